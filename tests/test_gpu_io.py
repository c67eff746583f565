"""Particles in and out through the C ABI: the device-side check, packing
and export of bd_set_particles / bd_get_particles."""
import numpy as np
import pytest

from gpusmoldyn_gb300 import _lib as L
from gpusmoldyn_gb300.configs import rng, uniform_positions
from gpusmoldyn_gb300.system import System

pytestmark = pytest.mark.gpu


def small(seed=51, n=5000):
    s = System((0, 0, 0), (3, 3, 3), dt=1e-3, seed=seed, normals="table")
    A, B, Cc = s.add_species(1.0), s.add_species(1.0), s.add_species(0.5)
    s.add_reaction(2, [A, B], [Cc], 5.0)
    s.finalize()
    pos = uniform_positions(rng(seed), n, (0, 0, 0), (3, 3, 3))
    sp = (np.arange(n) % 2).astype(np.int32)
    return s, pos, sp


def test_upload_round_trip_and_rejects_bad_input():
    s, pos, sp = small()
    s.set_particles(pos, sp)
    p4, q = s.particles4()
    np.testing.assert_array_equal(p4[:, :3], pos)
    assert (p4[:, 3] == 1.0).all()
    np.testing.assert_array_equal(q, sp)
    s.step(10)
    s.synchronize()
    before = s.slots()
    n_before = s.count()
    bad_species = sp.copy()
    bad_species[1234] = 7
    outside = pos.copy()
    outside[99, 2] = 3.5
    for args in ((pos, bad_species), (outside, sp), (pos, -np.ones_like(sp))):
        with pytest.raises(L.BDError) as e:
            s.set_particles(*args)
        assert e.value.code == L.BD_ERR_INVALID_ARGUMENT
    # nothing of the handle changed
    assert s.count() == n_before
    after = s.slots()
    np.testing.assert_array_equal(before[0], after[0])
    np.testing.assert_array_equal(before[1], after[1])
    s.step(5)
    s.synchronize()


def test_export_is_the_live_slots_in_order():
    s, pos, sp = small(seed=52, n=20000)
    s.set_particles(pos, sp)
    s.step(30)
    s.synchronize()
    xyz, w = s.slots()
    live = w != L.DEAD
    assert (~live).sum() > 0  # pair reactions left holes
    p4, q = s.particles4()
    np.testing.assert_array_equal(p4[:, :3], xyz[live])
    np.testing.assert_array_equal(q, (w[live] & 0xFFFF).astype(np.int32))
    # into arrays the caller keeps
    out = (np.full((30000, 4), -1, np.float32), np.full(30000, -1, np.int32))
    p4b, qb = s.particles4(out=out)
    np.testing.assert_array_equal(p4b, p4)
    np.testing.assert_array_equal(qb, q)
    assert out[1][len(q)] == -1  # nothing written past the live count
    xyz3, q3 = s.particles()
    np.testing.assert_array_equal(xyz3, p4[:, :3])


def test_ensemble_upload_assigns_instances():
    counts = [700, 0, 1300, 400]
    inst = [dict(box_lo=(0.0, 0.0, 0.0), box_hi=(1.0 + k, 1.0, 1.0), seed=60 + k) for k in range(4)]
    s = System(dt=1e-3, seed=1, normals="table", instances=inst)
    s.add_species(1.0)
    s.add_species(2.0)
    s.add_reaction(1, [0], [1], 1.0)
    s.finalize()
    g = rng(61)
    pos = np.concatenate([uniform_positions(g, n, d["box_lo"], d["box_hi"]) for d, n in zip(inst, counts)])
    sp = (np.arange(len(pos)) % 2).astype(np.int32)
    s.set_ensemble_particles(pos, sp, counts)
    np.testing.assert_array_equal(s.instance_counts(), counts)
    for k in range(4):
        p4, q = s.particles4(instance=k)
        off = sum(counts[:k])
        np.testing.assert_array_equal(p4[:, :3], pos[off:off + counts[k]])
        np.testing.assert_array_equal(q, sp[off:off + counts[k]])
    # instance 0's box is the unit cube: a particle of instance 0 at x = 1.5 is outside
    bad = pos.copy()
    bad[5, 0] = 1.5
    with pytest.raises(L.BDError):
        s.set_ensemble_particles(bad, sp, counts)


def test_export_into_short_and_pinned_arrays():
    """An array shorter than the live count receives its first entries and
    nothing past them; positions alone may be asked for; pinned arrays
    receive the same result as pageable ones."""
    import ctypes as C

    import torch

    from gpusmoldyn_gb300.system import _ptr

    s, pos, sp = small(seed=53, n=20000)
    s.set_particles(pos, sp)
    s.step(20)
    s.synchronize()
    p4, q = s.particles4()
    m = len(q) // 3
    short = (np.full((m + 8, 4), -1, np.float32), np.full(m + 8, -1, np.int32))
    got = C.c_size_t()
    L.check(s.lib.bd_get_instance_particles(s.h, -1, _ptr(short[0]), _ptr(short[1]), m, C.byref(got)),
            "bd_get_particles")
    assert got.value == len(q)
    np.testing.assert_array_equal(short[0][:m], p4[:m])
    np.testing.assert_array_equal(short[1][:m], q[:m])
    assert (short[0][m:] == -1).all() and (short[1][m:] == -1).all()
    # positions only
    only = np.full((len(q), 4), -1, np.float32)
    L.check(s.lib.bd_get_instance_particles(s.h, -1, _ptr(only), None, len(q), C.byref(got)), "bd_get_particles")
    np.testing.assert_array_equal(only, p4)
    pin_p = torch.full((len(q) + 8, 4), -1.0, dtype=torch.float32).pin_memory()
    pin_s = torch.full((len(q) + 8,), -1, dtype=torch.int32).pin_memory()
    p4c, qc = s.particles4(out=(pin_p.numpy(), pin_s.numpy()))
    np.testing.assert_array_equal(p4c, p4)
    np.testing.assert_array_equal(qc, q)
    assert (pin_s.numpy()[len(q):] == -1).all()
    s.close()
