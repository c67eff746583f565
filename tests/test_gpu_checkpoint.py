"""Checkpoint and resume: a handle built the same way and loaded from a
checkpoint continues bit for bit as the original."""
import numpy as np
import pytest

from gpusmoldyn_gb300 import _lib as L
from gpusmoldyn_gb300.configs import rng, uniform_positions
from gpusmoldyn_gb300.system import System
from test_gpu_parity import SORTS, gpu_records

pytestmark = pytest.mark.gpu


def build(sort, instances=None):
    kw = dict(dt=1e-3, seed=9, normals="boxmuller", sort=sort)
    s = System((0, 0, 0), (4, 4, 4), instances=instances, **kw) if instances else System((0, 0, 0), (4, 4, 4), **kw)
    A, B, Cc = s.add_species(1.0), s.add_species(1.0), s.add_species(0.5)
    s.add_reaction(2, [A, B], [Cc], 4.0)
    back = s.add_reaction(1, [Cc], [A, B], 30.0)
    s.set_product_placement(back, L.BD_PP_UNBINDRAD, 0.02)
    s.add_reaction(0, [], [A], 2000.0)
    s.finalize()
    return s


def populate(s, instances=None):
    g = rng(9)
    if instances:
        counts = [3000, 5000, 2000]
        pos = np.concatenate([uniform_positions(g, n, d["box_lo"], d["box_hi"]) for d, n in zip(instances, counts)])
        s.set_ensemble_particles(pos, (np.arange(len(pos)) % 2).astype(np.int32), counts)
    else:
        pos = uniform_positions(g, 20000, (0, 0, 0), (4, 4, 4))
        s.set_particles(pos, (np.arange(20000) % 2).astype(np.int32))


@pytest.mark.parametrize("sort", SORTS)
@pytest.mark.parametrize("ensemble", [False, True])
def test_resume_is_bit_exact(tmp_path, sort, ensemble):
    inst = [dict(box_lo=(0.0, 0.0, 0.0), box_hi=(2.0 + k, 2.0, 2.0), seed=40 + k, d_scale=1.0 + 0.3 * k)
            for k in range(3)] if ensemble else None
    a = build(sort, inst)
    populate(a, inst)
    a.step(15)
    a.synchronize()
    path = tmp_path / "run.ckpt"
    a.save_checkpoint(path)
    a.step(12)
    a.synchronize()
    want = gpu_records(a)
    want_events = a.event_counts()

    b = build(sort, inst)
    b.load_checkpoint(path)
    assert b.step_count() == 15
    b.step(12)
    b.synchronize()
    np.testing.assert_array_equal(gpu_records(b), want)
    np.testing.assert_array_equal(b.event_counts(), want_events)
    assert b.step_count() == 27 and want_events.sum() > 100


def test_checkpoint_of_another_build_is_refused(tmp_path):
    a = build("binned")
    populate(a)
    a.step(3)
    a.synchronize()
    path = tmp_path / "run.ckpt"
    a.save_checkpoint(path)
    other = System((0, 0, 0), (4, 4, 4), dt=2e-3, seed=9)  # another time step
    for d in (1.0, 1.0, 0.5):
        other.add_species(d)
    other.finalize()
    with pytest.raises(L.BDError) as e:
        other.load_checkpoint(path)
    assert e.value.code == L.BD_ERR_INVALID_ARGUMENT
    bad = tmp_path / "bad.ckpt"
    bad.write_bytes(b"not a checkpoint")
    with pytest.raises(L.BDError):
        a.load_checkpoint(bad)
