"""Continuous batching: simulations admitted into a running serving handle
give the same result as when each runs alone, bit for bit, and stop exactly
at their requested step count."""
import numpy as np
import pytest

from gpusmoldyn_gb300 import _lib as L
from gpusmoldyn_gb300.configs import rng, uniform_positions
from gpusmoldyn_gb300.system import System

pytestmark = pytest.mark.gpu


def network(s):
    A, B, Cc = s.add_species(1.0), s.add_species(1.0), s.add_species(0.5)
    s.add_reaction(2, [A, B], [Cc], 2.0)
    back = s.add_reaction(1, [Cc], [A, B], 40.0)
    s.set_product_placement(back, L.BD_PP_UNBINDRAD, 0.01)
    s.add_reaction(0, [], [A], 300.0)
    s.finalize()


def job(k):
    n = [3000, 12000, 700, 6000][k]
    side = float((n / 2000.0) ** (1 / 3))
    desc = dict(box_lo=(0.0, 0.0, 0.0), box_hi=(side, side, side), seed=77 + k, d_scale=[1.0, 0.7, 1.4, 1.1][k],
                k2_scale=[1.0, 2.0, 0.5, 1.5][k])
    g = rng(500 + k)
    pos = uniform_positions(g, n, desc["box_lo"], desc["box_hi"])
    sp = (np.arange(n) % 2).astype(np.int32)
    return desc, pos, sp, [30, 55, 80, 41][k]


def run_until_frozen(s, slot, chunk=7):
    while True:
        if slot in s.poll():
            return s.harvest(slot)
        s.step(chunk)
        s.synchronize()


def test_same_alone_and_in_the_mix():
    alone = {}
    for k in range(4):
        s = System(dt=1e-3, instances=1)
        network(s)
        desc, pos, sp, steps = job(k)
        slot = s.admit(desc, pos, sp, steps)
        alone[k] = run_until_frozen(s, slot)
        s.close()

    mix = System(dt=1e-3, instances=3)
    network(mix)
    results, slots, admitted = {}, {}, []
    pending = [0, 1, 2, 3]
    t = 0
    while pending or slots:
        # admit as slots free up, at staggered times
        if pending and len(slots) < 3 and t % 9 == 0:
            k = pending.pop(0)
            desc, pos, sp, steps = job(k)
            slots[mix.admit(desc, pos, sp, steps)] = k
        mix.step(3)
        t += 3
        for slot in mix.poll():
            steps_done, flags = mix.instance_state(slot)
            k = slots.pop(slot)
            assert steps_done == job(k)[3] and flags & 2
            results[k] = mix.harvest(slot)
    mix.close()
    for k in range(4):
        pa, sa = alone[k]
        pm, sm = results[k]
        assert pa.shape == pm.shape and len(pa) > 0
        np.testing.assert_array_equal(pa, pm, err_msg=f"job {k}")
        np.testing.assert_array_equal(sa, sm, err_msg=f"job {k}")


def test_server_slots_are_reused():
    s = System(dt=1e-3, instances=2)
    network(s)
    for rnd in range(3):
        got = []
        for k in (0, 2):
            desc, pos, sp, _ = job(k)
            got.append(s.admit(desc, pos, sp, 5))
        assert sorted(got) == [0, 1]
        done = []
        while len(done) < 2:
            s.step(2)
            s.synchronize()
            for slot in s.poll():
                done.append(slot)
                p, q = s.harvest(slot)
                assert len(p) > 0
        s.step(1)  # drops the harvested records, frees the slots
        s.synchronize()
    s.close()


def test_harvest_after_frozen_steps_equals_harvest_at_the_freeze():
    """Right after the freeze the harvest sorts on the host (products still
    sit in their reactants' slots); after a frozen step the records are in
    canonical order on the device and the harvest exports them as they lie.
    Both give the same particles, in the same order."""
    results = []
    for extra in (0, 1, 5):
        s = System(dt=1e-3, instances=2)
        network(s)
        desc, pos, sp, steps = job(1)
        slot = s.admit(desc, pos, sp, steps)
        other = s.admit(*job(0))  # a neighbour that keeps running
        s.step(steps)
        s.synchronize()
        assert slot in s.poll()
        s.step(extra)
        s.synchronize()
        results.append(s.harvest(slot))
        s.close()
        del other
    for pos, sp in results[1:]:
        np.testing.assert_array_equal(pos, results[0][0])
        np.testing.assert_array_equal(sp, results[0][1])
    assert len(results[0][1]) > 1000


def test_cancel_mid_flight_leaves_the_others_unchanged():
    """A request cancelled while it runs takes no further step and its
    records are gone after the next one; the other instances still evolve
    bit for bit as alone, the cancelled slot is never polled, and the next
    admission takes it."""
    alone = {}
    for k in (0, 2):
        s = System(dt=1e-3, instances=1)
        network(s)
        desc, pos, sp, steps = job(k)
        slot = s.admit(desc, pos, sp, steps)
        alone[k] = run_until_frozen(s, slot)
        s.close()
    mix = System(dt=1e-3, instances=3)
    network(mix)
    slots = {}
    for k in (0, 1, 2):
        desc, pos, sp, steps = job(k)
        slots[k] = mix.admit(desc, pos, sp, steps)
    mix.step(10)
    mix.synchronize()
    assert mix.instance_counts()[slots[1]] > 0
    mix.cancel(slots[1])
    with pytest.raises(L.BDError) as e:
        mix.cancel(slots[1])
    assert e.value.code == L.BD_ERR_INVALID_ARGUMENT
    mix.step(1)
    mix.synchronize()
    assert mix.instance_counts()[slots[1]] == 0
    # the only free slot is the cancelled one
    desc, pos, sp, _ = job(3)
    new = mix.admit(desc, pos, sp, 5)
    assert new == slots[1]
    results, pending = {}, {slots[0]: 0, slots[2]: 2, new: 3}
    while pending:
        for slot in mix.poll():
            assert slot in pending
            results[pending.pop(slot)] = mix.harvest(slot)
        mix.step(3)
        mix.synchronize()
    mix.close()
    assert len(results[3][0]) > 0
    for k in (0, 2):
        np.testing.assert_array_equal(alone[k][0], results[k][0], err_msg=f"job {k}")
        np.testing.assert_array_equal(alone[k][1], results[k][1], err_msg=f"job {k}")
