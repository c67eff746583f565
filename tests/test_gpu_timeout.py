"""The bounded waits on the device: the grid barriers of the cell scan and
of the matcher on steps with many candidate pairs.  With a test switch on,
CTA 0 of the kernel never arrives at its barrier; the other CTAs' waits run
out, the step stops with BD_ERR_TIMEOUT, and the context stays usable
(nothing faults, traps or hangs)."""
import time

import numpy as np
import pytest

from gpusmoldyn_gb300 import _lib as L
from gpusmoldyn_gb300.configs import rng, uniform_positions
from gpusmoldyn_gb300.system import System

pytestmark = pytest.mark.gpu


def system(seed):
    # 40^3 cells: several scan tiles of 8,192 cells, so the scan runs over several CTAs
    s = System((0, 0, 0), (20, 20, 20), dt=1e-3, seed=seed, normals="table", cell_size=0.5)
    A, B = s.add_species(1.0), s.add_species(1.0)
    s.add_reaction(2, [A, B], [A], 1.0)
    s.finalize()
    s.set_particles(uniform_positions(rng(seed), 20000, (0, 0, 0), (20, 20, 20)), (np.arange(20000) % 2).astype(np.int32))
    return s


def test_scan_wait_runs_out_and_reports_timeout():
    s = system(71)
    dims, _, _ = s.grid()
    assert int(np.prod(dims.astype(np.int64))) > 2 * 8192
    s.step(2)
    s.synchronize()
    L.check(s.lib.bd_debug_withhold_scan(s.h, 1), "withhold")
    t0 = time.perf_counter()
    s.step(1)
    with pytest.raises(L.BDError) as e:
        s.synchronize()
    assert e.value.code == L.BD_ERR_TIMEOUT
    assert time.perf_counter() - t0 < 30.0
    # the context is fine: another handle steps normally
    other = system(72)
    other.step(5)
    other.synchronize()
    assert other.step_count() == 5


def dense_system(seed):
    # the smoke system: its first step has about 24,500 candidate pairs, so
    # the matcher runs over its whole grid with barriers between passes
    s = System((0, 0, 0), (2.0, 2.0, 2.0), dt=1e-3, seed=seed, normals="table")
    A, B, Cc = s.add_species(1.0), s.add_species(1.0), s.add_species(0.5)
    s.add_reaction(2, [A, B], [Cc], 5.0)
    s.finalize()
    s.set_particles(uniform_positions(rng(seed), 4000, (0, 0, 0), (2, 2, 2)), (np.arange(4000) % 2).astype(np.int32))
    return s


def test_matcher_grid_barrier_wait_runs_out_and_reports_timeout():
    """The grid matcher's barrier waits are bounded: with the test switch on,
    CTA 0 never arrives, the other CTAs give up, the step stops with
    BD_ERR_TIMEOUT, and the context stays usable."""
    s = dense_system(73)
    L.check(s.lib.bd_debug_withhold_match(s.h, 1), "withhold")
    t0 = time.perf_counter()
    s.step(1)
    with pytest.raises(L.BDError) as e:
        s.synchronize()
    assert e.value.code == L.BD_ERR_TIMEOUT
    assert time.perf_counter() - t0 < 30.0
    # the same system without the switch reacts normally, and so does
    # another handle on the same context
    other = dense_system(73)
    other.step(2)
    other.synchronize()
    assert other.step_count() == 2 and other.event_counts()[0] > 1000
