"""The one bounded wait on the device: the single-pass cell scan's look-back.
With the test switch on, the scan's first tile keeps its sum to itself; the
next tile's wait for it runs out, the step stops with BD_ERR_TIMEOUT, and the
context stays usable (nothing faults, traps or hangs)."""
import time

import numpy as np
import pytest

from gpusmoldyn_gb300 import _lib as L
from gpusmoldyn_gb300.configs import rng, uniform_positions
from gpusmoldyn_gb300.system import System

pytestmark = pytest.mark.gpu


def system(seed):
    # 40^3 cells: several scan tiles of 16,384 cells, so a tile has a predecessor
    s = System((0, 0, 0), (20, 20, 20), dt=1e-3, seed=seed, normals="table", cell_size=0.5)
    A, B = s.add_species(1.0), s.add_species(1.0)
    s.add_reaction(2, [A, B], [A], 1.0)
    s.finalize()
    s.set_particles(uniform_positions(rng(seed), 20000, (0, 0, 0), (20, 20, 20)), (np.arange(20000) % 2).astype(np.int32))
    return s


def test_scan_wait_runs_out_and_reports_timeout():
    s = system(71)
    dims, _, _ = s.grid()
    assert int(np.prod(dims.astype(np.int64))) > 2 * 16384
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
