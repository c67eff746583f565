"""The launch count a handle reports (bd_get_kernels_per_step, which the
benchmark multiplies into its count of launches) equals the number of
kernels one profiled step enqueues, on every path: the binned and compact
sorts, with and without zeroth- and second-order reactions, with surfaces,
and the diffusion-only path."""
import numpy as np
import pytest

from gpusmoldyn_gb300 import _lib as L
from gpusmoldyn_gb300.configs import rng, uniform_positions
from gpusmoldyn_gb300.system import System

pytestmark = pytest.mark.gpu


def make(sort="binned", zeroth=False, first=True, second=True, panels=False):
    side = 4.0
    s = System((0, 0, 0), (side,) * 3, dt=1e-3, seed=61, normals="table", sort=sort)
    A, B, Cc = s.add_species(1.0), s.add_species(1.0), s.add_species(0.5)
    if second:
        s.add_reaction(2, [A, B], [Cc], 1.0)
    if first:
        s.add_reaction(1, [Cc], [], 1.0)
    if zeroth:
        s.add_reaction(0, [], [A], 50.0)
    if panels:
        f = s.add_surface()
        s.set_surface_action(f, L.BD_ALL_SPECIES, "both", "reflect")
        s.add_panel(f, "rect", [1.0, 0, 0, side, side], axis=0)
    s.finalize()
    n = 6000
    s.set_particles(uniform_positions(rng(61), n, (0, 0, 0), (side,) * 3), (np.arange(n) % 3).astype(np.int32))
    return s


@pytest.mark.parametrize("kw", [
    dict(sort="binned"),
    dict(sort="binned", zeroth=True),
    dict(sort="binned", second=False),
    dict(sort="binned", panels=True),
    dict(sort="compact"),
    dict(sort="compact", zeroth=True),
    dict(sort="compact", panels=True),
    dict(first=False, second=False),
    dict(first=False, second=False, zeroth=True),
], ids=lambda kw: "-".join(f"{k}={v}" for k, v in kw.items()))
def test_kernels_per_step_matches_the_profiled_step(kw):
    s = make(**kw)
    s.step(2)
    s.synchronize()
    prof = s.profile_steps(1)
    assert s.kernels_per_step() == len(prof), sorted(prof)
    s.close()
