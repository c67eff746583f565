"""The benchmark configurations' derived inputs, on host-only handles (no GPU).

The oracle takes the grid, the reaction parameters and the Poisson CDFs from
the library's handle, so these inputs are checked here on their own, at the
configurations' full sizes:

* grid sizing: every instance's cell edge is at least 1.01 x the largest
  binding radius of that instance, so every reacting pair lies within the
  27-cell neighbourhood that the step (and the oracle) searches -- the
  reference's cell of 2 x particleRadius (particleSystem.cpp:69-76) is
  unrelated to the binding radius and is not kept;
* the planned occupancy is near the target of 3 records per cell;
* the zeroth-order Poisson CDFs at the c3 rates: their exact mean and
  variance equal the Poisson mean k dt V (smolreact.cpp:295-303) and their
  lost tail mass is negligible (poisrandF, stats.cpp:234-275, is pinned
  against the reference's own sampler in test_rxnparam.py).
"""
import numpy as np
import pytest

from gpusmoldyn_gb300 import configs
from gpusmoldyn_gb300.system import System


def zero_particles(n):
    # calloc'd pages read as zeros without being backed: (0, 0, 0) lies in
    # every configuration's box
    return np.zeros((n, 4), np.float32), np.zeros(n, np.int32)


def check_grid(s, instance, n):
    dims, cell, inv = s.grid(instance)
    radii = [s.reaction_info(r, instance)["bind_radius"] for r in range(s.n_reactions)
             if s.reaction_info(r, instance)["order"] == 2]
    a_max = max(radii)
    assert np.all(cell >= 1.01 * a_max * (1 - 1e-6)), (instance, cell, a_max)
    # cell[a] * dims[a] spans the box, and inv is dims / L in float
    n_cells = int(np.prod(dims.astype(np.int64)))
    occ = n / n_cells
    return occ, a_max


def test_c1_grid():
    s = System((0, 0, 0), (10, 10, 10), dt=1e-3, seed=1, device=-1)
    A, B, Cc = s.add_species(1.0), s.add_species(1.0), s.add_species(0.5)
    s.add_reaction(2, [A, B], [Cc], 0.01)
    s.finalize()
    s.set_particles(*zero_particles(40000))
    occ, a = check_grid(s, 0, 40000)
    assert abs(a - 0.0133939) < 1e-6   # the reference's own bindingradius (F4)
    assert 2.0 < occ < 4.5
    s.close()


def test_c2_grid():
    s = configs.c2_system(device=-1)
    s.set_particles(*zero_particles(1_000_000))
    occ, a = check_grid(s, 0, 1_000_000)
    assert abs(a - 0.0181319) < 1e-6   # b = 0 fallback of the unattainable pgem 0.2
    assert 2.0 < occ < 4.5
    s.close()


def test_c3_grid_and_poisson_cdfs():
    n = 16_000_000
    s = configs.c3_system(n=n, device=-1)
    s.set_particles(*zero_particles(n))
    occ, a = check_grid(s, 0, n)
    assert 2.0 < occ < 4.5
    V = 200.0 ** 3
    for r in range(s.n_reactions):
        info = s.reaction_info(r)
        if info["order"] != 0:
            continue
        lam = float(np.float32(info["rate"]) * np.float32(1e-3) * np.float32(V))
        cdf, kmin = s.poisson_cdf(r)
        pmf = np.diff(np.concatenate([[0.0], cdf]))
        k = kmin + np.arange(len(pmf))
        mean = float(np.sum(k * pmf))
        var = float(np.sum((k - mean) ** 2 * pmf))
        assert abs(info["prob"] - lam) <= 1e-6 * lam
        assert abs(mean - info["prob"]) < 1e-9 * info["prob"], (mean, info["prob"])
        assert abs(var - info["prob"]) < 1e-6 * info["prob"], (var, info["prob"])
        assert cdf[-1] > 1 - 1e-12
        assert np.all(np.diff(cdf) >= 0)
    s.close()


def test_c4_grids_per_instance():
    inst, counts = configs.c4_instances()
    s = System(dt=5e-4, seed=4, instances=inst, device=-1)
    configs.c2_network(s)
    s.finalize()
    total = int(np.sum(counts))
    pos, sp = zero_particles(total)
    s.set_ensemble_particles(pos, sp, counts)
    occs = []
    for k in range(len(inst)):
        occ, a = check_grid(s, k, int(counts[k]))
        occs.append(occ)
        # the binding radius grows with the instance's rate scale
        assert a > 0
    assert 2.0 < np.median(occs) < 4.5
    s.close()


@pytest.mark.parametrize("job", range(4))
def test_c5_request_grids(job):
    from gpusmoldyn_gb300.serve import c3_request

    j = configs.c5_jobs(4, seed=5)[job]
    desc, pos, sp, _ = c3_request(j)
    side = desc["box_hi"][0]
    s = configs.c3_system(n=len(sp), side=side, seed=j["seed"], device=-1)
    s.set_particles(pos, sp)
    occ, _ = check_grid(s, 0, len(sp))
    assert 1.0 < occ < 6.0
    s.close()
