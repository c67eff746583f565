"""The benchmark configurations themselves, GPU against the oracle, bit-exact.

Each configuration is built by the same `configs` functions the benchmark
uses, in table-normal mode (the reference's 4096 quantiles,
particles_kernel.cu:57, 156-162), and stepped on the GPU and by the CPU
oracle from the same state.  Slots, cell starts, candidate pairs with their
accept flags and event counters must be identical, in both sort modes, as
for ParticleSystem::update (particleSystem.cpp:829-1001):

* c1 as specified: 20k A + 20k B in a 10 um cube, k = 0.01 um^3/s,
  dt = 1 ms, 1,000 steps;
* the c2 network (reversible, pgemmax 0.2 falling back to b = 0) at 100k
  particles at the c2 density, 200 steps;
* the c3 network (8 species, 12 reactions) on a 262,144-particle cube at
  the c3 density, 20 steps;
* a c4-shaped ensemble of 16 instances with log-uniform sizes and scaled D
  and k_on, each instance checked against the oracle running it alone.

The candidate-pair search is also checked against an independent
brute-force neighbour search (a k-d tree over the records, distances in
float32 in the step's operation order): no pair of reactants within its
binding radius is left unreacted, so neither the grid nor the 27-cell walk
(collideD, particles_kernel.cu:444-497) loses a pair.
"""
import math

import numpy as np
import pytest

from gpusmoldyn_gb300 import _lib as L
from gpusmoldyn_gb300 import configs
from gpusmoldyn_gb300.system import System
from oracle import py as orc

from test_gpu_parity import gpu_records, run_parity, sort_pairs

pytestmark = pytest.mark.gpu

SORTS = ["binned", "compact"]


@pytest.mark.parametrize("sort", SORTS)
def test_c1_as_specified_bit_exact(sort):
    s = configs.build_c1(normals="table", sort=sort)
    assert abs(s.reaction_info(0)["bind_radius"] - 0.0133939) < 1e-6
    _, npairs, ev = run_parity(s, 1000, batch=50)
    # about 4 reactions per step: k [A][B] V dt = 0.01 * 20 * 20 * 1000 * 1e-3
    assert 2000 < ev[0] < 6000, ev
    s.close()


@pytest.mark.parametrize("sort", SORTS)
def test_c2_network_bit_exact(sort):
    n = 100_000
    side = float((n / configs.C2_DENSITY) ** (1 / 3))
    s = configs.c2_system(side=side, normals="table", sort=sort)
    fwd, back = s.reaction_info(0), s.reaction_info(1)
    assert back["flags"] & 1, "pgem 0.2 is unattainable: b falls back to 0"
    assert back["unbind_radius"] == 0.0
    assert abs(fwd["bind_radius"] - 0.0181319) < 1e-6
    s.set_particles(*configs.c2_particles(n // 2, n - n // 2, side))
    _, npairs, ev = run_parity(s, 200, batch=20)
    assert ev[0] > 100 and ev[1] > 0, ev
    s.close()


@pytest.mark.parametrize("sort", SORTS)
def test_c3_network_bit_exact(sort):
    n = 262_144
    side = (n / 2.0) ** (1 / 3)
    s = configs.build_c3(n=n, side=side, normals="table", sort=sort)
    _, npairs, ev = run_parity(s, 20)
    orders = [s.reaction_info(r)["order"] for r in range(s.n_reactions)]
    # births, first-order and second-order events all happen
    for order in (0, 1, 2):
        assert sum(int(ev[r]) for r in range(len(orders)) if orders[r] == order) > 0, (order, ev)
    assert npairs > 0
    s.close()


@pytest.mark.parametrize("sort", SORTS)
def test_c4_shaped_ensemble_instances_match_oracle_alone(sort):
    inst, counts = configs.c4_instances(16, seed=4, n_lo=1e3, n_hi=1e5)
    s = System(dt=5e-4, seed=4, normals="table", instances=inst, sort=sort)
    configs.c2_network(s)
    s.finalize()
    pos, sp = configs.c4_positions(inst, counts)
    s.set_ensemble_particles(pos, sp, counts)
    oracles = [orc.OracleSystem(s, instance=k) for k in range(len(inst))]
    off = np.concatenate([[0], np.cumsum(counts)])
    recs = [orc.records(pos[off[k]:off[k + 1]], sp[off[k]:off[k + 1]], inst=k) for k in range(len(inst))]
    ev = np.zeros(2, np.uint64)
    for t in range(20):
        s.step(1)
        s.synchronize()
        xyz, w = s.slots()
        got = orc.slots_to_records(xyz, w)
        for k, o in enumerate(oracles):
            recs[k] = o.step(t, recs[k], events=ev)["recs"]
            live = recs[k][recs[k][:, 3] != 0xFFFFFFFF]
            mine = got[(got[:, 3] != 0xFFFFFFFF) & ((got[:, 3] >> 16) == k)]
            np.testing.assert_array_equal(mine, live, err_msg=f"instance {k} step {t}")
    np.testing.assert_array_equal(s.instance_counts(), [int(np.sum(r[:, 3] != 0xFFFFFFFF)) for r in recs])
    np.testing.assert_array_equal(s.event_counts(), ev)
    assert ev[0] > 0
    s.close()


def brute_force_pairs(recs, radius2, n_species):
    """Unordered pairs (i < j) of live records whose species pair has a
    second-order reaction and whose squared distance, computed in float32 as
    (dx^2 + dy^2) + dz^2, is at most that reaction's radius^2 (in float)."""
    from scipy.spatial import cKDTree

    live = np.nonzero(recs[:, 3] != 0xFFFFFFFF)[0]
    xyz = recs[live, :3].view(np.float32)
    sp = (recs[live, 3] & 0xFFFF).astype(np.int64)
    rmax = math.sqrt(float(max(radius2.values())))
    cand = cKDTree(xyz.astype(np.float64)).query_pairs(rmax * 1.001, output_type="ndarray")
    if len(cand) == 0:
        return set()
    a, b = cand[:, 0], cand[:, 1]
    d = xyz[a] - xyz[b]
    d2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
    lim = np.full((n_species, n_species), -1.0, np.float32)
    for (p, q), r2 in radius2.items():
        lim[p, q] = lim[q, p] = r2
    keep = d2 <= lim[sp[a], sp[b]]
    i, j = live[a[keep]], live[b[keep]]
    return set(zip(np.minimum(i, j).tolist(), np.maximum(i, j).tolist()))


@pytest.mark.parametrize("sort", SORTS)
def test_c3_pair_search_misses_no_pair(sort):
    """The c3 network's six second-order reactions alone (no births, so no
    record is excluded as a newborn), at 50x their rates, on a
    262,144-particle cube.  Every reaction has probability 1, so the greedy
    matching accepts each candidate pair whose two records are still free:
    after the step no two records that did not react may lie within their
    binding radius.  A pair the grid or the 27-cell walk missed would be
    such a pair; a brute-force search over the unreacted records (which
    still hold the positions the pair search saw) finds none."""
    n = 262_144
    side = (n / 2.0) ** (1 / 3)
    D, rx = configs.c3_network()
    s = System((0, 0, 0), (side, side, side), dt=1e-3, seed=3, normals="table", sort=sort)
    for d in D:
        s.add_species(float(d))
    for order, rc, pr, k in rx:
        if order == 2:
            s.add_reaction(order, rc, pr, float(k) * 50.0)
    s.finalize()
    pos, sp = configs.c3_particles(n, side)
    s.set_particles(pos, sp)
    radius2 = {}
    for r in range(s.n_reactions):
        info = s.reaction_info(r)
        a = np.float32(info["bind_radius"])
        radius2[tuple(sorted(info["reactants"]))] = np.float32(a * a)
    for t in range(3):
        s.step(1)
        s.synchronize()
        got = gpu_records(s)
        pairs = sort_pairs(s.pairs())
        acc = pairs[pairs[:, 3] == 1]
        reacted = np.zeros(len(got), bool)
        reacted[acc[:, 0]] = True
        reacted[acc[:, 1]] = True
        assert len(acc) > 300, len(acc)
        # every candidate pair has a reacted end
        assert np.all(reacted[pairs[:, 0]] | reacted[pairs[:, 1]])
        recs = got.copy()
        recs[reacted, 3] = 0xFFFFFFFF
        missed = brute_force_pairs(recs, radius2, len(D))
        assert not missed, (t, len(missed), sorted(missed)[:5])
    s.close()
