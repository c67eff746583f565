"""The oracle's own derivation of the step's inputs (oracle/params.py)
against the library's, on the CPU.

Parity tests feed the oracle the library's derived inputs; here the same
inputs are derived a second time by an independent restatement of the
reference's setup code (rxnparam.cpp:42-308, smolreact.cpp:283-483,
stats.cpp:202-275) and of the grid rule, and must agree exactly: species D,
reaction probabilities, binding radii, unbinding offsets, Poisson CDFs,
each instance's grid and the normal table.  A wrong derived input in the
library would therefore no longer be copied unnoticed into the oracle.
"""
import numpy as np
import pytest

from gpusmoldyn_gb300 import _lib as L
from gpusmoldyn_gb300 import configs
from gpusmoldyn_gb300.system import System, gauss_table
from oracle import params as P
from oracle import py as orc


def compare(s, o, instance=0):
    """Library handle s against OracleSystem o built by from_network."""
    dims, cell, inv = s.grid(instance)
    odims, ocell, oinv = o.grid
    np.testing.assert_array_equal(dims, odims)
    np.testing.assert_array_equal(cell.view(np.uint32), ocell.view(np.uint32))
    np.testing.assert_array_equal(inv.view(np.uint32), oinv.view(np.uint32))
    np.testing.assert_array_equal(s.species_d(instance).view(np.uint32), o.arrs["D"].view(np.uint32))
    for r in range(s.n_reactions):
        info = s.reaction_info(r, instance)
        for key, arr in (("prob", "prob"), ("bind_radius", "bind_radius")):
            assert np.float32(info[key]).view(np.uint32) == o.arrs[arr][r].view(np.uint32), (r, key, info[key],
                                                                                           o.arrs[arr][r])
        assert np.float32(info["product_offsets"][0]) == o.arrs["off0"][r], r
        assert np.float32(info["product_offsets"][1]) == o.arrs["off1"][r], r
        assert (info["flags"] & 1) == (o.derived["flags"][r] & 1), r
        if info["order"] == 0:
            cdf, kmin = s.poisson_cdf(r, instance)
            ocdf = o.derived["cdf"][r]
            assert kmin == o.derived["cdf_kmin"][r]
            np.testing.assert_array_equal(cdf.view(np.uint64), ocdf.view(np.uint64))


def reactions_of(rx, placements=None):
    placements = placements or {}
    out = []
    for r, (order, rc, pr, k) in enumerate(rx):
        kind, param, prob = placements.get(r, (P.PP_DEFAULT, 0.0, -1.0))
        out.append(P.Reaction(order, rc, pr, k, kind, param, prob))
    return out


def zero_particles(n):
    return np.zeros((n, 4), np.float32), np.zeros(n, np.int32)


@pytest.mark.parametrize("n", [262_144, 16_000_000])
def test_c3_inputs(n):
    side = 200.0 * (n / 16_000_000) ** (1 / 3)
    s = configs.c3_system(n=n, side=side, device=-1)
    s.set_particles(*zero_particles(n))
    D, rx, _ = configs.c3_reactions(n / side ** 3)
    o = orc.OracleSystem.from_network(D, reactions_of(rx), (0, 0, 0), (side,) * 3, 1e-3, 3, n)
    compare(s, o)
    s.close()


def test_c1_and_c2_inputs():
    s = configs.build_c1(device=-1)
    o = orc.OracleSystem.from_network([1.0, 1.0, 0.5], reactions_of([(2, [0, 1], [2], 0.01)]), (0, 0, 0),
                                      (10.0,) * 3, 1e-3, 1, 40000)
    compare(s, o)
    s.close()
    s = configs.c2_system(device=-1)
    s.set_particles(*zero_particles(1_000_000))
    rx = [(2, [0, 1], [2], 0.05), (1, [2], [0, 1], 10.0)]
    o = orc.OracleSystem.from_network([1.0, 1.0, 0.5], reactions_of(rx, {1: (P.PP_PGEMMAX, 0.2, -1.0)}),
                                      (0, 0, 0), (60.0,) * 3, 5e-4, 2, 1_000_000)
    compare(s, o)
    assert o.derived["flags"][1] & 1  # pgem 0.2 is unattainable: b = 0
    s.close()


def test_c4_instance_inputs():
    inst, counts = configs.c4_instances()
    s = System(dt=5e-4, seed=4, instances=inst, device=-1)
    configs.c2_network(s)
    s.finalize()
    s.set_ensemble_particles(*zero_particles(int(np.sum(counts))), counts)
    rx = reactions_of([(2, [0, 1], [2], 0.05), (1, [2], [0, 1], 10.0)], {1: (P.PP_PGEMMAX, 0.2, -1.0)})
    for k in range(0, len(inst), 17):
        d = inst[k]
        o = orc.OracleSystem.from_network([1.0, 1.0, 0.5], rx, d["box_lo"], d["box_hi"], 5e-4, d["seed"],
                                          int(counts[k]), d_scale=d["d_scale"], k2_scale=d["k2_scale"])
        compare(s, o, k)
    s.close()


@pytest.mark.parametrize("kind,param", [(P.PP_UNBINDRAD, 0.02), (P.PP_PGEM, 0.1), (P.PP_PGEMMAX, 0.05),
                                        (P.PP_OFFSET0, 0.0)])
def test_reversible_placements(kind, param):
    s = System((0, 0, 0), (2.0, 2.0, 2.0), dt=5e-4, seed=14, device=-1)
    A, B, Cc = s.add_species(1.0), s.add_species(0.7), s.add_species(0.5)
    s.add_reaction(2, [A, B], [Cc], 2.0)
    u = s.add_reaction(1, [Cc], [A, B], 30.0)
    s.set_product_placement(u, kind, param)
    s.finalize()
    s.set_particles(*zero_particles(5000))
    rx = reactions_of([(2, [0, 1], [2], 2.0), (1, [2], [0, 1], 30.0)], {1: (kind, param, -1.0)})
    o = orc.OracleSystem.from_network([1.0, 0.7, 0.5], rx, (0, 0, 0), (2.0,) * 3, 5e-4, 14, 5000)
    compare(s, o)
    s.close()


def test_mixed_network_inputs():
    """Zeroth order with one and two products, competing first-order
    reactions of one species, a homodimer and a per-encounter probability."""
    s = System((0, 0, 0), (3.0, 4.0, 5.0), dt=1e-3, seed=9, device=-1)
    for d in (1.0, 0.4, 2.0, 0.0):
        s.add_species(d)
    rx = [(0, [], [0], 30.0), (0, [], [1, 2], 5.0), (1, [0], [1], 4.0), (1, [0], [], 2.5), (1, [0], [2, 2], 7.0),
          (2, [1, 1], [3], 0.3), (2, [0, 2], [1], 1.2), (1, [3], [1, 1], 1.0)]
    for order, rc, pr, k in rx:
        s.add_reaction(order, rc, pr, k)
    s.set_reaction_probability(6, 0.4)
    s.set_product_placement(4, L.BD_PP_UNBINDRAD, 0.015)
    s.finalize()
    s.set_particles(*zero_particles(20000))
    o = orc.OracleSystem.from_network([1.0, 0.4, 2.0, 0.0],
                                      reactions_of(rx, {6: (P.PP_DEFAULT, 0.0, 0.4),
                                                        4: (P.PP_UNBINDRAD, 0.015, -1.0)}),
                                      (0, 0, 0), (3.0, 4.0, 5.0), 1e-3, 9, 20000)
    compare(s, o)
    s.close()


def test_gauss_quantiles():
    np.testing.assert_array_equal(P.gauss_quantiles().view(np.uint32), gauss_table().view(np.uint32))
