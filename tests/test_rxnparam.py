"""Parameter derivation pinned against the reference's own compiled code.

tests/golden/reference_kat.json was produced by oracle/ref_kat.cpp linked
with the reference's rxnparam.cpp / smolreact.cpp / stats.cpp (see
tests/golden/make_golden.py).  The library's rate tables are regenerated by
its own solver (gpusmoldyn_gb300/rate_tables_gen.py) and agree with the
reference's printed tables to their 6 decimals, so rates agree to ~1e-6 a^3.
"""
import json
import math
import os

import numpy as np
import pytest

from gpusmoldyn_gb300 import _lib as L
from gpusmoldyn_gb300.system import System, actrxnrate, bindingradius, gauss_table, numrxnrate, unbindingradius

KAT = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_kat.json")))


def test_numrxnrate_grid():
    worst = 0.0
    for step, a, b, ref in KAT["numrxnrate"]:
        v = numrxnrate(step, a, b)
        # table entries agree to 1e-6; cubic weights amplify by at most ~10
        tol = 2e-5 * a ** 3 + 1e-12 * abs(ref)
        assert abs(v - ref) <= tol, (step, a, b, v, ref)
        worst = max(worst, abs(v - ref) / a ** 3)
    assert worst < 2e-5


def test_actrxnrate():
    for step, a, ref in KAT["actrxnrate"]:
        assert actrxnrate(step, a) == pytest.approx(ref, rel=1e-6)


def test_bindingradius():
    for rate, dt, difc, b, rel, ref in KAT["bindingradius"]:
        v = bindingradius(rate, dt, difc, b, rel)
        assert v == pytest.approx(ref, rel=1e-4, abs=1e-12), (rate, dt, difc, b, rel)


def test_bindingradius_config_values():
    # the binding radii of the benchmark configurations
    assert bindingradius(0.01, 1e-3, 2.0, -1, 0) == pytest.approx(0.0133939, rel=1e-5)
    assert bindingradius(0.05, 5e-4, 2.0, -1, 0) == pytest.approx(0.018413, rel=1e-5)
    assert bindingradius(0.05, 5e-4, 2.0, 0, 0) == pytest.approx(0.0181319, rel=1e-5)
    assert numrxnrate(1, 1, -1) == pytest.approx(2.72398, rel=1e-5)
    assert actrxnrate(1, 1) == pytest.approx(3.53276, rel=1e-5)


def test_unbindingradius():
    for pgem, dt, difc, a, ref in KAT["unbindingradius"]:
        v = unbindingradius(pgem, dt, difc, a)
        assert v == pytest.approx(ref, rel=1e-4, abs=1e-9), (pgem, dt, difc, a)
    # maximum geminate probability of config 2 (returned negated) at the
    # irreversible radius and at the b = 0 radius
    a_irr = bindingradius(0.05, 5e-4, 2.0, -1, 0)
    assert unbindingradius(0.2, 5e-4, 2.0, a_irr) == pytest.approx(-0.0452765, rel=1e-4)
    a2 = bindingradius(0.05, 5e-4, 2.0, 0, 0)
    assert unbindingradius(0.2, 5e-4, 2.0, a2) == pytest.approx(KAT["unbindingradius"][0][4], rel=1e-6)


def test_gauss_table_matches_reference_quantiles():
    mine = gauss_table()
    ref = np.array(KAT["gauss_table"], np.float32)
    assert mine.shape == ref.shape == (4096,)
    # the reference bisects a float erf approximation (30 steps on [-20, 20]);
    # ours is exact in double: they agree to 1e-5 relative, tails included
    assert np.max(np.abs(mine - ref) / np.maximum(np.abs(ref), 0.01)) < 1e-5
    assert np.all(np.diff(mine[:2048]) > 0)
    assert float(np.mean(mine)) == pytest.approx(0.0, abs=1e-7)
    assert float(np.var(mine.astype(np.float64))) == pytest.approx(0.99968, abs=2e-4)


def _host(box_hi=(10.0, 10.0, 10.0), dt=1e-3):
    return System((0, 0, 0), box_hi, dt=dt, device=-1)


def _network(name, box_hi):
    net = KAT["networks"][name]
    s = _host(box_hi, net["dt"])
    return s, net


def test_irreversible_network_matches_reference():
    s, net = _network("irreversible", (10.0, 10.0, 10.0))
    for d in (0.0, 1.0, 1.0, 0.5):
        s.add_species(d)
    r = s.add_reaction(2, [1, 2], [3], 0.01)
    s.finalize()
    info = s.reaction_info(r)
    ref = net["reactions"][0]
    assert np.float32(info["bind_radius"]) ** 2 == pytest.approx(ref["bind_r2"], rel=1e-6)
    assert info["prob"] == ref["prob"] == 1.0


def test_mixed_network_matches_reference():
    # box volume 90, the reference's systemVolume for zeroth order
    s, net = _network("mixed", (90.0, 1.0, 1.0))
    for d in (0.0, 0.7, 0.3, 2.0, 0.1):
        s.add_species(d)
    s.add_reaction(1, [1], [2], 5.0)
    s.add_reaction(1, [1], [], 3.0)
    s.add_reaction(1, [1], [2, 3], 7.5)
    s.add_reaction(2, [3, 3], [4], 0.08)
    s.add_reaction(0, [], [1], 2.5)
    s.add_reaction(1, [4], [], 1.0)
    s.add_reaction(2, [2, 4], [1], 0.02)
    s.finalize()
    for r, ref in enumerate(net["reactions"]):
        info = s.reaction_info(r)
        assert ref["rxnsetrate"] == 0 and ref["rxnsetproduct"] == 0
        assert info["prob"] == pytest.approx(ref["prob"], rel=2e-7), r
        if ref["order"] == 2:
            assert np.float32(info["bind_radius"]) ** 2 == pytest.approx(ref["bind_r2"], rel=2e-4), r
        assert info["product_offsets"] == pytest.approx(ref["offsets"], abs=1e-12)


def test_reversible_network_semantics():
    """A + B <-> C.  The reference computes the forward radius with the
    irreversible formula and fails to set the unbinding radius (error 7,
    geminate probability read from the wrong reaction).  The library uses
    Smoldyn's intended rule: pgemmax 0.2 is above the attainable 4.5%, so
    b = 0 and the forward radius is calibrated at b = 0."""
    s, net = _network("reversible", (60.0, 60.0, 60.0))
    for d in (0.0, 1.0, 1.0, 0.5):
        s.add_species(d)
    f = s.add_reaction(2, [1, 2], [3], 0.05)
    u = s.add_reaction(1, [3], [1, 2], 10.0)
    s.set_product_placement(u, L.BD_PP_PGEMMAX, 0.2)
    assert s.finalize() == L.BD_OK
    fi, ui = s.reaction_info(f), s.reaction_info(u)
    ref_f, ref_u = net["reactions"]
    assert ref_u["rxnsetproduct"] == 7
    assert ui["prob"] == pytest.approx(ref_u["prob"], rel=1e-7)  # 0.00498754
    assert ui["prob"] == pytest.approx(0.00498754, rel=1e-5)
    assert fi["bind_radius"] == pytest.approx(0.0181319, rel=1e-5)
    assert ui["unbind_radius"] == 0.0 and ui["flags"] & 1
    # the attainable maximum at this radius (0.0452765 at the irreversible one)
    assert ui["geminate_prob"] == pytest.approx(-KAT["unbindingradius"][0][4], rel=1e-5)
    assert fi["reverse"] == u and ui["reverse"] == f


def test_reversible_attainable_pgem_is_self_consistent():
    s = _host((60.0, 60.0, 60.0), 5e-4)
    for d in (1.0, 1.0, 0.5):
        s.add_species(d)
    f = s.add_reaction(2, [0, 1], [2], 0.05)
    u = s.add_reaction(1, [2], [0, 1], 10.0)
    s.set_product_placement(u, L.BD_PP_PGEM, 0.02)
    assert s.finalize() == L.BD_OK
    fi, ui = s.reaction_info(f), s.reaction_info(u)
    a, b = fi["bind_radius"], ui["unbind_radius"]
    step = math.sqrt(2 * 2.0 * 5e-4)
    assert b > a
    # forward rate reproduced with rebinding, pgem reproduced at that a
    assert numrxnrate(step, a, b) == pytest.approx(0.05 * 5e-4, rel=2e-4)
    pg = 1 - numrxnrate(step, a, -1) / numrxnrate(step, a, b)
    assert pg == pytest.approx(0.02, rel=2e-3)
    assert ui["product_offsets"][0] == pytest.approx(b * 0.5, rel=1e-6)
    assert ui["product_offsets"][1] == pytest.approx(-b * 0.5, rel=1e-6)
    # pgem above the maximum is an error (rxnsetproduct's code 8)
    s2 = _host((60.0, 60.0, 60.0), 5e-4)
    for d in (1.0, 1.0, 0.5):
        s2.add_species(d)
    s2.add_reaction(2, [0, 1], [2], 0.05)
    u2 = s2.add_reaction(1, [2], [0, 1], 10.0)
    s2.set_product_placement(u2, L.BD_PP_PGEM, 0.2)
    assert s2.lib.bd_finalize(s2.h) == L.BD_ERR_PGEM_UNATTAINABLE


def test_poisson_cdf_against_reference_sampler():
    """Zeroth-order counts come from inversion of a Poisson CDF; its moments
    match the mean and the reference sampler's (poisrandF) sample moments."""
    g = np.random.Generator(np.random.Philox(7))
    for mean, n, ref_mu, ref_var in KAT["poisson"]:
        s = _host((1.0, 1.0, 1.0), 1.0)
        s.add_species(1.0)
        r = s.add_reaction(0, [], [0], mean)
        s.finalize()
        assert s.reaction_info(r)["prob"] == pytest.approx(mean, rel=1e-6)
        cdf, kmin = s.poisson_cdf(r)
        assert cdf[-1] == 1.0 and np.all(np.diff(cdf) >= 0)
        k = kmin + np.arange(len(cdf))
        pmf = np.diff(np.concatenate([[0.0], cdf]))
        mu = float(np.sum(k * pmf))
        var = float(np.sum(k * k * pmf) - mu * mu)
        assert mu == pytest.approx(mean, rel=1e-9)
        assert var == pytest.approx(mean, rel=1e-6)
        sd = math.sqrt(mean / n)
        assert abs(ref_mu - mean) < 5 * sd  # the reference sampler agrees with the law
        u = g.random(n)
        samples = kmin + np.searchsorted(cdf, u, side="right")
        assert abs(samples.mean() - ref_mu) < 7 * sd
        assert samples.var() == pytest.approx(ref_var, rel=0.05)


def test_poisson_inversion_by_count_equals_binary_search():
    """The device inverts a zeroth-order CDF either by binary search for the
    smallest k with CDF(k) > u or, with few entries, by counting the values
    at or below u; the tables never decrease, so the two agree, here at
    means from 0.3 to 40,000 births per step."""
    g = np.random.Generator(np.random.Philox(8))
    for mean in (0.3, 7.5, 1.2e3, 4.0e4):
        s = _host((1.0, 1.0, 1.0), 1.0)
        s.add_species(1.0)
        r = s.add_reaction(0, [], [0], mean)
        s.finalize()
        cdf, kmin = s.poisson_cdf(r)
        assert np.all(np.diff(cdf) >= 0) and cdf[-1] == 1.0
        for u in g.random(200):
            lo, hi = 0, len(cdf) - 1
            while lo < hi:
                mid = (lo + hi) // 2
                if cdf[mid] > u:
                    hi = mid
                else:
                    lo = mid + 1
            assert min(int(np.count_nonzero(cdf <= u)), len(cdf) - 1) == lo


@pytest.mark.slow
def test_rate_tables_regenerate():
    """The committed header is what the generator produces (irreversible table)."""
    from gpusmoldyn_gb300 import rate_tables_gen as g

    up = g.sweep("i", 600, 1e-5, True)
    dn = g.sweep("i", 600, 1e-5, False)
    yi = g._mean6(up, dn)
    hdr = open(os.path.join(os.path.dirname(g.__file__), "csrc", "rate_tables.h")).read()
    body = hdr.split("kIrrev[31] = {")[1].split("};")[0]
    vals = [float(v) for v in body.replace("\n", " ").split(",") if v.strip()]
    assert np.allclose(vals, yi, atol=1e-7)
