"""The CPU oracle itself: Philox known answers, its arithmetic against an
independent Python restatement, and its physics against theory.

The reference ships no golden outputs for the step (its -qatest files are
not in the repository), so the oracle's step is pinned by theory: the
mean-squared displacement of free diffusion, reflection, Poisson births and
the reference's own Andrews-Bray reaction rate."""
import math

import numpy as np
import pytest

from gpusmoldyn_gb300 import _lib as L
from gpusmoldyn_gb300.configs import rng, uniform_positions
from gpusmoldyn_gb300.system import System, gauss_table, numrxnrate
from oracle import py as orc


def test_philox_known_answers():
    # Random123 known-answer vectors for philox4x32-10
    assert list(orc.philox([0, 0, 0, 0], 0, 0)) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert list(orc.philox([0xFFFFFFFF] * 4, 0xFFFFFFFF, 0xFFFFFFFF)) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6,
                                                                          0x6D5451FD]
    assert list(orc.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], 0xA4093822, 0x299F31D0)) == [
        0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def host_system(box=((0, 0, 0), (10, 10, 10)), dt=1e-3, D=(1.0,), normals="table", seed=3):
    s = System(box[0], box[1], dt=dt, seed=seed, normals=normals, device=-1)
    for d in D:
        s.add_species(d)
    return s


def test_diffusion_step_matches_python_restatement():
    """x' = fma(sqrt(2 D dt), table[word >> 20], x) per axis, keyed by slot."""
    s = host_system(D=(0.7,), dt=2e-3, seed=0x1234567890)
    s.finalize()
    g = rng(1)
    pos = uniform_positions(g, 64, (2, 2, 2), (8, 8, 8))
    s.set_particles(pos, np.zeros(64, np.int32))
    o = orc.OracleSystem(s)
    out = o.step(9, orc.records(pos, np.zeros(64)))["recs"]
    table = gauss_table()
    sigma = np.float32(math.sqrt(2.0 * np.float32(0.7) * np.float32(2e-3)))
    sigma = np.sqrt(np.float32(2.0) * np.float32(0.7) * np.float32(2e-3), dtype=np.float32)
    for i in range(64):
        w = orc.philox([i, 9, 1 << 24, 0], 0x34567890, 0x12)
        for a in range(3):
            g_ = table[w[a] >> 20]
            exp = np.float32(np.float64(sigma) * np.float64(g_) + np.float64(pos[i, a]))  # fma in double, rounded once
            assert out[i, a] == np.float32(exp).view(np.uint32), (i, a)


def test_reflection_keeps_particles_in_box():
    s = host_system(D=(50.0,), dt=1e-3)
    s.finalize()
    g = rng(2)
    pos = uniform_positions(g, 5000, (0, 0, 0), (10, 10, 10))
    pos[:2500, 0] = 9.999
    s.set_particles(pos, np.zeros(5000, np.int32))
    o = orc.OracleSystem(s)
    recs = orc.records(pos, np.zeros(5000))
    for t in range(20):
        recs = o.step(t, recs)["recs"]
    xyz = recs[:, :3].view(np.float32)
    assert np.all(xyz >= 0) and np.all(xyz <= 10)


@pytest.mark.parametrize("normals", ["table", "boxmuller"])
def test_oracle_msd(normals):
    n, steps, D, dt = 40000, 20, 1.0, 1e-3
    s = host_system(box=((-1e3, -1e3, -1e3), (1e3, 1e3, 1e3)), D=(D,), dt=dt, normals=normals)
    s.finalize()
    pos = np.zeros((n, 3), np.float32)
    s.set_particles(pos, np.zeros(n, np.int32))
    o = orc.OracleSystem(s)
    recs = orc.records(pos, np.zeros(n))
    for t in range(steps):
        recs = o.step(t, recs)["recs"]
    xyz = recs[:, :3].view(np.float32).astype(np.float64)
    msd = np.mean(np.sum(xyz ** 2, axis=1))
    var = 0.99968 if normals == "table" else 1.0
    theory = 6 * D * dt * steps * var
    # relative standard error sqrt(2/3/n) = 0.4%
    assert msd / theory == pytest.approx(1.0, abs=0.02)


def test_oracle_irreversible_rate_matches_rxnparam():
    """A + B -> B (B catalytic, so its density stays fixed) at low B density:
    the events per step equal numrxnrate(step, a, -1) nA nB / V, the
    Andrews-Bray rate the binding radius was solved for, times the
    Smoluchowski transient 1 + R/sqrt(pi D t) (R = k / 4 pi D) of a system
    that starts well mixed, within 3.5 sigma and 1%."""
    side, nA, nB, dt, k, D = 10.0, 30000, 2000, 1e-3, 2.0, 10.0
    s = host_system(box=((0, 0, 0), (side, side, side)), D=(D, D), dt=dt, normals="boxmuller")
    r = s.add_reaction(2, [0, 1], [1], k)
    s.finalize()
    a = s.reaction_info(r)["bind_radius"]
    g = rng(4)
    pos = uniform_positions(g, nA + nB, (0, 0, 0), (side, side, side))
    sp = np.concatenate([np.zeros(nA), np.ones(nB)]).astype(np.int32)
    s.set_particles(pos, sp)
    o = orc.OracleSystem(s)
    recs = orc.records(pos, sp)
    kstep = numrxnrate(math.sqrt(2 * 2 * D * dt), a, -1)
    assert kstep == pytest.approx(k * dt, rel=1e-3)
    R = k / (4 * math.pi * 2 * D)
    expect = observed = 0.0
    for t in range(60):
        live = recs[:, 3] != 0xFFFFFFFF
        na = int(np.sum(live & ((recs[:, 3] & 0xFFFF) == 0)))
        res = o.step(t, recs)
        recs = res["recs"]
        if t >= 3:  # after the first steps' relaxation from uniform
            observed += float(res["events"][0])
            transient = 1 + R / math.sqrt(math.pi * 2 * D * (t + 0.5) * dt)
            expect += kstep * transient * na * nB / side ** 3
    assert abs(observed - expect) < 3.5 * math.sqrt(expect) + 0.01 * expect, (observed, expect)


def test_oracle_zeroth_order_births_are_poisson():
    s = host_system(box=((0, 0, 0), (2, 3, 4)), D=(0.5,), dt=1e-2)
    r = s.add_reaction(0, [], [0], 25.0)
    s.finalize()
    s.set_particles(np.zeros((0, 3), np.float32), np.zeros(0, np.int32))
    o = orc.OracleSystem(s)
    lam = 25.0 * 1e-2 * 24.0
    counts = []
    recs = np.zeros((0, 4), np.uint32)
    for t in range(400):
        n0 = recs.shape[0]
        recs = o.step(t, recs)["recs"]
        counts.append(recs.shape[0] - n0)
    counts = np.array(counts, np.float64)
    assert counts.mean() == pytest.approx(lam, rel=4 * math.sqrt(lam / 400) / lam)
    assert counts.var() == pytest.approx(lam, rel=0.25)
    xyz = recs[:, :3].view(np.float32)
    assert np.all(xyz >= 0) and np.all(xyz[:, 0] <= 2) and np.all(xyz[:, 2] <= 4)
