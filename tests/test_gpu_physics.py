"""Statistical checks of the production path (Philox Box-Muller normals)
against theory, each within 1% as the step is specified:

* mean-squared displacement 6 D t (in-place and sorted pipelines);
* the bimolecular rate equals the Andrews-Bray rate numrxnrate(step, a, b)/dt
  that the binding radius was solved for (with the Smoluchowski transient of
  a system that starts well mixed);
* the reversible A + B <-> C equilibrium equals mass action k_on / k_off;
* first-order decay and branching, zeroth-order Poisson production.

Tolerances are written in each test; sample sizes make the statistical
error a fraction of them.
"""
import math

import numpy as np
import pytest

from gpusmoldyn_gb300 import _lib as L
from gpusmoldyn_gb300.configs import rng, uniform_positions
from gpusmoldyn_gb300.system import System, numrxnrate

pytestmark = pytest.mark.gpu


def test_msd_in_place_path():
    n, steps, dt = 1_000_000, 50, 1e-3
    s = System((-1e3,) * 3, (1e3,) * 3, dt=dt, seed=21)
    s.add_species(1.0)
    s.add_species(0.25)
    s.finalize()
    sp = (np.arange(n) % 2).astype(np.int32)
    s.set_particles(np.zeros((n, 3), np.float32), sp)
    s.step(steps)
    s.synchronize()
    xyz, w = s.slots()  # in-place path keeps slot order
    r2 = np.sum(xyz.astype(np.float64) ** 2, axis=1)
    for species, D in ((0, 1.0), (1, 0.25)):
        msd = r2[(w & 0xFFFF) == species].mean()
        theory = 6 * D * dt * steps
        # relative standard error sqrt(2/3 / 5e5) = 0.12%; tolerance 1%
        assert msd / theory == pytest.approx(1.0, abs=0.01), (species, msd / theory)


def test_msd_sorted_path_and_table_mode():
    """All particles start at the centre, so |x|^2 needs no identity."""
    n, steps, dt = 600_000, 40, 1e-3
    for normals, var in (("boxmuller", 1.0), ("table", 0.99968)):
        s = System((-1e2,) * 3, (1e2,) * 3, dt=dt, seed=22, normals=normals)
        s.add_species(2.0)
        s.add_species(0.5)
        s.add_reaction(2, [0, 1], [0], 1e-9)  # forces the sorted pipeline, never fires
        s.finalize()
        s.set_particles(np.zeros((n, 3), np.float32), (np.arange(n) % 2).astype(np.int32))
        s.step(steps)
        s.synchronize()
        pos, sp = s.particles()
        r2 = np.sum(pos.astype(np.float64) ** 2, axis=1)
        for species, D in ((0, 2.0), (1, 0.5)):
            ratio = r2[sp == species].mean() / (6 * D * dt * steps * var)
            assert ratio == pytest.approx(1.0, abs=0.01), (normals, species, ratio)


def test_reflection_keeps_uniform_density():
    n, side = 400_000, 5.0
    s = System((0, 0, 0), (side,) * 3, dt=1e-3, seed=23)
    s.add_species(30.0)
    s.add_species(30.0)
    s.add_reaction(2, [0, 1], [0], 1e-9)
    s.finalize()
    g = rng(23)
    s.set_particles(uniform_positions(g, n, (0, 0, 0), (side,) * 3), (np.arange(n) % 2).astype(np.int32))
    s.step(200)
    s.synchronize()
    pos, _ = s.particles()
    assert np.all(pos >= 0) and np.all(pos <= side)
    h, _ = np.histogram(pos[:, 0], bins=50, range=(0, side))
    exp = n / 50
    chi2 = float(np.sum((h - exp) ** 2 / exp))
    assert chi2 < 100  # 49 degrees of freedom


def test_bimolecular_rate_matches_rxnparam():
    """B + A -> B with immobile B catalysts (D_B = 0, so the product stays
    exactly where B was and the B's stay uniform) and D_A = 2, the c2
    mutual diffusion: -d ln N_A / dt = k_eff rho_B with
    k_eff = numrxnrate(step, a, -1)/dt x (1 + 2R/sqrt(pi D T)), the time
    average of the Smoluchowski transient over the run (R = k / 4 pi D)."""
    side, rho, dt, k, steps = 50.0, 10.0, 5e-4, 0.05, 2000
    n = int(rho * side ** 3)
    s = System((0, 0, 0), (side,) * 3, dt=dt, seed=24)
    A, B = s.add_species(2.0), s.add_species(0.0)
    r = s.add_reaction(2, [B, A], [B], k)
    s.finalize()
    a = s.reaction_info(r)["bind_radius"]
    g = rng(24)
    s.set_particles(uniform_positions(g, 2 * n, (0, 0, 0), (side,) * 3),
                    np.concatenate([np.zeros(n), np.ones(n)]).astype(np.int32))
    s.step(steps)
    s.synchronize()
    na, nb = s.species_counts()
    assert nb == n
    events = int(s.event_counts()[0])
    assert events == n - na and events > 300_000
    T = steps * dt
    Dsum = 2.0
    kstep = numrxnrate(math.sqrt(2 * Dsum * dt), a, -1)
    R = k / (4 * math.pi * Dsum)
    k_theory = kstep / dt * (1 + 2 * R / math.sqrt(math.pi * Dsum * T))
    k_meas = -math.log(na / n) / (T * n / side ** 3)
    # statistical error ~0.15%; tolerance 1%
    assert k_meas / k_theory == pytest.approx(1.0, abs=0.01), (k_meas, k_theory)


def test_reversible_equilibrium_mass_action():
    """A + B <-> C at the c2 density, k_on 0.05, k_off 10, dt 0.5 ms: the
    time-averaged C count equals the mass-action solution of
    c = (k_on / k_off) (A0 - c)(B0 - c) / V within 1%."""
    n0, dens, dt = 200_000, 1_000_000 / 60.0 ** 3, 5e-4
    side = float((2 * n0 / dens) ** (1 / 3))
    V = side ** 3
    s = System((0, 0, 0), (side,) * 3, dt=dt, seed=25)
    A, B, Cc = s.add_species(1.0), s.add_species(1.0), s.add_species(0.5)
    s.add_reaction(2, [A, B], [Cc], 0.05)
    back = s.add_reaction(1, [Cc], [A, B], 10.0)
    s.set_product_placement(back, L.BD_PP_PGEMMAX, 0.2)
    s.finalize()
    g = rng(25)
    s.set_particles(uniform_positions(g, 2 * n0, (0, 0, 0), (side,) * 3),
                    np.concatenate([np.zeros(n0), np.ones(n0)]).astype(np.int32))
    s.step(3000)  # ~15 relaxation times
    samples = []
    for _ in range(400):
        s.step(20)
        samples.append(int(s.species_counts()[Cc]))
    c_mean = float(np.mean(samples))
    K = 0.05 / 10.0
    # K (n0 - c)^2 / V = c  ->  quadratic in c
    qa, qb, qc = K / V, -(2 * K * n0 / V + 1), K * n0 * n0 / V
    c_theory = (-qb - math.sqrt(qb * qb - 4 * qa * qc)) / (2 * qa)
    assert c_mean / c_theory == pytest.approx(1.0, abs=0.01), (c_mean, c_theory)


def test_first_order_decay_and_branching():
    n, dt, steps = 2_000_000, 1e-3, 100
    s = System((0, 0, 0), (100.0,) * 3, dt=dt, seed=26)
    A, B, Cc = s.add_species(1.0), s.add_species(1.0), s.add_species(1.0)
    r1 = s.add_reaction(1, [A], [B], 3.0)
    r2 = s.add_reaction(1, [A], [Cc], 1.0)
    s.finalize()
    g = rng(26)
    s.set_particles(uniform_positions(g, n, (0, 0, 0), (100.0,) * 3), np.zeros(n, np.int32))
    s.step(steps)
    s.synchronize()
    na, nb, nc = (int(v) for v in s.species_counts())
    assert na + nb + nc == n
    frac = na / n
    theory = math.exp(-4.0 * dt * steps)
    assert frac / theory == pytest.approx(1.0, abs=0.005)
    assert nb / (nb + nc) == pytest.approx(0.75, abs=0.005)
    ev = s.event_counts()
    assert ev[r1] == nb and ev[r2] == nc


def test_zeroth_order_production_is_poisson():
    dt, k, side = 1e-3, 2000.0, 5.0
    s = System((0, 0, 0), (side,) * 3, dt=dt, seed=27)
    s.add_species(1.0)
    s.add_reaction(0, [], [0], k)
    s.finalize()
    s.set_particles(np.full((1, 3), 1.0, np.float32), np.zeros(1, np.int32))
    lam = k * dt * side ** 3
    counts, prev = [], s.count()
    for _ in range(300):
        s.step(1)
        c = s.count()
        counts.append(c - prev)
        prev = c
    counts = np.array(counts, np.float64)
    assert counts.mean() == pytest.approx(lam, rel=0.02)
    assert counts.var() == pytest.approx(lam, rel=0.2)
    pos, _ = s.particles()
    assert np.all(pos >= 0) and np.all(pos <= side)


def test_competing_reactions_split_the_rate():
    """B + A -> B (k0) and B + A -> B + C (k1) compete for the same pairs
    (immobile catalysts B): A decays at the rate of the summed k0 + k1, as
    numrxnrate predicts for the shared binding radius, and the reactions
    fire in the ratio k0 : k1 (binomial error ~0.3%; tolerance 2%)."""
    side, rho, dt, k0, k1, steps = 50.0, 10.0, 5e-4, 0.0125, 0.0375, 2000
    n = int(rho * side ** 3)
    s = System((0, 0, 0), (side,) * 3, dt=dt, seed=30, pairs="channels")
    A, B, Cc = s.add_species(2.0), s.add_species(0.0), s.add_species(2.0)
    s.add_reaction(2, [B, A], [B], k0)
    s.add_reaction(2, [B, A], [B, Cc], k1)
    s.finalize()
    a = s.reaction_info(0)["bind_radius"]
    g = rng(30)
    s.set_particles(uniform_positions(g, 2 * n, (0, 0, 0), (side,) * 3),
                    np.concatenate([np.zeros(n), np.ones(n)]).astype(np.int32))
    s.step(steps)
    s.synchronize()
    na, nb, nc = s.species_counts()
    e0, e1 = (int(v) for v in s.event_counts()[:2])
    assert nb == n and e0 + e1 == n - na and nc == e1 and e0 + e1 > 300_000
    assert e1 / (e0 + e1) == pytest.approx(k1 / (k0 + k1), rel=0.02)
    T, Dsum, k = steps * dt, 2.0, k0 + k1
    kstep = numrxnrate(math.sqrt(2 * Dsum * dt), a, -1)
    k_theory = kstep / dt * (1 + 2 * (k / (4 * math.pi * Dsum)) / math.sqrt(math.pi * Dsum * T))
    k_meas = -math.log(na / n) / (T * n / side ** 3)
    assert k_meas / k_theory == pytest.approx(1.0, abs=0.01), (k_meas, k_theory)


def test_ensemble_msd_per_instance_with_scaled_d():
    """A batched ensemble (one pipeline per step over every instance): each
    instance diffuses with its own D scale, and its MSD is 6 D d_scale t
    within 1%.  All particles of an instance start at its box centre, so
    |x - centre|^2 needs no identity."""
    n, steps, dt = 300_000, 40, 1e-3
    scales = [0.5, 1.0, 2.0, 3.0]
    inst = [dict(box_lo=(0.0, 0.0, 0.0), box_hi=(200.0, 200.0, 200.0), seed=300 + k, d_scale=d, k2_scale=1.0)
            for k, d in enumerate(scales)]
    s = System(dt=dt, seed=30, instances=inst)
    s.add_species(1.0)
    s.add_species(0.4)
    s.add_reaction(2, [0, 1], [0], 1e-9)  # a second-order reaction that never fires
    s.finalize()
    pos = np.full((n * len(scales), 3), 100.0, np.float32)
    sp = (np.arange(n * len(scales)) % 2).astype(np.int32)
    s.set_ensemble_particles(pos, sp, [n] * len(scales))
    s.step(steps)
    s.synchronize()
    for k, d in enumerate(scales):
        p, q = s.particles(k)
        r2 = np.sum((p.astype(np.float64) - 100.0) ** 2, axis=1)
        for species, D in ((0, 1.0), (1, 0.4)):
            ratio = r2[q == species].mean() / (6 * D * d * dt * steps)
            # relative standard error sqrt(2/3 / 1.5e5) = 0.2%; tolerance 1%
            assert ratio == pytest.approx(1.0, abs=0.01), (k, species, ratio)
    s.close()


def test_ensemble_equilibrium_per_instance_with_scaled_kon():
    """Three instances of A + B <-> C at the c2 density (k_off 10 /s, pgemmax
    0.2) with k_on scaled 0.5, 1 and 2 from 0.05 um^3/s, in one pipeline:
    each instance's time-averaged C count equals its own mass-action
    solution c = (k_on k2_scale / k_off) (A0 - c)(B0 - c) / V within 1%."""
    n0, dens, dt = 150_000, 1_000_000 / 60.0 ** 3, 5e-4
    side = float((2 * n0 / dens) ** (1 / 3))
    V = side ** 3
    scales = [0.5, 1.0, 2.0]
    inst = [dict(box_lo=(0.0, 0.0, 0.0), box_hi=(side,) * 3, seed=310 + k, d_scale=1.0, k2_scale=ks)
            for k, ks in enumerate(scales)]
    s = System(dt=dt, seed=31, instances=inst)
    A, B, Cc = s.add_species(1.0), s.add_species(1.0), s.add_species(0.5)
    s.add_reaction(2, [A, B], [Cc], 0.05)
    back = s.add_reaction(1, [Cc], [A, B], 10.0)
    s.set_product_placement(back, L.BD_PP_PGEMMAX, 0.2)
    s.finalize()
    g = rng(31)
    pos = np.concatenate([uniform_positions(g, 2 * n0, (0, 0, 0), (side,) * 3) for _ in scales])
    sp = np.tile(np.concatenate([np.zeros(n0), np.ones(n0)]).astype(np.int32), len(scales))
    s.set_ensemble_particles(pos, sp, [2 * n0] * len(scales))
    s.step(3000)  # ~15 relaxation times
    samples = [[] for _ in scales]
    for _ in range(400):
        s.step(20)
        for k in range(len(scales)):
            samples[k].append(int(s.species_counts(k)[Cc]))
    for k, ks in enumerate(scales):
        c_mean = float(np.mean(samples[k]))
        K = 0.05 * ks / 10.0
        qa, qb, qc = K / V, -(2 * K * n0 / V + 1), K * n0 * n0 / V
        c_theory = (-qb - math.sqrt(qb * qb - 4 * qa * qc)) / (2 * qa)
        assert c_mean / c_theory == pytest.approx(1.0, abs=0.01), (k, ks, c_mean, c_theory)
    s.close()


@pytest.mark.parametrize("normals,var", [("boxmuller", 1.0), ("table", 0.99968)])
def test_msd_observable_equals_6_d_dt(normals, var):
    """bd_measure_msd: the mean squared diffusion move per step of each
    species is 6 D dt (times the table's variance in table mode) within 1%,
    in a box so large that walls reflect almost nothing; every live
    particle's move is counted once per step; the steps are taken."""
    n, steps, dt = 400_000, 10, 1e-3
    s = System((0, 0, 0), (500.0,) * 3, dt=dt, seed=41, normals=normals)
    s.add_species(1.5)
    s.add_species(0.2)
    s.add_reaction(2, [0, 1], [0], 1e-9)
    s.finalize()
    g = rng(41)
    s.set_particles(uniform_positions(g, n, (100.0,) * 3, (400.0,) * 3), (np.arange(n) % 2).astype(np.int32))
    step0 = s.step_count()
    msd, cnt = s.measure_msd(steps)
    assert s.step_count() == step0 + steps
    np.testing.assert_array_equal(cnt, [steps * n // 2, steps * n // 2])
    for species, D in ((0, 1.5), (1, 0.2)):
        assert msd[species] / (6 * D * dt * var) == pytest.approx(1.0, abs=0.01), (species, msd[species])
    s.close()


def test_msd_observable_per_instance():
    scales = [0.5, 2.0]
    inst = [dict(box_lo=(0.0,) * 3, box_hi=(300.0,) * 3, seed=420 + k, d_scale=d, k2_scale=1.0)
            for k, d in enumerate(scales)]
    s = System(dt=1e-3, seed=42, instances=inst)
    s.add_species(1.0)
    s.add_reaction(2, [0, 0], [0], 1e-9)
    s.finalize()
    n = 200_000
    g = rng(42)
    pos = np.concatenate([uniform_positions(g, n, (50.0,) * 3, (250.0,) * 3) for _ in scales])
    s.set_ensemble_particles(pos, np.zeros(2 * n, np.int32), [n, n])
    for k, d in enumerate(scales):
        msd, cnt = s.measure_msd(8, instance=k)
        assert int(cnt[0]) == 8 * n
        assert msd[0] / (6 * d * 1e-3) == pytest.approx(1.0, abs=0.01), (k, msd[0])
    s.close()
