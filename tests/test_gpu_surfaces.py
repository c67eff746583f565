"""Surfaces on the GPU, through the C ABI: bit-exact against the oracle on a
scene with every panel shape and action (both sort modes, products placed
across panels), transmitting panels are invisible, and the physics at sizes
the oracle cannot reach (absorption against erf, a reflecting sphere that
keeps a million molecules on their side)."""
from math import erf, sqrt

import numpy as np
import pytest

from gpusmoldyn_gb300 import _lib as L
from gpusmoldyn_gb300.configs import rng, uniform_positions
from gpusmoldyn_gb300.system import System
from surface_cases import mixed_scene
from test_gpu_parity import SORTS, gpu_records, run_parity

pytestmark = pytest.mark.gpu


def scene_system(sort, with_panels=True, transmit_only=False, seed=21):
    s = System((0, 0, 0), (6, 6, 6), dt=4e-3, seed=seed, normals="table", sort=sort)
    A, B, C, D = s.add_species(1.0), s.add_species(0.5), s.add_species(2.0), s.add_species(1.5)
    # reversible A + B <-> C: the unbinding places A and B apart across panels;
    # C + D -> A + B with an unbinding radius: pair products walk too
    fwd = s.add_reaction(2, [A, B], [C], 3.0)
    back = s.add_reaction(1, [C], [A, B], 20.0)
    s.set_product_placement(back, L.BD_PP_UNBINDRAD, 0.15)
    r = s.add_reaction(2, [C, D], [A, B], 2.0)
    s.set_product_placement(r, L.BD_PP_UNBINDRAD, 0.2)
    assert fwd == 0
    if with_panels:
        ids = mixed_scene(s, A, B, C, D)
        if transmit_only:
            for f in ids:
                s.set_surface_action(f, L.BD_ALL_SPECIES, "both", "transmit")
    s.finalize()
    g = rng(seed)
    pos = uniform_positions(g, 8000, (0, 0, 0), (6, 6, 6))
    s.set_particles(pos, (np.arange(8000) % 4).astype(np.int32))
    return s


@pytest.mark.parametrize("sort", SORTS)
def test_mixed_scene_bit_exact(sort):
    s = scene_system(sort)
    n0 = s.count()
    recs, _, ev = run_parity(s, 30)
    assert ev[1] > 20 and ev[2] > 5       # unbinding and pair products were placed
    assert s.count() < n0 - 50            # absorptions happened


def test_transmitting_panels_are_invisible():
    a = scene_system("binned", with_panels=False)
    b = scene_system("binned", with_panels=True, transmit_only=True)
    a.step(20)
    b.step(20)
    a.synchronize()
    b.synchronize()
    np.testing.assert_array_equal(gpu_records(a), gpu_records(b))


def test_absorbing_plane_survival_large():
    n, steps, dt = 1_000_000, 2000, 1e-4
    s = System((0, 0, 0), (10, 10, 10), dt=dt, seed=31, normals="boxmuller")
    s.add_species(1.0)
    f = s.add_surface()
    s.set_surface_action(f, L.BD_ALL_SPECIES, "both", "absorb")
    s.add_panel(f, "rect", [1.0, 0, 0, 10, 10], axis=0)
    s.finalize()
    g = rng(31)
    pos = np.column_stack([np.full(n, 2.0), g.random(n) * 10, g.random(n) * 10]).astype(np.float32)
    s.set_particles(pos, np.zeros(n, np.int32))
    s.step(steps)
    s.synchronize()
    t, sigma = steps * dt, sqrt(2 * dt)
    expect = erf((1.0 + 0.5826 * sigma) / sqrt(4 * t))
    got = s.count() / n
    assert got == pytest.approx(expect, abs=0.003)
    xyz, _ = s.particles()
    assert (xyz[:, 0] > 1.0).all()


def outside_sphere(xyz, c, r2):
    """The panel's side test in float32: (wx^2 + wy^2) + wz^2 - r^2 > 0."""
    w = np.asarray(xyz, np.float32) - np.float32(c)
    q = (w[:, 0] * w[:, 0] + w[:, 1] * w[:, 1]) + w[:, 2] * w[:, 2]
    return (q - np.float32(r2)) > 0


def test_reflecting_sphere_holds_a_million():
    n = 1_000_000
    s = System((0, 0, 0), (10, 10, 10), dt=1e-3, seed=32, normals="boxmuller")
    s.add_species(1.0)
    f = s.add_surface()
    s.set_surface_action(f, L.BD_ALL_SPECIES, "both", "reflect")
    s.add_panel(f, "sph", [5, 5, 5, 3])
    s.finalize()
    g = rng(32)
    pos = uniform_positions(g, n, (0, 0, 0), (10, 10, 10))
    inside = int((~outside_sphere(pos, 5, 9)).sum())
    s.set_particles(pos, np.zeros(n, np.int32))
    s.step(1500)
    s.synchronize()
    xyz, _ = s.particles()
    inn = ~outside_sphere(xyz, 5, 9)
    assert len(xyz) == n and int(inn.sum()) == inside
    d2 = ((xyz[inn].astype(np.float64) - 5) ** 2).sum(1)
    assert d2.mean() == pytest.approx(0.6 * 9, rel=0.01)
