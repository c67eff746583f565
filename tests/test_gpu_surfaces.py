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


@pytest.mark.parametrize("sort", SORTS)
def test_cell_scene_bit_exact(sort):
    # the bench's cell: a sphere membrane listed only in the grid boxes its
    # surface passes through and a nucleus of 1280 triangles; molecules
    # crowd both so that the walk meets every kind of box
    from gpusmoldyn_gb300 import configs
    side = 20.0
    s = System((0, 0, 0), (side, side, side), dt=2e-3, seed=41, normals="table", sort=sort)
    D = [0.5, 1.0, 4.0, 2.0]
    for d in D:
        s.add_species(d)
    s.add_reaction(2, [0, 1], [2], 0.5)
    r = s.add_reaction(1, [2], [0, 1], 5.0)
    s.set_product_placement(r, L.BD_PP_UNBINDRAD, 0.1)
    configs.c3_cell_surfaces(s, side)
    assert s.surface_counts() == (2, 1281)
    s.finalize()
    g = rng(41)
    n = 12000
    u = g.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    rad = np.where(np.arange(n) % 2 == 0, 0.4 * side, 0.12 * side) + g.normal(size=n) * 0.15
    pos = np.clip(side / 2 + u * rad[:, None], 0.01, side - 0.01).astype(np.float32)
    s.set_particles(pos, (np.arange(n) % 4).astype(np.int32))
    recs, _, ev = run_parity(s, 20)
    assert ev[0] > 10 and ev[1] > 10


@pytest.mark.parametrize("sort", SORTS)
def test_ensemble_with_surfaces_matches_oracle_alone(sort):
    """Instances of different sizes share the panels (in each instance's own
    coordinates): every instance evolves exactly as the oracle runs it alone."""
    from gpusmoldyn_gb300.configs import uniform_positions
    from oracle import py as orc
    counts = [1500, 4000, 2500]
    sides = [2.0, 3.0, 2.5]
    inst = [dict(box_lo=(0.0, 0.0, 0.0), box_hi=(sd, sd, sd), seed=300 + k, d_scale=[0.5, 1.0, 2.0][k],
                 k2_scale=[1.0, 2.0, 0.5][k]) for k, sd in enumerate(sides)]
    s = System(dt=2e-3, seed=1, normals="table", instances=inst, sort=sort)
    A, B, Cc = s.add_species(1.0), s.add_species(1.0), s.add_species(0.5)
    s.add_reaction(2, [A, B], [Cc], 3.0)
    u = s.add_reaction(1, [Cc], [A, B], 50.0)
    s.set_product_placement(u, L.BD_PP_UNBINDRAD, 0.02)
    f = s.add_surface()
    s.set_surface_action(f, L.BD_ALL_SPECIES, "both", "reflect")
    s.set_surface_action(f, A, "front", "absorb")
    s.add_panel(f, "sph", [1.0, 1.0, 1.0, 0.6])
    g2 = s.add_surface()
    s.set_surface_action(g2, B, "both", "reflect")
    s.add_panel(g2, "rect", [1.6, 0.0, 0.0, 3.0, 3.0], axis=0, front=-1)
    s.finalize()
    g = rng(22)
    pos, sp = [], []
    for d, n in zip(inst, counts):
        pos.append(uniform_positions(g, n, d["box_lo"], d["box_hi"]))
        sp.append((np.arange(n) % 3).astype(np.int32))
    s.set_ensemble_particles(np.concatenate(pos), np.concatenate(sp), counts)
    oracles = [orc.OracleSystem(s, instance=k) for k in range(len(counts))]
    recs = [orc.records(p, q, inst=k) for k, (p, q) in enumerate(zip(pos, sp))]
    for t in range(15):
        s.step(1)
        s.synchronize()
        got = gpu_records(s)
        for k, o in enumerate(oracles):
            recs[k] = o.step(t, recs[k])["recs"]
            live = recs[k][recs[k][:, 3] != 0xFFFFFFFF]
            mine = got[(got[:, 3] != 0xFFFFFFFF) & ((got[:, 3] >> 16) == k)]
            np.testing.assert_array_equal(mine, live, err_msg=f"instance {k} step {t}")
