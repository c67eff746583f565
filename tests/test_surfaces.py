"""Surfaces on the CPU: the C ABI's checks and derived panel geometry
(host-only handles), and the surface walk's physics on the oracle, which
states the same walk independently of the kernels (the GPU is checked
against it bit for bit in test_gpu_surfaces.py)."""
from math import erf, sqrt

import numpy as np
import pytest

from gpusmoldyn_gb300 import _lib as L
from gpusmoldyn_gb300.system import System
from oracle import py as orc
from surface_cases import capped_cylinder, mixed_scene, tri_box


def host(box=10.0, dt=1e-3, n_species=1, D=1.0):
    s = System((0, 0, 0), (box, box, box), dt=dt, seed=5, normals="table", device=L.BD_DEVICE_NONE)
    for _ in range(n_species):
        s.add_species(D)
    return s


def oracle_run(s, pos, steps, species=None):
    s.finalize(allow=(L.BD_OK, L.BD_ERR_ALREADY_FINALIZED))
    pos = np.asarray(pos, np.float32)
    species = np.zeros(len(pos), np.int32) if species is None else np.asarray(species, np.int32)
    s.set_particles(pos, species)
    o = orc.OracleSystem(s)
    recs = orc.records(pos, species)
    for t in range(steps):
        recs = o.step(t, recs)["recs"]
    return recs[:, :3].copy().view(np.float32), recs[:, 3]


def test_panel_checks():
    s = host()
    f = s.add_surface()
    bad = [("rect", [0, 0, 0, 1, 1], dict(axis=3)), ("rect", [0, 0, 0, 0, 1], {}),
           ("rect", [0, 0, 0, 1, 1], dict(front=0)), ("tri", [0, 0, 0, 1, 1, 1, 2, 2, 2], {}),
           ("sph", [1, 1, 1, 0], {}), ("sph", [1, 1, 1, 1], dict(front=2)),
           ("cyl", [1, 1, 1, 1, 1, 1, 0.5], {}), ("disk", [1, 1, 1, 1, 0, 0, 0], {}),
           ("hemi", [1, 1, 1, -1, 0, 0, 1], {}), ("sph", [1, 1, float("nan"), 1], {}), (9, [0] * 10, {})]
    for shape, p, kw in bad:
        with pytest.raises(L.BDError) as e:
            s.add_panel(f, shape, p, **kw)
        assert e.value.code == L.BD_ERR_INVALID_ARGUMENT, (shape, p, kw)
    with pytest.raises(L.BDError):
        s.add_panel(f + 1, "sph", [1, 1, 1, 1])           # no such surface
    with pytest.raises(L.BDError):
        s.set_surface_action(f, 3, "both", "reflect")     # no such species
    with pytest.raises(L.BDError):
        s.set_surface_action(f, 0, 7, "reflect")          # no such face
    with pytest.raises(L.BDError):
        s.set_surface_action(f, 0, "both", 9)             # no such action
    s.add_panel(f, "sph", [5, 5, 5, 1])
    s.finalize()
    with pytest.raises(L.BDError) as e:
        s.add_panel(f, "sph", [5, 5, 5, 2])
    assert e.value.code == L.BD_ERR_ALREADY_FINALIZED
    with pytest.raises(L.BDError) as e:
        s.add_surface()
    assert e.value.code == L.BD_ERR_ALREADY_FINALIZED
    assert s.surface_counts() == (1, 1)


def test_derived_geometry():
    s = host()
    f = s.add_surface()
    r = s.panel_info(s.add_panel(f, "rect", [1, 2, 3, 4, -1.5], axis=1, front=-1))
    assert (r["axis"], r["front"]) == (1, -1.0) and r["bounds"] == [1, 5, 1.5, 3]
    t = s.panel_info(s.add_panel(f, "tri", [0, 0, 0, 2, 0, 0, 0, 3, 0]))
    np.testing.assert_allclose(t["n"], [0, 0, 1], atol=1e-7)
    assert t["v1"] == [2, 0, 0] and t["v2"] == [0, 3, 0]
    c = s.panel_info(s.add_panel(f, "cyl", [1, 1, 1, 4, 5, 1, 0.5], front=-1))
    np.testing.assert_allclose(c["n"], [0.6, 0.8, 0], rtol=1e-6)
    assert c["len"] == pytest.approx(5.0) and c["r2"] == pytest.approx(0.25) and c["front"] == -1.0
    d = s.panel_info(s.add_panel(f, "disk", [1, 1, 1, 2, 0, 0, -3]))
    np.testing.assert_allclose(d["n"], [0, 0, -1])
    h = s.panel_info(s.add_panel(f, "hemi", [1, 1, 1, 2, 1, 1, 0]))
    np.testing.assert_allclose(h["n"], [2 ** -0.5, 2 ** -0.5, 0], rtol=1e-6)
    assert [p["surface"] for p in (r, t, c, d, h)] == [f] * 5


def test_actions_apply_in_order():
    s = host(n_species=3)
    f = s.add_surface()
    assert all(s.surface_action(f, sp, face) == L.BD_SURF_TRANSMIT for sp in range(3) for face in (0, 1))
    s.set_surface_action(f, L.BD_ALL_SPECIES, "both", "reflect")
    s.set_surface_action(f, 1, "front", "absorb")
    assert [s.surface_action(f, 1, face) for face in (0, 1)] == [L.BD_SURF_ABSORB, L.BD_SURF_REFLECT]
    assert s.surface_action(f, 2, "front") == L.BD_SURF_REFLECT
    # a later statement for all species overrides the earlier one for species 1
    s.set_surface_action(f, L.BD_ALL_SPECIES, "front", "transmit")
    assert s.surface_action(f, 1, "front") == L.BD_SURF_TRANSMIT
    assert s.surface_action(f, 1, "back") == L.BD_SURF_REFLECT


def test_reflecting_sphere_keeps_both_sides():
    # molecules inside stay inside and molecules outside stay outside; the
    # inside ones spread to the uniform density (mean r^2 = 3/5 R^2)
    s = host()
    f = s.add_surface()
    s.set_surface_action(f, L.BD_ALL_SPECIES, "both", "reflect")
    s.add_panel(f, "sph", [5, 5, 5, 3])
    g = np.random.default_rng(1)
    pos = g.random((12000, 3)) * 10
    inside = np.linalg.norm(pos - 5, axis=1) < 3
    xyz, _ = oracle_run(s, pos, 600)
    # records come back in cell order: match them up by side counts
    d = np.linalg.norm(xyz - 5, axis=1)
    assert len(xyz) == len(pos)
    assert (d < 3).sum() == inside.sum() and (d <= 3).sum() == inside.sum()
    assert (d[d < 3] ** 2).mean() == pytest.approx(0.6 * 9, rel=0.03)


def test_absorbing_plane_survival():
    # 1D first passage to an absorbing plane at distance 0.5: survival
    # erf(x0 / sqrt(4 D t)); stepping at discrete times shifts the effective
    # plane by 0.5826 sigma away (sigma = sqrt(2 D dt))
    s = host(dt=1e-4)
    f = s.add_surface()
    s.set_surface_action(f, L.BD_ALL_SPECIES, "both", "absorb")
    s.add_panel(f, "rect", [1.0, 0, 0, 10, 10], axis=0)
    n, steps = 40000, 1000
    g = np.random.default_rng(2)
    pos = np.column_stack([np.full(n, 1.5), g.random(n) * 10, g.random(n) * 10])
    xyz, _ = oracle_run(s, pos, steps)
    t, sigma = steps * 1e-4, sqrt(2e-4)
    expect = erf((0.5 + 0.5826 * sigma) / sqrt(4 * t))
    assert len(xyz) / n == pytest.approx(expect, abs=0.01)
    assert (xyz[:, 0] > 1.0).all()


def test_closed_triangle_box_and_capped_cylinder_contain():
    s = host()
    f = s.add_surface()
    s.set_surface_action(f, L.BD_ALL_SPECIES, "both", "reflect")
    tri_box(s, f, (3, 3, 3), (7, 7, 7))
    g = np.random.default_rng(3)
    pos = 3.02 + g.random((6000, 3)) * 3.96
    xyz, _ = oracle_run(s, pos, 400)
    assert len(xyz) == 6000 and xyz.min() >= 3.0 and xyz.max() <= 7.0

    s = host()
    f = s.add_surface()
    s.set_surface_action(f, L.BD_ALL_SPECIES, "both", "reflect")
    capped_cylinder(s, f, 5, 5, 2, 8, 2)
    ang, rad = g.random(6000) * 2 * np.pi, 1.95 * np.sqrt(g.random(6000))
    pos = np.column_stack([5 + rad * np.cos(ang), 5 + rad * np.sin(ang), 2.05 + g.random(6000) * 5.9])
    xyz, _ = oracle_run(s, pos, 400)
    assert len(xyz) == 6000
    assert np.hypot(xyz[:, 0] - 5, xyz[:, 1] - 5).max() <= 2.0
    assert xyz[:, 2].min() >= 2.0 and xyz[:, 2].max() <= 8.0


def test_one_way_membrane_and_transmitting_surface():
    # front reflects, back transmits: molecules only cross toward +x
    s = host(n_species=2)
    f = s.add_surface()
    s.set_surface_action(f, 0, "front", "reflect")
    s.set_surface_action(f, 1, "both", "transmit")
    s.add_panel(f, "rect", [5, 0, 0, 10, 10], axis=0)
    g = np.random.default_rng(4)
    pos = g.random((8000, 3)) * 10
    sp = (np.arange(8000) % 2).astype(np.int32)
    xyz, w = oracle_run(s, pos, 800, sp)
    a = (w & 0x7FFF) == 0
    right0 = (pos[sp == 0, 0] > 5).sum()
    assert (xyz[a, 0] > 5).sum() > right0 + 200          # species 0 piles up in front
    assert abs((xyz[~a, 0] > 5).mean() - 0.5) < 0.03     # species 1 does not see the panel


def test_mixed_scene_runs_on_the_oracle():
    s = host(box=6.0, n_species=0)
    A, B, C, D = (s.add_species(d) for d in (1.0, 0.5, 2.0, 1.5))
    mixed_scene(s, A, B, C, D)
    s.finalize()
    g = np.random.default_rng(6)
    pos = g.random((4000, 3)) * 6
    xyz, w = oracle_run(s, pos, 50, np.arange(4000) % 4)
    assert 0 < 4000 - len(xyz) < 600  # A and B are absorbed, C and D never
    assert np.bincount(w & 0x7FFF, minlength=4)[2:].tolist() == [1000, 1000]
