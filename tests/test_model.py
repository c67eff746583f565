"""The model reader (bd_create_from_model): a Smoldyn-style text gives the
same network, derived parameters and grid as the same model built through
the C ABI, and malformed models fail with the line named.  Host-only
handles: no GPU needed."""
import numpy as np
import pytest

from gpusmoldyn_gb300 import _lib as L
from gpusmoldyn_gb300.system import System

C2_MODEL = """
# reversible A + B <-> C at the c2 density, in a 20 um cube
dim 3
boundaries 0 0 20
boundaries 1 0 20 r
boundaries 2 0 20
species A B C
difc A 1
difc B(all) 1
difc C 0.5
time_start 0
time_stop 5
time_step 0.0005
random_seed 2
reaction fwd A + B -> C 0.05
reaction back C -> A + B 10
product_placement back pgemmax 0.2
reaction make 0 -> A 3
mol 18000 A u u u
mol 18000 B u u 7.5
graphics opengl     # display statements are ignored
end_file
this line is after end_file and never read
"""


def api_c2(device=None):
    s = System((0, 0, 0), (20, 20, 20), dt=5e-4, seed=2, device=L.BD_DEVICE_NONE if device is None else device)
    A, B, Cc = s.add_species(1.0), s.add_species(1.0), s.add_species(0.5)
    s.add_reaction(2, [A, B], [Cc], 0.05)
    back = s.add_reaction(1, [Cc], [A, B], 10.0)
    s.set_product_placement(back, L.BD_PP_PGEMMAX, 0.2)
    s.add_reaction(0, [], [A], 3.0)
    s.finalize()
    return s


def test_model_matches_the_same_network_built_through_the_abi():
    m, info = System.from_model(C2_MODEL, device=None)
    assert info == dict(time_start=0.0, time_stop=5.0, steps=10000, n_molecules=36000)
    assert (m.n_species, m.n_reactions) == (3, 3)
    assert [m.species_id(n) for n in "ABC"] == [0, 1, 2]
    assert [m.reaction_id(n) for n in ("fwd", "back", "make")] == [0, 1, 2]
    a = api_c2()
    np.testing.assert_array_equal(m.species_d(), a.species_d())
    for r in range(3):
        assert m.reaction_info(r) == a.reaction_info(r)
    assert m.reaction_info(0)["bind_radius"] == pytest.approx(0.0181319, rel=1e-5)  # b = 0 fallback
    cfg = m.cfg
    assert list(cfg.box_lo) == [0, 0, 0] and list(cfg.box_hi) == [20, 20, 20]
    assert cfg.dt == pytest.approx(5e-4) and cfg.seed == 2
    a.set_particles(np.full((36000, 3), 1.0, np.float32), np.zeros(36000, np.int32))
    for k in range(3):
        np.testing.assert_array_equal(m.grid()[k], a.grid()[k])


def test_reference_preset_as_a_model():
    # the enzyme preset of the reference (test2Reactions / test2Types) as text
    text = """
    dim 3
    boundaries x -1 1
    boundaries y -1 1
    boundaries z -1 1
    species E S ES P
    difc E 0.05
    difc S 0.05
    difc ES 0.05
    difc P 0.05
    time_step 0.001
    reaction fwd E + S -> ES 0.01
    reaction back ES -> E + S 1
    reaction prod ES -> E + P 1
    product_placement back pgemmax 0.2
    mol 100 E u u u
    mol 1000 S u u u
    mol 3 P 0 0 0.5
    """
    m, info = System.from_model(text, device=None)
    assert info["n_molecules"] == 1103 and info["steps"] == 0
    assert m.reaction_info(m.reaction_id("back"))["reverse"] == m.reaction_id("fwd")


@pytest.mark.parametrize("bad, code, where", [
    ("frobnicate 3", L.BD_ERR_INVALID_ARGUMENT, "line 2"),
    ("boundaries 0 0 20 p", L.BD_ERR_UNSUPPORTED, "line 2"),
    ("reaction r A + Q -> C 1", L.BD_ERR_INVALID_ARGUMENT, "unknown species Q"),
    ("dim 2", L.BD_ERR_UNSUPPORTED, "dim 3"),
    ("reaction r A + B + C -> A 1", L.BD_ERR_UNSUPPORTED, "two reactants"),
    ("product_placement fwd ratio 2", L.BD_ERR_UNSUPPORTED, "ratio"),
    ("mol 5 A 30 u u", L.BD_ERR_INVALID_ARGUMENT, "outside the box"),
])
def test_malformed_models_name_the_line(bad, code, where):
    text = "species A B C\n" + bad + "\n" + "\n".join(
        ["boundaries 0 0 20", "boundaries 1 0 20", "boundaries 2 0 20", "time_step 0.001",
         "difc A 1", "difc B 1", "difc C 1", "reaction fwd A + B -> C 0.05"])
    with pytest.raises(L.BDError) as e:
        System.from_model(text, device=None)
    assert e.value.code == code and where in str(e.value)


def test_missing_time_step_and_boundaries():
    with pytest.raises(L.BDError, match="time_step"):
        System.from_model("species A\nboundaries 0 0 1\nboundaries 1 0 1\nboundaries 2 0 1\n", device=None)
    with pytest.raises(L.BDError, match="boundaries"):
        System.from_model("species A\ntime_step 0.1\n", device=None)


def test_model_file(tmp_path):
    p = tmp_path / "c2.txt"
    p.write_text(C2_MODEL)
    m, info = System.from_model(path=p, device=None)
    assert info["n_molecules"] == 36000
    with pytest.raises(L.BDError, match="cannot read"):
        System.from_model(path=tmp_path / "missing.txt", device=None)


SURF_MODEL = """
dim 3
boundaries x 0 10
boundaries y 0 10
boundaries z 0 10
species A B
difc all 1
time_step 0.001
max_surface 3
start_surface membrane
  action all both reflect
  action B front absorb
  color both 0.5 0.5 0.5     # display: ignored
  panel sph 5 5 5 3 20 20 ball
end_surface
start_surface walls
  action front all transmit
  action back A reflect
  panel rect +x 8 0 0 10 10
  panel rect -2 0 0 9.5 10 10
  panel tri 1 1 1 2 1 1 1 2 1
  panel cyl 2 2 2 2 2 8 -1 12 12
  panel hemi 7 7 7 1 0 0 1 10 10
  panel disk 3 3 3 0.5 0 1 0
end_surface
surface walls action A both absorb
mol 100 A u u u
"""


def test_model_surfaces():
    m, info = System.from_model(SURF_MODEL, device=None)
    assert m.surface_counts() == (2, 7)
    A, B = m.species_id("A"), m.species_id("B")
    assert m.surface_action(0, A, "front") == L.BD_SURF_REFLECT
    assert [m.surface_action(0, B, f) for f in ("front", "back")] == [L.BD_SURF_ABSORB, L.BD_SURF_REFLECT]
    assert [m.surface_action(1, A, f) for f in ("front", "back")] == [L.BD_SURF_ABSORB] * 2
    assert [m.surface_action(1, B, f) for f in ("front", "back")] == [L.BD_SURF_TRANSMIT] * 2
    p = [m.panel_info(k) for k in range(7)]
    assert [q["shape"] for q in p] == [L.BD_PANEL_SPH, L.BD_PANEL_RECT, L.BD_PANEL_RECT, L.BD_PANEL_TRI,
                                       L.BD_PANEL_CYL, L.BD_PANEL_HEMI, L.BD_PANEL_DISK]
    assert p[0]["r"] == 3 and p[0]["front"] == 1.0
    assert (p[1]["axis"], p[1]["front"], p[1]["bounds"]) == (0, 1.0, [0, 10, 0, 10])
    assert (p[2]["axis"], p[2]["front"], p[2]["a"]) == (2, -1.0, [0, 0, 9.5])
    assert p[4]["front"] == -1.0 and p[4]["r"] == 1 and p[4]["len"] == 6
    assert [q["surface"] for q in p] == [0, 1, 1, 1, 1, 1, 1]


@pytest.mark.parametrize("bad, code, where", [
    ("start_surface s\n  action all both jump\nend_surface", L.BD_ERR_UNSUPPORTED, "line 8"),
    ("start_surface s\n  rate A fsoln bsoln 1\nend_surface", L.BD_ERR_UNSUPPORTED, "line 8"),
    ("start_surface s\n  panel rect x 0 0 0 1 1\nend_surface", L.BD_ERR_INVALID_ARGUMENT, "line 8"),
    ("start_surface s\n  panel sph 1 1 1\nend_surface", L.BD_ERR_INVALID_ARGUMENT, "needs 4"),
    ("start_surface s\n  panel tri 0 0 0 1 1 1 2 2 2\nend_surface", L.BD_ERR_INVALID_ARGUMENT, "degenerate"),
    ("start_surface s\n  panel box 0 0 0 1\nend_surface", L.BD_ERR_UNSUPPORTED, "box"),
    ("start_surface s\n  action Q both reflect\nend_surface", L.BD_ERR_INVALID_ARGUMENT, "unknown species Q"),
    ("start_surface s\n  panel sph 1 1 1 1", L.BD_ERR_INVALID_ARGUMENT, "without end_surface"),
])
def test_malformed_surfaces_name_the_line(bad, code, where):
    text = "species A B C\n" + bad.replace("start_surface", "\n".join(
        ["boundaries 0 0 20", "boundaries 1 0 20", "boundaries 2 0 20", "time_step 0.001", "difc all 1",
         "start_surface"]))
    with pytest.raises(L.BDError) as e:
        System.from_model(text, device=None)
    assert e.value.code == code and where in str(e.value)
