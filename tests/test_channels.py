"""Competing second-order reactions of one reactant pair (pair_mode
CHANNELS): one binding radius from the summed rate, each reaction's share
of it as cumulative thresholds; the reference's rule (the last reaction
listed for a pair is its only reaction) stays the default.  Host-only."""
import pytest

from gpusmoldyn_gb300 import _lib as L
from gpusmoldyn_gb300.system import System


def network(pairs, probability=None):
    s = System((0, 0, 0), (5, 5, 5), dt=1e-3, device=L.BD_DEVICE_NONE, pairs=pairs)
    A, B, Cc, D = (s.add_species(d) for d in (1.0, 1.0, 0.5, 0.3))
    s.add_reaction(2, [A, B], [Cc], 0.03)
    s.add_reaction(2, [B, A], [D], 0.01)       # same pair, reactants listed the other way round
    s.add_reaction(2, [A, B], [Cc, D], 0.06)
    s.add_reaction(2, [Cc, D], [A], 0.02)      # a pair with one reaction
    if probability is not None:
        s.set_reaction_probability(1, probability)
    return s


def test_competing_reactions_share_one_radius_and_split_the_rate():
    s = network("channels")
    s.finalize()
    lib = L.load()
    a = lib.bd_bindingradius(0.03 + 0.01 + 0.06, 1e-3, 2.0, -1, 0)
    info = [s.reaction_info(r) for r in range(4)]
    for r in range(3):
        assert info[r]["bind_radius"] == pytest.approx(a, rel=1e-6)
        assert info[r]["prob"] == 1.0
    assert [info[r]["channel_threshold"] for r in range(3)] == pytest.approx([0.3, 0.4, 1.0], rel=1e-6)
    # a pair with a single reaction is calibrated on its own rate
    assert info[3]["bind_radius"] == pytest.approx(lib.bd_bindingradius(0.02, 1e-3, 0.8, -1, 0), rel=1e-6)
    assert info[3]["channel_threshold"] == 1.0


def test_last_listed_reaction_is_the_pair_reaction_by_default():
    s = network("last")
    s.finalize()
    lib = L.load()
    info = [s.reaction_info(r) for r in range(3)]
    for r, k in enumerate((0.03, 0.01, 0.06)):
        assert info[r]["bind_radius"] == pytest.approx(lib.bd_bindingradius(k, 1e-3, 2.0, -1, 0), rel=1e-6)
        assert info[r]["channel_threshold"] == 1.0


def test_reaction_probability_on_a_competing_reaction_is_unsupported():
    s = network("channels", probability=0.5)
    with pytest.raises(L.BDError) as e:
        s.finalize()
    assert e.value.code == L.BD_ERR_UNSUPPORTED
    s = network("last", probability=0.5)
    s.finalize()  # allowed when reactions do not compete
