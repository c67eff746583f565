"""The c3 workload at its full size (16M particles, 8 species, 12
reactions, 200 um cube), checked through properties that hold at any size:
the two sort modes are independent GPU paths that must agree bit for bit,
every record stays in the box, the state is in canonical order (by cell,
then by the record's words), and the composition stays at the stationary
state the run starts from."""
import numpy as np
import pytest

from gpusmoldyn_gb300 import _lib as L
from gpusmoldyn_gb300 import configs

pytestmark = pytest.mark.gpu

N = 16_000_000
STEPS = 20


def cell_keys(xyz, lo, inv, dims):
    """The step's cell key in float32, the kernels' operations (cell_coord)."""
    key = np.zeros(len(xyz), np.int64)
    for a in (2, 1, 0):
        f = (xyz[:, a].astype(np.float32) - np.float32(lo[a])) * np.float32(inv[a])
        c = np.clip(np.floor(f).astype(np.int64), 0, int(dims[a]) - 1)
        key = key * int(dims[a]) + c
    return key


@pytest.fixture(scope="module")
def runs():
    out = {}
    for sort in ("binned", "compact"):
        s = configs.build_c3(n=N, sort=sort)
        s.step(STEPS)
        s.synchronize()
        xyz, w = s.slots()
        out[sort] = dict(xyz=xyz, w=w, events=s.event_counts(), grid=s.grid(), counts=s.species_counts(),
                         n=s.count())
        s.close()
    return out


def test_sort_modes_agree_bit_for_bit(runs):
    a, b = runs["binned"], runs["compact"]
    np.testing.assert_array_equal(a["w"], b["w"])
    np.testing.assert_array_equal(a["xyz"].view(np.uint32), b["xyz"].view(np.uint32))
    np.testing.assert_array_equal(a["events"], b["events"])
    assert a["events"].sum() > 3_000  # every reaction fires (about 6,000 events in 20 steps)


def test_records_in_the_box_and_canonical(runs):
    r = runs["binned"]
    live = r["w"] != L.DEAD
    xyz = r["xyz"][live]
    assert (xyz >= 0).all() and (xyz <= 200.0).all()
    dims, cell, inv = r["grid"]
    keys = cell_keys(xyz, (0.0, 0.0, 0.0), inv, dims)
    # the step leaves the products of its last phase in their reactants'
    # slots: apart from those few, records follow cell order
    assert np.mean(np.diff(keys) >= 0) > 0.999
    # and inside each cell the order is by x bits (then the other words)
    same = np.diff(keys) == 0
    xb = xyz[:, 0].view(np.uint32)
    assert np.mean(np.diff(xb.astype(np.int64))[same] >= 0) > 0.99


def test_composition_stays_stationary(runs):
    r = runs["binned"]
    _, rx = configs.c3_network()
    _, frac = configs.c3_steady_state(rx, N / 200.0 ** 3)
    got = r["counts"] / r["counts"].sum()
    np.testing.assert_allclose(got, frac, atol=0.01)
    assert abs(r["n"] - N) < 0.01 * N
