"""A model read from text steps exactly like the same model built through
the C ABI with the same molecules (positions compared bit for bit)."""
import numpy as np
import pytest

from gpusmoldyn_gb300.system import System
from test_model import C2_MODEL, api_c2

pytestmark = pytest.mark.gpu


def test_model_steps_like_the_abi_build():
    m, info = System.from_model(C2_MODEL, device=0)
    pos, sp = m.particles()
    assert len(sp) == info["n_molecules"] == 36000
    assert np.all(pos >= 0) and np.all(pos <= 20) and np.all(pos[18000:, 2] == 7.5)
    a = api_c2(device=0)
    a.set_particles(pos, sp)
    for s in (m, a):
        s.step(40)
        s.synchronize()
    xm, wm = m.slots()
    xa, wa = a.slots()
    np.testing.assert_array_equal(xm.view(np.uint32), xa.view(np.uint32))
    np.testing.assert_array_equal(wm, wa)
    np.testing.assert_array_equal(m.event_counts(), a.event_counts())
    assert m.event_counts()[0] > 0


def read_binary_snapshot(path):
    raw = open(path, "rb").read()
    step, n = np.frombuffer(raw[:16], np.uint64)
    rec = np.frombuffer(raw[16:], np.dtype([("p", np.float32, 3), ("s", np.int32)]))
    assert len(rec) == n
    return int(step), rec["p"], rec["s"]


def test_snapshots_restore_the_molecules(tmp_path):
    m, _ = System.from_model(C2_MODEL, device=0)
    m.step(25)
    m.synchronize()
    pos, sp = m.particles()
    m.write_snapshot(tmp_path / "s.txt")
    m.write_snapshot(tmp_path / "s.bin", binary=True)
    lines = open(tmp_path / "s.txt").read().splitlines()
    assert lines[0] == f"# step 25 molecules {len(sp)} species 3"
    assert [int(v) for v in lines[1].split()[2:]] == list(np.bincount(sp, minlength=3))
    txt = np.loadtxt(tmp_path / "s.txt")
    np.testing.assert_array_equal(txt[:, :3].astype(np.float32), pos)
    np.testing.assert_array_equal(txt[:, 3].astype(np.int32), sp)
    step, p2, s2 = read_binary_snapshot(tmp_path / "s.bin")
    assert step == 25
    np.testing.assert_array_equal(p2, pos)
    np.testing.assert_array_equal(s2, sp)
