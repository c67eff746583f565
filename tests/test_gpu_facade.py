"""The reference-shaped front ends: the C++ ParticleSystem drop-in (compiled
against include/ and linked with the library) and the Python mirror."""
import os
import subprocess

import numpy as np
import pytest

from gpusmoldyn_gb300 import ParticleSystem, _lib as L

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_particle_system(tmp_path):
    exe = str(tmp_path / "facade")
    lib_dir = os.path.dirname(L.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "facade_main.cpp"), "-L", lib_dir, "-lgpusmoldyn",
                    "-Wl,-rpath," + lib_dir, "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.count("preset") == 3


def test_python_particle_system_presets():
    for preset in ("test1", "test2", "test3"):
        # test1's rates make every A-B pair of the [-1,1]^3 world a candidate
        n = 1000 if preset == "test1" else 10000
        ps = ParticleSystem(n, (64, 64, 64), preset=preset)
        n0 = ps.getNumParticles()
        ok = all(ps.update() for _ in range(5 if preset == "test1" else 20))
        a = ps.getArray(ParticleSystem.POSITION)
        assert a.shape == (ps.getNumParticles(), 4)
        assert np.all(np.abs(a[:, :3]) <= 1.0)
        if preset == "test3":
            assert ok and ps.getNumParticles() == n0 == 10000
            assert ps.reactionOrderInfo[2]["reactionsPerOrder"] == 0
        if preset == "test2":
            assert ps.reactionOrderInfo[1]["reactionsPerOrder"] == 2
            assert ps.reactionList["order"] == [2, 1, 1]
