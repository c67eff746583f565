"""Build recipe for the test oracle (TEST INFRASTRUCTURE, not product).

* ``build_oracle()`` compiles oracle.cpp (the CPU restatement of the step)
  into ``oracle/_build/liboracle.so`` with -ffp-contract=off so every float
  operation is a single IEEE operation, with OpenMP when available.
* ``build_ref(ref_dir)`` compiles ref_kat.cpp against the reference's own
  host sources *where they lie* in ``ref_dir`` (nothing is copied) into
  ``oracle/_ref/ref_kat``.  ``ref_dir`` defaults to $REF_DIR, else to a
  ``reference`` directory beside the repository.  It is skipped when the
  reference tree is absent.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
ORACLE_LIB = os.path.join(BUILD, "liboracle.so")
REF_KAT = os.path.join(REF_OUT, "ref_kat")
REF_SOURCES = ["rxnparam.cpp", "smolreact.cpp", "stats.cpp", "SFMT/SFMT.cpp", "rnd/genmtrand.cpp",
               "reaction_cpu.cpp"]


def _cxx():
    return os.environ.get("CXX") or shutil.which("g++") or "g++"


def build_oracle(force: bool = False) -> str:
    src = [os.path.join(HERE, "oracle.cpp"), os.path.join(HERE, "oracle.h"), os.path.abspath(__file__)]
    if not force and os.path.exists(ORACLE_LIB) and all(
            os.path.getmtime(s) <= os.path.getmtime(ORACLE_LIB) for s in src):
        return ORACLE_LIB
    os.makedirs(BUILD, exist_ok=True)
    base = [_cxx(), "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared",
            os.path.join(HERE, "oracle.cpp"), "-o", ORACLE_LIB + ".tmp"]
    res = subprocess.run(base[:1] + ["-fopenmp"] + base[1:], capture_output=True, text=True)
    if res.returncode != 0:
        res = subprocess.run(base, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + res.stderr)
    os.replace(ORACLE_LIB + ".tmp", ORACLE_LIB)
    return ORACLE_LIB


def build_ref(ref_dir: str | None = None, force: bool = False) -> str | None:
    ref_dir = ref_dir or os.environ.get("REF_DIR") or os.path.join(HERE, "..", "..", "reference")
    if not os.path.exists(os.path.join(ref_dir, "rxnparam.cpp")):
        return None
    if not force and os.path.exists(REF_KAT) and os.path.getmtime(REF_KAT) >= os.path.getmtime(
            os.path.join(HERE, "ref_kat.cpp")):
        return REF_KAT
    os.makedirs(REF_OUT, exist_ok=True)
    cuda_inc = os.environ.get("CUDA_INC", "/usr/local/cuda/include")
    cmd = [_cxx(), "-O2", "-w", "-I", ref_dir, "-I", cuda_inc, os.path.join(HERE, "ref_kat.cpp")]
    cmd += [os.path.join(ref_dir, s) for s in REF_SOURCES]
    cmd += ["-o", REF_KAT]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("reference KAT build failed:\n" + res.stderr)
    return REF_KAT


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
