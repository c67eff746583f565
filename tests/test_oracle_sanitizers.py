"""The oracle under AddressSanitizer and UndefinedBehaviorSanitizer: its
step, built from oracle/oracle.cpp with a small driver
(oracle/sanitize_main.cpp), runs reacting systems with panels and a
diffusion-only system without a memory error, a leak or undefined
behaviour."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE = os.path.join(ROOT, "oracle")
FLAGS = ["-O1", "-g", "-std=c++17", "-ffp-contract=off", "-fsanitize=address,undefined",
         "-fno-sanitize-recover=all", "-fno-omit-frame-pointer"]


def _cxx():
    return os.environ.get("CXX") or shutil.which("g++")


def test_oracle_step_is_clean_under_asan_and_ubsan(tmp_path):
    cxx = _cxx()
    if not cxx:
        pytest.skip("no C++ compiler")
    probe = tmp_path / "probe.cpp"
    probe.write_text("int main() { return 0; }\n")
    if subprocess.run([cxx, *FLAGS, str(probe), "-o", str(tmp_path / "probe")], capture_output=True).returncode:
        pytest.skip("the compiler has no sanitizer runtimes")
    exe = tmp_path / "oracle_san"
    build = subprocess.run([cxx, *FLAGS, "-I" + ORACLE, os.path.join(ORACLE, "oracle.cpp"),
                            os.path.join(ORACLE, "sanitize_main.cpp"), "-o", str(exe)],
                           capture_output=True, text=True)
    assert build.returncode == 0, build.stderr
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0", UBSAN_OPTIONS="print_stacktrace=1")
    run = subprocess.run([str(exe)], capture_output=True, text=True, env=env, timeout=300)
    assert run.returncode == 0, run.stdout + run.stderr
    assert "runtime error" not in run.stderr and "ERROR: AddressSanitizer" not in run.stderr
    assert run.stdout.count("steps") == 4
