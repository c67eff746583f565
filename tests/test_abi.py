"""The C-ABI library loads and exports every declared entry point; host-only
set-up works without a GPU (no compute calls)."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from gpusmoldyn_gb300 import _lib as L
from gpusmoldyn_gb300.system import System

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            txt = open(os.path.join(inc, f)).read()
            names |= set(re.findall(r"BD_API\s+[\w\s\*]+?\b(bd_\w+)\s*\(", txt))
    return names


def test_library_exports_every_declared_symbol():
    lib = L.load()
    names = declared_symbols()
    assert len(names) >= 35
    for n in sorted(names):
        assert hasattr(lib, n), n
    out = subprocess.run(["nm", "-D", "--defined-only", L.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (bd_\w+)", out))
    assert names <= exported
    # the ctypes binding covers the whole ABI
    assert names <= set(L.exported_symbols()) | {"bd_config_default"}


def test_cpp_facade_exported():
    out = subprocess.run(["nm", "-DC", "--defined-only", L.LIB_PATH], capture_output=True, text=True).stdout
    for m in ("gpusmoldyn::ParticleSystem::ParticleSystem", "gpusmoldyn::ParticleSystem::update()",
              "gpusmoldyn::ParticleSystem::getArray"):
        assert m in out, m


def test_version_and_status_strings():
    lib = L.load()
    assert b"sm_103a" in lib.bd_version()
    assert lib.bd_status_string(L.BD_ERR_PGEM_UNATTAINABLE) == b"geminate probability unattainable"


def test_host_only_handle_derives_parameters():
    s = System((0, 0, 0), (10, 10, 10), dt=1e-3, device=-1)
    a, b, c = s.add_species(1.0), s.add_species(1.0), s.add_species(0.5)
    r = s.add_reaction(2, [a, b], [c], 0.01)
    s.finalize()
    info = s.reaction_info(r)
    assert abs(info["bind_radius"] - 0.0133939) < 1e-6
    s.set_particles(np.full((100, 3), 5.0, np.float32), np.zeros(100, np.int32))
    dims, cell, inv = s.grid()
    assert np.all(cell >= 1.01 * info["bind_radius"])
    assert np.all(dims >= 1)
    assert s.lib.bd_step(s.h, 1) == L.BD_ERR_NO_DEVICE
    s.close()


def test_setup_errors_mirror_reference_codes():
    s = System(device=-1)
    s.add_species(0.0)
    with pytest.raises(L.BDError) as e:
        s.add_reaction(2, [0, 0], [0], -1.0)
    assert e.value.code == L.BD_ERR_NEGATIVE_RATE
    s.add_reaction(2, [0, 0], [0], 1.0)
    # both reactants immobile: rxnsetrate returns 4
    assert s.lib.bd_finalize(s.h) == L.BD_ERR_ZERO_DIFFUSION
    s.close()


def test_invalid_arguments():
    lib = L.load()
    cfg = L.bd_config()
    lib.bd_config_default(C.byref(cfg))
    cfg.dt = -1.0
    h = C.c_void_p()
    assert lib.bd_create(C.byref(cfg), C.byref(h)) == L.BD_ERR_INVALID_ARGUMENT
    s = System(device=-1)
    s.add_species(1.0)
    with pytest.raises(L.BDError):
        s.add_reaction(1, [5], [], 1.0)
    s.finalize()
    with pytest.raises(L.BDError):
        s.set_particles(np.full((1, 3), 2.0, np.float32), np.zeros(1, np.int32))  # outside the box


def _static_sort_args(dims, d_in, d_out, d_start, n=4):
    lo = (C.c_float * 3)(0.0, 0.0, 0.0)
    hi = (C.c_float * 3)(1.0, 1.0, 1.0)
    dm = (C.c_uint32 * 3)(*dims)
    return (C.c_void_p(d_in), n, lo, hi, dm, C.c_void_p(d_out), C.c_void_p(d_start), None)


def test_static_sort_rejects_wrapping_and_overlapping_arguments():
    """The allocation-free sort checks its grid and buffers before it touches
    the GPU: these calls return before any CUDA call, with placeholder
    addresses that are never dereferenced."""
    lib = L.load()
    a, b, c = 1 << 20, 2 << 20, 3 << 20
    # 2^22 * 2^22 * 2^20 = 2^64 wraps a 64-bit product to 0
    assert lib.bd_cell_sort_static(*_static_sort_args((1 << 22, 1 << 22, 1 << 20), a, b, c)) == L.BD_ERR_CAPACITY
    assert lib.bd_cell_sort_static(*_static_sort_args((1 << 21, 1, 1), a, b, c)) == L.BD_ERR_CAPACITY
    assert lib.bd_cell_sort_static(*_static_sort_args((128, 128, 65), a, b, c)) == L.BD_ERR_CAPACITY
    assert lib.bd_cell_sort_static(*_static_sort_args((0, 4, 4), a, b, c)) == L.BD_ERR_INVALID_ARGUMENT
    # in place, and cell starts inside the record buffers
    assert lib.bd_cell_sort_static(*_static_sort_args((4, 4, 4), a, a, c)) == L.BD_ERR_INVALID_ARGUMENT
    assert lib.bd_cell_sort_static(*_static_sort_args((4, 4, 4), a, a + 32, c)) == L.BD_ERR_INVALID_ARGUMENT
    assert lib.bd_cell_sort_static(*_static_sort_args((4, 4, 4), a, b, b + 16)) == L.BD_ERR_INVALID_ARGUMENT
    assert lib.bd_cell_sort_static(*_static_sort_args((4, 4, 4), a, b, a + 60)) == L.BD_ERR_INVALID_ARGUMENT
