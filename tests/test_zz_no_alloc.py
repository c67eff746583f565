"""The allocation-free cell sort, bd_cell_sort_static.

It exists for callers that cannot call cudaMalloc (a host application that
owns all device memory, a time-critical loop that cannot take cudaMalloc's
implicit synchronisation): its scratch lives in one file-scope device array
instead of buffers a handle allocates.  Its output must equal the sort the
simulation handle performs in a step -- records ordered by cell, then by
their bits -- through the C ABI, on two calls in a row: the shared scratch
keeps the last call's contents, so the second call shows that each call
clears what must start at zero.  Comparison is exact (integer keys and
copied records; the tolerance is zero).
"""
import ctypes as C

import numpy as np
import pytest

from gpusmoldyn_gb300 import _lib as L
from gpusmoldyn_gb300.configs import rng, uniform_positions
from gpusmoldyn_gb300.system import System

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

BOX = ((0.0, 0.0, 0.0), (12.0, 9.0, 7.5))


def handle_sort(pos, species, cell):
    """The existing path: one step of immobile particles (D = 0) whose only
    reaction never fires (rate 0) -- the step sorts them and moves nothing."""
    s = System(BOX[0], BOX[1], dt=1e-3, seed=3, cell_size=cell, normals="table")
    for _ in range(3):
        s.add_species(0.0)
    s.add_reaction(1, [2], [], 0.0)
    s.finalize()
    s.set_particles(pos, species)
    s.step(1)
    s.synchronize()
    xyz, w = s.slots()
    cells = s.cells()
    dims, _, _ = s.grid()
    s.close()
    return xyz, w, cells, dims


def static_sort(pos, species, dims):
    lib = L.load()
    n = len(pos)
    rec = np.zeros((n, 4), np.float32)
    rec[:, :3] = pos
    rec[:, 3] = np.asarray(species, np.uint32).view(np.float32)
    n_cells = int(np.prod(dims.astype(np.int64)))
    d_in = torch.from_numpy(rec).cuda()
    d_out = torch.full_like(d_in, float("nan"))
    d_start = torch.full((n_cells + 1,), -1, dtype=torch.int32, device="cuda")
    lo = (C.c_float * 3)(*BOX[0])
    hi = (C.c_float * 3)(*BOX[1])
    dm = (C.c_uint32 * 3)(*[int(v) for v in dims])
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.bd_cell_sort_static(C.c_void_p(d_in.data_ptr()), n, lo, hi, dm, C.c_void_p(d_out.data_ptr()),
                                 C.c_void_p(d_start.data_ptr()), C.c_void_p(stream))
    assert rc == L.BD_OK, lib.bd_status_string(rc)
    torch.cuda.synchronize()
    return d_out.cpu().numpy(), d_start.cpu().numpy().view(np.uint32)


def dataset(seed, n):
    g = rng(seed)
    pos = uniform_positions(g, n, BOX[0], BOX[1])
    pos[: n // 10] = pos[n // 10: 2 * (n // 10)]  # duplicate positions share cells and bits
    species = (np.arange(n) % 3).astype(np.int32)
    return pos, species


def test_static_sort_matches_handle_sort_twice():
    cell = 0.5
    for call, (seed, n) in enumerate(((31, 60000), (32, 23456))):
        pos, sp = dataset(seed, n)
        xyz, w, cells, dims = handle_sort(pos, sp, cell)
        out, start = static_sort(pos, sp, dims)
        assert out.shape == (n, 4) and len(start) == len(cells)
        np.testing.assert_array_equal(start, cells, err_msg=f"call {call}: cell starts")
        np.testing.assert_array_equal(out[:, :3].view(np.uint32), xyz.view(np.uint32),
                                      err_msg=f"call {call}: positions")
        np.testing.assert_array_equal(out[:, 3].view(np.uint32), w, err_msg=f"call {call}: species words")


def test_static_sort_rejects_grids_beyond_its_scratch():
    lib = L.load()
    lo = (C.c_float * 3)(*BOX[0])
    hi = (C.c_float * 3)(*BOX[1])
    dm = (C.c_uint32 * 3)(128, 128, 65)  # 1,064,960 cells > 2^20
    buf = torch.zeros((4, 4), device="cuda")
    start = torch.zeros(8, dtype=torch.int32, device="cuda")
    rc = lib.bd_cell_sort_static(C.c_void_p(buf.data_ptr()), 4, lo, hi, dm, C.c_void_p(buf.data_ptr()),
                                 C.c_void_p(start.data_ptr()), None)
    assert rc == L.BD_ERR_CAPACITY


def crowded_dataset(seed, n):
    """Uniform records plus two crowded cells: about 2,000 records in one
    (ordered in shared memory) and 5,000 in another (ordered in place in
    global memory), some of them exact duplicates."""
    pos, species = dataset(seed, n)
    g = rng(seed + 100)
    a = (1.1 + 0.3 * g.random((2000, 3))).astype(np.float32)      # inside cell [1.0, 1.5)^3
    b = (6.05 + 0.4 * g.random((5000, 3))).astype(np.float32)     # inside cell [6.0, 6.5)^3
    b[:700] = b[700:1400]
    pos = np.concatenate([pos, a, b])
    species = np.concatenate([species, np.arange(7000, dtype=np.int32) % 3])
    perm = g.permutation(len(pos))
    return pos[perm], species[perm]


def test_static_sort_orders_crowded_cells():
    cell = 0.5
    for call, (seed, n) in enumerate(((41, 30000), (42, 12345))):
        pos, sp = crowded_dataset(seed, n)
        xyz, w, cells, dims = handle_sort(pos, sp, cell)
        out, start = static_sort(pos, sp, dims)
        assert np.max(np.diff(start.astype(np.int64))) >= 5000
        np.testing.assert_array_equal(start, cells, err_msg=f"call {call}: cell starts")
        np.testing.assert_array_equal(out[:, :3].view(np.uint32), xyz.view(np.uint32),
                                      err_msg=f"call {call}: positions")
        np.testing.assert_array_equal(out[:, 3].view(np.uint32), w, err_msg=f"call {call}: species words")
