// bd_static_sort.cu -- the uniform-grid cell sort without any allocation.
//
// Some callers cannot call cudaMalloc: a host application that owns every
// byte of device memory and forbids its plugins to grow the footprint, or a
// time-critical loop where cudaMalloc's implicit device-wide
// synchronisation is not acceptable.  bd_cell_sort_static gives them the
// step's counting sort (cell histogram, exclusive scan, scatter, canonical
// order inside each cell) with its scratch -- the per-cell counts and the
// scan's tile sums -- in a file-scope device array of fixed size instead of
// buffers a handle allocates.  The caller passes the input records and the
// output buffers.
//
// The array holds kStaticMaxCells + kStaticMaxTiles 32-bit words (about
// 4 MiB); every GPU that loads this library keeps it until the process
// exits.  All calls share it and it keeps the last call's contents, so each
// call clears the counts it uses first, and calls whose work overlaps on
// the GPU (different streams, no ordering between them) race on it.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "../../include/gpusmoldyn.h"
#include "bd_device.cuh"

namespace {

using bd::rec_equal;
using bd::rec_less;

constexpr uint32_t kStaticMaxCells = 1u << 20;
constexpr uint32_t kStaticTile = 4096;
constexpr uint32_t kStaticMaxTiles = kStaticMaxCells / kStaticTile;
constexpr unsigned kFull = 0xFFFFFFFFu;
constexpr int kMaxDevices = 64;

// counts [0, kStaticMaxCells), tile sums after them
static __device__ __align__(256) uint32_t g_static_scratch[kStaticMaxCells + kStaticMaxTiles];

struct StaticGrid {
  float lo[3], inv[3];
  uint32_t dims[3];
  uint32_t n_cells;
};

__device__ __forceinline__ uint32_t grid_key(const StaticGrid& g, const float4& r) {
  const int cx = bd::cell_coord(r.x, g.lo[0], g.inv[0], g.dims[0]);
  const int cy = bd::cell_coord(r.y, g.lo[1], g.inv[1], g.dims[1]);
  const int cz = bd::cell_coord(r.z, g.lo[2], g.inv[2], g.dims[2]);
  return ((uint32_t)cz * g.dims[1] + (uint32_t)cy) * g.dims[0] + (uint32_t)cx;
}

__global__ void k_static_clear(uint32_t* __restrict__ s, uint32_t n) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) s[i] = 0u;
}

__global__ void __launch_bounds__(256) k_static_count(const float4* __restrict__ in, uint32_t n, StaticGrid g,
                                                      uint32_t* __restrict__ counts) {
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
    const uint32_t i = base + threadIdx.x;
    const uint32_t key = i < n ? grid_key(g, in[i]) : 0xFFFFFFFFu;
    const uint32_t peers = __match_any_sync(kFull, key);
    if (key != 0xFFFFFFFFu && (threadIdx.x & 31u) == (uint32_t)(__ffs(peers) - 1))
      atomicAdd(&counts[key], (uint32_t)__popc(peers));
  }
}

template <int kThreads>
__device__ __forceinline__ uint32_t block_scan_excl(uint32_t v, uint32_t* total) {
  __shared__ uint32_t warp_sums[kThreads / 32];
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t incl = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t t = __shfl_up_sync(kFull, incl, d);
    if (lane >= (uint32_t)d) incl += t;
  }
  if (lane == 31) warp_sums[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    const uint32_t s = lane < kThreads / 32 ? warp_sums[lane] : 0u;
    uint32_t si = s;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t t = __shfl_up_sync(kFull, si, d);
      if (lane >= (uint32_t)d) si += t;
    }
    if (lane < kThreads / 32) warp_sums[lane] = si - s;
    const uint32_t tot = __shfl_sync(kFull, si, 31);
    if (lane == 0) *total = tot;
  }
  __syncthreads();
  const uint32_t r = warp_sums[warp] + incl - v;
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(1024) k_static_scan_tiles(const uint32_t* __restrict__ counts, uint32_t n_cells,
                                                            uint32_t* __restrict__ tiles) {
  __shared__ uint32_t total;
  uint32_t sum = 0;
  for (uint32_t k = 0; k < kStaticTile / 1024; ++k) {
    const uint32_t idx = blockIdx.x * kStaticTile + k * 1024 + threadIdx.x;
    if (idx < n_cells) sum += counts[idx];
  }
  block_scan_excl<1024>(sum, &total);
  if (threadIdx.x == 0) tiles[blockIdx.x] = total;
}

__global__ void __launch_bounds__(1024) k_static_scan_top(uint32_t* __restrict__ tiles, uint32_t n_tiles) {
  __shared__ uint32_t total;
  const uint32_t v = threadIdx.x < n_tiles ? tiles[threadIdx.x] : 0u;  // n_tiles <= 256
  const uint32_t ex = block_scan_excl<1024>(v, &total);
  if (threadIdx.x < n_tiles) tiles[threadIdx.x] = ex;
}

__global__ void __launch_bounds__(1024) k_static_scan_down(const uint32_t* __restrict__ counts, uint32_t n_cells,
                                                           const uint32_t* __restrict__ tiles,
                                                           uint32_t* __restrict__ start, uint32_t n) {
  __shared__ uint32_t total;
  constexpr uint32_t kPer = kStaticTile / 1024;
  const uint32_t base = blockIdx.x * kStaticTile + threadIdx.x * kPer;
  uint32_t v[kPer], sum = 0;
#pragma unroll
  for (uint32_t k = 0; k < kPer; ++k) {
    v[k] = base + k < n_cells ? counts[base + k] : 0u;
    sum += v[k];
  }
  uint32_t run = tiles[blockIdx.x] + block_scan_excl<1024>(sum, &total);
#pragma unroll
  for (uint32_t k = 0; k < kPer; ++k) {
    if (base + k < n_cells) start[base + k] = run;
    run += v[k];
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) start[n_cells] = n;
}

__global__ void __launch_bounds__(256) k_static_scatter(const float4* __restrict__ in, uint32_t n, StaticGrid g,
                                                        uint32_t* __restrict__ counts,
                                                        const uint32_t* __restrict__ start,
                                                        float4* __restrict__ out) {
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
    const uint32_t i = base + threadIdx.x;
    float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
    uint32_t key = 0xFFFFFFFFu;
    if (i < n) {
      r = in[i];
      key = grid_key(g, r);
    }
    const uint32_t peers = __match_any_sync(kFull, key);
    const int leader = __ffs(peers) - 1;
    const uint32_t rank = __popc(peers & ((1u << (threadIdx.x & 31u)) - 1u));
    uint32_t old = 0;
    if (key != 0xFFFFFFFFu && (threadIdx.x & 31u) == (uint32_t)leader)
      old = atomicSub(&counts[key], (uint32_t)__popc(peers));
    old = __shfl_sync(kFull, old, leader);
    if (key != 0xFFFFFFFFu) {
      const uint32_t slot = start[key] + old - 1u - rank;
      if (slot < n) out[slot] = r;
    }
  }
}

// Canonical order inside each cell (x, y, z, w bits), in place: one thread
// per cell, selection sort; cells are disjoint, so threads never share data.
__global__ void __launch_bounds__(256) k_static_canon(float4* __restrict__ out, const uint32_t* __restrict__ start,
                                                      uint32_t n_cells) {
  for (uint32_t cell = blockIdx.x * blockDim.x + threadIdx.x; cell < n_cells; cell += gridDim.x * blockDim.x) {
    const uint32_t s = start[cell], e = start[cell + 1];
    for (uint32_t a = s; a + 1 < e; ++a) {
      uint32_t m = a;
      float4 best = out[a];
      for (uint32_t b = a + 1; b < e; ++b) {
        const float4 q = out[b];
        if (rec_less(q, best)) {
          best = q;
          m = b;
        }
      }
      if (m != a) {
        out[m] = out[a];
        out[a] = best;
      }
    }
  }
}

std::mutex g_addr_mutex;
uint32_t* g_addr[kMaxDevices] = {nullptr};

}  // namespace

// Cell sort of n records with all scratch in a file-scope device array; no
// cudaMalloc, cudaFree or allocating library call.  See the file comment
// and include/gpusmoldyn.h for the contract.
BD_API bd_status bd_cell_sort_static(const float* d_in, uint64_t n, const float box_lo[3], const float box_hi[3],
                                     const uint32_t dims[3], float* d_out, uint32_t* d_cell_start, void* stream) {
  if (!d_in || !d_out || !d_cell_start || !box_lo || !box_hi || !dims) return BD_ERR_INVALID_ARGUMENT;
  uint64_t n_cells = 1;
  for (int a = 0; a < 3; a++) {
    if (!(box_hi[a] > box_lo[a]) || dims[a] == 0) return BD_ERR_INVALID_ARGUMENT;
    n_cells *= dims[a];
  }
  // the fixed scratch bounds the grid; records are limited by 32-bit slots
  if (n_cells > kStaticMaxCells || n > 0x7FFFFFFFull) return BD_ERR_CAPACITY;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return BD_ERR_CUDA;
  uint32_t* scratch;
  {
    // first call on a device: look up the array's device address (host code
    // cannot use the symbol itself, which names a host-side stand-in)
    std::lock_guard<std::mutex> lock(g_addr_mutex);
    if (!g_addr[dev]) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_static_scratch) != cudaSuccess || !p) return BD_ERR_CUDA;
      g_addr[dev] = (uint32_t*)p;
    }
    scratch = g_addr[dev];
  }
  uint32_t* counts = scratch;
  uint32_t* tiles = scratch + kStaticMaxCells;
  StaticGrid g;
  for (int a = 0; a < 3; a++) {
    g.lo[a] = box_lo[a];
    g.dims[a] = dims[a];
    // the same float factor the simulation handle computes for its grid
    g.inv[a] = (float)dims[a] / (float)((double)box_hi[a] - (double)box_lo[a]);
  }
  g.n_cells = (uint32_t)n_cells;
  const uint32_t nc = (uint32_t)n_cells, nn = (uint32_t)n;
  const uint32_t n_tiles = (nc + kStaticTile - 1) / kStaticTile;
  cudaStream_t s = (cudaStream_t)stream;
  const float4* in = (const float4*)d_in;
  float4* out = (float4*)d_out;
  k_static_clear<<<(nc + 255) / 256 < 1024 ? (nc + 255) / 256 : 1024, 256, 0, s>>>(counts, nc);
  const int gs = nn ? (int)((nn + 255) / 256 < 4096 ? (nn + 255) / 256 : 4096) : 1;
  if (nn) k_static_count<<<gs, 256, 0, s>>>(in, nn, g, counts);
  k_static_scan_tiles<<<n_tiles, 1024, 0, s>>>(counts, nc, tiles);
  k_static_scan_top<<<1, 1024, 0, s>>>(tiles, n_tiles);
  k_static_scan_down<<<n_tiles, 1024, 0, s>>>(counts, nc, tiles, d_cell_start, nn);
  if (nn) k_static_scatter<<<gs, 256, 0, s>>>(in, nn, g, counts, d_cell_start, out);
  k_static_canon<<<(nc + 255) / 256 < 4096 ? (nc + 255) / 256 : 4096, 256, 0, s>>>(out, d_cell_start, nc);
  return cudaGetLastError() == cudaSuccess ? BD_OK : BD_ERR_CUDA;
}
