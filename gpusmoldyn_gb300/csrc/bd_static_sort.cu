// bd_static_sort.cu -- the uniform-grid cell sort without any allocation.
//
// Some callers cannot call cudaMalloc: a host application that owns every
// byte of device memory and forbids its plugins to grow the footprint, or a
// time-critical loop where cudaMalloc's implicit device-wide
// synchronisation is not acceptable.  bd_cell_sort_static gives them the
// step's counting sort (cell histogram, exclusive scan, scatter, canonical
// order inside each cell) with its scratch -- the per-cell counts, the
// scan's tile sums and two control words -- in a file-scope device array of
// fixed size instead of buffers a handle allocates.  The caller passes the
// input records and the output buffers.
//
// The array holds kStaticMaxCells + kStaticMaxTiles + 2 32-bit words (about
// 4 MiB); every GPU that loads this library keeps it until the process
// exits.  All calls share it and it keeps the last call's contents, so each
// call clears the counts and control words it uses first, and calls whose
// work overlaps on the GPU (different streams, no ordering between them)
// race on it.
//
// Canonical order inside a cell costs a bounded amount of work whatever the
// cell holds: cells of up to kThreadCell records are ordered by one thread
// each; larger ("crowded") cells are listed and each is ordered by one
// thread block with a bitonic network -- in shared memory up to kChunk
// records, in place in the output above that (O(m log^2 m) for a cell of m
// records).
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "../../include/gpusmoldyn.h"
#include "bd_device.cuh"

namespace {

using bd::rec_less;

constexpr uint32_t kStaticMaxCells = 1u << 20;
constexpr uint32_t kStaticTile = 4096;
constexpr uint32_t kStaticMaxTiles = kStaticMaxCells / kStaticTile;
constexpr uint32_t kCtrlWords = 2;  // crowded-cell count, crowded-cell ticket
constexpr unsigned kFull = 0xFFFFFFFFu;
constexpr int kMaxDevices = 64;
constexpr uint32_t kThreadCell = 32;    // largest cell ordered by a single thread
constexpr uint32_t kChunk = 2048;       // records a block orders in shared memory (32 KiB)
constexpr int kCrowdThreads = 512;

// counts [0, kStaticMaxCells) -- after the scatter they are all zero again
// and the same words hold the list of crowded cells --, tile sums after
// them, then the control words
static __device__ __align__(256) uint32_t g_static_scratch[kStaticMaxCells + kStaticMaxTiles + kCtrlWords];

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

__global__ void k_static_clear(uint32_t* __restrict__ s, uint32_t n, uint32_t* __restrict__ ctrl) {
  if (blockIdx.x == 0 && threadIdx.x < kCtrlWords) ctrl[threadIdx.x] = 0u;
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

// Canonical order inside each cell (x, y, z, w bits), in place.  One thread
// per cell orders a cell of at most kThreadCell records by selection sort
// (at most 496 comparisons); a larger cell goes to the crowded list, which
// reuses the count words (all zero once the scatter has consumed them).
// Cells are disjoint, so threads never share records.
__global__ void __launch_bounds__(256) k_static_canon(float4* __restrict__ out, const uint32_t* __restrict__ start,
                                                      uint32_t n_cells, uint32_t* __restrict__ crowded,
                                                      uint32_t* __restrict__ n_crowded) {
  for (uint32_t cell = blockIdx.x * blockDim.x + threadIdx.x; cell < n_cells; cell += gridDim.x * blockDim.x) {
    const uint32_t s = start[cell], e = start[cell + 1];
    if (e - s > kThreadCell) {
      crowded[atomicAdd(n_crowded, 1u)] = cell;  // each cell once: fewer than n_cells entries
      continue;
    }
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

__device__ __forceinline__ float4 sentinel_rec() {
  const float m = __uint_as_float(0xFFFFFFFFu);  // no record compares above it
  return make_float4(m, m, m, m);
}

__device__ __forceinline__ void order_pair(float4& a, float4& b) {
  if (rec_less(b, a)) {
    const float4 t = a;
    a = b;
    b = t;
  }
}

// The bitonic network in its flip form (every compare-exchange puts the
// smaller record at the lower index; the first stage of each block size k
// pairs i with the mirror position in its block), so that positions past
// the cell's end act as records above every real one and pairs reaching
// them can be skipped.  half_cleaners runs the stages of distance j_max
// down to 1 on sh[0, p); block_sort runs the whole network on sh[0, p).
__device__ void half_cleaners(float4* sh, uint32_t p, uint32_t j_max) {
  for (uint32_t j = j_max; j >= 1; j >>= 1) {
    for (uint32_t t = threadIdx.x; t < p / 2; t += blockDim.x) {
      const uint32_t i = (t & ~(j - 1)) * 2 + (t & (j - 1));
      order_pair(sh[i], sh[i + j]);
    }
    __syncthreads();
  }
}

__device__ void block_sort(float4* sh, uint32_t p) {
  for (uint32_t k = 2; k <= p; k <<= 1) {
    const uint32_t half = k / 2;
    for (uint32_t t = threadIdx.x; t < p / 2; t += blockDim.x) {
      const uint32_t base = (t & ~(half - 1)) * 2, off = t & (half - 1);
      order_pair(sh[base + off], sh[base + k - 1 - off]);
    }
    __syncthreads();
    if (half > 1) half_cleaners(sh, p, half / 2);
  }
}

// rec[c, c + kChunk) <-> shared memory, positions at or past m as sentinels
__device__ void load_chunk(float4* sh, const float4* rec, uint64_t c, uint64_t m) {
  for (uint32_t i = threadIdx.x; i < kChunk; i += blockDim.x) sh[i] = c + i < m ? rec[c + i] : sentinel_rec();
  __syncthreads();
}
__device__ void store_chunk(const float4* sh, float4* rec, uint64_t c, uint64_t m) {
  for (uint32_t i = threadIdx.x; i < kChunk; i += blockDim.x)
    if (c + i < m) rec[c + i] = sh[i];
  __syncthreads();
}

// Crowded cells, one thread block each, taken from the list by a ticket.
// A cell of m <= kChunk records is ordered in shared memory.  A larger one
// is ordered in place: each kChunk run in shared memory, then for every
// block size k > kChunk the stages of distance >= kChunk in global memory
// and the rest in shared memory, run by run -- O(m log^2 m) work, no
// scratch beyond the block's shared memory.  The block's records are
// touched by no other block, so its barriers order every stage.
__global__ void __launch_bounds__(kCrowdThreads) k_static_canon_crowded(float4* out, const uint32_t* start,
                                                                        const uint32_t* crowded,
                                                                        const uint32_t* n_crowded,
                                                                        uint32_t* ticket) {
  __shared__ float4 sh[kChunk];
  __shared__ uint32_t job;
  const uint32_t n_jobs = *n_crowded;
  for (;;) {
    if (threadIdx.x == 0) job = atomicAdd(ticket, 1u);
    __syncthreads();
    const uint32_t jb = job;
    __syncthreads();
    if (jb >= n_jobs) return;
    const uint32_t cell = crowded[jb];
    const uint32_t s = start[cell];
    const uint64_t m = start[cell + 1] - s;
    float4* rec = out + s;
    if (m <= kChunk) {
      uint32_t p = 2;
      while (p < m) p <<= 1;
      for (uint32_t i = threadIdx.x; i < p; i += blockDim.x) sh[i] = i < m ? rec[i] : sentinel_rec();
      __syncthreads();
      block_sort(sh, p);
      for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) rec[i] = sh[i];
      __syncthreads();
      continue;
    }
    uint64_t P = kChunk;
    while (P < m) P <<= 1;
    for (uint64_t c = 0; c < m; c += kChunk) {
      load_chunk(sh, rec, c, m);
      block_sort(sh, kChunk);
      store_chunk(sh, rec, c, m);
    }
    for (uint64_t k = 2ull * kChunk; k <= P; k <<= 1) {
      const uint64_t half = k / 2;
      for (uint64_t t = threadIdx.x; t < P / 2; t += blockDim.x) {
        const uint64_t base = (t / half) * k, off = t % half;
        const uint64_t i = base + off, l = base + k - 1 - off;
        if (l < m) {
          float4 a = rec[i], b = rec[l];
          if (rec_less(b, a)) {
            rec[i] = b;
            rec[l] = a;
          }
        }
      }
      __syncthreads();
      for (uint64_t j = k / 4; j >= kChunk; j >>= 1) {
        for (uint64_t t = threadIdx.x; t < P / 2; t += blockDim.x) {
          const uint64_t i = (t / j) * 2 * j + t % j, l = i + j;
          if (l < m) {
            float4 a = rec[i], b = rec[l];
            if (rec_less(b, a)) {
              rec[i] = b;
              rec[l] = a;
            }
          }
        }
        __syncthreads();
      }
      for (uint64_t c = 0; c < m; c += kChunk) {
        load_chunk(sh, rec, c, m);
        half_cleaners(sh, kChunk, kChunk / 2);
        store_chunk(sh, rec, c, m);
      }
    }
  }
}

// Device address of the scratch array, per device, tagged with the driver
// context it was looked up in: a device reset (or another context on the
// same device) loads the module again at a new address, so a changed
// context id makes the next call look it up again.
struct ScratchSite {
  uint32_t* addr = nullptr;
  unsigned long long ctx_id = 0;
  int sms = 0;
};
std::mutex g_site_mutex;
ScratchSite g_site[kMaxDevices];

typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);
CtxGetCurrentFn g_ctx_current = nullptr;
CtxGetIdFn g_ctx_id = nullptr;
bool g_ctx_fns_tried = false;

// id of the current driver context (0 when none is current or the driver
// entry points are not available)
unsigned long long current_ctx_id() {
  if (!g_ctx_fns_tried) {
    g_ctx_fns_tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_ctx_current = (CtxGetCurrentFn)p;
    p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_ctx_id = (CtxGetIdFn)p;
  }
  if (!g_ctx_current || !g_ctx_id) return 0;
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (g_ctx_current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
  if (g_ctx_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

bool ranges_overlap(const void* a, uint64_t na, const void* b, uint64_t nb) {
  const uintptr_t x = (uintptr_t)a, y = (uintptr_t)b;
  return x < y + nb && y < x + na;
}

}  // namespace

// Cell sort of n records with all scratch in a file-scope device array; no
// cudaMalloc, cudaFree or allocating library call.  The contract is stated
// with the declaration in include/gpusmoldyn.h.
BD_API bd_status bd_cell_sort_static(const float* d_in, uint64_t n, const float box_lo[3], const float box_hi[3],
                                     const uint32_t dims[3], float* d_out, uint32_t* d_cell_start, void* stream) {
  if (!d_in || !d_out || !d_cell_start || !box_lo || !box_hi || !dims) return BD_ERR_INVALID_ARGUMENT;
  for (int a = 0; a < 3; a++)
    if (!(box_hi[a] > box_lo[a]) || dims[a] == 0) return BD_ERR_INVALID_ARGUMENT;
  // each axis is bounded before the product is formed, so the product
  // (below 2^60) cannot wrap past the bound
  for (int a = 0; a < 3; a++)
    if (dims[a] > kStaticMaxCells) return BD_ERR_CAPACITY;
  const uint64_t n_cells = (uint64_t)dims[0] * dims[1] * dims[2];
  // the fixed scratch bounds the grid; records are limited by 32-bit slots
  if (n_cells > kStaticMaxCells || n > 0x7FFFFFFFull) return BD_ERR_CAPACITY;
  // the kernels read d_in while they write d_out and d_cell_start
  const uint64_t rec_bytes = 16 * n, start_bytes = 4 * (n_cells + 1);
  if (ranges_overlap(d_in, rec_bytes, d_out, rec_bytes) || ranges_overlap(d_in, rec_bytes, d_cell_start, start_bytes) ||
      ranges_overlap(d_out, rec_bytes, d_cell_start, start_bytes))
    return BD_ERR_INVALID_ARGUMENT;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return BD_ERR_CUDA;
  uint32_t* scratch;
  int sms;
  {
    // set-up, once per device and driver context: look up the array's
    // device address (host code cannot use the symbol itself, which names a
    // host-side stand-in) with this device current
    std::lock_guard<std::mutex> lock(g_site_mutex);
    ScratchSite& site = g_site[dev];
    const unsigned long long id = current_ctx_id();
    if (!site.addr || id == 0 || id != site.ctx_id) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_static_scratch) != cudaSuccess || !p) return BD_ERR_CUDA;
      int nsm = 0;
      if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm <= 0)
        return BD_ERR_CUDA;
      site.addr = (uint32_t*)p;
      site.sms = nsm;
      site.ctx_id = current_ctx_id();  // the lookup made the device's context current
    }
    scratch = site.addr;
    sms = site.sms;
  }
  uint32_t* counts = scratch;
  uint32_t* tiles = scratch + kStaticMaxCells;
  uint32_t* ctrl = tiles + kStaticMaxTiles;  // [0] crowded cells, [1] ticket
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
  k_static_clear<<<(nc + 255) / 256 < 1024 ? (nc + 255) / 256 : 1024, 256, 0, s>>>(counts, nc, ctrl);
  const int gs = nn ? (int)((nn + 255) / 256 < 4096 ? (nn + 255) / 256 : 4096) : 1;
  if (nn) k_static_count<<<gs, 256, 0, s>>>(in, nn, g, counts);
  k_static_scan_tiles<<<n_tiles, 1024, 0, s>>>(counts, nc, tiles);
  k_static_scan_top<<<1, 1024, 0, s>>>(tiles, n_tiles);
  k_static_scan_down<<<n_tiles, 1024, 0, s>>>(counts, nc, tiles, d_cell_start, nn);
  if (nn) {
    k_static_scatter<<<gs, 256, 0, s>>>(in, nn, g, counts, d_cell_start, out);
    k_static_canon<<<(nc + 255) / 256 < 4096 ? (nc + 255) / 256 : 4096, 256, 0, s>>>(out, d_cell_start, nc, counts,
                                                                                       ctrl);
    k_static_canon_crowded<<<2 * sms, kCrowdThreads, 0, s>>>(out, d_cell_start, counts, ctrl, ctrl + 1);
  }
  return cudaGetLastError() == cudaSuccess ? BD_OK : BD_ERR_CUDA;
}
