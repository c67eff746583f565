// bd_io.cu -- particles between the caller's arrays and the device state.
//
// The reference copies its float4 positions and int types with blocking
// cudaMemcpy (setArray / getArray, particleSystem.cpp:729-751) and packs
// nothing.  Here the caller's arrays (float4 x, y, z, w and int species per
// particle) travel whole, with one copy each; the checks, the packing into
// 16-byte records and the export of the live records in slot order run as
// kernels, so no host loop touches the particles.
#include <cuda_runtime.h>
#include <stdint.h>

#include "bd_io.h"

namespace bd {

namespace {

constexpr uint32_t kIoThreads = 1024, kIoTile = 4096;  // slots per export tile (4 per thread)
constexpr uint32_t kFull = 0xFFFFFFFFu;

// Instance of upload index i: the k with start[k] <= i < start[k + 1].
__device__ __forceinline__ int instance_of(const uint64_t* start, int n_inst, uint64_t i) {
  int lo = 0, hi = n_inst;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (start[mid] <= i) lo = mid;
    else hi = mid;
  }
  return lo;
}

__global__ void __launch_bounds__(256) k_upload_check(UploadArgs a) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride) {
    const int k = instance_of(a.start, a.n_inst, i);
    const float4 r = a.xyz4[i];
    const int s = a.species[i];
    const float* b = a.boxes + 6 * k;
    const bool ok = s >= 0 && s < a.n_species && r.x >= b[0] && r.x <= b[3] && r.y >= b[1] && r.y <= b[4] &&
                    r.z >= b[2] && r.z <= b[5];
    if (!ok) atomicOr(a.bad, 1u);
  }
}

__global__ void __launch_bounds__(256) k_upload_pack(UploadArgs a, float4* __restrict__ out) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride) {
    const float4 r = a.xyz4[i];
    const uint32_t w = ((a.inst_offset + (uint32_t)instance_of(a.start, a.n_inst, i)) << 16) | (uint32_t)a.species[i];
    out[i] = make_float4(r.x, r.y, r.z, __uint_as_float(w));
  }
}

__device__ __forceinline__ bool exported(const float4& r, int inst) {
  const uint32_t w = __float_as_uint(r.w);
  return w != 0xFFFFFFFFu && (inst < 0 || (int)(w >> 16) == inst);
}

// Exclusive scan of v over the 1024 threads of a block; *total receives the sum.
__device__ __forceinline__ uint32_t block_scan(uint32_t v, uint32_t* total) {
  __shared__ uint32_t s_warp[32];
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t t = __shfl_up_sync(kFull, x, d);
    if (lane >= (uint32_t)d) x += t;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t y = s_warp[lane];
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t t = __shfl_up_sync(kFull, y, d);
      if (lane >= (uint32_t)d) y += t;
    }
    s_warp[lane] = y;
  }
  __syncthreads();
  const uint32_t before = warp ? s_warp[warp - 1] : 0u;
  *total = s_warp[31];
  __syncthreads();
  return before + x - v;
}

__global__ void __launch_bounds__(kIoThreads) k_export_count(ExportArgs a) {
  uint32_t total;
  const uint64_t base = (uint64_t)blockIdx.x * kIoTile + (uint64_t)threadIdx.x * 4u;
  uint32_t c = 0;
#pragma unroll
  for (uint32_t k = 0; k < 4; ++k)
    if (base + k < a.n_slots && exported(a.state[base + k], a.inst)) ++c;
  block_scan(c, &total);
  if (threadIdx.x == 0) a.tile_offset[blockIdx.x] = total;
}

// Tile offsets in place (exclusive); *count receives the total.
__global__ void __launch_bounds__(kIoThreads) k_export_scan(ExportArgs a) {
  uint32_t carry = 0, total;
  for (uint32_t base = 0; base < a.n_tiles; base += kIoThreads) {
    const uint32_t t = base + threadIdx.x;
    const uint32_t v = t < a.n_tiles ? a.tile_offset[t] : 0u;
    const uint32_t ex = block_scan(v, &total);
    if (t < a.n_tiles) a.tile_offset[t] = carry + ex;
    carry += total;
  }
  if (threadIdx.x == 0) *a.count = carry;
}

__global__ void __launch_bounds__(kIoThreads) k_export_write(ExportArgs a) {
  uint32_t total;
  const uint64_t base = (uint64_t)blockIdx.x * kIoTile + (uint64_t)threadIdx.x * 4u;
  float4 r[4];
  uint32_t c = 0;
#pragma unroll
  for (uint32_t k = 0; k < 4; ++k) {
    r[k] = base + k < a.n_slots ? a.state[base + k] : make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(0xFFFFFFFFu));
    if (exported(r[k], a.inst)) ++c;
  }
  uint32_t o = a.tile_offset[blockIdx.x] + block_scan(c, &total);
#pragma unroll
  for (uint32_t k = 0; k < 4; ++k) {
    if (!exported(r[k], a.inst)) continue;
    a.xyz4[o] = make_float4(r[k].x, r[k].y, r[k].z, 1.0f);
    a.species[o] = (int)(__float_as_uint(r[k].w) & 0xFFFFu);
    ++o;
  }
}

int grid_for(uint64_t n) {
  const uint64_t g = (n + 255) / 256;
  return (int)(g < 1 ? 1 : (g > 152 * 16 ? 152 * 16 : g));
}

}  // namespace

void enqueue_upload_check(const UploadArgs& a, cudaStream_t s) {
  k_upload_check<<<grid_for(a.n), 256, 0, s>>>(a);
}

void enqueue_upload_pack(const UploadArgs& a, float4* out, cudaStream_t s) {
  k_upload_pack<<<grid_for(a.n), 256, 0, s>>>(a, out);
}

uint32_t export_tiles(uint64_t n_slots) { return (uint32_t)((n_slots + kIoTile - 1) / kIoTile); }

void enqueue_export(const ExportArgs& a, cudaStream_t s) {
  if (a.n_tiles == 0) {
    cudaMemsetAsync(a.count, 0, sizeof(uint32_t), s);
    return;
  }
  k_export_count<<<a.n_tiles, kIoThreads, 0, s>>>(a);
  k_export_scan<<<1, kIoThreads, 0, s>>>(a);
  k_export_write<<<a.n_tiles, kIoThreads, 0, s>>>(a);
}

}  // namespace bd
