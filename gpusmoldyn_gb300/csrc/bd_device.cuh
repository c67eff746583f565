// bd_device.cuh -- per-particle arithmetic of the Brownian-dynamics step.
//
// Every floating-point operation whose result decides a cell, a pair or a
// reaction is written with an explicitly rounded intrinsic (__fmaf_rn,
// __fmul_rn, __fadd_rn, __fsqrt_rn), so the compiler cannot contract or
// reorder it and a CPU program that performs the same IEEE operations gets
// the same bits.  Only the production normal generator (Box-Muller with
// the hardware approximations __logf / __sincosf) is not bit-reproducible
// on a CPU; the table mode is.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "bd_layout.h"

namespace bd {

struct U4 {
  uint32_t x, y, z, w;
};

// Philox4x32-10 (J. K. Salmon, M. A. Moraes, R. O. Dror, D. E. Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC'11): 10 rounds of two
// 32x32->64 multiplies with a Weyl-sequence key schedule.  Stateless: the
// counter (particle, step, stream tag, partner) replaces the reference's
// 32768 shared Mersenne-Twister states (MersenneTwister.cuh:40-91,
// particles_kernel.cu:140-141), whose read-modify-write raced between
// threads i and i + 32768.
__device__ __forceinline__ U4 philox(U4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    // one 32x32->64 multiply each (IMAD.WIDE) gives both halves
    const uint64_t p0 = (uint64_t)0xD2511F53u * c.x;
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c.z;
    c = U4{(uint32_t)(p1 >> 32) ^ c.y ^ k0, (uint32_t)p1, (uint32_t)(p0 >> 32) ^ c.w ^ k1, (uint32_t)p0};
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

// The reference's randReal: a 32-bit word scaled by 2^-32 in float
// (rand_kernel.cuh:32-36).  May round to 1.0f, which no coin accepts.
__device__ __forceinline__ float u32_to_unit(uint32_t v) {
  return __fmul_rn(__uint2float_rn(v), 2.3283064365386963e-10f);
}

// 24-bit uniform in [0, 1).
__device__ __forceinline__ float u24_to_unit(uint32_t v) {
  return __fmul_rn(__uint2float_rn(v >> 8), 5.9604644775390625e-08f);
}

// 53-bit uniform in [0, 1) from two words (Poisson inversion).
__device__ __forceinline__ double u53_to_unit(uint32_t a, uint32_t b) {
  const uint64_t m = ((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6);
  return (double)m * 1.1102230246251565e-16;
}

// Three standard normals from words x, y, z of one Philox block; word w is
// left for the first first-order coin.
// Table mode: the top 12 bits of x, y, z index the 4096 quantiles of
// N(0,1) (the reference's gaussianLookupTable, particles_kernel.cu:156-162).
// Box-Muller mode (G. E. P. Box and M. E. Muller, Ann. Math. Stat. 29:610,
// 1958): two pairs of 24-bit uniforms give four normals, three are used;
// the fourth uniform is made of the low bytes of x, y, z.
template <bool kTable>
__device__ __forceinline__ void normals3(const U4& r, const float* __restrict__ table, float& g0,
                                         float& g1, float& g2) {
  if (kTable) {
    g0 = table[r.x >> 20];
    g1 = table[r.y >> 20];
    g2 = table[r.z >> 20];
  } else {
    // hardware approximations (MUFU lg2 / rsqrt / sin / cos): absolute
    // errors ~1e-6, far below the statistical resolution of the step
    const float a = u24_to_unit(r.x) + 2.98023223876953125e-08f;  // (0, 1)
    const float c = u24_to_unit(r.z) + 2.98023223876953125e-08f;
    // __logf may round to 0 just below 1: keep the radius finite (0)
    const float la = fmaxf(-2.0f * __logf(a), 1e-30f), lc = fmaxf(-2.0f * __logf(c), 1e-30f);
    const float ra = la * rsqrtf(la);
    const float rc = lc * rsqrtf(lc);
    float sa, ca, sc, cc;
    __sincosf(6.2831853071795865f * u24_to_unit(r.y), &sa, &ca);
    const uint32_t low = ((r.x & 0xFFu) << 24) | ((r.y & 0xFFu) << 16) | ((r.z & 0xFFu) << 8);
    __sincosf(6.2831853071795865f * u24_to_unit(low), &sc, &cc);
    g0 = ra * ca;
    g1 = ra * sa;
    g2 = rc * cc;
  }
}

// Uniform random unit vector (G. Marsaglia, "Choosing a point from the
// surface of a sphere", Ann. Math. Stat. 43:645, 1972): rejection from the
// unit disk, then (2u sqrt(1-s), 2v sqrt(1-s), 1-2s).  Only correctly
// rounded operations, so the result is bit-identical on any IEEE machine.
// Replaces the rotation DirCosM(acos(1-2u), 2 pi u, 2 pi u) applied to an
// x-axis offset (reaction_kernel.cuh:177-200, 249-257), which has the same
// distribution.  At most 8 Philox blocks (16 tries); the 2^-34 case where
// all fail returns +z.
__device__ __forceinline__ void unit_vector(uint32_t c0, uint32_t c1, uint32_t tag, uint32_t c3,
                                            uint32_t k0, uint32_t k1, float& dx, float& dy,
                                            float& dz) {
  for (uint32_t a = 0; a < 8; ++a) {
    const U4 r = philox(U4{c0, c1, tag | a, c3}, k0, k1);
    const uint32_t w[4] = {r.x, r.y, r.z, r.w};
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const float u = __fsub_rn(__fmul_rn(__uint2float_rn(w[2 * h] >> 8), 1.1920928955078125e-07f), 1.0f);
      const float v = __fsub_rn(__fmul_rn(__uint2float_rn(w[2 * h + 1] >> 8), 1.1920928955078125e-07f), 1.0f);
      const float s = __fadd_rn(__fmul_rn(u, u), __fmul_rn(v, v));
      if (s < 1.0f && s > 0.0f) {
        const float q = __fmul_rn(2.0f, __fsqrt_rn(__fsub_rn(1.0f, s)));
        dx = __fmul_rn(u, q);
        dy = __fmul_rn(v, q);
        dz = __fsub_rn(1.0f, __fmul_rn(2.0f, s));
        return;
      }
    }
  }
  dx = 0.0f;
  dy = 0.0f;
  dz = 1.0f;
}

// Specular reflection into [lo, hi] (x -> 2 hi - x, x -> 2 lo - x), repeated
// for steps longer than the box, then clamped.  Replaces the clamp to
// [-1 + r, 1 - r] of adjustPositions (particles_kernel.cu:61-95).
__device__ __forceinline__ float reflect(float x, float lo, float hi) {
  // the common case, inside the box, with one test and no loop (k_bin
  // 0.2305 -> 0.2270 ms on the 16M c3 step); the loop returns x unchanged
  // there too
  if (x >= lo && x <= hi) return x;
#pragma unroll 1
  for (int k = 0; k < 8; ++k) {
    if (x > hi) {
      x = __fsub_rn(__fmul_rn(2.0f, hi), x);
    } else if (x < lo) {
      x = __fsub_rn(__fmul_rn(2.0f, lo), x);
    } else {
      return x;
    }
  }
  return fminf(fmaxf(x, lo), hi);
}

// Cell coordinate along one axis, clamped to the grid (the reference wraps
// with & (gridSize-1), particles_kernel.cu:170-186; walls make the grid
// non-periodic here).
__device__ __forceinline__ int cell_coord(float x, float lo, float inv, uint32_t n) {
  const float f = __fmul_rn(__fsub_rn(x, lo), inv);
  int c = (int)floorf(f);
  c = c < 0 ? 0 : c;
  c = c > (int)n - 1 ? (int)n - 1 : c;
  return c;
}

__device__ __forceinline__ uint32_t cell_key(const DevInstance& I, float x, float y, float z) {
  const int cx = cell_coord(x, I.lo[0], I.inv[0], I.dims[0]);
  const int cy = cell_coord(y, I.lo[1], I.inv[1], I.dims[1]);
  const int cz = cell_coord(z, I.lo[2], I.inv[2], I.dims[2]);
  return I.cell_base + ((uint32_t)cz * I.dims[1] + (uint32_t)cy) * I.dims[0] + (uint32_t)cx;
}

__device__ __forceinline__ uint32_t rec_w(const float4& r) { return __float_as_uint(r.w); }
__device__ __forceinline__ uint32_t pack_w(uint32_t inst, uint32_t species) {
  return (inst << 16) | (species & 0xFFFFu);
}

// Canonical order of records that share a cell: x, y, z and w compared as
// unsigned words.  Records equal in all four words are indistinguishable,
// so any order among them gives the same array.
__device__ __forceinline__ bool rec_less(const float4& a, const float4& b) {
  const uint32_t ax = __float_as_uint(a.x), bx = __float_as_uint(b.x);
  if (ax != bx) return ax < bx;
  const uint32_t ay = __float_as_uint(a.y), by = __float_as_uint(b.y);
  if (ay != by) return ay < by;
  const uint32_t az = __float_as_uint(a.z), bz = __float_as_uint(b.z);
  if (az != bz) return az < bz;
  return __float_as_uint(a.w) < __float_as_uint(b.w);
}
__device__ __forceinline__ bool rec_equal(const float4& a, const float4& b) {
  return __float_as_uint(a.x) == __float_as_uint(b.x) && __float_as_uint(a.y) == __float_as_uint(b.y) &&
         __float_as_uint(a.z) == __float_as_uint(b.z) && __float_as_uint(a.w) == __float_as_uint(b.w);
}

}  // namespace bd
