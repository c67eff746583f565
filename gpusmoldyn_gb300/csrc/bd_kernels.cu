// bd_kernels.cu -- the per-timestep kernels of the Brownian-dynamics step.
//
// Sorted path (any first- or second-order reaction, or an ensemble), one
// step = 7 or 8 launches, no host synchronisation, all counts on the device:
//
//   k_zeroth    1 CTA      Poisson birth counts of the zeroth-order reactions
//                          (zeroReact + poisrandF on the host in the
//                          reference, reaction_cpu.cpp:36-63, stats.cpp:234-275)
//   k_count     streaming  diffuse + reflect + first-order reactions + cell key,
//                          warp-aggregated cell histogram; writes nothing else
//                          (diffuse, uniReact, adjustPositions, calcHashD:
//                          particles_kernel.cu:61-95, 127-207,
//                          reaction_kernel.cuh:263-342)
//   k_scan_*    3 launches exclusive scan of the cell histogram = cell starts
//                          (replaces RadixSort's 5 passes + CUDPP scans,
//                          radixsort.cu:1045-1143, and the cellStart memset)
//   k_scatter   streaming  recomputes k_count's records (counter-based RNG makes
//                          them identical) and scatters each into its cell;
//                          dead particles get no slot, births get one
//                          (compactPosAndTypeD, particles_kernel.cu:98-123)
//   k_pairs     streaming  canonical order inside each cell + pair search over
//                          the neighbour cells within the binding radius
//                          (reorderDataAndFindCellStartD, collideD, collideCell:
//                          particles_kernel.cu:212-272, 318-497)
//   k_match     1 CTA      one reaction per particle (greedy matching in pair
//                          order), product placement, counters, commit
//                          (bimReact, resetNonInteracting: reaction_kernel.cuh:
//                          202-258, particles_kernel.cu:499-508)
//
// HBM traffic per particle-step: k_count R16, k_scatter R16 + W16, k_pairs
// R16 + W16 = 80 B, plus 4-12 B per cell for the histogram and the starts.
//
// Diffusion-only path (no first- or second-order reaction, one instance):
// k_diffuse updates the records in place (R16 + W16) and zeroth-order births
// are appended by k_append.
#include "bd_device.cuh"
#include "bd_kernels.h"
#include "bd_surface.cuh"

namespace bd {
namespace {

constexpr uint32_t kNoKey = 0xFFFFFFFFu;
constexpr unsigned long long kFree64 = ~0ull;  // matcher word of a record not in a pending pair
constexpr unsigned kFull = 0xFFFFFFFFu;

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

__device__ __forceinline__ uint32_t ld_u32(const uint32_t* p) { return __ldcg(p); }

// ctrl words are written by earlier kernels and read here through L2.
__device__ __forceinline__ uint32_t ctrl_status_warp(const DevCtrl* c) {
  uint32_t s = 0;
  if (lane_id() == 0) s = ld_u32(&c->status);
  return __shfl_sync(kFull, s, 0);
}

// Grid-stride loop over the records [0, n_total) of the step: body(i, rec)
// with rec the current record for i < n_real (indices from n_real on are the
// step's zeroth-order births).  The next iteration's record is loaded before
// the body runs, so each thread keeps two 16-byte loads in flight.  Every
// thread of a warp makes the same number of calls (warp collectives allowed).
template <class Body>
__device__ __forceinline__ void stream_records(const float4* __restrict__ st, uint32_t n_real, uint32_t n_total,
                                               Body&& body) {
  const uint32_t stride = gridDim.x * blockDim.x;
  uint32_t base = blockIdx.x * blockDim.x;
  const float4 none = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  float4 next = base + threadIdx.x < n_real ? __ldcs(&st[base + threadIdx.x]) : none;
  for (; base < n_total; base += stride) {
    const uint32_t i = base + threadIdx.x;
    const float4 rec = next;
    const uint32_t ahead = i + stride;
    next = ahead < n_real && ahead > i ? __ldcs(&st[ahead]) : none;
    // and the record after that towards L2
    const uint32_t far = ahead + stride;
    if (far < n_real && far > ahead) asm volatile("prefetch.global.L2 [%0];" ::"l"(st + far));
    body(i, rec);
  }
}

__device__ __forceinline__ const float4* cur_state(const KParams& p, uint32_t cur) {
  return cur ? p.state[1] : p.state[0];
}
__device__ __forceinline__ float4* next_state(const KParams& p, uint32_t cur) {
  return cur ? p.state[0] : p.state[1];
}

// An instance advances when it is active, not frozen and not removed.
__device__ __forceinline__ bool advancing(uint32_t flags) {
  return (flags & kInstActive) && !(flags & (kInstFrozen | kInstRemoved));
}

// Commit one step (global index `step`) of an instance; it freezes when it
// reaches its target, so a request never runs past the step count it asked
// for, and the step it froze at is kept (inst_frozen: the state is in
// canonical order again after one more step).
__device__ __forceinline__ void advance_instance_step(const KParams& p, uint32_t inst, uint32_t step) {
  const uint32_t f = p.inst_flags[inst];
  if (!advancing(f)) return;
  const uint32_t s = p.inst_step[inst] + 1;
  p.inst_step[inst] = s;
  if (s >= p.inst_target[inst]) {
    p.inst_flags[inst] = f | kInstFrozen;
    p.inst_frozen[inst] = step;
  }
}

struct Out2 {
  float4 r[2];
  uint32_t key[2];
  int n;
};

__device__ __forceinline__ uint32_t word_of(const U4& c, uint32_t k) {
  switch (k & 3u) {
    case 0: return c.x;
    case 1: return c.y;
    case 2: return c.z;
    default: return c.w;
  }
}

// Instance parameters.  kSingle (a handle with one instance) reads the copy
// in the kernel parameters, which the compiler folds into constant-bank
// operands; ensembles read the instance table in global memory.
template <bool kSingle>
__device__ __forceinline__ const DevInstance& inst_of(const KParams& p, uint32_t inst) {
  if (kSingle) return p.inst0;
  return p.inst[inst];
}

// What every record of a one-instance handle reads, loaded once per CTA:
// the instance's flags, step and first slot in registers, its species and
// first-order tables in shared memory (at most kCtxSpecies / kCtxUni
// entries; larger networks run the generic kernels).
constexpr uint32_t kCtxSpecies = 64, kCtxUni = 64;
struct SingleCtx {
  uint32_t flags, step, slot_base;
  const DevSpecies* species;
  const DevUni* uni;
};

// Fills the shared tables (all threads of the CTA call it; one barrier).
__device__ __forceinline__ SingleCtx single_ctx(const KParams& p, DevSpecies* s_species, DevUni* s_uni) {
  for (uint32_t t = threadIdx.x; t < p.S; t += blockDim.x) s_species[t] = p.species[t];
  for (uint32_t t = threadIdx.x; t < p.U; t += blockDim.x) s_uni[t] = p.uni[t];
  __syncthreads();
  return SingleCtx{ld_u32(&p.inst_flags[0]), ld_u32(&p.inst_step[0]), ld_u32(&p.inst_slot_base[0]), s_species,
                   s_uni};
}

// Advance the record in slot i by one step: diffusion, reflection and the
// first successful first-order reaction (reaction_kernel.cuh:303-341: coins
// in list order, decay when the first product is absent, a second product
// becomes a birth).  kCount adds fired reactions to the event counters.
// The surface walk of a move from x0 to (x, y, z), a point the walls have
// already reflected into the box: the chord stays inside the box, so a panel
// that reaches a wall cannot be passed by way of the wall.  A reflection off
// a panel can leave the box, so the walls reflect the end once more.
// False = absorbed.
__device__ __forceinline__ bool surface_walk(const KParams& p, const DevInstance& I, uint32_t sp, const V3& x0,
                                             float& x, float& y, float& z) {
  V3 e{x, y, z};
  if (!surface_move(surf_view(p), sp, x0, e)) return false;
  x = reflect(e.x, I.lo[0], I.hi[0]);
  y = reflect(e.y, I.lo[1], I.hi[1]);
  z = reflect(e.z, I.lo[2], I.hi[2]);
  return true;
}

// kSurf = 1 walks each displacement (the diffusion step, product offsets)
// through the surface panels.  kSurf = 2 looks up the species mask of the
// cell where the step starts (cell_surf): a set bit means a panel the
// species sees lies within reach of the step or of the products it may
// place, and the record stops after its diffusion with o.n = -1 so that
// the caller queues it for a walk (k_bin_surface); other records finish
// here, and no panel could have changed their step.
template <bool kTable, bool kCount, bool kSingle, int kSurf = 0>
__device__ __forceinline__ void advance_rec(const KParams& p, const SingleCtx& ctx, const float4 rec, uint32_t i,
                                            Out2& o) {
  o.n = 0;
  const uint32_t w = rec_w(rec);
  if (w == kDead) return;
  const uint32_t inst = w >> 16, sp = w & kSpeciesMask;
  const DevInstance& I = inst_of<kSingle>(p, inst);
  const uint32_t flags = kSingle ? ctx.flags : p.inst_flags[inst];
  if (flags & kInstRemoved) return;
  if ((flags & kInstFrozen) || !(flags & kInstActive)) {
    o.r[0] = rec;
    o.key[0] = cell_key(I, rec.x, rec.y, rec.z);
    o.n = 1;
    return;
  }
  const uint32_t local = i - (kSingle ? ctx.slot_base : p.inst_slot_base[inst]);
  const uint32_t t = kSingle ? ctx.step : p.inst_step[inst];
  const uint32_t k0 = I.key_lo, k1 = I.key_hi;
  const DevSpecies S = kSingle ? ctx.species[sp] : p.species[I.block * p.S + sp];
  // the species mask of the cell the step starts in, loaded before the
  // arithmetic that hides its latency
  const uint32_t near = kSurf == 2 ? __ldg(&p.cell_surf[cell_key(I, rec.x, rec.y, rec.z)]) : 0u;

  const U4 rn = philox(U4{local, t, kTagDiffuse, 0u}, k0, k1);
  float g0, g1, g2;
  normals3<kTable>(rn, p.gauss, g0, g1, g2);
  float x = reflect(__fmaf_rn(S.sigma, g0, rec.x), I.lo[0], I.hi[0]);
  float y = reflect(__fmaf_rn(S.sigma, g1, rec.y), I.lo[1], I.hi[1]);
  float z = reflect(__fmaf_rn(S.sigma, g2, rec.z), I.lo[2], I.hi[2]);
  if (kSurf == 2 && ((near >> (sp < 7u ? sp : 7u)) & 1u)) {
    o.n = -1;
    return;
  }
  if (kSurf == 1 && !surface_walk(p, I, sp, V3{rec.x, rec.y, rec.z}, x, y, z)) return;  // absorbed
  uint32_t species = sp;
  int n = 1;

  // coin 0 is the diffusion block's spare word; coins 1.. come 4 per block
  U4 coins = rn;
  for (uint32_t k = 0; k < S.uni_count; ++k) {
    if (k > 0 && ((k - 1) & 3u) == 0) coins = philox(U4{local, t, kTagUniCoin | ((k - 1) >> 2), 0u}, k0, k1);
    const DevUni& u = kSingle ? ctx.uni[S.uni_begin + k] : p.uni[I.block * p.U + S.uni_begin + k];
    if (u32_to_unit(k == 0 ? rn.w : word_of(coins, k - 1)) < u.prob) {
      if (kCount) atomicAdd(&p.pending[(size_t)inst * p.R + u.rxn], 1ull);
      if (u.prod0 < 0) return;  // decay: no record
      species = (uint32_t)u.prod0;
      if (u.prod1 >= 0) {
        float bx = x, by = y, bz = z;
        bool keep0 = true, keep1 = true;
        if (u.off0 != 0.0f || u.off1 != 0.0f) {
          float dx, dy, dz;
          unit_vector(local, t, kTagUniDir, 0u, k0, k1, dx, dy, dz);
          bx = reflect(__fmaf_rn(u.off1, dx, x), I.lo[0], I.hi[0]);
          by = reflect(__fmaf_rn(u.off1, dy, y), I.lo[1], I.hi[1]);
          bz = reflect(__fmaf_rn(u.off1, dz, z), I.lo[2], I.hi[2]);
          const V3 from{x, y, z};
          x = reflect(__fmaf_rn(u.off0, dx, x), I.lo[0], I.hi[0]);
          y = reflect(__fmaf_rn(u.off0, dy, y), I.lo[1], I.hi[1]);
          z = reflect(__fmaf_rn(u.off0, dz, z), I.lo[2], I.hi[2]);
          if (kSurf == 1) {
            // both products move from the reaction point
            keep1 = surface_walk(p, I, (uint32_t)u.prod1, from, bx, by, bz);
            keep0 = surface_walk(p, I, (uint32_t)u.prod0, from, x, y, z);
          }
        }
        const float4 born = make_float4(bx, by, bz, __uint_as_float(pack_w(inst, (uint32_t)u.prod1) | kNewborn));
        if (kSurf == 1 && !keep0) {  // the first product was absorbed: the birth takes its place
          if (!keep1) return;
          o.r[0] = born;
          o.key[0] = cell_key(I, bx, by, bz);
          o.n = 1;
          return;
        }
        o.r[1] = born;
        o.key[1] = cell_key(I, bx, by, bz);
        n = (kSurf == 1 && !keep1) ? 1 : 2;
      }
      break;
    }
  }
  o.r[0] = make_float4(x, y, z, __uint_as_float(pack_w(inst, species)));
  o.key[0] = cell_key(I, x, y, z);
  o.n = n;
}

// Zeroth-order birth number v of this step: uniform position in the box
// (reaction_cpu.cpp:44-60 with randPos, particleSystem.h:115-120).
template <bool kSingle>
__device__ __forceinline__ void advance_virtual(const KParams& p, uint32_t v, Out2& o) {
  const uint32_t nz = p.n_inst * p.Z;
  // entry e with zero_off[e] <= v < zero_off[e + 1]
  uint32_t lo = 0, hi = nz;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (p.zero_off[mid] <= v) lo = mid;
    else hi = mid;
  }
  const uint32_t inst = lo / p.Z, zr = lo % p.Z;
  const uint32_t k_local = v - p.zero_off[inst * p.Z];
  const DevInstance& I = inst_of<kSingle>(p, inst);
  const uint32_t t = p.inst_step[inst];
  const U4 r = philox(U4{k_local, t, kTagZeroPos, 0u}, I.key_lo, I.key_hi);
  const float x = fminf(__fmaf_rn(u24_to_unit(r.x), __fsub_rn(I.hi[0], I.lo[0]), I.lo[0]), I.hi[0]);
  const float y = fminf(__fmaf_rn(u24_to_unit(r.y), __fsub_rn(I.hi[1], I.lo[1]), I.lo[1]), I.hi[1]);
  const float z = fminf(__fmaf_rn(u24_to_unit(r.z), __fsub_rn(I.hi[2], I.lo[2]), I.lo[2]), I.hi[2]);
  const DevZero& Zr = p.zero[I.block * p.Z + zr];
  const uint32_t key = cell_key(I, x, y, z);
  o.r[0] = make_float4(x, y, z, __uint_as_float(pack_w(inst, (uint32_t)Zr.prod0) | kNewborn));
  o.key[0] = key;
  o.n = 1;
  if (Zr.prod1 >= 0) {
    o.r[1] = make_float4(x, y, z, __uint_as_float(pack_w(inst, (uint32_t)Zr.prod1) | kNewborn));
    o.key[1] = key;
    o.n = 2;
  }
}

// Lanes with equal keys add their count with one atomic.
__device__ __forceinline__ void warp_count(uint32_t* cnt, uint32_t key) {
  const uint32_t peers = __match_any_sync(kFull, key);
  if (key != kNoKey && lane_id() == (uint32_t)(__ffs(peers) - 1)) atomicAdd(&cnt[key], (uint32_t)__popc(peers));
}

// Lanes with equal keys take consecutive places of their cell with one
// atomic; the count goes back to zero as the cell fills.
__device__ __forceinline__ uint32_t warp_claim(uint32_t* cnt, uint32_t key) {
  const uint32_t peers = __match_any_sync(kFull, key);
  const int leader = __ffs(peers) - 1;
  const uint32_t rank = __popc(peers & ((1u << lane_id()) - 1u));
  uint32_t old = 0;
  if (key != kNoKey && lane_id() == (uint32_t)leader) old = atomicSub(&cnt[key], (uint32_t)__popc(peers));
  old = __shfl_sync(kFull, old, leader);
  return old - 1u - rank;
}

template <int kThreads>
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total) {
  __shared__ uint32_t warp_sums[kThreads / 32];
  const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
  uint32_t incl = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t n = __shfl_up_sync(kFull, incl, d);
    if (lane >= (uint32_t)d) incl += n;
  }
  if (lane == 31) warp_sums[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t s = lane < kThreads / 32 ? warp_sums[lane] : 0u;
    uint32_t si = s;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t n = __shfl_up_sync(kFull, si, d);
      if (lane >= (uint32_t)d) si += n;
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

// ---------------------------------------------------------------- kernels

// Fields of entry g (< 4) of KParams::zero0, read at fixed offsets.
__device__ __forceinline__ void zero0_entry(const KParams& p, uint32_t g, uint32_t& off, uint32_t& len,
                                            int32_t& kmin, uint32_t& rxn) {
  off = p.zero0[0].cdf_off, len = p.zero0[0].cdf_len, kmin = p.zero0[0].kmin, rxn = p.zero0[0].rxn;
#pragma unroll
  for (uint32_t z = 1; z < 4; ++z)
    if (g == z) off = p.zero0[z].cdf_off, len = p.zero0[z].cdf_len, kmin = p.zero0[z].kmin, rxn = p.zero0[z].rxn;
}

__global__ void __launch_bounds__(1024) k_zeroth(KParams p, int check_append) {
  __shared__ uint32_t s_total;
  DevCtrl* c = p.ctrl;
  const uint32_t nz = p.n_inst * p.Z;
  if (p.n_inst == 1 && nz <= 4u) {
    // One instance, at most four reactions: the entries come from the
    // kernel parameters and the status, step and flags are loaded
    // together, so the counts wait on one round of global loads (the
    // CDFs) instead of a chain of four.  Counting as below.
    __shared__ uint32_t s_part[32], s_cnt[4];
    const uint32_t status = ld_u32(&c->status), step = p.inst_step[0];
    const bool adv = advancing(p.inst_flags[0]);
    const uint32_t G = nz > 2u ? 256u : (nz > 1u ? 512u : 1024u);  // threads per entry
    const uint32_t g = threadIdx.x / G, t = threadIdx.x % G;
    uint32_t off, len, rxn;
    int32_t kmin;
    uint32_t le = 0;
    if (g < nz && adv) {
      zero0_entry(p, g, off, len, kmin, rxn);
      const U4 r = philox(U4{g, step, kTagZeroCount, 0u}, p.inst0.key_lo, p.inst0.key_hi);
      const double u = u53_to_unit(r.x, r.y);
      const double* cdf = p.cdf + off;
      for (uint32_t k = t; k < len; k += G) le += cdf[k] <= u ? 1u : 0u;
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) le += __shfl_xor_sync(kFull, le, d);
    if ((threadIdx.x & 31u) == 0) s_part[threadIdx.x >> 5] = le;
    __syncthreads();
    if (threadIdx.x < nz) {
      uint32_t cnt = 0;
      if (adv) {
        zero0_entry(p, threadIdx.x, off, len, kmin, rxn);
        uint32_t below = 0;
        for (uint32_t w = 0; w < G / 32u; ++w) below += s_part[threadIdx.x * (G / 32u) + w];
        cnt = (uint32_t)kmin + min(below, len - 1u);
        if (cnt && !status) atomicAdd(&p.pending[rxn], (unsigned long long)cnt);
      }
      s_cnt[threadIdx.x] = cnt;
    }
    __syncthreads();
    if (threadIdx.x == 0 && !status) {
      uint32_t carry = 0;
      for (uint32_t e = 0; e < nz; ++e) {
        p.zero_off[e] = carry;
        carry += s_cnt[e];
      }
      p.zero_off[nz] = carry;
      c->n_virtual = carry;
      if (check_append && (uint64_t)c->n_slots + carry > p.capacity) atomicOr(&c->status, kStatCapacity);
    }
    return;
  }
  if (ld_u32(&c->status)) return;
  if (nz <= 32u) {
    // Few entries (one instance, a few reactions): a group of at least 32
    // threads per entry counts the CDF values at or below u.  The CDF does
    // not decrease, so that count is the smallest k with CDF(k) > u, the
    // index the binary search below finds, and its loads are all in flight
    // at once instead of one dependent load per halving.
    __shared__ uint32_t s_part[32], s_cnt[32];
    uint32_t groups = 1;
    while (groups < nz) groups <<= 1;
    const uint32_t G = 1024u / groups;  // threads per entry, a multiple of 32
    const uint32_t g = threadIdx.x / G, t = threadIdx.x % G;
    uint32_t le = 0;
    if (g < nz) {
      const uint32_t inst = g / p.Z, zr = g % p.Z;
      const DevInstance& I = p.inst[inst];
      if (advancing(p.inst_flags[inst])) {
        const DevZero& Zr = p.zero[I.block * p.Z + zr];
        const U4 r = philox(U4{zr, p.inst_step[inst], kTagZeroCount, 0u}, I.key_lo, I.key_hi);
        const double u = u53_to_unit(r.x, r.y);
        const double* cdf = p.cdf + Zr.cdf_off;
        for (uint32_t k = t; k < Zr.cdf_len; k += G) le += cdf[k] <= u ? 1u : 0u;
      }
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) le += __shfl_xor_sync(kFull, le, d);
    if ((threadIdx.x & 31u) == 0) s_part[threadIdx.x >> 5] = le;
    __syncthreads();
    if (threadIdx.x < nz) {
      const uint32_t e = threadIdx.x, inst = e / p.Z, zr = e % p.Z;
      const DevInstance& I = p.inst[inst];
      uint32_t cnt = 0;
      if (advancing(p.inst_flags[inst])) {
        const DevZero& Zr = p.zero[I.block * p.Z + zr];
        uint32_t below = 0;
        for (uint32_t w = 0; w < G / 32u; ++w) below += s_part[e * (G / 32u) + w];
        cnt = (uint32_t)Zr.kmin + min(below, Zr.cdf_len - 1u);
        if (cnt) atomicAdd(&p.pending[(size_t)inst * p.R + Zr.rxn], (unsigned long long)cnt);
      }
      s_cnt[e] = cnt;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      uint32_t carry = 0;
      for (uint32_t e = 0; e < nz; ++e) {
        p.zero_off[e] = carry;
        carry += s_cnt[e];
      }
      p.zero_off[nz] = carry;
      c->n_virtual = carry;
      if (check_append && (uint64_t)c->n_slots + carry > p.capacity) atomicOr(&c->status, kStatCapacity);
    }
    return;
  }
  uint32_t carry = 0;
  for (uint32_t base = 0; base < nz; base += 1024) {
    const uint32_t e = base + threadIdx.x;
    uint32_t cnt = 0;
    if (e < nz) {
      const uint32_t inst = e / p.Z, zr = e % p.Z;
      const DevInstance& I = p.inst[inst];
      if (advancing(p.inst_flags[inst])) {
        const DevZero& Zr = p.zero[I.block * p.Z + zr];
        const U4 r = philox(U4{zr, p.inst_step[inst], kTagZeroCount, 0u}, I.key_lo, I.key_hi);
        const double u = u53_to_unit(r.x, r.y);
        // inversion: smallest k with CDF(k) > u
        const double* cdf = p.cdf + Zr.cdf_off;
        uint32_t lo = 0, hi = Zr.cdf_len - 1;
        while (lo < hi) {
          const uint32_t mid = (lo + hi) >> 1;
          if (cdf[mid] > u) hi = mid;
          else lo = mid + 1;
        }
        cnt = (uint32_t)Zr.kmin + lo;
        if (cnt) atomicAdd(&p.pending[(size_t)inst * p.R + Zr.rxn], (unsigned long long)cnt);
      }
    }
    uint32_t tot;
    const uint32_t ex = block_exclusive_scan<1024>(cnt, &s_total);
    tot = s_total;
    if (e < nz) p.zero_off[e] = carry + ex;
    carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    p.zero_off[nz] = carry;
    c->n_virtual = carry;
    if (check_append && (uint64_t)c->n_slots + carry > p.capacity) atomicOr(&c->status, kStatCapacity);
  }
}

// kMinBlocks 4 / 6 cap registers at 64 / 40 (50% / 75% occupancy, the
// latter with a few spills); the launch shape picks the variant.
template <bool kTable, int kMinBlocks, bool kSingle, int kSurf = 0>
__global__ void __launch_bounds__(256, kMinBlocks) k_count(KParams p) {
  __shared__ DevSpecies s_species[kSingle ? kCtxSpecies : 1];
  __shared__ DevUni s_uni[kSingle ? kCtxUni : 1];
  SingleCtx ctx{};
  if (kSingle) ctx = single_ctx(p, s_species, s_uni);
  DevCtrl* c = p.ctrl;
  if (ctrl_status_warp(c)) return;
  const uint32_t cur = ld_u32(&c->cur);
  const float4* __restrict__ st = cur_state(p, cur);
  const uint32_t n_real = ld_u32(&c->n_slots), n_total = n_real + ld_u32(&c->n_virtual);
  stream_records(st, n_real, n_total, [&](uint32_t i, const float4& rec) {
    Out2 o;
    o.n = 0;
    if (i < n_real) advance_rec<kTable, true, kSingle, kSurf>(p, ctx, rec, i, o);
    else if (i < n_total) advance_virtual<kSingle>(p, i - n_real, o);
    warp_count(p.cell_count, o.n > 0 ? o.key[0] : kNoKey);
    if (__any_sync(kFull, o.n > 1)) warp_count(p.cell_count, o.n > 1 ? o.key[1] : kNoKey);
  });
}

// Grid-wide barrier of a cooperative launch (every CTA resident): thread 0
// of each CTA reads the generation, arrives on the counter, and either (the
// last to arrive) resets the counter and advances the generation, or waits
// for the generation to change.  The wait is bounded: after kGridSpins polls
// the CTA raises kStatTimeout and the barrier returns false; the other CTAs
// then run out at the same barrier or the next, so every CTA returns.
constexpr uint32_t kGridSpins = 1u << 22;

__device__ bool grid_barrier(DevCtrl* c) {
  __shared__ uint32_t s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    s_ok = 1u;
    const uint32_t gen = *(volatile uint32_t*)&c->bar_gen;
    __threadfence();
    if (atomicAdd(&c->bar_count, 1u) == gridDim.x - 1u) {
      atomicExch(&c->bar_count, 0u);
      __threadfence();
      atomicAdd(&c->bar_gen, 1u);
    } else {
      for (uint32_t spins = 0; *(volatile uint32_t*)&c->bar_gen == gen; ++spins) {
        if (spins > kGridSpins) {
          atomicOr(&c->status, kStatTimeout);
          s_ok = 0u;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return s_ok != 0u;
}

template <bool kTable, int kMinBlocks, bool kSingle, int kSurf = 0>
__global__ void __launch_bounds__(256, kMinBlocks) k_scatter(KParams p) {
  __shared__ DevSpecies s_species[kSingle ? kCtxSpecies : 1];
  __shared__ DevUni s_uni[kSingle ? kCtxUni : 1];
  SingleCtx ctx{};
  if (kSingle) ctx = single_ctx(p, s_species, s_uni);
  DevCtrl* c = p.ctrl;
  if (ctrl_status_warp(c)) return;
  const uint32_t cur = ld_u32(&c->cur);
  const float4* __restrict__ st = cur_state(p, cur);
  const uint32_t n_real = ld_u32(&c->n_slots), n_total = n_real + ld_u32(&c->n_virtual);
  stream_records(st, n_real, n_total, [&](uint32_t i, const float4& rec) {
    Out2 o;
    o.n = 0;
    if (i < n_real) advance_rec<kTable, false, kSingle, kSurf>(p, ctx, rec, i, o);
    else if (i < n_total) advance_virtual<kSingle>(p, i - n_real, o);
    const int kmax = __any_sync(kFull, o.n > 1) ? 2 : 1;
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      if (k >= kmax) break;  // warp-uniform
      const uint32_t key = o.n > k ? o.key[k] : kNoKey;
      const uint32_t off = warp_claim(p.cell_count, key);
      if (key != kNoKey) {
        const uint32_t slot = p.cell_start[key] + off;
        if (slot < p.capacity) p.scatter[slot] = o.r[k];
        else atomicOr(&c->status, kStatBounds);
      }
    }
  });
}

// Bin layout.  A cell's places come in groups of kBinGroup, stored
// together, and group g of every cell forms one contiguous array:
// place off of a cell is bins[(g * n_cells + cell) * kBinGroup + off %
// kBinGroup], g = off / kBinGroup.  The records a warp bins belong to a
// few consecutive cells (the state is in cell order), so their stores fall
// on a few contiguous lines, and a cell's first records fill whole 32-byte
// sectors rather than half of one shared with a neighbour cell.  The pair
// kernel reads a cell's first kBinGroup places from one group.
__device__ __forceinline__ size_t bin_index(const KParams& p, uint32_t cell, uint32_t off) {
  return ((size_t)(off / kBinGroup) * p.n_cells + cell) * kBinGroup + off % kBinGroup;
}

// A record waiting for its place in a bin: the warp's claim (atomicAdd on
// the cell count by the lane that leads the cell's peers) is issued when
// the record is made and consumed one record later, so the atomic's round
// trip to L2 overlaps the next record's arithmetic instead of stalling it.
struct PendingClaim {
  float4 r;
  uint32_t key;     // kNoKey: nothing pending in this lane
  uint32_t old;     // leader lane: count before the warp's claim
  uint32_t leader;  // lane holding `old` for this lane's cell
  uint32_t rank;    // this lane's place among its cell's peers
};

__device__ __forceinline__ PendingClaim claim_issue(uint32_t* cnt, uint32_t key, const float4& r) {
  PendingClaim c;
  c.r = r;
  c.key = key;
  const uint32_t peers = __match_any_sync(kFull, key);
  c.leader = (uint32_t)(__ffs(peers) - 1);
  c.rank = __popc(peers & ((1u << lane_id()) - 1u));
  c.old = 0;
  if (key != kNoKey && lane_id() == c.leader) c.old = atomicAdd(&cnt[key], (uint32_t)__popc(peers));
  return c;
}

__device__ __forceinline__ void claim_retire(const KParams& p, DevCtrl* c, const PendingClaim& pc) {
  const uint32_t off = __shfl_sync(kFull, pc.old, pc.leader) + pc.rank;
  if (pc.key == kNoKey) return;
  if (off < p.bin_cap) {
    p.bins[bin_index(p, pc.key, off)] = pc.r;
  } else {
    atomicOr(&c->status, kStatBins);
    atomicMax(&c->bin_need, off + 1u);
  }
}

// Binned path, pass 1 of 2: advance every record (as k_count) and write it
// into the next free place of its cell's bin.  Replaces k_count + k_scatter:
// the step's arithmetic runs once and nothing is recomputed.  First
// products keep the deferred claim above; the rare second products (births)
// claim and store at once.
// Slots a warp queues for k_bin_surface, written out 32 at a time with one
// atomicAdd on the queue count (a record per lane and atomic would all meet
// on that one word).
struct DeferBuffer {
  uint32_t slot[64];
};

__device__ __forceinline__ void defer_flush(const KParams& p, DevCtrl* c, DeferBuffer& b, uint32_t n) {
  __syncwarp();
  uint32_t base = 0;
  if (lane_id() == 0) base = atomicAdd(&c->n_surf, n);
  base = __shfl_sync(kFull, base, 0);
  if (lane_id() < n) {
    const uint32_t e = base + lane_id();
    if (e < p.capacity) p.surf_queue[e] = b.slot[lane_id()];
    else atomicOr(&c->status, kStatBounds);
  }
  __syncwarp();
}

template <bool kTable, int kMinBlocks, bool kSingle, int kSurf = 0>
__global__ void __launch_bounds__(256, kMinBlocks) k_bin(KParams p) {
  __shared__ DevSpecies s_species[kSingle ? kCtxSpecies : 1];
  __shared__ DevUni s_uni[kSingle ? kCtxUni : 1];
  __shared__ DeferBuffer s_defer[kSurf == 2 ? 8 : 1];  // one per warp (blocks of at most 256 threads)
  DeferBuffer& defer_buf = s_defer[kSurf == 2 ? threadIdx.x >> 5 : 0];
  uint32_t n_defer = 0;  // slots in defer_buf (warp-uniform)
  SingleCtx ctx{};
  if (kSingle) ctx = single_ctx(p, s_species, s_uni);
  DevCtrl* c = p.ctrl;
  if (ctrl_status_warp(c)) return;
  const uint32_t cur = ld_u32(&c->cur);
  const float4* __restrict__ st = cur_state(p, cur);
  const uint32_t n_real = ld_u32(&c->n_slots), n_total = n_real + ld_u32(&c->n_virtual);
  PendingClaim pending;
  pending.key = kNoKey;
  pending.old = 0;
  pending.leader = 0;
  pending.rank = 0;
  stream_records(st, n_real, n_total, [&](uint32_t i, const float4& rec) {
    Out2 o;
    o.n = 0;
    if (i < n_real) advance_rec<kTable, true, kSingle, kSurf>(p, ctx, rec, i, o);
    else if (i < n_total) advance_virtual<kSingle>(p, i - n_real, o);
    if (kSurf == 2) {
      // records near a panel go to k_bin_surface
      const bool defer = o.n < 0;
      const uint32_t ball = __ballot_sync(kFull, defer);
      if (ball) {
        if (defer) {
          defer_buf.slot[n_defer + __popc(ball & ((1u << lane_id()) - 1u))] = i;
          o.n = 0;
        }
        n_defer += __popc(ball);
        if (n_defer >= 32u) {
          defer_flush(p, c, defer_buf, 32u);
          if (lane_id() + 32u < n_defer) defer_buf.slot[lane_id()] = defer_buf.slot[lane_id() + 32u];
          __syncwarp();
          n_defer -= 32u;
        }
      }
    }
    const PendingClaim next = claim_issue(p.cell_count, o.n > 0 ? o.key[0] : kNoKey, o.r[0]);
    if (__any_sync(kFull, o.n > 1)) claim_retire(p, c, claim_issue(p.cell_count, o.n > 1 ? o.key[1] : kNoKey, o.r[1]));
    claim_retire(p, c, pending);
    pending = next;
  });
  claim_retire(p, c, pending);
  if (kSurf == 2 && n_defer > 0) defer_flush(p, c, defer_buf, n_defer);
}

// Binned path with surfaces, pass 1b: the records k_bin queued because
// their move meets a panel box, advanced with the surface walk (the same
// Philox counters, so the same step) and put into their bins.  A walk's
// cost varies with the panels near the record (one sphere against a mesh
// of many triangles), and the queue holds neighbouring records together,
// so warps take 32 queue entries at a time from a counter until the queue
// is empty: a warp of slow walks does not hold the others' share.
template <bool kTable, bool kSingle>
__global__ void __launch_bounds__(256, 4) k_bin_surface(KParams p) {
  __shared__ DevSpecies s_species[kSingle ? kCtxSpecies : 1];
  __shared__ DevUni s_uni[kSingle ? kCtxUni : 1];
  SingleCtx ctx{};
  if (kSingle) ctx = single_ctx(p, s_species, s_uni);
  DevCtrl* c = p.ctrl;
  if (ctrl_status_warp(c)) return;
  const float4* __restrict__ st = cur_state(p, ld_u32(&c->cur));
  const uint32_t n = min(ld_u32(&c->n_surf), p.capacity);
  const uint32_t lane = lane_id();
  // first products keep k_bin's deferred claim (consumed one record later)
  PendingClaim pending;
  pending.key = kNoKey;
  pending.old = 0;
  pending.leader = 0;
  pending.rank = 0;
  for (;;) {  // warp-uniform trip count
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(&c->surf_ticket, 32u);
    base = __shfl_sync(kFull, base, 0);
    if (base >= n) break;
    const uint32_t e = base + lane;
    Out2 o;
    o.n = 0;
    if (e < n) {
      const uint32_t i = p.surf_queue[e];
      advance_rec<kTable, true, kSingle, 1>(p, ctx, st[i], i, o);
    }
    const PendingClaim next = claim_issue(p.cell_count, o.n > 0 ? o.key[0] : kNoKey, o.r[0]);
    if (__any_sync(kFull, o.n > 1)) claim_retire(p, c, claim_issue(p.cell_count, o.n > 1 ? o.key[1] : kNoKey, o.r[1]));
    claim_retire(p, c, pending);
    pending = next;
  }
  claim_retire(p, c, pending);
}

// The records of one cell, m-th at base[(m / kBinGroup) * stride + m %
// kBinGroup]: a bin of the binned sort (stride = kBinGroup x the number of
// cells) or a range of the compact scatter buffer (stride kBinGroup, so
// the m-th record is base[m]).
struct CellView {
  const float4* base;
  size_t stride;
  __device__ __forceinline__ size_t at(uint32_t m) const { return (size_t)(m / kBinGroup) * stride + m % kBinGroup; }
  __device__ __forceinline__ float4 operator[](uint32_t m) const { return base[at(m)]; }
  __device__ __forceinline__ float4 ldg(uint32_t m) const { return __ldg(base + at(m)); }
  __device__ __forceinline__ float ldg_x(uint32_t m) const {
    return __ldg(reinterpret_cast<const float*>(base + at(m)));
  }
  __device__ __forceinline__ float2 ldg_xy(uint32_t m) const {
    return __ldg(reinterpret_cast<const float2*>(base + at(m)));
  }
};

// A cell's bin with its first kBinGroup places staged in shared memory by
// a bulk copy (kStage); the rest of the bin is read from global memory.
template <bool kStage>
struct BinView {
  const float4* sm;
  CellView g;
  __device__ __forceinline__ float4 operator[](uint32_t m) const {
    if (kStage && m < kBinGroup) return sm[m];
    return g[m];
  }
  __device__ __forceinline__ float4 ldg(uint32_t m) const {
    if (kStage && m < kBinGroup) return sm[m];
    return g.ldg(m);
  }
  __device__ __forceinline__ float ldg_x(uint32_t m) const {
    if (kStage && m < kBinGroup) return sm[m].x;
    return g.ldg_x(m);
  }
  __device__ __forceinline__ float2 ldg_xy(uint32_t m) const {
    if (kStage && m < kBinGroup) return make_float2(sm[m].x, sm[m].y);
    return g.ldg_xy(m);
  }
};

// Bulk global -> shared copies completed on an mbarrier (the copy engine
// moves the bytes; no thread issues a load per word).
__device__ __forceinline__ uint32_t smem_u32(const void* ptr) {
  return (uint32_t)__cvta_generic_to_shared(ptr);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// One thread: announce `bytes` and start the copy that will deliver them.
// The fence orders this thread's earlier generic-proxy accesses of the
// buffer (the warp's reads of its previous contents) before the copy.
__device__ __forceinline__ void bulk_to_smem(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
// Wait for the phase with parity `parity` of `bar` to complete; false after
// 2^20 polls (each poll suspends the thread for at most a short
// hardware-defined time).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (uint32_t it = 0; it < (1u << 20); ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Exclusive scan of the cell counts into cell_start, by a cooperative grid
// of two CTAs per SM (every CTA resident).  CTA b owns a contiguous range of
// cells and moves it through shared memory in chunks of up to kScanChunk
// counts, each brought in by one bulk copy (the copy engine, not a load
// per word): pass 1 sums the range and publishes the sum (tile_sums[b]);
// after one grid barrier, pass 2 adds the sums of the CTAs before it,
// scans each chunk in shared memory (a contiguous run of counts per
// thread) and writes it out by one bulk copy.  On the 16M c3 step a range
// is one chunk, so pass 2 finds it still in shared memory.  The last 1..3
// counts of the grid that do not fill 16 bytes go by plain loads and
// stores.  20.8 us on the 16M c3 step; chunks of 49,152 counts (one CTA
// per SM) took 22.4 us, of 12,288 (four) 26.3 us.  Earlier forms: a
// single-pass scan by decoupled look-back, 27 us (643 tiles, and the
// frontier of known prefixes moved by the 32 flags one poll reads per round
// trip); this grid scan reading tiles of 8,192 counts with vector loads
// instead of staging them, 24.6 us.
constexpr uint32_t kScanChunk = 24576;  // counts per chunk: 96 KiB of shared memory
constexpr uint32_t kScanSmem = kScanChunk * 4u;  // dynamic shared memory of k_scan

__device__ __forceinline__ void bulk_to_global(void* dst, const void* src, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_u32(src)),
               "r"(bytes)
               : "memory");
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}

// Chunk [c0, c0 + len) of the counts into s_cnt: the 16-byte-aligned part
// by one bulk copy (thread 0) on `bar`, the rest by plain loads.  False when
// the copy's wait runs out.
__device__ __forceinline__ bool scan_stage(const KParams& p, uint32_t* s_cnt, uint64_t* bar, uint32_t c0,
                                           uint32_t len, uint32_t& phase) {
  const uint32_t bulk = len & ~3u;
  if (bulk) {
    if (threadIdx.x == 0) bulk_to_smem(s_cnt, p.cell_count + c0, bulk * 4u, bar);
  }
  if (threadIdx.x < len - bulk) s_cnt[bulk + threadIdx.x] = __ldcg(&p.cell_count[c0 + bulk + threadIdx.x]);
  bool ok = true;
  if (bulk) {
    ok = mbar_wait(bar, phase);
    if (!ok) mbar_wait(bar, phase);  // give the copy in flight more time to land before the CTA leaves
    phase ^= 1u;
  }
  // one answer for the whole CTA, so that its threads leave or go on together
  return __syncthreads_and(ok) != 0;
}

__global__ void __launch_bounds__(1024) k_scan(KParams p) {
  extern __shared__ __align__(128) uint32_t s_cnt[];
  __shared__ __align__(8) uint64_t s_bar;
  __shared__ uint32_t s_stop, s_total, s_prefix, s_warp[32];
  DevCtrl* c = p.ctrl;
  if (threadIdx.x == 0) {
    s_stop = ld_u32(&c->status) != 0u;
    mbar_init(&s_bar);
    mbar_init_fence();
  }
  __syncthreads();
  // the status is the previous kernels' and the same for every CTA: all
  // return here together or none does
  if (s_stop) return;
  if (p.scan_withhold && blockIdx.x == 0) {  // test switch: CTA 0 never arrives
    if (gridDim.x == 1 && threadIdx.x == 0) atomicOr(&c->status, kStatTimeout);
    return;
  }
  // ranges of a multiple of 4 counts (16-byte aligned bulk copies)
  const uint32_t per = ((p.n_cells + gridDim.x - 1u) / gridDim.x + 3u) & ~3u;
  const uint32_t lo = min(blockIdx.x * per, p.n_cells), hi = min(lo + per, p.n_cells);
  const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
  uint32_t phase = 0;
  bool ok = true;
  // pass 1: the range's sum
  uint32_t sum = 0;
  for (uint32_t c0 = lo; c0 < hi && ok; c0 += kScanChunk) {
    const uint32_t len = min(kScanChunk, hi - c0);
    if (c0 != lo) __syncthreads();  // the previous chunk is summed
    ok = scan_stage(p, s_cnt, &s_bar, c0, len, phase);
    for (uint32_t i = threadIdx.x; i < len; i += 1024u) sum += s_cnt[i];
  }
  if (!ok) {
    if (threadIdx.x == 0) atomicOr(&c->status, kStatTimeout);
    return;
  }
  sum = __reduce_add_sync(kFull, sum);
  if (lane == 0) s_warp[warp] = sum;
  __syncthreads();
  if (warp == 0) {
    const uint32_t t = __reduce_add_sync(kFull, lane < (blockDim.x >> 5) ? s_warp[lane] : 0u);
    if (lane == 0) p.tile_sums[blockIdx.x] = t;
  }
  if (!grid_barrier(c)) return;
  // the counts before the range
  if (warp == 0) {
    uint32_t v = 0;
    for (uint32_t b = lane; b < blockIdx.x; b += 32u) v += __ldcg(&p.tile_sums[b]);
    v = __reduce_add_sync(kFull, v);
    if (lane == 0) s_prefix = v;
  }
  __syncthreads();
  // pass 2: each chunk scanned in shared memory, a run of q counts per thread
  uint32_t carry = s_prefix;
  const bool resident = hi - lo <= kScanChunk;  // the one chunk is still staged
  for (uint32_t c0 = lo; c0 < hi; c0 += kScanChunk) {
    const uint32_t len = min(kScanChunk, hi - c0);
    if (!resident) {
      __syncthreads();
      if (threadIdx.x == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");  // last chunk's store has read its source
      __syncthreads();
      if (!scan_stage(p, s_cnt, &s_bar, c0, len, phase)) {
        if (threadIdx.x == 0) atomicOr(&c->status, kStatTimeout);
        break;
      }
    }
    const uint32_t q = (len + 1023u) >> 10;
    const uint32_t b0 = min(threadIdx.x * q, len), b1 = min(b0 + q, len);
    uint32_t s = 0;
    for (uint32_t i = b0; i < b1; ++i) s += s_cnt[i];
    uint32_t run = carry + block_exclusive_scan<1024>(s, &s_total);
    carry += s_total;
    for (uint32_t i = b0; i < b1; ++i) {
      const uint32_t x = s_cnt[i];
      s_cnt[i] = run;
      run += x;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the writes above, seen by the bulk copy
    __syncthreads();
    const uint32_t bulk = len & ~3u;
    if (threadIdx.x == 0 && bulk) bulk_to_global(p.cell_start + c0, s_cnt, bulk * 4u);
    if (threadIdx.x < len - bulk) p.cell_start[c0 + bulk + threadIdx.x] = s_cnt[bulk + threadIdx.x];
  }
  if (threadIdx.x == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
  if (blockIdx.x == gridDim.x - 1u && threadIdx.x == 0) {  // every count lies at or before its range's end
    p.cell_start[p.n_cells] = carry;
    c->n_sorted = carry;
    if (carry > p.capacity) atomicOr(&c->status, kStatCapacity);
  }
}

// Position of record r among the records of its cell [s, e) in canonical
// order; ties between identical records go by slot.
template <class View>
__device__ __forceinline__ uint32_t canonical_rank(const View sc, uint32_t s, uint32_t e, uint32_t slot,
                                                   const float4& r) {
  uint32_t rank = 0;
  for (uint32_t m = s; m < e; ++m) {
    const float4 q = sc[m];
    rank += (rec_less(q, r) || (m < slot && rec_equal(q, r))) ? 1u : 0u;
  }
  return rank;
}

__device__ __forceinline__ float dist2(const float4& a, const float4& b) {
  const float dx = __fsub_rn(a.x, b.x), dy = __fsub_rn(a.y, b.y), dz = __fsub_rn(a.z, b.z);
  return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}

// Append candidate pair (lo < hi, canonical slots) of local reaction b,
// after its coin when the reaction probability is below 1.
__device__ __forceinline__ void emit_pair(const KParams& p, DevCtrl* c, uint32_t lo, uint32_t hi, int32_t b,
                                          float prob, uint32_t inst, const DevInstance& I) {
  if (prob < 1.0f) {
    const uint32_t base_new = __ldg(&p.cell_start[I.cell_base]);
    const U4 u = philox(U4{lo - base_new, __ldg(&p.inst_step[inst]), kTagBimCoin, hi - base_new}, I.key_lo,
                        I.key_hi);
    if (!(u32_to_unit(u.x) < prob)) return;
  }
  const uint32_t idx = atomicAdd(&c->n_pairs, 1u);
  if (idx < p.pair_cap) p.pairs[idx] = DevPair{lo, hi, (uint32_t)b | (inst << 16), 0u};
  else atomicOr(&c->status, kStatPairs);
}

// Cells with more records than this are handed from k_pairs_cells to
// k_pairs_big, which gives each of them a whole CTA.
constexpr uint32_t kBigCell = 128;
constexpr int kBigGrid = 304;  // most CTAs of the large-cell kernel (cells they take in turn)

// First record of a cell: its bin, or its range of the compact scatter buffer.
template <bool kBinned>
__device__ __forceinline__ CellView cell_records(const KParams& p, uint32_t cell, uint32_t cs) {
  if (kBinned) return CellView{p.bins + bin_index(p, cell, 0), (size_t)p.n_cells * kBinGroup};
  return CellView{p.scatter + cs, kBinGroup};
}

// A record looking for partners.
struct Seeker {
  float4 r;
  uint32_t inst, block;
  float max_r, r2max;
  float xlim;          // |dx| bound of every pair within its binding radii
  const int32_t* row;  // second-order table row of its species
};

// False when the record takes no part in this step's pair search: born in
// this step, instance not advancing, or a species without second-order
// reactions.
// s_maxr (one-instance kernels): the species' largest radii in shared
// memory, with adv0 the instance's advancing state, read once per kernel.
template <bool kSingle>
__device__ __forceinline__ bool seeker_init(const KParams& p, const float4& r, Seeker& k,
                                            const float* s_maxr = nullptr, bool adv0 = true) {
  const uint32_t w = rec_w(r);
  if (w & kNewborn) return false;
  k.r = r;
  k.inst = w >> 16;
  const uint32_t sa = w & kSpeciesMask;
  if (kSingle && s_maxr) {
    if (!adv0) return false;
    k.block = p.inst0.block;
    k.max_r = s_maxr[sa];
  } else {
    if (!advancing(__ldg(&p.inst_flags[k.inst]))) return false;
    k.block = inst_of<kSingle>(p, k.inst).block;
    k.max_r = __ldg(&p.species[k.block * p.S + sa].max_r);
  }
  // a bound on every squared radius of the species (float rounding of max_r^2)
  k.r2max = k.max_r * k.max_r * 1.0001f;
  // fl(dx^2) <= d2 <= r2max, so |dx| <= max_r * 1.00005
  k.xlim = k.max_r * 1.001f;
  k.row = p.bim_table + sa * p.S;
  return k.max_r > 0.0f;
}

// Local second-order reaction of k with record q when q lies within its
// binding radius, else -1.
__device__ __forceinline__ int32_t pair_reaction(const KParams& p, const Seeker& k, const float4& q) {
  if (fabsf(__fsub_rn(q.x, k.r.x)) > k.xlim) return -1;
  const uint32_t wq = rec_w(q);
  if (wq & kNewborn) return -1;
  const float d2 = dist2(k.r, q);
  if (d2 > k.r2max) return -1;
  const int32_t b = __ldg(&k.row[wq & kSpeciesMask]);
  if (b < 0 || d2 > __ldg(&p.bim[k.block * p.B + (uint32_t)b].r2)) return -1;
  return b;
}

template <bool kSingle>
__device__ __forceinline__ void emit(const KParams& p, DevCtrl* c, const Seeker& k, uint32_t ca, uint32_t cq,
                                     int32_t b) {
  emit_pair(p, c, min(ca, cq), max(ca, cq), b, __ldg(&p.bim[k.block * p.B + (uint32_t)b].prob), k.inst,
            inst_of<kSingle>(p, k.inst));
}

// True when record k may lie within its largest binding radius (plus the
// pruning margin) of a +x, +y or +z face of its cell, i.e. when
// forward_mask may return a neighbour; false for most records, which lie
// deeper inside their cell.  The test runs on the fractional grid
// coordinates: frac = g - floor(g) is exact (Sterbenz), and the 1% slack
// exceeds the rounding of forward_mask's face distances, so it never
// rejects a record that forward_mask would give a neighbour.
template <bool kSingle>
__device__ __forceinline__ bool near_forward_face(const KParams& p, const Seeker& k) {
  const DevInstance& I = inst_of<kSingle>(p, k.inst);
  const float gx = __fmul_rn(__fsub_rn(k.r.x, I.lo[0]), I.inv[0]);
  const float gy = __fmul_rn(__fsub_rn(k.r.y, I.lo[1]), I.inv[1]);
  const float gz = __fmul_rn(__fsub_rn(k.r.z, I.lo[2]), I.inv[2]);
  const float slack = 1.01f * (k.max_r + p.prune_margin * fminf(I.cell[0], fminf(I.cell[1], I.cell[2])));
  return !(1.0f - (gx - floorf(gx)) > slack * I.inv[0] && 1.0f - (gy - floorf(gy)) > slack * I.inv[1] &&
           1.0f - (gz - floorf(gz)) > slack * I.inv[2]);
}

// The forward neighbour cells (higher key) of record k that its largest
// binding radius reaches: the cells whose shared face, edge or corner lies
// within it.  Every cross-cell pair within range is found from its
// lower-key side only, so each is tested once.  Bit b of the result names
// neighbour b: 0 = (+1, 0, 0); 1..3 = (-1..+1, +1, 0); 4..12 = (-1..+1,
// -1..+1, +1) in (dx, dy, dz), dx fastest.  *key0 receives the record's own
// cell key.  The cell coordinates are recomputed from the position exactly
// as the sort computed the key (cell_coord), which avoids integer division.
template <bool kSingle>
__device__ __forceinline__ uint32_t forward_mask(const KParams& p, const Seeker& k, uint32_t* key0) {
  const DevInstance& I = inst_of<kSingle>(p, k.inst);
  const float cl0 = I.cell[0], cl1 = I.cell[1], cl2 = I.cell[2];
  const uint32_t d0 = I.dims[0], d1 = I.dims[1], d2 = I.dims[2];
  const float gx = __fmul_rn(__fsub_rn(k.r.x, I.lo[0]), I.inv[0]);
  const float gy = __fmul_rn(__fsub_rn(k.r.y, I.lo[1]), I.inv[1]);
  const float gz = __fmul_rn(__fsub_rn(k.r.z, I.lo[2]), I.inv[2]);
  const int cx = min(max((int)floorf(gx), 0), (int)d0 - 1);
  const int cy = min(max((int)floorf(gy), 0), (int)d1 - 1);
  const int cz = min(max((int)floorf(gz), 0), (int)d2 - 1);
  *key0 = I.cell_base + ((uint32_t)cz * d1 + (uint32_t)cy) * d0 + (uint32_t)cx;
  const float margin = p.prune_margin * fminf(cl0, fminf(cl1, cl2));
  const float need = k.max_r + margin;
  const float fx = __fsub_rn(gx, (float)cx), fy = __fsub_rn(gy, (float)cy), fz = __fsub_rn(gz, (float)cz);
  const float hix = (1.0f - fx) * cl0, hiy = (1.0f - fy) * cl1, hiz = (1.0f - fz) * cl2;
  // Every forward neighbour lies across the +x, +y or +z face.  Squared
  // distance to the -/+ face along each axis, infinite where no
  // cell lies beyond the face; a neighbour is marked when the sum over its
  // axes, added as (x + y) + z, is within need^2.  No branch: the warp
  // takes the records of a drain together, so every lane's marking used to
  // run the loops of the slowest.
  const float far = __int_as_float(0x7f800000);
  const float lox = fx * cl0, loy = fy * cl1;
  const float need2 = need * need;
  const float xm = cx > 0 ? lox * lox : far, xp = cx + 1 < (int)d0 ? hix * hix : far;
  const float ym = cy > 0 ? loy * loy : far, yp = cy + 1 < (int)d1 ? hiy * hiy : far;
  const float zp = cz + 1 < (int)d2 ? hiz * hiz : far;
  uint32_t mask = xp <= need2 ? 1u : 0u;  // (+1, 0, 0)
  mask |= (xm + yp <= need2 ? 1u : 0u) << 1;
  mask |= (yp <= need2 ? 1u : 0u) << 2;
  mask |= (xp + yp <= need2 ? 1u : 0u) << 3;
  const float ey[3] = {ym, 0.0f, yp}, ex[3] = {xm, 0.0f, xp};
#pragma unroll
  for (int dy = 0; dy < 3; ++dy) {
#pragma unroll
    for (int dx = 0; dx < 3; ++dx) mask |= ((ex[dx] + ey[dy]) + zp <= need2 ? 1u : 0u) << (4 + dy * 3 + dx);
  }
  return mask;
}

// Key of forward neighbour b (bit numbering of forward_mask) of cell key0.
__device__ __forceinline__ uint32_t forward_key(uint32_t key0, uint32_t b, uint32_t d0, uint32_t d1) {
  int dx, dy, dz;
  if (b == 0) {
    dx = 1, dy = 0, dz = 0;
  } else if (b < 4) {
    dx = (int)b - 2, dy = 1, dz = 0;
  } else {
    const int q = (int)b - 4;
    dx = q % 3 - 1, dy = q / 3 - 1, dz = 1;
  }
  return (uint32_t)((int)key0 + (dz * (int)d1 + dy) * (int)d0 + dx);
}

// Pairs of seeker k (canonical slot ca) with the records of neighbour cell
// nkey (first slot ns, nn records), found from k's side.
template <bool kBinned, bool kSingle>
__device__ __forceinline__ void visit_cell(const KParams& p, DevCtrl* c, const Seeker& k, uint32_t ca,
                                           uint32_t nkey, uint32_t ns, uint32_t nn) {
  if (nn > kBigCell) return;  // pairs with large cells are found by k_pairs_big
  const CellView nb = cell_records<kBinned>(p, nkey, ns);
  // x words of the first members together (overlapping latencies); a full
  // record only for members within the x window, taken from a bit mask
  // (places past the cell read as all-ones bits, a NaN |dx|).  The mask in
  // place of a branch per member: 0.248 against 0.261 ms on the 16M c3
  // step, although only the records near a +face come here.
  constexpr uint32_t kBatch = 8;
  float xs[kBatch];
#pragma unroll
  for (uint32_t m = 0; m < kBatch; ++m) xs[m] = m < nn ? nb.ldg_x(m) : __uint_as_float(0xFFFFFFFFu);
  uint32_t inx = 0;
#pragma unroll
  for (uint32_t m = 0; m < kBatch; ++m) inx |= (fabsf(__fsub_rn(xs[m], k.r.x)) <= k.xlim ? 1u : 0u) << m;
  while (inx) {
    const uint32_t m = (uint32_t)(__ffs(inx) - 1);
    inx &= inx - 1u;
    const float4 q = nb.ldg(m);
    const int32_t b = pair_reaction(p, k, q);
    if (b >= 0) emit<kSingle>(p, c, k, ca, ns + canonical_rank(nb, 0, nn, m, q), b);
  }
  for (uint32_t m = kBatch; m < nn; ++m) {
    const float4 q = nb.ldg(m);
    const int32_t b = pair_reaction(p, k, q);
    if (b >= 0) emit<kSingle>(p, c, k, ca, ns + canonical_rank(nb, 0, nn, m, q), b);
  }
}

// Canonical order + pair search.  A warp takes tasks of 32 consecutive
// cells, from the highest key down, and strings the tasks' records
// together into one stream: round r of the warp takes stream records
// 32r .. 32r+31, one per lane, whatever cells and tasks they come from, so
// only the warp's last round runs partly empty.  (Rounds that stopped at
// each task's end left 14% of the lanes idle on the 16M c3 step, whose
// tasks hold about 97 records.)  At most two tasks are open at a time:
// their non-empty cells sit in a per-warp ring, and a task is opened (its
// cell ranges read and scanned) when the stream runs short of the next
// round and the task before the last one has ended.  There are no CTA-wide
// barriers.  For its record a lane
//   * counts the records of its cell that precede it in canonical order,
//     reading only their x words (records whose x bits occur twice in the
//     cell are ranked again on all four words), and writes it to
//     cell_start[cell] + that rank in the next state;
//   * in the same loop marks the cell's later records (storage order)
//     whose x lies within its largest binding radius; only those are read
//     in full and tested, each in-cell pair once;
//   * tests, cheaply and with no branch, whether its record lies within
//     its largest binding radius of a +face of its cell (near_forward_face)
//     and queues those few records in the warp's shared queue; the warp
//     takes them 32 at a time, one per lane, marks their forward neighbour
//     cells (forward_mask) and visits them.  Marking the neighbours of
//     every record in line, and visiting them from the record's own lane,
//     held whole warps for the sake of one or two lanes.
// Canonical slots of partners are computed only for pairs within range.
// Cells above kBigCell records are queued for the large-cell kernels.  kBinned: the
// records come from the cell bins, whose counts are cleared here for the
// next step; otherwise from the compact scatter buffer.
//
// Binned path: bulk-copy staging of each task's first bin group (kStage).
// Measured slower on the 16M c3 step (0.325 against 0.272 ms with the
// record stream; 0.360 against 0.338 ms before it): four CTAs' staging
// buffers take the L1 space that the rank loads and neighbour visits hit
// in.  Kept selectable; the parity tests pass with it.
constexpr bool kStagePairs = false;

constexpr uint32_t kFaceQueue = 64;  // queued records per warp (< 32 between drains, + one round's push)
constexpr uint32_t kCellRing = 64;   // open cells per warp: two tasks of at most 32 non-empty cells

// Records near a +face queued by a warp.
struct FaceQueue {
  float4 rec[kFaceQueue];
  uint32_t ca[kFaceQueue];
};

// Take the first 32 queued records, one per lane (lane < n), move the rest
// (n - 32 < 32 entries) to the front, then mark and visit the forward
// neighbour cells of the lane's record.  Warp-uniform call.
template <bool kBinned, bool kSingle>
__device__ __forceinline__ void drain_faces(const KParams& p, DevCtrl* c, FaceQueue& q, uint32_t n,
                                            const float* s_maxr, bool adv0) {
  const uint32_t lane = lane_id();
  __syncwarp();
  const float4 r = q.rec[lane];
  const uint32_t ca = q.ca[lane];
  __syncwarp();
  if (lane + 32u < n) {
    q.rec[lane] = q.rec[lane + 32u];
    q.ca[lane] = q.ca[lane + 32u];
  }
  __syncwarp();
  if (lane >= n) return;
  Seeker k;
  if (!seeker_init<kSingle>(p, r, k, s_maxr, adv0)) return;
  uint32_t key0 = 0;
  uint32_t nbm = forward_mask<kSingle>(p, k, &key0);
  const DevInstance& I = inst_of<kSingle>(p, k.inst);
  while (nbm) {
    const uint32_t nkey = forward_key(key0, (uint32_t)(__ffs(nbm) - 1), I.dims[0], I.dims[1]);
    nbm &= nbm - 1u;
    const uint32_t ns = __ldg(&p.cell_start[nkey]);
    visit_cell<kBinned, kSingle>(p, c, k, ca, nkey, ns, __ldg(&p.cell_start[nkey + 1]) - ns);
  }
}

// kStage (binned path): group 0 of a task's 32 cells -- their first
// kBinGroup places, one contiguous 2 KiB run of the bins -- is brought into
// shared memory by a bulk copy into the stage buffer of the task's slot
// (its index among the warp's tasks, mod 2).  The copy for a task is
// started as soon as the task two before it has ended, so the copy engine
// moves it while the warp works on the task in between; it is waited for
// when the task is opened.  Places beyond the first group are read from
// global memory.
template <bool kHasBim, bool kBinned, bool kSingle, bool kStage>
__global__ void __launch_bounds__(256, 4) k_pairs_cells(KParams p) {
  // ring of the open tasks' non-empty cells: (key, first slot) and
  // (records | task slot << 8, stream offset of the cell's first record)
  __shared__ uint2 s_cell[8][kCellRing];
  __shared__ uint2 s_meta[8][kCellRing];
  __shared__ FaceQueue s_face[kHasBim ? 8 : 1];
  __shared__ float s_maxr[kSingle ? kCtxSpecies : 1];
  // one-instance kernels: per species, the near-face thresholds of
  // near_forward_face in grid units (x, y, z), computed once per CTA with
  // the same operations (0.2412 -> 0.2403 ms on the 16M c3 step)
  __shared__ float4 s_near[kSingle ? kCtxSpecies : 1];
  __shared__ __align__(128) float4 s_stage[kStage ? 8 : 1][kStage ? 2 : 1][kStage ? 32 * kBinGroup : 1];
  __shared__ uint64_t s_bar[kStage ? 8 : 1][2];
  if (kSingle) {  // before any warp may leave: one barrier for the whole CTA
    for (uint32_t t = threadIdx.x; t < p.S; t += blockDim.x) {
      const float mr = p.species[p.inst0.block * p.S + t].max_r;
      s_maxr[t] = mr;
      const DevInstance& I = p.inst0;
      const float slack = 1.01f * (mr + p.prune_margin * fminf(I.cell[0], fminf(I.cell[1], I.cell[2])));
      s_near[t] = make_float4(slack * I.inv[0], slack * I.inv[1], slack * I.inv[2], 0.0f);
    }
    __syncthreads();
  }
  const bool adv0 = kSingle ? advancing(ld_u32(&p.inst_flags[0])) : true;
  DevCtrl* c = p.ctrl;
  if (ctrl_status_warp(c)) return;
  const uint32_t cur = ld_u32(&c->cur);
  float4* __restrict__ nx = next_state(p, cur);
  const uint32_t warp = threadIdx.x >> 5, lane = lane_id();
  const uint32_t n_tasks = (p.n_cells + 31u) >> 5;
  const uint32_t nw = gridDim.x * (blockDim.x >> 5);
  const uint32_t tk0 = blockIdx.x * (blockDim.x >> 5) + warp;
  const uint32_t my_tasks = tk0 < n_tasks ? (n_tasks - 1u - tk0) / nw + 1u : 0u;
  const uint32_t le_mask = lane == 31 ? kFull : ((2u << lane) - 1u);
  FaceQueue& fqueue = s_face[kHasBim ? warp : 0];
  uint32_t fq = 0;  // queued records (warp-uniform)
  // The warp's i-th task.  Cells are taken from the highest key down: the
  // bins written last by k_bin (its records stream in ascending cell
  // order) are still in L2, and the next state's low slots, written last
  // here, are the first the next step's k_bin reads.
  auto task_of = [&](uint32_t i) { return n_tasks - 1u - (tk0 + i * nw); };
  // group 0 of the i-th task's cells into stage buffer i & 1 (lane 0)
  auto stage = [&](uint32_t i) {
    const uint32_t first = task_of(i) * 32u, cells = min(32u, p.n_cells - first);
    bulk_to_smem(&s_stage[kStage ? warp : 0][kStage ? (i & 1u) : 0][0], p.bins + bin_index(p, first, 0),
                 cells * kBinGroup * (uint32_t)sizeof(float4), &s_bar[kStage ? warp : 0][kStage ? (i & 1u) : 0]);
  };
  uint32_t staged = 0;  // tasks whose copies have been started
  if (kStage) {
    staged = min(my_tasks, 2u);
    if (lane == 0) {
      mbar_init(&s_bar[warp][0]);
      mbar_init(&s_bar[warp][1]);
      mbar_init_fence();
      for (uint32_t i = 0; i < staged; ++i) stage(i);
    }
    __syncwarp();
  }
  // The two task slots (slot = task index & 1): the stream offset of the
  // lane's cell in each, ~0 for an empty cell.
  uint32_t o0 = ~0u, o1 = ~0u;
  uint32_t opened = 0;   // tasks opened
  uint32_t last = 0;     // stream offset of the last opened task (the end of the one before it)
  uint32_t loaded = 0;   // stream records of the opened tasks
  uint32_t entries = 0;  // ring entries written
  uint32_t before = 0;   // ring entries whose cells start before the round
  // A round takes stream records [rb, rb + 32); one that the open tasks
  // cannot fill (the last task before it still open, or no task left)
  // ends at `loaded`, where the next round starts.
  for (uint32_t rb = 0;;) {
    // Open tasks while the stream falls short of this round and the slot
    // to be reused holds a task that has ended.
    while (loaded < rb + 32u && opened < my_tasks && last <= rb) {
      const uint32_t sl = opened & 1u;
      if (kStage && staged == opened) {  // its copy was not started early
        if (lane == 0) stage(opened);
        ++staged;
      }
      const uint32_t cell = task_of(opened) * 32u + lane;
      uint32_t cs = 0, n = 0;
      if (cell < p.n_cells) {
        cs = __ldg(&p.cell_start[cell]);
        n = __ldg(&p.cell_start[cell + 1]) - cs;
        if (kBinned) p.cell_count[cell] = 0u;
        if (n > kBigCell) {
          const uint32_t b = atomicAdd(&c->n_big, 1u);
          if (b < p.big_cap) p.big[b] = cell;
          else atomicOr(&c->status, kStatBounds);
          n = 0;
        }
      }
      const uint32_t ball = __ballot_sync(kFull, n > 0);
      uint32_t incl = n;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const uint32_t t = __shfl_up_sync(kFull, incl, d);
        if (lane >= (uint32_t)d) incl += t;
      }
      const uint32_t off = loaded + incl - n;
      __syncwarp();  // the ring entries about to be replaced are no longer read
      if (n > 0) {
        const uint32_t e = (entries + __popc(ball & ((1u << lane) - 1u))) & (kCellRing - 1u);
        s_cell[warp][e] = make_uint2(cell, cs);
        s_meta[warp][e] = make_uint2(n | (sl << 8), off);
      }
      entries += __popc(ball);
      last = loaded;
      loaded += __shfl_sync(kFull, incl, 31);
      if (sl) o1 = n > 0 ? off : ~0u;
      else o0 = n > 0 ? off : ~0u;
      // (one answer for the warp: its lanes leave or go on together)
      if (kStage && !__all_sync(kFull, mbar_wait(&s_bar[warp][sl], (opened >> 1) & 1u))) {
        // give up: record the timeout and let the copies still in flight land
        if (lane == 0) atomicOr(&c->status, kStatTimeout);
        for (uint32_t i = opened; i < staged; ++i) mbar_wait(&s_bar[warp][i & 1u], (i >> 1) & 1u);
        return;
      }
      ++opened;
      __syncwarp();
    }
    if (rb >= loaded) break;  // every task opened and taken
    // lanes at which a cell starts in this round
    const uint32_t M = __reduce_or_sync(kFull, (o0 - rb < 32u ? 1u << (o0 - rb) : 0u) |
                                                   (o1 - rb < 32u ? 1u << (o1 - rb) : 0u));
    const uint32_t t = rb + lane;
    bool near = false;  // this lane's record may have partners in forward neighbour cells
    uint32_t ca = 0;
    float4 ra = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (t < loaded) {
      const uint32_t e = (before + __popc(M & le_mask) - 1u) & (kCellRing - 1u);
      const uint2 cc = s_cell[warp][e];
      const uint2 meta = s_meta[warp][e];
      const uint32_t ocell = cc.x, ocs = cc.y, on = meta.x & 0xFFu;
      const uint32_t j = t - meta.y;
      const BinView<kStage> cb{&s_stage[kStage ? warp : 0][kStage ? (meta.x >> 8) : 0][kStage ? (ocell & 31u) * kBinGroup : 0],
                               cell_records<kBinned>(p, ocell, ocs)};
      ra = cb.ldg(j);
      Seeker k;
      const bool search = kHasBim && seeker_init<kSingle>(p, ra, k, kSingle ? s_maxr : nullptr, adv0);
      const float xlim = search ? k.xlim : -1.0f;
      const uint32_t rx = __float_as_uint(ra.x);
      // rank: members with smaller x bits; le also counts equal ones (the
      // record itself among them), so le - rank > 1 means a tie to break
      // on all four words.  cand: bit m = member m < 32 within xlim in both
      // x and y (a bound on |dx| and |dy| of any pair within range), so
      // only members near in two coordinates are read in full and tested:
      // 0.246 -> 0.242 ms on the 16M c3 step against x alone.  The first
      // kRankBatch members' x and y are loaded together (one 8-byte load
      // each), so their latencies overlap; larger cells continue one member
      // at a time on x.  The batch runs without a branch per member
      // (0.272 -> 0.261 ms): places past the cell read as all-ones x bits,
      // which count in neither rank nor le and give a NaN |dx| that is
      // never in range.
      constexpr uint32_t kRankBatch = 8;
      uint32_t rank = 0, le = 0, cand = 0;
      // members [0, 6) always, [6, 8) only when a lane of the warp has more
      // than six (0.2386 -> 0.2378 ms on the 16M c3 step)
      constexpr uint32_t kRankFirst = 6;
      float2 xs[kRankBatch];
      auto rank_members = [&](uint32_t m0, uint32_t m1) {
#pragma unroll
        for (uint32_t m = m0; m < m1; ++m) xs[m] = m < on ? cb.ldg_xy(m) : make_float2(__uint_as_float(0xFFFFFFFFu), 0.0f);
#pragma unroll
        for (uint32_t m = m0; m < m1; ++m) {
          const uint32_t qb = __float_as_uint(xs[m].x);
          rank += qb < rx ? 1u : 0u;
          le += qb <= rx ? 1u : 0u;
          cand |= (fabsf(__fsub_rn(xs[m].x, ra.x)) <= xlim && fabsf(__fsub_rn(xs[m].y, ra.y)) <= xlim ? 1u : 0u) << m;
        }
      };
      rank_members(0, kRankFirst);
      if (__any_sync(__activemask(), on > kRankFirst)) rank_members(kRankFirst, kRankBatch);
      for (uint32_t m = kRankBatch; m < on; ++m) {
        const float qx = cb.ldg_x(m);
        const uint32_t qb = __float_as_uint(qx);
        rank += qb < rx ? 1u : 0u;
        le += qb <= rx ? 1u : 0u;
        if (m < 32u && fabsf(__fsub_rn(qx, ra.x)) <= xlim) cand |= 1u << m;
      }
      cand &= j >= 31u ? 0u : ~((2u << j) - 1u);  // later members only
      if (le - rank > 1u) rank = canonical_rank(cb, 0, on, j, ra);
      ca = ocs + rank;
      if (ca < p.capacity) nx[ca] = make_float4(ra.x, ra.y, ra.z, __uint_as_float(rec_w(ra) & ~kNewborn));
      else atomicOr(&c->status, kStatBounds);
      if (search) {
        while (cand) {
          const uint32_t m = (uint32_t)(__ffs(cand) - 1);
          cand &= cand - 1u;
          const float4 qm = cb.ldg(m);
          const int32_t bb = pair_reaction(p, k, qm);
          if (bb >= 0) emit<kSingle>(p, c, k, ca, ocs + canonical_rank(cb, 0, on, m, qm), bb);
        }
        for (uint32_t m = max(j + 1u, 32u); m < on; ++m) {  // cells of 33..kBigCell records
          const float4 qm = cb.ldg(m);
          const int32_t bb = pair_reaction(p, k, qm);
          if (bb >= 0) emit<kSingle>(p, c, k, ca, ocs + canonical_rank(cb, 0, on, m, qm), bb);
        }
        if (kSingle) {
          const float4 sn = s_near[rec_w(ra) & kSpeciesMask];
          const DevInstance& I = p.inst0;
          const float gx = __fmul_rn(__fsub_rn(ra.x, I.lo[0]), I.inv[0]);
          const float gy = __fmul_rn(__fsub_rn(ra.y, I.lo[1]), I.inv[1]);
          const float gz = __fmul_rn(__fsub_rn(ra.z, I.lo[2]), I.inv[2]);
          near = !(1.0f - (gx - floorf(gx)) > sn.x && 1.0f - (gy - floorf(gy)) > sn.y && 1.0f - (gz - floorf(gz)) > sn.z);
        } else {
          near = near_forward_face<kSingle>(p, k);
        }
      }
    }
    if (kHasBim) {
      // records near a +face into the warp's queue, visited 32 at a time
      const uint32_t ball = __ballot_sync(kFull, near);
      if (near) {
        const uint32_t pos = fq + __popc(ball & ((1u << lane) - 1u));
        fqueue.rec[pos] = ra;
        fqueue.ca[pos] = ca;
      }
      fq += __popc(ball);
      if (fq >= 32u) {
        drain_faces<kBinned, kSingle>(p, c, fqueue, fq, kSingle ? s_maxr : nullptr, adv0);
        fq -= 32u;
      }
    }
    before += __popc(M);
    rb = min(rb + 32u, loaded);
    // kStage: once the task two before the next unstaged one (the last
    // opened task, or the one before it) has ended with this round, its
    // buffer takes that task's copy
    if (kStage && staged < my_tasks && staged <= opened + 1u && (staged > opened ? loaded : last) <= rb) {
      __syncwarp();
      if (lane == 0) stage(staged);
      ++staged;
    }
    __syncwarp();
  }
  if (kHasBim && fq > 0) drain_faces<kBinned, kSingle>(p, c, fqueue, fq, kSingle ? s_maxr : nullptr, adv0);
}

constexpr uint32_t kBigChunk = 2048;  // records sorted per shared-memory pass

// Records in [0, len) of the sorted run `run` that order before `e`
// (kOrEqual: before or equal).
template <bool kOrEqual>
__device__ __forceinline__ uint32_t run_rank(const float4* run, uint32_t len, const float4& e) {
  uint32_t lo = 0, hi = len;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    const float4 q = run[mid];
    if (rec_less(q, e) || (kOrEqual && rec_equal(q, e))) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// CTA-uniform status read (the large-cell kernels use barriers).
__device__ __forceinline__ bool stop_block(const DevCtrl* c) {
  __shared__ uint32_t s_stop;
  if (threadIdx.x == 0) s_stop = ld_u32(&c->status);
  __syncthreads();
  const bool stop = s_stop != 0;
  __syncthreads();
  return stop;
}

// Large cells, part 1 of 2 (k_pairs_big): the cells queued by
// k_pairs_cells (more than kBigCell records, e.g. particles released at one
// point), one CTA per cell, sorted in O(n log^2 n) rather than ranked in
// O(n^2):
//   1. chunks of 2048 records are sorted in shared memory (bitonic network,
//      padded with all-ones records) into big_scratch;
//   2. merge passes (each record finds its place in the partner run by
//      binary search) double the sorted runs, alternating between
//      big_scratch and the next state, until the cell is one canonical run;
//   3. the run is left in both places: in the next state without newborn
//      marks, in big_scratch (indexed by canonical slot) with them, where
//      part 2 reads it.
template <bool kBinned>
__device__ void big_sort(const KParams& p, DevCtrl* c, uint32_t nbig, float4* s_rec) {
  const uint32_t cur = ld_u32(&c->cur);
  float4* nx = next_state(p, cur);
  const float4 pad = make_float4(__uint_as_float(kFull), __uint_as_float(kFull), __uint_as_float(kFull),
                                 __uint_as_float(kFull));
  for (uint32_t bi = blockIdx.x; bi < nbig; bi += gridDim.x) {
    const uint32_t cell = p.big[bi];
    const uint32_t cs = p.cell_start[cell], n = p.cell_start[cell + 1] - cs;
    if ((uint64_t)cs + n > p.capacity) {
      if (threadIdx.x == 0) atomicOr(&c->status, kStatBounds);
      continue;  // uniform over the CTA
    }
    const CellView cb = cell_records<kBinned>(p, cell, cs);
    float4* out = nx + cs;
    float4* tmp = p.big_scratch + cs;
    for (uint32_t c0 = 0; c0 < n; c0 += kBigChunk) {
      const uint32_t len = min(kBigChunk, n - c0);
      for (uint32_t i = threadIdx.x; i < kBigChunk; i += blockDim.x) s_rec[i] = i < len ? cb[c0 + i] : pad;
      __syncthreads();
      for (uint32_t k = 2; k <= kBigChunk; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
          for (uint32_t i = threadIdx.x; i < kBigChunk; i += blockDim.x) {
            const uint32_t ixj = i ^ j;
            if (ixj > i) {
              const float4 a = s_rec[i], b = s_rec[ixj];
              const bool up = (i & k) == 0;
              if (rec_less(b, a) == up) {
                s_rec[i] = b;
                s_rec[ixj] = a;
              }
            }
          }
          __syncthreads();
        }
      }
      for (uint32_t i = threadIdx.x; i < len; i += blockDim.x) tmp[c0 + i] = s_rec[i];
      __syncthreads();
    }
    float4* src = tmp;
    float4* dst = out;
    for (uint32_t w = kBigChunk; w < n; w <<= 1) {
      for (uint32_t idx = threadIdx.x; idx < n; idx += blockDim.x) {
        const uint32_t lo = idx / (2 * w) * (2 * w);
        const uint32_t mid = min(lo + w, n), hi = min(lo + 2 * w, n);
        const float4 e = src[idx];
        const uint32_t pos = idx < mid ? (idx - lo) + run_rank<false>(src + mid, hi - mid, e)
                                       : (idx - mid) + run_rank<true>(src + lo, mid - lo, e);
        dst[lo + pos] = e;
      }
      __syncthreads();
      float4* t = src;
      src = dst;
      dst = t;
    }
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
      const float4 r = src[i];
      tmp[i] = r;
      out[i] = make_float4(r.x, r.y, r.z, __uint_as_float(rec_w(r) & ~kNewborn));
    }
    __syncthreads();
  }
}

// Index of the first record of the sorted run [0, n) whose x has its sign
// bit set: canonical order sorts x >= 0 ascending, then negative x by |x|.
__device__ __forceinline__ uint32_t run_negative_start(const float4* run, uint32_t n) {
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (__float_as_uint(run[mid].x) & 0x80000000u) hi = mid;
    else lo = mid + 1;
  }
  return lo;
}

// First record of [lo, hi) (sorted by |x| within one sign) with |x| >= v.
__device__ __forceinline__ uint32_t run_abs_lower(const float4* run, uint32_t lo, uint32_t hi, float v) {
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (fabsf(run[mid].x) < v) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// Pairs of seeker k (canonical slot ca) with the records of a sorted run
// (canonical slots base + m) whose |x - k.x| is within k.xlim, skipping
// m <= skip_to (in-cell: only later records; else pass -1).
template <bool kSingle>
__device__ void sweep_sorted(const KParams& p, DevCtrl* c, const Seeker& k, uint32_t ca, const float4* run,
                             uint32_t n, uint32_t base, int64_t skip_to) {
  const uint32_t npos = run_negative_start(run, n);
  // bounds widened well past any rounding of x0 +- xlim; the pair test decides
  const float x0 = k.r.x, w = 2.0f * k.xlim + 1e-6f * fabsf(x0);
  const float lo = x0 - w, hi = x0 + w;
  if (hi >= 0.0f) {  // x >= 0 part, ascending
    for (uint32_t m = run_abs_lower(run, 0, npos, fmaxf(lo, 0.0f)); m < npos; ++m) {
      const float4 q = run[m];
      if (q.x > hi) break;
      if ((int64_t)m <= skip_to) continue;
      const int32_t b = pair_reaction(p, k, q);
      if (b >= 0) emit<kSingle>(p, c, k, ca, base + m, b);
    }
  }
  if (lo <= 0.0f) {  // x < 0 part, ascending |x|
    for (uint32_t m = run_abs_lower(run, npos, n, fmaxf(-hi, 0.0f)); m < n; ++m) {
      const float4 q = run[m];
      if (fabsf(q.x) > -lo) break;
      if ((int64_t)m <= skip_to) continue;
      const int32_t b = pair_reaction(p, k, q);
      if (b >= 0) emit<kSingle>(p, c, k, ca, base + m, b);
    }
  }
}

// Large cells, part 2 of 2 (k_pairs_big), one CTA per queued cell, on the
// canonical runs left by part 1.  Each pair involving a large cell is
// tested once:
//   * inside the cell, by x sweeps over the run;
//   * with a large neighbour, from the lower-key cell of the two, by x
//     sweeps over the neighbour's run (binary search to |dx| <= radius);
//   * with an ordinary neighbour, here, in either direction, by a loop
//     over its records (k_pairs_cells skips large forward neighbours).
template <bool kBinned>
__device__ void big_pairs(const KParams& p, DevCtrl* c, uint32_t nbig) {
  for (uint32_t bi = blockIdx.x; bi < nbig; bi += gridDim.x) {
    const uint32_t cell = p.big[bi];
    const uint32_t cs = p.cell_start[cell], n = p.cell_start[cell + 1] - cs;
    if ((uint64_t)cs + n > p.capacity) continue;
    const float4* run = p.big_scratch + cs;
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
      Seeker k;
      if (!seeker_init<false>(p, run[i], k)) continue;
      const uint32_t ca = cs + i;
      sweep_sorted<false>(p, c, k, ca, run, n, cs, (int64_t)i);
      const DevInstance& I = p.inst[k.inst];
      const float cl0 = I.cell[0], cl1 = I.cell[1], cl2 = I.cell[2];
      const uint32_t d0 = I.dims[0], d1 = I.dims[1], d2 = I.dims[2];
      const float gx = __fmul_rn(__fsub_rn(k.r.x, I.lo[0]), I.inv[0]);
      const float gy = __fmul_rn(__fsub_rn(k.r.y, I.lo[1]), I.inv[1]);
      const float gz = __fmul_rn(__fsub_rn(k.r.z, I.lo[2]), I.inv[2]);
      const int cx = min(max((int)floorf(gx), 0), (int)d0 - 1);
      const int cy = min(max((int)floorf(gy), 0), (int)d1 - 1);
      const int cz = min(max((int)floorf(gz), 0), (int)d2 - 1);
      const float margin = p.prune_margin * fminf(cl0, fminf(cl1, cl2));
      const float need = k.max_r + margin, need2 = need * need;
      const float fx = __fsub_rn(gx, (float)cx), fy = __fsub_rn(gy, (float)cy), fz = __fsub_rn(gz, (float)cz);
      const float dlo[3] = {fx * cl0, fy * cl1, fz * cl2};
      const float dhi[3] = {(1.0f - fx) * cl0, (1.0f - fy) * cl1, (1.0f - fz) * cl2};
      const int c3[3] = {cx, cy, cz};
      const int dm[3] = {(int)d0, (int)d1, (int)d2};
      int lo3[3], hi3[3];
      for (int a = 0; a < 3; ++a) {
        lo3[a] = (c3[a] > 0 && dlo[a] <= need) ? -1 : 0;
        hi3[a] = (c3[a] + 1 < dm[a] && dhi[a] <= need) ? 1 : 0;
      }
      for (int dz = lo3[2]; dz <= hi3[2]; ++dz) {
        const float ddz = dz < 0 ? dlo[2] : (dz > 0 ? dhi[2] : 0.0f);
        for (int dy = lo3[1]; dy <= hi3[1]; ++dy) {
          const float ddy = dy < 0 ? dlo[1] : (dy > 0 ? dhi[1] : 0.0f);
          for (int dx = lo3[0]; dx <= hi3[0]; ++dx) {
            if (dx == 0 && dy == 0 && dz == 0) continue;
            const float ddx = dx < 0 ? dlo[0] : (dx > 0 ? dhi[0] : 0.0f);
            if (ddx * ddx + ddy * ddy + ddz * ddz > need2) continue;
            const bool forward = dz > 0 || (dz == 0 && (dy > 0 || (dy == 0 && dx > 0)));
            const uint32_t nkey =
                I.cell_base + ((uint32_t)(cz + dz) * d1 + (uint32_t)(cy + dy)) * d0 + (uint32_t)(cx + dx);
            const uint32_t ns = __ldg(&p.cell_start[nkey]), nn = __ldg(&p.cell_start[nkey + 1]) - ns;
            if (nn > kBigCell) {
              if (forward) sweep_sorted<false>(p, c, k, ca, p.big_scratch + ns, nn, ns, -1);
              continue;  // a large lower-key neighbour finds this pair itself
            }
            const CellView nb = cell_records<kBinned>(p, nkey, ns);
            for (uint32_t m = 0; m < nn; ++m) {
              const float4 q = nb.ldg(m);
              const int32_t b = pair_reaction(p, k, q);
              if (b >= 0) emit<false>(p, c, k, ca, ns + canonical_rank(nb, 0, nn, m, q), b);
            }
          }
        }
      }
    }
  }
}

// Large cells: part 1 (sort) by every CTA, a grid barrier, part 2 (pairs)
// by every CTA, in one launch (cooperative when there are pairs to find,
// so that the barrier waits only on resident CTAs).  Every CTA reads the
// same final count of queued cells, so when none is large they all leave
// at once: one empty launch per step instead of two (the two empty
// launches cost 3.3 us per 16M c3 step; the one measured within noise of
// them).  The first step that queues a cell without big_scratch in place
// raises kStatScratch; the host allocates it and replays the step.
template <bool kHasBim, bool kBinned>
__global__ void __launch_bounds__(256) k_pairs_big(KParams p) {
  __shared__ float4 s_rec[kBigChunk];
  DevCtrl* c = p.ctrl;
  if (stop_block(c)) return;
  const uint32_t nbig = min(ld_u32(&c->n_big), p.big_cap);
  if (nbig == 0) return;
  if (p.big_scratch_cap < p.capacity) {
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&c->status, kStatScratch);
    return;
  }
  big_sort<kBinned>(p, c, nbig, s_rec);
  if (!kHasBim) return;
  if (!grid_barrier(c)) return;
  big_pairs<kBinned>(p, c, nbig);
}

// Move the events of the committed step into the cumulative counters.
__device__ __forceinline__ void commit_events(const KParams& p) {
  const uint32_t n = p.n_inst * p.R;
  for (uint32_t e = threadIdx.x; e < n; e += blockDim.x) {
    const unsigned long long v = p.pending[e];
    if (v) {
      p.events[e] += v;
      p.pending[e] = 0;
    }
  }
}

// Candidate pairs above which the matching runs over the whole grid.
constexpr uint32_t kMatchOneCta = 8192;

// Rounds of locally dominant pairs over K candidates, by the threads of one
// CTA (kGrid false: __syncthreads, counters in shared memory) or of the
// whole cooperative grid (kGrid: grid barriers, counters in DevCtrl).
//
// In round r a pending pair (i, j) offers tag(r) | j to best[i] and
// tag(r) | i to best[j] (atomicMin); the pairs that are each other's
// minimum are matched (best = 0 at both ends), and a pending pair with a
// matched end is dropped.  tag(r) falls with r, so values of earlier rounds
// lose every minimum and best needs no reset between rounds: two passes and
// two barriers per round.  The pairs still pending are compacted, with
// their ends, into one of two lists for the next round.  Each round matches
// the smallest pending pair at least, so there are at most K rounds; the
// result is the greedy matching in (lower slot, upper slot) order.
// False when a grid barrier ran out (kStatTimeout is set).
template <bool kGrid>
__device__ bool match_rounds(const KParams& p, DevCtrl* c, uint32_t K, uint32_t* next) {
  DevPair* pr = p.pairs;
  unsigned long long* best = p.best;
  uint4* lists[2] = {p.match_list, p.match_list + p.pair_cap};
  const uint32_t tid = kGrid ? blockIdx.x * blockDim.x + threadIdx.x : threadIdx.x;
  const uint32_t nthr = kGrid ? gridDim.x * blockDim.x : blockDim.x;
  const uint32_t lane = lane_id();
  auto sync = [&]() -> bool {
    if (kGrid) return grid_barrier(c);
    __syncthreads();
    return true;
  };
  // Each thread takes kMatchIlp list entries at a time, so that their
  // loads (entry, then the two matcher words) are in flight together.
  constexpr uint32_t kMatchIlp = 4;
  uint32_t n_pend = K;
  for (uint32_t round = 0; n_pend > 0 && round <= K; ++round) {
    const uint4* in = round == 0 ? nullptr : lists[(round - 1) & 1];
    uint4* out = lists[round & 1];
    const unsigned long long tag = (unsigned long long)(0xFFFFFFFFu - round) << 32;
    const uint32_t span = nthr * kMatchIlp;
    // pass A: offers, except from pairs with an end matched in an earlier round
    for (uint32_t e0 = tid; e0 < n_pend; e0 += span) {
      uint4 ent[kMatchIlp];
      unsigned long long bi[kMatchIlp], bj[kMatchIlp];
#pragma unroll
      for (uint32_t u = 0; u < kMatchIlp; ++u) {
        const uint32_t e = e0 + u * nthr;
        if (e < n_pend) ent[u] = in ? in[e] : make_uint4(e, pr[e].i, pr[e].j, 0u);
      }
#pragma unroll
      for (uint32_t u = 0; u < kMatchIlp; ++u) {
        bi[u] = bj[u] = kFree64;
        if (round > 0 && e0 + u * nthr < n_pend) {
          bi[u] = __ldcg(&best[ent[u].y]);
          bj[u] = __ldcg(&best[ent[u].z]);
        }
      }
#pragma unroll
      for (uint32_t u = 0; u < kMatchIlp; ++u)
        if (e0 + u * nthr < n_pend && bi[u] != 0ull && bj[u] != 0ull) {
          atomicMin(&best[ent[u].y], tag | ent[u].z);
          atomicMin(&best[ent[u].z], tag | ent[u].y);
        }
    }
    if (!sync()) return false;
    // pass B: match mutual minima, drop pairs with a matched end, keep the
    // rest (the loop runs over whole warps: the ballot needs every lane)
    const uint32_t warp_first = tid - lane;
    for (uint32_t e0 = warp_first; e0 < n_pend; e0 += span) {
      uint4 ent[kMatchIlp];
      unsigned long long bi[kMatchIlp], bj[kMatchIlp];
#pragma unroll
      for (uint32_t u = 0; u < kMatchIlp; ++u) {
        const uint32_t e = e0 + u * nthr + lane;
        if (e < n_pend) ent[u] = in ? in[e] : make_uint4(e, pr[e].i, pr[e].j, 0u);
      }
#pragma unroll
      for (uint32_t u = 0; u < kMatchIlp; ++u)
        if (e0 + u * nthr + lane < n_pend) {
          bi[u] = __ldcg(&best[ent[u].y]);
          bj[u] = __ldcg(&best[ent[u].z]);
        }
#pragma unroll
      for (uint32_t u = 0; u < kMatchIlp; ++u) {
        bool keep = false;
        if (e0 + u * nthr + lane < n_pend) {
          if (bi[u] == (tag | ent[u].z) && bj[u] == (tag | ent[u].y)) {
            best[ent[u].y] = 0ull;
            best[ent[u].z] = 0ull;
            pr[ent[u].x].state = 1;
          } else if (bi[u] == 0ull || bj[u] == 0ull) {
            pr[ent[u].x].state = 2;
          } else {
            keep = true;
          }
        }
        // survivors to the next list, one atomic per warp
        const uint32_t ball = __ballot_sync(kFull, keep);
        uint32_t base = 0;
        if (ball && lane == 0) base = atomicAdd(&next[round & 1], (uint32_t)__popc(ball));
        base = __shfl_sync(kFull, base, 0);
        if (keep) out[base + __popc(ball & ((1u << lane) - 1u))] = ent[u];
      }
    }
    if (!sync()) return false;
    n_pend = kGrid ? *(volatile uint32_t*)&next[round & 1] : next[round & 1];
    // The other counter was last read before this round's first barrier,
    // and the next round appends to it only after its own first barrier;
    // this round's counter is reset only after the next round's second
    // barrier, when every thread has read it.  No third barrier is needed.
    if (tid == 0) next[(round + 1) & 1] = 0;
  }
  return true;
}

// Resolve the candidate pairs into a matching, apply the reactions and
// commit the step.  Each particle reacts at most once; the pairs accepted
// are those of the greedy scan in (lower slot, upper slot) order, found in
// parallel as rounds of locally dominant pairs (match_rounds).  Launched
// cooperatively over the grid: with at most kMatchOneCta candidates (most
// steps) CTA 0 does everything and the other CTAs leave at once; with more,
// every CTA takes part in the rounds and the products, and CTA 0 commits.
template <bool kSurf>
__global__ void __launch_bounds__(1024) k_match(KParams p) {
  __shared__ uint32_t s_next[2], s_deaths;
  DevCtrl* c = p.ctrl;
  if (ld_u32(&c->status)) return;
  // read before the barriers below; thread 0 of CTA 0 advances it at the end
  const uint32_t step_now = (uint32_t)*(volatile uint64_t*)&c->step;
  const uint32_t K = ld_u32(&c->n_pairs);
  if (K > p.pair_cap) {
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&c->status, kStatPairs);
    return;
  }
  const bool grid = gridDim.x > 1 && K > kMatchOneCta;  // the same in every CTA
  if (!grid && blockIdx.x != 0) return;
  const uint32_t cur = ld_u32(&c->cur);
  float4* __restrict__ nx = next_state(p, cur);
  DevPair* pr = p.pairs;
  unsigned long long* best = p.best;
  if (threadIdx.x < 2) s_next[threadIdx.x] = 0;
  if (threadIdx.x == 0) s_deaths = 0;
  if (grid) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      c->match_next[0] = c->match_next[1] = 0;
      c->match_deaths = 0;
    }
    if (p.match_withhold && blockIdx.x == 0) return;  // test switch: the other CTAs' waits run out
    if (!grid_barrier(c)) return;
    if (!match_rounds<true>(p, c, K, c->match_next)) return;
  } else {
    __syncthreads();
    match_rounds<false>(p, c, K, s_next);
  }
  const uint32_t tid = grid ? blockIdx.x * blockDim.x + threadIdx.x : threadIdx.x;
  const uint32_t nthr = grid ? gridDim.x * blockDim.x : blockDim.x;

  // products: at the D-weighted reaction point, displaced along a random
  // direction when the reaction has an unbinding radius
  for (uint32_t k = tid; k < K; k += nthr) {
    const DevPair q = pr[k];
    if (q.state != 1) continue;
    const uint32_t inst = q.b >> 16;
    const DevInstance& I = p.inst[inst];
    DevBim br = p.bim[I.block * p.B + (q.b & 0xFFFFu)];
    if (br.next >= 0) {
      // competing reactions of this pair: the one whose share of the
      // pair's summed rate holds the coin
      const uint32_t base_new = p.cell_start[I.cell_base];
      const U4 u = philox(U4{q.i - base_new, p.inst_step[inst], kTagBimChannel, q.j - base_new}, I.key_lo,
                          I.key_hi);
      const float coin = u24_to_unit(u.x);
      for (uint32_t hop = 0; hop < p.B && !(coin < br.thresh) && br.next >= 0; ++hop)
        br = p.bim[I.block * p.B + (uint32_t)br.next];
    }
    const float4 ri = nx[q.i], rj = nx[q.j];
    const bool i_first = (int32_t)(rec_w(ri) & kSpeciesMask) == br.react0;
    const uint32_t m1 = i_first ? q.i : q.j, m2 = i_first ? q.j : q.i;
    const float4 p1 = i_first ? ri : rj, p2 = i_first ? rj : ri;
    const float rx = __fmaf_rn(br.x, p1.x, __fmul_rn(br.omx, p2.x));
    const float ry = __fmaf_rn(br.x, p1.y, __fmul_rn(br.omx, p2.y));
    const float rz = __fmaf_rn(br.x, p1.z, __fmul_rn(br.omx, p2.z));
    float dx = 0.0f, dy = 0.0f, dz = 0.0f;
    if (br.off0 != 0.0f || br.off1 != 0.0f) {
      const uint32_t base_new = p.cell_start[I.cell_base];
      unit_vector(q.i - base_new, p.inst_step[inst], kTagBimDir, q.j - base_new, I.key_lo, I.key_hi, dx, dy,
                  dz);
    }
    uint32_t dead = 0;
    const float4 none = make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(kDead));
    float4 n1 = none, n2 = none;
    // each product moves from the reaction point by its offset, through the
    // surfaces when there are any, then the walls
    auto place = [&](int32_t prod, float off, float4& out) {
      if (prod < 0) {
        ++dead;
        return;
      }
      float ex = reflect(__fmaf_rn(off, dx, rx), I.lo[0], I.hi[0]);
      float ey = reflect(__fmaf_rn(off, dy, ry), I.lo[1], I.hi[1]);
      float ez = reflect(__fmaf_rn(off, dz, rz), I.lo[2], I.hi[2]);
      if (kSurf && off != 0.0f && !surface_walk(p, I, (uint32_t)prod, V3{rx, ry, rz}, ex, ey, ez)) {
        ++dead;
        return;
      }
      out = make_float4(ex, ey, ez, __uint_as_float(pack_w(inst, (uint32_t)prod)));
    };
    place(br.prod0, br.off0, n1);
    place(br.prod1, br.off1, n2);
    nx[m1] = n1;
    nx[m2] = n2;
    atomicAdd(&p.pending[(size_t)inst * p.R + br.rxn], 1ull);
    if (dead) atomicAdd(&s_deaths, dead);
  }
  for (uint32_t k = tid; k < K; k += nthr) {
    best[pr[k].i] = kFree64;
    best[pr[k].j] = kFree64;
  }
  __syncthreads();
  if (grid) {
    // every CTA's products and deaths are in before CTA 0 commits
    if (threadIdx.x == 0 && s_deaths) atomicAdd(&c->match_deaths, s_deaths);
    if (!grid_barrier(c)) return;
    if (blockIdx.x != 0) return;
    if (threadIdx.x == 0) s_deaths = *(volatile uint32_t*)&c->match_deaths;
    __syncthreads();
  }
  commit_events(p);
  for (uint32_t inst = threadIdx.x; inst < p.n_inst; inst += blockDim.x) {
    const DevInstance& I = p.inst[inst];
    advance_instance_step(p, inst, step_now);
    p.inst_slot_base[inst] = p.cell_start[I.cell_base];
  }
  if (threadIdx.x == 0) {
    c->n_pairs_last = K;
    c->n_pairs = 0;
    c->n_big = 0;
    c->n_surf = 0;
    c->surf_ticket = 0;
    c->deaths_last = s_deaths;
    c->n_slots = c->n_sorted;
    c->n_virtual = 0;
    c->cur = cur ^ 1u;
    c->step += 1;
    c->steps_done += 1;
  }
}

template <bool kTable>
__global__ void __launch_bounds__(256) k_diffuse(KParams p) {
  const DevCtrl* c = p.ctrl;
  if (ctrl_status_warp(c)) return;
  const uint32_t cur = ld_u32(&c->cur);
  float4* st = cur ? p.state[1] : p.state[0];
  const uint32_t n = ld_u32(&c->n_slots);
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    Out2 o;
    advance_rec<kTable, false, false>(p, SingleCtx{}, st[i], i, o);
    if (o.n > 0) st[i] = o.r[0];
  }
}

__global__ void __launch_bounds__(256) k_append(KParams p) {
  const DevCtrl* c = p.ctrl;
  if (ctrl_status_warp(c)) return;
  const uint32_t cur = ld_u32(&c->cur);
  float4* st = cur ? p.state[1] : p.state[0];
  const uint32_t n = ld_u32(&c->n_slots), nv = ld_u32(&c->n_virtual);
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += stride) {
    Out2 o;
    advance_virtual<false>(p, v, o);
    st[n + v] = make_float4(o.r[0].x, o.r[0].y, o.r[0].z, __uint_as_float(rec_w(o.r[0]) & ~kNewborn));
  }
}

__global__ void k_finalize_inplace(KParams p) {
  DevCtrl* c = p.ctrl;
  if (ld_u32(&c->status)) return;
  const uint32_t step_now = (uint32_t)*(volatile uint64_t*)&c->step;
  commit_events(p);
  for (uint32_t inst = threadIdx.x; inst < p.n_inst; inst += blockDim.x) advance_instance_step(p, inst, step_now);
  __syncthreads();  // every thread has read the step before thread 0 advances it
  if (threadIdx.x == 0) {
    c->n_slots += c->n_virtual;
    c->n_virtual = 0;
    c->n_pairs_last = 0;
    c->deaths_last = 0;
    c->step += 1;
    c->steps_done += 1;
  }
}

__global__ void __launch_bounds__(256) k_instance_counts(KParams p, unsigned long long* counts) {
  const DevCtrl* c = p.ctrl;
  const uint32_t cur = ld_u32(&c->cur);
  const float4* st = cur_state(p, cur);
  const uint32_t n = ld_u32(&c->n_slots);
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
    const uint32_t i = base + threadIdx.x;
    uint32_t key = kNoKey;
    if (i < n) {
      const uint32_t w = rec_w(st[i]);
      if (w != kDead) key = w >> 16;
    }
    const uint32_t peers = __match_any_sync(kFull, key);
    if (key != kNoKey && lane_id() == (uint32_t)(__ffs(peers) - 1))
      atomicAdd(&counts[key], (unsigned long long)__popc(peers));
  }
}

__global__ void __launch_bounds__(256) k_species_counts(KParams p, unsigned long long* counts) {
  const DevCtrl* c = p.ctrl;
  const uint32_t cur = ld_u32(&c->cur);
  const float4* st = cur_state(p, cur);
  const uint32_t n = ld_u32(&c->n_slots);
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
    const uint32_t i = base + threadIdx.x;
    uint32_t key = kNoKey;
    if (i < n) {
      const uint32_t w = rec_w(st[i]);
      if (w != kDead) key = (w >> 16) * p.S + (w & kSpeciesMask);
    }
    const uint32_t peers = __match_any_sync(kFull, key);
    if (key != kNoKey && lane_id() == (uint32_t)(__ffs(peers) - 1))
      atomicAdd(&counts[key], (unsigned long long)__popc(peers));
  }
}

// Squared diffusion moves of the coming step, summed per (instance,
// species): the step's own Philox counters, normals and wall reflections
// (advance_rec, before its reactions), read only.  An observable
// (bd_measure_msd), launched before a step, not part of it.  Sums go
// through shared memory when the (instance, species) table fits.
constexpr uint32_t kMsdShared = 512;

template <bool kTable>
__global__ void __launch_bounds__(256) k_msd(KParams p, double* sum, unsigned long long* cnt) {
  __shared__ double s_sum[kMsdShared];
  __shared__ unsigned long long s_cnt[kMsdShared];
  const DevCtrl* c = p.ctrl;
  if (ld_u32(&c->status)) return;  // the step will not run: nothing to measure
  const uint32_t keys = p.n_inst * p.S;
  const bool in_smem = keys <= kMsdShared;
  if (in_smem)
    for (uint32_t k = threadIdx.x; k < keys; k += blockDim.x) {
      s_sum[k] = 0.0;
      s_cnt[k] = 0ull;
    }
  __syncthreads();
  const uint32_t cur = ld_u32(&c->cur);
  const float4* st = cur_state(p, cur);
  const uint32_t n = ld_u32(&c->n_slots);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 rec = st[i];
    const uint32_t w = rec_w(rec);
    if (w == kDead) continue;
    const uint32_t inst = w >> 16, sp = w & kSpeciesMask;
    if (!advancing(p.inst_flags[inst])) continue;
    const DevInstance& I = p.inst[inst];
    const uint32_t local = i - p.inst_slot_base[inst];
    const float sigma = p.species[I.block * p.S + sp].sigma;
    const U4 rn = philox(U4{local, p.inst_step[inst], kTagDiffuse, 0u}, I.key_lo, I.key_hi);
    float g0, g1, g2;
    normals3<kTable>(rn, p.gauss, g0, g1, g2);
    const double dx = (double)reflect(__fmaf_rn(sigma, g0, rec.x), I.lo[0], I.hi[0]) - rec.x;
    const double dy = (double)reflect(__fmaf_rn(sigma, g1, rec.y), I.lo[1], I.hi[1]) - rec.y;
    const double dz = (double)reflect(__fmaf_rn(sigma, g2, rec.z), I.lo[2], I.hi[2]) - rec.z;
    const double d2 = dx * dx + dy * dy + dz * dz;
    const uint32_t key = inst * p.S + sp;
    if (in_smem) {
      atomicAdd(&s_sum[key], d2);
      atomicAdd(&s_cnt[key], 1ull);
    } else {
      atomicAdd(&sum[key], d2);
      atomicAdd(&cnt[key], 1ull);
    }
  }
  __syncthreads();
  if (in_smem)
    for (uint32_t k = threadIdx.x; k < keys; k += blockDim.x)
      if (s_cnt[k]) {
        atomicAdd(&sum[k], s_sum[k]);
        atomicAdd(&cnt[k], s_cnt[k]);
      }
}

}  // namespace

// The matcher, cooperatively over shape.grid_match CTAs (all resident, so
// its grid barriers cannot wait on a CTA that never runs).
void launch_match(const KParams& p, const LaunchShape& shape, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(shape.grid_match > 1 ? shape.grid_match : 1));
  cfg.blockDim = dim3(1024);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr;
  attr.id = cudaLaunchAttributeCooperative;
  attr.val.cooperative = 1;
  cfg.attrs = &attr;
  cfg.numAttrs = shape.grid_match > 1 ? 1 : 0;
  if (p.n_panels) cudaLaunchKernelEx(&cfg, k_match<true>, p);
  else cudaLaunchKernelEx(&cfg, k_match<false>, p);
}

// The large-cell kernel over shape.grid_big CTAs, cooperatively when it
// has pairs to find (its grid barrier waits only on resident CTAs).
void launch_big(const KParams& p, bool has_bim, bool binned, const LaunchShape& shape, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)std::max(shape.grid_big, 1));
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr;
  attr.id = cudaLaunchAttributeCooperative;
  attr.val.cooperative = 1;
  cfg.attrs = &attr;
  cfg.numAttrs = has_bim && shape.grid_big > 1 ? 1 : 0;
  if (has_bim) {
    if (binned) cudaLaunchKernelEx(&cfg, k_pairs_big<true, true>, p);
    else cudaLaunchKernelEx(&cfg, k_pairs_big<true, false>, p);
  } else {
    if (binned) cudaLaunchKernelEx(&cfg, k_pairs_big<false, true>, p);
    else cudaLaunchKernelEx(&cfg, k_pairs_big<false, false>, p);
  }
}

// The cell scan, cooperatively over at most shape.grid_scan CTAs (all
// resident) and at most one per kScanTile cells.
void launch_scan(const KParams& p, const LaunchShape& shape, cudaStream_t s) {
  const uint32_t g = std::max(1u, std::min((uint32_t)std::max(shape.grid_scan, 1), p.n_tiles));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(g);
  cfg.blockDim = dim3(1024);
  cfg.dynamicSmemBytes = kScanSmem;
  cfg.stream = s;
  cudaLaunchAttribute attr;
  attr.id = cudaLaunchAttributeCooperative;
  attr.val.cooperative = 1;
  cfg.attrs = &attr;
  cfg.numAttrs = g > 1 ? 1 : 0;
  cudaLaunchKernelEx(&cfg, k_scan, p);
}

int enqueue_step(const KParams& p, Path path, bool table, bool has_zero, bool has_uni, bool has_bim,
                 const LaunchShape& shape, cudaStream_t s, StageHook hook, void* ctx) {
  (void)has_uni;
  const int gs = shape.grid_stream, bs = shape.block_stream;
  int n = 0;
  auto done = [&](const char* name) {
    ++n;
    if (hook) hook(ctx, name);
  };
  if (has_zero) {
    k_zeroth<<<1, 1024, 0, s>>>(p, path == Path::kDiffuseOnly ? 1 : 0);
    done("k_zeroth");
  }
  if (path == Path::kDiffuseOnly) {
    if (table) k_diffuse<true><<<gs, bs, 0, s>>>(p);
    else k_diffuse<false><<<gs, bs, 0, s>>>(p);
    done("k_diffuse");
    if (has_zero) {
      k_append<<<gs, bs, 0, s>>>(p);
      done("k_append");
    }
    k_finalize_inplace<<<1, 256, 0, s>>>(p);
    done("k_finalize_inplace");
    return n;
  }
  // Register-capped variants of the streaming kernels, picked by the launch
  // shape's resident CTAs per SM: 1 = no cap, 4 = 64 registers, 6 = 40.
#define BD_STREAM_LAUNCH3(KERNEL, MINB, SURF)                                              \
  do {                                                                                     \
    if (single) {                                                                          \
      if (table) KERNEL<true, MINB, true, SURF><<<gs, bs, 0, s>>>(p);                       \
      else KERNEL<false, MINB, true, SURF><<<gs, bs, 0, s>>>(p);                            \
    } else {                                                                               \
      if (table) KERNEL<true, MINB, false, SURF><<<gs, bs, 0, s>>>(p);                      \
      else KERNEL<false, MINB, false, SURF><<<gs, bs, 0, s>>>(p);                           \
    }                                                                                      \
  } while (0)
  // With surfaces: one variant per kernel, no register cap.
#define BD_STREAM_LAUNCH(KERNEL, SURF)                   \
  do {                                                   \
    switch (shape.min_blocks) {                          \
      case 6: BD_STREAM_LAUNCH3(KERNEL, 6, SURF); break; \
      case 4: BD_STREAM_LAUNCH3(KERNEL, 4, SURF); break; \
      default: BD_STREAM_LAUNCH3(KERNEL, 1, SURF);       \
    }                                                    \
  } while (0)
  // The compact path walks the surfaces inline: one variant per kernel, no
  // register cap.
#define BD_STREAM_LAUNCH_COMPACT(KERNEL)          \
  do {                                            \
    if (p.n_panels) BD_STREAM_LAUNCH3(KERNEL, 1, 1); \
    else BD_STREAM_LAUNCH(KERNEL, 0);             \
  } while (0)
#define BD_PAIRS_LAUNCH(BINNED, STAGE)                                                               \
  do {                                                                                               \
    if (single) {                                                                                    \
      if (has_bim) k_pairs_cells<true, BINNED, true, STAGE><<<shape.grid_pairs, 256, 0, s>>>(p);  \
      else k_pairs_cells<false, BINNED, true, STAGE><<<shape.grid_pairs, 256, 0, s>>>(p);         \
    } else {                                                                                         \
      if (has_bim) k_pairs_cells<true, BINNED, false, STAGE><<<shape.grid_pairs, 256, 0, s>>>(p); \
      else k_pairs_cells<false, BINNED, false, STAGE><<<shape.grid_pairs, 256, 0, s>>>(p);        \
    }                                                                                                \
  } while (0)
  const bool single = p.n_inst == 1 && p.S <= kCtxSpecies && p.U <= kCtxUni;
  if (path == Path::kBinned) {
    if (p.n_panels) {
      BD_STREAM_LAUNCH(k_bin, 2);
      done("k_bin");
      if (single) {
        if (table) k_bin_surface<true, true><<<gs, bs, 0, s>>>(p);
        else k_bin_surface<false, true><<<gs, bs, 0, s>>>(p);
      } else {
        if (table) k_bin_surface<true, false><<<gs, bs, 0, s>>>(p);
        else k_bin_surface<false, false><<<gs, bs, 0, s>>>(p);
      }
      done("k_bin_surface");
    } else {
      BD_STREAM_LAUNCH(k_bin, 0);
      done("k_bin");
    }
    launch_scan(p, shape, s);
    done("k_scan");
    BD_PAIRS_LAUNCH(true, kStagePairs);
    done("k_pairs_cells");
    launch_big(p, has_bim, true, shape, s);
    done("k_pairs_big");
    launch_match(p, shape, s);
    done("k_match");
    return n;
  }
  BD_STREAM_LAUNCH_COMPACT(k_count);
  done("k_count");
  launch_scan(p, shape, s);
  done("k_scan");
  BD_STREAM_LAUNCH_COMPACT(k_scatter);
  done("k_scatter");
  BD_PAIRS_LAUNCH(false, false);
  done("k_pairs_cells");
#undef BD_STREAM_LAUNCH
#undef BD_STREAM_LAUNCH_COMPACT
#undef BD_STREAM_LAUNCH3
#undef BD_PAIRS_LAUNCH
  launch_big(p, has_bim, false, shape, s);
  done("k_pairs_big");
  launch_match(p, shape, s);
  done("k_match");
  return n;
}

void enqueue_instance_counts(const KParams& p, unsigned long long* counts, cudaStream_t s) {
  k_instance_counts<<<152 * 4, 256, 0, s>>>(p, counts);
}

// At most kMatchGrid CTAs: on the dense smoke step (24,509 candidates, 119
// rounds) 32 CTAs took 0.985 ms against 1.06 ms for 152 (one per SM) and
// 1.07 ms for 16, and a grid launch costs the small-K steps of c3 about
// 2 us over a single CTA (14.3 against 12.3 us) with 16 to 64 CTAs, 4 us
// with 152.
constexpr int kMatchGrid = 32;

int match_grid(int n_sm) {
  int a = 0, b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_match<false>, 1024, 0) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_match<true>, 1024, 0) != cudaSuccess)
    return 1;
  const int per_sm = a < b ? a : b;
  const int resident = per_sm > 0 ? per_sm * n_sm : 1;
  return resident < kMatchGrid ? resident : kMatchGrid;
}

int big_grid(int n_sm) {
  int a = 0, b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_pairs_big<true, true>, 256, 0) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_pairs_big<true, false>, 256, 0) != cudaSuccess)
    return 1;
  const int resident = (a < b ? a : b) * n_sm;
  return resident < 1 ? 1 : (resident < kBigGrid ? resident : kBigGrid);
}

int scan_grid(int n_sm) {
  int a = 0;
  if (cudaFuncSetAttribute(k_scan, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kScanSmem) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_scan, 1024, kScanSmem) != cudaSuccess || a < 1)
    return 0;
  return a * n_sm;
}

void enqueue_species_counts(const KParams& p, unsigned long long* counts, cudaStream_t s) {
  k_species_counts<<<152 * 4, 256, 0, s>>>(p, counts);
}

void enqueue_msd(const KParams& p, bool table, double* sum, unsigned long long* counts, cudaStream_t s) {
  if (table) k_msd<true><<<152 * 4, 256, 0, s>>>(p, sum, counts);
  else k_msd<false><<<152 * 4, 256, 0, s>>>(p, sum, counts);
}

}  // namespace bd
