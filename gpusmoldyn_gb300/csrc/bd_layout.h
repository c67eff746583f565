// bd_layout.h -- device-side data layout of one simulation handle, shared by
// the host packer (bd_api.cpp) and the kernels (bd_kernels.cu).
//
// Particle record: one float4 per slot, x, y, z and a 32-bit word w holding
// species (bits 0-14) and instance (bits 16-31); w = 0xFFFFFFFF marks an empty
// slot (a particle that died in the bimolecular phase).  The reference keeps
// positions (float4, w = radius/flag) and types (int) in two arrays
// (particleSystem.h:151-152, 204-205); one 16-byte record halves the number
// of memory transactions per particle.
//
// Parameters live in "blocks": one block per ensemble instance (a single
// system has one).  Every block has the same shape (species S, first-order
// reactions U, second-order reactions B, zeroth-order reactions Z) because
// the instances of an ensemble share one reaction network and differ only in
// numbers.  The second-order lookup table (S x S -> local reaction index) is
// shared by all blocks, like the reference's reactionTable
// (particleSystem.cpp:653-673).
#pragma once
#include <stdint.h>

namespace bd {

constexpr uint32_t kDead = 0xFFFFFFFFu;
// Bit 15 of w marks a particle born in the step in flight (second product
// of a first-order reaction, zeroth-order birth).  It exists only between
// the scatter and the pair kernel: newborns are sorted into their cells but
// take no part in that step's bimolecular search, as the reference appends
// them only after collide (particleSystem.cpp:984-991).
constexpr uint32_t kNewborn = 0x8000u;
constexpr uint32_t kSpeciesMask = 0x7FFFu;
constexpr uint32_t kMaxSpecies = 0x7FFEu;
constexpr uint32_t kMaxInstances = 0xFFFFu;

// Philox counter word 2 carries a stream tag in its top byte.
enum StreamTag : uint32_t {
  kTagDiffuse = 1u << 24,   // 3 normals per particle per step
  kTagUniCoin = 2u << 24,   // first-order coins, 4 per counter (low bits = k/4)
  kTagUniDir = 3u << 24,    // product direction of a first-order birth
  kTagZeroCount = 4u << 24, // Poisson count of one zeroth-order reaction
  kTagZeroPos = 5u << 24,   // position of one zeroth-order birth
  kTagBimCoin = 6u << 24,   // coin of one candidate pair
  kTagBimDir = 7u << 24,    // product direction of one accepted pair
  kTagBimChannel = 8u << 24,// which competing reaction an accepted pair fires
};

struct DevSpecies {        // 16 B
  float sigma;             // rms step per axis, sqrt(2 D dt) (molSetTimestep)
  float max_r;             // largest binding radius over this species' pairs (0 = inert)
  uint32_t uni_begin;      // first-order reactions of this species: [begin, begin+count)
  uint32_t uni_count;      // in the block's DevUni array (reactionOrderInfo[1] CSR)
};

struct DevUni {            // 32 B
  float prob;              // conditional per-step probability (rxnsetrate order 1)
  int32_t prod0, prod1;    // product species, -1 = none (prod0 < 0: decay)
  float off0, off1;        // product displacements along a random unit vector
  uint32_t rxn;            // global reaction index (event counters)
  uint32_t pad[2];
};

struct DevBim {            // 48 B
  float r2;                // squared binding radius
  float prob;              // reaction probability once within r2 (1 = always)
  float x, omx;            // reaction point x*p1 + omx*p2 (p1 = first reactant)
  int32_t react0;          // species of the first reactant
  int32_t prod0, prod1;    // product species, -1 = none
  float off0, off1;        // product displacements along a random unit vector
  uint32_t rxn;            // global reaction index
  float thresh;            // competing reactions: cumulative share of the pair's rate
  int32_t next;            // next competing reaction of the pair (local index), -1 = last
};

struct DevZero {           // 32 B
  int32_t prod0, prod1;    // product species (prod1 = -1 for one product)
  uint32_t cdf_off;        // offset of the Poisson CDF in the block's CDF array
  uint32_t cdf_len;        // entries: P(X <= kmin + k), k = 0..len-1
  int32_t kmin;
  uint32_t rxn;            // global reaction index
  uint32_t pad[2];
};

enum InstanceFlags : uint32_t {
  kInstActive = 1u,        // advanced every step
  kInstFrozen = 2u,        // kept in place, not advanced (finished request)
  kInstRemoved = 4u,       // dropped at the next sort
};

struct DevInstance {       // 80 B
  float lo[3], hi[3];      // reflecting box
  float inv[3];            // cells per unit length per axis
  float cell[3];           // cell edge per axis
  uint32_t dims[3];        // cells per axis
  uint32_t cell_base;      // first global cell key of this instance
  uint32_t key_lo, key_hi; // Philox key (instance seed)
  uint32_t block;          // parameter block
  uint32_t flags;          // InstanceFlags
};

// Mutable per-step control words, one per handle, in device memory.
struct DevCtrl {
  uint32_t cur;            // state buffer holding the current step (0/1)
  uint32_t n_slots;        // slots of the current state (holes included)
  uint32_t n_virtual;      // zeroth-order births of the step in flight
  uint32_t n_sorted;       // slots of the next state
  uint32_t n_pairs;        // candidate pairs appended by the pair kernel
  uint32_t n_pairs_last;   // candidate pairs of the last completed step
  uint32_t status;         // StatusBits, 0 = healthy
  uint32_t steps_done;     // completed steps since the last host reset
  uint64_t step;           // global step counter
  uint32_t deaths_last;    // bimolecular deaths of the last step
  uint32_t bin_need;       // largest cell occupancy seen by a bin that overflowed
  uint32_t n_big;          // cells queued for the large-cell pair kernel
  uint32_t n_surf;         // records whose move meets a panel box (binned path with surfaces)
  uint32_t surf_ticket;    // queued records taken by k_bin_surface in the step in flight
  // the grid barrier (cell scan; k_match over the whole grid when a step
  // has many candidate pairs): arrival count and generation; the matcher's
  // pending-pair counts of two rounds and the bimolecular deaths of the step
  uint32_t bar_count, bar_gen;
  uint32_t match_next[2];
  uint32_t match_deaths;
};

enum StatusBits : uint32_t {
  kStatCapacity = 1u,      // next state would exceed the slot capacity
  kStatPairs = 2u,         // candidate pairs exceed the pair capacity
  kStatBounds = 4u,        // a device-side bounds check failed
  kStatTimeout = 8u,       // a bounded wait ran out
  kStatBins = 16u,         // a cell held more records than its bin
  kStatScratch = 32u,      // the large-cell kernel needs its sort buffer
};

// Surface panels.  The shape codes and the field meanings are those of the
// public bd_panel_info (one float/int per field, same order), so the host
// fills a DevPanel by copying a bd_panel_info.
enum PanelShape : uint32_t { kPanelRect = 0, kPanelTri = 1, kPanelSph = 2, kPanelCyl = 3, kPanelHemi = 4,
                             kPanelDisk = 5 };
enum SurfaceAction : uint8_t { kActTransmit = 0, kActReflect = 1, kActAbsorb = 2 };
constexpr int kMaxSurfaceHits = 8;  // crossings handled per segment and step

struct DevPanel {          // 96 B
  uint32_t shape;          // PanelShape
  uint32_t surface;        // owning surface (index of its action table)
  uint32_t axis;           // rect: axis perpendicular to the panel
  float front;             // +1 / -1: which way the front face looks
  float a[3];              // rect corner, tri v0, sph/hemi/disk centre, cyl end 0
  float r, r2;             // radius and its square
  float n[3];              // tri/disk unit front normal, cyl unit axis, hemi unit opening direction
  float len;               // cyl axis length
  float v1[3], v2[3];      // tri vertices 1 and 2
  float bounds[4];         // rect: lower in-plane axis lo, hi; higher one lo, hi
  uint32_t pad;
};

// Pair list entry written by the pair kernel and resolved by the matcher.
struct DevPair {           // 16 B
  uint32_t i, j;           // canonical slots, i < j
  uint32_t b;              // local second-order reaction index | instance << 16
  uint32_t state;          // 0 undecided, 1 accepted, 2 rejected
};

}  // namespace bd
