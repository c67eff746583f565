// bd_kernels.h -- launch interface of the step kernels (host side).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "bd_layout.h"

namespace bd {

// Everything a step kernel reads or writes, passed by value.
struct KParams {
  float4* state[2];           // ping-pong state buffers, DevCtrl::cur selects
  float4* scatter;            // cell-ordered staging buffer of the compact sort
  float4* bins;               // [n_cells][bin_cap] records per cell (binned sort)
  DevCtrl* ctrl;
  const DevInstance* inst;
  DevInstance inst0;          // copy of instance 0 (kernels specialised for one instance)
  const DevSpecies* species;  // [block][S]
  const DevUni* uni;          // [block][U]
  const DevBim* bim;          // [block][B]
  const DevZero* zero;        // [block][Z]
  const double* cdf;          // Poisson CDFs (absolute offsets in DevZero)
  const int32_t* bim_table;   // [S][S] -> local second-order index or -1
  const float* gauss;         // 4096 N(0,1) quantiles (table mode)
  uint32_t* inst_step;        // [I] steps taken by each instance
  uint32_t* inst_flags;       // [I] InstanceFlags (frozen on device at the target)
  const uint32_t* inst_target;// [I] step count at which an instance freezes
  uint32_t* inst_frozen;      // [I] global step (low 32 bits) at which an instance froze
  uint32_t* inst_slot_base;   // [I] first slot of each instance in the current state
  uint32_t* zero_off;         // [I*Z + 1] prefix of zeroth-order births
  DevZero zero0[4];           // instance 0's zeroth-order entries when Z <= 4 (k_zeroth's one-instance path)
  uint32_t* cell_count;       // [n_cells] particles per cell (returns to 0 each step)
  uint32_t* cell_start;       // [n_cells + 1] exclusive prefix of cell_count
  uint32_t* tile_sums;        // [n_tiles] the cell scan's per-CTA sums
  uint32_t scan_withhold;     // test switch: CTA 0 of the cell scan never reaches its grid barrier
  uint32_t match_withhold;    // test switch: CTA 0 of the grid matcher never arrives (the others time out)
  DevPair* pairs;             // [pair_cap]
  unsigned long long* best;   // [capacity] matcher words, all ones between steps
  uint4* match_list;          // [2 * pair_cap] pending pairs (index, ends) of the matcher's rounds
  unsigned long long* events; // [I * R] reaction event counters (committed steps)
  unsigned long long* pending;// [I * R] events of the step in flight, added at commit
  uint32_t n_inst, S, U, B, Z, R;
  uint32_t n_cells, n_tiles;
  uint32_t capacity, pair_cap;
  uint32_t bin_cap;           // records per cell bin (binned sort)
  uint32_t* big;              // [big_cap] cells queued for k_pairs_big
  float4* big_scratch;        // [big_scratch_cap] merge-sort buffer of k_pairs_big
  uint32_t big_cap, big_scratch_cap;
  float prune_margin;         // fraction of a cell edge added to pruning distances
  // surfaces (n_panels = 0: none)
  const DevPanel* panels;     // [n_panels]
  const uint8_t* surf_act;    // [n_surfaces][S][2] SurfaceAction per (species, front/back face)
  const uint32_t* pbox_start; // [n_pbox + 1] panel lists of the coarse panel grid
  const uint32_t* pbox_list;  // panel ids, box by box
  float pbox_lo[3], pbox_inv[3];
  uint32_t pbox_dims[3];
  uint32_t n_panels;
  uint32_t* surf_queue;       // [capacity] slots whose move may meet a panel (k_bin -> k_bin_surface)
  const uint8_t* cell_surf;   // [n_cells] species masks: a step starting here may meet a panel (species_bit)
};

// kSorted: counting sort into compact cell ranges (k_count, scans,
// k_scatter) before the pair kernel.  kBinned: each record goes straight
// into a fixed-size bin of its cell (k_bin), the scans give the compact
// output ranges and the pair kernel reads the bins.  Same results.
enum class Path { kDiffuseOnly, kSorted, kBinned };

struct LaunchShape {
  int grid_stream;            // blocks of the grid-stride particle kernels
  int block_stream;           // threads per block of those kernels
  int grid_pairs, block_pairs;
  int min_blocks;             // register-capped streaming kernels: 1 (none), 4 (64 regs), 6 (40 regs)
  int grid_match;             // CTAs of the cooperative matcher (1 = one CTA, plain launch)
  int grid_scan;              // most CTAs of the cooperative cell scan (all resident)
  int grid_big;               // CTAs of the large-cell kernel (all resident)
};

// CTAs of 1024 threads that the matcher can keep resident on n_sm SMs (the
// size of its cooperative launch).
int match_grid(int n_sm);
// CTAs of 1024 threads that the cell scan can keep resident on n_sm SMs.
int scan_grid(int n_sm);
// CTAs of the large-cell kernel: at most 304, all resident on n_sm SMs.
int big_grid(int n_sm);

// Called after each kernel of a step is enqueued (stage name); lets the
// profiler record an event between kernels.  nullptr = no callback.
typedef void (*StageHook)(void* ctx, const char* stage);

// Enqueue one full step on `stream`.  table selects the normal generator.
// Returns the number of kernels enqueued.
int enqueue_step(const KParams& p, Path path, bool table, bool has_zero, bool has_uni, bool has_bim,
                 const LaunchShape& shape, cudaStream_t stream, StageHook hook = nullptr, void* ctx = nullptr);

// Count live records per instance (counts[I] must be zeroed).
void enqueue_instance_counts(const KParams& p, unsigned long long* counts, cudaStream_t stream);
// Count live records per (instance, species): counts[I * S] must be zeroed.
void enqueue_species_counts(const KParams& p, unsigned long long* counts, cudaStream_t stream);
// Squared diffusion moves of the coming step per (instance, species), added
// into sum / counts (bd_measure_msd).
void enqueue_msd(const KParams& p, bool table, double* sum, unsigned long long* counts, cudaStream_t stream);

// Tile size of the cell scan.
constexpr uint32_t kScanTile = 8192;

// Places of a cell bin stored together (64 bytes); the bin capacity is a
// multiple of it.
constexpr uint32_t kBinGroup = 4;

}  // namespace bd
