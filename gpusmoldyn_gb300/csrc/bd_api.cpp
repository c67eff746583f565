// bd_api.cpp -- implementation of the C ABI declared in include/gpusmoldyn.h.
//
// The handle owns the reaction network, the derived parameter blocks, every
// device buffer and a CUDA graph of one (and of kGraphBatch) timesteps.  A
// step never synchronises with the host: counts, capacity checks and the
// step counter live in a device control block, so bd_step only launches
// graphs.  bd_synchronize is where the host looks at the control block,
// grows buffers after an overflow and replays the steps that did not commit
// (a step that overflows writes only into buffers that the next attempt
// overwrites, so replay is exact).
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <initializer_list>
#include <string>
#include <vector>

#include "../../include/gpusmoldyn.h"
#include "bd_io.h"
#include "bd_kernels.h"
#include "bd_layout.h"
#include "bd_params.h"
#include "bd_surface.h"

using namespace bd;

namespace {

constexpr int kGraphBatch = 16;
// Largest bin array the automatic sort mode accepts.
constexpr uint64_t kBinBudgetBytes = 32ull << 30;

thread_local std::string g_last_error;

bool cuda_ok(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
  return false;
}

// NVTX range over one C-ABI call (host timeline of nsys / ncu; a no-op
// without a tool attached).  The step graphs' kernels carry their own names.
struct Range {
  explicit Range(const char* name) { nvtxRangePushA(name); }
  ~Range() { nvtxRangePop(); }
  Range(const Range&) = delete;
  Range& operator=(const Range&) = delete;
};

#define BD_CUDA(call)                                   \
  do {                                                  \
    if (!cuda_ok((call), #call)) return BD_ERR_CUDA;    \
  } while (0)

template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  cudaError_t alloc(size_t count) {
    free();
    n = count;
    if (count == 0) return cudaSuccess;
    return cudaMalloc((void**)&p, count * sizeof(T));
  }
  void free() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

}  // namespace

struct bd_system {
  bd_config cfg{};
  std::vector<bd_instance_desc> idesc;
  std::vector<float> D;
  std::vector<ReactionDef> rx;
  std::vector<std::string> species_names, reaction_names;  // optional, "" when unnamed
  bool finalized = false;
  std::vector<DerivedParams> derived;  // one per instance (= parameter block)

  // network shape
  int S = 0, U = 0, B = 0, Z = 0, R = 0;
  std::vector<int> uni_list;    // order-1 reactions grouped by reactant
  std::vector<int> bim_list;    // order-2 reactions, local index -> global
  std::vector<int> zero_list;   // order-0 reactions
  std::vector<int32_t> bim_table;
  bool zero_two_products = false;

  // surfaces: per surface the action of every species not set one by one
  // (BD_ALL_SPECIES) and the per-species settings (-1 = that default), for
  // the front and the back face
  struct Surface {
    uint8_t all[2] = {kActTransmit, kActTransmit};
    std::vector<int16_t> species[2];
  };
  std::vector<Surface> surfaces;
  std::vector<bd_panel_info> panels;
  DevBuf<DevPanel> dpanels;
  DevBuf<uint8_t> dsurf_act;
  DevBuf<uint32_t> dpbox_start, dpbox_list;
  DevBuf<uint32_t> surf_queue;  // [capacity] when there are panels
  DevBuf<uint8_t> dcell_surf;    // [n_cells] species masks of the cells near panels
  std::vector<uint8_t> panel_species;  // per panel: species_bit of every species whose step may meet it
  PanelGrid pgrid{};

  // device
  int device = 0, n_sm = 152;
  cudaStream_t stream = nullptr;
  DevBuf<DevCtrl> ctrl;
  DevCtrl* hctrl = nullptr;  // pinned mirror
  DevBuf<DevInstance> dinst;
  DevBuf<DevSpecies> dspecies;
  DevBuf<DevUni> duni;
  DevBuf<DevBim> dbim;
  DevBuf<DevZero> dzero;
  std::vector<DevZero> hzero;  // host copy of dzero
  DevBuf<double> dcdf;
  DevBuf<int32_t> dtable;
  DevBuf<float> dgauss;
  DevBuf<uint32_t> inst_step, inst_slot_base, zero_off;
  DevBuf<unsigned long long> events, pending;
  DevBuf<float4> state0, state1, scatter, bins;
  cudaMemPool_t pool = nullptr;  // stream-ordered scratch of host transfers (keeps its memory)
  DevBuf<unsigned long long> best;
  DevBuf<uint32_t> cell_count, cell_start, tile_sums, big;
  DevBuf<uint4> match_list;
  DevBuf<float4> big_scratch;  // allocated when a cell first outgrows the pair kernel
  DevBuf<DevPair> pairs;

  std::vector<DevInstance> hinst;
  uint32_t n_cells = 0, n_tiles = 0;
  uint64_t capacity = 0;
  uint32_t pair_cap = 0;
  bool binned = false;             // Path::kBinned (else the compact counting sort)
  uint32_t bin_cap = 0;            // records per cell bin
  std::vector<uint64_t> plan_n;    // particles each instance's grid was planned for
  bool have_particles = false;
  uint64_t target_step = 0;  // absolute step the enqueued work ends at
  float cell_override = 0.0f;

  cudaGraphExec_t graph1 = nullptr, graphN = nullptr;
  KParams graph_params{};     // what the graphs in hand were captured with
  LaunchShape graph_shape{};
  Path graph_path = Path::kBinned;
  LaunchShape shape{};

  bool host_only = false;  // BD_DEVICE_NONE: parameters and grid only
  bool scan_withhold = false;  // bd_debug_withhold_scan
  bool match_withhold = false; // bd_debug_withhold_match
  std::vector<std::string> stage_names;  // kernels of one step (bd_profile_steps)

  // serving: instance slots filled and emptied while the handle runs
  bool server = false;
  std::vector<uint8_t> slot_used;        // admitted, not yet harvested
  std::vector<uint64_t> slot_free_after; // removed: free once ctrl.step exceeds this
  std::vector<uint32_t> h_flags, h_target;
  DevBuf<uint32_t> inst_flags, inst_target, inst_frozen;

  bool diffuse_only() const {
    return U == 0 && B == 0 && idesc.size() == 1 && !zero_two_products && !server && panels.empty();
  }
  Path path() const { return diffuse_only() ? Path::kDiffuseOnly : (binned ? Path::kBinned : Path::kSorted); }
  int n_inst() const { return (int)idesc.size(); }
};

namespace {

void destroy_graphs(bd_system* h) {
  if (h->graph1) cudaGraphExecDestroy(h->graph1);
  if (h->graphN) cudaGraphExecDestroy(h->graphN);
  h->graph1 = h->graphN = nullptr;
}

KParams make_params(bd_system* h) {
  KParams p{};
  p.state[0] = h->state0.p;
  p.state[1] = h->state1.p;
  p.scatter = h->scatter.p;
  p.bins = h->bins.p;
  p.bin_cap = h->bin_cap;
  p.big = h->big.p;
  p.big_scratch = h->big_scratch.p;
  p.big_cap = (uint32_t)h->big.n;
  p.big_scratch_cap = (uint32_t)h->big_scratch.n;
  p.ctrl = h->ctrl.p;
  p.inst = h->dinst.p;
  if (!h->hinst.empty()) p.inst0 = h->hinst[0];
  p.species = h->dspecies.p;
  p.uni = h->duni.p;
  p.bim = h->dbim.p;
  p.zero = h->dzero.p;
  if (!h->hinst.empty() && h->Z > 0 && h->Z <= 4) {
    const size_t z0 = (size_t)h->hinst[0].block * h->Z;
    for (int z = 0; z < h->Z; z++)
      if (z0 + z < h->hzero.size()) p.zero0[z] = h->hzero[z0 + z];
  }
  p.cdf = h->dcdf.p;
  p.bim_table = h->dtable.p;
  p.gauss = h->dgauss.p;
  p.inst_step = h->inst_step.p;
  p.inst_flags = h->inst_flags.p;
  p.inst_target = h->inst_target.p;
  p.inst_frozen = h->inst_frozen.p;
  p.inst_slot_base = h->inst_slot_base.p;
  p.zero_off = h->zero_off.p;
  p.cell_count = h->cell_count.p;
  p.cell_start = h->cell_start.p;
  p.tile_sums = h->tile_sums.p;
  p.scan_withhold = h->scan_withhold ? 1u : 0u;
  p.match_withhold = h->match_withhold ? 1u : 0u;
  p.pairs = h->pairs.p;
  p.best = h->best.p;
  p.match_list = h->match_list.p;
  p.events = h->events.p;
  p.pending = h->pending.p;
  p.n_inst = (uint32_t)h->n_inst();
  p.S = (uint32_t)h->S;
  p.U = (uint32_t)h->U;
  p.B = (uint32_t)h->B;
  p.Z = (uint32_t)h->Z;
  p.R = (uint32_t)h->R;
  p.n_cells = h->n_cells;
  p.n_tiles = h->n_tiles;
  p.capacity = (uint32_t)h->capacity;
  p.pair_cap = h->pair_cap;
  p.prune_margin = 1e-3f;
  p.n_panels = (uint32_t)h->panels.size();
  if (p.n_panels) {
    p.panels = h->dpanels.p;
    p.surf_act = h->dsurf_act.p;
    p.pbox_start = h->dpbox_start.p;
    p.pbox_list = h->dpbox_list.p;
    p.surf_queue = h->surf_queue.p;
    p.cell_surf = h->dcell_surf.p;
    for (int k = 0; k < 3; k++) {
      p.pbox_lo[k] = h->pgrid.lo[k];
      p.pbox_inv[k] = h->pgrid.inv[k];
      p.pbox_dims[k] = h->pgrid.dims[k];
    }
  }
  return p;
}

bd_status build_graphs(bd_system* h) {
  const KParams p = make_params(h);
  const bool table = h->cfg.normal_mode == BD_NORMALS_TABLE;
  const Path path = h->path();
  // the graphs capture the parameter block, the launch shape and the path:
  // when none of them changed (a new upload into the same buffers), the
  // graphs in hand are still right
  if (h->graph1 && h->graphN && path == h->graph_path && memcmp(&p, &h->graph_params, sizeof p) == 0 &&
      memcmp(&h->shape, &h->graph_shape, sizeof h->shape) == 0)
    return BD_OK;
  destroy_graphs(h);
  const bool has_zero = h->Z > 0, has_uni = h->U > 0, has_bim = h->B > 0;
  for (int g = 0; g < 2; g++) {
    const int nsteps = g == 0 ? 1 : kGraphBatch;
    cudaGraph_t graph;
    BD_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < nsteps; k++) enqueue_step(p, path, table, has_zero, has_uni, has_bim, h->shape, h->stream);
    BD_CUDA(cudaStreamEndCapture(h->stream, &graph));
    cudaGraphExec_t exec;
    const cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    BD_CUDA(e);
    (g == 0 ? h->graph1 : h->graphN) = exec;
  }
  h->graph_params = p;
  h->graph_shape = h->shape;
  h->graph_path = path;
  return BD_OK;
}

// Uniform grid of one instance: cells at least 1% wider than the largest
// binding radius (so every reacting pair lies in the 27-cell neighbourhood),
// otherwise sized for `occupancy` particles per cell.
void choose_grid(bd_system* h, int k, uint64_t n_particles, DevInstance* I) {
  const bd_instance_desc& d = h->idesc[k];
  float rmax = 0.0f;
  for (int b = 0; b < h->B; b++) rmax = std::max(rmax, h->derived[k].rx[h->bim_list[b]].bind_radius);
  double L[3], vol = 1.0;
  for (int a = 0; a < 3; a++) {
    L[a] = (double)d.box_hi[a] - (double)d.box_lo[a];
    vol *= L[a];
  }
  double cs;
  const float want = h->cell_override > 0 ? h->cell_override : (d.cell_size > 0 ? d.cell_size : h->cfg.cell_size);
  if (want > 0) {
    cs = want;
  } else {
    const double occ = h->cfg.cell_occupancy > 0 ? h->cfg.cell_occupancy : 3.0;
    cs = cbrt(occ * vol / (double)std::max<uint64_t>(n_particles, 1));
  }
  cs = std::max(cs, 1.01 * (double)rmax);
  uint64_t total = 0;
  for (int guard = 0; guard < 64; guard++) {
    total = 1;
    for (int a = 0; a < 3; a++) total *= (uint64_t)std::max(1.0, floor(L[a] / cs));
    if (total <= (1ull << 28)) break;
    cs *= 1.25;
  }
  for (int a = 0; a < 3; a++) {
    I->lo[a] = d.box_lo[a];
    I->hi[a] = d.box_hi[a];
    I->dims[a] = (uint32_t)std::max(1.0, floor(L[a] / cs));
    I->cell[a] = (float)(L[a] / I->dims[a]);
    I->inv[a] = (float)I->dims[a] / (float)L[a];
  }
}

bd_status validate_config(const bd_config* c) {
  if (!c) return BD_ERR_INVALID_ARGUMENT;
  for (int a = 0; a < 3; a++)
    if (!(c->box_hi[a] > c->box_lo[a])) return BD_ERR_INVALID_ARGUMENT;
  if (!(c->dt > 0)) return BD_ERR_INVALID_ARGUMENT;
  if (c->normal_mode != BD_NORMALS_BOXMULLER && c->normal_mode != BD_NORMALS_TABLE) return BD_ERR_INVALID_ARGUMENT;
  if (c->sort_mode > BD_SORT_BINNED) return BD_ERR_INVALID_ARGUMENT;
  if (c->pair_mode > BD_PAIR_CHANNELS) return BD_ERR_INVALID_ARGUMENT;
  return BD_OK;
}

// The handle's pool for the scratch of host transfers, on its device; it
// keeps the memory it maps until the handle is destroyed.
cudaError_t create_pool(bd_system* h) {
  cudaMemPoolProps props = {};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = h->device;
  cudaError_t e = cudaMemPoolCreate(&h->pool, &props);
  if (e != cudaSuccess) {
    h->pool = nullptr;
    return e;
  }
  uint64_t keep = UINT64_MAX;
  return cudaMemPoolSetAttribute(h->pool, cudaMemPoolAttrReleaseThreshold, &keep);
}
bd_status create_common(const bd_config* cfg, const bd_instance_desc* inst, int n, bd_handle* out) {
  if (!out) return BD_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  bd_status st = validate_config(cfg);
  if (st) return st;
  if (n < 1 || (uint32_t)n > kMaxInstances) return BD_ERR_INVALID_ARGUMENT;
  const bool host_only = cfg->device == BD_DEVICE_NONE;
  int ndev = 0;
  if (!host_only) {
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
      g_last_error = "no CUDA device";
      return BD_ERR_NO_DEVICE;
    }
    if (cfg->device < 0 || cfg->device >= ndev) return BD_ERR_INVALID_ARGUMENT;
  }
  bd_system* h = new bd_system();
  h->host_only = host_only;
  h->cfg = *cfg;
  h->device = cfg->device;
  if (inst) {
    h->idesc.assign(inst, inst + n);
    for (auto& d : h->idesc) {
      for (int a = 0; a < 3; a++)
        if (!(d.box_hi[a] > d.box_lo[a])) {
          delete h;
          return BD_ERR_INVALID_ARGUMENT;
        }
      if (!(d.d_scale > 0)) d.d_scale = 1.0f;
      if (!(d.k2_scale > 0)) d.k2_scale = 1.0f;
    }
  } else {
    bd_instance_desc d{};
    memcpy(d.box_lo, cfg->box_lo, sizeof(d.box_lo));
    memcpy(d.box_hi, cfg->box_hi, sizeof(d.box_hi));
    d.seed = cfg->seed;
    d.d_scale = d.k2_scale = 1.0f;
    d.cell_size = 0.0f;
    h->idesc.push_back(d);
  }
  if (host_only) {
    *out = h;
    return BD_OK;
  }
  if (!cuda_ok(cudaSetDevice(h->device), "cudaSetDevice") ||
      !cuda_ok(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking), "cudaStreamCreate") ||
      !cuda_ok(create_pool(h), "cudaMemPoolCreate") ||
      !cuda_ok(h->ctrl.alloc(1), "cudaMalloc ctrl") ||
      !cuda_ok(cudaMallocHost((void**)&h->hctrl, sizeof(DevCtrl)), "cudaMallocHost")) {
    bd_destroy(h);
    return BD_ERR_CUDA;
  }
  cudaDeviceGetAttribute(&h->n_sm, cudaDevAttrMultiProcessorCount, h->device);
  // 4 resident CTAs of 256 threads per SM with the 64-register variants
  // (measured on the 16M c3 step: 0.90 ms against 1.00 ms uncapped)
  h->shape.block_stream = 256;
  h->shape.grid_stream = h->n_sm * 4;
  h->shape.min_blocks = 4;
  h->shape.block_pairs = 256;
  // one wave of the pair kernel (4 resident CTAs of 256 per SM): 0.2752
  // against 0.2786 ms for two waves on the 16M c3 step
  h->shape.grid_pairs = h->n_sm * 4;
  h->shape.grid_match = h->host_only ? 1 : match_grid(h->n_sm);
  h->shape.grid_scan = h->host_only ? 1 : scan_grid(h->n_sm);
  h->shape.grid_big = h->host_only ? 1 : big_grid(h->n_sm);
  memset(h->hctrl, 0, sizeof(DevCtrl));
  cudaMemset(h->ctrl.p, 0, sizeof(DevCtrl));
  *out = h;
  return BD_OK;
}

template <class T>
bd_status upload(DevBuf<T>& buf, const std::vector<T>& v, cudaStream_t s) {
  BD_CUDA(buf.alloc(std::max<size_t>(v.size(), 1)));
  if (!v.empty()) BD_CUDA(cudaMemcpyAsync(buf.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
  return BD_OK;
}

bd_status sync_ctrl(bd_system* h) {
  BD_CUDA(cudaMemcpyAsync(h->hctrl, h->ctrl.p, sizeof(DevCtrl), cudaMemcpyDeviceToHost, h->stream));
  BD_CUDA(cudaStreamSynchronize(h->stream));
  return BD_OK;
}

bd_status push_ctrl(bd_system* h) {
  BD_CUDA(cudaMemcpyAsync(h->ctrl.p, h->hctrl, sizeof(DevCtrl), cudaMemcpyHostToDevice, h->stream));
  BD_CUDA(cudaStreamSynchronize(h->stream));
  return BD_OK;
}

// (Re)allocate the particle-sized buffers for `cap` slots, keeping the
// current state (n_slots records of the current buffer) in buffer 0.
bd_status grow_particles(bd_system* h, uint64_t cap) {
  if (cap > 0xFFFFFFF0ull) return BD_ERR_CAPACITY;
  DevBuf<float4> s0, s1, sc;
  DevBuf<unsigned long long> best;
  BD_CUDA(s0.alloc(cap));
  BD_CUDA(s1.alloc(cap));
  if (!h->binned) BD_CUDA(sc.alloc(cap));
  BD_CUDA(best.alloc(cap));
  BD_CUDA(cudaMemsetAsync(best.p, 0xFF, cap * sizeof(unsigned long long), h->stream));
  if (!h->panels.empty()) BD_CUDA(h->surf_queue.alloc(cap));
  // cells above 128 records (the large-cell kernel's queue) number at most cap / 129
  BD_CUDA(h->big.alloc(cap / 129 + 2));
  if (h->big_scratch.n) BD_CUDA(h->big_scratch.alloc(cap));
  if (h->have_particles && h->hctrl->n_slots > 0) {
    const float4* src = h->hctrl->cur ? h->state1.p : h->state0.p;
    BD_CUDA(cudaMemcpyAsync(s0.p, src, (size_t)h->hctrl->n_slots * sizeof(float4), cudaMemcpyDeviceToDevice,
                            h->stream));
  }
  BD_CUDA(cudaStreamSynchronize(h->stream));
  h->state0.free();
  h->state1.free();
  h->scatter.free();
  h->best.free();
  h->state0 = s0;
  h->state1 = s1;
  h->scatter = sc;
  h->best = best;
  s0.p = s1.p = sc.p = nullptr;
  best.p = nullptr;
  h->hctrl->cur = 0;
  h->capacity = cap;
  return BD_OK;
}

bd_status grow_pairs(bd_system* h, uint32_t cap) {
  BD_CUDA(h->pairs.alloc(cap));
  BD_CUDA(h->match_list.alloc(2 * (uint64_t)cap));
  h->pair_cap = cap;
  return BD_OK;
}

// The buffer the current sort mode writes: the cell bins (bin_cap records
// per cell) or the compact scatter buffer (one record per slot).
bd_status ensure_sort_buffers(bd_system* h, uint32_t K) {
  if (h->binned) {
    h->bin_cap = K;
    const size_t need = (size_t)h->n_cells * K;
    if (h->bins.n < need) BD_CUDA(h->bins.alloc(need));
    h->scatter.free();
  } else {
    h->bins.free();
    if (h->capacity > 0 && h->scatter.n < h->capacity) BD_CUDA(h->scatter.alloc(h->capacity));
  }
  return BD_OK;
}

// Grid and Philox key of instance k, planned from its particle count.  An
// instance keeps its grid for life: the cell grid decides the canonical
// order, so it must not depend on the other instances.
void plan_instance(bd_system* h, int k, uint64_t n) {
  DevInstance& D = h->hinst[k];
  choose_grid(h, k, n, &D);
  if (h->plan_n.size() != h->hinst.size()) h->plan_n.assign(h->hinst.size(), 0);
  h->plan_n[k] = n;
  D.key_lo = (uint32_t)(h->idesc[k].seed & 0xFFFFFFFFu);
  D.key_hi = (uint32_t)(h->idesc[k].seed >> 32);
  D.block = (uint32_t)k;
  D.flags = kInstActive;
}

bd_status upload_cell_masks(bd_system* h);

// Consecutive cell ranges for the instances in instance order (unused
// server slots get a single cell), the cell arrays and the instance table.
bd_status layout_cells(bd_system* h) {
  const int I = h->n_inst();
  uint64_t base = 0;
  for (int k = 0; k < I; k++) {
    DevInstance& D = h->hinst[k];
    if (h->server && !h->slot_used[k]) {
      for (int a = 0; a < 3; a++) {
        D.dims[a] = 1;
        D.lo[a] = 0.0f;
        D.hi[a] = 1.0f;
        D.cell[a] = 1.0f;
        D.inv[a] = 1.0f;
      }
    }
    D.cell_base = (uint32_t)base;
    base += (uint64_t)D.dims[0] * D.dims[1] * D.dims[2];
  }
  if (base > 0xFFFFFFF0ull) return BD_ERR_CAPACITY;
  h->n_cells = (uint32_t)base;
  h->n_tiles = (uint32_t)((base + kScanTile - 1) / kScanTile);
  if (h->host_only) return BD_OK;
  // grow-only: a serving handle lays its cells out again at every admission,
  // and cudaFree would wait for the whole device
  auto ensure = [](auto& buf, size_t count) { return buf.p && buf.n >= count ? cudaSuccess : buf.alloc(count); };
  BD_CUDA(ensure(h->dinst, (size_t)I));
  BD_CUDA(cudaMemcpyAsync(h->dinst.p, h->hinst.data(), I * sizeof(DevInstance), cudaMemcpyHostToDevice, h->stream));
  BD_CUDA(ensure(h->cell_count, (size_t)h->n_cells));
  BD_CUDA(cudaMemsetAsync(h->cell_count.p, 0, (size_t)h->n_cells * sizeof(uint32_t), h->stream));
  BD_CUDA(ensure(h->cell_start, (size_t)h->n_cells + 1));
  BD_CUDA(cudaMemsetAsync(h->cell_start.p, 0, ((size_t)h->n_cells + 1) * sizeof(uint32_t), h->stream));
  BD_CUDA(ensure(h->tile_sums, (size_t)std::max<uint32_t>(h->n_tiles, 1)));
  BD_CUDA(cudaStreamSynchronize(h->stream));
  if (!h->panels.empty()) {
    const bd_status st = upload_cell_masks(h);
    if (st) return st;
  }
  // Bins hold the planned occupancy of the densest instance with room for
  // Poisson fluctuations (mean + 7 sd + 8: an overflow at mean 3 has
  // probability ~1e-14 per cell and step); they only grow.
  double lam = 0.0;
  for (int k = 0; k < I; k++) {
    if (h->server && !h->slot_used[k]) continue;
    const DevInstance& D = h->hinst[k];
    const double cells = (double)D.dims[0] * D.dims[1] * D.dims[2];
    if (k < (int)h->plan_n.size()) lam = std::max(lam, (double)h->plan_n[k] / cells);
  }
  uint32_t K = (uint32_t)ceil(lam + 7.0 * sqrt(lam) + 8.0);
  K = std::max<uint32_t>((K + kBinGroup - 1) / kBinGroup * kBinGroup, h->bin_cap);
  const uint64_t bytes = (uint64_t)h->n_cells * K * sizeof(float4);
  const uint32_t mode = h->cfg.sort_mode;
  h->binned = mode == BD_SORT_BINNED || (mode == BD_SORT_AUTO && bytes <= kBinBudgetBytes);
  return ensure_sort_buffers(h, K);
}

// Device scratch of one call, taken from the stream-ordered pool and given
// back on the stream when the call returns.
// Stream-ordered scratch of one call (uploads, readbacks, admissions,
// harvests), from the handle's own memory pool: the pool keeps the memory
// it has mapped (release threshold: never), so a call that repeats a size
// maps nothing new, where the device's default pool would hand the memory
// back at each synchronisation and map it again on the next call.
struct Scratch {
  cudaStream_t stream = nullptr;
  char* p = nullptr;
  size_t used = 0;
  ~Scratch() {
    if (p) cudaFreeAsync(p, stream);
  }
  cudaError_t alloc(size_t bytes, cudaStream_t s, cudaMemPool_t pool) {
    stream = s;
    if (pool) return cudaMallocFromPoolAsync((void**)&p, bytes, pool, s);
    return cudaMallocAsync((void**)&p, bytes, s);
  }
  template <class T>
  T* take(size_t count) {  // 256-byte aligned pieces
    T* q = reinterpret_cast<T*>(p + used);
    used += (count * sizeof(T) + 255) & ~(size_t)255;
    return q;
  }
};

size_t scratch_bytes(std::initializer_list<size_t> sizes) {
  size_t b = 0;
  for (size_t x : sizes) b += (x + 255) & ~(size_t)255;
  return b;
}

// The caller's particles (float4 x, y, z, w and int species, counts[k] for
// instance k in instance order) become the current state.  On a device
// handle they are copied whole to device scratch, checked there (species
// range, inside the instance's box) before anything of the handle changes,
// and packed into records by a kernel.
bd_status upload_particles(bd_system* h, const float* xyz4, const int* species, const uint64_t* counts) {
  const Range range("bd_set_particles");
  if (!h->finalized) return BD_ERR_NOT_FINALIZED;
  const int I = h->n_inst();
  uint64_t n = 0;
  for (int k = 0; k < I; k++) n += counts[k];
  if (n > 0 && (!xyz4 || !species)) return BD_ERR_INVALID_ARGUMENT;
  std::vector<uint32_t> slot_base(I, 0);
  std::vector<uint64_t> start(I + 1, 0);
  std::vector<float> boxes(6 * (size_t)I);
  for (int k = 0; k < I; k++) {
    start[k + 1] = start[k] + counts[k];
    slot_base[k] = (uint32_t)start[k];
    for (int a = 0; a < 3; a++) {
      boxes[6 * k + a] = h->idesc[k].box_lo[a];
      boxes[6 * k + 3 + a] = h->idesc[k].box_hi[a];
    }
  }
  Scratch scratch;
  UploadArgs up{};
  if (h->host_only) {
    for (int k = 0; k < I; k++)
      for (uint64_t i = start[k]; i < start[k + 1]; i++) {
        const int s = species[i];
        const float x = xyz4[4 * i], y = xyz4[4 * i + 1], z = xyz4[4 * i + 2];
        const float* b = &boxes[6 * k];
        if (s < 0 || s >= h->S || !(x >= b[0] && x <= b[3] && y >= b[1] && y <= b[4] && z >= b[2] && z <= b[5]))
          return BD_ERR_INVALID_ARGUMENT;
      }
  } else if (n > 0) {
    BD_CUDA(cudaSetDevice(h->device));
    BD_CUDA(scratch.alloc(scratch_bytes({n * sizeof(float4), n * sizeof(int), (I + 1) * sizeof(uint64_t),
                                         boxes.size() * sizeof(float), sizeof(uint32_t)}),
                          h->stream, h->pool));
    float4* d_xyz4 = scratch.take<float4>(n);
    int* d_species = scratch.take<int>(n);
    uint64_t* d_start = scratch.take<uint64_t>(I + 1);
    float* d_boxes = scratch.take<float>(boxes.size());
    uint32_t* d_bad = scratch.take<uint32_t>(1);
    BD_CUDA(cudaMemcpyAsync(d_xyz4, xyz4, n * sizeof(float4), cudaMemcpyHostToDevice, h->stream));
    BD_CUDA(cudaMemcpyAsync(d_species, species, n * sizeof(int), cudaMemcpyHostToDevice, h->stream));
    BD_CUDA(cudaMemcpyAsync(d_start, start.data(), (I + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, h->stream));
    BD_CUDA(cudaMemcpyAsync(d_boxes, boxes.data(), boxes.size() * sizeof(float), cudaMemcpyHostToDevice, h->stream));
    BD_CUDA(cudaMemsetAsync(d_bad, 0, sizeof(uint32_t), h->stream));
    up = UploadArgs{d_xyz4, d_species, d_start, d_boxes, n, I, h->S, d_bad, 0u};
    enqueue_upload_check(up, h->stream);
    BD_CUDA(cudaGetLastError());
    uint32_t bad = 0;
    BD_CUDA(cudaMemcpyAsync(&bad, d_bad, sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream));
    BD_CUDA(cudaStreamSynchronize(h->stream));
    if (bad) return BD_ERR_INVALID_ARGUMENT;
  }
  h->hinst.assign(I, DevInstance{});
  for (int k = 0; k < I; k++) plan_instance(h, k, counts[k]);
  bd_status st = layout_cells(h);
  if (st) return st;
  if (h->host_only) return BD_OK;
  uint64_t cap = h->cfg.capacity ? h->cfg.capacity : std::max<uint64_t>(2 * n, 4096);
  if (cap < n) cap = n;
  h->have_particles = false;
  memset(h->hctrl, 0, sizeof(DevCtrl));
  // buffers of the same size are kept (the matcher scratch is all ones
  // again after every step)
  const bool same = cap == h->capacity && h->state0.p && h->state1.p && (h->binned || h->scatter.n >= cap) &&
                    (h->panels.empty() || h->surf_queue.n >= cap);
  if (same) {
    h->hctrl->cur = 0;
  } else {
    st = grow_particles(h, cap);
    if (st) return st;
  }
  uint32_t pc = h->cfg.pair_capacity ? h->cfg.pair_capacity : (uint32_t)std::max<uint64_t>(65536, cap / 32);
  if (pc != h->pair_cap || !h->pairs.p) {
    st = grow_pairs(h, pc);
    if (st) return st;
  }
  if (n) {
    enqueue_upload_pack(up, h->state0.p, h->stream);
    BD_CUDA(cudaGetLastError());
  }
  std::vector<uint32_t> zeros(I, 0);
  st = upload(h->inst_step, zeros, h->stream);
  if (st) return st;
  st = upload(h->inst_slot_base, slot_base, h->stream);
  if (st) return st;
  h->h_flags.assign(I, kInstActive);
  h->h_target.assign(I, 0xFFFFFFFFu);
  if ((st = upload(h->inst_flags, h->h_flags, h->stream)) || (st = upload(h->inst_target, h->h_target, h->stream)) ||
      (st = upload(h->inst_frozen, zeros, h->stream)))
    return st;
  BD_CUDA(h->zero_off.alloc((size_t)I * h->Z + 1));
  BD_CUDA(cudaMemsetAsync(h->zero_off.p, 0, ((size_t)I * h->Z + 1) * sizeof(uint32_t), h->stream));
  BD_CUDA(h->events.alloc((size_t)I * std::max(h->R, 1)));
  BD_CUDA(cudaMemsetAsync(h->events.p, 0, (size_t)I * std::max(h->R, 1) * sizeof(unsigned long long), h->stream));
  BD_CUDA(h->pending.alloc((size_t)I * std::max(h->R, 1)));
  BD_CUDA(cudaMemsetAsync(h->pending.p, 0, (size_t)I * std::max(h->R, 1) * sizeof(unsigned long long), h->stream));
  memset(h->hctrl, 0, sizeof(DevCtrl));
  h->hctrl->n_slots = (uint32_t)n;
  st = push_ctrl(h);
  if (st) return st;
  h->have_particles = true;
  h->target_step = 0;
  return build_graphs(h);
}

}  // namespace

// ======================================================================= ABI

BD_API void bd_config_default(bd_config* c) {
  if (!c) return;
  memset(c, 0, sizeof(*c));
  for (int a = 0; a < 3; a++) {
    c->box_lo[a] = 0.0f;
    c->box_hi[a] = 1.0f;
  }
  c->dt = 1e-3f;
  c->seed = 1;
  c->normal_mode = BD_NORMALS_BOXMULLER;
}

BD_API bd_status bd_create(const bd_config* cfg, bd_handle* out) { return create_common(cfg, nullptr, 1, out); }

BD_API bd_status bd_create_ensemble(const bd_config* cfg, const bd_instance_desc* inst, int n, bd_handle* out) {
  if (!inst) return BD_ERR_INVALID_ARGUMENT;
  return create_common(cfg, inst, n, out);
}

BD_API bd_status bd_destroy(bd_handle h) {
  if (!h) return BD_ERR_INVALID_ARGUMENT;
  if (!h->host_only) cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  destroy_graphs(h);
  h->ctrl.free();
  if (h->hctrl) cudaFreeHost(h->hctrl);
  h->dinst.free();
  h->dspecies.free();
  h->duni.free();
  h->dbim.free();
  h->dzero.free();
  h->dcdf.free();
  h->dtable.free();
  h->dgauss.free();
  h->inst_step.free();
  h->inst_flags.free();
  h->inst_target.free();
  h->inst_frozen.free();
  h->inst_slot_base.free();
  h->zero_off.free();
  h->events.free();
  h->pending.free();
  h->state0.free();
  h->state1.free();
  h->scatter.free();
  h->bins.free();
  h->big.free();
  h->big_scratch.free();
  h->best.free();
  h->cell_count.free();
  h->cell_start.free();
  h->tile_sums.free();
  h->pairs.free();
  h->match_list.free();
  h->dpanels.free();
  h->dsurf_act.free();
  h->dpbox_start.free();
  h->dpbox_list.free();
  h->surf_queue.free();
  h->dcell_surf.free();
  if (h->pool) cudaMemPoolDestroy(h->pool);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return BD_OK;
}

BD_API bd_status bd_add_species(bd_handle h, float D, int* id) {
  if (!h) return BD_ERR_INVALID_ARGUMENT;
  if (h->finalized) return BD_ERR_ALREADY_FINALIZED;
  if (!(D >= 0) || h->D.size() >= kMaxSpecies) return BD_ERR_INVALID_ARGUMENT;
  h->D.push_back(D);
  if (id) *id = (int)h->D.size() - 1;
  return BD_OK;
}

BD_API bd_status bd_add_reaction(bd_handle h, int order, const int reactants[2], const int products[2], float rate,
                                 int* id) {
  if (!h) return BD_ERR_INVALID_ARGUMENT;
  if (h->finalized) return BD_ERR_ALREADY_FINALIZED;
  if (order < 0 || order > 2) return BD_ERR_INVALID_ARGUMENT;
  if (rate < 0) return BD_ERR_NEGATIVE_RATE;
  const int S = (int)h->D.size();
  ReactionDef r;
  r.order = order;
  r.rate = rate;
  for (int k = 0; k < 2; k++) {
    r.reactants[k] = reactants ? reactants[k] : -1;
    r.products[k] = products ? products[k] : -1;
  }
  for (int k = 0; k < order; k++)
    if (r.reactants[k] < 0 || r.reactants[k] >= S) return BD_ERR_INVALID_ARGUMENT;
  for (int k = order; k < 2; k++) r.reactants[k] = -1;
  if (r.products[0] < 0 && r.products[1] >= 0) std::swap(r.products[0], r.products[1]);
  for (int k = 0; k < 2; k++)
    if (r.products[k] >= S) return BD_ERR_INVALID_ARGUMENT;
  r.nprod = (r.products[0] >= 0) + (r.products[1] >= 0);
  if (order == 0 && r.nprod == 0) return BD_ERR_INVALID_ARGUMENT;
  h->rx.push_back(r);
  if (id) *id = (int)h->rx.size() - 1;
  return BD_OK;
}

BD_API bd_status bd_set_product_placement(bd_handle h, int rxn, int kind, float param) {
  if (!h || rxn < 0 || rxn >= (int)h->rx.size()) return BD_ERR_INVALID_ARGUMENT;
  if (h->finalized) return BD_ERR_ALREADY_FINALIZED;
  if (kind < BD_PP_DEFAULT || kind > BD_PP_OFFSET0) return BD_ERR_INVALID_ARGUMENT;
  h->rx[rxn].pp_kind = kind;
  h->rx[rxn].pp_param = param;
  return BD_OK;
}

namespace {
// Pack every instance's derived parameters into the device blocks.
static_assert(sizeof(bd_panel_info) <= sizeof(DevPanel), "DevPanel holds a bd_panel_info");

uint8_t surface_action(const bd_system* h, int surf, int sp, int face) {
  const bd_system::Surface& S = h->surfaces[surf];
  const int v = sp < (int)S.species[face].size() ? S.species[face][sp] : -1;
  return v >= 0 ? (uint8_t)v : S.all[face];
}

// [surface][species][front, back] actions for the kernels.
std::vector<uint8_t> surface_table(const bd_system* h) {
  const int S = (int)h->D.size();
  std::vector<uint8_t> t(h->surfaces.size() * (size_t)S * 2);
  for (size_t f = 0; f < h->surfaces.size(); f++)
    for (int sp = 0; sp < S; sp++)
      for (int face = 0; face < 2; face++) t[(f * S + sp) * 2 + face] = surface_action(h, (int)f, sp, face);
  return t;
}

// The panel grid spans the union of the instances' boxes (positions outside
// it map to its edge boxes, so any box is correct, only slower).
void plan_panel_grid(bd_system* h) {
  float lo[3], hi[3];
  for (int k = 0; k < 3; k++) {
    lo[k] = h->idesc[0].box_lo[k];
    hi[k] = h->idesc[0].box_hi[k];
  }
  for (const bd_instance_desc& d : h->idesc)
    for (int k = 0; k < 3; k++) {
      lo[k] = std::min(lo[k], d.box_lo[k]);
      hi[k] = std::max(hi[k], d.box_hi[k]);
    }
  build_panel_grid(h->panels, lo, hi, &h->pgrid);
  // a step of species s walks s and the products of its first-order
  // reactions: the panel counts for s when any of them sees it
  const int S = (int)h->D.size();
  std::vector<std::vector<int>> walked(S);
  for (int sp = 0; sp < S; sp++) walked[sp].push_back(sp);
  for (const ReactionDef& r : h->rx)
    if (r.order == 1)
      for (int k = 0; k < 2; k++)
        if (r.products[k] >= 0) walked[r.reactants[0]].push_back(r.products[k]);
  h->panel_species.assign(h->panels.size(), 0);
  for (size_t id = 0; id < h->panels.size(); id++)
    for (int sp = 0; sp < S; sp++)
      for (int t : walked[sp])
        if (surface_action(h, h->panels[id].surface, t, 0) != kActTransmit ||
            surface_action(h, h->panels[id].surface, t, 1) != kActTransmit)
          h->panel_species[id] |= (uint8_t)(1u << species_bit(sp));
}

// Species masks of every cell (build_cell_masks), instance by instance,
// looked up at the cell a step starts in.  The reach of an instance bounds
// how far a molecule's diffusion step goes (Box-Muller and table normals
// stay within 5.9 sigma per axis) plus the largest first-order product
// offset from the step's end.
bd_status upload_cell_masks(bd_system* h) {
  std::vector<uint8_t> m(h->n_cells, 0xFF);
  for (int k = 0; k < h->n_inst(); k++) {
    if (h->server && !h->slot_used[k]) continue;  // a single cell, nothing moves there
    const DevInstance& D = h->hinst[k];
    const DerivedParams& P = h->derived[k];
    double smax = 0.0, omax = 0.0;
    for (float sg : P.sigma) smax = std::max(smax, (double)sg);
    for (int r = 0; r < h->R; r++)
      if (h->rx[r].order == 1) omax = std::max({omax, (double)fabsf(P.rx[r].off[0]), (double)fabsf(P.rx[r].off[1])});
    double box = 0.0;
    for (int a = 0; a < 3; a++) box = std::max({box, (double)fabsf(D.lo[a]), (double)fabsf(D.hi[a])});
    const double reach = (6.0 * smax + omax) * 1.001 + 1e-5 * (box + 1.0);
    build_cell_masks(h->panels, h->panel_species, h->pgrid, D.lo, D.cell, D.dims, reach, &m[D.cell_base]);
  }
  BD_CUDA(h->dcell_surf.alloc(std::max<size_t>(m.size(), 1)));
  BD_CUDA(cudaMemcpyAsync(h->dcell_surf.p, m.data(), m.size(), cudaMemcpyHostToDevice, h->stream));
  BD_CUDA(cudaStreamSynchronize(h->stream));
  return BD_OK;
}

bd_status pack_blocks(bd_system* h) {
  const int I = h->n_inst(), S = h->S, U = h->U, B = h->B, Z = h->Z;
  std::vector<DevSpecies> sp((size_t)I * S);
  std::vector<DevUni> un((size_t)I * U);
  std::vector<DevBim> bi((size_t)I * B);
  std::vector<DevZero> ze((size_t)I * Z);
  std::vector<double> cdf;
  for (int k = 0; k < I; k++) {
    const DerivedParams& P = h->derived[k];
    int u = 0;
    for (int s = 0; s < S; s++) {
      DevSpecies& ds = sp[(size_t)k * S + s];
      ds.sigma = P.sigma[s];
      ds.uni_begin = (uint32_t)u;
      ds.uni_count = 0;
      ds.max_r = 0.0f;
      while (u < U && h->rx[h->uni_list[u]].reactants[0] == s) {
        const int r = h->uni_list[u];
        DevUni& du = un[(size_t)k * U + u];
        du.prob = P.rx[r].prob;
        du.prod0 = h->rx[r].products[0];
        du.prod1 = h->rx[r].products[1];
        du.off0 = P.rx[r].off[0];
        du.off1 = P.rx[r].off[1];
        du.rxn = (uint32_t)r;
        ds.uni_count++;
        u++;
      }
      for (int s2 = 0; s2 < S; s2++) {
        const int b = h->bim_table[(size_t)s * S + s2];
        if (b >= 0) ds.max_r = std::max(ds.max_r, P.rx[h->bim_list[b]].bind_radius);
      }
    }
    for (int b = 0; b < B; b++) {
      const int r = h->bim_list[b];
      DevBim& db = bi[(size_t)k * B + b];
      db.r2 = P.rx[r].bind_r2;
      db.prob = P.rx[r].prob;
      db.x = P.rx[r].x;
      db.omx = P.rx[r].omx;
      db.react0 = h->rx[r].reactants[0];
      db.prod0 = h->rx[r].products[0];
      db.prod1 = h->rx[r].products[1];
      db.off0 = P.rx[r].off[0];
      db.off1 = P.rx[r].off[1];
      db.rxn = (uint32_t)r;
      db.thresh = P.rx[r].thresh;
      db.next = -1;
      if (P.rx[r].next >= 0)
        for (int b2 = 0; b2 < B; b2++)
          if (h->bim_list[b2] == P.rx[r].next) db.next = b2;
    }
    for (int z = 0; z < Z; z++) {
      const int r = h->zero_list[z];
      DevZero& dz = ze[(size_t)k * Z + z];
      dz.prod0 = h->rx[r].products[0];
      dz.prod1 = h->rx[r].products[1];
      dz.cdf_off = (uint32_t)cdf.size();
      dz.cdf_len = (uint32_t)P.cdf[r].size();
      dz.kmin = P.cdf_kmin[r];
      dz.rxn = (uint32_t)r;
      cdf.insert(cdf.end(), P.cdf[r].begin(), P.cdf[r].end());
    }
  }
  h->hzero = ze;
  if (h->host_only) return BD_OK;
  std::vector<float> gauss(4096);
  gauss_quantiles(gauss.data(), 4096);
  bd_status st;
  if ((st = upload(h->dspecies, sp, h->stream)) || (st = upload(h->duni, un, h->stream)) ||
      (st = upload(h->dbim, bi, h->stream)) || (st = upload(h->dzero, ze, h->stream)) ||
      (st = upload(h->dcdf, cdf, h->stream)) || (st = upload(h->dtable, h->bim_table, h->stream)) ||
      (st = upload(h->dgauss, gauss, h->stream)))
    return st;
  if (!h->panels.empty()) {
    std::vector<DevPanel> dp(h->panels.size());
    for (size_t k = 0; k < dp.size(); k++) {
      memset(&dp[k], 0, sizeof(DevPanel));
      memcpy(&dp[k], &h->panels[k], sizeof(bd_panel_info));
    }
    if ((st = upload(h->dpanels, dp, h->stream)) || (st = upload(h->dsurf_act, surface_table(h), h->stream)) ||
        (st = upload(h->dpbox_start, h->pgrid.start, h->stream)) ||
        (st = upload(h->dpbox_list, h->pgrid.list, h->stream)))
      return st;
  }
  BD_CUDA(cudaStreamSynchronize(h->stream));
  return BD_OK;
}
}  // namespace

BD_API bd_status bd_set_reaction_probability(bd_handle h, int rxn, float prob) {
  if (!h || rxn < 0 || rxn >= (int)h->rx.size()) return BD_ERR_INVALID_ARGUMENT;
  if (h->finalized) return BD_ERR_ALREADY_FINALIZED;
  if (h->rx[rxn].order != 2 || !(prob >= 0.0f && prob <= 1.0f)) return BD_ERR_INVALID_ARGUMENT;
  h->rx[rxn].user_prob = prob;
  return BD_OK;
}

BD_API bd_status bd_finalize(bd_handle h) {
  const Range range("bd_finalize");
  if (!h) return BD_ERR_INVALID_ARGUMENT;
  if (h->finalized) return BD_ERR_ALREADY_FINALIZED;
  if (h->D.empty()) return BD_ERR_INVALID_ARGUMENT;
  if (!h->host_only) BD_CUDA(cudaSetDevice(h->device));
  const int I = h->n_inst();
  h->S = (int)h->D.size();
  h->R = (int)h->rx.size();
  bd_status first = BD_OK;
  h->derived.clear();
  for (int k = 0; k < I; k++) {
    const bd_instance_desc& d = h->idesc[k];
    const float vol = (d.box_hi[0] - d.box_lo[0]) * (d.box_hi[1] - d.box_lo[1]) * (d.box_hi[2] - d.box_lo[2]);
    h->derived.push_back(derive_params(h->D, h->rx, h->cfg.dt, vol, d.d_scale, d.k2_scale,
                                       h->cfg.pair_mode == BD_PAIR_CHANNELS));
    if (!first && h->derived.back().status) {
      first = h->derived.back().status;
      g_last_error = h->derived.back().message;
    }
  }
  // fatal setup errors leave the handle unfinalized
  if (first == BD_ERR_NEGATIVE_RATE || first == BD_ERR_ZERO_DIFFUSION || first == BD_ERR_ILLEGAL_UNBIND ||
      first == BD_ERR_UNSUPPORTED)
    return first;

  // network shape
  h->uni_list.clear();
  h->bim_list.clear();
  h->zero_list.clear();
  h->zero_two_products = false;
  for (int s = 0; s < h->S; s++)
    for (int r = 0; r < h->R; r++)
      if (h->rx[r].order == 1 && h->rx[r].reactants[0] == s) h->uni_list.push_back(r);
  for (int r = 0; r < h->R; r++) {
    if (h->rx[r].order == 2) h->bim_list.push_back(r);
    if (h->rx[r].order == 0) {
      h->zero_list.push_back(r);
      if (h->rx[r].nprod == 2) h->zero_two_products = true;
    }
  }
  h->U = (int)h->uni_list.size();
  h->B = (int)h->bim_list.size();
  h->Z = (int)h->zero_list.size();
  const int S = h->S, B = h->B;

  // pair table: the last reaction listed for a pair wins (particleSystem.cpp:656-669),
  // or, with competing reactions, the first of the pair's chain; a reaction
  // with zero rate never fires
  h->bim_table.assign((size_t)S * S, -1);
  const bool channels = h->cfg.pair_mode == BD_PAIR_CHANNELS;
  for (int b = 0; b < B; b++) {
    const ReactionDef& r = h->rx[h->bim_list[b]];
    if (!(r.rate > 0)) {
      if (!channels) {
        h->bim_table[(size_t)r.reactants[0] * S + r.reactants[1]] = -1;
        h->bim_table[(size_t)r.reactants[1] * S + r.reactants[0]] = -1;
      }
      continue;
    }
    int32_t& e0 = h->bim_table[(size_t)r.reactants[0] * S + r.reactants[1]];
    int32_t& e1 = h->bim_table[(size_t)r.reactants[1] * S + r.reactants[0]];
    if (channels && e0 >= 0) continue;  // the chain starts at the pair's first reaction
    e0 = b;
    e1 = b;
  }

  if (!h->panels.empty()) plan_panel_grid(h);
  bd_status st = pack_blocks(h);
  if (st) return st;
  h->finalized = true;
  return first;
}

BD_API bd_status bd_add_surface(bd_handle h, int* surface) {
  if (!h) return BD_ERR_INVALID_ARGUMENT;
  if (h->finalized) return BD_ERR_ALREADY_FINALIZED;
  if (h->surfaces.size() >= 0x10000) return BD_ERR_CAPACITY;
  h->surfaces.emplace_back();
  if (surface) *surface = (int)h->surfaces.size() - 1;
  return BD_OK;
}

BD_API bd_status bd_set_surface_action(bd_handle h, int surface, int species, int face, int action) {
  if (!h || surface < 0 || surface >= (int)h->surfaces.size()) return BD_ERR_INVALID_ARGUMENT;
  if (h->finalized) return BD_ERR_ALREADY_FINALIZED;
  if (species != BD_ALL_SPECIES && (species < 0 || species >= (int)h->D.size())) return BD_ERR_INVALID_ARGUMENT;
  if (face < BD_FACE_FRONT || face > BD_FACE_BOTH) return BD_ERR_INVALID_ARGUMENT;
  if (action != BD_SURF_TRANSMIT && action != BD_SURF_REFLECT && action != BD_SURF_ABSORB)
    return BD_ERR_INVALID_ARGUMENT;
  bd_system::Surface& S = h->surfaces[surface];
  for (int f = 0; f < 2; f++) {
    if (face != BD_FACE_BOTH && face != f) continue;
    if (species == BD_ALL_SPECIES) {
      // a later "all" statement overrides the earlier per-species ones
      S.all[f] = (uint8_t)action;
      S.species[f].clear();
    } else {
      if ((int)S.species[f].size() <= species) S.species[f].resize(species + 1, -1);
      S.species[f][species] = (int16_t)action;
    }
  }
  return BD_OK;
}

BD_API bd_status bd_get_surface_action(bd_handle h, int surface, int species, int face, int* action) {
  if (!h || !action || surface < 0 || surface >= (int)h->surfaces.size()) return BD_ERR_INVALID_ARGUMENT;
  if (species < 0 || species >= (int)h->D.size() || (face != BD_FACE_FRONT && face != BD_FACE_BACK))
    return BD_ERR_INVALID_ARGUMENT;
  *action = surface_action(h, surface, species, face);
  return BD_OK;
}

BD_API bd_status bd_add_panel(bd_handle h, int surface, const bd_panel* panel, int* id) {
  if (!h || !panel || surface < 0 || surface >= (int)h->surfaces.size()) return BD_ERR_INVALID_ARGUMENT;
  if (h->finalized) return BD_ERR_ALREADY_FINALIZED;
  if (h->panels.size() >= (1u << 24)) return BD_ERR_CAPACITY;
  bd_panel_info info;
  std::string msg;
  const bd_status st = derive_panel(*panel, surface, &info, &msg);
  if (st) {
    g_last_error = msg;
    return st;
  }
  h->panels.push_back(info);
  if (id) *id = (int)h->panels.size() - 1;
  return BD_OK;
}

BD_API bd_status bd_get_panel(bd_handle h, int id, bd_panel_info* out) {
  if (!h || !out || id < 0 || id >= (int)h->panels.size()) return BD_ERR_INVALID_ARGUMENT;
  *out = h->panels[id];
  return BD_OK;
}

BD_API bd_status bd_get_surface_counts(bd_handle h, int* n_surfaces, int* n_panels) {
  if (!h) return BD_ERR_INVALID_ARGUMENT;
  if (n_surfaces) *n_surfaces = (int)h->surfaces.size();
  if (n_panels) *n_panels = (int)h->panels.size();
  return BD_OK;
}

BD_API bd_status bd_get_counts(bd_handle h, int* n_species, int* n_reactions) {
  if (!h) return BD_ERR_INVALID_ARGUMENT;
  if (n_species) *n_species = (int)h->D.size();
  if (n_reactions) *n_reactions = (int)h->rx.size();
  return BD_OK;
}

BD_API bd_status bd_get_instance_reaction_info(bd_handle h, int inst, int rxn, bd_reaction_info* out) {
  if (!h || !out || rxn < 0 || rxn >= (int)h->rx.size() || inst < 0 || inst >= h->n_inst())
    return BD_ERR_INVALID_ARGUMENT;
  if (!h->finalized) return BD_ERR_NOT_FINALIZED;
  const ReactionDef& r = h->rx[rxn];
  const DerivedReaction& d = h->derived[inst].rx[rxn];
  memset(out, 0, sizeof(*out));
  out->order = r.order;
  out->nprod = r.nprod;
  for (int k = 0; k < 2; k++) {
    out->reactants[k] = r.reactants[k];
    out->products[k] = r.products[k];
    out->product_offsets[k] = d.off[k];
  }
  out->rate = r.rate;
  out->prob = d.prob;
  out->bind_radius = d.bind_radius;
  out->unbind_radius = d.unbind_radius;
  out->geminate_prob = d.gem_prob;
  out->reverse = d.reverse;
  out->flags = d.flags;
  out->channel_threshold = d.thresh;
  return BD_OK;
}

BD_API bd_status bd_get_reaction_info(bd_handle h, int rxn, bd_reaction_info* out) {
  return bd_get_instance_reaction_info(h, 0, rxn, out);
}

BD_API bd_status bd_set_particles(bd_handle h, const float* xyz4, const int* species, size_t n) {
  if (!h || h->n_inst() != 1) return BD_ERR_INVALID_ARGUMENT;
  if (!h->host_only) BD_CUDA(cudaSetDevice(h->device));
  const uint64_t c = n;
  return upload_particles(h, xyz4, species, &c);
}

BD_API bd_status bd_set_ensemble_particles(bd_handle h, const float* xyz4, const int* species, const uint64_t* counts,
                                           int n_instances) {
  if (!h || !counts || n_instances != h->n_inst()) return BD_ERR_INVALID_ARGUMENT;
  if (!h->host_only) BD_CUDA(cudaSetDevice(h->device));
  return upload_particles(h, xyz4, species, counts);
}

BD_API bd_status bd_step(bd_handle h, int nsteps) {
  const Range range("bd_step");
  if (!h || nsteps < 0) return BD_ERR_INVALID_ARGUMENT;
  if (!h->finalized) return BD_ERR_NOT_FINALIZED;
  if (h->host_only) return BD_ERR_NO_DEVICE;
  if (!h->have_particles) return BD_ERR_NOT_FINALIZED;
  BD_CUDA(cudaSetDevice(h->device));
  if (!h->graph1) {
    const bd_status st = build_graphs(h);
    if (st) return st;
  }
  int left = nsteps;
  while (left >= kGraphBatch) {
    BD_CUDA(cudaGraphLaunch(h->graphN, h->stream));
    left -= kGraphBatch;
  }
  while (left-- > 0) BD_CUDA(cudaGraphLaunch(h->graph1, h->stream));
  h->target_step += (uint64_t)nsteps;
  return BD_OK;
}

BD_API bd_status bd_measure_msd(bd_handle h, int inst, int nsteps, double* msd, uint64_t* counts, int n) {
  const Range range("bd_measure_msd");
  if (!h || nsteps < 0 || n < 0 || inst < -1) return BD_ERR_INVALID_ARGUMENT;
  if (!h->finalized) return BD_ERR_NOT_FINALIZED;
  if (inst >= h->n_inst()) return BD_ERR_INVALID_ARGUMENT;
  for (int s = 0; s < n; s++) {
    if (msd) msd[s] = 0.0;
    if (counts) counts[s] = 0;
  }
  if (h->host_only) return BD_ERR_NO_DEVICE;
  if (!h->have_particles) return BD_ERR_NOT_FINALIZED;
  if (!h->panels.empty()) return BD_ERR_UNSUPPORTED;  // the move would also need the surface walk
  BD_CUDA(cudaSetDevice(h->device));
  bd_status st = bd_synchronize(h);
  if (st && st != BD_ERR_EMPTY) return st;
  if (!h->graph1) {
    st = build_graphs(h);
    if (st) return st;
  }
  const size_t m = (size_t)h->n_inst() * h->S;
  DevBuf<double> sum;
  DevBuf<unsigned long long> cnt;
  BD_CUDA(sum.alloc(m));
  BD_CUDA(cnt.alloc(m));
  BD_CUDA(cudaMemsetAsync(sum.p, 0, m * sizeof(double), h->stream));
  BD_CUDA(cudaMemsetAsync(cnt.p, 0, m * sizeof(unsigned long long), h->stream));
  const bool table = h->cfg.normal_mode == BD_NORMALS_TABLE;
  for (int k = 0; k < nsteps; k++) {
    // one step at a time, synchronised: a step that overflows is replayed
    // by bd_synchronize at once (with grown buffers, so the parameters are
    // taken again); its moves were measured before it first ran and the
    // replay repeats the same moves unmeasured
    enqueue_msd(make_params(h), table, sum.p, cnt.p, h->stream);
    BD_CUDA(cudaGetLastError());
    if (!h->graph1) {
      st = build_graphs(h);
      if (st) return st;
    }
    BD_CUDA(cudaGraphLaunch(h->graph1, h->stream));
    h->target_step += 1;
    st = bd_synchronize(h);
    if (st && st != BD_ERR_EMPTY) return st;
  }
  std::vector<double> hs(m);
  std::vector<unsigned long long> hc(m);
  BD_CUDA(cudaMemcpyAsync(hs.data(), sum.p, m * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  BD_CUDA(cudaMemcpyAsync(hc.data(), cnt.p, m * sizeof(unsigned long long), cudaMemcpyDeviceToHost, h->stream));
  BD_CUDA(cudaStreamSynchronize(h->stream));
  sum.free();
  cnt.free();
  for (int s = 0; s < std::min(n, h->S); s++) {
    double a = 0.0;
    unsigned long long b = 0;
    for (int k = 0; k < h->n_inst(); k++) {
      if (inst >= 0 && k != inst) continue;
      a += hs[(size_t)k * h->S + s];
      b += hc[(size_t)k * h->S + s];
    }
    if (msd) msd[s] = b ? a / (double)b : 0.0;
    if (counts) counts[s] = b;
  }
  return BD_OK;
}

BD_API bd_status bd_step_async(bd_handle h, int nsteps, void* stream) {
  const Range range("bd_step_async");
  if (!h || nsteps < 0) return BD_ERR_INVALID_ARGUMENT;
  if (h->host_only) return BD_ERR_NO_DEVICE;
  BD_CUDA(cudaSetDevice(h->device));
  cudaStream_t caller = (cudaStream_t)stream;
  cudaEvent_t before, after;
  BD_CUDA(cudaEventCreateWithFlags(&before, cudaEventDisableTiming));
  if (!cuda_ok(cudaEventCreateWithFlags(&after, cudaEventDisableTiming), "cudaEventCreate")) {
    cudaEventDestroy(before);
    return BD_ERR_CUDA;
  }
  bd_status st = BD_OK;
  if (!cuda_ok(cudaEventRecord(before, caller), "cudaEventRecord") ||
      !cuda_ok(cudaStreamWaitEvent(h->stream, before, 0), "cudaStreamWaitEvent"))
    st = BD_ERR_CUDA;
  if (!st) st = bd_step(h, nsteps);
  if (!st && (!cuda_ok(cudaEventRecord(after, h->stream), "cudaEventRecord") ||
              !cuda_ok(cudaStreamWaitEvent(caller, after, 0), "cudaStreamWaitEvent")))
    st = BD_ERR_CUDA;
  cudaEventDestroy(before);
  cudaEventDestroy(after);
  return st;
}

BD_API bd_status bd_synchronize(bd_handle h) {
  const Range range("bd_synchronize");
  if (!h) return BD_ERR_INVALID_ARGUMENT;
  if (!h->have_particles) return BD_OK;
  BD_CUDA(cudaSetDevice(h->device));
  for (int attempt = 0; attempt < 64; attempt++) {
    bd_status st = sync_ctrl(h);
    if (st) return st;
    DevCtrl& c = *h->hctrl;
    if (c.status == 0) {
      if (c.step >= h->target_step) break;
      // a previous failed step stopped the queue; replay the rest
    } else {
      if (c.status & (kStatBounds | kStatTimeout)) {
        g_last_error = "device reported an inconsistent state";
        return (c.status & kStatTimeout) ? BD_ERR_TIMEOUT : BD_ERR_DEVICE_STATE;
      }
      if (c.status & kStatCapacity) {
        uint64_t need = std::max<uint64_t>(c.n_sorted, (uint64_t)c.n_slots + c.n_virtual);
        uint64_t cap = std::max<uint64_t>(2 * h->capacity, need + need / 2 + 1024);
        st = grow_particles(h, cap);
        if (st) return st;
      }
      if (c.status & kStatBins) {
        // a cell outgrew its bin: larger bins, or the compact sort when
        // they would not fit the automatic budget
        uint64_t K = std::max<uint64_t>((uint64_t)c.bin_need + c.bin_need / 4 + 4, (uint64_t)h->bin_cap + 8);
        K = (K + kBinGroup - 1) / kBinGroup * kBinGroup;
        const bool fits = (uint64_t)h->n_cells * K * sizeof(float4) <= kBinBudgetBytes;
        if (K > 0xFFFFFFF0ull || (!fits && h->cfg.sort_mode != BD_SORT_BINNED)) {
          h->binned = false;
          st = ensure_sort_buffers(h, h->bin_cap);
        } else {
          st = ensure_sort_buffers(h, (uint32_t)K);
        }
        if (st) return st;
        c.bin_need = 0;
      }
      if (c.status & kStatScratch) BD_CUDA(h->big_scratch.alloc(h->capacity));
      if (c.status & kStatPairs) {
        uint64_t cap = std::max<uint64_t>(2ull * h->pair_cap, (uint64_t)c.n_pairs + c.n_pairs / 2 + 1024);
        if (cap > 0x7FFFFFFFull) return BD_ERR_CAPACITY;
        st = grow_pairs(h, (uint32_t)cap);
        if (st) return st;
      }
      BD_CUDA(cudaMemsetAsync(h->cell_count.p, 0, (size_t)h->n_cells * sizeof(uint32_t), h->stream));
      BD_CUDA(cudaMemsetAsync(h->pending.p, 0, h->pending.n * sizeof(unsigned long long), h->stream));
      c.status = 0;
      c.n_pairs = 0;
      c.n_big = 0;
      c.n_surf = 0;
      c.surf_ticket = 0;
      c.n_virtual = 0;
      c.bar_count = 0;
      st = push_ctrl(h);
      if (st) return st;
      st = build_graphs(h);
      if (st) return st;
    }
    const uint64_t left = h->target_step - c.step;
    if (left == 0) break;
    h->target_step = c.step;
    st = bd_step(h, (int)left);
    if (st) return st;
  }
  const DevCtrl& c = *h->hctrl;
  if (c.step < h->target_step) return BD_ERR_CAPACITY;
  if ((uint64_t)c.n_slots - c.deaths_last == 0) return BD_ERR_EMPTY;
  return BD_OK;
}

BD_API bd_status bd_get_step(bd_handle h, uint64_t* step) {
  if (!h || !step) return BD_ERR_INVALID_ARGUMENT;
  bd_status st = bd_synchronize(h);
  if (st && st != BD_ERR_EMPTY) return st;
  *step = h->hctrl->step;
  return BD_OK;
}

BD_API bd_status bd_get_count(bd_handle h, uint64_t* n) {
  if (!h || !n) return BD_ERR_INVALID_ARGUMENT;
  if (!h->have_particles) {
    *n = 0;
    return BD_OK;
  }
  bd_status st = bd_synchronize(h);
  if (st && st != BD_ERR_EMPTY) return st;
  *n = (uint64_t)h->hctrl->n_slots - h->hctrl->deaths_last;
  return BD_OK;
}

namespace {
bd_status read_slots(bd_system* h, std::vector<float4>* out) {
  bd_status st = bd_synchronize(h);
  if (st && st != BD_ERR_EMPTY) return st;
  const uint32_t n = h->hctrl->n_slots;
  out->resize(n);
  const float4* src = h->hctrl->cur ? h->state1.p : h->state0.p;
  if (n) BD_CUDA(cudaMemcpy(out->data(), src, (size_t)n * sizeof(float4), cudaMemcpyDeviceToHost));
  return BD_OK;
}
}  // namespace

BD_API bd_status bd_get_particles(bd_handle h, float* xyz4, int* species, size_t cap, size_t* n) {
  return bd_get_instance_particles(h, -1, xyz4, species, cap, n);
}

BD_API bd_status bd_get_instance_particles(bd_handle h, int inst, float* xyz4, int* species, size_t cap,
                                           size_t* n) {
  const Range range("bd_get_particles");
  if (!h || !n) return BD_ERR_INVALID_ARGUMENT;
  if (inst >= h->n_inst()) return BD_ERR_INVALID_ARGUMENT;
  *n = 0;
  if (!h->have_particles) return BD_OK;
  bd_status st = bd_synchronize(h);
  if (st && st != BD_ERR_EMPTY) return st;
  // the live records in slot order, exported on the device and copied whole
  const uint64_t slots = h->hctrl->n_slots;
  const uint32_t tiles = export_tiles(slots);
  Scratch scratch;
  BD_CUDA(scratch.alloc(scratch_bytes({slots * sizeof(float4), slots * sizeof(int), tiles * sizeof(uint32_t),
                                       sizeof(uint32_t)}),
                        h->stream, h->pool));
  ExportArgs a{};
  a.state = h->hctrl->cur ? h->state1.p : h->state0.p;
  a.n_slots = slots;
  a.inst = inst;
  a.n_tiles = tiles;
  a.xyz4 = scratch.take<float4>(slots);
  a.species = scratch.take<int>(slots);
  a.tile_offset = scratch.take<uint32_t>(tiles);
  a.count = scratch.take<uint32_t>(1);
  enqueue_export(a, h->stream);
  BD_CUDA(cudaGetLastError());
  uint32_t total = 0;
  BD_CUDA(cudaMemcpyAsync(&total, a.count, sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream));
  BD_CUDA(cudaStreamSynchronize(h->stream));
  const size_t m = std::min<size_t>(total, cap);
  if (m && xyz4) BD_CUDA(cudaMemcpyAsync(xyz4, a.xyz4, m * sizeof(float4), cudaMemcpyDeviceToHost, h->stream));
  if (m && species) BD_CUDA(cudaMemcpyAsync(species, a.species, m * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  BD_CUDA(cudaStreamSynchronize(h->stream));
  *n = total;
  return BD_OK;
}

BD_API bd_status bd_get_state_pointer(bd_handle h, void** dev_records, uint64_t* n_slots) {
  if (!h || !dev_records || !n_slots) return BD_ERR_INVALID_ARGUMENT;
  *dev_records = nullptr;
  *n_slots = 0;
  if (!h->have_particles) return BD_OK;
  bd_status st = bd_synchronize(h);
  if (st && st != BD_ERR_EMPTY) return st;
  *dev_records = h->hctrl->cur ? (void*)h->state1.p : (void*)h->state0.p;
  *n_slots = h->hctrl->n_slots;
  return BD_OK;
}

// ------------------------------------------------------------------ serving

BD_API bd_status bd_create_server(const bd_config* cfg, int max_instances, bd_handle* out) {
  if (!cfg || max_instances < 1 || (uint32_t)max_instances > kMaxInstances) return BD_ERR_INVALID_ARGUMENT;
  std::vector<bd_instance_desc> d(max_instances);
  for (int k = 0; k < max_instances; k++) {
    memset(&d[k], 0, sizeof(d[k]));
    memcpy(d[k].box_lo, cfg->box_lo, sizeof(d[k].box_lo));
    memcpy(d[k].box_hi, cfg->box_hi, sizeof(d[k].box_hi));
    d[k].seed = cfg->seed + (uint64_t)k;
    d[k].d_scale = d[k].k2_scale = 1.0f;
  }
  bd_status st = create_common(cfg, d.data(), max_instances, out);
  if (st) return st;
  bd_system* h = *out;
  h->server = true;
  h->slot_used.assign(max_instances, 0);
  h->slot_free_after.assign(max_instances, UINT64_MAX);
  return BD_OK;
}

namespace {

// Records in the order a sort of one step leaves them: by cell key (the
// device's cell_key, the same correctly rounded float operations), then by
// the record's words as unsigned integers.  Empty slots go last.
void canonical_sort(const DevInstance& I, std::vector<float4>* recs) {
  struct Keyed {
    uint32_t key, x, y, z, w;
  };
  std::vector<Keyed> v(recs->size());
  for (size_t i = 0; i < recs->size(); i++) {
    const float4 q = (*recs)[i];
    Keyed& e = v[i];
    memcpy(&e.x, &q.x, 4);
    memcpy(&e.y, &q.y, 4);
    memcpy(&e.z, &q.z, 4);
    memcpy(&e.w, &q.w, 4);
    if (e.w == kDead) {
      e.key = 0xFFFFFFFFu;
      continue;
    }
    const float xyz[3] = {q.x, q.y, q.z};
    uint32_t c[3];
    for (int a = 0; a < 3; a++) {
      const float f = (xyz[a] - I.lo[a]) * I.inv[a];
      int ci = (int)floorf(f);
      ci = ci < 0 ? 0 : (ci > (int)I.dims[a] - 1 ? (int)I.dims[a] - 1 : ci);
      c[a] = (uint32_t)ci;
    }
    e.key = (c[2] * I.dims[1] + c[1]) * I.dims[0] + c[0];
  }
  std::sort(v.begin(), v.end(), [](const Keyed& a, const Keyed& b) {
    if (a.key != b.key) return a.key < b.key;
    if (a.x != b.x) return a.x < b.x;
    if (a.y != b.y) return a.y < b.y;
    if (a.z != b.z) return a.z < b.z;
    return a.w < b.w;
  });
  for (size_t i = 0; i < v.size(); i++) {
    float4& q = (*recs)[i];
    memcpy(&q.x, &v[i].x, 4);
    memcpy(&q.y, &v[i].y, 4);
    memcpy(&q.z, &v[i].z, 4);
    memcpy(&q.w, &v[i].w, 4);
  }
}

// Slots whose instance was harvested become free once a step has dropped
// its records.
void release_slots(bd_system* h) {
  for (int k = 0; k < h->n_inst(); k++)
    if (h->slot_free_after[k] != UINT64_MAX && h->hctrl->step > h->slot_free_after[k]) {
      h->slot_used[k] = 0;
      h->slot_free_after[k] = UINT64_MAX;
      h->h_flags[k] = 0;
    }
}

template <class T>
bd_status put1(DevBuf<T>& buf, int k, T v, cudaStream_t s) {
  BD_CUDA(cudaMemcpyAsync(buf.p + k, &v, sizeof(T), cudaMemcpyHostToDevice, s));
  BD_CUDA(cudaStreamSynchronize(s));
  return BD_OK;
}

}  // namespace

BD_API bd_status bd_instance_admit(bd_handle h, const bd_instance_desc* d, const float* xyz4, const int* species,
                                   size_t n, uint32_t steps, int* slot_out) {
  const Range range("bd_instance_admit");
  if (!h || !h->server || !d || !slot_out || steps == 0 || (n > 0 && (!xyz4 || !species)))
    return BD_ERR_INVALID_ARGUMENT;
  if (!h->finalized) return BD_ERR_NOT_FINALIZED;
  if (h->host_only) return BD_ERR_NO_DEVICE;
  for (int a = 0; a < 3; a++)
    if (!(d->box_hi[a] > d->box_lo[a])) return BD_ERR_INVALID_ARGUMENT;
  BD_CUDA(cudaSetDevice(h->device));
  const int I = h->n_inst();
  bd_status st;
  if (h->have_particles) {
    st = bd_synchronize(h);
    if (st && st != BD_ERR_EMPTY) return st;
  }
  if (h->h_flags.size() != (size_t)I) {
    h->h_flags.assign(I, 0);
    h->h_target.assign(I, 0xFFFFFFFFu);
  }
  release_slots(h);
  int k = -1;
  for (int j = 0; j < I && k < 0; j++)
    if (!h->slot_used[j] && h->slot_free_after[j] == UINT64_MAX) k = j;
  if (k < 0) return BD_ERR_CAPACITY;
  bd_instance_desc dd = *d;
  if (!(dd.d_scale > 0)) dd.d_scale = 1.0f;
  if (!(dd.k2_scale > 0)) dd.k2_scale = 1.0f;
  const float vol = (dd.box_hi[0] - dd.box_lo[0]) * (dd.box_hi[1] - dd.box_lo[1]) * (dd.box_hi[2] - dd.box_lo[2]);
  DerivedParams P = derive_params(h->D, h->rx, h->cfg.dt, vol, dd.d_scale, dd.k2_scale,
                                  h->cfg.pair_mode == BD_PAIR_CHANNELS);
  if (P.status == BD_ERR_NEGATIVE_RATE || P.status == BD_ERR_ZERO_DIFFUSION || P.status == BD_ERR_ILLEGAL_UNBIND)
    return P.status;
  // the request's particles: copied whole, checked on the device before
  // the handle changes, packed into the state after its current records
  Scratch scratch;
  UploadArgs up{};
  if (n) {
    const uint64_t start[2] = {0, (uint64_t)n};
    const float box[6] = {dd.box_lo[0], dd.box_lo[1], dd.box_lo[2], dd.box_hi[0], dd.box_hi[1], dd.box_hi[2]};
    BD_CUDA(scratch.alloc(scratch_bytes({n * sizeof(float4), n * sizeof(int), sizeof(start), sizeof(box),
                                         sizeof(uint32_t)}),
                          h->stream, h->pool));
    float4* d_xyz4 = scratch.take<float4>(n);
    int* d_species = scratch.take<int>(n);
    uint64_t* d_start = scratch.take<uint64_t>(2);
    float* d_box = scratch.take<float>(6);
    uint32_t* d_bad = scratch.take<uint32_t>(1);
    BD_CUDA(cudaMemcpyAsync(d_xyz4, xyz4, n * sizeof(float4), cudaMemcpyHostToDevice, h->stream));
    BD_CUDA(cudaMemcpyAsync(d_species, species, n * sizeof(int), cudaMemcpyHostToDevice, h->stream));
    BD_CUDA(cudaMemcpyAsync(d_start, start, sizeof(start), cudaMemcpyHostToDevice, h->stream));
    BD_CUDA(cudaMemcpyAsync(d_box, box, sizeof(box), cudaMemcpyHostToDevice, h->stream));
    BD_CUDA(cudaMemsetAsync(d_bad, 0, sizeof(uint32_t), h->stream));
    up = UploadArgs{d_xyz4, d_species, d_start, d_box, (uint64_t)n, 1, h->S, d_bad, (uint32_t)k};
    enqueue_upload_check(up, h->stream);
    BD_CUDA(cudaGetLastError());
    uint32_t bad = 0;
    BD_CUDA(cudaMemcpyAsync(&bad, d_bad, sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream));
    BD_CUDA(cudaStreamSynchronize(h->stream));
    if (bad) return BD_ERR_INVALID_ARGUMENT;
  }
  h->idesc[k] = dd;
  h->derived[k] = P;
  if ((st = pack_blocks(h))) return st;
  if (h->hinst.size() != (size_t)I) h->hinst.assign(I, DevInstance{});
  h->slot_used[k] = 1;
  plan_instance(h, k, n);
  if ((st = layout_cells(h))) return st;
  if (!h->have_particles) {
    const uint64_t cap = std::max<uint64_t>(h->cfg.capacity, std::max<uint64_t>(2 * n, 1u << 20));
    memset(h->hctrl, 0, sizeof(DevCtrl));
    if ((st = grow_particles(h, cap))) return st;
    const uint32_t pc = h->cfg.pair_capacity ? h->cfg.pair_capacity : (uint32_t)std::max<uint64_t>(65536, cap / 32);
    if ((st = grow_pairs(h, pc))) return st;
    std::vector<uint32_t> zeros(I, 0);
    if ((st = upload(h->inst_step, zeros, h->stream)) || (st = upload(h->inst_slot_base, zeros, h->stream)) ||
        (st = upload(h->inst_flags, h->h_flags, h->stream)) || (st = upload(h->inst_target, h->h_target, h->stream)) ||
        (st = upload(h->inst_frozen, zeros, h->stream)))
      return st;
    BD_CUDA(h->zero_off.alloc((size_t)I * h->Z + 1));
    BD_CUDA(cudaMemsetAsync(h->zero_off.p, 0, ((size_t)I * h->Z + 1) * sizeof(uint32_t), h->stream));
    BD_CUDA(h->events.alloc((size_t)I * std::max(h->R, 1)));
    BD_CUDA(h->pending.alloc((size_t)I * std::max(h->R, 1)));
    BD_CUDA(cudaMemsetAsync(h->pending.p, 0, h->pending.n * sizeof(unsigned long long), h->stream));
    h->have_particles = true;
    h->target_step = 0;
    if ((st = push_ctrl(h))) return st;
  }
  const uint64_t n_slots = h->hctrl->n_slots;
  if (n_slots + n > h->capacity) {
    if ((st = grow_particles(h, std::max<uint64_t>(2 * h->capacity, (n_slots + n) * 3 / 2)))) return st;
    if ((st = push_ctrl(h))) return st;
  }
  float4* cur = h->hctrl->cur ? h->state1.p : h->state0.p;
  if (n) {
    enqueue_upload_pack(up, cur + n_slots, h->stream);
    BD_CUDA(cudaGetLastError());
  }
  BD_CUDA(cudaMemsetAsync(h->events.p + (size_t)k * std::max(h->R, 1), 0,
                          std::max(h->R, 1) * sizeof(unsigned long long), h->stream));
  h->h_flags[k] = kInstActive;
  h->h_target[k] = steps;
  if ((st = put1(h->inst_step, k, 0u, h->stream)) || (st = put1(h->inst_slot_base, k, (uint32_t)n_slots, h->stream)) ||
      (st = put1(h->inst_flags, k, (uint32_t)kInstActive, h->stream)) || (st = put1(h->inst_target, k, steps, h->stream)))
    return st;
  h->hctrl->n_slots = (uint32_t)(n_slots + n);
  if ((st = push_ctrl(h))) return st;
  if ((st = build_graphs(h))) return st;
  *slot_out = k;
  return BD_OK;
}

BD_API bd_status bd_instance_state(bd_handle h, int k, uint32_t* steps, uint32_t* flags) {
  if (!h || !h->server || k < 0 || k >= h->n_inst()) return BD_ERR_INVALID_ARGUMENT;
  if (!h->have_particles) {
    if (steps) *steps = 0;
    if (flags) *flags = 0;
    return BD_OK;
  }
  bd_status st = bd_synchronize(h);
  if (st && st != BD_ERR_EMPTY) return st;
  uint32_t s = 0, f = 0;
  BD_CUDA(cudaMemcpy(&s, h->inst_step.p + k, 4, cudaMemcpyDeviceToHost));
  BD_CUDA(cudaMemcpy(&f, h->inst_flags.p + k, 4, cudaMemcpyDeviceToHost));
  if (steps) *steps = s;
  if (flags) *flags = h->slot_used[k] ? f : 0;
  return BD_OK;
}

BD_API bd_status bd_instance_poll(bd_handle h, int* slots, int cap, int* n_finished) {
  if (!h || !h->server || !n_finished) return BD_ERR_INVALID_ARGUMENT;
  *n_finished = 0;
  if (!h->have_particles) return BD_OK;
  bd_status st = bd_synchronize(h);
  if (st && st != BD_ERR_EMPTY) return st;
  const int I = h->n_inst();
  std::vector<uint32_t> f(I);
  BD_CUDA(cudaMemcpy(f.data(), h->inst_flags.p, I * sizeof(uint32_t), cudaMemcpyDeviceToHost));
  int m = 0;
  for (int k = 0; k < I; k++)
    if (h->slot_used[k] && h->slot_free_after[k] == UINT64_MAX && (f[k] & kInstFrozen)) {
      if (slots && m < cap) slots[m] = k;
      m++;
    }
  *n_finished = m;
  return BD_OK;
}

BD_API bd_status bd_instance_harvest(bd_handle h, int k, float* xyz4, int* species, size_t cap, size_t* n) {
  const Range range("bd_instance_harvest");
  if (!h || !h->server || !n || k < 0 || k >= h->n_inst()) return BD_ERR_INVALID_ARGUMENT;
  *n = 0;
  if (!h->slot_used[k] || h->slot_free_after[k] != UINT64_MAX) return BD_ERR_INVALID_ARGUMENT;
  bd_status st = bd_synchronize(h);
  if (st && st != BD_ERR_EMPTY) return st;
  const int I = h->n_inst();
  std::vector<uint32_t> base(I), f(I);
  uint32_t frozen_at = 0;
  BD_CUDA(cudaMemcpy(base.data(), h->inst_slot_base.p, I * sizeof(uint32_t), cudaMemcpyDeviceToHost));
  BD_CUDA(cudaMemcpy(f.data(), h->inst_flags.p, I * sizeof(uint32_t), cudaMemcpyDeviceToHost));
  BD_CUDA(cudaMemcpy(&frozen_at, h->inst_frozen.p + k, sizeof(uint32_t), cudaMemcpyDeviceToHost));
  if (!(f[k] & kInstFrozen)) return BD_ERR_INVALID_ARGUMENT;
  // the instance's records are contiguous: up to the next instance's first slot
  uint64_t end = h->hctrl->n_slots;
  for (int j = 0; j < I; j++)
    if (j != k && h->slot_used[j] && base[j] > base[k] && base[j] < end) end = base[j];
  const uint64_t len = end > base[k] ? end - base[k] : 0;
  const float4* cur = h->hctrl->cur ? h->state1.p : h->state0.p;
  // The step's last phase puts reaction products in their reactants' slots,
  // so the state is in canonical order only up to those slots; the next
  // sort restores it (a frozen instance neither moves nor reacts).  Harvest
  // in canonical order, so the result does not depend on how many frozen
  // steps ran before it: after a frozen step the records are exported as
  // they lie, on the device; right after the freeze they are sorted here.
  const bool sorted = (uint32_t)((uint32_t)h->hctrl->step - frozen_at) >= 2u;
  if (sorted) {
    const uint32_t tiles = export_tiles(len);
    Scratch scratch;
    BD_CUDA(scratch.alloc(scratch_bytes({len * sizeof(float4), len * sizeof(int), tiles * sizeof(uint32_t),
                                         sizeof(uint32_t)}),
                          h->stream, h->pool));
    ExportArgs a{};
    a.state = cur + base[k];
    a.n_slots = len;
    a.inst = k;
    a.n_tiles = tiles;
    a.xyz4 = scratch.take<float4>(len);
    a.species = scratch.take<int>(len);
    a.tile_offset = scratch.take<uint32_t>(tiles);
    a.count = scratch.take<uint32_t>(1);
    enqueue_export(a, h->stream);
    BD_CUDA(cudaGetLastError());
    uint32_t total = 0;
    BD_CUDA(cudaMemcpyAsync(&total, a.count, sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream));
    BD_CUDA(cudaStreamSynchronize(h->stream));
    const size_t m = std::min<size_t>(total, cap);
    if (m && xyz4) BD_CUDA(cudaMemcpyAsync(xyz4, a.xyz4, m * sizeof(float4), cudaMemcpyDeviceToHost, h->stream));
    if (m && species)
      BD_CUDA(cudaMemcpyAsync(species, a.species, m * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    BD_CUDA(cudaStreamSynchronize(h->stream));
    *n = total;
    h->h_flags[k] = f[k] | kInstRemoved;
    if ((st = put1(h->inst_flags, k, h->h_flags[k], h->stream))) return st;
    h->slot_free_after[k] = h->hctrl->step;
    return BD_OK;
  }
  std::vector<float4> r(len);
  if (len) BD_CUDA(cudaMemcpy(r.data(), cur + base[k], len * sizeof(float4), cudaMemcpyDeviceToHost));
  canonical_sort(h->hinst[k], &r);
  size_t m = 0;
  for (const float4& q : r) {
    uint32_t w;
    memcpy(&w, &q.w, 4);
    if (w == kDead || (int)(w >> 16) != k) continue;
    if (m < cap) {
      if (xyz4) {
        xyz4[4 * m] = q.x;
        xyz4[4 * m + 1] = q.y;
        xyz4[4 * m + 2] = q.z;
        xyz4[4 * m + 3] = 1.0f;
      }
      if (species) species[m] = (int)(w & 0xFFFFu);
    }
    m++;
  }
  *n = m;
  h->h_flags[k] = f[k] | kInstRemoved;
  if ((st = put1(h->inst_flags, k, h->h_flags[k], h->stream))) return st;
  h->slot_free_after[k] = h->hctrl->step;
  return BD_OK;
}

BD_API bd_status bd_instance_cancel(bd_handle h, int k) {
  const Range range("bd_instance_cancel");
  if (!h || !h->server || k < 0 || k >= h->n_inst()) return BD_ERR_INVALID_ARGUMENT;
  if (!h->slot_used[k] || h->slot_free_after[k] != UINT64_MAX) return BD_ERR_INVALID_ARGUMENT;
  bd_status st = bd_synchronize(h);
  if (st && st != BD_ERR_EMPTY) return st;
  // the device may have frozen it meanwhile: start from its flags there
  uint32_t f = 0;
  BD_CUDA(cudaMemcpy(&f, h->inst_flags.p + k, sizeof(uint32_t), cudaMemcpyDeviceToHost));
  h->h_flags[k] = f | kInstRemoved;
  if ((st = put1(h->inst_flags, k, h->h_flags[k], h->stream))) return st;
  h->slot_free_after[k] = h->hctrl->step;
  return BD_OK;
}

BD_API bd_status bd_get_instance_counts(bd_handle h, uint64_t* counts, int n_instances) {
  if (!h || !counts || n_instances != h->n_inst()) return BD_ERR_INVALID_ARGUMENT;
  if (!h->have_particles) {
    for (int k = 0; k < n_instances; k++) counts[k] = 0;
    return BD_OK;
  }
  bd_status st = bd_synchronize(h);
  if (st && st != BD_ERR_EMPTY) return st;
  DevBuf<unsigned long long> d;
  BD_CUDA(d.alloc(n_instances));
  BD_CUDA(cudaMemsetAsync(d.p, 0, n_instances * sizeof(unsigned long long), h->stream));
  enqueue_instance_counts(make_params(h), d.p, h->stream);
  BD_CUDA(cudaGetLastError());
  BD_CUDA(cudaMemcpyAsync(counts, d.p, n_instances * sizeof(unsigned long long), cudaMemcpyDeviceToHost, h->stream));
  BD_CUDA(cudaStreamSynchronize(h->stream));
  d.free();
  return BD_OK;
}

BD_API bd_status bd_get_species_counts(bd_handle h, int inst, uint64_t* counts, int n) {
  if (!h || !counts || n < 0 || inst < -1 || inst >= h->n_inst()) return BD_ERR_INVALID_ARGUMENT;
  for (int s = 0; s < n; s++) counts[s] = 0;
  if (!h->have_particles) return BD_OK;
  bd_status st = bd_synchronize(h);
  if (st && st != BD_ERR_EMPTY) return st;
  const size_t m = (size_t)h->n_inst() * h->S;
  DevBuf<unsigned long long> d;
  BD_CUDA(d.alloc(m));
  BD_CUDA(cudaMemsetAsync(d.p, 0, m * sizeof(unsigned long long), h->stream));
  enqueue_species_counts(make_params(h), d.p, h->stream);
  BD_CUDA(cudaGetLastError());
  std::vector<unsigned long long> hv(m);
  BD_CUDA(cudaMemcpyAsync(hv.data(), d.p, m * sizeof(unsigned long long), cudaMemcpyDeviceToHost, h->stream));
  BD_CUDA(cudaStreamSynchronize(h->stream));
  d.free();
  for (int k = 0; k < h->n_inst(); k++) {
    if (inst >= 0 && k != inst) continue;
    for (int s = 0; s < std::min(n, h->S); s++) counts[s] += hv[(size_t)k * h->S + s];
  }
  return BD_OK;
}

BD_API bd_status bd_get_event_counts(bd_handle h, uint64_t* counts, int n) {
  if (!h || !counts || n < 0) return BD_ERR_INVALID_ARGUMENT;
  for (int r = 0; r < n; r++) counts[r] = 0;
  if (!h->have_particles) return BD_OK;
  bd_status st = bd_synchronize(h);
  if (st && st != BD_ERR_EMPTY) return st;
  const int I = h->n_inst(), R = std::max(h->R, 1);
  std::vector<unsigned long long> ev((size_t)I * R);
  BD_CUDA(cudaMemcpy(ev.data(), h->events.p, ev.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
  for (int k = 0; k < I; k++)
    for (int r = 0; r < std::min(n, h->R); r++) counts[r] += ev[(size_t)k * R + r];
  return BD_OK;
}

BD_API bd_status bd_time_steps(bd_handle h, int nsteps, float* ms) {
  if (!h || !ms || nsteps < 0) return BD_ERR_INVALID_ARGUMENT;
  if (h->host_only) return BD_ERR_NO_DEVICE;
  BD_CUDA(cudaSetDevice(h->device));
  cudaEvent_t e0, e1;
  BD_CUDA(cudaEventCreate(&e0));
  BD_CUDA(cudaEventCreate(&e1));
  BD_CUDA(cudaEventRecord(e0, h->stream));
  bd_status st = bd_step(h, nsteps);
  if (!st) {
    BD_CUDA(cudaEventRecord(e1, h->stream));
    BD_CUDA(cudaEventSynchronize(e1));
    BD_CUDA(cudaEventElapsedTime(ms, e0, e1));
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st) return st;
  return bd_synchronize(h);
}

namespace {
struct ProfileCtx {
  cudaStream_t stream;
  std::vector<cudaEvent_t>* events;
  std::vector<std::string>* names;
  bool record_names;
};
void profile_hook(void* c, const char* name) {
  ProfileCtx* p = (ProfileCtx*)c;
  cudaEvent_t e;
  cudaEventCreate(&e);
  cudaEventRecord(e, p->stream);
  p->events->push_back(e);
  if (p->record_names) p->names->push_back(name);
}
}  // namespace

BD_API bd_status bd_profile_steps(bd_handle h, int nsteps, float* stage_ms, int cap, int* n_stages) {
  if (!h || nsteps < 1 || !n_stages) return BD_ERR_INVALID_ARGUMENT;
  if (h->host_only) return BD_ERR_NO_DEVICE;
  if (!h->finalized || !h->have_particles) return BD_ERR_NOT_FINALIZED;
  BD_CUDA(cudaSetDevice(h->device));
  bd_status st = bd_synchronize(h);
  if (st && st != BD_ERR_EMPTY) return st;
  const KParams p = make_params(h);
  const bool table = h->cfg.normal_mode == BD_NORMALS_TABLE;
  const Path path = h->path();
  std::vector<float> acc;
  h->stage_names.clear();
  for (int k = 0; k < nsteps; k++) {
    std::vector<cudaEvent_t> ev;
    cudaEvent_t e0;
    BD_CUDA(cudaEventCreate(&e0));
    BD_CUDA(cudaEventRecord(e0, h->stream));
    ev.push_back(e0);
    ProfileCtx ctx{h->stream, &ev, &h->stage_names, k == 0};
    const int nk = enqueue_step(p, path, table, h->Z > 0, h->U > 0, h->B > 0, h->shape, h->stream, profile_hook,
                                &ctx);
    BD_CUDA(cudaGetLastError());
    BD_CUDA(cudaEventSynchronize(ev.back()));
    if (acc.empty()) acc.assign(nk, 0.0f);
    for (int s = 0; s < nk && s + 1 < (int)ev.size(); s++) {
      float ms = 0;
      cudaEventElapsedTime(&ms, ev[s], ev[s + 1]);
      acc[s] += ms;
    }
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
    h->target_step += 1;
  }
  *n_stages = (int)acc.size();
  if (stage_ms)
    for (int s = 0; s < (int)acc.size() && s < cap; s++) stage_ms[s] = acc[s];
  st = bd_synchronize(h);
  return st == BD_ERR_EMPTY ? BD_OK : st;
}

BD_API const char* bd_stage_name(bd_handle h, int k) {
  if (!h || k < 0 || k >= (int)h->stage_names.size()) return "";
  return h->stage_names[k].c_str();
}

BD_API bd_status bd_get_kernels_per_step(bd_handle h, int* n) {
  if (!h || !n) return BD_ERR_INVALID_ARGUMENT;
  if (h->diffuse_only()) *n = (h->Z > 0 ? 2 : 0) + 2;
  // binned: k_bin, k_scan, k_pairs_cells, k_pairs_big, k_match (+ k_bin_surface
  // with panels); compact: k_count, k_scan, k_scatter, k_pairs_cells,
  // k_pairs_big, k_match; k_zeroth first with zeroth-order reactions
  else *n = (h->Z > 0 ? 1 : 0) + (h->binned ? 5 : 6) + (h->binned && !h->panels.empty() ? 1 : 0);
  return BD_OK;
}

BD_API bd_status bd_debug_get_slots(bd_handle h, float* xyz4, uint32_t* w, size_t cap, size_t* n) {
  if (!h || !n) return BD_ERR_INVALID_ARGUMENT;
  *n = 0;
  if (!h->have_particles) return BD_OK;
  std::vector<float4> slots;
  bd_status st = read_slots(h, &slots);
  if (st) return st;
  *n = slots.size();
  for (size_t i = 0; i < slots.size() && i < cap; i++) {
    if (xyz4) {
      xyz4[4 * i] = slots[i].x;
      xyz4[4 * i + 1] = slots[i].y;
      xyz4[4 * i + 2] = slots[i].z;
      xyz4[4 * i + 3] = 0.0f;
    }
    if (w) memcpy(&w[i], &slots[i].w, 4);
  }
  return BD_OK;
}

BD_API bd_status bd_debug_withhold_scan(bd_handle h, int on) {
  if (!h) return BD_ERR_INVALID_ARGUMENT;
  h->scan_withhold = on != 0;
  if (h->graph1 || h->graphN) return build_graphs(h);
  return BD_OK;
}

BD_API bd_status bd_debug_withhold_match(bd_handle h, int on) {
  if (!h) return BD_ERR_INVALID_ARGUMENT;
  h->match_withhold = on != 0;
  if (h->graph1 || h->graphN) return build_graphs(h);
  return BD_OK;
}

BD_API bd_status bd_debug_get_cells(bd_handle h, uint32_t* start, size_t cap, size_t* ncells) {
  if (!h || !ncells) return BD_ERR_INVALID_ARGUMENT;
  *ncells = h->n_cells;
  if (!h->have_particles) return BD_OK;
  bd_status st = bd_synchronize(h);
  if (st && st != BD_ERR_EMPTY) return st;
  if (start) {
    const size_t m = std::min<size_t>(cap, (size_t)h->n_cells + 1);
    BD_CUDA(cudaMemcpy(start, h->cell_start.p, m * sizeof(uint32_t), cudaMemcpyDeviceToHost));
  }
  return BD_OK;
}

BD_API bd_status bd_debug_get_pairs(bd_handle h, uint32_t* quads, size_t cap, size_t* n) {
  if (!h || !n) return BD_ERR_INVALID_ARGUMENT;
  *n = 0;
  if (!h->have_particles) return BD_OK;
  bd_status st = bd_synchronize(h);
  if (st && st != BD_ERR_EMPTY) return st;
  const uint32_t K = h->hctrl->n_pairs_last;
  *n = K;
  if (quads && K) {
    std::vector<DevPair> v(K);
    BD_CUDA(cudaMemcpy(v.data(), h->pairs.p, K * sizeof(DevPair), cudaMemcpyDeviceToHost));
    for (size_t k = 0; k < K && k < cap; k++) {
      quads[4 * k] = v[k].i;
      quads[4 * k + 1] = v[k].j;
      quads[4 * k + 2] = (uint32_t)h->bim_list[v[k].b & 0xFFFFu];
      quads[4 * k + 3] = v[k].state == 1 ? 1u : 0u;
    }
  }
  return BD_OK;
}

BD_API bd_status bd_get_grid(bd_handle h, int inst, uint32_t dims[3], float cell[3], float inv[3]) {
  if (!h || inst < 0) return BD_ERR_INVALID_ARGUMENT;
  if (h->hinst.empty()) return BD_ERR_NOT_FINALIZED;
  if (inst >= (int)h->hinst.size()) return BD_ERR_INVALID_ARGUMENT;
  for (int a = 0; a < 3; a++) {
    if (dims) dims[a] = h->hinst[inst].dims[a];
    if (cell) cell[a] = h->hinst[inst].cell[a];
    if (inv) inv[a] = h->hinst[inst].inv[a];
  }
  return BD_OK;
}

BD_API bd_status bd_get_poisson_cdf(bd_handle h, int inst, int rxn, double* cdf, size_t cap, int* kmin, size_t* len) {
  if (!h || inst < 0 || inst >= h->n_inst() || rxn < 0 || rxn >= (int)h->rx.size()) return BD_ERR_INVALID_ARGUMENT;
  if (!h->finalized) return BD_ERR_NOT_FINALIZED;
  const std::vector<double>& v = h->derived[inst].cdf[rxn];
  if (len) *len = v.size();
  if (kmin) *kmin = h->derived[inst].cdf_kmin[rxn];
  if (cdf)
    for (size_t k = 0; k < v.size() && k < cap; k++) cdf[k] = v[k];
  return BD_OK;
}

BD_API bd_status bd_get_species_d(bd_handle h, int inst, int species, float* D) {
  if (!h || !D || inst < 0 || inst >= h->n_inst() || species < 0 || species >= (int)h->D.size())
    return BD_ERR_INVALID_ARGUMENT;
  if (!h->finalized) return BD_ERR_NOT_FINALIZED;
  *D = h->derived[inst].D[species];
  return BD_OK;
}

BD_API bd_status bd_set_launch_shape(bd_handle h, int bs, int cs, int bp, int cp) {
  if (!h) return BD_ERR_INVALID_ARGUMENT;
  if (bs < 32 || bs > 256 || bs % 32 || bp != 256) return BD_ERR_INVALID_ARGUMENT;
  if (cs < 1 || cs > 64 || cp < 1 || cp > 64) return BD_ERR_INVALID_ARGUMENT;
  h->shape.block_stream = bs;
  h->shape.grid_stream = h->n_sm * cs;
  // a grid of exactly 48 or 32 warps per SM selects the register cap that
  // keeps all of it resident (40 or 64 registers); other grids run uncapped
  const int warps = bs / 32 * cs;
  h->shape.min_blocks = warps == 48 ? 6 : (warps == 32 ? 4 : 1);
  h->shape.block_pairs = bp;
  h->shape.grid_pairs = h->n_sm * cp;
  if (h->host_only || !h->have_particles) return BD_OK;
  bd_status st = bd_synchronize(h);
  if (st && st != BD_ERR_EMPTY) return st;
  return build_graphs(h);
}

BD_API bd_status bd_set_cell_size(bd_handle h, float cell_size) {
  if (!h || !(cell_size >= 0)) return BD_ERR_INVALID_ARGUMENT;
  h->cell_override = cell_size;
  return BD_OK;
}

namespace {
bd_status set_name(std::vector<std::string>* names, size_t n, int id, const char* name) {
  if (!name || id < 0 || (size_t)id >= n) return BD_ERR_INVALID_ARGUMENT;
  names->resize(n);
  (*names)[id] = name;
  return BD_OK;
}
bd_status find_name(const std::vector<std::string>& names, const char* name, int* id) {
  if (!name || !id) return BD_ERR_INVALID_ARGUMENT;
  for (size_t k = 0; k < names.size(); k++)
    if (names[k] == name) {
      *id = (int)k;
      return BD_OK;
    }
  return BD_ERR_INVALID_ARGUMENT;
}
}  // namespace

// ------------------------------------------------------------ checkpoints
namespace {

constexpr char kCkptMagic[8] = {'B', 'D', 'C', 'K', 'P', 'T', '0', '1'};

// What a handle must match to load a checkpoint: the network's shape and
// time step, the normal and pair modes, each instance's box, seed and scales.
std::vector<uint8_t> fingerprint(const bd_system* h) {
  std::vector<uint8_t> f;
  auto put = [&f](const void* p, size_t n) {
    const uint8_t* b = (const uint8_t*)p;
    f.insert(f.end(), b, b + n);
  };
  const int32_t shape[6] = {h->S, h->R, h->n_inst(), h->cfg.normal_mode, (int32_t)h->cfg.pair_mode,
                            (int32_t)h->panels.size()};
  put(shape, sizeof(shape));
  put(&h->cfg.dt, sizeof(float));
  put(h->D.data(), h->D.size() * sizeof(float));
  for (const ReactionDef& r : h->rx) {
    const int32_t v[5] = {r.order, r.reactants[0], r.reactants[1], r.products[0], r.products[1]};
    put(v, sizeof(v));
    put(&r.rate, sizeof(r.rate));
  }
  for (const bd_instance_desc& d : h->idesc) {
    put(d.box_lo, sizeof(d.box_lo));
    put(d.box_hi, sizeof(d.box_hi));
    put(&d.seed, sizeof(d.seed));
    put(&d.d_scale, sizeof(float));
    put(&d.k2_scale, sizeof(float));
    put(&d.cell_size, sizeof(float));
  }
  return f;
}

struct File {
  FILE* f = nullptr;
  ~File() {
    if (f) fclose(f);
  }
};

}  // namespace

BD_API bd_status bd_save_checkpoint(bd_handle h, const char* path) {
  const Range range("bd_save_checkpoint");
  if (!h || !path || h->server) return BD_ERR_INVALID_ARGUMENT;
  if (h->host_only) return BD_ERR_NO_DEVICE;
  if (!h->have_particles) return BD_ERR_NOT_FINALIZED;
  bd_status st = bd_synchronize(h);
  if (st && st != BD_ERR_EMPTY) return st;
  const int I = h->n_inst();
  const DevCtrl c = *h->hctrl;
  std::vector<float4> slots(c.n_slots);
  std::vector<uint32_t> step(I), flags(I), target(I), base(I);
  std::vector<unsigned long long> events((size_t)I * std::max(h->R, 1));
  const float4* cur = c.cur ? h->state1.p : h->state0.p;
  if (c.n_slots) BD_CUDA(cudaMemcpy(slots.data(), cur, slots.size() * sizeof(float4), cudaMemcpyDeviceToHost));
  BD_CUDA(cudaMemcpy(step.data(), h->inst_step.p, I * sizeof(uint32_t), cudaMemcpyDeviceToHost));
  BD_CUDA(cudaMemcpy(flags.data(), h->inst_flags.p, I * sizeof(uint32_t), cudaMemcpyDeviceToHost));
  BD_CUDA(cudaMemcpy(target.data(), h->inst_target.p, I * sizeof(uint32_t), cudaMemcpyDeviceToHost));
  BD_CUDA(cudaMemcpy(base.data(), h->inst_slot_base.p, I * sizeof(uint32_t), cudaMemcpyDeviceToHost));
  BD_CUDA(cudaMemcpy(events.data(), h->events.p, events.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
  const std::vector<uint8_t> fp = fingerprint(h);
  File out;
  out.f = fopen(path, "wb");
  if (!out.f) return BD_ERR_INVALID_ARGUMENT;
  const uint64_t head[5] = {(uint64_t)fp.size(), c.step, c.n_slots, c.deaths_last, (uint64_t)I};
  bool ok = fwrite(kCkptMagic, 8, 1, out.f) == 1 && fwrite(head, sizeof(head), 1, out.f) == 1 &&
            (fp.empty() || fwrite(fp.data(), fp.size(), 1, out.f) == 1);
  for (int k = 0; k < I && ok; k++) {
    const uint64_t planned = k < (int)h->plan_n.size() ? h->plan_n[k] : 0;
    const uint32_t v[4] = {step[k], flags[k], target[k], base[k]};
    ok = fwrite(&planned, sizeof(planned), 1, out.f) == 1 && fwrite(v, sizeof(v), 1, out.f) == 1;
  }
  ok = ok && fwrite(events.data(), sizeof(unsigned long long), events.size(), out.f) == events.size();
  ok = ok && (slots.empty() || fwrite(slots.data(), sizeof(float4), slots.size(), out.f) == slots.size());
  ok = (fclose(out.f) == 0) && ok;
  out.f = nullptr;
  return ok ? BD_OK : BD_ERR_INVALID_ARGUMENT;
}

BD_API bd_status bd_load_checkpoint(bd_handle h, const char* path) {
  const Range range("bd_load_checkpoint");
  if (!h || !path || h->server) return BD_ERR_INVALID_ARGUMENT;
  if (!h->finalized) return BD_ERR_NOT_FINALIZED;
  if (h->host_only) return BD_ERR_NO_DEVICE;
  File in;
  in.f = fopen(path, "rb");
  if (!in.f) return BD_ERR_INVALID_ARGUMENT;
  char magic[8];
  uint64_t head[5];
  if (fread(magic, 8, 1, in.f) != 1 || memcmp(magic, kCkptMagic, 8) != 0 || fread(head, sizeof(head), 1, in.f) != 1)
    return BD_ERR_INVALID_ARGUMENT;
  const std::vector<uint8_t> fp = fingerprint(h);
  const int I = h->n_inst();
  if (head[0] != fp.size() || head[4] != (uint64_t)I || head[2] > 0xFFFFFFF0ull) {
    g_last_error = "checkpoint of a differently built handle";
    return BD_ERR_INVALID_ARGUMENT;
  }
  std::vector<uint8_t> fp_file(fp.size());
  if ((!fp.empty() && fread(fp_file.data(), fp.size(), 1, in.f) != 1) || fp_file != fp) {
    g_last_error = "checkpoint of a differently built handle";
    return BD_ERR_INVALID_ARGUMENT;
  }
  const uint64_t n_slots = head[2];
  std::vector<uint64_t> planned(I);
  std::vector<uint32_t> step(I), flags(I), target(I), base(I);
  for (int k = 0; k < I; k++) {
    uint32_t v[4];
    if (fread(&planned[k], sizeof(uint64_t), 1, in.f) != 1 || fread(v, sizeof(v), 1, in.f) != 1)
      return BD_ERR_INVALID_ARGUMENT;
    step[k] = v[0], flags[k] = v[1], target[k] = v[2], base[k] = v[3];
  }
  std::vector<unsigned long long> events((size_t)I * std::max(h->R, 1));
  std::vector<float4> slots(n_slots);
  if (fread(events.data(), sizeof(unsigned long long), events.size(), in.f) != events.size() ||
      (n_slots && fread(slots.data(), sizeof(float4), n_slots, in.f) != n_slots))
    return BD_ERR_INVALID_ARGUMENT;
  BD_CUDA(cudaSetDevice(h->device));
  if (h->have_particles) {
    const bd_status st = bd_synchronize(h);
    if (st && st != BD_ERR_EMPTY) return st;
  }
  // the grids the original planned, then the buffers and the state
  h->hinst.assign(I, DevInstance{});
  for (int k = 0; k < I; k++) plan_instance(h, k, planned[k]);
  bd_status st = layout_cells(h);
  if (st) return st;
  uint64_t cap = h->cfg.capacity ? h->cfg.capacity : std::max<uint64_t>(2 * n_slots, 4096);
  cap = std::max<uint64_t>(cap, n_slots);
  h->have_particles = false;
  memset(h->hctrl, 0, sizeof(DevCtrl));
  if ((st = grow_particles(h, cap))) return st;
  const uint32_t pc = h->cfg.pair_capacity ? h->cfg.pair_capacity : (uint32_t)std::max<uint64_t>(65536, cap / 32);
  if ((st = grow_pairs(h, pc))) return st;
  if (n_slots)
    BD_CUDA(cudaMemcpyAsync(h->state0.p, slots.data(), n_slots * sizeof(float4), cudaMemcpyHostToDevice, h->stream));
  h->h_flags = flags;
  h->h_target = target;
  std::vector<uint32_t> zeros(I, 0);
  if ((st = upload(h->inst_step, step, h->stream)) || (st = upload(h->inst_slot_base, base, h->stream)) ||
      (st = upload(h->inst_flags, flags, h->stream)) || (st = upload(h->inst_target, target, h->stream)) ||
      (st = upload(h->inst_frozen, zeros, h->stream)) || (st = upload(h->events, events, h->stream)))
    return st;
  BD_CUDA(h->zero_off.alloc((size_t)I * h->Z + 1));
  BD_CUDA(cudaMemsetAsync(h->zero_off.p, 0, ((size_t)I * h->Z + 1) * sizeof(uint32_t), h->stream));
  BD_CUDA(h->pending.alloc((size_t)I * std::max(h->R, 1)));
  BD_CUDA(cudaMemsetAsync(h->pending.p, 0, h->pending.n * sizeof(unsigned long long), h->stream));
  memset(h->hctrl, 0, sizeof(DevCtrl));
  h->hctrl->n_slots = (uint32_t)n_slots;
  h->hctrl->step = head[1];
  h->hctrl->deaths_last = (uint32_t)head[3];
  if ((st = push_ctrl(h))) return st;
  BD_CUDA(cudaStreamSynchronize(h->stream));
  h->have_particles = true;
  h->target_step = head[1];
  return build_graphs(h);
}

BD_API bd_status bd_get_config(bd_handle h, bd_config* out) {
  if (!h || !out) return BD_ERR_INVALID_ARGUMENT;
  *out = h->cfg;
  return BD_OK;
}

BD_API bd_status bd_set_species_name(bd_handle h, int species, const char* name) {
  if (!h) return BD_ERR_INVALID_ARGUMENT;
  return set_name(&h->species_names, h->D.size(), species, name);
}
BD_API bd_status bd_find_species(bd_handle h, const char* name, int* species) {
  if (!h) return BD_ERR_INVALID_ARGUMENT;
  return find_name(h->species_names, name, species);
}
BD_API bd_status bd_set_reaction_name(bd_handle h, int rxn, const char* name) {
  if (!h) return BD_ERR_INVALID_ARGUMENT;
  return set_name(&h->reaction_names, h->rx.size(), rxn, name);
}
BD_API bd_status bd_find_reaction(bd_handle h, const char* name, int* rxn) {
  if (!h) return BD_ERR_INVALID_ARGUMENT;
  return find_name(h->reaction_names, name, rxn);
}

BD_API double bd_numrxnrate(double step, double a, double b) { return numrxnrate(step, a, b); }
BD_API double bd_actrxnrate(double step, double a) { return actrxnrate(step, a); }
BD_API double bd_bindingradius(double rate, double dt, double difc, double b, int rel) {
  return bindingradius(rate, dt, difc, b, rel);
}
BD_API double bd_unbindingradius(double pgem, double dt, double difc, double a) {
  return unbindingradius(pgem, dt, difc, a);
}
BD_API int bd_gauss_table(float* out, int n) {
  if (!out || n <= 0 || (n & 1)) return -1;
  gauss_quantiles(out, n);
  return n;
}

BD_API const char* bd_status_string(bd_status s) {
  switch (s) {
    case BD_OK: return "ok";
    case BD_ERR_NEGATIVE_RATE: return "negative reaction rate";
    case BD_ERR_STATE_DEPENDENT: return "state-dependent reaction probability";
    case BD_ERR_ZERO_DIFFUSION: return "diffusion coefficients sum to zero";
    case BD_ERR_ILLEGAL_UNBIND: return "illegal input for the unbinding radius";
    case BD_ERR_PGEM_UNATTAINABLE: return "geminate probability unattainable";
    case BD_ERR_INVALID_ARGUMENT: return "invalid argument";
    case BD_ERR_NOT_FINALIZED: return "not finalized / no particles";
    case BD_ERR_ALREADY_FINALIZED: return "already finalized";
    case BD_ERR_CAPACITY: return "capacity exceeded";
    case BD_ERR_EMPTY: return "no particles left";
    case BD_ERR_CUDA: return g_last_error.empty() ? "CUDA error" : g_last_error.c_str();
    case BD_ERR_TIMEOUT: return "device wait timed out";
    case BD_ERR_NO_DEVICE: return "no CUDA device";
    case BD_ERR_DEVICE_STATE: return "device state check failed";
    case BD_ERR_UNSUPPORTED: return "unsupported";
    default: return "unknown status";
  }
}

BD_API const char* bd_version(void) { return "gpusmoldyn-gb300 0.1 (sm_103a)"; }
