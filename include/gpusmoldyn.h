/*
 * gpusmoldyn.h -- C ABI of the GB300 Brownian-dynamics step (libgpusmoldyn.so).
 *
 * One handle owns one simulation (or a batched ensemble of independent
 * instances) resident on one GPU: species with per-species diffusion
 * coefficients, zeroth-, first- and second-order reactions whose probabilities
 * and binding / unbinding radii are derived with the Andrews-Bray rxnparam
 * method, reflecting walls in a rectangular box, and a per-timestep pipeline
 * of hand-written sm_103a kernels.  All entry points take plain pointers and
 * sizes and return a bd_status (0 = success); none aborts the process.
 *
 * This ABI replaces the reference's extern "C" CUDA layer
 * (particleSystem.cuh:29-110) and the device-facing part of its
 * ParticleSystem class (particleSystem.h:50-218); each declaration below
 * names the reference function(s) it stands in for.  Handles are independent:
 * there is no file-scope device state (the reference keeps SimParams, the
 * Gaussian table and textures in file-static device symbols,
 * particles_kernel.cu:42-57), so several handles may live in one process.
 */
#ifndef GPUSMOLDYN_H
#define GPUSMOLDYN_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
#define BD_EXTERN extern "C"
#else
#define BD_EXTERN
#endif
#define BD_API BD_EXTERN __attribute__((visibility("default")))

/* ------------------------------------------------------------------ status */
/* The setup codes 1, 2, 4, 7 and 8 keep the numbers the reference's
 * rxnsetrate / rxnsetproduct return (smolreact.cpp:274-282, 455-469). */
typedef int bd_status;
enum {
  BD_OK = 0,
  BD_ERR_NEGATIVE_RATE = 1,        /* rate < 0 (rxnsetrate return 1) */
  BD_ERR_STATE_DEPENDENT = 2,      /* reserved: per-state probabilities (return 2) */
  BD_ERR_ZERO_DIFFUSION = 4,       /* both reactants (or products) have D = 0 */
  BD_ERR_ILLEGAL_UNBIND = 7,       /* unbinding radius from illegal input (er = 7) */
  BD_ERR_PGEM_UNATTAINABLE = 8,    /* requested geminate probability too high (er = 8) */
  BD_ERR_INVALID_ARGUMENT = 16,
  BD_ERR_NOT_FINALIZED = 17,       /* step/particles before bd_finalize */
  BD_ERR_ALREADY_FINALIZED = 18,   /* species/reactions after bd_finalize */
  BD_ERR_CAPACITY = 19,            /* particle or pair capacity exceeded, no room to grow */
  BD_ERR_EMPTY = 20,               /* no particles left: reference update() returns false */
  BD_ERR_CUDA = 21,                /* a CUDA runtime call failed */
  BD_ERR_TIMEOUT = 22,             /* a bounded device-side wait ran out */
  BD_ERR_NO_DEVICE = 23,
  BD_ERR_DEVICE_STATE = 24,        /* device reported an inconsistent state (bounds check) */
  BD_ERR_UNSUPPORTED = 25
};

/* ------------------------------------------------------------------ types */
typedef struct bd_system *bd_handle;

enum { BD_NORMALS_BOXMULLER = 0, BD_NORMALS_TABLE = 1 };

/* bd_config.device value for a host-only handle: set-up, parameter
 * derivation, grid planning and the getters work without a GPU; stepping
 * returns BD_ERR_NO_DEVICE. */
#define BD_DEVICE_NONE (-1)

/* Product-placement kinds for reactions with two products (Smoldyn's rparam
 * types; the reference hard-codes pgem = 0.2, smolreact.cpp:373-376). */
enum {
  BD_PP_DEFAULT = 0,     /* irreversible: products at the reaction point;
                            reversible pair: PGEMMAX 0.2 (Smoldyn's default) */
  BD_PP_PGEM = 1,        /* param = geminate probability; error 8 if unattainable */
  BD_PP_PGEMMAX = 2,     /* param = max geminate probability; b = 0 if the
                            attainable maximum is below it */
  BD_PP_UNBINDRAD = 3,   /* param = unbinding radius b (length) */
  BD_PP_OFFSET0 = 4      /* products exactly at the reaction point (b = 0) */
};

/* bd_config.sort_mode.  Both modes give identical results (records in
 * canonical cell order, same pairs); they differ in memory and speed.
 * BINNED writes each advanced record straight into a fixed-size bin of its
 * cell (bins sized from the planned occupancy, grown and the step replayed
 * when one overflows) and needs n_cells x bin size x 16 bytes.  COMPACT
 * counts, scans and scatters into exact cell ranges (the reference's
 * calcHash + RadixSort + reorderDataAndFindCellStart in one counting sort)
 * and needs 16 bytes per slot.  AUTO takes BINNED while its bins fit in
 * 32 GiB. */
enum { BD_SORT_AUTO = 0, BD_SORT_COMPACT = 1, BD_SORT_BINNED = 2 };

/* bd_config.pair_mode.  LAST: the last second-order reaction listed for a
 * reactant pair is the pair's only reaction, as in the reference
 * (particleSystem.cpp:656-669).  CHANNELS: all of them compete: the pair's
 * binding radius comes from their summed rate (irreversible calibration,
 * b = 0) and an accepted pair fires reaction i with probability
 * rate_i / sum (bd_reaction_info.channel_threshold holds the cumulative
 * shares).  A reaction probability on a competing reaction is
 * BD_ERR_UNSUPPORTED. */
enum { BD_PAIR_LAST = 0, BD_PAIR_CHANNELS = 1 };

typedef struct bd_config {
  float box_lo[3];           /* reflecting box, replaces the fixed [-1,1]^3 world */
  float box_hi[3];           /* (particleSystem.cpp:73, particleSystem.h:114-120) */
  float dt;                  /* time step (particleSystem.h:147 deltaTime) */
  uint64_t seed;             /* Philox key; replaces srand(time(0)) MT seeding */
  uint64_t capacity;         /* particle slots; 0 = 2x the first particle upload */
  float cell_size;           /* uniform-grid cell edge; 0 = automatic */
  float cell_occupancy;      /* target particles per cell for automatic sizing (0 = 3) */
  int normal_mode;           /* BD_NORMALS_* */
  int device;                /* CUDA device ordinal */
  uint32_t pair_capacity;    /* candidate-pair list length; 0 = automatic */
  uint32_t sort_mode;        /* BD_SORT_*: how records reach their cells */
  uint32_t pair_mode;        /* BD_PAIR_*: several second-order reactions of one pair */
  uint32_t reserved[5];
} bd_config;

/* Derived parameters of one reaction, as the reference stores them in its
 * struct-of-arrays Reaction (reaction.h:36-48). */
typedef struct bd_reaction_info {
  int order, nprod;
  int reactants[2], products[2];
  float rate;                 /* as given */
  float prob;                 /* per-step probability (order 0: Poisson mean) */
  float bind_radius;          /* order 2: a */
  float unbind_radius;        /* b for the products of this reaction (0 if none) */
  float geminate_prob;        /* the pgem actually achieved (order 1 reverse) */
  float product_offsets[2];   /* signed displacement of each product along a
                                 random unit vector (rxnsetproduct x offsets) */
  int reverse;                /* index of the reverse reaction, -1 if none */
  int flags;                  /* bit 0: pgem fell back to b = 0 */
  float channel_threshold;    /* BD_PAIR_CHANNELS: cumulative share of the pair's rate (1 = last) */
} bd_reaction_info;

/* ----------------------------------------------------- lifetime & set-up */

/* Fill a config with defaults (unit box, dt = 1e-3, seed 1). */
BD_API void bd_config_default(bd_config *cfg);

/* Create a simulation on cfg->device.  Replaces ParticleSystem::ParticleSystem
 * + _initialize (particleSystem.cpp:49-88, 573-751), cudaInit
 * (particleSystemCuda.cu:46-54) and initializeMT (:139-145). */
BD_API bd_status bd_create(const bd_config *cfg, bd_handle *out);

/* Free every host and device allocation.  Replaces ~ParticleSystem /
 * _finalize (particleSystem.cpp:90-94, 753-826) and freeArray (:72-75). */
BD_API bd_status bd_destroy(bd_handle h);

/* Add a species with diffusion coefficient D; *id receives its index.
 * Replaces the hard-coded test*Types presets (particleSystem.cpp:381-571)
 * and molSetTimestep (:137-142). */
BD_API bd_status bd_add_species(bd_handle h, float D, int *id);

/* Add a reaction of order 0, 1 or 2; unused reactant/product slots are -1.
 * Replaces the test*Reactions presets (particleSystem.cpp:319-542). */
BD_API bd_status bd_add_reaction(bd_handle h, int order, const int reactants[2],
                                 const int products[2], float rate, int *id);

/* Per-encounter probability of a second-order reaction (Smoldyn's reaction
 * probability; the reference keeps Reaction::prob = 1, smolreact.cpp:382-383,
 * and draws a coin only when it is below 1, particles_kernel.cu:395-396). */
BD_API bd_status bd_set_reaction_probability(bd_handle h, int rxn, float prob);

/* Choose how the two products of reaction rxn are placed (BD_PP_*). */
BD_API bd_status bd_set_product_placement(bd_handle h, int rxn, int kind, float param);

/* Derive probabilities, binding and unbinding radii and product offsets and
 * upload the reaction tables.  Replaces fillReactionOrderInfo, rxnsetrate,
 * rxnsetproduct (smolreact.cpp:173-483), the reaction-table fill and upload
 * (particleSystem.cpp:635-700), createGaussTable + copyGaussianToConstant
 * (stats.cpp:277-282, particleSystemCuda.cu:134-137) and setParameters
 * (:121-125).  Returns the first setup error code; a pgem fallback to b = 0
 * is not an error (see bd_reaction_info.flags). */
BD_API bd_status bd_finalize(bd_handle h);

BD_API bd_status bd_get_reaction_info(bd_handle h, int rxn, bd_reaction_info *out);
BD_API bd_status bd_get_counts(bd_handle h, int *n_species, int *n_reactions);

/* ------------------------------------------------------------ particles */

/* Upload n particles from host memory: xyz4 holds x,y,z,(ignored) per
 * particle, species[i] the species id.  Replaces reset / setArray
 * (particleSystem.cpp:1057-1161, which never upload in headless mode) and
 * copyArrayToDevice (particleSystemCuda.cu:93-96). */
BD_API bd_status bd_set_particles(bd_handle h, const float *xyz4, const int *species, size_t n);

/* Live particle count (synchronises).  Replaces getNumParticles
 * (particleSystem.h:86) and the per-step count readbacks of
 * compactPosAndType (particleSystemCuda.cu:298-306). */
BD_API bd_status bd_get_count(bd_handle h, uint64_t *n);

/* Copy live particles to host memory (synchronises): up to cap particles,
 * *n receives the live count.  Replaces getArray / copyArrayFromDevice
 * (particleSystem.cpp:1031-1055, particleSystemCuda.cu:82-91). */
BD_API bd_status bd_get_particles(bd_handle h, float *xyz4, int *species, size_t cap, size_t *n);

/* Device address of the current record array (float4 x, y, z, w where w's
 * bits hold species | instance << 16, 0xFFFFFFFF = empty slot) and its slot
 * count, after synchronising; valid until the next bd_step.  Replaces
 * getCudaPosVBO / getCudaTypesVBO (particleSystem.h:94-95). */
BD_API bd_status bd_get_state_pointer(bd_handle h, void **dev_records, uint64_t *n_slots);

/* ----------------------------------------------------------------- step */

/* Enqueue nsteps timesteps on the handle's stream without host
 * synchronisation.  Replaces ParticleSystem::update (particleSystem.cpp:
 * 829-1001) and through it integrateSystem, adjustPositions, calcHash,
 * RadixSort::sort, reorderDataAndFindCellStart, collide and
 * compactPosAndType (particleSystemCuda.cu:148-367) and zeroReact
 * (reaction_cpu.cpp:36-63). */
BD_API bd_status bd_step(bd_handle h, int nsteps);
/* bd_step ordered on a caller's stream (a cudaStream_t; NULL = legacy
 * default): the steps start after the work already enqueued on `stream`,
 * and work enqueued on `stream` afterwards starts after the steps.  For a
 * caller that produces or consumes the device records
 * (bd_get_state_pointer) on its own stream.  A step that must grow a buffer
 * and be replayed completes only at the next bd_synchronize. */
BD_API bd_status bd_step_async(bd_handle h, int nsteps, void *stream);

/* Wait for enqueued steps; if a step ran out of particle or pair capacity
 * the buffers grow and the remaining steps are replayed, so the state after
 * return is the state after every requested step.  Returns BD_ERR_EMPTY when
 * no particle is left (update() returning false, particleSystem.cpp:892,963).
 * Replaces threadSync (particleSystemCuda.cu:77-80). */
BD_API bd_status bd_synchronize(bd_handle h);

/* Completed steps. */
BD_API bd_status bd_get_step(bd_handle h, uint64_t *step);

/* Cumulative event count per reaction (n entries). */
BD_API bd_status bd_get_event_counts(bd_handle h, uint64_t *counts, int n);

/* Run nsteps timesteps (as bd_step) bracketed by CUDA events recorded on the
 * handle's stream; *ms receives the device time between them.  Synchronises.
 * The reference times update() with a host timer around
 * cudaThreadSynchronize (particles.cpp:213-226). */
BD_API bd_status bd_time_steps(bd_handle h, int nsteps, float *ms);

/* Run nsteps timesteps launching the kernels one by one with a CUDA event
 * between consecutive kernels; stage_ms[k] receives the summed device time
 * of kernel k of the step (n_stages of them, at most cap).  Diagnostics for
 * the per-kernel roofline; the production path launches graphs. */
BD_API bd_status bd_profile_steps(bd_handle h, int nsteps, float *stage_ms, int cap, int *n_stages);
/* Name of kernel k of the step, as profiled by bd_profile_steps. */
BD_API const char *bd_stage_name(bd_handle h, int k);

/* Kernel launches in one timestep of the current configuration. */
BD_API bd_status bd_get_kernels_per_step(bd_handle h, int *n);

/* --------------------------------------------------- parity / inspection */

/* Raw slot array of the current state, holes included (w = 0xFFFFFFFF). */
BD_API bd_status bd_debug_get_slots(bd_handle h, float *xyz4, uint32_t *w, size_t cap, size_t *n);
/* Cell start offsets of the last sorted step (ncells + 1 entries). */
BD_API bd_status bd_debug_get_cells(bd_handle h, uint32_t *start, size_t cap, size_t *ncells);
/* Test switch for the bounded waits of the cell scan's grid barrier: with
 * on, CTA 0 of the scan never arrives at the barrier, so the other CTAs'
 * waits run out (after about a second) and the step reports BD_ERR_TIMEOUT
 * instead of hanging.  No fault, trap or endless loop. */
BD_API bd_status bd_debug_withhold_scan(bd_handle h, int on);
/* Test switch for the bounded waits of the matcher's grid barrier (steps
 * with more than 8,192 candidate pairs): with on, CTA 0 of the matcher
 * never arrives at its first barrier, so the other CTAs' waits run out
 * (after about a second) and the step reports BD_ERR_TIMEOUT. */
BD_API bd_status bd_debug_withhold_match(bd_handle h, int on);
/* Candidate pairs (slot_i, slot_j, reaction, accepted) of the last step. */
BD_API bd_status bd_debug_get_pairs(bd_handle h, uint32_t *quads, size_t cap, size_t *n);
/* Uniform-grid geometry of one instance: cells per axis, cell edge lengths
 * and cells per unit length (the float factors the cell key is computed
 * with).  Replaces getGridSize / getCellSize / getWorldOrigin
 * (particleSystem.h:110-112). */
BD_API bd_status bd_get_grid(bd_handle h, int instance, uint32_t dims[3], float cell[3], float inv[3]);
/* Poisson CDF of zeroth-order reaction rxn for one instance: P(X <= kmin+k)
 * for k < *len (copies up to cap entries). */
BD_API bd_status bd_get_poisson_cdf(bd_handle h, int instance, int rxn, double *cdf, size_t cap, int *kmin,
                                    size_t *len);
/* Diffusion coefficient of a species after the instance's scaling. */
BD_API bd_status bd_get_species_d(bd_handle h, int instance, int species, float *D);
/* Cell edge override before the first step (autotuner). */
BD_API bd_status bd_set_cell_size(bd_handle h, float cell_size);
/* Launch shape of the particle kernels (autotuner): threads per CTA (a
 * multiple of 32, at most 256) and CTAs per SM of the grid-stride grids, for
 * the streaming kernels and for the pair kernel (whose CTA is always 256
 * threads, one per cell of a tile: block_pairs must be 256).  A streaming grid of
 * exactly 48 or 32 warps per SM runs register-capped kernel variants (40 or
 * 64 registers) so that all of it is resident.  The result of a step does
 * not depend on it. */
BD_API bd_status bd_set_launch_shape(bd_handle h, int block_stream, int ctas_per_sm_stream, int block_pairs,
                                     int ctas_per_sm_pairs);

/* ------------------------------------------------------------- ensemble */

/* Per-instance description for a batched ensemble: every instance shares the
 * species and reaction network of the handle but has its own box, seed,
 * particles and parameter scaling (D x d_scale, second-order rates x
 * k2_scale).  The reference runs one system per process; this is new. */
typedef struct bd_instance_desc {
  float box_lo[3], box_hi[3];
  uint64_t seed;
  float d_scale, k2_scale;
  float cell_size;           /* 0 = automatic */
  uint32_t reserved[3];
} bd_instance_desc;

/* Create an ensemble handle of n instances (species/reactions then added as
 * for a single system). */
BD_API bd_status bd_create_ensemble(const bd_config *cfg, const bd_instance_desc *inst,
                                    int n_instances, bd_handle *out);
/* Upload the particles of all instances: counts[k] particles of instance k,
 * concatenated in instance order. */
BD_API bd_status bd_set_ensemble_particles(bd_handle h, const float *xyz4, const int *species,
                                           const uint64_t *counts, int n_instances);
/* Live particles per species (synchronises): counts[s] for s < n, summed
 * over instances (instance = -1) or for one instance.  Replaces reading
 * the whole type array back (particles.cpp:509-552 debug dumps). */
BD_API bd_status bd_get_species_counts(bd_handle h, int instance, uint64_t *counts, int n);
/* Mean squared displacement per species over the next nsteps steps, which
 * are taken as bd_step takes them (synchronises).  msd[s] is the mean,
 * over the moves of species s's particles (of one instance, or of all for
 * instance = -1), of |x' - x|^2 with x' the position after the step's
 * diffusion move and the wall reflections, before the step's reactions;
 * counts[s] is the number of moves averaged.  In the bulk it equals
 * 6 D dt.  The moves are recomputed from each step's own random counters
 * by a read-only kernel launched before the step.  Handles with surface
 * panels return BD_ERR_UNSUPPORTED.  Replaces watching the particles move
 * in the viewer (particles.cpp:254-275, render_particles.cpp). */
BD_API bd_status bd_measure_msd(bd_handle h, int instance, int nsteps, double *msd, uint64_t *counts, int n);

/* Live counts per instance (synchronises). */
BD_API bd_status bd_get_instance_counts(bd_handle h, uint64_t *counts, int n_instances);
/* Copy the live particles of one instance (synchronises). */
BD_API bd_status bd_get_instance_particles(bd_handle h, int instance, float *xyz4, int *species,
                                           size_t cap, size_t *n);
/* Derived parameters of reaction rxn for one instance. */
BD_API bd_status bd_get_instance_reaction_info(bd_handle h, int instance, int rxn,
                                               bd_reaction_info *out);

/* -------------------------------------------------------------- serving */
/* A serving handle: an ensemble of max_instances slots that are filled and
 * emptied while it runs (continuous batching).  Species and reactions are
 * added and finalized as usual; then bd_instance_admit adds a simulation,
 * bd_step advances every admitted instance together, an instance freezes on
 * the device when it reaches its step count, bd_instance_poll lists frozen
 * instances and bd_instance_harvest copies one out (in canonical order: by
 * cell, then by record bits) and frees its slot.  An instance evolves
 * exactly as it would alone.  The reference runs one system per process and
 * has no counterpart. */
BD_API bd_status bd_create_server(const bd_config *cfg, int max_instances, bd_handle *out);
BD_API bd_status bd_instance_admit(bd_handle h, const bd_instance_desc *d, const float *xyz4, const int *species,
                                   size_t n, uint32_t steps, int *slot);
BD_API bd_status bd_instance_poll(bd_handle h, int *slots, int cap, int *n_finished);
BD_API bd_status bd_instance_harvest(bd_handle h, int slot, float *xyz4, int *species, size_t cap, size_t *n);
/* Drops an admitted instance, frozen or still running (a cancelled
 * request): it takes no further step, its records are gone after the next
 * step, and its slot is free for bd_instance_admit from then on.  The other
 * instances are not affected. */
BD_API bd_status bd_instance_cancel(bd_handle h, int slot);
/* Steps taken by the instance in a slot and its flags (1 active, 2 frozen). */
BD_API bd_status bd_instance_state(bd_handle h, int slot, uint32_t *steps, uint32_t *flags);

/* ------------------------------------------------- allocation-free sort */
/* No counterpart in the reference.  For callers that cannot call cudaMalloc
 * -- a host application that owns all device memory and forbids its
 * plugins to grow the footprint, or a time-critical loop that cannot afford
 * cudaMalloc's implicit device synchronisation -- this sorts n records
 * (device float4 x, y, z, w) into the uniform grid of `dims` cells over the
 * box, exactly as a step orders its state: by cell, then by record bits
 * inside a cell.  d_out receives the n sorted records and d_cell_start the
 * n_cells + 1 cell starts; both are the caller's device buffers, and the
 * call is enqueued on `stream` (a cudaStream_t; NULL = legacy default).
 * Nothing is allocated: the per-cell counts, scan partials and two control
 * words live in one file-scope device array of 2^20 + 258 words (about
 * 4 MiB) that every GPU loading the library keeps until the process exits.
 * More than 2^20 cells (or any single dims[a] above 2^20) or more than
 * 2^31 - 1 records returns BD_ERR_CAPACITY before anything is enqueued.
 * d_in, d_out and d_cell_start must be disjoint (an overlap returns
 * BD_ERR_INVALID_ARGUMENT): the kernels read the input while they write the
 * outputs.  Ordering inside a cell is bounded work: a cell of up to 32
 * records costs one thread at most 496 comparisons, a larger cell is sorted
 * by one thread block with a bitonic network, O(m log^2 m) for m records.
 * The first call on a device (and the first after a device reset, which
 * reloads the module) looks up that array's device address
 * (cudaGetSymbolAddress), so make the first call before any stream capture.
 * Calls share the array and each clears its counts first; calls that
 * overlap on the GPU race on it and must be serialised. */
BD_API bd_status bd_cell_sort_static(const float *d_in, uint64_t n, const float box_lo[3], const float box_hi[3],
                                     const uint32_t dims[3], float *d_out, uint32_t *d_cell_start, void *stream);

/* ------------------------------------------------------------ surfaces */
/* Surfaces made of panels that reflect, absorb or transmit molecules, per
 * species and per face (Smoldyn's surfaces).  The reference only drafts
 * them: panel geometry and the crossing test in surfaces_kernel.cuh:97-248,
 * a per-cell panel walk in checkSurfaceCollisions (particles_kernel.cu:
 * 414-440) that is never launched and does not compile.  Here every step
 * tests the segment from a molecule's old position to its diffused one
 * against the panels (found through a coarse grid of panel lists), takes
 * the first crossing along it and applies the surface's action for the
 * molecule's species on the face it arrives from: ABSORB removes it,
 * TRANSMIT lets it through, REFLECT mirrors the rest of the step in the
 * panel's tangent plane at the crossing point; the walk continues with what
 * is left of the segment (at most 8 crossings a step, after which the
 * molecule stays at its last crossing point).  The box walls reflect after
 * the surfaces.  The segments from a reaction point to its displaced
 * products are tested the same way.  Pairs react whatever panel lies
 * between them, and zeroth-order births are uniform in the box.  A panel
 * whose surface transmits a species on both faces (the default action) is
 * invisible to that species.  Surfaces and panels are added before
 * bd_finalize; panels are shared by all instances of an ensemble, in each
 * instance's coordinates. */
enum {
  BD_PANEL_RECT = 0,  /* axis-aligned rectangle */
  BD_PANEL_TRI = 1,   /* triangle */
  BD_PANEL_SPH = 2,   /* sphere */
  BD_PANEL_CYL = 3,   /* open cylinder (no end caps) */
  BD_PANEL_HEMI = 4,  /* hemisphere */
  BD_PANEL_DISK = 5   /* flat disk */
};
enum { BD_FACE_FRONT = 0, BD_FACE_BACK = 1, BD_FACE_BOTH = 2 };
enum { BD_SURF_TRANSMIT = 0, BD_SURF_REFLECT = 1, BD_SURF_ABSORB = 2 };
#define BD_ALL_SPECIES (-1)

/* One panel as given.  p[] by shape:
 *   RECT  corner x, y, z; side along the lower-numbered other axis; side along
 *         the higher-numbered one (sides may be negative).  axis = the axis the
 *         rectangle is perpendicular to; front = +1: the front face looks
 *         toward +axis, -1 toward -axis.
 *   TRI   vertices v0, v1, v2; the front face is the one (v1-v0) x (v2-v0)
 *         points to.
 *   SPH   centre, radius.  front = +1: the front face is outside, -1 inside.
 *   CYL   axis end 0, axis end 1, radius; front as SPH.
 *   HEMI  centre, radius, opening direction (the shell is the half of the
 *         sphere away from it); front as SPH.
 *   DISK  centre, radius, normal (the front face is the one it points to).
 * Points exactly on a panel belong to its back face. */
typedef struct bd_panel {
  int shape;
  int axis;
  int front;
  float p[10];
} bd_panel;

/* The geometry a step uses for one panel, derived from bd_panel in float
 * (unit normals, squared radius, rectangle bounds). */
typedef struct bd_panel_info {
  int shape, surface, axis;
  float front;                /* +1 / -1 (RECT, SPH, CYL, HEMI) */
  float a[3];                 /* RECT corner, TRI v0, SPH/HEMI/DISK centre, CYL end 0 */
  float r, r2;                /* radius and its square */
  float n[3];                 /* TRI, DISK unit front normal; CYL unit axis; HEMI unit opening direction */
  float len;                  /* CYL axis length */
  float v1[3], v2[3];         /* TRI vertices 1 and 2 */
  float bounds[4];            /* RECT: lower axis lo, hi; higher axis lo, hi */
} bd_panel_info;

BD_API bd_status bd_add_surface(bd_handle h, int *surface);
/* species = BD_ALL_SPECIES for every species defined so far; face one of
 * BD_FACE_*; action one of BD_SURF_*.  The default is TRANSMIT. */
BD_API bd_status bd_set_surface_action(bd_handle h, int surface, int species, int face, int action);
BD_API bd_status bd_get_surface_action(bd_handle h, int surface, int species, int face, int *action);
BD_API bd_status bd_add_panel(bd_handle h, int surface, const bd_panel *panel, int *id);
BD_API bd_status bd_get_panel(bd_handle h, int id, bd_panel_info *out);
BD_API bd_status bd_get_surface_counts(bd_handle h, int *n_surfaces, int *n_panels);

/* ----------------------------------------------------------- snapshots */
/* The molecules written to a file (no display: replaces the reference's
 * OpenGL viewer, render_particles.cpp / particles.cpp).  TEXT: "# step s
 * molecules n species S", "# counts c0 c1 ...", then "x y z species" per
 * molecule with 9 significant digits (exact for float).  BINARY: uint64
 * step, uint64 n, then n records of float x, y, z and int32 species. */
enum { BD_SNAPSHOT_TEXT = 0, BD_SNAPSHOT_BINARY = 1 };
BD_API bd_status bd_write_snapshot(bd_handle h, const char *path, int format);

/* ---------------------------------------------------------- checkpoints */
/* The whole dynamic state of a handle, to stop a run and resume it: every
 * slot in slot order (empty ones too), the step counters of the handle and
 * of each instance, the event counters, and the particle counts each
 * instance's grid was planned for.  A handle built the same way (network,
 * configuration and instances; checked against a fingerprint stored in the
 * file) and loaded from it continues bit for bit as the original would
 * have.  The reference has no checkpoint (its debug dumps, particleSystem.
 * cpp:1003-1030, cannot be read back).  Not for serving handles. */
BD_API bd_status bd_save_checkpoint(bd_handle h, const char *path);
BD_API bd_status bd_load_checkpoint(bd_handle h, const char *path);

/* The configuration a handle was created with (box, dt, seed, ...). */
BD_API bd_status bd_get_config(bd_handle h, bd_config *out);

/* ------------------------------------------------------------- names */
/* Optional names of species and reactions (the model reader sets them). */
BD_API bd_status bd_set_species_name(bd_handle h, int species, const char *name);
BD_API bd_status bd_find_species(bd_handle h, const char *name, int *species);
BD_API bd_status bd_set_reaction_name(bd_handle h, int rxn, const char *name);
BD_API bd_status bd_find_reaction(bd_handle h, const char *name, int *rxn);

/* ------------------------------------------------------- model reader */
/* What a model text declared besides the network (all zero when absent). */
typedef struct bd_model_info {
  double time_start, time_stop;
  uint64_t steps;             /* (time_stop - time_start) / time_step, rounded */
  uint64_t n_molecules;       /* placed by mol statements */
  int n_species, n_reactions;
} bd_model_info;

/* A finalized handle with its molecules placed, from a model in a subset of
 * Smoldyn's configuration language: dim 3, boundaries / low_wall /
 * high_wall (reflecting), species, difc, time_start / time_stop /
 * time_step, random_seed, reaction, reaction_rate, reaction_probability,
 * product_placement (irrev, pgem, pgemmax, unbindrad), mol (coordinates or
 * u for uniform, from a splitmix64 stream seeded by random_seed),
 * end_file; display and output statements are ignored.  Replaces the
 * reference's hard-coded presets ParticleSystem::test1Reactions ..
 * test3Types (particleSystem.cpp:319-571), whose comments quote these
 * statements.  device may be BD_DEVICE_NONE.  On failure err (if given)
 * receives "line N: reason". */
BD_API bd_status bd_create_from_model(const char *text, int device, bd_handle *out, bd_model_info *info, char *err,
                                      size_t err_cap);
BD_API bd_status bd_create_from_model_file(const char *path, int device, bd_handle *out, bd_model_info *info,
                                           char *err, size_t err_cap);

/* ------------------------------------------------------ rxnparam (host) */
/* Restatements of rxnparam.h:39-42 (Andrews-Bray rate tables, rxnparam.cpp:
 * 42-308): rate per step in length^3, binding radius, unbinding radius. */
BD_API double bd_numrxnrate(double step, double a, double b);
BD_API double bd_actrxnrate(double step, double a);
BD_API double bd_bindingradius(double rate, double dt, double difc, double b, int rel);
BD_API double bd_unbindingradius(double pgem, double dt, double difc, double a);
/* The 4096-entry table of standard-normal quantiles used in BD_NORMALS_TABLE
 * mode (replaces createGaussTable, stats.cpp:202-232, 277-282). */
BD_API int bd_gauss_table(float *out, int n);

BD_API const char *bd_status_string(bd_status s);
BD_API const char *bd_version(void);

#endif /* GPUSMOLDYN_H */
