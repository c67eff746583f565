/*
 * oracle.h -- TEST INFRASTRUCTURE, not part of the product.
 *
 * A CPU restatement of one timestep of the Smoldyn Brownian-dynamics loop
 * (ParticleSystem::update, particleSystem.cpp:829-1001) with the semantics
 * the GPU library implements, written independently of the library's
 * kernels.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg load it, to check the GPU path or to time the CPU.  Parameters (species
 * step lengths, reaction probabilities, radii, offsets, grid, Poisson CDFs,
 * the normal table) are inputs: the library's host derivation of them is
 * pinned separately against the reference's own compiled setup code.
 */
#ifndef BD_ORACLE_H
#define BD_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One surface panel with its derived geometry, word for word the library's
 * bd_panel_info (shape 0 rect, 1 tri, 2 sphere, 3 cylinder, 4 hemisphere,
 * 5 disk). */
typedef struct or_panel {
  int shape, surface, axis;
  float front;
  float a[3];
  float r, r2;
  float n[3];
  float len;
  float v1[3], v2[3];
  float bounds[4];
} or_panel;

typedef struct or_system {
  float lo[3], hi[3], inv[3];
  float cell[3];
  uint32_t dims[3];
  uint32_t key_lo, key_hi;
  int normal_mode;          /* 0 Box-Muller, 1 table */
  const float *gauss;       /* 4096 quantiles */
  int S;
  const float *D;           /* per species (already scaled) */
  float dt;
  int R;                    /* reactions */
  const int *order, *react0, *react1, *prod0, *prod1;
  const float *prob, *bind_radius, *off0, *off1;
  const double *cdf;        /* concatenated Poisson CDFs of order-0 reactions */
  const int *cdf_off, *cdf_len, *cdf_kmin; /* per reaction (order 0 only) */
  int sorted;               /* 1: cell-sorted pipeline, 0: in-place diffusion */
  uint32_t inst;            /* instance id written into w */
  int threads;              /* OpenMP threads, 0 = default */
  int channels;             /* 1: second-order reactions of one pair compete */
  const float *thresh;      /* per reaction: cumulative share of its pair's rate */
  int n_panels;             /* surface panels (0 = none) */
  const or_panel *panels;
  const uint8_t *surf_act;  /* [surface][species][front, back]: 0 transmit, 1 reflect, 2 absorb */
} or_system;

/* One step.  in/out hold n records of 4 words (x, y, z as float bits, w).
 * cells (optional) receives ncells + 1 starts, pairs (optional) 4 words per
 * candidate pair (i, j, reaction, accepted).  events (optional) accumulates
 * per-reaction counts.  Returns 0 or a negative error. */
int or_step(const or_system *sys, uint32_t step, const uint32_t *in, uint32_t n, uint32_t *out, uint32_t cap,
            uint32_t *n_out, uint32_t *cells, uint64_t cells_cap, uint32_t *pairs, uint32_t pairs_cap,
            uint32_t *n_pairs, uint64_t *events);

/* Philox4x32-10 of one counter (known-answer checks). */
void or_philox(const uint32_t ctr[4], uint32_t k0, uint32_t k1, uint32_t out[4]);

#ifdef __cplusplus
}
#endif
#endif
