// bd_io.h -- kernels that move particles between the caller's arrays and
// the device state (bd_io.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace bd {

// An upload staged on the device: n particles (float4 x, y, z, w and int
// species), instance k owning [start[k], start[k + 1]), its box at
// boxes[6k .. 6k + 5] (lo x, y, z, hi x, y, z).
struct UploadArgs {
  const float4* xyz4;
  const int* species;
  const uint64_t* start;
  const float* boxes;
  uint64_t n;
  int n_inst, n_species;
  uint32_t* bad;  // set to 1 when a particle has a bad species or lies outside its box
  uint32_t inst_offset;  // instance index of start[0]'s instance in the records' w
};

// Checks (sets *bad) and packs the staged particles into records
// (w = instance << 16 | species), out[i] for particle i.
void enqueue_upload_check(const UploadArgs& a, cudaStream_t s);
void enqueue_upload_pack(const UploadArgs& a, float4* out, cudaStream_t s);

// The live records of state[0, n_slots) (of instance `inst`, or all when
// inst < 0), in slot order: positions as (x, y, z, 1) and species.
struct ExportArgs {
  const float4* state;
  uint64_t n_slots;
  int inst;
  uint32_t n_tiles;       // export_tiles(n_slots)
  uint32_t* tile_offset;  // [n_tiles] scratch
  uint32_t* count;        // receives the number exported
  float4* xyz4;           // [n_slots] out
  int* species;           // [n_slots] out
};
uint32_t export_tiles(uint64_t n_slots);
void enqueue_export(const ExportArgs& a, cudaStream_t s);

}  // namespace bd
