// hs_batch.h -- batched update and its autotuner (host side).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <tuple>
#include <vector>

#include "hairsim.h"
#include "hs_device.cuh"
#include "hs_internal.h"

namespace hs {

// One warp's worth of work: 32 consecutive strands of one groom.
struct BatchTile {
  uint32_t groom;
  uint32_t strand0;
};

// Device table entry, one per groom of the batch (a multiple of 16 bytes:
// warps stage it in shared memory ahead of their velocity columns).
struct BatchGroomDev {
  GroomView view;
  FrameConst fc;
};
static_assert(sizeof(BatchGroomDev) % 16 == 0, "table entries must keep float4 alignment");

// Tiles of one (capacity, mode) and how they are launched.
struct Bucket {
  int cap = 0;
  bool ref = false;
  uint32_t ntiles = 0;
  BatchTile* d_tiles = nullptr;
  int warps_per_block = 4;
  bool vsmem = false;  // velocity slots in shared memory (else registers)
  uint32_t grid = 1;
};

struct BatchState {
  std::vector<uint64_t> signature;  // groom pointers and (mode, npoints)
  uint32_t ngrooms = 0;
  std::vector<Bucket> buckets;
  BatchGroomDev* d_table = nullptr;
  BatchGroomDev* h_table[2] = {nullptr, nullptr};  // pinned staging, alternating
  cudaEvent_t done[2] = {nullptr, nullptr};
  cudaGraphExec_t exec[2] = {nullptr, nullptr};
  int next = 0;
  uint32_t* d_counters = nullptr;  // one tile counter per bucket
  std::vector<cudaStream_t> aux;   // one branch per bucket
  std::vector<cudaEvent_t> fork_join;
  ~BatchState();
  void release();
};

// Launch shape of a bucket, chosen by the autotuner.
struct TuneChoice {
  int warps_per_block = 4;
  int waves = 1;       // persistent grid = SMs x resident blocks per SM x waves
  bool vsmem = false;  // velocity slots in shared memory (else registers)
};

// Key: (capacity, reference mode, log2 of the bucket's tile count).
using TuneKey = std::tuple<int, bool, int>;

struct TuneCache {
  std::map<TuneKey, TuneChoice> best;
  std::map<TuneKey, float> best_ms;
};

TuneKey tune_key(int cap, bool ref, uint32_t ntiles);
TuneChoice tuned_choice(hs_ctx* ctx, int cap, bool ref, uint32_t ntiles);
int batch_occupancy(int cap, bool ref, bool vsmem, int warps_per_block);
hs_status batch_update(hs_ctx* ctx, hs_groom* const* grooms, uint32_t n, float dt, bool use_graph);

}  // namespace hs
