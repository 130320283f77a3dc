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

// Kernel variants of a bucket (the autotuner's mapping choice):
// positions and velocities in registers, or positions in registers and
// velocities in shared memory (up to 8 points); the streaming form (all in
// shared memory, runtime loops, any point count); the streaming form with
// the velocities in tensor memory; a lane group per strand (hs_lanes.cuh:
// warps per block = lanes per strand; DFTL buckets whose grooms all have
// one iteration and at most that many substeps). Values 3-5 are not built.
constexpr int kVariantRegs = 0;
constexpr int kVariantRegsVsmem = 1;
constexpr int kVariantStream = 2;
constexpr int kVariantStreamTmem = 6;  // 4 or 8 warps per block
constexpr int kVariantLanes = 7;       // 2, 4, 8 or 16 warps (lanes per strand) per block
constexpr int kVariants = 8;
inline bool is_stream(int variant) { return variant == kVariantStream; }
inline bool is_tmem(int variant) { return variant == kVariantStreamTmem; }
inline bool is_lanes(int variant) { return variant == kVariantLanes; }
// Variants with a runtime point loop (any capacity up to 64 points).
inline bool any_capacity(int variant) { return is_stream(variant) || is_tmem(variant) || is_lanes(variant); }

// Step classes: reference mode, DFTL under the EXACT contract, DFTL under
// the FAST contract (hs_contract); each runs kernels of its own.
constexpr int kClassRef = 0;
constexpr int kClassExact = 1;
constexpr int kClassFast = 2;
constexpr int kClasses = 3;
inline int step_class(const hs_sim_params& p) {
  if (p.mode == HS_MODE_REFERENCE) return kClassRef;
  return p.contract == HS_CONTRACT_FAST ? kClassFast : kClassExact;
}

// Buckets: one per (capacity, class); capacities 4, 8, 16, 24, 32, 64.
constexpr int kMaxBuckets = 6 * kClasses;

// Device table entry, one per groom of the batch (a multiple of 16 bytes:
// warps stage it in shared memory ahead of their state).
struct BatchGroomDev {
  GroomView view;
  FrameConst fc;
};
static_assert(sizeof(BatchGroomDev) % 16 == 0, "table entries must keep float4 alignment");

// Per-bucket header, in device memory.
struct BucketHeader {
  uint32_t ndir;        // grooms in the bucket
  uint32_t ntiles;      // 32-strand tiles in the bucket
  uint32_t dir_offset;  // first directory entry of the bucket
  uint32_t pad;
};

// Directory entry: a groom of the bucket and its first tile (sorted).
struct BucketDir {
  uint32_t groom;
  uint32_t first_tile;
};

// One bucket of the current groom set and how it is launched.
struct Bucket {
  int cap = 0;
  int cls = kClassExact;  // step class
  int variant = kVariantRegs;
  int warps_per_block = 4;
  uint32_t grid = 1;
  uint32_t ntiles = 0;
  int lanes_k = 0;  // smallest lane group every groom of the bucket fits (0: none, lane_group)
};

struct BatchState {
  // Persistent buffers, grown geometrically, never shrunk while in use.
  // Layout: [headers][directory (cap_grooms)][table (cap_grooms)].
  char* d_buf = nullptr;
  char* h_buf[2] = {nullptr, nullptr};  // pinned staging, alternating
  uint32_t cap_grooms = 0;
  uint32_t* d_counters = nullptr;       // one tile counter per bucket slot
  cudaEvent_t done[2] = {nullptr, nullptr};
  int next = 0;
  // Current groom set.
  std::vector<uint64_t> signature;
  uint32_t ngrooms = 0;
  std::vector<Bucket> buckets;          // bucket b uses header/counter slot b
  std::vector<BucketDir> dirs;          // grouped by bucket
  std::vector<BucketHeader> headers;
  // The frame graph: counter reset, table copy, one kernel per bucket.
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraphNode_t copy_node = nullptr;
  std::vector<int64_t> graph_shape;     // buckets and buffers the graph was built for
  ~BatchState();
  void release();
  void release_graph();
  size_t dir_offset() const;
  size_t table_offset() const;
  size_t bytes_used(uint32_t n) const;
};

// Launch shape of a bucket, chosen by the autotuner.
struct TuneChoice {
  int warps_per_block = 4;
  int waves = 1;  // persistent grid = SMs x resident blocks per SM x waves
  int variant = kVariantRegs;
};

// Key: (capacity, step class, log2 of the bucket's tile count).
using TuneKey = std::tuple<int, int, int>;

struct TuneCache {
  std::map<TuneKey, TuneChoice> best;
  std::map<TuneKey, float> best_ms;
  std::map<std::pair<int, bool>, TuneChoice> pinned;  // hs_tune_override
};

TuneKey tune_key(int cap, int cls, uint32_t ntiles);
TuneChoice tuned_choice(hs_ctx* ctx, int cap, int cls, uint32_t ntiles);
TuneChoice default_choice(int cap);  // the untuned shape of a capacity
int batch_occupancy(int cap, int cls, int variant, int warps_per_block);
hs_status batch_update(hs_ctx* ctx, hs_groom* const* grooms, uint32_t n, float dt);

}  // namespace hs
