// hs_batch.cu -- batched update: many grooms of uneven strand and point
// counts advanced together, one CUDA graph launch per frame.
//
// Work decomposition. Every groom is cut into tiles of 32 consecutive
// strands (one warp, thread per strand). Grooms are grouped in buckets by
// (point capacity, mode): each bucket has its own compiled step and
// register budget. A bucket is advanced by one persistent kernel whose
// warps take tiles from a shared counter, so grooms with many spheres or
// substeps leave no warp idle; a warp finds the groom of tile t by binary
// search in the bucket's directory of (groom, first tile). The per-frame
// constants of every groom live in a device table; a warp stages its
// current groom's entry (spheres included) in shared memory.
//
// One frame = one graph launch: counter reset, one host-to-device copy of
// headers + directory + table, the bucket kernels as independent nodes.
// The graph is built once per bucket shape. Grooms arriving or leaving
// change only the copied contents (and the copy's size, updated in the
// executable graph), so a served stream whose set changes every tick does
// not rebuild anything. Staging alternates between two pinned buffers,
// each guarded by an event.
//
// Results are bit-identical to hs_update on each groom alone: a strand's
// frame depends only on its own state and its groom's constants.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <cstring>
#include <map>
#include <mutex>
#include <set>
#include <vector>

#include "hs_api_internal.h"
#include "hs_batch.h"
#include "hs_lanes.cuh"
#include "hs_step.cuh"
#include "hs_stream.cuh"
#include "hs_tmem.cuh"

namespace hs {

namespace {

constexpr int kWarp = 32;
constexpr size_t kAlign = 256;

size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

// Copies a table entry into this warp's shared slot.
__device__ __forceinline__ void warp_copy(void* dst, const void* src, size_t bytes, int lane) {
  const uint32_t* s = static_cast<const uint32_t*>(src);
  uint32_t* d = static_cast<uint32_t*>(dst);
  for (size_t w = lane; w < bytes / 4; w += kWarp) d[w] = __ldg(s + w);
  __syncwarp();
}

// Next tile of the bucket for this warp: false when none is left.
__device__ __forceinline__ bool next_tile(const BucketHeader& H, const BucketDir* __restrict__ dirs,
                                          uint32_t* counter, int lane, uint32_t* groom, uint32_t* strand0) {
  uint32_t t = 0;
  if (lane == 0) t = atomicAdd(counter, 1u);
  t = __shfl_sync(0xffffffffu, t, 0);
  if (t >= H.ntiles) return false;
  const BucketDir* d = dirs + H.dir_offset;
  uint32_t lo = 0, hi = H.ndir - 1;
  while (lo < hi) {
    const uint32_t mid = (lo + hi + 1) / 2;
    if (d[mid].first_tile <= t) lo = mid;
    else hi = mid - 1;
  }
  *groom = d[lo].groom;
  *strand0 = (t - d[lo].first_tile) * kWarp;
  return true;
}

// Largest block the autotuner tries: 8 warps.
constexpr int kMaxBatchBlock = 256;

// Register cap per (capacity, velocity storage). With the velocity slots in
// shared memory, about what the plain step needs for the same capacity, so
// that registers and shared memory allow a similar number of warps; with
// them in registers, no cap below the hardware's.
template <int CAP, bool VSMEM>
struct RegBudget {
  static constexpr int value = VSMEM ? 128 : 255;
};

// FAST (every batched kernel): the bucket's grooms run the FAST contract;
// a kernel of its own, with no code of the other contract in it.
template <int CAP, bool REF, bool VSMEM, bool FAST>
__global__ void __launch_bounds__(kMaxBatchBlock) __maxnreg__((RegBudget<CAP, VSMEM>::value))
    k_step_batch(const BucketHeader* __restrict__ hdr, const BucketDir* __restrict__ dirs,
                 const BatchGroomDev* __restrict__ table, uint32_t* __restrict__ counters, int bucket, int cap) {
  extern __shared__ float4 s_raw[];
  const int warps = blockDim.x / kWarp;
  const int warp = threadIdx.x / kWarp;
  const int lane = threadIdx.x % kWarp;
  BatchGroomDev* s_entry = reinterpret_cast<BatchGroomDev*>(s_raw);
  float4* s_vel = s_raw + (sizeof(BatchGroomDev) / sizeof(float4)) * warps;  // per-thread velocity rows (VSMEM)
  BatchGroomDev& e = s_entry[warp];
  const BucketHeader H = hdr[bucket];
  uint32_t cur = 0xffffffffu, g = 0, strand0 = 0;
  (void)cap;
  while (next_tile(H, dirs, counters + bucket, lane, &g, &strand0)) {
    if (g != cur) {
      __syncwarp();
      warp_copy(&e, &table[g], sizeof(BatchGroomDev), lane);
      cur = g;
    }
    const uint32_t s = strand0 + lane;
    const SphereSet S{e.fc.spheres, e.fc.r2, e.fc.adj, e.fc.nspheres};
    if constexpr (REF) strand_frame_ref<CAP, VSMEM>(e.fc, S, e.view, s, s < e.view.nstrands, s_vel, threadIdx.x);
    else strand_frame_regs_dftl<CAP, VSMEM, FAST>(e.fc, S, e.view, s, s < e.view.nstrands, s_vel, threadIdx.x);
  }
}

// Streaming form: any point count up to `cap`; the block's shared state
// is [cap][blockDim] positions then [cap][blockDim] velocities.
template <bool REF, bool FAST>
__global__ void __maxnreg__(128)
    k_step_batch_stream(const BucketHeader* __restrict__ hdr, const BucketDir* __restrict__ dirs,
                        const BatchGroomDev* __restrict__ table, uint32_t* __restrict__ counters, int bucket,
                        int cap) {
  extern __shared__ float4 s_raw[];
  const int B = blockDim.x;
  const int warps = B / kWarp;
  const int warp = threadIdx.x / kWarp;
  const int lane = threadIdx.x % kWarp;
  BatchGroomDev* s_entry = reinterpret_cast<BatchGroomDev*>(s_raw);
  float4* Xs = s_raw + (sizeof(BatchGroomDev) / sizeof(float4)) * warps;
  float4* Vs = Xs + cap * B;
  BatchGroomDev& e = s_entry[warp];
  const BucketHeader H = hdr[bucket];
  uint32_t cur = 0xffffffffu, g = 0, strand0 = 0;
  while (next_tile(H, dirs, counters + bucket, lane, &g, &strand0)) {
    if (g != cur) {
      __syncwarp();
      warp_copy(&e, &table[g], sizeof(BatchGroomDev), lane);
      cur = g;
    }
    const uint32_t s = strand0 + lane;
    const SphereSet S{e.fc.spheres, e.fc.r2, e.fc.adj, e.fc.nspheres};
    strand_frame_stream<REF, XShared4, VShared, kCachedSpheres, false, false, FAST>(
        e.fc, S, e.view, s, s < e.view.nstrands, XShared4{Xs + threadIdx.x, B},
                             VShared{Vs + threadIdx.x, B});
  }
}

// Streaming form with the velocities in tensor memory (hs_tmem.cuh). Warp w
// of a block owns TMEM lane quadrant w % 4 and column slice w / 4; shared
// memory holds the table entries and the positions, 12 bytes a point.
// WARPS (4 or 8) is compile-time, so the shared-memory strides are
// immediates; resident blocks are bounded by TMEM and shared memory at 16
// warps per SM, so registers are held to 128 a thread.
template <bool REF, int WARPS, bool FAST>
__global__ void __launch_bounds__(WARPS * 32, 16 / WARPS)
    k_step_batch_stream_tmem(const BucketHeader* __restrict__ hdr, const BucketDir* __restrict__ dirs,
                             const BatchGroomDev* __restrict__ table, uint32_t* __restrict__ counters, int bucket,
                             int cap) {
  extern __shared__ float4 s_raw[];
  __shared__ uint32_t s_taddr;
  constexpr int B = WARPS * kWarp;
  constexpr int warps = WARPS;
  const int warp = threadIdx.x / kWarp;
  const int lane = threadIdx.x % kWarp;
  const uint32_t slice = tmem::cols_for(static_cast<uint32_t>(cap));
  const uint32_t ncols = slice * static_cast<uint32_t>(warps / 4);
  if (warp == 0) {
    tmem::alloc(&s_taddr, ncols);
    tmem::relinquish();
  }
  tmem::fence_before_sync();
  __syncthreads();
  tmem::fence_after_sync();
  const uint32_t base = s_taddr;
  const VTmem V{base + ((static_cast<uint32_t>(warp % 4) * 32u) << 16) + static_cast<uint32_t>(warp / 4) * slice};
  BatchGroomDev* s_entry = reinterpret_cast<BatchGroomDev*>(s_raw);
  // Positions, compact: float2 (x, y) then float z, each [cap][B].
  float2* xy = reinterpret_cast<float2*>(s_raw + (sizeof(BatchGroomDev) / sizeof(float4)) * warps);
  float* zs = reinterpret_cast<float*>(xy + cap * B);
  const XShared3 X{xy + threadIdx.x, zs + threadIdx.x, B};
  BatchGroomDev& e = s_entry[warp];
  const BucketHeader H = hdr[bucket];
  uint32_t cur = 0xffffffffu, g = 0, strand0 = 0;
  while (next_tile(H, dirs, counters + bucket, lane, &g, &strand0)) {
    if (g != cur) {
      __syncwarp();
      warp_copy(&e, &table[g], sizeof(BatchGroomDev), lane);
      cur = g;
    }
    const uint32_t s = strand0 + lane;
    const SphereSet S{e.fc.spheres, e.fc.r2, e.fc.adj, e.fc.nspheres};
    strand_frame_stream<REF, XShared3, VTmem, kCachedSpheres, false, false, FAST>(e.fc, S, e.view, s,
                                                                                 s < e.view.nstrands, X, V);
  }
  tmem::fence_before_sync();
  __syncthreads();
  tmem::fence_after_sync();
  if (warp == 0) tmem::dealloc(base, ncols);
}

// Lane groups (hs_lanes.cuh): a block of K warps takes one 32-strand tile
// at a time from the bucket's counter. Shared memory: the groom's table
// entry, then the tile's starting state ([cap][32] positions, then
// velocities). Register cap 128 (16 warps a SM).
template <int K, bool FAST>
__global__ void __launch_bounds__(K * 32, 16 / K)
    k_step_batch_lanes(const BucketHeader* __restrict__ hdr, const BucketDir* __restrict__ dirs,
                       const BatchGroomDev* __restrict__ table, uint32_t* __restrict__ counters, int bucket,
                       int cap) {
  extern __shared__ float4 s_raw[];
  __shared__ TileStats s_ts[32];
  __shared__ uint32_t s_next[2];
  BatchGroomDev& e = *reinterpret_cast<BatchGroomDev*>(s_raw);
  float4* s_p = s_raw + sizeof(BatchGroomDev) / sizeof(float4);
  float4* s_v = s_p + cap * 32;
  const BucketHeader H = hdr[bucket];
  uint32_t cur = 0xffffffffu;
  for (;;) {
    if (threadIdx.x < kWarp) {
      uint32_t g = 0, strand0 = 0;
      const bool more = next_tile(H, dirs, counters + bucket, static_cast<int>(threadIdx.x), &g, &strand0);
      if (threadIdx.x == 0) {
        s_next[0] = more ? g : 0xffffffffu;
        s_next[1] = strand0;
      }
    }
    __syncthreads();
    const uint32_t g = s_next[0], strand0 = s_next[1];
    if (g == 0xffffffffu) break;
    if (g != cur) {
      const uint32_t* src = reinterpret_cast<const uint32_t*>(&table[g]);
      uint32_t* dst = reinterpret_cast<uint32_t*>(&e);
      for (uint32_t w = threadIdx.x; w < sizeof(BatchGroomDev) / 4; w += blockDim.x) dst[w] = __ldg(src + w);
      cur = g;
      __syncthreads();
    }
    const SphereSet S{e.fc.spheres, e.fc.r2, e.fc.adj, e.fc.nspheres};
    tile_frame_lanes<K, kCachedSpheres, false, FAST>(e.fc, S, e.view, strand0 / kWarp, s_p, s_v, s_ts);
    __syncthreads();  // the next tile rewrites s_next, the entry and the state
  }
}

template <bool REF, bool FAST>
const void* any_cap_kernel(int variant, int warps) {
  if (is_lanes(variant)) {
    if (REF) return nullptr;
    if (warps == 2) return reinterpret_cast<const void*>(&k_step_batch_lanes<2, FAST>);
    if (warps == 4) return reinterpret_cast<const void*>(&k_step_batch_lanes<4, FAST>);
    if (warps == 8) return reinterpret_cast<const void*>(&k_step_batch_lanes<8, FAST>);
    if (warps == 16) return reinterpret_cast<const void*>(&k_step_batch_lanes<16, FAST>);
    return nullptr;
  }
  if (is_tmem(variant)) {
    if (warps == 4) return reinterpret_cast<const void*>(&k_step_batch_stream_tmem<REF, 4, FAST>);
    if (warps == 8) return reinterpret_cast<const void*>(&k_step_batch_stream_tmem<REF, 8, FAST>);
    return nullptr;
  }
  if (is_stream(variant)) return reinterpret_cast<const void*>(&k_step_batch_stream<REF, FAST>);
  return nullptr;
}

// Register variants exist for short strands only (up to 8 points): longer
// register-resident strands spill.
template <int CAP, bool REF, bool FAST>
const void* batch_kernel(int variant, int warps) {
  if (any_capacity(variant)) return any_cap_kernel<REF, FAST>(variant, warps);
  if (variant == kVariantRegsVsmem) return reinterpret_cast<const void*>(&k_step_batch<CAP, REF, true, FAST>);
  if (variant == kVariantRegs) return reinterpret_cast<const void*>(&k_step_batch<CAP, REF, false, FAST>);
  return nullptr;
}

template <int CAP>
const void* class_kernel(int cls, int variant, int warps) {
  if constexpr (CAP <= 8) {
    if (cls == kClassRef) return batch_kernel<CAP, true, false>(variant, warps);
    if (cls == kClassFast) return batch_kernel<CAP, false, true>(variant, warps);
    return batch_kernel<CAP, false, false>(variant, warps);
  } else {
    if (cls == kClassRef) return any_cap_kernel<true, false>(variant, warps);
    if (cls == kClassFast) return any_cap_kernel<false, true>(variant, warps);
    return any_cap_kernel<false, false>(variant, warps);
  }
}

// The kernel of a bucket shape (null where the shape is not built).
const void* kernel_for(int cap, int cls, int variant, int warps) {
  switch (cap) {
    case 4: return class_kernel<4>(cls, variant, warps);
    case 8: return class_kernel<8>(cls, variant, warps);
    case 16:
    case 24:
    case 32:
    case 64: return class_kernel<64>(cls, variant, warps);
    default: return nullptr;
  }
}

size_t smem_bytes(int cap, int warps, int variant) {
  if (is_lanes(variant)) return sizeof(BatchGroomDev) + 2 * sizeof(float4) * cap * kWarp;
  const size_t entries = sizeof(BatchGroomDev) * warps;
  if (is_tmem(variant)) return entries + (sizeof(float2) + sizeof(float)) * cap * warps * kWarp;
  if (is_stream(variant)) return entries + 2 * sizeof(float4) * cap * warps * kWarp;
  if (variant == kVariantRegsVsmem) return entries + sizeof(float4) * (cap + 1) * warps * kWarp;
  return entries;
}

int bucket_slot(int cap, int cls) {
  int c = 0;
  switch (cap) {
    case 4: c = 0; break;
    case 8: c = 1; break;
    case 16: c = 2; break;
    case 24: c = 3; break;
    case 32: c = 4; break;
    default: c = 5; break;
  }
  return kClasses * c + cls;
}

// Kernel arguments of one bucket launch (kept alive while a launch or a
// graph node is being made from them).
struct LaunchArgs {
  const BucketHeader* hdr;
  const BucketDir* dirs;
  const BatchGroomDev* table;
  uint32_t* counters;
  int bucket;
  int cap;
  void* ptrs[6];
  void bind() {
    ptrs[0] = &hdr;
    ptrs[1] = &dirs;
    ptrs[2] = &table;
    ptrs[3] = &counters;
    ptrs[4] = &bucket;
    ptrs[5] = &cap;
  }
};

void fill_args(const BatchState& B, int b, LaunchArgs* a) {
  a->hdr = reinterpret_cast<const BucketHeader*>(B.d_buf);
  a->dirs = reinterpret_cast<const BucketDir*>(B.d_buf + B.dir_offset());
  a->table = reinterpret_cast<const BatchGroomDev*>(B.d_buf + B.table_offset());
  a->counters = B.d_counters;
  a->bucket = b;
  a->cap = B.buckets[b].cap;
  a->bind();
}

cudaKernelNodeParams node_params(const Bucket& bk, LaunchArgs* a) {
  cudaKernelNodeParams p{};
  p.func = const_cast<void*>(kernel_for(bk.cap, bk.cls, bk.variant, bk.warps_per_block));
  p.gridDim = dim3(bk.grid);
  p.blockDim = dim3(bk.warps_per_block * kWarp);
  p.sharedMemBytes = static_cast<unsigned>(smem_bytes(bk.cap, bk.warps_per_block, bk.variant));
  p.kernelParams = a->ptrs;
  p.extra = nullptr;
  return p;
}

}  // namespace

int batch_occupancy(int cap, int cls, int variant, int warps_per_block) {
  const void* fn = kernel_for(cap, cls, variant, warps_per_block);
  if (!fn) return 0;
  const size_t smem = smem_bytes(cap, warps_per_block, variant);
  // Buckets of different capacities share the streaming kernel: opt every
  // kernel in to the device's largest dynamic shared memory once.
  const int optin = device_attribute(cudaDevAttrMaxSharedMemoryPerBlockOptin, 48 * 1024);
  // The dynamic part may use what the kernel's static shared memory leaves.
  cudaFuncAttributes fa;
  if (cudaFuncGetAttributes(&fa, fn) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  const int max_dynamic = optin - static_cast<int>(fa.sharedSizeBytes);
  if (smem > static_cast<size_t>(max_dynamic)) return 0;
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, max_dynamic) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  int blocks = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, warps_per_block * kWarp, smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  if (is_tmem(variant)) {
    // Every resident block holds its TMEM columns (512 per SM) for its life.
    if (warps_per_block % 4 != 0) return 0;
    const int cols = static_cast<int>(tmem::cols_for(static_cast<uint32_t>(cap))) * (warps_per_block / 4);
    if (cols > 512) return 0;
    blocks = std::min(blocks, 512 / cols);
  }
  return blocks;
}

// ---- persistent state ---------------------------------------------------

BatchState::~BatchState() { release(); }

void BatchState::release_graph() {
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  exec = nullptr;
  graph = nullptr;
  copy_node = nullptr;
  graph_shape.clear();
}

void BatchState::release() {
  release_graph();
  cudaFree(d_buf);
  d_buf = nullptr;
  cudaFree(d_counters);
  d_counters = nullptr;
  for (int k = 0; k < 2; ++k) {
    if (h_buf[k]) cudaFreeHost(h_buf[k]);
    h_buf[k] = nullptr;
    if (done[k]) cudaEventDestroy(done[k]);
    done[k] = nullptr;
  }
  cap_grooms = 0;
  signature.clear();
  buckets.clear();
  dirs.clear();
  headers.clear();
  ngrooms = 0;
}

size_t BatchState::dir_offset() const { return align_up(sizeof(BucketHeader) * kMaxBuckets); }
size_t BatchState::table_offset() const { return align_up(dir_offset() + sizeof(BucketDir) * cap_grooms); }
size_t BatchState::bytes_used(uint32_t n) const { return table_offset() + sizeof(BatchGroomDev) * n; }

// Makes room for n grooms (buffers grow by doubling; the graph is rebuilt).
static cudaError_t ensure_capacity(hs_ctx* ctx, BatchState& B, uint32_t n) {
  cudaError_t e = cudaSuccess;
  if (!B.d_counters) {
    e = cudaMalloc(&B.d_counters, sizeof(uint32_t) * kMaxBuckets);
    if (e != cudaSuccess) return e;
    for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
      e = cudaEventCreateWithFlags(&B.done[k], cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventRecord(B.done[k], ctx->stream);
    }
    if (e != cudaSuccess) return e;
  }
  if (n <= B.cap_grooms) return cudaSuccess;
  uint32_t cap = std::max<uint32_t>(64, B.cap_grooms);
  while (cap < n) cap *= 2;
  // Frames in flight read the old buffers.
  e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return e;
  B.release_graph();
  cudaFree(B.d_buf);
  B.d_buf = nullptr;
  for (int k = 0; k < 2; ++k) {
    if (B.h_buf[k]) cudaFreeHost(B.h_buf[k]);
    B.h_buf[k] = nullptr;
  }
  B.cap_grooms = cap;
  const size_t bytes = B.bytes_used(cap);
  e = cudaMalloc(&B.d_buf, bytes);
  for (int k = 0; k < 2 && e == cudaSuccess; ++k) e = cudaMallocHost(&B.h_buf[k], bytes);
  if (e != cudaSuccess) B.cap_grooms = 0;
  B.signature.clear();
  return e;
}

// A groom set's shape: grooms, modes, point counts, and what decides
// whether a bucket can take lane groups (substeps, iterations).
static std::vector<uint64_t> signature_of(hs_groom* const* grooms, uint32_t n) {
  std::vector<uint64_t> sig;
  sig.reserve(3 * n);
  for (uint32_t i = 0; i < n; ++i) {
    sig.push_back(reinterpret_cast<uint64_t>(grooms[i]));
    sig.push_back((static_cast<uint64_t>(grooms[i]->sim.mode) << 32) | grooms[i]->npoints);
    sig.push_back((static_cast<uint64_t>(grooms[i]->sim.substeps) << 32) |
                  (static_cast<uint64_t>(grooms[i]->sim.iterations) << 8) | grooms[i]->sim.contract);
  }
  return sig;
}

// The lane group every groom of a bucket fits (the largest of their
// lane_group sizes), 0 if one of them has no lane-group form.
static int bucket_lanes(hs_groom* const* grooms, const std::vector<uint32_t>& members) {
  int k = 0;
  for (uint32_t i : members) {
    const hs_sim_params& p = grooms[i]->sim;
    const int ki = lane_group(static_cast<int>(p.mode), static_cast<int>(p.substeps), static_cast<int>(p.iterations));
    if (ki == 0) return 0;
    k = std::max(k, ki);
  }
  return k;
}

// A lane-group shape runs a bucket only if every groom fits its groups.
static bool shape_fits(const Bucket& bk, const TuneChoice& c) {
  return !is_lanes(c.variant) || (bk.lanes_k > 0 && c.warps_per_block >= bk.lanes_k);
}

// Groups a new groom set into buckets with their directories and shapes.
static void regroup(hs_ctx* ctx, BatchState& B, hs_groom* const* grooms, uint32_t n) {
  // One flat work list: every DFTL groom of up to 32 points shares one
  // bucket (one persistent kernel) at the largest capacity among them, the
  // kernels taking each groom's point count at run time; reference-mode
  // grooms, longer strands and point classes with a pinned shape
  // (hs_tune_override) keep buckets of their own. (Per-capacity buckets ran
  // the same frame time and a 4 % longer served tick.)
  auto pinned = [&](int cap) {
    return ctx->tune && ctx->tune->pinned.count(std::make_pair(cap, false)) != 0;
  };
  auto flat = [&](const hs_groom* g, int cap) {
    return g->sim.mode != HS_MODE_REFERENCE && cap <= 32 && !pinned(cap);
  };  // one flat bucket per contract
  std::map<int, std::vector<uint32_t>> by_slot;
  std::map<int, int> slot_cap;
  int flat_cap = 0;
  for (uint32_t i = 0; i < n; ++i) {
    const int cap = step_capacity(grooms[i]->npoints);
    if (flat(grooms[i], cap)) flat_cap = std::max(flat_cap, cap);
  }
  for (uint32_t i = 0; i < n; ++i) {
    const int cls = step_class(grooms[i]->sim);
    int cap = step_capacity(grooms[i]->npoints);
    if (flat(grooms[i], cap)) cap = flat_cap;  // never a pinned class: distinct slots
    const int slot = bucket_slot(cap, cls);
    by_slot[slot].push_back(i);
    slot_cap[slot] = cap;
  }
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
  B.buckets.clear();
  B.dirs.clear();
  B.headers.assign(kMaxBuckets, BucketHeader{0, 0, 0, 0});
  // Longest tiles first, so that the frame ends on the shortest ones and
  // its last partial wave is short: buckets launch in descending point
  // capacity, and within a bucket longer strands, then grooms with more
  // spheres, come first. Measured on the 64-groom workload: 1.273 ->
  // 1.254 -> 1.222 ms per frame.
  for (auto it = by_slot.rbegin(); it != by_slot.rend(); ++it) {
    auto& kv = *it;
    std::stable_sort(kv.second.begin(), kv.second.end(), [&](uint32_t a, uint32_t b) {
      if (grooms[a]->npoints != grooms[b]->npoints) return grooms[a]->npoints > grooms[b]->npoints;
      return grooms[a]->spheres.size() > grooms[b]->spheres.size();
    });
    Bucket bk;
    const hs_groom* g0 = grooms[kv.second.front()];
    bk.cap = slot_cap[kv.first];
    bk.cls = step_class(g0->sim);
    BucketHeader h{};
    h.dir_offset = static_cast<uint32_t>(B.dirs.size());
    uint32_t tiles = 0;
    for (uint32_t i : kv.second) {
      B.dirs.push_back(BucketDir{i, tiles});
      tiles += (grooms[i]->nstrands + kWarp - 1) / kWarp;
    }
    h.ndir = static_cast<uint32_t>(kv.second.size());
    h.ntiles = tiles;
    bk.ntiles = tiles;
    bk.lanes_k = bk.cls == kClassRef ? 0 : bucket_lanes(grooms, kv.second);
    TuneChoice tc = tuned_choice(ctx, bk.cap, bk.cls, tiles);
    // A lane-group shape tuned or pinned for this class does not run a
    // bucket with a groom of more substeps (or iterations): the default.
    if (!shape_fits(bk, tc)) tc = default_choice(bk.cap);
    bk.variant = tc.variant;
    bk.warps_per_block = tc.warps_per_block;
    const int occ = std::max(1, batch_occupancy(bk.cap, bk.cls, bk.variant, bk.warps_per_block));
    bk.grid = static_cast<uint32_t>(sms * occ * tc.waves);
    // Bucket b of the launch reads header and counter slot b.
    B.headers[B.buckets.size()] = h;
    B.buckets.push_back(bk);
  }
  B.signature = signature_of(grooms, n);
  B.ngrooms = n;
}

// Fills a staging slot: headers, directory, table.
static hs_status fill(BatchState& B, int slot, hs_groom* const* grooms, uint32_t n, float dt) {
  char* h = B.h_buf[slot];
  std::memcpy(h, B.headers.data(), sizeof(BucketHeader) * kMaxBuckets);
  std::memcpy(h + B.dir_offset(), B.dirs.data(), sizeof(BucketDir) * B.dirs.size());
  BatchGroomDev* table = reinterpret_cast<BatchGroomDev*>(h + B.table_offset());
  for (uint32_t i = 0; i < n; ++i) {
    hs_status st = make_frame_const(grooms[i], dt, &table[i].fc);
    if (st != HS_OK) return st;
    table[i].view = view_of(grooms[i]);
  }
  return HS_OK;
}

static std::vector<int64_t> shape_of(const BatchState& B) {
  std::vector<int64_t> s{reinterpret_cast<int64_t>(B.d_buf), static_cast<int64_t>(B.cap_grooms)};
  for (const Bucket& bk : B.buckets) {
    s.push_back(bk.cap);
    s.push_back(bk.cls);
    s.push_back(bk.variant);
    s.push_back(bk.warps_per_block);
    s.push_back(bk.grid);
  }
  return s;
}

// Builds the frame graph: counter reset and table copy, then the buckets.
static cudaError_t build_graph(BatchState& B, int slot, size_t bytes) {
  B.release_graph();
  cudaError_t e = cudaGraphCreate(&B.graph, 0);
  cudaGraphNode_t reset = nullptr;
  if (e == cudaSuccess) {
    cudaMemsetParams mp{};
    mp.dst = B.d_counters;
    mp.value = 0;
    mp.elementSize = sizeof(uint32_t);
    mp.width = kMaxBuckets;
    mp.height = 1;
    e = cudaGraphAddMemsetNode(&reset, B.graph, nullptr, 0, &mp);
  }
  if (e == cudaSuccess)
    e = cudaGraphAddMemcpyNode1D(&B.copy_node, B.graph, nullptr, 0, B.d_buf, B.h_buf[slot], bytes,
                                 cudaMemcpyHostToDevice);
  std::vector<LaunchArgs> args(B.buckets.size());
  for (size_t b = 0; b < B.buckets.size() && e == cudaSuccess; ++b) {
    fill_args(B, static_cast<int>(b), &args[b]);
    cudaKernelNodeParams p = node_params(B.buckets[b], &args[b]);
    cudaGraphNode_t deps[2] = {reset, B.copy_node};
    cudaGraphNode_t kn = nullptr;
    e = cudaGraphAddKernelNode(&kn, B.graph, deps, 2, &p);
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&B.exec, B.graph, 0);
  if (e != cudaSuccess) {
    cudaGetLastError();
    B.release_graph();
    return e;
  }
  B.graph_shape = shape_of(B);
  return cudaSuccess;
}

hs_status batch_update(hs_ctx* ctx, hs_groom* const* grooms, uint32_t n, float dt) {
  if (!ctx->batch) ctx->batch = new BatchState();
  BatchState& B = *ctx->batch;
  cudaError_t e = ensure_capacity(ctx, B, n);
  if (e != cudaSuccess) return cuda_fail(e, "hs_update_many: buffers");
  if (B.signature != signature_of(grooms, n)) regroup(ctx, B, grooms, n);
  const int slot = B.next;
  e = cudaEventSynchronize(B.done[slot]);
  if (e != cudaSuccess) return cuda_fail(e, "hs_update_many: wait for staging slot");
  hs_status st = fill(B, slot, grooms, n, dt);
  if (st != HS_OK) return st;
  const size_t bytes = B.bytes_used(n);
  if (!B.exec || B.graph_shape != shape_of(B)) {
    e = build_graph(B, slot, bytes);
    if (e != cudaSuccess) return cuda_fail(e, "hs_update_many: graph");
  } else {
    e = cudaGraphExecMemcpyNodeSetParams1D(B.exec, B.copy_node, B.d_buf, B.h_buf[slot], bytes,
                                           cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "hs_update_many: graph copy update");
  }
  e = cudaGraphLaunch(B.exec, ctx->stream);
  if (e == cudaSuccess) e = cudaEventRecord(B.done[slot], ctx->stream);
  if (e != cudaSuccess) return cuda_fail(e, "hs_update_many: launch");
  for (uint32_t i = 0; i < n; ++i) grooms[i]->stats_valid = true;
  ctx->launches += B.buckets.size();
  B.next ^= 1;
  return HS_OK;
}

// ---- autotuner ------------------------------------------------------------

TuneKey tune_key(int cap, int cls, uint32_t ntiles) {
  int lg = 0;
  while (lg < 31 && (1u << (lg + 1)) <= ntiles) ++lg;
  return TuneKey{cap, cls, lg};
}

// Pins (hs_tune_override) are per (capacity, mode): both contracts of a
// DFTL class take them.
TuneChoice tuned_choice(hs_ctx* ctx, int cap, int cls, uint32_t ntiles) {
  if (ctx->tune) {
    auto ov = ctx->tune->pinned.find(std::make_pair(cap, cls == kClassRef));
    if (ov != ctx->tune->pinned.end()) return ov->second;
    auto it = ctx->tune->best.find(tune_key(cap, cls, ntiles));
    if (it != ctx->tune->best.end()) return it->second;
  }
  return default_choice(cap);
}

TuneChoice default_choice(int cap) {
  // Untuned: the streaming form, one substep at a time; from 16 points up
  // with the velocities in tensor memory (4 warps per block, a grid of 4
  // waves of resident blocks: the fastest fixed shape measured on the
  // batched workload), below that in shared memory with one warp per block.
  TuneChoice c;
  if (cap >= 16) {
    c.variant = kVariantStreamTmem;
    c.warps_per_block = 4;
    c.waves = 4;
  } else {
    c.variant = kVariantStream;
    c.warps_per_block = 1;
  }
  return c;
}

// Times the candidate launch shapes of every bucket of the groom set on the
// live state, keeps the fastest in the context's cache, then restores the
// state the trials advanced.
static hs_status autotune(hs_ctx* ctx, hs_groom* const* grooms, uint32_t n, float dt, uint32_t* out_trials) {
  if (!ctx->tune) ctx->tune = new TuneCache();
  if (!ctx->batch) ctx->batch = new BatchState();
  BatchState& B = *ctx->batch;
  cudaStream_t s = ctx->stream;
  cudaError_t e = ensure_capacity(ctx, B, n);
  if (e != cudaSuccess) return cuda_fail(e, "hs_autotune: buffers");
  regroup(ctx, B, grooms, n);
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "hs_autotune");
  hs_status st = fill(B, 0, grooms, n, dt);
  if (st != HS_OK) return st;
  e = cudaMemcpyAsync(B.d_buf, B.h_buf[0], B.bytes_used(n), cudaMemcpyHostToDevice, s);
  // Snapshot of every groom's state.
  std::vector<float4*> snap(2 * n, nullptr);
  for (uint32_t i = 0; i < n && e == cudaSuccess; ++i) {
    const size_t bytes = sizeof(float4) * static_cast<size_t>(grooms[i]->stride) * grooms[i]->npoints;
    e = cudaMalloc(&snap[2 * i], bytes);
    if (e == cudaSuccess) e = cudaMalloc(&snap[2 * i + 1], bytes);
    if (e == cudaSuccess) e = cudaMemcpyAsync(snap[2 * i], grooms[i]->d_pos, bytes, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(snap[2 * i + 1], grooms[i]->d_vel, bytes, cudaMemcpyDeviceToDevice, s);
  }
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  if (e == cudaSuccess) e = cudaEventCreate(&t0);
  if (e == cudaSuccess) e = cudaEventCreate(&t1);
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
  uint32_t trials = 0;
  for (size_t b = 0; b < B.buckets.size() && e == cudaSuccess; ++b) {
    const Bucket& bk = B.buckets[b];
    float best = 1e30f;
    TuneChoice best_c = tuned_choice(ctx, bk.cap, bk.cls, bk.ntiles);
    for (int variant = 0; variant < kVariants && e == cudaSuccess; ++variant) {
      if (bk.cap > 32 && !any_capacity(variant)) continue;
      for (int wpb : {1, 2, 4, 8, 16}) {
        if (!shape_fits(bk, TuneChoice{wpb, 1, variant})) continue;
        if (wpb == 16 && !is_lanes(variant)) continue;
        const int occ = batch_occupancy(bk.cap, bk.cls, variant, wpb);
        if (occ <= 0) continue;
        for (int waves : {1, 2, 4}) {
          Bucket trial = bk;
          trial.variant = variant;
          trial.warps_per_block = wpb;
          trial.grid = static_cast<uint32_t>(sms * occ * waves);
          LaunchArgs a;
          fill_args(B, static_cast<int>(b), &a);
          const cudaKernelNodeParams p = node_params(trial, &a);
          float ms_sum = 0.0f;
          const int reps = 3;
          for (int r = 0; r < reps + 1 && e == cudaSuccess; ++r) {
            e = cudaMemsetAsync(B.d_counters + b, 0, sizeof(uint32_t), s);
            if (e == cudaSuccess) e = cudaEventRecord(t0, s);
            if (e == cudaSuccess)
              e = cudaLaunchKernel(p.func, p.gridDim, p.blockDim, p.kernelParams, p.sharedMemBytes, s);
            if (e == cudaSuccess) e = cudaEventRecord(t1, s);
            if (e == cudaSuccess) e = cudaEventSynchronize(t1);
            float ms = 0.0f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, t0, t1);
            if (r > 0) ms_sum += ms;  // the first run warms up
            ctx->launches += 1;
          }
          ++trials;
          const float ms = ms_sum / reps;
          if (e == cudaSuccess && ms < best) {
            best = ms;
            best_c = TuneChoice{wpb, waves, variant};
          }
        }
      }
    }
    const TuneKey key = tune_key(bk.cap, bk.cls, bk.ntiles);
    ctx->tune->best[key] = best_c;
    ctx->tune->best_ms[key] = best;
  }
  // Restore the state the trials advanced.
  for (uint32_t i = 0; i < n; ++i) {
    const size_t bytes = sizeof(float4) * static_cast<size_t>(grooms[i]->stride) * grooms[i]->npoints;
    if (snap[2 * i] && e == cudaSuccess)
      e = cudaMemcpyAsync(grooms[i]->d_pos, snap[2 * i], bytes, cudaMemcpyDeviceToDevice, s);
    if (snap[2 * i + 1] && e == cudaSuccess)
      e = cudaMemcpyAsync(grooms[i]->d_vel, snap[2 * i + 1], bytes, cudaMemcpyDeviceToDevice, s);
  }
  cudaError_t e2 = cudaStreamSynchronize(s);
  if (e == cudaSuccess) e = e2;
  for (float4* p : snap) cudaFree(p);
  if (t0) cudaEventDestroy(t0);
  if (t1) cudaEventDestroy(t1);
  B.signature.clear();  // the next update regroups with the tuned shapes
  for (uint32_t i = 0; i < n; ++i) grooms[i]->stats_valid = false;  // the trials' frames were undone
  if (out_trials) *out_trials = trials;
  if (e != cudaSuccess) return cuda_fail(e, "hs_autotune");
  return HS_OK;
}

void destroy_ctx_extensions(hs_ctx* ctx) {
  delete ctx->batch;
  ctx->batch = nullptr;
  delete ctx->tune;
  ctx->tune = nullptr;
}

}  // namespace hs

using namespace hs;

extern "C" {

static hs_status validate_set(hs_ctx* ctx, hs_groom* const* grooms, uint32_t n, const char* what) {
  if (!ctx || (n > 0 && !grooms)) return fail(HS_ERR_INVALID_ARG, "%s: null argument", what);
  std::set<const hs_groom*> seen;
  for (uint32_t i = 0; i < n; ++i) {
    if (!grooms[i] || grooms[i]->ctx != ctx)
      return fail(HS_ERR_INVALID_ARG, "%s: groom %u is null or belongs to another context", what, i);
    if (!seen.insert(grooms[i]).second) return fail(HS_ERR_INVALID_ARG, "%s: groom %u listed twice", what, i);
  }
  return HS_OK;
}

HS_API hs_status hs_update_many(hs_ctx* ctx, hs_groom* const* grooms, uint32_t n, float dt) {
  hs_status st = validate_set(ctx, grooms, n, "hs_update_many");
  if (st != HS_OK || n == 0) return st;
  HS_ON_DEVICE(ctx, "hs_update_many");
  return batch_update(ctx, grooms, n, dt);
}

HS_API hs_status hs_tune_override(hs_ctx* ctx, uint32_t points, uint32_t mode, uint32_t variant,
                                  uint32_t warps_per_block, uint32_t waves) {
  if (!ctx) return fail(HS_ERR_INVALID_ARG, "hs_tune_override: null context");
  const int cap = step_capacity(points);
  if (cap == 0) return fail(HS_ERR_INVALID_ARG, "hs_tune_override: %u points per strand", points);
  if (mode > HS_MODE_DFTL) return fail(HS_ERR_INVALID_ARG, "hs_tune_override: unknown mode %u", mode);
  if (variant >= static_cast<uint32_t>(kVariants) || (cap > 32 && !any_capacity(static_cast<int>(variant))))
    return fail(HS_ERR_INVALID_ARG, "hs_tune_override: variant %u unavailable for %u points", variant, points);
  if (warps_per_block != 1 && warps_per_block != 2 && warps_per_block != 4 && warps_per_block != 8 &&
      !(warps_per_block == 16 && is_lanes(static_cast<int>(variant))))
    return fail(HS_ERR_INVALID_ARG, "hs_tune_override: warps per block must be 1, 2, 4 or 8 (16: lane groups)");
  if (is_lanes(static_cast<int>(variant)) && mode != HS_MODE_DFTL)
    return fail(HS_ERR_UNSUPPORTED, "hs_tune_override: lane groups run DFTL mode only");
  if (waves != 1 && waves != 2 && waves != 4) return fail(HS_ERR_INVALID_ARG, "hs_tune_override: waves must be 1, 2 or 4");
  if (batch_occupancy(cap, mode == HS_MODE_REFERENCE ? kClassRef : kClassExact, static_cast<int>(variant),
                      static_cast<int>(warps_per_block)) <= 0)
    return fail(HS_ERR_UNSUPPORTED, "hs_tune_override: that shape does not fit on an SM");
  if (!ctx->tune) ctx->tune = new TuneCache();
  ctx->tune->pinned[std::make_pair(cap, mode == HS_MODE_REFERENCE)] =
      TuneChoice{static_cast<int>(warps_per_block), static_cast<int>(waves), static_cast<int>(variant)};
  if (ctx->batch) ctx->batch->signature.clear();  // the next update regroups
  return HS_OK;
}

HS_API hs_status hs_tune_entries(hs_ctx* ctx, hs_tune_entry* out, uint32_t capacity, uint32_t* out_count) {
  if (!ctx || !out_count || (capacity > 0 && !out)) return fail(HS_ERR_INVALID_ARG, "hs_tune_entries: null argument");
  uint32_t n = 0;
  if (ctx->tune) {
    for (const auto& kv : ctx->tune->best) {
      if (n < capacity) {
        hs_tune_entry& e = out[n];
        e.capacity = static_cast<uint32_t>(std::get<0>(kv.first));
        e.mode = std::get<1>(kv.first) == kClassRef ? HS_MODE_REFERENCE : HS_MODE_DFTL;
        e.tiles_log2 = static_cast<uint32_t>(std::get<2>(kv.first));
        e.variant = static_cast<uint32_t>(kv.second.variant);
        e.warps_per_block = static_cast<uint32_t>(kv.second.warps_per_block);
        e.waves = static_cast<uint32_t>(kv.second.waves);
        auto ms = ctx->tune->best_ms.find(kv.first);
        e.ms = ms != ctx->tune->best_ms.end() ? ms->second : 0.0f;
        e.contract = std::get<1>(kv.first) == kClassFast ? HS_CONTRACT_FAST : HS_CONTRACT_EXACT;
      }
      ++n;
    }
  }
  *out_count = n;
  return HS_OK;
}

HS_API hs_status hs_autotune(hs_ctx* ctx, hs_groom* const* grooms, uint32_t n, float dt, uint32_t* out_trials) {
  hs_status st = validate_set(ctx, grooms, n, "hs_autotune");
  if (st != HS_OK) return st;
  HS_ON_DEVICE(ctx, "hs_autotune");
  if (n == 0) {
    if (out_trials) *out_trials = 0;
    return HS_OK;
  }
  return autotune(ctx, grooms, n, dt, out_trials);
}

}  // extern "C"

// ---- update without allocation ---------------------------------------------
//
// hs_update_many_noalloc is the batched step for callers that must not
// allocate device memory once their grooms exist: engines and renderers
// that reserve their whole GPU budget at load time and forbid allocation in
// the frame loop (cudaMalloc and cudaFree can synchronise the device and
// stall a frame; a list that grows mid-session would grow hs_update_many's
// buffers past the reserved budget). hs_update_many keeps its tile counters,
// bucket directory and groom table in buffers it allocates, grows and
// captures into a graph on demand; this entry point keeps the same scratch
// in one file-scope device array of fixed size instead and launches the
// same streaming kernel on it, so its results are bit-identical.
//
// Every call looks up the array's address on its device
// (cudaGetSymbolAddress with the device current, no allocation); the first
// call on a device also reads its launch limits, and should come before any
// stream capture. The host stages the per-call
// contents through kernel parameters (stream-ordered, nothing on the host
// outlives the call). Every call on a device shares the array and finds the
// previous call's contents there: the tile counters are cleared each call.
// Calls on one stream are ordered; calls that overlap on the GPU (two
// streams, two contexts of one device, two host threads) race on the array.

namespace hs {
namespace {

constexpr uint32_t kNoAllocMaxGrooms = HS_NOALLOC_MAX_GROOMS;
constexpr uint32_t kNoAllocCounters = 32;  // >= kMaxBuckets, one 128-byte line

struct NoAllocScratch {
  uint32_t counters[kNoAllocCounters];   // tile counter per bucket slot
  BucketHeader headers[kMaxBuckets];     // indexed by bucket slot
  BucketDir dirs[kNoAllocMaxGrooms];     // grouped by bucket slot
  BatchGroomDev table[kNoAllocMaxGrooms];
};
static_assert(kNoAllocCounters >= kMaxBuckets, "one counter per bucket slot");
static_assert(offsetof(NoAllocScratch, table) % 16 == 0, "table entries keep float4 alignment");

// Kernel parameters are limited to 32,764 bytes: the table is staged in
// chunks of this many entries.
constexpr uint32_t kStageEntries = 24;

struct StageDir {
  BucketHeader headers[kMaxBuckets];
  BucketDir dirs[kNoAllocMaxGrooms];
  uint32_t ndirs;
};

struct StageTable {
  uint32_t first;  // first table slot written
  uint32_t count;  // entries in this chunk
  uint32_t pad[2];
  BatchGroomDev entries[kStageEntries];
};
static_assert(sizeof(StageDir) + sizeof(void*) <= 32764, "kernel parameter limit");
static_assert(sizeof(StageTable) + sizeof(void*) <= 32764, "kernel parameter limit");

constexpr int kNoAllocMaxDevices = 64;

struct NoAllocDevice {
  bool ready = false;
  NoAllocScratch* scratch = nullptr;  // this device's address of the scratch array (this call's lookup)
  int sms = 0;
  int occupancy[kMaxBuckets] = {0};   // resident blocks per SM, by bucket slot
};

std::mutex g_noalloc_mu;
NoAllocDevice g_noalloc_dev[kNoAllocMaxDevices];

constexpr int kNoAllocCaps[] = {4, 8, 16, 24, 32, 64};

// Clears the tile counters and writes the bucket headers and directory.
__global__ void k_noalloc_stage_dir(const __grid_constant__ StageDir p, NoAllocScratch* s) {
  for (uint32_t i = threadIdx.x; i < kNoAllocCounters; i += blockDim.x) s->counters[i] = 0u;
  for (uint32_t i = threadIdx.x; i < static_cast<uint32_t>(kMaxBuckets); i += blockDim.x) s->headers[i] = p.headers[i];
  for (uint32_t i = threadIdx.x; i < p.ndirs; i += blockDim.x) s->dirs[i] = p.dirs[i];
}

// Writes table entries [first, first + count).
__global__ void k_noalloc_stage_table(const __grid_constant__ StageTable p, NoAllocScratch* s) {
  const uint32_t* src = reinterpret_cast<const uint32_t*>(p.entries);
  uint32_t* dst = reinterpret_cast<uint32_t*>(s->table + p.first);
  const uint32_t words = p.count * static_cast<uint32_t>(sizeof(BatchGroomDev) / 4);
  for (uint32_t w = threadIdx.x; w < words; w += blockDim.x) dst[w] = src[w];
}

}  // namespace

// The scratch: every GPU that loads this library holds it until exit.
static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocScratch)];

namespace {

// With the device current: the scratch array's device address, looked up
// on every call (cheap, allocates nothing, and still right after a
// cudaDeviceReset reloads the module), and once per device the persistent
// grid of every bucket slot.
hs_status noalloc_setup(int device, NoAllocDevice* out) {
  if (device < 0 || device >= kNoAllocMaxDevices)
    return fail(HS_ERR_UNSUPPORTED, "hs_update_many_noalloc: device %d beyond the %d supported", device,
                kNoAllocMaxDevices);
  void* ptr = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
  if (e != cudaSuccess) return cuda_fail(e, "hs_update_many_noalloc: scratch address");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  NoAllocDevice& d = g_noalloc_dev[device];
  if (!d.ready) {
    e = cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) return cuda_fail(e, "hs_update_many_noalloc: SM count");
    for (int cap : kNoAllocCaps) {
      for (int cls = 0; cls < kClasses; ++cls) {
        const int occ = batch_occupancy(cap, cls, kVariantStream, 1);
        if (occ <= 0) return fail(HS_ERR_UNSUPPORTED, "hs_update_many_noalloc: %d-point step does not fit", cap);
        d.occupancy[bucket_slot(cap, cls)] = occ;
      }
    }
    d.ready = true;
  }
  *out = d;
  out->scratch = static_cast<NoAllocScratch*>(ptr);
  return HS_OK;
}

hs_status noalloc_update(hs_ctx* ctx, hs_groom* const* grooms, uint32_t n, float dt) {
  DeviceScope scope(ctx->device);
  if (scope.err != cudaSuccess) return cuda_fail(scope.err, "hs_update_many_noalloc: device");
  NoAllocDevice devs;
  hs_status st = noalloc_setup(ctx->device, &devs);
  if (st != HS_OK) return st;
  const NoAllocDevice* dev = &devs;
  // Buckets by slot (fixed arrays: nothing here allocates).
  StageDir dir;
  std::memset(&dir, 0, sizeof(dir));
  uint8_t slot_of[kNoAllocMaxGrooms];
  uint32_t count[kMaxBuckets] = {0};
  for (uint32_t i = 0; i < n; ++i) {
    const int cap = step_capacity(grooms[i]->npoints);
    slot_of[i] = static_cast<uint8_t>(bucket_slot(cap, step_class(grooms[i]->sim)));
    ++count[slot_of[i]];
  }
  uint32_t offset = 0;
  for (int b = 0; b < kMaxBuckets; ++b) {
    dir.headers[b].dir_offset = offset;
    dir.headers[b].ndir = count[b];
    offset += count[b];
  }
  uint32_t placed[kMaxBuckets] = {0};
  for (uint32_t i = 0; i < n; ++i) {
    const int b = slot_of[i];
    BucketHeader& h = dir.headers[b];
    dir.dirs[h.dir_offset + placed[b]++] = BucketDir{i, h.ntiles};
    h.ntiles += (grooms[i]->nstrands + kWarp - 1) / kWarp;
  }
  dir.ndirs = n;
  // Frame constants of every groom, validated before anything is launched.
  for (uint32_t i = 0; i < n; ++i) {
    FrameConst fc;
    st = make_frame_const(grooms[i], dt, &fc);
    if (st != HS_OK) return st;
  }
  StageTable chunk;  // on the stack: copied into the launch's parameters
  cudaStream_t stream = ctx->stream;
  NoAllocScratch* s = dev->scratch;
  k_noalloc_stage_dir<<<1, 256, 0, stream>>>(dir, s);
  cudaError_t e = cudaGetLastError();
  uint64_t launches = 1;
  for (uint32_t first = 0; first < n && e == cudaSuccess; first += kStageEntries) {
    chunk.first = first;
    chunk.count = std::min(kStageEntries, n - first);
    for (uint32_t k = 0; k < chunk.count; ++k) {
      make_frame_const(grooms[first + k], dt, &chunk.entries[k].fc);
      chunk.entries[k].view = view_of(grooms[first + k]);
    }
    k_noalloc_stage_table<<<1, 256, 0, stream>>>(chunk, s);
    e = cudaGetLastError();
    ++launches;
  }
  for (int b = 0; b < kMaxBuckets && e == cudaSuccess; ++b) {
    if (dir.headers[b].ntiles == 0) continue;
    const int cap = kNoAllocCaps[b / kClasses];
    const int cls = b % kClasses;
    const BucketHeader* hdr = s->headers;
    const BucketDir* dirs = s->dirs;
    const BatchGroomDev* table = s->table;
    uint32_t* counters = s->counters;
    int bucket = b;
    int cap_arg = cap;
    void* args[6] = {&hdr, &dirs, &table, &counters, &bucket, &cap_arg};
    const dim3 grid(static_cast<unsigned>(dev->sms * dev->occupancy[b]));
    e = cudaLaunchKernel(kernel_for(cap, cls, kVariantStream, 1), grid, dim3(kWarp), args,
                         smem_bytes(cap, 1, kVariantStream), stream);
    ++launches;
  }
  if (e != cudaSuccess) return cuda_fail(e, "hs_update_many_noalloc: launch");
  ctx->launches += launches;
  for (uint32_t i = 0; i < n; ++i) grooms[i]->stats_valid = true;
  return HS_OK;
}

}  // namespace
}  // namespace hs

extern "C" {

HS_API hs_status hs_update_many_noalloc(hs_ctx* ctx, hs_groom* const* grooms, uint32_t n, float dt) {
  if (!ctx || (n > 0 && !grooms)) return fail(HS_ERR_INVALID_ARG, "hs_update_many_noalloc: null argument");
  if (n > kNoAllocMaxGrooms)
    return fail(HS_ERR_INVALID_ARG, "hs_update_many_noalloc: %u grooms exceed the maximum of %u per call", n,
                kNoAllocMaxGrooms);
  for (uint32_t i = 0; i < n; ++i) {
    if (!grooms[i] || grooms[i]->ctx != ctx)
      return fail(HS_ERR_INVALID_ARG, "hs_update_many_noalloc: groom %u is null or belongs to another context", i);
    for (uint32_t j = 0; j < i; ++j)
      if (grooms[j] == grooms[i]) return fail(HS_ERR_INVALID_ARG, "hs_update_many_noalloc: groom %u listed twice", i);
  }
  if (n == 0) return HS_OK;
  return noalloc_update(ctx, grooms, n, dt);
}

}  // extern "C"
