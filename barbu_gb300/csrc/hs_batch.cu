// hs_batch.cu -- batched update: many grooms of uneven strand and point
// counts advanced together, one CUDA graph launch per frame.
//
// Work decomposition. Every groom is cut into tiles of 32 consecutive
// strands (one warp, thread per strand). Tiles are grouped in buckets by
// (capacity, mode): each bucket has its own compiled step and register
// budget. A bucket is advanced by one persistent kernel whose warps take
// tiles from a shared counter, so grooms with many spheres or substeps do
// not leave other warps idle. The per-frame constants of every groom live
// in a device table filled by one host-to-device copy per frame; a warp
// stages its current groom's entry (spheres included) in shared memory.
//
// One frame = one graph: table copy, counter reset, the bucket kernels on
// parallel branches. The graph is captured once per groom set and replayed;
// the host only rewrites the pinned table between frames (two slots,
// alternating, each guarded by an event).
//
// Results are bit-identical to hs_update on each groom alone: a strand's
// frame depends only on its own state and its groom's constants.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <set>
#include <vector>

#include "hs_api_internal.h"
#include "hs_batch.h"
#include "hs_step.cuh"

namespace hs {

namespace {

constexpr int kWarp = 32;

// Copies the groom's table entry into this warp's shared slot.
__device__ __forceinline__ void warp_copy(void* dst, const void* src, size_t bytes, int lane) {
  const uint32_t* s = static_cast<const uint32_t*>(src);
  uint32_t* d = static_cast<uint32_t*>(dst);
  for (size_t w = lane; w < bytes / 4; w += kWarp) d[w] = __ldg(s + w);
  __syncwarp();
}

// Largest block the autotuner tries: 8 warps.
constexpr int kMaxBatchBlock = 256;

// Register cap per (capacity, velocity storage). With the velocity slots in
// shared memory, about what the plain step needs for the same capacity, so
// that registers and shared memory allow a similar number of warps; with
// them in registers, no cap below the hardware's.
template <int CAP, bool VSMEM>
struct RegBudget {
  static constexpr int value =
      VSMEM ? (CAP >= 32 ? 200 : CAP >= 24 ? 168 : CAP >= 16 ? 128 : CAP >= 8 ? 104 : 72) : 255;
};

template <int CAP, bool REF, bool VSMEM>
__global__ void __launch_bounds__(kMaxBatchBlock) __maxnreg__((RegBudget<CAP, VSMEM>::value))
    k_step_batch(const BatchGroomDev* __restrict__ table, const BatchTile* __restrict__ tiles, uint32_t ntiles,
                 uint32_t* __restrict__ counter) {
  extern __shared__ float4 s_raw[];
  const int warps = blockDim.x / kWarp;
  const int warp = threadIdx.x / kWarp;
  const int lane = threadIdx.x % kWarp;
  BatchGroomDev* s_entry = reinterpret_cast<BatchGroomDev*>(s_raw);
  float4* s_vel = s_raw + (sizeof(BatchGroomDev) / sizeof(float4)) * warps;  // per-thread velocity rows (VSMEM)
  BatchGroomDev& e = s_entry[warp];
  uint32_t cur = 0xffffffffu;
  for (;;) {
    uint32_t t = 0;
    if (lane == 0) t = atomicAdd(counter, 1u);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= ntiles) break;
    const BatchTile tile = tiles[t];
    if (tile.groom != cur) {
      __syncwarp();
      warp_copy(&e, &table[tile.groom], sizeof(BatchGroomDev), lane);
      cur = tile.groom;
    }
    const uint32_t s = tile.strand0 + lane;
    const SphereSet S{e.fc.spheres, e.fc.r2, e.fc.adj, e.fc.nspheres};
    strand_frame<CAP, REF, VSMEM>(e.fc, S, e.view, s, s < e.view.nstrands, s_vel, threadIdx.x);
  }
}

template <int CAP, bool REF>
const void* batch_kernel(bool vsmem) {
  return vsmem ? reinterpret_cast<const void*>(&k_step_batch<CAP, REF, true>)
               : reinterpret_cast<const void*>(&k_step_batch<CAP, REF, false>);
}

const void* kernel_for(int cap, bool ref, bool vsmem) {
  switch (cap) {
    case 4: return ref ? batch_kernel<4, true>(vsmem) : batch_kernel<4, false>(vsmem);
    case 8: return ref ? batch_kernel<8, true>(vsmem) : batch_kernel<8, false>(vsmem);
    case 16: return ref ? batch_kernel<16, true>(vsmem) : batch_kernel<16, false>(vsmem);
    case 24: return ref ? batch_kernel<24, true>(vsmem) : batch_kernel<24, false>(vsmem);
    case 32: return ref ? batch_kernel<32, true>(vsmem) : batch_kernel<32, false>(vsmem);
    default: return nullptr;
  }
}

size_t smem_bytes(int cap, int warps, bool vsmem) {
  return sizeof(BatchGroomDev) * warps + (vsmem ? sizeof(float4) * (cap + 1) * warps * kWarp : 0);
}

cudaError_t launch_bucket(const BatchGroomDev* table, const Bucket& b, uint32_t* counter, cudaStream_t st) {
  const void* fn = kernel_for(b.cap, b.ref, b.vsmem);
  if (!fn) return cudaErrorInvalidValue;
  const size_t smem = smem_bytes(b.cap, b.warps_per_block, b.vsmem);
  uint32_t ntiles = b.ntiles;
  const BatchTile* tiles = b.d_tiles;
  void* args[] = {const_cast<BatchGroomDev**>(&table), const_cast<BatchTile**>(&tiles), &ntiles, &counter};
  return cudaLaunchKernel(fn, dim3(b.grid), dim3(b.warps_per_block * kWarp), args, smem, st);
}

}  // namespace

int batch_occupancy(int cap, bool ref, bool vsmem, int warps_per_block) {
  const void* fn = kernel_for(cap, ref, vsmem);
  if (!fn) return 0;
  const size_t smem = smem_bytes(cap, warps_per_block, vsmem);
  if (smem > 48 * 1024) cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  int blocks = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, warps_per_block * kWarp, smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return blocks;
}

BatchState::~BatchState() { release(); }

void BatchState::release() {
  for (int k = 0; k < 2; ++k) {
    if (exec[k]) cudaGraphExecDestroy(exec[k]);
    exec[k] = nullptr;
  }
  for (Bucket& b : buckets) cudaFree(b.d_tiles);
  buckets.clear();
  cudaFree(d_table);
  d_table = nullptr;
  cudaFree(d_counters);
  d_counters = nullptr;
  for (int k = 0; k < 2; ++k) {
    if (h_table[k]) cudaFreeHost(h_table[k]);
    h_table[k] = nullptr;
    if (done[k]) cudaEventDestroy(done[k]);
    done[k] = nullptr;
  }
  for (cudaStream_t s : aux) cudaStreamDestroy(s);
  aux.clear();
  for (cudaEvent_t e : fork_join) cudaEventDestroy(e);
  fork_join.clear();
  signature.clear();
  ngrooms = 0;
}

static std::vector<uint64_t> signature_of(hs_groom* const* grooms, uint32_t n) {
  std::vector<uint64_t> sig;
  sig.reserve(2 * n);
  for (uint32_t i = 0; i < n; ++i) {
    sig.push_back(reinterpret_cast<uint64_t>(grooms[i]));
    sig.push_back((static_cast<uint64_t>(grooms[i]->sim.mode) << 32) | grooms[i]->npoints);
  }
  return sig;
}

// Rebuilds buckets, tiles and device buffers for a new groom set.
static hs_status rebuild(hs_ctx* ctx, BatchState& B, hs_groom* const* grooms, uint32_t n) {
  cudaStreamSynchronize(ctx->stream);  // frames in flight still read the old table
  B.release();
  std::map<std::pair<int, bool>, std::vector<BatchTile>> by_key;
  for (uint32_t i = 0; i < n; ++i) {
    const hs_groom* g = grooms[i];
    const int cap = step_capacity(g->npoints);
    const bool ref = g->sim.mode == HS_MODE_REFERENCE;
    auto& v = by_key[{cap, ref}];
    for (uint32_t s0 = 0; s0 < g->nstrands; s0 += kWarp) v.push_back(BatchTile{i, s0});
  }
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
  cudaError_t e = cudaSuccess;
  for (auto& kv : by_key) {
    Bucket b;
    b.cap = kv.first.first;
    b.ref = kv.first.second;
    b.ntiles = static_cast<uint32_t>(kv.second.size());
    const TuneChoice tc = tuned_choice(ctx, b.cap, b.ref, b.ntiles);
    b.warps_per_block = tc.warps_per_block;
    b.vsmem = tc.vsmem;
    const int occ = std::max(1, batch_occupancy(b.cap, b.ref, b.vsmem, b.warps_per_block));
    const uint32_t resident = static_cast<uint32_t>(sms * occ * tc.waves);
    const uint32_t need = (b.ntiles + b.warps_per_block - 1) / b.warps_per_block;
    b.grid = std::max(1u, std::min(resident, need));
    e = cudaMalloc(&b.d_tiles, sizeof(BatchTile) * b.ntiles);
    if (e == cudaSuccess)
      e = cudaMemcpy(b.d_tiles, kv.second.data(), sizeof(BatchTile) * b.ntiles, cudaMemcpyHostToDevice);
    B.buckets.push_back(b);
    if (e != cudaSuccess) break;
  }
  if (e == cudaSuccess) e = cudaMalloc(&B.d_table, sizeof(BatchGroomDev) * n);
  if (e == cudaSuccess) e = cudaMalloc(&B.d_counters, sizeof(uint32_t) * std::max<size_t>(1, B.buckets.size()));
  for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
    e = cudaMallocHost(&B.h_table[k], sizeof(BatchGroomDev) * n);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&B.done[k], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventRecord(B.done[k], ctx->stream);
  }
  for (size_t j = 0; j < B.buckets.size() && e == cudaSuccess; ++j) {
    cudaStream_t s = nullptr;
    e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) B.aux.push_back(s);
  }
  for (size_t j = 0; j < B.buckets.size() + 1 && e == cudaSuccess; ++j) {
    cudaEvent_t ev = nullptr;
    e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e == cudaSuccess) B.fork_join.push_back(ev);
  }
  if (e != cudaSuccess) {
    B.release();
    return cuda_fail(e, "hs_update_many: set-up");
  }
  B.signature = signature_of(grooms, n);
  B.ngrooms = n;
  return HS_OK;
}

// Records one frame (table copy, counter reset, bucket kernels on parallel
// branches) on the context stream; used both for capture and direct runs.
static cudaError_t record_frame(hs_ctx* ctx, BatchState& B, int slot) {
  cudaStream_t st = ctx->stream;
  cudaError_t e = cudaMemcpyAsync(B.d_table, B.h_table[slot], sizeof(BatchGroomDev) * B.ngrooms,
                                  cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(B.d_counters, 0, sizeof(uint32_t) * B.buckets.size(), st);
  if (e == cudaSuccess && B.buckets.size() == 1) {
    return launch_bucket(B.d_table, B.buckets[0], B.d_counters, st);
  }
  if (e == cudaSuccess) e = cudaEventRecord(B.fork_join[0], st);
  for (size_t j = 0; j < B.buckets.size() && e == cudaSuccess; ++j) {
    e = cudaStreamWaitEvent(B.aux[j], B.fork_join[0], 0);
    if (e == cudaSuccess) e = launch_bucket(B.d_table, B.buckets[j], B.d_counters + j, B.aux[j]);
    if (e == cudaSuccess) e = cudaEventRecord(B.fork_join[j + 1], B.aux[j]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(st, B.fork_join[j + 1], 0);
  }
  return e;
}

hs_status batch_update(hs_ctx* ctx, hs_groom* const* grooms, uint32_t n, float dt, bool use_graph) {
  if (!ctx->batch) ctx->batch = new BatchState();
  BatchState& B = *ctx->batch;
  if (B.signature != signature_of(grooms, n)) {
    hs_status st = rebuild(ctx, B, grooms, n);
    if (st != HS_OK) return st;
  }
  const int slot = B.next;
  cudaError_t e = cudaEventSynchronize(B.done[slot]);
  if (e != cudaSuccess) return cuda_fail(e, "hs_update_many: wait for staging slot");
  for (uint32_t i = 0; i < n; ++i) {
    BatchGroomDev& d = B.h_table[slot][i];
    hs_status st = make_frame_const(grooms[i], dt, &d.fc);
    if (st != HS_OK) return st;
    d.view = view_of(grooms[i]);
  }
  if (use_graph) {
    if (!B.exec[slot]) {
      cudaGraph_t graph = nullptr;
      e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
      if (e == cudaSuccess) {
        cudaError_t er = record_frame(ctx, B, slot);
        e = cudaStreamEndCapture(ctx->stream, &graph);
        if (er != cudaSuccess) e = er;
      }
      if (e == cudaSuccess) e = cudaGraphInstantiate(&B.exec[slot], graph, 0);
      if (graph) cudaGraphDestroy(graph);
      if (e != cudaSuccess) {
        cudaGetLastError();
        return cuda_fail(e, "hs_update_many: graph capture");
      }
    }
    e = cudaGraphLaunch(B.exec[slot], ctx->stream);
  } else {
    e = record_frame(ctx, B, slot);
  }
  if (e == cudaSuccess) e = cudaEventRecord(B.done[slot], ctx->stream);
  if (e != cudaSuccess) return cuda_fail(e, "hs_update_many: launch");
  ctx->launches += B.buckets.size();
  B.next ^= 1;
  return HS_OK;
}

TuneKey tune_key(int cap, bool ref, uint32_t ntiles) {
  int lg = 0;
  while (lg < 31 && (1u << (lg + 1)) <= ntiles) ++lg;
  return TuneKey{cap, ref, lg};
}

TuneChoice tuned_choice(hs_ctx* ctx, int cap, bool ref, uint32_t ntiles) {
  if (ctx->tune) {
    auto it = ctx->tune->best.find(tune_key(cap, ref, ntiles));
    if (it != ctx->tune->best.end()) return it->second;
  }
  return TuneChoice{};  // 4 warps per block, one resident wave
}

// Times the candidate launch shapes of every bucket of the groom set on the
// live state, keeps the fastest in the context's cache, then restores the
// state the trials advanced.
static hs_status autotune(hs_ctx* ctx, hs_groom* const* grooms, uint32_t n, float dt, uint32_t* out_trials) {
  if (!ctx->tune) ctx->tune = new TuneCache();
  if (!ctx->batch) ctx->batch = new BatchState();
  BatchState& B = *ctx->batch;
  hs_status st = rebuild(ctx, B, grooms, n);
  if (st != HS_OK) return st;
  cudaStream_t s = ctx->stream;
  // Snapshot of every groom's state.
  std::vector<float4*> snap(2 * n, nullptr);
  cudaError_t e = cudaSuccess;
  for (uint32_t i = 0; i < n && e == cudaSuccess; ++i) {
    const size_t bytes = sizeof(float4) * static_cast<size_t>(grooms[i]->stride) * grooms[i]->npoints;
    e = cudaMalloc(&snap[2 * i], bytes);
    if (e == cudaSuccess) e = cudaMalloc(&snap[2 * i + 1], bytes);
    if (e == cudaSuccess) e = cudaMemcpyAsync(snap[2 * i], grooms[i]->d_pos, bytes, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(snap[2 * i + 1], grooms[i]->d_vel, bytes, cudaMemcpyDeviceToDevice, s);
  }
  for (uint32_t i = 0; i < n && e == cudaSuccess; ++i) {
    BatchGroomDev& d = B.h_table[0][i];
    st = make_frame_const(grooms[i], dt, &d.fc);
    if (st != HS_OK) break;
    d.view = view_of(grooms[i]);
  }
  if (e == cudaSuccess && st == HS_OK)
    e = cudaMemcpyAsync(B.d_table, B.h_table[0], sizeof(BatchGroomDev) * n, cudaMemcpyHostToDevice, s);
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  if (e == cudaSuccess) e = cudaEventCreate(&t0);
  if (e == cudaSuccess) e = cudaEventCreate(&t1);
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
  uint32_t trials = 0;
  for (size_t j = 0; j < B.buckets.size() && e == cudaSuccess && st == HS_OK; ++j) {
    Bucket& b = B.buckets[j];
    float best = 1e30f;
    TuneChoice best_c{};
    for (int vsm = 0; vsm < 2; ++vsm)
    for (int wpb : {1, 2, 4, 8}) {
      const int occ = batch_occupancy(b.cap, b.ref, vsm != 0, wpb);
      if (occ <= 0) continue;
      for (int waves : {1, 2, 4}) {
        const uint32_t need = (b.ntiles + wpb - 1) / wpb;
        const uint32_t grid = std::max(1u, std::min(static_cast<uint32_t>(sms * occ * waves), need));
        if (waves > 1 && grid == need) continue;  // same shape as a smaller wave count
        b.warps_per_block = wpb;
        b.vsmem = vsm != 0;
        b.grid = grid;
        float ms_sum = 0.0f;
        const int reps = 4;
        for (int r = 0; r < reps + 1 && e == cudaSuccess; ++r) {
          e = cudaMemsetAsync(B.d_counters + j, 0, sizeof(uint32_t), s);
          if (e == cudaSuccess) e = cudaEventRecord(t0, s);
          if (e == cudaSuccess) e = launch_bucket(B.d_table, b, B.d_counters + j, s);
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
          best_c = TuneChoice{wpb, waves, vsm != 0};
        }
      }
    }
    const TuneKey key = tune_key(b.cap, b.ref, b.ntiles);
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
  B.release();  // the next update rebuilds with the tuned shapes
  if (out_trials) *out_trials = trials;
  if (st != HS_OK) return st;
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
  return batch_update(ctx, grooms, n, dt, true);
}

HS_API hs_status hs_autotune(hs_ctx* ctx, hs_groom* const* grooms, uint32_t n, float dt, uint32_t* out_trials) {
  hs_status st = validate_set(ctx, grooms, n, "hs_autotune");
  if (st != HS_OK) return st;
  if (n == 0) {
    if (out_trials) *out_trials = 0;
    return HS_OK;
  }
  return autotune(ctx, grooms, n, dt, out_trials);
}

}  // extern "C"
