// hs_kernels.cu -- the per-groom kernels: step, init, layout transposes.
#include <algorithm>

#include "hs_internal.h"
#include "hs_lanes.cuh"
#include "hs_step.cuh"
#include "hs_stream.cuh"
#include "hs_tmem.cuh"

namespace hs {

namespace {

constexpr int kStepBlock = 64;

// AUTO mapping of the plain step: lane groups while they make at most this
// many warps per SM (32-strand tiles x lanes per strand) for strands of up
// to 16 points, proportionally more for longer strands.
constexpr int kLanesWarpsPerSm = 16;

// Overlapped frames (programmatic dependent launch). A groom's frames are
// back-to-back kernels on one stream; launched by launch_overlapped, a
// frame's blocks may become resident while the previous kernel's last
// blocks still run: each block signals at its start that the next kernel
// may be scheduled (frame_release), does the set-up that touches no
// simulation state (spheres into shared memory, tensor-memory allocation),
// then waits in frame_acquire until the previous kernel has completed and
// its writes are visible, before its first load of the state. Launched
// the ordinary way, both are no-ops.
__device__ __forceinline__ void frame_release() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void frame_acquire() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... Params, typename... Args>
cudaError_t launch_overlapped(void (*kernel)(Params...), unsigned grid, unsigned block, size_t smem, cudaStream_t st,
                              Args... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

// Copies the groom's spheres and overlap masks from the kernel parameters
// into shared memory (constant indices only, so the parameter block is
// never copied to local memory). Ends with a barrier.
__device__ __forceinline__ SphereSet stage_spheres(const FrameConst& fc, float4* s_c, float* s_r2, uint32_t* s_adj) {
#pragma unroll
  for (int k = 0; k < HS_MAX_SPHERES; ++k) {
    if (threadIdx.x == k && k < fc.nspheres) {
      s_c[k] = fc.spheres[k];
      s_r2[k] = fc.r2[k];
      s_adj[k] = fc.adj[k];
    }
  }
  __syncthreads();
  return SphereSet{s_c, s_r2, s_adj, fc.nspheres};
}

// Velocity slots of the plain step: registers up to 16 points per strand,
// shared memory above (keeps the register file for the positions).
template <int CAP>
struct PlainVsmem {
  static constexpr bool value = CAP > 16;
};

// FAST (every kernel below): the groom's FAST contract, a kernel of its own
// (no code of the other contract in it).
template <int CAP, bool REF, bool FAST>
__global__ void __launch_bounds__(kStepBlock) k_step(GroomView g, FrameConst fc) {
  extern __shared__ float4 s_vel[];  // per-thread velocity rows, when in shared memory
  __shared__ float4 s_c[HS_MAX_SPHERES];
  __shared__ float s_r2[HS_MAX_SPHERES];
  __shared__ uint32_t s_adj[HS_MAX_SPHERES];
  frame_release();
  const SphereSet S = stage_spheres(fc, s_c, s_r2, s_adj);
  frame_acquire();
  const uint32_t s = blockIdx.x * kStepBlock + threadIdx.x;
  if constexpr (REF) strand_frame_ref<CAP, PlainVsmem<CAP>::value>(fc, S, g, s, s < g.nstrands, s_vel, threadIdx.x);
  else strand_frame_regs_dftl<CAP, PlainVsmem<CAP>::value, FAST>(fc, S, g, s, s < g.nstrands, s_vel, threadIdx.x);
}

template <int CAP, bool REF, bool FAST>
cudaError_t launch_step_cap(const GroomView& g, const FrameConst& fc, cudaStream_t st) {
  const unsigned grid = (g.nstrands + kStepBlock - 1) / kStepBlock;
  const size_t smem = PlainVsmem<CAP>::value ? vslot_bytes<CAP>(kStepBlock) : 0;
  return launch_overlapped(k_step<CAP, REF, FAST>, grid, kStepBlock, smem, st, g, fc);
}

bool fast_frame(const FrameConst& fc) { return fc.mode == HS_MODE_DFTL && fc.contract == HS_CONTRACT_FAST; }

template <int CAP>
cudaError_t launch_step_mode(const GroomView& g, const FrameConst& fc, cudaStream_t st) {
  if (fc.mode == HS_MODE_REFERENCE) return launch_step_cap<CAP, true, false>(g, fc, st);
  return fast_frame(fc) ? launch_step_cap<CAP, false, true>(g, fc, st) : launch_step_cap<CAP, false, false>(g, fc, st);
}

// Streaming form (hs_stream.cuh): state in shared memory, one runtime loop
// per pass, any point count. One warp per block: the shared state is what
// bounds residency, and single-warp blocks pack it tightest.
constexpr int kStreamBlock = 32;

template <bool REF, bool FAST>
__global__ void __launch_bounds__(kStreamBlock) k_step_stream(GroomView g, FrameConst fc) {
  extern __shared__ float4 s_state[];  // X then V, each [npoints][kStreamBlock]
  __shared__ float4 s_c[HS_MAX_SPHERES];
  __shared__ float s_r2[HS_MAX_SPHERES];
  __shared__ uint32_t s_adj[HS_MAX_SPHERES];
  frame_release();
  const SphereSet S = stage_spheres(fc, s_c, s_r2, s_adj);
  frame_acquire();
  const uint32_t s = blockIdx.x * kStreamBlock + threadIdx.x;
  float4* Xs = s_state + threadIdx.x;
  float4* Vs = s_state + g.npoints * kStreamBlock + threadIdx.x;
  strand_frame_stream<REF, XShared4, VShared, kCachedSpheres, false, false, FAST>(
      fc, S, g, s, s < g.nstrands, XShared4{Xs, kStreamBlock}, VShared{Vs, kStreamBlock});
}

// Streaming form with the velocities in tensor memory (hs_tmem.cuh): a
// block is 4 warps, one per TMEM lane quadrant; shared memory holds the
// positions only, 12 bytes a point (the rest lengths ride in the w of the
// TMEM velocity slots).
constexpr int kTmemBlock = 128;

// CACHED: pushes from the register sphere cache (hs_stream.cuh, push_seg),
// for grooms among many spheres.
template <bool REF, bool CACHED, bool FAST>
__global__ void __launch_bounds__(kTmemBlock) k_step_stream_tmem(GroomView g, FrameConst fc) {
  extern __shared__ float4 s_pos[];  // positions, compact: float2 (x, y) then float z, each [npoints][kTmemBlock]
  __shared__ float4 s_c[HS_MAX_SPHERES];
  __shared__ float s_r2[HS_MAX_SPHERES];
  __shared__ uint32_t s_adj[HS_MAX_SPHERES];
  __shared__ uint32_t s_taddr;
  frame_release();
  const SphereSet S = stage_spheres(fc, s_c, s_r2, s_adj);
  const uint32_t warp = threadIdx.x / 32;
  const uint32_t ncols = tmem::cols_for(g.npoints);
  if (warp == 0) {
    tmem::alloc(&s_taddr, ncols);
    tmem::relinquish();
  }
  tmem::fence_before_sync();
  __syncthreads();
  tmem::fence_after_sync();
  frame_acquire();
  const uint32_t base = s_taddr;
  const VTmem V{base + ((warp * 32u) << 16)};
  const uint32_t s = blockIdx.x * kTmemBlock + threadIdx.x;
  float2* xy = reinterpret_cast<float2*>(s_pos);
  float* z = reinterpret_cast<float*>(xy + g.npoints * kTmemBlock);
  const XShared3 X{xy + threadIdx.x, z + threadIdx.x, kTmemBlock};
  strand_frame_stream<REF, XShared3, VTmem, 8, true, CACHED, FAST>(fc, S, g, s, s < g.nstrands, X, V);
  tmem::fence_before_sync();
  __syncthreads();
  tmem::fence_after_sync();
  if (warp == 0) tmem::dealloc(base, ncols);
}

// Blocks of the tensor-memory step resident on one SM are bounded by its
// 512 TMEM columns as well as by shared memory: the dynamic shared memory
// is padded so that shared memory is the tighter bound, and no block waits
// in its allocation.
size_t tmem_step_smem(uint32_t npoints) {
  const int sm_smem = device_attribute(cudaDevAttrMaxSharedMemoryPerMultiprocessor, 228 * 1024);
  const size_t need = (sizeof(float2) + sizeof(float)) * npoints * kTmemBlock;
  const size_t blocks_by_tmem = 512 / tmem::cols_for(npoints);
  const size_t per_block = static_cast<size_t>(sm_smem) / blocks_by_tmem + 1;  // one more block would not fit
  const size_t fixed = 1024 + 3 * 1024;  // reserved + static (spheres, masks, TMEM slot), rounded up
  return std::max(need, per_block > fixed ? per_block - fixed : need);
}

cudaError_t launch_step_stream_tmem(const GroomView& g, const FrameConst& fc, cudaStream_t st) {
  const unsigned grid = (g.nstrands + kTmemBlock - 1) / kTmemBlock;
  const size_t smem = tmem_step_smem(g.npoints);
  static std::atomic<uint64_t> optin{0};
  once_per_device(optin, [] {
    const int bytes = 200 * 1024;
    cudaFuncSetAttribute(k_step_stream_tmem<true, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(k_step_stream_tmem<false, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(k_step_stream_tmem<false, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(k_step_stream_tmem<false, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(k_step_stream_tmem<false, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  });
  // Grooms among many spheres push at most points: the register-cached
  // push pays there (skinned groom, 32 spheres: 5.53 -> 4.60 ms a frame)
  // and costs elsewhere in instruction-cache space (large groom, 16
  // spheres: 0.364 -> 0.462 ms).
  const bool cached = fc.nspheres > 16;
  const bool fast = fast_frame(fc);
  if (fc.mode == HS_MODE_REFERENCE) {
    return launch_overlapped(k_step_stream_tmem<true, false, false>, grid, kTmemBlock, smem, st, g, fc);
  } else if (cached) {
    if (fast) return launch_overlapped(k_step_stream_tmem<false, true, true>, grid, kTmemBlock, smem, st, g, fc);
    return launch_overlapped(k_step_stream_tmem<false, true, false>, grid, kTmemBlock, smem, st, g, fc);
  } else {
    if (fast) return launch_overlapped(k_step_stream_tmem<false, false, true>, grid, kTmemBlock, smem, st, g, fc);
    return launch_overlapped(k_step_stream_tmem<false, false, false>, grid, kTmemBlock, smem, st, g, fc);
  }
}

// Lane groups (hs_lanes.cuh): a block of K warps per 32-strand tile, the
// tile's starting state in shared memory ([npoints][32] positions, then
// velocities). Register cap 128 (16 warps a SM). CACHED: as the
// tensor-memory step (grooms among many spheres).
template <int K, bool CACHED, bool FAST>
__global__ void __launch_bounds__(K * 32, 16 / K) k_step_lanes(GroomView g, FrameConst fc) {
  extern __shared__ float4 s_state[];
  __shared__ float4 s_c[HS_MAX_SPHERES];
  __shared__ float s_r2[HS_MAX_SPHERES];
  __shared__ uint32_t s_adj[HS_MAX_SPHERES];
  __shared__ TileStats s_ts[32];
  frame_release();
  const SphereSet S = stage_spheres(fc, s_c, s_r2, s_adj);
  frame_acquire();
  tile_frame_lanes<K, 8, CACHED, FAST>(fc, S, g, blockIdx.x, s_state, s_state + g.npoints * 32, s_ts);
}

template <int K>
cudaError_t launch_step_lanes_k(const GroomView& g, const FrameConst& fc, cudaStream_t st) {
  const unsigned grid = (g.nstrands + 31) / 32;
  const size_t smem = 2 * sizeof(float4) * 32 * g.npoints;
  static std::atomic<uint64_t> optin{0};
  once_per_device(optin, [] {
    const int bytes = 2 * static_cast<int>(sizeof(float4)) * 32 * HS_MAX_POINTS_PER_STRAND;
    cudaFuncSetAttribute(k_step_lanes<K, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(k_step_lanes<K, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(k_step_lanes<K, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(k_step_lanes<K, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  });
  const bool cached = fc.nspheres > 16, fast = fast_frame(fc);
  const unsigned block = K * 32;
  if (cached && fast) return launch_overlapped(k_step_lanes<K, true, true>, grid, block, smem, st, g, fc);
  if (cached) return launch_overlapped(k_step_lanes<K, true, false>, grid, block, smem, st, g, fc);
  if (fast) return launch_overlapped(k_step_lanes<K, false, true>, grid, block, smem, st, g, fc);
  return launch_overlapped(k_step_lanes<K, false, false>, grid, block, smem, st, g, fc);
}

cudaError_t launch_step_lanes(const GroomView& g, const FrameConst& fc, cudaStream_t st) {
  switch (lane_group(fc.mode, fc.substeps, fc.iterations)) {
    case 2: return launch_step_lanes_k<2>(g, fc, st);
    case 4: return launch_step_lanes_k<4>(g, fc, st);
    case 8: return launch_step_lanes_k<8>(g, fc, st);
    case 16: return launch_step_lanes_k<16>(g, fc, st);
    default: return cudaErrorNotSupported;
  }
}

// Point counts the plain step runs with its velocities in tensor memory
// (all that take the streaming form).
bool plain_uses_tmem(const GroomView& g) { return g.npoints > 8 && g.npoints <= HS_MAX_POINTS_PER_STRAND; }

cudaError_t launch_step_stream(const GroomView& g, const FrameConst& fc, cudaStream_t st) {
  if (plain_uses_tmem(g)) return launch_step_stream_tmem(g, fc, st);
  const unsigned grid = (g.nstrands + kStreamBlock - 1) / kStreamBlock;
  const size_t smem = 2 * sizeof(float4) * g.npoints * kStreamBlock;
  // 64 points x 32 threads x 2 arrays = 64 KB: above the default 48 KB.
  static std::atomic<uint64_t> optin{0};
  once_per_device(optin, [] {
    const int bytes = 2 * static_cast<int>(sizeof(float4)) * HS_MAX_POINTS_PER_STRAND * kStreamBlock;
    cudaFuncSetAttribute(k_step_stream<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(k_step_stream<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    cudaFuncSetAttribute(k_step_stream<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  });
  if (fc.mode == HS_MODE_REFERENCE) {
    return launch_overlapped(k_step_stream<true, false>, grid, kStreamBlock, smem, st, g, fc);
  } else if (fast_frame(fc)) {
    return launch_overlapped(k_step_stream<false, true>, grid, kStreamBlock, smem, st, g, fc);
  } else {
    return launch_overlapped(k_step_stream<false, false>, grid, kStreamBlock, smem, st, g, fc);
  }
}

}  // namespace

namespace {

// Hair::init_simulation (src/fx/hair.cc:262-288), one thread per strand.
__global__ void k_init(GroomView g, InitArgs a, float4* root_rest) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= g.nstrands) return;
  const V3 r = v3(a.roots[3 * s], a.roots[3 * s + 1], a.roots[3 * s + 2]);
  const V3 nrm = v3(a.normals[3 * s], a.normals[3 * s + 1], a.normals[3 * s + 2]);
  const float u = hash_u01(a.length_key, a.strand_base + g.order[s]);  // the caller's index
  // rv = 1 + jitter * (1 - 2u)   (src/fx/hair.cc:268-270)
  const float rv = __fadd_rn(1.0f, __fmul_rn(a.length_jitter, __fsub_rn(1.0f, __fmul_rn(2.0f, u))));
  const int n = static_cast<int>(g.npoints);
  if (a.length_rule == HS_LENGTH_REFERENCE) {
    const float scale_offset = __fdiv_rn(a.max_length, static_cast<float>(n));
    float last = 0.0f;
    for (int i = 0; i < n; ++i) {
      const float offset = __fmul_rn(__fmul_rn(static_cast<float>(i), scale_offset), rv);
      const V3 q = add(r, mul(offset, nrm));
      g.pos[static_cast<size_t>(i) * g.stride + s] = make_float4(q.x, q.y, q.z, __fsub_rn(offset, last));
      g.vel[static_cast<size_t>(i) * g.stride + s] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      last = offset;
    }
  } else {
    const float L = a.lengths ? a.lengths[s] : __fmul_rn(a.max_length, rv);
    const float seg = __fdiv_rn(L, static_cast<float>(n - 1));
    for (int i = 0; i < n; ++i) {
      const float offset = __fmul_rn(static_cast<float>(i), seg);
      const V3 q = add(r, mul(offset, nrm));
      g.pos[static_cast<size_t>(i) * g.stride + s] = make_float4(q.x, q.y, q.z, i == 0 ? 0.0f : seg);
      g.vel[static_cast<size_t>(i) * g.stride + s] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
  }
  if (root_rest) root_rest[s] = make_float4(r.x, r.y, r.z, 0.0f);
}

// Transposes between strand-major (s*N + i) and [point][strand] (i*stride + s).
// A block moves 32 strands: their N float4 are contiguous in strand-major
// order, and each point row of 32 strands is 512 contiguous bytes.
// `order` (the caller's index of each stored strand) places stored strand s
// at strand-major row order[s]: the outside sees the caller's order.
constexpr int kTileStrands = 32;

// Tile rows are padded by one float4 so that the 32 strands of a point
// (one row each) fall in different shared-memory banks.
__global__ void k_to_strand_major(const float4* __restrict__ soa, float4* __restrict__ out,
                                  const uint32_t* __restrict__ order, uint32_t nstrands, uint32_t npoints,
                                  uint32_t stride) {
  __shared__ float4 tile[kTileStrands * (HS_MAX_POINTS_PER_STRAND + 1)];
  const uint32_t s0 = blockIdx.x * kTileStrands;
  const uint32_t ns = min(static_cast<uint32_t>(kTileStrands), nstrands - s0);
  const uint32_t total = ns * npoints;
  const uint32_t row = npoints + 1;
  for (uint32_t t = threadIdx.x; t < kTileStrands * npoints; t += blockDim.x) {
    const uint32_t i = t / kTileStrands, sl = t % kTileStrands;
    if (sl < ns) tile[sl * row + i] = soa[static_cast<size_t>(i) * stride + s0 + sl];
  }
  __syncthreads();
  for (uint32_t t = threadIdx.x; t < total; t += blockDim.x) {
    const uint32_t sl = t / npoints, i = t % npoints;
    out[static_cast<size_t>(order[s0 + sl]) * npoints + i] = tile[sl * row + i];
  }
}

// The same transpose to (x, y, z) only, 12 bytes a point. Block 32 x 8:
// a warp writes 32 consecutive points of one strand (384 contiguous bytes
// in three 4-byte stores a thread), with no division in the index math.
__global__ void k_to_strand_major_xyz(const float4* __restrict__ soa, float* __restrict__ out,
                                      const uint32_t* __restrict__ order, uint32_t nstrands, uint32_t npoints,
                                      uint32_t stride) {
  __shared__ float4 tile[kTileStrands * (HS_MAX_POINTS_PER_STRAND + 1)];
  const uint32_t s0 = blockIdx.x * kTileStrands;
  const uint32_t ns = min(static_cast<uint32_t>(kTileStrands), nstrands - s0);
  const uint32_t row = npoints + 1;
  const uint32_t sl_in = threadIdx.x;  // strand of the tile, loads
  for (uint32_t i = threadIdx.y; i < npoints; i += blockDim.y)
    if (sl_in < ns) tile[sl_in * row + i] = soa[static_cast<size_t>(i) * stride + s0 + sl_in];
  __syncthreads();
  for (uint32_t sl = threadIdx.y; sl < ns; sl += blockDim.y) {
    float* o = out + static_cast<size_t>(order[s0 + sl]) * 3 * npoints;
    for (uint32_t i = threadIdx.x; i < npoints; i += blockDim.x) {
      const float4 p = tile[sl * row + i];
      o[3 * i] = p.x;
      o[3 * i + 1] = p.y;
      o[3 * i + 2] = p.z;
    }
  }
}

__global__ void k_from_strand_major(const float4* __restrict__ in, float4* __restrict__ soa,
                                    const uint32_t* __restrict__ order, uint32_t nstrands, uint32_t npoints,
                                    uint32_t stride) {
  __shared__ float4 tile[kTileStrands * (HS_MAX_POINTS_PER_STRAND + 1)];
  const uint32_t s0 = blockIdx.x * kTileStrands;
  const uint32_t ns = min(static_cast<uint32_t>(kTileStrands), nstrands - s0);
  const uint32_t total = ns * npoints;
  const uint32_t row = npoints + 1;
  for (uint32_t t = threadIdx.x; t < total; t += blockDim.x) {
    const uint32_t sl = t / npoints, i = t % npoints;
    tile[sl * row + i] = in[static_cast<size_t>(order[s0 + sl]) * npoints + i];
  }
  __syncthreads();
  for (uint32_t t = threadIdx.x; t < kTileStrands * npoints; t += blockDim.x) {
    const uint32_t i = t / kTileStrands, sl = t % kTileStrands;
    if (sl < ns) soa[static_cast<size_t>(i) * stride + s0 + sl] = tile[sl * row + i];
  }
}

// [point][stride] -> [point][nstrands] in the caller's strand order.
__global__ void k_to_point_major(const float4* __restrict__ soa, float4* __restrict__ out,
                                 const uint32_t* __restrict__ order, uint32_t nstrands, uint32_t npoints,
                                 uint32_t stride) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nstrands) return;
  const uint32_t c = order[s];
  for (uint32_t i = 0; i < npoints; ++i)
    out[static_cast<size_t>(i) * nstrands + c] = soa[static_cast<size_t>(i) * stride + s];
}

__global__ void k_copy_roots(const float4* __restrict__ soa, float4* __restrict__ root_rest, uint32_t nstrands) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < nstrands) {
    const float4 p = soa[s];
    root_rest[s] = make_float4(p.x, p.y, p.z, 0.0f);
  }
}

}  // namespace

int step_capacity(uint32_t npoints) {
  if (npoints < HS_MIN_POINTS_PER_STRAND) return 0;
  if (npoints <= 4) return 4;
  if (npoints <= 8) return 8;
  if (npoints <= 16) return 16;
  if (npoints <= 24) return 24;
  if (npoints <= 32) return 32;
  if (npoints <= HS_MAX_POINTS_PER_STRAND) return 64;
  return 0;
}

int plain_mapping(const GroomView& g, const FrameConst& fc, int mapping) {
  const int K = lane_group(fc.mode, fc.substeps, fc.iterations);
  if (mapping == HS_MAPPING_LANES || K == 0) return mapping == HS_MAPPING_LANES ? HS_MAPPING_LANES : HS_MAPPING_THREAD;
  if (mapping == HS_MAPPING_THREAD) return HS_MAPPING_THREAD;
  // AUTO: lane groups while a thread per strand leaves the SMs' schedulers
  // short of warps and the lane groups do not crowd them. Measured on
  // 1,024-65,536 strands x 16-64 points, 4 and 8 substeps: lane groups are
  // faster up to about 16 of their warps per SM at 16 points, about N at
  // N points (a longer chain gains more from the wavefront), slower beyond,
  // where the idle lanes of the wavefront's head and tail and its shuffles
  // cost more than the shorter chain saves.
  const int sms = device_attribute(cudaDevAttrMultiProcessorCount, 152);
  const uint64_t warps = static_cast<uint64_t>((g.nstrands + 31) / 32) * static_cast<uint64_t>(K);
  const uint64_t per_sm = static_cast<uint64_t>(kLanesWarpsPerSm) * std::max<uint32_t>(16u, g.npoints) / 16u;
  return warps <= per_sm * static_cast<uint64_t>(sms) ? HS_MAPPING_LANES : HS_MAPPING_THREAD;
}

cudaError_t launch_step(const GroomView& g, const FrameConst& fc, int mapping, cudaStream_t st) {
  if (g.nstrands == 0) return cudaSuccess;
  if (plain_mapping(g, fc, mapping) == HS_MAPPING_LANES) return launch_step_lanes(g, fc, st);
  // Short strands: everything in registers. Longer: the streaming form.
  if (g.npoints > 8) return launch_step_stream(g, fc, st);
  switch (step_capacity(g.npoints)) {
    case 4: return launch_step_mode<4>(g, fc, st);
    case 8: return launch_step_mode<8>(g, fc, st);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_init(const GroomView& g, const InitArgs& a, float4* root_rest, cudaStream_t st) {
  if (g.nstrands == 0) return cudaSuccess;
  k_init<<<(g.nstrands + 127) / 128, 128, 0, st>>>(g, a, root_rest);
  return cudaGetLastError();
}

cudaError_t launch_to_strand_major(const float4* soa, float4* out, const uint32_t* order, uint32_t nstrands,
                                   uint32_t npoints, uint32_t stride, cudaStream_t st) {
  if (nstrands == 0) return cudaSuccess;
  k_to_strand_major<<<(nstrands + kTileStrands - 1) / kTileStrands, 256, 0, st>>>(soa, out, order, nstrands,
                                                                                    npoints, stride);
  return cudaGetLastError();
}

cudaError_t launch_to_strand_major_xyz(const float4* soa, float* out, const uint32_t* order, uint32_t nstrands,
                                       uint32_t npoints, uint32_t stride, cudaStream_t st) {
  if (nstrands == 0) return cudaSuccess;
  k_to_strand_major_xyz<<<(nstrands + kTileStrands - 1) / kTileStrands, dim3(kTileStrands, 8), 0, st>>>(
      soa, out, order, nstrands, npoints, stride);
  return cudaGetLastError();
}

cudaError_t launch_from_strand_major(const float4* in, float4* soa, const uint32_t* order, uint32_t nstrands,
                                     uint32_t npoints, uint32_t stride, cudaStream_t st) {
  if (nstrands == 0) return cudaSuccess;
  k_from_strand_major<<<(nstrands + kTileStrands - 1) / kTileStrands, 256, 0, st>>>(in, soa, order, nstrands,
                                                                                      npoints, stride);
  return cudaGetLastError();
}

cudaError_t launch_to_point_major(const float4* soa, float4* out, const uint32_t* order, uint32_t nstrands,
                                  uint32_t npoints, uint32_t stride, cudaStream_t st) {
  if (nstrands == 0) return cudaSuccess;
  k_to_point_major<<<(nstrands + 255) / 256, 256, 0, st>>>(soa, out, order, nstrands, npoints, stride);
  return cudaGetLastError();
}

cudaError_t launch_copy_roots(const float4* soa, float4* root_rest, uint32_t nstrands, cudaStream_t st) {
  if (nstrands == 0) return cudaSuccess;
  k_copy_roots<<<(nstrands + 255) / 256, 256, 0, st>>>(soa, root_rest, nstrands);
  return cudaGetLastError();
}

// A few attributes per device are asked for; each slot caches one as a
// single 64-bit word (attribute + 1 in the high half, 0 = empty; the value
// in the low half), so that a reader sees a pair or nothing.
int device_attribute(cudaDeviceAttr attr, int fallback) {
  static std::atomic<uint64_t> cache[kMaxDevices][4];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return fallback;
  }
  const uint64_t key = static_cast<uint64_t>(static_cast<uint32_t>(attr) + 1u) << 32;
  for (std::atomic<uint64_t>& slot : cache[dev]) {
    uint64_t w = slot.load(std::memory_order_acquire);
    if ((w & ~uint64_t{0xffffffffu}) == key) return static_cast<int>(static_cast<uint32_t>(w));
    if (w != 0) continue;
    int v = 0;
    if (cudaDeviceGetAttribute(&v, attr, dev) != cudaSuccess) {
      cudaGetLastError();
      return fallback;
    }
    const uint64_t entry = key | static_cast<uint32_t>(v);
    if (slot.compare_exchange_strong(w, entry, std::memory_order_acq_rel) || w == entry) return v;
  }
  int v = 0;
  if (cudaDeviceGetAttribute(&v, attr, dev) != cudaSuccess) {
    cudaGetLastError();
    return fallback;
  }
  return v;
}

}  // namespace hs
