// hs_api_internal.h -- host-side objects behind the C-ABI handles.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <deque>
#include <set>
#include <vector>

#include "hairsim.h"
#include "hs_device.cuh"

namespace hs {
struct BatchState;  // batched update machinery (hs_batch.cu)
struct TuneCache;   // autotuned launch shapes (hs_batch.cu)
}

// A context: one device, one stream, the grooms created on it.
struct hs_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t copy_stream = nullptr;  // asynchronous readbacks, created on first use
  std::set<hs_groom*> grooms;
  uint64_t launches = 0;         // kernels launched (each graph node counts)
  hs::BatchState* batch = nullptr;
  hs::TuneCache* tune = nullptr;
  // Asynchronous readbacks: an event on the copy stream after each one's
  // copy, oldest first (hs_readback_drain), and spare events.
  std::deque<cudaEvent_t> pending;
  std::vector<cudaEvent_t> spare_events;
  // Staging of hs_readback_many_async: two buffers taken in turn, so that
  // the snapshot of one call overlaps the copy of the previous one.
  float* d_many[2] = {nullptr, nullptr};
  size_t many_cap[2] = {0, 0};       // floats
  cudaEvent_t many_ready[2] = {nullptr, nullptr};
  cudaEvent_t many_free[2] = {nullptr, nullptr};
  int many_next = 0;
};

// A groom: the device slabs of one set of strands and its per-frame inputs.
struct hs_groom {
  hs_ctx* ctx = nullptr;
  uint32_t nstrands = 0, npoints = 0, stride = 0;
  uint64_t seed = 0;
  uint32_t strand_base = 0;  // global index of strand 0 (split grooms)
  hs_sim_params sim{};
  char* d_mem = nullptr;            // one block holding the three arrays below
  bool pool_owned = false;          // d_mem belongs to a server's slab pool
  float4* d_pos = nullptr;          // [npoints][stride] (x, y, z, restlength)
  float4* d_vel = nullptr;          // [npoints][stride] (x, y, z, 0)
  float4* d_root_rest = nullptr;    // [stride] rest roots (RIGID, SKINNED)
  float4* d_stats = nullptr;        // [2 * stride / 32] frame statistics per tile (TileStats)
  uint32_t* d_order = nullptr;      // [stride] the caller's index of each stored strand
  std::vector<uint32_t> order;      // the same on the host (identity past nstrands)
  std::vector<uint32_t> inv;        // [nstrands] stored index of each caller strand
  bool stats_valid = false;         // a frame has written d_stats
  uint32_t mapping = HS_MAPPING_AUTO;  // hs_mapping of hs_update
  float4* d_root_target = nullptr;  // [stride] explicit targets, allocated on first hs_set_roots
  // Strand-major readback staging, two buffers allocated on first use and
  // taken in turn by asynchronous readbacks (the blocking readback uses the
  // first), so that a snapshot overlaps the previous readback's copy.
  float4* d_out[2] = {nullptr, nullptr};
  cudaEvent_t out_ready[2] = {nullptr, nullptr};  // d_out[i] written (context stream)
  cudaEvent_t out_free[2] = {nullptr, nullptr};   // d_out[i] copied to host (copy stream): it may be rewritten
  int out_next = 0;                               // the buffer of the next asynchronous readback
  uint4* d_skin = nullptr;          // [stride] bone influences (SKINNED), allocated on first hs_set_skin
  uint32_t skin_max_bone = 0;       // largest bone index the influences use
  uint32_t nbones = 0;              // bones in the current palette
  float4 bone_real[HS_MAX_BONES] = {};
  float4 bone_dual[HS_MAX_BONES] = {};
  // Tessellation stream (hs_tess.cu): static inputs and the output buffer.
  uint32_t* d_tess_faces = nullptr;  // 3 strand indices per triangle
  float4* d_tess_tangents = nullptr; // [npoints][stride]
  float* d_tess_random = nullptr;    // HS_TESS_RANDOM_SIZE floats
  uint32_t tess_nfaces = 0;
  float4* d_tess = nullptr;          // 2 vertices per line segment
  uint64_t tess_cap = 0, tess_count = 0;
  size_t state_bytes = 0;
  std::vector<float4> spheres;
  uint32_t adj[HS_MAX_SPHERES] = {0};  // overlap masks of `spheres` (culling)
  std::vector<float4> h_targets;
  float wind[3] = {0.0f, 0.0f, 0.0f};
  float m[16] = {0};
};

namespace hs {

// Makes `device` current for the duration of a call and restores the
// caller's device afterwards.
struct DeviceScope {
  int prev = -1;
  cudaError_t err = cudaSuccess;
  explicit DeviceScope(int device) {
    err = cudaGetDevice(&prev);
    if (err == cudaSuccess && prev != device) err = cudaSetDevice(device);
  }
  ~DeviceScope() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
  DeviceScope(const DeviceScope&) = delete;
  DeviceScope& operator=(const DeviceScope&) = delete;
};

hs_status fail(hs_status st, const char* fmt, ...);
hs_status cuda_fail(cudaError_t e, const char* what);
hs_status validate_sim(const hs_sim_params* p);
GroomView view_of(const hs_groom* g);
hs_status make_frame_const(const hs_groom* g, float dt, FrameConst* out);
void free_groom(hs_groom* g);

// Groom construction in pieces, for callers that own the device memory.
// Bytes of a groom's state block: positions, velocities, rest roots, tile
// statistics, strand order.
size_t groom_state_bytes(uint32_t nstrands, uint32_t npoints);
// The order a groom stores its strands in: order[j] = the caller's index of
// stored strand j, `stride` entries (identity past n). keep: the caller's
// order; else a Z-order (Morton) curve over the roots' bounding box, so
// that the 32 strands of a warp are spatial neighbours (sphere culling and
// the instruction stream of a warp are per warp).
void strand_order(const float* roots, size_t root_stride_floats, uint32_t n, uint32_t stride, bool keep,
                  std::vector<uint32_t>* order, std::vector<uint32_t>* inv);
// Host rows permuted into the groom's stored order: out[j] = in[order[j]].
template <typename T>
void to_stored(const hs_groom* g, const T* in, size_t width, std::vector<T>* out) {
  out->resize(static_cast<size_t>(g->nstrands) * width);
  for (uint32_t j = 0; j < g->nstrands; ++j)
    for (size_t k = 0; k < width; ++k) (*out)[j * width + k] = in[static_cast<size_t>(g->order[j]) * width + k];
}
// Validates and creates a groom without device memory.
hs_status make_groom_shell(hs_ctx* ctx, uint32_t nstrands, uint32_t npoints, uint64_t seed,
                           const hs_sim_params* sim, hs_groom** out);
// Points the groom's arrays into `mem` (groom_state_bytes long, 256-aligned).
void place_groom(hs_groom* g, char* mem, bool pool_owned);
// Expands strands from device-resident roots/normals (lengths optional).
cudaError_t init_groom_on_device(hs_groom* g, const float* d_roots, const float* d_normals, const float* d_lengths,
                                 const hs_strand_params* strand, cudaStream_t st);
hs_status validate_strand(const hs_strand_params* strand, const float* roots, const float* normals,
                          const float* lengths, uint32_t nstrands);
hs_status set_spheres(hs_groom* g, const float* xyzr, uint32_t n);
// Packs per-strand bone influences as the step kernel reads them (4 bone
// bytes, 3 weights as float bits), `stride` entries; validates them.
hs_status pack_skin(const uint8_t* bones, const float* weights, uint32_t nstrands, uint32_t stride,
                    std::vector<uint4>* out, uint32_t* max_bone, const char* what);
// Rigid column-major 4x4 -> dual quaternion (real xyzw, dual xyzw).
void matrix_to_dual_quat(const float* m, float* dq);
// Releases what hs_batch.cu attached to the context.
void destroy_ctx_extensions(hs_ctx* ctx);

}  // namespace hs

// Every entry point that touches the device runs on its context's device,
// whichever device the calling thread has selected.
#define HS_ON_DEVICE(ctx, what)                           \
  ::hs::DeviceScope hs_device_scope_((ctx)->device);      \
  if (hs_device_scope_.err != cudaSuccess) return ::hs::cuda_fail(hs_device_scope_.err, what)
