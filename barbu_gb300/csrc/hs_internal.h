// hs_internal.h -- launchers shared between the C-ABI layer and the kernels.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>

#include "hs_device.cuh"

namespace hs {

// Devices the per-device caches below track (a bit or a slot each).
constexpr int kMaxDevices = 64;

// Runs `set_up` once per device, on the current one: kernel attributes are
// kept per device by the runtime. Concurrent first calls may both run it
// (it only sets attributes, so that is harmless).
template <typename F>
inline void once_per_device(std::atomic<uint64_t>& done, F&& set_up) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    set_up();
    return;
  }
  const uint64_t bit = uint64_t{1} << dev;
  if (done.load(std::memory_order_acquire) & bit) return;
  set_up();
  done.fetch_or(bit, std::memory_order_acq_rel);
}

// An attribute of the current device, cached per device; `fallback` where
// the query fails.
int device_attribute(cudaDeviceAttr attr, int fallback);

// Capacities (points per strand) with a compiled step kernel; a groom of N
// points runs on the smallest capacity >= N.
int step_capacity(uint32_t npoints);

// Lane-group size of a frame (hs_lanes.cuh): the smallest power of two >=
// S for DFTL frames with one constraint iteration and 2 <= S <= 16, else 0
// (the frame has no lane-group form).
inline int lane_group(int mode, int substeps, int iterations) {
  if (mode != HS_MODE_DFTL || iterations != 1 || substeps < 2 || substeps > 16) return 0;
  int k = 2;
  while (k < substeps) k *= 2;
  return k;
}

// One frame of one groom. mapping (hs_mapping): a thread per strand, or a
// lane group per strand (lane_group must be nonzero), or AUTO: lane groups
// for grooms too small to fill the GPU a thread per strand.
cudaError_t launch_step(const GroomView& g, const FrameConst& fc, int mapping, cudaStream_t st);
// The mapping launch_step takes for `mapping` (HS_MAPPING_THREAD or _LANES).
int plain_mapping(const GroomView& g, const FrameConst& fc, int mapping);

// Strand expansion of hs_groom_init (src/fx/hair.cc:262-288) on the device.
struct InitArgs {
  const float* roots;    // nstrands * 3
  const float* normals;  // nstrands * 3
  const float* lengths;  // nstrands or null
  uint32_t length_rule;
  float max_length, length_jitter;
  uint32_t length_key;
  uint32_t strand_base;
};
cudaError_t launch_init(const GroomView& g, const InitArgs& a, float4* root_rest, cudaStream_t st);

// [point][strand] <-> strand-major float4 transposes; `order` gives the
// caller's index of each stored strand (strand-major rows are the caller's).
cudaError_t launch_to_strand_major(const float4* soa, float4* out, const uint32_t* order, uint32_t nstrands,
                                   uint32_t npoints, uint32_t stride, cudaStream_t st);
cudaError_t launch_from_strand_major(const float4* in, float4* soa, const uint32_t* order, uint32_t nstrands,
                                     uint32_t npoints, uint32_t stride, cudaStream_t st);
// [point][strand] float4 -> strand-major (x, y, z), 3 floats a point.
cudaError_t launch_to_strand_major_xyz(const float4* soa, float* out, const uint32_t* order, uint32_t nstrands,
                                       uint32_t npoints, uint32_t stride, cudaStream_t st);
// [point][stride] -> [point][nstrands] in the caller's order.
cudaError_t launch_to_point_major(const float4* soa, float4* out, const uint32_t* order, uint32_t nstrands,
                                  uint32_t npoints, uint32_t stride, cudaStream_t st);
// root_rest[s] = pos[0][s] (point 0 of every strand).
cudaError_t launch_copy_roots(const float4* soa, float4* root_rest, uint32_t nstrands, cudaStream_t st);

}  // namespace hs
