// hs_internal.h -- launchers shared between the C-ABI layer and the kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "hs_device.cuh"

namespace hs {

// Capacities (points per strand) with a compiled step kernel; a groom of N
// points runs on the smallest capacity >= N.
int step_capacity(uint32_t npoints);

// One frame of one groom, thread per strand.
cudaError_t launch_step(const GroomView& g, const FrameConst& fc, cudaStream_t st);

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

// [point][strand] <-> strand-major float4 transposes.
cudaError_t launch_to_strand_major(const float4* soa, float4* out, uint32_t nstrands, uint32_t npoints,
                                   uint32_t stride, cudaStream_t st);
cudaError_t launch_from_strand_major(const float4* in, float4* soa, uint32_t nstrands, uint32_t npoints,
                                     uint32_t stride, cudaStream_t st);
// root_rest[s] = pos[0][s] (point 0 of every strand).
cudaError_t launch_copy_roots(const float4* soa, float4* root_rest, uint32_t nstrands, cudaStream_t st);

}  // namespace hs
