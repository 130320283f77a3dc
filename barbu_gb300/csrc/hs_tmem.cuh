// hs_tmem.cuh -- strand velocities in tensor memory (TMEM).
//
// The streaming step keeps a strand's positions and velocities on chip for
// the whole frame; shared memory alone holds 6 warps of 32-point strands
// per SM, too few to hide the step's dependent arithmetic. Each SM also
// has 256 KB of tensor memory (128 lanes x 512 columns of 32 bits), which
// the step does not otherwise use: here it holds the velocities, so shared
// memory holds only positions and twice as many warps fit.
//
// Layout: a CTA of 4 warps (one per TMEM lane quadrant: warp w may only
// touch lanes 32w..32w+31) allocates the columns for its point capacity;
// thread t of warp w owns lane 32w + t, and point i's velocity is columns
// 4i..4i+3 of that lane. Loads and stores are the 32x32b shape (each
// thread moves its own lane), warp-collective, so every lane of the warp
// executes them, inactive strands included.
#pragma once

#include <cstdint>

#include "hs_device.cuh"

namespace hs {
namespace tmem {

// Columns a CTA allocates for strands of up to n points: a power of two,
// at least 32 (the allocation granule).
__host__ __device__ __forceinline__ uint32_t cols_for(uint32_t n) {
  uint32_t c = 32;
  while (c < 4 * n) c *= 2;
  return c;
}

__device__ __forceinline__ void alloc(uint32_t* slot, uint32_t ncols) {
  const uint32_t dst = static_cast<uint32_t>(__cvta_generic_to_shared(slot));
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst), "r"(ncols) : "memory");
}
__device__ __forceinline__ void relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// Four columns of this thread's lane; the wait is in the same statement,
// so the values are complete when it returns.
__device__ __forceinline__ float4 load4(uint32_t taddr) {
  uint32_t a, b, c, d;
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(a), "=r"(b), "=r"(c), "=r"(d)
      : "r"(taddr)
      : "memory");
  return make_float4(__uint_as_float(a), __uint_as_float(b), __uint_as_float(c), __uint_as_float(d));
}

// Four columns of this thread's lane; completion is awaited by wait_st().
__device__ __forceinline__ void store4(uint32_t taddr, float4 v) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1, %2, %3, %4};" ::"r"(taddr),
               "r"(__float_as_uint(v.x)), "r"(__float_as_uint(v.y)), "r"(__float_as_uint(v.z)),
               "r"(__float_as_uint(v.w))
               : "memory");
}

}  // namespace tmem

// Velocity slots in tensor memory: `lane_addr` is this warp's TMEM address
// (lane quadrant in bits 31:16, first column in bits 15:0). Stores become
// visible to later loads after fence() (tcgen05.wait::st).
// Loads and stores are issued where the warp is converged (outside the
// divergent push-out, which the compiler closes with a reconvergence
// point); each substep ends with a __syncwarp and the store wait.
struct VTmem {
  static constexpr bool kShared = false;
  static constexpr bool kPrefetch = false;  // a load is waited for where it is issued
  using Pending = float4;
  uint32_t lane_addr;
  __device__ __forceinline__ float4 load(int i) const {
    return tmem::load4(lane_addr + 4u * static_cast<uint32_t>(i));
  }
  __device__ __forceinline__ void store(int i, float4 v) const {
    tmem::store4(lane_addr + 4u * static_cast<uint32_t>(i), v);
  }
  __device__ __forceinline__ void fence() const {
    __syncwarp();
    tmem::wait_st();
  }
  __device__ __forceinline__ Pending issue(int i) const { return load(i); }
  __device__ __forceinline__ float4 complete(Pending t) const { return t; }
};

}  // namespace hs
