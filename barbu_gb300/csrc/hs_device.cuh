// hs_device.cuh -- device types and the arithmetic contract of the step.
//
// Every floating-point operation of the simulation is spelled with an
// explicitly rounded intrinsic (__fadd_rn, __fmul_rn, __fmaf_rn,
// __fsqrt_rn, __fdiv_rn), so nvcc cannot contract or reassociate it. The
// contract is the one cs_simulation.glsl's builtins are given here:
//   dot(a,b)       = fma(a.z,b.z, fma(a.y,b.y, a.x*b.x))
//   inversesqrt(x) = magic-constant estimate (C. Lomont, "Fast Inverse
//                    Square Root", 2003), two Newton-Raphson steps
//                    y *= 1.5 - (x/2) y^2, then y += (y/2)(1 - x y^2) with
//                    the residual by fma: < 1 ulp, no MUFU, no branch
//   normalize(v)   = v * inversesqrt(dot(v,v)), guarded at dot == 0
//   reflect(I,N)   = I - (2*dot(N,I)) * N
// With it, FP32 results are identical to a CPU evaluation of the same
// expressions, which is how the tests hold the kernels to the reference.
// Only IEEE add, multiply and fma are used in the step itself: each is
// correctly rounded on both sides, so no vendor approximation enters.
#pragma once

#include <cstdint>

#include "hairsim.h"

namespace hs {

struct V3 {
  float x, y, z;
};

__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 add(V3 a, V3 b) {
  return V3{__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z)};
}
__device__ __forceinline__ V3 sub(V3 a, V3 b) {
  return V3{__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)};
}
__device__ __forceinline__ V3 mul(float s, V3 a) {
  return V3{__fmul_rn(s, a.x), __fmul_rn(s, a.y), __fmul_rn(s, a.z)};
}
__device__ __forceinline__ V3 mul(V3 a, float s) {
  return V3{__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s)};
}
// fma(a, b, c) with scalar a.
__device__ __forceinline__ V3 fmas(float a, V3 b, V3 c) {
  return V3{__fmaf_rn(a, b.x, c.x), __fmaf_rn(a, b.y, c.y), __fmaf_rn(a, b.z, c.z)};
}
__device__ __forceinline__ float dot(V3 a, V3 b) {
  return __fmaf_rn(a.z, b.z, __fmaf_rn(a.y, b.y, __fmul_rn(a.x, b.x)));
}
__device__ __forceinline__ float inversesqrt(float x) {
  float y = __uint_as_float(0x5f3759dfu - (__float_as_uint(x) >> 1));
  const float hx = __fmul_rn(0.5f, x);
  y = __fmul_rn(y, __fmaf_rn(-hx, __fmul_rn(y, y), 1.5f));
  y = __fmul_rn(y, __fmaf_rn(-hx, __fmul_rn(y, y), 1.5f));
  const float r = __fmaf_rn(-__fmul_rn(x, y), y, 1.0f);
  return __fmaf_rn(__fmul_rn(0.5f, y), r, y);
}
__device__ __forceinline__ V3 reflect(V3 i, V3 n) { return sub(i, mul(__fmul_rn(2.0f, dot(n, i)), n)); }

// Seeded counter hash (lowbias32, C. Wellons), standing in for the
// reference's time-seeded rand() (src/core/app.cc:96-97, src/fx/hair.cc:269).
__host__ __device__ __forceinline__ uint32_t lowbias32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x;
}
__host__ __device__ __forceinline__ uint32_t stream_key(uint64_t seed, uint32_t stream) {
  return lowbias32(static_cast<uint32_t>(seed) ^
                   lowbias32(static_cast<uint32_t>(seed >> 32) + 0x9E3779B9U * (stream + 1U)));
}
// u in [0,1), a multiple of 2^-24 (exact in float).
__device__ __forceinline__ float hash_u01(uint32_t key, uint32_t idx) {
  return __fmul_rn(static_cast<float>(lowbias32(idx + key) >> 8), 1.0f / 16777216.0f);
}
constexpr uint32_t kStreamLength = 1;
constexpr uint32_t kStreamWind = 2;

// Per-groom, per-frame constants of one update. Plain path: passed by value
// as a kernel parameter. Batched path: one entry per groom in a device table.
struct FrameConst {
  float h, h2, inv_h;       // substep, its square, its inverse (float ops)
  float damping, length_scale, wind_jitter;
  float Gx, Gy, Gz;         // gravity_scale * gravity
  float wx, wy, wz;         // wind
  float m[16];              // root transform (RIGID), column-major
  int32_t substeps, iterations, mode, root_mode;
  int32_t nspheres;
  uint32_t wind_key;
  float sphere_rmax;        // largest sphere radius (culling bound)
  int32_t pad;
  float4 spheres[HS_MAX_SPHERES];  // (x, y, z, r)
  float r2[HS_MAX_SPHERES];        // r * r
  uint32_t adj[HS_MAX_SPHERES];    // adj[k] bit j: spheres k and j overlap (with margin)
};

// Device view of a groom's state. Structure of arrays [point][strand]:
// point i of strand s at i * stride + s.
struct GroomView {
  float4* pos;               // (x, y, z, restlength)
  float4* vel;               // (x, y, z, 0)
  const float4* root_rest;   // rest root (RIGID), or null
  const float4* root_target; // explicit target (EXPLICIT), or null
  uint32_t nstrands, stride, npoints, strand_base;
};

}  // namespace hs
