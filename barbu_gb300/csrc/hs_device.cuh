// hs_device.cuh -- device types and the arithmetic contract of the step.
//
// Every floating-point operation of the simulation is spelled with an
// explicitly rounded intrinsic (__fadd_rn, __fmul_rn, __fmaf_rn,
// __fsqrt_rn, __fdiv_rn) or an explicitly rounded two-wide instruction
// ({add,sub,fma}.rn.f32x2, below), so the compilers cannot contract or
// reassociate it. The contract is the one cs_simulation.glsl's builtins
// are given here:
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

// The (x, y) halves of the vector additions, subtractions and fmas run as
// one two-wide FP32 instruction ({add,sub,fma}.rn.f32x2, sm_100 and later)
// on a 64-bit register pair, z as a scalar one. Each half of a .rn.f32x2
// instruction is rounded as the scalar .rn instruction rounds it, so a
// vector operation gives the bits of three scalar intrinsics in two
// instructions. The vector multiply stays scalar: ptxas (CUDA 13.0) fuses
// a mul.rn.f32x2 whose result feeds an add.rn.f32x2 or sub.rn.f32x2 into
// one fused multiply-add despite the rounding modifiers (so does the
// __fmul2_rn / __fadd2_rn pair), which changes the bits; a scalar multiply
// feeding a packed add is left alone. Measured on 2^21 random pairs.
__device__ __forceinline__ uint64_t pair(float a, float b) {
  uint64_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ V3 with_z(uint64_t xy, float z) {
  V3 o;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(o.x), "=f"(o.y) : "l"(xy));
  o.z = z;
  return o;
}
__device__ __forceinline__ V3 add(V3 a, V3 b) {
  uint64_t r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pair(a.x, a.y)), "l"(pair(b.x, b.y)));
  return with_z(r, __fadd_rn(a.z, b.z));
}
__device__ __forceinline__ V3 sub(V3 a, V3 b) {
  uint64_t r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(pair(a.x, a.y)), "l"(pair(b.x, b.y)));
  return with_z(r, __fsub_rn(a.z, b.z));
}
__device__ __forceinline__ V3 mul(float s, V3 a) {
  return V3{__fmul_rn(s, a.x), __fmul_rn(s, a.y), __fmul_rn(s, a.z)};
}
__device__ __forceinline__ V3 mul(V3 a, float s) {
  return V3{__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s)};
}
// fma(a, b, c) with scalar a.
__device__ __forceinline__ V3 fmas(float a, V3 b, V3 c) {
  uint64_t r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(pair(a, a)), "l"(pair(b.x, b.y)), "l"(pair(c.x, c.y)));
  return with_z(r, __fmaf_rn(a, b.z, c.z));
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
// The FAST contract's reciprocal square root: the hardware approximation
// (flush-to-zero; the argument held at or above the smallest normal float,
// so that a zero link length gives a finite scale and normalize(0) = 0).
__device__ __forceinline__ float rsqrt_fast(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(fmaxf(x, 1.17549435e-38f)));
  return y;
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
  int32_t contract;         // hs_contract of the DFTL chain link
  float4 spheres[HS_MAX_SPHERES];  // (x, y, z, r)
  float r2[HS_MAX_SPHERES];        // r * r
  uint32_t adj[HS_MAX_SPHERES];    // adj[k] bit j: spheres k and j overlap (with margin)
  float4 bone_real[HS_MAX_BONES];  // bone palette (SKINNED): dual quaternions,
  float4 bone_dual[HS_MAX_BONES];  // (x, y, z, w) real and dual parts
};

// Device view of a groom's state. Structure of arrays [point][strand]:
// point i of strand s at i * stride + s.
struct GroomView {
  float4* pos;               // (x, y, z, restlength)
  float4* vel;               // (x, y, z, 0)
  const float4* root_rest;   // rest root (RIGID), or null
  const float4* root_target; // explicit target (EXPLICIT), or null
  const uint4* skin;         // per strand (SKINNED): 4 bone indices (bytes), weights 0..2 as float bits
  float4* stats;             // 2 per 32-strand tile, written every frame (TileStats)
  const uint32_t* order;     // [stride]: the caller's index of each stored strand
  uint32_t nstrands, stride, npoints, strand_base;
};

// Statistics of one frame of a 32-strand tile: bounds of the control points,
// kinetic energy (0.5 |v|^2 per point, unit mass) and the largest |v|^2.
// Each thread accumulates its strand in point order, the warp reduces with
// shuffles (an xor tree: every lane ends with the same bits), lane 0 writes
// (min.xyz, energy) and (max.xyz, max |v|^2). The host combines the tiles
// (hs_groom_stats).
struct TileStats {
  float mnx, mny, mnz, mxx, mxy, mxz, ke, v2;
  __device__ __forceinline__ void init() {
    mnx = mny = mnz = __int_as_float(0x7f800000);   // +inf
    mxx = mxy = mxz = __int_as_float(0xff800000);   // -inf
    ke = 0.0f;
    v2 = 0.0f;
  }
  __device__ __forceinline__ void add(float4 p, float4 v) {
    mnx = fminf(mnx, p.x);
    mny = fminf(mny, p.y);
    mnz = fminf(mnz, p.z);
    mxx = fmaxf(mxx, p.x);
    mxy = fmaxf(mxy, p.y);
    mxz = fmaxf(mxz, p.z);
    const float s = __fmaf_rn(v.z, v.z, __fmaf_rn(v.y, v.y, __fmul_rn(v.x, v.x)));
    ke = __fmaf_rn(0.5f, s, ke);
    v2 = fmaxf(v2, s);
  }
  // Warps past the groom's last tile (blocks wider than the groom) write nothing.
  __device__ __forceinline__ void store(float4* stats, uint32_t tile, uint32_t ntiles, int lane) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      mnx = fminf(mnx, __shfl_xor_sync(0xffffffffu, mnx, off));
      mny = fminf(mny, __shfl_xor_sync(0xffffffffu, mny, off));
      mnz = fminf(mnz, __shfl_xor_sync(0xffffffffu, mnz, off));
      mxx = fmaxf(mxx, __shfl_xor_sync(0xffffffffu, mxx, off));
      mxy = fmaxf(mxy, __shfl_xor_sync(0xffffffffu, mxy, off));
      mxz = fmaxf(mxz, __shfl_xor_sync(0xffffffffu, mxz, off));
      ke = __fadd_rn(ke, __shfl_xor_sync(0xffffffffu, ke, off));
      v2 = fmaxf(v2, __shfl_xor_sync(0xffffffffu, v2, off));
    }
    if (lane == 0 && stats && tile < ntiles) {
      stats[2 * tile] = make_float4(mnx, mny, mnz, ke);
      stats[2 * tile + 1] = make_float4(mxx, mxy, mxz, v2);
    }
  }
};

// 4-component dot in the order of dot(): fma(a.w,b.w, fma(a.z,b.z, fma(a.y,b.y, a.x*b.x))).
__device__ __forceinline__ float dot4(float4 a, float4 b) {
  return __fmaf_rn(a.w, b.w, __fmaf_rn(a.z, b.z, __fmaf_rn(a.y, b.y, __fmul_rn(a.x, b.x))));
}
// cross(a, b), each component as fma(p, q, -(r * t)).
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
  return V3{__fmaf_rn(a.y, b.z, -__fmul_rn(a.z, b.y)), __fmaf_rn(a.z, b.x, -__fmul_rn(a.x, b.z)),
            __fmaf_rn(a.x, b.y, -__fmul_rn(a.y, b.x))};
}
__device__ __forceinline__ float sign_of(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }

// Dual-quaternion blend of a rest point (Kavan et al. 2008), the
// reference's apply_skinning + skinning_DQBS (inc_skinning.glsl:22-82),
// operation for operation (the blend and 4-dots as fma chains, the rest as
// the shader writes it):
// no skinning when the first weight is <= 1e-6; the fourth weight is
// 1 - (w0 + w1 + w2); weights 0..2 flip sign where their bone's rotation is
// antipodal to bone 3's; the blend is normalised by its real part's norm.
__device__ __forceinline__ V3 skin_point(const FrameConst& fc, V3 v, uint4 sk) {
  float w0 = __uint_as_float(sk.y), w1 = __uint_as_float(sk.z), w2 = __uint_as_float(sk.w);
  if (w0 <= 1e-6f) return v;
  const float w3 = __fsub_rn(1.0f, __fadd_rn(__fadd_rn(w0, w1), w2));
  const uint32_t b0 = sk.x & 0xffu, b1 = (sk.x >> 8) & 0xffu, b2 = (sk.x >> 16) & 0xffu, b3 = sk.x >> 24;
  const float4 r0 = fc.bone_real[b0], r1 = fc.bone_real[b1], r2 = fc.bone_real[b2], r3 = fc.bone_real[b3];
  const float4 d0 = fc.bone_dual[b0], d1 = fc.bone_dual[b1], d2 = fc.bone_dual[b2], d3 = fc.bone_dual[b3];
  w0 = __fmul_rn(w0, sign_of(dot4(r3, r0)));
  w1 = __fmul_rn(w1, sign_of(dot4(r3, r1)));
  w2 = __fmul_rn(w2, sign_of(dot4(r3, r2)));
  // A = Ma * w, B = Mb * w, summed in column order.
  float4 A, B;
  A.x = __fmaf_rn(r3.x, w3, __fmaf_rn(r2.x, w2, __fmaf_rn(r1.x, w1, __fmul_rn(r0.x, w0))));
  A.y = __fmaf_rn(r3.y, w3, __fmaf_rn(r2.y, w2, __fmaf_rn(r1.y, w1, __fmul_rn(r0.y, w0))));
  A.z = __fmaf_rn(r3.z, w3, __fmaf_rn(r2.z, w2, __fmaf_rn(r1.z, w1, __fmul_rn(r0.z, w0))));
  A.w = __fmaf_rn(r3.w, w3, __fmaf_rn(r2.w, w2, __fmaf_rn(r1.w, w1, __fmul_rn(r0.w, w0))));
  B.x = __fmaf_rn(d3.x, w3, __fmaf_rn(d2.x, w2, __fmaf_rn(d1.x, w1, __fmul_rn(d0.x, w0))));
  B.y = __fmaf_rn(d3.y, w3, __fmaf_rn(d2.y, w2, __fmaf_rn(d1.y, w1, __fmul_rn(d0.y, w0))));
  B.z = __fmaf_rn(d3.z, w3, __fmaf_rn(d2.z, w2, __fmaf_rn(d1.z, w1, __fmul_rn(d0.z, w0))));
  B.w = __fmaf_rn(d3.w, w3, __fmaf_rn(d2.w, w2, __fmaf_rn(d1.w, w1, __fmul_rn(d0.w, w0))));
  const float inv = inversesqrt(dot4(A, A));
  const V3 a = v3(__fmul_rn(A.x, inv), __fmul_rn(A.y, inv), __fmul_rn(A.z, inv));
  const float aw = __fmul_rn(A.w, inv);
  const V3 b = v3(__fmul_rn(B.x, inv), __fmul_rn(B.y, inv), __fmul_rn(B.z, inv));
  const float bw = __fmul_rn(B.w, inv);
  // Rotate: v += 2 cross(a, cross(a, v) + aw v) (:77), unfused as written.
  v = add(v, mul(2.0f, cross(a, add(cross(a, v), mul(aw, v)))));
  // Translate: v += 2 ((aw b - bw a) + cross(a, b)) (:78).
  const V3 t = add(sub(mul(aw, b), mul(bw, a)), cross(a, b));
  return add(v, mul(2.0f, t));
}

}  // namespace hs
