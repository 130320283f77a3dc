// hs_step.cuh -- one frame of one strand, thread-per-strand.
//
// The frame restates src/shaders/hair/01_simulation/cs_simulation.glsl
// (reference mode) and Mueller et al. 2012 (DFTL mode). Per iteration the
// reference runs the whole follow-the-leader chain (:109-117), then the
// tip-ward velocity shift (:119-121), then each point's push-out against
// the spheres (:149-153). Here the velocity shift is done inside the chain
// (link i+1 is what produces point i's velocity) and the push-out loops over
// spheres outside and points inside; each point still meets the spheres in
// the same order with the same arithmetic, so results are bit-identical.
//
// A strand's control points live in registers for the whole frame: HBM is
// read once and written once per frame, whatever the substep count.
//
// Sphere culling. Before the push-out of a substep, the spheres that no
// point of the strand can reach are skipped. After the chain every point is
// within R = sum of link lengths of the root p0; each push moves a point by
// at most the pushing sphere's radius, and a point meets each sphere once
// per pass, so with M the set of spheres kept, every point stays within
// B = R + sum_{j in M} r_j of p0. M is grown until every sphere outside it
// lies farther than r_k + B (with a relative margin far above FP32
// rounding); a skipped sphere's test is then provably false, so skipping it
// changes no bit. A warp processes the union of its lanes' sets.
#pragma once

#include "hs_device.cuh"

namespace hs {

// Rest lengths of a strand: registers for short strands, a column of
// shared memory (one float per point, stride = block size) for long ones.
template <int CAP, bool SMEM>
struct RestLengths {
  float r[CAP];
  __device__ __forceinline__ void bind(float*, int) {}
  __device__ __forceinline__ float get(int i) const { return r[i]; }
  __device__ __forceinline__ void set(int i, float v) { r[i] = v; }
};
template <int CAP>
struct RestLengths<CAP, true> {
  float* base;
  int stride;
  __device__ __forceinline__ void bind(float* b, int st) {
    base = b;
    stride = st;
  }
  __device__ __forceinline__ float get(int i) const { return base[i * stride]; }
  __device__ __forceinline__ void set(int i, float v) { base[i * stride] = v; }
};

// Capacities above this keep rest lengths in shared memory.
constexpr int kRestInRegistersMax = 16;

// Spheres of the groom being advanced, staged in shared memory.
struct SphereSet {
  const float4* c;   // (x, y, z, r)
  const float* r2;   // r * r
  int n;
};

// Set of spheres a strand rooted at p0 with total link length R can touch
// during one push-out pass (see the header comment).
__device__ __forceinline__ uint32_t reachable_spheres(const SphereSet& S, V3 p0, float R) {
  if (S.n == 0) return 0u;
  const float mag = fmaxf(fmaxf(fabsf(p0.x), fabsf(p0.y)), fmaxf(fabsf(p0.z), R)) + 1.0f;
  const float slack = mag * 1.0e-4f;
  uint32_t m = 0u;
  float B = R;
  for (int round = 0; round <= S.n; ++round) {
    uint32_t m2 = 0u;
    float sum = 0.0f;
    for (int k = 0; k < S.n; ++k) {
      const float4 c = S.c[k];
      const float dx = c.x - p0.x, dy = c.y - p0.y, dz = c.z - p0.z;
      const float d2 = dx * dx + dy * dy + dz * dz;
      const float reach = (c.w + B) * 1.001f + slack;
      if (d2 < reach * reach) {
        m2 |= 1u << k;
        sum += c.w;
      }
    }
    if (m2 == m) break;
    m = m2;
    B = (R + sum) * 1.001f + slack;
  }
  return m;
}

// One frame of strand s. CAP: compile-time capacity (register arrays);
// n = g.npoints <= CAP at run time (uniform across the groom).
// rest_smem: this thread's column of CAP floats (stride rest_stride) when
// CAP > kRestInRegistersMax, else unused. active: false for the padding
// lanes of the last warp (they join the warp votes but touch no memory).
template <int CAP, bool REF>
__device__ __forceinline__ void strand_frame(const FrameConst& fc, const SphereSet& S, const GroomView& g,
                                             uint32_t s, bool active, float* rest_smem, int rest_stride) {
  const int n = static_cast<int>(g.npoints);
  V3 X[CAP], V[CAP];
  RestLengths<CAP, (CAP > kRestInRegistersMax)> rest;
  rest.bind(rest_smem, rest_stride);
  float R = 0.0f;  // total link length, for culling
#pragma unroll
  for (int i = 0; i < CAP; ++i) {
    X[i] = v3(0.0f, 0.0f, 0.0f);
    V[i] = v3(0.0f, 0.0f, 0.0f);
    rest.set(i, 0.0f);
    if (i < n && active) {
      const float4 p = g.pos[static_cast<size_t>(i) * g.stride + s];
      const float4 v = g.vel[static_cast<size_t>(i) * g.stride + s];
      X[i] = v3(p.x, p.y, p.z);
      rest.set(i, p.w);
      V[i] = v3(v.x, v.y, v.z);
      if (i > 0) R += fabsf(fc.length_scale * p.w);
    }
  }

  // Force per unit mass: gravity (CalculateForces, :70-77) + jittered wind.
  const float u = hash_u01(fc.wind_key, g.strand_base + s);
  const float j = __fadd_rn(1.0f, __fmul_rn(fc.wind_jitter, __fsub_rn(1.0f, __fmul_rn(2.0f, u))));
  const V3 F = v3(__fmaf_rn(j, fc.wx, fc.Gx), __fmaf_rn(j, fc.wy, fc.Gy), __fmaf_rn(j, fc.wz, fc.Gz));

  // Root target for this frame.
  const V3 x0_start = X[0];
  V3 target = x0_start;
  const bool moving = fc.root_mode != HS_ROOT_PINNED;
  if (active) {
    if (fc.root_mode == HS_ROOT_RIGID) {
      const float4 r = g.root_rest[s];
      target = v3(__fmaf_rn(fc.m[8], r.z, __fmaf_rn(fc.m[4], r.y, __fmaf_rn(fc.m[0], r.x, fc.m[12]))),
                  __fmaf_rn(fc.m[9], r.z, __fmaf_rn(fc.m[5], r.y, __fmaf_rn(fc.m[1], r.x, fc.m[13]))),
                  __fmaf_rn(fc.m[10], r.z, __fmaf_rn(fc.m[6], r.y, __fmaf_rn(fc.m[2], r.x, fc.m[14]))));
    } else if (fc.root_mode == HS_ROOT_EXPLICIT || fc.root_mode == HS_ROOT_SKINNED) {
      const float4 t = g.root_target[s];
      target = v3(t.x, t.y, t.z);
    }
  }
  const V3 root_delta = sub(target, x0_start);

  for (int k = 0; k < fc.substeps; ++k) {
    // Root (:184-193): kinematic, linear to its target over the frame.
    V3 p0 = X[0];
    if (moving) {
      const float alpha = __fdiv_rn(static_cast<float>(k + 1), static_cast<float>(fc.substeps));
      p0 = fmas(alpha, root_delta, x0_start);
    }
    const V3 x0_old = X[0];
    X[0] = p0;
    // Integrate (:179-183). DFTL keeps the start position x_i in V until
    // the velocity is formed; reference mode overwrites V in the chain.
#pragma unroll
    for (int i = 1; i < CAP; ++i) {
      if (i < n) {
        const V3 pr = fmas(fc.h2, F, fmas(fc.h, V[i], X[i]));
        if (!REF) V[i] = X[i];
        X[i] = pr;
      }
    }
    const uint32_t reach = __reduce_or_sync(0xffffffffu, active ? reachable_spheres(S, p0, R) : 0u);

    for (int it = 0; it < fc.iterations; ++it) {
      const bool last = it + 1 == fc.iterations;
      // DistanceConstraint (:109-121): follow the leader, root to tip.
      V3 nprev = v3(0.0f, -1.0f, 0.0f);
#pragma unroll
      for (int i = 1; i < CAP; ++i) {
        if (i < n) {
          const V3 p1 = X[i];
          const V3 d = sub(p1, X[i - 1]);
          const float d2 = dot(d, d);
          const V3 nd = d2 > 0.0f ? mul(d, inversesqrt(d2)) : nprev;
          nprev = nd;
          X[i] = add(X[i - 1], mul(__fmul_rn(fc.length_scale, rest.get(i)), nd));
          const V3 corr = sub(X[i], p1);
          if (REF) {
            // :116 then :119-121: each point takes its own correction, then
            // the next link replaces it with the next point's, damped; the
            // tip, last in the chain, keeps its own.
            V[i] = corr;
            if (i >= 2) V[i - 1] = mul(corr, fc.damping);
          } else if (last && i >= 2) {
            // Eq. 9 as v = (p - y) / h with y = x + damping * d_{i+1}.
            V[i - 1] = fmas(fc.damping, corr, V[i - 1]);
          }
        }
      }
      // CollisionConstraint (:149-153): every point but the root.
      uint32_t todo = reach;
      while (todo) {
        const int k2 = __ffs(todo) - 1;
        todo &= todo - 1u;
        const float4 c = S.c[k2];
        const float r2 = S.r2[k2];
        const V3 cc = v3(c.x, c.y, c.z);
#pragma unroll
        for (int i = 1; i < CAP; ++i) {
          if (i < n) {
            const V3 pt = sub(X[i], cc);
            const float dp = dot(pt, pt);
            if (dp < r2) {
              const V3 nn = dp > 0.0f ? mul(pt, inversesqrt(dp)) : v3(0.0f, 1.0f, 0.0f);
              X[i] = add(cc, mul(c.w, nn));
              if (REF) V[i] = reflect(V[i], nn);  // :137
            }
          }
        }
      }
    }
    if (REF) {
      V[0] = sub(X[0], x0_old);  // :192
    } else {
      V[0] = mul(sub(X[0], x0_old), fc.inv_h);
#pragma unroll
      for (int i = 1; i < CAP; ++i)
        if (i < n) V[i] = mul(sub(X[i], V[i]), fc.inv_h);
    }
  }

  if (!active) return;
#pragma unroll
  for (int i = 0; i < CAP; ++i) {
    if (i < n) {
      g.pos[static_cast<size_t>(i) * g.stride + s] = make_float4(X[i].x, X[i].y, X[i].z, rest.get(i));
      g.vel[static_cast<size_t>(i) * g.stride + s] = make_float4(V[i].x, V[i].y, V[i].z, 0.0f);
    }
  }
}

}  // namespace hs
