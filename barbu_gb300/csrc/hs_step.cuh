// hs_step.cuh -- one frame of one strand, thread-per-strand.
//
// Reference mode restates src/shaders/hair/01_simulation/cs_simulation.glsl.
// Per iteration the reference runs the whole follow-the-leader chain
// (:109-117), then the tip-ward velocity shift (:119-121), then each
// point's push-out (:149-153). Here the velocity shift is written inside
// the chain (link i+1 is what produces point i's velocity) and the push-out
// loops over spheres outside and points inside; each point still meets the
// spheres in index order with the same arithmetic, so results are
// bit-identical to the reference's phase-by-phase order.
//
// DFTL mode (Mueller et al. 2012) runs in the segment form (hs_stream.cuh):
// per point its segment s_i = p_i - p_{i-1} and, within a substep, its
// displacement D_i = p_i - x_i, instead of world positions. The algorithm is
// the same; the rounding is not: world coordinates round at ~6e-8 |p| per
// operation and Eq. 9 divides position differences by the substep h, so
// every substep would inject ~6e-8 |p| / h of velocity noise; segments and
// displacements are a segment's length or a substep's motion in size.
//
// Storage. A strand's positions live in registers for the whole frame.
// Velocities (x, y, z) with the rest length in .w live either in registers
// too (VSMEM = false) or in a float4 column of shared memory (VSMEM =
// true); the autotuner picks per bucket. HBM is read once and written once
// per frame, whatever the substep count.
//
// Sphere culling, exact. After the chain every point is within R = sum of
// link lengths of the root p0, and p0 stays within |target - x0|/2 of the
// midpoint of its path over the frame. A push moves a point onto the
// pushing sphere's surface, so a point can enter sphere k only if k reaches
// that ball (the near set: |c_k - mid| < r_k + R + |target - x0|/2) or the
// point sits on a sphere j that overlaps k. The spheres a strand can touch
// in the frame are therefore the closure of the near set under overlap;
// every other sphere's test is provably false (margins far above FP32
// rounding), so skipping it changes no bit. The reference-mode register
// form here tests, per warp, the closure of its lanes' union; the DFTL
// forms (hs_stream.cuh, hs_lanes.cuh) keep each strand's own closure.
#pragma once

#include "hs_device.cuh"

namespace hs {

// Spheres of the groom being advanced, staged in shared memory.
struct SphereSet {
  const float4* c;     // (x, y, z, r)
  const float* r2;     // r * r
  const uint32_t* adj; // adj[k]: spheres overlapping sphere k
  int n;
};

// Near set of one strand (see the header comment): spheres reaching the
// ball of radius `reach_extra` around `mid`.
__device__ __forceinline__ uint32_t near_spheres(const SphereSet& S, V3 mid, float reach_extra) {
  const float mag = fmaxf(fmaxf(fabsf(mid.x), fabsf(mid.y)), fmaxf(fabsf(mid.z), reach_extra)) + 1.0f;
  const float slack = mag * 1.0e-4f;
  uint32_t m = 0u;
  for (int k = 0; k < S.n; ++k) {
    const float4 c = S.c[k];
    const float dx = c.x - mid.x, dy = c.y - mid.y, dz = c.z - mid.z;
    const float d2 = dx * dx + dy * dy + dz * dz;
    const float reach = (c.w + reach_extra) * 1.001f + slack;
    if (d2 < reach * reach) m |= 1u << k;
  }
  return m;
}

// Smallest summed link length at which a point of the strand may touch a
// sphere: min over spheres k of the distance from `mid` to k's surface less
// the root's half path, with near_spheres' margins (reach_extra: its
// argument, R + half_path). A point whose links from the root sum to less
// cannot be inside any sphere this frame.
__device__ __forceinline__ float reach_threshold(const SphereSet& S, V3 mid, float reach_extra, float half_path) {
  const float mag = fmaxf(fmaxf(fabsf(mid.x), fabsf(mid.y)), fmaxf(fabsf(mid.z), reach_extra)) + 1.0f;
  const float slack = mag * 1.0e-4f;
  float t = 3.0e38f;
  for (int k = 0; k < S.n; ++k) {
    const float4 c = S.c[k];
    const float dx = c.x - mid.x, dy = c.y - mid.y, dz = c.z - mid.z;
    const float d = sqrtf(dx * dx + dy * dy + dz * dz);
    t = fminf(t, (d - slack) / 1.001f - c.w - half_path);
  }
  return t;
}

// Closure of a sphere set under overlap.
__device__ __forceinline__ uint32_t overlap_closure(const SphereSet& S, uint32_t m) {
  for (;;) {
    uint32_t m2 = m, todo = m;
    while (todo) {
      const int k = __ffs(todo) - 1;
      todo &= todo - 1u;
      m2 |= S.adj[k];
    }
    if (m2 == m) return m;
    m = m2;
  }
}

// Velocity slots (velocity or parked position in xyz, rest length in w).
template <int CAP, bool SMEM>
struct VStore {
  float4 v[CAP];
  __device__ __forceinline__ void bind(float4*, int) {}
  __device__ __forceinline__ float4 get(int i) const { return v[i]; }
  __device__ __forceinline__ float get_w(int i) const { return v[i].w; }
  __device__ __forceinline__ void set(int i, float4 x) { v[i] = x; }
};
// Shared-memory slots: each thread owns CAP consecutive float4 (its row),
// rows padded to CAP + 1 float4 so that the eight threads of a 128-bit
// shared-memory phase fall on distinct banks. Offsets are compile-time.
template <int CAP>
struct VStore<CAP, true> {
  static constexpr int kRow = CAP + 1;
  float4* base;
  __device__ __forceinline__ void bind(float4* rows, int thread) { base = rows + thread * kRow; }
  __device__ __forceinline__ float4 get(int i) const { return base[i]; }
  __device__ __forceinline__ float get_w(int i) const { return reinterpret_cast<const float*>(base + i)[3]; }
  __device__ __forceinline__ void set(int i, float4 x) { base[i] = x; }
};
// Shared memory of the velocity slots for `threads` threads.
template <int CAP>
constexpr size_t vslot_bytes(int threads) {
  return sizeof(float4) * (CAP + 1) * threads;
}

__device__ __forceinline__ float4 f4(V3 a, float w) { return make_float4(a.x, a.y, a.z, w); }
__device__ __forceinline__ V3 xyz(float4 a) { return v3(a.x, a.y, a.z); }

// One frame of strand s in reference mode. CAP: compile-time capacity
// (register arrays); n = g.npoints <= CAP at run time (uniform across the
// groom). VSMEM: where the velocity slots live; vs_rows/thread: the block's
// shared rows and this thread's index when they live in shared memory.
// active: false for the padding lanes of a warp (they follow the warp
// through the vote but touch no memory). DFTL mode's register form is
// strand_frame_regs_dftl (hs_stream.cuh).
template <int CAP, bool VSMEM>
__device__ __forceinline__ void strand_frame_ref(const FrameConst& fc, const SphereSet& S, const GroomView& g,
                                             uint32_t s, bool active, float4* vs_rows, int thread) {
  // Frame constants: kernel parameters (plain step) or this warp's table
  // entry in shared memory (batched step); either way read where used.
  const int n = static_cast<int>(g.npoints);

  V3 X[CAP];
  VStore<CAP, VSMEM> vs;
  vs.bind(vs_rows, thread);
  float R = 0.0f;  // total link length, for culling
#pragma unroll
  for (int i = 0; i < CAP; ++i) {
    X[i] = v3(0.0f, 0.0f, 0.0f);
    if (i < n) {
      float4 p = make_float4(0.0f, 0.0f, 0.0f, 0.0f), v = p;
      if (active) {
        p = g.pos[static_cast<size_t>(i) * g.stride + s];
        v = g.vel[static_cast<size_t>(i) * g.stride + s];
      }
      X[i] = v3(p.x, p.y, p.z);
      vs.set(i, make_float4(v.x, v.y, v.z, p.w));
      if (i > 0) R += fabsf(fc.length_scale * p.w);
    }
  }

  // Force per unit mass: gravity (CalculateForces, :70-77) + jittered wind.
  // Per-strand hashes use the caller's strand index (the library stores
  // strands in its own order).
  const float u = hash_u01(fc.wind_key, g.strand_base + (active ? g.order[s] : s));
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
    } else if (fc.root_mode == HS_ROOT_EXPLICIT) {
      const float4 t = g.root_target[s];
      target = v3(t.x, t.y, t.z);
    } else if (fc.root_mode == HS_ROOT_SKINNED) {
      const float4 r = g.root_rest[s];
      target = skin_point(fc, v3(r.x, r.y, r.z), g.skin[s]);
    }
  }
  const V3 root_delta = sub(target, x0_start);

  // Spheres this warp can touch during the frame.
  uint32_t reach = 0u;
  if (S.n > 0) {
    const V3 mid = v3(0.5f * (x0_start.x + target.x), 0.5f * (x0_start.y + target.y), 0.5f * (x0_start.z + target.z));
    const float half_path = 0.5f * sqrtf(root_delta.x * root_delta.x + root_delta.y * root_delta.y +
                                         root_delta.z * root_delta.z);
    reach = __reduce_or_sync(0xffffffffu, active ? near_spheres(S, mid, R + half_path) : 0u);
    reach = overlap_closure(S, reach);
  }

  for (int k = 0; k < fc.substeps; ++k) {
    // Root (:184-193): kinematic, linear to its target, on it at the end.
    V3 p0 = X[0];
    if (moving) {
      const float alpha = __fdiv_rn(static_cast<float>(k + 1), static_cast<float>(fc.substeps));
      p0 = (k + 1 == fc.substeps) ? target : fmas(alpha, root_delta, x0_start);
    }
    const V3 x0_old = X[0];
    X[0] = p0;
    // Integrate (:179-183).
#pragma unroll
    for (int i = 1; i < CAP; ++i) {
      if (i < n) {
        const float4 v = vs.get(i);
        X[i] = fmas(fc.h2, F, fmas(fc.h, xyz(v), X[i]));
      }
    }

    for (int it = 0; it < fc.iterations; ++it) {
      // DistanceConstraint (:109-121): follow the leader, root to tip.
      V3 nprev = v3(0.0f, -1.0f, 0.0f);
      float rest_prev = 0.0f;
#pragma unroll
      for (int i = 1; i < CAP; ++i) {
        if (i < n) {
          const float rest_i = vs.get_w(i);
          const V3 p1 = X[i];
          const V3 d = sub(p1, X[i - 1]);
          const float d2 = dot(d, d);
          const V3 nd = d2 > 0.0f ? mul(d, inversesqrt(d2)) : nprev;
          nprev = nd;
          X[i] = add(X[i - 1], mul(__fmul_rn(fc.length_scale, rest_i), nd));
          const V3 corr = sub(X[i], p1);
          // :116 then :119-121: each point takes its own correction and
          // the next link replaces it with the next point's, damped; the
          // tip, last in the chain, keeps its own.
          vs.set(i, f4(corr, rest_i));
          if (i >= 2) vs.set(i - 1, f4(mul(corr, fc.damping), rest_prev));
          rest_prev = rest_i;
        }
      }
      // CollisionConstraint (:149-153): every point but the root, each
      // against the reachable spheres in index order (CollideSphere, :129-139).
      uint32_t todo = reach;
      while (todo) {
        const int kk = __ffs(todo) - 1;
        todo &= todo - 1u;
        const float4 c = S.c[kk];
        const float r2 = S.r2[kk];
        const V3 cc = v3(c.x, c.y, c.z);
#pragma unroll
        for (int i = 1; i < CAP; ++i) {
          if (i < n) {
            const V3 pt = sub(X[i], cc);
            const float dp = dot(pt, pt);
            if (dp < r2) {
              const V3 nn = dp > 0.0f ? mul(pt, inversesqrt(dp)) : v3(0.0f, 1.0f, 0.0f);
              X[i] = add(cc, mul(c.w, nn));
              const float4 sl = vs.get(i);
              vs.set(i, f4(reflect(xyz(sl), nn), sl.w));  // :137
            }
          }
        }
      }
    }
    const float4 s0 = vs.get(0);
    vs.set(0, f4(sub(X[0], x0_old), s0.w));  // :192
  }

  TileStats ts;
  ts.init();
  if (active) {
#pragma unroll
    for (int i = 0; i < CAP; ++i) {
      if (i < n) {
        const float4 v = vs.get(i);
        const float4 x = make_float4(X[i].x, X[i].y, X[i].z, v.w);
        g.pos[static_cast<size_t>(i) * g.stride + s] = x;
        g.vel[static_cast<size_t>(i) * g.stride + s] = make_float4(v.x, v.y, v.z, 0.0f);
        ts.add(x, v);
      }
    }
  }
  ts.store(g.stats, s / 32u, (g.nstrands + 31u) / 32u, static_cast<int>(threadIdx.x % 32u));
}

}  // namespace hs
