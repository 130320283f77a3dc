// hs_stream.cuh -- one frame of one strand, streaming form.
//
// Same frame as strand_frame (hs_step.cuh), bit for bit, arranged for small
// code: the strand's positions and velocities live in shared memory and
// every pass over the strand is one runtime loop over its points. With one
// constraint iteration per substep (the DFTL default) a substep is a single
// pass in which iteration i predicts point i, runs chain link i, and
// finishes point i-1 (push-out, velocity, store): only the chain link is on
// the loop-carried path, so the rest fills its latency. More iterations
// (reference mode: 8) run a predict pass then one pass per iteration.
//
// Shared layout: [point][thread] float4, so a warp touches 512 contiguous
// bytes per access (no bank conflicts, no padding). Xs[i*B] = (position,
// rest length), Vs[i*B] = velocity, or the parked start position x_i in
// DFTL until Eq. 9 is formed (then y_i = x_i + damping * d_{i+1}).
// Any point count up to HS_MAX_POINTS_PER_STRAND.
#pragma once

#include "hs_step.cuh"

namespace hs {

// Velocity slots in shared memory, [point][thread] (any pass). The other
// store, in tensor memory, is VTmem (hs_tmem.cuh).
// kPrefetch: the single pass reads a velocity one point ahead of its use
// (issue, then complete), which hides the shared-memory latency.
struct VShared {
  static constexpr bool kShared = true;
  static constexpr bool kPrefetch = true;
  using Pending = float4;
  float4* p;
  int B;
  __device__ __forceinline__ float4 load(int i) const { return p[i * B]; }
  __device__ __forceinline__ void store(int i, float4 v) const { p[i * B] = v; }
  __device__ __forceinline__ void fence() const {}
  __device__ __forceinline__ Pending issue(int i) const { return p[i * B]; }
  __device__ __forceinline__ float4 complete(Pending t) const { return t; }
};

// Position slots. XShared4: float4 [point][thread] (position, rest length).
// XShared3: the compact form beside tensor-memory velocities, float2 (x, y)
// and float z arrays [point][thread], 12 bytes a point; the rest length
// then travels in the w of the point's velocity slot (kRestInV).
struct XShared4 {
  static constexpr bool kRestInV = false;
  float4* p;
  int B;
  __device__ __forceinline__ float4 load(int i) const { return p[i * B]; }
  __device__ __forceinline__ void store(int i, float4 v) const { p[i * B] = v; }
};
struct XShared3 {
  static constexpr bool kRestInV = true;
  float2* xy;
  float* z;
  int B;
  __device__ __forceinline__ float4 load(int i) const {
    const float2 a = xy[i * B];
    return make_float4(a.x, a.y, z[i * B], 0.0f);
  }
  __device__ __forceinline__ void store(int i, float4 v) const {
    xy[i * B] = make_float2(v.x, v.y);
    z[i * B] = v.z;
  }
};
// A position load with its rest length in w, wherever it is kept.
template <typename XS>
__device__ __forceinline__ float4 with_rest(float4 x, float4 v) {
  if constexpr (XS::kRestInV) return make_float4(x.x, x.y, x.z, v.w);
  else return x;
}
// The w a velocity slot stores: the rest length where it lives there.
template <typename XS>
__device__ __forceinline__ float vel_w(float rest) {
  if constexpr (XS::kRestInV) return rest;
  else return 0.0f;
}

// Up to M of the warp's reachable spheres sit in registers; the rest are
// read from shared memory. kCachedSpheres is the width of the batched
// kernels' cache; the plain step also has an 8-wide one (strand_frame_stream).
constexpr int kCachedSpheres = 4;

template <int M>
struct SphereCache {
  float cx[M], cy[M], cz[M], r[M], r2[M];
  float2 ncx[M / 2], ncy[M / 2], ncz[M / 2];  // negated centres, in pairs
  int ncached;      // uniform
  uint32_t rest;    // reachable spheres beyond the cached ones, in index order
};

template <int M>
__device__ __forceinline__ SphereCache<M> cache_spheres(const SphereSet& S, uint32_t reach) {
  SphereCache<M> C;
  C.ncached = 0;
#pragma unroll
  for (int q = 0; q < M; ++q) {
    C.cx[q] = C.cy[q] = C.cz[q] = C.r[q] = 0.0f;
    C.r2[q] = -1.0f;
    if (reach) {
      const int k = __ffs(reach) - 1;
      reach &= reach - 1u;
      const float4 c = S.c[k];
      C.cx[q] = c.x;
      C.cy[q] = c.y;
      C.cz[q] = c.z;
      C.r[q] = c.w;
      C.r2[q] = S.r2[k];
      C.ncached = q + 1;
    }
  }
  C.rest = reach;
#pragma unroll
  for (int q = 0; q < M / 2; ++q) {
    C.ncx[q] = make_float2(-C.cx[2 * q], -C.cx[2 * q + 1]);
    C.ncy[q] = make_float2(-C.cy[2 * q], -C.cy[2 * q + 1]);
    C.ncz[q] = make_float2(-C.cz[2 * q], -C.cz[2 * q + 1]);
  }
  return C;
}

// CollideSphere(+1, c, r, p) (cs_simulation.glsl:129-139) of one sphere.
template <bool REF>
__device__ __forceinline__ void push_out(V3 cc, float r, float r2, V3& p, V3& v) {
  const V3 pt = sub(p, cc);
  const float dp = dot(pt, pt);
  if (dp < r2) {
    const V3 nn = dp > 0.0f ? mul(pt, inversesqrt(dp)) : v3(0.0f, 1.0f, 0.0f);
    p = add(cc, mul(r, nn));
    if (REF) v = reflect(v, nn);  // :137
  }
}

// Push-out of one point against all reachable spheres, in index order.
template <bool REF, int M>
__device__ __forceinline__ void collide_cached(const SphereCache<M>& C, const SphereSet& S, V3& p, V3& v) {
#pragma unroll
  for (int q = 0; q < M; ++q)
    if (q < C.ncached) push_out<REF>(v3(C.cx[q], C.cy[q], C.cz[q]), C.r[q], C.r2[q], p, v);
  uint32_t more = C.rest;
  while (more) {
    const int k = __ffs(more) - 1;
    more &= more - 1u;
    const float4 c = S.c[k];
    push_out<REF>(v3(c.x, c.y, c.z), c.w, S.r2[k], p, v);
  }
}

// Collision of one point, split so the cheap part can be scheduled with
// other work: tests() checks the cached spheres branch-free; only if one
// of them is hit (or the warp reaches spheres beyond the cache) does
// push_all() run the exact in-order push-out. With no hit the in-order
// result is the untouched point, so both paths agree.
// NC is the number of cache slots tested; unused slots have r2 = -1 and
// never hit, so NC may exceed the number of spheres cached.
template <int NC, int M>
__device__ __forceinline__ bool tests(const SphereCache<M>& C, V3 p) {
  static_assert(NC <= M, "tests reach past the cache");
  bool hit = C.rest != 0u;
  // Two spheres per packed operation: p - c as p + (-c), then the dot
  // product in the contract's order, lane by lane. The packed forms keep
  // the scalar contract's bits here because no packed product feeds a
  // packed add: the compiler fuses __fadd2_rn(a, __fmul2_rn(b, c)) into
  // one packed fma (one rounding), even with -fmad=false, which the
  // contract's separate multiply and add would not match.
  const float2 px = make_float2(p.x, p.x), py = make_float2(p.y, p.y), pz = make_float2(p.z, p.z);
#pragma unroll
  for (int q = 0; q < NC / 2; ++q) {
    const float2 dx = __fadd2_rn(px, C.ncx[q]);
    const float2 dy = __fadd2_rn(py, C.ncy[q]);
    const float2 dz = __fadd2_rn(pz, C.ncz[q]);
    const float2 d2 = __ffma2_rn(dz, dz, __ffma2_rn(dy, dy, __fmul2_rn(dx, dx)));
    hit |= (d2.x < C.r2[2 * q]) | (d2.y < C.r2[2 * q + 1]);
  }
  return hit;
}

// The exact in-order push-out (rare), kept inline: an out-of-line call
// would take the addresses of the callers' per-lane arrays and move them
// to local memory.
template <bool REF, int NC, int M>
__device__ __forceinline__ void push_all(const SphereCache<M>& C, const SphereSet& S, V3& p, V3& v) {
#pragma unroll
  for (int q = 0; q < M; ++q)
    if (q < C.ncached) push_out<REF>(v3(C.cx[q], C.cy[q], C.cz[q]), C.r[q], C.r2[q], p, v);
  uint32_t more = C.rest;
  while (more) {
    const int k = __ffs(more) - 1;
    more &= more - 1u;
    const float4 c = S.c[k];
    push_out<REF>(v3(c.x, c.y, c.z), c.w, S.r2[k], p, v);
  }
}

template <bool REF, int NC, int M>
__device__ __forceinline__ void collide_fast(const SphereCache<M>& C, const SphereSet& S, V3& p, V3& v) {
  if (tests<NC>(C, p)) push_all<REF, NC>(C, S, p, v);
}

// Per-strand constants of a frame.
struct StrandConsts {
  V3 F;            // force per unit mass
  float h, h2, inv_h, damping, lscale;
};

// Chain link (DistanceConstraint, :109-117): point p follows `prev`.
__device__ __forceinline__ V3 link(const StrandConsts& K, V3 prev, V3 p, float rest, V3& nprev, V3& corr) {
  const V3 d = sub(p, prev);
  const float d2 = dot(d, d);
  const V3 nd = d2 > 0.0f ? mul(d, inversesqrt(d2)) : nprev;
  nprev = nd;
  const V3 pc = add(prev, mul(__fmul_rn(K.lscale, rest), nd));
  corr = sub(pc, p);
  return pc;
}

// Velocity of a finished point: reference mode, the next point's
// correction damped (the tip: its own), reflected on contact (the push-out
// path handles the reflection); DFTL, Eq. 9 as v = (q - y) / h with
// y = x + damping * d_{j+1} (the tip: y = x).
template <bool REF>
__device__ __forceinline__ V3 initial_velocity(const StrandConsts& K, V3 corr_next, V3 corr_own, bool tip) {
  return tip ? corr_own : mul(corr_next, K.damping);
}

// Finishes point j after its chain link: push-out, velocity, store.
template <bool REF, int NC, typename XS, typename VS, int M>
__device__ __forceinline__ void finish_point(const StrandConsts& K, const SphereCache<M>& C, const SphereSet& S,
                                             V3 q, bool hit, V3 corr_next, V3 x_start, float rest, bool tip,
                                             V3 corr_own, const XS& X, const VS& V, int j) {
  V3 v = v3(0.0f, 0.0f, 0.0f);
  if (REF) v = initial_velocity<true>(K, corr_next, corr_own, tip);
  if (hit) push_all<REF, NC>(C, S, q, v);
  if (!REF) {
    const V3 y = tip ? x_start : fmas(K.damping, corr_next, x_start);
    v = mul(sub(q, y), K.inv_h);
  }
  X.store(j, f4(q, rest));
  V.store(j, f4(v, vel_w<XS>(rest)));
}

__device__ __forceinline__ V3 predict(const StrandConsts& K, float4 x, float4 v) {
  return fmas(K.h2, K.F, fmas(K.h, xyz(v), xyz(x)));  // :179-183
}

// One substep with one constraint iteration, as a single software-pipelined
// pass. The loop body predicts point i+1, runs chain link i and tests point
// i-1 against the spheres in one branch-free block (three independent
// streams of work for the scheduler), then finishes point i-1.
template <bool REF, int NC, typename XS, typename VS, int M>
__device__ __forceinline__ void substep_single_pass(const StrandConsts& K, const SphereCache<M>& C, const SphereSet& S,
                                                    int n, V3 p0, const XS& X, const VS& V) {
  V3 nprev = v3(0.0f, -1.0f, 0.0f);
  // Link 1.
  const float4 v1 = V.load(1);
  const float4 x1 = with_rest<XS>(X.load(1), v1);
  V3 corr_prev;
  V3 prev = link(K, p0, predict(K, x1, v1), x1.w, nprev, corr_prev);
  V3 x_prev = xyz(x1);
  float rest_prev = x1.w;
  if (n >= 3) {
    const float4 v2 = V.load(2);
    float4 xc = with_rest<XS>(X.load(2), v2);
    V3 p_cur = predict(K, xc, v2);
    typename VS::Pending pend{};
    if constexpr (VS::kPrefetch) {
      if (n > 3) pend = V.issue(3);
    }
    // Links 2 .. n-2, with point i+1 predicted and point i-1 finished.
    // Unrolled by two so the carried values change registers instead of
    // being copied each iteration.
#pragma unroll 2
    for (int i = 2; i < n - 1; ++i) {
      const float4 xr = X.load(i + 1);
      float4 vn;
      if constexpr (VS::kPrefetch) {
        vn = V.complete(pend);
        if (i + 2 < n) pend = V.issue(i + 2);
      } else {
        vn = V.load(i + 1);
      }
      const float4 xn = with_rest<XS>(xr, vn);
      const V3 p_next = predict(K, xn, vn);
      V3 corr;
      const V3 pc = link(K, prev, p_cur, xc.w, nprev, corr);
      const bool hit = tests<NC>(C, prev);
      finish_point<REF, NC>(K, C, S, prev, hit, corr, x_prev, rest_prev, false, corr_prev, X, V, i - 1);
      prev = pc;
      corr_prev = corr;
      x_prev = xyz(xc);
      rest_prev = xc.w;
      xc = xn;
      p_cur = p_next;
    }
    // Link n-1 and point n-2.
    V3 corr;
    const V3 pc = link(K, prev, p_cur, xc.w, nprev, corr);
    const bool hit = tests<NC>(C, prev);
    finish_point<REF, NC>(K, C, S, prev, hit, corr, x_prev, rest_prev, false, corr_prev, X, V, n - 2);
    prev = pc;
    corr_prev = corr;
    x_prev = xyz(xc);
    rest_prev = xc.w;
  }
  // The tip keeps its own correction (:116); its y is its start position.
  const bool hit = tests<NC>(C, prev);
  finish_point<REF, NC>(K, C, S, prev, hit, v3(0.0f, 0.0f, 0.0f), x_prev, rest_prev, true, corr_prev, X, V,
                        n - 1);
}

// Root of substep k (:184-193): kinematic, linear from x0 to the frame's
// target, on it at the last substep.
__device__ __forceinline__ V3 root_at(int k, int substeps, bool moving, V3 x0, V3 target, V3 delta) {
  if (!moving) return x0;
  if (k + 1 == substeps) return target;
  const float alpha = __fdiv_rn(static_cast<float>(k + 1), static_cast<float>(substeps));
  return fmas(alpha, delta, x0);
}

// W substeps at once, as a diagonal wavefront. Substep k+1's chain link j
// needs point j as substep k leaves it, which substep k finishes right
// after its link j+1; so with substep k+w running link i - 2w while
// substep k runs link i, the W links of one loop iteration are independent
// (W chains for the scheduler), and every point still sees the same
// arithmetic in the same order as one substep after another. Point i of
// lane w is read in iteration i + 2w and written (as point i of the next
// lane's substep) in iteration i + 2w + 1; reads and writes of one
// iteration fall on points of different parity. Substeps run in groups of
// W; the wavefront fills and drains over 2(W-1) iterations per group.
template <bool REF, int NC, int W, int M>
__device__ __forceinline__ void substep_group(const FrameConst& fc, const StrandConsts& K, const SphereCache<M>& C,
                                              const SphereSet& S, int n, int k0, int nsub, V3 x0, V3 target,
                                              float4* Xs, float4* Vs, int B) {
  const bool moving = fc.root_mode != HS_ROOT_PINNED;
  const V3 delta = sub(target, x0);
  V3 prev[W], nprev[W], corr_prev[W], x_prev[W];
  float rest_prev[W];
#pragma unroll
  for (int w = 0; w < W; ++w) {
    prev[w] = nprev[w] = corr_prev[w] = x_prev[w] = v3(0.0f, 0.0f, 0.0f);
    rest_prev[w] = 0.0f;
  }
  const int last = 2 * (nsub - 1) + n;
  for (int tau = 0; tau <= last; ++tau) {
    V3 pc[W], corr[W];
    float4 xi[W];
    bool hit[W];
    bool any_hit = false;
    // Loads, predictions, chain links and sphere tests of every lane.
#pragma unroll
    for (int w = 0; w < W; ++w) {
      const int i = tau - 2 * w;
      if (w < nsub && i == 0) {  // substep starts at the root
        prev[w] = root_at(k0 + w, fc.substeps, moving, x0, target, delta);
        nprev[w] = v3(0.0f, -1.0f, 0.0f);
      }
      const int li = min(max(i, 1), n - 1);
      xi[w] = Xs[li * B];
      const float4 vi = Vs[li * B];
      V3 nd = nprev[w];
      pc[w] = link(K, prev[w], predict(K, xi[w], vi), xi[w].w, nd, corr[w]);
      if (w < nsub && i >= 1 && i <= n - 1) nprev[w] = nd;
      hit[w] = (w < nsub && i >= 2 && i <= n) && tests<NC>(C, prev[w]);
      any_hit |= hit[w];
    }
    // Exact in-order push-out where a sphere was hit (rare).
    V3 v[W];
#pragma unroll
    for (int w = 0; w < W; ++w) {
      const bool tip = tau - 2 * w == n;
      v[w] = REF ? (tip ? corr_prev[w] : mul(corr[w], K.damping)) : v3(0.0f, 0.0f, 0.0f);
    }
    if (any_hit) {
#pragma unroll
      for (int w = 0; w < W; ++w)
        if (hit[w]) push_all<REF, NC>(C, S, prev[w], v[w]);
    }
    // Velocities and stores of the finished points, then carry the chains.
#pragma unroll
    for (int w = 0; w < W; ++w) {
      const int i = tau - 2 * w;
      if (w < nsub && i >= 2 && i <= n) {
        const bool tip = i == n;
        V3 vel = v[w];
        if (!REF) {
          const V3 y = tip ? x_prev[w] : fmas(K.damping, corr[w], x_prev[w]);
          vel = mul(sub(prev[w], y), K.inv_h);
        }
        Xs[(i - 1) * B] = f4(prev[w], rest_prev[w]);
        Vs[(i - 1) * B] = f4(vel, 0.0f);
      }
      if (w < nsub && i >= 1 && i <= n - 1) {
        prev[w] = pc[w];
        corr_prev[w] = corr[w];
        x_prev[w] = xyz(xi[w]);
        rest_prev[w] = xi[w].w;
      }
    }
  }
}

// One substep with several constraint iterations (reference mode: 8): a
// predict pass, then one pass per iteration.
template <bool REF, int NC, typename XS, typename VS, int M>
__device__ __forceinline__ void substep_multi_pass(const StrandConsts& K, const SphereCache<M>& C, const SphereSet& S,
                                                   int n, int iterations, V3 p0, const XS& X, const VS& V) {
  // Predict pass; DFTL parks x_i in the velocity slot.
  for (int i = 1; i < n; ++i) {
    const float4 vi = V.load(i);
    const float4 xi = with_rest<XS>(X.load(i), vi);
    X.store(i, f4(fmas(K.h2, K.F, fmas(K.h, xyz(vi), xyz(xi))), xi.w));
    if (!REF) V.store(i, f4(xyz(xi), vel_w<XS>(xi.w)));
  }
  V.fence();
  for (int it = 0; it < iterations; ++it) {
    const bool last = it + 1 == iterations;
    V3 prev = p0;
    V3 nprev = v3(0.0f, -1.0f, 0.0f);
    V3 corr_prev = v3(0.0f, 0.0f, 0.0f);
    float rest_prev = 0.0f;
    for (int i = 1; i <= n; ++i) {
      V3 corr = v3(0.0f, 0.0f, 0.0f);
      float rest_i = 0.0f;
      V3 pc = prev;
      if (i < n) {
        float4 pi4 = X.load(i);
        if constexpr (XS::kRestInV) pi4.w = V.load(i).w;
        const V3 pi = xyz(pi4);
        rest_i = pi4.w;
        const V3 d = sub(pi, prev);
        const float d2 = dot(d, d);
        const V3 nd = d2 > 0.0f ? mul(d, inversesqrt(d2)) : nprev;
        nprev = nd;
        pc = add(prev, mul(__fmul_rn(K.lscale, rest_i), nd));
        corr = sub(pc, pi);
      }
      if (i >= 2) {
        const bool tip = i == n;
        V3 q = prev;
        if (REF) {
          V3 v = tip ? corr_prev : mul(corr, K.damping);
          collide_fast<true, NC>(C, S, q, v);
          V.store(i - 1, f4(v, vel_w<XS>(rest_prev)));
        } else {
          V3 unused = v3(0.0f, 0.0f, 0.0f);
          collide_fast<false, NC>(C, S, q, unused);
          if (last) {
            const V3 x = xyz(V.load(i - 1));
            const V3 y = tip ? x : fmas(K.damping, corr, x);
            V.store(i - 1, f4(mul(sub(q, y), K.inv_h), vel_w<XS>(rest_prev)));
          }
        }
        X.store(i - 1, f4(q, rest_prev));
      }
      prev = pc;
      corr_prev = corr;
      rest_prev = rest_i;
    }
  }
}

template <bool REF, int NC, int W, typename XS, typename VS, int M>
__device__ __forceinline__ void substeps(const FrameConst& fc, const StrandConsts& K, const SphereCache<M>& C,
                                         const SphereSet& S, int n, V3 x0_start, V3 target, float rest0,
                                         const XS& X, const VS& V) {
  const bool moving = fc.root_mode != HS_ROOT_PINNED;
  if constexpr (VS::kShared && !XS::kRestInV) {
  float4* const Vs = V.p;
  float4* const Xs = X.p;
  const int B = X.B;
  if (W > 1 && fc.iterations == 1 && n >= 2) {
    for (int k0 = 0; k0 < fc.substeps; k0 += W)
      substep_group<REF, NC, W>(fc, K, C, S, n, k0, min(W, fc.substeps - k0), x0_start, target, Xs, Vs, B);
    // The root's final position and its velocity over the last substep.
    const V3 delta = sub(target, x0_start);
    const int k = fc.substeps - 1;
    const V3 p0 = root_at(k, fc.substeps, moving, x0_start, target, delta);
    const V3 pm = k > 0 ? root_at(k - 1, fc.substeps, moving, x0_start, target, delta) : x0_start;
    const V3 v0 = REF ? sub(p0, pm) : mul(sub(p0, pm), K.inv_h);  // :192
    Xs[0] = f4(p0, rest0);
    Vs[0] = f4(v0, 0.0f);
    return;
  }
  }
  const V3 root_delta = sub(target, x0_start);
  V3 root = x0_start;  // root position at the start of the substep
  for (int k = 0; k < fc.substeps; ++k) {
    // Root (:184-193): kinematic, linear to its target, on it at the end.
    V3 p0 = root;
    if (moving) {
      const float alpha = __fdiv_rn(static_cast<float>(k + 1), static_cast<float>(fc.substeps));
      p0 = (k + 1 == fc.substeps) ? target : fmas(alpha, root_delta, x0_start);
    }
    const V3 v0 = REF ? sub(p0, root) : mul(sub(p0, root), K.inv_h);  // :192
    root = p0;
    X.store(0, f4(p0, rest0));
    V.store(0, f4(v0, vel_w<XS>(rest0)));
    if (n >= 2) {
      if (fc.iterations == 1) substep_single_pass<REF, NC>(K, C, S, n, p0, X, V);
      else substep_multi_pass<REF, NC>(K, C, S, n, fc.iterations, p0, X, V);
    }
    V.fence();
  }
}

// One frame of strand s. X: the position slots (XShared4 or XShared3, this
// thread's column of the block's shared [point][thread] arrays); V: the
// velocity slots (VShared, or VTmem: whose loads and stores are
// warp-collective, so every lane runs every pass, active or not).
// M: sphere-cache width. With M = 8 a warp that reaches more than
// kCachedSpheres spheres tests 8 cached ones instead of running the exact
// push-out at every point; the others keep the 4-wide tests.
template <bool REF, int W, typename XS, typename VS, int M = kCachedSpheres>
__device__ __forceinline__ void strand_frame_stream(const FrameConst& fc, const SphereSet& S, const GroomView& g,
                                                    uint32_t s, bool active, const XS& X, const VS& V) {
  const int n = static_cast<int>(g.npoints);
  float R = 0.0f;  // total link length, for culling
  // The strand comes in kLoadBatch points at a time: all their HBM loads
  // are issued before the first on-chip store (a TMEM store is a compiler
  // barrier, which would otherwise leave one load in flight per thread).
  constexpr int kLoadBatch = 8;
  for (int i0 = 0; i0 < n; i0 += kLoadBatch) {
    float4 p[kLoadBatch], v[kLoadBatch];
#pragma unroll
    for (int k = 0; k < kLoadBatch; ++k) {
      p[k] = v[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      if (active && i0 + k < n) {
        p[k] = g.pos[static_cast<size_t>(i0 + k) * g.stride + s];
        v[k] = g.vel[static_cast<size_t>(i0 + k) * g.stride + s];
      }
    }
#pragma unroll
    for (int k = 0; k < kLoadBatch; ++k) {
      const int i = i0 + k;
      if (i < n) {  // uniform over the warp (TMEM stores are warp-collective)
        X.store(i, p[k]);
        V.store(i, make_float4(v[k].x, v[k].y, v[k].z, XS::kRestInV ? p[k].w : v[k].w));
        if (i > 0) R += fabsf(fc.length_scale * p[k].w);
      }
    }
  }
  V.fence();

  // Force per unit mass: gravity (CalculateForces, :70-77) + jittered wind.
  StrandConsts K;
  const float u = hash_u01(fc.wind_key, g.strand_base + s);
  const float j = __fadd_rn(1.0f, __fmul_rn(fc.wind_jitter, __fsub_rn(1.0f, __fmul_rn(2.0f, u))));
  K.F = v3(__fmaf_rn(j, fc.wx, fc.Gx), __fmaf_rn(j, fc.wy, fc.Gy), __fmaf_rn(j, fc.wz, fc.Gz));
  K.h = fc.h;
  K.h2 = fc.h2;
  K.inv_h = fc.inv_h;
  K.damping = fc.damping;
  K.lscale = fc.length_scale;

  // Root target for this frame.
  const float4 x00 = with_rest<XS>(X.load(0), V.load(0));
  const V3 x0_start = xyz(x00);
  V3 target = x0_start;
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

  // Spheres this warp can touch during the frame (see hs_step.cuh).
  uint32_t reach = 0u;
  if (S.n > 0) {
    const V3 root_delta = sub(target, x0_start);
    const V3 mid = v3(0.5f * (x0_start.x + target.x), 0.5f * (x0_start.y + target.y), 0.5f * (x0_start.z + target.z));
    const float half_path = 0.5f * sqrtf(root_delta.x * root_delta.x + root_delta.y * root_delta.y +
                                         root_delta.z * root_delta.z);
    reach = __reduce_or_sync(0xffffffffu, active ? near_spheres(S, mid, R + half_path) : 0u);
    reach = overlap_closure(S, reach);
  }
  const SphereCache<M> C = cache_spheres<M>(S, reach);
  // One code path per cache width: all tested slots are tested whether
  // filled or not (empty ones never hit). A second path without sphere
  // tests saved their cost for warps that reach no sphere, but warps on
  // different paths at once thrashed the instruction cache of the batched
  // kernels (measured: one path is 13-16 % faster on the batched workload
  // and no slower on a single groom).
  if (M > kCachedSpheres && C.ncached > kCachedSpheres)
    substeps<REF, M, W>(fc, K, C, S, n, x0_start, target, x00.w, X, V);
  else
    substeps<REF, kCachedSpheres, W>(fc, K, C, S, n, x0_start, target, x00.w, X, V);

  TileStats ts;
  ts.init();
  for (int i = 0; i < n; ++i) {
    const float4 v = V.load(i);
    if (active) {
      const float4 x = with_rest<XS>(X.load(i), v);
      g.pos[static_cast<size_t>(i) * g.stride + s] = x;
      g.vel[static_cast<size_t>(i) * g.stride + s] = make_float4(v.x, v.y, v.z, 0.0f);
      ts.add(x, v);
    }
  }
  ts.store(g.stats, s / 32u, (g.nstrands + 31u) / 32u, static_cast<int>(threadIdx.x % 32u));
}

}  // namespace hs
