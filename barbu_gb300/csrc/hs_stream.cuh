// hs_stream.cuh -- one frame of one strand, streaming form.
//
// Same frame as strand_frame (hs_step.cuh), bit for bit, arranged for small
// code: the strand's state lives on chip and every pass over the strand is
// one runtime loop over its points. With one constraint iteration per
// substep (the DFTL default) a substep is a single pass in which iteration
// i loads point i+1, runs chain link i, and finishes point i-1 (push-out,
// velocity, store): only the chain link is on the loop-carried path, so the
// rest fills its latency. More iterations (reference mode: 8) run a predict
// pass then one pass per iteration.
//
// Slots: X[i] holds point i's position (reference mode) or its segment
// s_i = p_i - p_{i-1} (DFTL mode, the segment form of hs_step.cuh), V[i]
// its velocity, or within a substep its displacement D_i. The rest length
// rides in the w of one of them. Any point count up to
// HS_MAX_POINTS_PER_STRAND.
#pragma once

#include "hs_step.cuh"

namespace hs {

// Velocity slots in shared memory, [point][thread] float4, so a warp
// touches 512 contiguous bytes per access (no bank conflicts, no padding).
// The other store, in tensor memory, is VTmem (hs_tmem.cuh).
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

// Position (or segment) slots. XShared4: float4 [point][thread] with the
// rest length in w. XShared3: the compact form beside tensor-memory
// velocities, float2 (x, y) and float z arrays [point][thread], 12 bytes a
// point; the rest length then travels in the w of the point's velocity
// slot (kRestInV).
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
// An X slot's load with its rest length in w, wherever it is kept.
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
  int ncached;      // spheres cached (this lane's)
  uint32_t rest;    // reachable spheres beyond the cached ones, in index order
  uint32_t reach;   // every reachable sphere
};

template <int M>
__device__ __forceinline__ SphereCache<M> cache_spheres(const SphereSet& S, uint32_t reach) {
  SphereCache<M> C;
  C.ncached = 0;
  C.reach = reach;
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

// CollideSphere(+1, c, r, p) (cs_simulation.glsl:129-139) of one sphere;
// true if the sphere pushed the point. FAST: the normal's reciprocal
// square root is the hardware's (the FAST contract, DFTL mode only).
template <bool REF, bool FAST = false>
__device__ __forceinline__ bool push_out(V3 cc, float r, float r2, V3& p, V3& v) {
  static_assert(!(REF && FAST), "reference mode has the EXACT contract only");
  const V3 pt = sub(p, cc);
  const float dp = dot(pt, pt);
  if (dp < r2) {
    const V3 nn = dp > 0.0f ? mul(pt, FAST ? rsqrt_fast(dp) : inversesqrt(dp)) : v3(0.0f, 1.0f, 0.0f);
    p = add(cc, mul(r, nn));
    if (REF) v = reflect(v, nn);  // :137
    return true;
  }
  return false;
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
// to local memory. True if any sphere pushed the point.
template <bool REF, int NC, bool FAST = false, int M>
__device__ __forceinline__ bool push_all(const SphereCache<M>& C, const SphereSet& S, V3& p, V3& v) {
  bool pushed = false;
#pragma unroll
  for (int q = 0; q < M; ++q)
    if (q < C.ncached) pushed |= push_out<REF, FAST>(v3(C.cx[q], C.cy[q], C.cz[q]), C.r[q], C.r2[q], p, v);
  uint32_t more = C.rest;
  while (more) {
    const int k = __ffs(more) - 1;
    more &= more - 1u;
    const float4 c = S.c[k];
    pushed |= push_out<REF, FAST>(v3(c.x, c.y, c.z), c.w, S.r2[k], p, v);
  }
  return pushed;
}

template <bool REF, int NC, int M>
__device__ __forceinline__ void collide_fast(const SphereCache<M>& C, const SphereSet& S, V3& p, V3& v) {
  if (tests<NC>(C, p)) push_all<REF, NC>(C, S, p, v);
}

// Per-strand constants of a frame.
struct StrandConsts {
  V3 F;            // force per unit mass
  V3 h2F;          // h^2 F (DFTL: the force's part of a substep's displacement)
  float h, h2, inv_h, damping, neg_damping, lscale;
  bool fast;       // DFTL chain links under the FAST contract (hs_contract)
};

// ---- reference mode: world coordinates (cs_simulation.glsl) -----------

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

// Finishes point j after its chain link: velocity (the next point's
// correction damped, the tip its own, :116-121), push-out with reflection
// (:129-153), store.
template <int NC, typename XS, typename VS, int M>
__device__ __forceinline__ void finish_point_ref(const StrandConsts& K, const SphereCache<M>& C, const SphereSet& S,
                                                 V3 q, bool hit, V3 corr_next, float rest, bool tip, V3 corr_own,
                                                 const XS& X, const VS& V, int j) {
  V3 v = tip ? corr_own : mul(corr_next, K.damping);
  if (hit) push_all<true, NC>(C, S, q, v);
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
template <int NC, typename XS, typename VS, int M>
__device__ __forceinline__ void substep_single_pass_ref(const StrandConsts& K, const SphereCache<M>& C,
                                                        const SphereSet& S, int n, V3 p0, const XS& X, const VS& V) {
  V3 nprev = v3(0.0f, -1.0f, 0.0f);
  // Link 1.
  const float4 v1 = V.load(1);
  const float4 x1 = with_rest<XS>(X.load(1), v1);
  V3 corr_prev;
  V3 prev = link(K, p0, predict(K, x1, v1), x1.w, nprev, corr_prev);
  float rest_prev = x1.w;
  if (n >= 3) {
    const float4 v2 = V.load(2);
    float4 xc = with_rest<XS>(X.load(2), v2);
    V3 p_cur = predict(K, xc, v2);
    typename VS::Pending pend{};
    if constexpr (VS::kPrefetch) {
      if (n > 3) pend = V.issue(3);
    }
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
      finish_point_ref<NC>(K, C, S, prev, hit, corr, rest_prev, false, corr_prev, X, V, i - 1);
      prev = pc;
      corr_prev = corr;
      rest_prev = xc.w;
      xc = xn;
      p_cur = p_next;
    }
    // Link n-1 and point n-2.
    V3 corr;
    const V3 pc = link(K, prev, p_cur, xc.w, nprev, corr);
    const bool hit = tests<NC>(C, prev);
    finish_point_ref<NC>(K, C, S, prev, hit, corr, rest_prev, false, corr_prev, X, V, n - 2);
    prev = pc;
    corr_prev = corr;
    rest_prev = xc.w;
  }
  // The tip keeps its own correction (:116).
  const bool hit = tests<NC>(C, prev);
  finish_point_ref<NC>(K, C, S, prev, hit, v3(0.0f, 0.0f, 0.0f), rest_prev, true, corr_prev, X, V, n - 1);
}

// One substep with several constraint iterations (reference mode: 8): a
// predict pass, then one pass per iteration.
template <int NC, typename XS, typename VS, int M>
__device__ __forceinline__ void substep_multi_pass_ref(const StrandConsts& K, const SphereCache<M>& C,
                                                       const SphereSet& S, int n, int iterations, V3 p0, const XS& X,
                                                       const VS& V) {
  for (int i = 1; i < n; ++i) {
    const float4 vi = V.load(i);
    const float4 xi = with_rest<XS>(X.load(i), vi);
    X.store(i, f4(fmas(K.h2, K.F, fmas(K.h, xyz(vi), xyz(xi))), xi.w));
  }
  V.fence();
  for (int it = 0; it < iterations; ++it) {
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
        V3 v = tip ? corr_prev : mul(corr, K.damping);
        collide_fast<true, NC>(C, S, q, v);
        V.store(i - 1, f4(v, vel_w<XS>(rest_prev)));
        X.store(i - 1, f4(q, rest_prev));
      }
      prev = pc;
      corr_prev = corr;
      rest_prev = rest_i;
    }
    V.fence();
  }
}

// ---- DFTL mode: segment form (see hs_step.cuh) ---------------------------

// Within a frame the velocity slots of the DFTL passes carry u = h v (the
// frame's load scales by h, its store by 1/h: frame_velocity): a substep's
// displacement from prediction is D = u + h^2 F, and a finished point's
// slot takes fma(-damping, e, D) as it is, where v would need a multiply
// by 1/h at every point-substep.
__device__ __forceinline__ V3 disp(const StrandConsts& K, float4 u) { return add(xyz(u), K.h2F); }
__device__ __forceinline__ V3 vel_of(const StrandConsts&, V3 x) { return x; }
// A velocity slot at a frame's start (LOAD: h v) or end (u / h), where the
// slots carry u (SCALE: the DFTL passes; w kept).
template <bool SCALE, bool LOAD>
__device__ __forceinline__ float4 frame_velocity(const FrameConst& fc, float4 v) {
  if constexpr (!SCALE) {
    return v;
  } else {
    const float f = LOAD ? fc.h : fc.inv_h;
    return make_float4(__fmul_rn(f, v.x), __fmul_rn(f, v.y), __fmul_rn(f, v.z), v.w);
  }
}

// Chain link in the segment form: d is the point's offset from its leader
// (already moved), s' = (L * inversesqrt(d.d)) d, e = s' - d.
// FAST: the hardware reciprocal square root (the FAST contract).
template <bool FAST = false>
__device__ __forceinline__ void link_seg(const StrandConsts& K, V3 d, float rest, V3& sn, V3& e) {
  const float d2 = dot(d, d);
  const float sc = __fmul_rn(__fmul_rn(K.lscale, rest), FAST ? rsqrt_fast(d2) : inversesqrt(d2));
  sn = mul(sc, d);
  e = sub(sn, d);
}

// Push-out of one point against the spheres of `reach`, in index order,
// read from shared memory: the exact in-order push of push_all (the cached
// spheres are copies of the same entries, taken in index order), as one
// small loop rather than push_all's unrolled cache.
struct Pushed {
  V3 p;
  bool pushed;
};
template <bool FAST = false>
__device__ __forceinline__ Pushed push_mask(uint32_t reach, const float4* c, const float* r2, V3 p) {
  bool pushed = false;
  V3 unused = v3(0.0f, 0.0f, 0.0f);
  while (reach) {
    const int k = __ffs(reach) - 1;
    reach &= reach - 1u;
    const float4 ck = c[k];
    pushed |= push_out<false, FAST>(v3(ck.x, ck.y, ck.z), ck.w, r2[k], p, unused);
  }
  return Pushed{p, pushed};
}
// Push-out of point j at its chain position w: a push by g moves D_j and
// s_j by +g and the next segment by -g (none at the tip). CACHED: the
// in-order push from the register cache (push_all, unrolled over its
// slots: more code, fewer instructions a push), for grooms among many
// spheres that push at most points; else the small loop of push_mask.
// FAST: the push-out of the FAST contract (push_out).
template <bool CACHED, int NC, bool FAST = false, int M>
__device__ __forceinline__ void push_seg(const SphereCache<M>& C, const SphereSet& S, V3 w, V3& D, V3& s,
                                         V3& s_next, bool tip) {
  Pushed r{w, false};
  if constexpr (CACHED) {
    V3 unused = v3(0.0f, 0.0f, 0.0f);
    r.pushed = push_all<false, NC, FAST>(C, S, r.p, unused);
  } else {
    r = push_mask<FAST>(C.reach, S.c, S.r2, w);
  }
  if (r.pushed) {
    const V3 g = sub(r.p, w);
    D = add(D, g);
    s = add(s, g);
    if (!tip) s_next = sub(s_next, g);
  }
}

// Iteration i of the single pass (2 <= i <= n - 2): uses point i's loads
// (a_cur = s_i + D_i, dp_cur, rest_cur), loads point i + 1, runs link i,
// finishes point i - 1, testing it against the spheres if TEST and
// i - 1 >= jmin.
template <bool TEST, bool CACHED, int NC, bool FAST, typename XS, typename VS, int M>
struct SegPass {
  const StrandConsts& K;
  const SphereCache<M>& C;
  const SphereSet& S;
  const XS& X;
  const VS& V;
  int n, jmin;
  V3 D_prev, w_prev, s_prev, a_cur, dp_cur;
  float rest_prev, rest_cur;
  typename VS::Pending pend;
  __device__ __forceinline__ void step(int i) {
    const float4 xr = X.load(i + 1);
    float4 vn;
    if constexpr (VS::kPrefetch) {
      vn = V.complete(pend);
      if (i + 2 < n) pend = V.issue(i + 2);
    } else {
      vn = V.load(i + 1);
    }
    const float4 xn = with_rest<XS>(xr, vn);
    const V3 dp_next = disp(K, vn);
    const V3 a_next = add(xyz(xn), dp_next);
    V3 sn, e;
    link_seg<FAST>(K, sub(a_cur, D_prev), rest_cur, sn, e);
    const V3 D_i = add(dp_cur, e);
    const V3 w_i = add(w_prev, sn);
    if (TEST && i - 1 >= jmin && tests<NC>(C, w_prev))
      push_seg<CACHED, NC, FAST>(C, S, w_prev, D_prev, s_prev, sn, false);
    X.store(i - 1, f4(s_prev, rest_prev));
    V.store(i - 1, f4(vel_of(K, fmas(K.neg_damping, e, D_prev)), vel_w<XS>(rest_prev)));
    s_prev = sn;
    D_prev = D_i;
    w_prev = w_i;
    rest_prev = rest_cur;
    a_cur = a_next;
    dp_cur = dp_next;
    rest_cur = xn.w;
  }
};

// One substep with one constraint iteration, one pass. Iteration i loads
// point i+1 (its segment plus displacement, independent of the chain),
// runs link i (d = (s_i + D_i) - D_{i-1}, the loop-carried path), and
// finishes point i-1: tests at its chain position, push-out, Eq. 9
// velocity v = fma(-damping, e_i, D_{i-1}) / h, stores. Points below jmin
// cannot reach a sphere this frame (strand_frame_stream) and skip the
// tests. Measured code shapes (the hot loop must stay in the instruction
// cache): SPLIT, a loop without tests up to jmin then one with them, else
// one loop with the jmin check; CACHED (8-wide cache only): the push from
// the register cache (push_seg).
template <int NC, bool SPLIT, bool CACHED, bool FAST, typename XS, typename VS, int M>
__device__ __forceinline__ void substep_single_pass_seg(const StrandConsts& K, const SphereCache<M>& C,
                                                        const SphereSet& S, int n, int jmin, V3 D0, V3 R,
                                                        const XS& X, const VS& V) {
  constexpr bool kSplit = SPLIT;
  constexpr bool kCached = CACHED && M > kCachedSpheres;
  // Link 1.
  const float4 v1 = V.load(1);
  const float4 x1 = with_rest<XS>(X.load(1), v1);
  const V3 dp1 = disp(K, v1);
  V3 sn, e;
  link_seg<FAST>(K, sub(add(xyz(x1), dp1), D0), x1.w, sn, e);
  V3 D_prev = add(dp1, e);
  V3 w_prev = add(R, sn);
  V3 s_prev = sn;
  float rest_prev = x1.w;
  if (n >= 3) {
    const float4 v2 = V.load(2);
    const float4 x2 = with_rest<XS>(X.load(2), v2);
    const V3 dp2 = disp(K, v2);
    SegPass<!kSplit, kCached, NC, FAST, XS, VS, M> A{K, C, S, X, V, n, jmin, D_prev, w_prev, s_prev,
                                               add(xyz(x2), dp2), dp2, rest_prev, x2.w, {}};
    if constexpr (VS::kPrefetch) {
      if (n > 3) A.pend = V.issue(3);
    }
    int i = 2;
    if constexpr (kSplit) {
      // Iterations finishing points below jmin: no tests.
      const int ia = min(max(jmin + 1, 2), n - 1);
      // Unrolled by two so the carried values change registers instead of
      // being copied each iteration.
#pragma unroll 2
      for (; i < ia; ++i) A.step(i);
    }
    SegPass<true, kCached, NC, FAST, XS, VS, M> B{K, C, S, X, V, n, jmin, A.D_prev, A.w_prev, A.s_prev, A.a_cur,
                                            A.dp_cur, A.rest_prev, A.rest_cur, A.pend};
#pragma unroll 2
    for (; i < n - 1; ++i) B.step(i);
    // Link n-1 and point n-2.
    link_seg<FAST>(K, sub(B.a_cur, B.D_prev), B.rest_cur, sn, e);
    const V3 D_i = add(B.dp_cur, e);
    const V3 w_i = add(B.w_prev, sn);
    D_prev = B.D_prev;
    s_prev = B.s_prev;
    if (n - 2 >= jmin && tests<NC>(C, B.w_prev))
      push_seg<kCached, NC, FAST>(C, S, B.w_prev, D_prev, s_prev, sn, false);
    X.store(n - 2, f4(s_prev, B.rest_prev));
    V.store(n - 2, f4(vel_of(K, fmas(K.neg_damping, e, D_prev)), vel_w<XS>(B.rest_prev)));
    s_prev = sn;
    D_prev = D_i;
    w_prev = w_i;
    rest_prev = B.rest_cur;
  }
  // The tip: no next correction, v = D / h.
  if (n - 1 >= jmin && tests<NC>(C, w_prev)) push_seg<kCached, NC, FAST>(C, S, w_prev, D_prev, s_prev, sn, true);
  X.store(n - 1, f4(s_prev, rest_prev));
  V.store(n - 1, f4(vel_of(K, D_prev), vel_w<XS>(rest_prev)));
}

// One substep with several constraint iterations: a predict pass (the
// velocity slots take D_i), then one pass per iteration. The first
// iteration's link is d = (s_i + D_i) - D_{i-1} (as in the single pass),
// later ones d = s_i - e_{i-1} (e: that iteration's correction of the
// leader); the last pass forms the velocities.
template <int NC, bool FAST, typename XS, typename VS, int M>
__device__ __forceinline__ void substep_multi_pass_seg(const StrandConsts& K, const SphereCache<M>& C,
                                                       const SphereSet& S, int n, int iterations, V3 D0, V3 R,
                                                       const XS& X, const VS& V) {
  for (int i = 1; i < n; ++i) {
    const float4 v = V.load(i);
    V.store(i, f4(disp(K, v), v.w));
  }
  V.fence();
  const V3 zero = v3(0.0f, 0.0f, 0.0f);
  for (int it = 0; it < iterations; ++it) {
    const bool last = it + 1 == iterations;
    V3 D_prev = D0, e_prev = zero, w_prev = R, s_prev = zero;
    float rest_prev = 0.0f;
    for (int i = 1; i <= n; ++i) {
      V3 sn = zero, e = zero, D_i = zero, w_i = zero;
      float rest_i = 0.0f;
      if (i < n) {
        const float4 vd = V.load(i);
        const float4 x = with_rest<XS>(X.load(i), vd);
        rest_i = x.w;
        const V3 d = it == 0 ? sub(add(xyz(x), xyz(vd)), D_prev) : sub(xyz(x), e_prev);
        link_seg<FAST>(K, d, rest_i, sn, e);
        D_i = add(xyz(vd), e);
        w_i = add(w_prev, sn);
      }
      if (i >= 2) {
        const bool tip = i == n;
        V3 Dj = D_prev, sj = s_prev;
        if (tests<NC>(C, w_prev)) push_seg<false, NC, FAST>(C, S, w_prev, Dj, sj, sn, tip);
        const V3 out = last ? vel_of(K, tip ? Dj : fmas(K.neg_damping, e, Dj)) : Dj;
        X.store(i - 1, f4(sj, rest_prev));
        V.store(i - 1, f4(out, vel_w<XS>(rest_prev)));
      }
      D_prev = D_i;
      e_prev = e;
      w_prev = w_i;
      s_prev = sn;
      rest_prev = rest_i;
    }
    V.fence();
  }
}

// ---- the frame ------------------------------------------------------------

// Per-strand constants of a frame: force per unit mass, gravity
// (CalculateForces, :70-77) plus the wind with its per-strand jitter. The
// jitter hashes the caller's strand index (the library stores strands in
// its own order).
__device__ __forceinline__ StrandConsts strand_consts(const FrameConst& fc, const GroomView& g, uint32_t s,
                                                      bool active) {
  StrandConsts K;
  const float u = hash_u01(fc.wind_key, g.strand_base + (active ? g.order[s] : s));
  const float j = __fadd_rn(1.0f, __fmul_rn(fc.wind_jitter, __fsub_rn(1.0f, __fmul_rn(2.0f, u))));
  K.F = v3(__fmaf_rn(j, fc.wx, fc.Gx), __fmaf_rn(j, fc.wy, fc.Gy), __fmaf_rn(j, fc.wz, fc.Gz));
  K.h = fc.h;
  K.h2 = fc.h2;
  K.h2F = mul(fc.h2, K.F);
  K.inv_h = fc.inv_h;
  K.damping = fc.damping;
  K.neg_damping = -fc.damping;
  K.lscale = fc.length_scale;
  K.fast = fc.contract == HS_CONTRACT_FAST;
  return K;
}

// The root's position at the end of the frame: the rest root moved by the
// groom's transform (RIGID) or skinned by its bones (SKINNED), the
// caller's target (EXPLICIT), else where it starts.
__device__ __forceinline__ V3 root_target(const FrameConst& fc, const GroomView& g, uint32_t s, bool active,
                                          V3 x0_start) {
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
  return target;
}

template <bool REF, int NC, bool SPLIT, bool CACHED, bool FAST, typename XS, typename VS, int M>
__device__ __forceinline__ void substeps(const FrameConst& fc, const StrandConsts& K, const SphereCache<M>& C,
                                         const SphereSet& S, int n, int jmin, V3 x0_start, V3 target, float rest0,
                                         const XS& X, const VS& V) {
  const bool moving = fc.root_mode != HS_ROOT_PINNED;
  if constexpr (REF) {
    const V3 root_delta = sub(target, x0_start);
    V3 root = x0_start;  // root position at the start of the substep
    for (int k = 0; k < fc.substeps; ++k) {
      // Root (:184-193): kinematic, linear to its target, on it at the end.
      V3 p0 = root;
      if (moving) {
        const float alpha = __fdiv_rn(static_cast<float>(k + 1), static_cast<float>(fc.substeps));
        p0 = (k + 1 == fc.substeps) ? target : fmas(alpha, root_delta, x0_start);
      }
      const V3 v0 = sub(p0, root);  // :192
      root = p0;
      X.store(0, f4(p0, rest0));
      V.store(0, f4(v0, vel_w<XS>(rest0)));
      if (n >= 2) {
        if (fc.iterations == 1) substep_single_pass_ref<NC>(K, C, S, n, p0, X, V);
        else substep_multi_pass_ref<NC>(K, C, S, n, fc.iterations, p0, X, V);
      }
      V.fence();
    }
  } else {
    // Root offsets from the frame's start: rel_k = alpha_k delta (delta
    // itself at the last substep), D_0 = rel_k - rel_{k-1}.
    const V3 delta = sub(target, x0_start);
    const V3 zero = v3(0.0f, 0.0f, 0.0f);
    V3 rel_prev = zero, D0 = zero;
    for (int k = 0; k < fc.substeps; ++k) {
      V3 rel = zero, R = x0_start;
      if (moving) {
        const bool last = k + 1 == fc.substeps;
        const float alpha = __fdiv_rn(static_cast<float>(k + 1), static_cast<float>(fc.substeps));
        rel = last ? delta : mul(alpha, delta);
        R = last ? target : add(x0_start, rel);
      }
      D0 = sub(rel, rel_prev);
      rel_prev = rel;
      if (n >= 2) {
        if (fc.iterations == 1) substep_single_pass_seg<NC, SPLIT, CACHED, FAST>(K, C, S, n, jmin, D0, R, X, V);
        else substep_multi_pass_seg<NC, FAST>(K, C, S, n, fc.iterations, D0, R, X, V);
      }
      V.fence();
    }
    X.store(0, f4(zero, rest0));
    V.store(0, f4(vel_of(K, D0), vel_w<XS>(rest0)));
    V.fence();
  }
}

// One frame of strand s. X: the position/segment slots (XShared4 or
// XShared3, this thread's column of the block's shared [point][thread]
// arrays); V: the velocity slots (VShared, or VTmem: whose loads and stores
// are warp-collective, so every lane runs every pass, active or not).
// M: sphere-cache width. With M = 8 a warp that reaches more than
// kCachedSpheres spheres tests 8 cached ones instead of running the exact
// push-out at every point; the others keep the 4-wide tests.
// SPLIT: the DFTL pass shape (substep_single_pass_seg). One code shape per
// kernel keeps the instruction cache warm: the batched kernels (4-wide
// cache) run one loop; the plain step, whose 8-wide path splits, splits
// both. CACHED: see push_seg (the plain step picks it for grooms with more
// than 16 spheres).
template <bool REF, typename XS, typename VS, int M = kCachedSpheres, bool SPLIT = (M > kCachedSpheres),
          bool CACHED = false, bool FAST = false>
__device__ __forceinline__ void strand_frame_stream(const FrameConst& fc, const SphereSet& S, const GroomView& g,
                                                    uint32_t s, bool active, const XS& X, const VS& V) {
  const int n = static_cast<int>(g.npoints);
  float R = 0.0f;  // total link length, for culling
  float rest0 = 0.0f;
  V3 x0_start = v3(0.0f, 0.0f, 0.0f);
  V3 last = x0_start;  // previous point (DFTL: segments are differences)
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
        float4 xs = p[k];
        if (i == 0) {
          x0_start = xyz(p[k]);
          rest0 = p[k].w;
        }
        if (!REF) {
          xs = f4(i == 0 ? v3(0.0f, 0.0f, 0.0f) : sub(xyz(p[k]), last), p[k].w);
          last = xyz(p[k]);
        }
        X.store(i, xs);
        const float4 vk = frame_velocity<!REF, true>(fc, v[k]);
        V.store(i, make_float4(vk.x, vk.y, vk.z, XS::kRestInV ? p[k].w : v[k].w));
        if (i > 0) R += fabsf(fc.length_scale * p[k].w);
      }
    }
  }
  V.fence();

  const StrandConsts K = strand_consts(fc, g, s, active);
  const V3 target = root_target(fc, g, s, active, x0_start);

  // Spheres this warp can touch during the frame (see hs_step.cuh), and
  // the first point that can touch one: point j stays within R_j (its
  // links' lengths summed from the root) of the root, so it cannot reach
  // sphere k before R_j covers the distance from the root's path to k's
  // surface (same margins as near_spheres). A sphere reached only through
  // an overlap is entered by a point another sphere pushed first.
  uint32_t reach = 0u;
  int jmin = n;
  if (S.n > 0) {
    const V3 root_delta = sub(target, x0_start);
    const V3 mid = v3(0.5f * (x0_start.x + target.x), 0.5f * (x0_start.y + target.y), 0.5f * (x0_start.z + target.z));
    const float half_path = 0.5f * sqrtf(root_delta.x * root_delta.x + root_delta.y * root_delta.y +
                                         root_delta.z * root_delta.z);
    // Per lane: each thread caches the spheres its own strand can reach, so
    // a warp whose strands lie far apart (a mesh's vertex order, or any
    // order) tests no more than spatially coherent ones do.
    reach = active ? overlap_closure(S, near_spheres(S, mid, R + half_path)) : 0u;
    const float thr = reach_threshold(S, mid, R + half_path, half_path);
    float Rj = 0.0f;
    int jl = n;
    for (int i = 1; i < n; ++i) {  // the same sum as R, point by point
      const float rest = with_rest<XS>(X.load(i), V.load(i)).w;
      Rj += fabsf(fc.length_scale * rest);
      if (jl == n && Rj >= thr) jl = i;
    }
    jmin = __reduce_min_sync(0xffffffffu, active ? jl : n);
  }
  const SphereCache<M> C = cache_spheres<M>(S, reach);
  // One code path per cache width: all tested slots are tested whether
  // filled or not (empty ones never hit). A second path without sphere
  // tests saved their cost for warps that reach no sphere, but warps on
  // different paths at once thrashed the instruction cache of the batched
  // kernels (measured: one path is 13-16 % faster on the batched workload
  // and no slower on a single groom). The width is chosen per warp.
  const int warp_cached = __reduce_max_sync(0xffffffffu, C.ncached);
  if (M > kCachedSpheres && warp_cached > kCachedSpheres)
    substeps<REF, M, SPLIT, CACHED, FAST>(fc, K, C, S, n, jmin, x0_start, target, rest0, X, V);
  else
    substeps<REF, kCachedSpheres, SPLIT, CACHED, FAST>(fc, K, C, S, n, jmin, x0_start, target, rest0, X, V);

  // Store: reference mode holds positions; DFTL mode rebuilds them from the
  // final root and the segments.
  const bool moving = fc.root_mode != HS_ROOT_PINNED;
  V3 w = moving ? target : x0_start;
  TileStats ts;
  ts.init();
  for (int i = 0; i < n; ++i) {
    const float4 vs = V.load(i);
    if (active) {
      float4 x = with_rest<XS>(X.load(i), vs);
      const float4 v = frame_velocity<!REF, false>(fc, vs);
      if (!REF) {
        if (i > 0) w = add(w, xyz(x));
        x = f4(w, x.w);
      }
      g.pos[static_cast<size_t>(i) * g.stride + s] = x;
      g.vel[static_cast<size_t>(i) * g.stride + s] = make_float4(v.x, v.y, v.z, 0.0f);
      ts.add(x, v);
    }
  }
  ts.store(g.stats, s / 32u, (g.nstrands + 31u) / 32u, static_cast<int>(threadIdx.x % 32u));
}

// Register form of a DFTL frame (short strands): the segments in
// registers, the velocity slots (then displacements) in registers or
// shared rows (VStore, hs_step.cuh). The passes of substep_multi_pass_seg,
// unrolled over CAP; with one iteration they compute what
// substep_single_pass_seg does, operation for operation.
template <int CAP, bool VSMEM, bool FAST = false>
__device__ __forceinline__ void strand_frame_regs_dftl(const FrameConst& fc, const SphereSet& S, const GroomView& g,
                                                       uint32_t s, bool active, float4* vs_rows, int thread) {
  const int n = static_cast<int>(g.npoints);
  const V3 zero = v3(0.0f, 0.0f, 0.0f);
  V3 Sg[CAP];
  VStore<CAP, VSMEM> vs;
  vs.bind(vs_rows, thread);
  float R = 0.0f, rest0 = 0.0f;
  V3 x0_start = zero, last = zero;
#pragma unroll
  for (int i = 0; i < CAP; ++i) {
    Sg[i] = zero;
    if (i < n) {
      float4 p = make_float4(0.0f, 0.0f, 0.0f, 0.0f), v = p;
      if (active) {
        p = g.pos[static_cast<size_t>(i) * g.stride + s];
        v = g.vel[static_cast<size_t>(i) * g.stride + s];
      }
      if (i == 0) {
        x0_start = xyz(p);
        rest0 = p.w;
      } else {
        Sg[i] = sub(xyz(p), last);
        R += fabsf(fc.length_scale * p.w);
      }
      last = xyz(p);
      const float4 vin = frame_velocity<true, true>(fc, v);
      vs.set(i, make_float4(vin.x, vin.y, vin.z, p.w));
    }
  }

  const StrandConsts K = strand_consts(fc, g, s, active);
  const V3 target = root_target(fc, g, s, active, x0_start);
  const bool moving = fc.root_mode != HS_ROOT_PINNED;
  uint32_t reach = 0u;
  if (S.n > 0) {
    const V3 root_delta = sub(target, x0_start);
    const V3 mid = v3(0.5f * (x0_start.x + target.x), 0.5f * (x0_start.y + target.y), 0.5f * (x0_start.z + target.z));
    const float half_path = 0.5f * sqrtf(root_delta.x * root_delta.x + root_delta.y * root_delta.y +
                                         root_delta.z * root_delta.z);
    reach = active ? overlap_closure(S, near_spheres(S, mid, R + half_path)) : 0u;  // per lane
  }
  const SphereCache<kCachedSpheres> C = cache_spheres<kCachedSpheres>(S, reach);

  const V3 delta = sub(target, x0_start);
  V3 rel_prev = zero, D0 = zero;
  for (int k = 0; k < fc.substeps; ++k) {
    V3 rel = zero, Rk = x0_start;
    if (moving) {
      const bool lastk = k + 1 == fc.substeps;
      const float alpha = __fdiv_rn(static_cast<float>(k + 1), static_cast<float>(fc.substeps));
      rel = lastk ? delta : mul(alpha, delta);
      Rk = lastk ? target : add(x0_start, rel);
    }
    D0 = sub(rel, rel_prev);
    rel_prev = rel;
#pragma unroll
    for (int i = 1; i < CAP; ++i) {
      if (i < n) {
        const float4 sl = vs.get(i);
        vs.set(i, f4(disp(K, sl), sl.w));
      }
    }
    for (int it = 0; it < fc.iterations; ++it) {
      const bool last_it = it + 1 == fc.iterations;
      V3 D_prev = D0, e_prev = zero, w_prev = Rk, s_prev = zero;
      float rest_prev = 0.0f;
#pragma unroll
      for (int i = 1; i <= CAP; ++i) {
        if (i <= n) {
          V3 sn = zero, e = zero, D_i = zero, w_i = zero;
          float rest_i = 0.0f;
          if (i < CAP && i < n) {
            const float4 sl = vs.get(i);
            rest_i = sl.w;
            const V3 d = it == 0 ? sub(add(Sg[i], xyz(sl)), D_prev) : sub(Sg[i], e_prev);
            link_seg<FAST>(K, d, rest_i, sn, e);
            D_i = add(xyz(sl), e);
            w_i = add(w_prev, sn);
          }
          if (i >= 2) {
            const bool tip = i == n;
            V3 Dj = D_prev, sj = s_prev;
            if (tests<kCachedSpheres>(C, w_prev))
              push_seg<false, kCachedSpheres, FAST>(C, S, w_prev, Dj, sj, sn, tip);
            const V3 out = last_it ? vel_of(K, tip ? Dj : fmas(K.neg_damping, e, Dj)) : Dj;
            Sg[i - 1] = sj;
            vs.set(i - 1, f4(out, rest_prev));
          }
          D_prev = D_i;
          e_prev = e;
          w_prev = w_i;
          s_prev = sn;
          rest_prev = rest_i;
        }
      }
    }
  }
  vs.set(0, f4(vel_of(K, D0), rest0));

  TileStats ts;
  ts.init();
  if (active) {
    V3 w = moving ? target : x0_start;
#pragma unroll
    for (int i = 0; i < CAP; ++i) {
      if (i < n) {
        const float4 v = frame_velocity<true, false>(fc, vs.get(i));
        if (i > 0) w = add(w, Sg[i]);
        const float4 x = f4(w, v.w);
        g.pos[static_cast<size_t>(i) * g.stride + s] = x;
        g.vel[static_cast<size_t>(i) * g.stride + s] = make_float4(v.x, v.y, v.z, 0.0f);
        ts.add(x, v);
      }
    }
  }
  ts.store(g.stats, s / 32u, (g.nstrands + 31u) / 32u, static_cast<int>(threadIdx.x % 32u));
}

}  // namespace hs
