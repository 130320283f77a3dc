// hair_oracle.cc -- CPU restatement of the hair-strand simulation step.
//
// TEST INFRASTRUCTURE ONLY. This file is the checker: tests/ compare the
// CUDA library against it, and bench.py times its FP32 instantiation as the
// CPU baseline. The library never links, loads or calls it.
//
// What it restates, and where parity comes from:
//  * HS_MODE_REFERENCE follows src/shaders/hair/01_simulation/cs_simulation.glsl
//    line by line (:53-66 pack/unpack, :70-77 forces, :93-127 the FTL
//    DistanceConstraint with its tip-ward velocity shift, :129-153 sphere
//    push-out, :155-161 the iteration loop, :170-207 main). Its FP32
//    instantiation is PINNED against that shader's own text compiled as C++
//    (oracle/ref_glsl, golden vectors in tests/golden/): bit for bit.
//  * HS_MODE_DFTL (substeps, wind, many spheres, Eq. 9 velocity, moving
//    roots) is written from Mueller et al. 2012, "Fast Simulation of
//    Inextensible Hair and Fur" (cited by the reference at README.md:98).
//    The reference has no such code: that mode's parity is unpinned.
//  * init follows src/fx/hair.cc:262-288, with the time-seeded rand()
//    (src/core/app.cc:96-97) replaced by a seeded counter hash.
//
// Layout follows the reference's position/velocity streams: float4 per
// control point, strand-major, point i of strand s at index s*N + i
// (src/fx/hair.cc:242-288, src/shaders/hair/interop.h:13-16).
//
// Arithmetic contract (the CUDA kernels follow the same one, which is what
// makes the FP32 comparison exact):
//   dot(a,b)       = fma(a.z,b.z, fma(a.y,b.y, a.x*b.x))
//   inversesqrt(x) = FP32: magic-constant estimate (C. Lomont, "Fast Inverse
//                    Square Root", 2003), two Newton-Raphson steps
//                    y *= 1.5 - (x/2) y^2, then y += (y/2)(1 - x y^2) with the
//                    residual by fma; < 1 ulp, within GLSL's 2-ulp bound.
//                    FP64: 1 / sqrt(x), the accuracy reference.
//   normalize(v)   = v * inversesqrt(dot(v,v)); if dot == 0, reference mode
//                    takes the previous link's direction (first link:
//                    (0,-1,0)) and DFTL mode the zero vector. The reference
//                    yields NaN there; both are documented choices.
// DFTL mode in FP32 runs in the segment form (frame_strand_seg), which
// keeps world coordinates out of the per-substep arithmetic.
//   reflect(I,N)   = I - (2*dot(N,I)) * N
// All other vector ops are per component and unfused unless written fma.
// Build with -ffp-contract=off so the compiler adds no fusion of its own.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <type_traits>
#include <vector>

#include "hairsim.h"

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

template <typename T>
struct V3 {
  T x, y, z;
};

template <typename T>
inline V3<T> add(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <typename T>
inline V3<T> sub(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <typename T>
inline V3<T> mul(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <typename T>
inline V3<T> mul(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
// fma(a, b, c) with a scalar a and vectors b, c.
template <typename T>
inline V3<T> fmas(T a, V3<T> b, V3<T> c) {
  return {std::fma(a, b.x, c.x), std::fma(a, b.y, c.y), std::fma(a, b.z, c.z)};
}
template <typename T>
inline T dot(V3<T> a, V3<T> b) { return std::fma(a.z, b.z, std::fma(a.y, b.y, a.x * b.x)); }
inline double inversesqrt(double x) { return 1.0 / std::sqrt(x); }
inline float inversesqrt(float x) {
  uint32_t i;
  std::memcpy(&i, &x, sizeof(i));
  i = 0x5f3759dfu - (i >> 1);
  float y;
  std::memcpy(&y, &i, sizeof(y));
  const float hx = 0.5f * x;
  for (int k = 0; k < 2; ++k) y = y * std::fma(-hx, y * y, 1.5f);
  const float r = std::fma(-(x * y), y, 1.0f);
  return std::fma(0.5f * y, r, y);
}
template <typename T>
inline V3<T> reflect(V3<T> i, V3<T> n) { return sub(i, mul(T(2) * dot(n, i), n)); }

// Seeded counter hash (lowbias32, C. Wellons) standing in for rand().
inline uint32_t lowbias32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x;
}
inline uint32_t stream_key(uint64_t seed, uint32_t stream) {
  return lowbias32(static_cast<uint32_t>(seed) ^
                   lowbias32(static_cast<uint32_t>(seed >> 32) + 0x9E3779B9U * (stream + 1U)));
}
// u in [0,1), a multiple of 2^-24, exact in float and double.
template <typename T>
inline T hash_u01(uint32_t key, uint32_t idx) {
  return static_cast<T>(lowbias32(idx + key) >> 8) * static_cast<T>(1.0 / 16777216.0);
}
constexpr uint32_t kStreamLength = 1;
constexpr uint32_t kStreamWind = 2;

template <typename T>
struct SimT {
  int mode, substeps, iterations;
  T h, h2, inv_h;
  V3<T> G;  // gravity_scale * gravity
  T damping, length_scale, wind_jitter;
  V3<T> wind;
  int nspheres;
  V3<T> c[HS_MAX_SPHERES];
  T r[HS_MAX_SPHERES], r2[HS_MAX_SPHERES];
  uint32_t wind_key;
};

template <typename T>
bool make_sim(SimT<T>& S, const hs_sim_params* sp, uint64_t seed, float dt, const float* wind,
              uint32_t nspheres, const float* spheres) {
  if (!sp || sp->substeps < 1 || sp->iterations < 1 || nspheres > HS_MAX_SPHERES) return false;
  S.mode = static_cast<int>(sp->mode);
  S.substeps = static_cast<int>(sp->substeps);
  S.iterations = static_cast<int>(sp->iterations);
  S.h = static_cast<T>(dt) / static_cast<T>(sp->substeps);
  S.h2 = S.h * S.h;
  S.inv_h = T(1) / S.h;
  const T gs = sp->gravity_scale;
  S.G = {gs * T(sp->gravity[0]), gs * T(sp->gravity[1]), gs * T(sp->gravity[2])};
  S.damping = sp->damping;
  S.length_scale = sp->length_scale;
  S.wind_jitter = sp->wind_jitter;
  S.wind = wind ? V3<T>{T(wind[0]), T(wind[1]), T(wind[2])} : V3<T>{T(0), T(0), T(0)};
  S.nspheres = static_cast<int>(nspheres);
  for (uint32_t k = 0; k < nspheres; ++k) {
    S.c[k] = {T(spheres[4 * k + 0]), T(spheres[4 * k + 1]), T(spheres[4 * k + 2])};
    S.r[k] = spheres[4 * k + 3];
    S.r2[k] = S.r[k] * S.r[k];
  }
  S.wind_key = stream_key(seed, kStreamWind);
  return true;
}

// CollideSphere(+1, c, r, p) of cs_simulation.glsl:129-139 for every sphere
// in order (the reference has one, :149-153). Updates p and, in reference
// mode, reflects v; returns whether any sphere pushed the point.
template <typename T>
inline bool collide(const SimT<T>& S, V3<T>& p, V3<T>& v, bool reflect_velocity) {
  bool pushed = false;
  for (int k = 0; k < S.nspheres; ++k) {
    const V3<T> pt = sub(p, S.c[k]);
    const T dp = dot(pt, pt);
    if (dp < S.r2[k]) {
      const V3<T> n = dp > T(0) ? mul(pt, inversesqrt(dp)) : V3<T>{T(0), T(1), T(0)};
      p = add(S.c[k], mul(S.r[k], n));
      if (reflect_velocity) v = reflect(v, n);
      pushed = true;
    }
  }
  return pushed;
}

// One frame of one strand in world coordinates. P, V: this strand's N
// float4 (strand-major). Reference mode always runs here; DFTL mode runs
// here in FP64 (the accuracy reference: Mueller et al.'s algorithm as
// written) and, for comparison, in FP32 (frame_strand_seg is the FP32
// contract of DFTL mode).
template <typename T>
void frame_strand(T* P, T* V, int N, const SimT<T>& S, uint32_t strand, const T* target) {
  V3<T> x[HS_MAX_POINTS_PER_STRAND], v[HS_MAX_POINTS_PER_STRAND];
  V3<T> p[HS_MAX_POINTS_PER_STRAND], corr[HS_MAX_POINTS_PER_STRAND];
  T l[HS_MAX_POINTS_PER_STRAND];
  for (int i = 0; i < N; ++i) {  // UnpackParticle (:53-61)
    x[i] = {P[4 * i + 0], P[4 * i + 1], P[4 * i + 2]};
    l[i] = P[4 * i + 3];
    v[i] = {V[4 * i + 0], V[4 * i + 1], V[4 * i + 2]};
  }
  const bool ref = S.mode == HS_MODE_REFERENCE;

  // Per-strand force: gravity (CalculateForces, :70-77) plus jittered wind.
  const T u = hash_u01<T>(S.wind_key, strand);
  const T j = T(1) + S.wind_jitter * (T(1) - T(2) * u);
  const V3<T> F = {std::fma(j, S.wind.x, S.G.x), std::fma(j, S.wind.y, S.G.y),
                   std::fma(j, S.wind.z, S.G.z)};
  const V3<T> x0_start = x[0];
  V3<T> tgt = x0_start;
  if (target) tgt = {target[0], target[1], target[2]};
  const V3<T> root_delta = sub(tgt, x0_start);

  for (int k = 0; k < S.substeps; ++k) {
    // Root (:184-193): kinematic. Moves linearly to its target over the frame.
    if (target) {
      const T alpha = static_cast<T>(k + 1) / static_cast<T>(S.substeps);
      p[0] = (k + 1 == S.substeps) ? tgt : fmas(alpha, root_delta, x0_start);
    } else {
      p[0] = x[0];
    }
    // Integrate (:179-183): p = fma(dt*dt, force, fma(dt, v, p)).
    for (int i = 1; i < N; ++i) p[i] = fmas(S.h2, F, fmas(S.h, v[i], x[i]));

    // SatisfyConstraints (:155-161).
    for (int it = 0; it < S.iterations; ++it) {
      // DistanceConstraint (:109-117): follow the leader, root to tip.
      V3<T> nprev = {T(0), T(-1), T(0)};
      for (int i = 1; i < N; ++i) {
        const V3<T> p1 = p[i];
        const V3<T> d = sub(p1, p[i - 1]);
        const T d2 = dot(d, d);
        // normalize(0): the previous link's direction in reference mode,
        // the zero vector in DFTL mode (the point lands on its leader).
        const V3<T> n = d2 > T(0) ? mul(d, inversesqrt(d2)) : (ref ? nprev : V3<T>{T(0), T(0), T(0)});
        nprev = n;
        p[i] = add(p[i - 1], mul(S.length_scale * l[i], n));
        corr[i] = sub(p[i], p1);
      }
      if (ref) {
        // :116 then :119-121: velocity := correction of the next point,
        // damped; the tip keeps its own correction.
        for (int i = 1; i < N - 1; ++i) v[i] = mul(corr[i + 1], S.damping);
        v[N - 1] = corr[N - 1];
      }
      // CollisionConstraint (:149-153): all but the root.
      for (int i = 1; i < N; ++i) collide(S, p[i], v[i], ref);
    }

    if (ref) {
      v[0] = sub(p[0], x[0]);  // :192
    } else {
      // Mueller 2012 Eq. 9, v_i = (p_i - x_i)/h - s * d_{i+1}/h, evaluated
      // as v_i = (p_i - y_i) * (1/h) with y_i = fma(s, d_{i+1}, x_i); the
      // tip has no d_{i+1} and uses y = x.
      v[0] = mul(sub(p[0], x[0]), S.inv_h);
      for (int i = 1; i < N; ++i) {
        const V3<T> y = (i + 1 < N) ? fmas(S.damping, corr[i + 1], x[i]) : x[i];
        v[i] = mul(sub(p[i], y), S.inv_h);
      }
    }
    for (int i = 0; i < N; ++i) x[i] = p[i];
  }
  for (int i = 0; i < N; ++i) {  // PackParticle (:63-66)
    P[4 * i + 0] = x[i].x;
    P[4 * i + 1] = x[i].y;
    P[4 * i + 2] = x[i].z;
    P[4 * i + 3] = l[i];
    V[4 * i + 0] = v[i].x;
    V[4 * i + 1] = v[i].y;
    V[4 * i + 2] = v[i].z;
    V[4 * i + 3] = T(0);
  }
}

// One frame of one strand in DFTL mode, segment form: the FP32 arithmetic
// contract of the library's DFTL kernels. The same algorithm as
// frame_strand (Mueller et al. 2012 with Eq. 9), carried in quantities
// whose magnitude is a segment or a substep's motion rather than a world
// coordinate: per point i >= 1 its segment s_i = p_i - p_{i-1} and, within
// a substep, its displacement D_i = p_i - x_i. World positions round at
// ~6e-8 |p| every operation; Eq. 9 divides position differences by h,
// so in world coordinates every substep injects ~6e-8 |p| / h of velocity
// noise, which the scheme integrates; here the same roundings are relative
// to segment lengths and displacements. Per substep k:
//   root offset rel_k = alpha_k * delta (delta = target - x0 at the last
//   substep exactly), D_0 = rel_k - rel_{k-1}, root R_k = x0 + rel_k
//   (the target at the last substep);
//   predict   D_i = fma(h, v_i, h^2 F);
//   chain, iteration 1: d = (s_i + D_i) - D_{i-1}; later iterations:
//             d = s_i - e_{i-1} (e: the iteration's correction of the
//             leader, 0 for the root); s_i' = (L_i * inversesqrt(d.d)) * d,
//             e_i = s_i' - d, D_i += e_i (L_i = uScaleFactor * rest length);
//   collide   each point at its chain position w_i = w_{i-1} + s_i'
//             (w_0 = R_k, the chain before any push); a pushed point moves
//             by g: D_i += g, s_i += g, s_{i+1} -= g;
//   velocity  v_i = fma(-damping, e_{i+1}, D_i) * (1/h) (tip: D_i / h),
//             v_0 = D_0 / h.
// Load: s_i = x_i - x_{i-1}. Store: p_0 = the root, p_i = p_{i-1} + s_i.
template <typename T>
void frame_strand_seg(T* P, T* V, int N, const SimT<T>& S, uint32_t strand, const T* target) {
  V3<T> s[HS_MAX_POINTS_PER_STRAND], v[HS_MAX_POINTS_PER_STRAND], D[HS_MAX_POINTS_PER_STRAND];
  V3<T> e[HS_MAX_POINTS_PER_STRAND + 1], sn[HS_MAX_POINTS_PER_STRAND];
  T l[HS_MAX_POINTS_PER_STRAND];
  const V3<T> zero = {T(0), T(0), T(0)};
  const V3<T> x0 = {P[0], P[1], P[2]};
  V3<T> xprev = x0;
  for (int i = 0; i < N; ++i) {
    const V3<T> xi = {P[4 * i + 0], P[4 * i + 1], P[4 * i + 2]};
    l[i] = P[4 * i + 3];
    // Within the frame v[] carries u = h v: the prediction is D = u + h^2 F
    // and a finished point's u is fma(-damping, e, D), without the divide
    // by h (the kernels' contract); v = u / h when the frame is stored.
    v[i] = mul(S.h, V3<T>{V[4 * i + 0], V[4 * i + 1], V[4 * i + 2]});
    s[i] = i > 0 ? sub(xi, xprev) : zero;
    xprev = xi;
  }
  const T u = hash_u01<T>(S.wind_key, strand);
  const T j = T(1) + S.wind_jitter * (T(1) - T(2) * u);
  const V3<T> F = {std::fma(j, S.wind.x, S.G.x), std::fma(j, S.wind.y, S.G.y),
                   std::fma(j, S.wind.z, S.G.z)};
  const V3<T> h2F = mul(S.h2, F);
  const bool moving = target != nullptr;
  const V3<T> tgt = moving ? V3<T>{target[0], target[1], target[2]} : x0;
  const V3<T> delta = sub(tgt, x0);
  V3<T> rel_prev = zero;
  for (int k = 0; k < S.substeps; ++k) {
    V3<T> rel = zero, root = x0;
    if (moving) {
      const T alpha = static_cast<T>(k + 1) / static_cast<T>(S.substeps);
      const bool last = k + 1 == S.substeps;
      rel = last ? delta : mul(alpha, delta);
      root = last ? tgt : add(x0, rel);
    }
    D[0] = sub(rel, rel_prev);
    rel_prev = rel;
    for (int i = 1; i < N; ++i) D[i] = add(v[i], h2F);
    e[0] = zero;
    e[N] = zero;
    for (int it = 0; it < S.iterations; ++it) {
      for (int i = 1; i < N; ++i) {
        const V3<T> d = it == 0 ? sub(add(s[i], D[i]), D[i - 1]) : sub(s[i], e[i - 1]);
        const T d2 = dot(d, d);
        // normalize(0) = 0: FP32's inversesqrt is finite at 0, so d = 0
        // gives s' = 0 unguarded (as the kernels compute it); FP64's is not.
        T sc = (S.length_scale * l[i]) * inversesqrt(d2);
        if (std::is_same<T, double>::value && !(d2 > T(0))) sc = T(0);
        sn[i] = mul(sc, d);
        e[i] = sub(sn[i], d);
        D[i] = add(D[i], e[i]);
        s[i] = sn[i];
      }
      V3<T> w = root;
      for (int i = 1; i < N; ++i) {
        w = add(w, sn[i]);
        V3<T> q = w, unused = zero;
        if (collide(S, q, unused, false)) {
          const V3<T> g = sub(q, w);
          D[i] = add(D[i], g);
          s[i] = add(s[i], g);
          if (i + 1 < N) s[i + 1] = sub(s[i + 1], g);
        }
      }
    }
    v[0] = D[0];
    for (int i = 1; i < N; ++i) v[i] = i + 1 < N ? fmas(-S.damping, e[i + 1], D[i]) : D[i];
  }
  for (int i = 0; i < N; ++i) v[i] = mul(v[i], S.inv_h);
  V3<T> w = tgt;
  for (int i = 0; i < N; ++i) {
    if (i > 0) w = add(w, s[i]);
    P[4 * i + 0] = w.x;
    P[4 * i + 1] = w.y;
    P[4 * i + 2] = w.z;
    P[4 * i + 3] = l[i];
    V[4 * i + 0] = v[i].x;
    V[4 * i + 1] = v[i].y;
    V[4 * i + 2] = v[i].z;
    V[4 * i + 3] = T(0);
  }
}

// Which restatement of DFTL mode runs: the library's contract (segment
// form in FP32, world form in FP64), or one form explicitly.
constexpr int kFormContract = 0;
constexpr int kFormWorld = 1;
constexpr int kFormSegment = 2;

template <typename T>
int frame_all(T* pos, T* vel, uint32_t nstrands, uint32_t npoints, uint32_t strand_base,
              const hs_sim_params* sp, uint64_t seed, float dt, const float* wind,
              uint32_t nspheres, const float* spheres, const T* root_targets, int nthreads, int form = kFormContract) {
  if (npoints < HS_MIN_POINTS_PER_STRAND || npoints > HS_MAX_POINTS_PER_STRAND) return 1;
  SimT<T> S;
  if (!make_sim(S, sp, seed, dt, wind, nspheres, spheres)) return 1;
  const int N = static_cast<int>(npoints);
  const int64_t ns = static_cast<int64_t>(nstrands);
  if (form == kFormContract) form = std::is_same<T, float>::value ? kFormSegment : kFormWorld;
  const bool seg = S.mode != HS_MODE_REFERENCE && form == kFormSegment;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
  for (int64_t s = 0; s < ns; ++s) {
    T* P = pos + s * N * 4;
    T* V = vel + s * N * 4;
    const uint32_t strand = strand_base + static_cast<uint32_t>(s);
    const T* tg = root_targets ? root_targets + 3 * s : nullptr;
    if (seg) frame_strand_seg<T>(P, V, N, S, strand, tg);
    else frame_strand<T>(P, V, N, S, strand, tg);
  }
  (void)nthreads;
  return 0;
}

// Hair::init_simulation, src/fx/hair.cc:262-288.
template <typename T>
int init_all(T* pos, T* vel, const float* roots, const float* normals, uint32_t nstrands,
             const hs_strand_params* sp) {
  if (!sp || sp->points_per_strand < HS_MIN_POINTS_PER_STRAND ||
      sp->points_per_strand > HS_MAX_POINTS_PER_STRAND)
    return 1;
  const int N = static_cast<int>(sp->points_per_strand);
  const uint32_t key = stream_key(sp->seed, kStreamLength);
  for (uint32_t s = 0; s < nstrands; ++s) {
    const V3<T> r = {T(roots[3 * s]), T(roots[3 * s + 1]), T(roots[3 * s + 2])};
    const V3<T> n = {T(normals[3 * s]), T(normals[3 * s + 1]), T(normals[3 * s + 2])};
    const T u = hash_u01<T>(key, sp->strand_base + s);
    const T rv = T(1) + T(sp->length_jitter) * (T(1) - T(2) * u);
    T* P = pos + static_cast<size_t>(s) * N * 4;
    T* V = vel + static_cast<size_t>(s) * N * 4;
    if (sp->length_rule == HS_LENGTH_REFERENCE) {
      const T scale_offset = T(sp->max_length) / static_cast<T>(N);
      T last = T(0);
      for (int i = 0; i < N; ++i) {
        const T offset = static_cast<T>(i) * scale_offset * rv;
        const V3<T> q = add(r, mul(offset, n));
        P[4 * i + 0] = q.x;
        P[4 * i + 1] = q.y;
        P[4 * i + 2] = q.z;
        P[4 * i + 3] = offset - last;
        last = offset;
      }
    } else {
      const T L = sp->lengths ? T(sp->lengths[s]) : T(sp->max_length) * rv;
      const T seg = L / static_cast<T>(N - 1);
      for (int i = 0; i < N; ++i) {
        const T offset = static_cast<T>(i) * seg;
        const V3<T> q = add(r, mul(offset, n));
        P[4 * i + 0] = q.x;
        P[4 * i + 1] = q.y;
        P[4 * i + 2] = q.z;
        P[4 * i + 3] = i == 0 ? T(0) : seg;
      }
    }
    for (int i = 0; i < 4 * N; ++i) V[i] = T(0);
  }
  return 0;
}

// Rigid root targets: t = M * r with M column-major,
// t.x = fma(m8, r.z, fma(m4, r.y, fma(m0, r.x, m12))) and so on.
template <typename T>
void rigid_targets(T* out, const float* rest, uint32_t nstrands, const float* m) {
  for (uint32_t s = 0; s < nstrands; ++s) {
    const T rx = rest[3 * s], ry = rest[3 * s + 1], rz = rest[3 * s + 2];
    for (int c = 0; c < 3; ++c) {
      out[3 * s + c] =
          std::fma(T(m[8 + c]), rz, std::fma(T(m[4 + c]), ry, std::fma(T(m[0 + c]), rx, T(m[12 + c]))));
    }
  }
}

// ---- skinned roots ------------------------------------------------------
//
// Dual-quaternion blend of the rest root, restating the reference's
// apply_skinning + skinning_DQBS (src/shaders/shared/inc_skinning.glsl:22-82,
// Kavan et al. 2008, "Geometric Skinning with Approximate Dual Quaternion
// Blending"): skip when w0 <= Epsilon() = 1e-6 (inc_constants.glsl:6) and
// :23-25; w3 = 1 - (w0 + w1 + w2) (:28); w0..w2 *= sign(dot(real[b3],
// real[bk])) (:65); A = Ma*w, B = Mb*w (:68-69); normalise both by
// inversesqrt(dot(A,A)) (:72-74); rotate and translate (:77-78).
// Op order (shared with the kernels): 4-dots and the blend sums as fma
// chains in index order, cross(a,b).x = fma(a.y, b.z, -(a.z*b.y)), every
// other operation as the shader writes it, unfused. Pinned bit for bit to
// the reference's inc_skinning.glsl compiled as C++ (tests/golden/ref_skin.npz).
template <typename T>
struct Q4 {
  T x, y, z, w;
};

template <typename T>
inline T dot4(Q4<T> a, Q4<T> b) {
  return std::fma(a.w, b.w, std::fma(a.z, b.z, std::fma(a.y, b.y, a.x * b.x)));
}
template <typename T>
inline V3<T> cross(V3<T> a, V3<T> b) {
  return {std::fma(a.y, b.z, -(a.z * b.y)), std::fma(a.z, b.x, -(a.x * b.z)), std::fma(a.x, b.y, -(a.y * b.x))};
}
template <typename T>
inline T sign_of(T x) {
  return x > T(0) ? T(1) : (x < T(0) ? T(-1) : T(0));
}

template <typename T>
V3<T> skin_point(V3<T> v, const uint8_t* b, const float* wts, const float* dq) {
  T w0 = wts[0], w1 = wts[1], w2 = wts[2];
  if (w0 <= T(1e-6f)) return v;
  const T w3 = T(1) - ((w0 + w1) + w2);
  Q4<T> r[4], d[4];
  for (int k = 0; k < 4; ++k) {
    const float* q = dq + 8 * b[k];
    r[k] = {T(q[0]), T(q[1]), T(q[2]), T(q[3])};
    d[k] = {T(q[4]), T(q[5]), T(q[6]), T(q[7])};
  }
  w0 = w0 * sign_of(dot4(r[3], r[0]));
  w1 = w1 * sign_of(dot4(r[3], r[1]));
  w2 = w2 * sign_of(dot4(r[3], r[2]));
  auto blend = [&](const Q4<T>* q) {
    Q4<T> o;
    o.x = std::fma(q[3].x, w3, std::fma(q[2].x, w2, std::fma(q[1].x, w1, q[0].x * w0)));
    o.y = std::fma(q[3].y, w3, std::fma(q[2].y, w2, std::fma(q[1].y, w1, q[0].y * w0)));
    o.z = std::fma(q[3].z, w3, std::fma(q[2].z, w2, std::fma(q[1].z, w1, q[0].z * w0)));
    o.w = std::fma(q[3].w, w3, std::fma(q[2].w, w2, std::fma(q[1].w, w1, q[0].w * w0)));
    return o;
  };
  const Q4<T> A = blend(r), B = blend(d);
  const T inv = inversesqrt(dot4(A, A));
  const V3<T> a{A.x * inv, A.y * inv, A.z * inv};
  const T aw = A.w * inv;
  const V3<T> bv{B.x * inv, B.y * inv, B.z * inv};
  const T bw = B.w * inv;
  // :77-78, as written: cross(a, v) + aw v, and (aw b - bw a) + cross(a, b).
  v = add(v, mul(T(2), cross(a, add(cross(a, v), mul(aw, v)))));
  const V3<T> t = add(sub(mul(aw, bv), mul(bw, a)), cross(a, bv));
  return add(v, mul(T(2), t));
}

template <typename T>
void skin_targets(T* out, const float* rest, const uint8_t* bones, const float* weights, uint32_t nstrands,
                  const float* dq) {
  for (uint32_t s = 0; s < nstrands; ++s) {
    const V3<T> v{T(rest[3 * s]), T(rest[3 * s + 1]), T(rest[3 * s + 2])};
    const V3<T> o = skin_point<T>(v, bones + 4 * s, weights + 3 * s, dq);
    out[3 * s] = o.x;
    out[3 * s + 1] = o.y;
    out[3 * s + 2] = o.z;
  }
}

// Rigid column-major 4x4 -> dual quaternion, in float as the library does
// it on the host: rotation by K. Shoemake's trace-branch construction
// (1985), dual = 0.5 * (t, 0) * real; glm 0.9.9.8's dualquat(mat3x4), which
// the reference calls (src/fx/animation/skeleton_controller.cc:262), builds
// the same quantity (glm is not vendored in the reference).
void matrix_to_dual_quat(const float* m, float* dq) {
  auto R = [m](int i, int j) { return m[4 * j + i]; };
  const float tr = (R(0, 0) + R(1, 1)) + R(2, 2);
  float x, y, z, w;
  if (tr > 0.0f) {
    const float s = 2.0f * std::sqrt(tr + 1.0f);
    w = 0.25f * s;
    x = (R(2, 1) - R(1, 2)) / s;
    y = (R(0, 2) - R(2, 0)) / s;
    z = (R(1, 0) - R(0, 1)) / s;
  } else if (R(0, 0) > R(1, 1) && R(0, 0) > R(2, 2)) {
    const float s = 2.0f * std::sqrt(((1.0f + R(0, 0)) - R(1, 1)) - R(2, 2));
    w = (R(2, 1) - R(1, 2)) / s;
    x = 0.25f * s;
    y = (R(0, 1) + R(1, 0)) / s;
    z = (R(0, 2) + R(2, 0)) / s;
  } else if (R(1, 1) > R(2, 2)) {
    const float s = 2.0f * std::sqrt(((1.0f + R(1, 1)) - R(0, 0)) - R(2, 2));
    w = (R(0, 2) - R(2, 0)) / s;
    x = (R(0, 1) + R(1, 0)) / s;
    y = 0.25f * s;
    z = (R(1, 2) + R(2, 1)) / s;
  } else {
    const float s = 2.0f * std::sqrt(((1.0f + R(2, 2)) - R(0, 0)) - R(1, 1));
    w = (R(1, 0) - R(0, 1)) / s;
    x = (R(0, 2) + R(2, 0)) / s;
    y = (R(1, 2) + R(2, 1)) / s;
    z = 0.25f * s;
  }
  const float tx = m[12], ty = m[13], tz = m[14];
  dq[0] = x;
  dq[1] = y;
  dq[2] = z;
  dq[3] = w;
  dq[4] = 0.5f * ((w * tx) + (ty * z - tz * y));
  dq[5] = 0.5f * ((w * ty) + (tz * x - tx * z));
  dq[6] = 0.5f * ((w * tz) + (tx * y - ty * x));
  dq[7] = -0.5f * ((tx * x + ty * y) + tz * z);
}

// ---- tessellation stream ------------------------------------------------
//
// The reference's second pass, restated per output vertex (float):
//   vs_stream_hair.glsl:19-24   relative position (vertex id mod N) / N;
//   tcs_stream_hair.glsl:34-41  levels (nlines, nsubsegments), tangent * uScaleFactor;
//   tes_stream_hair.glsl:27-73  hermite_mix of the 3 strands' segment, a point of
//                               the triangle at random coordinates, smoothstep2;
//   gs_stream_hair.glsl:20-28   each line segment as 2 vertices;
// with the isoline tessellator's coordinates u = s / nsub, v = l / nlines,
// and the output order [instance][triangle][segment][line][subsegment].
// Op order (shared with the kernel): 4-dots as fma chains, row vector x
// matrix by columns, mat3x4 * c = fma(p2, c.z, fma(p1, c.y, p0 * c.x)).
inline float dot4f(float a0, float a1, float a2, float a3, float b0, float b1, float b2, float b3) {
  return std::fma(a3, b3, std::fma(a2, b2, std::fma(a1, b1, a0 * b0)));
}

// hermite_mix (inc_maths.glsl:210-228), xyz.
inline void hermite(const float* p0, const float* p1, const float* t0, const float* t1, float u, float* out) {
  const float uu = u * u;
  const float u3 = uu * u;
  const float c0 = dot4f(u3, uu, u, 1.0f, 2.0f, -3.0f, 0.0f, 1.0f);
  const float c1 = dot4f(u3, uu, u, 1.0f, -2.0f, 3.0f, 0.0f, 0.0f);
  const float c2 = dot4f(u3, uu, u, 1.0f, 1.0f, -2.0f, 1.0f, 0.0f);
  const float c3 = dot4f(u3, uu, u, 1.0f, 1.0f, -1.0f, 0.0f, 0.0f);
  for (int k = 0; k < 3; ++k) out[k] = dot4f(c0, c1, c2, c3, p0[k], p1[k], t0[k], t1[k]);
}

// smoothstep2(0, 1, x) (inc_maths.glsl:263-266): t = clamp(x, 0, 1).
inline float smoothstep01(float x) {
  const float t = std::fmin(std::fmax(x, 0.0f), 1.0f);
  return ((t * t) * t) * (10.0f + t * (-15.0f + 6.0f * t));
}

void tess_vertex(const float (*P)[3], const float (*T)[3], float u, float rx, float ry, float rel0, float n,
                 float* out) {
  float p[3][3];
  for (int k = 0; k < 3; ++k) hermite(P[2 * k], P[2 * k + 1], T[2 * k], T[2 * k + 1], u, p[k]);
  // sample_triangle2 (inc_maths.glsl:107-115), st.y reassigned after st.x.
  float sx = rx, sy = ry;
  if (sx + sy > 1.0f) {
    sx = std::fmax(sx, sy);
    sy = std::fmin(sx, sy);
    sx = 1.0f - sx;
  }
  const float cz = 1.0f - (sx + sy);
  for (int k = 0; k < 3; ++k) out[k] = std::fma(p[2][k], cz, std::fma(p[1][k], sy, p[0][k] * sx));
  out[3] = smoothstep01(rel0 + u / n);
}

void tess_all(const float* pos, const float* tan, uint32_t npoints, const uint32_t* faces, uint32_t nfaces,
              const float* random, uint32_t ninst, uint32_t nlines, uint32_t nsub, float scale, float* out) {
  size_t t = 0;
  const float n = static_cast<float>(npoints);
  for (uint32_t inst = 0; inst < ninst; ++inst)
    for (uint32_t f = 0; f < nfaces; ++f)
      for (uint32_t j = 0; j + 1 < npoints; ++j) {
        float P[6][3], T[6][3];
        for (int k = 0; k < 6; ++k) {
          const size_t idx = (static_cast<size_t>(faces[3 * f + k / 2]) * npoints + j + (k & 1)) * 4;
          for (int c = 0; c < 3; ++c) {
            P[k][c] = pos[idx + c];
            T[k][c] = tan[idx + c] * scale;
          }
        }
        const float rel0 = static_cast<float>(j) / n;
        for (uint32_t l = 0; l < nlines; ++l) {
          const float v = static_cast<float>(l) / static_cast<float>(nlines);
          const int r = static_cast<int>(v * 40.0f + static_cast<float>(inst)) % HS_TESS_RANDOM_SIZE;
          const float rx = random[4 * r], ry = random[4 * r + 1];
          for (uint32_t s = 0; s < nsub; ++s, ++t) {
            const float u0 = static_cast<float>(s) / static_cast<float>(nsub);
            const float u1 = static_cast<float>(s + 1) / static_cast<float>(nsub);
            tess_vertex(P, T, u0, rx, ry, rel0, n, out + 8 * t);
            tess_vertex(P, T, u1, rx, ry, rel0, n, out + 8 * t + 4);
          }
        }
      }
}

// ---- Marschner lookup tables ---------------------------------------------
//
// cs_marschner_m.glsl:33-61 and cs_marschner_n.glsl:25-84 with
// inc_marschner_n.glsl:40-118, inc_solver.glsl:31-122, inc_fresnel.glsl:17-58,
// per texel, in T (float or double) with the C library's transcendental
// functions. Pi() = 3.141564 and Epsilon() = 1e-6 as in the reference
// (inc_constants.glsl:6-7); degrees() is the GLSL builtin (180 / pi);
// pow(x, 2) is x * x.
template <typename T>
struct MRoots {
  T r[3];
  int n;
};

template <typename T>
MRoots<T> m_linear(T a, T b) {
  MRoots<T> z{{0, 0, 0}, 0};
  if (std::fabs(a) > T(1e-6f)) {
    z.r[0] = -b / a;
    z.n = 1;
  }
  return z;
}
template <typename T>
MRoots<T> m_quadratic(T a, T b, T c) {
  if (std::fabs(a) < T(1e-6f)) return m_linear(b, c);
  T delta = b * b - T(4) * a * c;
  MRoots<T> z{{0, 0, 0}, 0};
  if (delta < T(0)) return z;
  delta = std::sqrt(delta);
  z.r[0] = (-b + delta) / (T(2) * a);
  z.r[1] = (-b - delta) / (T(2) * a);
  z.n = 1 + (delta >= T(1e-6f) ? 1 : 0);
  return z;
}
template <typename T>
T m_sign(T x) {
  return x > T(0) ? T(1) : (x < T(0) ? T(-1) : T(0));
}
template <typename T>
MRoots<T> m_cubic_normalized(T a, T b, T c) {
  const T pi = T(3.141564f);
  MRoots<T> z{{0, 0, 0}, 0};
  if (std::fabs(c) < T(1e-6f)) {
    z = m_quadratic(T(1), a, b);
    z.r[z.n] = T(0);
    z.n += 1;
    return z;
  }
  const T Q = (T(3) * b - a * a) / T(9);
  const T R = (T(9) * a * b - T(27) * c - T(2) * a * a * a) / T(54);
  const T Q3 = Q * Q * Q;
  const T D = Q3 + R * R;
  const T third_a = a / T(3);
  if (D > T(0)) {
    const T sqrtD = std::sqrt(D);
    const T s = m_sign(R + sqrtD) * std::pow(std::fabs(R + sqrtD), T(0.333f));
    const T t = m_sign(R - sqrtD) * std::pow(std::fabs(R - sqrtD), T(0.333f));
    z.r[0] = s + t - third_a;
    z.n = 1;
  } else {
    const T theta = std::acos(R * inversesqrt(-Q3));  // inc_solver.glsl:91
    const T two_sqrt_q = T(2) * std::sqrt(-Q);
    z.r[0] = std::fma(two_sqrt_q, std::cos(theta / T(3)), -third_a);
    z.r[1] = std::fma(two_sqrt_q, std::cos((theta + T(2) * pi) / T(3)), -third_a);
    z.r[2] = std::fma(two_sqrt_q, std::cos((theta + T(4) * pi) / T(3)), -third_a);
    z.n = 3;
  }
  return z;
}
template <typename T>
MRoots<T> m_cubic(T a, T b, T c, T d) {
  return std::fabs(a) < T(1e-6f) ? m_quadratic(b, c, d) : m_cubic_normalized(b / a, c / a, d / a);
}
// GLSL pow: x * x for an exponent of 2 (the shaders square signed values,
// for which GLSL leaves pow undefined), else the C library's pow.
template <typename T>
T m_pow(T x, T y) {
  return y == T(2) ? x * x : std::pow(x, y);
}
template <typename T>
T m_power_ratio(T eta_ratio, T na, T nb, T cos_i, T sin_i) {
  const T e = eta_ratio * sin_i;
  const T sin_t2 = e * e;
  if (sin_t2 > T(1)) return T(1);
  const T cos_t = std::sqrt(T(1) - sin_t2);
  const T A = na * cos_i;
  const T B = nb * cos_t;
  const T R = (A - B) / (A + B);
  return std::fmin(T(1), R * R);
}
template <typename T>
T m_fresnel(T eta0, T eta_perp, T eta_par, T cos_a, T sin_a) {
  const T refl = m_power_ratio(eta0 / eta_perp, eta0, eta_perp, cos_a, sin_a);
  const T trans = m_power_ratio(eta0 / eta_par, eta_par, eta0, cos_a, sin_a);
  return refl * (T(1) - T(0.5)) + trans * T(0.5);
}
template <typename T>
T m_absorption(int p, T absorption, T eta_perp, T eta_par, T cos_gi, T sin_gi) {
  if (p == 0) return m_fresnel(T(1), eta_perp, eta_par, cos_gi, sin_gi);
  const T sin_gt = sin_gi / eta_perp;
  const T gt = std::asin(sin_gt);
  const T cos_gt = std::cos(gt);
  const T fi = m_fresnel(T(1), eta_perp, eta_par, cos_gi, sin_gi);
  const T ft = m_fresnel(T(1), T(1) / eta_perp, T(1) / eta_par, cos_gt, sin_gt);
  const T t = std::exp(T(-4) * absorption * (cos_gt * cos_gt));
  const T om = T(1) - fi;
  return (om * om) * m_pow(ft, T(p - 1)) * m_pow(t, T(p));
}
template <typename T>
T m_np(int p, T absorption, T eta_perp, T eta_par, T c, T phi) {
  const T pf = T(p);
  const T a = pf * c * T(-0.25801227547f);
  const T cc = pf * c * T(1.90985931710f) - T(2);
  const T d = pf * T(3.141564f) - phi;
  const MRoots<T> z = m_cubic(a, T(0), cc, d);
  T L = T(0);
  for (int i = 0; i < z.n; ++i) {
    const T gi = z.r[i];
    const T A = m_absorption(p, absorption, eta_perp, eta_par, std::cos(gi), std::sin(gi));
    const T f1 = (T(3) * a * (gi * gi) + cc) / std::cos(gi);
    L += A * (T(1) / std::fabs(T(2) * f1));
  }
  return std::fmin(L, T(1));
}
template <typename T>
void marschner_luts(uint32_t res, T eta, T absorption, T ar, T br, T* m, T* n) {
  const T inv = T(1) / T(res);
  for (uint32_t y = 0; y < res; ++y) {
    for (uint32_t x = 0; x < res; ++x) {
      T* mo = m + 4 * (static_cast<size_t>(y) * res + x);
      T* no = n + 4 * (static_cast<size_t>(y) * res + x);
      {
        const T ti = std::asin(T(2) * T(x) * inv - T(1));
        const T tr = std::asin(T(2) * T(y) * inv - T(1));
        const T th = (ti + tr) / T(2), td = (ti - tr) / T(2);
        const T deg = th * T(57.2957795131f);
        const T shifts[3] = {T(1) * ar, T(-0.5f) * ar, T(-1.5f) * ar};
        const T widths[3] = {T(1) * br, T(0.5f) * br, T(2) * br};
        for (int k = 0; k < 3; ++k) {
          const T xm = deg - shifts[k];
          mo[k] = std::exp(-(xm * xm) / (T(2) * widths[k] * widths[k])) / (T(2.5066282f) * std::fabs(widths[k]));
        }
        mo[3] = std::cos(td);
      }
      {
        const T cos_phi_d = T(2) * T(x) * inv - T(1);
        const T cos_theta_d = T(2) * T(y) * inv - T(1);
        const T sin_td2 = T(1) - cos_theta_d * cos_theta_d;
        const T eta2 = eta * eta;
        const T eta_perp = std::sqrt(eta2 - sin_td2) / cos_theta_d;
        const T eta_par = eta2 / eta_perp;
        const T phi_d = std::acos(cos_phi_d);
        const T c = std::asin(T(1) / eta_perp);
        no[0] = m_np(0, absorption, eta_perp, eta_par, c, phi_d);
        no[1] = m_np(1, absorption, eta_perp, eta_par, c, phi_d);
        no[2] = m_np(2, absorption, eta_perp, eta_par, c, phi_d);
        no[3] = T(1);
      }
    }
  }
}

}  // namespace

extern "C" {

// One frame (Hair::update) for nstrands strands of N points, in place.
// strand_base: global index of the first strand (seeds the wind jitter).
// root_targets: nstrands*3 values of the array's type, or NULL (pinned).
int oracle_frame_f32(float* pos, float* vel, uint32_t nstrands, uint32_t npoints, uint32_t strand_base,
                     const hs_sim_params* sp, uint64_t seed, float dt, const float* wind,
                     uint32_t nspheres, const float* spheres, const float* root_targets, int nthreads) {
  return frame_all<float>(pos, vel, nstrands, npoints, strand_base, sp, seed, dt, wind, nspheres,
                          spheres, root_targets, nthreads);
}
int oracle_frame_f64(double* pos, double* vel, uint32_t nstrands, uint32_t npoints, uint32_t strand_base,
                     const hs_sim_params* sp, uint64_t seed, float dt, const float* wind,
                     uint32_t nspheres, const float* spheres, const double* root_targets, int nthreads) {
  return frame_all<double>(pos, vel, nstrands, npoints, strand_base, sp, seed, dt, wind, nspheres,
                           spheres, root_targets, nthreads);
}
// The same frame with DFTL mode in a chosen form: 1 world coordinates,
// 2 segment form (see frame_strand_seg); 0 is the contract above.
int oracle_frame_form_f32(float* pos, float* vel, uint32_t nstrands, uint32_t npoints, uint32_t strand_base,
                          const hs_sim_params* sp, uint64_t seed, float dt, const float* wind, uint32_t nspheres,
                          const float* spheres, const float* root_targets, int nthreads, int form) {
  return frame_all<float>(pos, vel, nstrands, npoints, strand_base, sp, seed, dt, wind, nspheres, spheres,
                          root_targets, nthreads, form);
}
int oracle_frame_form_f64(double* pos, double* vel, uint32_t nstrands, uint32_t npoints, uint32_t strand_base,
                          const hs_sim_params* sp, uint64_t seed, float dt, const float* wind, uint32_t nspheres,
                          const float* spheres, const double* root_targets, int nthreads, int form) {
  return frame_all<double>(pos, vel, nstrands, npoints, strand_base, sp, seed, dt, wind, nspheres, spheres,
                           root_targets, nthreads, form);
}
int oracle_init_f32(float* pos, float* vel, const float* roots, const float* normals, uint32_t nstrands,
                    const hs_strand_params* sp) {
  return init_all<float>(pos, vel, roots, normals, nstrands, sp);
}
int oracle_init_f64(double* pos, double* vel, const float* roots, const float* normals, uint32_t nstrands,
                    const hs_strand_params* sp) {
  return init_all<double>(pos, vel, roots, normals, nstrands, sp);
}
void oracle_rigid_targets_f32(float* out, const float* rest, uint32_t nstrands, const float* m) {
  rigid_targets<float>(out, rest, nstrands, m);
}
void oracle_rigid_targets_f64(double* out, const float* rest, uint32_t nstrands, const float* m) {
  rigid_targets<double>(out, rest, nstrands, m);
}
// Skinned root targets: nstrands*3 outputs from rest roots (3 floats),
// influences (4 bone bytes, 3 weights per strand) and a palette of dual
// quaternions (8 floats per bone).
void oracle_skin_targets_f32(float* out, const float* rest, const uint8_t* bones, const float* weights,
                             uint32_t nstrands, const float* dq) {
  skin_targets<float>(out, rest, bones, weights, nstrands, dq);
}
void oracle_skin_targets_f64(double* out, const float* rest, const uint8_t* bones, const float* weights,
                             uint32_t nstrands, const float* dq) {
  skin_targets<double>(out, rest, bones, weights, nstrands, dq);
}
void oracle_matrix_to_dual_quat(const float* m, float* dq) { matrix_to_dual_quat(m, dq); }
// Tessellation stream: pos and tan strand-major (nstrands * N * 4 floats),
// out 8 floats per line segment (see tess_all for the order).
void oracle_tess_f32(const float* pos, const float* tan, uint32_t npoints, const uint32_t* faces, uint32_t nfaces,
                     const float* random, uint32_t ninst, uint32_t nlines, uint32_t nsub, float scale, float* out) {
  tess_all(pos, tan, npoints, faces, nfaces, random, ninst, nlines, nsub, scale, out);
}
// Marschner tables: res * res RGBA texels each (see marschner_luts).
void oracle_marschner_f32(uint32_t res, float eta, float absorption, float ar, float br, float* m, float* n) {
  marschner_luts<float>(res, eta, absorption, ar, br, m, n);
}
void oracle_marschner_f64(uint32_t res, float eta, float absorption, float ar, float br, double* m, double* n) {
  marschner_luts<double>(res, eta, absorption, ar, br, m, n);
}
// The wind-jitter and length-jitter draws, for tests of the hash itself.
float oracle_hash_u01(uint64_t seed, uint32_t stream, uint32_t idx) {
  return hash_u01<float>(stream_key(seed, stream), idx);
}
int oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
