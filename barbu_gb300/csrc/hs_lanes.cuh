// hs_lanes.cuh -- one frame of a 32-strand tile, a group of K lanes per
// strand (DFTL mode, one constraint iteration per substep).
//
// The thread-per-strand forms run a strand's S substeps one after the
// other, each a pass over its N points whose chain link i needs link i-1:
// S x N dependent steps per thread. A groom of a few thousand strands
// then occupies a few warps per SM, each waiting on its own chain. Here
// the K lanes of a group take one substep each (lane k: substep k, S <= K)
// and run as a wavefront: at time step T lane k is at point j = T - 2k of
// its pass, so a frame takes N + 2 (S - 1) + 1 steps instead of S x N, on
// K times the lanes. The reference also spreads a strand over a work
// group, one invocation per particle (cs_simulation.glsl:89, :169).
//
// Data flow. Step j of a pass loads point j+1 (used by link j+1), runs
// link j and finishes point j-1 (push-out, Eq. 9 velocity), as the single
// pass of hs_stream.cuh does, operation for operation. Lane k's input,
// point j+1 as substep k-1 left it, is what lane k-1 finished at step
// j+2: in the same time step with the lag of 2, handed over by a shuffle
// between its finish and lane k's load.
// Lane 0 reads the frame's starting state from the tile's shared-memory
// copy (segments and velocities) instead, and lane S-1 writes the
// finished points (world positions rebuilt from the final root and the
// segments, as strand_frame_stream stores them). The pass carries are
// registers.
//
// The arithmetic of every point and substep is that of
// substep_single_pass_seg, so the frames are bit-identical to the
// thread-per-strand kernels'. Which points test the spheres (jmin, per
// strand here) and how (the cache width) change no result: a point that
// cannot reach a sphere is never pushed.
#pragma once

#include "hs_stream.cuh"

namespace hs {

// Lag between the passes of consecutive substeps, in time steps.
constexpr int kLaneLag = 2;

// Lane 0's input: point i of the frame's start (segment and rest length,
// velocity), loaded straight into the registers the shuffle filled, as one
// predicated pair of shared-memory loads.
__device__ __forceinline__ void load_start(bool take, const float4* sp, const float4* sv, float& x, float& y,
                                           float& z, float& rest, float& vx, float& vy, float& vz) {
  float vw = 0.0f;
  const uint32_t ap = static_cast<uint32_t>(__cvta_generic_to_shared(sp));
  const uint32_t av = static_cast<uint32_t>(__cvta_generic_to_shared(sv));
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.u32 p, %8, 0;\n\t"
      "@p ld.shared.v4.f32 {%0, %1, %2, %3}, [%9];\n\t"
      "@p ld.shared.v4.f32 {%4, %5, %6, %7}, [%10];\n\t}"
      : "+f"(x), "+f"(y), "+f"(z), "+f"(rest), "+f"(vx), "+f"(vy), "+f"(vz), "+f"(vw)
      : "r"(static_cast<uint32_t>(take)), "r"(ap), "r"(av)
      : "memory");
}

// The wavefront of one strand's substeps (see the header). NC: sphere
// slots tested; CACHED: push from the register cache (push_seg). s_p holds
// the strand's starting segments (point 0: its world position) with the
// rest lengths in w, s_v its velocities, [point][32] at column c. The lane
// of the last substep stores the finished points and adds them to `ts`.
template <int K, int NC, bool CACHED, bool FAST, int M>
__device__ __forceinline__ void lanes_pass(const FrameConst& fc, const StrandConsts& Kc, const SphereCache<M>& C,
                                           const SphereSet& S, const GroomView& g, uint32_t s, bool active, int c,
                                           int k, int n, int jmin, V3 x0_start, V3 target, float rest0,
                                           const float4* s_p, const float4* s_v, TileStats& ts) {
  constexpr bool kCached = CACHED && M > kCachedSpheres;
  const V3 zero = v3(0.0f, 0.0f, 0.0f);
  const int nsub = fc.substeps;
  const bool worker = k < nsub;
  const bool writer = active && k == nsub - 1;

  // This lane's substep: its root offset rel_k = alpha_k delta (delta at
  // the last substep), chain start R and root displacement D0.
  const bool moving = fc.root_mode != HS_ROOT_PINNED;
  const V3 delta = sub(target, x0_start);
  V3 rel = zero, rel_prev = zero, R = x0_start;
  if (moving) {
    const bool lastk = k + 1 == nsub;
    const float alpha = __fdiv_rn(static_cast<float>(k + 1), static_cast<float>(nsub));
    rel = lastk ? delta : mul(alpha, delta);
    R = lastk ? target : add(x0_start, rel);
    if (k > 0) rel_prev = mul(__fdiv_rn(static_cast<float>(k), static_cast<float>(nsub)), delta);
  }
  const V3 D0 = sub(rel, rel_prev);

  // The root, final after the last substep.
  V3 wout = R;
  if (writer) {
    const float4 x = f4(R, rest0);
    const float4 v = f4(mul(D0, Kc.inv_h), 0.0f);
    g.pos[s] = x;
    g.vel[s] = v;
    ts.add(x, v);
  }

  V3 D_prev = D0, w_prev = R, s_prev = zero, a_cur = zero, dp_cur = zero;
  float rest_prev = 0.0f, rest_cur = 0.0f;
  const int steps = n + kLaneLag * (nsub - 1) + 1;
  // Lane 0 takes point j + 1 = T + 1 of the frame's start at step T.
  const float4* lp = s_p + 32 + c;
  const float4* lv = s_v + 32 + c;
  for (int T = 0; T < steps; ++T) {
    const int j = T - kLaneLag * k;
    const bool tip = j == n;
    // Link j (kept for 1 <= j <= n - 1).
    V3 sn, e;
    link_seg<FAST>(Kc, sub(a_cur, D_prev), rest_cur, sn, e);
    const V3 D_i = add(dp_cur, e);
    const V3 w_i = add(w_prev, sn);
    // Finish point j - 1 (2 <= j <= n).
    const bool fin = worker && j >= 2 && j <= n;
    if (fin && j - 1 >= jmin && tests<NC>(C, w_prev))
      push_seg<kCached, NC, FAST>(C, S, w_prev, D_prev, s_prev, sn, tip);
    const V3 vel = vel_of(Kc, tip ? D_prev : fmas(Kc.neg_damping, e, D_prev));
    if (writer && fin) {
      wout = add(wout, s_prev);
      const float4 x = f4(wout, rest_prev);
      const float4 v = frame_velocity<true, false>(fc, f4(vel, 0.0f));
      const size_t at = static_cast<size_t>(j - 1) * g.stride + s;
      g.pos[at] = x;
      g.vel[at] = v;
      ts.add(x, v);
    }
    // Hand point j - 1 to the next substep's lane, which takes it as its
    // point j' + 1 (j' = j - 2, this step). Lane k takes lane k-1's; lane 0
    // the frame's start. Values outside 2 <= j <= n are never linked.
    float ix = __shfl_up_sync(0xffffffffu, s_prev.x, 1, K);
    float iy = __shfl_up_sync(0xffffffffu, s_prev.y, 1, K);
    float iz = __shfl_up_sync(0xffffffffu, s_prev.z, 1, K);
    float irest = __shfl_up_sync(0xffffffffu, rest_prev, 1, K);
    float ivx = __shfl_up_sync(0xffffffffu, vel.x, 1, K);
    float ivy = __shfl_up_sync(0xffffffffu, vel.y, 1, K);
    float ivz = __shfl_up_sync(0xffffffffu, vel.z, 1, K);
    load_start(k == 0 && T + 1 < n, lp, lv, ix, iy, iz, irest, ivx, ivy, ivz);
    lp += 32;
    lv += 32;
    if (j >= 1) {  // nothing after the tip is used
      s_prev = sn;
      D_prev = D_i;
      w_prev = w_i;
      rest_prev = rest_cur;
    }
    // Point j + 1, for link j + 1 (a stash before j = 0 is replaced at
    // j = 0, one at j >= n - 1 is never linked).
    dp_cur = disp(Kc, make_float4(ivx, ivy, ivz, 0.0f));
    a_cur = add(v3(ix, iy, iz), dp_cur);
    rest_cur = irest;
  }
}

// One frame of tile `tile` of groom g, by a block of 32 K threads (K warps;
// warp w takes strands [w 32/K, (w + 1) 32/K) of the tile, lane l strand
// l / K as substep lane l % K). s_p, s_v: [n][32] float4 each, the tile's
// starting state; s_ts: 32 TileStats. Every thread of the block calls it.
template <int K, int M, bool CACHED, bool FAST>
__device__ __forceinline__ void tile_frame_lanes(const FrameConst& fc, const SphereSet& S, const GroomView& g,
                                                 uint32_t tile, float4* s_p, float4* s_v, TileStats* s_ts) {
  static_assert(K == 2 || K == 4 || K == 8 || K == 16, "lane groups of 2, 4, 8 or 16");
  constexpr int G = 32 / K;  // strands per warp
  constexpr int B = 32 * K;  // threads
  constexpr int U = 4;       // loads in flight per thread
  const int n = static_cast<int>(g.npoints);
  const int t = static_cast<int>(threadIdx.x);
  // The tile's state, one coalesced 512-byte row per point and array, the
  // positions as segments s_i = p_i - p_{i-1} (point 0 as it is; row i-1
  // comes again from the L1).
  for (int base = t; base < n * 32; base += U * B) {
    float4 p[U], pm[U], v[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int idx = base + u * B;
      const int i = idx / 32;
      const uint32_t s = tile * 32u + static_cast<uint32_t>(idx % 32);
      p[u] = pm[u] = v[u] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      if (idx < n * 32 && s < g.nstrands) {
        p[u] = g.pos[static_cast<size_t>(i) * g.stride + s];
        v[u] = g.vel[static_cast<size_t>(i) * g.stride + s];
        if (i > 0) pm[u] = g.pos[static_cast<size_t>(i - 1) * g.stride + s];
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int idx = base + u * B;
      if (idx < n * 32) {
        s_p[idx] = idx >= 32 ? f4(sub(xyz(p[u]), xyz(pm[u])), p[u].w) : p[u];
        s_v[idx] = frame_velocity<true, true>(fc, v[u]);
      }
    }
  }
  __syncthreads();

  const int warp = t / 32, lane = t % 32;
  const int k = lane % K;
  const int c = warp * G + lane / K;  // the strand's column in the tile
  const uint32_t s = tile * 32u + static_cast<uint32_t>(c);
  const bool active = s < g.nstrands;
  const float4 p0 = s_p[c];
  const V3 x0_start = xyz(p0);
  const float rest0 = p0.w;
  float Rlen = 0.0f;  // total link length, for culling (the sum of strand_frame_stream)
  for (int i = 1; i < n; ++i) Rlen += fabsf(fc.length_scale * s_p[i * 32 + c].w);

  const StrandConsts Kc = strand_consts(fc, g, s, active);
  const V3 target = root_target(fc, g, s, active, x0_start);

  // Spheres this strand can touch during the frame and the first point
  // that can touch one (strand_frame_stream), per strand.
  uint32_t reach = 0u;
  int jmin = n;
  if (S.n > 0 && active) {
    const V3 root_delta = sub(target, x0_start);
    const V3 mid = v3(0.5f * (x0_start.x + target.x), 0.5f * (x0_start.y + target.y), 0.5f * (x0_start.z + target.z));
    const float half_path = 0.5f * sqrtf(root_delta.x * root_delta.x + root_delta.y * root_delta.y +
                                         root_delta.z * root_delta.z);
    reach = overlap_closure(S, near_spheres(S, mid, Rlen + half_path));
    const float thr = reach_threshold(S, mid, Rlen + half_path, half_path);
    float Rj = 0.0f;
    for (int i = 1; i < n; ++i) {
      Rj += fabsf(fc.length_scale * s_p[i * 32 + c].w);
      if (jmin == n && Rj >= thr) jmin = i;
    }
  }
  const SphereCache<M> C = cache_spheres<M>(S, reach);
  TileStats ts;
  ts.init();
  const int warp_cached = __reduce_max_sync(0xffffffffu, C.ncached);
  if (M > kCachedSpheres && warp_cached > kCachedSpheres)
    lanes_pass<K, M, CACHED, FAST>(fc, Kc, C, S, g, s, active, c, k, n, jmin, x0_start, target, rest0, s_p, s_v, ts);
  else
    lanes_pass<K, kCachedSpheres, CACHED, FAST>(fc, Kc, C, S, g, s, active, c, k, n, jmin, x0_start, target, rest0,
                                                s_p, s_v, ts);

  // Tile statistics: the strands' own (from their last substep's lane, in
  // point order), reduced by one warp as the thread-per-strand kernels do.
  if (k == fc.substeps - 1) s_ts[c] = ts;
  __syncthreads();
  if (warp == 0) {
    TileStats tt = s_ts[lane];
    tt.store(g.stats, tile, (g.nstrands + 31u) / 32u, lane);
  }
}

}  // namespace hs
