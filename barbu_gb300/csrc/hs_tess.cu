// hs_tess.cu -- the tessellation stream pass: interpolated render strands
// from the simulated control points, into a device buffer.
//
// The reference runs this pass on the GL tessellator (src/fx/hair.cc:145-170:
// vs/tcs/tes/gs_stream_hair.glsl, captured by transform feedback). Here one
// thread takes one isoline: it gathers the patch (6 control points and
// tangents from the groom's [point][strand] arrays) and the line's triangle
// sample once, evaluates the tessellation evaluation shader at each of the
// line's nsub + 1 vertices, and writes the line's 2 nsub segment ends into
// shared memory; the warp then stores its 32 lines, which are contiguous in
// the output, with coalesced writes. The shader's divisions, the Hermite
// basis at each u and the smoothstep of each (point, u) pair come from
// per-block tables (one entry per distinct operand).
//
// Arithmetic contract (shared with the oracle, which matches bit for bit):
//   4-component dot = fma(a.w,b.w, fma(a.z,b.z, fma(a.y,b.y, a.x*b.x)));
//   row vector x matrix: component j = dot(v, column j);
//   mat3x4 * c        = fma(p2, c.z, fma(p1, c.y, p0 * c.x)) per component;
//   u^3 = (u*u)*u; smoothstep2(0,1,x) = ((t*t)*t) * (10 + t*(-15 + 6t)),
//   t = clamp(x, 0, 1), each operation rounded.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "hs_api_internal.h"
#include "hs_internal.h"

namespace hs {
namespace {

// Unsigned 32-bit division by a divisor fixed for the launch, by a
// multiply-high and shifts (T. Granlund, P. Montgomery, "Division by
// Invariant Integers using Multiplication", PLDI 1994, section 4): for
// d > 1, l = ceil(log2 d), m = floor(2^32 (2^l - d) / d) + 1,
// q = (t + ((n - t) >> 1)) >> (l - 1) with t = mulhi(m, n).
struct FastDiv {
  uint32_t d, m, l;
  static FastDiv make(uint32_t d) {
    FastDiv f{d, 0u, 0u};
    if (d > 1) {
      uint32_t l = 0;
      while ((1ull << l) < d) ++l;
      f.l = l;
      f.m = static_cast<uint32_t>(((1ull << 32) * ((1ull << l) - d)) / d + 1);
    }
    return f;
  }
  __device__ __forceinline__ uint32_t div(uint32_t n) const {
    if (d == 1) return n;
    const uint32_t t = __umulhi(m, n);
    return (t + ((n - t) >> 1)) >> (l - 1);
  }
};

struct TessArgs {
  const float4* pos;      // [N][stride] (x, y, z, rest length)
  const float4* tangent;  // [N][stride]
  const uint3* faces;     // strand indices of each triangle
  const float* random;    // HS_TESS_RANDOM_SIZE floats
  float4* out;            // 2 vertices per line segment
  uint32_t stride, npoints, nfaces;
  uint32_t ninstances, nlines, nsub;
  float scale;            // uScaleFactor
  uint64_t nvertices;     // tessellated vertices: lines * (nsub + 1)
  FastDiv lines, segs, faces_div;  // divisors of the line index decomposition (< 2^32 lines)
};

// The shader's divisions, one table entry per distinct operand pair:
// u = s / nsub, u / N, j / N, v = l / nlines (IEEE divisions, as the oracle).
struct TessTables {
  float4 basis[17];                                  // Hermite basis (c0..c3) at u = s / nsub
  float rel[(HS_MAX_POINTS_PER_STRAND - 1) * 17];    // smoothstep(j / N + u / N), [j][s]
  float v[16];                                       // l / nlines
};

__device__ __forceinline__ float dot4(float a0, float a1, float a2, float a3, float b0, float b1, float b2,
                                      float b3) {
  return __fmaf_rn(a3, b3, __fmaf_rn(a2, b2, __fmaf_rn(a1, b1, __fmul_rn(a0, b0))));
}

// vU * mHermit (hermite_mix, inc_maths.glsl:210-228): the basis weights at
// u, mHermit's columns (2,-3,0,1), (-2,3,0,0), (1,-2,1,0), (1,-1,0,0).
__device__ __forceinline__ float4 hermite_basis(float u) {
  const float uu = __fmul_rn(u, u);
  const float u3 = __fmul_rn(uu, u);
  return make_float4(dot4(u3, uu, u, 1.0f, 2.0f, -3.0f, 0.0f, 1.0f), dot4(u3, uu, u, 1.0f, -2.0f, 3.0f, 0.0f, 0.0f),
                     dot4(u3, uu, u, 1.0f, 1.0f, -2.0f, 1.0f, 0.0f), dot4(u3, uu, u, 1.0f, 1.0f, -1.0f, 0.0f, 0.0f));
}

__device__ __forceinline__ float smoothstep01(float x);

__device__ __forceinline__ void tess_tables(const TessArgs& a, TessTables& T) {
  const float n = static_cast<float>(a.npoints);
  const uint32_t ns = a.nsub + 1;
  for (uint32_t k = threadIdx.x; k < ns; k += blockDim.x)
    T.basis[k] = hermite_basis(__fdiv_rn(static_cast<float>(k), static_cast<float>(a.nsub)));
  for (uint32_t k = threadIdx.x; k < (a.npoints - 1) * ns; k += blockDim.x) {
    const uint32_t j = k / ns, sub = k - j * ns;
    const float u = __fdiv_rn(static_cast<float>(sub), static_cast<float>(a.nsub));
    T.rel[k] = smoothstep01(__fadd_rn(__fdiv_rn(static_cast<float>(j), n), __fdiv_rn(u, n)));  // tes :65-66
  }
  for (uint32_t k = threadIdx.x; k < a.nlines; k += blockDim.x)
    T.v[k] = __fdiv_rn(static_cast<float>(k), static_cast<float>(a.nlines));
}

// hermite_mix (inc_maths.glsl:210-228): vU * mHermit * B, xyz only (the w
// of the result is not used by the pass).
// (...) * B with the basis c: B's columns (p0.x, p1.x, t0.x, t1.x) and so on.
__device__ __forceinline__ float3 hermite(float3 p0, float3 p1, float3 t0, float3 t1, float4 c) {
  return make_float3(dot4(c.x, c.y, c.z, c.w, p0.x, p1.x, t0.x, t1.x), dot4(c.x, c.y, c.z, c.w, p0.y, p1.y, t0.y, t1.y),
                     dot4(c.x, c.y, c.z, c.w, p0.z, p1.z, t0.z, t1.z));
}

// smoothstep2(0, 1, x) (inc_maths.glsl:263-266, maprange :239-241).
__device__ __forceinline__ float smoothstep01(float x) {
  const float t = fminf(fmaxf(x, 0.0f), 1.0f);
  const float inner = __fadd_rn(10.0f, __fmul_rn(t, __fadd_rn(-15.0f, __fmul_rn(6.0f, t))));
  return __fmul_rn(__fmul_rn(__fmul_rn(t, t), t), inner);
}

__device__ __forceinline__ float3 xyz3(float4 v) { return make_float3(v.x, v.y, v.z); }
__device__ __forceinline__ float3 scaled(float4 v, float s) {
  return make_float3(__fmul_rn(v.x, s), __fmul_rn(v.y, s), __fmul_rn(v.z, s));
}

// Blocks of 4 warps. The staging row of a line holds its nsub + 1 vertices
// (each vertex ends one segment and starts the next, so the output row of
// 2 nsub segment ends repeats them); 17 float4 a row, an odd stride, keep
// the lanes' rows in different banks.
constexpr int kTessBlock = 128;
constexpr int kTessRow = 17;

// One tessellation-evaluation vertex (tes_stream_hair.glsl:27-73) per
// (line, u): the three strands' Hermite curves at the basis c, mixed by the
// line's triangle sample (sx, sy, cz).
__device__ __forceinline__ float4 tes_vertex(const float3 (&P)[6], const float3 (&T)[6], float4 c, float sx, float sy,
                                             float cz, float rel) {
  const float3 p0 = hermite(P[0], P[1], T[0], T[1], c);
  const float3 p1 = hermite(P[2], P[3], T[2], T[3], c);
  const float3 p2 = hermite(P[4], P[5], T[4], T[5], c);
  const float x = __fmaf_rn(p2.x, cz, __fmaf_rn(p1.x, sy, __fmul_rn(p0.x, sx)));
  const float y = __fmaf_rn(p2.y, cz, __fmaf_rn(p1.y, sy, __fmul_rn(p0.y, sx)));
  const float z = __fmaf_rn(p2.z, cz, __fmaf_rn(p1.z, sy, __fmul_rn(p0.z, sx)));
  return make_float4(x, y, z, rel);
}

// A grid-stride loop over groups of 32 lines, one group per warp.
// Line index = ((instance * nfaces + face) * (N - 1) + j) * nlines + l.
__global__ void __launch_bounds__(kTessBlock) k_tess(TessArgs a) {
  __shared__ TessTables tab;
  __shared__ float4 stage[kTessBlock / 32][32 * kTessRow];
  tess_tables(a, tab);
  __syncthreads();
  const uint32_t warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  float4* const st = stage[warp];
  const uint32_t ns = a.nsub + 1, row = 2 * a.nsub;
  const uint64_t nlines_total = a.nvertices / ns;
  const uint64_t groups = (nlines_total + 31) / 32;
  const uint64_t step = static_cast<uint64_t>(gridDim.x) * (kTessBlock / 32);
  for (uint64_t grp = static_cast<uint64_t>(blockIdx.x) * (kTessBlock / 32) + warp; grp < groups; grp += step) {
    const uint64_t line0 = grp * 32;
    const uint64_t li = line0 + lane;
    if (li < nlines_total) {
      uint32_t line, j, face, inst;
      if (nlines_total <= 0xffffffffull) {
        const uint32_t l32 = static_cast<uint32_t>(li);
        const uint32_t q1 = a.lines.div(l32);
        line = l32 - q1 * a.nlines;
        const uint32_t q2 = a.segs.div(q1);
        j = q1 - q2 * (a.npoints - 1);
        inst = a.faces_div.div(q2);
        face = q2 - inst * a.nfaces;
      } else {
        uint64_t q = li;
        line = static_cast<uint32_t>(q % a.nlines);
        q /= a.nlines;
        j = static_cast<uint32_t>(q % (a.npoints - 1));
        q /= (a.npoints - 1);
        face = static_cast<uint32_t>(q % a.nfaces);
        inst = static_cast<uint32_t>(q / a.nfaces);
      }
      // The patch (hair.cc:400-408): points j, j+1 of the triangle's strands.
      const uint3 f = a.faces[face];
      const uint32_t strand[3] = {f.x, f.y, f.z};
      float3 P[6], T[6];
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        const size_t idx = static_cast<size_t>(j + (k & 1)) * a.stride + strand[k >> 1];
        P[k] = xyz3(__ldg(a.pos + idx));
        T[k] = scaled(__ldg(a.tangent + idx), a.scale);  // tcs :41
      }
      // gl_TessCoord v = line / nlines; the random offset (tes :55-58);
      // randbuffer is vec3 under std430: element r starts at float 4r.
      const float v = tab.v[line];
      const int r = static_cast<int>(__fadd_rn(__fmul_rn(v, 40.0f), static_cast<float>(inst))) % HS_TESS_RANDOM_SIZE;
      // sample_triangle2 (inc_maths.glsl:107-115); st.y is min(st.x, st.y)
      // after st.x has become the max, i.e. st.y itself.
      float sx = __ldg(a.random + 4 * r), sy = __ldg(a.random + 4 * r + 1);
      if (__fadd_rn(sx, sy) > 1.0f) {
        sx = fmaxf(sx, sy);
        sy = fminf(sx, sy);
        sx = __fsub_rn(1.0f, sx);
      }
      const float cz = __fsub_rn(1.0f, __fadd_rn(sx, sy));
      // The geometry shader's lines (gs :20-28): vertex s ends segment
      // s - 1 and starts segment s (expanded when the rows are stored).
      float4* const mine = st + lane * kTessRow;
      const float* const rel = tab.rel + j * ns;
      // Fully unrolled over the 17 possible vertices: independent vertices
      // in flight (few warps fit an SM).
#pragma unroll
      for (uint32_t sub = 0; sub < 17; ++sub) {
        if (sub < ns) mine[sub] = tes_vertex(P, T, tab.basis[sub], sx, sy, cz, rel[sub]);
      }
    }
    __syncwarp();
    // The warp's lines are contiguous in the output: row by row, coalesced;
    // segment end k of a line is its vertex (k + 1) / 2.
    const uint64_t nl = min(static_cast<uint64_t>(32), nlines_total - line0);
    float4* const out = a.out + line0 * row;
    for (uint32_t l = 0; l < nl; ++l)
      for (uint32_t k = lane; k < row; k += 32) out[static_cast<size_t>(l) * row + k] = st[l * kTessRow + (k + 1) / 2];
    __syncwarp();
  }
}

}  // namespace
}  // namespace hs

namespace hs {

uint64_t tess_segments(const hs_groom* g, const hs_tess_params* p) {
  return static_cast<uint64_t>(p->ninstances) * g->tess_nfaces * (g->npoints - 1) * p->nlines * p->nsubsegments;
}

static hs_status validate_tess(const hs_groom* g, const hs_tess_params* p, const char* what) {
  if (!g || !p) return fail(HS_ERR_INVALID_ARG, "%s: null argument", what);
  if (p->ninstances < 1 || p->ninstances > 16 || p->nlines < 1 || p->nlines > 16 || p->nsubsegments < 1 ||
      p->nsubsegments > 16)
    return fail(HS_ERR_INVALID_ARG, "%s: instances, lines and subsegments must be in 1..16", what);
  if (!std::isfinite(p->length_scale)) return fail(HS_ERR_INVALID_ARG, "%s: non-finite length scale", what);
  return HS_OK;
}

}  // namespace hs

using namespace hs;

extern "C" {

HS_API void hs_tess_params_reference(hs_tess_params* p) {
  if (!p) return;
  p->ninstances = 3;      // Parameters_t::tess (src/fx/hair.h:33-37)
  p->nlines = 2;
  p->nsubsegments = 16;
  p->length_scale = 1.45f;  // render.lengthScale (:42)
}

HS_API hs_status hs_tess_setup(hs_groom* g, const uint32_t* faces, uint32_t nfaces, const float* tangents_xyzw,
                               const float* random, uint32_t nrandom) {
  if (!g || (nfaces > 0 && !faces) || !tangents_xyzw || !random)
    return fail(HS_ERR_INVALID_ARG, "hs_tess_setup: null argument");
  HS_ON_DEVICE(g->ctx, "hs_tess_setup");
  if (nrandom != HS_TESS_RANDOM_SIZE)
    return fail(HS_ERR_INVALID_ARG, "hs_tess_setup: the random buffer has %d floats, got %u", HS_TESS_RANDOM_SIZE,
                nrandom);
  for (size_t k = 0; k < 3 * static_cast<size_t>(nfaces); ++k)
    if (faces[k] >= g->nstrands)
      return fail(HS_ERR_INVALID_ARG, "hs_tess_setup: face %zu uses strand %u of %u", k / 3, faces[k], g->nstrands);
  const size_t nt = 4 * static_cast<size_t>(g->nstrands) * g->npoints;
  for (size_t k = 0; k < nt; ++k)
    if (!std::isfinite(tangents_xyzw[k])) return fail(HS_ERR_INVALID_ARG, "hs_tess_setup: non-finite tangent");
  for (uint32_t k = 0; k < nrandom; ++k)
    if (!std::isfinite(random[k])) return fail(HS_ERR_INVALID_ARG, "hs_tess_setup: non-finite random value");
  cudaStream_t st = g->ctx->stream;
  cudaError_t e = cudaStreamSynchronize(st);  // a pass in flight may read the old inputs
  cudaFree(g->d_tess_faces);
  cudaFree(g->d_tess_tangents);
  cudaFree(g->d_tess_random);
  g->d_tess_faces = nullptr;
  g->d_tess_tangents = nullptr;
  g->d_tess_random = nullptr;
  g->tess_nfaces = 0;
  float4* d_strand_major = nullptr;
  const size_t plane = sizeof(float4) * static_cast<size_t>(g->stride) * g->npoints;
  if (e == cudaSuccess) e = cudaMalloc(&g->d_tess_faces, sizeof(uint3) * std::max<uint32_t>(nfaces, 1));
  if (e == cudaSuccess) e = cudaMalloc(&g->d_tess_tangents, plane);
  if (e == cudaSuccess) e = cudaMalloc(&g->d_tess_random, sizeof(float) * HS_TESS_RANDOM_SIZE);
  if (e == cudaSuccess) e = cudaMalloc(&d_strand_major, sizeof(float) * nt);
  // Faces name caller strands; the state columns are the stored strands.
  std::vector<uint32_t> stored_faces(3 * static_cast<size_t>(nfaces));
  for (size_t k = 0; k < stored_faces.size(); ++k) stored_faces[k] = g->inv[faces[k]];
  if (e == cudaSuccess && nfaces > 0)
    e = cudaMemcpyAsync(g->d_tess_faces, stored_faces.data(), sizeof(uint3) * nfaces, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(g->d_tess_random, random, sizeof(float) * HS_TESS_RANDOM_SIZE, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(g->d_tess_tangents, 0, plane, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_strand_major, tangents_xyzw, sizeof(float) * nt, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = launch_from_strand_major(d_strand_major, g->d_tess_tangents, g->d_order, g->nstrands, g->npoints, g->stride,
                                 st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(d_strand_major);
  if (e != cudaSuccess) return cuda_fail(e, "hs_tess_setup");
  g->ctx->launches += 1;
  g->tess_nfaces = nfaces;
  return HS_OK;
}

HS_API hs_status hs_tess_count(const hs_groom* g, const hs_tess_params* p, uint64_t* out_vertices) {
  hs_status st = validate_tess(g, p, "hs_tess_count");
  if (st != HS_OK) return st;
  if (!out_vertices) return fail(HS_ERR_INVALID_ARG, "hs_tess_count: null output");
  *out_vertices = 2 * tess_segments(g, p);
  return HS_OK;
}

HS_API hs_status hs_tess_stream(hs_groom* g, const hs_tess_params* p, uint64_t* out_vertices) {
  hs_status st = validate_tess(g, p, "hs_tess_stream");
  if (st != HS_OK) return st;
  HS_ON_DEVICE(g->ctx, "hs_tess_stream");
  if (!g->d_tess_tangents) return fail(HS_ERR_NOT_INITIALIZED, "hs_tess_stream: call hs_tess_setup first");
  const uint64_t segs = tess_segments(g, p);
  cudaStream_t s = g->ctx->stream;
  cudaError_t e = cudaSuccess;
  if (2 * segs > g->tess_cap) {
    e = cudaStreamSynchronize(s);  // the old buffer may still be read
    cudaFree(g->d_tess);
    g->d_tess = nullptr;
    g->tess_cap = 0;
    if (e == cudaSuccess) e = cudaMalloc(&g->d_tess, sizeof(float4) * 2 * std::max<uint64_t>(segs, 1));
    if (e != cudaSuccess) {
      g->d_tess = nullptr;
      return cuda_fail(e, "hs_tess_stream: device allocation");
    }
    g->tess_cap = 2 * std::max<uint64_t>(segs, 1);
  }
  g->tess_count = 2 * segs;
  if (out_vertices) *out_vertices = 2 * segs;
  if (segs == 0) return HS_OK;
  TessArgs a;
  a.pos = g->d_pos;
  a.tangent = g->d_tess_tangents;
  a.faces = reinterpret_cast<const uint3*>(g->d_tess_faces);
  a.random = g->d_tess_random;
  a.out = g->d_tess;
  a.stride = g->stride;
  a.npoints = g->npoints;
  a.nfaces = g->tess_nfaces;
  a.ninstances = p->ninstances;
  a.nlines = p->nlines;
  a.nsub = p->nsubsegments;
  a.scale = p->length_scale;
  a.nvertices = segs / p->nsubsegments * (p->nsubsegments + 1);
  a.lines = FastDiv::make(p->nlines);
  a.segs = FastDiv::make(g->npoints - 1);
  a.faces_div = FastDiv::make(g->tess_nfaces);
  // One wave of resident blocks: each builds the tables once.
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tess, kTessBlock, 0) != cudaSuccess) {
    cudaGetLastError();
    per_sm = 1;
  }
  const uint64_t resident = static_cast<uint64_t>(std::max(1, per_sm)) *
                            static_cast<uint64_t>(device_attribute(cudaDevAttrMultiProcessorCount, 1));
  const uint64_t groups = (a.nvertices / (p->nsubsegments + 1) + 31) / 32;
  const uint64_t blocks = std::min<uint64_t>((groups + kTessBlock / 32 - 1) / (kTessBlock / 32), resident);
  k_tess<<<static_cast<unsigned>(std::max<uint64_t>(blocks, 1)), kTessBlock, 0, s>>>(a);
  e = cudaGetLastError();
  g->ctx->launches += 1;
  if (e != cudaSuccess) return cuda_fail(e, "hs_tess_stream: launch");
  return HS_OK;
}

HS_API hs_status hs_tess_device(hs_groom* g, const void** out_dptr, uint64_t* out_vertices) {
  if (!g || !out_dptr || !out_vertices) return fail(HS_ERR_INVALID_ARG, "hs_tess_device: null argument");
  *out_dptr = g->d_tess;
  *out_vertices = g->tess_count;
  return HS_OK;
}

HS_API hs_status hs_tess_readback(hs_groom* g, float* host_xyzw, size_t capacity_floats) {
  if (!g || !host_xyzw) return fail(HS_ERR_INVALID_ARG, "hs_tess_readback: null argument");
  HS_ON_DEVICE(g->ctx, "hs_tess_readback");
  const size_t need = 4 * static_cast<size_t>(g->tess_count);
  if (capacity_floats < need)
    return fail(HS_ERR_INVALID_ARG, "hs_tess_readback: capacity %zu < %zu floats", capacity_floats, need);
  if (need == 0) return HS_OK;
  cudaStream_t s = g->ctx->stream;
  cudaError_t e = cudaMemcpyAsync(host_xyzw, g->d_tess, sizeof(float) * need, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "hs_tess_readback");
  return HS_OK;
}

}  // extern "C"
