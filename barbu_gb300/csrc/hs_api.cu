// hs_api.cu -- the C-ABI of include/hairsim.h: contexts, grooms, per-frame
// inputs, the plain per-groom update and readback.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <set>
#include <string>
#include <vector>

#include "hairsim.h"
#include "hs_api_internal.h"
#include "hs_internal.h"

namespace {

thread_local std::string g_last_error;

}  // namespace

namespace hs {

hs_status fail(hs_status st, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return st;
}

hs_status cuda_fail(cudaError_t e, const char* what) {
  return fail(e == cudaErrorMemoryAllocation ? HS_ERR_OUT_OF_MEMORY : HS_ERR_CUDA, "%s: %s", what,
              cudaGetErrorString(e));
}

bool finite3(const float* v) { return std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]); }

hs_status validate_sim(const hs_sim_params* p) {
  if (!p) return fail(HS_ERR_INVALID_ARG, "sim params: null");
  if (p->mode != HS_MODE_REFERENCE && p->mode != HS_MODE_DFTL)
    return fail(HS_ERR_INVALID_ARG, "sim params: unknown mode %u", p->mode);
  if (p->substeps < 1 || p->substeps > HS_MAX_SUBSTEPS)
    return fail(HS_ERR_INVALID_ARG, "sim params: substeps %u outside [1, %d]", p->substeps, HS_MAX_SUBSTEPS);
  if (p->iterations < 1 || p->iterations > HS_MAX_ITERATIONS)
    return fail(HS_ERR_INVALID_ARG, "sim params: iterations %u outside [1, %d]", p->iterations,
                HS_MAX_ITERATIONS);
  if (p->root_mode > HS_ROOT_SKINNED) return fail(HS_ERR_INVALID_ARG, "sim params: unknown root mode %u", p->root_mode);
  if (!finite3(p->gravity) || !std::isfinite(p->gravity_scale) || !std::isfinite(p->damping) ||
      !std::isfinite(p->length_scale) || !std::isfinite(p->wind_jitter))
    return fail(HS_ERR_INVALID_ARG, "sim params: non-finite value");
  if (p->contract > HS_CONTRACT_FAST) return fail(HS_ERR_INVALID_ARG, "sim params: unknown contract %u", p->contract);
  if (p->contract == HS_CONTRACT_FAST && p->mode != HS_MODE_DFTL)
    return fail(HS_ERR_INVALID_ARG, "sim params: the FAST contract is for DFTL mode (reference mode is exact)");
  return HS_OK;
}

GroomView view_of(const hs_groom* g) {
  GroomView v;
  v.pos = g->d_pos;
  v.vel = g->d_vel;
  v.root_rest = g->d_root_rest;
  v.root_target = g->d_root_target;
  v.skin = g->d_skin;
  v.stats = g->d_stats;
  v.order = g->d_order;
  v.nstrands = g->nstrands;
  v.stride = g->stride;
  v.npoints = g->npoints;
  v.strand_base = g->strand_base;
  return v;
}

hs_status make_frame_const(const hs_groom* g, float dt, FrameConst* out) {
  const hs_sim_params& p = g->sim;
  if (!std::isfinite(dt) || dt < 0.0f) return fail(HS_ERR_INVALID_ARG, "update: dt must be finite and >= 0");
  if (p.mode == HS_MODE_DFTL && !(dt > 0.0f)) return fail(HS_ERR_INVALID_ARG, "update: DFTL mode needs dt > 0");
  if (p.root_mode == HS_ROOT_EXPLICIT && !g->d_root_target)
    return fail(HS_ERR_NOT_INITIALIZED, "update: root mode needs targets (hs_set_roots) first");
  if (p.root_mode == HS_ROOT_SKINNED) {
    if (!g->d_skin) return fail(HS_ERR_NOT_INITIALIZED, "update: skinned roots need influences (hs_set_skin) first");
    if (g->nbones <= g->skin_max_bone)
      return fail(HS_ERR_NOT_INITIALIZED, "update: influences use bone %u but the palette has %u bones",
                  g->skin_max_bone, g->nbones);
  }
  FrameConst fc;
  std::memset(&fc, 0, sizeof(fc));
  // These host float operations mirror the oracle's: one rounding each.
  fc.h = dt / static_cast<float>(p.substeps);
  fc.h2 = fc.h * fc.h;
  fc.inv_h = 1.0f / fc.h;
  fc.damping = p.damping;
  fc.length_scale = p.length_scale;
  fc.wind_jitter = p.wind_jitter;
  fc.Gx = p.gravity_scale * p.gravity[0];
  fc.Gy = p.gravity_scale * p.gravity[1];
  fc.Gz = p.gravity_scale * p.gravity[2];
  fc.wx = g->wind[0];
  fc.wy = g->wind[1];
  fc.wz = g->wind[2];
  std::memcpy(fc.m, g->m, sizeof(fc.m));
  fc.substeps = static_cast<int32_t>(p.substeps);
  fc.iterations = static_cast<int32_t>(p.iterations);
  fc.mode = static_cast<int32_t>(p.mode);
  fc.root_mode = static_cast<int32_t>(p.root_mode);
  fc.nspheres = static_cast<int32_t>(g->spheres.size());
  fc.wind_key = stream_key(g->seed, kStreamWind);
  fc.contract = static_cast<int32_t>(p.contract);
  float rmax = 0.0f;
  const size_t K = g->spheres.size();
  for (size_t k = 0; k < K; ++k) {
    fc.spheres[k] = g->spheres[k];
    fc.r2[k] = g->spheres[k].w * g->spheres[k].w;
    rmax = std::fmax(rmax, g->spheres[k].w);
  }
  fc.sphere_rmax = rmax;
  std::memcpy(fc.adj, g->adj, sizeof(fc.adj));
  std::memcpy(fc.bone_real, g->bone_real, sizeof(fc.bone_real));
  std::memcpy(fc.bone_dual, g->bone_dual, sizeof(fc.bone_dual));
  *out = fc;
  return HS_OK;
}

// Rigid 4x4 transform (column-major) to a unit dual quaternion, 8 floats:
// real (x, y, z, w), then dual (x, y, z, w). The rotation quaternion is
// K. Shoemake's trace-branch construction ("Animating rotation with
// quaternion curves", 1985): w from the trace when it is positive, else the
// largest diagonal term gives the first component. The dual part is
// 0.5 * (t, 0) * real. This is the conversion the reference makes on the CPU
// before skinning (src/fx/animation/skeleton_controller.cc:259-264).
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
  // (t, 0) * (v, w) = (w t + t x v, -t . v)
  dq[4] = 0.5f * ((w * tx) + (ty * z - tz * y));
  dq[5] = 0.5f * ((w * ty) + (tz * x - tx * z));
  dq[6] = 0.5f * ((w * tz) + (tx * y - ty * x));
  dq[7] = -0.5f * ((tx * x + ty * y) + tz * z);
}

}  // namespace hs

using namespace hs;

extern "C" {

HS_API const char* hs_last_error_string(void) { return g_last_error.c_str(); }

HS_API void hs_sim_params_reference(hs_sim_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->mode = HS_MODE_REFERENCE;
  p->substeps = 1;
  p->iterations = 8;          // kNumContraintsIteration, cs_simulation.glsl:197
  p->root_mode = HS_ROOT_PINNED;
  p->gravity[1] = -9.81f;     // :71
  p->gravity_scale = 20.0f;   // kForceCoeff, :72
  p->damping = 0.80f;         // mix(0.80, 0.94, 0), :100-102
  p->length_scale = 1.0f;     // uScaleFactor default, :41
  p->wind_jitter = 0.0f;
}

HS_API void hs_sim_params_dftl(hs_sim_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->mode = HS_MODE_DFTL;
  p->substeps = 4;
  p->iterations = 1;
  p->root_mode = HS_ROOT_PINNED;
  p->gravity[1] = -9.81f;
  p->gravity_scale = 1.0f;
  p->damping = 0.9f;
  p->length_scale = 1.0f;
  p->wind_jitter = 0.0f;
}

HS_API void hs_strand_params_reference(hs_strand_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->points_per_strand = 4;   // HAIR_MAX_PARTICLE_PER_STRAND, interop.h:8
  p->length_rule = HS_LENGTH_REFERENCE;
  p->max_length = 0.5f;       // Parameters_t::sim.maxlength, hair.h:29
  p->length_jitter = 0.1f;    // hair.cc:269
  p->seed = 0;
  p->lengths = nullptr;
}

HS_API hs_status hs_create(hs_ctx** out_ctx) {
  if (!out_ctx) return fail(HS_ERR_INVALID_ARG, "hs_create: null output");
  *out_ctx = nullptr;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "hs_create: cudaGetDevice");
  hs_ctx* ctx = new (std::nothrow) hs_ctx();
  if (!ctx) return fail(HS_ERR_OUT_OF_MEMORY, "hs_create: host allocation");
  ctx->device = dev;
  e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete ctx;
    return cuda_fail(e, "hs_create: cudaStreamCreate");
  }
  *out_ctx = ctx;
  return HS_OK;
}

HS_API hs_status hs_destroy(hs_ctx* ctx) {
  if (!ctx) return fail(HS_ERR_INVALID_ARG, "hs_destroy: null context");
  HS_ON_DEVICE(ctx, "hs_destroy");
  cudaStreamSynchronize(ctx->stream);
  destroy_ctx_extensions(ctx);
  std::set<hs_groom*> grooms = ctx->grooms;
  for (hs_groom* g : grooms) hs_groom_destroy(g);
  if (ctx->copy_stream) {
    cudaStreamSynchronize(ctx->copy_stream);
    cudaStreamDestroy(ctx->copy_stream);
  }
  for (cudaEvent_t ev : ctx->pending) cudaEventDestroy(ev);
  for (cudaEvent_t ev : ctx->spare_events) cudaEventDestroy(ev);
  for (int i = 0; i < 2; ++i) {
    cudaFree(ctx->d_many[i]);
    if (ctx->many_ready[i]) cudaEventDestroy(ctx->many_ready[i]);
    if (ctx->many_free[i]) cudaEventDestroy(ctx->many_free[i]);
  }
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return HS_OK;
}

HS_API hs_status hs_ctx_stream(hs_ctx* ctx, void** out_stream) {
  if (!ctx || !out_stream) return fail(HS_ERR_INVALID_ARG, "hs_ctx_stream: null argument");
  *out_stream = static_cast<void*>(ctx->stream);
  return HS_OK;
}

HS_API hs_status hs_sync(hs_ctx* ctx) {
  if (!ctx) return fail(HS_ERR_INVALID_ARG, "hs_sync: null context");
  HS_ON_DEVICE(ctx, "hs_sync");
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_fail(e, "hs_sync");
  return HS_OK;
}

HS_API hs_status hs_ctx_launch_count(hs_ctx* ctx, uint64_t* out_count) {
  if (!ctx || !out_count) return fail(HS_ERR_INVALID_ARG, "hs_ctx_launch_count: null argument");
  *out_count = ctx->launches;
  return HS_OK;
}

}  // extern "C"

namespace hs {

hs_status pack_skin(const uint8_t* bones, const float* weights, uint32_t nstrands, uint32_t stride,
                    std::vector<uint4>* out, uint32_t* max_bone, const char* what) {
  out->assign(stride, make_uint4(0u, 0u, 0u, 0u));
  *max_bone = 0;
  for (uint32_t s = 0; s < nstrands; ++s) {
    uint32_t packed = 0;
    for (int k = 0; k < 4; ++k) {
      const uint32_t b = bones[4 * static_cast<size_t>(s) + k];
      if (b >= HS_MAX_BONES) return fail(HS_ERR_INVALID_ARG, "%s: strand %u bone %u >= %d", what, s, b, HS_MAX_BONES);
      *max_bone = std::max(*max_bone, b);
      packed |= b << (8 * k);
    }
    const float* w = weights + 3 * static_cast<size_t>(s);
    if (!std::isfinite(w[0]) || !std::isfinite(w[1]) || !std::isfinite(w[2]))
      return fail(HS_ERR_INVALID_ARG, "%s: strand %u has a non-finite weight", what, s);
    uint32_t wb[3];
    std::memcpy(wb, w, sizeof(wb));
    (*out)[s] = make_uint4(packed, wb[0], wb[1], wb[2]);
  }
  return HS_OK;
}

size_t groom_state_bytes(uint32_t nstrands, uint32_t npoints) {
  const size_t stride = (static_cast<size_t>(nstrands) + 31u) & ~static_cast<size_t>(31u);
  // positions and velocities [npoints][stride], rest roots [stride], the
  // frame statistics (2 float4 per 32-strand tile), the strand order
  // [stride] (stride is a multiple of 32: every part stays 16-byte aligned).
  return sizeof(float4) * stride * (2 * static_cast<size_t>(npoints) + 1) + 2 * sizeof(float4) * (stride / 32) +
         sizeof(uint32_t) * stride;
}

void strand_order(const float* roots, size_t root_stride_floats, uint32_t n, uint32_t stride, bool keep,
                  std::vector<uint32_t>* order, std::vector<uint32_t>* inv) {
  order->resize(stride);
  for (uint32_t j = 0; j < stride; ++j) (*order)[j] = j;
  if (!keep && n > 32) {
    float lo[3] = {roots[0], roots[1], roots[2]}, hi[3] = {roots[0], roots[1], roots[2]};
    for (uint32_t s = 0; s < n; ++s)
      for (int a = 0; a < 3; ++a) {
        lo[a] = std::min(lo[a], roots[s * root_stride_floats + a]);
        hi[a] = std::max(hi[a], roots[s * root_stride_floats + a]);
      }
    std::vector<std::pair<uint32_t, uint32_t>> key(n);
    for (uint32_t s = 0; s < n; ++s) {
      uint32_t q[3];
      for (int a = 0; a < 3; ++a) {
        const float ext = hi[a] - lo[a];
        const float t = ext > 0.0f ? (roots[s * root_stride_floats + a] - lo[a]) / ext : 0.0f;
        q[a] = static_cast<uint32_t>(std::min(1023.0f, std::max(0.0f, t * 1023.0f)));
      }
      uint32_t code = 0;
      for (int b = 0; b < 10; ++b)
        for (int a = 0; a < 3; ++a) code |= ((q[a] >> b) & 1u) << (3 * b + a);
      key[s] = std::make_pair(code, s);
    }
    std::sort(key.begin(), key.end());  // ties by caller index: deterministic
    for (uint32_t j = 0; j < n; ++j) (*order)[j] = key[j].second;
  }
  inv->resize(n);
  for (uint32_t j = 0; j < n; ++j) (*inv)[(*order)[j]] = j;
}

hs_status make_groom_shell(hs_ctx* ctx, uint32_t nstrands, uint32_t npoints, uint64_t seed,
                           const hs_sim_params* sim, hs_groom** out) {
  if (nstrands == 0) return fail(HS_ERR_INVALID_ARG, "groom: nstrands must be > 0");
  if (npoints < HS_MIN_POINTS_PER_STRAND || npoints > HS_MAX_POINTS_PER_STRAND)
    return fail(HS_ERR_INVALID_ARG, "groom: points per strand %u outside [%d, %d]", npoints,
                HS_MIN_POINTS_PER_STRAND, HS_MAX_POINTS_PER_STRAND);
  if (step_capacity(npoints) == 0)
    return fail(HS_ERR_UNSUPPORTED, "groom: %u points per strand has no compiled kernel", npoints);
  hs_status st = validate_sim(sim);
  if (st != HS_OK) return st;
  hs_groom* g = new (std::nothrow) hs_groom();
  if (!g) return fail(HS_ERR_OUT_OF_MEMORY, "groom: host allocation");
  g->ctx = ctx;
  g->nstrands = nstrands;
  g->npoints = npoints;
  g->stride = (nstrands + 31u) & ~31u;
  g->seed = seed;
  g->sim = *sim;
  g->state_bytes = groom_state_bytes(nstrands, npoints);
  // Identity root transform (the reference's uModel default, :37).
  for (int c = 0; c < 16; ++c) g->m[c] = (c % 5 == 0) ? 1.0f : 0.0f;
  *out = g;
  return HS_OK;
}

void place_groom(hs_groom* g, char* mem, bool pool_owned) {
  g->d_mem = mem;
  g->pool_owned = pool_owned;
  const size_t plane = static_cast<size_t>(g->stride) * g->npoints;
  g->d_pos = reinterpret_cast<float4*>(mem);
  g->d_vel = g->d_pos + plane;
  g->d_root_rest = g->d_vel + plane;
  g->d_stats = g->d_root_rest + g->stride;
  g->d_order = reinterpret_cast<uint32_t*>(g->d_stats + 2 * (g->stride / 32));
}

cudaError_t init_groom_on_device(hs_groom* g, const float* d_roots, const float* d_normals, const float* d_lengths,
                                 const hs_strand_params* strand, cudaStream_t st) {
  InitArgs a;
  a.roots = d_roots;
  a.normals = d_normals;
  a.lengths = d_lengths;
  a.length_rule = strand->length_rule;
  a.max_length = strand->max_length;
  a.length_jitter = strand->length_jitter;
  a.length_key = stream_key(strand->seed, kStreamLength);
  a.strand_base = strand->strand_base;
  g->strand_base = strand->strand_base;
  g->ctx->launches += 1;
  return launch_init(view_of(g), a, g->d_root_rest, st);
}

hs_status validate_strand(const hs_strand_params* strand, const float* roots, const float* normals,
                          const float* lengths, uint32_t nstrands) {
  if (strand->length_rule > HS_LENGTH_TOTAL) return fail(HS_ERR_INVALID_ARG, "groom: unknown length rule");
  if (!std::isfinite(strand->max_length) || !std::isfinite(strand->length_jitter) || strand->max_length < 0.0f)
    return fail(HS_ERR_INVALID_ARG, "groom: bad max_length / length_jitter");
  for (size_t k = 0; k < 3 * static_cast<size_t>(nstrands); ++k) {
    if (!std::isfinite(roots[k]) || !std::isfinite(normals[k]))
      return fail(HS_ERR_INVALID_ARG, "groom: non-finite root or normal at strand %zu", k / 3);
  }
  if (lengths) {
    for (uint32_t s = 0; s < nstrands; ++s)
      if (!std::isfinite(lengths[s]) || lengths[s] < 0.0f)
        return fail(HS_ERR_INVALID_ARG, "groom: bad length at strand %u", s);
  }
  return HS_OK;
}

}  // namespace hs

extern "C" {

static hs_status alloc_groom(hs_ctx* ctx, uint32_t nstrands, uint32_t npoints, uint64_t seed,
                             const hs_sim_params* sim, hs_groom** out) {
  hs_groom* g = nullptr;
  hs_status st = make_groom_shell(ctx, nstrands, npoints, seed, sim, &g);
  if (st != HS_OK) return st;
  char* mem = nullptr;
  cudaError_t e = cudaMalloc(&mem, g->state_bytes);
  if (e != cudaSuccess) {
    delete g;
    cudaGetLastError();
    return cuda_fail(e, "groom: device allocation");
  }
  place_groom(g, mem, false);
  *out = g;
  return HS_OK;
}

HS_API hs_status hs_groom_init(hs_ctx* ctx, const float* root_pos, const float* root_nrm, uint32_t nstrands,
                               const hs_strand_params* strand, const hs_sim_params* sim, hs_groom** out_groom) {
  if (!ctx || !root_pos || !root_nrm || !strand || !out_groom)
    return fail(HS_ERR_INVALID_ARG, "hs_groom_init: null argument");
  HS_ON_DEVICE(ctx, "hs_groom_init");
  *out_groom = nullptr;
  hs_status st = validate_strand(strand, root_pos, root_nrm, strand->lengths, nstrands);
  if (st != HS_OK) return st;
  hs_groom* g = nullptr;
  st = alloc_groom(ctx, nstrands, strand->points_per_strand, strand->seed, sim, &g);
  if (st != HS_OK) return st;
  strand_order(root_pos, 3, nstrands, g->stride, strand->keep_order != 0, &g->order, &g->inv);
  std::vector<float> roots, normals, lengths;
  to_stored(g, root_pos, 3, &roots);
  to_stored(g, root_nrm, 3, &normals);
  if (strand->lengths) to_stored(g, strand->lengths, 1, &lengths);

  // Stage roots, normals (and lengths) in the stored order on the device,
  // then expand there.
  const size_t n3 = sizeof(float) * 3 * static_cast<size_t>(nstrands);
  float* d_in = nullptr;
  const size_t in_bytes = 2 * n3 + (strand->lengths ? sizeof(float) * nstrands : 0);
  cudaError_t e = cudaMalloc(&d_in, in_bytes);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(g->d_order, g->order.data(), sizeof(uint32_t) * g->stride, cudaMemcpyHostToDevice,
                        ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_in, roots.data(), n3, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_in + 3 * static_cast<size_t>(nstrands), normals.data(), n3, cudaMemcpyHostToDevice,
                        ctx->stream);
  if (e == cudaSuccess && strand->lengths)
    e = cudaMemcpyAsync(d_in + 6 * static_cast<size_t>(nstrands), lengths.data(), sizeof(float) * nstrands,
                        cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess)
    e = init_groom_on_device(g, d_in, d_in + 3 * static_cast<size_t>(nstrands),
                             strand->lengths ? d_in + 6 * static_cast<size_t>(nstrands) : nullptr, strand, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(d_in);
  if (e != cudaSuccess) {
    free_groom(g);
    return cuda_fail(e, "hs_groom_init");
  }
  ctx->grooms.insert(g);
  *out_groom = g;
  return HS_OK;
}

HS_API hs_status hs_groom_init_from_state(hs_ctx* ctx, const float* pos_xyzw, const float* vel_xyzw,
                                          uint32_t nstrands, uint32_t npoints, uint64_t seed,
                                          const hs_sim_params* sim, hs_groom** out_groom) {
  if (!ctx || !pos_xyzw || !vel_xyzw || !out_groom)
    return fail(HS_ERR_INVALID_ARG, "hs_groom_init_from_state: null argument");
  HS_ON_DEVICE(ctx, "hs_groom_init_from_state");
  *out_groom = nullptr;
  const size_t nfl = 4 * static_cast<size_t>(nstrands) * npoints;
  for (size_t k = 0; k < nfl; ++k) {
    if (!std::isfinite(pos_xyzw[k]) || !std::isfinite(vel_xyzw[k]))
      return fail(HS_ERR_INVALID_ARG, "hs_groom_init_from_state: non-finite value at float %zu", k);
  }
  hs_groom* g = nullptr;
  hs_status st = alloc_groom(ctx, nstrands, npoints, seed, sim, &g);
  if (st != HS_OK) return st;
  // Stored in the spatial order of the roots (point 0 of each strand).
  strand_order(pos_xyzw, 4 * static_cast<size_t>(npoints), nstrands, g->stride, false, &g->order, &g->inv);
  float4* d_tmp = nullptr;
  const size_t bytes = sizeof(float) * nfl;
  cudaError_t e = cudaMalloc(&d_tmp, bytes);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(g->d_order, g->order.data(), sizeof(uint32_t) * g->stride, cudaMemcpyHostToDevice,
                        ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_tmp, pos_xyzw, bytes, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess)
    e = launch_from_strand_major(d_tmp, g->d_pos, g->d_order, nstrands, npoints, g->stride, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_tmp, vel_xyzw, bytes, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess)
    e = launch_from_strand_major(d_tmp, g->d_vel, g->d_order, nstrands, npoints, g->stride, ctx->stream);
  if (e == cudaSuccess) e = launch_copy_roots(g->d_pos, g->d_root_rest, nstrands, ctx->stream);
  ctx->launches += 3;
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(d_tmp);
  if (e != cudaSuccess) {
    free_groom(g);
    return cuda_fail(e, "hs_groom_init_from_state");
  }
  ctx->grooms.insert(g);
  *out_groom = g;
  return HS_OK;
}

HS_API hs_status hs_groom_destroy(hs_groom* g) {
  if (!g) return fail(HS_ERR_INVALID_ARG, "hs_groom_destroy: null groom");
  HS_ON_DEVICE(g->ctx, "hs_groom_destroy");
  cudaStreamSynchronize(g->ctx->stream);
  g->ctx->grooms.erase(g);
  free_groom(g);
  return HS_OK;
}

HS_API hs_status hs_groom_set_params(hs_groom* g, const hs_sim_params* sim) {
  if (!g) return fail(HS_ERR_INVALID_ARG, "hs_groom_set_params: null groom");
  hs_status st = validate_sim(sim);
  if (st != HS_OK) return st;
  g->sim = *sim;
  return HS_OK;
}

HS_API hs_status hs_groom_info(const hs_groom* g, uint32_t* out_nstrands, uint32_t* out_npoints) {
  if (!g) return fail(HS_ERR_INVALID_ARG, "hs_groom_info: null groom");
  if (out_nstrands) *out_nstrands = g->nstrands;
  if (out_npoints) *out_npoints = g->npoints;
  return HS_OK;
}

HS_API hs_status hs_set_bounding_sphere(hs_groom* g, const float xyzr[4]) {
  return hs_set_spheres(g, xyzr, 1);
}

HS_API hs_status hs_set_spheres(hs_groom* g, const float* xyzr, uint32_t n) { return set_spheres(g, xyzr, n); }

}  // extern "C"

hs_status hs::set_spheres(hs_groom* g, const float* xyzr, uint32_t n) {
  if (!g || (n > 0 && !xyzr)) return fail(HS_ERR_INVALID_ARG, "hs_set_spheres: null argument");
  if (n > HS_MAX_SPHERES) return fail(HS_ERR_INVALID_ARG, "hs_set_spheres: %u spheres > %d", n, HS_MAX_SPHERES);
  for (uint32_t k = 0; k < n; ++k) {
    const float* s = xyzr + 4 * k;
    if (!finite3(s) || !std::isfinite(s[3]) || s[3] < 0.0f)
      return fail(HS_ERR_INVALID_ARG, "hs_set_spheres: sphere %u not finite or negative radius", k);
  }
  g->spheres.resize(n);
  for (uint32_t k = 0; k < n; ++k) g->spheres[k] = make_float4(xyzr[4 * k], xyzr[4 * k + 1], xyzr[4 * k + 2], xyzr[4 * k + 3]);
  // Overlap masks for the exact sphere culling of the step kernel: a point
  // pushed onto sphere k can only be inside sphere j if the two overlap.
  // The margin is far above FP32 rounding of the push-out.
  std::memset(g->adj, 0, sizeof(g->adj));
  for (uint32_t k = 0; k < n; ++k) {
    const float4 a = g->spheres[k];
    for (uint32_t j = 0; j < n; ++j) {
      if (j == k) continue;
      const float4 b = g->spheres[j];
      const double dx = double(a.x) - b.x, dy = double(a.y) - b.y, dz = double(a.z) - b.z;
      const double mag = 1.0 + std::fmax(std::fmax(std::fabs(a.x), std::fabs(a.y)),
                                         std::fmax(std::fmax(std::fabs(a.z), std::fabs(b.x)),
                                                   std::fmax(std::fabs(b.y), std::fabs(b.z))));
      const double lim = (double(a.w) + b.w) * 1.001 + 1.0e-4 * (mag + a.w + b.w);
      if (dx * dx + dy * dy + dz * dz < lim * lim) g->adj[k] |= 1u << j;
    }
  }
  return HS_OK;
}

extern "C" {

HS_API hs_status hs_set_wind(hs_groom* g, const float wind[3]) {
  if (!g || !wind) return fail(HS_ERR_INVALID_ARG, "hs_set_wind: null argument");
  if (!finite3(wind)) return fail(HS_ERR_INVALID_ARG, "hs_set_wind: non-finite wind");
  std::memcpy(g->wind, wind, sizeof(g->wind));
  return HS_OK;
}

HS_API hs_status hs_set_root_transform(hs_groom* g, const float m[16]) {
  if (!g || !m) return fail(HS_ERR_INVALID_ARG, "hs_set_root_transform: null argument");
  for (int c = 0; c < 16; ++c)
    if (!std::isfinite(m[c])) return fail(HS_ERR_INVALID_ARG, "hs_set_root_transform: non-finite entry %d", c);
  std::memcpy(g->m, m, sizeof(g->m));
  return HS_OK;
}

HS_API hs_status hs_set_root_transforms(hs_groom* const* grooms, uint32_t n, const float* m) {
  if (n > 0 && (!grooms || !m)) return fail(HS_ERR_INVALID_ARG, "hs_set_root_transforms: null argument");
  for (uint32_t i = 0; i < n; ++i) {
    if (!grooms[i]) return fail(HS_ERR_INVALID_ARG, "hs_set_root_transforms: groom %u is null", i);
    for (int c = 0; c < 16; ++c)
      if (!std::isfinite(m[16 * i + c]))
        return fail(HS_ERR_INVALID_ARG, "hs_set_root_transforms: non-finite entry in matrix %u", i);
  }
  for (uint32_t i = 0; i < n; ++i) std::memcpy(grooms[i]->m, m + 16 * i, sizeof(grooms[i]->m));
  return HS_OK;
}

HS_API hs_status hs_set_roots(hs_groom* g, const float* xyz, uint32_t nstrands) {
  if (!g || !xyz) return fail(HS_ERR_INVALID_ARG, "hs_set_roots: null argument");
  HS_ON_DEVICE(g->ctx, "hs_set_roots");
  if (nstrands != g->nstrands)
    return fail(HS_ERR_INVALID_ARG, "hs_set_roots: %u targets for %u strands", nstrands, g->nstrands);
  for (size_t k = 0; k < 3 * static_cast<size_t>(nstrands); ++k)
    if (!std::isfinite(xyz[k])) return fail(HS_ERR_INVALID_ARG, "hs_set_roots: non-finite target");
  cudaStream_t st = g->ctx->stream;
  cudaError_t e = cudaSuccess;
  if (!g->d_root_target) e = cudaMalloc(&g->d_root_target, sizeof(float4) * g->stride);
  if (e != cudaSuccess) {
    g->d_root_target = nullptr;
    return cuda_fail(e, "hs_set_roots: device allocation");
  }
  g->h_targets.resize(g->nstrands);
  for (uint32_t j = 0; j < nstrands; ++j) {
    const float* t = xyz + 3 * static_cast<size_t>(g->order[j]);  // stored order
    g->h_targets[j] = make_float4(t[0], t[1], t[2], 0.0f);
  }
  // The copy is ordered before the next update on the stream; wait for it so
  // the staging vector can be reused by the next call.
  e = cudaMemcpyAsync(g->d_root_target, g->h_targets.data(), sizeof(float4) * nstrands, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "hs_set_roots: copy");
  return HS_OK;
}

HS_API hs_status hs_set_skin(hs_groom* g, const uint8_t* bones, const float* weights, uint32_t nstrands) {
  if (!g || !bones || !weights) return fail(HS_ERR_INVALID_ARG, "hs_set_skin: null argument");
  HS_ON_DEVICE(g->ctx, "hs_set_skin");
  if (nstrands != g->nstrands)
    return fail(HS_ERR_INVALID_ARG, "hs_set_skin: influences for %u strands, groom has %u", nstrands, g->nstrands);
  std::vector<uint4> hc, h(g->stride, make_uint4(0u, 0u, 0u, 0u));
  uint32_t max_bone = 0;
  hs_status pst = pack_skin(bones, weights, nstrands, g->stride, &hc, &max_bone, "hs_set_skin");
  if (pst != HS_OK) return pst;
  for (uint32_t j = 0; j < nstrands; ++j) h[j] = hc[g->order[j]];  // stored order
  cudaStream_t st = g->ctx->stream;
  cudaError_t e = cudaSuccess;
  if (!g->d_skin) e = cudaMalloc(&g->d_skin, sizeof(uint4) * g->stride);
  if (e != cudaSuccess) {
    g->d_skin = nullptr;
    return cuda_fail(e, "hs_set_skin: device allocation");
  }
  // Ordered before the next update; waited for so `h` can go.
  e = cudaMemcpyAsync(g->d_skin, h.data(), sizeof(uint4) * g->stride, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "hs_set_skin: copy");
  g->skin_max_bone = max_bone;
  return HS_OK;
}

HS_API hs_status hs_set_bone_dual_quats(hs_groom* g, const float* dq, uint32_t nbones) {
  if (!g || (nbones > 0 && !dq)) return fail(HS_ERR_INVALID_ARG, "hs_set_bone_dual_quats: null argument");
  if (nbones > HS_MAX_BONES)
    return fail(HS_ERR_INVALID_ARG, "hs_set_bone_dual_quats: %u bones > %d", nbones, HS_MAX_BONES);
  for (uint32_t b = 0; b < nbones; ++b) {
    const float* q = dq + 8 * static_cast<size_t>(b);
    for (int k = 0; k < 8; ++k)
      if (!std::isfinite(q[k])) return fail(HS_ERR_INVALID_ARG, "hs_set_bone_dual_quats: bone %u non-finite", b);
    if (q[0] == 0.0f && q[1] == 0.0f && q[2] == 0.0f && q[3] == 0.0f)
      return fail(HS_ERR_INVALID_ARG, "hs_set_bone_dual_quats: bone %u has a zero rotation part", b);
  }
  for (uint32_t b = 0; b < HS_MAX_BONES; ++b) {
    const float* q = dq + 8 * static_cast<size_t>(b);
    g->bone_real[b] = b < nbones ? make_float4(q[0], q[1], q[2], q[3]) : make_float4(0.0f, 0.0f, 0.0f, 1.0f);
    g->bone_dual[b] = b < nbones ? make_float4(q[4], q[5], q[6], q[7]) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  }
  g->nbones = nbones;
  return HS_OK;
}

HS_API hs_status hs_set_bone_matrices(hs_groom* g, const float* m, uint32_t nbones) {
  if (!g || (nbones > 0 && !m)) return fail(HS_ERR_INVALID_ARG, "hs_set_bone_matrices: null argument");
  if (nbones > HS_MAX_BONES) return fail(HS_ERR_INVALID_ARG, "hs_set_bone_matrices: %u bones > %d", nbones, HS_MAX_BONES);
  float dq[8 * HS_MAX_BONES];
  for (uint32_t b = 0; b < nbones; ++b) {
    const float* mb = m + 16 * static_cast<size_t>(b);
    for (int k = 0; k < 16; ++k)
      if (!std::isfinite(mb[k])) return fail(HS_ERR_INVALID_ARG, "hs_set_bone_matrices: bone %u non-finite", b);
    matrix_to_dual_quat(mb, dq + 8 * b);
  }
  return hs_set_bone_dual_quats(g, dq, nbones);
}

HS_API hs_status hs_update(hs_groom* g, float dt) {
  if (!g) return fail(HS_ERR_INVALID_ARG, "hs_update: null groom");
  HS_ON_DEVICE(g->ctx, "hs_update");
  FrameConst fc;
  hs_status st = make_frame_const(g, dt, &fc);
  if (st != HS_OK) return st;
  if (g->mapping == HS_MAPPING_LANES && lane_group(fc.mode, fc.substeps, fc.iterations) == 0)
    return fail(HS_ERR_UNSUPPORTED, "hs_update: lane groups need DFTL mode, one iteration and 2..16 substeps");
  cudaError_t e = launch_step(view_of(g), fc, static_cast<int>(g->mapping), g->ctx->stream);
  g->ctx->launches += 1;
  if (e != cudaSuccess) return cuda_fail(e, "hs_update: launch");
  g->stats_valid = true;
  return HS_OK;
}

HS_API hs_status hs_groom_set_mapping(hs_groom* g, uint32_t mapping) {
  if (!g) return fail(HS_ERR_INVALID_ARG, "hs_groom_set_mapping: null groom");
  if (mapping > HS_MAPPING_LANES) return fail(HS_ERR_INVALID_ARG, "hs_groom_set_mapping: unknown mapping %u", mapping);
  g->mapping = mapping;
  return HS_OK;
}

HS_API hs_status hs_groom_mapping(hs_groom* g, uint32_t* out) {
  if (!g || !out) return fail(HS_ERR_INVALID_ARG, "hs_groom_mapping: null argument");
  HS_ON_DEVICE(g->ctx, "hs_groom_mapping");
  FrameConst fc;
  hs_status st = make_frame_const(g, 1.0f / 60.0f, &fc);
  if (st != HS_OK) return st;
  *out = static_cast<uint32_t>(plain_mapping(view_of(g), fc, static_cast<int>(g->mapping)));
  return HS_OK;
}

HS_API hs_status hs_groom_stats(hs_groom* g, hs_frame_stats* out) {
  if (!g || !out) return fail(HS_ERR_INVALID_ARG, "hs_groom_stats: null argument");
  HS_ON_DEVICE(g->ctx, "hs_groom_stats");
  std::memset(out, 0, sizeof(*out));
  if (!g->stats_valid) return HS_OK;
  const size_t ntiles = (static_cast<size_t>(g->nstrands) + 31) / 32;
  std::vector<float4> h(2 * ntiles);
  cudaStream_t st = g->ctx->stream;
  cudaError_t e = cudaMemcpyAsync(h.data(), g->d_stats, sizeof(float4) * h.size(), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "hs_groom_stats");
  float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY}, v2 = 0.0f;
  double ke = 0.0;
  for (size_t t = 0; t < ntiles; ++t) {
    const float4 a = h[2 * t], b = h[2 * t + 1];
    mn[0] = std::fmin(mn[0], a.x);
    mn[1] = std::fmin(mn[1], a.y);
    mn[2] = std::fmin(mn[2], a.z);
    mx[0] = std::fmax(mx[0], b.x);
    mx[1] = std::fmax(mx[1], b.y);
    mx[2] = std::fmax(mx[2], b.z);
    ke += static_cast<double>(a.w);
    v2 = std::fmax(v2, b.w);
  }
  for (int k = 0; k < 3; ++k) {
    out->bounds_min[k] = mn[k];
    out->bounds_max[k] = mx[k];
  }
  out->max_speed = std::sqrt(v2);
  out->kinetic_energy = ke;
  out->valid = 1;
  return HS_OK;
}

// comps: 4 = (x, y, z, w) per point, 3 = (x, y, z).
static cudaError_t snapshot_into(hs_groom* g, const float4* src, int comps, float* dst, cudaStream_t st) {
  g->ctx->launches += 1;
  return comps == 4 ? launch_to_strand_major(src, reinterpret_cast<float4*>(dst), g->d_order, g->nstrands,
                                             g->npoints, g->stride, st)
                    : launch_to_strand_major_xyz(src, dst, g->d_order, g->nstrands, g->npoints, g->stride, st);
}

static cudaError_t ensure_event(cudaEvent_t* ev) {
  if (*ev) return cudaSuccess;
  const cudaError_t e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
  if (e != cudaSuccess) *ev = nullptr;
  return e;
}

// Staging buffer `slot` of the groom, with its two events.
static cudaError_t ensure_out(hs_groom* g, int slot) {
  cudaError_t e = ensure_event(&g->out_ready[slot]);
  if (e == cudaSuccess) e = ensure_event(&g->out_free[slot]);
  if (e != cudaSuccess || g->d_out[slot]) return e;
  e = cudaMalloc(&g->d_out[slot], sizeof(float4) * static_cast<size_t>(g->nstrands) * g->npoints);
  if (e != cudaSuccess) g->d_out[slot] = nullptr;
  return e;
}

static cudaError_t ensure_copy_stream(hs_ctx* ctx) {
  if (ctx->copy_stream) return cudaSuccess;
  const cudaError_t e = cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) ctx->copy_stream = nullptr;
  return e;
}

// Marks the end of an asynchronous readback (the copy stream's work queued
// so far) for hs_readback_drain.
static cudaError_t push_pending(hs_ctx* ctx) {
  cudaEvent_t ev = nullptr;
  if (!ctx->spare_events.empty()) {
    ev = ctx->spare_events.back();
    ctx->spare_events.pop_back();
  } else {
    const cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e != cudaSuccess) return e;
  }
  const cudaError_t e = cudaEventRecord(ev, ctx->copy_stream);
  if (e != cudaSuccess) {
    ctx->spare_events.push_back(ev);
    return e;
  }
  ctx->pending.push_back(ev);
  return cudaSuccess;
}

static hs_status readback(hs_groom* g, const float4* src, int comps, float* host, size_t capacity_floats,
                          const char* what) {
  if (!g || !host) return fail(HS_ERR_INVALID_ARG, "%s: null argument", what);
  HS_ON_DEVICE(g->ctx, what);
  const size_t need = static_cast<size_t>(comps) * g->nstrands * g->npoints;
  if (capacity_floats < need) return fail(HS_ERR_INVALID_ARG, "%s: capacity %zu < %zu floats", what, capacity_floats, need);
  cudaStream_t st = g->ctx->stream;
  cudaError_t e = ensure_out(g, 0);
  // An asynchronous readback may still be copying out of the buffer.
  if (e == cudaSuccess) e = cudaStreamWaitEvent(st, g->out_free[0], 0);
  float* staging = reinterpret_cast<float*>(g->d_out[0]);
  if (e == cudaSuccess) e = snapshot_into(g, src, comps, staging, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(host, staging, sizeof(float) * need, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, what);
  return HS_OK;
}

// Asynchronous readback: the strand-major snapshot is written into one of
// the groom's two staging buffers on the context stream (after the updates
// queued before it), and copied to host on the context's copy stream, so
// that the copy of frame f overlaps the update of frame f + 1; the buffers
// take turns, so the snapshot of frame f + 1 overlaps that copy too.
// out_free[i] orders the next snapshot into buffer i after its copy;
// hs_readback_wait and hs_readback_drain wait for the copies.
static hs_status readback_async(hs_groom* g, int comps, float* host, size_t capacity_floats, const char* what) {
  if (!g || !host) return fail(HS_ERR_INVALID_ARG, "%s: null argument", what);
  HS_ON_DEVICE(g->ctx, what);
  const size_t need = static_cast<size_t>(comps) * g->nstrands * g->npoints;
  if (capacity_floats < need) return fail(HS_ERR_INVALID_ARG, "%s: capacity %zu < %zu floats", what, capacity_floats, need);
  hs_ctx* ctx = g->ctx;
  const int slot = g->out_next;
  cudaError_t e = ensure_copy_stream(ctx);
  if (e == cudaSuccess) e = ensure_out(g, slot);
  if (e != cudaSuccess) return cuda_fail(e, what);
  cudaStream_t st = ctx->stream;
  float* staging = reinterpret_cast<float*>(g->d_out[slot]);
  e = cudaStreamWaitEvent(st, g->out_free[slot], 0);  // the previous copy out of this buffer is done
  if (e == cudaSuccess) e = snapshot_into(g, g->d_pos, comps, staging, st);
  if (e == cudaSuccess) e = cudaEventRecord(g->out_ready[slot], st);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->copy_stream, g->out_ready[slot], 0);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(host, staging, sizeof(float) * need, cudaMemcpyDeviceToHost, ctx->copy_stream);
  if (e == cudaSuccess) e = cudaEventRecord(g->out_free[slot], ctx->copy_stream);
  if (e == cudaSuccess) e = push_pending(ctx);
  if (e != cudaSuccess) return cuda_fail(e, what);
  g->out_next = slot ^ 1;
  return HS_OK;
}

HS_API hs_status hs_readback_async(hs_groom* g, float* host_xyzw, size_t capacity_floats) {
  return readback_async(g, 4, host_xyzw, capacity_floats, "hs_readback_async");
}

HS_API hs_status hs_readback_xyz_async(hs_groom* g, float* host_xyz, size_t capacity_floats) {
  return readback_async(g, 3, host_xyz, capacity_floats, "hs_readback_xyz_async");
}

// Several grooms into one host buffer: their snapshots into one of the
// context's two staging buffers (in list order, each strand-major), then
// one copy of the whole.
HS_API hs_status hs_readback_many_async(hs_ctx* ctx, hs_groom* const* grooms, uint32_t n, uint32_t comps,
                                        float* host, size_t capacity_floats) {
  const char* what = "hs_readback_many_async";
  if (!ctx || !host || (n > 0 && !grooms)) return fail(HS_ERR_INVALID_ARG, "%s: null argument", what);
  if (comps != 3 && comps != 4) return fail(HS_ERR_INVALID_ARG, "%s: comps must be 3 or 4, not %u", what, comps);
  HS_ON_DEVICE(ctx, what);
  size_t need = 0;
  for (uint32_t i = 0; i < n; ++i) {
    if (!grooms[i]) return fail(HS_ERR_INVALID_ARG, "%s: groom %u is null", what, i);
    if (grooms[i]->ctx != ctx) return fail(HS_ERR_INVALID_ARG, "%s: groom %u belongs to another context", what, i);
    need += static_cast<size_t>(comps) * grooms[i]->nstrands * grooms[i]->npoints;
  }
  if (capacity_floats < need) return fail(HS_ERR_INVALID_ARG, "%s: capacity %zu < %zu floats", what, capacity_floats, need);
  if (need == 0) return HS_OK;
  const int slot = ctx->many_next;
  cudaError_t e = ensure_copy_stream(ctx);
  if (e == cudaSuccess) e = ensure_event(&ctx->many_ready[slot]);
  if (e == cudaSuccess) e = ensure_event(&ctx->many_free[slot]);
  if (e == cudaSuccess && ctx->many_cap[slot] < need) {
    // A copy out of the old buffer may be in flight.
    e = cudaEventSynchronize(ctx->many_free[slot]);
    if (e == cudaSuccess) {
      cudaFree(ctx->d_many[slot]);
      ctx->d_many[slot] = nullptr;
      ctx->many_cap[slot] = 0;
      e = cudaMalloc(&ctx->d_many[slot], sizeof(float) * need);
      if (e == cudaSuccess) ctx->many_cap[slot] = need;
      else ctx->d_many[slot] = nullptr;
    }
  }
  if (e != cudaSuccess) return cuda_fail(e, what);
  cudaStream_t st = ctx->stream;
  e = cudaStreamWaitEvent(st, ctx->many_free[slot], 0);  // the previous copy out of this buffer is done
  size_t at = 0;
  for (uint32_t i = 0; i < n && e == cudaSuccess; ++i) {
    hs_groom* g = grooms[i];
    e = snapshot_into(g, g->d_pos, static_cast<int>(comps), ctx->d_many[slot] + at, st);
    at += static_cast<size_t>(comps) * g->nstrands * g->npoints;
  }
  if (e == cudaSuccess) e = cudaEventRecord(ctx->many_ready[slot], st);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->copy_stream, ctx->many_ready[slot], 0);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(host, ctx->d_many[slot], sizeof(float) * need, cudaMemcpyDeviceToHost, ctx->copy_stream);
  if (e == cudaSuccess) e = cudaEventRecord(ctx->many_free[slot], ctx->copy_stream);
  if (e == cudaSuccess) e = push_pending(ctx);
  if (e != cudaSuccess) return cuda_fail(e, what);
  ctx->many_next = slot ^ 1;
  return HS_OK;
}

HS_API hs_status hs_readback_drain(hs_ctx* ctx, uint32_t keep) {
  if (!ctx) return fail(HS_ERR_INVALID_ARG, "hs_readback_drain: null context");
  HS_ON_DEVICE(ctx, "hs_readback_drain");
  while (ctx->pending.size() > keep) {
    cudaEvent_t ev = ctx->pending.front();
    const cudaError_t e = cudaEventSynchronize(ev);
    if (e != cudaSuccess) return cuda_fail(e, "hs_readback_drain");
    ctx->pending.pop_front();
    ctx->spare_events.push_back(ev);
  }
  return HS_OK;
}

HS_API hs_status hs_readback_wait(hs_ctx* ctx) {
  if (!ctx) return fail(HS_ERR_INVALID_ARG, "hs_readback_wait: null context");
  HS_ON_DEVICE(ctx, "hs_readback_wait");
  if (!ctx->copy_stream) return HS_OK;
  cudaError_t e = cudaStreamSynchronize(ctx->copy_stream);
  if (e != cudaSuccess) return cuda_fail(e, "hs_readback_wait");
  while (!ctx->pending.empty()) {
    ctx->spare_events.push_back(ctx->pending.front());
    ctx->pending.pop_front();
  }
  return HS_OK;
}

HS_API hs_status hs_export(hs_groom* g, uint32_t field, uint32_t layout, void* d_dst, size_t capacity_floats) {
  if (!g || !d_dst) return fail(HS_ERR_INVALID_ARG, "hs_export: null argument");
  HS_ON_DEVICE(g->ctx, "hs_export");
  if (field > HS_FIELD_VELOCITIES || layout > HS_EXPORT_POINT_MAJOR)
    return fail(HS_ERR_INVALID_ARG, "hs_export: unknown field %u or layout %u", field, layout);
  if (reinterpret_cast<uintptr_t>(d_dst) % 16 != 0)
    return fail(HS_ERR_INVALID_ARG, "hs_export: destination not 16-byte aligned");
  const size_t need = 4 * static_cast<size_t>(g->nstrands) * g->npoints;
  if (capacity_floats < need) return fail(HS_ERR_INVALID_ARG, "hs_export: capacity %zu < %zu floats", capacity_floats, need);
  cudaPointerAttributes pa;
  if (cudaPointerGetAttributes(&pa, d_dst) != cudaSuccess || pa.devicePointer == nullptr || pa.device != g->ctx->device) {
    cudaGetLastError();
    return fail(HS_ERR_INVALID_ARG, "hs_export: destination is not device memory of the context's device");
  }
  const float4* src = field == HS_FIELD_POSITIONS ? g->d_pos : g->d_vel;
  float4* dst = static_cast<float4*>(d_dst);
  cudaStream_t st = g->ctx->stream;
  cudaError_t e = cudaSuccess;
  if (layout == HS_EXPORT_STRAND_MAJOR) {
    e = launch_to_strand_major(src, dst, g->d_order, g->nstrands, g->npoints, g->stride, st);
  } else {
    e = launch_to_point_major(src, dst, g->d_order, g->nstrands, g->npoints, g->stride, st);
  }
  g->ctx->launches += 1;
  if (e != cudaSuccess) return cuda_fail(e, "hs_export");
  return HS_OK;
}

HS_API hs_status hs_readback(hs_groom* g, float* host_xyzw, size_t capacity_floats) {
  return readback(g, g ? g->d_pos : nullptr, 4, host_xyzw, capacity_floats, "hs_readback");
}

HS_API hs_status hs_readback_xyz(hs_groom* g, float* host_xyz, size_t capacity_floats) {
  return readback(g, g ? g->d_pos : nullptr, 3, host_xyz, capacity_floats, "hs_readback_xyz");
}

HS_API hs_status hs_readback_velocities(hs_groom* g, float* host_xyzw, size_t capacity_floats) {
  return readback(g, g ? g->d_vel : nullptr, 4, host_xyzw, capacity_floats, "hs_readback_velocities");
}

HS_API hs_status hs_device_positions(hs_groom* g, const void** out_dptr, hs_layout* out_layout) {
  if (!g || !out_dptr) return fail(HS_ERR_INVALID_ARG, "hs_device_positions: null argument");
  *out_dptr = g->d_pos;
  if (out_layout) {
    out_layout->nstrands = g->nstrands;
    out_layout->points_per_strand = g->npoints;
    out_layout->strand_stride = g->stride;
    out_layout->reserved = 0;
  }
  return HS_OK;
}

HS_API hs_status hs_groom_strand_order(hs_groom* g, uint32_t* out, uint32_t capacity, uint32_t* out_count) {
  if (!g || !out_count || (capacity > 0 && !out)) return fail(HS_ERR_INVALID_ARG, "hs_groom_strand_order: null argument");
  const uint32_t n = std::min(capacity, g->nstrands);
  for (uint32_t j = 0; j < n; ++j) out[j] = g->order[j];
  *out_count = g->nstrands;
  return HS_OK;
}

}  // extern "C"

namespace hs {

void free_groom(hs_groom* g) {
  if (!g) return;
  for (int i = 0; i < 2; ++i) {
    if (g->out_free[i]) cudaEventSynchronize(g->out_free[i]);  // a copy out of d_out[i] in flight
    if (g->out_ready[i]) cudaEventDestroy(g->out_ready[i]);
    if (g->out_free[i]) cudaEventDestroy(g->out_free[i]);
  }
  if (!g->pool_owned) cudaFree(g->d_mem);
  cudaFree(g->d_root_target);
  cudaFree(g->d_skin);
  cudaFree(g->d_tess_faces);
  cudaFree(g->d_tess_tangents);
  cudaFree(g->d_tess_random);
  cudaFree(g->d_tess);
  cudaFree(g->d_out[0]);
  cudaFree(g->d_out[1]);
  delete g;
}

}  // namespace hs
