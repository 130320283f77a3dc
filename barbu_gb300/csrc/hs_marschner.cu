// hs_marschner.cu -- the Marschner reflectance lookup tables.
//
// The reference precomputes two RGBA16F tables for its hair shading with two
// compute shaders (src/fx/marschner.cc:33-67): the longitudinal scattering
// M (cs_marschner_m.glsl: three Gaussian lobes R, TT, TRT of the half angle
// and cos(theta_d)) and the azimuthal scattering N (cs_marschner_n.glsl:
// N_p for p = 0, 1, 2 by inc_marschner_n.glsl:87-118, the cubic root solver
// of inc_solver.glsl and the Fresnel terms of inc_fresnel.glsl). Marschner
// et al. 2003, "Light Scattering from Human Hair Fibers". Here they are two
// kernels, one thread per texel, writing into the caller's device buffers
// (the headless stand-in for the GL textures), as half or float RGBA.
//
// The arithmetic follows the shaders' expressions; the transcendental
// functions are CUDA's (asinf, acosf, sinf, cosf, expf, powf), so the
// tables match a CPU evaluation to the functions' ulps, not bit for bit.
// Constants are the reference's: Pi() = 3.141564 (inc_constants.glsl:7),
// Epsilon() = 1e-6. pow(x, 2) is taken as x * x (GLSL leaves pow undefined
// for x < 0, and the shaders square signed values).
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cmath>

#include "hs_api_internal.h"
#include "hs_internal.h"

namespace hs {
namespace {

constexpr float kPi = 3.141564f;     // the reference's Pi() (inc_constants.glsl:7)
constexpr float kEps = 1e-6f;        // Epsilon() (inc_constants.glsl:6)
constexpr float kEtaOrigin = 1.0f;   // inc_marschner_n.glsl:38

struct Roots {
  float r[3];
  int n;
};

__device__ __forceinline__ float sgn(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }

// inc_solver.glsl:31-58.
__device__ __forceinline__ Roots solve_linear(float a, float b) {
  Roots z{{0.0f, 0.0f, 0.0f}, 0};
  if (fabsf(a) > kEps) {
    z.r[0] = -b / a;
    z.n = 1;
  }
  return z;
}
__device__ __forceinline__ Roots solve_quadratic(float a, float b, float c) {
  if (fabsf(a) < kEps) return solve_linear(b, c);
  float delta = b * b - 4.0f * a * c;
  Roots z{{0.0f, 0.0f, 0.0f}, 0};
  if (delta < 0.0f) return z;
  delta = sqrtf(delta);
  z.r[0] = (-b + delta) / (2.0f * a);
  z.r[1] = (-b - delta) / (2.0f * a);
  z.n = 1 + (delta >= kEps ? 1 : 0);  // 1 + step(Epsilon(), delta)
  return z;
}
// inc_solver.glsl:71-122 (x^3 + a x^2 + b x + c).
__device__ __forceinline__ Roots solve_cubic_normalized(float a, float b, float c) {
  Roots z{{0.0f, 0.0f, 0.0f}, 0};
  if (fabsf(c) < kEps) {
    z = solve_quadratic(1.0f, a, b);
    z.r[z.n] = 0.0f;  // roots[int(roots.w)] = 0
    z.n += 1;
    return z;
  }
  const float Q = (3.0f * b - a * a) / 9.0f;
  const float R = (9.0f * a * b - 27.0f * c - 2.0f * a * a * a) / 54.0f;
  const float Q3 = Q * Q * Q;
  const float D = Q3 + R * R;
  const float third_a = a / 3.0f;
  if (D > 0.0f) {
    const float sqrtD = sqrtf(D);
    const float s = sgn(R + sqrtD) * powf(fabsf(R + sqrtD), 0.333f);
    const float t = sgn(R - sqrtD) * powf(fabsf(R - sqrtD), 0.333f);
    z.r[0] = s + t - third_a;
    z.n = 1;
  } else {
    const float theta = acosf(R * (1.0f / sqrtf(-Q3)));
    const float two_sqrt_q = 2.0f * sqrtf(-Q);
    z.r[0] = fmaf(two_sqrt_q, cosf(theta / 3.0f), -third_a);
    z.r[1] = fmaf(two_sqrt_q, cosf((theta + 2.0f * kPi) / 3.0f), -third_a);
    z.r[2] = fmaf(two_sqrt_q, cosf((theta + 4.0f * kPi) / 3.0f), -third_a);
    z.n = 3;
  }
  return z;
}
__device__ __forceinline__ Roots solve_cubic(float a, float b, float c, float d) {
  return fabsf(a) < kEps ? solve_quadratic(b, c, d) : solve_cubic_normalized(b / a, c / a, d / a);
}

// inc_fresnel.glsl:17-58.
__device__ __forceinline__ float fresnel_power_ratio(float eta_ratio, float na, float nb, float cos_i, float sin_i) {
  const float e = eta_ratio * sin_i;
  const float sin_t2 = e * e;
  if (sin_t2 > 1.0f) return 1.0f;
  const float cos_t = sqrtf(1.0f - sin_t2);
  const float A = na * cos_i;
  const float B = nb * cos_t;
  const float R = (A - B) / (A + B);
  return fminf(1.0f, R * R);
}
__device__ __forceinline__ float fresnel(float eta0, float eta_perp, float eta_par, float cos_a, float sin_a) {
  const float refl = fresnel_power_ratio(eta0 / eta_perp, eta0, eta_perp, cos_a, sin_a);
  const float trans = fresnel_power_ratio(eta0 / eta_par, eta_par, eta0, cos_a, sin_a);
  return refl * (1.0f - 0.5f) + trans * 0.5f;  // mix(refl, trans, 0.5)
}

// inc_marschner_n.glsl:45-118.
__device__ __forceinline__ float absorption_term(int p, float absorption, float eta_perp, float eta_par,
                                                 float cos_gi, float sin_gi) {
  if (p == 0) return fresnel(kEtaOrigin, eta_perp, eta_par, cos_gi, sin_gi);
  const float sin_gt = sin_gi / eta_perp;
  const float gt = asinf(sin_gt);
  const float cos_gt = cosf(gt);
  const float fi = fresnel(kEtaOrigin, eta_perp, eta_par, cos_gi, sin_gi);
  const float ft = fresnel(kEtaOrigin, 1.0f / eta_perp, 1.0f / eta_par, cos_gt, sin_gt);
  const float t = expf(-4.0f * absorption * (cos_gt * cos_gt));
  const float one_minus = 1.0f - fi;
  return (one_minus * one_minus) * powf(ft, static_cast<float>(p - 1)) * powf(t, static_cast<float>(p));
}

__device__ __forceinline__ float n_p(int p, float absorption, float eta_perp, float eta_par, float c, float phi) {
  // get_polynomial_coefficients (:40-49).
  const float pf = static_cast<float>(p);
  const float a = pf * c * -0.25801227547f;
  const float cc = pf * c * 1.90985931710f - 2.0f;
  const float d = pf * kPi - phi;
  const Roots z = solve_cubic(a, 0.0f, cc, d);
  float L = 0.0f;
  for (int i = 0; i < z.n; ++i) {
    const float gi = z.r[i];
    const float s = sinf(gi), co = cosf(gi);
    const float A = absorption_term(p, absorption, eta_perp, eta_par, co, s);
    // inv_first_derivative_factor (:55-62): 1 / |2 (3 a g^2 + c) / cos g|.
    const float f1 = (3.0f * a * (gi * gi) + cc) / co;
    L += A * (1.0f / fabsf(2.0f * f1));
  }
  return fminf(L, 1.0f);
}

template <typename Out>
__device__ __forceinline__ void put(Out* out, size_t i, float x, float y, float z, float w);
template <>
__device__ __forceinline__ void put<float4>(float4* out, size_t i, float x, float y, float z, float w) {
  out[i] = make_float4(x, y, z, w);
}
template <>
__device__ __forceinline__ void put<__half>(__half* out, size_t i, float x, float y, float z, float w) {
  out[4 * i] = __float2half_rn(x);
  out[4 * i + 1] = __float2half_rn(y);
  out[4 * i + 2] = __float2half_rn(z);
  out[4 * i + 3] = __float2half_rn(w);
}

// cs_marschner_m.glsl:33-61.
template <typename Out>
__global__ void k_marschner_m(Out* out, int res, float inv_res, float shift, float width) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= res || y >= res) return;
  const float sin_ti = 2.0f * static_cast<float>(x) * inv_res - 1.0f;
  const float sin_tr = 2.0f * static_cast<float>(y) * inv_res - 1.0f;
  const float ti = asinf(sin_ti);
  const float tr = asinf(sin_tr);
  const float th = (ti + tr) / 2.0f;
  const float td = (ti - tr) / 2.0f;
  const float deg = th * 57.2957795131f;  // degrees(): the GLSL builtin, 180 / pi
  const float shifts[3] = {1.0f * shift, -0.5f * shift, -1.5f * shift};
  const float widths[3] = {1.0f * width, 0.5f * width, 2.0f * width};
  float lobe[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float xm = deg - shifts[k];
    // gaussian (inc_maths.glsl:274-276).
    lobe[k] = expf(-(xm * xm) / (2.0f * widths[k] * widths[k])) / (2.5066282f * fabsf(widths[k]));
  }
  put(out, static_cast<size_t>(y) * res + x, lobe[0], lobe[1], lobe[2], cosf(td));
}

// cs_marschner_n.glsl:25-84 (the generic branch: N_p for p = 0, 1, 2).
template <typename Out>
__global__ void k_marschner_n(Out* out, int res, float inv_res, float eta, float absorption) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= res || y >= res) return;
  const float cos_phi_d = 2.0f * static_cast<float>(x) * inv_res - 1.0f;
  const float cos_theta_d = 2.0f * static_cast<float>(y) * inv_res - 1.0f;
  const float sin_td2 = 1.0f - cos_theta_d * cos_theta_d;
  const float eta2 = eta * eta;
  const float eta_perp = sqrtf(eta2 - sin_td2) / cos_theta_d;
  const float eta_par = eta2 / eta_perp;
  const float phi_d = acosf(cos_phi_d);
  const float c = asinf(1.0f / eta_perp);
  const float R = n_p(0, absorption, eta_perp, eta_par, c, phi_d);
  const float TT = n_p(1, absorption, eta_perp, eta_par, c, phi_d);
  const float TRT = n_p(2, absorption, eta_perp, eta_par, c, phi_d);
  put(out, static_cast<size_t>(y) * res + x, R, TT, TRT, 1.0f);
}

}  // namespace
}  // namespace hs

using namespace hs;

extern "C" {

HS_API void hs_marschner_params_reference(hs_marschner_params* p) {
  if (!p) return;
  // Marschner::ShadingParameters_t (src/fx/marschner.h:31-45).
  p->eta = 1.55f;
  p->absorption = 0.20f;
  p->eccentricity = 0.85f;
  p->ar = -5.0f;
  p->br = 5.0f;
  p->glint_scale = 0.5f;
  p->azimuthal_width = 10.0f;
  p->delta_caustic = 0.2f;
  p->delta_hm = 0.5f;
  p->resolution = 128;  // kTextureResolution (:24)
}

HS_API hs_status hs_marschner_luts(hs_ctx* ctx, const hs_marschner_params* p, uint32_t format, void* d_m, void* d_n) {
  if (!ctx || !p || (!d_m && !d_n)) return fail(HS_ERR_INVALID_ARG, "hs_marschner_luts: null argument");
  HS_ON_DEVICE(ctx, "hs_marschner_luts");
  if (format > HS_LUT_FLOAT4) return fail(HS_ERR_INVALID_ARG, "hs_marschner_luts: unknown format %u", format);
  if (p->resolution < 2 || p->resolution > 4096)
    return fail(HS_ERR_INVALID_ARG, "hs_marschner_luts: resolution %u outside [2, 4096]", p->resolution);
  if (!std::isfinite(p->eta) || !std::isfinite(p->absorption) || !std::isfinite(p->ar) || !std::isfinite(p->br))
    return fail(HS_ERR_INVALID_ARG, "hs_marschner_luts: non-finite parameter");
  const int res = static_cast<int>(p->resolution);
  const float inv = 1.0f / static_cast<float>(res);  // kInvTextureResolution (marschner.h:29)
  const dim3 block(16, 16);  // kComputeBlockSize (:25)
  const dim3 grid((res + 15) / 16, (res + 15) / 16);
  cudaStream_t st = ctx->stream;
  cudaError_t e = cudaSuccess;
  if (format == HS_LUT_HALF4) {
    if (d_m) k_marschner_m<__half><<<grid, block, 0, st>>>(static_cast<__half*>(d_m), res, inv, p->ar, p->br);
    if (d_n) k_marschner_n<__half><<<grid, block, 0, st>>>(static_cast<__half*>(d_n), res, inv, p->eta, p->absorption);
  } else {
    if (d_m) k_marschner_m<float4><<<grid, block, 0, st>>>(static_cast<float4*>(d_m), res, inv, p->ar, p->br);
    if (d_n)
      k_marschner_n<float4><<<grid, block, 0, st>>>(static_cast<float4*>(d_n), res, inv, p->eta, p->absorption);
  }
  e = cudaGetLastError();
  ctx->launches += (d_m ? 1 : 0) + (d_n ? 1 : 0);
  if (e != cudaSuccess) return cuda_fail(e, "hs_marschner_luts: launch");
  return HS_OK;
}

}  // extern "C"
