// glsl_shim.h -- just enough of GLSL 4.30 for the reference's hair
// simulation compute shader and its tessellation evaluation shader
// (src/shaders/hair/02_tess_stream/tes_stream_hair.glsl) to compile as C++.
//
// TEST INFRASTRUCTURE ONLY: used by make_ref.py to build the reference
// shader (src/shaders/hair/01_simulation/cs_simulation.glsl) into
// oracle/_ref/, which pins the oracle through golden vectors.
//
// Builtins are restated from their definitions in the GLSL 4.30
// specification (section 8), in IEEE binary32, with these choices where
// the specification leaves the rounding to the implementation:
//   dot(a,b)       = fma(a.z,b.z, fma(a.y,b.y, a.x*b.x))
//   inversesqrt(x) = a magic-constant first estimate (C. Lomont, "Fast
//                    Inverse Square Root", 2003: bits 0x5f3759df - (bits(x)>>1)),
//                    two Newton-Raphson steps y *= 1.5 - (x/2) y^2, and a
//                    last step in residual form, r = 1 - x y^2 by fma,
//                    y += (y/2) r. Error < 1 ulp for normal x (GLSL allows 2).
//   normalize(v)   = v * inversesqrt(dot(v,v))
//   reflect(I,N)   = I - 2 * dot(N,I) * N
//   smoothstep     = t*t*(3-2t), t = clamp((x-e0)/(e1-e0), 0, 1)
//   mix(x,y,a)     = x*(1-a) + y*a
//   vec4 * mat4    = component j: fma(v.w,m[j].w, fma(v.z,m[j].z, fma(v.y,m[j].y, v.x*m[j].x)))
//   mat3x4 * vec3  = fma(m[2], v.z, fma(m[1], v.y, m[0] * v.x)) per component
//   max(x,y)       = x < y ? y : x;  min(x,y) = y < x ? y : x
// (the skinning and Marschner shaders' builtins are listed further down)
// Compile with -ffp-contract=off: the operators below round every step.
//
// Work-group execution: a shader invocation is a host thread; the
// local_size_x invocations of a work group run concurrently and
// memoryBarrierShared() / groupMemoryBarrier() are execution barriers
// across them. That is the order the shader intends (all write shared,
// invocation 0 solves, all read back); on the GPU it holds because a
// 4-invocation group runs inside one warp.
#ifndef ORACLE_GLSL_SHIM_H_
#define ORACLE_GLSL_SHIM_H_

#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>

namespace glsl {

typedef uint32_t uint;

struct vec4;

struct vec2 {
  float x, y;
  vec2() : x(0.f), y(0.f) {}
  vec2(float a, float b) : x(a), y(b) {}
  vec2 xy_swizzle() const { return *this; }
};

struct vec3 {
  float x, y, z;
  vec3() : x(0.f), y(0.f), z(0.f) {}
  explicit vec3(float s) : x(s), y(s), z(s) {}
  vec3(float a, float b, float c) : x(a), y(b), z(c) {}
  vec3(const vec2& v, float c) : x(v.x), y(v.y), z(c) {}
  explicit vec3(const vec4& v);
  vec2 xy_swizzle() const { return vec2(x, y); }
  vec3& operator*=(float s) {
    x = x * s;
    y = y * s;
    z = z * s;
    return *this;
  }
};

struct vec4 {
  float x, y, z, w;
  vec4() : x(0.f), y(0.f), z(0.f), w(0.f) {}
  explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
  vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
  vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
  vec3 xyz_swizzle() const { return vec3(x, y, z); }
  float& operator[](int i) { return i == 0 ? x : i == 1 ? y : i == 2 ? z : w; }
  float operator[](int i) const { return i == 0 ? x : i == 1 ? y : i == 2 ? z : w; }
  vec4& operator*=(float s) {
    x = x * s;
    y = y * s;
    z = z * s;
    w = w * s;
    return *this;
  }
};

inline vec3::vec3(const vec4& v) : x(v.x), y(v.y), z(v.z) {}

// Column-major, as GLSL: m[c] is column c.
struct mat4 {
  vec4 c[4];
  mat4() {}
  vec4& operator[](int i) { return c[i]; }
  const vec4& operator[](int i) const { return c[i]; }
  explicit mat4(float s) {
    c[0] = vec4(s, 0.f, 0.f, 0.f);
    c[1] = vec4(0.f, s, 0.f, 0.f);
    c[2] = vec4(0.f, 0.f, s, 0.f);
    c[3] = vec4(0.f, 0.f, 0.f, s);
  }
  mat4(vec4 a, vec4 b, vec4 d, vec4 e) {
    c[0] = a;
    c[1] = b;
    c[2] = d;
    c[3] = e;
  }
};

// Three columns of four.
struct mat3x4 {
  vec4 c[3];
  explicit mat3x4(const mat4& m) {
    c[0] = m.c[0];
    c[1] = m.c[1];
    c[2] = m.c[2];
  }
  mat3x4(vec4 a, vec4 b, vec4 d) {
    c[0] = a;
    c[1] = b;
    c[2] = d;
  }
};

inline vec3 operator+(vec3 a, vec3 b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(vec3 a, vec3 b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(vec3 a, vec3 b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator*(float s, vec3 a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator*(vec3 a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator-(vec3 a) { return vec3(-a.x, -a.y, -a.z); }
// mat4 * vec4: columns scaled by the vector's components, accumulated in
// order with fma (as mat3x4 * vec3).
inline vec4 operator*(const mat4& m, vec4 v) {
  vec4 r;
  r.x = std::fma(m.c[3].x, v.w, std::fma(m.c[2].x, v.z, std::fma(m.c[1].x, v.y, m.c[0].x * v.x)));
  r.y = std::fma(m.c[3].y, v.w, std::fma(m.c[2].y, v.z, std::fma(m.c[1].y, v.y, m.c[0].y * v.x)));
  r.z = std::fma(m.c[3].z, v.w, std::fma(m.c[2].z, v.z, std::fma(m.c[1].z, v.y, m.c[0].z * v.x)));
  r.w = std::fma(m.c[3].w, v.w, std::fma(m.c[2].w, v.z, std::fma(m.c[1].w, v.y, m.c[0].w * v.x)));
  return r;
}

inline float dot4(vec4 a, vec4 b) { return std::fma(a.w, b.w, std::fma(a.z, b.z, std::fma(a.y, b.y, a.x * b.x))); }
// Row vector times matrix.
inline vec4 operator*(vec4 v, const mat4& m) { return vec4(dot4(v, m.c[0]), dot4(v, m.c[1]), dot4(v, m.c[2]), dot4(v, m.c[3])); }
inline vec4 operator*(const mat3x4& m, vec3 v) {
  return vec4(std::fma(m.c[2].x, v.z, std::fma(m.c[1].x, v.y, m.c[0].x * v.x)),
              std::fma(m.c[2].y, v.z, std::fma(m.c[1].y, v.y, m.c[0].y * v.x)),
              std::fma(m.c[2].z, v.z, std::fma(m.c[1].z, v.y, m.c[0].z * v.x)),
              std::fma(m.c[2].w, v.z, std::fma(m.c[1].w, v.y, m.c[0].w * v.x)));
}
inline float max(float x, float y) { return x < y ? y : x; }
inline float min(float x, float y) { return y < x ? y : x; }

inline float fma(float a, float b, float c) { return std::fma(a, b, c); }
inline vec3 fma(vec3 a, vec3 b, vec3 c) {
  return vec3(std::fma(a.x, b.x, c.x), std::fma(a.y, b.y, c.y), std::fma(a.z, b.z, c.z));
}
inline float dot(vec3 a, vec3 b) { return std::fma(a.z, b.z, std::fma(a.y, b.y, a.x * b.x)); }
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
inline vec3 normalize(vec3 v) { return v * inversesqrt(dot(v, v)); }
inline vec3 reflect(vec3 i, vec3 n) { return i - 2.0f * dot(n, i) * n; }
inline float clamp(float x, float lo, float hi) { return x < lo ? lo : (x > hi ? hi : x); }
inline float smoothstep(float e0, float e1, float x) {
  const float t = clamp((x - e0) / (e1 - e0), 0.0f, 1.0f);
  return t * t * (3.0f - 2.0f * t);
}
inline float mix(float x, float y, float a) { return x * (1.0f - a) + y * a; }
inline vec3 mix(vec3 x, vec3 y, float a) { return vec3(mix(x.x, y.x, a), mix(x.y, y.y, a), mix(x.z, y.z, a)); }


// ---- for the skinning and Marschner shaders ---------------------------------
//   cross(a,b)      = (fma(a.y,b.z, -(a.z*b.y)), fma(a.z,b.x, -(a.x*b.z)), fma(a.x,b.y, -(a.y*b.x)))
//   vec4 * mat3x4   = row vector times matrix: component j = dot4(v, m[j])
//   pow(x, 2)       = x * x (GLSL leaves pow undefined for x < 0 and the
//                     shaders square signed values); other exponents powf
//   degrees(x)      = x * 57.2957795131, radians(x) = x * 0.0174532925199
//   asin, acos, sin, cos, exp, sqrt: the C library's float functions.
struct uvec4 {
  uint x, y, z, w;
  uvec4() : x(0), y(0), z(0), w(0) {}
  uvec4(uint a, uint b, uint c, uint d) : x(a), y(b), z(c), w(d) {}
};
struct ivec4 {
  int x, y, z, w;
  explicit ivec4(const uvec4& u) : x(int(u.x)), y(int(u.y)), z(int(u.z)), w(int(u.w)) {}
  ivec4(int a, int b, int c, int d) : x(a), y(b), z(c), w(d) {}
};
inline ivec4 operator*(int s, const ivec4& v) { return ivec4(s * v.x, s * v.y, s * v.z, s * v.w); }
struct uvec2_t {
  uint x, y;
};
struct ivec2 {
  int x, y;
  explicit ivec2(const uvec2_t& v) : x(int(v.x)), y(int(v.y)) {}
  ivec2(int a, int b) : x(a), y(b) {}
};
inline vec3& operator+=(vec3& a, vec3 b) { return a = a + b; }
inline vec3 cross(vec3 a, vec3 b) {
  return vec3(std::fma(a.y, b.z, -(a.z * b.y)), std::fma(a.z, b.x, -(a.x * b.z)), std::fma(a.x, b.y, -(a.y * b.x)));
}
inline float dot(vec4 a, vec4 b) { return dot4(a, b); }
inline vec3 operator*(vec4 v, const mat3x4& m) { return vec3(dot4(v, m.c[0]), dot4(v, m.c[1]), dot4(v, m.c[2])); }
inline float sign(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
inline vec3 sign(vec3 v) { return vec3(sign(v.x), sign(v.y), sign(v.z)); }
inline float abs(float x) { return std::fabs(x); }
inline vec3 abs(vec3 v) { return vec3(std::fabs(v.x), std::fabs(v.y), std::fabs(v.z)); }
inline float sqrt(float x) { return std::sqrt(x); }
inline float asin(float x) { return std::asin(x); }
inline float acos(float x) { return std::acos(x); }
inline float sin(float x) { return std::sin(x); }
inline float cos(float x) { return std::cos(x); }
inline float exp(float x) { return std::exp(x); }
inline vec3 exp(vec3 v) { return vec3(std::exp(v.x), std::exp(v.y), std::exp(v.z)); }
inline float pow(float x, float y) { return y == 2.0f ? x * x : std::pow(x, y); }
inline float step(float edge, float x) { return x < edge ? 0.0f : 1.0f; }
inline float degrees(float x) { return x * 57.2957795131f; }
inline float radians(float x) { return x * 0.0174532925199f; }
inline vec3 operator/(vec3 a, vec3 b) { return vec3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline vec4 operator*(float s, vec4 v) { return vec4(s * v.x, s * v.y, s * v.z, s * v.w); }
inline vec4 operator*(vec4 v, float s) { return vec4(v.x * s, v.y * s, v.z * s, v.w * s); }
inline vec4 operator*(vec4 a, vec4 b) { return vec4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
// Swizzle assignments, which make_ref.py rewrites into calls.
inline void glsl_set_xyz(vec4& v, vec3 a) {
  v.x = a.x;
  v.y = a.y;
  v.z = a.z;
}
inline void glsl_mul_xyz(vec4& v, vec3 a) {
  v.x = v.x * a.x;
  v.y = v.y * a.y;
  v.z = v.z * a.z;
}
// A buffer texture of vec4 texels.
typedef const vec4* samplerBuffer;
inline vec4 texelFetch(samplerBuffer b, int i) { return b[i]; }

// ---- work-group emulation -------------------------------------------------

// Sense-reversing spin barrier for the invocations of one work group.
struct SpinBarrier {
  std::atomic<unsigned> count{0};
  std::atomic<unsigned> phase{0};
  unsigned n = 1;
  void wait() {
    const unsigned ph = phase.load(std::memory_order_acquire);
    if (count.fetch_add(1, std::memory_order_acq_rel) + 1 == n) {
      count.store(0, std::memory_order_relaxed);
      phase.store(ph + 1, std::memory_order_release);
    } else {
      while (phase.load(std::memory_order_acquire) == ph) std::this_thread::yield();
    }
  }
};

inline SpinBarrier& group_barrier() {
  static SpinBarrier b;
  return b;
}
inline void memoryBarrierShared() { group_barrier().wait(); }
inline void groupMemoryBarrier() { group_barrier().wait(); }

struct uvec3_t {
  uint x, y, z;
  uvec2_t xy_swizzle() const { return uvec2_t{x, y}; }
};
inline thread_local uvec3_t gl_GlobalInvocationID{0, 0, 0};
inline thread_local uint gl_LocalInvocationIndex = 0;

}  // namespace glsl

#endif  // ORACLE_GLSL_SHIM_H_
