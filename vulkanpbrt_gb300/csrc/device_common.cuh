// Device-side helpers shared by the per-frame kernels: GLSL-like float3 math,
// storage-format conversions of the reference's Vulkan image formats, and the
// level-0 bilinear/REPEAT sampler the reference binds by default
// (external/vsg/include/vsg/state/Sampler.h:29-42).
#pragma once
#include <cuda_fp16.h>
#include <stdint.h>

#define PBRT_HD __host__ __device__ __forceinline__
#define PBRT_D __device__ __forceinline__

namespace pbrt {

PBRT_HD float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
PBRT_HD float3 f3(float s) { return make_float3(s, s, s); }
PBRT_HD float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
PBRT_HD float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
PBRT_HD float3 operator*(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
PBRT_HD float3 operator/(float3 a, float3 b) { return f3(a.x / b.x, a.y / b.y, a.z / b.z); }
PBRT_HD float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
PBRT_HD float3 operator*(float s, float3 a) { return f3(a.x * s, a.y * s, a.z * s); }
PBRT_HD float3 operator/(float3 a, float s) { return f3(a.x / s, a.y / s, a.z / s); }
PBRT_HD float3 operator-(float3 a) { return f3(-a.x, -a.y, -a.z); }
PBRT_HD float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
PBRT_HD float3 cross(float3 a, float3 b) {
  return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
PBRT_D float length(float3 a) { return sqrtf(dot(a, a)); }
PBRT_D float3 normalize(float3 a) { return a / length(a); }
PBRT_D float3 fmin3(float3 a, float3 b) { return f3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)); }
PBRT_D float3 fmax3(float3 a, float3 b) { return f3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)); }
PBRT_D float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
PBRT_D float3 clamp3(float3 x, float lo, float hi) {
  return f3(clampf(x.x, lo, hi), clampf(x.y, lo, hi), clampf(x.z, lo, hi));
}
PBRT_D float mixf(float x, float y, float a) { return x * (1.f - a) + y * a; }
PBRT_D float3 mix3(float3 x, float3 y, float a) { return x * (1.f - a) + y * a; }

// Column-major 4x4 (GLSL / vsg convention): c[col] = column.
struct Mat4 {
  float4 c[4];
};
// Unfused forms (each product and sum rounded on its own, in the shader's
// left-to-right order): the hit position, the ray origins built from it and
// the G-buffer depth come out bit-identical to an unfused FP32 evaluation.
PBRT_D float3 mul_rn(float3 a, float s) { return f3(__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s)); }
PBRT_D float3 add_rn(float3 a, float3 b) { return f3(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z)); }
PBRT_D float length_rn(float3 a) {
  return sqrtf(__fadd_rn(__fadd_rn(__fmul_rn(a.x, a.x), __fmul_rn(a.y, a.y)), __fmul_rn(a.z, a.z)));
}
PBRT_D float3 normalize_rn(float3 a) {
  const float l = length_rn(a);
  return f3(__fdiv_rn(a.x, l), __fdiv_rn(a.y, l), __fdiv_rn(a.z, l));
}
PBRT_D float4 mul(const Mat4& m, float4 v) {
  float4 r;
  r.x = m.c[0].x * v.x + m.c[1].x * v.y + m.c[2].x * v.z + m.c[3].x * v.w;
  r.y = m.c[0].y * v.x + m.c[1].y * v.y + m.c[2].y * v.z + m.c[3].y * v.w;
  r.z = m.c[0].z * v.x + m.c[1].z * v.y + m.c[2].z * v.z + m.c[3].z * v.w;
  r.w = m.c[0].w * v.x + m.c[1].w * v.y + m.c[2].w * v.z + m.c[3].w * v.w;
  return r;
}
// m * (p, 1), xyz, unfused: ((c0 p.x + c1 p.y) + c2 p.z) + c3.
PBRT_D float3 mul_point_rn(const Mat4& m, float3 p) {
  float3 r;
  r.x = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m.c[0].x, p.x), __fmul_rn(m.c[1].x, p.y)), __fmul_rn(m.c[2].x, p.z)), m.c[3].x);
  r.y = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m.c[0].y, p.x), __fmul_rn(m.c[1].y, p.y)), __fmul_rn(m.c[2].y, p.z)), m.c[3].y);
  r.z = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m.c[0].z, p.x), __fmul_rn(m.c[1].z, p.y)), __fmul_rn(m.c[2].z, p.z)), m.c[3].z);
  return r;
}

// Storage conversions: R16F/RGBA16F stores round to nearest even; UNORM8
// stores clamp to [0,1] and round to nearest.
PBRT_D float h2f(__half h) { return __half2float(h); }
PBRT_D __half f2h(float f) { return __float2half_rn(f); }
PBRT_D uint8_t f2u8(float f) { return (uint8_t)floorf(clampf(f, 0.f, 1.f) * 255.f + 0.5f); }
PBRT_D float u82f(uint8_t u) { return (float)u / 255.f; }

struct Half4 {
  __half x, y, z, w;
};
static_assert(sizeof(Half4) == 8, "RGBA16F texel is 8 bytes");
PBRT_D float4 load_half4(const Half4* p) {
  uint2 raw = *reinterpret_cast<const uint2*>(p);
  __half2 a = *reinterpret_cast<__half2*>(&raw.x), b = *reinterpret_cast<__half2*>(&raw.y);
  float2 fa = __half22float2(a), fb = __half22float2(b);
  return make_float4(fa.x, fa.y, fb.x, fb.y);
}
PBRT_D void store_half4(Half4* p, float x, float y, float z, float w) {
  __half2 a = __floats2half2_rn(x, y), b = __floats2half2_rn(z, w);
  uint2 raw;
  raw.x = *reinterpret_cast<uint32_t*>(&a);
  raw.y = *reinterpret_cast<uint32_t*>(&b);
  *reinterpret_cast<uint2*>(p) = raw;
}

// REPEAT addressing of a floored texel coordinate; NaN/inf map to texel 0.
PBRT_D int wrap_repeat(float c, int n) {
  if (!isfinite(c)) return 0;
  float m = c - (float)n * floorf(c / (float)n);
  int i = (int)m;
  return min(max(i, 0), n - 1);
}
// Level-0 bilinear sample at normalized uv: lerp along x, then along y.
template <class Fetch>
PBRT_D float4 bilinear(int W, int H, float u, float v, Fetch fetch) {
  float x = u * (float)W - 0.5f, y = v * (float)H - 0.5f;
  float x0 = floorf(x), y0 = floorf(y);
  float fx = x - x0, fy = y - y0;
  if (!isfinite(fx)) fx = 0.f;
  if (!isfinite(fy)) fy = 0.f;
  int i0 = wrap_repeat(x0, W), i1 = wrap_repeat(x0 + 1.f, W);
  int j0 = wrap_repeat(y0, H), j1 = wrap_repeat(y0 + 1.f, H);
  float4 t00 = fetch(i0, j0), t10 = fetch(i1, j0), t01 = fetch(i0, j1), t11 = fetch(i1, j1);
  float4 r;
  r.x = mixf(mixf(t00.x, t10.x, fx), mixf(t01.x, t11.x, fx), fy);
  r.y = mixf(mixf(t00.y, t10.y, fx), mixf(t01.y, t11.y, fx), fy);
  r.z = mixf(mixf(t00.z, t10.z, fx), mixf(t01.z, t11.z, fx), fy);
  r.w = mixf(mixf(t00.w, t10.w, fx), mixf(t01.w, t11.w, fx), fy);
  return r;
}

// Mirror addressing of the denoisers' padded block grid
// (shaders/bmfrGeneral.comp:93-101).
PBRT_HD int mirror1(int x, int s) {
  if (x < 0) return (x < 0 ? -x : x) - 1;
  if (x >= s) return 2 * s - x - 1;
  return x;
}

// Spherical normal decode (shaders/bmfrPre.comp:27-30).
PBRT_D float3 decode_normal(float th, float ph) {
  float st = sinf(th);
  return f3(cosf(ph) * st, sinf(ph) * st, cosf(th));
}

}  // namespace pbrt
