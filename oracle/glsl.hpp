// Oracle (test infrastructure only): GLSL value semantics on the CPU.
//
// This header is part of the CPU oracle that the tests, smoke() and the
// bench's cpu_baseline leg use as the checker for the CUDA path. Nothing in
// the product links it.
//
// It gives the oracle GLSL 4.60 semantics for the handful of built-ins the
// VulkanPBRT shaders use: column-major mat4 (m[c][r]), mix(x,y,a)=x*(1-a)+y*a,
// clamp(x,lo,hi)=min(max(x,lo),hi) with IEEE minNum/maxNum (NaN-dropping,
// as fminf/fmaxf), reflect, smoothstep, sign, normalize = v / length(v).
// The scalar type T is float for the "as-shader" FP32 mode and double for the
// FP64 convergence oracle. Build with -ffp-contract=off so a*b+c is never fused.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

namespace orc {

template <class T> struct V2 { T x, y; };
template <class T> struct V3 {
  T x, y, z;
  T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template <class T> struct V4 {
  T x, y, z, w;
  T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
  T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
  V3<T> xyz() const { return {x, y, z}; }
};

template <class T> inline V2<T> v2(T x, T y) { return {x, y}; }
template <class T> inline V3<T> v3(T x, T y, T z) { return {x, y, z}; }
template <class T> inline V3<T> v3(T s) { return {s, s, s}; }
template <class T> inline V4<T> v4(T x, T y, T z, T w) { return {x, y, z, w}; }
template <class T> inline V4<T> v4(V3<T> a, T w) { return {a.x, a.y, a.z, w}; }

#define ORC_BIN(OP)                                                                        \
  template <class T> inline V3<T> operator OP(V3<T> a, V3<T> b) { return {a.x OP b.x, a.y OP b.y, a.z OP b.z}; } \
  template <class T> inline V3<T> operator OP(V3<T> a, T b) { return {a.x OP b, a.y OP b, a.z OP b}; }            \
  template <class T> inline V3<T> operator OP(T a, V3<T> b) { return {a OP b.x, a OP b.y, a OP b.z}; }            \
  template <class T> inline V2<T> operator OP(V2<T> a, V2<T> b) { return {a.x OP b.x, a.y OP b.y}; }              \
  template <class T> inline V2<T> operator OP(V2<T> a, T b) { return {a.x OP b, a.y OP b}; }                      \
  template <class T> inline V4<T> operator OP(V4<T> a, V4<T> b) { return {a.x OP b.x, a.y OP b.y, a.z OP b.z, a.w OP b.w}; } \
  template <class T> inline V4<T> operator OP(V4<T> a, T b) { return {a.x OP b, a.y OP b, a.z OP b, a.w OP b}; }
ORC_BIN(+)
ORC_BIN(-)
ORC_BIN(*)
ORC_BIN(/)
#undef ORC_BIN
template <class T> inline V3<T> operator-(V3<T> a) { return {-a.x, -a.y, -a.z}; }

template <class T> inline T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> inline T dot(V4<T> a, V4<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
template <class T> inline T length(V3<T> a) { return std::sqrt(dot(a, a)); }
template <class T> inline T distance(V3<T> a, V3<T> b) { return length(a - b); }
template <class T> inline V3<T> normalize(V3<T> a) { return a / length(a); }
template <class T> inline V3<T> cross(V3<T> a, V3<T> b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// IEEE minNum / maxNum: a NaN operand is dropped (GPU min/max behaviour).
template <class T> inline T gmin(T a, T b) { return std::fmin(a, b); }
template <class T> inline T gmax(T a, T b) { return std::fmax(a, b); }
template <class T> inline T clampf(T x, T lo, T hi) { return gmin(gmax(x, lo), hi); }
template <class T> inline V3<T> gmin(V3<T> a, V3<T> b) { return {gmin(a.x, b.x), gmin(a.y, b.y), gmin(a.z, b.z)}; }
template <class T> inline V3<T> gmax(V3<T> a, V3<T> b) { return {gmax(a.x, b.x), gmax(a.y, b.y), gmax(a.z, b.z)}; }
template <class T> inline V3<T> clamp3(V3<T> x, T lo, T hi) {
  return {clampf(x.x, lo, hi), clampf(x.y, lo, hi), clampf(x.z, lo, hi)};
}
template <class T> inline T mix(T x, T y, T a) { return x * (T(1) - a) + y * a; }
template <class T> inline V3<T> mix(V3<T> x, V3<T> y, T a) { return x * (T(1) - a) + y * a; }
template <class T> inline V3<T> mix(V3<T> x, V3<T> y, V3<T> a) { return x * (v3<T>(T(1)) - a) + y * a; }
template <class T> inline V3<T> reflect(V3<T> i, V3<T> n) { return i - T(2) * dot(n, i) * n; }
template <class T> inline T smoothstep(T e0, T e1, T x) {
  T t = clampf((x - e0) / (e1 - e0), T(0), T(1));
  return t * t * (T(3) - T(2) * t);
}
template <class T> inline T signf(T x) { return x > T(0) ? T(1) : (x < T(0) ? T(-1) : T(0)); }
template <class T> inline bool eq(V3<T> a, V3<T> b) { return a.x == b.x && a.y == b.y && a.z == b.z; }

// Column-major 4x4: m[c] is column c, m[c][r] row r, as GLSL mat4.
template <class T> struct M4 {
  V4<T> c[4];
  V4<T> operator*(V4<T> v) const {
    return c[0] * v.x + c[1] * v.y + c[2] * v.z + c[3] * v.w;
  }
  M4 operator*(const M4& b) const {
    M4 r;
    for (int i = 0; i < 4; ++i) r.c[i] = (*this) * b.c[i];
    return r;
  }
};
template <class T> inline M4<T> load_m4(const float* p) {
  M4<T> m;
  for (int i = 0; i < 4; ++i) m.c[i] = {T(p[4 * i]), T(p[4 * i + 1]), T(p[4 * i + 2]), T(p[4 * i + 3])};
  return m;
}
// 3x3 column-major (TBN basis); b * v = c0*v.x + c1*v.y + c2*v.z.
template <class T> struct M3 {
  V3<T> c[3];
  V3<T> operator*(V3<T> v) const { return c[0] * v.x + c[1] * v.y + c[2] * v.z; }
};

// General 4x4 inverse by cofactor expansion, evaluated in double and rounded
// to T (the host-side inverse the path uses where a shader calls inverse()).
template <class T> inline M4<T> inverse(const M4<T>& mi) {
  double m[16], inv[16];
  for (int c = 0; c < 4; ++c)
    for (int r = 0; r < 4; ++r) m[c * 4 + r] = (double)mi.c[c][r];
  inv[0] = m[5] * m[10] * m[15] - m[5] * m[11] * m[14] - m[9] * m[6] * m[15] + m[9] * m[7] * m[14] + m[13] * m[6] * m[11] - m[13] * m[7] * m[10];
  inv[4] = -m[4] * m[10] * m[15] + m[4] * m[11] * m[14] + m[8] * m[6] * m[15] - m[8] * m[7] * m[14] - m[12] * m[6] * m[11] + m[12] * m[7] * m[10];
  inv[8] = m[4] * m[9] * m[15] - m[4] * m[11] * m[13] - m[8] * m[5] * m[15] + m[8] * m[7] * m[13] + m[12] * m[5] * m[11] - m[12] * m[7] * m[9];
  inv[12] = -m[4] * m[9] * m[14] + m[4] * m[10] * m[13] + m[8] * m[5] * m[14] - m[8] * m[6] * m[13] - m[12] * m[5] * m[10] + m[12] * m[6] * m[9];
  inv[1] = -m[1] * m[10] * m[15] + m[1] * m[11] * m[14] + m[9] * m[2] * m[15] - m[9] * m[3] * m[14] - m[13] * m[2] * m[11] + m[13] * m[3] * m[10];
  inv[5] = m[0] * m[10] * m[15] - m[0] * m[11] * m[14] - m[8] * m[2] * m[15] + m[8] * m[3] * m[14] + m[12] * m[2] * m[11] - m[12] * m[3] * m[10];
  inv[9] = -m[0] * m[9] * m[15] + m[0] * m[11] * m[13] + m[8] * m[1] * m[15] - m[8] * m[3] * m[13] - m[12] * m[1] * m[11] + m[12] * m[3] * m[9];
  inv[13] = m[0] * m[9] * m[14] - m[0] * m[10] * m[13] - m[8] * m[1] * m[14] + m[8] * m[2] * m[13] + m[12] * m[1] * m[10] - m[12] * m[2] * m[9];
  inv[2] = m[1] * m[6] * m[15] - m[1] * m[7] * m[14] - m[5] * m[2] * m[15] + m[5] * m[3] * m[14] + m[13] * m[2] * m[7] - m[13] * m[3] * m[6];
  inv[6] = -m[0] * m[6] * m[15] + m[0] * m[7] * m[14] + m[4] * m[2] * m[15] - m[4] * m[3] * m[14] - m[12] * m[2] * m[7] + m[12] * m[3] * m[6];
  inv[10] = m[0] * m[5] * m[15] - m[0] * m[7] * m[13] - m[4] * m[1] * m[15] + m[4] * m[3] * m[13] + m[12] * m[1] * m[7] - m[12] * m[3] * m[5];
  inv[14] = -m[0] * m[5] * m[14] + m[0] * m[6] * m[13] + m[4] * m[1] * m[14] - m[4] * m[2] * m[13] - m[12] * m[1] * m[6] + m[12] * m[2] * m[5];
  inv[3] = -m[1] * m[6] * m[11] + m[1] * m[7] * m[10] + m[5] * m[2] * m[11] - m[5] * m[3] * m[10] - m[9] * m[2] * m[7] + m[9] * m[3] * m[6];
  inv[7] = m[0] * m[6] * m[11] - m[0] * m[7] * m[10] - m[4] * m[2] * m[11] + m[4] * m[3] * m[10] + m[8] * m[2] * m[7] - m[8] * m[3] * m[6];
  inv[11] = -m[0] * m[5] * m[11] + m[0] * m[7] * m[9] + m[4] * m[1] * m[11] - m[4] * m[3] * m[9] - m[8] * m[1] * m[7] + m[8] * m[3] * m[5];
  inv[15] = m[0] * m[5] * m[10] - m[0] * m[6] * m[9] - m[4] * m[1] * m[10] + m[4] * m[2] * m[9] + m[8] * m[1] * m[6] - m[8] * m[2] * m[5];
  double det = m[0] * inv[0] + m[1] * inv[4] + m[2] * inv[8] + m[3] * inv[12];
  M4<T> r;
  for (int c = 0; c < 4; ++c)
    for (int rr = 0; rr < 4; ++rr) r.c[c][rr] = (T)(inv[c * 4 + rr] / det);
  return r;
}

// ---------------------------------------------------------------------------
// Storage-format conversions (Vulkan image formats the reference uses).
// float -> binary16 with round-to-nearest-even (R16F / RGBA16F stores).
inline uint16_t f2h(float f) {
  uint32_t x;
  std::memcpy(&x, &f, 4);
  uint32_t sign = (x >> 16) & 0x8000u;
  uint32_t ax = x & 0x7fffffffu;
  if (ax >= 0x7f800000u) return (uint16_t)(sign | 0x7c00u | (ax > 0x7f800000u ? 0x200u : 0u));
  if (ax >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u);  // rounds to +-inf
  if (ax < 0x38800000u) {                                      // half subnormal or zero
    uint32_t e = ax >> 23;
    if (e < 102) return (uint16_t)sign;  // below half of the smallest subnormal
    uint32_t m = (ax & 0x7fffffu) | 0x800000u;
    uint32_t shift = 126 - e;  // value in units of 2^-24 is m >> shift
    uint32_t q = m >> shift;
    uint32_t rem = m & ((1u << shift) - 1u);
    uint32_t half = 1u << (shift - 1);
    if (rem > half || (rem == half && (q & 1u))) q++;
    return (uint16_t)(sign | q);
  }
  uint32_t e = (ax >> 23) - 112;  // rebias 127 -> 15
  uint32_t m = ax & 0x7fffffu;
  uint32_t h = (e << 10) | (m >> 13);
  uint32_t rem = m & 0x1fffu;
  if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h++;
  return (uint16_t)(sign | h);
}
inline float h2f(uint16_t h) {
  uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
  uint32_t e = (h >> 10) & 0x1fu, m = h & 0x3ffu, x;
  if (e == 0) {
    if (m == 0) {
      x = sign;
    } else {  // subnormal: m * 2^-24
      float v = (float)m * 5.9604644775390625e-8f;
      std::memcpy(&x, &v, 4);
      x |= sign;
    }
  } else if (e == 31) {
    x = sign | 0x7f800000u | (m << 13);
  } else {
    x = sign | ((e + 112) << 23) | (m << 13);
  }
  float f;
  std::memcpy(&f, &x, 4);
  return f;
}
inline float q16(float f) { return h2f(f2h(f)); }
// float -> UNORM8 (R8 / RGBA8 stores): clamp to [0,1], round to nearest.
inline uint8_t f2u8(float f) {
  float c = clampf(f, 0.f, 1.f);
  return (uint8_t)std::floor(c * 255.f + 0.5f);
}
inline float u82f(uint8_t u) { return (float)u / 255.f; }

}  // namespace orc
