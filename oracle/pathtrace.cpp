// Oracle (test infrastructure only): CPU restatement of VulkanPBRT's per-frame
// path tracer -- ptRaygen.rgen with ptClosesthit / ptAlphaHit / ptMiss /
// shadow.rmiss, lighting.glsl, sampling.glsl, brdf.glsl, geometry.glsl,
// color.glsl, random.glsl, camera.glsl -- in FP32 "as shader" (T = float,
// no FP contraction) or FP64 (T = double) arithmetic.
//
// Used only by tests/, smoke() and the bench's CPU legs as the checker.
//
// Parity pin: the reference's shaders cannot be compiled or run here and its
// traversal is the closed Vulkan driver's; this restatement is pinned by the
// integer known-answer vectors under tests/golden and by citation. The
// closest hit is defined geometrically: watertight ray/triangle test
// (Woop, Benthin & Wald 2013), smallest t, ties to the lowest instance-major
// triangle index. Where the shaders leave behaviour open the oracle makes the
// same choices as the CUDA path: a path ends when indirectLighting() returns
// early or misses; min/max/clamp drop NaN operands (IEEE minNum/maxNum);
// texture filtering is FP32 bilinear with REPEAT addressing at level 0.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "glsl.hpp"

using namespace orc;

extern "C" {
// Scene arrays, in the layout the CUDA library uploads (packed u16 pairs or
// u32 words for indices; column-major object matrices).
struct OrcScene {
  uint32_t mesh_count;
  const uint32_t* mesh_vbase;
  const uint32_t* mesh_ibase;
  const int32_t* mesh_tex;  // 5 per mesh
  const float* pos;
  const float* nor;
  const float* uv;
  const uint32_t* idx;
  uint32_t instance_count;
  const float* inst_mat;  // 16 per instance
  const int32_t* inst_mesh;
  const uint32_t* inst_stride;
  const uint8_t* inst_opaque;
  const uint32_t* inst_tri_count;
  const float* materials;  // 24 per mesh
  uint32_t light_count;
  const float* lights;  // 32 per light
  uint32_t texture_count;
  const uint64_t* tex_offset;  // in texels
  const uint32_t* tex_w;
  const uint32_t* tex_h;
  const uint8_t* texels;  // RGBA8
};
}

namespace {

template <class F> void parallel_rows(int n, int threads, F f) {
  if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
  threads = std::min(threads, std::max(1, n));
  std::atomic<int> next(0);
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; ++t)
    pool.emplace_back([&]() {
      for (int i = next++; i < n; i = next++) f(i);
    });
  for (auto& th : pool) th.join();
}

// T-typed libm
inline float Pow(float a, float b) { return std::pow(a, b); }
inline double Pow(double a, double b) { return std::pow(a, b); }

// ---------------------------------------------------------------------------
// random.glsl:16-96
struct RandomEngine {
  uint32_t x, y, z, w;
};
inline uint32_t taus(uint32_t z, int s1, int s2, int s3, uint32_t m) {
  uint32_t b = (((z << s1) ^ z) >> s2);
  return (((z & m) << s3) ^ b);
}
inline uint32_t wang(uint32_t s) {
  s = (s ^ 61u) ^ (s >> 16);
  s *= 9u;
  s = s ^ (s >> 4);
  s *= 0x27d4eb2du;
  s = s ^ (s >> 15);
  return s;
}
template <class T> inline T random_float(RandomEngine& e) {
  e.x = taus(e.x, 13, 19, 12, 4294967294u);
  e.y = taus(e.y, 2, 25, 4, 4294967288u);
  e.z = taus(e.z, 3, 11, 17, 4294967280u);
  e.w = 1664525u * e.w + 1013904223u;
  uint32_t u = e.x ^ e.y ^ e.z ^ e.w;
  return (T)2.3283064365387e-10f * (T)u;  // float(u) for T=float (round to nearest), exact for double
}
inline RandomEngine re_init(uint32_t x, uint32_t y, uint32_t frame) {
  return RandomEngine{wang(x), wang(y), wang(frame), wang((x + y) * frame)};
}

// ---------------------------------------------------------------------------
template <class T> struct World {
  const OrcScene* sc;
  std::vector<T> tri;  // 9 per triangle, world space
  std::vector<uint32_t> tri_inst, tri_prim;
  // simple binary BVH (median split), double bounds
  struct BNode {
    double lo[3], hi[3];
    int left, right;  // -1 leaf
    uint32_t begin, count;
  };
  std::vector<BNode> nodes;
  std::vector<uint32_t> order;

  void build(const OrcScene* s) {
    sc = s;
    size_t total = 0;
    for (uint32_t i = 0; i < s->instance_count; ++i) total += s->inst_tri_count[i];
    tri.resize(9 * total);
    tri_inst.resize(total);
    tri_prim.resize(total);
    size_t t = 0;
    for (uint32_t i = 0; i < s->instance_count; ++i) {
      const float* M = s->inst_mat + 16 * i;
      const int m = s->inst_mesh[i];
      for (uint32_t p = 0; p < s->inst_tri_count[i]; ++p, ++t) {
        uint32_t ix[3];
        unpack_index(m, p, s->inst_stride[i], ix);
        for (int k = 0; k < 3; ++k) {
          const float* v = s->pos + 3 * (size_t)(s->mesh_vbase[m] + ix[k]);
          for (int a = 0; a < 3; ++a) {
            // (objectMat * vec4(v, 1)).xyz, column order
            T acc = (T)M[0 * 4 + a] * (T)v[0];
            acc = acc + (T)M[1 * 4 + a] * (T)v[1];
            acc = acc + (T)M[2 * 4 + a] * (T)v[2];
            acc = acc + (T)M[3 * 4 + a] * (T)1;
            tri[9 * t + 3 * k + a] = acc;
          }
        }
        tri_inst[t] = i;
        tri_prim[t] = p;
      }
    }
    order.resize(total);
    for (size_t i = 0; i < total; ++i) order[i] = (uint32_t)i;
    nodes.clear();
    nodes.reserve(2 * total / 2 + 8);
    build_node(0, (uint32_t)total);
  }

  int build_node(uint32_t begin, uint32_t count) {
    BNode n;
    for (int a = 0; a < 3; ++a) {
      n.lo[a] = INFINITY;
      n.hi[a] = -INFINITY;
    }
    double clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t i = begin; i < begin + count; ++i) {
      const T* v = &tri[9 * (size_t)order[i]];
      for (int a = 0; a < 3; ++a) {
        double mn = std::min({(double)v[a], (double)v[3 + a], (double)v[6 + a]});
        double mx = std::max({(double)v[a], (double)v[3 + a], (double)v[6 + a]});
        n.lo[a] = std::min(n.lo[a], mn);
        n.hi[a] = std::max(n.hi[a], mx);
        double c = 0.5 * (mn + mx);
        clo[a] = std::min(clo[a], c);
        chi[a] = std::max(chi[a], c);
      }
    }
    n.begin = begin;
    n.count = count;
    n.left = n.right = -1;
    int id = (int)nodes.size();
    nodes.push_back(n);
    if (count <= 4) return id;
    int ax = 0;
    for (int a = 1; a < 3; ++a)
      if (chi[a] - clo[a] > chi[ax] - clo[ax]) ax = a;
    uint32_t mid = begin + count / 2;
    auto cen = [&](uint32_t ti) {
      const T* v = &tri[9 * (size_t)ti];
      double mn = std::min({(double)v[ax], (double)v[3 + ax], (double)v[6 + ax]});
      double mx = std::max({(double)v[ax], (double)v[3 + ax], (double)v[6 + ax]});
      return 0.5 * (mn + mx);
    };
    std::nth_element(order.begin() + begin, order.begin() + mid, order.begin() + begin + count,
                     [&](uint32_t a, uint32_t b) { return cen(a) < cen(b); });
    int l = build_node(begin, mid - begin);
    int r = build_node(mid, begin + count - mid);
    nodes[id].left = l;
    nodes[id].right = r;
    return id;
  }

  void unpack_index(int m, uint32_t prim, uint32_t stride, uint32_t ix[3]) const {
    // geometry.glsl:4-26
    const uint32_t* ind = sc->idx + sc->mesh_ibase[m];
    if (stride == 4) {
      ix[0] = ind[3 * prim];
      ix[1] = ind[3 * prim + 1];
      ix[2] = ind[3 * prim + 2];
      return;
    }
    int full = 3 * (int)prim;
    uint32_t p = (uint32_t)((float)full * .5f);
    if (full & 1) {
      ix[0] = ind[p] >> 16;
      uint32_t t = ind[p + 1];
      ix[2] = t >> 16;
      ix[1] = t & 0xffffu;
    } else {
      uint32_t t = ind[p];
      ix[1] = t >> 16;
      ix[0] = t & 0xffffu;
      ix[2] = ind[p + 1] & 0xffffu;
    }
  }
};

// Watertight test, the same operation order as the CUDA path.
template <class T> struct RayT {
  V3<T> o, d;
  int kx, ky, kz;
  T Sx, Sy, Sz;
};
template <class T> inline T compo(const V3<T>& v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }
template <class T> RayT<T> make_ray(V3<T> o, V3<T> d) {
  RayT<T> r;
  r.o = o;
  r.d = d;
  T ax = std::fabs(d.x), ay = std::fabs(d.y), az = std::fabs(d.z);
  r.kz = (ax > ay && ax > az) ? 0 : (ay > az ? 1 : 2);
  r.kx = (r.kz + 1) % 3;
  r.ky = (r.kx + 1) % 3;
  T dz = compo(d, r.kz);
  if (dz < 0) std::swap(r.kx, r.ky);
  r.Sx = compo(d, r.kx) / dz;
  r.Sy = compo(d, r.ky) / dz;
  r.Sz = (T)1 / dz;
  return r;
}
template <class T> bool tri_test(const RayT<T>& r, const T* v, T tmin, T& t, T& u, T& w2) {
  V3<T> A{v[0] - r.o.x, v[1] - r.o.y, v[2] - r.o.z};
  V3<T> B{v[3] - r.o.x, v[4] - r.o.y, v[5] - r.o.z};
  V3<T> C{v[6] - r.o.x, v[7] - r.o.y, v[8] - r.o.z};
  T Akz = compo(A, r.kz), Bkz = compo(B, r.kz), Ckz = compo(C, r.kz);
  T Ax = compo(A, r.kx) - r.Sx * Akz, Ay = compo(A, r.ky) - r.Sy * Akz;
  T Bx = compo(B, r.kx) - r.Sx * Bkz, By = compo(B, r.ky) - r.Sy * Bkz;
  T Cx = compo(C, r.kx) - r.Sx * Ckz, Cy = compo(C, r.ky) - r.Sy * Ckz;
  T U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
  if (U == 0 || V == 0 || W == 0) {
    U = (T)((double)Cx * (double)By - (double)Cy * (double)Bx);
    V = (T)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
    W = (T)((double)Bx * (double)Ay - (double)By * (double)Ax);
  }
  if ((U < 0 || V < 0 || W < 0) && (U > 0 || V > 0 || W > 0)) return false;
  T det = (U + V) + W;
  if (det == 0) return false;
  T Az = r.Sz * Akz, Bz = r.Sz * Bkz, Cz = r.Sz * Ckz;
  T Tt = (U * Az + V * Bz) + W * Cz;
  T rcp = (T)1 / det;
  t = Tt * rcp;
  if (!(t > tmin)) return false;
  u = V * rcp;
  w2 = W * rcp;
  return true;
}

template <class T> struct Tracer {
  World<T>& w;
  const OrcScene* sc;
  int light_mode, min_depth, max_depth;
  float light_strength_sum;

  // ---- textures (FP32 bilinear, REPEAT, level 0) ----
  void tex(int t, float u, float v, float out[4]) const {
    const uint32_t W = sc->tex_w[t], H = sc->tex_h[t];
    const uint8_t* base = sc->texels + 4 * sc->tex_offset[t];
    float x = u * (float)W - 0.5f, y = v * (float)H - 0.5f;
    float x0 = std::floor(x), y0 = std::floor(y);
    float fx = x - x0, fy = y - y0;
    if (!std::isfinite(fx)) fx = 0.f;
    if (!std::isfinite(fy)) fy = 0.f;
    auto wrap = [](float c, int n) {
      if (!std::isfinite(c)) return 0;
      float m = c - (float)n * std::floor(c / (float)n);
      int i = (int)m;
      return std::min(std::max(i, 0), n - 1);
    };
    int i0 = wrap(x0, (int)W), i1 = wrap(x0 + 1.f, (int)W), j0 = wrap(y0, (int)H), j1 = wrap(y0 + 1.f, (int)H);
    for (int c = 0; c < 4; ++c) {
      float t00 = u82f(base[4 * ((size_t)j0 * W + i0) + c]), t10 = u82f(base[4 * ((size_t)j0 * W + i1) + c]);
      float t01 = u82f(base[4 * ((size_t)j1 * W + i0) + c]), t11 = u82f(base[4 * ((size_t)j1 * W + i1) + c]);
      out[c] = mix(mix(t00, t10, fx), mix(t01, t11, fx), fy);
    }
  }
  bool tex1x1(int t) const { return sc->tex_w[t] == 1 && sc->tex_h[t] == 1; }

  bool alpha_ok(uint32_t inst, uint32_t prim, T bu, T bv) const {
    if (sc->inst_opaque[inst]) return true;
    const int m = sc->inst_mesh[inst];
    uint32_t ix[3];
    w.unpack_index(m, prim, sc->inst_stride[inst], ix);
    const float* uv = sc->uv;
    const uint32_t vb = sc->mesh_vbase[m];
    T b0 = (T)1 - bu - bv;
    T u = (T)uv[2 * (vb + ix[0])] * b0 + (T)uv[2 * (vb + ix[1])] * bu + (T)uv[2 * (vb + ix[2])] * bv;
    T v = (T)uv[2 * (vb + ix[0]) + 1] * b0 + (T)uv[2 * (vb + ix[1]) + 1] * bu + (T)uv[2 * (vb + ix[2]) + 1] * bv;
    float d[4];
    tex(sc->mesh_tex[5 * m + 0], (float)u, (float)v, d);
    return !(d[3] < .01f);
  }

  // closest (any = false) or first (any = true) hit; returns flat triangle index or -1
  long trace(V3<T> o, V3<T> d, T tmin, T tmax, bool any, T& th, T& tu, T& tv, uint64_t& rays) const {
    rays++;
    RayT<T> r = make_ray(o, d);
    long best = -1;
    T bt = tmax, bu = 0, bv = 0;
    int stack[128];
    int sp = 0;
    stack[sp++] = 0;
    double od[3] = {(double)o.x, (double)o.y, (double)o.z}, dd[3] = {(double)d.x, (double)d.y, (double)d.z};
    while (sp) {
      const auto& n = w.nodes[stack[--sp]];
      // slab test in double with a margin (conservative; decisions come from the triangle test)
      double t0 = -INFINITY, t1 = INFINITY;
      for (int a = 0; a < 3; ++a) {
        if (dd[a] == 0.0) {
          if (od[a] < n.lo[a] || od[a] > n.hi[a]) {
            t0 = INFINITY;
            break;
          }
          continue;
        }
        double inv = 1.0 / dd[a];
        double ta = (n.lo[a] - od[a]) * inv, tb = (n.hi[a] - od[a]) * inv;
        if (ta > tb) std::swap(ta, tb);
        t0 = std::max(t0, ta);
        t1 = std::min(t1, tb);
      }
      double pad = 1e-6 * std::max(1.0, std::fabs(t1));
      if (!(t0 <= t1 + pad) || t1 + pad < (double)tmin || t0 - pad > (double)bt) continue;
      if (n.left < 0) {
        for (uint32_t i = n.begin; i < n.begin + n.count; ++i) {
          uint32_t ti = w.order[i];
          T t, u, v;
          if (!tri_test(r, &w.tri[9 * (size_t)ti], tmin, t, u, v)) continue;
          if (!(t < bt || (t == bt && (long)ti < best))) continue;
          if (!alpha_ok(w.tri_inst[ti], w.tri_prim[ti], u, v)) continue;
          best = (long)ti;
          bt = t;
          bu = u;
          bv = v;
          if (any) {
            th = bt;
            return best;
          }
        }
      } else {
        stack[sp++] = n.left;
        stack[sp++] = n.right;
      }
    }
    th = bt;
    tu = bu;
    tv = bv;
    return best;
  }

  struct SI {
    T pr, metal, ar;
    int illum;
    V3<T> r0, r90, diffuse, specular, emissive, transmissive, normal, b0, b1, b2;
    T ior;
  };

  static V3<T> srgb2lin(V3<T> c) { return V3<T>{Pow(c.x, (T)2.2f), Pow(c.y, (T)2.2f), Pow(c.z, (T)2.2f)}; }
  static T luminance(V3<T> c) { return dot(c, V3<T>{(T)0.2126f, (T)0.7152f, (T)0.0722f}); }
  static T convert_metallic(V3<T> d, V3<T> s, T maxs) {  // color.glsl:32-47
    T pd = std::sqrt((T)0.299f * d.x * d.x + (T)0.587f * d.y * d.y + (T)0.114f * d.z * d.z);
    T ps = std::sqrt((T)0.299f * s.x * s.x + (T)0.587f * s.y * s.y + (T)0.114f * s.z * s.z);
    const T mr = (T)0.04f;
    if (ps < mr) return 0;
    T a = mr;
    T b = pd * ((T)1 - maxs) / ((T)1 - mr) + ps - (T)2 * mr;
    T c = mr - ps;
    T D = gmax(b * b - (T)4 * a * c, (T)0);
    return clampf((-b + std::sqrt(D)) / ((T)2 * a), (T)0, (T)1);
  }
  static V3<T> get_tangent(V3<T> A, V3<T> B, V3<T> C, V2<T> Au, V2<T> Bu, V2<T> Cu) {  // geometry.glsl:59-69
    T bc = Bu.y - Cu.y;
    if (bc == 0) return (B - C) / (Bu.x - Cu.x);
    T q = (Au.y - Cu.y) / bc;
    V3<T> D = C + (B - C) * q;
    V2<T> Du{Cu.x + (Bu.x - Cu.x) * q, Cu.y + (Bu.y - Cu.y) * q};
    return (D - A) / (Du.x - Au.x);
  }
  static V3<T> project(V3<T> a, V3<T> b) { return dot(a, b) / dot(b, b) * b; }

  // ptClosesthit.rchit:18-92
  V3<T> closest_hit(V3<T> ray_dir, uint32_t inst, uint32_t prim, T bu, T bv, SI& si, uint32_t& cat) const {
    const T eps = (T)1e-6f;
    const int m = sc->inst_mesh[inst];
    uint32_t ix[3];
    w.unpack_index(m, prim, sc->inst_stride[inst], ix);
    const uint32_t vb = sc->mesh_vbase[m];
    V3<T> p[3], n[3];
    V2<T> t[3];
    for (int k = 0; k < 3; ++k) {
      size_t vi = vb + ix[k];
      p[k] = V3<T>{(T)sc->pos[3 * vi], (T)sc->pos[3 * vi + 1], (T)sc->pos[3 * vi + 2]};
      n[k] = V3<T>{(T)sc->nor[3 * vi], (T)sc->nor[3 * vi + 1], (T)sc->nor[3 * vi + 2]};
      t[k] = V2<T>{(T)sc->uv[2 * vi], (T)sc->uv[2 * vi + 1]};
    }
    const T b0 = (T)1 - bu - bv, b1 = bu, b2 = bv;
    V2<T> tc{t[0].x * b0 + t[1].x * b1 + t[2].x * b2, t[0].y * b0 + t[1].y * b1 + t[2].y * b2};
    const int* mt = sc->mesh_tex + 5 * m;
    float dm[4];
    tex(mt[0], (float)tc.x, (float)tc.y, dm);
    V3<T> diffuse = srgb2lin(V3<T>{(T)dm[0], (T)dm[1], (T)dm[2]});
    diffuse = diffuse * (T)dm[3];
    V3<T> position = p[0] * b0 + p[1] * b1 + p[2] * b2;
    const float* M = sc->inst_mat + 16 * inst;
    V3<T> wp;
    for (int a = 0; a < 3; ++a) {
      T acc = (T)M[0 * 4 + a] * position.x;
      acc = acc + (T)M[1 * 4 + a] * position.y;
      acc = acc + (T)M[2 * 4 + a] * position.z;
      acc = acc + (T)M[3 * 4 + a] * (T)1;
      wp[a] = acc;
    }
    position = wp;
    V3<T> normal = normalize(n[0] * b0 + n[1] * b1 + n[2] * b2);
    if (std::isinf(normal.x) || std::isnan(normal.x)) normal = V3<T>{0, 1, 0};
    // transpose(inverse(objectMat)), evaluated in double, upper 3x3 columns
    M4<double> Md;
    for (int c = 0; c < 4; ++c) Md.c[c] = V4<double>{M[4 * c], M[4 * c + 1], M[4 * c + 2], M[4 * c + 3]};
    M4<double> inv = orc::inverse(Md);
    V3<T> nc[3];
    for (int c = 0; c < 3; ++c) {
      nc[c] = V3<T>{(T)(float)inv.c[0][c], (T)(float)inv.c[1][c], (T)(float)inv.c[2][c]};
      if (sizeof(T) == 8) nc[c] = V3<T>{(T)inv.c[0][c], (T)inv.c[1][c], (T)inv.c[2][c]};
    }
    normal = normalize(nc[0] * normal.x + nc[1] * normal.y + nc[2] * normal.z);
    if (t[0].x == t[1].x && t[0].y == t[1].y) t[1].x += eps;
    if (t[0].x == t[2].x && t[0].y == t[2].y) t[2].y += eps;
    if (t[1].x == t[2].x && t[1].y == t[2].y) {
      t[2].x += eps;
      t[2].y += eps;
    }
    V3<T> tg = get_tangent(p[0], p[1], p[2], t[0], t[1], t[2]);
    V3<T> Tn = nc[0] * tg.x + nc[1] * tg.y + nc[2] * tg.z;
    V3<T> bt = get_tangent(p[0], p[2], p[1], V2<T>{t[0].y, t[0].x}, V2<T>{t[2].y, t[2].x}, V2<T>{t[1].y, t[1].x});
    V3<T> Bn = nc[0] * bt.x + nc[1] * bt.y + nc[2] * bt.z;
    V3<T> tt = Tn - project(Tn, normal);
    V3<T> bb = Bn - project(Bn, tt) - project(Bn, normal);
    si.b0 = normalize(tt);
    si.b1 = normalize(bb);
    si.b2 = normal;
    if (!tex1x1(mt[2])) {
      float nm[4];
      tex(mt[2], (float)tc.x, (float)tc.y, nm);
      V3<T> tn{(T)nm[0] * (T)2 - (T)1, (T)nm[1] * (T)2 - (T)1, (T)nm[2] * (T)2 - (T)1};
      normal = normalize(si.b0 * tn.x + si.b1 * tn.y + si.b2 * tn.z);
    }
    const float* mat = sc->materials + 24 * m;
    diffuse = diffuse * V3<T>{(T)mat[4], (T)mat[5], (T)mat[6]};
    V3<T> spec;
    T pr;
    if (tex1x1(mt[4])) {
      spec = V3<T>{(T)mat[8], (T)mat[9], (T)mat[10]};
      pr = (T)mat[3];
    } else {
      float sm[4];
      tex(mt[4], (float)tc.x, (float)tc.y, sm);
      spec = srgb2lin(V3<T>{(T)sm[0], (T)sm[1], (T)sm[2]});
      pr = (T)sm[3];
    }
    const T mr = (T)0.04f;
    T maxs = gmax(gmax(spec.x, spec.y), spec.z);
    T metal = convert_metallic(diffuse, spec, maxs);
    V3<T> bcd = diffuse * (((T)1 - maxs) / ((T)1 - mr) / gmax((T)1 - metal, eps));
    V3<T> bcs = spec - (v3<T>(mr) * ((T)1 - metal) * ((T)1 / gmax(metal, eps)));
    V3<T> base = mix(bcd, bcs, metal * metal);
    V3<T> dcol = base * (v3<T>((T)1) - v3<T>((T)0.04f));
    dcol = dcol * ((T)1 - metal);
    V3<T> scol = mix(v3<T>((T)0.04f), base, metal);
    T refl = gmax(gmax(scol.x, scol.y), scol.z);
    T r90 = clampf(refl * (T)25, (T)0, (T)1);
    V3<T> v = normalize(-ray_dir);
    float em[4];
    tex(mt[3], (float)tc.x, (float)tc.y, em);
    V3<T> emissive = V3<T>{(T)mat[16], (T)mat[17], (T)mat[18]} * srgb2lin(V3<T>{(T)em[0], (T)em[1], (T)em[2]});
    if (dot(v, normal) < 0) emissive = v3<T>((T)0);
    si.pr = pr;
    si.metal = metal;
    si.ar = pr * pr;
    si.illum = (int)mat[15];
    si.r0 = scol;
    si.r90 = v3<T>((T)1) * r90;
    si.diffuse = dcol;
    si.specular = scol;
    si.emissive = emissive;
    si.transmissive = V3<T>{(T)mat[12], (T)mat[13], (T)mat[14]};
    si.normal = normal;
    si.ior = (T)mat[7];
    uint32_t c;
    std::memcpy(&c, &mat[20], 4);
    cat = c;
    return position;
  }

  // brdf.glsl
  static T spec_weight(const SI& s) {
    T wd = mix(luminance(s.diffuse), (T)0, s.metal);
    T ws = luminance(s.specular);
    return gmin((T)1, ws / (wd + wd));
  }
  static T pdf_brdf(const SI& s, V3<T> v, V3<T> l, V3<T> h) {
    (void)v;
    T pd = (T)0.31830988618f * dot(l, s.normal);
    T a2 = s.ar * s.ar;
    T nh = dot(h, s.normal);
    T q = nh * nh * (a2 - (T)1) + (T)1;
    T ps = a2 / ((T)3.14159265359f * (q * q));
    ps = ps * nh;
    return mix(pd, ps, spec_weight(s));
  }
  static V3<T> brdf(V3<T> v, V3<T> l, V3<T> h, const SI& s) {
    V3<T> n = s.normal;
    T NdotL = clampf(dot(n, l), (T)0.001f, (T)1);
    T NdotV = clampf(std::fabs(dot(n, v)), (T)0.001f, (T)1);
    T NdotH = clampf(dot(n, h), (T)0, (T)1);
    T VdotH = clampf(dot(v, h), (T)0, (T)1);
    V3<T> F = s.r0 + (s.r90 - s.r90 * s.r0) * std::exp2(((T)-5.55473f * VdotH - (T)6.98316f) * VdotH);
    T r = s.ar * s.ar;
    T aL = (T)2 * NdotL / (NdotL + std::sqrt(r + ((T)1 - r) * (NdotL * NdotL)));
    T aV = (T)2 * NdotV / (NdotV + std::sqrt(r + ((T)1 - r) * (NdotV * NdotV)));
    T G = aL * aV;
    T f = (NdotH * r - NdotH) * NdotH + (T)1;
    T D = r / ((T)3.14159265359f * f * f);
    T fd90 = (T)0.5f + (T)2 * s.pr * VdotH * VdotH;
    T dim = (T)1 - (T)0.1f;
    if (sizeof(T) == 4) dim = (T)(1.0f - 0.1f);
    T dis = (((T)1 + (fd90 - (T)1) * Pow((T)1 - NdotL, (T)5)) * ((T)1 + (fd90 - (T)1) * Pow((T)1 - NdotV, (T)5))) *
            (T)0.31830988618f * dim;
    V3<T> dc = (v3<T>((T)1) - F) * (s.diffuse * dis);
    V3<T> sp = F * G * D / ((T)4 * NdotL * NdotV);
    if (dot(n, l) <= 0) sp = v3<T>((T)0);
    return dc + sp;
  }
  // sampling.glsl:29-78 (engine by value)
  V3<T> sample_brdf(const SI& s, RandomEngine re, V3<T> v, V3<T>& l, T& pdf) const {
    const T PI = (T)3.14159265359f;
    T ux = random_float<T>(re), uy = random_float<T>(re), uz = random_float<T>(re);
    T sw = spec_weight(s);
    V3<T> b2 = s.b2;
    bool entering = dot(v, s.normal) >= 0;
    if (s.illum == 7 && !entering) b2 = -b2;
    V3<T> h;
    if (uz < sw) {
      T a2 = s.ar * s.ar;
      T phi = (T)2 * PI * ux;
      T ch = std::sqrt(((T)1 - uy) / ((T)1 + (a2 - (T)1) * uy));
      T sh = std::sqrt((T)1 - ch * ch);
      V3<T> hl{sh * std::cos(phi), sh * std::sin(phi), ch};
      h = s.b0 * hl.x + s.b1 * hl.y + b2 * hl.z;
      l = -(v - (T)2 * dot(h, v) * h);
    } else {
      T t = (T)2 * PI * uy;
      T sr = std::sqrt(ux);
      T dx = sr * std::cos(t), dy = sr * std::sin(t);
      V3<T> hs{dx, dy, std::sqrt(gmax((T)0, (T)1 - dx * dx - dy * dy))};
      l = s.b0 * hs.x + s.b1 * hs.y + b2 * hs.z;
      h = normalize(v + l);
    }
    pdf = pdf_brdf(s, v, l, h);
    V3<T> b = brdf(v, l, h, s);
    if (s.illum == 7) {
      T vh = dot(v, h);
      T fr = (T)1 + ((T)0 - (T)1) * Pow(clampf((T)1 - vh, (T)0, (T)1), (T)5);
      if (random_float<T>(re) < fr || !entering) {
        T t = !entering ? s.ior : (T)1 / s.ior;
        T ci = dot(b2, l);
        T st2 = t * t * ((T)1 - ci * ci);
        if (st2 <= (T)1) {
          l = l - (T)2 * ci * b2;
          T ct = std::sqrt((T)1 - st2);
          l = t * l + (t * ci - ct) * b2;
        }
        b = s.transmissive;
        pdf = 1;
      } else {
        pdf = 1;
        b = v3<T>((T)1);
      }
    }
    return b;
  }

  static V3<T> sky(V3<T> d) {  // lighting.glsl:233-240
    V3<T> up = srgb2lin(V3<T>{(T)0.3f, (T)0.5f, (T)0.92f});
    up = mix(v3<T>((T)1), up, gmax(d.z, (T)0));
    V3<T> lo = v3<T>((T)0.2f);
    T w = smoothstep((T)-0.02f, (T)0.02f, d.z);
    return mix(lo, up, w);
  }

  // sampleLight (lighting.glsl:19-227); traced = a shadow ray is cast
  V3<T> sample_light(V3<T> pos, V3<T> n, RandomEngine& re, V3<T>& l, T& pdf, bool& lit, uint64_t& rays) const {
    const T tmin = (T)0.001f;
    pdf = 0;
    l = v3<T>((T)0);
    lit = false;
    auto L = [&](uint32_t i) { return sc->lights + 32 * (size_t)i; };
    auto occluded = [&](V3<T> dir, T tmax) {
      T th, tu, tv;
      return trace(pos, dir, tmin, tmax, true, th, tu, tv, rays) >= 0;
    };
    if (light_mode == 0) {
      T ssum = 0, pstr = 0;
      V3<T> pls = v3<T>((T)0);
      T tmax = (T)1000;
      for (uint32_t i = 0; i < sc->light_count; ++i) {
        const float* lp = L(i);
        V3<T> ca{(T)lp[16], (T)lp[17], (T)lp[18]}, cd{(T)lp[20], (T)lp[21], (T)lp[22]}, cs{(T)lp[24], (T)lp[25], (T)lp[26]};
        V3<T> csum = ca + cd + cs;
        T csw = ((T)lp[19] + (T)lp[23]) + (T)lp[27];
        T power = ((csum.x + csum.y) + csum.z) + csw;
        T strength = 0;
        V3<T> ls = csum;
        T ctmax = (T)1000;
        V3<T> cl = v3<T>((T)0);
        int type = (int)lp[3];
        V3<T> v0{(T)lp[0], (T)lp[1], (T)lp[2]};
        T sx = (T)lp[28], sy = (T)lp[29], sz = (T)lp[30];
        if (type == 1) {
          T d = length(pos - v0);
          T att = (T)1 / (sx + sy * d + sz * d * d);
          V3<T> nd = -V3<T>{(T)lp[12], (T)lp[13], (T)lp[14]};
          strength = gmax(dot(n, nd), (T)0) * power * att;
          ls = ls * (dot(n, nd) * att);
          cl = normalize(nd);
        } else if (type == 2) {
          T d = length(pos - v0);
          T att = (T)1 / (sx + sy * d + sz * d * d);
          V3<T> to = normalize(v0 - pos);
          strength = gmax(dot(n, to), (T)0) * power * att;
          ls = ls * (dot(n, to) * att);
          cl = to;
        } else if (type == 5) {
          T ux = random_float<T>(re), uy = random_float<T>(re);
          T sq = std::sqrt(ux);
          T bx = (T)1 - sq, by = uy * sq;
          V3<T> p2{(T)lp[4], (T)lp[5], (T)lp[6]}, p3{(T)lp[8], (T)lp[9], (T)lp[10]};
          V3<T> lpt = v0 * ((T)1 - bx - by) + p2 * bx + p3 * by;
          V3<T> ld = lpt - pos;
          V3<T> ln = normalize(cross(p2 - v0, p3 - v0));
          T d = length(ld);
          ld = ld / d;
          T att = (T)1 / (sx + sy * d + sz * d * d);
          strength = gmax(dot(n, ld), (T)0) * gmax(dot(-ld, ln), (T)0) * power * att;
          ls = ls * (gmax(dot(n, ld), (T)0) * gmax(dot(-ld, ln), (T)0) * att);
          cl = ld;
          ctmax = d - tmin;
        }
        ssum = ssum + strength;
        if (random_float<T>(re) < strength / ssum) {
          pstr = strength;
          pls = ls;
          tmax = ctmax;
          l = cl;
        }
      }
      if (ssum < (T)1e-6f || pstr < (T)1e-6f) {
        pdf = 0;
        l = v3<T>((T)0);
        return v3<T>((T)0);
      }
      pdf = pstr / ssum;
      lit = !occluded(l, tmax);
      return pls;
    }
    T rnd = random_float<T>(re);
    int i;
    T lstr = 1;
    if (light_mode == 1) {
      T picked = rnd * (T)light_strength_sum;
      int begin = 0, end = (int)sc->light_count, mid = (begin + end) / 2, c = 0;
      while (end - begin > 1 && ++c < 100) {
        if (picked <= (T)L(mid)[31]) end = mid + 1;
        else begin = mid;
        mid = (begin + end) / 2;
      }
      lstr = (T)L(begin)[31];
      if (begin > 0) lstr = lstr - (T)L(begin - 1)[31];
      i = begin;
    } else {
      i = (int)(rnd * (T)sc->light_count) - (int)rnd;
    }
    const float* lp = L(i);
    V3<T> ls = V3<T>{(T)lp[16], (T)lp[17], (T)lp[18]} + V3<T>{(T)lp[20], (T)lp[21], (T)lp[22]} +
               V3<T>{(T)lp[24], (T)lp[25], (T)lp[26]};
    T tmax = (T)1000;
    int type = (int)lp[3];
    V3<T> v0{(T)lp[0], (T)lp[1], (T)lp[2]};
    T sx = (T)lp[28], sy = (T)lp[29], sz = (T)lp[30];
    if (type == 1) {
      T d = length(pos - v0);
      T att = (T)1 / (sx + sy * d + sz * d * d);
      V3<T> nd = -V3<T>{(T)lp[12], (T)lp[13], (T)lp[14]};
      ls = ls * (gmax(dot(n, nd), (T)0) * att);
      l = normalize(nd);
    } else if (type == 2) {
      T d = length(pos - v0);
      T att = (T)1 / (sx + sy * d + sz * d * d);
      V3<T> to = normalize(v0 - pos);
      ls = ls * (gmax(dot(n, to), (T)0) * att);
      l = to;
    } else if (type == 5) {
      T ux = random_float<T>(re), uy = random_float<T>(re);
      T sq = std::sqrt(ux);
      T bx = (T)1 - sq, by = uy * sq;
      V3<T> p2{(T)lp[4], (T)lp[5], (T)lp[6]}, p3{(T)lp[8], (T)lp[9], (T)lp[10]};
      V3<T> lpt = v0 * ((T)1 - bx - by) + p2 * bx + p3 * by;
      V3<T> ld = lpt - pos;
      V3<T> lnr = cross(p2 - v0, p3 - v0);
      T area = (T)0.5f * length(lnr);
      V3<T> ln = normalize(lnr);
      T d = length(ld);
      ld = ld / d;
      T att = (T)1 / (sx + sy * d + sz * d * d);
      ls = ls * (gmax(dot(n, ld), (T)0) * gmax(dot(-ld, ln), (T)0) * att * area);
      l = ld;
      tmax = d - tmin;
    }
    if (length(ls) < (T)1e-6f) {
      pdf = 0;
      l = v3<T>((T)0);
      return v3<T>((T)0);
    }
    pdf = 1;
    lit = !occluded(l, tmax);
    if (light_mode == 1) return ls * (T)light_strength_sum / lstr;
    return ls * (T)sc->light_count;
  }

  // nextEventEsitmation (lighting.glsl:246-261)
  V3<T> nee(V3<T> pos, V3<T> o, const SI& s, bool miss, V3<T> thr, RandomEngine& re, uint64_t& srays) const {
    if (miss) return sky(-o) * thr;
    V3<T> l;
    T lpdf;
    bool lit;
    V3<T> lc = sample_light(pos, s.normal, re, l, lpdf, lit, srays);
    if (!lit) return v3<T>((T)0);
    if (lc.x == 0 && lc.y == 0 && lc.z == 0) return lc;
    V3<T> lh = normalize(l + o);
    V3<T> b = brdf(o, l, lh, s);
    T bp = pdf_brdf(s, o, l, lh);
    T f = lpdf * lpdf, g = bp * bp;
    T wgt = f / (f + g);
    V3<T> light = v3<T>((T)0) + lc * b * wgt / lpdf;
    return gmin(thr * light, v3<T>((T)10));
  }

  void miss_si(SI& s, V3<T>& pos, uint32_t& cat) const {
    pos = v3<T>((T)1.0e10f);
    cat = 0xffffffffu;
    s.normal = v3<T>((T)1);
    s.emissive = s.diffuse = s.specular = s.r0 = s.r90 = s.transmissive = v3<T>((T)0);
    s.pr = s.metal = s.ar = 0;
    s.illum = 0;
    s.b0 = s.b1 = s.b2 = v3<T>((T)0);
    s.ior = 1;
  }

  // One sample of ptRaygen main (ptRaygen.rgen:24-104).
  struct Out {
    V3<T> final_color;  // clamped
    V3<T> albedo;
    T depth;
    V3<T> normal;
    uint32_t cat;
    long prim_tri;
  };
  Out sample(int x, int y, int W, int H, const M4<T>& iv, const M4<T>& ip, uint32_t frame, uint32_t sample_n,
             bool final_image, uint64_t rays[3]) const {
    RandomEngine re = re_init((uint32_t)x, (uint32_t)y, frame);
    V3<T> thr = v3<T>((T)1);
    // createRay (camera.glsl:6-16)
    T pcx = (T)x + (T)0.5f, pcy = (T)y + (T)0.5f;
    if (final_image && sample_n > 0) {
      T jx = random_float<T>(re), jy = random_float<T>(re);
      pcx = pcx + (jx - (T)0.5f);
      pcy = pcy + (jy - (T)0.5f);
    }
    T cx = pcx / (T)W * (T)2 - (T)1, cy = pcy / (T)H * (T)2 - (T)1;
    V4<T> wsp = iv.c[3];
    V4<T> d4 = ip * V4<T>{cx, cy, (T)1, (T)1};
    V3<T> nd = normalize(d4.xyz());
    V4<T> wsd = iv * V4<T>{nd.x, nd.y, nd.z, (T)0};
    V3<T> org = wsp.xyz(), dir = wsd.xyz();
    T th = 0, tu = 0, tv = 0;
    long tri = trace(org, dir, (T)0.001f, (T)10000, false, th, tu, tv, rays[0]);
    SI si;
    V3<T> pos;
    uint32_t cat;
    bool miss = tri < 0;
    if (miss) miss_si(si, pos, cat);
    else pos = closest_hit(dir, w.tri_inst[tri], w.tri_prim[tri], tu, tv, si, cat);
    V3<T> fc = v3<T>((T)0);
    fc = fc + nee(pos, -normalize(dir), si, miss, thr, re, rays[2]);
    fc = fc + si.emissive;
    Out out;
    out.albedo = si.diffuse + si.specular;
    out.depth = distance(pos, org);
    out.normal = si.normal;
    out.cat = cat;
    out.prim_tri = tri;
    if (!miss) {
      V3<T> wpos = org;
      int trans = 0;
      for (int i = 0; (uint32_t)i < (uint32_t)max_depth && trans < 10; ++i) {
        if (si.illum == 7) {
          --i;
          ++trans;
        }
        V3<T> v = normalize(wpos - pos);
        wpos = pos;
        // indirectLighting (lighting.glsl:263-287)
        V3<T> l;
        T pdf;
        V3<T> b = sample_brdf(si, re, v, l, pdf);
        if ((b.x == 0 && b.y == 0 && b.z == 0) || pdf < (T)1e-6f) break;  // path ends
        T t = dot(l, si.normal);
        if (si.illum == 7) t = 1;
        V3<T> pt = thr * (b * t) / pdf;
        if ((uint32_t)i > (uint32_t)min_depth) {
          if (random_float<T>(re) < (T)0.05f) break;  // path ends
          pt = pt / ((T)1 - (T)0.05f);
        }
        thr = pt;
        tri = trace(pos, l, (T)0.001f, (T)10000, false, th, tu, tv, rays[1]);
        bool m2 = tri < 0;
        SI s2;
        V3<T> p2;
        uint32_t c2;
        if (m2) miss_si(s2, p2, c2);
        else p2 = closest_hit(l, w.tri_inst[tri], w.tri_prim[tri], tu, tv, s2, c2);
        V3<T> indir = nee(p2, -l, s2, m2, thr, re, rays[2]) + s2.emissive * thr;
        fc = fc + indir;
        si = s2;
        pos = p2;
        if (m2) break;  // later iterations add nothing
      }
    }
    out.final_color = clamp3(fc, (T)0, (T)10);
    return out;
  }
};

// The last scene's world-space triangles and BVH are kept, keyed by the
// scene arrays' identity, so repeated renders of one scene build them once.
template <class T> World<T>& cached_world(const OrcScene* sc) {
  static World<T> w;
  static const void* key[4] = {nullptr, nullptr, nullptr, nullptr};
  const void* k[4] = {sc->idx, sc->inst_mat, sc->pos, (const void*)(uintptr_t)sc->instance_count};
  if (std::memcmp(k, key, sizeof(k)) != 0) {
    w = World<T>();
    w.build(sc);
    std::memcpy(key, k, sizeof(k));
  }
  w.sc = sc;
  return w;
}

template <class T>
int render(const OrcScene* sc, int W, int H, const float* inv_view, const float* inv_proj, uint32_t frame,
           uint32_t sample_n, int min_depth, int max_depth, int light_mode, int final_image, int frames, float* illum,
           float* depth, float* normal, uint8_t* material, uint8_t* albedo, uint32_t* hit_key, uint64_t* ray_counts,
           int threads) {
  World<T>& w = cached_world<T>(sc);
  Tracer<T> tr{w, sc, light_mode, min_depth, max_depth,
               sc->light_count ? sc->lights[32 * (sc->light_count - 1) + 31] : 0.f};
  M4<T> iv, ip;
  for (int c = 0; c < 4; ++c) {
    iv.c[c] = V4<T>{(T)inv_view[4 * c], (T)inv_view[4 * c + 1], (T)inv_view[4 * c + 2], (T)inv_view[4 * c + 3]};
    ip.c[c] = V4<T>{(T)inv_proj[4 * c], (T)inv_proj[4 * c + 1], (T)inv_proj[4 * c + 2], (T)inv_proj[4 * c + 3]};
  }
  std::atomic<uint64_t> r0(0), r1(0), r2(0);
  // map instance-major flat index -> key (the flat index itself)
  parallel_rows(H, threads, [&](int y) {
    uint64_t rays[3] = {0, 0, 0};
    for (int x = 0; x < W; ++x) {
      size_t p = (size_t)y * W + x;
      V3<T> acc = v3<T>((T)0);
      typename Tracer<T>::Out o0{};
      for (int f = 0; f < frames; ++f) {
        auto o = tr.sample(x, y, W, H, iv, ip, frame + (uint32_t)f, sample_n, final_image != 0, rays);
        if (f == 0) o0 = o;
        acc = acc + o.final_color;
      }
      V3<T> fc = frames == 1 ? o0.final_color : acc / (T)frames;
      if (!final_image) {
        V3<T> dm = gmin(fc / (o0.albedo + v3<T>((T)1e-6f)), v3<T>((T)1e3f));
        illum[4 * p] = (float)dm.x;
        illum[4 * p + 1] = (float)dm.y;
        illum[4 * p + 2] = (float)dm.z;
        illum[4 * p + 3] = 1.f;
      } else {
        // FINAL_IMAGE with sample_n == 0 (no previous frame blended here)
        const T g = (T)(1.0f / 2.2f);
        V3<T> s = clamp3(V3<T>{Pow(fc.x, g), Pow(fc.y, g), Pow(fc.z, g)}, (T)0, (T)1);
        illum[4 * p] = (float)s.x;
        illum[4 * p + 1] = (float)s.y;
        illum[4 * p + 2] = (float)s.z;
        illum[4 * p + 3] = 1.f;
      }
      if (depth) depth[p] = (float)o0.depth;
      if (normal) {
        normal[2 * p] = (float)std::acos(o0.normal.z);
        normal[2 * p + 1] = (float)std::atan2(o0.normal.y, o0.normal.x);
      }
      if (material) {
        material[4 * p] = f2u8((float)o0.cat / 255.0f);
        material[4 * p + 1] = material[4 * p + 2] = material[4 * p + 3] = 0;
      }
      if (albedo) {
        albedo[4 * p] = f2u8((float)o0.albedo.x);
        albedo[4 * p + 1] = f2u8((float)o0.albedo.y);
        albedo[4 * p + 2] = f2u8((float)o0.albedo.z);
        albedo[4 * p + 3] = 255;
      }
      if (hit_key) hit_key[p] = o0.prim_tri < 0 ? 0xffffffffu : (uint32_t)o0.prim_tri;
    }
    r0 += rays[0];
    r1 += rays[1];
    r2 += rays[2];
  });
  if (ray_counts) {
    ray_counts[0] = r0;
    ray_counts[1] = r1;
    ray_counts[2] = r2;
  }
  return 0;
}

}  // namespace

extern "C" {

// precision 32: FP32 as the shaders; 64: FP64. frames > 1 averages that many
// consecutive frame numbers (independent RNG streams) before demodulating.
int oracle_render(const OrcScene* sc, int W, int H, const float* inv_view, const float* inv_proj, uint32_t frame,
                  uint32_t sample_n, int min_depth, int max_depth, int light_mode, int final_image, int precision,
                  int frames, float* illum, float* depth, float* normal, uint8_t* material, uint8_t* albedo,
                  uint32_t* hit_key, uint64_t* ray_counts, int threads) {
  if (!sc || W <= 0 || H <= 0 || frames <= 0 || !illum) return -1;
  if (precision == 64)
    return render<double>(sc, W, H, inv_view, inv_proj, frame, sample_n, min_depth, max_depth, light_mode, final_image,
                          frames, illum, depth, normal, material, albedo, hit_key, ray_counts, threads);
  return render<float>(sc, W, H, inv_view, inv_proj, frame, sample_n, min_depth, max_depth, light_mode, final_image,
                       frames, illum, depth, normal, material, albedo, hit_key, ray_counts, threads);
}

// Ray queries against the oracle's world triangles (FP64 watertight test).
int oracle_trace_rays(const OrcScene* sc, const float* org_tmin, const float* dir_tmax, uint32_t n, int any_hit,
                      float* hits, int precision, int threads) {
  auto run = [&](auto tag) {
    using T = decltype(tag);
    World<T>& w = cached_world<T>(sc);
    Tracer<T> tr{w, sc, 0, 0, 0, 0.f};
    parallel_rows((int)((n + 255) / 256), threads, [&](int blk) {
      uint64_t rays = 0;
      for (uint32_t i = (uint32_t)blk * 256; i < std::min(n, (uint32_t)blk * 256 + 256); ++i) {
        V3<T> o{(T)org_tmin[4 * i], (T)org_tmin[4 * i + 1], (T)org_tmin[4 * i + 2]};
        V3<T> d{(T)dir_tmax[4 * i], (T)dir_tmax[4 * i + 1], (T)dir_tmax[4 * i + 2]};
        T th, tu = 0, tv = 0;
        long t = tr.trace(o, d, (T)org_tmin[4 * i + 3], (T)dir_tmax[4 * i + 3], any_hit != 0, th, tu, tv, rays);
        hits[4 * i] = (float)th;
        hits[4 * i + 1] = (float)tu;
        hits[4 * i + 2] = (float)tv;
        uint32_t key = t < 0 ? 0xffffffffu : (uint32_t)t;
        std::memcpy(&hits[4 * i + 3], &key, 4);
      }
    });
  };
  if (precision == 64) run(0.0);
  else run(0.0f);
  return 0;
}

// Known-answer helpers: n numbers of the stream of pixel (x, y) at frame.
void oracle_rng_stream(uint32_t x, uint32_t y, uint32_t frame, int n, float* out) {
  RandomEngine re = re_init(x, y, frame);
  for (int i = 0; i < n; ++i) out[i] = random_float<float>(re);
}

}  // extern "C"
