// Oracle (test infrastructure only): CPU restatement of VulkanPBRT's
// accumulator and regression denoisers, in the reference's own FP32 "as
// shader" arithmetic and with its storage quantisation points.
//
// Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference
// legs load this code, as the checker of the CUDA path; the product never does.
//
// Parity pin: the reference ships no tests, golden images or known-answer
// vectors, and its GLSL cannot be compiled or run in this environment (no
// shader compiler, no Vulkan). This restatement is therefore pinned only by
// its own known-answer tests (tests/golden) and by line-by-line citations of
// the shaders below: parity unpinned against the shaders themselves.
//
// Image layouts follow the reference's Vulkan formats, stored row-major
// (index = y * width + x):
//   depth R32F float, normal RG32F float2 (theta, phi), albedo RGBA8,
//   noisy / accumulated illumination RGBA16F (4 x binary16),
//   motion RG16F, spp R8_UNORM, denoised RGBA16F x 2 layers,
//   final B8G8R8A8_UNORM (bytes B,G,R,A), feature buffer R16F x 13 layers at
//   padded size, weights R32F x 30 layers at block-grid size.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <limits>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "glsl.hpp"

using namespace orc;
typedef V2<float> vec2;
typedef V3<float> vec3;
typedef V4<float> vec4;
typedef M4<float> mat4;

namespace {

// Run f(i) for i in [0, n) over the machine's cores (one task per row/block).
template <class F> void parallel_for(int n, F f, int threads = 0) {
  if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
  threads = std::min(threads, std::max(1, n));
  if (threads == 1) {
    for (int i = 0; i < n; ++i) f(i);
    return;
  }
  std::vector<std::thread> pool;
  std::atomic_int next(0);
  for (int t = 0; t < threads; ++t)
    pool.emplace_back([&]() {
      for (int i = next++; i < n; i = next++) f(i);
    });
  for (auto& th : pool) th.join();
}

inline int wrap_repeat(float c, int n) {
  // REPEAT addressing of texel index c (already floored); NaN/inf map to 0.
  if (!std::isfinite(c)) return 0;
  float m = c - (float)n * std::floor(c / (float)n);
  int i = (int)m;
  if (i < 0) i = 0;
  if (i >= n) i = n - 1;
  return i;
}

// Bilinear filtering of a level-0 image with REPEAT addressing, as the
// reference's default sampler (LINEAR/LINEAR, REPEAT, maxLod 0;
// external/vsg/include/vsg/state/Sampler.h:29-42). fetch(x, y, out[4]).
template <class Fetch> void bilinear(int W, int H, vec2 uv, Fetch fetch, float out[4]) {
  float x = uv.x * (float)W - 0.5f, y = uv.y * (float)H - 0.5f;
  float x0 = std::floor(x), y0 = std::floor(y);
  float fx = x - x0, fy = y - y0;
  if (!std::isfinite(fx)) fx = 0.f;
  if (!std::isfinite(fy)) fy = 0.f;
  int i0 = wrap_repeat(x0, W), i1 = wrap_repeat(x0 + 1.f, W);
  int j0 = wrap_repeat(y0, H), j1 = wrap_repeat(y0 + 1.f, H);
  float t00[4], t10[4], t01[4], t11[4];
  fetch(i0, j0, t00);
  fetch(i1, j0, t10);
  fetch(i0, j1, t01);
  fetch(i1, j1, t11);
  for (int c = 0; c < 4; ++c) {
    float a = mix(t00[c], t10[c], fx);
    float b = mix(t01[c], t11[c], fx);
    out[c] = mix(a, b, fy);
  }
}

// Normal decode used by bmfrPre/bmfrPost/bfr (shaders/bmfrPre.comp:27-30).
inline vec3 decode_normal(float th, float ph) {
  return vec3{std::cos(ph) * std::sin(th), std::sin(ph) * std::sin(th), std::cos(th)};
}

// shaders/bmfrGeneral.comp:93-101
inline int mirror1(int x, int s) {
  if (x < 0) return std::abs(x) - 1;
  if (x >= s) return 2 * s - x - 1;
  return x;
}

// shaders/bmfrGeneral.comp:36 (float pairs, scaled by the block edge and
// truncated toward zero by ivec2()).
const float kBmfrOffsets[16][2] = {{.7f, .85f}, {.95f, .5f}, {.43f, .76f}, {.97f, .03f}, {.37f, .58f}, {.03f, .36f},
                                   {.81f, .46f}, {0.f, .78f}, {.36f, -.08f}, {-.06f, 0.f}, {.95f, .1f}, {.85f, .61f},
                                   {.06f, .1f},  {.43f, .16f}, {0.f, .5f},  {.73f, .38f}};
// shaders/bfr.comp:92
const int kBfrOffsets[16][2] = {{-7, -11}, {-14, -8}, {-5, -12}, {-15, -1}, {-5, -9}, {-1, -4}, {-14, -7}, {0, -13},
                                {-5, -1},  {-1, 0},   {-15, -2}, {-14, -10}, {-1, -1}, {-6, -3}, {0, -8},  {-10, -4}};

// shaders/bmfrGeneral.comp:103-113 (Wang-style integer hash to [0,1]).
inline float bmfr_random(uint32_t a) {
  a = (a + 0x7ed55d16u) + (a << 12);
  a = (a ^ 0xc761c23cu) ^ (a >> 19);
  a = (a + 0x165667b1u) + (a << 5);
  a = (a + 0xd3a2646cu) ^ (a << 9);
  a = (a + 0xfd7046c5u) + (a << 3);
  a = (a ^ 0xb55a4f09u) ^ (a >> 16);
  return (float)a / (float)0xffffffffu;
}

// Block-wide sum in the order the CUDA kernels use: per-lane partials, an
// xor-butterfly over each 32-lane subgroup, then subgroups in index order
// (shaders/bmfrGeneral.comp:79-91 leaves the in-subgroup order open).
inline float subgroup_sum(const float* v) {
  float t[32];
  for (int i = 0; i < 32; ++i) t[i] = v[i];
  for (int off = 16; off >= 1; off >>= 1) {
    float n[32];
    for (int i = 0; i < 32; ++i) n[i] = t[i] + t[i ^ off];
    std::memcpy(t, n, sizeof(t));
  }
  return t[0];
}
inline float block_sum(const std::vector<float>& v) {
  int n = (int)v.size(), groups = (n + 31) / 32;
  float acc = 0.f;
  for (int g = 0; g < groups; ++g) {
    float lanes[32];
    for (int i = 0; i < 32; ++i) lanes[i] = (g * 32 + i < n) ? v[g * 32 + i] : 0.f;
    float s = subgroup_sum(lanes);
    acc = (g == 0) ? s : acc + s;
  }
  return acc;
}

struct Cam {
  mat4 inv_view, inv_proj;
};

// Position feature per POSITION_TYPE (shaders/bmfrPre.comp:38-76); returns the
// un-normalised value the reductions run over.
inline vec3 world_pos(const Cam& c, int W, int H, int ix, int iy, float depth, bool add_origin) {
  vec2 pc{(float)ix + .5f, (float)iy + .5f};
  vec2 npc{pc.x / (float)W, pc.y / (float)H};
  vec2 clip{npc.x * 2.f - 1.f, npc.y * 2.f - 1.f};
  vec4 wsp = c.inv_view * vec4{0, 0, 0, 1};
  vec4 vsd = c.inv_proj * vec4{clip.x, clip.y, 1, 1};
  vec4 wsd = c.inv_view * v4(normalize(vsd.xyz()), 0.f);
  vec3 p = wsd.xyz() * depth;
  if (add_origin) p = wsp.xyz() + p;
  return p;
}

// Per-block feature computation shared by bmfrPre and bmfrPost
// (shaders/bmfrPre.comp:5-98, shaders/bmfrPost.comp:5-163). Fills, for each
// of the bw*bh invocations (local index ly*bw+lx), the 10 regression features
// in FP32 plus the image position and whether it lies inside the image.
struct BlockPix {
  float f[10];
  int ix, iy;
  bool inside;
};
void bmfr_block_features(int W, int H, int bw, int bh, int gx, int gy, uint32_t frame, int position_type,
                         const Cam& cam, const float* depth, const float* normal, std::vector<BlockPix>& out) {
  int n = bw * bh;
  out.resize(n);
  std::vector<vec3> pos(n), nor(n);
  int offx = (int)((float)bw * kBmfrOffsets[frame % 16][0]);
  int offy = (int)((float)bh * kBmfrOffsets[frame % 16][1]);
  for (int ly = 0; ly < bh; ++ly)
    for (int lx = 0; lx < bw; ++lx) {
      int li = ly * bw + lx;
      int ax = gx * bw + lx - offx, ay = gy * bh + ly - offy;
      int ix = mirror1(ax, W), iy = mirror1(ay, H);
      out[li].ix = ix;
      out[li].iy = iy;
      out[li].inside = (ax == ix && ay == iy);
      size_t p = (size_t)iy * W + ix;
      float d = depth[p];
      nor[li] = decode_normal(normal[2 * p], normal[2 * p + 1]);
      pos[li] = vec3{0.f, 0.f, d};
      if (position_type == 1) pos[li] = vec3{0.f, 0.f, d};
      if (position_type == 2) pos[li] = world_pos(cam, W, H, ix, iy, d, true);
    }
  const float EPS = 1e-6f;
  if (position_type == 0 || position_type == 1) {
    float mn = pos[0].z, mx = pos[0].z;
    for (int i = 0; i < n; ++i) {
      mn = gmin(mn, pos[i].z);
      mx = gmax(mx, pos[i].z);
    }
    for (int ly = 0; ly < bh; ++ly)
      for (int lx = 0; lx < bw; ++lx) {
        int li = ly * bw + lx;
        float z = pos[li].z;
        z -= mn;
        z /= mx - mn + EPS;
        if (position_type == 0) {
          pos[li] = vec3{(float)lx / ((float)bw - 1.f), (float)ly / ((float)bh - 1.f), z};
        } else {
          pos[li] = world_pos(cam, W, H, out[li].ix, out[li].iy, z, false);
        }
      }
  } else {
    for (int a = 0; a < 3; ++a) {
      float mn = pos[0][a], mx = pos[0][a];
      for (int i = 0; i < n; ++i) {
        mn = gmin(mn, pos[i][a]);
        mx = gmax(mx, pos[i][a]);
      }
      for (int i = 0; i < n; ++i) {
        float v = pos[i][a];
        v -= mn;
        v /= mx - mn + EPS;
        pos[i][a] = v;
      }
    }
  }
  for (int i = 0; i < n; ++i) {
    vec3 p = pos[i], q = nor[i];
    float* f = out[i].f;
    f[0] = 1.f;
    f[1] = q.x;
    f[2] = q.y;
    f[3] = q.z;
    f[4] = p.x;
    f[5] = p.y;
    f[6] = p.z;
    f[7] = p.x * p.x;
    f[8] = p.y * p.y;
    f[9] = p.z * p.z;
  }
}

inline void load_half4(const uint16_t* img, size_t p, float o[4]) {
  for (int c = 0; c < 4; ++c) o[c] = h2f(img[4 * p + c]);
}

// Temporal blend, albedo remodulation and tone map shared by bmfrPost and bfr
// (shaders/bmfrPost.comp:194-214, shaders/bfr.comp:289-308).
void post_store(int W, int H, uint32_t frame, vec3 dc, int ix, int iy, const uint8_t* albedo, const uint16_t* motion,
                const uint8_t* spp, uint16_t* denoised, uint8_t* final_bgra) {
  size_t p = (size_t)iy * W + ix;
  size_t layer = (size_t)W * H;
  dc = clamp3(dc, 0.f, 10.f);
  vec2 uv{h2f(motion[2 * p]), h2f(motion[2 * p + 1])};
  bool accept = uv.x >= 0.f;
  float pixel_spp = u82f(spp[p]) * 256.f;
  vec3 prev{0, 0, 0};
  float a = 1.f;
  if (frame > 0 && accept) {
    const uint16_t* src = denoised + (size_t)(frame & 1) * layer * 4;
    float s[4];
    bilinear(W, H, uv, [&](int x, int y, float o[4]) { load_half4(src, (size_t)y * W + x, o); }, s);
    prev = prev + vec3{s[0], s[1], s[2]};
    a = gmax(1.f / pixel_spp, 0.1f);
  }
  dc = a * dc + (1.f - a) * prev;
  uint16_t* dst = denoised + (size_t)((frame & 1) ^ 1) * layer * 4;
  dst[4 * p + 0] = f2h(dc.x);
  dst[4 * p + 1] = f2h(dc.y);
  dst[4 * p + 2] = f2h(dc.z);
  dst[4 * p + 3] = f2h(1.f);
  vec3 alb{u82f(albedo[4 * p]) + 1e-6f, u82f(albedo[4 * p + 1]) + 1e-6f, u82f(albedo[4 * p + 2]) + 1e-6f};
  vec3 t = gmax(v3(0.f), alb * dc);
  vec3 tm{std::pow(t.x, .454545f), std::pow(t.y, .454545f), std::pow(t.z, .454545f)};
  tm = clamp3(tm, 0.f, 1.f);
  final_bgra[4 * p + 0] = f2u8(tm.z);
  final_bgra[4 * p + 1] = f2u8(tm.y);
  final_bgra[4 * p + 2] = f2u8(tm.x);
  final_bgra[4 * p + 3] = 255;
}

Cam make_cam(const float* inv_view, const float* inv_proj) {
  Cam c;
  c.inv_view = load_m4<float>(inv_view);
  c.inv_proj = load_m4<float>(inv_proj);
  return c;
}

}  // namespace

extern "C" {

// accumulator.comp main (shaders/accumulator.comp:33-105) with the push
// constants Accumulator::set_camera_matrices writes
// (source/renderModules/Accumulator.cpp:85-117). separate=1 is the live
// renderer's SEPARATE_MATRICES variant: view = cur.inv_proj,
// inverse_view = cur.inv_view, prev_view = prev.view,
// prev_origin = inverse(prev.view)[3]. motion is written as RG (both
// components; the shader's r16f qualifier on an RG16F image is read as RG).
int oracle_accumulate(int W, int H, uint32_t frame, int separate, const float* view, const float* inverse_view,
                      const float* prev_view, const float* prev_origin, const float* src_rgba32f, const float* depth,
                      const float* prev_depth, const uint8_t* prev_spp, const uint16_t* prev_output,
                      uint16_t* motion_out, uint8_t* spp_out, uint16_t* illum_out, int threads) {
  mat4 V = load_m4<float>(view), IV = load_m4<float>(inverse_view), PV = load_m4<float>(prev_view);
  mat4 proj = inverse(V);
  mat4 proj_prev = proj * PV;  // GLSL evaluates proj * prevView * p left to right
  vec4 porg{prev_origin[0], prev_origin[1], prev_origin[2], prev_origin[3]};
  parallel_for(H, [&](int y) {
    for (int x = 0; x < W; ++x) {
      size_t p = (size_t)y * W + x;
      bool reprojected = false;
      float pixel_spp = 1.f / 256.f;
      float d = depth[p];
      vec4 pp, prev_pos;
      if (separate) {
        vec4 pos = IV.c[3];
        pos.w = 1.f;
        vec2 pc{(float)x + .5f, (float)y + .5f};
        vec2 clip{pc.x / (float)W * 2.f - 1.f, pc.y / (float)H * 2.f - 1.f};
        vec4 dir = V * vec4{clip.x, clip.y, 1, 1};
        dir = IV * v4(normalize(dir.xyz()), 0.f);
        pp = pos + dir * d;
        prev_pos = proj_prev * pp;
      } else {
        vec4 org = IV.c[2];
        org = org / org.w;
        vec2 clip{((float)x + .5f) / (float)W * 2.f - 1.f, ((float)y + .5f) / (float)H * 2.f - 1.f};
        vec4 cd = IV * vec4{clip.x, clip.y, 1, 1};
        cd = cd / (cd.w + 1e-9f);
        vec4 diff = cd - org;  // normalize() of a vec4 uses all four components
        float len = std::sqrt(dot(diff, diff));
        cd = diff / len;
        cd = vec4{-cd.x, -cd.y, -cd.z, -cd.w};
        pp = org + cd * d;
        prev_pos = PV * pp;
      }
      float pre_depth = length(pp.xyz() - porg.xyz());
      prev_pos = prev_pos / prev_pos.w;
      prev_pos.x += 1.f;
      prev_pos.y += 1.f;
      prev_pos.x *= .5f;
      prev_pos.y *= .5f;
      prev_pos.x *= (float)W / ((float)W - .5f);
      prev_pos.y *= (float)H / ((float)H - .5f);
      vec3 prev_color{0, 0, 0};
      vec2 uv{prev_pos.x, prev_pos.y};
      if (frame > 0) {
        float s[4];
        bilinear(W, H, uv, [&](int i, int j, float o[4]) { o[0] = prev_depth[(size_t)j * W + i]; o[1] = o[2] = o[3] = 0; }, s);
        float dissim = (s[0] / pre_depth) - 1.f;
        if (uv.x >= 0.f && uv.y >= 0.f && uv.x <= 1.f && uv.y <= 1.f && std::fabs(dissim) <= .01f) {
          reprojected = true;
          float c[4];
          bilinear(W, H, uv, [&](int i, int j, float o[4]) { load_half4(prev_output, (size_t)j * W + i, o); }, c);
          prev_color = vec3{c[0], c[1], c[2]};
          float sp[4];
          bilinear(W, H, uv, [&](int i, int j, float o[4]) { o[0] = u82f(prev_spp[(size_t)j * W + i]); o[1] = o[2] = o[3] = 0; }, sp);
          pixel_spp += sp[0];
        }
      }
      if (reprojected) {
        motion_out[2 * p] = f2h(uv.x);
        motion_out[2 * p + 1] = f2h(uv.y);
      } else {
        motion_out[2 * p] = f2h(-1.f);
        motion_out[2 * p + 1] = f2h(-1.f);
      }
      spp_out[p] = f2u8(pixel_spp);
      vec3 demod{src_rgba32f[4 * p], src_rgba32f[4 * p + 1], src_rgba32f[4 * p + 2]};
      if (reprojected) {
        float a = gmax(1.f / (pixel_spp * 256.f), .1f);
        demod = mix(prev_color, demod, a);
      }
      illum_out[4 * p + 0] = f2h(demod.x);
      illum_out[4 * p + 1] = f2h(demod.y);
      illum_out[4 * p + 2] = f2h(demod.z);
      illum_out[4 * p + 3] = f2h(1.f);
    }
  }, threads);
  return 0;
}

// bmfrPre main (shaders/bmfrPre.comp:5-98): 13 R16F feature layers at padded
// size ((W/bw+2)*bw x (H/bh+2)*bh), layer-major.
int oracle_bmfr_pre(int W, int H, int bw, uint32_t frame, int position_type, const float* inv_view,
                    const float* inv_proj, const float* depth, const float* normal, const uint16_t* noisy,
                    uint16_t* features, int threads) {
  int gw = W / bw + 2, gh = H / bw + 2, PW = gw * bw, PH = gh * bw;
  Cam cam = make_cam(inv_view, inv_proj);
  parallel_for(gw * gh, [&](int b) {
    int gx = b % gw, gy = b / gw;
    std::vector<BlockPix> px;
    bmfr_block_features(W, H, bw, bw, gx, gy, frame, position_type, cam, depth, normal, px);
    for (int ly = 0; ly < bw; ++ly)
      for (int lx = 0; lx < bw; ++lx) {
        const BlockPix& q = px[ly * bw + lx];
        size_t ip = (size_t)q.iy * W + q.ix;
        size_t gp = (size_t)(gy * bw + ly) * PW + (gx * bw + lx);
        for (int c = 0; c < 10; ++c) features[(size_t)c * PW * PH + gp] = f2h(q.f[c]);
        for (int c = 0; c < 3; ++c) features[(size_t)(10 + c) * PW * PH + gp] = f2h(h2f(noisy[4 * ip + c]));
      }
  }, threads);
  return 0;
}

// bmfrFit main (shaders/bmfrFit.comp:5-92): per block, Householder QR of the
// 1024x13 (bw*bw rows) feature matrix with 1e-4 hash noise on the 10 feature
// columns, back substitution for 10 RGB weights; weights R32F x 30 layers at
// block-grid size, layer index feature*3+channel. fit_threads = the fitting
// kernel's invocation count (256, or 64 for 8x8 blocks).
int oracle_bmfr_fit(int W, int H, int bw, int fit_threads, uint32_t frame, const uint16_t* features, float* weights,
                    int threads) {
  int gw = W / bw + 2, gh = H / bw + 2, PW = gw * bw, PH = gh * bw;
  int P = bw * bw, K = fit_threads, SV = P / K;
  if (SV < 1 || P % K) return -1;
  parallel_for(gw * gh, [&](int b) {
    int gx = b % gw, gy = b / gw;
    // A[row][col], row = id + sv*K = pixel (row / bw, row % bw) of the block.
    std::vector<float> A((size_t)P * 13);
    for (int col = 0; col < 13; ++col)
      for (int sv = 0; sv < SV; ++sv)
        for (int id = 0; id < K; ++id) {
          int index = id + sv * K;
          int px = index / bw + gx * bw, py = index % bw + gy * bw;
          float t = h2f(features[(size_t)col * PW * PH + (size_t)py * PW + px]);
          if (col < 10) {
            uint32_t h = (uint32_t)id + (uint32_t)sv * (uint32_t)K + (uint32_t)col * (uint32_t)P * (uint32_t)P +
                         frame * 13u * (uint32_t)P * (uint32_t)P;
            t = t + 1e-4f * 2.f * (bmfr_random(h) - .5f);
          }
          A[(size_t)index * 13 + col] = t;
        }
    std::vector<float> part(K), u(P);
    float ulen2 = 0.f;
    float R[10][13];
    for (int col = 0; col < 10; ++col) {
      for (int id = 0; id < K; ++id) {
        float v2 = 0.f;
        for (int sv = 0; sv < SV; ++sv) {
          int index = id + sv * K;
          float uu = A[(size_t)index * 13 + col];
          u[index] = uu;
          if (index > col) v2 += uu * uu;
        }
        part[id] = v2;
      }
      float vls = block_sum(part);
      for (int sv = 0; sv < SV; ++sv)
        for (int id = 0; id < K; ++id) {
          int index = id + sv * K;
          if (index < col) u[index] = 0.f;  // u[0] = 0 for id < col (sv = 0 rows)
        }
      float vlen = std::sqrt(vls + u[col] * u[col]);
      u[col] -= vlen;
      vls += u[col] * u[col];
      ulen2 = vls;
      R[col][col] = vlen;
      for (int f = col + 1; f < 13; ++f) {
        for (int id = 0; id < K; ++id) {
          float v = 0.f;
          for (int sv = 0; sv < SV; ++sv) {
            int index = id + sv * K;
            if (index >= col) v += A[(size_t)index * 13 + f] * u[index];
          }
          part[id] = v;
        }
        float v = block_sum(part);
        // features -= 2 * u * v / uLengthSquared, with the division taken as a
        // product with the correctly rounded reciprocal (within the 2.5 ULP
        // Vulkan allows a shader's x / y).
        float rl = 1.f / ulen2;
        for (int index = col; index < P; ++index) A[(size_t)index * 13 + f] -= 2.f * u[index] * v * rl;
      }
      for (int f = col + 1; f < 13; ++f) R[col][f] = A[(size_t)col * 13 + f];
    }
    vec3 ws[10];
    for (int i = 9; i >= 0; --i) {
      ws[i] = vec3{R[i][10], R[i][11], R[i][12]};
      for (int x = i + 1; x < 10; ++x) ws[i] = ws[i] - ws[x] * R[i][x];
      ws[i] = ws[i] / R[i][i];
    }
    for (int id = 0; id < 10; ++id) {
      vec3 w = ws[id];
      if (ulen2 == 0.f) w = v3(.2f);
      size_t L = (size_t)gw * gh;
      weights[(size_t)(id * 3 + 0) * L + (size_t)gy * gw + gx] = w.x;
      weights[(size_t)(id * 3 + 1) * L + (size_t)gy * gw + gx] = w.y;
      weights[(size_t)(id * 3 + 2) * L + (size_t)gy * gw + gx] = w.z;
    }
  }, threads);
  return 0;
}

// bmfrPost main (shaders/bmfrPost.comp:5-124).
int oracle_bmfr_post(int W, int H, int bw, uint32_t frame, int position_type, const float* inv_view,
                     const float* inv_proj, const float* depth, const float* normal, const uint8_t* albedo,
                     const uint16_t* motion, const uint8_t* spp, const float* weights, uint16_t* denoised,
                     uint8_t* final_bgra, int threads) {
  int gw = W / bw + 2, gh = H / bw + 2;
  Cam cam = make_cam(inv_view, inv_proj);
  size_t L = (size_t)gw * gh;
  // Blocks write disjoint in-image pixels; rows of blocks run in parallel.
  parallel_for(gh, [&](int gy) {
    std::vector<BlockPix> px;
    for (int gx = 0; gx < gw; ++gx) {
      bmfr_block_features(W, H, bw, bw, gx, gy, frame, position_type, cam, depth, normal, px);
      float w[10][3];
      for (int f = 0; f < 10; ++f)
        for (int c = 0; c < 3; ++c) {
          float v = weights[(size_t)(f * 3 + c) * L + (size_t)gy * gw + gx];
          if (std::isinf(v) || std::isnan(v)) v = 0.f;
          w[f][c] = v;
        }
      for (auto& q : px) {
        if (!q.inside) continue;
        vec3 dc{0, 0, 0};
        for (int f = 0; f < 10; ++f) dc = dc + vec3{w[f][0], w[f][1], w[f][2]} * q.f[f];
        post_store(W, H, frame, dc, q.ix, q.iy, albedo, motion, spp, denoised, final_bgra);
      }
    }
  }, threads);
  return 0;
}

// bfr.comp main (shaders/bfr.comp:202-309): per bw x bh block, 40 Adam-style
// descent steps on 7 features (L1 when spp >= 10), then the shared post.
int oracle_bfr(int W, int H, int bw, int bh, uint32_t frame, const float* depth, const float* normal,
               const uint8_t* albedo, const uint16_t* motion, const uint8_t* spp, const uint16_t* noisy,
               uint16_t* denoised, uint8_t* final_bgra, int threads) {
  int gw = W / bw + 2, gh = H / bh + 2, n = bw * bh;
  int ox = kBfrOffsets[frame % 16][0], oy = kBfrOffsets[frame % 16][1];
  const int ASZ = 7;
  // Threads with ID = lx*bh+ly < 7 sharing thread 0's 32-lane subgroup
  // contribute to the stopping test (shaders/bfr.comp:136-137, 276-277).
  int n_stop = std::min(ASZ, (32 + bw - 1) / bw);
  parallel_for(gh, [&](int gy) {
    std::vector<float> feat((size_t)n * ASZ), part(n);
    std::vector<vec3> col(n);
    std::vector<int> l1(n), ix(n), iy(n);
    std::vector<bool> inside(n);
    for (int gx = 0; gx < gw; ++gx) {
      std::vector<float> dep(n);
      std::vector<vec3> nor(n);
      for (int ly = 0; ly < bh; ++ly)
        for (int lx = 0; lx < bw; ++lx) {
          int li = ly * bw + lx;
          int ax = gx * bw + lx + ox, ay = gy * bh + ly + oy;
          ix[li] = mirror1(ax, W);
          iy[li] = mirror1(ay, H);
          inside[li] = (ax == ix[li] && ay == iy[li]);
          size_t p = (size_t)iy[li] * W + ix[li];
          float s[4];
          load_half4(noisy, p, s);
          col[li] = vec3{s[0], s[1], s[2]};
          dep[li] = depth[p];
          nor[li] = decode_normal(normal[2 * p], normal[2 * p + 1]);
          l1[li] = (u82f(spp[p]) * 256.f >= 10.f) ? 1 : 0;
        }
      float mn = dep[0], mx = dep[0];
      for (int i = 0; i < n; ++i) {
        mn = gmin(mn, dep[i]);
        mx = gmax(mx, dep[i]);
      }
      for (int ly = 0; ly < bh; ++ly)
        for (int lx = 0; lx < bw; ++lx) {
          int li = ly * bw + lx;
          float d = dep[li];
          d -= mn;
          d /= mx - mn + 1e-8f;
          d = d * 2.f - 1.f;
          float* f = &feat[(size_t)li * ASZ];
          f[0] = 1.f;
          f[1] = (float)lx / ((float)bw - 1.f) - 0.5f;
          f[2] = (float)ly / ((float)bh - 1.f) - 0.5f;
          f[3] = d;
          f[4] = nor[li].x;
          f[5] = nor[li].y;
          f[6] = nor[li].z;
        }
      int l1sum = 0;
      for (int i = 0; i < n; ++i) l1sum += l1[i];
      vec3 alpha[ASZ], m[ASZ], v[ASZ];
      for (int j = 0; j < ASZ; ++j) alpha[j] = m[j] = v[j] = v3(0.f);
      float grad_rest = 0.f;
      for (int it = 0; grad_rest >= 0.f && it < 40; ++it) {
        std::vector<vec3> cdel(n);
        for (int i = 0; i < n; ++i) {
          vec3 c{0, 0, 0};
          for (int j = 0; j < ASZ; ++j) c = c + feat[(size_t)i * ASZ + j] * alpha[j];
          c = col[i] - c;
          if (l1[i]) c = vec3{signf(c.x), signf(c.y), signf(c.z)};
          cdel[i] = c;
        }
        vec3 delta[ASZ];
        for (int j = 0; j < ASZ; ++j) {
          float d3[3];
          for (int ch = 0; ch < 3; ++ch) {
            for (int i = 0; i < n; ++i) part[i] = feat[(size_t)i * ASZ + j] * cdel[i][ch];
            d3[ch] = block_sum(part);
          }
          delta[j] = vec3{d3[0], d3[1], d3[2]};
        }
        float t = (float)(it + 1);
        float l1r = (float)l1sum * 1.0f / (float)n;
        float a = l1r * 1.1f + (1.f - l1r) * .863f;
        float b1 = l1r * .45f + (1.f - l1r) * .3f;
        float b2 = l1r * .75f + (1.f - l1r) * .7314f;
        float step = a * std::exp(-.116f * t) * std::sqrt(1.f - std::pow(.7314f, t)) / (1.f - std::pow(.3f, t));
        for (int j = 0; j < ASZ; ++j) {
          vec3 dd = delta[j];
          m[j] = b1 * m[j] + (1.f - .3f) * dd;
          vec3 ad{std::fabs(dd.x), std::fabs(dd.y), std::fabs(dd.z)};
          v[j] = b2 * v[j] + (1.f - .7314f) * (ad * ad);
          vec3 den{std::sqrt(v[j].x) + 1e-8f, std::sqrt(v[j].y) + 1e-8f, std::sqrt(v[j].z) + 1e-8f};
          alpha[j] = alpha[j] + step * (m[j] / den);
        }
        vec3 g{0, 0, 0};
        for (int j = 0; j < n_stop; ++j) g = g + vec3{std::fabs(delta[j].x), std::fabs(delta[j].y), std::fabs(delta[j].z)};
        grad_rest = g.x + g.y + g.z;
      }
      for (int i = 0; i < n; ++i) {
        if (!inside[i]) continue;
        vec3 dc{0, 0, 0};
        for (int j = 0; j < ASZ; ++j) dc = dc + feat[(size_t)i * ASZ + j] * alpha[j];
        post_store(W, H, frame, dc, ix[i], iy[i], albedo, motion, spp, denoised, final_bgra);
      }
    }
  }, threads);
  return 0;
}

// TAA (shaders/taa.comp:48-103) with the history the reference keeps: the
// previous final B8G8R8A8 image copied byte for byte into an R8G8B8A8 image
// (source/renderModules/Taa.cpp:121-159), so the bilinear history sample
// returns the previous frame's (b, g, r). denoised / final: B8G8R8A8 bytes;
// history / history_next: the copied bytes; motion: RG16F.
int oracle_taa(int W, int H, uint32_t frame, const uint16_t* motion, const uint8_t* denoised, const uint8_t* history,
               uint8_t* final_bgra, uint8_t* history_next, int threads) {
  auto fetch = [&](size_t p) { return vec3{u82f(denoised[4 * p + 2]), u82f(denoised[4 * p + 1]), u82f(denoised[4 * p])}; };
  auto ycocg = [](vec3 c) {
    return vec3{c.x * 1.f + c.y * 2.f + c.z * 1.f, c.x * 2.f + c.y * 0.f + c.z * -2.f,
                c.x * -1.f + c.y * 2.f + c.z * -1.f};
  };
  parallel_for(H, [&](int y) {
    for (int x = 0; x < W; ++x) {
      const size_t p = (size_t)y * W + x;
      const vec3 cur = fetch(p);
      const vec2 uv{h2f(motion[2 * p]), h2f(motion[2 * p + 1])};
      vec3 res = cur;
      if (!(frame == 0 || uv.x < 0.f || uv.y < 0.f || uv.x > 1.f || uv.y > 1.f)) {
        const float inf = std::numeric_limits<float>::infinity();
        vec3 mn_box{inf, inf, inf}, mn_cross = mn_box, mx_box{-inf, -inf, -inf}, mx_cross = mx_box;
        for (int dy = -1; dy <= 1; ++dy)
          for (int dx = -1; dx <= 1; ++dx) {
            const int sx = x + dx, sy = y + dy;
            if (sx < 0 || sy < 0 || sx >= W || sy >= H) continue;
            const vec3 c = ycocg((dx == 0 && dy == 0) ? cur : fetch((size_t)sy * W + sx));
            if (dx == 0 || dy == 0) {
              mn_cross = gmin(mn_cross, c);
              mx_cross = gmax(mx_cross, c);
            }
            mn_box = gmin(mn_box, c);
            mx_box = gmax(mx_box, c);
          }
        float h[4];
        bilinear(W, H, uv, [&](int i, int j, float o[4]) {
          const size_t q = 4 * ((size_t)j * W + i);
          for (int k = 0; k < 4; ++k) o[k] = u82f(history[q + k]);
        }, h);
        const vec3 prev{h[0], h[1], h[2]};
        const vec3 pc = ycocg(prev);
        const vec3 mn = (mn_box + mn_cross) * .5f, mx = (mx_box + mx_cross) * .5f;
        const bool inside = pc.x >= mn.x && pc.y >= mn.y && pc.z >= mn.z && pc.x <= mx.x && pc.y <= mx.y && pc.z <= mx.z;
        if (inside) res = .4f * cur + (1.f - .4f) * prev;
      }
      const uint8_t o[4] = {f2u8(res.z), f2u8(res.y), f2u8(res.x), 255};
      for (int k = 0; k < 4; ++k) final_bgra[4 * p + k] = history_next[4 * p + k] = o[k];
    }
  }, threads);
  return 0;
}

// BFRBlender (shaders/bfrBlender.comp:31-68): blend of the 8x8 / 16x16 /
// 32x32 denoisers' 8-bit final images (den8 / den16 / den32, blended byte for
// byte) by the standard deviation of the average image's luminance over a
// (2 radius + 1)^2 window, each running mean blended 1:1 with the pixel's own
// average / average-square luminance. avg / avg_sq: RGBA16F (is_float32 = 0)
// or RGBA32F (1). Window taps outside the image read zero and still count
// (robust-access imageLoad); min(t, 1) of a NaN deviation is 1, the GPU's
// IEEE minNum. out: 8-bit, alpha 255.
int oracle_bfr_blend(int W, int H, int radius, int is_float32, const void* avg, const void* avg_sq,
                     const uint8_t* den8, const uint8_t* den16, const uint8_t* den32, uint8_t* out, int threads) {
  auto load = [&](const void* im, int x, int y) {
    const size_t p = (size_t)y * W + x;
    if (is_float32) {
      const float* f = (const float*)im + 4 * p;
      return vec3{f[0], f[1], f[2]};
    }
    const uint16_t* h = (const uint16_t*)im + 4 * p;
    return vec3{h2f(h[0]), h2f(h[1]), h2f(h[2])};
  };
  auto lum = [](vec3 c) {
    const float k = 1.0f / 3.0f;
    return (c.x * k + c.y * k) + c.z * k;
  };
  auto mix3 = [](float a, float b, float c, float t) {
    const float mid = .5f, max_dev = 1.f;
    t = t / max_dev;
    t = std::fmin(t, 1.f);
    const float af = std::fmax(1.0f - (t / mid), 0.f);
    const float bf = (t < mid) ? t / mid : 1.f - (t - mid) / (1.0f - mid);
    const float cf = (1.0f - af) - bf;
    return (af * a + bf * b) + cf * c;
  };
  parallel_for(H, [&](int y) {
    for (int x = 0; x < W; ++x) {
      float sq = 0.f, av = 0.f;
      int count = 0;
      for (int dy = -radius; dy <= radius; ++dy)
        for (int dx = -radius; dx <= radius; ++dx) {
          const int sx = x + dx, sy = y + dy;
          const bool in = sx >= 0 && sy >= 0 && sx < W && sy < H;
          const float cur = in ? lum(load(avg, sx, sy)) : 0.f;
          ++count;
          const float w = 1.0f / (float)count;
          sq = mix(sq, cur * cur, w);
          av = mix(av, cur, w);
        }
      av = mix(av, lum(load(avg, x, y)), .5f);
      sq = mix(sq, lum(load(avg_sq, x, y)), .5f);
      const float sd = std::sqrt(sq - av * av);
      const size_t p = 4 * ((size_t)y * W + x);
      for (int c = 0; c < 3; ++c)
        out[p + c] = f2u8(mix3(u82f(den32[p + c]), u82f(den16[p + c]), u82f(den8[p + c]), sd));
      out[p + 3] = 255;
    }
  }, threads);
  return 0;
}

// Known-answer helpers for the tests.
float oracle_bmfr_random(uint32_t a) { return bmfr_random(a); }
uint16_t oracle_f2h(float f) { return f2h(f); }
float oracle_h2f(uint16_t h) { return h2f(h); }
int oracle_mirror(int x, int s) { return mirror1(x, s); }

}  // extern "C"
