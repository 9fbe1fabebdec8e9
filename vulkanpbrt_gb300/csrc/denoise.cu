// Accumulator, BMFR and BFR on sm_103a.
//
// accumulator.comp  -> accumulate_kernel      (one thread per pixel)
// bmfrPre/Fit/Post  -> bmfr_fused_kernel      (one CTA per block: features,
//                      Householder fit and output without an HBM round trip)
// bfr.comp          -> bfr_kernel             (one CTA per block)
//
// This translation unit is compiled with -fmad=false: the reference shaders'
// arithmetic is restated operation by operation, and none of these kernels is
// bound by FP32 issue, so contraction would only move results away from the
// shader rounding.
#include <cuda.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <new>

#include "device_common.cuh"
#include "internal.hpp"

namespace pbrt {

// shaders/bmfrGeneral.comp:36
__constant__ float c_bmfr_offsets[16][2] = {
    {.7f, .85f}, {.95f, .5f}, {.43f, .76f}, {.97f, .03f}, {.37f, .58f}, {.03f, .36f}, {.81f, .46f}, {0.f, .78f},
    {.36f, -.08f}, {-.06f, 0.f}, {.95f, .1f}, {.85f, .61f}, {.06f, .1f}, {.43f, .16f}, {0.f, .5f}, {.73f, .38f}};
// shaders/bfr.comp:92
__constant__ int c_bfr_offsets[16][2] = {{-7, -11}, {-14, -8}, {-5, -12}, {-15, -1}, {-5, -9},  {-1, -4},
                                         {-14, -7}, {0, -13},  {-5, -1},  {-1, 0},   {-15, -2}, {-14, -10},
                                         {-1, -1},  {-6, -3},  {0, -8},   {-10, -4}};

constexpr unsigned kFull = 0xffffffffu;

// ---------------------------------------------------------------------------
// Accumulator (shaders/accumulator.comp:33-105).
struct AccKernelParams {
  Mat4 view, inverse_view, proj_prev_view, prev_view;
  float4 prev_origin;
  uint32_t frame;
  int separate;
  int W, H;
};

__global__ void accumulate_kernel(AccKernelParams p, const float4* __restrict__ src_f32,
                                  const Half4* __restrict__ src_f16, const float* __restrict__ depth,
                                  const float* __restrict__ prev_depth, const uint8_t* __restrict__ prev_spp,
                                  const Half4* __restrict__ prev_output, __half2* __restrict__ motion,
                                  uint8_t* __restrict__ spp, Half4* __restrict__ illum) {
  int x = blockIdx.x * blockDim.x + threadIdx.x;
  int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= p.W || y >= p.H) return;
  const int W = p.W, H = p.H;
  size_t idx = (size_t)y * W + x;
  bool reprojected = false;
  float pixel_spp = 1.f / 256.f;
  float d = depth[idx];
  float4 pp, prev_pos;
  if (p.separate) {
    float4 pos = p.inverse_view.c[3];
    pos.w = 1.f;
    float cx = ((float)x + .5f) / (float)W * 2.f - 1.f;
    float cy = ((float)y + .5f) / (float)H * 2.f - 1.f;
    float4 dir = mul(p.view, make_float4(cx, cy, 1.f, 1.f));
    float3 nd = normalize(f3(dir.x, dir.y, dir.z));
    dir = mul(p.inverse_view, make_float4(nd.x, nd.y, nd.z, 0.f));
    pp = make_float4(pos.x + dir.x * d, pos.y + dir.y * d, pos.z + dir.z * d, pos.w + dir.w * d);
    prev_pos = mul(p.proj_prev_view, pp);
  } else {
    float4 org = p.inverse_view.c[2];
    org = make_float4(org.x / org.w, org.y / org.w, org.z / org.w, org.w / org.w);
    float cx = ((float)x + .5f) / (float)W * 2.f - 1.f;
    float cy = ((float)y + .5f) / (float)H * 2.f - 1.f;
    float4 cd = mul(p.inverse_view, make_float4(cx, cy, 1.f, 1.f));
    float wd = cd.w + 1e-9f;
    cd = make_float4(cd.x / wd, cd.y / wd, cd.z / wd, cd.w / wd);
    float4 df = make_float4(cd.x - org.x, cd.y - org.y, cd.z - org.z, cd.w - org.w);
    float len = sqrtf(df.x * df.x + df.y * df.y + df.z * df.z + df.w * df.w);
    cd = make_float4(-(df.x / len), -(df.y / len), -(df.z / len), -(df.w / len));
    pp = make_float4(org.x + cd.x * d, org.y + cd.y * d, org.z + cd.z * d, org.w + cd.w * d);
    prev_pos = mul(p.prev_view, pp);
  }
  float pre_depth = length(f3(pp.x - p.prev_origin.x, pp.y - p.prev_origin.y, pp.z - p.prev_origin.z));
  float pw = prev_pos.w;
  prev_pos = make_float4(prev_pos.x / pw, prev_pos.y / pw, prev_pos.z / pw, prev_pos.w / pw);
  float u = (prev_pos.x + 1.f) * .5f * ((float)W / ((float)W - .5f));
  float v = (prev_pos.y + 1.f) * .5f * ((float)H / ((float)H - .5f));
  float3 prev_color = f3(0.f);
  if (p.frame > 0) {
    float4 pd = bilinear(W, H, u, v, [&](int i, int j) {
      return make_float4(prev_depth[(size_t)j * W + i], 0.f, 0.f, 0.f);
    });
    float dissim = (pd.x / pre_depth) - 1.f;
    if (u >= 0.f && v >= 0.f && u <= 1.f && v <= 1.f && fabsf(dissim) <= .01f) {
      reprojected = true;
      float4 c = bilinear(W, H, u, v, [&](int i, int j) { return load_half4(prev_output + (size_t)j * W + i); });
      prev_color = f3(c.x, c.y, c.z);
      float4 s = bilinear(W, H, u, v, [&](int i, int j) {
        return make_float4(u82f(prev_spp[(size_t)j * W + i]), 0.f, 0.f, 0.f);
      });
      pixel_spp += s.x;
    }
  }
  motion[idx] = reprojected ? __floats2half2_rn(u, v) : __floats2half2_rn(-1.f, -1.f);
  spp[idx] = f2u8(pixel_spp);
  float3 demod;
  if (src_f32) {
    float4 s = src_f32[idx];
    demod = f3(s.x, s.y, s.z);
  } else {
    float4 s = load_half4(src_f16 + idx);
    demod = f3(s.x, s.y, s.z);
  }
  if (reprojected) {
    float a = fmaxf(1.f / (pixel_spp * 256.f), .1f);
    demod = mix3(prev_color, demod, a);
  }
  store_half4(illum + idx, demod.x, demod.y, demod.z, 1.f);
}

// ---------------------------------------------------------------------------
// Shared tail of bmfrPost / bfr (shaders/bmfrPost.comp:194-214,
// shaders/bfr.comp:289-308): clamp, temporal blend with the previous denoised
// layer at the motion uv, store to the other layer, remodulate and tone map.
struct PostArgs {
  const __half2* motion;
  const uint8_t* spp;
  const uint8_t* albedo;  // RGBA8
  Half4* denoised;        // 2 layers
  uchar4* final_bgra;
  int W, H;
  uint32_t frame;
};

PBRT_D void post_store(const PostArgs& a, float3 dc, int ix, int iy) {
  const int W = a.W, H = a.H;
  size_t p = (size_t)iy * W + ix;
  size_t layer = (size_t)W * H;
  dc = clamp3(dc, 0.f, 10.f);
  float2 uv = __half22float2(a.motion[p]);
  bool accept = uv.x >= 0.f;
  float pixel_spp = u82f(a.spp[p]) * 256.f;
  float3 prev = f3(0.f);
  float alpha = 1.f;
  if (a.frame > 0 && accept) {
    const Half4* src = a.denoised + (size_t)(a.frame & 1) * layer;
    float4 s = bilinear(W, H, uv.x, uv.y, [&](int i, int j) { return load_half4(src + (size_t)j * W + i); });
    prev = prev + f3(s.x, s.y, s.z);
    alpha = fmaxf(1.f / pixel_spp, 0.1f);
  }
  dc = alpha * dc + (1.f - alpha) * prev;
  store_half4(a.denoised + (size_t)((a.frame & 1) ^ 1) * layer + p, dc.x, dc.y, dc.z, 1.f);
  uchar4 al = reinterpret_cast<const uchar4*>(a.albedo)[p];
  float3 alb = f3(u82f(al.x) + 1e-6f, u82f(al.y) + 1e-6f, u82f(al.z) + 1e-6f);
  float3 t = fmax3(f3(0.f), alb * dc);
  float3 tm = f3(powf(t.x, .454545f), powf(t.y, .454545f), powf(t.z, .454545f));
  tm = clamp3(tm, 0.f, 1.f);
  a.final_bgra[p] = make_uchar4(f2u8(tm.z), f2u8(tm.y), f2u8(tm.x), 255);
}

// Warp transpose-reduction: each lane starts with N partial values; after
// log2(32) xor-butterfly levels lane L holds the warp total of value
// (L >> (5 - log2 N)) -- every total is the same pairwise tree a full
// xor-butterfly builds, at N-1 shuffles instead of 5N.
template <int N> PBRT_D void warp_transpose_reduce(float (&v)[N], int lane) {
  static_assert(N == 32 || N == 16, "N must be 16 or 32");
  int half = N / 2;
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    if (half >= 1) {
      bool upper = (lane & o) != 0;
#pragma unroll
      for (int j = 0; j < N / 2; ++j) {
        if (j < half) {
          float keep = upper ? v[j + half] : v[j];
          float send = upper ? v[j] : v[j + half];
          v[j] = keep + __shfl_xor_sync(kFull, send, o);
        }
      }
      half >>= 1;
    } else {
      v[0] = v[0] + __shfl_xor_sync(kFull, v[0], o);
    }
  }
}

// bmfrGeneral.comp:103-113
PBRT_D float bmfr_random(uint32_t a) {
  a = (a + 0x7ed55d16u) + (a << 12);
  a = (a ^ 0xc761c23cu) ^ (a >> 19);
  a = (a + 0x165667b1u) + (a << 5);
  a = (a + 0xd3a2646cu) ^ (a << 9);
  a = (a + 0xfd7046c5u) + (a << 3);
  a = (a ^ 0xb55a4f09u) ^ (a >> 16);
  return __uint2float_rn(a) / 4294967296.f;
}

// ---------------------------------------------------------------------------
// BMFR: bmfrPre + bmfrFit + bmfrPost for one BW x BW block per CTA.
struct BmfrParams {
  Mat4 inv_view, inv_proj;
  int W, H, gw, gh;
  uint32_t frame;
  int position_type;
  int fp64_resolve;
  float cond_limit;  // R-diagonal ratio above which a block is re-solved in FP64
  const float* depth;
  const float2* normal;
  const Half4* noisy_f16;
  const float4* noisy_f32;
  float* weights;  // 30 layers x gh x gw
  uint32_t* flagged;  // [0] = count, [1] = largest R-diagonal ratio (float bits), [2..] = block ids to re-solve
  uint32_t* last_layer;  // device word: the denoised layer this dispatch writes (null: not recorded)
  PostArgs post;
};

template <int BW> struct BmfrShape {
  static constexpr int P = BW * BW;
  static constexpr int NT = BW == 8 ? 64 : 256;
  static constexpr int SV = P / NT;
  static constexpr int NW = NT / 32;
  static constexpr int PAD = P + P / 32;  // one spare word per 32 rows: conflict-free transpose
};

// Block min/max of K values per thread across the CTA (warp butterfly, then
// one partial per warp in shared memory read back by every thread).
template <int K, int NW>
PBRT_D void block_minmax(float (&mn)[K], float (&mx)[K], float* red, int warp, int lane) {
#pragma unroll
  for (int k = 0; k < K; ++k) {
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
      mn[k] = fminf(mn[k], __shfl_xor_sync(kFull, mn[k], o));
      mx[k] = fmaxf(mx[k], __shfl_xor_sync(kFull, mx[k], o));
    }
  }
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      red[warp * 2 * K + k] = mn[k];
      red[warp * 2 * K + K + k] = mx[k];
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < K; ++k) {
    float a = red[k], b = red[K + k];
    for (int w = 1; w < NW; ++w) {
      a = fminf(a, red[w * 2 * K + k]);
      b = fmaxf(b, red[w * 2 * K + K + k]);
    }
    mn[k] = a;
    mx[k] = b;
  }
}

PBRT_D float3 bmfr_world_dir(const BmfrParams& p, int ix, int iy) {
  float cx = ((float)ix + .5f) / (float)p.W * 2.f - 1.f;
  float cy = ((float)iy + .5f) / (float)p.H * 2.f - 1.f;
  float4 vsd = mul(p.inv_proj, make_float4(cx, cy, 1.f, 1.f));
  float3 n = normalize(f3(vsd.x, vsd.y, vsd.z));
  float4 wsd = mul(p.inv_view, make_float4(n.x, n.y, n.z, 0.f));
  return f3(wsd.x, wsd.y, wsd.z);
}

template <int BW>
__global__ void __launch_bounds__(BmfrShape<BW>::NT, BW == 8 ? 8 : 3) bmfr_fused_kernel(BmfrParams p) {
  using S = BmfrShape<BW>;
  constexpr int NT = S::NT, SV = S::SV, NW = S::NW, P = S::P;
  extern __shared__ float smem[];
  float* fq = smem;                                     // [13][PAD] quantised + noised features
  float(*red)[NW][16] = reinterpret_cast<float(*)[NW][16]>(fq + 13 * S::PAD);  // [2 buffers][NW][16]
  float(*rowc)[16] = reinterpret_cast<float(*)[16]>(fq + 13 * S::PAD + 2 * NW * 16);  // [2][16]
  float(*Rm)[13] = reinterpret_cast<float(*)[13]>(fq + 13 * S::PAD + 2 * NW * 16 + 32);  // [10][13]
  float* wsm = fq + 13 * S::PAD + 2 * NW * 16 + 32 + 130;                               // [30]
  float(*mmred)[6] = reinterpret_cast<float(*)[6]>(wsm + 32);                          // [NW][6]
  float(*redS)[NW] = reinterpret_cast<float(*)[NW]>(wsm + 32 + NW * 6);                  // [2][NW]

  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int gx = blockIdx.x, gy = blockIdx.y;
  if (p.last_layer && gx == 0 && gy == 0 && t == 0) *p.last_layer = (p.frame & 1u) ^ 1u;
  const int offx = (int)((float)BW * c_bmfr_offsets[p.frame % 16][0]);
  const int offy = (int)((float)BW * c_bmfr_offsets[p.frame % 16][1]);
  const float EPS = 1e-6f;

  // ---- phase 1: load (coalesced: q = t + s*NT, lx = q % BW, ly = q / BW) --
  float3 nor[SV], pos[SV], noisy[SV];
  int ixs[SV], iys[SV];
  bool inside[SV];
#pragma unroll
  for (int s = 0; s < SV; ++s) {
    int q = t + s * NT, lx = q % BW, ly = q / BW;
    int ax = gx * BW + lx - offx, ay = gy * BW + ly - offy;
    int ix = mirror1(ax, p.W), iy = mirror1(ay, p.H);
    ixs[s] = ix;
    iys[s] = iy;
    inside[s] = (ax == ix && ay == iy);
    size_t pi = (size_t)iy * p.W + ix;
    float d = p.depth[pi];
    float2 nn = p.normal[pi];
    nor[s] = decode_normal(nn.x, nn.y);
    float4 c = p.noisy_f16 ? load_half4(p.noisy_f16 + pi) : p.noisy_f32[pi];
    noisy[s] = f3(c.x, c.y, c.z);
    if (p.position_type == 2) {
      float3 o = f3(p.inv_view.c[3].x, p.inv_view.c[3].y, p.inv_view.c[3].z);
      // inverseViewMatrix * vec4(0,0,0,1) is column 3.
      pos[s] = o + bmfr_world_dir(p, ix, iy) * d;
    } else {
      pos[s] = f3(0.f, 0.f, d);
    }
  }
  // ---- block normalisation of the position features (bmfrPre.comp:38-76) --
  if (p.position_type == 2) {
    float mn[3], mx[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      float a = k == 0 ? pos[0].x : (k == 1 ? pos[0].y : pos[0].z);
      mn[k] = a;
      mx[k] = a;
#pragma unroll
      for (int s = 1; s < SV; ++s) {
        float b = k == 0 ? pos[s].x : (k == 1 ? pos[s].y : pos[s].z);
        mn[k] = fminf(mn[k], b);
        mx[k] = fmaxf(mx[k], b);
      }
    }
    block_minmax<3, NW>(mn, mx, &mmred[0][0], warp, lane);
#pragma unroll
    for (int s = 0; s < SV; ++s) {
      float3 v = pos[s];
      v.x = (v.x - mn[0]) / (mx[0] - mn[0] + EPS);
      v.y = (v.y - mn[1]) / (mx[1] - mn[1] + EPS);
      v.z = (v.z - mn[2]) / (mx[2] - mn[2] + EPS);
      pos[s] = v;
    }
  } else {
    float mn[1] = {pos[0].z}, mx[1] = {pos[0].z};
#pragma unroll
    for (int s = 1; s < SV; ++s) {
      mn[0] = fminf(mn[0], pos[s].z);
      mx[0] = fmaxf(mx[0], pos[s].z);
    }
    block_minmax<1, NW>(mn, mx, &mmred[0][0], warp, lane);
#pragma unroll
    for (int s = 0; s < SV; ++s) {
      int q = t + s * NT, lx = q % BW, ly = q / BW;
      float z = pos[s].z;
      z -= mn[0];
      z /= mx[0] - mn[0] + EPS;
      if (p.position_type == 0) {
        pos[s] = f3((float)lx / ((float)BW - 1.f), (float)ly / ((float)BW - 1.f), z);
      } else {
        pos[s] = bmfr_world_dir(p, ixs[s], iys[s]) * z;
      }
    }
  }
  // ---- quantised (R16F) features + hash noise into shared memory ----------
  // Fit row r of pixel (lx, ly) is r = lx * BW + ly (bmfrFit.comp:18-19).
#pragma unroll
  for (int s = 0; s < SV; ++s) {
    int q = t + s * NT, lx = q % BW, ly = q / BW;
    int r = lx * BW + ly;
    int ri = r + r / 32;
    float3 n = nor[s], ps = pos[s];
    float f[13] = {1.f, n.x, n.y, n.z, ps.x, ps.y, ps.z, ps.x * ps.x, ps.y * ps.y, ps.z * ps.z,
                   noisy[s].x, noisy[s].y, noisy[s].z};
#pragma unroll
    for (int c = 0; c < 13; ++c) {
      float v = __half2float(__float2half_rn(f[c]));
      if (c < 10) {
        uint32_t h = (uint32_t)r + (uint32_t)c * (uint32_t)P * (uint32_t)P + p.frame * 13u * (uint32_t)P * (uint32_t)P;
        v = v + (1e-4f * 2.f) * (bmfr_random(h) - .5f);
      }
      fq[c * S::PAD + ri] = v;
    }
  }
  __syncthreads();

  // ---- phase 2: Householder QR (bmfrFit.comp:26-69), rows r = t + s*NT ----
  float X[SV][13];
#pragma unroll
  for (int s = 0; s < SV; ++s) {
    int r = t + s * NT, ri = r + r / 32;
#pragma unroll
    for (int c = 0; c < 13; ++c) X[s][c] = fq[c * S::PAD + ri];
  }
  // The staging area is dead now: park each pixel's decoded normal and
  // normalised position there until the output pass (keeps them out of
  // registers during the QR).
  __syncthreads();
#pragma unroll
  for (int s = 0; s < SV; ++s) {
    int q = t + s * NT;
    fq[0 * P + q] = nor[s].x;
    fq[1 * P + q] = nor[s].y;
    fq[2 * P + q] = nor[s].z;
    fq[3 * P + q] = pos[s].x;
    fq[4 * P + q] = pos[s].y;
    fq[5 * P + q] = pos[s].z;
  }
  float ulen2 = 0.f;
#pragma unroll
  for (int col = 0; col < 10; ++col) {
    const int buf = col & 1;
    // (1) squared length of the column below the diagonal, summed per thread
    // in row order, then a 32-lane xor butterfly, then warps in order -- the
    // order the oracle restates (bmfrFit.comp:28-36).
    float sp = 0.f;
#pragma unroll
    for (int s = 0; s < SV; ++s) {
      int r = t + s * NT;
      if (r > col) sp = sp + X[s][col] * X[s][col];
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) sp = sp + __shfl_xor_sync(kFull, sp, o);
    if (lane == 0) redS[buf][warp] = sp;
    if (t == col) {
#pragma unroll
      for (int f = 0; f < 13; ++f) rowc[buf][f] = X[0][f];
    }
    __syncthreads();
    float S2 = redS[buf][0];
    for (int w = 1; w < NW; ++w) S2 = S2 + redS[buf][w];
    const float xcc = rowc[buf][col];
    const float vlen = sqrtf(S2 + xcc * xcc);  // bmfrFit.comp:41-44
    const float ucol = xcc - vlen;
    ulen2 = S2 + ucol * ucol;
    // (2) v_f = sum over rows r >= col of x_f * u (bmfrFit.comp:53-61),
    // all trailing columns in one transpose reduction.
    float v[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = 0.f;
#pragma unroll
    for (int s = 0; s < SV; ++s) {
      int r = t + s * NT;
      if (r >= col) {
        float u = (r == col) ? ucol : X[s][col];
#pragma unroll
        for (int f = 0; f < 13; ++f)
          if (f > col) v[f] = v[f] + X[s][f] * u;
      }
    }
    warp_transpose_reduce<16>(v, lane);
    if ((lane & 1) == 0 && (lane >> 1) < 13) red[buf][warp][lane >> 1] = v[0];
    __syncthreads();
    float tot = 0.f;
    if (lane < 13) {
      tot = red[buf][0][lane];
      for (int w = 1; w < NW; ++w) tot = tot + red[buf][w][lane];
    }
    // (3) reflect the trailing columns (bmfrFit.comp:62-67); the shader's
    // division by |u|^2 is a product with its reciprocal (Vulkan allows
    // 2.5 ULP for x / y).
    const float rl = 1.f / ulen2;
#pragma unroll
    for (int f = 0; f < 13; ++f) {
      const float vf = __shfl_sync(kFull, tot, f);
      if (f > col) {
#pragma unroll
        for (int s = 0; s < SV; ++s) {
          int r = t + s * NT;
          if (r >= col) {
            float u = (r == col) ? ucol : X[s][col];
            X[s][f] = X[s][f] - 2.f * u * vf * rl;
          }
        }
      }
    }
    if (t == col) {
#pragma unroll
      for (int f = 0; f < 13; ++f) Rm[col][f] = (f == col) ? vlen : (f > col ? X[0][f] : 0.f);
    }
  }
  __syncthreads();
  // ---- back substitution (bmfrFit.comp:71-81) and weight store -----------
  if (t < 3) {
    float ws[10];
#pragma unroll
    for (int i = 9; i >= 0; --i) {
      float b = Rm[i][10 + t];
#pragma unroll
      for (int x = i + 1; x < 10; ++x) b = b - ws[x] * Rm[i][x];
      ws[i] = b / Rm[i][i];
    }
    size_t L = (size_t)p.gw * p.gh, bidx = (size_t)gy * p.gw + gx;
#pragma unroll
    for (int i = 0; i < 10; ++i) {
      float w = (ulen2 == 0.f) ? .2f : ws[i];
      wsm[i * 3 + t] = w;
      p.weights[(size_t)(i * 3 + t) * L + bidx] = w;
    }
  }
  if (p.fp64_resolve && t == 0) {
    float dmax = 0.f, dmin = INFINITY;
#pragma unroll
    for (int i = 0; i < 10; ++i) {
      float a = fabsf(Rm[i][i]);
      dmax = fmaxf(dmax, a);
      dmin = fminf(dmin, a);
    }
    const float ratio = dmax <= 3.0e38f * dmin ? dmax / dmin : INFINITY;  // dmin = 0 or NaN: infinite
    atomicMax(p.flagged + 1, __float_as_uint(ratio));  // non-negative floats order as their bits
    if (!(dmax <= p.cond_limit * dmin)) {
      uint32_t slot = atomicAdd(p.flagged, 1u);
      p.flagged[2 + slot] = (uint32_t)(gy * p.gw + gx);
    }
  }
  __syncthreads();
  // ---- phase 3: weighted sum + temporal blend (bmfrPost.comp:164-214) -----
  float w[30];
#pragma unroll
  for (int i = 0; i < 30; ++i) {
    float a = wsm[i];
    w[i] = (isinf(a) || isnan(a)) ? 0.f : a;
  }
#pragma unroll
  for (int s = 0; s < SV; ++s) {
    const int q = t + s * NT, lx = q % BW, ly = q / BW;
    const int ax = gx * BW + lx - offx, ay = gy * BW + ly - offy;
    const int ix = mirror1(ax, p.W), iy = mirror1(ay, p.H);
    if (ax != ix || ay != iy) continue;
    float3 n = f3(fq[0 * P + q], fq[1 * P + q], fq[2 * P + q]);
    float3 ps = f3(fq[3 * P + q], fq[4 * P + q], fq[5 * P + q]);
    float f[10] = {1.f, n.x, n.y, n.z, ps.x, ps.y, ps.z, ps.x * ps.x, ps.y * ps.y, ps.z * ps.z};
    float3 dc = f3(0.f);
#pragma unroll
    for (int i = 0; i < 10; ++i) dc = dc + f3(w[i * 3], w[i * 3 + 1], w[i * 3 + 2]) * f[i];
    post_store(p.post, dc, ix, iy);
  }
}

// FP64 re-solve of flagged blocks: recompute the block's quantised features,
// Householder QR in FP64 in shared memory, then redo the block's output.
// No reference counterpart (the reference keeps the FP32 solution).
template <int BW>
__global__ void __launch_bounds__(256) bmfr_fp64_kernel(BmfrParams p) {
  constexpr int P = BW * BW, NT = 256;
  extern __shared__ double dsm[];
  double* A = dsm;                 // [13][P]
  double* red = dsm + 13 * P;      // [NT/32][14]
  __shared__ float wsm[30];
  __shared__ float mm[2];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const uint32_t nflag = p.flagged[0];
  for (uint32_t k = blockIdx.x; k < nflag; k += gridDim.x) {
    const int bid = (int)p.flagged[2 + k];
    const int gx = bid % p.gw, gy = bid / p.gw;
    const int offx = (int)((float)BW * c_bmfr_offsets[p.frame % 16][0]);
    const int offy = (int)((float)BW * c_bmfr_offsets[p.frame % 16][1]);
    const float EPS = 1e-6f;
    // Depth (or world position) range of the block.
    float lmn[3] = {INFINITY, INFINITY, INFINITY}, lmx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int q = t; q < P; q += NT) {
      int lx = q % BW, ly = q / BW;
      int ix = mirror1(gx * BW + lx - offx, p.W), iy = mirror1(gy * BW + ly - offy, p.H);
      float d = p.depth[(size_t)iy * p.W + ix];
      float3 ps = f3(0.f, 0.f, d);
      if (p.position_type == 2) ps = f3(p.inv_view.c[3].x, p.inv_view.c[3].y, p.inv_view.c[3].z) + bmfr_world_dir(p, ix, iy) * d;
      lmn[0] = fminf(lmn[0], ps.x); lmx[0] = fmaxf(lmx[0], ps.x);
      lmn[1] = fminf(lmn[1], ps.y); lmx[1] = fmaxf(lmx[1], ps.y);
      lmn[2] = fminf(lmn[2], ps.z); lmx[2] = fmaxf(lmx[2], ps.z);
    }
    float (*mmr)[6] = reinterpret_cast<float(*)[6]>(red);
    block_minmax<3, NT / 32>(lmn, lmx, &mmr[0][0], warp, lane);
    __syncthreads();
    for (int q = t; q < P; q += NT) {
      int lx = q % BW, ly = q / BW;
      int ix = mirror1(gx * BW + lx - offx, p.W), iy = mirror1(gy * BW + ly - offy, p.H);
      size_t pi = (size_t)iy * p.W + ix;
      float d = p.depth[pi];
      float2 nn = p.normal[pi];
      float3 n = decode_normal(nn.x, nn.y);
      float3 ps;
      if (p.position_type == 2) {
        ps = f3(p.inv_view.c[3].x, p.inv_view.c[3].y, p.inv_view.c[3].z) + bmfr_world_dir(p, ix, iy) * d;
        ps.x = (ps.x - lmn[0]) / (lmx[0] - lmn[0] + EPS);
        ps.y = (ps.y - lmn[1]) / (lmx[1] - lmn[1] + EPS);
        ps.z = (ps.z - lmn[2]) / (lmx[2] - lmn[2] + EPS);
      } else {
        float z = (d - lmn[2]) / (lmx[2] - lmn[2] + EPS);
        ps = p.position_type == 0 ? f3((float)lx / ((float)BW - 1.f), (float)ly / ((float)BW - 1.f), z)
                                  : bmfr_world_dir(p, ix, iy) * z;
      }
      float4 c = p.noisy_f16 ? load_half4(p.noisy_f16 + pi) : p.noisy_f32[pi];
      float f[13] = {1.f, n.x, n.y, n.z, ps.x, ps.y, ps.z, ps.x * ps.x, ps.y * ps.y, ps.z * ps.z, c.x, c.y, c.z};
      int r = lx * BW + ly;
      for (int cc = 0; cc < 13; ++cc) {
        float v = __half2float(__float2half_rn(f[cc]));
        if (cc < 10) {
          uint32_t h = (uint32_t)r + (uint32_t)cc * (uint32_t)P * (uint32_t)P + p.frame * 13u * (uint32_t)P * (uint32_t)P;
          v = v + (1e-4f * 2.f) * (bmfr_random(h) - .5f);
        }
        A[cc * P + r] = (double)v;
      }
    }
    __syncthreads();
    double ulen2 = 0.0;
    for (int col = 0; col < 10; ++col) {
      double part[14];
      for (int i = 0; i < 14; ++i) part[i] = 0.0;
      for (int r = t; r < P; r += NT) {
        if (r <= col) continue;
        double xc = A[col * P + r];
        part[13] += xc * xc;
        for (int f = col + 1; f < 13; ++f) part[f] += A[f * P + r] * xc;
      }
      for (int i = 0; i < 14; ++i)
        for (int o = 16; o >= 1; o >>= 1) part[i] += __shfl_xor_sync(kFull, part[i], o);
      if (lane == 0)
        for (int i = 0; i < 14; ++i) red[warp * 14 + i] = part[i];
      __syncthreads();
      double tot[14];
      for (int i = 0; i < 14; ++i) {
        tot[i] = 0.0;
        for (int w = 0; w < NT / 32; ++w) tot[i] += red[w * 14 + i];
      }
      double xcc = A[col * P + col];
      double vlen = sqrt(tot[13] + xcc * xcc);
      double ucol = xcc - vlen;
      ulen2 = tot[13] + ucol * ucol;
      double vf[13];
      for (int f = 0; f < 13; ++f) vf[f] = (f > col) ? (tot[f] + A[f * P + col] * ucol) / ulen2 : 0.0;
      __syncthreads();  // row col is read above by every thread before its owner updates it
      for (int r = t; r < P; r += NT) {
        if (r < col) continue;
        double u = (r == col) ? ucol : A[col * P + r];
        for (int f = col + 1; f < 13; ++f) A[f * P + r] -= 2.0 * u * vf[f];
      }
      __syncthreads();
      if (t == 0) A[col * P + col] = vlen;
      __syncthreads();
    }
    if (t < 3) {
      double ws[10];
      for (int i = 9; i >= 0; --i) {
        double b = A[(10 + t) * P + i];
        for (int x = i + 1; x < 10; ++x) b -= ws[x] * A[x * P + i];
        ws[i] = b / A[i * P + i];
      }
      size_t L = (size_t)p.gw * p.gh, bidx = (size_t)gy * p.gw + gx;
      for (int i = 0; i < 10; ++i) {
        float w = (ulen2 == 0.0) ? .2f : (float)ws[i];
        wsm[i * 3 + t] = w;
        p.weights[(size_t)(i * 3 + t) * L + bidx] = w;
      }
    }
    __syncthreads();
    for (int q = t; q < P; q += NT) {
      int lx = q % BW, ly = q / BW;
      int ax = gx * BW + lx - offx, ay = gy * BW + ly - offy;
      int ix = mirror1(ax, p.W), iy = mirror1(ay, p.H);
      if (ax != ix || ay != iy) continue;
      size_t pi = (size_t)iy * p.W + ix;
      float d = p.depth[pi];
      float2 nn = p.normal[pi];
      float3 n = decode_normal(nn.x, nn.y);
      float3 ps;
      if (p.position_type == 2) {
        ps = f3(p.inv_view.c[3].x, p.inv_view.c[3].y, p.inv_view.c[3].z) + bmfr_world_dir(p, ix, iy) * d;
        ps.x = (ps.x - lmn[0]) / (lmx[0] - lmn[0] + EPS);
        ps.y = (ps.y - lmn[1]) / (lmx[1] - lmn[1] + EPS);
        ps.z = (ps.z - lmn[2]) / (lmx[2] - lmn[2] + EPS);
      } else {
        float z = (d - lmn[2]) / (lmx[2] - lmn[2] + EPS);
        ps = p.position_type == 0 ? f3((float)lx / ((float)BW - 1.f), (float)ly / ((float)BW - 1.f), z)
                                  : bmfr_world_dir(p, ix, iy) * z;
      }
      float f[10] = {1.f, n.x, n.y, n.z, ps.x, ps.y, ps.z, ps.x * ps.x, ps.y * ps.y, ps.z * ps.z};
      float3 dc = f3(0.f);
      for (int i = 0; i < 10; ++i) {
        float a = wsm[i * 3], b = wsm[i * 3 + 1], c = wsm[i * 3 + 2];
        a = (isinf(a) || isnan(a)) ? 0.f : a;
        b = (isinf(b) || isnan(b)) ? 0.f : b;
        c = (isinf(c) || isnan(c)) ? 0.f : c;
        dc = dc + f3(a, b, c) * f[i];
      }
      post_store(p.post, dc, ix, iy);
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// BFR (shaders/bfr.comp:202-309), one BW x BH block per CTA, thread t owns
// local pixel (t % BW, t / BW) -- the shader's gl_LocalInvocationIndex, so
// warps are its 32-wide subgroups.
struct BfrParams {
  int W, H;
  uint32_t frame;
  const float* depth;
  const float2* normal;
  const Half4* noisy_f16;
  const float4* noisy_f32;
  PostArgs post;
};

template <int BW, int BH>
__global__ void __launch_bounds__(BW * BH) bfr_kernel(BfrParams p) {
  constexpr int NT = BW * BH, NW = NT / 32, ASZ = 7;
  constexpr int NSTOP = (32 + BW - 1) / BW < ASZ ? (32 + BW - 1) / BW : ASZ;
  __shared__ float red[2][NW][32];
  __shared__ float mmred[NW][2];
  __shared__ int lred[NW];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int lx = t % BW, ly = t / BW;
  const int ax = blockIdx.x * BW + lx + c_bfr_offsets[p.frame % 16][0];
  const int ay = blockIdx.y * BH + ly + c_bfr_offsets[p.frame % 16][1];
  const int ix = mirror1(ax, p.W), iy = mirror1(ay, p.H);
  const bool inside = (ax == ix && ay == iy);
  const size_t pi = (size_t)iy * p.W + ix;
  float4 c4 = p.noisy_f16 ? load_half4(p.noisy_f16 + pi) : p.noisy_f32[pi];
  const float3 col = f3(c4.x, c4.y, c4.z);
  float d = p.depth[pi];
  float2 nn = p.normal[pi];
  const float3 n = decode_normal(nn.x, nn.y);
  const float spp = u82f(p.post.spp[pi]) * 256.f;
  const int l1 = spp >= 10.f ? 1 : 0;
  // depth range and the block's L1 count
  float mn[1] = {d}, mx[1] = {d};
  int lc = l1;
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) lc += __shfl_xor_sync(kFull, lc, o);
  if (lane == 0) lred[warp] = lc;
  block_minmax<1, NW>(mn, mx, &mmred[0][0], warp, lane);
  int l1sum = 0;
#pragma unroll
  for (int w = 0; w < NW; ++w) l1sum += lred[w];
  d = d - mn[0];
  d = d / (mx[0] - mn[0] + 1e-8f);
  d = d * 2.f - 1.f;
  const float f[ASZ] = {1.f, (float)lx / ((float)BW - 1.f) - 0.5f, (float)ly / ((float)BH - 1.f) - 0.5f, d, n.x, n.y, n.z};

  float alpha[3 * ASZ];
#pragma unroll
  for (int i = 0; i < 3 * ASZ; ++i) alpha[i] = 0.f;
  float m_l = 0.f, v_l = 0.f, a_l = 0.f;  // Adam state of slot `lane` (= feature*3 + channel)
  const float l1r = (float)l1sum * 1.0f / (float)NT;
  const float lr = l1r * 1.1f + (1.f - l1r) * .863f;
  const float b1 = l1r * .45f + (1.f - l1r) * .3f;
  const float b2 = l1r * .75f + (1.f - l1r) * .7314f;
#pragma unroll 1
  for (int it = 0; it < 40; ++it) {
    float3 c = f3(0.f);
#pragma unroll
    for (int j = 0; j < ASZ; ++j) c = c + f[j] * f3(alpha[3 * j], alpha[3 * j + 1], alpha[3 * j + 2]);
    c = col - c;
    if (l1) {
      c.x = c.x > 0.f ? 1.f : (c.x < 0.f ? -1.f : 0.f);
      c.y = c.y > 0.f ? 1.f : (c.y < 0.f ? -1.f : 0.f);
      c.z = c.z > 0.f ? 1.f : (c.z < 0.f ? -1.f : 0.f);
    }
    float v[32];
#pragma unroll
    for (int j = 0; j < ASZ; ++j) {
      v[3 * j] = f[j] * c.x;
      v[3 * j + 1] = f[j] * c.y;
      v[3 * j + 2] = f[j] * c.z;
    }
#pragma unroll
    for (int j = 3 * ASZ; j < 32; ++j) v[j] = 0.f;
    warp_transpose_reduce<32>(v, lane);
    const int buf = it & 1;
    red[buf][warp][lane] = v[0];
    __syncthreads();
    float delta = red[buf][0][lane];
#pragma unroll
    for (int w = 1; w < NW; ++w) delta = delta + red[buf][w][lane];
    const float tt = (float)(it + 1);
    const float step = lr * expf(-.116f * tt) * sqrtf(1.f - powf(.7314f, tt)) / (1.f - powf(.3f, tt));
    m_l = b1 * m_l + (1.f - .3f) * delta;
    float ad = fabsf(delta);
    v_l = b2 * v_l + (1.f - .7314f) * (ad * ad);
    a_l = a_l + step * (m_l / (sqrtf(v_l) + 1e-8f));
#pragma unroll
    for (int i = 0; i < 3 * ASZ; ++i) alpha[i] = __shfl_sync(kFull, a_l, i);
    const bool stop = __any_sync(kFull, lane < 3 * NSTOP && isnan(delta));
    if (stop) break;
  }
  if (!inside) return;
  float3 dc = f3(0.f);
#pragma unroll
  for (int j = 0; j < ASZ; ++j) dc = dc + f[j] * f3(alpha[3 * j], alpha[3 * j + 1], alpha[3 * j + 2]);
  post_store(p.post, dc, ix, iy);
}

// ---------------------------------------------------------------------------
// Host-side matrix helpers (column-major, FP32 products in GLSL order; the
// inverse by cofactors in FP64).
static void mat_mul(const float* a, const float* b, float* out) {
  float r[16];
  for (int c = 0; c < 4; ++c)
    for (int row = 0; row < 4; ++row)
      r[c * 4 + row] = a[0 * 4 + row] * b[c * 4 + 0] + a[1 * 4 + row] * b[c * 4 + 1] + a[2 * 4 + row] * b[c * 4 + 2] +
                       a[3 * 4 + row] * b[c * 4 + 3];
  memcpy(out, r, sizeof(r));
}

static bool mat_inverse(const float* in, float* out) {
  double a[4][4];  // a[row][col]
  for (int c = 0; c < 4; ++c)
    for (int r = 0; r < 4; ++r) a[r][c] = in[c * 4 + r];
  double inv[4][4] = {{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}};
  // Gauss-Jordan with partial pivoting.
  for (int c = 0; c < 4; ++c) {
    int piv = c;
    for (int r = c + 1; r < 4; ++r)
      if (fabs(a[r][c]) > fabs(a[piv][c])) piv = r;
    if (a[piv][c] == 0.0) return false;
    for (int k = 0; k < 4; ++k) {
      std::swap(a[c][k], a[piv][k]);
      std::swap(inv[c][k], inv[piv][k]);
    }
    double d = a[c][c];
    for (int k = 0; k < 4; ++k) {
      a[c][k] /= d;
      inv[c][k] /= d;
    }
    for (int r = 0; r < 4; ++r) {
      if (r == c) continue;
      double f = a[r][c];
      for (int k = 0; k < 4; ++k) {
        a[r][k] -= f * a[c][k];
        inv[r][k] -= f * inv[c][k];
      }
    }
  }
  for (int c = 0; c < 4; ++c)
    for (int r = 0; r < 4; ++r) out[c * 4 + r] = (float)inv[r][c];
  return true;
}

static Mat4 to_mat4(const float* m) {
  Mat4 r;
  for (int c = 0; c < 4; ++c) r.c[c] = make_float4(m[4 * c], m[4 * c + 1], m[4 * c + 2], m[4 * c + 3]);
  return r;
}

static size_t bmfr_smem_bytes(int bw) {
  int P = bw * bw, NT = bw == 8 ? 64 : 256, NW = NT / 32;
  int pad = P + P / 32;
  return sizeof(float) * (size_t)(13 * pad + 2 * NW * 16 + 32 + 130 + 32 + NW * 6 + 2 * NW);
}

}  // namespace pbrt

using namespace pbrt;

PbrtAccumulator::~PbrtAccumulator() {
  release(gbuffer);
  release(source);
  release(accumulated);
  release(acc);
}
PbrtBMFR::~PbrtBMFR() {
  denoised.free_();
  final_image.free_();
  weights.free_();
  flags.free_();
  release(gbuffer);
  release(illumination);
  release(acc);
}
PbrtBFR::~PbrtBFR() {
  denoised.free_();
  final_image.free_();
  release(gbuffer);
  release(illumination);
  release(acc);
}

template <int BW> static int launch_bmfr(PbrtBMFR* b, const BmfrParams& kp, pbrt_stream_t stream) {
  size_t smem = bmfr_smem_bytes(BW);
  static PerDeviceOnce attrs;
  int ast = once_per_device(attrs, [&]() -> int {
    PBRT_CUDA(cudaFuncSetAttribute(bmfr_fused_kernel<BW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    PBRT_CUDA(cudaFuncSetAttribute(bmfr_fp64_kernel<BW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)(sizeof(double) * (13 * BW * BW + 8 * 14))));
    return PBRT_OK;
  });
  if (ast) return ast;
  dim3 grid(kp.gw, kp.gh);
  bmfr_fused_kernel<BW><<<grid, BmfrShape<BW>::NT, smem, stream>>>(kp);
  int st = check_launch("bmfr_fused_kernel");
  if (st) return st;
  if (kp.fp64_resolve) {
    bmfr_fp64_kernel<BW><<<152, 256, sizeof(double) * (13 * BW * BW + 8 * 14), stream>>>(kp);
    st = check_launch("bmfr_fp64_kernel");
  }
  return st;
}

extern "C" {

PBRT_API int pbrt_accumulator_create(PbrtGBuffer* g, PbrtIlluminationBuffer* illumination, int32_t separate_matrices,
                                     int32_t work_width, int32_t work_height, PbrtAccumulator** out) {
  if (!out) return fail(PBRT_ERROR_INVALID_ARGUMENT, "accumulator: null output");
  *out = nullptr;
  if (!checked<PbrtGBuffer>(g, Kind::GBuffer) || !checked<PbrtIlluminationBuffer>(illumination, Kind::Illumination))
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "accumulator: bad GBuffer or IlluminationBuffer handle");
  if (g->width != illumination->width || g->height != illumination->height)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "accumulator: GBuffer and illumination sizes differ");
  PbrtFormat f = (PbrtFormat)illumination->images[0].view.format;
  if (f != PBRT_FORMAT_R32G32B32A32_SFLOAT && f != PBRT_FORMAT_R16G16B16A16_SFLOAT)
    return fail(PBRT_ERROR_UNSUPPORTED, "accumulator: source image 0 must be RGBA32F or RGBA16F");
  if (work_width <= 0 || work_height <= 0 || work_width * work_height > 1024)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "accumulator: bad work group %dx%d", work_width, work_height);
  auto* a = new (std::nothrow) PbrtAccumulator();
  if (!a) return fail(PBRT_ERROR_OUT_OF_MEMORY, "accumulator: host allocation");
  a->separate = separate_matrices != 0;
  a->work_w = work_width;
  a->work_h = work_height;
  a->gbuffer = g;
  retain(g);
  a->source = illumination;
  retain(illumination);
  int st = pbrt_illumination_buffer_create(PBRT_ILLUMINATION_DEMODULATED, g->width, g->height, &a->accumulated);
  if (!st) st = pbrt_accumulation_buffer_create(g->width, g->height, &a->acc);
  if (st) {
    delete a;
    return st;
  }
  *out = a;
  return PBRT_OK;
}

PBRT_API int pbrt_accumulator_set_camera_matrices(PbrtAccumulator* a, int32_t frame_index,
                                                  const PbrtCameraMatrices* cur, const PbrtCameraMatrices* prev) {
  if (!checked<PbrtAccumulator>(a, Kind::Accumulator) || !cur || !prev)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "set_camera_matrices: bad arguments");
  AccumulatorParams& p = a->params;
  if (a->separate) {
    if (!cur->has_proj)
      return fail(PBRT_ERROR_INVALID_ARGUMENT,
                  "Accumulator::set_camera_matrices: created with separate matrices, but the current "
                  "CameraMatrices has no proj / inv_proj");
    memcpy(p.view, cur->inv_proj, 64);
    memcpy(p.inverse_view, cur->inv_view, 64);
    if (frame_index != 0) {
      memcpy(p.prev_view, prev->view, 64);
      float inv[16];
      if (!mat_inverse(prev->view, inv)) return fail(PBRT_ERROR_INVALID_ARGUMENT, "prev.view is singular");
      p.prev_origin[0] = inv[12];
      p.prev_origin[1] = inv[13];
      p.prev_origin[2] = inv[14];
      p.prev_origin[3] = 1.f;
    }
    if (!mat_inverse(p.view, p.proj)) return fail(PBRT_ERROR_INVALID_ARGUMENT, "inv_proj is singular");
  } else {
    memcpy(p.view, cur->view, 64);
    memcpy(p.inverse_view, cur->inv_view, 64);
    if (frame_index != 0) {
      memcpy(p.prev_view, prev->view, 64);
      float w = prev->inv_view[11];
      for (int i = 0; i < 4; ++i) p.prev_origin[i] = prev->inv_view[8 + i] / w;
    }
  }
  p.frame_number = (uint32_t)frame_index;
  return PBRT_OK;
}

PBRT_API int pbrt_accumulator_dispatch(PbrtAccumulator* a, pbrt_stream_t stream) {
  if (!checked<PbrtAccumulator>(a, Kind::Accumulator)) return fail(PBRT_ERROR_INVALID_ARGUMENT, "not an Accumulator");
  const AccumulatorParams& hp = a->params;
  AccKernelParams kp;
  kp.view = to_mat4(hp.view);
  kp.inverse_view = to_mat4(hp.inverse_view);
  kp.prev_view = to_mat4(hp.prev_view);
  float ppv[16];
  mat_mul(hp.proj, hp.prev_view, ppv);
  kp.proj_prev_view = to_mat4(ppv);
  kp.prev_origin = make_float4(hp.prev_origin[0], hp.prev_origin[1], hp.prev_origin[2], hp.prev_origin[3]);
  kp.frame = hp.frame_number;
  kp.separate = a->separate ? 1 : 0;
  kp.W = (int)a->gbuffer->width;
  kp.H = (int)a->gbuffer->height;
  const DeviceImage& src = a->source->images[0];
  bool f32 = src.view.format == PBRT_FORMAT_R32G32B32A32_SFLOAT;
  dim3 block(a->work_w, a->work_h);
  dim3 grid((kp.W + a->work_w - 1) / a->work_w, (kp.H + a->work_h - 1) / a->work_h);
  accumulate_kernel<<<grid, block, 0, stream>>>(
      kp, f32 ? src.ptr<float4>() : nullptr, f32 ? nullptr : src.ptr<Half4>(), a->gbuffer->depth.ptr<float>(),
      a->acc->prev_depth.ptr<float>(), a->acc->prev_spp.ptr<uint8_t>(), a->acc->prev_illu.ptr<Half4>(),
      a->acc->motion.ptr<__half2>(), a->acc->spp.ptr<uint8_t>(), a->accumulated->images[0].ptr<Half4>());
  return check_launch("accumulate_kernel");
}

PBRT_API int pbrt_accumulator_get_accumulated_illumination(PbrtAccumulator* a, PbrtIlluminationBuffer** out) {
  if (!checked<PbrtAccumulator>(a, Kind::Accumulator) || !out) return fail(PBRT_ERROR_INVALID_ARGUMENT, "bad arguments");
  *out = a->accumulated;
  return PBRT_OK;
}

PBRT_API int pbrt_accumulator_get_accumulation_buffer(PbrtAccumulator* a, PbrtAccumulationBuffer** out) {
  if (!checked<PbrtAccumulator>(a, Kind::Accumulator) || !out) return fail(PBRT_ERROR_INVALID_ARGUMENT, "bad arguments");
  *out = a->acc;
  return PBRT_OK;
}

static int denoiser_inputs_ok(const char* who, uint32_t w, uint32_t h, PbrtGBuffer* g,
                              PbrtIlluminationBuffer* illumination, PbrtAccumulationBuffer* acc) {
  if (!checked<PbrtGBuffer>(g, Kind::GBuffer) || !checked<PbrtIlluminationBuffer>(illumination, Kind::Illumination) ||
      !checked<PbrtAccumulationBuffer>(acc, Kind::Accumulation))
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "%s: bad GBuffer / IlluminationBuffer / AccumulationBuffer handle", who);
  if (illumination->type != PBRT_ILLUMINATION_DEMODULATED && illumination->type != PBRT_ILLUMINATION_DEMODULATED_FLOAT)
    return fail(PBRT_ERROR_UNSUPPORTED,
                "%s: Illumination Buffer type is required to be IlluminationBufferDemodulated/Float", who);
  if (g->width != w || g->height != h || illumination->width != w || illumination->height != h || acc->width != w ||
      acc->height != h)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "%s: buffer sizes differ from %ux%u", who, w, h);
  return PBRT_OK;
}

PBRT_API int pbrt_bmfr_create(uint32_t width, uint32_t height, uint32_t work_width, uint32_t work_height,
                              PbrtGBuffer* g, PbrtIlluminationBuffer* illumination, PbrtAccumulationBuffer* acc,
                              uint32_t fitting_kernel, PbrtBMFR** out) {
  if (!out) return fail(PBRT_ERROR_INVALID_ARGUMENT, "bmfr: null output");
  *out = nullptr;
  int st = denoiser_inputs_ok("BMFR", width, height, g, illumination, acc);
  if (st) return st;
  if (work_width != work_height || (work_width != 8 && work_width != 16 && work_width != 32))
    return fail(PBRT_ERROR_UNSUPPORTED, "BMFR: work size %ux%u (supported: 8x8, 16x16, 32x32)", work_width, work_height);
  // The fit's reduction grouping is its invocation count: DenoiserUtils.cpp
  // uses 64 invocations for 8x8 blocks and 256 otherwise (BMFR.hpp:19).
  uint32_t want_k = work_width == 8 ? 64u : 256u;
  if (fitting_kernel != want_k)
    return fail(PBRT_ERROR_UNSUPPORTED, "BMFR: fitting kernel %u for %ux%u blocks (supported: %u)", fitting_kernel,
                work_width, work_height, want_k);
  if (width < 2 * work_width + 2 || height < 2 * work_height + 2)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "BMFR: image %ux%u smaller than the mirror padding allows (>= %u)",
                width, height, 2 * work_width + 2);
  auto* b = new (std::nothrow) PbrtBMFR();
  if (!b) return fail(PBRT_ERROR_OUT_OF_MEMORY, "bmfr: host allocation");
  b->width = width;
  b->height = height;
  b->bw = work_width;
  b->fitting_kernel = fitting_kernel;
  b->gbuffer = g;
  retain(g);
  b->illumination = illumination;
  retain(illumination);
  b->acc = acc;
  retain(acc);
  uint32_t gw = width / work_width + 2, gh = height / work_height + 2;
  if ((st = b->denoised.alloc(width, height, 2, PBRT_FORMAT_R16G16B16A16_SFLOAT)) ||
      (st = b->final_image.alloc(width, height, 1, PBRT_FORMAT_B8G8R8A8_UNORM)) ||
      (st = b->weights.alloc(gw, gh, 30, PBRT_FORMAT_R32_SFLOAT)) ||
      (st = b->flags.alloc(gw * gh + 3, 1, 1, PBRT_FORMAT_R32_SFLOAT))) {
    delete b;
    return st;
  }
  b->counter = b->flags.ptr<uint32_t>();
  b->last_layer = b->counter + gw * gh + 2;
  *out = b;
  return PBRT_OK;
}

PBRT_API int pbrt_bmfr_set_options(PbrtBMFR* b, int32_t position_type, int32_t fp64_resolve) {
  if (!checked<PbrtBMFR>(b, Kind::BMFR)) return fail(PBRT_ERROR_INVALID_ARGUMENT, "not a BMFR");
  if (position_type < 0 || position_type > 2)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "BMFR: POSITION_TYPE %d (0 depth, 1 world/depth-norm, 2 world)",
                position_type);
  b->position_type = position_type;
  b->fp64_resolve = fp64_resolve ? 1 : 0;
  return PBRT_OK;
}

PBRT_API int pbrt_bmfr_dispatch(PbrtBMFR* b, const PbrtPushConstants* pc, pbrt_stream_t stream) {
  if (!checked<PbrtBMFR>(b, Kind::BMFR) || !pc) return fail(PBRT_ERROR_INVALID_ARGUMENT, "bmfr_dispatch: bad arguments");
  BmfrParams kp;
  kp.inv_view = to_mat4(pc->view_inverse);
  kp.inv_proj = to_mat4(pc->proj_inverse);
  kp.W = (int)b->width;
  kp.H = (int)b->height;
  kp.gw = (int)(b->width / b->bw + 2);
  kp.gh = (int)(b->height / b->bw + 2);
  kp.frame = pc->frame_number;
  kp.position_type = b->position_type;
  kp.fp64_resolve = b->fp64_resolve;
  kp.cond_limit = b->cond_limit;
  kp.depth = b->gbuffer->depth.ptr<float>();
  kp.normal = b->gbuffer->normal.ptr<float2>();
  const DeviceImage& noisy = b->illumination->images[0];
  bool f32 = noisy.view.format == PBRT_FORMAT_R32G32B32A32_SFLOAT;
  kp.noisy_f16 = f32 ? nullptr : noisy.ptr<Half4>();
  kp.noisy_f32 = f32 ? noisy.ptr<float4>() : nullptr;
  kp.weights = b->weights.ptr<float>();
  kp.flagged = b->counter;
  kp.last_layer = b->last_layer;
  kp.post.motion = b->acc->motion.ptr<__half2>();
  kp.post.spp = b->acc->spp.ptr<uint8_t>();
  kp.post.albedo = b->gbuffer->albedo.ptr<uint8_t>();
  kp.post.denoised = b->denoised.ptr<Half4>();
  kp.post.final_bgra = b->final_image.ptr<uchar4>();
  kp.post.W = kp.W;
  kp.post.H = kp.H;
  kp.post.frame = kp.frame;
  if (b->fp64_resolve) PBRT_CUDA(cudaMemsetAsync(b->counter, 0, 2 * sizeof(uint32_t), stream));
  switch (b->bw) {
    case 8: return launch_bmfr<8>(b, kp, stream);
    case 16: return launch_bmfr<16>(b, kp, stream);
    default: return launch_bmfr<32>(b, kp, stream);
  }
}

PBRT_API int pbrt_bmfr_final_image(const PbrtBMFR* b, PbrtImage* out) {
  if (!checked<const PbrtBMFR>((void*)b, Kind::BMFR) || !out) return fail(PBRT_ERROR_INVALID_ARGUMENT, "bad arguments");
  *out = b->final_image.view;
  return PBRT_OK;
}

PBRT_API int pbrt_bmfr_images(const PbrtBMFR* b, PbrtImage* denoised, PbrtImage* weights) {
  if (!checked<const PbrtBMFR>((void*)b, Kind::BMFR)) return fail(PBRT_ERROR_INVALID_ARGUMENT, "not a BMFR");
  if (denoised) *denoised = b->denoised.view;
  if (weights) *weights = b->weights.view;
  return PBRT_OK;
}

PBRT_API int pbrt_bmfr_fp64_block_count(PbrtBMFR* b, pbrt_stream_t stream, uint32_t* count) {
  if (!checked<PbrtBMFR>(b, Kind::BMFR) || !count) return fail(PBRT_ERROR_INVALID_ARGUMENT, "bad arguments");
  *count = 0;
  if (!b->fp64_resolve) return PBRT_OK;
  PBRT_CUDA(cudaMemcpyAsync(count, b->counter, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
  PBRT_CUDA(cudaStreamSynchronize(stream));
  return PBRT_OK;
}

PBRT_API int pbrt_bmfr_set_condition_limit(PbrtBMFR* b, float limit) {
  if (!checked<PbrtBMFR>(b, Kind::BMFR)) return fail(PBRT_ERROR_INVALID_ARGUMENT, "not a BMFR");
  if (!(limit >= 1.f) || !std::isfinite(limit))
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "BMFR: condition limit %g (finite, >= 1)", (double)limit);
  b->cond_limit = limit;
  return PBRT_OK;
}

PBRT_API int pbrt_bmfr_condition_stats(PbrtBMFR* b, pbrt_stream_t stream, uint32_t* flagged, float* max_ratio) {
  if (!checked<PbrtBMFR>(b, Kind::BMFR) || !flagged || !max_ratio)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "bad arguments");
  *flagged = 0;
  *max_ratio = 0.f;
  if (!b->fp64_resolve) return fail(PBRT_ERROR_INVALID_ARGUMENT, "BMFR: condition statistics need fp64_resolve");
  uint32_t w[2];
  PBRT_CUDA(cudaMemcpyAsync(w, b->counter, sizeof(w), cudaMemcpyDeviceToHost, stream));
  PBRT_CUDA(cudaStreamSynchronize(stream));
  *flagged = w[0];
  std::memcpy(max_ratio, &w[1], sizeof(float));
  return PBRT_OK;
}

PBRT_API int pbrt_bfr_create(uint32_t width, uint32_t height, uint32_t work_width, uint32_t work_height,
                             PbrtGBuffer* g, PbrtIlluminationBuffer* illumination, PbrtAccumulationBuffer* acc,
                             PbrtBFR** out) {
  if (!out) return fail(PBRT_ERROR_INVALID_ARGUMENT, "bfr: null output");
  *out = nullptr;
  int st = denoiser_inputs_ok("BFR", width, height, g, illumination, acc);
  if (st) return st;
  if (work_width != work_height || (work_width != 8 && work_width != 16 && work_width != 32))
    return fail(PBRT_ERROR_UNSUPPORTED, "BFR: work size %ux%u (supported: 8x8, 16x16, 32x32)", work_width, work_height);
  uint32_t minw = 2 * work_width > 16 ? 2 * work_width : 16;
  if (width < minw || height < minw)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "BFR: image %ux%u smaller than the mirror padding allows (>= %u)", width,
                height, minw);
  auto* b = new (std::nothrow) PbrtBFR();
  if (!b) return fail(PBRT_ERROR_OUT_OF_MEMORY, "bfr: host allocation");
  b->width = width;
  b->height = height;
  b->bw = work_width;
  b->bh = work_height;
  b->gbuffer = g;
  retain(g);
  b->illumination = illumination;
  retain(illumination);
  b->acc = acc;
  retain(acc);
  if ((st = b->denoised.alloc(width, height, 2, PBRT_FORMAT_R16G16B16A16_SFLOAT)) ||
      (st = b->final_image.alloc(width, height, 1, PBRT_FORMAT_B8G8R8A8_UNORM))) {
    delete b;
    return st;
  }
  *out = b;
  return PBRT_OK;
}

PBRT_API int pbrt_bfr_dispatch(PbrtBFR* b, const PbrtPushConstants* pc, pbrt_stream_t stream) {
  if (!checked<PbrtBFR>(b, Kind::BFR) || !pc) return fail(PBRT_ERROR_INVALID_ARGUMENT, "bfr_dispatch: bad arguments");
  BfrParams kp;
  kp.W = (int)b->width;
  kp.H = (int)b->height;
  kp.frame = pc->frame_number;
  kp.depth = b->gbuffer->depth.ptr<float>();
  kp.normal = b->gbuffer->normal.ptr<float2>();
  const DeviceImage& noisy = b->illumination->images[0];
  bool f32 = noisy.view.format == PBRT_FORMAT_R32G32B32A32_SFLOAT;
  kp.noisy_f16 = f32 ? nullptr : noisy.ptr<Half4>();
  kp.noisy_f32 = f32 ? noisy.ptr<float4>() : nullptr;
  kp.post.motion = b->acc->motion.ptr<__half2>();
  kp.post.spp = b->acc->spp.ptr<uint8_t>();
  kp.post.albedo = b->gbuffer->albedo.ptr<uint8_t>();
  kp.post.denoised = b->denoised.ptr<Half4>();
  kp.post.final_bgra = b->final_image.ptr<uchar4>();
  kp.post.W = kp.W;
  kp.post.H = kp.H;
  kp.post.frame = kp.frame;
  dim3 grid(b->width / b->bw + 2, b->height / b->bh + 2);
  switch (b->bw) {
    case 8: bfr_kernel<8, 8><<<grid, 64, 0, stream>>>(kp); break;
    case 16: bfr_kernel<16, 16><<<grid, 256, 0, stream>>>(kp); break;
    default: bfr_kernel<32, 32><<<grid, 1024, 0, stream>>>(kp); break;
  }
  return check_launch("bfr_kernel");
}

PBRT_API int pbrt_bfr_final_image(const PbrtBFR* b, PbrtImage* out) {
  if (!checked<const PbrtBFR>((void*)b, Kind::BFR) || !out) return fail(PBRT_ERROR_INVALID_ARGUMENT, "bad arguments");
  *out = b->final_image.view;
  return PBRT_OK;
}

PBRT_API int pbrt_bfr_images(const PbrtBFR* b, PbrtImage* denoised) {
  if (!checked<const PbrtBFR>((void*)b, Kind::BFR)) return fail(PBRT_ERROR_INVALID_ARGUMENT, "not a BFR");
  if (denoised) *denoised = b->denoised.view;
  return PBRT_OK;
}

}  // extern "C"

// ===========================================================================
// BMFR without device allocation.
//
// Some callers cannot call cudaMalloc: a host engine or compositor that owns
// the device-memory budget and hands plugins only the images they work on,
// per-frame code that must not run into the device-wide synchronisation
// cudaMalloc / cudaFree can cause, or code that runs while its stream is being
// captured. For them the fit's per-block weights -- the only memory the fused
// kernel needs beyond its inputs and outputs -- live in the file-scope array
// below, which every GPU that loads this library holds until the process
// exits (kNoAllocMaxBlocks * 30 floats = 1.9 MiB).
namespace pbrt {
constexpr uint32_t kNoAllocMaxBlocks = PBRT_BMFR_NOALLOC_MAX_BLOCKS;
static __device__ __align__(256) float g_bmfr_noalloc_weights[kNoAllocMaxBlocks * 30];

// Device address of g_bmfr_noalloc_weights for each device, resolved with
// that device current (host code cannot use the symbol itself), together
// with the id of the context it was resolved in: after cudaDeviceReset the
// device's next context loads the module anew, so the address and the
// kernel attributes are resolved again.
typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);
static std::mutex g_noalloc_mutex;
static float* g_noalloc_ptr[kMaxDevices] = {nullptr};
static unsigned long long g_noalloc_ctx[kMaxDevices] = {0};

// Unique id of the calling thread's current context (0 if unavailable).
static unsigned long long current_context_id() {
  static const std::pair<CtxGetCurrentFn, CtxGetIdFn> fns = []() {
    void* a = nullptr;
    void* b = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
        q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      return std::pair<CtxGetCurrentFn, CtxGetIdFn>(nullptr, nullptr);
    }
    return std::pair<CtxGetCurrentFn, CtxGetIdFn>((CtxGetCurrentFn)a, (CtxGetIdFn)b);
  }();
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (!fns.first || !fns.second || fns.first(&ctx) != CUDA_SUCCESS || !ctx || fns.second(ctx, &id) != CUDA_SUCCESS)
    return 0;
  return id;
}

static int noalloc_weights(float** out) {
  int dev = 0;
  PBRT_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(PBRT_ERROR_UNSUPPORTED, "BMFR no-alloc: device ordinal %d", dev);
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev] || current_context_id() != g_noalloc_ctx[dev]) {
    void* p = nullptr;
    // (also makes the device's primary context current on a thread's first call)
    cudaError_t e = cudaGetSymbolAddress(&p, g_bmfr_noalloc_weights);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_bmfr_noalloc_weights)");
    for (int bw : {8, 16, 32}) {  // shared-memory opt-in of the kernel this entry point launches
      size_t smem = bmfr_smem_bytes(bw);
      cudaError_t a = bw == 8    ? cudaFuncSetAttribute(bmfr_fused_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
                      : bw == 16 ? cudaFuncSetAttribute(bmfr_fused_kernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
                                 : cudaFuncSetAttribute(bmfr_fused_kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (a != cudaSuccess) return cuda_fail(a, "cudaFuncSetAttribute(bmfr_fused_kernel)");
    }
    g_noalloc_ptr[dev] = static_cast<float*>(p);
    g_noalloc_ctx[dev] = current_context_id();
  }
  *out = g_noalloc_ptr[dev];
  return PBRT_OK;
}
}  // namespace pbrt

extern "C" PBRT_API int pbrt_bmfr_dispatch_noalloc(uint32_t width, uint32_t height, uint32_t block_size,
                                                   int32_t position_type, const PbrtBmfrNoAllocImages* im,
                                                   const PbrtPushConstants* pc, pbrt_stream_t stream) {
  using namespace pbrt;
  if (!im || !pc || !im->depth || !im->normal || !im->albedo || !im->noisy || !im->motion || !im->spp ||
      !im->denoised || !im->final_bgra)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "BMFR no-alloc: null image pointer or push constants");
  {
    // the kernel reads noisy / denoised as 8-byte half4, normal as float2, motion
    // as half2, depth as float and albedo / final as 4-byte texels
    const struct { const void* p; unsigned align; const char* name; } req[] = {
        {im->noisy, 8, "noisy"}, {im->denoised, 8, "denoised"}, {im->normal, 8, "normal"}, {im->depth, 4, "depth"},
        {im->motion, 4, "motion"}, {im->albedo, 4, "albedo"}, {im->final_bgra, 4, "final_bgra"}};
    for (const auto& r : req)
      if (reinterpret_cast<uintptr_t>(r.p) % r.align)
        return fail(PBRT_ERROR_INVALID_ARGUMENT, "BMFR no-alloc: %s pointer %p is not %u-byte aligned", r.name, r.p,
                    r.align);
  }
  if (block_size != 8 && block_size != 16 && block_size != 32)
    return fail(PBRT_ERROR_UNSUPPORTED, "BMFR no-alloc: block size %u (supported: 8, 16, 32)", block_size);
  if (position_type < 0 || position_type > 2)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "BMFR no-alloc: POSITION_TYPE %d", position_type);
  if (width < 2 * block_size + 2 || height < 2 * block_size + 2)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "BMFR no-alloc: image %ux%u smaller than the mirror padding allows",
                width, height);
  const uint64_t gw = width / block_size + 2, gh = height / block_size + 2;
  if (gw * gh > kNoAllocMaxBlocks)
    return fail(PBRT_ERROR_INVALID_ARGUMENT,
                "BMFR no-alloc: %ux%u with %ux%u blocks needs %llu blocks of weight scratch, above the fixed maximum "
                "of %u (use pbrt_bmfr_create / pbrt_bmfr_dispatch, or larger blocks)",
                width, height, block_size, block_size, (unsigned long long)(gw * gh), kNoAllocMaxBlocks);
  float* weights = nullptr;
  int st = noalloc_weights(&weights);
  if (st) return st;
  BmfrParams kp;
  kp.inv_view = to_mat4(pc->view_inverse);
  kp.inv_proj = to_mat4(pc->proj_inverse);
  kp.W = (int)width;
  kp.H = (int)height;
  kp.gw = (int)gw;
  kp.gh = (int)gh;
  kp.frame = pc->frame_number;
  kp.position_type = position_type;
  kp.fp64_resolve = 0;
  kp.depth = im->depth;
  kp.normal = reinterpret_cast<const float2*>(im->normal);
  kp.noisy_f16 = reinterpret_cast<const Half4*>(im->noisy);
  kp.noisy_f32 = nullptr;
  kp.weights = weights;  // every block writes all 30 of its weights before reading them back
  kp.flagged = nullptr;
  kp.last_layer = nullptr;
  kp.post.motion = reinterpret_cast<const __half2*>(im->motion);
  kp.post.spp = im->spp;
  kp.post.albedo = im->albedo;
  kp.post.denoised = reinterpret_cast<Half4*>(im->denoised);
  kp.post.final_bgra = reinterpret_cast<uchar4*>(im->final_bgra);
  kp.post.W = kp.W;
  kp.post.H = kp.H;
  kp.post.frame = kp.frame;
  dim3 grid((unsigned)gw, (unsigned)gh);
  switch (block_size) {
    case 8: bmfr_fused_kernel<8><<<grid, BmfrShape<8>::NT, bmfr_smem_bytes(8), stream>>>(kp); break;
    case 16: bmfr_fused_kernel<16><<<grid, BmfrShape<16>::NT, bmfr_smem_bytes(16), stream>>>(kp); break;
    default: bmfr_fused_kernel<32><<<grid, BmfrShape<32>::NT, bmfr_smem_bytes(32), stream>>>(kp); break;
  }
  return check_launch("bmfr_fused_kernel (no-alloc)");
}
