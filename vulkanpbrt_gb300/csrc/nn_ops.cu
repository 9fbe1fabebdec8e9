// Non-convolution operators of the kernel-predicting denoiser (FP32 on the
// CUDA cores): input features from the G-buffer, 2x2 pooling, the backward
// helpers of the U-Net (ReLU mask, bias gradient, concat split and upsample
// sum), the multi-scale kernel-prediction heads, the relMSE loss and Adam.
// No reference counterpart: the reference's denoisers are BMFR and BFR.
#include <cuda_bf16.h>

#include <cstdint>

#include "device_common.cuh"
#include "internal.hpp"

namespace pbrt {
namespace nn {

typedef __nv_bfloat16 bf16;
constexpr int kKP = 25;  // 5x5 kernel taps

#define GRID_STRIDE(i, n) for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < (n); i += (long)gridDim.x * blockDim.x)

// Network input (16 BF16 channels at the padded size PH x PW; edge pixels
// replicated): log1p(illumination rgb), albedo rgb, normal xyz (decoded from
// the G-buffer's spherical angles), log1p(depth) / 8, samples per pixel
// (min(spp, 16) / 16, from the accumulation buffer's R8 spp image in the
// accumulator's 1/256 steps; one sample without it), zeros. Also the
// illumination the kernel-prediction heads filter (FP32 rgb), clamped to
// [0, 10] as BMFR clamps its output (shaders/bmfrPost.comp:99).
constexpr float kRadianceClamp = 10.f;
__global__ void features_kernel(const float4* __restrict__ illum32, const Half4* __restrict__ illum16,
                                const uchar4* __restrict__ albedo, const float2* __restrict__ normal,
                                const float* __restrict__ depth, const uint8_t* __restrict__ spp, int W, int H, int PW,
                                int PH, int n_img, bf16* __restrict__ feat, float* __restrict__ rad) {
  const long total = (long)n_img * PH * PW;
  GRID_STRIDE(i, total) {
    const int x = (int)(i % PW), y = (int)((i / PW) % PH), n = (int)(i / ((long)PW * PH));
    const int sx = min(x, W - 1), sy = min(y, H - 1);
    const size_t p = ((size_t)n * H + sy) * W + sx;
    float4 c = illum32 ? illum32[p] : load_half4(illum16 + p);
    c.x = fminf(fmaxf(c.x, 0.f), kRadianceClamp);
    c.y = fminf(fmaxf(c.y, 0.f), kRadianceClamp);
    c.z = fminf(fmaxf(c.z, 0.f), kRadianceClamp);
    const uchar4 a = albedo[p];
    const float2 th = normal[p];
    const float3 nn3 = decode_normal(th.x, th.y);
    const float s = spp ? fminf((float)spp[p] / 255.f * 256.f, 16.f) / 16.f : 1.f / 16.f;
    float f[16] = {log1pf(c.x), log1pf(c.y), log1pf(c.z), a.x / 255.f, a.y / 255.f, a.z / 255.f, nn3.x, nn3.y,
                   nn3.z, log1pf(fmaxf(depth[p], 0.f)) * 0.125f, s, 0, 0, 0, 0, 0};
    bf16* o = feat + i * 16;
#pragma unroll
    for (int k = 0; k < 16; k += 2) *reinterpret_cast<__nv_bfloat162*>(o + k) = __floats2bfloat162_rn(f[k], f[k + 1]);
    rad[i * 3 + 0] = c.x;
    rad[i * 3 + 1] = c.y;
    rad[i * 3 + 2] = c.z;
  }
}

__global__ void avgpool2_bf16_kernel(const bf16* __restrict__ src, bf16* __restrict__ dst, int n_img, int H, int W,
                                     int C) {
  const int H2 = H / 2, W2 = W / 2;
  const long total = (long)n_img * H2 * W2 * (C / 2);
  GRID_STRIDE(i, total) {
    const int c = (int)(i % (C / 2)) * 2;
    const long q = i / (C / 2);
    const int x = (int)(q % W2), yy = (int)((q / W2) % H2), n = (int)(q / ((long)W2 * H2));
    float2 s = make_float2(0.f, 0.f);
#pragma unroll
    for (int d = 0; d < 4; ++d) {
      const size_t p = (((size_t)n * H + 2 * yy + (d >> 1)) * W + 2 * x + (d & 1)) * C + c;
      float2 v = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(src + p));
      s.x += v.x;
      s.y += v.y;
    }
    *reinterpret_cast<__nv_bfloat162*>(dst + q * C + c) = __floats2bfloat162_rn(0.25f * s.x, 0.25f * s.y);
  }
}

__global__ void avgpool2_f32_kernel(const float* __restrict__ src, float* __restrict__ dst, int n_img, int H, int W,
                                    int C) {
  const int H2 = H / 2, W2 = W / 2;
  const long total = (long)n_img * H2 * W2 * C;
  GRID_STRIDE(i, total) {
    const int c = (int)(i % C);
    const long q = i / C;
    const int x = (int)(q % W2), yy = (int)((q / W2) % H2), n = (int)(q / ((long)W2 * H2));
    float s = 0.f;
#pragma unroll
    for (int d = 0; d < 4; ++d) s += src[(((size_t)n * H + 2 * yy + (d >> 1)) * W + 2 * x + (d & 1)) * C + c];
    dst[i] = 0.25f * s;
  }
}

// dx[2i+a][2j+b] += dy[i][j] / 4   (FP32)
__global__ void avgpool2_bwd_add_kernel(const float* __restrict__ dy, float* __restrict__ dx, int n_img, int H, int W,
                                        int C) {
  const long total = (long)n_img * H * W * C;
  GRID_STRIDE(i, total) {
    const int c = (int)(i % C);
    const long p = i / C;
    const int x = (int)(p % W), y = (int)((p / W) % H), n = (int)(p / ((long)W * H));
    dx[i] += 0.25f * dy[(((size_t)n * (H / 2) + y / 2) * (W / 2) + x / 2) * C + c];
  }
}

// out = bf16(dy * (y > 0)) and db[c] += sum of it (block partials, one
// atomic per channel per block).
// ReLU backward, 8 channels (16 bytes of BF16) a thread: out = bf16(dy) where
// y > 0, else 0, and the bias gradient db += sum over pixels of out. 192
// threads a block (a multiple of every channel-group count C / 8 up to 24),
// so a thread keeps one channel group for all its pixels and sums its 8
// bias partials in registers; one shared-memory and one global atomic a
// channel, thread and block at the end.
constexpr int kReluBwdThreads = 192;
__global__ void __launch_bounds__(kReluBwdThreads) relu_bwd_kernel(const float* __restrict__ dy,
                                                                   const bf16* __restrict__ y, bf16* __restrict__ out,
                                                                   float* __restrict__ db, long P, int C) {
  extern __shared__ float sdb[];
  for (int c = threadIdx.x; c < C; c += blockDim.x) sdb[c] = 0.f;
  __syncthreads();
  const int G = C / 8, per_block = kReluBwdThreads / G;
  const int gi = threadIdx.x % G, c0 = gi * 8;
  float part[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if ((int)threadIdx.x < per_block * G) {
    for (long p = (long)blockIdx.x * per_block + threadIdx.x / G; p < P; p += (long)gridDim.x * per_block) {
      const size_t i = (size_t)p * C + c0;
      const uint4 yr = *reinterpret_cast<const uint4*>(y + i);
      const float4 d0 = *reinterpret_cast<const float4*>(dy + i), d1 = *reinterpret_cast<const float4*>(dy + i + 4);
      const uint32_t yw[4] = {yr.x, yr.y, yr.z, yr.w};
      const float dv[8] = {d0.x, d0.y, d0.z, d0.w, d1.x, d1.y, d1.z, d1.w};
      uint32_t o[4];
#pragma unroll
      for (int h = 0; h < 4; ++h) {
        const float2 yv = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&yw[h]));
        const __nv_bfloat162 g2 = __floats2bfloat162_rn(yv.x > 0.f ? dv[2 * h] : 0.f, yv.y > 0.f ? dv[2 * h + 1] : 0.f);
        const float2 gf = __bfloat1622float2(g2);
        part[2 * h] += gf.x;
        part[2 * h + 1] += gf.y;
        o[h] = *reinterpret_cast<const uint32_t*>(&g2);
      }
      *reinterpret_cast<uint4*>(out + i) = make_uint4(o[0], o[1], o[2], o[3]);
    }
  }
  if (db) {
#pragma unroll
    for (int e = 0; e < 8; ++e) atomicAdd(&sdb[c0 + e], part[e]);
    __syncthreads();
    for (int c = threadIdx.x; c < C; c += blockDim.x) atomicAdd(&db[c], sdb[c]);
  }
}

// Backward of "concat(x1, upsample2(x2))": dx1 += dcat[:, :c1];
// dx2 += sum over each 2x2 of dcat[:, c1:].
__global__ void split_upsum_kernel(const float* __restrict__ dcat, int c1, int c2, int n_img, int H, int W,
                                   float* __restrict__ dx1, float* __restrict__ dx2) {
  const int C = c1 + c2, H2 = H / 2, W2 = W / 2;
  const long t1 = (long)n_img * H * W * c1;
  GRID_STRIDE(i, t1) {
    const int c = (int)(i % c1);
    const long p = i / c1;
    dx1[i] += dcat[p * C + c];
  }
  const long t2 = (long)n_img * H2 * W2 * c2;
  GRID_STRIDE(i, t2) {
    const int c = (int)(i % c2);
    const long q = i / c2;
    const int x = (int)(q % W2), y = (int)((q / W2) % H2), n = (int)(q / ((long)W2 * H2));
    float s = 0.f;
#pragma unroll
    for (int d = 0; d < 4; ++d) s += dcat[((((size_t)n * H + 2 * y + (d >> 1)) * W + 2 * x + (d & 1))) * C + c1 + c];
    dx2[i] += s;
  }
}

// ---------------------------------------------------------------------------
// Kernel-prediction head at one scale. Per pixel: logits = Wh . F + bh;
// 5x5 kernel = softmax(logits[0:25]) applied to the scale's noisy
// illumination (edge-clamped); with a coarser result, alpha =
// sigmoid(logits[25]) blends it in (o = (1 - a) f + a up(o_coarse)); at
// scale 0 logits[26] is the predicted log squared error (variance gate).
struct HeadArgs {
  const bf16* F;       // [N][H][W][C]
  const float* Wh;     // [K][C]
  const float* bh;     // [K]
  const float* R;      // [N][H][W][3]
  const float* coarse; // [N][H/2][W/2][3] or null
  float* out;          // [N][H][W][3]
  float* kw;           // [N][H][W][25] softmax weights, saved for backward (optional)
  float* filt;         // [N][H][W][3] filtered, before the blend (optional)
  float* alpha;        // [N][H][W] blend weight (optional)
  float* var;          // [N][H][W] or null (log squared-error prediction)
  int N, H, W, C, K;
};

// CT, KT > 0: channel and logit counts fixed at compile time (the network's
// three heads), so the logits stay in registers; 0: any (runtime loops).
template <int CT, int KT>
__global__ void kp_head_fwd_kernel(HeadArgs a) {
  extern __shared__ float sW[];  // [K][C]
  const int C = CT > 0 ? CT : a.C, K = KT > 0 ? KT : a.K;
  for (int i = threadIdx.x; i < K * C; i += blockDim.x) sW[i] = a.Wh[i];
  __syncthreads();
  const long P = (long)a.N * a.H * a.W;
  GRID_STRIDE(p, P) {
    const int x = (int)(p % a.W), y = (int)((p / a.W) % a.H), n = (int)(p / ((long)a.W * a.H));
    float lg[27];
#pragma unroll
    for (int k = 0; k < 27; ++k)
      if (k < K) lg[k] = a.bh[k];
    const bf16* f = a.F + p * C;
#pragma unroll 1
    for (int c = 0; c < C; c += 8) {
      const uint4 raw = *reinterpret_cast<const uint4*>(f + c);  // 8 channels
      const uint32_t w4[4] = {raw.x, raw.y, raw.z, raw.w};
#pragma unroll
      for (int h = 0; h < 4; ++h) {
        const float2 v = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&w4[h]));
        const int cc = c + 2 * h;
#pragma unroll
        for (int k = 0; k < 27; ++k)
          if (k < K) lg[k] += sW[k * C + cc] * v.x + sW[k * C + cc + 1] * v.y;
      }
    }
    float mx = lg[0];
#pragma unroll
    for (int k = 1; k < kKP; ++k) mx = fmaxf(mx, lg[k]);
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < kKP; ++k) {
      lg[k] = __expf(lg[k] - mx);
      s += lg[k];
    }
    const float inv = 1.f / s;
    float3 acc = f3(0.f);
#pragma unroll
    for (int k = 0; k < kKP; ++k) {
      const float w = lg[k] * inv;
      if (a.kw) a.kw[p * kKP + k] = w;
      const int sx = min(max(x + k % 5 - 2, 0), a.W - 1), sy = min(max(y + k / 5 - 2, 0), a.H - 1);
      const float* r = a.R + (((size_t)n * a.H + sy) * a.W + sx) * 3;
      acc = acc + w * f3(r[0], r[1], r[2]);
    }
    if (a.filt) {
      a.filt[p * 3 + 0] = acc.x;
      a.filt[p * 3 + 1] = acc.y;
      a.filt[p * 3 + 2] = acc.z;
    }
    float3 o = acc;
    if (a.coarse) {
      const float al = 1.f / (1.f + __expf(-lg[kKP]));
      if (a.alpha) a.alpha[p] = al;
      const float* cc = a.coarse + (((size_t)n * (a.H / 2) + y / 2) * (a.W / 2) + x / 2) * 3;
      o = (1.f - al) * acc + al * f3(cc[0], cc[1], cc[2]);
    }
    if (a.var) a.var[p] = a.coarse ? lg[kKP + 1] : lg[kKP];
    a.out[p * 3 + 0] = o.x;
    a.out[p * 3 + 1] = o.y;
    a.out[p * 3 + 2] = o.z;
  }
}

// The network's three heads, a block per tile of 4 rows x 32 pixels (one
// row a warp, grid-stride over tiles). The 1x1 convolution runs on the
// tensor cores: per 16-pixel group the logits are a [16 x C] x [C x 32]
// product (27 logits padded to 32) by mma.sync m16n8k16 with FP32
// accumulation; the FP32 head weights are split into three BF16 parts
// (w = hi + mid + lo to ~24 bits) and the features are BF16 already, so the
// three products add up to the FP32 logits. The logits go through shared
// memory to one lane a pixel, which takes the softmax and the 5x5 filter as
// the per-pixel kernel does, reading the radiance from the tile's halo,
// staged once in shared memory with the edge replication of that kernel
// (the radiance gather, not the projection, bounds the per-pixel kernel).
template <int C, int K>
__global__ void __launch_bounds__(128) kp_head_fwd_tile_kernel(HeadArgs a) {
  constexpr int KS = C / 16;             // k steps of 16 channels
  constexpr int TW = 32, TH = 4;         // tile: one 32-pixel row a warp
  constexpr int RW = TW + 4, RH = TH + 4;  // radiance halo (5x5 taps)
  constexpr int LS = 27;                 // logits a pixel in shared memory (odd: no bank conflicts)
  __shared__ uint2 sB[3][KS][4][32];     // B fragments of the three weight parts: [part][ks][nt][lane]
  __shared__ float sBias[32];
  __shared__ float sR[RH * RW * 3];
  __shared__ float sL[TH][TW * LS];
  for (int i = threadIdx.x; i < 3 * KS * 4 * 32; i += blockDim.x) {
    const int ln = i % 32, nt = (i / 32) % 4, ks = (i / 128) % KS, part = i / (128 * KS);
    const int g = ln >> 2, t = ln & 3, n = nt * 8 + g;
    uint32_t r[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {  // b0: k = 2t, 2t + 1; b1: k = 2t + 8, 2t + 9
      const int k0 = ks * 16 + 2 * t + 8 * h;
      float w[2];
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        float v = n < K ? a.Wh[n * C + k0 + j] : 0.f;
        for (int q = 0; q < part; ++q) v -= __bfloat162float(__float2bfloat16_rn(v));
        w[j] = v;
      }
      const __nv_bfloat162 b2 = __floats2bfloat162_rn(w[0], w[1]);
      r[h] = *reinterpret_cast<const uint32_t*>(&b2);
    }
    sB[part][ks][nt][ln] = make_uint2(r[0], r[1]);
  }
  for (int i = threadIdx.x; i < 32; i += blockDim.x) sBias[i] = i < K ? a.bh[i] : 0.f;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int tiles_x = (a.W + TW - 1) / TW, tiles_y = (a.H + TH - 1) / TH;
  const long tiles = (long)tiles_x * tiles_y * a.N;
  for (long tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    const int n = (int)(tile / ((long)tiles_x * tiles_y));
    const int rem = (int)(tile % ((long)tiles_x * tiles_y));
    const int x0 = (rem % tiles_x) * TW, y0 = (rem / tiles_x) * TH;
    __syncthreads();  // the previous tile's shared-memory reads are done (and sB, sBias written)
    for (int i = threadIdx.x; i < RH * RW * 3; i += blockDim.x) {
      const int q = i / 3, hx = q % RW, hy = q / RW;
      const int sx = min(max(x0 - 2 + hx, 0), a.W - 1), sy = min(max(y0 - 2 + hy, 0), a.H - 1);
      sR[i] = a.R[(((size_t)n * a.H + sy) * a.W + sx) * 3 + i % 3];
    }
    const int y = y0 + warp, yc = min(y, a.H - 1);
    const size_t row = ((size_t)n * a.H + yc) * a.W;
#pragma unroll 1
    for (int grp = 0; grp < 2; ++grp) {
      const int xa = min(x0 + grp * 16 + g, a.W - 1), xb = min(x0 + grp * 16 + g + 8, a.W - 1);
      const uint32_t* fa = reinterpret_cast<const uint32_t*>(a.F + (row + xa) * C);
      const uint32_t* fb = reinterpret_cast<const uint32_t*>(a.F + (row + xb) * C);
      float acc[4][4];
#pragma unroll
      for (int nt = 0; nt < 4; ++nt) {
        const float b0 = sBias[nt * 8 + 2 * t], b1 = sBias[nt * 8 + 2 * t + 1];
        acc[nt][0] = b0;
        acc[nt][1] = b1;
        acc[nt][2] = b0;
        acc[nt][3] = b1;
      }
#pragma unroll
      for (int ks = 0; ks < KS; ++ks) {
        const uint32_t a0 = fa[ks * 8 + t], a1 = fb[ks * 8 + t], a2 = fa[ks * 8 + 4 + t], a3 = fb[ks * 8 + 4 + t];
#pragma unroll
        for (int part = 2; part >= 0; --part)  // smallest parts first
#pragma unroll
          for (int nt = 0; nt < 4; ++nt) {
            const uint2 b = sB[part][ks][nt][lane];
            asm volatile(
                "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                "{%0,%1,%2,%3};\n"
                : "+f"(acc[nt][0]), "+f"(acc[nt][1]), "+f"(acc[nt][2]), "+f"(acc[nt][3])
                : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b.x), "r"(b.y));
          }
      }
      // lane (g, t) holds logits 8 nt + 2t + j of the group's pixels g (c0, c1) and g + 8 (c2, c3)
      float* la = &sL[warp][(grp * 16 + g) * LS];
      float* lb = la + 8 * LS;
#pragma unroll
      for (int nt = 0; nt < 4; ++nt)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          const int k = nt * 8 + 2 * t + j;
          if (k < K) {
            la[k] = acc[nt][j];
            lb[k] = acc[nt][2 + j];
          }
        }
    }
    __syncthreads();  // the halo and this warp's logits in place
    const int x = x0 + lane;
    if (x >= a.W || y >= a.H) continue;
    const long p = (long)row + x;
    const float* lg = &sL[warp][lane * LS];
    float mx = lg[0];
#pragma unroll
    for (int k = 1; k < kKP; ++k) mx = fmaxf(mx, lg[k]);
    float e[kKP], sum = 0.f;
#pragma unroll
    for (int k = 0; k < kKP; ++k) {
      e[k] = __expf(lg[k] - mx);
      sum += e[k];
    }
    const float inv = 1.f / sum;
    float3 acc3 = f3(0.f);
#pragma unroll
    for (int k = 0; k < kKP; ++k) {
      const float w = e[k] * inv;
      if (a.kw) a.kw[p * kKP + k] = w;
      const float* r = &sR[((warp + k / 5) * RW + lane + k % 5) * 3];
      acc3 = acc3 + w * f3(r[0], r[1], r[2]);
    }
    if (a.filt) {
      a.filt[p * 3 + 0] = acc3.x;
      a.filt[p * 3 + 1] = acc3.y;
      a.filt[p * 3 + 2] = acc3.z;
    }
    float3 o = acc3;
    if (a.coarse) {
      const float al = 1.f / (1.f + __expf(-lg[kKP]));
      if (a.alpha) a.alpha[p] = al;
      const float* cc = a.coarse + (((size_t)n * (a.H / 2) + y / 2) * (a.W / 2) + x / 2) * 3;
      o = (1.f - al) * acc3 + al * f3(cc[0], cc[1], cc[2]);
    }
    if (a.var) a.var[p] = a.coarse ? lg[kKP + 1] : lg[kKP];
    a.out[p * 3 + 0] = o.x;
    a.out[p * 3 + 1] = o.y;
    a.out[p * 3 + 2] = o.z;
  }
}

struct HeadBwdArgs {
  HeadArgs f;
  const float* dout;   // [N][H][W][3]
  const float* dvar;   // [N][H][W] or null
  float* dF;           // [N][H][W][C] accumulated
  float* dWh;          // [K][C] accumulated
  float* dbh;          // [K] accumulated
  float* dcoarse;      // [N][H/2][W/2][3] accumulated, or null
};

// Backward of a head, 128 pixels a block per batch (one a thread): the
// thread takes its pixel's softmax, filter and blend backward and the
// feature gradient (dF += W^T dl), and leaves dl and the pixel's features
// in shared memory; then the block sums the weight gradient dW = sum over
// the batch of dl F^T with each thread owning (logit, 8 channels) blocks in
// registers -- no shared-memory atomics on addresses every lane shares --
// and adds its blocks to dWh once at the end.
constexpr int kHeadBwdThreads = 128;
__host__ __device__ constexpr int head_bwd_dl_stride(int k) { return k | 1; }  // odd: no bank conflicts
__host__ __device__ constexpr int head_bwd_f_stride(int c) { return c + 8; }   // BF16, 16-byte rows
__host__ __device__ constexpr size_t head_bwd_smem(int k, int c) {
  return ((size_t)k * c + (size_t)kHeadBwdThreads * head_bwd_dl_stride(k)) * sizeof(float) +
         (size_t)kHeadBwdThreads * head_bwd_f_stride(c) * sizeof(bf16);
}

// CT, KT > 0: the network's three heads (sizes fixed at compile time, so the
// per-pixel logit gradients stay in registers); 0: any.
template <int CT, int KT>
__global__ void __launch_bounds__(kHeadBwdThreads) kp_head_bwd_kernel(HeadBwdArgs b) {
  extern __shared__ __align__(16) float sm[];
  const HeadArgs& a = b.f;
  const int K = KT > 0 ? KT : a.K, C = CT > 0 ? CT : a.C, DLS = head_bwd_dl_stride(K), FS = head_bwd_f_stride(C);
  float* sW = sm;                                          // [K][C]
  float* sDL = sW + K * C;                                 // [128][DLS]
  bf16* sF = reinterpret_cast<bf16*>(sDL + kHeadBwdThreads * DLS);  // [128][FS]
  const int tid = threadIdx.x;
  for (int i = tid; i < K * C; i += blockDim.x) sW[i] = a.Wh[i];
  const int cb = C / 8, owners = K * cb;
  float acc[2][8];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int e = 0; e < 8; ++e) acc[i][e] = 0.f;
  float accb = 0.f;
  const long P = (long)a.N * a.H * a.W;
  for (long base = (long)blockIdx.x * kHeadBwdThreads; base < P; base += (long)gridDim.x * kHeadBwdThreads) {
    __syncthreads();  // sW written; the previous batch's shared-memory reads done
    const long p = base + tid;
    float dl[27];
#pragma unroll
    for (int k = 0; k < 27; ++k) dl[k] = 0.f;
    if (p < P) {
      const int x = (int)(p % a.W), y = (int)((p / a.W) % a.H), n = (int)(p / ((long)a.W * a.H));
      const float3 dout = f3(b.dout[p * 3], b.dout[p * 3 + 1], b.dout[p * 3 + 2]);
      float3 df = dout;
      if (a.coarse) {
        const float al = a.alpha[p];
        const float* cc = a.coarse + (((size_t)n * (a.H / 2) + y / 2) * (a.W / 2) + x / 2) * 3;
        const float3 fl = f3(a.filt[p * 3], a.filt[p * 3 + 1], a.filt[p * 3 + 2]);
        const float da = dot(dout, f3(cc[0], cc[1], cc[2]) - fl);
        dl[kKP] = da * al * (1.f - al);
        df = (1.f - al) * dout;
        if (b.dcoarse) {
          float* dc = b.dcoarse + (((size_t)n * (a.H / 2) + y / 2) * (a.W / 2) + x / 2) * 3;
          atomicAdd(dc + 0, al * dout.x);
          atomicAdd(dc + 1, al * dout.y);
          atomicAdd(dc + 2, al * dout.z);
        }
      }
      if (b.dvar) dl[a.coarse ? kKP + 1 : kKP] = b.dvar[p];
      // softmax backward
      float dw[kKP], sum = 0.f;
      for (int k = 0; k < kKP; ++k) {
        const int sx = min(max(x + k % 5 - 2, 0), a.W - 1), sy = min(max(y + k / 5 - 2, 0), a.H - 1);
        const float* r = a.R + (((size_t)n * a.H + sy) * a.W + sx) * 3;
        dw[k] = dot(df, f3(r[0], r[1], r[2]));
        sum += a.kw[p * kKP + k] * dw[k];
      }
      for (int k = 0; k < kKP; ++k) dl[k] = a.kw[p * kKP + k] * (dw[k] - sum);
      const bf16* f = a.F + p * C;
      float* dF = b.dF + p * C;
      for (int c = 0; c < C; c += 8) {
        const uint4 raw = *reinterpret_cast<const uint4*>(f + c);
        *reinterpret_cast<uint4*>(&sF[tid * FS + c]) = raw;
        for (int h = 0; h < 8; h += 2) {
          float g0 = 0.f, g1 = 0.f;
#pragma unroll
          for (int k = 0; k < 27; ++k) {
            if (k >= K) break;
            g0 += sW[k * C + c + h] * dl[k];
            g1 += sW[k * C + c + h + 1] * dl[k];
          }
          dF[c + h] += g0;
          dF[c + h + 1] += g1;
        }
      }
    } else {
      for (int c = 0; c < C; c += 8) *reinterpret_cast<uint4*>(&sF[tid * FS + c]) = make_uint4(0u, 0u, 0u, 0u);
    }
#pragma unroll
    for (int k = 0; k < 27; ++k)
      if (k < K) sDL[tid * DLS + k] = dl[k];
    __syncthreads();
    // dW over the batch: thread owns (k, channels c0 .. c0 + 7) for j = tid, tid + 128
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const int j = tid + i * kHeadBwdThreads;
      if (j >= owners) break;
      const int k = j / cb, c0 = (j % cb) * 8;
      for (int q = 0; q < kHeadBwdThreads; ++q) {
        const float d = sDL[q * DLS + k];
        const uint4 raw = *reinterpret_cast<const uint4*>(&sF[q * FS + c0]);
        const uint32_t w4[4] = {raw.x, raw.y, raw.z, raw.w};
#pragma unroll
        for (int h = 0; h < 4; ++h) {
          const float2 v = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&w4[h]));
          acc[i][2 * h] += d * v.x;
          acc[i][2 * h + 1] += d * v.y;
        }
      }
    }
    if (tid < K)
      for (int q = 0; q < kHeadBwdThreads; ++q) accb += sDL[q * DLS + tid];
  }
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const int j = tid + i * kHeadBwdThreads;
    if (j >= owners) break;
    const int k = j / cb, c0 = (j % cb) * 8;
#pragma unroll
    for (int e = 0; e < 8; ++e) atomicAdd(&b.dWh[k * C + c0 + e], acc[i][e]);
  }
  if (tid < K) atomicAdd(&b.dbh[tid], accb);
}

// relMSE of the remodulated output against the remodulated target:
// mean over valid pixels and channels of (A o - A t)^2 / ((A t)^2 + 0.01);
// dout = dL/do. The predicted log squared error v (if given) is regressed on
// log(e + 1e-4) of the pixel's error e with weight var_w. loss[0] += L,
// loss[1] += variance loss.
__global__ void relmse_loss_kernel(const float* __restrict__ out, const float* __restrict__ target,
                                   const uchar4* __restrict__ albedo, const float* __restrict__ var, int N, int PH,
                                   int PW, int H, int W, float var_w, float* __restrict__ dout,
                                   float* __restrict__ dvar, float* __restrict__ loss) {
  __shared__ float s_l[2];
  if (threadIdx.x < 2) s_l[threadIdx.x] = 0.f;
  __syncthreads();
  const long P = (long)N * PH * PW;
  const float norm = 1.f / (3.f * (float)N * H * W);
  const float vnorm = 1.f / ((float)N * H * W);
  GRID_STRIDE(p, P) {
    const int x = (int)(p % PW), y = (int)((p / PW) % PH), n = (int)(p / ((long)PW * PH));
    if (x >= W || y >= H) {
      dout[p * 3] = dout[p * 3 + 1] = dout[p * 3 + 2] = 0.f;
      if (dvar) dvar[p] = 0.f;
      continue;
    }
    const uchar4 a4 = albedo[((size_t)n * H + y) * W + x];
    const float A[3] = {a4.x / 255.f, a4.y / 255.f, a4.z / 255.f};
    const float* t = target + (((size_t)n * H + y) * W + x) * 3;
    float l = 0.f;
    for (int c = 0; c < 3; ++c) {
      const float r = A[c] * t[c], xo = A[c] * out[p * 3 + c];
      const float den = r * r + 0.01f;
      const float d = xo - r;
      l += d * d / den;
      dout[p * 3 + c] = norm * 2.f * d / den * A[c];
    }
    atomicAdd(&s_l[0], l * norm);
    if (var) {
      const float tgt = logf(l / 3.f + 1e-4f);
      const float dv = var[p] - tgt;
      dvar[p] = var_w * 2.f * dv * vnorm;
      atomicAdd(&s_l[1], dv * dv * vnorm);
    }
  }
  __syncthreads();
  if (threadIdx.x < 2) atomicAdd(&loss[threadIdx.x], s_l[threadIdx.x]);
}

// Adam on FP32 master weights; writes the BF16 copy the convolutions read.
__global__ void adam_kernel(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, bf16* __restrict__ w16, long n, float lr, float b1, float b2,
                            float eps, float c1, float c2, float grad_scale) {
  GRID_STRIDE(i, n) {
    const float gi = g[i] * grad_scale;
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    if (w16) w16[i] = __float2bfloat16_rn(wi);
  }
}

// Variance gate: one CTA per tile x tile block; the block falls back when
// the mean over its pixels of the predicted relative squared error
// (exp of the error head's log output) exceeds the threshold.
__global__ void gate_kernel(const float* __restrict__ var, int PW, int W, int H, float threshold, int tile,
                            uint8_t* __restrict__ mask, uint32_t* __restrict__ count) {
  __shared__ float part[8];
  const int tiles_x = (W + tile - 1) / tile;
  const int tx = blockIdx.x % tiles_x, ty = blockIdx.x / tiles_x;
  const int x0 = tx * tile, y0 = ty * tile;
  const int tw = min(tile, W - x0), th = min(tile, H - y0);
  float s = 0.f;
  for (int i = threadIdx.x; i < tw * th; i += blockDim.x) s += __expf(var[(size_t)(y0 + i / tw) * PW + x0 + i % tw]);
  for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += part[w];
    const bool fb = t / (float)(tw * th) > threshold;
    mask[blockIdx.x] = fb ? 1 : 0;
    if (fb) atomicAdd(count, 1u);
  }
}

// Learned tile gate (no reference counterpart). Per tile of the frame, eight
// features that need no reference image -- the error head's mean predicted
// relative squared error, the mean squared difference between the
// network's and BMFR's final images, the mean accumulated sample count, the
// variance of log(1 + luminance) and the mean luminance of the noisy input,
// the mean depth gradient |d log depth|, the normals' spread 1 - |mean n|,
// the mean albedo -- each as a logarithm, enter four linear predictions of
// how much the tile's relative squared error changes when the shown
// illumination is alpha * network + (1 - alpha) * BMFR for alpha = 0.75,
// 0.5, 0.25 and 0 instead of the network alone (regressions fitted offline
// on tiles of held-out frames against converged renders). The tile takes the
// alpha with the lowest prediction (alpha 1, the network, when none is
// below zero). Runs after the network's final image is composed: tiles with
// alpha < 1 get the blend of the network's FP32 output and BMFR's denoised
// (RGBA16F) illumination in `denoised` and, remodulated and tone mapped as
// the compose pass does, in the final image (alpha 0: BMFR's own final
// pixels).
struct GateModelArgs {
  const float* var;  // padded (PW) log predicted relative squared error
  const float* nn_out;  // padded (PW) network output, 3 floats a pixel
  int PW, W, H, tile;
  const uchar4* bm_final;  // BMFR final image
  const Half4* bm_denoised;  // BMFR denoised, 2 layers of W x H
  const uint32_t* bm_layer;  // device word: the layer BMFR wrote this frame
  const uint8_t* spp;      // accumulated samples (null: 1)
  const Half4* noisy16;    // noisy demodulated input (one of the two)
  const float4* noisy32;
  const float* depth;
  const float2* normal;    // (theta, phi)
  const uchar4* albedo;
  float coef[36];          // per alpha 0.75, 0.5, 0.25, 0: 8 weights, then the bias
  uint8_t* mask;           // per tile: 0 network, 1..4 alpha 0.75 .. 0
  uint32_t* count;         // tiles with alpha < 1
  uchar4* final_out;       // the composed network image, rewritten in blended tiles
  float4* denoised;        // the network's output image, rewritten in blended tiles
};
constexpr int kGateSums = 11;
__global__ void __launch_bounds__(256) gate_model_kernel(GateModelArgs a) {
  __shared__ float part[8][kGateSums];
  __shared__ int choice;
  const int tiles_x = (a.W + a.tile - 1) / a.tile;
  const int tx = blockIdx.x % tiles_x, ty = blockIdx.x / tiles_x;
  const int x0 = tx * a.tile, y0 = ty * a.tile;
  const int tw = min(a.tile, a.W - x0), th = min(a.tile, a.H - y0);
  float acc[kGateSums];
#pragma unroll
  for (int k = 0; k < kGateSums; ++k) acc[k] = 0.f;
  for (int i = threadIdx.x; i < tw * th; i += blockDim.x) {
    const int x = x0 + i % tw, y = y0 + i / tw;
    const size_t p = (size_t)y * a.W + x;
    acc[0] += expf(a.var[(size_t)y * a.PW + x]);
    const uchar4 n = a.final_out[p], b = a.bm_final[p];
    const float dx = ((float)b.x - (float)n.x) / 255.f, dy = ((float)b.y - (float)n.y) / 255.f,
                dz = ((float)b.z - (float)n.z) / 255.f;
    acc[1] += (dx * dx + dy * dy + dz * dz) / 3.f;
    acc[2] += a.spp ? (float)a.spp[p] : 1.f;
    const float4 c = a.noisy32 ? a.noisy32[p] : load_half4(a.noisy16 + p);
    const float lum = 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z;
    const float ll = log1pf(fmaxf(lum, 0.f));
    acc[3] += ll;
    acc[4] += ll * ll;
    const float ld = logf(fminf(fmaxf(a.depth[p], 1e-3f), 1e4f));
    float g = 0.f;
    if (x + 1 < a.W) g += fabsf(logf(fminf(fmaxf(a.depth[p + 1], 1e-3f), 1e4f)) - ld);
    if (y + 1 < a.H) g += fabsf(logf(fminf(fmaxf(a.depth[p + a.W], 1e-3f), 1e4f)) - ld);
    acc[5] += g;
    const float2 tp = a.normal[p];
    float st, ct, sp, cp;
    sincosf(tp.x, &st, &ct);
    sincosf(tp.y, &sp, &cp);
    acc[6] += st * cp;
    acc[7] += st * sp;
    acc[8] += ct;
    acc[9] += lum;
    const uchar4 al = a.albedo[p];
    acc[10] += ((float)al.x + (float)al.y + (float)al.z) / (3.f * 255.f);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < kGateSums; ++k) {
    for (int o = 16; o; o >>= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
    if (lane == 0) part[warp][k] = acc[k];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float m[kGateSums];
    for (int k = 0; k < kGateSums; ++k) {
      m[k] = 0.f;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m[k] += part[w][k];
      m[k] /= (float)(tw * th);
    }
    const float e = 1e-8f;
    const float nl = sqrtf(m[6] * m[6] + m[7] * m[7] + m[8] * m[8]);
    const float f[8] = {logf(m[0] + e), logf(m[1] + e), logf(m[2] + e), logf(fmaxf(m[4] - m[3] * m[3], 0.f) + e),
                        logf(m[5] + e), logf(fmaxf(1.f - nl, 0.f) + e), logf(m[9] + e), logf(m[10] + e)};
    int best = 0;
    float best_d = 0.f;  // the network alone
    for (int c = 0; c < 4; ++c) {
      float d = a.coef[9 * c + 8];
      for (int k = 0; k < 8; ++k) d += a.coef[9 * c + k] * f[k];
      if (d < best_d) {
        best_d = d;
        best = c + 1;
      }
    }
    choice = best;
    a.mask[blockIdx.x] = (uint8_t)best;
    if (best) atomicAdd(a.count, 1u);
  }
  __syncthreads();
  if (!choice) return;
  const float alpha = 1.f - 0.25f * (float)choice;
  const Half4* bm = a.bm_denoised + (size_t)(*a.bm_layer & 1u) * a.W * a.H;
  for (int i = threadIdx.x; i < tw * th; i += blockDim.x) {
    const int x = x0 + i % tw, y = y0 + i / tw;
    const size_t p = (size_t)y * a.W + x, q = (size_t)y * a.PW + x;
    const float4 b = load_half4(bm + p);
    const float3 o = f3(a.nn_out[q * 3], a.nn_out[q * 3 + 1], a.nn_out[q * 3 + 2]);
    const float3 c = o * alpha + f3(b.x, b.y, b.z) * (1.f - alpha);
    a.denoised[p] = make_float4(c.x, c.y, c.z, 1.f);
    if (choice == 4) {
      a.final_out[p] = a.bm_final[p];
      continue;
    }
    const uchar4 al = a.albedo[p];
    float3 t = fmax3(f3(0.f), f3(al.x / 255.f + 1e-6f, al.y / 255.f + 1e-6f, al.z / 255.f + 1e-6f) * c);
    t = clamp3(f3(powf(t.x, .454545f), powf(t.y, .454545f), powf(t.z, .454545f)), 0.f, 1.f);
    a.final_out[p] = make_uchar4(f2u8(t.z), f2u8(t.y), f2u8(t.x), 255);
  }
}

// Final image of the neural path: the network's denoised illumination
// (always written to `denoised`) remodulated by the albedo and tone mapped
// as bmfrPost does (shaders/bmfrPost.comp:211-214); pixels of tiles the gate
// marked take the fallback (BMFR) final image instead.
__global__ void compose_kernel(const float* __restrict__ out, int PW, int W, int H, const uchar4* __restrict__ albedo,
                               const uint8_t* __restrict__ mask, int tile, const uchar4* __restrict__ fallback,
                               uchar4* __restrict__ final_bgra, float4* __restrict__ denoised) {
  const long P = (long)W * H;
  const int tiles_x = mask ? (W + tile - 1) / tile : 1;
  GRID_STRIDE(i, P) {
    const int x = (int)(i % W), y = (int)(i / W);
    const size_t p = (size_t)y * PW + x;
    const float3 o = f3(out[p * 3], out[p * 3 + 1], out[p * 3 + 2]);
    if (denoised) denoised[i] = make_float4(o.x, o.y, o.z, 1.f);
    if (mask && mask[(y / tile) * tiles_x + x / tile]) {
      final_bgra[i] = fallback[i];
      continue;
    }
    const uchar4 a = albedo[i];
    float3 t = fmax3(f3(0.f), f3(a.x / 255.f + 1e-6f, a.y / 255.f + 1e-6f, a.z / 255.f + 1e-6f) * o);
    t = clamp3(f3(powf(t.x, .454545f), powf(t.y, .454545f), powf(t.z, .454545f)), 0.f, 1.f);
    final_bgra[i] = make_uchar4(f2u8(t.z), f2u8(t.y), f2u8(t.x), 255);
  }
}

}  // namespace nn
}  // namespace pbrt

using namespace pbrt;
using namespace pbrt::nn;

namespace {
inline int grid_for(long n, int block = 256) { return (int)std::min<long>((n + block - 1) / block, 152L * 16); }
// Blocks of 128 threads of `kernel` resident on the device at once (at
// least one an SM), capped at `work` units.
template <class Kernel> int head_grid(Kernel kernel, long work) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 128, 0) != cudaSuccess || per_sm < 1) {
    cudaGetLastError();
    per_sm = 1;
  }
  return (int)std::max<long>(1, std::min<long>(work, (long)sms * per_sm));
}
}  // namespace

extern "C" {

PBRT_API int pbrt_nn_features(const void* illum, int32_t illum_is_half, const void* albedo, const void* normal,
                              const void* depth, const void* spp, int32_t w, int32_t h, int32_t pw, int32_t ph,
                              int32_t n_img, void* feat, float* rad, pbrt_stream_t s) {
  if (!illum || !albedo || !normal || !depth || !feat || !rad || pw < w || ph < h || w <= 0 || h <= 0 || n_img <= 0)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "nn features: bad arguments");
  const long total = (long)n_img * ph * pw;
  features_kernel<<<grid_for(total), 256, 0, s>>>(illum_is_half ? nullptr : (const float4*)illum,
                                                  illum_is_half ? (const Half4*)illum : nullptr, (const uchar4*)albedo,
                                                  (const float2*)normal, (const float*)depth, (const uint8_t*)spp, w, h,
                                                  pw, ph, n_img,
                                                  (bf16*)feat, rad);
  return check_launch("features_kernel");
}

PBRT_API int pbrt_nn_avgpool2(const void* x, void* y, int32_t is_f32, int32_t n, int32_t h, int32_t w, int32_t c,
                              pbrt_stream_t s) {
  if (!x || !y || h % 2 || w % 2 || c <= 0 || (!is_f32 && c % 2)) return fail(PBRT_ERROR_INVALID_ARGUMENT, "avgpool2");
  const long total = (long)n * (h / 2) * (w / 2) * c;
  if (is_f32) avgpool2_f32_kernel<<<grid_for(total), 256, 0, s>>>((const float*)x, (float*)y, n, h, w, c);
  else avgpool2_bf16_kernel<<<grid_for(total / 2), 256, 0, s>>>((const bf16*)x, (bf16*)y, n, h, w, c);
  return check_launch("avgpool2");
}

PBRT_API int pbrt_nn_avgpool2_bwd_add(const float* dy, float* dx, int32_t n, int32_t h, int32_t w, int32_t c,
                                      pbrt_stream_t s) {
  if (!dy || !dx || h % 2 || w % 2) return fail(PBRT_ERROR_INVALID_ARGUMENT, "avgpool2 bwd");
  avgpool2_bwd_add_kernel<<<grid_for((long)n * h * w * c), 256, 0, s>>>(dy, dx, n, h, w, c);
  return check_launch("avgpool2_bwd_add");
}

PBRT_API int pbrt_nn_relu_bwd(const float* dy, const void* y, void* out, float* db, int64_t pixels, int32_t c,
                              pbrt_stream_t s) {
  if (!dy || !y || !out || c <= 0 || c % 8 || kReluBwdThreads % (c / 8) || ((uintptr_t)dy & 15) ||
      ((uintptr_t)y & 15) || ((uintptr_t)out & 15))
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "relu bwd: channels a multiple of 8 dividing 192 x 8, 16-byte aligned");
  const long groups = pixels * (c / 8);
  relu_bwd_kernel<<<grid_for(groups, kReluBwdThreads), kReluBwdThreads, c * sizeof(float), s>>>(
      dy, (const bf16*)y, (bf16*)out, db, pixels, c);
  return check_launch("relu_bwd");
}

PBRT_API int pbrt_nn_split_upsum(const float* dcat, int32_t c1, int32_t c2, int32_t n, int32_t h, int32_t w,
                                 float* dx1, float* dx2, pbrt_stream_t s) {
  if (!dcat || !dx1 || !dx2 || h % 2 || w % 2) return fail(PBRT_ERROR_INVALID_ARGUMENT, "split upsum");
  split_upsum_kernel<<<grid_for((long)n * h * w * c1), 256, 0, s>>>(dcat, c1, c2, n, h, w, dx1, dx2);
  return check_launch("split_upsum");
}

PBRT_API int pbrt_nn_kp_head(const void* F, const float* Wh, const float* bh, const float* R, const float* coarse,
                             float* out, float* kw, float* filt, float* alpha, float* var, int32_t n, int32_t h,
                             int32_t w, int32_t c, int32_t k, pbrt_stream_t s) {
  if (!F || !Wh || !bh || !R || !out || k < kKP || k > 27 || c % 2 || (size_t)k * c * sizeof(float) > 48 * 1024 ||
      (var && k <= (coarse ? kKP + 1 : kKP)) || (coarse && k < kKP + 1))
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "kp head: bad arguments");
  HeadArgs a{(const bf16*)F, Wh, bh, R, coarse, out, kw, filt, alpha, var, n, h, w, c, k};
  const int g = grid_for((long)n * h * w, 128);
  const size_t sm = (size_t)k * c * sizeof(float);
  // the network's heads: tiles of 4 x 32 pixels, the 1x1 convolution on the
  // tensor cores; one wave of resident blocks walks the tiles
  const long tiles = (long)n * ((h + 3) / 4) * ((w + 31) / 32);
  if (c == 64 && k == 25) {
    kp_head_fwd_tile_kernel<64, 25><<<head_grid(kp_head_fwd_tile_kernel<64, 25>, tiles), 128, 0, s>>>(a);
  } else if (c == 48 && k == 26) {
    kp_head_fwd_tile_kernel<48, 26><<<head_grid(kp_head_fwd_tile_kernel<48, 26>, tiles), 128, 0, s>>>(a);
  } else if (c == 32 && k == 27) {
    kp_head_fwd_tile_kernel<32, 27><<<head_grid(kp_head_fwd_tile_kernel<32, 27>, tiles), 128, 0, s>>>(a);
  } else if (c % 8 == 0) {
    kp_head_fwd_kernel<0, 0><<<g, 128, sm, s>>>(a);
  } else {
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "kp head: channels must be a multiple of 8");
  }
  return check_launch("kp_head_fwd");
}

PBRT_API int pbrt_nn_kp_head_bwd(const void* F, const float* Wh, const float* bh, const float* R, const float* coarse,
                                 float* kw, float* filt, float* alpha, int32_t n, int32_t h, int32_t w, int32_t c,
                                 int32_t k, const float* dout, const float* dvar, float* dF, float* dWh, float* dbh,
                                 float* dcoarse, pbrt_stream_t s) {
  if (!F || !Wh || !R || !kw || !filt || (coarse && !alpha) || !dout || !dF || !dWh || !dbh || k < kKP || k > 27 ||
      c % 8 || c <= 0 || head_bwd_smem(k, c) > 48 * 1024 || k * (c / 8) > 2 * kHeadBwdThreads ||
      (dvar && k <= (coarse ? kKP + 1 : kKP)) || (coarse && k < kKP + 1) || ((uintptr_t)F & 15))
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "kp head bwd: bad arguments");
  HeadBwdArgs b;
  b.f = HeadArgs{(const bf16*)F, Wh, bh, R, coarse, nullptr, kw, filt, alpha, nullptr, n, h, w, c, k};
  b.dout = dout;
  b.dvar = dvar;
  b.dF = dF;
  b.dWh = dWh;
  b.dbh = dbh;
  b.dcoarse = dcoarse;
  const int g = grid_for((long)n * h * w, kHeadBwdThreads);
  const size_t sm = head_bwd_smem(k, c);
  if (c == 64 && k == 25) kp_head_bwd_kernel<64, 25><<<g, kHeadBwdThreads, sm, s>>>(b);
  else if (c == 48 && k == 26) kp_head_bwd_kernel<48, 26><<<g, kHeadBwdThreads, sm, s>>>(b);
  else if (c == 32 && k == 27) kp_head_bwd_kernel<32, 27><<<g, kHeadBwdThreads, sm, s>>>(b);
  else kp_head_bwd_kernel<0, 0><<<g, kHeadBwdThreads, sm, s>>>(b);
  return check_launch("kp_head_bwd");
}

PBRT_API int pbrt_nn_relmse_loss(const float* out, const float* target, const void* albedo, const float* var,
                                 int32_t n, int32_t ph, int32_t pw, int32_t h, int32_t w, float var_weight, float* dout,
                                 float* dvar, float* loss, pbrt_stream_t s) {
  if (!out || !target || !albedo || !dout || !loss || (var && !dvar))
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "relmse loss: bad arguments");
  relmse_loss_kernel<<<grid_for((long)n * ph * pw), 256, 0, s>>>(out, target, (const uchar4*)albedo, var, n, ph, pw,
                                                                h, w, var_weight, dout, dvar, loss);
  return check_launch("relmse_loss");
}

PBRT_API int pbrt_nn_adam(float* w, const float* g, float* m, float* v, void* w_bf16, int64_t n, float lr, float b1,
                          float b2, float eps, int32_t step, float grad_scale, pbrt_stream_t s) {
  if (!w || !g || !m || !v || n <= 0 || step < 1) return fail(PBRT_ERROR_INVALID_ARGUMENT, "adam: bad arguments");
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  adam_kernel<<<grid_for(n), 256, 0, s>>>(w, g, m, v, (bf16*)w_bf16, n, lr, b1, b2, eps, c1, c2, grad_scale);
  return check_launch("adam");
}

PBRT_API int pbrt_nn_gate(const float* var, int32_t pw, int32_t w, int32_t h, float threshold, int32_t tile,
                          uint8_t* mask, uint32_t* count, pbrt_stream_t s) {
  if (!var || !mask || !count || tile < 4 || tile > 256 || w <= 0 || h <= 0 || pw < w)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "gate: bad arguments");
  const int tiles = ((w + tile - 1) / tile) * ((h + tile - 1) / tile);
  gate_kernel<<<tiles, 256, 0, s>>>(var, pw, w, h, threshold, tile, mask, count);
  return check_launch("gate");
}

PBRT_API int pbrt_nn_gate_model(const float* var, const float* nn_out, int32_t pw, int32_t w, int32_t h,
                                int32_t tile, const void* bmfr_final_bgra, const void* bmfr_denoised,
                                const uint32_t* bmfr_layer, const uint8_t* spp, const void* noisy,
                                int32_t noisy_is_half, const float* depth, const void* normal, const void* albedo,
                                const float* coef, uint8_t* mask, uint32_t* count, void* final_bgra,
                                float* denoised_rgba32f, pbrt_stream_t s) {
  if (!var || !nn_out || !bmfr_final_bgra || !bmfr_denoised || !bmfr_layer || !noisy || !depth || !normal ||
      !albedo || !coef || !mask || !count || !final_bgra || !denoised_rgba32f || tile < 4 || tile > 256 || w <= 0 ||
      h <= 0 || pw < w)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "gate model: bad arguments");
  GateModelArgs a;
  a.var = var;
  a.nn_out = nn_out;
  a.PW = pw;
  a.W = w;
  a.H = h;
  a.tile = tile;
  a.bm_final = (const uchar4*)bmfr_final_bgra;
  a.bm_denoised = (const Half4*)bmfr_denoised;
  a.bm_layer = bmfr_layer;
  a.spp = spp;
  a.noisy16 = noisy_is_half ? (const Half4*)noisy : nullptr;
  a.noisy32 = noisy_is_half ? nullptr : (const float4*)noisy;
  a.depth = depth;
  a.normal = (const float2*)normal;
  a.albedo = (const uchar4*)albedo;
  for (int k = 0; k < 36; ++k) a.coef[k] = coef[k];
  a.mask = mask;
  a.count = count;
  a.final_out = (uchar4*)final_bgra;
  a.denoised = (float4*)denoised_rgba32f;
  const int tiles = ((w + tile - 1) / tile) * ((h + tile - 1) / tile);
  gate_model_kernel<<<tiles, 256, 0, s>>>(a);
  return check_launch("gate model");
}

PBRT_API int pbrt_nn_compose(const float* out, int32_t pw, int32_t w, int32_t h, const void* albedo,
                             const uint8_t* mask, int32_t tile, const void* fallback_bgra, void* final_bgra,
                             float* denoised_rgba32f, pbrt_stream_t s) {
  if (!out || !albedo || !final_bgra || pw < w || (mask && (!fallback_bgra || tile < 4 || tile > 256)))
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "compose: bad arguments");
  compose_kernel<<<grid_for((long)w * h), 256, 0, s>>>(out, pw, w, h, (const uchar4*)albedo, mask, tile,
                                                      (const uchar4*)fallback_bgra, (uchar4*)final_bgra,
                                                      (float4*)denoised_rgba32f);
  return check_launch("compose");
}

}  // extern "C"
