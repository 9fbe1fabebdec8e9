// 3x3 convolutions of the kernel-predicting denoiser on tensor cores (BF16
// operands, FP32 accumulation), as implicit GEMMs -- no im2col buffer.
//
// Activations are NHWC BF16 with channel counts that are multiples of 16.
// Weights are [Cout][9][Cin] BF16 (tap = ky * 3 + kx). The forward kernel
// reads its input from one tensor, or from two tensors concatenated along C
// where the second is at half resolution and upsampled (nearest) on load --
// the U-Net decoder's "upsample, then concatenate the skip" without
// materialising either. The backward-data pass is the same kernel run on the
// spatially flipped, channel-transposed weights; the backward-weight pass is
// a GEMM over pixels (dW = dY^T . im2col(X)), split over pixel chunks.
#include <cuda_bf16.h>
#include <cuda_fp8.h>

#include <algorithm>
#include <cstdint>

#include "internal.hpp"

namespace pbrt {
namespace nn {

typedef __nv_bfloat16 bf16;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void cp_async16(void* dst, const void* src, bool valid) {
  const int n = valid ? 16 : 0;  // src-size 0: zero fill
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(smem_u32(dst)), "l"(src), "r"(n));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N> __device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }
__device__ __forceinline__ void ldsm_x4(uint32_t addr, uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(addr));
}
__device__ __forceinline__ void ldsm_x2(uint32_t addr, uint32_t& r0, uint32_t& r1) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];\n" : "=r"(r0), "=r"(r1) : "r"(addr));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t addr, uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(addr));
}
__device__ __forceinline__ void mma_bf16(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

struct ConvArgs {
  const bf16* x1;  // [N][H][W][c1]
  const bf16* x2;  // [N][H/2][W/2][c2] (upsampled on load) or null
  int c1, c2;
  const bf16* w;       // [cout][9][c1 + c2]
  const float* bias;   // [cout] or null
  bf16* y;             // [N][H][W][cout] (ldy = cout)
  float* y32;          // optional FP32 copy of the output
  int N, H, W, cout;
  int relu;            // bit 0: ReLU; bit 1: add into y32 instead of overwriting; bit 2: k-step kernel;
                       // bit 3: no wide-tile kernel
};

// Output tile: 8 rows x 16 columns = 128 pixels; BN output channels; K steps
// of 16 input channels per tap. 8 warps: 4 along pixels (32 each) x 2 along
// channels (BN / 2 each, WN n8-tiles).
constexpr int kTH = 8, kTW = 16, kBM = 128, kStages = 4;
constexpr int kRowA = 24;  // smem row stride in bf16 (16 + 8 pad): conflict-free ldmatrix

template <int WN>
__global__ void __launch_bounds__(256) conv3x3_fwd_kernel(ConvArgs a) {
  constexpr int BN = 16 * WN;
  __shared__ __align__(128) bf16 sA[kStages][kBM * kRowA];
  __shared__ __align__(128) bf16 sB[kStages][BN * kRowA];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp & 3, wn = warp >> 2;
  const int tiles_x = (a.W + kTW - 1) / kTW;
  const int x0 = (blockIdx.x % tiles_x) * kTW, y0 = (blockIdx.x / tiles_x) * kTH;
  const int n = blockIdx.y;
  const int co0 = blockIdx.z * BN;
  const int cin = a.c1 + a.c2;
  const int kchunks = cin / 16;
  const int ksteps = 9 * kchunks;
  // this thread's A load: pixel tid / 2, 16-byte half tid % 2
  const int lp = tid >> 1, lh = tid & 1;
  const int py = y0 + lp / kTW, px = x0 + lp % kTW;
  const int H2 = a.H >> 1, W2 = a.W >> 1;
  auto load_stage = [&](int stage, int ks) {
    const int tap = ks / kchunks, kc = ks % kchunks;
    const int dy = tap / 3 - 1, dx = tap % 3 - 1;
    const int ci = kc * 16;
    {
      const int yy = py + dy, xx = px + dx;
      const bool in = (yy >= 0 && yy < a.H && xx >= 0 && xx < a.W);
      const bf16* src;
      if (ci < a.c1) {
        src = a.x1 + (((size_t)n * a.H + (in ? yy : 0)) * a.W + (in ? xx : 0)) * a.c1 + ci + lh * 8;
      } else {
        const int y2 = in ? (yy >> 1) : 0, x2 = in ? (xx >> 1) : 0;
        src = a.x2 + (((size_t)n * H2 + y2) * W2 + x2) * a.c2 + (ci - a.c1) + lh * 8;
      }
      cp_async16(&sA[stage][lp * kRowA + lh * 8], src, in);
    }
    for (int i = tid; i < BN * 2; i += 256) {
      const int row = i >> 1, h = i & 1;
      const int co = co0 + row;
      const bool ok = co < a.cout;
      const bf16* src = a.w + ((size_t)(ok ? co : 0) * 9 + tap) * cin + ci + h * 8;
      cp_async16(&sB[stage][row * kRowA + h * 8], src, ok);
    }
  };
  float acc[2][WN][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < WN; ++j)
#pragma unroll
      for (int k = 0; k < 4; ++k) acc[i][j][k] = 0.f;
#pragma unroll
  for (int s = 0; s < kStages - 1; ++s) {
    if (s < ksteps) load_stage(s, s);
    cp_async_commit();
  }
  for (int ks = 0; ks < ksteps; ++ks) {
    cp_async_wait<kStages - 2>();
    __syncthreads();
    const int nxt = ks + kStages - 1;
    if (nxt < ksteps) load_stage(nxt % kStages, nxt);
    cp_async_commit();
    const int st = ks % kStages;
    uint32_t af[2][4];
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const int row = wm * 32 + i * 16 + (lane & 7) + 8 * ((lane >> 3) & 1);
      const int col = 8 * (lane >> 4);
      ldsm_x4(smem_u32(&sA[st][row * kRowA + col]), af[i][0], af[i][1], af[i][2], af[i][3]);
    }
#pragma unroll
    for (int j = 0; j < WN; ++j) {
      uint32_t b0, b1;
      const int row = wn * (8 * WN) + j * 8 + (lane & 7);
      const int col = 8 * ((lane >> 3) & 1);
      ldsm_x2(smem_u32(&sB[st][row * kRowA + col]), b0, b1);
#pragma unroll
      for (int i = 0; i < 2; ++i) mma_bf16(acc[i][j], af[i][0], af[i][1], af[i][2], af[i][3], b0, b1);
    }
  }
  cp_async_wait<0>();
  // epilogue: bias, ReLU, store
#pragma unroll
  for (int i = 0; i < 2; ++i) {
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const int p = wm * 32 + i * 16 + (lane >> 2) + 8 * half;
      const int oy = y0 + p / kTW, ox = x0 + p % kTW;
      if (oy >= a.H || ox >= a.W) continue;
      const size_t base = (((size_t)n * a.H + oy) * a.W + ox) * a.cout;
#pragma unroll
      for (int j = 0; j < WN; ++j) {
        const int co = co0 + wn * (8 * WN) + j * 8 + 2 * (lane & 3);
        if (co >= a.cout) continue;
        float v0 = acc[i][j][2 * half], v1 = acc[i][j][2 * half + 1];
        if (a.bias) {
          v0 += a.bias[co];
          v1 += a.bias[co + 1];
        }
        if (a.relu & 1) {
          v0 = fmaxf(v0, 0.f);
          v1 = fmaxf(v1, 0.f);
        }
        if (a.y) *reinterpret_cast<__nv_bfloat162*>(a.y + base + co) = __floats2bfloat162_rn(v0, v1);
        if (a.y32) {
          float2* d = reinterpret_cast<float2*>(a.y32 + base + co);
          if (a.relu & 2) {
            const float2 o = *d;
            v0 += o.x;
            v1 += o.y;
          }
          *d = make_float2(v0, v1);
        }
      }
    }
  }
}

// Halo-tile forward: per chunk of KC input channels the CTA stages the
// (8+2) x (16+2) input halo of its 8 x 16 output tile and the BN x 9 x KC
// weight slab in shared memory (cp.async, double-buffered across chunks)
// and runs all nine taps from there: each input pixel is read from global
// memory once per chunk instead of once per tap, and the CTA synchronises
// once per chunk instead of once per (tap, 16 channels). ldmatrix takes the
// A rows straight from the halo (row addresses per lane), so no im2col copy
// is made. Rows are padded by 16 bytes (conflict-free ldmatrix).
constexpr int kHaloH = kTH + 2, kHaloW = kTW + 2, kHaloPx = kHaloH * kHaloW;

template <int WN, int KC>
struct HaloCfg {
  static constexpr int BN = 16 * WN;
  static constexpr int kRowHalo = KC + (KC == 16 ? 0 : 8);   // bf16 per halo pixel row
  static constexpr int kRowW = 9 * KC + 8;                    // bf16 per weight row (one co)
  static constexpr int kStageElems = kHaloPx * kRowHalo + BN * kRowW;
  static constexpr size_t kSmem = 2 * (size_t)kStageElems * sizeof(bf16);
};

template <int WN, int KC>
__global__ void __launch_bounds__(256) conv3x3_halo_kernel(ConvArgs a) {
  typedef HaloCfg<WN, KC> Cfg;
  constexpr int BN = Cfg::BN, RH = Cfg::kRowHalo, RW = Cfg::kRowW;
  extern __shared__ __align__(128) bf16 smem[];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp & 3, wn = warp >> 2;
  const int tiles_x = (a.W + kTW - 1) / kTW;
  const int x0 = (blockIdx.x % tiles_x) * kTW, y0 = (blockIdx.x / tiles_x) * kTH;
  const int n = blockIdx.y;
  const int co0 = blockIdx.z * BN;
  const int cin = a.c1 + a.c2;
  const int nchunks = (cin + KC - 1) / KC;
  const int H2 = a.H >> 1, W2 = a.W >> 1;
  auto halo = [&](int st) { return smem + (size_t)st * Cfg::kStageElems; };
  auto wts = [&](int st) { return smem + (size_t)st * Cfg::kStageElems + kHaloPx * RH; };
  auto load_chunk = [&](int st, int ch) {
    const int c0 = ch * KC;
    bf16* sh = halo(st);
    constexpr int kPieces = KC / 8;  // 16-byte pieces per pixel
    for (int i = tid; i < kHaloPx * kPieces; i += 256) {
      const int hp = i / kPieces, pc = i % kPieces;
      const int yy = y0 - 1 + hp / kHaloW, xx = x0 - 1 + hp % kHaloW;
      const int ci = c0 + pc * 8;
      const bool ok = yy >= 0 && yy < a.H && xx >= 0 && xx < a.W && ci < cin;
      const bf16* src = a.x1;
      if (ok) {
        if (ci < a.c1) src = a.x1 + (((size_t)n * a.H + yy) * a.W + xx) * a.c1 + ci;
        else src = a.x2 + (((size_t)n * H2 + (yy >> 1)) * W2 + (xx >> 1)) * a.c2 + (ci - a.c1);
      }
      cp_async16(sh + hp * RH + pc * 8, src, ok);
    }
    bf16* sw = wts(st);
    for (int i = tid; i < BN * 9 * kPieces; i += 256) {
      const int row = i / (9 * kPieces), r = i % (9 * kPieces);
      const int tap = r / kPieces, pc = r % kPieces;
      const int co = co0 + row, ci = c0 + pc * 8;
      const bool ok = co < a.cout && ci < cin;
      const bf16* src = ok ? a.w + ((size_t)co * 9 + tap) * cin + ci : a.w;
      cp_async16(sw + row * RW + tap * KC + pc * 8, src, ok);
    }
  };
  float acc[2][WN][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < WN; ++j)
#pragma unroll
      for (int k = 0; k < 4; ++k) acc[i][j][k] = 0.f;
  // this lane's A rows: output pixel (row r, column c) of the tile for each m16 tile i
  int pr[2], pcl[2];
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const int m = wm * 32 + i * 16 + (lane & 7) + 8 * ((lane >> 3) & 1);
    pr[i] = m / kTW;
    pcl[i] = m % kTW;
  }
  const int acol = 8 * (lane >> 4);
  load_chunk(0, 0);
  cp_async_commit();
  for (int ch = 0; ch < nchunks; ++ch) {
    const int st = ch & 1;
    if (ch + 1 < nchunks) load_chunk(st ^ 1, ch + 1);
    cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();
    const uint32_t hbase = smem_u32(halo(st)), wbase = smem_u32(wts(st));
#pragma unroll
    for (int tap = 0; tap < 9; ++tap) {
      const int dy = tap / 3, dx = tap % 3;  // halo offset = output + (dy, dx)
#pragma unroll
      for (int kk = 0; kk < KC; kk += 16) {
        uint32_t af[2][4];
#pragma unroll
        for (int i = 0; i < 2; ++i) {
          const int hp = (pr[i] + dy) * kHaloW + pcl[i] + dx;
          ldsm_x4(hbase + (uint32_t)((hp * RH + kk + acol) * 2), af[i][0], af[i][1], af[i][2], af[i][3]);
        }
#pragma unroll
        for (int j = 0; j < WN; ++j) {
          uint32_t b0, b1;
          const int row = wn * (8 * WN) + j * 8 + (lane & 7);
          const int col = tap * KC + kk + 8 * ((lane >> 3) & 1);
          ldsm_x2(wbase + (uint32_t)((row * RW + col) * 2), b0, b1);
#pragma unroll
          for (int i = 0; i < 2; ++i) mma_bf16(acc[i][j], af[i][0], af[i][1], af[i][2], af[i][3], b0, b1);
        }
      }
    }
    __syncthreads();
  }
  cp_async_wait<0>();
#pragma unroll
  for (int i = 0; i < 2; ++i) {
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const int p = wm * 32 + i * 16 + (lane >> 2) + 8 * half;
      const int oy = y0 + p / kTW, ox = x0 + p % kTW;
      if (oy >= a.H || ox >= a.W) continue;
      const size_t base = (((size_t)n * a.H + oy) * a.W + ox) * a.cout;
#pragma unroll
      for (int j = 0; j < WN; ++j) {
        const int co = co0 + wn * (8 * WN) + j * 8 + 2 * (lane & 3);
        if (co >= a.cout) continue;
        float v0 = acc[i][j][2 * half], v1 = acc[i][j][2 * half + 1];
        if (a.bias) {
          v0 += a.bias[co];
          v1 += a.bias[co + 1];
        }
        if (a.relu & 1) {
          v0 = fmaxf(v0, 0.f);
          v1 = fmaxf(v1, 0.f);
        }
        if (a.y) *reinterpret_cast<__nv_bfloat162*>(a.y + base + co) = __floats2bfloat162_rn(v0, v1);
        if (a.y32) {
          float2* d = reinterpret_cast<float2*>(a.y32 + base + co);
          if (a.relu & 2) {
            const float2 o = *d;
            v0 += o.x;
            v1 += o.y;
          }
          *d = make_float2(v0, v1);
        }
      }
    }
  }
}

// Wide-tile variant for narrow outputs (Cout <= 64): all eight warps split
// the pixels of a 16 x 16 tile (32 each) and every warp computes all of the
// CTA's output channels, so one A fragment feeds NT/2..NT MMAs and B
// fragments come two n-tiles per ldmatrix.x4 (about half the ldmatrix
// traffic per MMA of the 4 x 2 warp layout).
constexpr int kMTH = 16;  // tile rows (x kTW = 16 columns)
constexpr int kMHaloH = kMTH + 2, kMHaloPx = kMHaloH * kHaloW;

template <int NT, int KC>
struct HaloMCfg {
  static constexpr int BN = 8 * NT;
  static constexpr int kRowHalo = KC + (KC == 16 ? 0 : 8);
  static constexpr int kRowW = 9 * KC + 8;
  static constexpr int kStageElems = kMHaloPx * kRowHalo + BN * kRowW;
  static constexpr size_t kSmem = 2 * (size_t)kStageElems * sizeof(bf16);
};

template <int NT, int KC>
__global__ void __launch_bounds__(256) conv3x3_halo_m_kernel(ConvArgs a) {
  typedef HaloMCfg<NT, KC> Cfg;
  constexpr int BN = Cfg::BN, RH = Cfg::kRowHalo, RW = Cfg::kRowW;
  extern __shared__ __align__(128) bf16 smem[];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int tiles_x = (a.W + kTW - 1) / kTW;
  const int x0 = (blockIdx.x % tiles_x) * kTW, y0 = (blockIdx.x / tiles_x) * kMTH;
  const int n = blockIdx.y;
  const int co0 = blockIdx.z * BN;
  const int cin = a.c1 + a.c2;
  const int nchunks = (cin + KC - 1) / KC;
  const int H2 = a.H >> 1, W2 = a.W >> 1;
  auto halo = [&](int st) { return smem + (size_t)st * Cfg::kStageElems; };
  auto wts = [&](int st) { return smem + (size_t)st * Cfg::kStageElems + kMHaloPx * RH; };
  auto load_chunk = [&](int st, int ch) {
    const int c0 = ch * KC;
    bf16* sh = halo(st);
    constexpr int kPieces = KC / 8;
    for (int i = tid; i < kMHaloPx * kPieces; i += 256) {
      const int hp = i / kPieces, pc = i % kPieces;
      const int yy = y0 - 1 + hp / kHaloW, xx = x0 - 1 + hp % kHaloW;
      const int ci = c0 + pc * 8;
      const bool ok = yy >= 0 && yy < a.H && xx >= 0 && xx < a.W && ci < cin;
      const bf16* src = a.x1;
      if (ok) {
        if (ci < a.c1) src = a.x1 + (((size_t)n * a.H + yy) * a.W + xx) * a.c1 + ci;
        else src = a.x2 + (((size_t)n * H2 + (yy >> 1)) * W2 + (xx >> 1)) * a.c2 + (ci - a.c1);
      }
      cp_async16(sh + hp * RH + pc * 8, src, ok);
    }
    bf16* sw = wts(st);
    for (int i = tid; i < BN * 9 * kPieces; i += 256) {
      const int row = i / (9 * kPieces), r = i % (9 * kPieces);
      const int tap = r / kPieces, pc = r % kPieces;
      const int co = co0 + row, ci = c0 + pc * 8;
      const bool ok = co < a.cout && ci < cin;
      const bf16* src = ok ? a.w + ((size_t)co * 9 + tap) * cin + ci : a.w;
      cp_async16(sw + row * RW + tap * KC + pc * 8, src, ok);
    }
  };
  float acc[2][NT][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < NT; ++j)
#pragma unroll
      for (int k = 0; k < 4; ++k) acc[i][j][k] = 0.f;
  int pr[2], pcl[2];
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const int m = warp * 32 + i * 16 + (lane & 7) + 8 * ((lane >> 3) & 1);
    pr[i] = m / kTW;
    pcl[i] = m % kTW;
  }
  const int acol = 8 * (lane >> 4);
  const int brow = (lane & 7) + 8 * (lane >> 4), bcol = 8 * ((lane >> 3) & 1);
  load_chunk(0, 0);
  cp_async_commit();
  for (int ch = 0; ch < nchunks; ++ch) {
    const int st = ch & 1;
    if (ch + 1 < nchunks) load_chunk(st ^ 1, ch + 1);
    cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();
    const uint32_t hbase = smem_u32(halo(st)), wbase = smem_u32(wts(st));
#pragma unroll
    for (int tap = 0; tap < 9; ++tap) {
      const int dy = tap / 3, dx = tap % 3;
#pragma unroll
      for (int kk = 0; kk < KC; kk += 16) {
        uint32_t af[2][4];
#pragma unroll
        for (int i = 0; i < 2; ++i) {
          const int hp = (pr[i] + dy) * kHaloW + pcl[i] + dx;
          ldsm_x4(hbase + (uint32_t)((hp * RH + kk + acol) * 2), af[i][0], af[i][1], af[i][2], af[i][3]);
        }
#pragma unroll
        for (int j = 0; j < NT; j += 2) {
          uint32_t b0, b1, b2, b3;
          ldsm_x4(wbase + (uint32_t)(((j * 8 + brow) * RW + tap * KC + kk + bcol) * 2), b0, b1, b2, b3);
#pragma unroll
          for (int i = 0; i < 2; ++i) {
            mma_bf16(acc[i][j], af[i][0], af[i][1], af[i][2], af[i][3], b0, b1);
            mma_bf16(acc[i][j + 1], af[i][0], af[i][1], af[i][2], af[i][3], b2, b3);
          }
        }
      }
    }
    __syncthreads();
  }
  cp_async_wait<0>();
#pragma unroll
  for (int i = 0; i < 2; ++i) {
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const int p = warp * 32 + i * 16 + (lane >> 2) + 8 * half;
      const int oy = y0 + p / kTW, ox = x0 + p % kTW;
      if (oy >= a.H || ox >= a.W) continue;
      const size_t base = (((size_t)n * a.H + oy) * a.W + ox) * a.cout;
#pragma unroll
      for (int j = 0; j < NT; ++j) {
        const int co = co0 + j * 8 + 2 * (lane & 3);
        if (co >= a.cout) continue;
        float v0 = acc[i][j][2 * half], v1 = acc[i][j][2 * half + 1];
        if (a.bias) {
          v0 += a.bias[co];
          v1 += a.bias[co + 1];
        }
        if (a.relu & 1) {
          v0 = fmaxf(v0, 0.f);
          v1 = fmaxf(v1, 0.f);
        }
        if (a.y) *reinterpret_cast<__nv_bfloat162*>(a.y + base + co) = __floats2bfloat162_rn(v0, v1);
        if (a.y32) {
          float2* d = reinterpret_cast<float2*>(a.y32 + base + co);
          if (a.relu & 2) {
            const float2 o = *d;
            v0 += o.x;
            v1 += o.y;
          }
          *d = make_float2(v0, v1);
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// FP8 (e4m3) inference variant of the halo kernel. Weights are stored FP8
// with one scale per output channel, after folding a per-input-channel
// activation scale into them: w8 = e4m3(w * sx[ci] / sw[co]). Activations
// stay BF16 in memory and are quantised on their way into shared memory,
// x8 = e4m3(x / sx[ci]) (saturating), so every other kernel is unchanged.
// The MMA is m16n8k32 e4m3 x e4m3 -> FP32; the epilogue multiplies by sw[co]
// before bias and ReLU. Chunks of 32 channels (32 bytes per pixel).
__device__ __forceinline__ void mma_e4m3(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k32.row.col.f32.e4m3.e4m3.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

struct Fp8ConvArgs {
  const bf16* x1;
  const bf16* x2;
  int c1, c2;
  const uint8_t* w8;         // [cout][9][cin] e4m3
  const float* wscale;       // [cout]
  const float* inv_xscale;   // [cin]: 1 / sx
  const float* bias;         // [cout] or null
  bf16* y;                   // [N][H][W][cout]
  int N, H, W, cout;
  int relu;
};

constexpr int kF8KC = 32;                 // channels (bytes) per chunk
constexpr int kF8RowHalo = kF8KC + 16;    // bytes per halo pixel row
constexpr int kF8RowW = 9 * kF8KC + 16;   // bytes per weight row
constexpr int kF8Pieces = kHaloPx * (kF8KC / 8);            // 8-channel halo pieces per chunk
constexpr int kF8PiecesPerThread = (kF8Pieces + 255) / 256;  // 3

template <int WN>
struct Fp8Cfg {
  static constexpr int BN = 16 * WN;
  static constexpr int kStageBytes = kHaloPx * kF8RowHalo + BN * kF8RowW;
  static constexpr size_t kSmem = 2 * (size_t)kStageBytes + 256 * sizeof(float);
};

template <int WN>
__global__ void __launch_bounds__(256) conv3x3_halo_fp8_kernel(Fp8ConvArgs a) {
  typedef Fp8Cfg<WN> Cfg;
  constexpr int BN = Cfg::BN;
  extern __shared__ __align__(128) uint8_t smem8[];
  float* s_inv = reinterpret_cast<float*>(smem8 + 2 * Cfg::kStageBytes);  // [256] >= cin
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp & 3, wn = warp >> 2;
  const int tiles_x = (a.W + kTW - 1) / kTW;
  const int x0 = (blockIdx.x % tiles_x) * kTW, y0 = (blockIdx.x / tiles_x) * kTH;
  const int n = blockIdx.y;
  const int co0 = blockIdx.z * BN;
  const int cin = a.c1 + a.c2;
  const int nchunks = (cin + kF8KC - 1) / kF8KC;
  const int H2 = a.H >> 1, W2 = a.W >> 1;
  for (int i = tid; i < 256; i += 256) s_inv[i] = i < cin ? a.inv_xscale[i] : 0.f;
  auto halo = [&](int st) { return smem8 + (size_t)st * Cfg::kStageBytes; };
  auto wts = [&](int st) { return smem8 + (size_t)st * Cfg::kStageBytes + kHaloPx * kF8RowHalo; };
  uint4 pre[kF8PiecesPerThread];
  auto fetch_halo = [&](int ch) {  // global BF16 pieces into registers
#pragma unroll
    for (int k = 0; k < kF8PiecesPerThread; ++k) {
      const int i = tid + k * 256;
      pre[k] = make_uint4(0, 0, 0, 0);
      if (i >= kF8Pieces) continue;
      const int hp = i / (kF8KC / 8), pc = i % (kF8KC / 8);
      const int yy = y0 - 1 + hp / kHaloW, xx = x0 - 1 + hp % kHaloW;
      const int ci = ch * kF8KC + pc * 8;
      if (yy < 0 || yy >= a.H || xx < 0 || xx >= a.W || ci >= cin) continue;
      const bf16* src = ci < a.c1 ? a.x1 + (((size_t)n * a.H + yy) * a.W + xx) * a.c1 + ci
                                  : a.x2 + (((size_t)n * H2 + (yy >> 1)) * W2 + (xx >> 1)) * a.c2 + (ci - a.c1);
      pre[k] = __ldg(reinterpret_cast<const uint4*>(src));
    }
  };
  auto store_halo = [&](int st, int ch) {  // quantise and store
    uint8_t* sh = halo(st);
#pragma unroll
    for (int k = 0; k < kF8PiecesPerThread; ++k) {
      const int i = tid + k * 256;
      if (i >= kF8Pieces) continue;
      const int hp = i / (kF8KC / 8), pc = i % (kF8KC / 8);
      const int ci = ch * kF8KC + pc * 8;
      const uint32_t w4[4] = {pre[k].x, pre[k].y, pre[k].z, pre[k].w};
      uint32_t q[2];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        uint32_t packed = 0;
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          const uint32_t wv = w4[h * 2 + e];
          const float2 f = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&wv));
          const int c = ci + h * 4 + e * 2;
          const float s0 = c < 256 ? s_inv[c] : 0.f, s1 = c + 1 < 256 ? s_inv[c + 1] : 0.f;
          const __nv_fp8x2_storage_t v = __nv_cvt_float2_to_fp8x2(make_float2(f.x * s0, f.y * s1), __NV_SATFINITE,
                                                                  __NV_E4M3);
          packed |= (uint32_t)v << (16 * e);
        }
        q[h] = packed;
      }
      *reinterpret_cast<uint2*>(sh + hp * kF8RowHalo + pc * 8) = make_uint2(q[0], q[1]);
    }
  };
  auto load_weights = [&](int st, int ch) {
    uint8_t* sw = wts(st);
    constexpr int kPieces = kF8KC / 16;  // 16-byte pieces per (co, tap)
    for (int i = tid; i < BN * 9 * kPieces; i += 256) {
      const int row = i / (9 * kPieces), r = i % (9 * kPieces);
      const int tap = r / kPieces, pc = r % kPieces;
      const int co = co0 + row, ci = ch * kF8KC + pc * 16;
      const bool ok = co < a.cout && ci < cin;
      const uint8_t* src = ok ? a.w8 + ((size_t)co * 9 + tap) * cin + ci : a.w8;
      cp_async16(sw + row * kF8RowW + tap * kF8KC + pc * 16, src, ok);
    }
  };
  float acc[2][WN][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < WN; ++j)
#pragma unroll
      for (int k = 0; k < 4; ++k) acc[i][j][k] = 0.f;
  int pr[2], pcl[2];
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const int m = wm * 32 + i * 16 + (lane & 7) + 8 * ((lane >> 3) & 1);
    pr[i] = m / kTW;
    pcl[i] = m % kTW;
  }
  const int acol = 16 * (lane >> 4);
  __syncthreads();  // s_inv
  fetch_halo(0);
  load_weights(0, 0);
  cp_async_commit();
  store_halo(0, 0);
  for (int ch = 0; ch < nchunks; ++ch) {
    const int st = ch & 1;
    const bool more = ch + 1 < nchunks;
    if (more) {
      load_weights(st ^ 1, ch + 1);
      fetch_halo(ch + 1);
    }
    cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();
    const uint32_t hbase = smem_u32(halo(st)), wbase = smem_u32(wts(st));
#pragma unroll
    for (int tap = 0; tap < 9; ++tap) {
      const int dy = tap / 3, dx = tap % 3;
      uint32_t af[2][4];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int hp = (pr[i] + dy) * kHaloW + pcl[i] + dx;
        ldsm_x4(hbase + (uint32_t)(hp * kF8RowHalo + acol), af[i][0], af[i][1], af[i][2], af[i][3]);
      }
#pragma unroll
      for (int j = 0; j < WN; ++j) {
        uint32_t b0, b1;
        const int row = wn * (8 * WN) + j * 8 + (lane & 7);
        ldsm_x2(wbase + (uint32_t)(row * kF8RowW + tap * kF8KC + 16 * ((lane >> 3) & 1)), b0, b1);
#pragma unroll
        for (int i = 0; i < 2; ++i) mma_e4m3(acc[i][j], af[i][0], af[i][1], af[i][2], af[i][3], b0, b1);
      }
    }
    __syncthreads();
    if (more) store_halo(st ^ 1, ch + 1);
  }
  cp_async_wait<0>();
#pragma unroll
  for (int i = 0; i < 2; ++i) {
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const int p = wm * 32 + i * 16 + (lane >> 2) + 8 * half;
      const int oy = y0 + p / kTW, ox = x0 + p % kTW;
      if (oy >= a.H || ox >= a.W) continue;
      const size_t base = (((size_t)n * a.H + oy) * a.W + ox) * a.cout;
#pragma unroll
      for (int j = 0; j < WN; ++j) {
        const int co = co0 + wn * (8 * WN) + j * 8 + 2 * (lane & 3);
        if (co >= a.cout) continue;
        float v0 = acc[i][j][2 * half] * a.wscale[co], v1 = acc[i][j][2 * half + 1] * a.wscale[co + 1];
        if (a.bias) {
          v0 += a.bias[co];
          v1 += a.bias[co + 1];
        }
        if (a.relu & 1) {
          v0 = fmaxf(v0, 0.f);
          v1 = fmaxf(v1, 0.f);
        }
        *reinterpret_cast<__nv_bfloat162*>(a.y + base + co) = __floats2bfloat162_rn(v0, v1);
      }
    }
  }
}

// Per-output-channel FP8 weights: sw[co] = max |w * sx| / 448 over the
// channel's 9 x cin weights, w8 = e4m3(w * sx / sw). One CTA per channel.
__global__ void quantize_weights_fp8_kernel(const float* __restrict__ w, const float* __restrict__ xscale, int cin,
                                            uint8_t* __restrict__ w8, float* __restrict__ wscale) {
  __shared__ float part[8];
  const int co = blockIdx.x, K = 9 * cin;
  const float* wr = w + (size_t)co * K;
  float m = 0.f;
  for (int i = threadIdx.x; i < K; i += blockDim.x) m = fmaxf(m, fabsf(wr[i] * xscale[i % cin]));
  for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = m;
  __syncthreads();
  float amax = 0.f;
  for (int k = 0; k < (int)(blockDim.x >> 5); ++k) amax = fmaxf(amax, part[k]);
  const float sw = amax > 0.f ? amax / 448.f : 1.f;
  if (threadIdx.x == 0) wscale[co] = sw;
  for (int i = threadIdx.x; i < K; i += blockDim.x)
    w8[(size_t)co * K + i] = (uint8_t)__nv_cvt_float_to_fp8(wr[i] * xscale[i % cin] / sw, __NV_SATFINITE, __NV_E4M3);
}

// amax[c] = max(amax[c], max over pixels |x[p][c]|) (non-negative floats
// compare as their bit patterns).
__global__ void channel_amax_kernel(const bf16* __restrict__ x, long pixels, int C, float* __restrict__ amax) {
  extern __shared__ float sm[];
  for (int c = threadIdx.x; c < C; c += blockDim.x) sm[c] = 0.f;
  __syncthreads();
  const long total = pixels * C;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const float v = fabsf(__bfloat162float(x[i]));
    atomicMax(reinterpret_cast<int*>(&sm[i % C]), __float_as_int(v));
  }
  __syncthreads();
  for (int c = threadIdx.x; c < C; c += blockDim.x) atomicMax(reinterpret_cast<int*>(&amax[c]), __float_as_int(sm[c]));
}

// dW[co][tap][ci] += sum over pixels of dY[p][co] * X[p + tap][ci]: one tap
// per CTA, 64 x 64 (co x ci) tile, 32-pixel K steps over a run of pixels.
struct WgradArgs {
  const bf16* dy;  // [N][H][W][cout]
  const bf16* x1;
  const bf16* x2;  // concat / upsampled second input, as in the forward
  int c1, c2;
  float* dw;  // [cout][9][c1 + c2] FP32, accumulated
  int N, H, W, cout;
  int pix_per_cta;
};
constexpr int kWM = 64, kWNt = 64, kWK = 32;
constexpr int kRowW = 64 + 8;  // bf16 per smem row (pad)

__global__ void __launch_bounds__(256) conv3x3_wgrad_kernel(WgradArgs a) {
  __shared__ __align__(128) bf16 sA[2][kWK * kRowW];  // [pixel][co]
  __shared__ __align__(128) bf16 sB[2][kWK * kRowW];  // [pixel][ci]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp & 1, wn = warp >> 1;  // 2 x 4 warps: 32 co x 16 ci each
  // blockIdx.x: tap + 9 x channel tile (consecutive CTAs read the same pixel
  // run: L2 reuse across the taps), blockIdx.y: pixel run
  const int tap = blockIdx.x % 9, tile = blockIdx.x / 9;
  const int dy = tap / 3 - 1, dx = tap % 3 - 1;
  const int ntile_ci = (a.c1 + a.c2 + kWNt - 1) / kWNt;
  const int co0 = (tile / ntile_ci) * kWM, ci0 = (tile % ntile_ci) * kWNt;
  const int cin = a.c1 + a.c2;
  const long P = (long)a.N * a.H * a.W;
  const long p_begin = (long)blockIdx.y * a.pix_per_cta;
  const long p_end = (p_begin + a.pix_per_cta < P) ? p_begin + a.pix_per_cta : P;
  const int H2 = a.H >> 1, W2 = a.W >> 1;
  // loads: 32 pixels x 64 channels = 256 x 16 B for each operand
  const int lp = tid >> 3, lc = (tid & 7) * 8;
  auto load = [&](int stage, long pb) {
    const long p = pb + lp;
    const bool pv = p < p_end;
    const long pp = pv ? p : 0;
    const int n = (int)(pp / ((long)a.H * a.W));
    const int rem = (int)(pp % ((long)a.H * a.W));
    const int y = rem / a.W, x = rem % a.W;
    {
      const int co = co0 + lc;
      const bool ok = pv && co < a.cout;
      const bf16* src = a.dy + (size_t)pp * a.cout + (ok ? co : 0);
      cp_async16(&sA[stage][lp * kRowW + lc], src, ok);
    }
    {
      const int ci = ci0 + lc;
      const int yy = y + dy, xx = x + dx;
      const bool ok = pv && ci < cin && yy >= 0 && yy < a.H && xx >= 0 && xx < a.W;
      const bf16* src = a.x1;
      if (ok) {
        if (ci < a.c1) src = a.x1 + (((size_t)n * a.H + yy) * a.W + xx) * a.c1 + ci;
        else src = a.x2 + (((size_t)n * H2 + (yy >> 1)) * W2 + (xx >> 1)) * a.c2 + (ci - a.c1);
      }
      cp_async16(&sB[stage][lp * kRowW + lc], src, ok);
    }
  };
  float acc[2][2][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
      for (int k = 0; k < 4; ++k) acc[i][j][k] = 0.f;
  if (p_begin < p_end) {
    load(0, p_begin);
    cp_async_commit();
    int stage = 0;
    for (long pb = p_begin; pb < p_end; pb += kWK) {
      if (pb + kWK < p_end) load(stage ^ 1, pb + kWK);
      cp_async_commit();
      cp_async_wait<1>();
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < kWK; kk += 16) {
        uint32_t af[2][4], bfr[2][2];
#pragma unroll
        for (int i = 0; i < 2; ++i) {  // A = dY^T: stored [pixel][co], transposed load
          const int prow = kk + (lane & 7) + 8 * (lane >> 4);
          const int col = wm * 32 + i * 16 + 8 * ((lane >> 3) & 1);
          ldsm_x4_t(smem_u32(&sA[stage][prow * kRowW + col]), af[i][0], af[i][1], af[i][2], af[i][3]);
        }
        {  // B = X: stored [pixel][ci], transposed load, two n8 tiles
          const int prow = kk + (lane & 7) + 8 * ((lane >> 3) & 1);
          const int col = wn * 16 + 8 * (lane >> 4);
          uint32_t r0, r1, r2, r3;
          ldsm_x4_t(smem_u32(&sB[stage][prow * kRowW + col]), r0, r1, r2, r3);
          bfr[0][0] = r0;
          bfr[0][1] = r1;
          bfr[1][0] = r2;
          bfr[1][1] = r3;
        }
#pragma unroll
        for (int i = 0; i < 2; ++i)
#pragma unroll
          for (int j = 0; j < 2; ++j) mma_bf16(acc[i][j], af[i][0], af[i][1], af[i][2], af[i][3], bfr[j][0], bfr[j][1]);
      }
      __syncthreads();
      stage ^= 1;
    }
    cp_async_wait<0>();
  }
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const int co = co0 + wm * 32 + i * 16 + (lane >> 2) + 8 * half;
      if (co >= a.cout) continue;
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const int ci = ci0 + wn * 16 + j * 8 + 2 * (lane & 3);
        if (ci >= cin) continue;
        float* d = a.dw + ((size_t)co * 9 + tap) * cin + ci;
        atomicAdd(d, acc[i][j][2 * half]);
        atomicAdd(d + 1, acc[i][j][2 * half + 1]);
      }
    }
}

// wt[ci][tap'][co] = w[co][8 - tap'][ci]: the backward-data weights.
__global__ void flip_weights_kernel(const bf16* __restrict__ w, bf16* __restrict__ wt, int cout, int cin) {
  const long total = (long)cout * 9 * cin;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const int ci = (int)(i % cin);
    const int tap = (int)((i / cin) % 9);
    const int co = (int)(i / ((long)cin * 9));
    wt[((size_t)ci * 9 + (8 - tap)) * cout + co] = w[i];
  }
}

}  // namespace nn
}  // namespace pbrt

using namespace pbrt;
using namespace pbrt::nn;

namespace {
template <int WN> void launch_fwd(const ConvArgs& a, cudaStream_t s) {
  constexpr int BN = 16 * WN;
  dim3 grid(((a.W + kTW - 1) / kTW) * ((a.H + kTH - 1) / kTH), a.N, (a.cout + BN - 1) / BN);
  conv3x3_fwd_kernel<WN><<<grid, 256, 0, s>>>(a);
}
template <int WN, int KC> int launch_halo(const ConvArgs& a, cudaStream_t s) {
  typedef HaloCfg<WN, KC> Cfg;
  static PerDeviceOnce attrs;
  int ast = once_per_device(attrs, [&]() -> int {
    cudaError_t e = cudaFuncSetAttribute(conv3x3_halo_kernel<WN, KC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)Cfg::kSmem);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(conv3x3_halo_kernel)");
    return PBRT_OK;
  });
  if (ast) return ast;
  dim3 grid(((a.W + kTW - 1) / kTW) * ((a.H + kTH - 1) / kTH), a.N, (a.cout + Cfg::BN - 1) / Cfg::BN);
  conv3x3_halo_kernel<WN, KC><<<grid, 256, Cfg::kSmem, s>>>(a);
  return PBRT_OK;
}
template <int NT, int KC> int launch_halo_m(const ConvArgs& a, cudaStream_t s) {
  typedef HaloMCfg<NT, KC> Cfg;
  static PerDeviceOnce attrs;
  int ast = once_per_device(attrs, [&]() -> int {
    cudaError_t e = cudaFuncSetAttribute(conv3x3_halo_m_kernel<NT, KC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)Cfg::kSmem);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(conv3x3_halo_m_kernel)");
    return PBRT_OK;
  });
  if (ast) return ast;
  dim3 grid(((a.W + kTW - 1) / kTW) * ((a.H + kMTH - 1) / kMTH), a.N, (a.cout + Cfg::BN - 1) / Cfg::BN);
  conv3x3_halo_m_kernel<NT, KC><<<grid, 256, Cfg::kSmem, s>>>(a);
  return PBRT_OK;
}
// Wide channel chunks (fewer barriers) while the weight slab stays small.
template <int WN> int launch_halo_for(const ConvArgs& a, cudaStream_t s) {
  if constexpr (WN <= 4) {
    if (a.c1 + a.c2 <= 16) return launch_halo<WN, 16>(a, s);  // one 16-channel chunk: no zero half
    return launch_halo<WN, 32>(a, s);
  } else {
    return launch_halo<WN, 16>(a, s);
  }
}
template <int WN> int launch_fp8(const Fp8ConvArgs& a, cudaStream_t s) {
  typedef Fp8Cfg<WN> Cfg;
  static PerDeviceOnce attrs;
  int ast = once_per_device(attrs, [&]() -> int {
    cudaError_t e = cudaFuncSetAttribute(conv3x3_halo_fp8_kernel<WN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)Cfg::kSmem);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(conv3x3_halo_fp8_kernel)");
    return PBRT_OK;
  });
  if (ast) return ast;
  dim3 grid(((a.W + kTW - 1) / kTW) * ((a.H + kTH - 1) / kTH), a.N, (a.cout + Cfg::BN - 1) / Cfg::BN);
  conv3x3_halo_fp8_kernel<WN><<<grid, 256, Cfg::kSmem, s>>>(a);
  return PBRT_OK;
}
}  // namespace

extern "C" {

PBRT_API int pbrt_nn_conv3x3(const void* x1, int32_t c1, const void* x2, int32_t c2, const void* w, const float* bias,
                             void* y, float* y32, int32_t n, int32_t h, int32_t wd, int32_t cout, int32_t relu,
                             pbrt_stream_t stream) {
  if (!x1 || !w || (!y && !y32) || ((relu & 2) && !y32) || c1 <= 0 || c1 % 16 || c2 < 0 || c2 % 16 || (c2 && !x2) || cout <= 0 || cout % 16 || n <= 0 ||
      h <= 0 || wd <= 0 || (c2 && (h % 2 || wd % 2)))
    return fail(PBRT_ERROR_INVALID_ARGUMENT,
                "nn conv3x3: channels must be multiples of 16 (c1 %d, c2 %d, cout %d); an upsampled second input "
                "needs even sizes",
                c1, c2, cout);
  ConvArgs a{(const bf16*)x1, (const bf16*)x2, c1, c2, (const bf16*)w, bias, (bf16*)y, y32, n, h, wd, cout, relu};
  // one n-tile of up to 128 channels; larger outputs split in two
  int bn = cout <= 128 ? cout : (cout / 2 <= 128 && (cout / 2) % 16 == 0 ? cout / 2 : 128);
  if (relu & 4) {  // the per-(tap, 16-channel) pipelined kernel
    switch (bn / 16) {
      case 1: launch_fwd<1>(a, stream); break;
      case 2: launch_fwd<2>(a, stream); break;
      case 3: launch_fwd<3>(a, stream); break;
      case 4: launch_fwd<4>(a, stream); break;
      case 5: launch_fwd<5>(a, stream); break;
      case 6: launch_fwd<6>(a, stream); break;
      case 7: launch_fwd<7>(a, stream); break;
      default: launch_fwd<8>(a, stream); break;
    }
    return check_launch("conv3x3_fwd_kernel");
  }
  int st;
  if ((relu & 8) == 0 && cout <= 48) {  // wide-tile kernel for narrow outputs (measured faster up to 48)
    const bool k16 = c1 + c2 <= 16;
    switch (cout / 16) {
      case 1: st = k16 ? launch_halo_m<2, 16>(a, stream) : launch_halo_m<2, 32>(a, stream); break;
      case 2: st = k16 ? launch_halo_m<4, 16>(a, stream) : launch_halo_m<4, 32>(a, stream); break;
      case 3: st = k16 ? launch_halo_m<6, 16>(a, stream) : launch_halo_m<6, 32>(a, stream); break;
      default: st = k16 ? launch_halo_m<8, 16>(a, stream) : launch_halo_m<8, 32>(a, stream); break;
    }
    if (st) return st;
    return check_launch("conv3x3_halo_m_kernel");
  }
  switch (bn / 16) {
    case 1: st = launch_halo_for<1>(a, stream); break;
    case 2: st = launch_halo_for<2>(a, stream); break;
    case 3: st = launch_halo_for<3>(a, stream); break;
    case 4: st = launch_halo_for<4>(a, stream); break;
    case 5: st = launch_halo_for<5>(a, stream); break;
    case 6: st = launch_halo_for<6>(a, stream); break;
    case 7: st = launch_halo_for<7>(a, stream); break;
    default: st = launch_halo_for<8>(a, stream); break;
  }
  if (st) return st;
  return check_launch("conv3x3_halo_kernel");
}

PBRT_API int pbrt_nn_conv3x3_wgrad(const void* dy, const void* x1, int32_t c1, const void* x2, int32_t c2, float* dw,
                                   int32_t n, int32_t h, int32_t wd, int32_t cout, pbrt_stream_t stream) {
  if (!dy || !x1 || !dw || c1 <= 0 || c1 % 16 || c2 < 0 || c2 % 16 || (c2 && !x2) || cout <= 0 || cout % 16)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "nn conv3x3 wgrad: bad arguments");
  WgradArgs a{(const bf16*)dy, (const bf16*)x1, (const bf16*)x2, c1, c2, dw, n, h, wd, cout, 0};
  const long P = (long)n * h * wd;
  const int tiles = ((cout + kWM - 1) / kWM) * ((c1 + c2 + kWNt - 1) / kWNt);
  // enough CTAs to fill the GPU: pixel runs of a multiple of 32
  long chunks = std::max(1L, std::min(P / 2048, (long)(152 * 8 * 4) / (9 * tiles) + 1));
  long ppc = (P + chunks - 1) / chunks;
  ppc = (ppc + kWK - 1) / kWK * kWK;
  a.pix_per_cta = (int)ppc;
  dim3 grid((unsigned)(9 * tiles), (unsigned)((P + ppc - 1) / ppc));
  conv3x3_wgrad_kernel<<<grid, 256, 0, stream>>>(a);
  return check_launch("conv3x3_wgrad_kernel");
}

PBRT_API int pbrt_nn_conv3x3_fp8(const void* x1, int32_t c1, const void* x2, int32_t c2, const void* w8,
                                 const float* wscale, const float* inv_xscale, const float* bias, void* y, int32_t n,
                                 int32_t h, int32_t wd, int32_t cout, int32_t flags, pbrt_stream_t stream) {
  if (!x1 || !w8 || !wscale || !inv_xscale || !y || c1 <= 0 || c1 % 16 || c2 < 0 || c2 % 16 || (c2 && !x2) ||
      c1 + c2 > 256 || cout <= 0 || cout % 16 || n <= 0 || h <= 0 || wd <= 0 || (c2 && (h % 2 || wd % 2)))
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "nn conv3x3 fp8: bad arguments (c1 %d, c2 %d, cout %d)", c1, c2, cout);
  // the tcgen05 form where it applies (flags bit 3: this kernel only)
  if (!(flags & 8) && cout <= 128 && nn_fp8_umma_fits(x1, c1, x2, c2, w8, cout, h, wd, false))
    return pbrt_nn_conv3x3_fp8_umma(x1, c1, x2, c2, w8, wscale, inv_xscale, bias, y, nullptr, n, h, wd, cout,
                                    flags & 17, stream);
  Fp8ConvArgs a{(const bf16*)x1, (const bf16*)x2, c1, c2, (const uint8_t*)w8, wscale, inv_xscale, bias, (bf16*)y,
                n, h, wd, cout, flags & 1};
  const int bn = cout <= 128 ? cout : (cout / 2 <= 128 && (cout / 2) % 16 == 0 ? cout / 2 : 128);
  int st;
  switch (bn / 16) {
    case 1: st = launch_fp8<1>(a, stream); break;
    case 2: st = launch_fp8<2>(a, stream); break;
    case 3: st = launch_fp8<3>(a, stream); break;
    case 4: st = launch_fp8<4>(a, stream); break;
    case 5: st = launch_fp8<5>(a, stream); break;
    case 6: st = launch_fp8<6>(a, stream); break;
    case 7: st = launch_fp8<7>(a, stream); break;
    default: st = launch_fp8<8>(a, stream); break;
  }
  if (st) return st;
  return check_launch("conv3x3_halo_fp8_kernel");
}

PBRT_API int pbrt_nn_quantize_weights_fp8(const float* w, const float* xscale, int32_t cout, int32_t cin, void* w8,
                                          float* wscale, pbrt_stream_t stream) {
  if (!w || !xscale || !w8 || !wscale || cout <= 0 || cin <= 0)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "quantize weights fp8: bad arguments");
  quantize_weights_fp8_kernel<<<cout, 256, 0, stream>>>(w, xscale, cin, (uint8_t*)w8, wscale);
  return check_launch("quantize_weights_fp8_kernel");
}

PBRT_API int pbrt_nn_channel_amax(const void* x, int64_t pixels, int32_t c, float* amax, pbrt_stream_t stream) {
  if (!x || !amax || c <= 0 || c > 1024 || pixels < 0) return fail(PBRT_ERROR_INVALID_ARGUMENT, "channel amax");
  const long total = (long)pixels * c;
  const int grid = (int)std::max<long>(1, std::min<long>((total + 255) / 256, 152L * 8));
  channel_amax_kernel<<<grid, 256, c * sizeof(float), stream>>>((const bf16*)x, (long)pixels, c, amax);
  return check_launch("channel_amax_kernel");
}

PBRT_API int pbrt_nn_flip_weights(const void* w, void* wt, int32_t cout, int32_t cin, pbrt_stream_t stream) {
  if (!w || !wt || cout <= 0 || cin <= 0) return fail(PBRT_ERROR_INVALID_ARGUMENT, "nn flip weights: bad arguments");
  flip_weights_kernel<<<256, 256, 0, stream>>>((const bf16*)w, (bf16*)wt, cout, cin);
  return check_launch("flip_weights_kernel");
}

}  // extern "C"
