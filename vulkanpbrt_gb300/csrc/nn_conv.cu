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
  int relu;            // bit 0: ReLU; bit 1: add into y32 instead of overwriting
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
  const int tap = blockIdx.y;
  const int dy = tap / 3 - 1, dx = tap % 3 - 1;
  const int ntile_ci = (a.c1 + a.c2 + kWNt - 1) / kWNt;
  const int co0 = (blockIdx.z / ntile_ci) * kWM, ci0 = (blockIdx.z % ntile_ci) * kWNt;
  const int cin = a.c1 + a.c2;
  const long P = (long)a.N * a.H * a.W;
  const long p_begin = (long)blockIdx.x * a.pix_per_cta;
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
  dim3 grid((unsigned)((P + ppc - 1) / ppc), 9, tiles);
  conv3x3_wgrad_kernel<<<grid, 256, 0, stream>>>(a);
  return check_launch("conv3x3_wgrad_kernel");
}

PBRT_API int pbrt_nn_flip_weights(const void* w, void* wt, int32_t cout, int32_t cin, pbrt_stream_t stream) {
  if (!w || !wt || cout <= 0 || cin <= 0) return fail(PBRT_ERROR_INVALID_ARGUMENT, "nn flip weights: bad arguments");
  flip_weights_kernel<<<256, 256, 0, stream>>>((const bf16*)w, (bf16*)wt, cout, cin);
  return check_launch("flip_weights_kernel");
}

}  // extern "C"
