// 3x3 convolution forward on the 5th-generation tensor cores (tcgen05): an
// implicit GEMM with the accumulator in tensor memory. One CTA (4 warps)
// computes a 16 x 8-pixel output tile (M = 128) for N = Cout <= 128 output
// channels. Per chunk of up to 32 input channels the CTA stages, with
// cp.async, the 18 x 10 input halo and the 9 x chunk x N weight slab in
// shared memory in the K-major "interleaved" layout of the MMA's matrix
// descriptors (8 x 16-byte core matrices): the halo is stored as planes of
// 8 channels, pixel rows of the halo 10 pixels apart, so the A operand of
// every tap is the same descriptor with its start address shifted by the
// tap's pixel offset (stride between 8-pixel row groups = one halo row).
// Thread 0 issues 9 x chunk/16 MMAs (kind::f16, BF16 x BF16 -> FP32) per
// chunk and commits them to an mbarrier, which gates the reuse of the
// stage two chunks later; the epilogue reads the accumulator with
// tcgen05.ld (each warp its 32 TMEM lanes = 32 pixels), adds the bias,
// applies ReLU and stores BF16. Every wait is bounded: on a timeout the
// kernel records an error (pbrt_nn_umma_status), waits again for its own
// MMAs, frees its tensor memory and returns.
#include <cuda.h>  // CUtensorMap (the encoder is fetched through the runtime)
#include <cuda_bf16.h>
#include <cuda_fp8.h>

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>

#include "internal.hpp"

namespace pbrt {
namespace nn {

typedef __nv_bfloat16 bf16;

__device__ uint32_t g_umma_error = 0;

namespace umma {

constexpr int kTileH = 16, kTileW = 8, kM = kTileH * kTileW;  // 128 pixels
constexpr int kHaloH = kTileH + 2, kHaloW = kTileW + 2, kHaloPx = kHaloH * kHaloW;  // 180
constexpr int kKC = 32;                    // input channels per chunk
constexpr int kPlanes = kKC / 8;           // 8-channel planes per chunk
constexpr int kPlaneBytes = kHaloPx * 16;  // one plane of the halo: 2880 B
// the half-resolution second input under a halo: 6 x 10 pixels a plane
constexpr int kStgW = kTileW / 2 + 2, kStgH = kTileH / 2 + 2;
constexpr int kStgPlaneBytes = kStgW * kStgH * 16;  // 960 B

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void cp16(uint32_t dst, const void* src, bool valid) {
  const int n = valid ? 16 : 0;
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(n));
}

// Shared-memory matrix descriptor, K-major, no swizzle: start address,
// leading (K-direction) and stride (M/N-direction) core-matrix offsets, in
// 16-byte units; version 1.
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo_bytes, uint32_t sbo_bytes) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3fffu);
  d |= (uint64_t)((lbo_bytes >> 4) & 0x3fffu) << 16;
  d |= (uint64_t)((sbo_bytes >> 4) & 0x3fffu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Shared-memory matrix descriptor, K-major, swizzled rows of `row_bytes`
// (32, 64 or 128: one pixel of 16, 32 or 64 BF16 channels, as a TMA with
// the same swizzle writes it): the stride between groups of 8 rows; the
// leading offset is unused (a K step of 16 elements stays inside a row and
// moves the start by 32 bytes). The swizzle is a function of the address
// bits, so a start shifted by whole rows (the taps) needs no base offset.
__device__ __forceinline__ uint64_t sdesc_sw(uint32_t addr, uint32_t sbo_bytes, uint32_t row_bytes) {
  const uint64_t layout = row_bytes == 128 ? 2u : (row_bytes == 64 ? 4u : 6u);
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3fffu);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)((sbo_bytes >> 4) & 0x3fffu) << 32;
  d |= (uint64_t)1 << 46;
  d |= layout << 61;
  return d;
}

// Instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, M = 128, N = n.
__host__ __device__ constexpr uint32_t idesc_bf16(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kM >> 4) << 24);
}

// Instruction descriptor, kind::f8f6f4: FP32 accumulator, E4M3 A and B
// (format code 0), both K-major, M = 128, N = n. K = 32 per instruction.
__host__ __device__ constexpr uint32_t idesc_e4m3(int n) {
  return (1u << 4) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kM >> 4) << 24);
}

// One tcgen05.mma with A and B in shared memory; accumulate = false
// overwrites D. kF8: kind::f8f6f4 (E4M3), else kind::f16 (BF16).
template <bool kF8>
__device__ __forceinline__ void mma_ss(uint32_t d, uint64_t da, uint64_t db, uint32_t idesc, bool accumulate) {
  if constexpr (kF8)
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
        "l"(da), "l"(db), "r"(idesc), "r"((uint32_t)accumulate));
  else
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
        "l"(da), "l"(db), "r"(idesc), "r"((uint32_t)accumulate));
}

__device__ __forceinline__ void mbar_init(uint32_t addr, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(addr), "r"(count));
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t addr, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(addr), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait for an mbarrier phase: false after ~2 s.
__device__ __forceinline__ bool mbar_wait(uint32_t addr, uint32_t parity) {
  if (mbar_try_wait(addr, parity)) return true;
  const unsigned long long t0 = now_ns();
  while (true) {
    if (mbar_try_wait(addr, parity)) return true;
    if (now_ns() - t0 > 2000000000ull) return false;
  }
}

}  // namespace umma

struct UmmaConvArgs {
  const bf16* x1;
  const bf16* x2;
  int c1, c2;
  const bf16* w;       // [cout][9][c1 + c2]
  const float* bias;   // [cout] or null
  bf16* y;             // [N][H][W][cout]
  int N, H, W, cout;
  int relu;
  bf16* pooled = nullptr;  // [N][H/2][W/2][cout]: 2x2 average of y (warp-specialised kernel only)
  // FP8 form of the warp-specialised kernel: e4m3 weights [cout][9][c1 + c2]
  // with one scale per output channel, and the per-input-channel scales
  // that quantise the BF16 activations on their way into shared memory
  const uint8_t* w8 = nullptr;
  const float* wscale = nullptr;      // [cout]
  const float* inv_xscale = nullptr;  // [c1 + c2]
  // FP32 output instead of y (warp-specialised BF16 kernel only): pixel p's
  // channels at y32[p * ldy32 .. + cout)
  float* y32 = nullptr;
  int ldy32 = 0;
};

template <int NC>  // output channels (= MMA N), multiple of 16, <= 128
__global__ void __launch_bounds__(128) conv3x3_umma_kernel(UmmaConvArgs a) {
  using namespace umma;
  constexpr int kWBytes = 9 * kPlanes * NC * 16;          // weight slab per stage
  constexpr int kStage = kPlanes * kPlaneBytes + kWBytes;  // halo + weights
  constexpr uint32_t kCols = NC <= 32 ? 32 : (NC <= 64 ? 64 : 128);
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ uint32_t tmem_base_slot;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int tiles_x = (a.W + kTileW - 1) / kTileW;
  const int x0 = (blockIdx.x % tiles_x) * kTileW, y0 = (blockIdx.x / tiles_x) * kTileH;
  const int n = blockIdx.y;
  const int cin = a.c1 + a.c2;
  const int nchunks = (cin + kKC - 1) / kKC;
  const int H2 = a.H >> 1, W2 = a.W >> 1;
  const uint32_t sbase = smem_addr(smem);
  const uint32_t mb0 = smem_addr(&mbar[0]), mb1 = smem_addr(&mbar[1]);

  if (tid == 0) {
    umma::mbar_init(mb0, 1);
    umma::mbar_init(mb1, 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     smem_addr(&tmem_base_slot)),
                 "r"(kCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_base_slot;

  auto load_chunk = [&](int st, int ch) {
    const uint32_t hb = sbase + st * kStage, wb = hb + kPlanes * kPlaneBytes;
    const int c0 = ch * kKC;
    for (int i = tid; i < kHaloPx * kPlanes; i += 128) {
      const int hp = i % kHaloPx, p = i / kHaloPx;
      const int yy = y0 - 1 + hp / kHaloW, xx = x0 - 1 + hp % kHaloW;
      const int ci = c0 + p * 8;
      const bool ok = yy >= 0 && yy < a.H && xx >= 0 && xx < a.W && ci < cin;
      const bf16* src = a.x1;
      if (ok) {
        if (ci < a.c1) src = a.x1 + (((size_t)n * a.H + yy) * a.W + xx) * a.c1 + ci;
        else src = a.x2 + (((size_t)n * H2 + (yy >> 1)) * W2 + (xx >> 1)) * a.c2 + (ci - a.c1);
      }
      umma::cp16(hb + p * kPlaneBytes + hp * 16, src, ok);
    }
    for (int i = tid; i < NC * 9 * kPlanes; i += 128) {
      const int co = i % NC, r = i / NC;
      const int p = r % kPlanes, tap = r / kPlanes;
      const int ci = c0 + p * 8;
      const bool ok = co < a.cout && ci < cin;
      const bf16* src = ok ? a.w + ((size_t)co * 9 + tap) * cin + ci : a.w;
      umma::cp16(wb + ((tap * kPlanes + p) * NC + co) * 16, src, ok);
    }
  };

  bool failed = false;
  load_chunk(0, 0);
  asm volatile("cp.async.commit_group;\n" ::);
  for (int ch = 0; ch < nchunks && !failed; ++ch) {
    const int st = ch & 1;
    if (ch + 1 < nchunks) {
      const int s1 = (ch + 1) & 1;
      bool ok = true;
      if (ch + 1 >= 2) ok = umma::mbar_wait(s1 ? mb1 : mb0, (uint32_t)(((ch - 1) >> 1) & 1));
      if (__syncthreads_or(!ok)) {  // the same decision in every thread
        failed = true;
        break;
      }
      load_chunk(s1, ch + 1);
    }
    asm volatile("cp.async.commit_group;\n" ::);
    asm volatile("cp.async.wait_group 1;\n" ::);
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      const uint32_t hb = sbase + st * kStage, wb = hb + kPlanes * kPlaneBytes;
      const int kc = cin - ch * kKC < kKC ? cin - ch * kKC : kKC;  // 16 or 32
      constexpr uint32_t idesc = umma::idesc_bf16(NC);
#pragma unroll 1
      for (int tap = 0; tap < 9; ++tap) {
        const int dy = tap / 3, dx = tap % 3;
        for (int ks = 0; ks < kc / 16; ++ks) {
          const uint64_t da =
              umma::sdesc(hb + (2 * ks) * kPlaneBytes + (dy * kHaloW + dx) * 16, kPlaneBytes, kHaloW * 16);
          const uint64_t db = umma::sdesc(wb + ((tap * kPlanes + 2 * ks) * NC) * 16, NC * 16, 8 * 16);
          const uint32_t acc = (ch > 0 || tap > 0 || ks > 0) ? 1u : 0u;
          asm volatile(
              "{\n\t.reg .pred p;\n\t"
              "setp.ne.b32 p, %4, 0;\n\t"
              "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
              "l"(da), "l"(db), "r"(idesc), "r"(acc));
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                       st ? mb1 : mb0)
                   : "memory");
    }
  }
  asm volatile("cp.async.wait_group 0;\n" ::);
  // all MMAs issued so far complete before the accumulator is read or freed
  const int last = nchunks - 1;
  bool done = umma::mbar_wait((last & 1) ? mb1 : mb0, (uint32_t)((last >> 1) & 1));
  if (!done) done = umma::mbar_wait((last & 1) ? mb1 : mb0, (uint32_t)((last >> 1) & 1));  // once more, bounded
  failed = __syncthreads_or(failed || !done);
  if (failed) {
    if (tid == 0) atomicOr(&g_umma_error, 1u);
  } else {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const int m = warp * 32 + lane;  // TMEM lane = pixel of the tile
    const int oy = y0 + m / kTileW, ox = x0 + m % kTileW;
    const bool inside = oy < a.H && ox < a.W;
    bf16* dst = a.y + (((size_t)n * a.H + (inside ? oy : 0)) * a.W + (inside ? ox : 0)) * a.cout;
#pragma unroll
    for (int c0 = 0; c0 < NC; c0 += 16) {
      uint32_t v[16];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
      if (inside) {
        uint32_t packed[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          float f0 = __uint_as_float(v[2 * j]), f1 = __uint_as_float(v[2 * j + 1]);
          if (a.bias) {
            f0 += a.bias[c0 + 2 * j];
            f1 += a.bias[c0 + 2 * j + 1];
          }
          if (a.relu & 1) {
            f0 = fmaxf(f0, 0.f);
            f1 = fmaxf(f1, 0.f);
          }
          const __nv_bfloat162 b2 = __floats2bfloat162_rn(f0, f1);
          packed[j] = *reinterpret_cast<const uint32_t*>(&b2);
        }
        uint4* d4 = reinterpret_cast<uint4*>(dst + c0);
        d4[0] = make_uint4(packed[0], packed[1], packed[2], packed[3]);
        d4[1] = make_uint4(packed[4], packed[5], packed[6], packed[7]);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kCols));
  }
}

// Persistent form for the large-image layers: the whole weight tensor
// (9 x Cin x N) stays in shared memory for the CTA's lifetime, and the CTA
// walks output tiles with a two-deep pipeline: while the tensor cores work
// on tile i (accumulator buffer i&1 in tensor memory), the CTA loads tile
// i+1's halo (all Cin channels) into the other halo buffer and drains tile
// i-1's accumulator (bias, ReLU, BF16 stores). Used when the weights and two
// halos fit in shared memory.
// With use_tma, the x1 part of each halo comes in one TMA load (x1 viewed as
// a 5-D tensor [8 channels][x][y][channel group][image], box
// [8][10][18][c1/8][1]: exactly the plane layout, out-of-image pixels filled
// with zeros) that completes on a per-buffer mbarrier; the upsampled x2 part
// is still gathered with cp.async.
template <int NC>
__global__ void __launch_bounds__(128) conv3x3_umma_persistent_kernel(UmmaConvArgs a, int tiles_per_image,
                                                                      const __grid_constant__ CUtensorMap x1map,
                                                                      int use_tma) {
  using namespace umma;
  constexpr uint32_t kCols = 2 * NC <= 64 ? 64 : (2 * NC <= 128 ? 128 : 256);
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ __align__(8) uint64_t tbar[2];  // TMA arrival per halo buffer
  __shared__ uint32_t tmem_base_slot;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int cin = a.c1 + a.c2, planes = cin / 8;
  const int halo_bytes = planes * kPlaneBytes;
  const int tiles_x = (a.W + kTileW - 1) / kTileW;
  const int total_tiles = tiles_per_image * a.N;
  const int H2 = a.H >> 1, W2 = a.W >> 1;
  const uint32_t sbase = smem_addr(smem);
  const uint32_t wbase = sbase;
  const uint32_t hbase0 = (sbase + 9 * planes * NC * 16 + 1023u) & ~1023u;
  const uint32_t hbase1 = (hbase0 + halo_bytes + 1023u) & ~1023u;
  const uint32_t mb0 = smem_addr(&mbar[0]), mb1 = smem_addr(&mbar[1]);
  const uint32_t tb0 = smem_addr(&tbar[0]), tb1 = smem_addr(&tbar[1]);
  const int x1_planes = use_tma ? a.c1 / 8 : 0;  // planes the TMA load fills
  if (tid == 0) {
    umma::mbar_init(mb0, 1);
    umma::mbar_init(mb1, 1);
    umma::mbar_init(tb0, 1);
    umma::mbar_init(tb1, 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     smem_addr(&tmem_base_slot)),
                 "r"(kCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_base_slot;

  // weights, once: [tap][plane][n][8 channels]
  for (int i = tid; i < NC * 9 * planes; i += 128) {
    const int co = i % NC, r = i / NC;
    const int p = r % planes, tap = r / planes;
    umma::cp16(wbase + ((tap * planes + p) * NC + co) * 16, a.w + ((size_t)co * 9 + tap) * cin + p * 8, true);
  }
  auto tile_origin = [&](int t, int& img, int& x0, int& y0) {
    img = t / tiles_per_image;
    const int r = t % tiles_per_image;
    x0 = (r % tiles_x) * kTileW;
    y0 = (r / tiles_x) * kTileH;
  };
  auto load_halo = [&](uint32_t hb, int t) {
    int img, x0, y0;
    tile_origin(t, img, x0, y0);
    if (x1_planes && tid == 0) {
      const uint32_t tb = hb == hbase0 ? tb0 : tb1;
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(tb),
                   "r"((uint32_t)(x1_planes * kPlaneBytes))
                   : "memory");
      asm volatile(
          "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, "
          "%6}], [%7];\n" ::"r"(hb),
          "l"(reinterpret_cast<uint64_t>(&x1map)), "r"(0), "r"(x0 - 1), "r"(y0 - 1), "r"(0), "r"(img), "r"(tb)
          : "memory");
    }
    for (int i = tid + x1_planes * kHaloPx; i < kHaloPx * planes; i += 128) {
      const int hp = i % kHaloPx, p = i / kHaloPx;
      const int yy = y0 - 1 + hp / kHaloW, xx = x0 - 1 + hp % kHaloW;
      const int ci = p * 8;
      const bool ok = yy >= 0 && yy < a.H && xx >= 0 && xx < a.W;
      const bf16* src = a.x1;
      if (ok) {
        if (ci < a.c1) src = a.x1 + (((size_t)img * a.H + yy) * a.W + xx) * a.c1 + ci;
        else src = a.x2 + (((size_t)img * H2 + (yy >> 1)) * W2 + (xx >> 1)) * a.c2 + (ci - a.c1);
      }
      umma::cp16(hb + p * kPlaneBytes + hp * 16, src, ok);
    }
  };
  auto epilogue = [&](int t, uint32_t buf) {
    int img, x0, y0;
    tile_origin(t, img, x0, y0);
    const int m = warp * 32 + lane;
    const int oy = y0 + m / kTileW, ox = x0 + m % kTileW;
    const bool inside = oy < a.H && ox < a.W;
    bf16* dst = a.y + (((size_t)img * a.H + (inside ? oy : 0)) * a.W + (inside ? ox : 0)) * a.cout;
#pragma unroll
    for (int c0 = 0; c0 < NC; c0 += 16) {
      uint32_t v[16];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + buf * NC + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
      if (inside) {
        uint32_t packed[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          float f0 = __uint_as_float(v[2 * j]), f1 = __uint_as_float(v[2 * j + 1]);
          if (a.bias) {
            f0 += a.bias[c0 + 2 * j];
            f1 += a.bias[c0 + 2 * j + 1];
          }
          if (a.relu & 1) {
            f0 = fmaxf(f0, 0.f);
            f1 = fmaxf(f1, 0.f);
          }
          const __nv_bfloat162 b2 = __floats2bfloat162_rn(f0, f1);
          packed[j] = *reinterpret_cast<const uint32_t*>(&b2);
        }
        uint4* d4 = reinterpret_cast<uint4*>(dst + c0);
        d4[0] = make_uint4(packed[0], packed[1], packed[2], packed[3]);
        d4[1] = make_uint4(packed[4], packed[5], packed[6], packed[7]);
      }
    }
  };

  bool failed = false;
  int i = 0, mma_issued = -1;  // index of the last tile whose MMAs were issued
  int t = blockIdx.x;
  if (t < total_tiles) load_halo(hbase0, t);
  asm volatile("cp.async.commit_group;\n" ::);  // weights + first halo
  for (; t < total_tiles; t += gridDim.x, ++i) {
    const uint32_t b = (uint32_t)(i & 1);
    const uint32_t hb = b ? hbase1 : hbase0;
    asm volatile("cp.async.wait_group 0;\n" ::);
    if (x1_planes) {  // halo i's TMA load: the (i >> 1)-th completion on this buffer's barrier
      const bool ok = umma::mbar_wait(b ? tb1 : tb0, (uint32_t)((i >> 1) & 1));
      if (__syncthreads_or(!ok)) {
        umma::mbar_wait(b ? tb1 : tb0, (uint32_t)((i >> 1) & 1));  // the copy in flight, once more
        failed = true;
        break;
      }
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();  // halo i in place; accumulator buffer b drained (epilogue of tile i-2)
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      constexpr uint32_t idesc = umma::idesc_bf16(NC);
      const uint32_t d = tmem + b * NC;
      // descriptors advance by constants (16-byte units)
      const uint64_t da0 = umma::sdesc(hb, kPlaneBytes, kHaloW * 16);
      const uint64_t db0 = umma::sdesc(wbase, NC * 16, 8 * 16);
#pragma unroll
      for (int tap = 0; tap < 9; ++tap) {
        uint64_t da = da0 + (uint64_t)((((tap / 3) * kHaloW + tap % 3) * 16) >> 4);
        uint64_t db = db0 + (uint64_t)(tap * planes * NC);
        for (int ks = 0; ks < planes / 2; ++ks, da += (2 * kPlaneBytes) >> 4, db += 2 * NC)
          umma::mma_ss<false>(d, da, db, idesc, tap > 0 || ks > 0);
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                       b ? mb1 : mb0)
                   : "memory");
    }
    mma_issued = i;
    // tile i-1's MMAs (which read the other halo buffer) must be done before
    // that buffer is refilled and before its accumulator is drained
    if (i >= 1) {
      const uint32_t pb = b ^ 1u;
      const bool ok = umma::mbar_wait(pb ? mb1 : mb0, (uint32_t)(((i - 1) >> 1) & 1));
      if (__syncthreads_or(!ok)) {
        failed = true;
        break;
      }
    }
    const int tn = t + gridDim.x;
    if (tn < total_tiles) load_halo(b ? hbase0 : hbase1, tn);
    asm volatile("cp.async.commit_group;\n" ::);
    if (i >= 1) {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      epilogue(t - (int)gridDim.x, b ^ 1u);
    }
  }
  asm volatile("cp.async.wait_group 0;\n" ::);
  if (failed && mma_issued > i - 1) {  // tile i's MMAs were issued and not waited for: once more, bounded
    umma::mbar_wait((i & 1) ? mb1 : mb0, (uint32_t)((i >> 1) & 1));
    __syncthreads();
  }
  if (!failed && i >= 1) {  // the last tile
    const int last = i - 1;
    bool ok = umma::mbar_wait((last & 1) ? mb1 : mb0, (uint32_t)((last >> 1) & 1));
    if (!ok) ok = umma::mbar_wait((last & 1) ? mb1 : mb0, (uint32_t)((last >> 1) & 1));
    failed = __syncthreads_or(!ok);
    if (!failed) {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      epilogue(blockIdx.x + last * (int)gridDim.x, (uint32_t)(last & 1));
    }
  }
  if (failed && tid == 0) atomicOr(&g_umma_error, 1u);
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kCols));
  }
}

// Warp-specialised persistent form. Warp 0 produces input halos into a
// ring of shared-memory stages (x1 by TMA; the upsampled x2 part by cp.async
// gathers, after which each lane waits for its copies, fences them for the
// tensor cores and arrives on the same "full" barrier); warp 1
// allocates tensor memory and, from one lane, issues each tile's MMAs into
// one of two accumulator buffers, committing to the stage's "empty" barrier
// (the producer may refill it) and to the buffer's "full" barrier; warps
// 2-5 drain finished accumulators (bias, ReLU, BF16 stores) and release the
// buffer. No block-wide barrier inside the tile loop. Every wait is bounded
// (2 s); a timeout raises a shared abort flag that ends every role's loop.
// warp 0: TMA producer; 1: MMA issue; 2-5: epilogue; 6-9: cp.async gather of
// the halo planes the TMA does not load (the upsampled second input), each
// stage owned by one gather warp, so a warp's wait for its own copies does
// not hold up the other stages
//
// FP8 form (kF8): a stage receives the BF16 halo planes as above (the TMA
// completes on a separate per-stage barrier); the stage's gather warp waits
// for them, quantises them in place with the per-input-channel scales
// (e4m3, saturating) into planes of 16 e4m3 channels (16 bytes a pixel:
// the plane geometry of 8 BF16 channels), zeros past the input channels up
// to a multiple of 32, and only then arrives on the "full" barrier; the MMA
// warp issues kind::f8f6f4 with K = 32 (two planes) per instruction, half
// the BF16 instruction count; the epilogue multiplies by the per-output-
// channel weight scale before the bias.
constexpr int kWsGatherWarps = 4;
constexpr int kWsThreads = 192 + 32 * kWsGatherWarps;

__device__ __forceinline__ void mbar_arrive(uint32_t addr) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(addr) : "memory");
}

// e4m3 codes (saturating) of four BF16 values (two packed pairs) scaled by
// s[0..3], in channel order from the low byte: the quantisation of the
// mma.sync FP8 kernel.
__device__ __forceinline__ uint32_t quant4_e4m3(uint32_t lo2, uint32_t hi2, const float* s) {
  const float2 f0 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&lo2));
  const float2 f1 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&hi2));
  const __nv_fp8x2_storage_t q0 = __nv_cvt_float2_to_fp8x2(make_float2(f0.x * s[0], f0.y * s[1]), __NV_SATFINITE,
                                                           __NV_E4M3);
  const __nv_fp8x2_storage_t q1 = __nv_cvt_float2_to_fp8x2(make_float2(f1.x * s[2], f1.y * s[3]), __NV_SATFINITE,
                                                           __NV_E4M3);
  return (uint32_t)q0 | ((uint32_t)q1 << 16);
}

// FP8: at most 64 registers, three CTAs an SM (the full-resolution layers
// run out of CTAs in flight with two); BF16: the compiler's allocation.
template <int NC, bool kF8, bool kSwz = false>
__global__ void __launch_bounds__(kWsThreads, kF8 ? 3 : 0) conv3x3_umma_ws_kernel(UmmaConvArgs a, int tiles_per_image,
                                                                     const __grid_constant__ CUtensorMap x1map,
                                                                     const __grid_constant__ CUtensorMap x2map,
                                                                     int use_tma, int stg_planes, int stages,
                                                                     int x1_swz) {
  using namespace umma;
  constexpr uint32_t kCols = 2 * NC <= 64 ? 64 : (2 * NC <= 128 ? 128 : 256);
  constexpr int kMaxStages = 6;
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) uint64_t full_bar[kMaxStages], empty_bar[kMaxStages], tfull_bar[2], tempty_bar[2];
  __shared__ __align__(8) uint64_t tma_bar[kF8 ? kMaxStages : 1];  // FP8: the TMA's arrival per stage
  __shared__ __align__(8) uint64_t stg_bar[kMaxStages];             // the half-resolution x2 box's arrival
  __shared__ uint32_t tmem_base_slot;
  __shared__ volatile int abort_flag;
  __shared__ __align__(16) float s_bias[NC];
  __shared__ __align__(16) float s_wsc[kF8 ? NC : 1];    // FP8: weight scale per output channel
  __shared__ __align__(16) float s_inv[kF8 ? 256 : 4];   // FP8: 1 / activation scale per input channel, 0 past cin
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int cin = a.c1 + a.c2;
  // MMA planes: 8 BF16 channels, or 16 e4m3 channels (input padded to a multiple of 32)
  const int planes = kF8 ? ((cin + 31) & ~31) / 16 : cin / 8;
  // BF16 planes a stage receives (8 channels each); the FP8 form quantises
  // them in place into its e4m3 planes (at most the same bytes)
  const int in_planes = cin / 8;
  const int halo_bytes = in_planes * kPlaneBytes;
  // stage: the halo planes, then (stg_planes > 0) the TMA's half-resolution
  // box of the second input, which the gather warp expands into its planes
  const int stg_off = (halo_bytes + 127) & ~127;
  const int halo_pitch = (stg_off + stg_planes * kStgPlaneBytes + 1023) & ~1023;
  const int tiles_x = (a.W + kTileW - 1) / kTileW;
  const int total_tiles = tiles_per_image * a.N;
  const int H2 = a.H >> 1, W2 = a.W >> 1;
  const int x1_planes = use_tma ? a.c1 / 8 : 0;
  const bool gather = kF8 || in_planes > x1_planes;  // cp.async part present (FP8: the quantising warps)
  const uint32_t sbase = smem_addr(smem);
  const uint32_t wbase = sbase;
  const uint32_t hbase = (sbase + 9 * planes * NC * 16 + 1023u) & ~1023u;
  auto fb = [&](int st) { return smem_addr(&full_bar[st]); };
  auto eb = [&](int st) { return smem_addr(&empty_bar[st]); };
  auto tfb = [&](int b) { return smem_addr(&tfull_bar[b]); };
  auto teb = [&](int b) { return smem_addr(&tempty_bar[b]); };
  auto tmb = [&](int st) { return smem_addr(&tma_bar[kF8 ? st : 0]); };
  auto sgb = [&](int st) { return smem_addr(&stg_bar[st]); };
  if (tid == 0) {
    for (int st = 0; st < stages; ++st) {
      umma::mbar_init(fb(st), kF8 ? 32u : (x1_planes ? 1u : 0u) + (gather ? 32u : 0u));
      umma::mbar_init(eb(st), 1);
      if (kF8) umma::mbar_init(tmb(st), 1);
      if (stg_planes) umma::mbar_init(sgb(st), 1);
    }
    for (int b = 0; b < 2; ++b) {
      umma::mbar_init(tfb(b), 1);
      umma::mbar_init(teb(b), 128);
    }
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     smem_addr(&tmem_base_slot)),
                 "r"(kCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
  }
  for (int i = tid; i < NC; i += (int)blockDim.x) s_bias[i] = a.bias ? a.bias[i] : 0.f;
  if constexpr (kF8) {
    for (int i = tid; i < NC; i += (int)blockDim.x) s_wsc[i] = a.wscale[i];
    for (int i = tid; i < 256; i += (int)blockDim.x) s_inv[i] = i < cin ? a.inv_xscale[i] : 0.f;
  }
  // weights, once, by every thread: [tap][plane][n][16 bytes]
  for (int i = tid; i < NC * 9 * planes; i += (int)blockDim.x) {
    const int co = i % NC, r = i / NC;
    const int p = r % planes, tap = r / planes;
    if constexpr (kF8) {  // e4m3, zeros for the padding channels
      const bool ok = p * 16 < cin;
      umma::cp16(wbase + ((tap * planes + p) * NC + co) * 16, ok ? a.w8 + ((size_t)co * 9 + tap) * cin + p * 16 : a.w8,
                 ok);
    } else {
      umma::cp16(wbase + ((tap * planes + p) * NC + co) * 16, a.w + ((size_t)co * 9 + tap) * cin + p * 8, true);
    }
  }
  asm volatile("cp.async.commit_group;\n" ::);
  asm volatile("cp.async.wait_group 0;\n" ::);
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_base_slot;
  auto tile_origin = [&](int t, int& img, int& x0, int& y0) {
    img = t / tiles_per_image;
    const int r = t % tiles_per_image;
    x0 = (r % tiles_x) * kTileW;
    y0 = (r / tiles_x) * kTileH;
  };
  auto wait = [&](uint32_t bar, uint32_t parity) {
    if (umma::mbar_wait(bar, parity)) return true;
    abort_flag = 1;
    return false;
  };

  int tma_issued = 0;  // producer: TMA loads issued (the abort path waits for the last one per stage)
  if (warp == 0) {
    // ---- producer (TMA of the x1 planes)
    int i = 0;
    for (int t = blockIdx.x; t < total_tiles && !abort_flag && (x1_planes || stg_planes); t += gridDim.x, ++i) {
      const int st = i % stages, k = i / stages;
      if (!wait(eb(st), (uint32_t)((k & 1) ^ 1))) break;  // the MMAs of the stage's previous tile are done
      const uint32_t hb = hbase + st * halo_pitch;
      int img, x0, y0;
      tile_origin(t, img, x0, y0);
      if (lane == 0 && x1_planes) {
        const uint32_t bar = kF8 ? tmb(st) : fb(st);  // FP8: the quantising warp waits for the load
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar),
                     "r"((uint32_t)(x1_planes * kPlaneBytes))
                     : "memory");
        if constexpr (kSwz)  // whole pixels, swizzled rows: [18][10][c1] (the same bytes as the planes)
          asm volatile(
              "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
              "%4, %5}], [%6];\n" ::"r"(hb),
              "l"(reinterpret_cast<uint64_t>(&x1map)), "r"(0), "r"(x0 - 1), "r"(y0 - 1), "r"(img), "r"(bar)
              : "memory");
        else
          asm volatile(
              "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
              "%4, %5, %6}], [%7];\n" ::"r"(hb),
              "l"(reinterpret_cast<uint64_t>(&x1map)), "r"(0), "r"(x0 - 1), "r"(y0 - 1), "r"(0), "r"(img), "r"(bar)
              : "memory");
      }
      if (lane == 0 && stg_planes) {
        // the 6 x 10 half-resolution pixels under the tile's halo (x0 % 8 == 0,
        // y0 % 16 == 0: columns x0/2 - 1 .. x0/2 + 4, rows y0/2 - 1 .. y0/2 + 8)
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(sgb(st)),
                     "r"((uint32_t)(stg_planes * kStgPlaneBytes))
                     : "memory");
        asm volatile(
            "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
            "%5, %6}], [%7];\n" ::"r"(hb + stg_off),
            "l"(reinterpret_cast<uint64_t>(&x2map)), "r"(0), "r"((x0 >> 1) - 1), "r"((y0 >> 1) - 1), "r"(0), "r"(img),
            "r"(sgb(st))
            : "memory");
      }
      ++tma_issued;
    }
  } else if (warp >= 6) {
    // ---- gather (cp.async of the planes after the TMA's). Stage st belongs
    // to warp st % kWsGatherWarps alone, so each stage's fills and arrivals
    // come in phase order from one warp: a warp cannot wait on a stage's
    // empty barrier two phases late (its parity would then read as done).
    const int gw = warp - 6;
    int i = 0;
    for (int t = blockIdx.x; t < total_tiles && !abort_flag && gather; t += gridDim.x, ++i) {
      if ((i % stages) % kWsGatherWarps != gw) continue;
      const int st = i % stages, k = i / stages;
      if (!wait(eb(st), (uint32_t)((k & 1) ^ 1))) break;
      const uint32_t hb = hbase + st * halo_pitch;
      int img, x0, y0;
      tile_origin(t, img, x0, y0);
      {
        const int gathered = stg_planes ? a.c1 / 8 : in_planes;  // planes fetched by cp.async end here
        for (int q = lane + x1_planes * kHaloPx; q < kHaloPx * gathered; q += 32) {
          const int hp = q % kHaloPx, p = q / kHaloPx;
          const int yy = y0 - 1 + hp / kHaloW, xx = x0 - 1 + hp % kHaloW;
          const int ci = p * 8;
          const bool ok = yy >= 0 && yy < a.H && xx >= 0 && xx < a.W;
          const bf16* src = a.x1;
          if (ok) {
            if (ci < a.c1) src = a.x1 + (((size_t)img * a.H + yy) * a.W + xx) * a.c1 + ci;
            else src = a.x2 + (((size_t)img * H2 + (yy >> 1)) * W2 + (xx >> 1)) * a.c2 + (ci - a.c1);
          }
          umma::cp16(hb + p * kPlaneBytes + hp * 16, src, ok);
        }
        // this lane's copies landed and made visible to the tensor cores, then one arrival
        asm volatile("cp.async.commit_group;\n" ::);
        asm volatile("cp.async.wait_group 0;\n" ::);
        if (stg_planes) {
          // nearest upsampling of the half-resolution box into the second
          // input's planes: halo pixel (hy, hx) is box pixel ((hy + 1) / 2,
          // (hx + 1) / 2); outside the frame the box holds the TMA's zeros
          if (!wait(sgb(st), (uint32_t)(k & 1))) break;
          const uint32_t sb = hb + stg_off, db = hb + (a.c1 / 8) * kPlaneBytes;
          for (int q = lane; q < stg_planes * kHaloPx; q += 32) {
            const int p = q / kHaloPx, hp = q - p * kHaloPx;
            const int hy = hp / kHaloW, hx = hp - hy * kHaloW;
            const uint32_t src = sb + p * kStgPlaneBytes + (((hy + 1) >> 1) * kStgW + ((hx + 1) >> 1)) * 16;
            uint32_t v0, v1, v2, v3;
            asm volatile("ld.shared.v4.b32 {%0, %1, %2, %3}, [%4];\n"
                         : "=r"(v0), "=r"(v1), "=r"(v2), "=r"(v3)
                         : "r"(src)
                         : "memory");
            asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};\n" ::"r"(db + p * kPlaneBytes + hp * 16), "r"(v0),
                         "r"(v1), "r"(v2), "r"(v3)
                         : "memory");
          }
        }
        if constexpr (kF8) {
          // every BF16 plane in place (the TMA's and the warp's copies), then
          // each 16-channel pair quantised into e4m3 plane p at the offset of
          // BF16 plane p: a lane rewrites only its own pixels, and plane p's
          // BF16 source planes 2p, 2p + 1 are not yet overwritten
          if (x1_planes && !wait(tmb(st), (uint32_t)(k & 1))) break;
          __syncwarp();
          for (int p = 0; p < planes; ++p) {
            const float* sc = s_inv + p * 16;
            const bool lo_in = 2 * p < in_planes, hi_in = 2 * p + 1 < in_planes;  // else padding channels
            for (int hp = lane; hp < kHaloPx; hp += 32) {
              uint4 lo = make_uint4(0u, 0u, 0u, 0u), hi = lo;
              const uint32_t src = hb + (2 * p) * kPlaneBytes + hp * 16;
              if (lo_in)
                asm volatile("ld.shared.v4.b32 {%0, %1, %2, %3}, [%4];\n"
                             : "=r"(lo.x), "=r"(lo.y), "=r"(lo.z), "=r"(lo.w)
                             : "r"(src)
                             : "memory");
              if (hi_in)
                asm volatile("ld.shared.v4.b32 {%0, %1, %2, %3}, [%4];\n"
                             : "=r"(hi.x), "=r"(hi.y), "=r"(hi.z), "=r"(hi.w)
                             : "r"(src + kPlaneBytes)
                             : "memory");
              const uint32_t o0 = quant4_e4m3(lo.x, lo.y, sc), o1 = quant4_e4m3(lo.z, lo.w, sc + 4);
              const uint32_t o2 = quant4_e4m3(hi.x, hi.y, sc + 8), o3 = quant4_e4m3(hi.z, hi.w, sc + 12);
              asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};\n" ::"r"(hb + p * kPlaneBytes + hp * 16),
                           "r"(o0), "r"(o1), "r"(o2), "r"(o3)
                           : "memory");
            }
          }
        }
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        mbar_arrive(fb(st));
      }
    }
    asm volatile("cp.async.wait_group 0;\n" ::);
  } else if (warp == 1) {
    // ---- MMA issue (one lane)
    if (lane == 0) {
      constexpr uint32_t idesc = kF8 ? umma::idesc_e4m3(NC) : umma::idesc_bf16(NC);
      int i = 0;
      for (int t = blockIdx.x; t < total_tiles && !abort_flag; t += gridDim.x, ++i) {
        const int st = i % stages, k = i / stages, b = i & 1, kb = i >> 1;
        if (!wait(fb(st), (uint32_t)(k & 1))) break;           // halo in place
        if (!wait(teb(b), (uint32_t)((kb & 1) ^ 1))) break;    // accumulator buffer drained
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        const uint32_t hb = hbase + st * halo_pitch, d = tmem + (uint32_t)b * NC;
        // The descriptors advance by constants (a tap shifts the halo's
        // start, a K step moves two planes -- or, kSwz, 32 bytes along the
        // swizzled pixel rows; every sum is a shared-memory address, so the
        // 14-bit address field never carries): a single issuing thread that
        // rebuilt them per instruction spent ~40 cycles an MMA on it, as much
        // as the ~50-cycle MMA itself at small N.
        const uint64_t db0 = umma::sdesc(wbase, NC * 16, 8 * 16);
        const int ksteps = planes / 2;
        if constexpr (kSwz) {
          const uint64_t da0 = umma::sdesc_sw(hb, kHaloW * x1_swz, x1_swz);
          const uint32_t px16 = (uint32_t)x1_swz >> 4;  // one pixel, 16-byte units
#pragma unroll
          for (int tap = 0; tap < 9; ++tap) {
            uint64_t da = da0 + (uint64_t)(((tap / 3) * kHaloW + tap % 3) * px16);
            uint64_t db = db0 + (uint64_t)(tap * planes * NC);
            for (int ks = 0; ks < ksteps; ++ks, da += 2, db += 2 * NC)
              umma::mma_ss<kF8>(d, da, db, idesc, tap > 0 || ks > 0);
          }
        } else {
          const uint64_t da0 = umma::sdesc(hb, kPlaneBytes, kHaloW * 16);
#pragma unroll
          for (int tap = 0; tap < 9; ++tap) {
            uint64_t da = da0 + (uint64_t)((((tap / 3) * kHaloW + tap % 3) * 16) >> 4);
            uint64_t db = db0 + (uint64_t)(tap * planes * NC);
            for (int ks = 0; ks < ksteps; ++ks, da += (2 * kPlaneBytes) >> 4, db += 2 * NC)
              umma::mma_ss<kF8>(d, da, db, idesc, tap > 0 || ks > 0);
          }
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(eb(st))
                     : "memory");
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(tfb(b))
                     : "memory");
      }
    }
    __syncwarp();
  } else {
    // ---- epilogue (warps 2-5: tensor-memory subpartitions 2, 3, 0, 1)
    const int sub = warp & 3;
    int i = 0;
    for (int t = blockIdx.x; t < total_tiles; t += gridDim.x, ++i) {
      const int b = i & 1, kb = i >> 1;
      const bool ok = umma::mbar_wait(tfb(b), (uint32_t)(kb & 1));
      if (__any_sync(0xffffffffu, !ok) || abort_flag) {
        abort_flag = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      int img, x0, y0;
      tile_origin(t, img, x0, y0);
      const int m = sub * 32 + lane;
      const int oy = y0 + m / kTileW, ox = x0 + m % kTileW;
      const bool inside = oy < a.H && ox < a.W;
      const size_t pix = ((size_t)img * a.H + (inside ? oy : 0)) * a.W + (inside ? ox : 0);
      bf16* dst = a.y32 ? nullptr : a.y + pix * a.cout;
      float* dst32 = a.y32 ? a.y32 + pix * a.ldy32 : nullptr;
      // two 16-column loads in flight before one wait (fewer tensor-memory round trips)
#pragma unroll
      for (int c00 = 0; c00 < NC; c00 += 32) {
      uint32_t vv[2][16];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        if (c00 + 16 * h >= NC) break;
        const uint32_t taddr = tmem + ((uint32_t)(sub * 32) << 16) + (uint32_t)b * NC + (uint32_t)(c00 + 16 * h);
        uint32_t* v = vv[h];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
            "[%16];\n"
            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
              "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
            : "r"(taddr));
      }
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int c0 = c00 + 16 * h;
        if (c0 >= NC) break;
        const uint32_t* v = vv[h];
        if (inside && dst32) {  // FP32 output (no FP8 scale, no pooling)
          float f[16];
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            f[j] = __uint_as_float(v[j]) + (a.bias ? s_bias[c0 + j] : 0.f);
            if (a.relu & 1) f[j] = fmaxf(f[j], 0.f);
          }
          float4* d4 = reinterpret_cast<float4*>(dst32 + c0);
#pragma unroll
          for (int j = 0; j < 4; ++j) d4[j] = make_float4(f[4 * j], f[4 * j + 1], f[4 * j + 2], f[4 * j + 3]);
        } else if (inside) {
          uint32_t packed[8];
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            float f0 = __uint_as_float(v[2 * j]), f1 = __uint_as_float(v[2 * j + 1]);
            if constexpr (kF8) {
              const float2 sw = *reinterpret_cast<const float2*>(&s_wsc[c0 + 2 * j]);
              f0 *= sw.x;
              f1 *= sw.y;
            }
            if (a.bias) {
              const float2 bb = *reinterpret_cast<const float2*>(&s_bias[c0 + 2 * j]);
              f0 += bb.x;
              f1 += bb.y;
            }
            if (a.relu & 1) {
              f0 = fmaxf(f0, 0.f);
              f1 = fmaxf(f1, 0.f);
            }
            const __nv_bfloat162 b2 = __floats2bfloat162_rn(f0, f1);
            packed[j] = *reinterpret_cast<const uint32_t*>(&b2);
          }
          uint4* d4 = reinterpret_cast<uint4*>(dst + c0);
          d4[0] = make_uint4(packed[0], packed[1], packed[2], packed[3]);
          d4[1] = make_uint4(packed[4], packed[5], packed[6], packed[7]);
          if (a.pooled) {
            // 2x2 average of the stored BF16 values (the frame divides into
            // tiles, so every lane is inside): a warp holds four 8-pixel rows
            // of the tile (lane = 8 row + column), so a pooled pixel's window
            // is lanes lane, lane ^ 1, lane ^ 8, lane ^ 9, summed in the
            // order of the stand-alone pooling kernel: the same bits
            uint32_t q1[8], q8[8], q9[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
              q1[j] = __shfl_xor_sync(0xffffffffu, packed[j], 1);
              q8[j] = __shfl_xor_sync(0xffffffffu, packed[j], 8);
              q9[j] = __shfl_xor_sync(0xffffffffu, packed[j], 9);
            }
            if ((lane & 9) == 0) {
              uint32_t po[8];
#pragma unroll
              for (int j = 0; j < 8; ++j) {
                const float2 v0 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&packed[j]));
                const float2 v1 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&q1[j]));
                const float2 v2 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&q8[j]));
                const float2 v3 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&q9[j]));
                const float sx = ((v0.x + v1.x) + v2.x) + v3.x, sy = ((v0.y + v1.y) + v2.y) + v3.y;
                const __nv_bfloat162 b2 = __floats2bfloat162_rn(0.25f * sx, 0.25f * sy);
                po[j] = *reinterpret_cast<const uint32_t*>(&b2);
              }
              bf16* pd = a.pooled + (((size_t)img * (a.H >> 1) + (oy >> 1)) * (a.W >> 1) + (ox >> 1)) * a.cout + c0;
              uint4* p4 = reinterpret_cast<uint4*>(pd);
              p4[0] = make_uint4(po[0], po[1], po[2], po[3]);
              p4[1] = make_uint4(po[4], po[5], po[6], po[7]);
            }
          }
        }
      }
      }
      asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
      mbar_arrive(teb(b));
    }
  }
  // every role is past its loop; the epilogue has waited for the last MMAs
  // (or a role gave up: then wait once more, bounded, for MMAs in flight)
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (abort_flag) {
    if (tid == 0) atomicOr(&g_umma_error, 1u);
    const int n_mine = (total_tiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x;
    if (n_mine > 0 && warp == 1 && lane == 0) {  // the last tile's accumulator commit, bounded
      const int last = n_mine - 1;
      umma::mbar_wait(tfb(last & 1), (uint32_t)((last >> 1) & 1));
    }
    if ((x1_planes || stg_planes) && warp == 0 && lane == 0) {
      // TMA loads still in flight land before the CTA's shared memory is
      // released: the last load into each stage, bounded (FP8: the load's own
      // barrier; BF16: the stage's full barrier, which with gather warps also
      // waits for their arrivals and may give up at the bound)
      for (int st = 0; st < stages && st < tma_issued; ++st) {
        const int j = tma_issued - 1 - (tma_issued - 1 - st) % stages;  // last tile loaded into stage st
        if (x1_planes) umma::mbar_wait(kF8 ? tmb(st) : fb(st), (uint32_t)((j / stages) & 1));
        if (stg_planes) umma::mbar_wait(sgb(st), (uint32_t)((j / stages) & 1));
      }
    }
    __syncthreads();
  }
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kCols));
  }
}

// Backward weights on tcgen05: dW[co][tap][ci] += sum over pixels p of
// dY[p][co] * X(p shifted by the tap)[ci]. A CTA walks 8x8-pixel tiles of
// the images (grid-stride) for a group of taps, the sums of the whole walk
// in tensor memory: per tile and tap a GEMM with M = 128 output channels
// (rows past cout are zeros), N = cin and K = the tile's 64 pixels, four
// K = 16 MMAs. Both operands sit in shared memory as they are stored in
// global memory -- each pixel's channels contiguous -- which is the MN-major
// no-swizzle layout: a core matrix is 8 pixels (K) x 8 channels (16 bytes).
// dY's tile: pixel rows 128 bytes apart (the K stride), channel groups 1 KB
// apart. X's 10x10-pixel halo of the tile: halo rows 160 bytes apart, channel
// groups 1600 bytes apart; the tap (dy, dx) is the same descriptor with its
// start moved by dy halo rows and dx pixels -- no copy per tap. dY's tile
// and x1's halo come by TMA (5-D maps [8 channels][x][y][channel group]
// [image] whose boxes land in exactly this layout). The accumulators (TMEM
// lane = co, column = tap x cin + ci) are added into dW with atomics once,
// at the end of the walk.
struct UmmaWgradArgs {
  const bf16* dy;  // [N][H][W][cout]
  const bf16* x1;  // [N][H][W][c1]
  const bf16* x2;  // [N][H/2][W/2][c2], upsampled on load, or null
  int c1, c2;
  float* dw;  // [cout][9][c1 + c2]
  int N, H, W, cout;
  int ntaps;   // taps a CTA: blockIdx.x * ntaps .. + ntaps - 1
  int stages;  // 3 or 4 input stages
};
constexpr int kWgT = 8, kWgHalo = kWgT + 2;  // 8x8-pixel tile, 10x10 halo
constexpr int kWgStages = 4;                 // at most
constexpr int kWgABytes = 16 * 64 * 16;                       // 128 rows (16 groups) x 64 pixels
constexpr int kWgBGroup = kWgHalo * kWgHalo * 16;             // one 8-channel group of the halo: 1600 B
__host__ __device__ constexpr int wgrad_stage_bytes(int cin) {
  return kWgABytes + (((cin / 8) * kWgBGroup + 127) & ~127);
}
__host__ __device__ constexpr uint32_t wgrad_cols(int cols) {
  return cols <= 32 ? 32u : (cols <= 64 ? 64u : (cols <= 128 ? 128u : (cols <= 256 ? 256u : 512u)));
}

// Warp-specialised: no block-wide barrier inside the tile loop. Warp 0's
// lane 0 loads dY's tile and x1's halo of each tile by TMA into a ring of S
// stages (stage "full" barrier: its transaction bytes); warps 2-3 gather the
// upsampled x2 part of the halo with cp.async and arrive on the same full
// barrier (64 arrivals); warp 1's lane 0 issues each tile's MMAs as soon as
// its stage is full and commits them to the stage's "empty" barrier, which
// the loaders wait for before refilling it. At the end every warp drains
// its 32 tensor-memory lanes into dW. Every wait is bounded (2 s); a
// timeout raises a shared abort flag that ends every role's loop; the MMA
// lane then waits (bounded) for its last commit and the TMA lane for its
// last load into each stage before the tensor memory is freed.
__global__ void __launch_bounds__(128) conv3x3_wgrad_umma_ws_kernel(UmmaWgradArgs a,
                                                                    const __grid_constant__ CUtensorMap dymap,
                                                                    const __grid_constant__ CUtensorMap x1map) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) uint64_t full_bar[kWgStages], empty_bar[kWgStages];
  __shared__ uint32_t tmem_base_slot;
  __shared__ volatile int abort_flag;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int cin = a.c1 + a.c2;
  const int tap0 = blockIdx.x * a.ntaps;
  const int tiles_x = (a.W + kWgT - 1) / kWgT, tiles_y = (a.H + kWgT - 1) / kWgT;
  const long tiles = (long)tiles_x * tiles_y * a.N;
  const int n_it = blockIdx.y < tiles ? (int)((tiles - 1 - blockIdx.y) / gridDim.y + 1) : 0;
  const int H2 = a.H >> 1, W2 = a.W >> 1;
  const uint32_t cols = wgrad_cols(a.ntaps * cin);
  const int S = a.stages;
  const int stage_bytes = wgrad_stage_bytes(cin);
  const int ga = a.cout / 8, gb = cin / 8, gb1 = a.c1 / 8;
  const bool gather = gb > gb1;  // the upsampled second input
  const uint32_t sbase = (umma::smem_addr(smem) + 1023u) & ~1023u;
  auto fb = [&](int st) { return umma::smem_addr(&full_bar[st]); };
  auto eb = [&](int st) { return umma::smem_addr(&empty_bar[st]); };
  if (tid == 0) {
    for (int st = 0; st < S; ++st) {
      umma::mbar_init(fb(st), 1u + (gather ? 64u : 0u));
      umma::mbar_init(eb(st), 1);
    }
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     umma::smem_addr(&tmem_base_slot)),
                 "r"(cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
  }
  // the A rows past cout stay zero in every stage
  for (int st = 0; st < S; ++st)
    for (int i = tid * 16 + ga * 1024; i < kWgABytes; i += 128 * 16)
      asm volatile("st.shared.v4.b32 [%0], {%1, %1, %1, %1};\n" ::"r"(sbase + st * stage_bytes + i), "r"(0)
                   : "memory");
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_base_slot;
  auto wait = [&](uint32_t bar, uint32_t parity) {
    if (umma::mbar_wait(bar, parity)) return true;
    abort_flag = 1;
    return false;
  };
  auto tile_origin = [&](int it, int& img, int& x0, int& y0) {
    const long t = blockIdx.y + (long)it * gridDim.y;
    img = (int)(t / ((long)tiles_x * tiles_y));
    const int rem = (int)(t - (long)img * tiles_x * tiles_y);
    x0 = (rem % tiles_x) * kWgT;
    y0 = (rem / tiles_x) * kWgT;
  };

  int loaded = 0;  // producer lane: tiles whose TMA loads were issued
  if (warp == 0) {
    if (lane == 0) {
      for (int it = 0; it < n_it && !abort_flag; ++it) {
        const int st = it % S, k = it / S;
        if (!wait(eb(st), (uint32_t)((k & 1) ^ 1))) break;  // the MMAs of the stage's previous tile are done
        int img, x0, y0;
        tile_origin(it, img, x0, y0);
        const uint32_t ab = sbase + st * stage_bytes, bb = ab + kWgABytes;
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(fb(st)),
                     "r"((uint32_t)(ga * 1024 + gb1 * kWgBGroup))
                     : "memory");
        asm volatile(
            "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
            "%5, %6}], [%7];\n" ::"r"(ab),
            "l"(reinterpret_cast<uint64_t>(&dymap)), "r"(0), "r"(x0), "r"(y0), "r"(0), "r"(img), "r"(fb(st))
            : "memory");
        asm volatile(
            "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
            "%5, %6}], [%7];\n" ::"r"(bb),
            "l"(reinterpret_cast<uint64_t>(&x1map)), "r"(0), "r"(x0 - 1), "r"(y0 - 1), "r"(0), "r"(img), "r"(fb(st))
            : "memory");
        ++loaded;
      }
    }
    __syncwarp();
  } else if (warp >= 2) {
    // ---- gather of the upsampled x2 planes of the halo (64 threads, every stage)
    const int tg = tid - 64;
    for (int it = 0; it < n_it && !abort_flag && gather; ++it) {
      const int st = it % S, k = it / S;
      if (!wait(eb(st), (uint32_t)((k & 1) ^ 1))) break;
      int img, x0, y0;
      tile_origin(it, img, x0, y0);
      const uint32_t bb = sbase + st * stage_bytes + kWgABytes;
      for (int q = tg; q < kWgHalo * kWgHalo * (gb - gb1); q += 64) {
        const int hp = q % (kWgHalo * kWgHalo), g = gb1 + q / (kWgHalo * kWgHalo);
        const int yy = y0 - 1 + hp / kWgHalo, xx = x0 - 1 + hp % kWgHalo;
        const bool ok = yy >= 0 && yy < a.H && xx >= 0 && xx < a.W;
        const bf16* src = ok ? a.x2 + (((size_t)img * H2 + (yy >> 1)) * W2 + (xx >> 1)) * a.c2 + (g * 8 - a.c1) : a.x1;
        umma::cp16(bb + g * kWgBGroup + hp * 16, src, ok);
      }
      asm volatile("cp.async.commit_group;\n" ::);
      asm volatile("cp.async.wait_group 0;\n" ::);
      asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
      asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(fb(st)) : "memory");
    }
    asm volatile("cp.async.wait_group 0;\n" ::);
  } else if (lane == 0) {
    // ---- MMA issue (warp 1, one lane)
    const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | (1u << 15) | (1u << 16) |
                           ((uint32_t)(cin >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
    for (int it = 0; it < n_it && !abort_flag; ++it) {
      const int st = it % S, k = it / S;
      if (!wait(fb(st), (uint32_t)(k & 1))) break;  // this tile's operands in place
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      const uint32_t ab = sbase + st * stage_bytes, bb = ab + kWgABytes;
      // descriptors advance by constants (16-byte units)
      const uint64_t da0 = umma::sdesc(ab, 128, 1024);
      const uint64_t db0 = umma::sdesc(bb, kWgHalo * 16, kWgBGroup);
      for (int tl = 0; tl < a.ntaps; ++tl) {
        const int tap = tap0 + tl, dy = tap / 3, dx = tap % 3;
        const uint32_t d = tmem + (uint32_t)(tl * cin);
        const uint64_t dbt = db0 + (uint64_t)(dy * kWgHalo + dx);
#pragma unroll
        for (int ks = 0; ks < 4; ++ks)  // K = 16: tile rows 2ks, 2ks + 1
          umma::mma_ss<false>(d, da0 + (uint64_t)(ks * 16), dbt + (uint64_t)(2 * ks * kWgHalo), idesc,
                              it > 0 || ks > 0);
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(eb(st))
                   : "memory");
    }
  }
  // every role is past its loop: the last tile's MMAs (and every earlier
  // one) complete before the accumulator is read or freed
  __syncthreads();
  bool ok = !abort_flag;
  if (n_it > 0) {
    const int last = n_it - 1;
    if (ok) {
      ok = umma::mbar_wait(eb(last % S), (uint32_t)((last / S) & 1));
      if (!ok) ok = umma::mbar_wait(eb(last % S), (uint32_t)((last / S) & 1));
    }
  }
  const bool failed = __syncthreads_or(!ok);
  if (failed) {
    if (tid == 0) {
      atomicOr(&g_umma_error, 1u);
      // TMA loads still in flight land before the shared memory is
      // released: the last load into each stage, bounded
      for (int st = 0; st < S && st < loaded; ++st) {
        const int jl = loaded - 1 - (loaded - 1 - st) % S;
        umma::mbar_wait(fb(st), (uint32_t)((jl / S) & 1));
      }
    }
    if (warp == 1 && lane == 0 && n_it > 0) {  // MMAs in flight, bounded
      const int last = n_it - 1;
      umma::mbar_wait(eb(last % S), (uint32_t)((last / S) & 1));
    }
  } else if (n_it > 0) {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const int co = warp * 32 + lane;  // TMEM lane
    for (int tl = 0; tl < a.ntaps; ++tl) {
      float* drow = a.dw + ((size_t)(co < a.cout ? co : 0) * 9 + tap0 + tl) * cin;
      for (int c0 = 0; c0 < cin; c0 += 16) {
        uint32_t v[16];
        const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(tl * cin + c0);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
            "[%16];\n"
            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
              "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
        if (co < a.cout) {
#pragma unroll
          for (int k = 0; k < 16; ++k) atomicAdd(drow + c0 + k, __uint_as_float(v[k]));
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(cols));
  }
}

}  // namespace nn
}  // namespace pbrt

using namespace pbrt;
using namespace pbrt::nn;

namespace {
template <int NC> int launch_umma(const UmmaConvArgs& a, cudaStream_t s) {
  constexpr int kStage = umma::kPlanes * umma::kPlaneBytes + 9 * umma::kPlanes * NC * 16;
  constexpr size_t kSmem = 2 * (size_t)kStage + 1024;  // two stages (+ alignment of the dynamic base)
  static PerDeviceOnce attrs;
  int ast = once_per_device(attrs, [&]() -> int {
    cudaError_t e = cudaFuncSetAttribute(conv3x3_umma_kernel<NC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kSmem);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(conv3x3_umma_kernel)");
    return PBRT_OK;
  });
  if (ast) return ast;
  dim3 grid(((a.W + umma::kTileW - 1) / umma::kTileW) * ((a.H + umma::kTileH - 1) / umma::kTileH), a.N, 1);
  conv3x3_umma_kernel<NC><<<grid, 128, kSmem, s>>>(a);
  return PBRT_OK;
}
// Shared memory of the persistent form: the weights and two halos (each
// 1024-byte aligned for the TMA destination).
size_t persistent_smem(int cin, int nc) { return (size_t)9 * cin * nc * 2 + 2 * (size_t)cin * 360 + 3 * 1024; }

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library).
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled() {
  // the driver entry point is process-wide; resolved once (thread-safe static)
  static const EncodeTiledFn fn = []() -> EncodeTiledFn {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      return (EncodeTiledFn)p;
    cudaGetLastError();
    return nullptr;
  }();
  return fn;
}

// x1 [N][H][W][c1] BF16 as [8][W][H][c1/8][N] with box [8][10][18][c1/8][1].
bool make_x1_map(CUtensorMap* m, const void* x1, int n, int h, int w, int c1) {
  EncodeTiledFn enc = encode_tiled();
  if (!enc || ((uintptr_t)x1 & 15) || c1 % 8 || c1 / 8 > 256) return false;
  const cuuint64_t dims[5] = {8, (cuuint64_t)w, (cuuint64_t)h, (cuuint64_t)(c1 / 8), (cuuint64_t)n};
  const cuuint64_t strides[4] = {(cuuint64_t)c1 * 2, (cuuint64_t)w * c1 * 2, 16, (cuuint64_t)h * w * c1 * 2};
  const cuuint32_t box[5] = {8, (cuuint32_t)umma::kHaloW, (cuuint32_t)umma::kHaloH, (cuuint32_t)(c1 / 8), 1};
  const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void*>(x1), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}
// x1 [N][H][W][c1] BF16, c1 in {16, 32, 64}, as [c1][W][H][N] with box
// [c1][10][18][1] and the swizzle of a c1 * 2-byte row: one request a pixel
// instead of one per 8 channels; lands as the halo's pixel rows.
bool make_x1_swz_map(CUtensorMap* m, const void* x1, int n, int h, int w, int c1) {
  EncodeTiledFn enc = encode_tiled();
  if (!enc || ((uintptr_t)x1 & 15) || (c1 != 16 && c1 != 32 && c1 != 64)) return false;
  const cuuint64_t dims[4] = {(cuuint64_t)c1, (cuuint64_t)w, (cuuint64_t)h, (cuuint64_t)n};
  const cuuint64_t strides[3] = {(cuuint64_t)c1 * 2, (cuuint64_t)w * c1 * 2, (cuuint64_t)h * w * c1 * 2};
  const cuuint32_t box[4] = {(cuuint32_t)c1, (cuuint32_t)umma::kHaloW, (cuuint32_t)umma::kHaloH, 1};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  const CUtensorMapSwizzle sw =
      c1 == 16 ? CU_TENSOR_MAP_SWIZZLE_32B : (c1 == 32 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_128B);
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(x1), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}
// x2 [N][H/2][W/2][c2] BF16 (the half-resolution second input) as
// [8][W/2][H/2][c2/8][N] with box [8][6][10][c2/8][1]: the pixels under one
// tile's halo, zeros outside the frame.
bool make_x2_map(CUtensorMap* m, const void* x2, int n, int h2, int w2, int c2) {
  EncodeTiledFn enc = encode_tiled();
  if (!enc || ((uintptr_t)x2 & 15) || c2 % 8 || c2 / 8 > 256 || h2 <= 0 || w2 <= 0) return false;
  const cuuint64_t dims[5] = {8, (cuuint64_t)w2, (cuuint64_t)h2, (cuuint64_t)(c2 / 8), (cuuint64_t)n};
  const cuuint64_t strides[4] = {(cuuint64_t)c2 * 2, (cuuint64_t)w2 * c2 * 2, 16, (cuuint64_t)h2 * w2 * c2 * 2};
  const cuuint32_t box[5] = {8, (cuuint32_t)umma::kStgW, (cuuint32_t)umma::kStgH, (cuuint32_t)(c2 / 8), 1};
  const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void*>(x2), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}
constexpr size_t kPersistentSmemMax = 200 * 1024;

// Warp-specialised form: weights + `stages` halo buffers (1024-aligned),
// each with room for `stg` planes of the second input's half-resolution box
// (the stage layout of conv3x3_umma_ws_kernel).
size_t ws_stage_bytes(int cin, int stg) {
  return ((((size_t)cin * 360 + 127) & ~(size_t)127) + (size_t)stg * umma::kStgPlaneBytes + 1023) & ~(size_t)1023;
}
size_t ws_smem(int cin, int nc, int stages, int stg = 0) {
  return (size_t)9 * cin * nc * 2 + 1024 + stages * ws_stage_bytes(cin, stg) + 1024;
}
constexpr size_t kWsSmemMax = 200 * 1024;
// the FP8 form (at most 3 KB of static shared memory): up to the 227 KB a CTA may hold
constexpr size_t kWsSmemMaxF8 = 220 * 1024;

// The FP8 form holds e4m3 planes of 16 channels, the input padded to a
// multiple of 32: the shared memory of the BF16 form at half the (padded)
// channel count.
size_t ws_smem_f8(int cin, int nc, int stages, int stg = 0) {
  // BF16 planes, quantised in place
  return (size_t)9 * ((cin + 31) & ~31) * nc + 1024 + stages * ws_stage_bytes(cin, stg) + 1024;
}

template <int NC, bool kF8> int launch_umma_ws(const UmmaConvArgs& a, cudaStream_t s, bool use_tma_flag,
                                               bool box_flag = true, bool swz_flag = true) {
  const int cin = a.c1 + a.c2;
  CUtensorMap map, map2;
  memset(&map, 0, sizeof(map));
  memset(&map2, 0, sizeof(map2));
  // BF16, one input of 16 or 32 channels, 32 or 48 out (the network's
  // full- and half-resolution first layers and e0b, d0b): the x1 halo as
  // swizzled pixel rows, one TMA request a pixel instead of one per 8
  // channels (1088x1920: e0b 87 -> 77 us, d0b 88 -> 79); elsewhere the
  // planes, which timed as fast or faster (64 channels; beside the
  // upsampled second input)
  constexpr bool kSwzForm = !kF8 && (NC == 32 || NC == 48);
  int x1_swz = 0;
  if (kSwzForm && use_tma_flag && swz_flag && a.c2 == 0 && (a.c1 == 16 || a.c1 == 32) &&
      make_x1_swz_map(&map, a.x1, a.N, a.H, a.W, a.c1))
    x1_swz = a.c1 * 2;
  const int use_tma = x1_swz || (use_tma_flag && make_x1_map(&map, a.x1, a.N, a.H, a.W, a.c1)) ? 1 : 0;
  const size_t smem_max = kF8 ? kWsSmemMaxF8 : kWsSmemMax;
  auto smem_at = [&](int st, int stg) { return kF8 ? ws_smem_f8(cin, NC, st, stg) : ws_smem(cin, NC, st, stg); };
  // input stages in flight: PBRT_WS_STAGES (2..6) fixes the count; by
  // default the count of 2..4 with the most resident CTAs, the deeper ring
  // among equals, and a shallower one only while every CTA still walks 16
  // tiles or more (d0a, 80 channels at 1080p: two CTAs an SM with two
  // stages, 245 us, against one with four, 302 us; e1a, 4080 tiles: four
  // stages and two CTAs, 36 us, against two and four, 42 us)
  static const int env_stages = [] {
    const char* e = std::getenv("PBRT_WS_STAGES");
    return e ? std::min(6, std::max(2, std::atoi(e))) : 0;
  }();
  static PerDeviceOnce attrs;
  int ast = once_per_device(attrs, [&]() -> int {
    cudaError_t e = cudaFuncSetAttribute(conv3x3_umma_ws_kernel<NC, kF8>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max);
    if (e == cudaSuccess && kSwzForm)
      e = cudaFuncSetAttribute(conv3x3_umma_ws_kernel<NC, kF8, kSwzForm>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem_max);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(conv3x3_umma_ws_kernel)");
    return PBRT_OK;
  });
  if (ast) return ast;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  constexpr int kCols = 2 * NC <= 64 ? 64 : (2 * NC <= 128 ? 128 : 256);
  // the gather warps only when some planes are not loaded by the TMA (FP8: always, they quantise)
  const bool gather = kF8 || !use_tma || a.c2 > 0;
  const int threads = gather ? kWsThreads : kWsThreads - 32 * kWsGatherWarps;
  // resident CTAs an SM at a given dynamic shared-memory size, from the
  // kernel's registers (warp granules of 256), its static shared memory and
  // the 1 KB the system reserves per CTA, within 228 KB an SM
  int regs_cta = 0, static_smem = 0;
  {
    cudaFuncAttributes fa;
    const cudaError_t e = x1_swz ? cudaFuncGetAttributes(&fa, conv3x3_umma_ws_kernel<NC, kF8, kSwzForm>)
                                 : cudaFuncGetAttributes(&fa, conv3x3_umma_ws_kernel<NC, kF8>);
    if (e == cudaSuccess && fa.numRegs > 0) {
      regs_cta = (threads / 32) * ((fa.numRegs * 32 + 255) / 256 * 256);
      static_smem = (int)fa.sharedSizeBytes;
    } else {
      cudaGetLastError();
    }
  }
  auto resident = [&](size_t smem) {
    const int fit = regs_cta ? std::min(65536 / regs_cta, (int)((228 * 1024) / (smem + static_smem + 1024))) : 1;
    return std::max(1, std::min({4, fit, 512 / kCols}));
  };
  const int tiles_per_image = ((a.W + umma::kTileW - 1) / umma::kTileW) * ((a.H + umma::kTileH - 1) / umma::kTileH);
  const long total_tiles = (long)tiles_per_image * a.N;
  // stage count for a stage layout (stg box planes a stage)
  auto pick_stages = [&](int stg) {
    int stages = env_stages ? env_stages : 4;
    while (stages > 2 && smem_at(stages, stg) > smem_max) --stages;
    if (!env_stages) {
      int best = stages, best_r = resident(smem_at(stages, stg));
      for (int st = stages - 1; st >= 2; --st) {
        const int r = resident(smem_at(st, stg));
        if (r > best_r && total_tiles >= 16L * sms * r) best = st, best_r = r;
      }
      stages = best;
    }
    return stages;
  };
  // the second input's half-resolution box by TMA (expanded in shared
  // memory by the gather warps) where the x1 halo comes by TMA, two stages
  // fit and the box's room costs no resident CTA; else its planes are
  // gathered with cp.async (BF16 d0a at 1080p: box 295 us with one CTA an
  // SM, gathers 245 us with two; d1a: box 108 us, gathers 148 us, one CTA
  // either way; FP8 d0a: box 242 us, gathers 309 us, two CTAs either way)
  int stg = 0;
  if (use_tma && box_flag && a.c2 > 0 && smem_at(2, a.c2 / 8) <= smem_max &&
      resident(smem_at(pick_stages(a.c2 / 8), a.c2 / 8)) >= resident(smem_at(pick_stages(0), 0)) &&
      make_x2_map(&map2, a.x2, a.N, a.H >> 1, a.W >> 1, a.c2))
    stg = a.c2 / 8;
  const int stages = pick_stages(stg);
  const size_t smem = smem_at(stages, stg);
  const int per_sm = resident(smem);
  const int grid = (int)std::min(total_tiles, (long)sms * per_sm);
  if (x1_swz)
    conv3x3_umma_ws_kernel<NC, kF8, kSwzForm><<<grid, threads, smem, s>>>(a, tiles_per_image, map, map2, use_tma, stg,
                                                                         stages, x1_swz);
  else
    conv3x3_umma_ws_kernel<NC, kF8><<<grid, threads, smem, s>>>(a, tiles_per_image, map, map2, use_tma, stg, stages,
                                                                 0);
  return PBRT_OK;
}

template <int NC> int launch_umma_persistent(const UmmaConvArgs& a, cudaStream_t s, bool use_tma_flag) {
  const size_t smem = persistent_smem(a.c1 + a.c2, NC);
  static PerDeviceOnce attrs;
  int ast = once_per_device(attrs, [&]() -> int {
    cudaError_t e = cudaFuncSetAttribute(conv3x3_umma_persistent_kernel<NC>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPersistentSmemMax);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(conv3x3_umma_persistent_kernel)");
    return PBRT_OK;
  });
  if (ast) return ast;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  constexpr int kCols = 2 * NC <= 64 ? 64 : (2 * NC <= 128 ? 128 : 256);  // tensor memory per CTA
  const int per_sm = std::max(1, std::min({4, (int)((227 * 1024) / smem), 512 / kCols}));
  const int tiles_per_image = ((a.W + umma::kTileW - 1) / umma::kTileW) * ((a.H + umma::kTileH - 1) / umma::kTileH);
  const int grid = std::min(tiles_per_image * a.N, sms * per_sm);
  CUtensorMap map;
  memset(&map, 0, sizeof(map));
  const int use_tma = use_tma_flag && make_x1_map(&map, a.x1, a.N, a.H, a.W, a.c1) ? 1 : 0;
  conv3x3_umma_persistent_kernel<NC><<<grid, 128, smem, s>>>(a, tiles_per_image, map, use_tma);
  return PBRT_OK;
}
}  // namespace

bool pbrt::nn_fp8_umma_fits(const void* x1, int c1, const void* x2, int c2, const void* w8, int cout, int h, int w,
                            bool pooled) {
  return ws_smem_f8(c1 + c2, cout, 2) <= kWsSmemMaxF8 && !((uintptr_t)x1 & 15) && !((uintptr_t)x2 & 15) &&
         !((uintptr_t)w8 & 15) && !(pooled && (h % umma::kTileH || w % umma::kTileW));
}

bool pbrt::nn_umma_pooled_fits(int c1, int cout, int h, int w) {
  return h % umma::kTileH == 0 && w % umma::kTileW == 0 && ws_smem(c1, cout, 2) <= kWsSmemMax;
}

extern "C" {

// tcgen05 forward convolution (BF16 output only): Cout in {16, 32, 48, 64,
// 80, 96, 112, 128}, channel counts multiples of 16; flags bit 0: ReLU,
// bit 1: the per-tile kernel only, bit 2: no TMA (cp.async gathers), bit 3:
// the single-role persistent kernel instead of the warp-specialised one,
// bit 4: the upsampled second input by cp.async gathers, not the TMA box,
// bit 5: the x1 halo as 8-channel planes, not swizzled pixel rows.
PBRT_API int pbrt_nn_conv3x3_umma(const void* x1, int32_t c1, const void* x2, int32_t c2, const void* w,
                                  const float* bias, void* y, int32_t n, int32_t h, int32_t wd, int32_t cout,
                                  int32_t flags, pbrt_stream_t stream) {
  if (!x1 || !w || !y || c1 <= 0 || c1 % 16 || c2 < 0 || c2 % 16 || (c2 && !x2) || cout < 16 || cout > 128 ||
      cout % 16 || n <= 0 || h <= 0 || wd <= 0 || (c2 && (h % 2 || wd % 2)))
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "nn conv3x3 umma: bad arguments (c1 %d, c2 %d, cout %d)", c1, c2, cout);
  UmmaConvArgs a{(const bf16*)x1, (const bf16*)x2, c1, c2, (const bf16*)w, bias, (bf16*)y, n, h, wd, cout, flags};
  int st;
  // warp-specialised form (the upsampled second input comes from its gather warps)
  if (!(flags & 10) && ws_smem(c1 + c2, cout, 2) <= kWsSmemMax) {
    switch (cout) {
      case 16: st = launch_umma_ws<16, false>(a, stream, !(flags & 4), !(flags & 16), !(flags & 32)); break;
      case 32: st = launch_umma_ws<32, false>(a, stream, !(flags & 4), !(flags & 16), !(flags & 32)); break;
      case 48: st = launch_umma_ws<48, false>(a, stream, !(flags & 4), !(flags & 16), !(flags & 32)); break;
      case 64: st = launch_umma_ws<64, false>(a, stream, !(flags & 4), !(flags & 16), !(flags & 32)); break;
      case 80: st = launch_umma_ws<80, false>(a, stream, !(flags & 4), !(flags & 16), !(flags & 32)); break;
      case 96: st = launch_umma_ws<96, false>(a, stream, !(flags & 4), !(flags & 16), !(flags & 32)); break;
      case 112: st = launch_umma_ws<112, false>(a, stream, !(flags & 4), !(flags & 16), !(flags & 32)); break;
      default: st = launch_umma_ws<128, false>(a, stream, !(flags & 4), !(flags & 16), !(flags & 32)); break;
    }
    if (st) return st;
    return check_launch("conv3x3_umma_ws_kernel");
  }
  if (!(flags & 2) && persistent_smem(c1 + c2, cout) <= kPersistentSmemMax) {
    switch (cout) {
      case 16: st = launch_umma_persistent<16>(a, stream, !(flags & 4)); break;
      case 32: st = launch_umma_persistent<32>(a, stream, !(flags & 4)); break;
      case 48: st = launch_umma_persistent<48>(a, stream, !(flags & 4)); break;
      case 64: st = launch_umma_persistent<64>(a, stream, !(flags & 4)); break;
      case 80: st = launch_umma_persistent<80>(a, stream, !(flags & 4)); break;
      case 96: st = launch_umma_persistent<96>(a, stream, !(flags & 4)); break;
      case 112: st = launch_umma_persistent<112>(a, stream, !(flags & 4)); break;
      default: st = launch_umma_persistent<128>(a, stream, !(flags & 4)); break;
    }
    if (st) return st;
    return check_launch("conv3x3_umma_persistent_kernel");
  }
  switch (cout) {
    case 16: st = launch_umma<16>(a, stream); break;
    case 32: st = launch_umma<32>(a, stream); break;
    case 48: st = launch_umma<48>(a, stream); break;
    case 64: st = launch_umma<64>(a, stream); break;
    case 80: st = launch_umma<80>(a, stream); break;
    case 96: st = launch_umma<96>(a, stream); break;
    case 112: st = launch_umma<112>(a, stream); break;
    default: st = launch_umma<128>(a, stream); break;
  }
  if (st) return st;
  return check_launch("conv3x3_umma_kernel");
}

// The warp-specialised convolution of a single input that also writes the
// 2x2 average pooling of its output (the next encoder level's input; the
// same bits as pbrt_nn_avgpool2 of y). Needs h % 16 == 0, wd % 8 == 0 and
// the warp-specialised kernel's shared memory; PBRT_ERROR_UNSUPPORTED
// otherwise (the caller pools separately).
PBRT_API int pbrt_nn_conv3x3_umma_pooled(const void* x1, int32_t c1, const void* w, const float* bias, void* y,
                                         void* pooled, int32_t n, int32_t h, int32_t wd, int32_t cout, int32_t flags,
                                         pbrt_stream_t stream) {
  if (!x1 || !w || !y || !pooled || c1 <= 0 || c1 % 16 || cout < 16 || cout > 128 || cout % 16 || n <= 0 || h <= 0 ||
      wd <= 0)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "nn conv3x3 umma pooled: bad arguments (c1 %d, cout %d)", c1, cout);
  if (!nn_umma_pooled_fits(c1, cout, h, wd))
    return fail(PBRT_ERROR_UNSUPPORTED, "nn conv3x3 umma pooled: %dx%d, c1 %d, cout %d", wd, h, c1, cout);
  UmmaConvArgs a{(const bf16*)x1, nullptr, c1, 0, (const bf16*)w, bias, (bf16*)y, n, h, wd, cout, flags};
  a.pooled = (bf16*)pooled;
  int st;
  switch (cout) {
    case 16: st = launch_umma_ws<16, false>(a, stream, true, true, !(flags & 32)); break;
    case 32: st = launch_umma_ws<32, false>(a, stream, true, true, !(flags & 32)); break;
    case 48: st = launch_umma_ws<48, false>(a, stream, true, true, !(flags & 32)); break;
    case 64: st = launch_umma_ws<64, false>(a, stream, true, true, !(flags & 32)); break;
    case 80: st = launch_umma_ws<80, false>(a, stream, true, true, !(flags & 32)); break;
    case 96: st = launch_umma_ws<96, false>(a, stream, true, true, !(flags & 32)); break;
    case 112: st = launch_umma_ws<112, false>(a, stream, true, true, !(flags & 32)); break;
    default: st = launch_umma_ws<128, false>(a, stream, true, true, !(flags & 32)); break;
  }
  if (st) return st;
  return check_launch("conv3x3_umma_ws_kernel (pooled)");
}

// Backward weights on tcgen05 (conv3x3_wgrad_umma_ws_kernel): the arguments of
// pbrt_nn_conv3x3_wgrad; dw is accumulated into.
PBRT_API int pbrt_nn_conv3x3_wgrad_umma(const void* dy, const void* x1, int32_t c1, const void* x2, int32_t c2,
                                        float* dw, int32_t n, int32_t h, int32_t wd, int32_t cout,
                                        pbrt_stream_t stream) {
  if (!dy || !x1 || !dw || c1 <= 0 || c1 % 16 || c2 < 0 || c2 % 16 || (c2 && !x2) || c1 + c2 > 256 || cout <= 0 ||
      cout % 16 || cout > 128 || n <= 0 || h <= 0 || wd <= 0 || (c2 && (h % 2 || wd % 2)) || ((uintptr_t)dy & 15) ||
      ((uintptr_t)x1 & 15) || ((uintptr_t)x2 & 15))
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "nn conv3x3 wgrad umma: bad arguments (c1 %d, c2 %d, cout %d)", c1, c2,
                cout);
  const int cin = c1 + c2;
  // taps a CTA: three while their accumulators take at most half the
  // tensor memory, else one; three stages. Two or three CTAs an SM on the
  // full- and half-resolution layers (one CTA of all nine taps, 512
  // columns and four stages, left the SM's issue slots 88 % idle: d0b
  // 310 us, d0a 808 us at 16 x 256^2)
  const int ntaps = wgrad_cols(3 * cin) <= 256 ? 3 : 1;
  const int cols = (int)wgrad_cols(ntaps * cin);
  constexpr size_t kMaxSmem = 210 * 1024;  // below the opt-in limit less the kernel's static shared memory
  const int stages = 3;
  const size_t smem = (size_t)stages * wgrad_stage_bytes(cin) + 1024;
  static PerDeviceOnce attrs;
  int ast = once_per_device(attrs, [&]() -> int {
    cudaError_t e = cudaFuncSetAttribute(conv3x3_wgrad_umma_ws_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kMaxSmem);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(conv3x3_wgrad_umma_ws_kernel)");
    return PBRT_OK;
  });
  if (ast) return ast;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  // resident CTAs an SM: shared memory and the 512 tensor-memory columns
  const int per_sm = std::max(1, std::min((int)((227 * 1024) / (smem + 1024)), 512 / cols));
  const long tiles = (long)n * ((h + kWgT - 1) / kWgT) * ((wd + kWgT - 1) / kWgT);
  const int groups = 9 / ntaps;
  // one wave: each CTA walks its share of the tiles for its taps
  const long per_group = std::max(1L, std::min(tiles, (long)sms * per_sm / groups));
  UmmaWgradArgs a{(const bf16*)dy, (const bf16*)x1, (const bf16*)x2, c1, c2, dw, n, h, wd, cout, ntaps, stages};
  // dY's 8x8 tile and x1's 10x10 halo by TMA: 5-D maps [8 channels][x][y]
  // [channel group][image] whose boxes land in the operands' layout
  CUtensorMap dymap, x1map;
  memset(&dymap, 0, sizeof(dymap));
  memset(&x1map, 0, sizeof(x1map));
  int use_tma = 0;
  if (EncodeTiledFn enc = encode_tiled()) {
    const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
    const cuuint64_t ddims[5] = {8, (cuuint64_t)wd, (cuuint64_t)h, (cuuint64_t)(cout / 8), (cuuint64_t)n};
    const cuuint64_t dstr[4] = {(cuuint64_t)cout * 2, (cuuint64_t)wd * cout * 2, 16, (cuuint64_t)h * wd * cout * 2};
    const cuuint32_t dbox[5] = {8, kWgT, kWgT, (cuuint32_t)(cout / 8), 1};
    const cuuint64_t xdims[5] = {8, (cuuint64_t)wd, (cuuint64_t)h, (cuuint64_t)(c1 / 8), (cuuint64_t)n};
    const cuuint64_t xstr[4] = {(cuuint64_t)c1 * 2, (cuuint64_t)wd * c1 * 2, 16, (cuuint64_t)h * wd * c1 * 2};
    const cuuint32_t xbox[5] = {8, kWgHalo, kWgHalo, (cuuint32_t)(c1 / 8), 1};
    use_tma = enc(&dymap, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void*>(dy), ddims, dstr, dbox, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS &&
              enc(&x1map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void*>(x1), xdims, xstr, xbox, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
  }
  if (!use_tma) return fail(PBRT_ERROR_UNSUPPORTED, "nn conv3x3 wgrad umma: no tensor maps (c1 %d, cout %d)", c1, cout);
  dim3 grid((unsigned)groups, (unsigned)per_group);
  conv3x3_wgrad_umma_ws_kernel<<<grid, 128, smem, stream>>>(a, dymap, x1map);
  return check_launch("conv3x3_wgrad_umma_ws_kernel");
}

// tcgen05 convolution of a single input with an FP32 output (the backward-
// data pass: dY convolved with the flipped weights), any Cout that is a
// multiple of 16: the output channels are split into slices whose weights
// and two input stages fit the warp-specialised kernel's shared memory, one
// launch a slice, each writing its columns of y32 (pixel stride cout).
// PBRT_ERROR_UNSUPPORTED when no slicing fits (c1 too large).
PBRT_API int pbrt_nn_conv3x3_umma_f32(const void* x1, int32_t c1, const void* w, const float* bias, float* y32,
                                      int32_t n, int32_t h, int32_t wd, int32_t cout, int32_t flags,
                                      pbrt_stream_t stream) {
  if (!x1 || !w || !y32 || c1 <= 0 || c1 % 16 || cout < 16 || cout % 16 || n <= 0 || h <= 0 || wd <= 0 ||
      ((uintptr_t)y32 & 15) || ((uintptr_t)x1 & 15) || ((uintptr_t)w & 15))
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "nn conv3x3 umma f32: bad arguments (c1 %d, cout %d)", c1, cout);
  int slice = 0;
  for (int parts = (cout + 127) / 128; parts <= cout / 16; ++parts) {
    const int nc = ((cout + parts - 1) / parts + 15) / 16 * 16;
    if (nc <= 128 && ws_smem(c1, nc, 2) <= kWsSmemMax) {
      slice = nc;
      break;
    }
  }
  if (!slice) return fail(PBRT_ERROR_UNSUPPORTED, "nn conv3x3 umma f32: c1 %d, cout %d", c1, cout);
  for (int o = 0; o < cout; o += slice) {
    const int nc = std::min(slice, cout - o);
    UmmaConvArgs a{(const bf16*)x1, nullptr, c1, 0, (const bf16*)w + (size_t)o * 9 * c1, bias ? bias + o : nullptr,
                   nullptr, n, h, wd, nc, flags & 1};
    a.y32 = y32 + o;
    a.ldy32 = cout;
    int st;
    switch (nc) {
      case 16: st = launch_umma_ws<16, false>(a, stream, !(flags & 4)); break;
      case 32: st = launch_umma_ws<32, false>(a, stream, !(flags & 4)); break;
      case 48: st = launch_umma_ws<48, false>(a, stream, !(flags & 4)); break;
      case 64: st = launch_umma_ws<64, false>(a, stream, !(flags & 4)); break;
      case 80: st = launch_umma_ws<80, false>(a, stream, !(flags & 4)); break;
      case 96: st = launch_umma_ws<96, false>(a, stream, !(flags & 4)); break;
      case 112: st = launch_umma_ws<112, false>(a, stream, !(flags & 4)); break;
      default: st = launch_umma_ws<128, false>(a, stream, !(flags & 4)); break;
    }
    if (st) return st;
    const int e = check_launch("conv3x3_umma_ws_kernel (f32)");
    if (e) return e;
  }
  return PBRT_OK;
}

// FP8 (e4m3) convolution on the tensor cores (kind::f8f6f4): the arguments
// and quantisation of pbrt_nn_conv3x3_fp8, plus the optional fused 2x2
// pooling of pbrt_nn_conv3x3_umma_pooled (single input only); flags bit 0:
// ReLU, bit 4: the upsampled second input by cp.async gathers.
// PBRT_ERROR_UNSUPPORTED when the weights and two input stages do not fit
// in shared memory, an operand is not 16-byte aligned, or (pooled) the
// frame does not divide into 16 x 8 tiles.
PBRT_API int pbrt_nn_conv3x3_fp8_umma(const void* x1, int32_t c1, const void* x2, int32_t c2, const void* w8,
                                      const float* wscale, const float* inv_xscale, const float* bias, void* y,
                                      void* pooled, int32_t n, int32_t h, int32_t wd, int32_t cout, int32_t flags,
                                      pbrt_stream_t stream) {
  if (!x1 || !w8 || !wscale || !inv_xscale || !y || c1 <= 0 || c1 % 16 || c2 < 0 || c2 % 16 || (c2 && !x2) ||
      c1 + c2 > 256 || cout < 16 || cout > 128 || cout % 16 || n <= 0 || h <= 0 || wd <= 0 ||
      (c2 && (h % 2 || wd % 2)) || (pooled && c2))
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "nn conv3x3 fp8 umma: bad arguments (c1 %d, c2 %d, cout %d)", c1, c2,
                cout);
  if (!nn_fp8_umma_fits(x1, c1, x2, c2, w8, cout, h, wd, pooled != nullptr))
    return fail(PBRT_ERROR_UNSUPPORTED, "nn conv3x3 fp8 umma: %dx%d, c1 %d, c2 %d, cout %d", wd, h, c1, c2, cout);
  UmmaConvArgs a{(const bf16*)x1, (const bf16*)x2, c1, c2, nullptr, bias, (bf16*)y, n, h, wd, cout, flags};
  a.pooled = (bf16*)pooled;
  a.w8 = (const uint8_t*)w8;
  a.wscale = wscale;
  a.inv_xscale = inv_xscale;
  int st;
  switch (cout) {
    case 16: st = launch_umma_ws<16, true>(a, stream, true, !(flags & 16)); break;
    case 32: st = launch_umma_ws<32, true>(a, stream, true, !(flags & 16)); break;
    case 48: st = launch_umma_ws<48, true>(a, stream, true, !(flags & 16)); break;
    case 64: st = launch_umma_ws<64, true>(a, stream, true, !(flags & 16)); break;
    case 80: st = launch_umma_ws<80, true>(a, stream, true, !(flags & 16)); break;
    case 96: st = launch_umma_ws<96, true>(a, stream, true, !(flags & 16)); break;
    case 112: st = launch_umma_ws<112, true>(a, stream, true, !(flags & 16)); break;
    default: st = launch_umma_ws<128, true>(a, stream, true, !(flags & 16)); break;
  }
  if (st) return st;
  return check_launch("conv3x3_umma_ws_kernel (fp8)");
}

// Error flags of the tcgen05 kernels since the last call (bit 0: an
// mbarrier wait timed out); resets them (stream-synchronising).
PBRT_API int pbrt_nn_umma_status(pbrt_stream_t stream, uint32_t* flags) {
  if (!flags) return fail(PBRT_ERROR_INVALID_ARGUMENT, "umma status: null output");
  PBRT_CUDA(cudaStreamSynchronize(stream));
  PBRT_CUDA(cudaMemcpyFromSymbol(flags, g_umma_error, sizeof(uint32_t)));
  const uint32_t zero = 0;
  PBRT_CUDA(cudaMemcpyToSymbol(g_umma_error, &zero, sizeof(uint32_t)));
  return PBRT_OK;
}

}  // extern "C"
