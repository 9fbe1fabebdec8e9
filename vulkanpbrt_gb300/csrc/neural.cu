// Inference object of the kernel-predicting denoiser: a render module like
// BMFR (reads the G-buffer and the 1-spp demodulated illumination, writes a
// denoised RGBA32F image and a tone-mapped B8G8R8A8 final image), with the
// per-tile variance gate that hands tiles back to a BMFR object's final
// image. The forward pass is the fixed launch sequence of the U-Net
// (features, 18 convolutions, 4 poolings, 3 heads, compose), captured in a
// CUDA graph on the first dispatch and replayed afterwards.
// No reference counterpart: the reference's denoisers are BMFR and BFR
// (source/renderModules/BMFR.cpp, source/renderModules/BFR.cpp).
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "internal.hpp"

namespace pbrt {
namespace neural {

typedef __nv_bfloat16 bf16;

struct ConvSpec {
  const char* name;
  int c1, c2, cout, level;
};
// Same order and shapes as vulkanpbrt_gb300/kpunet.py (ENCODER + DECODER).
constexpr ConvSpec kConvs[] = {
    {"e0a", 16, 0, 32, 0},  {"e0b", 32, 0, 32, 0},   {"e1a", 32, 0, 48, 1},  {"e1b", 48, 0, 48, 1},
    {"e2a", 48, 0, 64, 2},  {"e2b", 64, 0, 64, 2},   {"e3a", 64, 0, 96, 3},  {"e3b", 96, 0, 96, 3},
    {"e4a", 96, 0, 128, 4}, {"e4b", 128, 0, 128, 4}, {"d3a", 96, 128, 96, 3}, {"d3b", 96, 0, 96, 3},
    {"d2a", 64, 96, 64, 2}, {"d2b", 64, 0, 64, 2},   {"d1a", 48, 64, 48, 1}, {"d1b", 48, 0, 48, 1},
    {"d0a", 32, 48, 32, 0}, {"d0b", 32, 0, 32, 0}};
constexpr int kNumConvs = sizeof(kConvs) / sizeof(kConvs[0]);
struct HeadSpec {
  int feature_conv, c, k, scale;
};
constexpr HeadSpec kHeads[] = {{13, 64, 25, 2}, {15, 48, 26, 1}, {17, 32, 27, 0}};  // d2b, d1b, d0b

struct Layout {
  size_t conv_w[kNumConvs], conv_b[kNumConvs], head_w[3], head_b[3], total, conv_w_total;
  Layout() {
    size_t off = 0;
    for (int i = 0; i < kNumConvs; ++i) {
      conv_w[i] = off;
      off += (size_t)kConvs[i].cout * 9 * (kConvs[i].c1 + kConvs[i].c2);
    }
    conv_w_total = off;
    for (int i = 0; i < kNumConvs; ++i) {
      conv_b[i] = off;
      off += kConvs[i].cout;
    }
    for (int h = 0; h < 3; ++h) {
      head_w[h] = off;
      off += (size_t)kHeads[h].k * kHeads[h].c;
      head_b[h] = off;
      off += kHeads[h].k;
    }
    total = off;
  }
};

__global__ void to_bf16_kernel(const float* __restrict__ src, bf16* __restrict__ dst, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = __float2bfloat16_rn(src[i]);
}

}  // namespace neural
}  // namespace pbrt

using namespace pbrt;
using namespace pbrt::neural;

struct PbrtNeural : pbrt::Object {
  PbrtNeural() : Object(pbrt::Kind::Neural) {}
  ~PbrtNeural() override;
  uint32_t width = 0, height = 0, pw = 0, ph = 0;
  PbrtGBuffer* gbuffer = nullptr;
  PbrtIlluminationBuffer* illumination = nullptr;
  PbrtAccumulationBuffer* acc = nullptr;  // optional: samples per pixel of accumulated input
  PbrtBMFR* fallback = nullptr;
  float threshold = 0.f;
  int32_t tile = 32;
  bool gate_model = false;  // the learned tile gate instead of the threshold on the predicted error
  float gate_coef[36] = {};
  Layout lay;
  float* params = nullptr;  // FP32, lay.total
  bf16* w16 = nullptr;      // BF16 convolution weights, lay.conv_w_total
  bf16* feat = nullptr;
  bf16* act[kNumConvs] = {};
  bf16* pool[5] = {};
  float* rad[3] = {};
  float* out[3] = {};
  pbrt::DeviceImage variance, denoised, final_image;
  pbrt::DeviceImage mask;  // R8 per gate tile: 1 = fallback
  uint32_t* counter = nullptr;
  cudaGraphExec_t graph = nullptr;
  // per layer: 0 = mma.sync kernels, 1 = tcgen05 kernel (chosen by timing both on the first dispatch)
  int32_t conv_kernel[kNumConvs] = {};
  bool tuned = false;
  // FP8 inference (pbrt_neural_calibrate / pbrt_neural_set_precision):
  // per layer, e4m3 where the calibration timed it faster than BF16
  int precision = 16;
  bool fp8_layer[kNumConvs] = {};
  bool calibrated = false;
  uint8_t* w8 = nullptr;      // e4m3 convolution weights, lay.conv_w_total
  float* wscale = nullptr;    // per output channel, all convolutions
  float* xscale = nullptr;    // per input channel, all convolutions
  float* inv_xscale = nullptr;
  size_t wsoff[kNumConvs] = {}, xsoff[kNumConvs] = {}, n_wscale = 0, n_xscale = 0;
};

namespace {

template <class T> int dalloc(T** p, size_t count) {
  *p = nullptr;
  cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc (neural)");
  return PBRT_OK;
}

// Convolution i of the forward pass (x: its input, or its skip-concatenated
// decoder input's upsampled part), in FP8 (e4m3, after calibration) or BF16
// on the layer's chosen kernel. *pooled: the convolution also wrote the next
// encoder level's 2x2-pooled input from its epilogue.
int conv_layer(PbrtNeural* nd, int i, const bf16* x, bool fp8, cudaStream_t s, bool* pooled) {
  const int n = 1;
  const ConvSpec& c = kConvs[i];
  const int h = nd->ph >> c.level, w = nd->pw >> c.level;
  const bf16* w16 = nd->w16 + nd->lay.conv_w[i];
  const float* b = nd->params + nd->lay.conv_b[i];
  const int skip_of[4] = {1, 3, 5, 7};  // e0b, e1b, e2b, e3b
  const bf16* in1 = c.c2 ? nd->act[skip_of[c.level]] : x;
  const bf16* in2 = c.c2 ? x : nullptr;
  *pooled = false;
  int st;
  // an encoder level's second convolution on the tcgen05 kernel pools its
  // output in the epilogue (levels 0-2; the frame must divide into tiles)
  const bool pool_here = i < 8 && (i & 1) && c.c2 == 0 && nd->conv_kernel[i] >= 1 && !fp8 &&
                         nn_umma_pooled_fits(c.c1, c.cout, h, w);
  // tcgen05: kind 1 loads the first input's halo as swizzled pixel rows
  // where the layer's shape allows, kind 2 as 8-channel planes (flags bit 5)
  const int umma_flags = 1 | (nd->conv_kernel[i] == 2 ? 32 : 0);
  if (fp8) {
    const uint8_t* w8 = nd->w8 + nd->lay.conv_w[i];
    const float* wsc = nd->wscale + nd->wsoff[i];
    const float* ixs = nd->inv_xscale + nd->xsoff[i];
    if (i < 8 && (i & 1) && c.c2 == 0 && nn_fp8_umma_fits(in1, c.c1, nullptr, 0, w8, c.cout, h, w, true)) {
      // the encoder's pooling in the FP8 convolution's epilogue
      st = pbrt_nn_conv3x3_fp8_umma(in1, c.c1, nullptr, 0, w8, wsc, ixs, b, nd->act[i], nd->pool[c.level + 1], n, h,
                                    w, c.cout, 1, s);
      *pooled = st == PBRT_OK;
      return st;
    }
    return pbrt_nn_conv3x3_fp8(in1, c.c1, in2, c.c2, w8, wsc, ixs, b, nd->act[i], n, h, w, c.cout, 1, s);
  }
  if (pool_here && (st = pbrt_nn_conv3x3_umma_pooled(in1, c.c1, w16, b, nd->act[i], nd->pool[c.level + 1], n, h, w,
                                                     c.cout, umma_flags, s)) != PBRT_ERROR_UNSUPPORTED) {
    *pooled = st == PBRT_OK;
    return st;
  }
  if (nd->conv_kernel[i] >= 1)
    return pbrt_nn_conv3x3_umma(in1, c.c1, in2, c.c2, w16, b, nd->act[i], n, h, w, c.cout, umma_flags, s);
  return pbrt_nn_conv3x3(in1, c.c1, in2, c.c2, w16, b, nd->act[i], nullptr, n, h, w, c.cout, 1, s);
}

int record_forward(PbrtNeural* nd, cudaStream_t s) {
  const int n = 1, PH = nd->ph, PW = nd->pw;
  const PbrtIlluminationBuffer* ib = nd->illumination;
  const DeviceImage& illum = ib->demodulated();
  const int is_half = illum.view.format == PBRT_FORMAT_R16G16B16A16_SFLOAT;
  int st;
  if ((st = pbrt_nn_features(illum.view.data, is_half, nd->gbuffer->albedo.view.data, nd->gbuffer->normal.view.data,
                             nd->gbuffer->depth.view.data, nd->acc ? nd->acc->spp.view.data : nullptr, nd->width,
                             nd->height, PW, PH, n, nd->feat, nd->rad[0], s)))
    return st;
  if ((st = pbrt_nn_avgpool2(nd->rad[0], nd->rad[1], 1, n, PH, PW, 3, s))) return st;
  if ((st = pbrt_nn_avgpool2(nd->rad[1], nd->rad[2], 1, n, PH / 2, PW / 2, 3, s))) return st;
  const bf16* x = nd->feat;
  bool pooled = false;  // the previous convolution also wrote the next level's pooled input
  for (int i = 0; i < kNumConvs; ++i) {
    const ConvSpec& c = kConvs[i];
    const int h = PH >> c.level, w = PW >> c.level;
    if (i < 10 && c.name[2] == 'a' && c.level > 0) {  // encoder: pool the previous level's output first
      if (!pooled && (st = pbrt_nn_avgpool2(x, nd->pool[c.level], 0, n, h * 2, w * 2, kConvs[i - 1].cout, s)))
        return st;
      x = nd->pool[c.level];
    }
    if ((st = conv_layer(nd, i, x, nd->precision == 8 && nd->fp8_layer[i], s, &pooled))) return st;
    x = nd->act[i];
  }
  for (int k = 0; k < 3; ++k) {
    const HeadSpec& hs = kHeads[k];
    const int h = PH >> hs.scale, w = PW >> hs.scale;
    const float* coarse = hs.scale < 2 ? nd->out[hs.scale + 1] : nullptr;
    float* var = hs.scale == 0 ? nd->variance.ptr<float>() : nullptr;
    if ((st = pbrt_nn_kp_head(nd->act[hs.feature_conv], nd->params + nd->lay.head_w[k], nd->params + nd->lay.head_b[k],
                              nd->rad[hs.scale], coarse, nd->out[hs.scale], nullptr, nullptr, nullptr, var, n, h, w,
                              hs.c, hs.k, s)))
      return st;
  }
  const bool gate = nd->fallback != nullptr && !nd->gate_model;
  if (nd->fallback) PBRT_CUDA(cudaMemsetAsync(nd->counter, 0, sizeof(uint32_t), s));
  if (gate) {
    if ((st = pbrt_nn_gate(nd->variance.ptr<float>(), PW, nd->width, nd->height, nd->threshold, nd->tile,
                           nd->mask.ptr<uint8_t>(), nd->counter, s)))
      return st;
  }
  if ((st = pbrt_nn_compose(nd->out[0], PW, nd->width, nd->height, nd->gbuffer->albedo.view.data,
                            gate ? nd->mask.ptr<uint8_t>() : nullptr, nd->tile,
                            gate ? nd->fallback->final_image.view.data : nullptr, nd->final_image.view.data,
                            nd->denoised.ptr<float>(), s)))
    return st;
  if (!nd->fallback || !nd->gate_model) return PBRT_OK;
  // the learned gate reads the composed network image and BMFR's and overwrites the tiles it hands to BMFR
  return pbrt_nn_gate_model(nd->variance.ptr<float>(), nd->out[0], PW, nd->width, nd->height, nd->tile,
                            nd->fallback->final_image.view.data, nd->fallback->denoised.view.data,
                            nd->fallback->last_layer, nd->acc ? nd->acc->spp.ptr<uint8_t>() : nullptr,
                            illum.view.data, is_half, nd->gbuffer->depth.ptr<float>(),
                            nd->gbuffer->normal.view.data, nd->gbuffer->albedo.view.data, nd->gate_coef,
                            nd->mask.ptr<uint8_t>(), nd->counter, nd->final_image.view.data,
                            nd->denoised.ptr<float>(), s);
}

void drop_graph(PbrtNeural* nd) {
  if (nd->graph) cudaGraphExecDestroy(nd->graph);
  nd->graph = nullptr;
}

}  // namespace

PbrtNeural::~PbrtNeural() {
  drop_graph(this);
  cudaFree(params);
  cudaFree(w16);
  cudaFree(feat);
  for (auto* p : act) cudaFree(p);
  for (auto* p : pool) cudaFree(p);
  for (auto* p : rad) cudaFree(p);
  for (auto* p : out) cudaFree(p);
  cudaFree(counter);
  cudaFree(w8);
  cudaFree(wscale);
  cudaFree(xscale);
  cudaFree(inv_xscale);
  variance.free_();
  denoised.free_();
  final_image.free_();
  mask.free_();
  release(gbuffer);
  release(illumination);
  release(acc);
  release(fallback);
}

extern "C" {

PBRT_API int pbrt_neural_param_count(int64_t* count) {
  if (!count) return fail(PBRT_ERROR_INVALID_ARGUMENT, "neural param count: null output");
  *count = (int64_t)Layout().total;
  return PBRT_OK;
}

PBRT_API int pbrt_neural_set_params(PbrtNeural* nd, const float* params_host, int64_t count) {
  if (!checked<PbrtNeural>(nd, Kind::Neural) || !params_host || count != (int64_t)nd->lay.total)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "neural set params: expected %lld parameters, got %lld",
                (long long)(nd ? nd->lay.total : 0), (long long)count);
  PBRT_CUDA(cudaMemcpy(nd->params, params_host, nd->lay.total * sizeof(float), cudaMemcpyHostToDevice));
  nd->calibrated = false;
  if (nd->precision == 8) {
    nd->precision = 16;
    drop_graph(nd);
  }
  to_bf16_kernel<<<256, 256>>>(nd->params, nd->w16, nd->lay.conv_w_total);
  int st = check_launch("to_bf16_kernel");
  if (st) return st;
  PBRT_CUDA(cudaDeviceSynchronize());
  return PBRT_OK;
}

PBRT_API int pbrt_neural_create(uint32_t width, uint32_t height, PbrtGBuffer* g, PbrtIlluminationBuffer* illu,
                                PbrtAccumulationBuffer* acc, const float* params_host, int64_t count,
                                PbrtNeural** out) {
  if (!out || !checked<PbrtGBuffer>(g, Kind::GBuffer) || !checked<PbrtIlluminationBuffer>(illu, Kind::Illumination) ||
      (acc && !checked<PbrtAccumulationBuffer>(acc, Kind::Accumulation)))
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "neural create: bad arguments");
  if (acc && (acc->width != width || acc->height != height))
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "neural create: accumulation buffer size differs");
  *out = nullptr;
  if (g->width != width || g->height != height || illu->width != width || illu->height != height || width < 16 ||
      height < 16)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "neural create: image sizes differ from %ux%u (or below 16)", width,
                height);
  const int32_t f = illu->demodulated().view.format;
  if (f != PBRT_FORMAT_R32G32B32A32_SFLOAT && f != PBRT_FORMAT_R16G16B16A16_SFLOAT)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "neural create: the illumination buffer holds no demodulated image");
  auto* nd = new (std::nothrow) PbrtNeural();
  if (!nd) return fail(PBRT_ERROR_OUT_OF_MEMORY, "neural: host allocation");
  nd->width = width;
  nd->height = height;
  nd->pw = (width + 15) / 16 * 16;
  nd->ph = (height + 15) / 16 * 16;
  retain(g);
  retain(illu);
  if (acc) retain(acc);
  nd->gbuffer = g;
  nd->illumination = illu;
  nd->acc = acc;
  const size_t P = (size_t)nd->pw * nd->ph;
  int st;
  for (int i = 0; i < kNumConvs; ++i) {
    nd->wsoff[i] = nd->n_wscale;
    nd->n_wscale += kConvs[i].cout;
    nd->xsoff[i] = nd->n_xscale;
    nd->n_xscale += kConvs[i].c1 + kConvs[i].c2;
  }
  if ((st = dalloc(&nd->params, nd->lay.total)) || (st = dalloc(&nd->w16, nd->lay.conv_w_total)) ||
      (st = dalloc(&nd->feat, P * 16)) || (st = dalloc(&nd->counter, 1)) ||
      (st = dalloc(&nd->w8, nd->lay.conv_w_total)) || (st = dalloc(&nd->wscale, nd->n_wscale)) ||
      (st = dalloc(&nd->xscale, nd->n_xscale)) || (st = dalloc(&nd->inv_xscale, nd->n_xscale))) {
    delete nd;
    return st;
  }
  for (int i = 0; i < kNumConvs && !st; ++i) st = dalloc(&nd->act[i], (P >> (2 * kConvs[i].level)) * kConvs[i].cout);
  for (int l = 1; l <= 4 && !st; ++l) st = dalloc(&nd->pool[l], (P >> (2 * l)) * kConvs[2 * l - 1].cout);
  for (int s = 0; s < 3 && !st; ++s) st = dalloc(&nd->rad[s], (P >> (2 * s)) * 3);
  for (int s = 0; s < 3 && !st; ++s) st = dalloc(&nd->out[s], (P >> (2 * s)) * 3);
  if (!st) st = nd->variance.alloc(nd->pw, nd->ph, 1, PBRT_FORMAT_R32_SFLOAT);
  if (!st) st = nd->denoised.alloc(width, height, 1, PBRT_FORMAT_R32G32B32A32_SFLOAT);
  if (!st) st = nd->final_image.alloc(width, height, 1, PBRT_FORMAT_B8G8R8A8_UNORM);
  if (!st && params_host) st = pbrt_neural_set_params(nd, params_host, count);
  if (st) {
    delete nd;
    return st;
  }
  *out = nd;
  return PBRT_OK;
}

PBRT_API int pbrt_neural_set_gate_model(PbrtNeural* nd, const float* coef, int32_t n) {
  if (!checked<PbrtNeural>(nd, Kind::Neural) || (coef && n != 36))
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "neural gate model: 36 coefficients (4 x (8 weights, bias)) or null");
  nd->gate_model = coef != nullptr;
  for (int k = 0; k < 36; ++k) nd->gate_coef[k] = coef ? coef[k] : 0.f;
  drop_graph(nd);  // the coefficients are baked into the captured launch
  return PBRT_OK;
}

PBRT_API int pbrt_neural_set_fallback(PbrtNeural* nd, PbrtBMFR* bmfr, float threshold, int32_t tile) {
  if (!checked<PbrtNeural>(nd, Kind::Neural) || (bmfr && !checked<PbrtBMFR>(bmfr, Kind::BMFR)) || tile < 4 ||
      tile > 256)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "neural set fallback: bad arguments");
  if (bmfr && (bmfr->width != nd->width || bmfr->height != nd->height))
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "neural set fallback: BMFR image size differs");
  if (bmfr && (nd->mask.view.width != (uint32_t)((nd->width + tile - 1) / tile) ||
               nd->mask.view.height != (uint32_t)((nd->height + tile - 1) / tile))) {
    nd->mask.free_();
    nd->mask.view = PbrtImage{};
    int st = nd->mask.alloc((nd->width + tile - 1) / tile, (nd->height + tile - 1) / tile, 1, PBRT_FORMAT_R8_UNORM);
    if (st) return st;
  }
  if (bmfr) retain(bmfr);
  release(nd->fallback);
  nd->fallback = bmfr;
  nd->threshold = threshold;
  nd->tile = tile;
  drop_graph(nd);
  return PBRT_OK;
}

// Per-layer kernel choice: one forward pass to have every layer's input,
// then each convolution timed with both kernels (median of 3 after a
// warm-up, CUDA events) and the faster kept. Stream-synchronising.
PBRT_API int pbrt_neural_autotune(PbrtNeural* nd, pbrt_stream_t stream) {
  if (!checked<PbrtNeural>(nd, Kind::Neural)) return fail(PBRT_ERROR_INVALID_ARGUMENT, "neural autotune: not a handle");
  for (int i = 0; i < kNumConvs; ++i) nd->conv_kernel[i] = 0;
  const int saved = nd->precision;
  nd->precision = 16;
  int st = record_forward(nd, stream);
  nd->precision = saved;
  if (st) return st;
  cudaEvent_t e0, e1;
  PBRT_CUDA(cudaEventCreate(&e0));
  PBRT_CUDA(cudaEventCreate(&e1));
  const int skip_of[4] = {1, 3, 5, 7};
  for (int i = 0; i < kNumConvs && !st; ++i) {
    const ConvSpec& c = kConvs[i];
    const int h = nd->ph >> c.level, w = nd->pw >> c.level;
    const bf16* in1;
    const bf16* in2 = nullptr;
    if (i == 0) in1 = nd->feat;
    else if (c.c2) {
      in1 = nd->act[skip_of[c.level]];
      in2 = nd->act[i - 1];
    } else if (i < 10 && c.name[2] == 'a') in1 = nd->pool[c.level];
    else in1 = nd->act[i - 1];
    const bf16* w16 = nd->w16 + nd->lay.conv_w[i];
    const float* b = nd->params + nd->lay.conv_b[i];
    // 0: mma.sync; 1: tcgen05 (swizzled pixel rows for one input of 16 or
    // 32 channels and 32 or 48 out); 2: tcgen05 with 8-channel planes
    // (timed only where 1 differs)
    float best[3] = {1e30f, 1e30f, 1e30f};
    const int kinds = (c.c1 == 16 || c.c1 == 32) && c.c2 == 0 && (c.cout == 32 || c.cout == 48) ? 3 : 2;
    for (int k = 0; k < kinds && !st; ++k) {
      float ms[3];
      for (int r = 0; r < 4 && !st; ++r) {
        cudaEventRecord(e0, stream);
        st = k ? pbrt_nn_conv3x3_umma(in1, c.c1, in2, c.c2, w16, b, nd->act[i], 1, h, w, c.cout, k == 2 ? 33 : 1,
                                      stream)
               : pbrt_nn_conv3x3(in1, c.c1, in2, c.c2, w16, b, nd->act[i], nullptr, 1, h, w, c.cout, 1, stream);
        cudaEventRecord(e1, stream);
        cudaError_t e = cudaEventSynchronize(e1);
        if (!st && e != cudaSuccess) st = cuda_fail(e, "neural autotune");
        if (r > 0) cudaEventElapsedTime(&ms[r - 1], e0, e1);
      }
      if (!st) {
        std::sort(ms, ms + 3);
        best[k] = ms[1];
      }
    }
    int pick = best[1] < best[0] ? 1 : 0;
    if (best[2] < best[pick]) pick = 2;
    nd->conv_kernel[i] = pick;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st) return st;
  uint32_t flags = 0;
  if ((st = pbrt_nn_umma_status(stream, &flags))) return st;
  if (flags) {  // a tcgen05 wait ran out: keep the mma.sync kernels
    for (int i = 0; i < kNumConvs; ++i) nd->conv_kernel[i] = 0;
    return fail(PBRT_ERROR_TIMEOUT, "neural autotune: a tcgen05 convolution timed out; using mma.sync");
  }
  nd->tuned = true;
  drop_graph(nd);
  return PBRT_OK;
}

PBRT_API int pbrt_neural_conv_kernels(const PbrtNeural* nd, int32_t* kinds, int32_t count) {
  if (!checked<const PbrtNeural>((void*)nd, Kind::Neural) || !kinds || count < kNumConvs)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "neural conv kernels: bad arguments");
  for (int i = 0; i < kNumConvs; ++i) kinds[i] = nd->conv_kernel[i];
  return PBRT_OK;
}

PBRT_API int pbrt_neural_set_conv_kernels(PbrtNeural* nd, const int32_t* kinds, int32_t count) {
  if (!checked<PbrtNeural>(nd, Kind::Neural) || !kinds || count != kNumConvs)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "neural set conv kernels: bad arguments");
  for (int i = 0; i < kNumConvs; ++i) {
    if (kinds[i] < 0 || kinds[i] > 2) return fail(PBRT_ERROR_INVALID_ARGUMENT, "neural set conv kernels: 0, 1 or 2");
    nd->conv_kernel[i] = kinds[i];
  }
  nd->tuned = true;
  drop_graph(nd);
  return PBRT_OK;
}

PBRT_API int pbrt_neural_dispatch(PbrtNeural* nd, pbrt_stream_t stream) {
  if (!checked<PbrtNeural>(nd, Kind::Neural)) return fail(PBRT_ERROR_INVALID_ARGUMENT, "neural dispatch: not a handle");
  if (!nd->tuned) {
    nd->tuned = true;  // once, whatever the outcome
    int st = pbrt_neural_autotune(nd, stream);
    if (st && st != PBRT_ERROR_TIMEOUT) return st;
  }
  if (!nd->graph) {
    cudaStream_t cap;
    PBRT_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    cudaGraph_t graph;
    cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    int st = e == cudaSuccess ? record_forward(nd, cap) : cuda_fail(e, "begin capture");
    cudaError_t e2 = cudaStreamEndCapture(cap, &graph);
    cudaStreamDestroy(cap);
    if (st) return st;
    if (e2 != cudaSuccess) return cuda_fail(e2, "end capture");
    e = cudaGraphInstantiate(&nd->graph, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(e, "graph instantiate");
  }
  PBRT_CUDA(cudaGraphLaunch(nd->graph, stream));
  return PBRT_OK;
}

PBRT_API int pbrt_neural_dispatch_direct(PbrtNeural* nd, pbrt_stream_t stream) {
  if (!checked<PbrtNeural>(nd, Kind::Neural)) return fail(PBRT_ERROR_INVALID_ARGUMENT, "neural dispatch: not a handle");
  return record_forward(nd, stream);
}

// FP8 calibration: one BF16 forward pass on the current inputs, the
// per-channel maximum |x| of every convolution's input, sx = amax / 448
// (e4m3's largest finite value), then the per-output-channel FP8 weights
// with sx folded in. Then the FP8 mode's per-layer choice: each
// convolution but the first (whose 16 input channels pad to 32 in e4m3, the
// BF16 instruction count) timed in BF16 on its chosen kernel and in FP8,
// each with the next level's pooling where the encoder needs it (fused in
// the epilogue or a separate launch), median of 3 after a warm-up on the
// activations of the BF16 pass; FP8 where it is faster.
PBRT_API int pbrt_neural_calibrate(PbrtNeural* nd, pbrt_stream_t stream) {
  if (!checked<PbrtNeural>(nd, Kind::Neural)) return fail(PBRT_ERROR_INVALID_ARGUMENT, "neural calibrate: not a handle");
  const int saved = nd->precision;
  nd->precision = 16;
  int st = record_forward(nd, stream);
  nd->precision = saved;
  if (st) return st;
  PBRT_CUDA(cudaMemsetAsync(nd->xscale, 0, nd->n_xscale * sizeof(float), stream));
  const size_t P = (size_t)nd->pw * nd->ph;
  const int skip_of[4] = {1, 3, 5, 7};
  for (int i = 0; i < kNumConvs && !st; ++i) {
    const ConvSpec& c = kConvs[i];
    const long px = (long)(P >> (2 * c.level));
    const bf16* in1;
    const bf16* in2 = nullptr;
    if (i == 0) in1 = nd->feat;
    else if (c.c2) {
      in1 = nd->act[skip_of[c.level]];
      in2 = nd->act[i - 1];
    } else if (i < 10 && c.name[2] == 'a') in1 = nd->pool[c.level];
    else in1 = nd->act[i - 1];
    st = pbrt_nn_channel_amax(in1, px, c.c1, nd->xscale + nd->xsoff[i], stream);
    if (!st && in2) st = pbrt_nn_channel_amax(in2, px / 4, c.c2, nd->xscale + nd->xsoff[i] + c.c1, stream);
  }
  if (st) return st;
  std::vector<float> amax(nd->n_xscale), sx(nd->n_xscale), inv(nd->n_xscale);
  PBRT_CUDA(cudaMemcpyAsync(amax.data(), nd->xscale, amax.size() * sizeof(float), cudaMemcpyDeviceToHost, stream));
  PBRT_CUDA(cudaStreamSynchronize(stream));
  for (size_t k = 0; k < amax.size(); ++k) {
    sx[k] = amax[k] > 0.f ? amax[k] / 448.f : 1.f;
    inv[k] = 1.f / sx[k];
  }
  PBRT_CUDA(cudaMemcpyAsync(nd->xscale, sx.data(), sx.size() * sizeof(float), cudaMemcpyHostToDevice, stream));
  PBRT_CUDA(cudaMemcpyAsync(nd->inv_xscale, inv.data(), inv.size() * sizeof(float), cudaMemcpyHostToDevice, stream));
  for (int i = 0; i < kNumConvs && !st; ++i)
    st = pbrt_nn_quantize_weights_fp8(nd->params + nd->lay.conv_w[i], nd->xscale + nd->xsoff[i], kConvs[i].cout,
                                      kConvs[i].c1 + kConvs[i].c2, nd->w8 + nd->lay.conv_w[i],
                                      nd->wscale + nd->wsoff[i], stream);
  if (st) return st;
  PBRT_CUDA(cudaStreamSynchronize(stream));
  nd->calibrated = true;
  if (!nd->tuned) {  // the BF16 kernels per layer first (as the first dispatch would)
    nd->tuned = true;
    st = pbrt_neural_autotune(nd, stream);
    if (st && st != PBRT_ERROR_TIMEOUT) return st;
    st = PBRT_OK;
  }
  cudaEvent_t e0, e1;
  PBRT_CUDA(cudaEventCreate(&e0));
  PBRT_CUDA(cudaEventCreate(&e1));
  nd->fp8_layer[0] = false;
  for (int i = 1; i < kNumConvs && !st; ++i) {
    const ConvSpec& c = kConvs[i];
    const int h = nd->ph >> c.level, w = nd->pw >> c.level;
    const bf16* x = (i < 10 && c.name[2] == 'a') ? nd->pool[c.level] : nd->act[i - 1];
    float best[2] = {1e30f, 1e30f};
    for (int k = 0; k < 2 && !st; ++k) {
      float ms[3];
      for (int r = 0; r < 4 && !st; ++r) {
        cudaEventRecord(e0, stream);
        bool pooled = false;
        st = conv_layer(nd, i, x, k == 1, stream, &pooled);
        if (!st && i < 8 && (i & 1) && !pooled)
          st = pbrt_nn_avgpool2(nd->act[i], nd->pool[c.level + 1], 0, 1, h, w, c.cout, stream);
        cudaEventRecord(e1, stream);
        cudaError_t e = cudaEventSynchronize(e1);
        if (!st && e != cudaSuccess) st = cuda_fail(e, "neural calibrate (timing)");
        if (r > 0) cudaEventElapsedTime(&ms[r - 1], e0, e1);
      }
      if (!st) {
        std::sort(ms, ms + 3);
        best[k] = ms[1];
      }
    }
    nd->fp8_layer[i] = best[1] < best[0];
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st) return st;
  uint32_t flags = 0;
  if ((st = pbrt_nn_umma_status(stream, &flags))) return st;
  if (flags) return fail(PBRT_ERROR_TIMEOUT, "neural calibrate: a tcgen05 convolution timed out");
  drop_graph(nd);
  return PBRT_OK;
}

// FP8 mode's per-layer precision: mask[i] = 1 where convolution i runs in
// e4m3 (set by the calibration's timing; the first convolution stays BF16).
PBRT_API int pbrt_neural_fp8_layers(const PbrtNeural* nd, int32_t* mask, int32_t count) {
  if (!checked<const PbrtNeural>((void*)nd, Kind::Neural) || !mask || count < kNumConvs)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "neural fp8 layers: bad arguments");
  for (int i = 0; i < kNumConvs; ++i) mask[i] = nd->fp8_layer[i] ? 1 : 0;
  return PBRT_OK;
}

PBRT_API int pbrt_neural_set_fp8_layers(PbrtNeural* nd, const int32_t* mask, int32_t count) {
  if (!checked<PbrtNeural>(nd, Kind::Neural) || !mask || count != kNumConvs)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "neural set fp8 layers: bad arguments");
  if (mask[0]) return fail(PBRT_ERROR_INVALID_ARGUMENT, "neural set fp8 layers: the first convolution stays BF16");
  for (int i = 0; i < kNumConvs; ++i) nd->fp8_layer[i] = mask[i] != 0;
  drop_graph(nd);
  return PBRT_OK;
}

PBRT_API int pbrt_neural_set_precision(PbrtNeural* nd, int32_t bits) {
  if (!checked<PbrtNeural>(nd, Kind::Neural) || (bits != 16 && bits != 8))
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "neural set precision: 16 (BF16) or 8 (FP8 e4m3)");
  if (bits == 8 && !nd->calibrated)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "neural set precision: FP8 needs pbrt_neural_calibrate first");
  if (nd->precision != bits) {
    nd->precision = bits;
    drop_graph(nd);
  }
  return PBRT_OK;
}

PBRT_API int pbrt_neural_final_image(const PbrtNeural* nd, PbrtImage* out) {
  if (!checked<const PbrtNeural>((void*)nd, Kind::Neural) || !out)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "neural final image: bad arguments");
  *out = nd->final_image.view;
  return PBRT_OK;
}

PBRT_API int pbrt_neural_images(const PbrtNeural* nd, PbrtImage* denoised, PbrtImage* variance) {
  if (!checked<const PbrtNeural>((void*)nd, Kind::Neural))
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "neural images: not a handle");
  if (denoised) *denoised = nd->denoised.view;
  if (variance) *variance = nd->variance.view;
  return PBRT_OK;
}

PBRT_API int pbrt_neural_fallback_mask(const PbrtNeural* nd, PbrtImage* mask) {
  if (!checked<const PbrtNeural>((void*)nd, Kind::Neural) || !mask)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "neural fallback mask: bad arguments");
  *mask = nd->mask.view;
  return PBRT_OK;
}

PBRT_API int pbrt_neural_fallback_tiles(const PbrtNeural* nd, pbrt_stream_t stream, uint32_t* count) {
  if (!checked<const PbrtNeural>((void*)nd, Kind::Neural) || !count)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "neural fallback tiles: bad arguments");
  PBRT_CUDA(cudaMemcpyAsync(count, nd->counter, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
  PBRT_CUDA(cudaStreamSynchronize(stream));
  if (!nd->fallback) *count = 0;
  return PBRT_OK;
}

}  // extern "C"
