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

#include <cstring>
#include <new>

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
  PbrtBMFR* fallback = nullptr;
  float threshold = 0.f;
  int32_t tile = 32;
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
};

namespace {

template <class T> int dalloc(T** p, size_t count) {
  *p = nullptr;
  cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc (neural)");
  return PBRT_OK;
}

int record_forward(PbrtNeural* nd, cudaStream_t s) {
  const int n = 1, PH = nd->ph, PW = nd->pw;
  const PbrtIlluminationBuffer* ib = nd->illumination;
  const DeviceImage& illum = ib->demodulated();
  const int is_half = illum.view.format == PBRT_FORMAT_R16G16B16A16_SFLOAT;
  int st;
  if ((st = pbrt_nn_features(illum.view.data, is_half, nd->gbuffer->albedo.view.data, nd->gbuffer->normal.view.data,
                             nd->gbuffer->depth.view.data, nd->width, nd->height, PW, PH, n, nd->feat, nd->rad[0], s)))
    return st;
  if ((st = pbrt_nn_avgpool2(nd->rad[0], nd->rad[1], 1, n, PH, PW, 3, s))) return st;
  if ((st = pbrt_nn_avgpool2(nd->rad[1], nd->rad[2], 1, n, PH / 2, PW / 2, 3, s))) return st;
  const bf16* x = nd->feat;
  const int skip_of[4] = {1, 3, 5, 7};  // e0b, e1b, e2b, e3b
  for (int i = 0; i < kNumConvs; ++i) {
    const ConvSpec& c = kConvs[i];
    const int h = PH >> c.level, w = PW >> c.level;
    const bf16* w16 = nd->w16 + nd->lay.conv_w[i];
    const float* b = nd->params + nd->lay.conv_b[i];
    if (i < 10 && c.name[2] == 'a' && c.level > 0) {  // encoder: pool the previous level's output first
      if ((st = pbrt_nn_avgpool2(x, nd->pool[c.level], 0, n, h * 2, w * 2, kConvs[i - 1].cout, s))) return st;
      x = nd->pool[c.level];
    }
    if (c.c2) {
      st = pbrt_nn_conv3x3(nd->act[skip_of[c.level]], c.c1, x, c.c2, w16, b, nd->act[i], nullptr, n, h, w, c.cout, 1, s);
    } else {
      st = pbrt_nn_conv3x3(x, c.c1, nullptr, 0, w16, b, nd->act[i], nullptr, n, h, w, c.cout, 1, s);
    }
    if (st) return st;
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
  const bool gate = nd->fallback != nullptr;
  if (gate) {
    PBRT_CUDA(cudaMemsetAsync(nd->counter, 0, sizeof(uint32_t), s));
    if ((st = pbrt_nn_gate(nd->variance.ptr<float>(), PW, nd->width, nd->height, nd->threshold, nd->tile,
                           nd->mask.ptr<uint8_t>(), nd->counter, s)))
      return st;
  }
  return pbrt_nn_compose(nd->out[0], PW, nd->width, nd->height, nd->gbuffer->albedo.view.data,
                         gate ? nd->mask.ptr<uint8_t>() : nullptr, nd->tile,
                         gate ? nd->fallback->final_image.view.data : nullptr, nd->final_image.view.data,
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
  variance.free_();
  denoised.free_();
  final_image.free_();
  mask.free_();
  release(gbuffer);
  release(illumination);
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
  to_bf16_kernel<<<256, 256>>>(nd->params, nd->w16, nd->lay.conv_w_total);
  int st = check_launch("to_bf16_kernel");
  if (st) return st;
  PBRT_CUDA(cudaDeviceSynchronize());
  return PBRT_OK;
}

PBRT_API int pbrt_neural_create(uint32_t width, uint32_t height, PbrtGBuffer* g, PbrtIlluminationBuffer* illu,
                                const float* params_host, int64_t count, PbrtNeural** out) {
  if (!out || !checked<PbrtGBuffer>(g, Kind::GBuffer) || !checked<PbrtIlluminationBuffer>(illu, Kind::Illumination))
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "neural create: bad arguments");
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
  nd->gbuffer = g;
  nd->illumination = illu;
  const size_t P = (size_t)nd->pw * nd->ph;
  int st;
  if ((st = dalloc(&nd->params, nd->lay.total)) || (st = dalloc(&nd->w16, nd->lay.conv_w_total)) ||
      (st = dalloc(&nd->feat, P * 16)) || (st = dalloc(&nd->counter, 1))) {
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

PBRT_API int pbrt_neural_dispatch(PbrtNeural* nd, pbrt_stream_t stream) {
  if (!checked<PbrtNeural>(nd, Kind::Neural)) return fail(PBRT_ERROR_INVALID_ARGUMENT, "neural dispatch: not a handle");
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
