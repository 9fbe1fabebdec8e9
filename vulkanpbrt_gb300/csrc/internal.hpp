// Internal object model behind the C ABI: reference-counted handles owning
// device images, and the status/error plumbing every entry point uses.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <cstdarg>
#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/vulkanpbrt_gb300.h"

namespace pbrt {

enum class Kind : uint32_t {
  GBuffer = 0x47425546,
  Illumination,
  Accumulation,
  Accumulator,
  BMFR,
  BFR,
  Scene,
  Pipeline,
  Neural,
  Taa,
  Batch,
  BfrBlender
};

struct Object {
  explicit Object(Kind k) : kind(k) {}
  virtual ~Object() = default;
  uint32_t magic = 0x50425254u;  // "PBRT"
  Kind kind;
  std::atomic<int> refs{1};
};

// Records msg as the calling thread's last error and returns status.
int fail(int status, const char* fmt, ...);
// Maps a CUDA error to PBRT_ERROR_CUDA / PBRT_ERROR_OUT_OF_MEMORY.
int cuda_fail(cudaError_t e, const char* what);
#define PBRT_CUDA(call)                                     \
  do {                                                      \
    cudaError_t _e = (call);                                \
    if (_e != cudaSuccess) return ::pbrt::cuda_fail(_e, #call); \
  } while (0)
// Checks the launch just issued on this thread.
int check_launch(const char* what);
// Whether the FP8 tcgen05 convolution (pbrt_nn_conv3x3_fp8_umma) takes
// these operands: shared memory for the weights and two input stages,
// 16-byte alignment, and (pooled) a frame of whole 16 x 8 tiles.
bool nn_fp8_umma_fits(const void* x1, int c1, const void* x2, int c2, const void* w8, int cout, int h, int w,
                      bool pooled);
// Whether pbrt_nn_conv3x3_umma_pooled takes this layer (whole 16 x 8 tiles,
// the weights and two input stages in shared memory).
bool nn_umma_pooled_fits(int c1, int cout, int h, int w);

// One-time setup per device (kernel attributes such as the dynamic
// shared-memory opt-in are recorded per device, not per process):
// once_per_device(flag, f) runs f() with the caller's current device the
// first time it is called on that device, and again after a failed f().
// Thread-safe.
constexpr int kMaxDevices = 64;
struct PerDeviceOnce {
  std::mutex m;
  bool done[kMaxDevices] = {};
};
template <class F> int once_per_device(PerDeviceOnce& o, F&& f) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return fail(PBRT_ERROR_UNSUPPORTED, "device ordinal %d beyond %d", dev, kMaxDevices);
  std::lock_guard<std::mutex> lock(o.m);
  if (o.done[dev]) return PBRT_OK;
  int st = f();
  if (st == PBRT_OK) o.done[dev] = true;
  return st;
}

void retain(Object* o);
void release(Object* o);
template <class T> T* checked(void* h, Kind k) {
  Object* o = static_cast<Object*>(h);
  if (!o || o->magic != 0x50425254u || o->kind != k) return nullptr;
  return static_cast<T*>(o);
}

// A device image the library owns (zero-initialised at creation).
struct DeviceImage {
  PbrtImage view{};
  int alloc(uint32_t w, uint32_t h, uint32_t layers, PbrtFormat fmt);
  void free_();
  template <class T> T* ptr() const { return static_cast<T*>(view.data); }
  size_t bytes() const { return view.layer_bytes * view.layers; }
};
uint32_t texel_bytes(PbrtFormat f);

}  // namespace pbrt

struct PbrtGBuffer : pbrt::Object {
  PbrtGBuffer() : Object(pbrt::Kind::GBuffer) {}
  ~PbrtGBuffer() override;
  uint32_t width = 0, height = 0;
  pbrt::DeviceImage depth, normal, material, albedo;
};

struct PbrtIlluminationBuffer : pbrt::Object {
  PbrtIlluminationBuffer() : Object(pbrt::Kind::Illumination) {}
  ~PbrtIlluminationBuffer() override;
  int32_t type = 0;
  uint32_t width = 0, height = 0;
  std::vector<pbrt::DeviceImage> images;
  // The demodulated illumination image the accumulator / denoisers read:
  // image 1 of FinalDemodulated, else image 0.
  const pbrt::DeviceImage& demodulated() const {
    return type == PBRT_ILLUMINATION_FINAL_DEMODULATED ? images[1] : images[0];
  }
};

struct PbrtAccumulationBuffer : pbrt::Object {
  PbrtAccumulationBuffer() : Object(pbrt::Kind::Accumulation) {}
  ~PbrtAccumulationBuffer() override;
  uint32_t width = 0, height = 0;
  pbrt::DeviceImage prev_illu, prev_illu_squared, prev_depth, prev_normal, spp, prev_spp, motion;
};

namespace pbrt {
// Push constants of accumulator.comp (shaders/accumulator.comp:20-27) plus
// the host-side inverse of `view` the SEPARATE_MATRICES variant needs.
struct AccumulatorParams {
  float view[16], inverse_view[16], prev_view[16], prev_origin[4];
  float proj[16];  // inverse(view), evaluated once on the host
  uint32_t frame_number;
};
}  // namespace pbrt

struct PbrtAccumulator : pbrt::Object {
  PbrtAccumulator() : Object(pbrt::Kind::Accumulator) {}
  ~PbrtAccumulator() override;
  PbrtGBuffer* gbuffer = nullptr;
  PbrtIlluminationBuffer* source = nullptr;
  PbrtIlluminationBuffer* accumulated = nullptr;
  PbrtAccumulationBuffer* acc = nullptr;
  bool separate = true;
  int32_t work_w = 16, work_h = 16;
  pbrt::AccumulatorParams params{};
};

struct PbrtBMFR : pbrt::Object {
  PbrtBMFR() : Object(pbrt::Kind::BMFR) {}
  ~PbrtBMFR() override;
  uint32_t width = 0, height = 0, bw = 32, fitting_kernel = 256;
  int32_t position_type = 0, fp64_resolve = 0;
  float cond_limit = 1e6f;  // FP64 re-solve above this R-diagonal ratio
  PbrtGBuffer* gbuffer = nullptr;
  PbrtIlluminationBuffer* illumination = nullptr;
  PbrtAccumulationBuffer* acc = nullptr;
  pbrt::DeviceImage denoised, final_image, weights;
  pbrt::DeviceImage flags;  // per block: condition estimate exceeded (FP64 re-solve list)
  uint32_t* counter = nullptr;  // device: [0] = number of flagged blocks, [1] = largest ratio (float bits)
  uint32_t* last_layer = nullptr;  // device: the denoised layer the last dispatch wrote (0 or 1)
};

struct PbrtBFR : pbrt::Object {
  PbrtBFR() : Object(pbrt::Kind::BFR) {}
  ~PbrtBFR() override;
  uint32_t width = 0, height = 0, bw = 16, bh = 16;
  PbrtGBuffer* gbuffer = nullptr;
  PbrtIlluminationBuffer* illumination = nullptr;
  PbrtAccumulationBuffer* acc = nullptr;
  pbrt::DeviceImage denoised, final_image;
};
