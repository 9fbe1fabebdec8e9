// C ABI plumbing and the image-holding objects: GBuffer, the
// IlluminationBuffer family and AccumulationBuffer
// (source/buffers/{GBuffer,IlluminationBuffer,AccumulationBuffer}.cpp).
#include <cstdio>
#include <cstring>
#include <new>

#include "internal.hpp"

namespace pbrt {

static thread_local std::string g_last_error;

int fail(int status, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return status;
}

int cuda_fail(cudaError_t e, const char* what) {
  // a failed call leaves its error as the runtime's last error; take it off
  // so that the next launch check reports its own (a sticky error stays)
  cudaGetLastError();
  int st = (e == cudaErrorMemoryAllocation) ? PBRT_ERROR_OUT_OF_MEMORY : PBRT_ERROR_CUDA;
  return fail(st, "%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
}

int check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, what);
  return PBRT_OK;
}

void retain(Object* o) { o->refs.fetch_add(1); }
void release(Object* o) {
  if (o && o->refs.fetch_sub(1) == 1) delete o;
}

uint32_t texel_bytes(PbrtFormat f) {
  switch (f) {
    case PBRT_FORMAT_R32_SFLOAT: return 4;
    case PBRT_FORMAT_R32G32_SFLOAT: return 8;
    case PBRT_FORMAT_R32G32B32A32_SFLOAT: return 16;
    case PBRT_FORMAT_R16_SFLOAT: return 2;
    case PBRT_FORMAT_R16G16_SFLOAT: return 4;
    case PBRT_FORMAT_R16G16B16A16_SFLOAT: return 8;
    case PBRT_FORMAT_R8_UNORM: return 1;
    case PBRT_FORMAT_R8G8B8A8_UNORM: return 4;
    case PBRT_FORMAT_B8G8R8A8_UNORM: return 4;
  }
  return 0;
}

int DeviceImage::alloc(uint32_t w, uint32_t h, uint32_t layers, PbrtFormat fmt) {
  view.width = w;
  view.height = h;
  view.layers = layers;
  view.format = fmt;
  view.texel_bytes = texel_bytes(fmt);
  view.row_bytes = (size_t)w * view.texel_bytes;
  view.layer_bytes = view.row_bytes * h;
  size_t n = view.layer_bytes * layers;
  if (n == 0) return fail(PBRT_ERROR_INVALID_ARGUMENT, "empty image %ux%ux%u", w, h, layers);
  void* p = nullptr;
  PBRT_CUDA(cudaMalloc(&p, n));
  cudaError_t e = cudaMemset(p, 0, n);
  if (e != cudaSuccess) {
    cudaFree(p);
    return cuda_fail(e, "cudaMemset(image)");
  }
  view.data = p;
  return PBRT_OK;
}

void DeviceImage::free_() {
  if (view.data) cudaFree(view.data);
  view.data = nullptr;
}

}  // namespace pbrt

using namespace pbrt;

PbrtGBuffer::~PbrtGBuffer() {
  depth.free_();
  normal.free_();
  material.free_();
  albedo.free_();
}
PbrtIlluminationBuffer::~PbrtIlluminationBuffer() {
  for (auto& i : images) i.free_();
}
PbrtAccumulationBuffer::~PbrtAccumulationBuffer() {
  for (DeviceImage* i : {&prev_illu, &prev_illu_squared, &prev_depth, &prev_normal, &spp, &prev_spp, &motion})
    i->free_();
}

extern "C" {

PBRT_API const char* pbrt_version(void) { return "vulkanpbrt_gb300 0.1 (sm_103a)"; }

PBRT_API int pbrt_last_error(char* buffer, size_t size) {
  if (!buffer || size == 0) return PBRT_ERROR_INVALID_ARGUMENT;
  snprintf(buffer, size, "%s", g_last_error.c_str());
  return PBRT_OK;
}

PBRT_API int pbrt_retain(void* handle) {
  Object* o = static_cast<Object*>(handle);
  if (!o || o->magic != 0x50425254u) return fail(PBRT_ERROR_INVALID_ARGUMENT, "pbrt_retain: not a handle");
  retain(o);
  return PBRT_OK;
}

PBRT_API int pbrt_release(void* handle) {
  Object* o = static_cast<Object*>(handle);
  if (!o) return PBRT_OK;
  if (o->magic != 0x50425254u) return fail(PBRT_ERROR_INVALID_ARGUMENT, "pbrt_release: not a handle");
  release(o);
  return PBRT_OK;
}

PBRT_API int pbrt_image_upload(const PbrtImage* dst, const void* host, size_t host_row_bytes, pbrt_stream_t stream) {
  if (!dst || !dst->data || !host || host_row_bytes < (size_t)dst->width * dst->texel_bytes)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "image upload: bad arguments");
  const size_t rows = (size_t)dst->height * (dst->layers ? dst->layers : 1);
  cudaError_t e = cudaMemcpy2DAsync(dst->data, dst->row_bytes, host, host_row_bytes,
                                    (size_t)dst->width * dst->texel_bytes, rows, cudaMemcpyHostToDevice,
                                    (cudaStream_t)stream);
  return e == cudaSuccess ? PBRT_OK : cuda_fail(e, "image upload");
}

PBRT_API int pbrt_image_download(const PbrtImage* src, void* host, size_t host_row_bytes, pbrt_stream_t stream) {
  if (!src || !src->data || !host || host_row_bytes < (size_t)src->width * src->texel_bytes)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "image download: bad arguments");
  const size_t rows = (size_t)src->height * (src->layers ? src->layers : 1);
  cudaError_t e = cudaMemcpy2DAsync(host, host_row_bytes, src->data, src->row_bytes,
                                    (size_t)src->width * src->texel_bytes, rows, cudaMemcpyDeviceToHost,
                                    (cudaStream_t)stream);
  return e == cudaSuccess ? PBRT_OK : cuda_fail(e, "image download");
}

PBRT_API int pbrt_stream_synchronize(pbrt_stream_t stream) {
  cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
  return e == cudaSuccess ? PBRT_OK : cuda_fail(e, "stream synchronize");
}

PBRT_API int pbrt_gbuffer_create(uint32_t width, uint32_t height, PbrtGBuffer** out) {
  if (!out || width == 0 || height == 0) return fail(PBRT_ERROR_INVALID_ARGUMENT, "gbuffer: bad size or output");
  *out = nullptr;
  auto* g = new (std::nothrow) PbrtGBuffer();
  if (!g) return fail(PBRT_ERROR_OUT_OF_MEMORY, "gbuffer: host allocation");
  g->width = width;
  g->height = height;
  int st;
  if ((st = g->depth.alloc(width, height, 1, PBRT_FORMAT_R32_SFLOAT)) ||
      (st = g->normal.alloc(width, height, 1, PBRT_FORMAT_R32G32_SFLOAT)) ||
      (st = g->material.alloc(width, height, 1, PBRT_FORMAT_R8G8B8A8_UNORM)) ||
      (st = g->albedo.alloc(width, height, 1, PBRT_FORMAT_R8G8B8A8_UNORM))) {
    delete g;
    return st;
  }
  *out = g;
  return PBRT_OK;
}

PBRT_API int pbrt_gbuffer_images(const PbrtGBuffer* g, PbrtImage* depth, PbrtImage* normal, PbrtImage* material,
                                 PbrtImage* albedo) {
  if (!checked<const PbrtGBuffer>((void*)g, Kind::GBuffer)) return fail(PBRT_ERROR_INVALID_ARGUMENT, "not a GBuffer");
  if (depth) *depth = g->depth.view;
  if (normal) *normal = g->normal.view;
  if (material) *material = g->material.view;
  if (albedo) *albedo = g->albedo.view;
  return PBRT_OK;
}

PBRT_API int pbrt_illumination_buffer_create(int32_t type, uint32_t width, uint32_t height,
                                             PbrtIlluminationBuffer** out) {
  if (!out || width == 0 || height == 0) return fail(PBRT_ERROR_INVALID_ARGUMENT, "illumination: bad size or output");
  *out = nullptr;
  std::vector<PbrtFormat> fmts;
  switch (type) {
    case PBRT_ILLUMINATION_FINAL: fmts = {PBRT_FORMAT_B8G8R8A8_UNORM}; break;
    case PBRT_ILLUMINATION_FINAL_DEMODULATED:
      fmts = {PBRT_FORMAT_B8G8R8A8_UNORM, PBRT_FORMAT_R16G16B16A16_SFLOAT, PBRT_FORMAT_R16G16B16A16_SFLOAT};
      break;
    case PBRT_ILLUMINATION_DEMODULATED:
      fmts = {PBRT_FORMAT_R16G16B16A16_SFLOAT, PBRT_FORMAT_R16G16B16A16_SFLOAT};
      break;
    case PBRT_ILLUMINATION_DEMODULATED_FLOAT: fmts = {PBRT_FORMAT_R32G32B32A32_SFLOAT}; break;
    case PBRT_ILLUMINATION_FINAL_FLOAT: fmts = {PBRT_FORMAT_R32G32B32A32_SFLOAT}; break;
    default: return fail(PBRT_ERROR_INVALID_ARGUMENT, "illumination: unknown type %d", type);
  }
  auto* b = new (std::nothrow) PbrtIlluminationBuffer();
  if (!b) return fail(PBRT_ERROR_OUT_OF_MEMORY, "illumination: host allocation");
  b->type = type;
  b->width = width;
  b->height = height;
  b->images.resize(fmts.size());
  for (size_t i = 0; i < fmts.size(); ++i) {
    int st = b->images[i].alloc(width, height, 1, fmts[i]);
    if (st) {
      delete b;
      return st;
    }
  }
  *out = b;
  return PBRT_OK;
}

PBRT_API int pbrt_illumination_buffer_images(const PbrtIlluminationBuffer* b, PbrtImage* images, uint32_t capacity,
                                             uint32_t* count) {
  if (!checked<const PbrtIlluminationBuffer>((void*)b, Kind::Illumination))
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "not an IlluminationBuffer");
  if (count) *count = (uint32_t)b->images.size();
  for (uint32_t i = 0; i < capacity && i < b->images.size(); ++i) images[i] = b->images[i].view;
  return PBRT_OK;
}

PBRT_API int pbrt_accumulation_buffer_create(uint32_t width, uint32_t height, PbrtAccumulationBuffer** out) {
  if (!out || width == 0 || height == 0) return fail(PBRT_ERROR_INVALID_ARGUMENT, "accumulation: bad size or output");
  *out = nullptr;
  auto* a = new (std::nothrow) PbrtAccumulationBuffer();
  if (!a) return fail(PBRT_ERROR_OUT_OF_MEMORY, "accumulation: host allocation");
  a->width = width;
  a->height = height;
  int st;
  if ((st = a->spp.alloc(width, height, 1, PBRT_FORMAT_R8_UNORM)) ||
      (st = a->prev_spp.alloc(width, height, 1, PBRT_FORMAT_R8_UNORM)) ||
      (st = a->prev_depth.alloc(width, height, 1, PBRT_FORMAT_R32_SFLOAT)) ||
      (st = a->prev_normal.alloc(width, height, 1, PBRT_FORMAT_R32G32_SFLOAT)) ||
      (st = a->motion.alloc(width, height, 1, PBRT_FORMAT_R16G16_SFLOAT)) ||
      (st = a->prev_illu.alloc(width, height, 1, PBRT_FORMAT_R16G16B16A16_SFLOAT)) ||
      (st = a->prev_illu_squared.alloc(width, height, 1, PBRT_FORMAT_R16G16B16A16_SFLOAT))) {
    delete a;
    return st;
  }
  *out = a;
  return PBRT_OK;
}

PBRT_API int pbrt_accumulation_buffer_images(const PbrtAccumulationBuffer* a, PbrtAccumulationImages* out) {
  if (!checked<const PbrtAccumulationBuffer>((void*)a, Kind::Accumulation) || !out)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "not an AccumulationBuffer");
  out->prev_illu = a->prev_illu.view;
  out->prev_illu_squared = a->prev_illu_squared.view;
  out->prev_depth = a->prev_depth.view;
  out->prev_normal = a->prev_normal.view;
  out->spp = a->spp.view;
  out->prev_spp = a->prev_spp.view;
  out->motion = a->motion.view;
  return PBRT_OK;
}

PBRT_API int pbrt_accumulation_buffer_copy_to_back_images(PbrtAccumulationBuffer* a, const PbrtGBuffer* g,
                                                          const PbrtIlluminationBuffer* illumination,
                                                          pbrt_stream_t stream) {
  if (!checked<PbrtAccumulationBuffer>(a, Kind::Accumulation) || !checked<const PbrtGBuffer>((void*)g, Kind::GBuffer) ||
      !checked<const PbrtIlluminationBuffer>((void*)illumination, Kind::Illumination))
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "copy_to_back_images: bad handle");
  if (g->width != a->width || g->height != a->height || illumination->width != a->width ||
      illumination->height != a->height)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "copy_to_back_images: size mismatch");
  const DeviceImage& src = illumination->demodulated();
  if (illumination->type != PBRT_ILLUMINATION_DEMODULATED && illumination->type != PBRT_ILLUMINATION_FINAL_DEMODULATED)
    return fail(PBRT_ERROR_UNSUPPORTED,
                "AccumulationBuffer::copy_to_back_images: illumination buffer not supported "
                "(needs Demodulated or FinalDemodulated)");
  PBRT_CUDA(cudaMemcpyAsync(a->prev_depth.view.data, g->depth.view.data, a->prev_depth.bytes(),
                            cudaMemcpyDeviceToDevice, stream));
  PBRT_CUDA(cudaMemcpyAsync(a->prev_normal.view.data, g->normal.view.data, a->prev_normal.bytes(),
                            cudaMemcpyDeviceToDevice, stream));
  PBRT_CUDA(cudaMemcpyAsync(a->prev_spp.view.data, a->spp.view.data, a->prev_spp.bytes(), cudaMemcpyDeviceToDevice,
                            stream));
  PBRT_CUDA(cudaMemcpyAsync(a->prev_illu.view.data, src.view.data, a->prev_illu.bytes(), cudaMemcpyDeviceToDevice,
                            stream));
  return PBRT_OK;
}

}  // extern "C"
