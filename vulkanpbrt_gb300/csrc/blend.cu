// BFRBlender (shaders/bfrBlender.comp:31-68, source/renderModules/denoisers/
// BFRBlender.cpp): the multi-scale combination of three denoiser outputs
// (block sizes 8, 16 and 32) used by DenoisingBlockSize::X8X16X32
// (source/util/DenoiserUtils.cpp:48-69, 103-124).
//
// Per pixel: the luminance (mean of r, g, b) of the average image over a
// (2r+1)^2 window gives a running mean and mean square, each blended 1:1
// with the pixel's own average and average-square luminance; their standard
// deviation picks the blend: 0 -> the 32x32 result, 0.5 -> the 16x16 result,
// >= 1 -> the 8x8 result, piecewise linear in between. Out-of-image window
// taps read zero (and still count), as a robust-access imageLoad does. A
// negative variance (rounding) gives a NaN deviation, which min(t, 1)
// resolves to 1 -- the hardware min returns the non-NaN operand -- so such
// pixels take the 8x8 result, as the shader does on the GPU it was written
// for. The denoised and final images are 8-bit with four channels, blended
// byte for byte (the shader's rgba8 view of B8G8R8A8 data swaps r and b on
// load and on store alike); alpha is stored as 255.
//
// Arithmetic is the shader's, unfused (this file is built with -fmad=false),
// so results match the oracle bit for bit.
#include "device_common.cuh"
#include "internal.hpp"

namespace pbrt {

struct BlendArgs {
  int W, H, R;
  PbrtImage avg, avg_sq;  // RGBA16F or RGBA32F
  const uchar4* den8;     // denoised0 (block 8)
  const uchar4* den16;    // denoised1 (block 16)
  const uchar4* den32;    // denoised2 (block 32)
  uchar4* out;            // B8G8R8A8
};

PBRT_D float3 load_rgb(const PbrtImage& im, int x, int y) {
  const char* row = (const char*)im.data + (size_t)y * im.row_bytes;
  if (im.format == PBRT_FORMAT_R16G16B16A16_SFLOAT) {
    const float4 v = load_half4((const Half4*)row + x);
    return f3(v.x, v.y, v.z);
  }
  const float4 v = ((const float4*)row)[x];
  return f3(v.x, v.y, v.z);
}

PBRT_D float lum3(float3 c) {  // dot(c, vec3(1.0 / 3.0))
  const float k = 1.0f / 3.0f;
  return (c.x * k + c.y * k) + c.z * k;
}

// mix3 of bfrBlender.comp:22-29 with mid 0.5 and maxDev 1.
PBRT_D float mix3(float a, float b, float c, float t) {
  const float mid = .5f, max_dev = 1.f;
  t = t / max_dev;
  t = fminf(t, 1.f);
  const float af = fmaxf(1.0f - (t / mid), 0.f);
  const float bf = (t < mid) ? t / mid : 1.f - (t - mid) / (1.0f - mid);
  const float cf = (1.0f - af) - bf;
  return (af * a + bf * b) + cf * c;
}

__global__ void bfr_blend_kernel(BlendArgs a) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= a.W || y >= a.H) return;
  float sq = 0.f, av = 0.f;
  int count = 0;
  for (int dy = -a.R; dy <= a.R; ++dy)
    for (int dx = -a.R; dx <= a.R; ++dx) {
      const int sx = x + dx, sy = y + dy;
      const bool in = sx >= 0 && sy >= 0 && sx < a.W && sy < a.H;
      const float cur = in ? lum3(load_rgb(a.avg, sx, sy)) : 0.f;
      ++count;
      const float w = 1.0f / (float)count;
      sq = mixf(sq, cur * cur, w);
      av = mixf(av, cur, w);
    }
  av = mixf(av, lum3(load_rgb(a.avg, x, y)), .5f);
  sq = mixf(sq, lum3(load_rgb(a.avg_sq, x, y)), .5f);
  const float sd = sqrtf(sq - av * av);
  const size_t p = (size_t)y * a.W + x;
  const uchar4 d2 = a.den8[p], d1 = a.den16[p], d0 = a.den32[p];
  const float c0 = mix3(u82f(d0.x), u82f(d1.x), u82f(d2.x), sd);
  const float c1 = mix3(u82f(d0.y), u82f(d1.y), u82f(d2.y), sd);
  const float c2 = mix3(u82f(d0.z), u82f(d1.z), u82f(d2.z), sd);
  a.out[p] = make_uchar4(f2u8(c0), f2u8(c1), f2u8(c2), 255);
}

}  // namespace pbrt

using namespace pbrt;

struct PbrtBFRBlender : pbrt::Object {
  PbrtBFRBlender() : Object(pbrt::Kind::BfrBlender) {}
  ~PbrtBFRBlender() override { final_image.free_(); }
  uint32_t width = 0, height = 0, work_w = 16, work_h = 16, radius = 2;
  PbrtImage avg{}, avg_sq{}, den[3]{};
  pbrt::DeviceImage final_image;
};

namespace {
bool float4_image(const PbrtImage* im, uint32_t w, uint32_t h) {
  return im && im->data && im->width == w && im->height == h &&
         (im->format == PBRT_FORMAT_R16G16B16A16_SFLOAT || im->format == PBRT_FORMAT_R32G32B32A32_SFLOAT) &&
         im->row_bytes >= (size_t)w * im->texel_bytes && im->row_bytes % 8 == 0;
}
bool packed_u8x4(const PbrtImage* im, uint32_t w, uint32_t h) {
  return im && im->data && im->width == w && im->height == h &&
         (im->format == PBRT_FORMAT_B8G8R8A8_UNORM || im->format == PBRT_FORMAT_R8G8B8A8_UNORM) &&
         im->row_bytes == (size_t)w * 4;
}
}  // namespace

extern "C" {

PBRT_API int pbrt_bfr_blender_create(uint32_t width, uint32_t height, const PbrtImage* average_image,
                                     const PbrtImage* average_squared_image, const PbrtImage* denoised0,
                                     const PbrtImage* denoised1, const PbrtImage* denoised2, uint32_t work_width,
                                     uint32_t work_height, uint32_t filter_radius, PbrtBFRBlender** out) {
  if (!out || width == 0 || height == 0 || work_width == 0 || work_height == 0 || work_width * work_height > 1024 ||
      filter_radius > 32)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "bfr blender create: bad arguments");
  *out = nullptr;
  if (!float4_image(average_image, width, height) || !float4_image(average_squared_image, width, height))
    return fail(PBRT_ERROR_INVALID_ARGUMENT,
                "bfr blender create: the average images must be %ux%u RGBA16F or RGBA32F images", width, height);
  if (!packed_u8x4(denoised0, width, height) || !packed_u8x4(denoised1, width, height) ||
      !packed_u8x4(denoised2, width, height))
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "bfr blender create: the denoised images must be packed %ux%u 8-bit RGBA",
                width, height);
  auto* b = new (std::nothrow) PbrtBFRBlender();
  if (!b) return fail(PBRT_ERROR_OUT_OF_MEMORY, "bfr blender: host allocation");
  b->width = width;
  b->height = height;
  b->work_w = work_width;
  b->work_h = work_height;
  b->radius = filter_radius;
  b->avg = *average_image;
  b->avg_sq = *average_squared_image;
  b->den[0] = *denoised0;
  b->den[1] = *denoised1;
  b->den[2] = *denoised2;
  if (int st = b->final_image.alloc(width, height, 1, PBRT_FORMAT_B8G8R8A8_UNORM)) {
    delete b;
    return st;
  }
  *out = b;
  return PBRT_OK;
}

PBRT_API int pbrt_bfr_blender_dispatch(PbrtBFRBlender* b, pbrt_stream_t stream) {
  if (!checked<PbrtBFRBlender>(b, Kind::BfrBlender)) return fail(PBRT_ERROR_INVALID_ARGUMENT, "bfr blender dispatch");
  BlendArgs a;
  a.W = (int)b->width;
  a.H = (int)b->height;
  a.R = (int)b->radius;
  a.avg = b->avg;
  a.avg_sq = b->avg_sq;
  a.den8 = (const uchar4*)b->den[0].data;
  a.den16 = (const uchar4*)b->den[1].data;
  a.den32 = (const uchar4*)b->den[2].data;
  a.out = b->final_image.ptr<uchar4>();
  dim3 block(b->work_w, b->work_h), grid((b->width + b->work_w - 1) / b->work_w, (b->height + b->work_h - 1) / b->work_h);
  bfr_blend_kernel<<<grid, block, 0, stream>>>(a);
  return check_launch("bfr_blend_kernel");
}

PBRT_API int pbrt_bfr_blender_final_image(const PbrtBFRBlender* b, PbrtImage* out) {
  if (!checked<const PbrtBFRBlender>((void*)b, Kind::BfrBlender) || !out)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "bfr blender final image");
  *out = b->final_image.view;
  return PBRT_OK;
}

}  // extern "C"
