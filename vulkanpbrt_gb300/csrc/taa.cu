// Temporal anti-aliasing (shaders/taa.comp:48-103, source/renderModules/Taa.cpp)
// and the format converter (shaders/formatConverter.comp:9-13,
// source/renderModules/FormatConverter.cpp): the two passes that follow the
// denoiser in the reference's frame (source/VulkanPBRT.cpp:448-484).
//
// TAA reads the denoiser's B8G8R8A8 final image (texelFetch returns it as
// rgb), clamps the history against the YCoCg min/max of the 3x3
// neighbourhood (average of the box and the cross), blends 0.4 current +
// 0.6 history when the history lies inside, and stores B8G8R8A8. The history
// is the previous final image copied byte for byte into an R8G8B8A8 image
// (Taa.cpp:121-159, vkCmdCopyImage between the two formats), so the
// bilinear history sample returns the previous frame's (b, g, r): that swap
// is the reference's behaviour and is kept. Here the copy is the kernel's
// second output into the other half of a ping-pong pair, which leaves the
// history it samples untouched while it runs.
#include "device_common.cuh"
#include "internal.hpp"

namespace pbrt {

PBRT_D float3 rgb_to_ycocg(float3 c) {
  return f3(c.x * 1.f + c.y * 2.f + c.z * 1.f, c.x * 2.f + c.y * 0.f + c.z * -2.f, c.x * -1.f + c.y * 2.f + c.z * -1.f);
}

struct TaaArgs {
  int W, H;
  uint32_t frame;
  const __half2* motion;       // RG16F
  const uchar4* denoised;      // B8G8R8A8
  const uchar4* history;       // bytes of the previous final image, read as R8G8B8A8
  uchar4* final_bgra;          // B8G8R8A8
  uchar4* history_next;        // copy of final_bgra
};

PBRT_D float3 fetch_bgra(const uchar4* im, size_t p) {
  const uchar4 b = im[p];
  return f3(u82f(b.z), u82f(b.y), u82f(b.x));  // texelFetch of a B8G8R8A8 image: (r, g, b)
}

__global__ void taa_kernel(TaaArgs a) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= a.W || y >= a.H) return;
  const size_t p = (size_t)y * a.W + x;
  const float3 cur = fetch_bgra(a.denoised, p);
  const float2 uv = __half22float2(a.motion[p]);
  float3 res = cur;
  if (!(a.frame == 0 || uv.x < 0.f || uv.y < 0.f || uv.x > 1.f || uv.y > 1.f)) {
    const float inf = __int_as_float(0x7f800000);
    float3 mn_box = f3(inf), mn_cross = f3(inf), mx_box = f3(-inf), mx_cross = f3(-inf);
    for (int dy = -1; dy <= 1; ++dy)
      for (int dx = -1; dx <= 1; ++dx) {
        const int sx = x + dx, sy = y + dy;
        if (sx < 0 || sy < 0 || sx >= a.W || sy >= a.H) continue;
        const float3 c = rgb_to_ycocg((dx == 0 && dy == 0) ? cur : fetch_bgra(a.denoised, (size_t)sy * a.W + sx));
        if (dx == 0 || dy == 0) {
          mn_cross = fmin3(mn_cross, c);
          mx_cross = fmax3(mx_cross, c);
        }
        mn_box = fmin3(mn_box, c);
        mx_box = fmax3(mx_box, c);
      }
    const float4 h = bilinear(a.W, a.H, uv.x, uv.y, [&](int i, int j) {
      const uchar4 b = a.history[(size_t)j * a.W + i];
      return make_float4(u82f(b.x), u82f(b.y), u82f(b.z), u82f(b.w));
    });
    const float3 prev = f3(h.x, h.y, h.z);
    const float3 pc = rgb_to_ycocg(prev);
    const float3 mn = (mn_box + mn_cross) * .5f, mx = (mx_box + mx_cross) * .5f;
    const bool inside = pc.x >= mn.x && pc.y >= mn.y && pc.z >= mn.z && pc.x <= mx.x && pc.y <= mx.y && pc.z <= mx.z;
    if (inside) res = .4f * cur + (1.f - .4f) * prev;
  }
  const uchar4 o = make_uchar4(f2u8(res.z), f2u8(res.y), f2u8(res.x), 255);
  a.final_bgra[p] = o;
  a.history_next[p] = o;
}

// formatConverter.comp: texelFetch of the source, imageStore to the target
// format (UNORM8 stores clamp and round).
__global__ void convert_kernel(PbrtImage src, PbrtImage dst) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= (int)src.width || y >= (int)src.height) return;
  const char* s = (const char*)src.data + (size_t)y * src.row_bytes + (size_t)x * src.texel_bytes;
  float4 v;
  switch (src.format) {
    case PBRT_FORMAT_R32G32B32A32_SFLOAT: v = *(const float4*)s; break;
    case PBRT_FORMAT_R16G16B16A16_SFLOAT: v = load_half4((const Half4*)s); break;
    case PBRT_FORMAT_R8G8B8A8_UNORM: {
      const uchar4 b = *(const uchar4*)s;
      v = make_float4(u82f(b.x), u82f(b.y), u82f(b.z), u82f(b.w));
      break;
    }
    default: {  // B8G8R8A8_UNORM
      const uchar4 b = *(const uchar4*)s;
      v = make_float4(u82f(b.z), u82f(b.y), u82f(b.x), u82f(b.w));
    }
  }
  char* d = (char*)dst.data + (size_t)y * dst.row_bytes + (size_t)x * dst.texel_bytes;
  switch (dst.format) {
    case PBRT_FORMAT_R32G32B32A32_SFLOAT: *(float4*)d = v; break;
    case PBRT_FORMAT_R8G8B8A8_UNORM: *(uchar4*)d = make_uchar4(f2u8(v.x), f2u8(v.y), f2u8(v.z), f2u8(v.w)); break;
    default: *(uchar4*)d = make_uchar4(f2u8(v.z), f2u8(v.y), f2u8(v.x), f2u8(v.w));
  }
}

}  // namespace pbrt

using namespace pbrt;

struct PbrtTaa : pbrt::Object {
  PbrtTaa() : Object(pbrt::Kind::Taa) {}
  ~PbrtTaa() override {
    final_image.free_();
    history.free_();
    release(gbuffer);
    release(acc);
  }
  uint32_t width = 0, height = 0, work_w = 16, work_h = 16;
  PbrtGBuffer* gbuffer = nullptr;
  PbrtAccumulationBuffer* acc = nullptr;
  PbrtImage denoised{};
  pbrt::DeviceImage final_image, history;  // history: 2 layers (ping-pong)
  uint32_t parity = 0;
};

namespace {
bool is_u8x4(int32_t f) { return f == PBRT_FORMAT_B8G8R8A8_UNORM || f == PBRT_FORMAT_R8G8B8A8_UNORM; }
}  // namespace

extern "C" {

PBRT_API int pbrt_taa_create(uint32_t width, uint32_t height, uint32_t work_width, uint32_t work_height,
                             PbrtGBuffer* g, PbrtAccumulationBuffer* acc, const PbrtImage* denoised, PbrtTaa** out) {
  if (!out || !checked<PbrtGBuffer>(g, Kind::GBuffer) || !checked<PbrtAccumulationBuffer>(acc, Kind::Accumulation) ||
      !denoised || !denoised->data || width == 0 || height == 0 || work_width == 0 || work_height == 0 ||
      work_width * work_height > 1024)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "taa create: bad arguments");
  *out = nullptr;
  if (denoised->format != PBRT_FORMAT_B8G8R8A8_UNORM || denoised->width != width || denoised->height != height ||
      denoised->row_bytes != (size_t)width * 4)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "taa create: the denoised image must be a packed %ux%u B8G8R8A8 image",
                width, height);
  if (acc->motion.view.width != width || acc->motion.view.height != height)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "taa create: accumulation buffer size differs");
  auto* t = new (std::nothrow) PbrtTaa();
  if (!t) return fail(PBRT_ERROR_OUT_OF_MEMORY, "taa: host allocation");
  t->width = width;
  t->height = height;
  t->work_w = work_width;
  t->work_h = work_height;
  retain(g);
  retain(acc);
  t->gbuffer = g;
  t->acc = acc;
  t->denoised = *denoised;
  int st;
  if ((st = t->final_image.alloc(width, height, 1, PBRT_FORMAT_B8G8R8A8_UNORM)) ||
      (st = t->history.alloc(width, height, 2, PBRT_FORMAT_R8G8B8A8_UNORM))) {
    delete t;
    return st;
  }
  *out = t;
  return PBRT_OK;
}

PBRT_API int pbrt_taa_dispatch(PbrtTaa* t, const PbrtPushConstants* pc, pbrt_stream_t stream) {
  if (!checked<PbrtTaa>(t, Kind::Taa) || !pc) return fail(PBRT_ERROR_INVALID_ARGUMENT, "taa dispatch: bad arguments");
  TaaArgs a;
  a.W = (int)t->width;
  a.H = (int)t->height;
  a.frame = pc->frame_number;
  a.motion = t->acc->motion.ptr<__half2>();
  a.denoised = (const uchar4*)t->denoised.data;
  const size_t layer = (size_t)t->width * t->height;
  a.history = t->history.ptr<uchar4>() + (size_t)t->parity * layer;
  a.history_next = t->history.ptr<uchar4>() + (size_t)(t->parity ^ 1u) * layer;
  a.final_bgra = t->final_image.ptr<uchar4>();
  dim3 block(t->work_w, t->work_h), grid((t->width + t->work_w - 1) / t->work_w, (t->height + t->work_h - 1) / t->work_h);
  taa_kernel<<<grid, block, 0, stream>>>(a);
  int st = check_launch("taa_kernel");
  if (!st) t->parity ^= 1u;
  return st;
}

PBRT_API int pbrt_taa_final_image(const PbrtTaa* t, PbrtImage* out) {
  if (!checked<const PbrtTaa>((void*)t, Kind::Taa) || !out) return fail(PBRT_ERROR_INVALID_ARGUMENT, "taa final image");
  *out = t->final_image.view;
  return PBRT_OK;
}

PBRT_API int pbrt_format_convert(const PbrtImage* src, const PbrtImage* dst, pbrt_stream_t stream) {
  if (!src || !dst || !src->data || !dst->data || src->width != dst->width || src->height != dst->height)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "format convert: bad images");
  const bool src_ok = src->format == PBRT_FORMAT_R32G32B32A32_SFLOAT || src->format == PBRT_FORMAT_R16G16B16A16_SFLOAT ||
                      is_u8x4(src->format);
  const bool dst_ok = dst->format == PBRT_FORMAT_R32G32B32A32_SFLOAT || is_u8x4(dst->format);
  if (!src_ok || !dst_ok) return fail(PBRT_ERROR_UNSUPPORTED, "format convert: %d -> %d", src->format, dst->format);
  dim3 block(16, 16), grid((src->width + 15) / 16, (src->height + 15) / 16);
  convert_kernel<<<grid, block, 0, stream>>>(*src, *dst);
  return check_launch("convert_kernel");
}

}  // extern "C"
