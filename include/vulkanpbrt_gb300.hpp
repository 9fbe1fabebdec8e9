/*
 * vulkanpbrt_gb300.hpp -- the render-module classes of VulkanPBRT as
 * header-only C++17 over the C ABI (vulkanpbrt_gb300.h).
 *
 * Class, attribute and method names follow the reference's render modules
 * and buffers so that host code written against them compiles against these
 * with the Vulkan types swapped for CUDA ones:
 *   GBuffer             source/buffers/GBuffer.hpp:9-26
 *   IlluminationBuffer* source/buffers/IlluminationBuffer.hpp:9-80
 *   AccumulationBuffer  source/buffers/AccumulationBuffer.hpp:10-30
 *   PBRTPipeline        source/renderModules/PBRTPipeline.hpp:19-60
 *   Accumulator         source/renderModules/Accumulator.hpp:8-49
 *   BMFR                source/renderModules/denoisers/BMFR.hpp:14-41
 *   BFR                 source/renderModules/denoisers/BFR.hpp:8-45
 *   BFRBlender          source/renderModules/denoisers/BFRBlender.hpp:6-27
 *   Taa                 source/renderModules/Taa.hpp:9-35
 * Objects are created with T::create(...) and held by ref_ptr<T> (the
 * intrusive reference count of vsg::Inherit / vsg::ref_ptr). Images are
 * public attributes: device buffers the library owns (the reference's
 * DescriptorImage attributes). add_*_to_command_graph records work into a
 * Commands list; Commands::submit(stream) replays it on a CUDA stream, reading
 * the PushConstants values current at submit time (the reference records
 * its command graph once and resubmits it every frame,
 * source/VulkanPBRT.cpp:397-505, 551-618). compile() and
 * update_image_layouts() do nothing: images exist from construction and CUDA
 * has no image layouts. Errors throw vkpbrt::Exception (the reference throws
 * vsg::Exception{message}). The classes are also visible in the global
 * namespace, as in the reference, unless VULKANPBRT_GB300_NO_GLOBAL_NAMES is
 * defined before the include.
 */
#ifndef VULKANPBRT_GB300_HPP
#define VULKANPBRT_GB300_HPP

#include <atomic>
#include <cstdint>
#include <functional>
#include <string>
#include <utility>
#include <vector>

#include "vulkanpbrt_gb300.h"

namespace vkpbrt {

// vsg::Exception: the message, plus the C ABI status it came from.
struct Exception {
  std::string message;
  int result = PBRT_OK;
};

// Throws Exception with the library's last message when status is not PBRT_OK.
inline void check(int status, const char* what) {
  if (status == PBRT_OK) return;
  char buf[1024];
  buf[0] = '\0';
  pbrt_last_error(buf, sizeof(buf));
  throw Exception{std::string(what) + ": " + buf, status};
}

// Intrusively reference-counted base (vsg::Object).
class Object {
 public:
  Object() = default;
  Object(const Object&) = delete;
  Object& operator=(const Object&) = delete;
  virtual ~Object() = default;
  void ref() const { refs_.fetch_add(1, std::memory_order_relaxed); }
  void unref() const {
    if (refs_.fetch_sub(1, std::memory_order_acq_rel) == 1) delete this;
  }
  unsigned referenceCount() const { return refs_.load(std::memory_order_relaxed); }

 private:
  mutable std::atomic<unsigned> refs_{0};
};

// vsg::ref_ptr: shared ownership through the object's own count.
template <class T> class ref_ptr {
 public:
  ref_ptr() = default;
  explicit ref_ptr(T* p) : p_(p) {
    if (p_) p_->ref();
  }
  ref_ptr(const ref_ptr& o) : ref_ptr(o.p_) {}
  template <class U> ref_ptr(const ref_ptr<U>& o) : ref_ptr(o.get()) {}
  ref_ptr(ref_ptr&& o) noexcept : p_(std::exchange(o.p_, nullptr)) {}
  ~ref_ptr() {
    if (p_) p_->unref();
  }
  ref_ptr& operator=(ref_ptr o) noexcept {
    std::swap(p_, o.p_);
    return *this;
  }
  T* get() const { return p_; }
  T* operator->() const { return p_; }
  T& operator*() const { return *p_; }
  explicit operator bool() const { return p_ != nullptr; }

 private:
  T* p_ = nullptr;
};

// vsg::Inherit<Object, T>: T::create(args...) -> ref_ptr<T>.
template <class Base, class T> class Inherit : public Base {
 public:
  using Base::Base;
  template <class... Args> static ref_ptr<T> create(Args&&... args) {
    return ref_ptr<T>(new T(std::forward<Args>(args)...));
  }
};

// The C handle behind a (possibly null) object: the C ABI reports a null
// handle as PBRT_ERROR_INVALID_ARGUMENT, which check() turns into Exception.
template <class T> auto c_handle_of(const ref_ptr<T>& p) -> decltype(p->c_handle()) {
  return p ? p->c_handle() : nullptr;
}

// A library handle of a C ABI object, released with the C++ object.
class Handle : public Object {
 public:
  ~Handle() override {
    if (handle_) pbrt_release(handle_);
  }

 protected:
  void* handle_ = nullptr;
};

// A device image owned by a library object (vsg::DescriptorImage's role).
struct Image {
  PbrtImage view{};
  void* data() const { return view.data; }
  uint32_t width() const { return view.width; }
  uint32_t height() const { return view.height; }
  uint32_t layers() const { return view.layers; }
  PbrtFormat format() const { return static_cast<PbrtFormat>(view.format); }
  size_t bytes() const { return view.layer_bytes * view.layers; }
  // Stream-ordered whole-image copies from / to host memory (rows host_row_bytes apart; 0 = packed).
  void upload(const void* host, size_t host_row_bytes = 0, pbrt_stream_t stream = nullptr) const {
    check(pbrt_image_upload(&view, host, host_row_bytes ? host_row_bytes : view.row_bytes, stream), "Image::upload");
  }
  void download(void* host, size_t host_row_bytes = 0, pbrt_stream_t stream = nullptr) const {
    check(pbrt_image_download(&view, host, host_row_bytes ? host_row_bytes : view.row_bytes, stream),
          "Image::download");
  }
};

// vsg::PushConstants holding RayTracingPushConstants
// (source/renderModules/PipelineStructs.hpp:6-13); recorded commands read
// `value` when they are submitted.
class PushConstants : public Inherit<Object, PushConstants> {
 public:
  PbrtPushConstants value{};
};

// vsg::Commands: recorded GPU work, replayed on a stream.
class Commands : public Inherit<Object, Commands> {
 public:
  void addChild(std::function<void(pbrt_stream_t)> call) { calls_.push_back(std::move(call)); }
  void submit(pbrt_stream_t stream = nullptr) const {
    for (const auto& c : calls_) c(stream);
  }
  size_t size() const { return calls_.size(); }

 private:
  std::vector<std::function<void(pbrt_stream_t)>> calls_;
};

// CameraMatrices (source/io/RenderIO.hpp), column-major.
using CameraMatrices = PbrtCameraMatrices;

// ---------------------------------------------------------------------------
class GBuffer : public Inherit<Handle, GBuffer> {
 public:
  GBuffer(uint32_t width_, uint32_t height_) : width(width_), height(height_) {
    PbrtGBuffer* g = nullptr;
    check(pbrt_gbuffer_create(width, height, &g), "GBuffer");
    handle_ = g;
    check(pbrt_gbuffer_images(g, &depth.view, &normal.view, &material.view, &albedo.view), "GBuffer images");
  }
  void compile(void* /*context*/ = nullptr) {}
  void update_image_layouts(void* /*context*/ = nullptr) {}
  PbrtGBuffer* c_handle() const { return static_cast<PbrtGBuffer*>(handle_); }

  uint32_t width, height;
  Image depth, normal, material, albedo;
};

class IlluminationBuffer : public Inherit<Handle, IlluminationBuffer> {
 public:
  void compile(void* /*context*/ = nullptr) {}
  void update_image_layouts(void* /*context*/ = nullptr) {}
  PbrtIlluminationBuffer* c_handle() const { return static_cast<PbrtIlluminationBuffer*>(handle_); }
  // Wraps a handle (takes over one reference).
  static ref_ptr<IlluminationBuffer> adopt(PbrtIlluminationBuffer* h, uint32_t w, uint32_t hh) {
    ref_ptr<IlluminationBuffer> b(new IlluminationBuffer());
    b->attach(h, w, hh);
    return b;
  }

  uint32_t width = 0, height = 0;
  std::vector<Image> illumination_images;

 protected:
  IlluminationBuffer() = default;
  IlluminationBuffer(PbrtIlluminationType type, uint32_t w, uint32_t h) {
    PbrtIlluminationBuffer* b = nullptr;
    check(pbrt_illumination_buffer_create(type, w, h, &b), "IlluminationBuffer");
    attach(b, w, h);
  }
  void attach(PbrtIlluminationBuffer* b, uint32_t w, uint32_t h) {
    handle_ = b;
    width = w;
    height = h;
    PbrtImage views[4];
    uint32_t n = 0;
    check(pbrt_illumination_buffer_images(b, views, 4, &n), "IlluminationBuffer images");
    illumination_images.resize(n);
    for (uint32_t i = 0; i < n; ++i) illumination_images[i].view = views[i];
  }
};

#define VKPBRT_ILLUMINATION_BUFFER(NAME, TYPE)                                         \
  class NAME : public IlluminationBuffer {                                            \
   public:                                                                            \
    NAME(uint32_t w, uint32_t h) : IlluminationBuffer(TYPE, w, h) {}                  \
    static ref_ptr<NAME> create(uint32_t w, uint32_t h) { return ref_ptr<NAME>(new NAME(w, h)); } \
  };
VKPBRT_ILLUMINATION_BUFFER(IlluminationBufferFinal, PBRT_ILLUMINATION_FINAL)
VKPBRT_ILLUMINATION_BUFFER(IlluminationBufferFinalDemodulated, PBRT_ILLUMINATION_FINAL_DEMODULATED)
VKPBRT_ILLUMINATION_BUFFER(IlluminationBufferDemodulated, PBRT_ILLUMINATION_DEMODULATED)
VKPBRT_ILLUMINATION_BUFFER(IlluminationBufferDemodulatedFloat, PBRT_ILLUMINATION_DEMODULATED_FLOAT)
VKPBRT_ILLUMINATION_BUFFER(IlluminationBufferFinalFloat, PBRT_ILLUMINATION_FINAL_FLOAT)
#undef VKPBRT_ILLUMINATION_BUFFER

class AccumulationBuffer : public Inherit<Handle, AccumulationBuffer> {
 public:
  AccumulationBuffer(uint32_t w, uint32_t h) {
    PbrtAccumulationBuffer* a = nullptr;
    check(pbrt_accumulation_buffer_create(w, h, &a), "AccumulationBuffer");
    attach(a, w, h);
  }
  static ref_ptr<AccumulationBuffer> adopt(PbrtAccumulationBuffer* a, uint32_t w, uint32_t h) {
    ref_ptr<AccumulationBuffer> b(new AccumulationBuffer(a, w, h));
    return b;
  }
  void compile(void* /*context*/ = nullptr) {}
  void update_image_layouts(void* /*context*/ = nullptr) {}
  // AccumulationBuffer::copy_to_back_images (AccumulationBuffer.cpp:72-244)
  void copy_to_back_images(ref_ptr<Commands> commands, ref_ptr<GBuffer> g_buffer,
                           ref_ptr<IlluminationBuffer> illumination_buffer) {
    ref_ptr<AccumulationBuffer> self(this);
    commands->addChild([self, g_buffer, illumination_buffer](pbrt_stream_t s) {
      check(pbrt_accumulation_buffer_copy_to_back_images(self->c_handle(), c_handle_of(g_buffer),
                                                         c_handle_of(illumination_buffer), s),
            "AccumulationBuffer::copy_to_back_images");
    });
  }
  PbrtAccumulationBuffer* c_handle() const { return static_cast<PbrtAccumulationBuffer*>(handle_); }

  uint32_t width = 0, height = 0;
  Image prev_illu, prev_illu_squared, prev_depth, prev_normal, spp, prev_spp, motion;

 private:
  AccumulationBuffer(PbrtAccumulationBuffer* a, uint32_t w, uint32_t h) { attach(a, w, h); }
  void attach(PbrtAccumulationBuffer* a, uint32_t w, uint32_t h) {
    handle_ = a;
    width = w;
    height = h;
    PbrtAccumulationImages im{};
    check(pbrt_accumulation_buffer_images(a, &im), "AccumulationBuffer images");
    prev_illu.view = im.prev_illu;
    prev_illu_squared.view = im.prev_illu_squared;
    prev_depth.view = im.prev_depth;
    prev_normal.view = im.prev_normal;
    spp.view = im.spp;
    prev_spp.view = im.prev_spp;
    motion.view = im.motion;
  }
};

class Accumulator : public Inherit<Handle, Accumulator> {
 public:
  Accumulator(ref_ptr<GBuffer> g_buffer, ref_ptr<IlluminationBuffer> illumination_buffer,
              bool separate_matrices = true, int32_t work_width = 16, int32_t work_height = 16)
      : g_buffer_(g_buffer), source_(illumination_buffer) {
    PbrtAccumulator* a = nullptr;
    check(pbrt_accumulator_create(c_handle_of(g_buffer), c_handle_of(illumination_buffer), separate_matrices ? 1 : 0,
                                  work_width, work_height, &a),
          "Accumulator");
    handle_ = a;
    PbrtIlluminationBuffer* ib = nullptr;
    PbrtAccumulationBuffer* ab = nullptr;
    check(pbrt_accumulator_get_accumulated_illumination(a, &ib), "Accumulator accumulated_illumination");
    check(pbrt_accumulator_get_accumulation_buffer(a, &ab), "Accumulator accumulation_buffer");
    check(pbrt_retain(ib), "retain");  // borrowed references: the C++ wrappers own one each
    check(pbrt_retain(ab), "retain");
    accumulated_illumination = IlluminationBuffer::adopt(ib, g_buffer->width, g_buffer->height);
    accumulation_buffer = AccumulationBuffer::adopt(ab, g_buffer->width, g_buffer->height);
  }
  void compile(void* /*context*/ = nullptr) {}
  void update_image_layouts(void* /*context*/ = nullptr) {}
  // Accumulator::set_camera_matrices (Accumulator.cpp:85-117)
  void set_camera_matrices(int32_t frame_index, const CameraMatrices& cur, const CameraMatrices& prev) {
    check(pbrt_accumulator_set_camera_matrices(c_handle(), frame_index, &cur, &prev),
          "Accumulator::set_camera_matrices");
  }
  // Accumulator::add_dispatch_to_command_graph (Accumulator.cpp:72-83)
  void add_dispatch_to_command_graph(ref_ptr<Commands> commands) {
    ref_ptr<Accumulator> self(this);
    commands->addChild([self](pbrt_stream_t s) {
      check(pbrt_accumulator_dispatch(self->c_handle(), s), "Accumulator::dispatch");
    });
  }
  PbrtAccumulator* c_handle() const { return static_cast<PbrtAccumulator*>(handle_); }

  ref_ptr<IlluminationBuffer> accumulated_illumination;
  ref_ptr<AccumulationBuffer> accumulation_buffer;

 private:
  ref_ptr<GBuffer> g_buffer_;
  ref_ptr<IlluminationBuffer> source_;
};

// The scene the pipeline traces: stands for the vsg scene graph after
// RayTracingSceneDescriptorCreationVisitor and the acceleration-structure
// build (pbrt_scene_create_ex builds the 8-wide BVH: binned SAH on the host
// by default, or PBRT_BUILD_PREFER_FAST_BUILD for the device build, as a
// Vulkan acceleration-structure build's PREFER_FAST_TRACE / FAST_BUILD flags).
class Scene : public Inherit<Handle, Scene> {
 public:
  explicit Scene(const PbrtSceneDesc& desc, uint32_t build_flags = PBRT_BUILD_PREFER_FAST_TRACE) {
    PbrtScene* s = nullptr;
    check(pbrt_scene_create_ex(&desc, build_flags, &s), "Scene");
    handle_ = s;
  }
  PbrtSceneInfo info() const {
    PbrtSceneInfo i{};
    check(pbrt_scene_info(c_handle(), &i), "Scene::info");
    return i;
  }
  PbrtScene* c_handle() const { return static_cast<PbrtScene*>(handle_); }
};

enum class RayTracingRayOrigin { CAMERA, GBUFFER };

class PBRTPipeline : public Inherit<Handle, PBRTPipeline> {
 public:
  // PBRTPipeline(scene, g_buffer, illumination_buffer, write_g_buffer,
  // ray_tracing_ray_origin) (PBRTPipeline.hpp:22-24). g_buffer may be null
  // when write_g_buffer is false. Rays start at the camera; GBUFFER origins
  // are not supported.
  PBRTPipeline(ref_ptr<Scene> scene, ref_ptr<GBuffer> g_buffer, ref_ptr<IlluminationBuffer> illumination_buffer,
               bool write_g_buffer, RayTracingRayOrigin ray_tracing_ray_origin = RayTracingRayOrigin::CAMERA)
      : scene_(scene), g_buffer_(g_buffer), illumination_buffer_(illumination_buffer) {
    if (ray_tracing_ray_origin != RayTracingRayOrigin::CAMERA)
      throw Exception{"PBRTPipeline: ray origins from the G-buffer are not supported", PBRT_ERROR_UNSUPPORTED};
    PbrtPipeline* p = nullptr;
    check(pbrt_pipeline_create(c_handle_of(scene), c_handle_of(g_buffer), c_handle_of(illumination_buffer),
                               write_g_buffer ? 1 : 0, &p),
          "PBRTPipeline");
    handle_ = p;
  }
  // PBRTPipeline::set_tlas (PBRTPipeline.cpp:38-56): here the scene carries
  // its own BVH; a pipeline traces the scene it was created with.
  void set_tlas(ref_ptr<Scene> scene) {
    if (scene.get() != scene_.get())
      throw Exception{"PBRTPipeline::set_tlas: create a pipeline per scene", PBRT_ERROR_UNSUPPORTED};
  }
  void compile(void* /*context*/ = nullptr) { apply_config(); }
  void update_image_layouts(void* /*context*/ = nullptr) {}
  // PBRTPipeline::add_trace_rays_to_command_graph (PBRTPipeline.cpp:65-80)
  void add_trace_rays_to_command_graph(ref_ptr<Commands> commands, ref_ptr<PushConstants> push_constants) {
    apply_config();
    ref_ptr<PBRTPipeline> self(this);
    commands->addChild([self, push_constants](pbrt_stream_t s) {
      check(pbrt_pipeline_trace(self->c_handle(), &push_constants->value, s), "PBRTPipeline::trace");
    });
  }
  ref_ptr<IlluminationBuffer> get_illumination_buffer() const { return illumination_buffer_; }
  PbrtTraceStats stats(pbrt_stream_t stream = nullptr) const {
    PbrtTraceStats st{};
    check(pbrt_pipeline_stats(c_handle(), stream, &st), "PBRTPipeline::stats");
    return st;
  }
  PbrtPipeline* c_handle() const { return static_cast<PbrtPipeline*>(handle_); }

  enum class LightSamplingMethod {
    SAMPLE_SURFACE_STRENGTH,
    SAMPLE_LIGHT_STRENGTH,
    SAMPLE_UNIFORM
  } light_sampling_method = LightSamplingMethod::SAMPLE_SURFACE_STRENGTH;
  // The Infos UBO's recursion depths (layoutPTUniform.glsl:4-9; the reference fixes 2 / 0).
  int32_t max_recursion_depth = 2, min_recursion_depth = 0;

 private:
  void apply_config() {
    check(pbrt_pipeline_set_config(c_handle(), static_cast<int32_t>(light_sampling_method), min_recursion_depth,
                                   max_recursion_depth),
          "PBRTPipeline config");
  }
  ref_ptr<Scene> scene_;
  ref_ptr<GBuffer> g_buffer_;
  ref_ptr<IlluminationBuffer> illumination_buffer_;
};

class BMFR : public Inherit<Handle, BMFR> {
 public:
  BMFR(uint32_t width, uint32_t height, uint32_t work_width, uint32_t work_height, ref_ptr<GBuffer> g_buffer,
       ref_ptr<IlluminationBuffer> illu_buffer, ref_ptr<AccumulationBuffer> acc_buffer, uint32_t fitting_kernel = 256)
      : inputs_{g_buffer, illu_buffer, acc_buffer} {
    PbrtBMFR* b = nullptr;
    check(pbrt_bmfr_create(width, height, work_width, work_height, c_handle_of(g_buffer), c_handle_of(illu_buffer),
                           c_handle_of(acc_buffer), fitting_kernel, &b),
          "BMFR");
    handle_ = b;
    check(pbrt_bmfr_final_image(b, &final_.view), "BMFR final image");
    check(pbrt_bmfr_images(b, &denoised.view, &weights.view), "BMFR images");
  }
  void compile(void* /*context*/ = nullptr) {}
  void update_image_layouts(void* /*context*/ = nullptr) {}
  // BMFR::add_dispatch_to_command_graph (BMFR.cpp:203-230)
  void add_dispatch_to_command_graph(ref_ptr<Commands> commands, ref_ptr<PushConstants> push_constants) {
    ref_ptr<BMFR> self(this);
    commands->addChild([self, push_constants](pbrt_stream_t s) {
      check(pbrt_bmfr_dispatch(self->c_handle(), &push_constants->value, s), "BMFR::dispatch");
    });
  }
  // BMFR::get_final_descriptor_image (BMFR.cpp:231-234): B8G8R8A8.
  const Image& get_final_descriptor_image() const { return final_; }
  PbrtBMFR* c_handle() const { return static_cast<PbrtBMFR*>(handle_); }

  Image denoised, weights;  // RGBA16F x 2 layers; R32F x 30 layers at block-grid size

 private:
  struct Inputs {
    ref_ptr<GBuffer> g;
    ref_ptr<IlluminationBuffer> illumination;
    ref_ptr<AccumulationBuffer> acc;
  } inputs_;
  Image final_;
};

class BFR : public Inherit<Handle, BFR> {
 public:
  BFR(uint32_t width, uint32_t height, uint32_t work_width, uint32_t work_height, ref_ptr<GBuffer> g_buffer,
      ref_ptr<IlluminationBuffer> illu_buffer, ref_ptr<AccumulationBuffer> acc_buffer)
      : g_(g_buffer), illumination_(illu_buffer), acc_(acc_buffer) {
    PbrtBFR* b = nullptr;
    check(pbrt_bfr_create(width, height, work_width, work_height, c_handle_of(g_buffer), c_handle_of(illu_buffer),
                          c_handle_of(acc_buffer), &b),
          "BFR");
    handle_ = b;
    check(pbrt_bfr_final_image(b, &final_.view), "BFR final image");
    check(pbrt_bfr_images(b, &denoised.view), "BFR images");
  }
  void compile(void* /*context*/ = nullptr) {}
  void update_image_layouts(void* /*context*/ = nullptr) {}
  // BFR::add_dispatch_to_command_graph (BFR.cpp:128-138)
  void add_dispatch_to_command_graph(ref_ptr<Commands> commands, ref_ptr<PushConstants> push_constants) {
    ref_ptr<BFR> self(this);
    commands->addChild([self, push_constants](pbrt_stream_t s) {
      check(pbrt_bfr_dispatch(self->c_handle(), &push_constants->value, s), "BFR::dispatch");
    });
  }
  const Image& get_final_descriptor_image() const { return final_; }
  PbrtBFR* c_handle() const { return static_cast<PbrtBFR*>(handle_); }

  Image denoised;

 private:
  ref_ptr<GBuffer> g_;
  ref_ptr<IlluminationBuffer> illumination_;
  ref_ptr<AccumulationBuffer> acc_;
  Image final_;
};

class Taa : public Inherit<Handle, Taa> {
 public:
  // Taa(width, height, work_width, work_height, g_buffer, acc_buffer,
  // denoised) (Taa.cpp:4-91); denoised is a denoiser's final image, whose
  // owner must outlive this object.
  Taa(uint32_t width, uint32_t height, uint32_t work_width, uint32_t work_height, ref_ptr<GBuffer> g_buffer,
      ref_ptr<AccumulationBuffer> acc_buffer, const Image& denoised)
      : g_(g_buffer), acc_(acc_buffer) {
    PbrtTaa* t = nullptr;
    check(pbrt_taa_create(width, height, work_width, work_height, c_handle_of(g_buffer), c_handle_of(acc_buffer),
                          &denoised.view, &t),
          "Taa");
    handle_ = t;
    check(pbrt_taa_final_image(t, &final_.view), "Taa final image");
  }
  void compile(void* /*context*/ = nullptr) {}
  void update_image_layouts(void* /*context*/ = nullptr) {}
  void add_dispatch_to_command_graph(ref_ptr<Commands> commands, ref_ptr<PushConstants> push_constants) {
    ref_ptr<Taa> self(this);
    commands->addChild([self, push_constants](pbrt_stream_t s) {
      check(pbrt_taa_dispatch(self->c_handle(), &push_constants->value, s), "Taa::dispatch");
    });
  }
  const Image& get_final_descriptor_image() const { return final_; }
  PbrtTaa* c_handle() const { return static_cast<PbrtTaa*>(handle_); }

 private:
  ref_ptr<GBuffer> g_;
  ref_ptr<AccumulationBuffer> acc_;
  Image final_;
};

class BFRBlender : public Inherit<Handle, BFRBlender> {
 public:
  // BFRBlender(width, height, average_image, average_squared_image,
  // denoised0..2, work_width = 16, work_height = 16, filter_radius = 2); the
  // images' owners must outlive this object.
  BFRBlender(uint32_t width, uint32_t height, const Image& average_image, const Image& average_squared_image,
             const Image& denoised0, const Image& denoised1, const Image& denoised2, uint32_t work_width = 16,
             uint32_t work_height = 16, uint32_t filter_radius = 2) {
    PbrtBFRBlender* b = nullptr;
    check(pbrt_bfr_blender_create(width, height, &average_image.view, &average_squared_image.view, &denoised0.view,
                                  &denoised1.view, &denoised2.view, work_width, work_height, filter_radius, &b),
          "BFRBlender");
    handle_ = b;
    check(pbrt_bfr_blender_final_image(b, &final_.view), "BFRBlender final image");
  }
  void compile(void* /*context*/ = nullptr) {}
  void update_image_layouts(void* /*context*/ = nullptr) {}
  void add_dispatch_to_command_graph(ref_ptr<Commands> commands) {
    ref_ptr<BFRBlender> self(this);
    commands->addChild([self](pbrt_stream_t s) {
      check(pbrt_bfr_blender_dispatch(self->c_handle(), s), "BFRBlender::dispatch");
    });
  }
  const Image& get_final_descriptor_image() const { return final_; }
  PbrtBFRBlender* c_handle() const { return static_cast<PbrtBFRBlender*>(handle_); }

 private:
  Image final_;
};

// FormatConverter (source/renderModules/FormatConverter.cpp): dst = src texel by texel.
inline void format_convert(const Image& src, const Image& dst, pbrt_stream_t stream = nullptr) {
  check(pbrt_format_convert(&src.view, &dst.view, stream), "FormatConverter");
}

}  // namespace vkpbrt

#ifndef VULKANPBRT_GB300_NO_GLOBAL_NAMES
using vkpbrt::AccumulationBuffer;
using vkpbrt::Accumulator;
using vkpbrt::BFR;
using vkpbrt::BFRBlender;
using vkpbrt::BMFR;
using vkpbrt::GBuffer;
using vkpbrt::IlluminationBuffer;
using vkpbrt::IlluminationBufferDemodulated;
using vkpbrt::IlluminationBufferDemodulatedFloat;
using vkpbrt::IlluminationBufferFinal;
using vkpbrt::IlluminationBufferFinalDemodulated;
using vkpbrt::IlluminationBufferFinalFloat;
using vkpbrt::PBRTPipeline;
using vkpbrt::RayTracingRayOrigin;
using vkpbrt::Taa;
#endif

#endif  // VULKANPBRT_GB300_HPP
