/*
 * vulkanpbrt_gb300.h -- C ABI of the GB300-native per-frame path of
 * VulkanPBRT: path tracer (PBRTPipeline), temporal accumulator and the BMFR /
 * BFR regression denoisers.
 *
 * Every entry point replaces a method of the reference's render-module C++
 * classes; the comment above each names the reference interface (file:line,
 * relative to the VulkanPBRT source tree). Conventions:
 *   - every call returns int status: PBRT_OK (0) or a negative PbrtStatus;
 *     pbrt_last_error() gives the calling thread's last message;
 *   - handles are opaque and reference counted (pbrt_retain/pbrt_release);
 *     an object retains the objects it was created from;
 *   - images are device buffers the library owns, exposed through PbrtImage
 *     views (the reference's public DescriptorImage attributes), rows packed,
 *     layers consecutive;
 *   - work is stream ordered on the cudaStream_t passed in (NULL = legacy
 *     default stream). Calls on one handle are not reentrant: use one handle
 *     per host thread or synchronise externally (the reference records and
 *     submits from a single thread).
 */
#ifndef VULKANPBRT_GB300_H
#define VULKANPBRT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define PBRT_API __attribute__((visibility("default")))
#else
#define PBRT_API
#endif

struct CUstream_st;
typedef struct CUstream_st* pbrt_stream_t; /* == cudaStream_t */

typedef enum PbrtStatus {
  PBRT_OK = 0,
  PBRT_ERROR_INVALID_ARGUMENT = -1,
  PBRT_ERROR_CUDA = -2,
  PBRT_ERROR_OUT_OF_MEMORY = -3,
  PBRT_ERROR_UNSUPPORTED = -4,
  PBRT_ERROR_ABORTED = -5,
  PBRT_ERROR_TIMEOUT = -6
} PbrtStatus;

/* Texel formats of the reference's images (Vulkan VK_FORMAT_* names). */
typedef enum PbrtFormat {
  PBRT_FORMAT_R32_SFLOAT = 1,
  PBRT_FORMAT_R32G32_SFLOAT = 2,
  PBRT_FORMAT_R32G32B32A32_SFLOAT = 3,
  PBRT_FORMAT_R16_SFLOAT = 4,
  PBRT_FORMAT_R16G16_SFLOAT = 5,
  PBRT_FORMAT_R16G16B16A16_SFLOAT = 6,
  PBRT_FORMAT_R8_UNORM = 7,
  PBRT_FORMAT_R8G8B8A8_UNORM = 8,
  PBRT_FORMAT_B8G8R8A8_UNORM = 9,
  PBRT_FORMAT_R32_UINT = 10
} PbrtFormat;

/* A device image: texel (x, y) of layer l is at
 * data + l * layer_bytes + y * row_bytes + x * texel_bytes. */
typedef struct PbrtImage {
  void* data;
  uint32_t width, height, layers;
  int32_t format; /* PbrtFormat */
  uint32_t texel_bytes;
  size_t row_bytes, layer_bytes;
} PbrtImage;

/* RayTracingPushConstants (source/renderModules/PipelineStructs.hpp:6-13);
 * matrices column-major as vsg::mat4 / GLSL mat4. */
typedef struct PbrtPushConstants {
  float view_inverse[16];
  float proj_inverse[16];
  float prev_view[16];
  uint32_t frame_number;
  uint32_t sample_number;
} PbrtPushConstants;

/* CameraMatrices (source/io/RenderIO.hpp) as Accumulator::set_camera_matrices
 * reads it; has_proj says whether proj / inv_proj are set. */
typedef struct PbrtCameraMatrices {
  float view[16];
  float inv_view[16];
  float proj[16];
  float inv_proj[16];
  int32_t has_proj;
} PbrtCameraMatrices;

typedef struct PbrtGBuffer PbrtGBuffer;
typedef struct PbrtIlluminationBuffer PbrtIlluminationBuffer;
typedef struct PbrtAccumulationBuffer PbrtAccumulationBuffer;
typedef struct PbrtAccumulator PbrtAccumulator;
typedef struct PbrtBMFR PbrtBMFR;
typedef struct PbrtBFR PbrtBFR;
typedef struct PbrtScene PbrtScene;
typedef struct PbrtPipeline PbrtPipeline;
typedef struct PbrtNeural PbrtNeural;
typedef struct PbrtTaa PbrtTaa;
typedef struct PbrtBFRBlender PbrtBFRBlender;
typedef struct PbrtBatch PbrtBatch;

/* ---- library ---------------------------------------------------------- */
PBRT_API const char* pbrt_version(void);
/* Copies the calling thread's last error message (NUL terminated). */
PBRT_API int pbrt_last_error(char* buffer, size_t size);
/* Reference counting for every handle type above. */
PBRT_API int pbrt_retain(void* handle);
PBRT_API int pbrt_release(void* handle);
/* Host <-> device copies of a whole image (all layers), stream ordered:
 * the staging-buffer copies of the reference's offline replay
 * (OfflineGBuffer / OfflineIllumination upload_* / download_*,
 * source/io/RenderIO.cpp:372-391, 718-1008). host rows are host_row_bytes
 * apart (>= width * texel bytes). */
PBRT_API int pbrt_image_upload(const PbrtImage* dst, const void* host, size_t host_row_bytes, pbrt_stream_t stream);
PBRT_API int pbrt_image_download(const PbrtImage* src, void* host, size_t host_row_bytes, pbrt_stream_t stream);
PBRT_API int pbrt_stream_synchronize(pbrt_stream_t stream);

/* ---- GBuffer (source/buffers/GBuffer.hpp:9-26) -------------------------
 * Public images depth R32F, normal RG32F (theta, phi), material RGBA8,
 * albedo RGBA8 (GBuffer.cpp:53-125). */
PBRT_API int pbrt_gbuffer_create(uint32_t width, uint32_t height, PbrtGBuffer** out);
PBRT_API int pbrt_gbuffer_images(const PbrtGBuffer* g, PbrtImage* depth, PbrtImage* normal, PbrtImage* material,
                                 PbrtImage* albedo);

/* ---- IlluminationBuffer family (source/buffers/IlluminationBuffer.hpp) --
 * type: the subclass name's suffix. Image lists follow
 * IlluminationBuffer.cpp:73-310: Final {BGRA8}, FinalDemodulated {BGRA8,
 * RGBA16F illumination, RGBA16F illuminationSquared}, Demodulated {RGBA16F
 * illumination, RGBA16F illuminationSquared}, DemodulatedFloat {RGBA32F},
 * FinalFloat {RGBA32F}. */
typedef enum PbrtIlluminationType {
  PBRT_ILLUMINATION_FINAL = 0,
  PBRT_ILLUMINATION_FINAL_DEMODULATED = 1,
  PBRT_ILLUMINATION_DEMODULATED = 2,
  PBRT_ILLUMINATION_DEMODULATED_FLOAT = 3,
  PBRT_ILLUMINATION_FINAL_FLOAT = 4
} PbrtIlluminationType;
PBRT_API int pbrt_illumination_buffer_create(int32_t type, uint32_t width, uint32_t height,
                                             PbrtIlluminationBuffer** out);
PBRT_API int pbrt_illumination_buffer_images(const PbrtIlluminationBuffer* b, PbrtImage* images, uint32_t capacity,
                                             uint32_t* count);

/* ---- AccumulationBuffer (source/buffers/AccumulationBuffer.hpp:10-30) ---
 * prev_illu, prev_illu_squared RGBA16F; prev_depth R32F; prev_normal RG32F;
 * spp, prev_spp R8_UNORM; motion RG16F (AccumulationBuffer.cpp:245-339). */
PBRT_API int pbrt_accumulation_buffer_create(uint32_t width, uint32_t height, PbrtAccumulationBuffer** out);
typedef struct PbrtAccumulationImages {
  PbrtImage prev_illu, prev_illu_squared, prev_depth, prev_normal, spp, prev_spp, motion;
} PbrtAccumulationImages;
PBRT_API int pbrt_accumulation_buffer_images(const PbrtAccumulationBuffer* a, PbrtAccumulationImages* out);
/* AccumulationBuffer::copy_to_back_images (AccumulationBuffer.cpp:72-244):
 * depth->prev_depth, normal->prev_normal, spp->prev_spp and the
 * demodulated illumination (image 0, or image 1 of FinalDemodulated) ->
 * prev_illu. */
PBRT_API int pbrt_accumulation_buffer_copy_to_back_images(PbrtAccumulationBuffer* a, const PbrtGBuffer* g,
                                                          const PbrtIlluminationBuffer* illumination,
                                                          pbrt_stream_t stream);

/* ---- Accumulator (source/renderModules/Accumulator.hpp:8-49) ----------- */
PBRT_API int pbrt_accumulator_create(PbrtGBuffer* g, PbrtIlluminationBuffer* illumination, int32_t separate_matrices,
                                     int32_t work_width, int32_t work_height, PbrtAccumulator** out);
/* Accumulator::set_camera_matrices (Accumulator.cpp:85-117). */
PBRT_API int pbrt_accumulator_set_camera_matrices(PbrtAccumulator* acc, int32_t frame_index,
                                                  const PbrtCameraMatrices* cur, const PbrtCameraMatrices* prev);
/* Accumulator::add_dispatch_to_command_graph (Accumulator.cpp:72-83). */
PBRT_API int pbrt_accumulator_dispatch(PbrtAccumulator* acc, pbrt_stream_t stream);
/* Public attributes accumulated_illumination (IlluminationBufferDemodulated)
 * and accumulation_buffer (Accumulator.hpp:24-25); borrowed references. */
PBRT_API int pbrt_accumulator_get_accumulated_illumination(PbrtAccumulator* acc, PbrtIlluminationBuffer** out);
PBRT_API int pbrt_accumulator_get_accumulation_buffer(PbrtAccumulator* acc, PbrtAccumulationBuffer** out);

/* ---- BMFR (source/renderModules/denoisers/BMFR.hpp:14-41) --------------
 * BMFR(width, height, work_width, work_height, g_buffer, illu_buffer,
 * acc_buffer, fitting_kernel = 256). illumination must be Demodulated or
 * DemodulatedFloat (BMFR.cpp:58-63; here: an error instead of a silent
 * half-built object). work sizes 8, 16 or 32 (square). */
PBRT_API int pbrt_bmfr_create(uint32_t width, uint32_t height, uint32_t work_width, uint32_t work_height,
                              PbrtGBuffer* g, PbrtIlluminationBuffer* illumination, PbrtAccumulationBuffer* acc,
                              uint32_t fitting_kernel, PbrtBMFR** out);
/* POSITION_TYPE specialisation constant (shaders/bmfrGeneral.comp:30-31;
 * BMFR.cpp never sets it, so the reference runs 0 = screen xy + block-
 * normalised depth). fp64_resolve = 1 re-solves, in FP64, every block whose
 * R-factor diagonal ratio exceeds 1e6 (no reference counterpart; 0 keeps
 * the reference's FP32 result). */
PBRT_API int pbrt_bmfr_set_options(PbrtBMFR* b, int32_t position_type, int32_t fp64_resolve);
/* BMFR::add_dispatch_to_command_graph (BMFR.cpp:203-230): the three
 * dispatches bmfrPre -> bmfrFit -> bmfrPost, fused here into one kernel per
 * 32x32 (or 16x16, 8x8) block. */
PBRT_API int pbrt_bmfr_dispatch(PbrtBMFR* b, const PbrtPushConstants* pc, pbrt_stream_t stream);
/* BMFR::get_final_descriptor_image (BMFR.cpp:231-234): B8G8R8A8_UNORM. */
PBRT_API int pbrt_bmfr_final_image(const PbrtBMFR* b, PbrtImage* out);
/* Private images exposed for inspection: denoised RGBA16F x 2 layers and
 * weights R32F x 30 layers at block-grid size (BMFR.cpp:97-133). */
PBRT_API int pbrt_bmfr_images(const PbrtBMFR* b, PbrtImage* denoised, PbrtImage* weights);
/* Number of blocks re-solved in FP64 by the last dispatch (stream-ordered
 * read; synchronises the stream). */
PBRT_API int pbrt_bmfr_fp64_block_count(PbrtBMFR* b, pbrt_stream_t stream, uint32_t* count);
/* R-diagonal ratio above which a block is re-solved in FP64 (default 1e6;
 * finite, >= 1). No reference counterpart. */
PBRT_API int pbrt_bmfr_set_condition_limit(PbrtBMFR* b, float limit);
/* Of the last dispatch with fp64_resolve on: the number of blocks re-solved
 * in FP64 and the largest R-diagonal ratio max|R_ii| / min|R_ii| of any
 * block's FP32 fit (infinite for a zero or NaN diagonal). Stream-ordered
 * read; synchronises the stream. No reference counterpart. */
PBRT_API int pbrt_bmfr_condition_stats(PbrtBMFR* b, pbrt_stream_t stream, uint32_t* flagged, float* max_ratio);

/* BMFR for callers that cannot allocate device memory. No counterpart in the
 * reference. Hosts that own the device-memory budget (an engine or compositor
 * handing a plugin only its images), per-frame code that must not hit the
 * device-wide synchronisation cudaMalloc / cudaFree can cause, and code that
 * runs while its stream is being captured cannot create a PbrtBMFR (which
 * allocates its weights and output images). This entry point runs the same
 * fused BMFR kernel on images the caller provides and allocates nothing: the
 * fit's per-block weights go to a fixed array inside the library, of
 * PBRT_BMFR_NOALLOC_MAX_BLOCKS x 30 floats (1.9 MiB), which every GPU that
 * loads the library holds until the process exits. Images whose block grid
 * ((width/b + 2) x (height/b + 2) for block size b) exceeds that maximum are
 * rejected with PBRT_ERROR_INVALID_ARGUMENT: 1080p fits with 16x16 and 32x32
 * blocks (8,418 and 2,170 blocks), 4K (3840x2160) only with 32x32 blocks
 * (8,418; at 16x16 it needs 33,154), and 1080p with 8x8 blocks (33,154) does
 * not. The first call on a device (and the first after that device's
 * context changes, e.g. after cudaDeviceReset) looks up that array's device
 * address (cudaGetSymbolAddress) and sets the kernel's shared-memory limit,
 * so make that first call before any stream capture. All calls share the one
 * array: calls whose kernels can overlap on the GPU (different streams, no
 * ordering between them) race on it; order them on one stream. Nothing in
 * the array has to start at zero (each block writes its weights before
 * reading them). The FP64 re-solve is not available here.
 * Images: width x height, rows packed; denoised holds 2 RGBA16F layers (layer
 * frame & 1 is read as the previous frame, layer (frame & 1) ^ 1 written).
 * Alignment (device addresses): noisy, denoised and normal 8 bytes; depth,
 * motion, albedo and final_bgra 4 bytes; a misaligned pointer is rejected
 * with PBRT_ERROR_INVALID_ARGUMENT. */
#define PBRT_BMFR_NOALLOC_MAX_BLOCKS 16384
typedef struct PbrtBmfrNoAllocImages {
  const float* depth;    /* R32F */
  const float* normal;   /* RG32F (theta, phi) */
  const uint8_t* albedo; /* RGBA8 */
  const void* noisy;     /* RGBA16F accumulated, demodulated illumination */
  const void* motion;    /* RG16F */
  const uint8_t* spp;    /* R8_UNORM */
  void* denoised;        /* RGBA16F x 2 layers, read and written */
  uint8_t* final_bgra;   /* B8G8R8A8, written */
} PbrtBmfrNoAllocImages;
PBRT_API int pbrt_bmfr_dispatch_noalloc(uint32_t width, uint32_t height, uint32_t block_size, int32_t position_type,
                                        const PbrtBmfrNoAllocImages* images, const PbrtPushConstants* pc,
                                        pbrt_stream_t stream);

/* ---- BFR (source/renderModules/denoisers/BFR.hpp:8-45) ----------------- */
PBRT_API int pbrt_bfr_create(uint32_t width, uint32_t height, uint32_t work_width, uint32_t work_height,
                             PbrtGBuffer* g, PbrtIlluminationBuffer* illumination, PbrtAccumulationBuffer* acc,
                             PbrtBFR** out);
/* BFR::add_dispatch_to_command_graph (BFR.cpp:128-138). */
PBRT_API int pbrt_bfr_dispatch(PbrtBFR* b, const PbrtPushConstants* pc, pbrt_stream_t stream);
PBRT_API int pbrt_bfr_final_image(const PbrtBFR* b, PbrtImage* out);
PBRT_API int pbrt_bfr_images(const PbrtBFR* b, PbrtImage* denoised);

/* ---- Scene (RayTracingSceneDescriptorCreationVisitor output) -----------
 * The shader-side data model of source/scene/RayTracingVisitor.{hpp,cpp}:
 * non-interleaved per-mesh positions / normals / uvs and u16 or u32 indices
 * (RayTracingVisitor.cpp:29-168), ObjectInstance (ptStructures.glsl:10-15,
 * RayTracingVisitor.hpp:37-43), WaveFrontMaterialPacked per mesh
 * (RayTracingVisitor.hpp:44-53), vsg::Light::PackedLight
 * (external/vsg/include/vsg/nodes/Light.h:23-37), five texture slots per
 * mesh (diffuse, mr, normal, emissive, specular; RGBA8, bilinear, REPEAT,
 * level 0) and the per-instance opacity flags PBRTPipeline::set_tlas reads
 * (PBRTPipeline.cpp:38-56). pbrt_scene_create replaces the visitor's
 * descriptor upload plus BuildAccelerationStructureTraversal: it flattens the
 * instances to world-space triangles and builds the 8-wide BVH. */
typedef struct PbrtMeshDesc {
  const float* positions; /* 3 per vertex */
  const float* normals;   /* 3 per vertex */
  const float* uvs;       /* 2 per vertex */
  uint32_t vertex_count;
  const void* indices; /* uint16 (index_stride 2) or uint32 (4) */
  uint32_t index_count;
  uint32_t index_stride;
} PbrtMeshDesc;
typedef struct PbrtObjectInstance {
  float object_mat[16]; /* column major */
  int32_t mesh_id;
  uint32_t index_stride;
  int32_t pad[2];
} PbrtObjectInstance;
typedef struct PbrtMaterialPacked {
  float ambient_roughness[4];
  float diffuse_ior[4];
  float specular_dissolve[4];
  float transmittance_illum[4];
  float emission_texture_id[4];
  uint32_t category_id;
  float pad[3];
} PbrtMaterialPacked;
typedef struct PbrtPackedLight {
  float v0[3];
  float type; /* 1 directional, 2 point, 5 area triangle */
  float v1[3];
  float radius;
  float v2[3];
  float angle;
  float dir[3];
  float angle2;
  float color_ambient[4];
  float color_diffuse[4];
  float color_specular[4];
  float strengths[3]; /* attenuation 1 / (x + y d + z d^2) */
  float inclusive_strength;
} PbrtPackedLight;
typedef struct PbrtTextureDesc {
  const uint8_t* rgba8;
  uint32_t width, height;
} PbrtTextureDesc;
typedef struct PbrtSceneDesc {
  uint32_t mesh_count;
  const PbrtMeshDesc* meshes;
  uint32_t instance_count;
  const PbrtObjectInstance* instances;
  const uint8_t* instance_opaque; /* NULL = all opaque */
  const PbrtMaterialPacked* materials; /* mesh_count entries, indexed by mesh id */
  uint32_t light_count;
  const PbrtPackedLight* lights;
  uint32_t texture_count; /* entry 0 should be the 1x1 white default */
  const PbrtTextureDesc* textures;
  const int32_t* mesh_textures; /* mesh_count x 5 texture indices */
} PbrtSceneDesc;
typedef struct PbrtSceneInfo {
  uint32_t triangle_count, instance_count, bvh_nodes, bvh_depth, light_count;
  uint64_t bvh_bytes, triangle_bytes;
  double build_ms;
} PbrtSceneInfo;
PBRT_API int pbrt_scene_create(const PbrtSceneDesc* desc, PbrtScene** out);
/* The build's speed-for-quality trade, as Vulkan's acceleration-structure
 * build flags offer it (VK_BUILD_ACCELERATION_STRUCTURE_PREFER_FAST_TRACE_BIT_KHR
 * / _PREFER_FAST_BUILD_BIT_KHR; the reference builds with vsg's defaults,
 * VulkanPBRT.cpp:365-367). FAST_TRACE (what pbrt_scene_create does): binned
 * SAH on the host, collapsed SAH-optimally to 8-wide nodes. FAST_BUILD: a
 * linear BVH (Morton order) built on the device and collapsed greedily;
 * lower quality, for scenes rendered few times. Hits, and so frames, are
 * identical under either build. */
enum { PBRT_BUILD_PREFER_FAST_TRACE = 0, PBRT_BUILD_PREFER_FAST_BUILD = 1 };
PBRT_API int pbrt_scene_create_ex(const PbrtSceneDesc* desc, uint32_t build_flags, PbrtScene** out);
/* Mesh preparation the visitor applies before it hands a mesh on
 * (RayTracingVisitor.cpp:52-127, 133-166), host side: area-weighted running
 * average of face normals into normals[3 * vertex_count] (not normalised,
 * as there; the visitor does this when the mesh's first normal is zero),
 * and texture coordinates (0,0), (0,1), (1,0) per triangle corner, later
 * triangles overwriting earlier ones, into uvs[2 * vertex_count] (when the
 * mesh has none). index_stride: 2 (uint16) or 4 (uint32). */
PBRT_API int pbrt_mesh_generate_normals(const float* positions, uint32_t vertex_count, const void* indices,
                                        uint32_t index_count, uint32_t index_stride, float* normals);
PBRT_API int pbrt_mesh_fill_uvs(uint32_t vertex_count, const void* indices, uint32_t index_count,
                                uint32_t index_stride, float* uvs);
PBRT_API int pbrt_scene_info(const PbrtScene* scene, PbrtSceneInfo* info);
/* Ray queries against the scene (no reference counterpart; the path tracer's
 * traversal exposed for tests and throughput measurement). Device arrays of n
 * float4 (origin, tmin) and (direction, tmax); hits_out float4 per ray
 * (t, u, v, triangle key bits -- the instance-major flat triangle index, or
 * 0xffffffff on a miss). scratch_u32x2: 8 bytes of device memory. */
PBRT_API int pbrt_scene_trace_rays(PbrtScene* scene, const void* origins_tmin, const void* directions_tmax, uint32_t n,
                                   int32_t any_hit, void* hits_out, void* scratch_u32x2, pbrt_stream_t stream);

/* ---- PBRTPipeline (source/renderModules/PBRTPipeline.hpp:19-60) ---------
 * PBRTPipeline(scene, g_buffer, illumination_buffer, write_g_buffer, ...):
 * illumination DemodulatedFloat selects DEMOD_ILLUMINATION_FLOAT, FinalFloat
 * selects FINAL_IMAGE (PBRTPipeline.cpp:171-229). Defaults follow the
 * reference: max recursion depth 2, min 0, surface-strength light sampling
 * (uniform above 800 lights, PBRTPipeline.cpp:92-96). */
PBRT_API int pbrt_pipeline_create(PbrtScene* scene, PbrtGBuffer* g, PbrtIlluminationBuffer* illumination,
                                  int32_t write_g_buffer, PbrtPipeline** out);
/* light_sampling: 0 SAMPLE_SURFACE_STRENGTH, 1 SAMPLE_LIGHT_STRENGTH,
 * 2 SAMPLE_UNIFORM (PBRTPipeline.hpp:32-37); the Infos UBO's
 * minRecursionDepth / maxRecursionDepth (layoutPTUniform.glsl:4-9). */
PBRT_API int pbrt_pipeline_set_config(PbrtPipeline* p, int32_t light_sampling, int32_t min_recursion_depth,
                                      int32_t max_recursion_depth);
/* PBRTPipeline::add_trace_rays_to_command_graph (PBRTPipeline.cpp:65-80):
 * one sample per pixel into the illumination (and G-) buffer. The frame's
 * launches are captured into a CUDA graph on first use. */
PBRT_API int pbrt_pipeline_trace(PbrtPipeline* p, const PbrtPushConstants* pc, pbrt_stream_t stream);
typedef struct PbrtTraceStats {
  uint64_t frames, primary_rays, extension_rays, shadow_rays;
  uint32_t error_flags; /* bit 0: a traversal ran out of stack */
} PbrtTraceStats;
/* BVH queries issued since creation / the last reset (stream-synchronising). */
PBRT_API int pbrt_pipeline_stats(PbrtPipeline* p, pbrt_stream_t stream, PbrtTraceStats* out);
PBRT_API int pbrt_pipeline_reset_stats(PbrtPipeline* p, pbrt_stream_t stream);
/* One frame launched stage by stage with CUDA events around every launch
 * (no graph), for per-kernel timing; counts BVH work. No reference
 * counterpart (the reference writes two timestamps it never reads,
 * source/VulkanPBRT.cpp:397-408). */
typedef struct PbrtStageTimes {
  float raygen_ms, trace_closest_ms, shade_ms, trace_shadow_ms, finalize_ms;
  uint64_t closest_rays, shadow_rays;
  uint64_t closest_nodes, closest_tris, shadow_nodes, shadow_tris; /* node / triangle visits */
  uint32_t closest_launches;
} PbrtStageTimes;
PBRT_API int pbrt_pipeline_profile(PbrtPipeline* p, const PbrtPushConstants* pc, pbrt_stream_t stream,
                                   PbrtStageTimes* out);
/* Launch shape of the tracer: persistent traversal CTAs and shading CTAs per
 * SM (1..16 each; default 8 and 8). No reference counterpart. */
PBRT_API int pbrt_pipeline_set_launch(PbrtPipeline* p, int32_t trace_blocks_per_sm, int32_t shade_blocks_per_sm);
/* Frame schedule (no reference counterpart; the results are the same either
 * way). sort_rays = 1: extension and shadow rays are reordered by direction
 * octant and origin cell (a counting sort on the GPU) before they are
 * traversed; its staging queues are allocated on first use. merge_shadow =
 * 1 (default): bounce k's closest-hit rays and bounce k-1's shadow rays are
 * traced in one launch; 0: one launch per queue. The frame graph is
 * recaptured on the next trace after a change. */
PBRT_API int pbrt_pipeline_set_schedule(PbrtPipeline* p, int32_t sort_rays, int32_t merge_shadow);

/* ---- batched requests (no reference counterpart) -----------------------
 * Many independent renders in one CUDA graph launch: each request names its
 * own pipeline (scene, resolution, depth, G-buffer, illumination buffer),
 * renders spp frames from pc (frame numbers pc.frame_number ...
 * pc.frame_number + spp - 1) and, optionally, accumulates them with its
 * accumulator (static camera: `camera` for both current and previous) and
 * denoises the result with its BMFR. Requests run as `branches` concurrent
 * chains, assigned longest first to the least loaded chain. A pipeline may
 * appear in one request of a batch only. */
typedef struct PbrtBatchRequest {
  PbrtPipeline* pipeline;
  PbrtAccumulator* accumulator; /* optional */
  PbrtBMFR* bmfr;               /* optional; reads the accumulator's output */
  PbrtPushConstants pc;
  PbrtCameraMatrices camera;    /* with proj, when accumulated */
  uint32_t spp;
} PbrtBatchRequest;
typedef struct PbrtBatchTuning {
  uint32_t branches;            /* concurrent chains (1..64) */
  uint32_t trace_blocks_per_sm; /* persistent traversal CTAs per SM */
  uint32_t shade_blocks_per_sm;
  uint32_t order;               /* 0: as added, 1: longest first */
} PbrtBatchTuning;
PBRT_API int pbrt_batch_create(PbrtBatch** out);
PBRT_API int pbrt_batch_add(PbrtBatch* b, const PbrtBatchRequest* request);
PBRT_API int pbrt_batch_size(const PbrtBatch* b, uint32_t* count);
PBRT_API int pbrt_batch_set_tuning(PbrtBatch* b, const PbrtBatchTuning* tuning);
PBRT_API int pbrt_batch_get_tuning(const PbrtBatch* b, PbrtBatchTuning* tuning);
/* One graph launch of every request (captured on first use or after a change). */
PBRT_API int pbrt_batch_submit(PbrtBatch* b, pbrt_stream_t stream);
/* Times each candidate tuning on this batch (median of `repeats` launches
 * after one warm-up) and keeps the fastest (stream-synchronising). */
PBRT_API int pbrt_batch_autotune(PbrtBatch* b, pbrt_stream_t stream, int32_t repeats, PbrtBatchTuning* best,
                                 float* best_ms);
/* The chain assignment the batch uses (host only): assign[i] in
 * 0..branches-1 for request costs[i]; order 1 = longest first onto the least
 * loaded chain, 0 = in the given order. */
PBRT_API int pbrt_batch_plan(const double* costs, uint32_t n, uint32_t branches, uint32_t order, uint32_t* assign);

/* Failure handling without a GPU fault (no reference counterpart; the
 * reference has none). abort_flag: a pinned host word mapped into the
 * device; writing nonzero makes frames in flight and later frames stop
 * taking rays (checked every 64 warp batches) and shade nothing, until the
 * host writes 0. set_budget: a frame whose traversal runs longer than
 * budget_ns (0 = no budget, the default) stops the same way. status
 * (stream-synchronising) gives PBRT_ERROR_ABORTED or PBRT_ERROR_TIMEOUT for a
 * stopped frame since the last call, else PBRT_OK, and clears it; the
 * pipeline stays usable. */
PBRT_API int pbrt_pipeline_abort_flag(PbrtPipeline* p, uint32_t** host_flag);
PBRT_API int pbrt_pipeline_set_budget(PbrtPipeline* p, uint64_t budget_ns);
PBRT_API int pbrt_pipeline_status(PbrtPipeline* p, pbrt_stream_t stream, int32_t* frame_status);
/* R32_UINT per pixel: key of the primary ray's closest triangle (see
 * pbrt_scene_trace_rays), 0xffffffff on a miss. */
PBRT_API int pbrt_pipeline_debug_images(const PbrtPipeline* p, PbrtImage* primary_hit_key);

/* ---- Taa (source/renderModules/Taa.hpp:9-35) ----------------------------
 * Taa(width, height, work_width, work_height, g_buffer, acc_buffer, denoised)
 * (Taa.cpp:4-91): denoised is the denoiser's final image (packed B8G8R8A8,
 * e.g. pbrt_bmfr_final_image; it must outlive the Taa object); motion comes
 * from acc_buffer. add_dispatch_to_command_graph (Taa.cpp:111-120) ->
 * pbrt_taa_dispatch (frame_number from the push constants; the history copy
 * of Taa.cpp:121-159 is part of the dispatch); get_final_descriptor_image ->
 * pbrt_taa_final_image (B8G8R8A8). */
PBRT_API int pbrt_taa_create(uint32_t width, uint32_t height, uint32_t work_width, uint32_t work_height,
                             PbrtGBuffer* g_buffer, PbrtAccumulationBuffer* acc_buffer, const PbrtImage* denoised,
                             PbrtTaa** out);
PBRT_API int pbrt_taa_dispatch(PbrtTaa* taa, const PbrtPushConstants* pc, pbrt_stream_t stream);
PBRT_API int pbrt_taa_final_image(const PbrtTaa* taa, PbrtImage* out);
/* ---- BFRBlender (source/renderModules/denoisers/BFRBlender.hpp:6-27) ----
 * BFRBlender(width, height, average_image, average_squared_image, denoised0,
 * denoised1, denoised2, work_width = 16, work_height = 16, filter_radius = 2)
 * (BFRBlender.cpp:5-70, shaders/bfrBlender.comp): blends the 8x8, 16x16 and
 * 32x32 denoisers' final images (denoised0/1/2: packed 8-bit RGBA or BGRA,
 * blended byte for byte) by the local standard deviation of the average
 * image's luminance. average / average_squared: RGBA16F (the accumulated
 * IlluminationBufferDemodulated's images 0 and 1) or RGBA32F. The images
 * must outlive the blender. add_dispatch_to_command_graph
 * (BFRBlender.cpp:84-91) -> pbrt_bfr_blender_dispatch;
 * get_final_descriptor_image -> pbrt_bfr_blender_final_image (B8G8R8A8). */
PBRT_API int pbrt_bfr_blender_create(uint32_t width, uint32_t height, const PbrtImage* average_image,
                                     const PbrtImage* average_squared_image, const PbrtImage* denoised0,
                                     const PbrtImage* denoised1, const PbrtImage* denoised2, uint32_t work_width,
                                     uint32_t work_height, uint32_t filter_radius, PbrtBFRBlender** out);
PBRT_API int pbrt_bfr_blender_dispatch(PbrtBFRBlender* blender, pbrt_stream_t stream);
PBRT_API int pbrt_bfr_blender_final_image(const PbrtBFRBlender* blender, PbrtImage* out);
/* FormatConverter (source/renderModules/FormatConverter.hpp,
 * shaders/formatConverter.comp:9-13): dst = src texel by texel, src
 * RGBA32F / RGBA16F / RGBA8 / BGRA8, dst RGBA32F / RGBA8 / BGRA8 (UNORM
 * stores clamp and round); same size. */
PBRT_API int pbrt_format_convert(const PbrtImage* src, const PbrtImage* dst, pbrt_stream_t stream);

/* ---- kernel-predicting denoiser operators (no reference counterpart) ----
 * Device pointers, NHWC layout, channel counts multiples of 16 for the
 * convolutions. BF16 activations and weights, FP32 accumulation, FP32
 * gradients and master weights. The network that strings them together is
 * vulkanpbrt_gb300/kpunet.py. */
/* y = relu?(conv3x3(concat(x1, upsample2(x2))) + bias), zero padding.
 * w [cout][9][c1+c2] BF16 (tap = ky*3+kx); x2 may be null (c2 = 0).
 * flags bit 0: ReLU; bit 1: add into y32 instead of storing; bit 2: the
 * per-(tap, 16-channel) pipelined kernel; bit 3: no 16 x 16-tile kernel for
 * cout <= 48 (kernel choice only, same result). y (BF16) and y32 (FP32) are
 * both optional, at least one is given. */
PBRT_API int pbrt_nn_conv3x3(const void* x1, int32_t c1, const void* x2, int32_t c2, const void* w, const float* bias,
                             void* y, float* y32, int32_t n, int32_t h, int32_t w_px, int32_t cout, int32_t flags,
                             pbrt_stream_t stream);
/* FP8 (e4m3) variant for inference: w8 [cout][9][c1+c2] e4m3 with per-output-
 * channel scales wscale and the per-input-channel activation scales folded
 * in (pbrt_nn_quantize_weights_fp8); BF16 inputs are quantised on load with
 * inv_xscale [c1+c2] (saturating); c1 + c2 <= 256; flags bit 0: ReLU,
 * bit 3: the mma.sync kernel only (default: pbrt_nn_conv3x3_fp8_umma where
 * it applies, this kernel otherwise), bit 4: see pbrt_nn_conv3x3_umma. */
PBRT_API int pbrt_nn_conv3x3_fp8(const void* x1, int32_t c1, const void* x2, int32_t c2, const void* w8,
                                 const float* wscale, const float* inv_xscale, const float* bias, void* y, int32_t n,
                                 int32_t h, int32_t w_px, int32_t cout, int32_t flags, pbrt_stream_t stream);
/* tcgen05 variant (5th-generation tensor cores, accumulator in tensor
 * memory): BF16 output only, cout in {16, 32, ..., 128}, flags bit 0 ReLU,
 * bit 1: the per-tile kernel only, bit 2: no TMA, bit 3: the single-role
 * persistent kernel, bit 4: the upsampled second input gathered with
 * cp.async (default: its half-resolution box by TMA, expanded in shared
 * memory, where two stages of it fit), bit 5: the first input's halo as
 * 8-channel planes (default for a single input of 16 or 32 channels and
 * cout 32 or 48: whole pixels by one swizzled TMA row each). */
PBRT_API int pbrt_nn_conv3x3_umma(const void* x1, int32_t c1, const void* x2, int32_t c2, const void* w,
                                  const float* bias, void* y, int32_t n, int32_t h, int32_t w_px, int32_t cout,
                                  int32_t flags, pbrt_stream_t stream);
/* The warp-specialised tcgen05 convolution of a single input (x1, c1) that
 * also writes the 2x2 average pooling of its BF16 output y into pooled
 * ([n][h/2][wd/2][cout], the same bits as pbrt_nn_avgpool2 of y): the
 * encoder's pooling fused into the producing convolution's epilogue. Needs
 * h % 16 == 0 and wd % 8 == 0 (else PBRT_ERROR_UNSUPPORTED). flags bit 0:
 * ReLU, bit 5: as pbrt_nn_conv3x3_umma. */
PBRT_API int pbrt_nn_conv3x3_umma_pooled(const void* x1, int32_t c1, const void* w, const float* bias, void* y,
                                         void* pooled, int32_t n, int32_t h, int32_t wd, int32_t cout, int32_t flags,
                                         pbrt_stream_t stream);
/* Backward weights on tcgen05: the arguments of pbrt_nn_conv3x3_wgrad (dw
 * [cout][9][c1+c2] FP32, added to), cout <= 128, c1 + c2 <= 256, 16-byte
 * aligned inputs. A CTA walks 8x8-pixel tiles for a group of taps: dY's tile
 * and the input's 10x10 halo (by TMA; the upsampled second input gathered)
 * are the MMA's MN-major operands as stored, each tap a shift of the halo
 * descriptor, the sums in tensor memory, then atomics into dw.
 * PBRT_ERROR_UNSUPPORTED when the tensor maps cannot be made. */
PBRT_API int pbrt_nn_conv3x3_wgrad_umma(const void* dy, const void* x1, int32_t c1, const void* x2, int32_t c2,
                                        float* dw, int32_t n, int32_t h, int32_t w_px, int32_t cout,
                                        pbrt_stream_t stream);
/* tcgen05 convolution of a single input with an FP32 output y32
 * [n][h][wd][cout] (16-byte aligned operands): the backward-data pass of
 * training (dY with pbrt_nn_flip_weights' weights). Any cout that is a
 * multiple of 16: the output channels run in slices whose weights fit in
 * shared memory, one launch a slice. flags bit 0: ReLU, bit 2: no TMA.
 * PBRT_ERROR_UNSUPPORTED when no slice fits (c1 too large). */
PBRT_API int pbrt_nn_conv3x3_umma_f32(const void* x1, int32_t c1, const void* w, const float* bias, float* y32,
                                      int32_t n, int32_t h, int32_t wd, int32_t cout, int32_t flags,
                                      pbrt_stream_t stream);
/* The FP8 convolution on the tcgen05 tensor cores (kind::f8f6f4, K = 32 per
 * instruction): the arguments and quantisation of pbrt_nn_conv3x3_fp8, cout
 * in {16, 32, ..., 128}, plus an optional pooled output as in
 * pbrt_nn_conv3x3_umma_pooled (x2 must then be NULL). PBRT_ERROR_UNSUPPORTED
 * when the weights and two input stages do not fit in shared memory, an
 * operand is not 16-byte aligned, or (pooled) h % 16 or wd % 8 is not 0. */
PBRT_API int pbrt_nn_conv3x3_fp8_umma(const void* x1, int32_t c1, const void* x2, int32_t c2, const void* w8,
                                      const float* wscale, const float* inv_xscale, const float* bias, void* y,
                                      void* pooled, int32_t n, int32_t h, int32_t w_px, int32_t cout, int32_t flags,
                                      pbrt_stream_t stream);
/* Error flags of the tcgen05 kernels since the last call (bit 0: a bounded
 * wait timed out), reset on read (stream-synchronising). */
PBRT_API int pbrt_nn_umma_status(pbrt_stream_t stream, uint32_t* flags);
/* wscale[co] = max |w x xscale| / 448 over the channel, w8 = e4m3(w x xscale / wscale). */
PBRT_API int pbrt_nn_quantize_weights_fp8(const float* w, const float* xscale, int32_t cout, int32_t cin, void* w8,
                                          float* wscale, pbrt_stream_t stream);
/* amax[c] = max(amax[c], max over pixels |x[p][c]|), x BF16 [pixels][c]. */
PBRT_API int pbrt_nn_channel_amax(const void* x, int64_t pixels, int32_t c, float* amax, pbrt_stream_t stream);
/* dw [cout][9][c1+c2] FP32 += sum over pixels of dy (BF16) x im2col(input). */
PBRT_API int pbrt_nn_conv3x3_wgrad(const void* dy, const void* x1, int32_t c1, const void* x2, int32_t c2, float* dw,
                                   int32_t n, int32_t h, int32_t w_px, int32_t cout, pbrt_stream_t stream);
/* [cout][9][cin] -> [cin][9][cout], taps reversed (backward-data weights). */
PBRT_API int pbrt_nn_flip_weights(const void* w, void* wt, int32_t cout, int32_t cin, pbrt_stream_t stream);
/* Network input: 16 BF16 channels per padded pixel (log1p radiance, albedo,
 * normal, log1p depth / 8, min(spp, 16) / 16, zeros; edges replicated) and
 * the radiance the heads filter (FP32 rgb, clamped to [0, 10]) from an
 * illumination image (RGBA32F, or RGBA16F when illum_is_half), the
 * G-buffer's albedo (RGBA8), normal (RG32F angles) and depth (R32F) images
 * and, optionally, the accumulation buffer's spp image (R8, 1/256 steps;
 * null = one sample); n_img images of w x h each, packed. */
PBRT_API int pbrt_nn_features(const void* illum, int32_t illum_is_half, const void* albedo, const void* normal,
                              const void* depth, const void* spp, int32_t w, int32_t h, int32_t pw, int32_t ph,
                              int32_t n_img, void* feat, float* rad, pbrt_stream_t stream);
/* 2x2 average pooling (BF16 when is_f32 = 0, else FP32) and its backward (adds). */
PBRT_API int pbrt_nn_avgpool2(const void* x, void* y, int32_t is_f32, int32_t n, int32_t h, int32_t w, int32_t c,
                              pbrt_stream_t stream);
PBRT_API int pbrt_nn_avgpool2_bwd_add(const float* dy, float* dx, int32_t n, int32_t h, int32_t w, int32_t c,
                                      pbrt_stream_t stream);
/* out = BF16(dy * (y > 0)); db (optional) += per-channel sums of out. */
PBRT_API int pbrt_nn_relu_bwd(const float* dy, const void* y, void* out, float* db, int64_t pixels, int32_t c,
                              pbrt_stream_t stream);
/* Backward of concat(x1, upsample2(x2)): dx1 += dcat[:c1], dx2 += 2x2 sums of dcat[c1:]. */
PBRT_API int pbrt_nn_split_upsum(const float* dcat, int32_t c1, int32_t c2, int32_t n, int32_t h, int32_t w,
                                 float* dx1, float* dx2, pbrt_stream_t stream);
/* Kernel-prediction head: logits = Wh . F + bh (k = 25, 26 or 27 outputs);
 * softmax 5x5 kernel over R; with coarse, alpha = sigmoid(logit 25) blends
 * the upsampled coarse result in; the last logit (k = 26 without coarse,
 * 27 with) is the predicted log squared error written to var. */
PBRT_API int pbrt_nn_kp_head(const void* F, const float* Wh, const float* bh, const float* R, const float* coarse,
                             float* out, float* kw, float* filt, float* alpha, float* var, int32_t n, int32_t h,
                             int32_t w, int32_t c, int32_t k, pbrt_stream_t stream);
PBRT_API int pbrt_nn_kp_head_bwd(const void* F, const float* Wh, const float* bh, const float* R, const float* coarse,
                                 float* kw, float* filt, float* alpha, int32_t n, int32_t h, int32_t w, int32_t c,
                                 int32_t k, const float* dout, const float* dvar, float* dF, float* dWh, float* dbh,
                                 float* dcoarse, pbrt_stream_t stream);
/* relMSE of albedo x out against albedo x target over the unpadded w x h
 * pixels, its gradient, and the variance head's regression on the
 * per-pixel error; loss[0] += relMSE, loss[1] += variance loss. */
PBRT_API int pbrt_nn_relmse_loss(const float* out, const float* target, const void* albedo, const float* var,
                                 int32_t n, int32_t ph, int32_t pw, int32_t h, int32_t w, float var_weight, float* dout,
                                 float* dvar, float* loss, pbrt_stream_t stream);
/* Adam step on FP32 master weights (bias-corrected for step >= 1); refreshes
 * the BF16 copy when w_bf16 is given. */
PBRT_API int pbrt_nn_adam(float* w, const float* g, float* m, float* v, void* w_bf16, int64_t n, float lr, float b1,
                          float b2, float eps, int32_t step, float grad_scale, pbrt_stream_t stream);
/* Variance gate: mask[t] = 1 for every tile x tile block (row-major tiles
 * over w x h) whose mean predicted relative squared error exp(var) exceeds
 * threshold; count += the number of such tiles. */
PBRT_API int pbrt_nn_gate(const float* var, int32_t pw, int32_t w, int32_t h, float threshold, int32_t tile,
                          uint8_t* mask, uint32_t* count, pbrt_stream_t stream);
/* Learned tile gate (no reference counterpart): per tile, eight features
 * (log of: the mean predicted relative squared error exp(var), the mean
 * squared difference between final_bgra -- the network's composed final
 * image -- and bmfr_final_bgra in [0,1] units, the mean spp byte, the
 * variance of log(1 + luminance) of the noisy input, the mean |d log depth|
 * (forward differences), 1 - |mean normal|, the mean noisy luminance, the
 * mean albedo) give four predictions coef[9c + 8] + sum_k coef[9c + k] *
 * feature[k] of the change in relative squared error from showing alpha *
 * network + (1 - alpha) * BMFR, alpha = 0.75, 0.5, 0.25, 0 (c = 0..3); the
 * tile takes the lowest prediction below zero, else the network alone.
 * mask: 0 network, 1..4 the chosen alpha; count: tiles with alpha < 1. In
 * those tiles denoised_rgba32f gets the blend of nn_out (padded rows of pw
 * pixels, 3 floats each) and BMFR's denoised layer *bmfr_layer (RGBA16F,
 * two layers of w x h), and final_bgra its remodulated, tone-mapped value
 * (alpha 0: bmfr_final_bgra's pixels). noisy: RGBA16F (noisy_is_half) or
 * RGBA32F; spp may be NULL. */
PBRT_API int pbrt_nn_gate_model(const float* var, const float* nn_out, int32_t pw, int32_t w, int32_t h,
                                int32_t tile, const void* bmfr_final_bgra, const void* bmfr_denoised,
                                const uint32_t* bmfr_layer, const uint8_t* spp, const void* noisy,
                                int32_t noisy_is_half, const float* depth, const void* normal, const void* albedo,
                                const float* coef, uint8_t* mask, uint32_t* count, void* final_bgra,
                                float* denoised_rgba32f, pbrt_stream_t s);
/* Final image of the neural path, tone-mapped as BMFR's final image; pixels
 * of masked tiles copy fallback_bgra (BMFR's final image). denoised_rgba32f
 * (optional) always receives the network's output. */
PBRT_API int pbrt_nn_compose(const float* out, int32_t pw, int32_t w, int32_t h, const void* albedo,
                             const uint8_t* mask, int32_t tile, const void* fallback_bgra, void* final_bgra,
                             float* denoised_rgba32f, pbrt_stream_t stream);

/* ---- neural denoiser render module (no reference counterpart) ---------
 * Reads the G-buffer and the demodulated illumination image of
 * `illumination` (RGBA32F or RGBA16F: one sample, or the accumulator's
 * output) and writes a denoised RGBA32F image and
 * a B8G8R8A8 final image tone-mapped as BMFR's. Parameters: the flat FP32
 * vector of vulkanpbrt_gb300/kpunet.py (convolution weights [cout][9][cin]
 * in layer order, convolution biases, then per head weights [k][c] and
 * biases), pbrt_neural_param_count floats. The forward pass is captured in
 * a CUDA graph on the first dispatch. */
PBRT_API int pbrt_neural_param_count(int64_t* count);
/* acc (optional): the accumulation buffer whose spp image counts the samples
 * behind `illumination` (the accumulator's output); null for 1-spp input. */
PBRT_API int pbrt_neural_create(uint32_t width, uint32_t height, PbrtGBuffer* gbuffer,
                                PbrtIlluminationBuffer* illumination, PbrtAccumulationBuffer* acc,
                                const float* params_host, int64_t count, PbrtNeural** out);
PBRT_API int pbrt_neural_set_params(PbrtNeural* nd, const float* params_host, int64_t count);
/* Variance gate: with bmfr given, every tile x tile block whose mean predicted
 * per-pixel relative squared error exceeds threshold shows BMFR's final image
 * in the final image (the denoised image keeps the network's output)
 * (bmfr must be dispatched before the neural module each frame); null bmfr
 * turns the gate off. */
PBRT_API int pbrt_neural_set_fallback(PbrtNeural* nd, PbrtBMFR* bmfr, float threshold, int32_t tile);
/* Learned tile gate in place of the threshold (no reference counterpart):
 * coef = the 4 x 9 coefficients of the predictions pbrt_nn_gate_model
 * describes (fitted offline; vulkanpbrt_gb300/weights/gate.json), n = 36;
 * tiles show alpha * network + (1 - alpha) * BMFR with the alpha in {1,
 * 0.75, 0.5, 0.25, 0} predicted best, in the final and the denoised images.
 * NULL returns to the threshold rule. Needs a fallback BMFR
 * (pbrt_neural_set_fallback), dispatched before the neural module. */
PBRT_API int pbrt_neural_set_gate_model(PbrtNeural* nd, const float* coef, int32_t n);
/* FP8 inference: calibrate runs one BF16 pass on the current inputs
 * (stream-synchronising) and derives per-input-channel activation scales
 * (max |x| / 448) and per-output-channel e4m3 weights, then times every
 * convolution but the first (16 input channels, which stays BF16) in BF16
 * and in e4m3 on those activations and marks the layers where e4m3 is
 * faster; set_precision(8) then runs the marked layers as e4m3 x e4m3 ->
 * FP32 on the tensor cores (tcgen05 kind::f8f6f4 where the layer fits in
 * shared memory, mma.sync otherwise), with the encoder's pooling fused as
 * in BF16, and the others in BF16; set_precision(16) returns to BF16. New
 * parameters drop the calibration. fp8_layers reads the marks (18 entries,
 * layer order of vulkanpbrt_gb300/kpunet.py), set_fp8_layers fixes them
 * (entry 0 must be 0). */
PBRT_API int pbrt_neural_calibrate(PbrtNeural* nd, pbrt_stream_t stream);
PBRT_API int pbrt_neural_set_precision(PbrtNeural* nd, int32_t bits);
PBRT_API int pbrt_neural_fp8_layers(const PbrtNeural* nd, int32_t* mask, int32_t count);
PBRT_API int pbrt_neural_set_fp8_layers(PbrtNeural* nd, const int32_t* mask, int32_t count);
/* Per-layer convolution kernel: 0 = warp-level mma.sync kernels, 1 =
 * tcgen05 (tensor memory, TMA; the first input's halo as swizzled pixel rows
 * for a single input of 16 or 32 channels and 32 or 48 out), 2 = tcgen05
 * with that halo as 8-channel planes (the same bits as 1). autotune (run by the first dispatch
 * when no choice was set) times them for every layer on the current inputs
 * and keeps the fastest (stream-synchronising); conv_kernels reads the choice
 * (18 entries, layer order of vulkanpbrt_gb300/kpunet.py), set_conv_kernels
 * fixes it. */
PBRT_API int pbrt_neural_autotune(PbrtNeural* nd, pbrt_stream_t stream);
PBRT_API int pbrt_neural_conv_kernels(const PbrtNeural* nd, int32_t* kinds, int32_t count);
PBRT_API int pbrt_neural_set_conv_kernels(PbrtNeural* nd, const int32_t* kinds, int32_t count);
PBRT_API int pbrt_neural_dispatch(PbrtNeural* nd, pbrt_stream_t stream);
/* The same launches without the graph (for per-kernel profiling). */
PBRT_API int pbrt_neural_dispatch_direct(PbrtNeural* nd, pbrt_stream_t stream);
PBRT_API int pbrt_neural_final_image(const PbrtNeural* nd, PbrtImage* out);
/* denoised: RGBA32F width x height; variance: R32F predicted log relative
 * squared error at the padded size (multiples of 16). */
PBRT_API int pbrt_neural_images(const PbrtNeural* nd, PbrtImage* denoised, PbrtImage* variance);
/* R8 image, one texel per gate tile (row-major): 1 where the last dispatch
 * showed the fallback; empty (data null) while the gate is off. */
PBRT_API int pbrt_neural_fallback_mask(const PbrtNeural* nd, PbrtImage* mask);
/* Tiles of the last dispatch that took the fallback (stream-synchronising). */
PBRT_API int pbrt_neural_fallback_tiles(const PbrtNeural* nd, pbrt_stream_t stream, uint32_t* count);

#ifdef __cplusplus
}
#endif
#endif /* VULKANPBRT_GB300_H */
