// Test driver for the C++ render-module layer (include/vulkanpbrt_gb300.hpp).
//
//   render_frame errors
//       host-only checks: reference counting of ref_ptr, and construction
//       errors surfacing as vkpbrt::Exception with the library's message
//       (no GPU needed: a null handle is rejected before any CUDA call).
//   render_frame frame SCENE FRAMES OUT_PREFIX
//       builds the scene written by the Python test (SCENE, format below),
//       records the reference's per-frame command graph once -- trace,
//       accumulate, BMFR 32x32, copy to the back images
//       (source/VulkanPBRT.cpp:397-445) -- and submits it for every frame
//       record in FRAMES (PbrtPushConstants + current and previous
//       PbrtCameraMatrices), then writes the last frame's illumination
//       (RGBA32F) and BMFR final image (BGRA8) to OUT_PREFIX.{illum,final}.
//
// Scene file: "PBRTSCN1", u32 mesh count, per mesh u32 vertex count, u32
// index count, u32 index stride, positions, normals, uvs, indices (padded to
// 4 bytes); u32 instance count, PbrtObjectInstance[], u8 opaque[] (padded to
// 4 bytes); PbrtMaterialPacked[mesh count]; u32 light count,
// PbrtPackedLight[]; u32 texture count, per texture u32 width, u32 height,
// RGBA8 texels; i32 mesh_textures[5 * mesh count]; u32 max depth, u32 min depth.
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iterator>
#include <stdexcept>
#include <vector>

#include "vulkanpbrt_gb300.hpp"

namespace {

struct Reader {
  std::vector<char> buf;
  size_t at = 0;
  explicit Reader(const char* path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error(std::string("cannot open ") + path);
    buf.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
  }
  const char* take(size_t n) {
    if (at + n > buf.size()) throw std::runtime_error("truncated file");
    const char* p = buf.data() + at;
    at += n;
    return p;
  }
  uint32_t u32() {
    uint32_t v;
    std::memcpy(&v, take(4), 4);
    return v;
  }
  void align4() { at = (at + 3) & ~size_t(3); }
};

int fail(const char* what) {
  std::fprintf(stderr, "FAIL %s\n", what);
  return 1;
}

int errors() {
  using namespace vkpbrt;
  // reference counting
  ref_ptr<Commands> cmds = Commands::create();
  if (cmds->referenceCount() != 1) return fail("create -> one reference");
  {
    ref_ptr<Commands> other = cmds;
    if (cmds->referenceCount() != 2) return fail("copy -> two references");
  }
  if (cmds->referenceCount() != 1) return fail("scope exit -> one reference");
  ref_ptr<PushConstants> pc = PushConstants::create();
  pc->value.frame_number = 7;
  int recorded = 0;
  cmds->addChild([&recorded, pc](pbrt_stream_t) { recorded += (int)pc->value.frame_number; });
  cmds->submit();
  pc->value.frame_number = 9;  // commands read the value current at submit time
  cmds->submit();
  if (recorded != 16 || cmds->size() != 1) return fail("commands replay the current push constants");
  // construction errors: the C ABI's status and message become Exception
  try {
    BMFR::create(64u, 64u, 32u, 32u, ref_ptr<GBuffer>(), ref_ptr<IlluminationBuffer>(),
                 ref_ptr<AccumulationBuffer>());
    return fail("BMFR without inputs must throw");
  } catch (const Exception& e) {
    if (e.result != PBRT_ERROR_INVALID_ARGUMENT || e.message.find("BMFR") == std::string::npos)
      return fail("BMFR exception: status and message");
    std::printf("BMFR error: %s\n", e.message.c_str());
  }
  try {
    PBRTPipeline::create(ref_ptr<Scene>(), ref_ptr<GBuffer>(), ref_ptr<IlluminationBuffer>(), true,
                         RayTracingRayOrigin::GBUFFER);
    return fail("G-buffer ray origins must throw");
  } catch (const Exception& e) {
    if (e.result != PBRT_ERROR_UNSUPPORTED) return fail("ray origin exception status");
  }
  try {
    PBRTPipeline::create(ref_ptr<Scene>(), ref_ptr<GBuffer>(), ref_ptr<IlluminationBuffer>(), true);
    return fail("a pipeline without a scene must throw");
  } catch (const Exception& e) {
    if (e.result != PBRT_ERROR_INVALID_ARGUMENT) return fail("pipeline exception status");
    std::printf("PBRTPipeline error: %s\n", e.message.c_str());
  }
  try {
    Accumulator::create(ref_ptr<GBuffer>(), ref_ptr<IlluminationBuffer>());
    return fail("an accumulator without buffers must throw");
  } catch (const Exception& e) {
    if (e.result != PBRT_ERROR_INVALID_ARGUMENT) return fail("accumulator exception status");
  }
  std::printf("errors: ok\n");
  return 0;
}

int frame(const char* scene_path, const char* frames_path, const std::string& out) {
  using namespace vkpbrt;
  Reader r(scene_path);
  if (std::memcmp(r.take(8), "PBRTSCN1", 8) != 0) throw std::runtime_error("not a scene file");
  const uint32_t nm = r.u32();
  std::vector<PbrtMeshDesc> meshes(nm);
  for (uint32_t m = 0; m < nm; ++m) {
    PbrtMeshDesc& d = meshes[m];
    d.vertex_count = r.u32();
    d.index_count = r.u32();
    d.index_stride = r.u32();
    d.positions = reinterpret_cast<const float*>(r.take(12 * (size_t)d.vertex_count));
    d.normals = reinterpret_cast<const float*>(r.take(12 * (size_t)d.vertex_count));
    d.uvs = reinterpret_cast<const float*>(r.take(8 * (size_t)d.vertex_count));
    d.indices = r.take((size_t)d.index_stride * d.index_count);
    r.align4();
  }
  const uint32_t ni = r.u32();
  const auto* inst = reinterpret_cast<const PbrtObjectInstance*>(r.take(sizeof(PbrtObjectInstance) * ni));
  const auto* opaque = reinterpret_cast<const uint8_t*>(r.take(ni));
  r.align4();
  const auto* mats = reinterpret_cast<const PbrtMaterialPacked*>(r.take(sizeof(PbrtMaterialPacked) * nm));
  const uint32_t nl = r.u32();
  const auto* lights = reinterpret_cast<const PbrtPackedLight*>(r.take(sizeof(PbrtPackedLight) * nl));
  const uint32_t nt = r.u32();
  std::vector<PbrtTextureDesc> tex(nt);
  for (uint32_t t = 0; t < nt; ++t) {
    tex[t].width = r.u32();
    tex[t].height = r.u32();
    tex[t].rgba8 = reinterpret_cast<const uint8_t*>(r.take(4 * (size_t)tex[t].width * tex[t].height));
  }
  const auto* mesh_tex = reinterpret_cast<const int32_t*>(r.take(4 * 5 * (size_t)nm));
  const uint32_t max_depth = r.u32(), min_depth = r.u32();
  PbrtSceneDesc desc{nm, meshes.data(), ni, inst, opaque, mats, nl, lights, nt, tex.data(), mesh_tex};

  Reader fr(frames_path);
  const uint32_t W = fr.u32(), H = fr.u32(), nf = fr.u32();

  ref_ptr<Scene> scene = Scene::create(desc);
  auto g_buffer = GBuffer::create(W, H);
  auto illumination = IlluminationBufferDemodulatedFloat::create(W, H);
  auto pipeline = PBRTPipeline::create(scene, g_buffer, illumination, true);
  pipeline->max_recursion_depth = (int32_t)max_depth;
  pipeline->min_recursion_depth = (int32_t)min_depth;
  pipeline->compile();
  auto accumulator = Accumulator::create(g_buffer, illumination);
  auto bmfr = BMFR::create(W, H, 32u, 32u, g_buffer, accumulator->accumulated_illumination,
                           accumulator->accumulation_buffer, 256u);
  auto push_constants = PushConstants::create();
  auto commands = Commands::create();
  pipeline->add_trace_rays_to_command_graph(commands, push_constants);
  accumulator->add_dispatch_to_command_graph(commands);
  bmfr->add_dispatch_to_command_graph(commands, push_constants);
  accumulator->accumulation_buffer->copy_to_back_images(commands, g_buffer, accumulator->accumulated_illumination);
  for (uint32_t f = 0; f < nf; ++f) {
    std::memcpy(&push_constants->value, fr.take(sizeof(PbrtPushConstants)), sizeof(PbrtPushConstants));
    CameraMatrices cur, prev;
    std::memcpy(&cur, fr.take(sizeof(CameraMatrices)), sizeof(CameraMatrices));
    std::memcpy(&prev, fr.take(sizeof(CameraMatrices)), sizeof(CameraMatrices));
    accumulator->set_camera_matrices((int32_t)push_constants->value.frame_number, cur, prev);
    commands->submit(nullptr);
  }
  std::vector<char> il(illumination->illumination_images[0].bytes());
  illumination->illumination_images[0].download(il.data());
  const Image& fin = bmfr->get_final_descriptor_image();
  std::vector<char> fb(fin.bytes());
  fin.download(fb.data());
  check(pbrt_stream_synchronize(nullptr), "synchronize");
  std::ofstream(out + ".illum", std::ios::binary).write(il.data(), (std::streamsize)il.size());
  std::ofstream(out + ".final", std::ios::binary).write(fb.data(), (std::streamsize)fb.size());
  const PbrtTraceStats st = pipeline->stats();
  std::printf("frame: %u frames, %llu primary, %llu extension, %llu shadow rays\n", nf,
              (unsigned long long)st.primary_rays, (unsigned long long)st.extension_rays,
              (unsigned long long)st.shadow_rays);
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  try {
    if (argc >= 2 && std::strcmp(argv[1], "errors") == 0) return errors();
    if (argc >= 5 && std::strcmp(argv[1], "frame") == 0) return frame(argv[2], argv[3], argv[4]);
  } catch (const vkpbrt::Exception& e) {
    std::fprintf(stderr, "vkpbrt::Exception (%d): %s\n", e.result, e.message.c_str());
    return 2;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 3;
  }
  std::fprintf(stderr, "usage: render_frame errors | frame SCENE FRAMES OUT_PREFIX\n");
  return 64;
}
