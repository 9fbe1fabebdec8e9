// Device scene layout and ray traversal (replaces the driver's TLAS/BLAS and
// traceRayEXT; shaders/ptRaygen.rgen:41, shaders/lighting.glsl:94,283).
//
// HBM layout (all arrays 16-byte aligned, read-only during a frame):
//   tris      float4[3 * ntri]  world-space v0|key, v1|instance, v2|primitive,
//                                in BVH leaf order (48 B per triangle);
//                                key = instance-major flat index (tie breaks)
//   nodes     Node8[nnodes]     80 B compressed 8-wide nodes, root at 0
//   instances DevInstance[]     object matrix, normal matrix, mesh, flags, the
//                                mesh's pool offsets and texture ids
//   meshes    DevMesh[]         offsets into the vertex / index pools
//   pos/nor/uv float pools      non-interleaved as the reference's SSBOs
//   idx       uint32 pool        u32 indices, or u16 pairs packed per word
//   materials DevMaterial[]     WaveFrontMaterialPacked (96 B)
//   lights    DevLight[]        PackedLight (128 B)
//   textures  DevTexture[] + one RGBA8 texel pool
#pragma once
#include <stdint.h>

#include "bvh.hpp"
#include "device_common.cuh"

namespace pbrt {

struct DevTexture {
  uint64_t offset;  // in texels; the texture in 4 x 2-texel tiles (texture_tile_index)
  uint32_t w, h;
};
struct DevMesh {
  uint32_t vbase;  // first vertex in the pos/nor/uv pools
  uint32_t ibase;  // first 32-bit word in the index pool
  uint32_t index_stride;
  int32_t tex[5];  // diffuse, mr, normal, emissive, specular
};
struct alignas(16) DevInstance {
  Mat4 obj;         // objectMat (column major)
  float4 nrm[3];    // columns of transpose(inverse(objectMat)), upper 3x3 (w unused)
  int32_t mesh;
  uint32_t index_stride;
  uint32_t opaque;  // 0: run the any-hit alpha test
  uint32_t pad;
  // the mesh's pool offsets and texture ids, copied here so a hit reaches
  // its vertices and textures one dependent load sooner
  uint32_t vbase, ibase;
  int32_t tex[5];
  uint32_t pad2;
};
struct alignas(16) DevMaterial {
  float4 ambient_roughness, diffuse_ior, specular_dissolve, transmittance_illum, emission_texture_id;
  uint32_t category_id;
  float pad[3];
};
struct alignas(16) DevLight {
  float4 v0_type, v1_strength, v2_angle, dir_angle2, col_ambient, col_diffuse, col_specular, strengths;
};
static_assert(sizeof(DevMaterial) == 96, "material is 96 B");
static_assert(sizeof(DevLight) == 128, "light is 128 B");

struct SceneView {
  const float4* tris;
  const Node8* nodes;
  const DevInstance* instances;
  const DevMesh* meshes;
  const DevMaterial* materials;
  const DevLight* lights;
  const float4* light_sum;  // per light: ambient + diffuse + specular colour (xyz), w = its power (sampleLight's sums)
  const float* pos;
  const float* nor;
  const float* uv;
  const uint32_t* idx;
  const DevTexture* textures;
  const uchar4* texels;
  uint32_t light_count;
  float light_strength_sum;
  uint32_t tri_count;
  int any_alpha;  // some instance needs the alpha test
};

constexpr int kStackSize = 64;

}  // namespace pbrt
