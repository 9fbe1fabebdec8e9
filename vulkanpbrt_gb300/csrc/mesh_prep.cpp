// Mesh preparation of the scene visitor (source/scene/RayTracingVisitor.cpp:
// 52-127 and 133-166), host side: vertex normals generated when a mesh
// arrives without them, texture coordinates filled when it arrives without
// any. Float arithmetic follows vsg's vec3 operators
// (external/vsg/include/vsg/maths/vec3.h: cross, length = sqrt of the
// left-to-right sum of squares, v / s = v * (1 / s)), FP contraction off.
#include <cmath>
#include <cstdint>
#include <cstring>

#include "internal.hpp"

namespace {

struct V3 {
  float x, y, z;
};
V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
V3 mul(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
V3 cross(V3 l, V3 r) { return {l.y * r.z - r.y * l.z, l.z * r.x - r.z * l.x, l.x * r.y - r.x * l.y}; }
float length(V3 v) { return std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z); }

template <class I>
int generate(const float* pos, uint32_t nv, const I* idx, uint32_t ni, float* nor) {
  for (uint32_t i = 0; i < ni; ++i)
    if (idx[i] >= nv) return pbrt::fail(PBRT_ERROR_INVALID_ARGUMENT, "mesh normals: index %u >= %u vertices", (unsigned)idx[i], nv);
  std::vector<float> weight(nv, 0.f);
  auto P = [&](uint32_t k) { return V3{pos[3 * k], pos[3 * k + 1], pos[3 * k + 2]}; };
  auto N = [&](uint32_t k) { return V3{nor[3 * k], nor[3 * k + 1], nor[3 * k + 2]}; };
  auto setN = [&](uint32_t k, V3 v) {
    nor[3 * k] = v.x;
    nor[3 * k + 1] = v.y;
    nor[3 * k + 2] = v.z;
  };
  for (uint32_t t = 0; t < ni / 3; ++t) {
    const uint32_t ia = idx[3 * t], ib = idx[3 * t + 1], ic = idx[3 * t + 2];
    const V3 a = P(ia), b = P(ib), c = P(ic);
    V3 fn = cross(sub(b, a), sub(c, a));
    const float w = length(fn);  // area-proportional weight
    fn = mul(fn, 1.0f / w);
    for (uint32_t k : {ia, ib, ic}) {
      const float nw = w + weight[k];
      setN(k, add(mul(N(k), weight[k] / nw), mul(fn, w / nw)));
      weight[k] = nw;
    }
  }
  return PBRT_OK;
}

}  // namespace

extern "C" {

PBRT_API int pbrt_mesh_generate_normals(const float* positions, uint32_t vertex_count, const void* indices,
                                        uint32_t index_count, uint32_t index_stride, float* normals) {
  if (!positions || !indices || !normals || (index_stride != 2 && index_stride != 4))
    return pbrt::fail(PBRT_ERROR_INVALID_ARGUMENT, "mesh normals: bad arguments");
  if (index_stride == 2)
    return generate(positions, vertex_count, static_cast<const uint16_t*>(indices), index_count, normals);
  return generate(positions, vertex_count, static_cast<const uint32_t*>(indices), index_count, normals);
}

PBRT_API int pbrt_mesh_fill_uvs(uint32_t vertex_count, const void* indices, uint32_t index_count,
                                uint32_t index_stride, float* uvs) {
  if (!indices || !uvs || (index_stride != 2 && index_stride != 4))
    return pbrt::fail(PBRT_ERROR_INVALID_ARGUMENT, "mesh uvs: bad arguments");
  std::memset(uvs, 0, sizeof(float) * 2 * (size_t)vertex_count);
  static const float corner[3][2] = {{0.f, 0.f}, {0.f, 1.f}, {1.f, 0.f}};
  for (uint32_t i = 0; i < index_count / 3 * 3; ++i) {
    const uint32_t k = index_stride == 2 ? static_cast<const uint16_t*>(indices)[i]
                                         : static_cast<const uint32_t*>(indices)[i];
    if (k >= vertex_count) return pbrt::fail(PBRT_ERROR_INVALID_ARGUMENT, "mesh uvs: index %u >= %u", k, vertex_count);
    uvs[2 * k] = corner[i % 3][0];
    uvs[2 * k + 1] = corner[i % 3][1];
  }
  return PBRT_OK;
}

}  // extern "C"
