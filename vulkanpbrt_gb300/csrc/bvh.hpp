// Compressed 8-wide BVH over world-space triangles.
//
// Built on the host: binned-SAH binary BVH (Wald 2007, 32 bins on 3 axes,
// leaves of at most 3 triangles), collapsed to 8-wide nodes by repeatedly
// opening the child with the largest surface area. A node stores its bounds'
// origin and per-axis power-of-two scale; each child box is 6 bytes of
// conservative 8-bit offsets (the quantised layout of Ylitie, Karras & Laine
// 2017, with a layout of this project's own). Child slots are assigned by
// octant of the child's centroid relative to the node's, so a ray visits
// slot (k ^ octant(ray)) in order k = 0..7, roughly near to far.
#pragma once
#include <cstddef>
#include <cstdint>
#include <vector>

#include <vector_types.h>

namespace pbrt {

struct alignas(16) Node8 {
  float px, py, pz;          // bounds origin
  uint8_t ex, ey, ez;        // biased exponents: scale = 2^(e - 127)
  uint8_t imask;             // slots holding internal children
  uint32_t child_base;       // node index of the first internal child (consecutive, slot order)
  uint32_t tri_base;         // first triangle of this node's leaves (consecutive, slot order)
  uint8_t meta[8];           // 0 empty; 0x80 internal; else (count << 5) | tri offset
  uint8_t qlo[3][8];         // per axis, per slot: child lo = p + scale * qlo
  uint8_t qhi[3][8];
};
static_assert(sizeof(Node8) == 80, "Node8 is 80 bytes");

struct Bvh8Stats {
  size_t nodes = 0, leaves = 0, tris = 0;
  int depth = 0;
  double sah = 0.0;
  double build_ms = 0.0;
};

// Builds over n triangles given as 9 floats each (v0, v1, v2, world space).
// tri_order receives, for every triangle slot of the BVH, the input index.
void build_bvh8(const float* verts9, size_t n, std::vector<Node8>& nodes, std::vector<uint32_t>& tri_order,
                Bvh8Stats* stats);

// Device build of the same layout (bvh_gpu.cu): a linear BVH collapsed to
// 8-wide nodes. Takes the triangles (9 floats each) and each triangle's
// instance and primitive; returns device arrays (cudaMalloc'd, the caller
// frees them): the nodes and the leaf-ordered triangle records, 3 float4 a
// triangle (v0 | flattening index, v1 | instance, v2 | primitive). Fails
// with PBRT_ERROR_UNSUPPORTED past max_depth wide levels.
int build_bvh8_device(const float* verts9, const uint32_t* instance, const uint32_t* primitive, size_t n,
                      int max_depth, Node8** nodes, float4** tris, Bvh8Stats* stats);

}  // namespace pbrt
