// Wavefront path tracer on sm_103a: the per-frame path of ptRaygen.rgen with
// ptClosesthit / ptAlphaHit / ptMiss / shadow.rmiss, NEE with multiple-
// importance light sampling (lighting.glsl) and BRDF importance sampling
// (sampling.glsl, brdf.glsl).
//
// One frame = raygen, then per bounce: closest-hit traversal of the ray
// queue (persistent warps), shading (surface, next-event light choice, BRDF
// sample, Russian roulette) that compacts surviving paths into the next ray
// queue and shadow rays into the shadow queue with warp-aggregated atomics,
// any-hit traversal of the shadow queue which resolves the pending NEE term,
// and a final pass that clamps and demodulates. The launch sequence of a
// frame is captured once in a CUDA graph and replayed.
//
// Path semantics follow the shaders, with one definition the shaders leave
// open: when indirectLighting() returns early (zero BRDF, pdf < 1e-6 or a
// Russian-roulette kill) the reference keeps iterating with a zero-length
// view vector (NaN) whose outcome depends on the driver's min/max/clamp NaN
// rules; here the path ends, which is what those early returns mean. A path
// that misses also ends (later iterations add nothing and draw no numbers).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "internal.hpp"
#include "shading.cuh"

namespace pbrt {

constexpr unsigned kFullMask = 0xffffffffu;

// ---------------------------------------------------------------------------
// Watertight ray/triangle test (Woop, Benthin & Wald, JCGT 2013), every
// operation rounded explicitly (no contraction) so that the CPU oracle's FP32
// test takes identical decisions.
struct RayPre {
  float3 o, d, inv;
  int kx, ky, kz, oct;
  float Sx, Sy, Sz;
};

PBRT_D float comp(float3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

PBRT_D RayPre ray_pre(float3 o, float3 d) {
  RayPre r;
  r.o = o;
  r.d = d;
  float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
  r.kz = (ax > ay && ax > az) ? 0 : (ay > az ? 1 : 2);
  r.kx = (r.kz + 1) % 3;
  r.ky = (r.kx + 1) % 3;
  float dz = comp(d, r.kz);
  if (dz < 0.f) {
    int t = r.kx;
    r.kx = r.ky;
    r.ky = t;
  }
  r.Sx = __fdiv_rn(comp(d, r.kx), dz);
  r.Sy = __fdiv_rn(comp(d, r.ky), dz);
  r.Sz = __fdiv_rn(1.0f, dz);
  // slab test reciprocals (tiny components clamped away from zero)
  auto safe = [](float x) { return fabsf(x) < 1e-20f ? copysignf(1e-20f, x) : x; };
  r.inv = f3(1.f / safe(d.x), 1.f / safe(d.y), 1.f / safe(d.z));
  r.oct = (d.x < 0.f ? 1 : 0) | (d.y < 0.f ? 2 : 0) | (d.z < 0.f ? 4 : 0);
  return r;
}

PBRT_D bool tri_intersect(const RayPre& r, float4 a, float4 b, float4 c, float tmin, float& t, float& u, float& v) {
  float3 A = f3(__fsub_rn(a.x, r.o.x), __fsub_rn(a.y, r.o.y), __fsub_rn(a.z, r.o.z));
  float3 B = f3(__fsub_rn(b.x, r.o.x), __fsub_rn(b.y, r.o.y), __fsub_rn(b.z, r.o.z));
  float3 C = f3(__fsub_rn(c.x, r.o.x), __fsub_rn(c.y, r.o.y), __fsub_rn(c.z, r.o.z));
  float Akz = comp(A, r.kz), Bkz = comp(B, r.kz), Ckz = comp(C, r.kz);
  float Ax = __fsub_rn(comp(A, r.kx), __fmul_rn(r.Sx, Akz)), Ay = __fsub_rn(comp(A, r.ky), __fmul_rn(r.Sy, Akz));
  float Bx = __fsub_rn(comp(B, r.kx), __fmul_rn(r.Sx, Bkz)), By = __fsub_rn(comp(B, r.ky), __fmul_rn(r.Sy, Bkz));
  float Cx = __fsub_rn(comp(C, r.kx), __fmul_rn(r.Sx, Ckz)), Cy = __fsub_rn(comp(C, r.ky), __fmul_rn(r.Sy, Ckz));
  float U = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
  float V = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
  float W = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
  if (U == 0.f || V == 0.f || W == 0.f) {  // edge cases re-evaluated exactly enough in FP64
    U = (float)__dsub_rn(__dmul_rn((double)Cx, (double)By), __dmul_rn((double)Cy, (double)Bx));
    V = (float)__dsub_rn(__dmul_rn((double)Ax, (double)Cy), __dmul_rn((double)Ay, (double)Cx));
    W = (float)__dsub_rn(__dmul_rn((double)Bx, (double)Ay), __dmul_rn((double)By, (double)Ax));
  }
  if ((U < 0.f || V < 0.f || W < 0.f) && (U > 0.f || V > 0.f || W > 0.f)) return false;
  float det = __fadd_rn(__fadd_rn(U, V), W);
  if (det == 0.f) return false;
  float Az = __fmul_rn(r.Sz, Akz), Bz = __fmul_rn(r.Sz, Bkz), Cz = __fmul_rn(r.Sz, Ckz);
  float T = __fadd_rn(__fadd_rn(__fmul_rn(U, Az), __fmul_rn(V, Bz)), __fmul_rn(W, Cz));
  float rcp = __fdiv_rn(1.0f, det);
  t = __fmul_rn(T, rcp);
  if (!(t > tmin)) return false;
  u = __fmul_rn(V, rcp);
  v = __fmul_rn(W, rcp);
  return true;
}

// ptAlphaHit out of line: it runs rarely, and inlined into the node visit it
// inflated the traversal loop (instruction-fetch stalls).
__device__ __noinline__ bool alpha_accept_slow(const DevInstance* instances, const DevMesh* meshes,
                                               const uint32_t* idx, const float* uvs, const DevTexture* textures,
                                               const uchar4* texels, uint32_t inst_id, uint32_t prim, float bu,
                                               float bv) {
  SceneView sc{};
  sc.instances = instances;
  sc.meshes = meshes;
  sc.idx = idx;
  sc.uv = uvs;
  sc.textures = textures;
  sc.texels = texels;
  return alpha_accept(sc, inst_id, prim, bu, bv);
}
PBRT_D bool alpha_accept_call(const SceneView& sc, uint32_t inst_id, uint32_t prim, float bu, float bv) {
  if (__ldg(&sc.instances[inst_id].opaque)) return true;
  return alpha_accept_slow(sc.instances, sc.meshes, sc.idx, sc.uv, sc.textures, sc.texels, inst_id, prim, bu, bv);
}

// Per-ray traversal state: the node to visit next, the short stack of node
// groups (child base, inner mask << 8 | remaining hits), the triangles of the
// last node visited that wait for their test, and the best hit.
struct TravState {
  uint32_t node;
  int sp;
  int best_tri;  // BVH-order triangle slot, -1 = miss
  float tbest, bu, bv;
  uint32_t best_key;
  uint32_t tri_base, tri_mask;    // pending triangles: slots tri_base + bit of tri_mask
  uint32_t tri_base2, tri_mask2;  // a second pending group (the triangle tests wait for a fuller warp)
};
constexpr uint32_t kNoNode = 0xffffffffu;

// Traversal stack in local memory (per lane; interleaved across lanes by the
// hardware). Shallow at the depths of these trees: pushes and pops hit L1.
constexpr int kTraverseThreads = 128;
struct TravStack {
  uint2 local[kStackSize];
  PBRT_D void put(int i, uint2 v) { local[i] = v; }
  PBRT_D uint2 get(int i) const { return local[i]; }
};

// The entry / exit distances of the three slabs; three-input min / max.
PBRT_D float fmax3f(float a, float b, float c) { return fmaxf(fmaxf(a, b), c); }
PBRT_D float fmin3f(float a, float b, float c) { return fminf(fminf(a, b), c); }
// byte k of w as a float (k is a constant once the child loop is unrolled)
PBRT_D float byte_to_float(uint32_t w, int k) { return (float)((w >> (8 * k)) & 0xffu); }
// Bits 0, 8, 16, 24 of x -> bits 0..3.
PBRT_D uint32_t gather_byte_lsbs(uint32_t x) { return ((x * 0x204081u) >> 21) & 0xFu; }
// 8-bit mask of the slots whose meta byte is a leaf (triangle count 1..3 in bits 5-6).
PBRT_D uint32_t leaf_slots(uint32_t meta_lo, uint32_t meta_hi) {
  const uint32_t c0 = (meta_lo >> 5) & 0x03030303u, c1 = (meta_hi >> 5) & 0x03030303u;
  return gather_byte_lsbs((c0 | (c0 >> 1)) & 0x01010101u) | (gather_byte_lsbs((c1 | (c1 >> 1)) & 0x01010101u) << 4);
}
// Moves bit s of an 8-bit mask to bit s ^ oct.
PBRT_D uint32_t octant_permute(uint32_t m, int oct) {
  if (oct & 1) m = ((m & 0x55u) << 1) | ((m >> 1) & 0x55u);
  if (oct & 2) m = ((m & 0x33u) << 2) | ((m >> 2) & 0x33u);
  if (oct & 4) m = ((m & 0x0Fu) << 4) | ((m >> 4) & 0x0Fu);
  return m;
}

// Node visit: box-tests st.node's children, records the triangles of the hit
// leaf children in st.tri_mask and moves to the next node -- the nearest hit
// inner child (octant order), else the next entry of the stack, else kNoNode.
// Each axis's near and far quantised plane words are chosen once per node by
// the sign of the ray's reciprocal direction (for a positive scale the fma of
// the smaller plane is the smaller t, so this is the per-child min / max, bit
// for bit); the hits are collected as an 8-bit mask and classified once per
// node (inner children: the node's inner mask moved to octant order; leaves:
// a mask built from the meta bytes' count fields).
PBRT_D void visit_node(const SceneView& sc, const RayPre& r, float tmin, TravState& st, TravStack& stack, int& err,
                       uint32_t& n_nodes) {
  const float4* nodes4 = reinterpret_cast<const float4*>(sc.nodes);
  const uint32_t node = st.node;
  ++n_nodes;
  const float4 n0 = __ldg(nodes4 + 5 * node + 0);
  const float4 n1 = __ldg(nodes4 + 5 * node + 1);
  const float4 n2 = __ldg(nodes4 + 5 * node + 2);
  const float4 n3 = __ldg(nodes4 + 5 * node + 3);
  const float4 n4 = __ldg(nodes4 + 5 * node + 4);
  const uint32_t emi = __float_as_uint(n0.w);
  const uint32_t imask = emi >> 24;
  const uint32_t child_base = __float_as_uint(n1.x), tri_base = __float_as_uint(n1.y);
  const uint32_t meta_lo = __float_as_uint(n1.z), meta_hi = __float_as_uint(n1.w);
  // t = (p + scale * q - o) * inv = q * (scale * inv) + (p - o) * inv
  const float adx = (n0.x - r.o.x) * r.inv.x, ady = (n0.y - r.o.y) * r.inv.y, adz = (n0.z - r.o.z) * r.inv.z;
  const float scx = __uint_as_float(((emi >> 0) & 0xffu) << 23) * r.inv.x;
  const float scy = __uint_as_float(((emi >> 8) & 0xffu) << 23) * r.inv.y;
  const float scz = __uint_as_float(((emi >> 16) & 0xffu) << 23) * r.inv.z;
  // near / far plane words: lo for a positive reciprocal, hi for a negative one
  const bool sx = scx < 0.f, sy = scy < 0.f, sz = scz < 0.f;
  const uint32_t lx0 = __float_as_uint(n2.x), lx1 = __float_as_uint(n2.y), ly0 = __float_as_uint(n2.z),
                 ly1 = __float_as_uint(n2.w), lz0 = __float_as_uint(n3.x), lz1 = __float_as_uint(n3.y);
  const uint32_t hx0 = __float_as_uint(n3.z), hx1 = __float_as_uint(n3.w), hy0 = __float_as_uint(n4.x),
                 hy1 = __float_as_uint(n4.y), hz0 = __float_as_uint(n4.z), hz1 = __float_as_uint(n4.w);
  const uint32_t nx0 = sx ? hx0 : lx0, nx1 = sx ? hx1 : lx1, fx0 = sx ? lx0 : hx0, fx1 = sx ? lx1 : hx1;
  const uint32_t ny0 = sy ? hy0 : ly0, ny1 = sy ? hy1 : ly1, fy0 = sy ? ly0 : hy0, fy1 = sy ? ly1 : hy1;
  const uint32_t nz0 = sz ? hz0 : lz0, nz1 = sz ? hz1 : lz1, fz0 = sz ? lz0 : hz0, fz1 = sz ? lz1 : hz1;
  uint32_t hitm = 0;
#pragma unroll
  for (int s = 0; s < 8; ++s) {
    const int K = s & 3;
    const float tnx = fmaf(byte_to_float(s < 4 ? nx0 : nx1, K), scx, adx);
    const float tny = fmaf(byte_to_float(s < 4 ? ny0 : ny1, K), scy, ady);
    const float tnz = fmaf(byte_to_float(s < 4 ? nz0 : nz1, K), scz, adz);
    const float tfx = fmaf(byte_to_float(s < 4 ? fx0 : fx1, K), scx, adx);
    const float tfy = fmaf(byte_to_float(s < 4 ? fy0 : fy1, K), scy, ady);
    const float tfz = fmaf(byte_to_float(s < 4 ? fz0 : fz1, K), scz, adz);
    float tn = fmaxf(fmax3f(tnx, tny, tnz), tmin);
    float tf = fminf(fmin3f(tfx, tfy, tfz), st.tbest);
    // widened by a few ulp: the quantised boxes are conservative, the slab
    // arithmetic must not undo that
    tn = tn - fabsf(tn) * 4e-7f;
    tf = tf + fabsf(tf) * 4e-7f;
    hitm |= (tn <= tf ? 1u : 0u) << s;
  }
  uint32_t inner = octant_permute(hitm & imask, r.oct);
  uint32_t tris = 0;
  uint32_t lh = hitm & leaf_slots(meta_lo, meta_hi);
  while (lh) {
    const int s = __ffs(lh) - 1;
    lh &= lh - 1;
    const uint32_t meta = ((s < 4 ? meta_lo : meta_hi) >> (8 * (s & 3))) & 0xffu;
    tris |= ((1u << (meta >> 5)) - 1u) << (meta & 31u);  // <= 8 leaves x 3 triangles: bits 0..23
  }
  if (tris) {  // the lane holds at most one group when it visits a node
    if (st.tri_mask) {
      st.tri_base2 = tri_base;
      st.tri_mask2 = tris;
    } else {
      st.tri_base = tri_base;
      st.tri_mask = tris;
    }
  }
  if (inner) {
    const int k = __ffs(inner) - 1;
    inner &= inner - 1;
    const int s = k ^ r.oct;
    if (inner) {
      if (st.sp == kStackSize) {
        err = 1;
        st.node = kNoNode;
        st.tri_mask = st.tri_mask2 = 0;
        return;
      }
      stack.put(st.sp++, make_uint2(child_base, (imask << 8) | inner));
    }
    st.node = child_base + __popc(imask & ((1u << s) - 1u));
    return;
  }
  if (st.sp == 0) {
    st.node = kNoNode;
    return;
  }
  uint2 g = stack.get(--st.sp);
  uint32_t m = g.y & 0xffu;
  const uint32_t im = g.y >> 8;
  const int k = __ffs(m) - 1;
  m &= m - 1;
  const int s = k ^ r.oct;
  if (m) stack.put(st.sp++, make_uint2(g.x, (im << 8) | m));
  st.node = g.x + __popc(im & ((1u << s) - 1u));
}

// Tests the lowest triangle of st.tri_mask (the packet traversal's form).
// Returns true for an accepted any-hit (the ray is finished).
PBRT_D bool test_one_triangle_rt(const SceneView& sc, const RayPre& r, float tmin, TravState& st, bool any_hit) {
  const int b = __ffs(st.tri_mask) - 1;
  st.tri_mask &= st.tri_mask - 1;
  const uint32_t ti = st.tri_base + (uint32_t)b;
  const float4 a = __ldg(sc.tris + 3 * ti), bb = __ldg(sc.tris + 3 * ti + 1), c = __ldg(sc.tris + 3 * ti + 2);
  float t, u, v;
  if (!tri_intersect(r, a, bb, c, tmin, t, u, v)) return false;
  const uint32_t key = __float_as_uint(a.w);
  if (!(t < st.tbest || (t == st.tbest && key < st.best_key))) return false;
  if (sc.any_alpha && !alpha_accept_call(sc, __float_as_uint(bb.w), __float_as_uint(c.w), u, v)) return false;
  st.best_tri = (int)ti;
  st.tbest = t;
  st.bu = u;
  st.bv = v;
  st.best_key = key;
  return any_hit;
}

// Cooperative triangle tests. A lane's node visit leaves 0 to 24 triangles
// to test, and only about a quarter of a warp's lanes have some at any step,
// so a per-lane triangle step runs with most lanes idle. Instead, after each
// step of node visits the warp lists every pending (ray, triangle) pair --
// lane i's pairs are numbers excl_i .. excl_i + count_i - 1 of an exclusive
// scan of the per-lane counts -- and tests them 32 at a time, lane j taking
// pair j of each pass: its owner is the largest i with excl_i <= j (a binary
// search over the scan, held in registers and read with shuffles), the
// triangle the owner's (j - excl_i)-th pending bit. The owner's ray (origin,
// the watertight test's shear and axis permutation, tmin, any-hit flag) is
// read from its record in shared memory; an accepted hit lowers the owner's
// best (t bits << 32 | triangle key) with a 64-bit shared-memory atomicMin --
// the nearest hit, ties to the lowest key, as the serial order gives -- and
// the lane holding the winning pair writes its u, v and triangle slot. The
// closest hit depends only on which triangles are tested, so the result is
// the serial traversal's, bit for bit.
struct TriRay {
  float ox, oy, oz, tmin;
  float sx, sy, sz;
  uint32_t perm;  // kx | ky << 2 | kz << 4 | any-hit << 6
};
struct TriBest {
  unsigned long long best;  // (t bits << 32) | key of the nearest accepted triangle
  float u, v;
  uint32_t tri;  // its BVH-order slot
  uint32_t pad;
};
PBRT_D unsigned long long pack_hit(float t, uint32_t key) {
  return ((unsigned long long)__float_as_uint(t) << 32) | key;  // t > 0: the bits order as the values
}
PBRT_D TriRay make_tri_ray(const RayPre& r, float tmin, bool any) {
  TriRay t;
  t.ox = r.o.x;
  t.oy = r.o.y;
  t.oz = r.o.z;
  t.tmin = tmin;
  t.sx = r.Sx;
  t.sy = r.Sy;
  t.sz = r.Sz;
  t.perm = (uint32_t)r.kx | ((uint32_t)r.ky << 2) | ((uint32_t)r.kz << 4) | (any ? 64u : 0u);
  return t;
}
// The watertight test (tri_intersect) with the ray read from its record.
PBRT_D bool tri_intersect_rec(const TriRay& q, float4 a, float4 b, float4 c, float& t, float& u, float& v) {
  RayPre r;
  r.o = f3(q.ox, q.oy, q.oz);
  r.kx = (int)(q.perm & 3u);
  r.ky = (int)((q.perm >> 2) & 3u);
  r.kz = (int)((q.perm >> 4) & 3u);
  r.Sx = q.sx;
  r.Sy = q.sy;
  r.Sz = q.sz;
  return tri_intersect(r, a, b, c, q.tmin, t, u, v);
}
// Tests every pending triangle of the warp's rays (all 32 lanes call it),
// once the warp has at least kCoopMinPairs of them or a lane cannot go on
// without its results (it holds two groups, or has no node left to visit);
// until then the lanes keep visiting nodes. Returns, per lane, whether its
// any-hit ray found an accepted triangle. kCoopMinPairs measured at 1080p
// (merged closest + shadow launches of a frame): 1 pair (test at every step)
// 4.35 ms, 12: 4.14, 20: 4.12, 28: 4.08 (5.73 ms with shading, against
// 5.70 at 20); the warps then test ~24 pairs a pass instead of ~13.
constexpr uint32_t kCoopMinPairs = 20;
PBRT_D bool coop_triangles(const SceneView& sc, TravState& st, const TriRay* rays, TriBest* best, int lane,
                           uint32_t& n_tris, uint32_t& n_tris_any) {
  const uint32_t cnt = __popc(st.tri_mask) + __popc(st.tri_mask2);
  uint32_t incl = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(kFullMask, incl, o);
    if (lane >= o) incl += y;
  }
  const uint32_t total = __shfl_sync(kFullMask, incl, 31);
  if (total == 0) return false;
  const bool urgent = st.tri_mask2 != 0 || (cnt != 0 && st.node == kNoNode);
  if (total < kCoopMinPairs && !__any_sync(kFullMask, urgent)) return false;
  const uint32_t excl = incl - cnt;
  const unsigned long long start = pack_hit(st.tbest, st.best_key);
  if (cnt) best[lane].best = start;
  __syncwarp();
  for (uint32_t base = 0; base < total; base += 32) {
    const uint32_t j = base + (uint32_t)lane;
    int owner = 0;  // the largest lane i with excl_i <= j
#pragma unroll
    for (int step = 16; step >= 1; step >>= 1) {
      const uint32_t e = __shfl_sync(kFullMask, excl, owner + step);
      if (e <= j) owner += step;
    }
    const uint32_t m0 = __shfl_sync(kFullMask, st.tri_mask, owner);
    const uint32_t b0 = __shfl_sync(kFullMask, st.tri_base, owner);
    const uint32_t m1 = __shfl_sync(kFullMask, st.tri_mask2, owner);
    const uint32_t b1 = __shfl_sync(kFullMask, st.tri_base2, owner);
    const uint32_t oexcl = __shfl_sync(kFullMask, excl, owner);
    bool won = false;
    unsigned long long cand = 0;
    float cu = 0.f, cv = 0.f;
    uint32_t ti = 0;
    if (j < total) {
      const uint32_t kk = j - oexcl, c0 = __popc(m0);
      ti = kk < c0 ? b0 + __fns(m0, 0, (int)kk + 1) : b1 + __fns(m1, 0, (int)(kk - c0) + 1);
      const TriRay q = rays[owner];
      const bool any = (q.perm & 64u) != 0;
      n_tris += any ? 0u : 1u;
      n_tris_any += any ? 1u : 0u;
      const float4 a = __ldg(sc.tris + 3 * ti), b = __ldg(sc.tris + 3 * ti + 1), c = __ldg(sc.tris + 3 * ti + 2);
      float t, u, v;
      if (tri_intersect_rec(q, a, b, c, t, u, v)) {
        cand = pack_hit(t, __float_as_uint(a.w));
        if (cand < *((volatile unsigned long long*)&best[owner].best) &&
            (!sc.any_alpha || alpha_accept_call(sc, __float_as_uint(b.w), __float_as_uint(c.w), u, v))) {
          atomicMin(&best[owner].best, cand);
          won = true;
          cu = u;
          cv = v;
        }
      }
    }
    __syncwarp();
    if (won && best[owner].best == cand) {  // the keys are distinct: one winner per owner
      best[owner].u = cu;
      best[owner].v = cv;
      best[owner].tri = ti;
    }
    __syncwarp();
  }
  bool accepted = false;
  if (cnt) {
    const TriBest b = best[lane];
    if (b.best != start) {
      st.tbest = __uint_as_float((uint32_t)(b.best >> 32));
      st.best_key = (uint32_t)b.best;
      st.bu = b.u;
      st.bv = b.v;
      st.best_tri = (int)b.tri;
      accepted = (rays[lane].perm & 64u) != 0;
    }
    st.tri_mask = st.tri_mask2 = 0;
  }
  __syncwarp();
  return accepted;
}

// ---------------------------------------------------------------------------
// Per-frame parameters and queues.
struct FrameParams {
  Mat4 inv_view, inv_proj;
  uint32_t frame, sample;
  int W, H;
  int min_depth, max_depth;  // Infos.minRecursionDepth / maxRecursionDepth
  int light_mode;            // 0 surface strength, 1 light strength, 2 uniform
  int final_image;           // FINAL_IMAGE (progressive sRGB) instead of DEMOD_ILLUMINATION_FLOAT
  int write_gbuffer;
  const volatile uint32_t* abort_flag;  // mapped host word, nonzero = stop (null: none)
  unsigned long long budget_ns;         // frame time budget (0: none)
};

struct Counters {
  uint32_t ray[2];       // ray queue sizes (ping-pong)
  uint32_t shadow;       // shadow queue size
  uint32_t work_trace;   // persistent-warp work index, closest hit
  uint32_t work_shadow;  // persistent-warp work index, any hit
  uint32_t error;        // bit 0 traversal stack overflow, bit 1 aborted, bit 2 budget exceeded
  uint32_t stop;         // nonzero: the frame was stopped (abort flag or budget); no more work is taken
  uint32_t pad;
  unsigned long long t0, budget_ns;      // frame start (%globaltimer) and budget
  const volatile uint32_t* abort_flag;
  unsigned long long rays_primary, rays_extension, rays_shadow, frames;
  unsigned long long nodes_closest, tris_closest, nodes_shadow, tris_shadow;  // BVH work (node / triangle visits)
};

// Adds a per-thread count to a 64-bit total with one atomic per warp.
PBRT_D void warp_add64(unsigned long long* dst, uint32_t v) {
  unsigned long long x = v;
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  if ((threadIdx.x & 31) == 0 && x) atomicAdd(dst, x);
}

struct Queues {
  // ray queues (2, ping-pong): path index, origin|tmin, direction|tmax
  uint32_t* pix[2];
  float4* org[2];
  float4* dir[2];
  float4* hit;    // t, u, v, key of the closest triangle (bits; 0xffffffff miss)
  uint2* hit_ip;  // instance and primitive of the closest triangle
  // shadow queue: path index, origin|tmin, direction|tmax, pending NEE, add term
  uint32_t* spix;
  float4* sorg;
  float4* sdir;
  float4* snee;  // unshadowed NEE contribution xyz, w = 0 primary / 1 indirect
  float4* sadd;  // emission term added with it
  // path state
  uint4* rng;
  float4* thr;   // throughput
  float4* rad;   // accumulated radiance (finalColor)
  float4* prev;  // previous vertex (worldSpacePos) xyz, w = loop index i (as int bits)
  float4* alb;   // primary albedo xyz (float, for demodulation), w = transDepth (int bits)
  uint32_t* prim_key;  // primary hit key per pixel (0xffffffff = miss), for parity tests
  // ray sorting (sort_rays schedule): shading appends to these, the sort scatters them
  // into the ray queue / shadow queue ordered by (direction octant, origin cell)
  uint32_t* pix_t;
  float4* org_t;
  float4* dir_t;
  uint16_t* key_t;
  uint32_t* spix_t;
  float4* sorg_t;
  float4* sdir_t;
  float4* snee_t;
  float4* sadd_t;
  uint16_t* skey_t;
  uint32_t* bins;  // [2][kSortBins]: extension rays, shadow rays
};

// Schedule options of a pipeline (pbrt_pipeline_set_schedule).
// Ray sorting: extension and shadow rays are reordered by a 12-bit key --
// the direction octant (3 bits) over a 3-bit-per-axis Morton cell of the
// origin in the scene box -- with a counting sort (histogram, scan,
// warp-aggregated scatter) before they are traversed, so a warp's rays take
// the same child order and start in the same region of the BVH. Results
// are per pixel, so the order changes nothing but speed. Shading appends to
// the staging queues (pix_t ... skey_t) when Queues::key_t is set.
// Merged schedule: bounce k's closest-hit rays and bounce k-1's shadow rays
// in one persistent launch (fewer launch tails, more rays per launch);
// per-pixel updates keep their order (shading of k-1, shadow resolve of
// k-1, shading of k). Otherwise one launch per queue.
constexpr int kSortBits = 12, kSortBins = 1 << kSortBits;

struct GBufferOut {
  float* depth;
  float2* normal;
  uchar4* material;
  uchar4* albedo;
};

// Warp-aggregated queue slot: one atomic per warp.
PBRT_D int warp_alloc(uint32_t* counter, bool want) {
  const unsigned active = __activemask();
  const unsigned m = __ballot_sync(active, want);
  if (m == 0) return -1;
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(m) - 1;
  uint32_t base = 0;
  if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(m));
  base = __shfl_sync(active, base, leader);
  if (!want) return -1;
  return (int)(base + __popc(m & ((1u << lane) - 1u)));
}

// ---------------------------------------------------------------------------
// Per-frame parameters travel as this launch's argument: no host buffer has
// to outlive the call, so consecutive frames need no host synchronisation.
__global__ void k_set_params(FrameParams* dst, FrameParams fp) { *dst = fp; }

PBRT_D unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Abort flag and frame budget: every traversal warp reads `stop` when it
// takes a batch; one batch in 64 also polls the host's abort word and the
// clock and raises `stop` (recording why in `error`). Stopped frames take no
// more rays and shade nothing, so the frame ends early and the host reads
// the reason with pbrt_pipeline_status; nothing waits on anything.
constexpr uint32_t kPollBatches = 64;
PBRT_D bool stop_requested(Counters* c, uint32_t batch) {
  if (*((volatile uint32_t*)&c->stop)) return true;
  if ((batch / 32u) % kPollBatches != 0) return false;
  uint32_t why = 0;
  if (c->abort_flag && *c->abort_flag) why = 2u;
  else if (c->budget_ns && global_ns() - c->t0 > c->budget_ns) why = 4u;
  if (!why) return false;
  atomicOr(&c->stop, why);
  atomicOr(&c->error, why);
  return true;
}

__global__ void k_frame_begin(Counters* c, const FrameParams* fp) {
  c->stop = 0;
  c->t0 = global_ns();
  c->budget_ns = fp->budget_ns;
  c->abort_flag = fp->abort_flag;
  c->ray[0] = (uint32_t)(fp->W * fp->H);
  c->ray[1] = 0;
  c->shadow = 0;
  c->work_trace = 0;
  c->work_shadow = 0;
  c->rays_primary += (unsigned long long)(fp->W * fp->H);
  c->frames += 1;
}

__global__ void k_bounce_begin(Counters* c, int k) {
  // queue k&1 was filled by the previous shade (or raygen)
  if (k > 0) c->rays_extension += c->ray[k & 1];
  c->ray[(k + 1) & 1] = 0;
  c->shadow = 0;
  c->work_trace = 0;
  c->work_shadow = 0;
}

__global__ void k_bounce_end(Counters* c) { c->rays_shadow += c->shadow; }

// Merged schedule: bounce k's launch also traces the shadow rays of bounce
// k-1, so the shadow queue is kept until that launch is done.
__global__ void k_bounce_begin_merged(Counters* c, int k) {
  if (k > 0) c->rays_extension += c->ray[k & 1];
  c->ray[(k + 1) & 1] = 0;
  c->work_trace = 0;
  c->work_shadow = 0;
  if (k == 0) c->shadow = 0;
}
__global__ void k_shadow_begin(Counters* c) { c->work_shadow = 0; }
__global__ void k_shadow_consumed(Counters* c) {
  c->rays_shadow += c->shadow;
  c->shadow = 0;
}

// createRay (camera.glsl:6-16) and the RNG seeding of ptRaygen.rgen:28-40.
// Primary rays enter the queue in 8x4-pixel tiles when the frame divides
// into them: the 32 rays a packet-traversal warp takes then cover a compact
// patch of the image (a smaller union of nodes than a 32-pixel row).
__global__ void k_raygen(const FrameParams* __restrict__ fpp, Queues q) {
  const FrameParams& fp = *fpp;
  const int N = fp.W * fp.H;
  const bool tiled = fp.W % 8 == 0 && fp.H % 4 == 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    int x, y;
    if (tiled) {
      const int tile = i >> 5, l = i & 31, tiles_x = fp.W >> 3;
      x = (tile % tiles_x) * 8 + (l & 7);
      y = (tile / tiles_x) * 4 + (l >> 3);
    } else {
      x = i % fp.W;
      y = i / fp.W;
    }
    const int p = y * fp.W + x;
    Rng re = rng_init((uint32_t)x, (uint32_t)y, fp.frame);
    float pcx = (float)x + .5f, pcy = (float)y + .5f;
    if (fp.final_image && fp.sample > 0) {  // antiAlias: only FINAL_IMAGE after the first sample
      float jx = rng_next(re), jy = rng_next(re);
      pcx += jx - .5f;
      pcy += jy - .5f;
    }
    const float cx = pcx / (float)fp.W * 2.0f - 1.0f, cy = pcy / (float)fp.H * 2.0f - 1.0f;
    const float4 org = fp.inv_view.c[3];
    float4 d = mul(fp.inv_proj, make_float4(cx, cy, 1.f, 1.f));
    float3 nd = normalize(f3(d.x, d.y, d.z));
    d = mul(fp.inv_view, make_float4(nd.x, nd.y, nd.z, 0.f));
    q.pix[0][i] = (uint32_t)p;
    q.org[0][i] = make_float4(org.x, org.y, org.z, 0.001f);
    q.dir[0][i] = make_float4(d.x, d.y, d.z, 10000.0f);
    q.rng[p] = make_uint4(re.x, re.y, re.z, re.w);
    q.thr[p] = make_float4(1.f, 1.f, 1.f, 0.f);
    q.rad[p] = make_float4(0.f, 0.f, 0.f, 0.f);
    q.prev[p] = make_float4(org.x, org.y, org.z, __int_as_float(0));
    q.alb[p] = make_float4(0.f, 0.f, 0.f, __int_as_float(0));
  }
}

// Persistent traversal. Each lane holds one ray; when it finishes, the lane
// takes the next ray of its warp's batch (32 ray indices fetched with one
// atomic) at once, so a warp never waits for its slowest ray. MODE 0: closest
// hit of the pipeline's ray queue; 1: any hit of the shadow queue, resolving
// the pending NEE term; 2 / 3: closest / any hit of a ray-query batch.
struct QueryIO {
  const float4* org;
  const float4* dir;
  float4* hits;
  uint32_t n;
  uint32_t* work;
  uint32_t* errflag;
};

// Traversal CTAs resident per SM the register allocation targets (7 x 128
// threads at <= 72 registers; 1080p tracer 5.66 -> 5.55 ms against 8 CTAs
// at 64 registers; 6 CTAs: 5.60 ms).
constexpr int kTraverseMinBlocks = 7;
template <int MODE>
__global__ void __launch_bounds__(128, kTraverseMinBlocks) k_traverse(SceneView sc, Queues q, Counters* c, int k,
                                                                    QueryIO io) {
  // MODE 4: the closest-hit rays of queue k&1 followed by the shadow rays
  // of the previous bounce, in one launch (one work counter over both)
  constexpr bool ANY = (MODE == 1 || MODE == 3);
  const int lane = threadIdx.x & 31;
  const unsigned lt_mask = (1u << lane) - 1u;
  const float4* org;
  const float4* dir;
  uint32_t count, count_c = 0;
  uint32_t* work;
  if (MODE == 4) {
    count_c = *((volatile uint32_t*)&c->ray[k & 1]);
    count = count_c + *((volatile uint32_t*)&c->shadow);
    org = q.org[k & 1];
    dir = q.dir[k & 1];
    work = &c->work_trace;
  } else if (MODE == 0) {
    count = *((volatile uint32_t*)&c->ray[k & 1]);
    org = q.org[k & 1];
    dir = q.dir[k & 1];
    work = &c->work_trace;
  } else if (MODE == 1) {
    count = *((volatile uint32_t*)&c->shadow);
    org = q.sorg;
    dir = q.sdir;
    work = &c->work_shadow;
  } else {
    count = io.n;
    org = io.org;
    dir = io.dir;
    work = io.work;
  }
  // per-lane ray records and best hits of the cooperative triangle tests
  __shared__ TriRay s_rays[kTraverseThreads];
  __shared__ TriBest s_best[kTraverseThreads];
  TriRay* const w_rays = s_rays + (threadIdx.x & ~31);
  TriBest* const w_best = s_best + (threadIdx.x & ~31);
  TravStack stack;
  TravState st;
  RayPre r;
  float tmin = 0.f;
  int idx = -1;
  uint32_t batch_next = 0, batch_end = 0;  // warp-uniform
  bool drained = false;                     // warp-uniform: no more batches
  int err = 0;
  uint32_t nn = 0, nt = 0, nn_s = 0, nt_s = 0;
  bool lane_any = ANY;
  st.tri_mask = st.tri_mask2 = 0;
  st.tri_base = st.tri_base2 = 0;
  while (true) {
    // ---- refill idle lanes from the warp's batch
    unsigned need = __ballot_sync(kFullMask, idx < 0);
    while (need && !drained) {
      if (batch_next >= batch_end) {
        uint32_t b = 0;
        if (lane == 0) {
          b = atomicAdd(work, 32u);
          if ((MODE <= 1 || MODE == 4) && b < count && stop_requested(c, b)) b = count;
        }
        b = __shfl_sync(kFullMask, b, 0);
        if (b >= count) {
          drained = true;
          break;
        }
        batch_next = b;
        batch_end = min(b + 32u, count);
      }
      const uint32_t avail = batch_end - batch_next;
      const uint32_t rank = __popc(need & lt_mask);
      if (((need >> lane) & 1u) && rank < avail) {
        idx = (int)(batch_next + rank);
        float4 o, d;
        if (MODE == 4) {
          lane_any = (uint32_t)idx >= count_c;
          const uint32_t j = lane_any ? (uint32_t)idx - count_c : (uint32_t)idx;
          o = lane_any ? q.sorg[j] : org[j];
          d = lane_any ? q.sdir[j] : dir[j];
        } else {
          o = org[idx];
          d = dir[idx];
        }
        r = ray_pre(f3(o.x, o.y, o.z), f3(d.x, d.y, d.z));
        tmin = o.w;
        w_rays[lane] = make_tri_ray(r, tmin, lane_any);
        st.node = 0;
        st.sp = 0;
        st.best_tri = -1;
        st.tbest = d.w;
        st.bu = st.bv = 0.f;
        st.best_key = 0xffffffffu;
        st.tri_mask = st.tri_mask2 = 0;
      }
      batch_next += min((uint32_t)__popc(need), avail);
      need = __ballot_sync(kFullMask, idx < 0);
    }
    if (__all_sync(kFullMask, idx < 0)) break;
    // ---- the triangles of the last node visits, the warp's lanes sharing them out
    const bool accepted = coop_triangles(sc, st, w_rays, w_best, lane, nt, nt_s);
    // ---- one node visit per busy lane
    if (idx >= 0 && !accepted && st.node != kNoNode) visit_node(sc, r, tmin, st, stack, err, lane_any ? nn_s : nn);
    if (idx < 0 || (!accepted && (st.node != kNoNode || st.tri_mask != 0))) continue;  // (tri_mask2 implies tri_mask)
    // ---- ray finished
    if (MODE == 0 || (MODE == 4 && !lane_any)) {
      // the hit's instance and primitive, read here where the triangle was
      // just tested (L1), so shading starts one dependent load later in the chain
      uint2 ip = make_uint2(0xffffffffu, 0u);
      if (st.best_tri >= 0)
        ip = make_uint2(__float_as_uint(__ldg(&sc.tris[3 * st.best_tri + 1].w)),
                        __float_as_uint(__ldg(&sc.tris[3 * st.best_tri + 2].w)));
      q.hit[idx] = make_float4(st.tbest, st.bu, st.bv, __uint_as_float(st.best_tri >= 0 ? st.best_key : 0xffffffffu));
      q.hit_ip[idx] = ip;
    } else if (MODE == 1 || MODE == 4) {
      const uint32_t j = MODE == 4 ? (uint32_t)idx - count_c : (uint32_t)idx;
      const uint32_t p = q.spix[j];
      const float4 nee4 = q.snee[j], add4 = q.sadd[j];
      const float3 nee = st.best_tri >= 0 ? f3(0.f) : f3(nee4.x, nee4.y, nee4.z);
      const float3 add = f3(add4.x, add4.y, add4.z);
      const float4 rd = q.rad[p];
      float3 rad = f3(rd.x, rd.y, rd.z);
      if (nee4.w == 0.f) rad = (f3(0.f) + nee) + add;  // finalColor = 0; += NEE; += emissive
      else rad = rad + (nee + add);                    // finalColor += NEE + emissive * throughput
      q.rad[p] = make_float4(rad.x, rad.y, rad.z, rd.w);
    } else {
      const uint32_t key = st.best_tri >= 0 ? __float_as_uint(sc.tris[3 * st.best_tri].w) : 0xffffffffu;
      io.hits[idx] = make_float4(st.tbest, st.bu, st.bv, __uint_as_float(key));
    }
    idx = -1;
    st.tri_mask = st.tri_mask2 = 0;
  }
  if (MODE == 4) {
    warp_add64(&c->nodes_closest, nn);
    warp_add64(&c->tris_closest, nt);
    warp_add64(&c->nodes_shadow, nn_s);
    warp_add64(&c->tris_shadow, nt_s);
  } else if (MODE == 0) {
    warp_add64(&c->nodes_closest, nn);
    warp_add64(&c->tris_closest, nt);
  } else if (MODE == 1) {
    warp_add64(&c->nodes_shadow, nn_s);
    warp_add64(&c->tris_shadow, nt_s);
  }
  if (err) atomicOr((MODE <= 1 || MODE == 4) ? &c->error : io.errflag, 1u);
}

// Packet traversal of the primary rays (bounce 0): a warp takes 32
// consecutive queue entries (an 8x4-pixel tile, see k_raygen) and walks the BVH
// together: every lane box-tests the same node's children against its own
// ray (its own t range), the warp follows the union of the hits (octant
// order of the warp's first ray) on one shared stack, and each lane tests
// the triangles of the union's leaves that its own ray hit. All lanes run the
// same node visit (a single ray's traversal keeps about half of them busy on
// primary rays); the closest hit is the same, as it depends only on which
// triangles a ray tests, never on the order. Node visits are counted once
// per warp (one fetch serves the 32 rays), triangle tests per ray.
__global__ void __launch_bounds__(128, kTraverseMinBlocks) k_traverse_packet(SceneView sc, Queues q, Counters* c) {
  __shared__ uint2 s_stack[kTraverseThreads / 32][kStackSize];
  const int lane = threadIdx.x & 31;
  uint2* stk = s_stack[threadIdx.x >> 5];
  const uint32_t count = *((volatile uint32_t*)&c->ray[0]);
  const float4* nodes4 = reinterpret_cast<const float4*>(sc.nodes);
  uint32_t nn = 0, nt = 0;
  int err = 0;
  while (true) {
    uint32_t base = 0;
    if (lane == 0) {
      base = atomicAdd(&c->work_trace, 32u);
      if (base < count && stop_requested(c, base)) base = count;
    }
    base = __shfl_sync(kFullMask, base, 0);
    if (base >= count) break;
    const uint32_t idx = base + (uint32_t)lane;
    const bool valid = idx < count;
    float4 o = make_float4(0.f, 0.f, 0.f, 0.f), d = make_float4(0.f, 0.f, 1.f, -1.f);
    if (valid) {
      o = q.org[0][idx];
      d = q.dir[0][idx];
    }
    const RayPre r = ray_pre(f3(o.x, o.y, o.z), f3(d.x, d.y, d.z));
    const float tmin = o.w;
    TravState st;
    st.best_tri = -1;
    st.tbest = d.w;  // invalid lanes: -1, so no box is ever hit
    st.bu = st.bv = 0.f;
    st.best_key = 0xffffffffu;
    const int oct = __shfl_sync(kFullMask, r.oct, 0);
    uint32_t node = 0;
    int sp = 0;  // warp-uniform
    while (true) {
      // ---- box tests of node's children, per lane (the deferred visit's slab code)
      ++nn;
      const float4 n0 = __ldg(nodes4 + 5 * node + 0), n1 = __ldg(nodes4 + 5 * node + 1);
      const float4 n2 = __ldg(nodes4 + 5 * node + 2), n3 = __ldg(nodes4 + 5 * node + 3);
      const float4 n4 = __ldg(nodes4 + 5 * node + 4);
      const uint32_t emi = __float_as_uint(n0.w), imask = emi >> 24;
      const uint32_t child_base = __float_as_uint(n1.x), tri_base = __float_as_uint(n1.y);
      const uint32_t meta_lo = __float_as_uint(n1.z), meta_hi = __float_as_uint(n1.w);
      const float adx = (n0.x - r.o.x) * r.inv.x, ady = (n0.y - r.o.y) * r.inv.y, adz = (n0.z - r.o.z) * r.inv.z;
      const float scx = __uint_as_float(((emi >> 0) & 0xffu) << 23) * r.inv.x;
      const float scy = __uint_as_float(((emi >> 8) & 0xffu) << 23) * r.inv.y;
      const float scz = __uint_as_float(((emi >> 16) & 0xffu) << 23) * r.inv.z;
      const bool sx = scx < 0.f, sy = scy < 0.f, sz = scz < 0.f;
      const uint32_t lx0 = __float_as_uint(n2.x), lx1 = __float_as_uint(n2.y), ly0 = __float_as_uint(n2.z),
                     ly1 = __float_as_uint(n2.w), lz0 = __float_as_uint(n3.x), lz1 = __float_as_uint(n3.y);
      const uint32_t hx0 = __float_as_uint(n3.z), hx1 = __float_as_uint(n3.w), hy0 = __float_as_uint(n4.x),
                     hy1 = __float_as_uint(n4.y), hz0 = __float_as_uint(n4.z), hz1 = __float_as_uint(n4.w);
      const uint32_t nx0 = sx ? hx0 : lx0, nx1 = sx ? hx1 : lx1, fx0 = sx ? lx0 : hx0, fx1 = sx ? lx1 : hx1;
      const uint32_t ny0 = sy ? hy0 : ly0, ny1 = sy ? hy1 : ly1, fy0 = sy ? ly0 : hy0, fy1 = sy ? ly1 : hy1;
      const uint32_t nz0 = sz ? hz0 : lz0, nz1 = sz ? hz1 : lz1, fz0 = sz ? lz0 : hz0, fz1 = sz ? lz1 : hz1;
      uint32_t hitm = 0;
#pragma unroll
      for (int s = 0; s < 8; ++s) {
        const int K = s & 3;
        const float tnx = fmaf(byte_to_float(s < 4 ? nx0 : nx1, K), scx, adx);
        const float tny = fmaf(byte_to_float(s < 4 ? ny0 : ny1, K), scy, ady);
        const float tnz = fmaf(byte_to_float(s < 4 ? nz0 : nz1, K), scz, adz);
        const float tfx = fmaf(byte_to_float(s < 4 ? fx0 : fx1, K), scx, adx);
        const float tfy = fmaf(byte_to_float(s < 4 ? fy0 : fy1, K), scy, ady);
        const float tfz = fmaf(byte_to_float(s < 4 ? fz0 : fz1, K), scz, adz);
        float tn = fmaxf(fmax3f(tnx, tny, tnz), tmin);
        float tf = fminf(fmin3f(tfx, tfy, tfz), st.tbest);
        tn = tn - fabsf(tn) * 4e-7f;
        tf = tf + fabsf(tf) * 4e-7f;
        hitm |= (tn <= tf ? 1u : 0u) << s;
      }
      uint32_t tris = 0;
      uint32_t lh = hitm & leaf_slots(meta_lo, meta_hi);
      while (lh) {
        const int s = __ffs(lh) - 1;
        lh &= lh - 1;
        const uint32_t meta = ((s < 4 ? meta_lo : meta_hi) >> (8 * (s & 3))) & 0xffu;
        tris |= ((1u << (meta >> 5)) - 1u) << (meta & 31u);
      }
      // ---- triangles of the union's leaves, each lane those its ray reached
      uint32_t utris = __reduce_or_sync(kFullMask, tris);
      while (utris) {
        const int b = __ffs(utris) - 1;
        utris &= utris - 1;
        if ((tris >> b) & 1u) {
          st.tri_base = tri_base;
          st.tri_mask = 1u << b;
          ++nt;
          test_one_triangle_rt(sc, r, tmin, st, false);
        }
      }
      // ---- next node: nearest inner child of the union (warp octant order), rest on the stack
      const uint32_t uinner = octant_permute(__reduce_or_sync(kFullMask, hitm & imask), oct);
      if (uinner) {
        const int k = __ffs(uinner) - 1;
        const uint32_t rest = uinner & (uinner - 1);
        if (rest) {
          if (sp == kStackSize) {
            err = 1;
            break;
          }
          if (lane == 0) stk[sp] = make_uint2(child_base, (imask << 8) | rest);
          ++sp;
        }
        const int s = k ^ oct;
        node = child_base + __popc(imask & ((1u << s) - 1u));
        __syncwarp();
        continue;
      }
      if (sp == 0) break;
      __syncwarp();
      const uint2 g = stk[sp - 1];
      uint32_t m = g.y & 0xffu;
      const uint32_t im = g.y >> 8;
      const int k = __ffs(m) - 1;
      m &= m - 1;
      __syncwarp();
      if (m) {
        if (lane == 0) stk[sp - 1] = make_uint2(g.x, (im << 8) | m);
      } else {
        --sp;
      }
      const int s = k ^ oct;
      node = g.x + __popc(im & ((1u << s) - 1u));
      __syncwarp();
    }
    if (valid) {
      uint2 ip = make_uint2(0xffffffffu, 0u);
      if (st.best_tri >= 0)
        ip = make_uint2(__float_as_uint(__ldg(&sc.tris[3 * st.best_tri + 1].w)),
                        __float_as_uint(__ldg(&sc.tris[3 * st.best_tri + 2].w)));
      q.hit[idx] = make_float4(st.tbest, st.bu, st.bv, __uint_as_float(st.best_tri >= 0 ? st.best_key : 0xffffffffu));
      q.hit_ip[idx] = ip;
    }
  }
  // nodes counted per warp (lane 0's count), triangles per ray
  warp_add64(&c->nodes_closest, lane == 0 ? nn : 0u);
  warp_add64(&c->tris_closest, nt);
  if (err) atomicOr(&c->error, 1u);
}

// sampleLight (lighting.glsl:19-227): returns the picked light's strength
// (lightStrength), fills the direction, the pick pdf and the shadow ray's
// tmax; traced = false when no shadow ray is cast. The per-light
// attenuation, direction and pick-probability divisions use the hardware
// reciprocal (GLSL's own division is only 2.5 ulp).
PBRT_D float3 sample_light(const SceneView& sc, int mode, float3 pos, float3 n, Rng& re, float3& l, float& pdf,
                           float& shadow_tmax, bool& traced) {
  const float tmin = 0.001f;
  traced = false;
  pdf = 0.f;
  l = f3(0.f);
  if (mode == 0) {
    float strength_sum = 0.f, picked_strength = 0.f;
    float3 picked_ls = f3(0.f);
    float tmax = 1000.0f;
    for (uint32_t i = 0; i < sc.light_count; ++i) {
      const DevLight L = sc.lights[i];
      const float4 lsum = sc.light_sum[i];  // colA + colD + colS, and dot(colA + colD + colS, vec4(1))
      const float3 csum = f3(lsum.x, lsum.y, lsum.z);
      const float power = lsum.w;
      float strength = 0.f;
      float3 ls = csum;
      float cur_tmax = 1000.0f;
      float3 cur_l = f3(0.f);
      const int type = (int)L.v0_type.w;
      const float3 v0 = f3(L.v0_type.x, L.v0_type.y, L.v0_type.z);
      if (type == 1) {  // directional
        float d = length(pos - v0);
        float att = __fdividef(1.0f, L.strengths.x + L.strengths.y * d + L.strengths.z * d * d);
        float3 ndir = -f3(L.dir_angle2.x, L.dir_angle2.y, L.dir_angle2.z);
        strength = fmaxf(dot(n, ndir), 0.f) * power * att;
        ls = ls * (dot(n, ndir) * att);
        cur_l = nrmz(ndir);
      } else if (type == 2) {  // point
        float d = length(pos - v0);
        float att = __fdividef(1.0f, L.strengths.x + L.strengths.y * d + L.strengths.z * d * d);
        float3 to = nrmz(v0 - pos);
        strength = fmaxf(dot(n, to), 0.f) * power * att;
        ls = ls * (dot(n, to) * att);
        cur_l = to;
      } else if (type == 5) {  // area triangle
        float ux = rng_next(re), uy = rng_next(re);
        float sq = sqrtf(ux);
        float bx = 1.0f - sq, by = uy * sq;  // sampleTriangle
        const float3 p2 = f3(L.v1_strength.x, L.v1_strength.y, L.v1_strength.z);
        const float3 p3 = f3(L.v2_angle.x, L.v2_angle.y, L.v2_angle.z);
        float3 lp = v0 * (1.0f - bx - by) + p2 * bx + p3 * by;  // blerp
        float3 ldir = lp - pos;
        float3 ln = nrmz(cross(p2 - v0, p3 - v0));
        float d = length(ldir);
        ldir = ldir * __fdividef(1.0f, d);
        float att = __fdividef(1.0f, L.strengths.x + L.strengths.y * d + L.strengths.z * d * d);
        strength = fmaxf(dot(n, ldir), 0.f) * fmaxf(dot(-ldir, ln), 0.f) * power * att;
        ls = ls * (fmaxf(dot(n, ldir), 0.f) * fmaxf(dot(-ldir, ln), 0.f) * att);
        cur_l = ldir;
        cur_tmax = d - tmin;
      }
      strength_sum += strength;
      if (rng_next(re) < __fdividef(strength, strength_sum)) {
        picked_strength = strength;
        picked_ls = ls;
        tmax = cur_tmax;
        l = cur_l;
      }
    }
    if (strength_sum < 1e-6f || picked_strength < 1e-6f) {
      pdf = 0.f;
      l = f3(0.f);
      return f3(0.f);
    }
    pdf = picked_strength / strength_sum;
    shadow_tmax = tmax;
    traced = true;
    return picked_ls;
  }
  // LIGHT_STRENGTH (binary search over inclusive strengths) or UNIFORM
  float rnd = rng_next(re);
  int i;
  float l_strength = 1.f;
  if (mode == 1) {
    float picked = rnd * sc.light_strength_sum;
    int begin = 0, end = (int)sc.light_count, mid = (begin + end) / 2, cnt = 0;
    while (end - begin > 1 && ++cnt < 100) {
      if (picked <= sc.lights[mid].strengths.w) end = mid + 1;
      else begin = mid;
      mid = (begin + end) / 2;
    }
    l_strength = sc.lights[begin].strengths.w;
    if (begin > 0) l_strength -= sc.lights[begin - 1].strengths.w;
    i = begin;
  } else {
    i = (int)(rnd * (float)sc.light_count) - (int)rnd;
  }
  const DevLight L = sc.lights[i];
  const float4 lsum = sc.light_sum[i];
  float3 ls = f3(lsum.x, lsum.y, lsum.z);
  float tmax = 1000.0f;
  const int type = (int)L.v0_type.w;
  const float3 v0 = f3(L.v0_type.x, L.v0_type.y, L.v0_type.z);
  if (type == 1) {
    float d = length(pos - v0);
    float att = __fdividef(1.0f, L.strengths.x + L.strengths.y * d + L.strengths.z * d * d);
    float3 ndir = -f3(L.dir_angle2.x, L.dir_angle2.y, L.dir_angle2.z);
    ls = ls * (fmaxf(dot(n, ndir), 0.f) * att);
    l = nrmz(ndir);
  } else if (type == 2) {
    float d = length(pos - v0);
    float att = __fdividef(1.0f, L.strengths.x + L.strengths.y * d + L.strengths.z * d * d);
    float3 to = nrmz(v0 - pos);
    ls = ls * (fmaxf(dot(n, to), 0.f) * att);
    l = to;
  } else if (type == 5) {
    float ux = rng_next(re), uy = rng_next(re);
    float sq = sqrtf(ux);
    float bx = 1.0f - sq, by = uy * sq;
    const float3 p2 = f3(L.v1_strength.x, L.v1_strength.y, L.v1_strength.z);
    const float3 p3 = f3(L.v2_angle.x, L.v2_angle.y, L.v2_angle.z);
    float3 lp = v0 * (1.0f - bx - by) + p2 * bx + p3 * by;
    float3 ldir = lp - pos;
    float3 lnr = cross(p2 - v0, p3 - v0);
    float area = .5f * length(lnr);
    float3 ln = nrmz(lnr);
    float d = length(ldir);
    ldir = ldir * __fdividef(1.0f, d);
    float att = __fdividef(1.0f, L.strengths.x + L.strengths.y * d + L.strengths.z * d * d);
    ls = ls * (fmaxf(dot(n, ldir), 0.f) * fmaxf(dot(-ldir, ln), 0.f) * att * area);
    l = ldir;
    tmax = d - tmin;
  }
  if (length(ls) < 1e-6f) {
    pdf = 0.f;
    l = f3(0.f);
    return f3(0.f);
  }
  pdf = 1.0f;
  shadow_tmax = tmax;
  traced = true;
  if (mode == 1) return ls * sc.light_strength_sum / l_strength;
  return ls * (float)sc.light_count;
}

// One bounce of shading for every entry of ray queue k&1.
PBRT_D uint32_t spread3(uint32_t v) {  // 3-bit value -> bits 0, 3, 6
  return (v & 1u) | ((v & 2u) << 2) | ((v & 4u) << 4);
}
// Sort key of a ray: octant of its direction over the Morton cell of its
// origin in the BVH root's box (8 cells per axis).
PBRT_D uint16_t ray_key(const SceneView& sc, float3 o, float3 d) {
  const float4 r0 = __ldg(reinterpret_cast<const float4*>(sc.nodes));
  const uint32_t e = __float_as_uint(r0.w);
  const float sx = __uint_as_float(((e >> 0) & 0xffu) << 23) * 255.f;
  const float sy = __uint_as_float(((e >> 8) & 0xffu) << 23) * 255.f;
  const float sz = __uint_as_float(((e >> 16) & 0xffu) << 23) * 255.f;
  const uint32_t cx = (uint32_t)min(max((int)((o.x - r0.x) / sx * 8.f), 0), 7);
  const uint32_t cy = (uint32_t)min(max((int)((o.y - r0.y) / sy * 8.f), 0), 7);
  const uint32_t cz = (uint32_t)min(max((int)((o.z - r0.z) / sz * 8.f), 0), 7);
  const uint32_t oct = (d.x < 0.f ? 1u : 0u) | (d.y < 0.f ? 2u : 0u) | (d.z < 0.f ? 4u : 0u);
  return (uint16_t)((oct << 9) | spread3(cx) | (spread3(cy) << 1) | (spread3(cz) << 2));
}

__global__ void k_sort_hist(const uint32_t* __restrict__ count_ptr, const uint16_t* __restrict__ keys,
                            uint32_t* __restrict__ bins) {
  __shared__ uint32_t h[kSortBins];
  for (int i = threadIdx.x; i < kSortBins; i += blockDim.x) h[i] = 0;
  __syncthreads();
  const uint32_t n = *((volatile const uint32_t*)count_ptr);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) atomicAdd(&h[keys[i]], 1u);
  __syncthreads();
  for (int i = threadIdx.x; i < kSortBins; i += blockDim.x)
    if (h[i]) atomicAdd(&bins[i], h[i]);
}

// Exclusive scan of the kSortBins counts in place (one CTA of 1024 threads).
__global__ void __launch_bounds__(1024) k_sort_scan(uint32_t* __restrict__ bins) {
  __shared__ uint32_t warp_sums[32];
  constexpr int kPer = kSortBins / 1024;
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  uint32_t v[kPer], sum = 0;
#pragma unroll
  for (int k = 0; k < kPer; ++k) {
    v[k] = bins[t * kPer + k];
    sum += v[k];
  }
  uint32_t incl = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) warp_sums[w] = incl;
  __syncthreads();
  if (w == 0) {
    uint32_t ws = warp_sums[lane], wi = ws;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += y;
    }
    warp_sums[lane] = wi - ws;
  }
  __syncthreads();
  uint32_t run = warp_sums[w] + incl - sum;
#pragma unroll
  for (int k = 0; k < kPer; ++k) {
    bins[t * kPer + k] = run;
    run += v[k];
  }
}

// Scatter by key: lanes with equal keys reserve their slots with one atomic.
template <bool SHADOW>
__global__ void k_sort_scatter(const uint32_t* __restrict__ count_ptr, Queues q, int nq, uint32_t* __restrict__ offs) {
  const uint32_t n = *((volatile const uint32_t*)count_ptr);
  const uint32_t n_round = (n + 31u) & ~31u;
  const int lane = threadIdx.x & 31;
  const uint16_t* keys = SHADOW ? q.skey_t : q.key_t;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_round; i += gridDim.x * blockDim.x) {
    const bool valid = i < n;
    const uint32_t key = valid ? (uint32_t)keys[i] : 0xffffffffu;
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    const int leader = __ffs(peers) - 1;
    uint32_t base = 0;
    if (valid && lane == leader) base = atomicAdd(&offs[key], (uint32_t)__popc(peers));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (!valid) continue;
    const uint32_t dst = base + __popc(peers & ((1u << lane) - 1u));
    if (SHADOW) {
      q.spix[dst] = q.spix_t[i];
      q.sorg[dst] = q.sorg_t[i];
      q.sdir[dst] = q.sdir_t[i];
      q.snee[dst] = q.snee_t[i];
      q.sadd[dst] = q.sadd_t[i];
    } else {
      q.pix[nq][dst] = q.pix_t[i];
      q.org[nq][dst] = q.org_t[i];
      q.dir[nq][dst] = q.dir_t[i];
    }
  }
}

// Shading CTAs resident per SM the register allocation targets (more CTAs,
// fewer registers per thread). Measured at 1080p: 8 (64 registers, a few
// spills) 1.52 ms per frame; 7 1.53; 6 1.56; 5 1.59; 4 (unbounded, ~110
// registers) 1.90; 10 1.79; 12 1.95; 16 2.38.
constexpr int kShadeMinBlocks = 8;
// LM: the light-sampling mode (FrameParams::light_mode) and FIRST: the
// primary bounce, both fixed per instantiation so each launch carries only
// the code of its own mode and bounce (a smaller loop body: fewer
// instruction-fetch stalls).
template <int LM, bool FIRST>
__global__ void __launch_bounds__(128, kShadeMinBlocks) k_shade(SceneView sc, const FrameParams* __restrict__ fpp, Queues q,
                                               Counters* c, GBufferOut g, int k) {
  const FrameParams& fp = *fpp;
  if (*((volatile uint32_t*)&c->stop)) return;  // stopped frame: shade nothing, queue nothing
  const uint32_t count = *((volatile uint32_t*)&c->ray[k & 1]);
  const uint32_t* qpix = q.pix[k & 1];
  const float4* qdir = q.dir[k & 1];
  const int nq = (k + 1) & 1;
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t n_round = (count + 31u) & ~31u;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n_round; i += stride) {
    bool push_ray = false, push_shadow = false;
    float4 ray_o = make_float4(0, 0, 0, 0), ray_d = ray_o, sh_o = ray_o, sh_d = ray_o, sh_nee = ray_o, sh_add = ray_o;
    uint32_t p = 0;
    if (i < count) {
      p = qpix[i];
      const float4 d4 = qdir[i];
      const float3 rdir = f3(d4.x, d4.y, d4.z);
      const float4 h = q.hit[i];
      const uint32_t hit_key = __float_as_uint(h.w);
      const uint2 hit_ip = q.hit_ip[i];
      uint4 r4 = q.rng[p];
      Rng re{r4.x, r4.y, r4.z, r4.w};
      const float4 th4 = q.thr[p];
      float3 thr = f3(th4.x, th4.y, th4.z);
      float4 pv = q.prev[p], al = q.alb[p];
      float3 prev = f3(pv.x, pv.y, pv.z);
      int it = __float_as_int(pv.w), trans = __float_as_int(al.w);
      SurfaceInfo si;
      float3 position;
      uint32_t category;
      const bool miss = hit_key == 0xffffffffu;
      if (miss) miss_payload(si, position, category);
      else position = closest_hit(sc, rdir, hit_ip.x, hit_ip.y, h.y, h.z, si, category);
      // ---- next-event estimation at this vertex (lighting.glsl:246-261) ----
      const float3 o = FIRST ? -nrmz(rdir) : -rdir;
      float3 nee = f3(0.f);
      bool nee_pending = false;
      float3 sl = f3(0.f);
      float shadow_tmax = 0.f;
      if (miss) {
        nee = sky_color(-o) * thr;
      } else {
        float lpdf;
        bool traced;
        const float3 lcol = sample_light(sc, LM, position, si.normal, re, sl, lpdf, shadow_tmax, traced);
        if (traced && !(lcol.x == 0.f && lcol.y == 0.f && lcol.z == 0.f)) {
          const float3 lh = nrmz(sl + o);
          const float3 brdf = brdf_eval(o, sl, lh, si);
          const float bpdf = pdf_brdf(si, o, sl, lh);
          const float w = power_heuristic(lpdf, bpdf);
          const float3 light = f3(0.f) + lcol * brdf * __fdividef(w, lpdf);
          nee = fmin3(thr * light, f3(kMaxRadiance));
          nee_pending = true;
        }
      }
      const float3 add = FIRST ? si.emissive : si.emissive * thr;
      if (FIRST) {
        // ---- G-buffer (ptRaygen.rgen:48-60) ----
        const float3 alb = si.diffuse + si.specular;
        al = make_float4(alb.x, alb.y, alb.z, al.w);
        q.prim_key[p] = hit_key;
        if (fp.write_gbuffer) {
          g.depth[p] = length_rn(position - prev);
          g.normal[p] = make_float2(acosf(si.normal.z), atan2f(si.normal.y, si.normal.x));
          const float cat = (float)category / 255.0f;
          g.material[p] = make_uchar4(f2u8(cat), 0, 0, 0);
          g.albedo[p] = make_uchar4(f2u8(alb.x), f2u8(alb.y), f2u8(alb.z), 255);
        }
      }
      if (nee_pending) {
        push_shadow = true;
        sh_o = make_float4(position.x, position.y, position.z, 0.001f);
        sh_d = make_float4(sl.x, sl.y, sl.z, shadow_tmax);
        sh_nee = make_float4(nee.x, nee.y, nee.z, FIRST ? 0.f : 1.f);
        sh_add = make_float4(add.x, add.y, add.z, 0.f);
      } else {
        float4 rd = q.rad[p];
        float3 rad = f3(rd.x, rd.y, rd.z);
        rad = FIRST ? (f3(0.f) + nee) + add : rad + (nee + add);
        q.rad[p] = make_float4(rad.x, rad.y, rad.z, rd.w);
      }
      // ---- next bounce (ptRaygen.rgen:66-75, lighting.glsl:263-283) ----
      if (!FIRST) it += 1;
      if (!miss && (uint32_t)it < (uint32_t)fp.max_depth && trans < 10) {
        if (si.illum == 7) {
          it -= 1;
          trans += 1;
        }
        const float3 v = nrmz(prev - position);
        prev = position;
        float3 l;
        float pdf;
        const float3 brdf = sample_brdf(si, re, v, l, pdf);
        if (!((brdf.x == 0.f && brdf.y == 0.f && brdf.z == 0.f) || pdf < kEpsilon)) {
          float t = dot(l, si.normal);
          if (si.illum == 7) t = 1.f;
          float3 pt = thr * (brdf * t) * __fdividef(1.0f, pdf);
          bool alive = true;
          if ((uint32_t)it > (uint32_t)fp.min_depth) {
            if (rng_next(re) < kMinTermination) alive = false;
            pt = pt * __fdividef(1.0f, 1.0f - kMinTermination);
          }
          if (alive) {
            thr = pt;
            push_ray = true;
            ray_o = make_float4(position.x, position.y, position.z, 0.001f);
            ray_d = make_float4(l.x, l.y, l.z, 10000.0f);
          }
        }
      }
      q.rng[p] = make_uint4(re.x, re.y, re.z, re.w);
      q.thr[p] = make_float4(thr.x, thr.y, thr.z, 0.f);
      q.prev[p] = make_float4(prev.x, prev.y, prev.z, __int_as_float(it));
      q.alb[p] = make_float4(al.x, al.y, al.z, __int_as_float(trans));
    }
    const int rs = warp_alloc(&c->ray[nq], push_ray);
    if (rs >= 0) {
      if (q.key_t) {
        q.pix_t[rs] = p;
        q.org_t[rs] = ray_o;
        q.dir_t[rs] = ray_d;
        q.key_t[rs] = ray_key(sc, f3(ray_o.x, ray_o.y, ray_o.z), f3(ray_d.x, ray_d.y, ray_d.z));
      } else {
        q.pix[nq][rs] = p;
        q.org[nq][rs] = ray_o;
        q.dir[nq][rs] = ray_d;
      }
    }
    const int ss = warp_alloc(&c->shadow, push_shadow);
    if (ss >= 0) {
      if (q.skey_t) {
        q.spix_t[ss] = p;
        q.sorg_t[ss] = sh_o;
        q.sdir_t[ss] = sh_d;
        q.snee_t[ss] = sh_nee;
        q.sadd_t[ss] = sh_add;
        q.skey_t[ss] = ray_key(sc, f3(sh_o.x, sh_o.y, sh_o.z), f3(sh_d.x, sh_d.y, sh_d.z));
      } else {
        q.spix[ss] = p;
        q.sorg[ss] = sh_o;
        q.sdir[ss] = sh_d;
        q.snee[ss] = sh_nee;
        q.sadd[ss] = sh_add;
      }
    }
  }
}

// ptRaygen.rgen:81-103: clamp, then demodulate (DEMOD_ILLUMINATION_FLOAT) or
// blend progressively in sRGB (FINAL_IMAGE).
__global__ void k_finalize(const FrameParams* __restrict__ fpp, Queues q, float4* __restrict__ out) {
  const FrameParams& fp = *fpp;
  const int N = fp.W * fp.H;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x) {
    const float4 r = q.rad[p];
    float3 fc = clamp3(f3(r.x, r.y, r.z), 0.f, kMaxRadiance);
    if (!fp.final_image) {
      const float4 a = q.alb[p];
      float3 dm = fmin3(fc / (f3(a.x, a.y, a.z) + f3(kEpsilon)), f3(1e3f));
      out[p] = make_float4(dm.x, dm.y, dm.z, 1.f);
    } else {
      if (fp.sample > 0) {
        const float4 pr = out[p];
        const float alpha = 1.0f / (float)(fp.sample + 1);
        fc = mix3(srgb_to_linear(f3(pr.x, pr.y, pr.z)), fc, alpha);
      }
      fc = clamp3(linear_to_srgb(fc), 0.f, 1.f);
      out[p] = make_float4(fc.x, fc.y, fc.z, 1.f);
    }
  }
}

// Row-major RGBA8 texture -> the pool's 4 x 2-texel tiles (texture_tile_index).
__global__ void k_tile_texture(const uchar4* __restrict__ src, uchar4* __restrict__ dst, uint32_t w, uint32_t h) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)w * h) return;
  const uint32_t x = (uint32_t)(i % w), y = (uint32_t)(i / w);
  dst[texture_tile_index(w, x, y)] = src[i];
}

}  // namespace pbrt

// ===========================================================================
// Host objects.
using namespace pbrt;

namespace {

template <class T> int dalloc(T** p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
  return PBRT_OK;
}
template <class T> int upload(T** p, const T* src, size_t count) {
  int st = dalloc(p, count);
  if (st) return st;
  if (count) PBRT_CUDA(cudaMemcpy(*p, src, count * sizeof(T), cudaMemcpyHostToDevice));
  return PBRT_OK;
}

float bits_f(uint32_t u) {
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}

// double-precision 4x4 inverse (column-major in/out), false if singular
bool inverse4(const double* m, double* out) {
  double a[4][8];
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) {
      a[r][c] = m[c * 4 + r];
      a[r][4 + c] = (r == c) ? 1.0 : 0.0;
    }
  for (int c = 0; c < 4; ++c) {
    int piv = c;
    for (int r = c + 1; r < 4; ++r)
      if (std::fabs(a[r][c]) > std::fabs(a[piv][c])) piv = r;
    if (a[piv][c] == 0.0) return false;
    for (int k = 0; k < 8; ++k) std::swap(a[c][k], a[piv][k]);
    double d = a[c][c];
    for (int k = 0; k < 8; ++k) a[c][k] /= d;
    for (int r = 0; r < 4; ++r) {
      if (r == c) continue;
      double f = a[r][c];
      for (int k = 0; k < 8; ++k) a[r][k] -= f * a[c][k];
    }
  }
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) out[c * 4 + r] = a[r][4 + c];
  return true;
}

}  // namespace

struct PbrtScene : pbrt::Object {
  PbrtScene() : Object(pbrt::Kind::Scene) {}
  ~PbrtScene() override {
    for (void* p : allocs) cudaFree(p);
  }
  std::vector<void*> allocs;
  SceneView view{};
  Bvh8Stats stats;
  uint32_t instance_count = 0, tri_count = 0;
  bool transmissive = false;  // some material has illum 7 (refraction)
  template <class T> int up(T** p, const T* src, size_t n) {
    int st = upload(p, src, n);
    if (!st) allocs.push_back((void*)*p);
    return st;
  }
};

struct PbrtPipeline : pbrt::Object {
  PbrtPipeline() : Object(pbrt::Kind::Pipeline) {}
  ~PbrtPipeline() override {
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    for (void* p : allocs) cudaFree(p);
    if (abort_host) cudaFreeHost(abort_host);
    release(scene);
    release(gbuffer);
    release(illumination);
  }
  PbrtScene* scene = nullptr;
  PbrtGBuffer* gbuffer = nullptr;
  PbrtIlluminationBuffer* illumination = nullptr;
  bool write_gbuffer = false;
  int W = 0, H = 0;
  int light_mode = 0, min_depth = 0, max_depth = 2;
  std::vector<void*> allocs;
  Queues q{};
  Counters* ctr = nullptr;
  FrameParams* dev_fp = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  int graph_depth = -1;
  int graph_light_mode = -1;  // the light-sampling mode the captured graph's shading kernels were built for
  int sort_rays = 0;        // schedule: counting sort of the ray and shadow queues before traversal
  int merge_shadow = 1;     // schedule: shadow rays of bounce k-1 traced in bounce k's launch
  int grid_persistent = 0;  // traversal CTAs (persistent warps)
  int grid_shade = 0;       // shading CTAs (grid-stride)
  uint32_t* abort_host = nullptr;  // mapped pinned word (pbrt_pipeline_abort_flag)
  uint32_t* abort_dev = nullptr;
  unsigned long long budget_ns = 0;
  template <class T> int a(T** p, size_t n) {
    int st = dalloc(p, n);
    if (!st) allocs.push_back((void*)*p);
    return st;
  }
};

// Optional per-stage timing (events summed over the frame's launches).
struct StageEvents {
  static constexpr int kCount = 5;  // raygen, closest, shade, shadow, finalize
  cudaEvent_t ev[kCount][2];
  float ms[kCount];
  cudaStream_t stream;
  void begin(int i) { cudaEventRecord(ev[i][0], stream); }
  void end(int i) {
    cudaEventRecord(ev[i][1], stream);
    cudaEventSynchronize(ev[i][1]);
    float t = 0.f;
    cudaEventElapsedTime(&t, ev[i][0], ev[i][1]);
    ms[i] += t;
  }
};

static void launch_shade(int grid, cudaStream_t s, const SceneView& sc, const FrameParams* fp, const Queues& q,
                         Counters* c, const GBufferOut& g, int k, int light_mode) {
  if (light_mode == 1) {
    if (k == 0) k_shade<1, true><<<grid, 128, 0, s>>>(sc, fp, q, c, g, k);
    else k_shade<1, false><<<grid, 128, 0, s>>>(sc, fp, q, c, g, k);
  } else if (light_mode == 2) {
    if (k == 0) k_shade<2, true><<<grid, 128, 0, s>>>(sc, fp, q, c, g, k);
    else k_shade<2, false><<<grid, 128, 0, s>>>(sc, fp, q, c, g, k);
  } else {
    if (k == 0) k_shade<0, true><<<grid, 128, 0, s>>>(sc, fp, q, c, g, k);
    else k_shade<0, false><<<grid, 128, 0, s>>>(sc, fp, q, c, g, k);
  }
}

static int record_frame(PbrtPipeline* pp, cudaStream_t s, StageEvents* ev) {
  const int N = pp->W * pp->H;
  const SceneView sc = pp->scene->view;
  Queues q = pp->q;
  if (!pp->sort_rays) {  // shading writes the queues directly
    q.key_t = nullptr;
    q.skey_t = nullptr;
  }
  const bool merge = pp->merge_shadow != 0;
  GBufferOut g{};
  if (pp->gbuffer) {
    g.depth = pp->gbuffer->depth.ptr<float>();
    g.normal = pp->gbuffer->normal.ptr<float2>();
    g.material = pp->gbuffer->material.ptr<uchar4>();
    g.albedo = pp->gbuffer->albedo.ptr<uchar4>();
  }
  float4* out = pp->illumination->images[0].ptr<float4>();
  const int blocks_px = std::min((N + 255) / 256, 152 * 8);
  k_frame_begin<<<1, 1, 0, s>>>(pp->ctr, pp->dev_fp);
  if (ev) ev->begin(0);
  k_raygen<<<blocks_px, 256, 0, s>>>(pp->dev_fp, q);
  if (ev) ev->end(0);
  // Bounce k traces the rays that leave vertex k-1. Transmissive vertices do
  // not count towards the depth (ptRaygen.rgen:69, up to 10 of them).
  const int bounces = pp->max_depth + 1 + (pp->scene->transmissive ? 10 : 0);
  for (int k = 0; k < bounces; ++k) {
    if (merge) {
      k_bounce_begin_merged<<<1, 1, 0, s>>>(pp->ctr, k);
      if (ev) ev->begin(1);
      if (k == 0) k_traverse_packet<<<pp->grid_persistent, 128, 0, s>>>(sc, q, pp->ctr);
      else k_traverse<4><<<pp->grid_persistent, 128, 0, s>>>(sc, q, pp->ctr, k, QueryIO{});
      if (ev) ev->end(1);
      k_shadow_consumed<<<1, 1, 0, s>>>(pp->ctr);
    } else {
      k_bounce_begin<<<1, 1, 0, s>>>(pp->ctr, k);
      if (ev) ev->begin(1);
      if (k == 0) k_traverse_packet<<<pp->grid_persistent, 128, 0, s>>>(sc, q, pp->ctr);
      else k_traverse<0><<<pp->grid_persistent, 128, 0, s>>>(sc, q, pp->ctr, k, QueryIO{});
      if (ev) ev->end(1);
    }
    if (ev) ev->begin(2);
    launch_shade(pp->grid_shade, s, sc, pp->dev_fp, q, pp->ctr, g, k, pp->light_mode);
    if (pp->sort_rays) {
      const int nq = (k + 1) & 1;
      uint32_t* bins_r = q.bins;
      uint32_t* bins_s = q.bins + kSortBins;
      const int sort_grid = std::min((N + 255) / 256, 152 * 4);
      cudaMemsetAsync(q.bins, 0, 2 * kSortBins * sizeof(uint32_t), s);
      if (k + 1 < bounces) {
        k_sort_hist<<<sort_grid, 256, 0, s>>>(&pp->ctr->ray[nq], q.key_t, bins_r);
        k_sort_scan<<<1, 1024, 0, s>>>(bins_r);
        k_sort_scatter<false><<<sort_grid, 256, 0, s>>>(&pp->ctr->ray[nq], q, nq, bins_r);
      }
      k_sort_hist<<<sort_grid, 256, 0, s>>>(&pp->ctr->shadow, q.skey_t, bins_s);
      k_sort_scan<<<1, 1024, 0, s>>>(bins_s);
      k_sort_scatter<true><<<sort_grid, 256, 0, s>>>(&pp->ctr->shadow, q, 0, bins_s);
    }
    if (ev) ev->end(2);
    if (!merge || k + 1 == bounces) {  // merged: the last bounce's shadow rays go alone
      if (ev) ev->begin(3);
      if (merge) k_shadow_begin<<<1, 1, 0, s>>>(pp->ctr);
      k_traverse<1><<<pp->grid_persistent, 128, 0, s>>>(sc, q, pp->ctr, k, QueryIO{});
      if (ev) ev->end(3);
      k_bounce_end<<<1, 1, 0, s>>>(pp->ctr);
    }
  }
  if (ev) ev->begin(4);
  k_finalize<<<blocks_px, 256, 0, s>>>(pp->dev_fp, q, out);
  if (ev) ev->end(4);
  return check_launch("path tracer frame");
}

extern "C" {

PBRT_API int pbrt_scene_create(const PbrtSceneDesc* d, PbrtScene** out) {
  return pbrt_scene_create_ex(d, PBRT_BUILD_PREFER_FAST_TRACE, out);
}

PBRT_API int pbrt_scene_create_ex(const PbrtSceneDesc* d, uint32_t build_flags, PbrtScene** out) {
  if (!out || !d) return fail(PBRT_ERROR_INVALID_ARGUMENT, "scene: null argument");
  if (build_flags & ~(uint32_t)PBRT_BUILD_PREFER_FAST_BUILD)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "scene: unknown build flags 0x%x", build_flags);
  const bool device_build = (build_flags & PBRT_BUILD_PREFER_FAST_BUILD) != 0;
  *out = nullptr;
  if (d->mesh_count == 0 || d->instance_count == 0 || !d->meshes || !d->instances || !d->materials)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "scene: needs meshes, instances and materials");
  if (d->light_count > 0 && !d->lights) return fail(PBRT_ERROR_INVALID_ARGUMENT, "scene: lights missing");
  if (d->texture_count == 0 || !d->textures || !d->mesh_textures)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "scene: needs a texture table (entry 0 = 1x1 white default)");
  auto* sc = new (std::nothrow) PbrtScene();
  if (!sc) return fail(PBRT_ERROR_OUT_OF_MEMORY, "scene: host allocation");
  // --- mesh pools
  std::vector<DevMesh> meshes(d->mesh_count);
  std::vector<float> pos, nor, uv;
  std::vector<uint32_t> idx;
  for (uint32_t m = 0; m < d->mesh_count; ++m) {
    const PbrtMeshDesc& md = d->meshes[m];
    if (!md.positions || !md.normals || !md.uvs || !md.indices || md.index_count % 3 != 0 ||
        (md.index_stride != 2 && md.index_stride != 4)) {
      delete sc;
      return fail(PBRT_ERROR_INVALID_ARGUMENT, "scene: mesh %u malformed (indices multiple of 3, stride 2 or 4)", m);
    }
    DevMesh& dm = meshes[m];
    dm.vbase = (uint32_t)(pos.size() / 3);
    dm.ibase = (uint32_t)idx.size();
    dm.index_stride = md.index_stride;
    for (int s = 0; s < 5; ++s) {
      int t = d->mesh_textures[5 * m + s];
      if (t < 0 || (uint32_t)t >= d->texture_count) {
        delete sc;
        return fail(PBRT_ERROR_INVALID_ARGUMENT, "scene: mesh %u texture slot %d -> %d out of range", m, s, t);
      }
      dm.tex[s] = t;
    }
    pos.insert(pos.end(), md.positions, md.positions + 3 * (size_t)md.vertex_count);
    nor.insert(nor.end(), md.normals, md.normals + 3 * (size_t)md.vertex_count);
    uv.insert(uv.end(), md.uvs, md.uvs + 2 * (size_t)md.vertex_count);
    if (md.index_stride == 4) {
      const uint32_t* ii = (const uint32_t*)md.indices;
      for (uint32_t k = 0; k < md.index_count; ++k) {
        if (ii[k] >= md.vertex_count) {
          delete sc;
          return fail(PBRT_ERROR_INVALID_ARGUMENT, "scene: mesh %u index %u out of range", m, ii[k]);
        }
      }
      idx.insert(idx.end(), ii, ii + md.index_count);
    } else {
      const uint16_t* ii = (const uint16_t*)md.indices;
      for (uint32_t k = 0; k < md.index_count; ++k)
        if (ii[k] >= md.vertex_count) {
          delete sc;
          return fail(PBRT_ERROR_INVALID_ARGUMENT, "scene: mesh %u index %u out of range", m, ii[k]);
        }
      for (uint32_t k = 0; k < md.index_count; k += 2) {
        uint32_t lo = ii[k], hi = (k + 1 < md.index_count) ? ii[k + 1] : 0u;
        idx.push_back(lo | (hi << 16));
      }
      idx.push_back(0u);  // unpackIndex may read one word past an odd-length buffer
    }
  }
  // --- instances: flatten to world-space triangles (instance-major order)
  std::vector<DevInstance> inst(d->instance_count);
  size_t total = 0;
  for (uint32_t i = 0; i < d->instance_count; ++i) {
    const PbrtObjectInstance& oi = d->instances[i];
    if (oi.mesh_id < 0 || (uint32_t)oi.mesh_id >= d->mesh_count) {
      delete sc;
      return fail(PBRT_ERROR_INVALID_ARGUMENT, "scene: instance %u mesh %d out of range", i, oi.mesh_id);
    }
    total += d->meshes[oi.mesh_id].index_count / 3;
  }
  if (total == 0 || total > 0x7fffffffu) {
    delete sc;
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "scene: %zu triangles", total);
  }
  std::vector<float> world(9 * total);
  std::vector<uint32_t> tri_inst(total), tri_prim(total);
  size_t t = 0;
  bool any_alpha = false;
  for (uint32_t i = 0; i < d->instance_count; ++i) {
    const PbrtObjectInstance& oi = d->instances[i];
    DevInstance& di = inst[i];
    const float* M = oi.object_mat;
    for (int c = 0; c < 4; ++c) di.obj.c[c] = make_float4(M[4 * c], M[4 * c + 1], M[4 * c + 2], M[4 * c + 3]);
    double md[16], inv[16];
    for (int k = 0; k < 16; ++k) md[k] = M[k];
    if (!inverse4(md, inv)) {
      delete sc;
      return fail(PBRT_ERROR_INVALID_ARGUMENT, "scene: instance %u object matrix is singular", i);
    }
    // transpose(inverse(M)) columns: column c = row c of inverse(M)
    for (int c = 0; c < 3; ++c)
      di.nrm[c] = make_float4((float)inv[0 * 4 + c], (float)inv[1 * 4 + c], (float)inv[2 * 4 + c], 0.f);
    di.mesh = oi.mesh_id;
    di.index_stride = oi.index_stride;
    di.vbase = meshes[oi.mesh_id].vbase;
    di.ibase = meshes[oi.mesh_id].ibase;
    for (int s = 0; s < 5; ++s) di.tex[s] = meshes[oi.mesh_id].tex[s];
    di.opaque = d->instance_opaque ? (d->instance_opaque[i] ? 1u : 0u) : 1u;
    di.pad = 0;
    if (!di.opaque) any_alpha = true;
    const PbrtMeshDesc& md_ = d->meshes[oi.mesh_id];
    const uint32_t ntri = md_.index_count / 3;
    for (uint32_t p = 0; p < ntri; ++p, ++t) {
      for (int k = 0; k < 3; ++k) {
        uint32_t vi = md_.index_stride == 4 ? ((const uint32_t*)md_.indices)[3 * p + k]
                                            : ((const uint16_t*)md_.indices)[3 * p + k];
        const float* v = md_.positions + 3 * (size_t)vi;
        // (objectMat * vec4(v, 1)).xyz in FP32, GLSL column order
        for (int a = 0; a < 3; ++a) {
          float s = M[0 * 4 + a] * v[0];
          s = s + M[1 * 4 + a] * v[1];
          s = s + M[2 * 4 + a] * v[2];
          s = s + M[3 * 4 + a] * 1.0f;
          world[9 * t + 3 * k + a] = s;
        }
      }
      tri_inst[t] = i;
      tri_prim[t] = p;
    }
  }
  std::vector<Node8> nodes;
  std::vector<float4> tris;
  float4* dtris = nullptr;
  Node8* dnodes = nullptr;
  if (device_build) {
    // linear BVH built on the device, written there (bvh_gpu.cu)
    const int bst = build_bvh8_device(world.data(), tri_inst.data(), tri_prim.data(), total, kStackSize - 3, &dnodes,
                                      &dtris, &sc->stats);
    if (bst) {
      delete sc;
      return bst;
    }
    sc->allocs.push_back(dnodes);
    sc->allocs.push_back(dtris);
  } else {
    std::vector<uint32_t> order;
    build_bvh8(world.data(), total, nodes, order, &sc->stats);
    tris.resize(3 * total);
    for (size_t s = 0; s < total; ++s) {
      const uint32_t o = order[s];
      const float* w = &world[9 * (size_t)o];
      tris[3 * s + 0] = make_float4(w[0], w[1], w[2], bits_f(o));
      tris[3 * s + 1] = make_float4(w[3], w[4], w[5], bits_f(tri_inst[o]));
      tris[3 * s + 2] = make_float4(w[6], w[7], w[8], bits_f(tri_prim[o]));
    }
  }
  if (sc->stats.depth >= kStackSize - 2) {
    delete sc;
    return fail(PBRT_ERROR_UNSUPPORTED, "scene: BVH depth %d exceeds the traversal stack", sc->stats.depth);
  }
  // --- textures
  std::vector<DevTexture> texd(d->texture_count);
  size_t texels = 0, max_texels = 0;
  for (uint32_t i = 0; i < d->texture_count; ++i) {
    const PbrtTextureDesc& td = d->textures[i];
    if (!td.rgba8 || td.width == 0 || td.height == 0) {
      delete sc;
      return fail(PBRT_ERROR_INVALID_ARGUMENT, "scene: texture %u empty", i);
    }
    texd[i].offset = texels;
    texd[i].w = td.width;
    texd[i].h = td.height;
    // 4 x 2-texel tiles: the width padded to a multiple of 4, the height of 2
    texels += (size_t)((td.width + 3) & ~3u) * ((td.height + 1) & ~1u);
    max_texels = std::max(max_texels, (size_t)td.width * td.height);
  }
  int st = PBRT_OK;
  uchar4* texpool = nullptr;
  st = dalloc(&texpool, texels);
  if (!st) sc->allocs.push_back(texpool);
  if (!st && cudaMemset(texpool, 0, texels * sizeof(uchar4)) != cudaSuccess) st = cuda_fail(cudaGetLastError(), "texture pool");
  // each texture uploaded row-major into a staging buffer, then tiled on the device
  uchar4* staging = nullptr;
  if (!st) st = dalloc(&staging, max_texels);
  for (uint32_t i = 0; !st && i < d->texture_count; ++i) {
    const uint32_t w = d->textures[i].width, h = d->textures[i].height;
    cudaError_t e = cudaMemcpy(staging, d->textures[i].rgba8, (size_t)w * h * 4, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      st = cuda_fail(e, "texture upload");
      break;
    }
    const size_t n = (size_t)w * h;
    k_tile_texture<<<(unsigned)((n + 255) / 256), 256>>>(staging, texpool + texd[i].offset, w, h);
    st = check_launch("texture tiling");
  }
  if (staging) {
    cudaDeviceSynchronize();  // the tiling kernels read the staging buffer
    cudaFree(staging);
  }
  std::vector<DevMaterial> mats(d->mesh_count);
  std::memcpy(mats.data(), d->materials, sizeof(DevMaterial) * d->mesh_count);
  for (const DevMaterial& m : mats)
    if ((int)m.transmittance_illum.w == 7) sc->transmissive = true;
  std::vector<DevLight> lights(std::max<uint32_t>(1, d->light_count));
  if (d->light_count) std::memcpy(lights.data(), d->lights, sizeof(DevLight) * d->light_count);
  // sampleLight's per-light colour sum and power, once (same FP32 order as the shader's expressions)
  std::vector<float4> light_sum(lights.size());
  for (size_t i = 0; i < lights.size(); ++i) {
    const DevLight& L = lights[i];
    const float sx = (L.col_ambient.x + L.col_diffuse.x) + L.col_specular.x;
    const float sy = (L.col_ambient.y + L.col_diffuse.y) + L.col_specular.y;
    const float sz = (L.col_ambient.z + L.col_diffuse.z) + L.col_specular.z;
    const float sw = (L.col_ambient.w + L.col_diffuse.w) + L.col_specular.w;
    light_sum[i] = make_float4(sx, sy, sz, ((sx + sy) + sz) + sw);
  }
  SceneView& v = sc->view;
  DevInstance* dinst = nullptr;
  DevMesh* dmesh = nullptr;
  DevMaterial* dmat = nullptr;
  DevLight* dlight = nullptr;
  float4* dlsum = nullptr;
  float *dpos = nullptr, *dnor = nullptr, *duv = nullptr;
  uint32_t* didx = nullptr;
  DevTexture* dtex = nullptr;
  if (!st && !device_build) st = sc->up(&dtris, tris.data(), tris.size());
  if (!st && !device_build) st = sc->up(&dnodes, nodes.data(), nodes.size());
  if (!st) st = sc->up(&dinst, inst.data(), inst.size());
  if (!st) st = sc->up(&dmesh, meshes.data(), meshes.size());
  if (!st) st = sc->up(&dmat, mats.data(), mats.size());
  if (!st) st = sc->up(&dlight, lights.data(), lights.size());
  if (!st) st = sc->up(&dlsum, light_sum.data(), light_sum.size());
  if (!st) st = sc->up(&dpos, pos.data(), pos.size());
  if (!st) st = sc->up(&dnor, nor.data(), nor.size());
  if (!st) st = sc->up(&duv, uv.data(), uv.size());
  if (!st) st = sc->up(&didx, idx.data(), idx.size());
  if (!st) st = sc->up(&dtex, texd.data(), texd.size());
  if (st) {
    delete sc;
    return st;
  }
  v.tris = dtris;
  v.nodes = dnodes;
  v.instances = dinst;
  v.meshes = dmesh;
  v.materials = dmat;
  v.lights = dlight;
  v.light_sum = dlsum;
  v.pos = dpos;
  v.nor = dnor;
  v.uv = duv;
  v.idx = didx;
  v.textures = dtex;
  v.texels = texpool;
  v.light_count = d->light_count;
  v.light_strength_sum = d->light_count ? d->lights[d->light_count - 1].inclusive_strength : 0.f;
  v.tri_count = (uint32_t)total;
  v.any_alpha = any_alpha ? 1 : 0;
  sc->instance_count = d->instance_count;
  sc->tri_count = (uint32_t)total;
  *out = sc;
  return PBRT_OK;
}

PBRT_API int pbrt_scene_info(const PbrtScene* s, PbrtSceneInfo* info) {
  if (!checked<const PbrtScene>((void*)s, Kind::Scene) || !info) return fail(PBRT_ERROR_INVALID_ARGUMENT, "not a scene");
  info->triangle_count = s->tri_count;
  info->instance_count = s->instance_count;
  info->bvh_nodes = (uint32_t)s->stats.nodes;
  info->bvh_depth = (uint32_t)s->stats.depth;
  info->bvh_bytes = (uint64_t)s->stats.nodes * sizeof(Node8);
  info->triangle_bytes = (uint64_t)s->tri_count * 48u;
  info->build_ms = s->stats.build_ms;
  info->light_count = s->view.light_count;
  return PBRT_OK;
}

PBRT_API int pbrt_scene_trace_rays(PbrtScene* s, const void* origins_tmin, const void* directions_tmax, uint32_t n,
                                   int32_t any_hit, void* hits_out, void* scratch_u32x2, pbrt_stream_t stream) {
  if (!checked<PbrtScene>(s, Kind::Scene) || (n && (!origins_tmin || !directions_tmax || !hits_out || !scratch_u32x2)))
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "trace_rays: bad arguments");
  if (n == 0) return PBRT_OK;
  uint32_t* work = (uint32_t*)scratch_u32x2;
  PBRT_CUDA(cudaMemsetAsync(work, 0, 2 * sizeof(uint32_t), stream));
  int dev = 0, sms = 0;
  PBRT_CUDA(cudaGetDevice(&dev));
  PBRT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  QueryIO io{(const float4*)origins_tmin, (const float4*)directions_tmax, (float4*)hits_out, n, work, work + 1};
  if (any_hit) k_traverse<3><<<sms * 8, 128, 0, stream>>>(s->view, Queues{}, nullptr, 0, io);
  else k_traverse<2><<<sms * 8, 128, 0, stream>>>(s->view, Queues{}, nullptr, 0, io);
  return check_launch("k_traverse (ray query)");
}

PBRT_API int pbrt_pipeline_create(PbrtScene* scene, PbrtGBuffer* g, PbrtIlluminationBuffer* illumination,
                                  int32_t write_g_buffer, PbrtPipeline** out) {
  if (!out) return fail(PBRT_ERROR_INVALID_ARGUMENT, "pipeline: null output");
  *out = nullptr;
  if (!checked<PbrtScene>(scene, Kind::Scene) || !checked<PbrtIlluminationBuffer>(illumination, Kind::Illumination))
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "pipeline: bad scene or illumination handle");
  if (g && !checked<PbrtGBuffer>(g, Kind::GBuffer)) return fail(PBRT_ERROR_INVALID_ARGUMENT, "pipeline: bad GBuffer");
  if (write_g_buffer && !g) return fail(PBRT_ERROR_INVALID_ARGUMENT, "pipeline: write_g_buffer needs a GBuffer");
  if (illumination->type != PBRT_ILLUMINATION_DEMODULATED_FLOAT && illumination->type != PBRT_ILLUMINATION_FINAL_FLOAT)
    return fail(PBRT_ERROR_UNSUPPORTED,
                "pipeline: illumination must be DemodulatedFloat (DEMOD_ILLUMINATION_FLOAT) or FinalFloat (FINAL_IMAGE)");
  if (g && (g->width != illumination->width || g->height != illumination->height))
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "pipeline: GBuffer and illumination sizes differ");
  auto* pp = new (std::nothrow) PbrtPipeline();
  if (!pp) return fail(PBRT_ERROR_OUT_OF_MEMORY, "pipeline: host allocation");
  pp->scene = scene;
  retain(scene);
  pp->illumination = illumination;
  retain(illumination);
  if (g) {
    pp->gbuffer = g;
    retain(g);
  }
  pp->write_gbuffer = write_g_buffer != 0;
  pp->W = (int)illumination->width;
  pp->H = (int)illumination->height;
  // PBRTPipeline.cpp:92-96: uniform light sampling above 800 lights
  pp->light_mode = scene->view.light_count > 800 ? 2 : 0;
  const size_t N = (size_t)pp->W * pp->H;
  int st = PBRT_OK;
  Queues& q = pp->q;
  for (int i = 0; i < 2 && !st; ++i) {
    st = pp->a(&q.pix[i], N);
    if (!st) st = pp->a(&q.org[i], N);
    if (!st) st = pp->a(&q.dir[i], N);
  }
  if (!st) st = pp->a(&q.hit, N);
  if (!st) st = pp->a(&q.hit_ip, N);
  if (!st) st = pp->a(&q.spix, N);
  if (!st) st = pp->a(&q.sorg, N);
  if (!st) st = pp->a(&q.sdir, N);
  if (!st) st = pp->a(&q.snee, N);
  if (!st) st = pp->a(&q.sadd, N);
  if (!st) st = pp->a(&q.rng, N);
  if (!st) st = pp->a(&q.thr, N);
  if (!st) st = pp->a(&q.rad, N);
  if (!st) st = pp->a(&q.prev, N);
  if (!st) st = pp->a(&q.alb, N);
  if (!st) st = pp->a(&q.prim_key, N);
  if (!st) st = pp->a(&pp->ctr, 1);
  if (!st) st = pp->a(&pp->dev_fp, 1);
  if (!st) {
    cudaError_t e = cudaMemset(pp->ctr, 0, sizeof(Counters));
    if (e != cudaSuccess) st = cuda_fail(e, "pipeline state");
  }
  if (!st) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    pp->grid_persistent = sms * kTraverseMinBlocks;  // the resident 128-thread traversal CTAs
    pp->grid_shade = sms * kShadeMinBlocks;
  }
  if (st) {
    delete pp;
    return st;
  }
  *out = pp;
  return PBRT_OK;
}

PBRT_API int pbrt_pipeline_set_config(PbrtPipeline* pp, int32_t light_sampling, int32_t min_recursion_depth,
                                      int32_t max_recursion_depth) {
  if (!checked<PbrtPipeline>(pp, Kind::Pipeline)) return fail(PBRT_ERROR_INVALID_ARGUMENT, "not a pipeline");
  if (light_sampling < 0 || light_sampling > 2 || min_recursion_depth < 0 || max_recursion_depth < 0 ||
      max_recursion_depth > 64)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "pipeline config: light_sampling %d, depth [%d, %d]", light_sampling,
                min_recursion_depth, max_recursion_depth);
  pp->light_mode = light_sampling;
  pp->min_depth = min_recursion_depth;
  pp->max_depth = max_recursion_depth;
  return PBRT_OK;
}

static FrameParams frame_params(const PbrtPipeline* pp, const PbrtPushConstants* pc) {
  FrameParams fp;
  for (int c = 0; c < 4; ++c) {
    fp.inv_view.c[c] = make_float4(pc->view_inverse[4 * c], pc->view_inverse[4 * c + 1], pc->view_inverse[4 * c + 2],
                                   pc->view_inverse[4 * c + 3]);
    fp.inv_proj.c[c] = make_float4(pc->proj_inverse[4 * c], pc->proj_inverse[4 * c + 1], pc->proj_inverse[4 * c + 2],
                                   pc->proj_inverse[4 * c + 3]);
  }
  fp.frame = pc->frame_number;
  fp.sample = pc->sample_number;
  fp.W = pp->W;
  fp.H = pp->H;
  fp.min_depth = pp->min_depth;
  fp.max_depth = pp->max_depth;
  fp.light_mode = pp->light_mode;
  fp.final_image = pp->illumination->type == PBRT_ILLUMINATION_FINAL_FLOAT ? 1 : 0;
  fp.write_gbuffer = pp->write_gbuffer ? 1 : 0;
  fp.abort_flag = pp->abort_dev;
  fp.budget_ns = pp->budget_ns;
  return fp;
}

PBRT_API int pbrt_pipeline_trace(PbrtPipeline* pp, const PbrtPushConstants* pc, pbrt_stream_t stream) {
  if (!checked<PbrtPipeline>(pp, Kind::Pipeline) || !pc) return fail(PBRT_ERROR_INVALID_ARGUMENT, "trace: bad arguments");
  k_set_params<<<1, 1, 0, stream>>>(pp->dev_fp, frame_params(pp, pc));
  int st = check_launch("k_set_params");
  if (st) return st;
  const int bounces = pp->max_depth + 1 + (pp->scene->transmissive ? 10 : 0);
  if (!pp->graph_exec || pp->graph_depth != bounces || pp->graph_light_mode != pp->light_mode) {
    if (pp->graph_exec) cudaGraphExecDestroy(pp->graph_exec);
    pp->graph_exec = nullptr;
    cudaStream_t cap;
    PBRT_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    cudaGraph_t graph;
    cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    st = e == cudaSuccess ? record_frame(pp, cap, nullptr) : cuda_fail(e, "begin capture");
    cudaError_t e2 = cudaStreamEndCapture(cap, &graph);
    cudaStreamDestroy(cap);
    if (st) return st;
    if (e2 != cudaSuccess) return cuda_fail(e2, "end capture");
    e = cudaGraphInstantiate(&pp->graph_exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(e, "graph instantiate");
    pp->graph_depth = bounces;
    pp->graph_light_mode = pp->light_mode;
  }
  PBRT_CUDA(cudaGraphLaunch(pp->graph_exec, stream));
  return PBRT_OK;
}

PBRT_API int pbrt_pipeline_profile(PbrtPipeline* pp, const PbrtPushConstants* pc, pbrt_stream_t stream,
                                   PbrtStageTimes* out) {
  if (!checked<PbrtPipeline>(pp, Kind::Pipeline) || !pc || !out)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "profile: bad arguments");
  StageEvents ev;
  for (int i = 0; i < StageEvents::kCount; ++i) {
    ev.ms[i] = 0.f;
    PBRT_CUDA(cudaEventCreate(&ev.ev[i][0]));
    PBRT_CUDA(cudaEventCreate(&ev.ev[i][1]));
  }
  ev.stream = stream;
  k_set_params<<<1, 1, 0, stream>>>(pp->dev_fp, frame_params(pp, pc));
  Counters before;
  PBRT_CUDA(cudaMemcpyAsync(&before, pp->ctr, sizeof(Counters), cudaMemcpyDeviceToHost, stream));
  PBRT_CUDA(cudaStreamSynchronize(stream));
  int st = record_frame(pp, stream, &ev);
  PBRT_CUDA(cudaStreamSynchronize(stream));
  Counters after;
  PBRT_CUDA(cudaMemcpy(&after, pp->ctr, sizeof(Counters), cudaMemcpyDeviceToHost));
  for (int i = 0; i < StageEvents::kCount; ++i) {
    cudaEventDestroy(ev.ev[i][0]);
    cudaEventDestroy(ev.ev[i][1]);
  }
  if (st) return st;
  out->raygen_ms = ev.ms[0];
  out->trace_closest_ms = ev.ms[1];
  out->shade_ms = ev.ms[2];
  out->trace_shadow_ms = ev.ms[3];
  out->finalize_ms = ev.ms[4];
  out->closest_rays = (after.rays_primary - before.rays_primary) + (after.rays_extension - before.rays_extension);
  out->shadow_rays = after.rays_shadow - before.rays_shadow;
  out->closest_nodes = after.nodes_closest - before.nodes_closest;
  out->closest_tris = after.tris_closest - before.tris_closest;
  out->shadow_nodes = after.nodes_shadow - before.nodes_shadow;
  out->shadow_tris = after.tris_shadow - before.tris_shadow;
  out->closest_launches = (uint32_t)(pp->graph_depth > 0 ? pp->graph_depth : pp->max_depth + 1);
  return PBRT_OK;
}

PBRT_API int pbrt_pipeline_stats(PbrtPipeline* pp, pbrt_stream_t stream, PbrtTraceStats* out) {
  if (!checked<PbrtPipeline>(pp, Kind::Pipeline) || !out) return fail(PBRT_ERROR_INVALID_ARGUMENT, "stats: bad arguments");
  Counters c;
  PBRT_CUDA(cudaMemcpyAsync(&c, pp->ctr, sizeof(Counters), cudaMemcpyDeviceToHost, stream));
  PBRT_CUDA(cudaStreamSynchronize(stream));
  out->frames = c.frames;
  out->primary_rays = c.rays_primary;
  out->extension_rays = c.rays_extension;
  out->shadow_rays = c.rays_shadow;
  out->error_flags = c.error;
  return PBRT_OK;
}

PBRT_API int pbrt_pipeline_reset_stats(PbrtPipeline* pp, pbrt_stream_t stream) {
  if (!checked<PbrtPipeline>(pp, Kind::Pipeline)) return fail(PBRT_ERROR_INVALID_ARGUMENT, "not a pipeline");
  PBRT_CUDA(cudaMemsetAsync(pp->ctr, 0, sizeof(Counters), stream));
  return PBRT_OK;
}

PBRT_API int pbrt_pipeline_abort_flag(PbrtPipeline* pp, uint32_t** host_flag) {
  if (!checked<PbrtPipeline>(pp, Kind::Pipeline) || !host_flag)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "abort flag: bad arguments");
  if (!pp->abort_host) {
    void* h = nullptr;
    PBRT_CUDA(cudaHostAlloc(&h, sizeof(uint32_t), cudaHostAllocMapped));
    *(volatile uint32_t*)h = 0;
    void* d = nullptr;
    cudaError_t e = cudaHostGetDevicePointer(&d, h, 0);
    if (e != cudaSuccess) {
      cudaFreeHost(h);
      return cuda_fail(e, "cudaHostGetDevicePointer");
    }
    pp->abort_host = (uint32_t*)h;
    pp->abort_dev = (uint32_t*)d;
  }
  *host_flag = pp->abort_host;
  return PBRT_OK;
}

PBRT_API int pbrt_pipeline_set_budget(PbrtPipeline* pp, uint64_t budget_ns) {
  if (!checked<PbrtPipeline>(pp, Kind::Pipeline)) return fail(PBRT_ERROR_INVALID_ARGUMENT, "not a pipeline");
  pp->budget_ns = budget_ns;
  return PBRT_OK;
}

PBRT_API int pbrt_pipeline_status(PbrtPipeline* pp, pbrt_stream_t stream, int32_t* frame_status) {
  if (!checked<PbrtPipeline>(pp, Kind::Pipeline) || !frame_status)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "status: bad arguments");
  uint32_t err = 0;
  PBRT_CUDA(cudaMemcpyAsync(&err, &pp->ctr->error, sizeof(err), cudaMemcpyDeviceToHost, stream));
  PBRT_CUDA(cudaStreamSynchronize(stream));
  *frame_status = (err & 2u) ? PBRT_ERROR_ABORTED : (err & 4u) ? PBRT_ERROR_TIMEOUT : PBRT_OK;
  const uint32_t keep = err & 1u;  // the stack-overflow record stays for pbrt_pipeline_stats
  PBRT_CUDA(cudaMemcpyAsync(&pp->ctr->error, &keep, sizeof(keep), cudaMemcpyHostToDevice, stream));
  PBRT_CUDA(cudaStreamSynchronize(stream));
  return PBRT_OK;
}

PBRT_API int pbrt_pipeline_debug_images(const PbrtPipeline* pp, PbrtImage* primary_hit_key) {
  if (!checked<const PbrtPipeline>((void*)pp, Kind::Pipeline)) return fail(PBRT_ERROR_INVALID_ARGUMENT, "not a pipeline");
  if (primary_hit_key) {
    PbrtImage& im = *primary_hit_key;
    im.data = pp->q.prim_key;
    im.width = (uint32_t)pp->W;
    im.height = (uint32_t)pp->H;
    im.layers = 1;
    im.format = PBRT_FORMAT_R32_UINT;
    im.texel_bytes = 4;
    im.row_bytes = (size_t)pp->W * 4;
    im.layer_bytes = im.row_bytes * pp->H;
  }
  return PBRT_OK;
}


PBRT_API int pbrt_pipeline_set_schedule(PbrtPipeline* pp, int32_t sort_rays, int32_t merge_shadow) {
  if (!checked<PbrtPipeline>(pp, Kind::Pipeline)) return fail(PBRT_ERROR_INVALID_ARGUMENT, "not a pipeline");
  if (sort_rays && !pp->q.key_t) {  // staging queues of the sort, allocated on first use
    Queues& q = pp->q;
    const size_t N = (size_t)pp->W * pp->H;
    int st = PBRT_OK;
    if (!st) st = pp->a(&q.pix_t, N);
    if (!st) st = pp->a(&q.org_t, N);
    if (!st) st = pp->a(&q.dir_t, N);
    if (!st) st = pp->a(&q.spix_t, N);
    if (!st) st = pp->a(&q.sorg_t, N);
    if (!st) st = pp->a(&q.sdir_t, N);
    if (!st) st = pp->a(&q.snee_t, N);
    if (!st) st = pp->a(&q.sadd_t, N);
    if (!st) st = pp->a(&q.skey_t, N);
    if (!st) st = pp->a(&q.bins, 2 * kSortBins);
    if (!st) st = pp->a(&q.key_t, N);  // last: key_t marks the staging queues as allocated
    if (st) return st;
  }
  const int sr = sort_rays ? 1 : 0, ms = merge_shadow ? 1 : 0;
  if (sr != pp->sort_rays || ms != pp->merge_shadow) {
    pp->sort_rays = sr;
    pp->merge_shadow = ms;
    pp->graph_depth = -1;  // the frame graph is recaptured on the next trace
  }
  return PBRT_OK;
}

PBRT_API int pbrt_pipeline_set_launch(PbrtPipeline* pp, int32_t trace_blocks_per_sm, int32_t shade_blocks_per_sm) {
  if (!checked<PbrtPipeline>(pp, Kind::Pipeline) || trace_blocks_per_sm < 1 || trace_blocks_per_sm > 16 ||
      shade_blocks_per_sm < 1 || shade_blocks_per_sm > 16)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "set launch: blocks per SM must be in 1..16");
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (pp->grid_persistent != sms * trace_blocks_per_sm || pp->grid_shade != sms * shade_blocks_per_sm) {
    pp->grid_persistent = sms * trace_blocks_per_sm;
    pp->grid_shade = sms * shade_blocks_per_sm;
    pp->graph_depth = -1;  // the frame graph is recaptured on the next trace
  }
  return PBRT_OK;
}

}  // extern "C"

// ===========================================================================
// Batched requests: many independent renders (own pipeline -- scene,
// resolution, depth -- own sample count, optional accumulator and BMFR) in
// one CUDA graph launch. The graph forks into `branches` concurrent chains;
// requests are assigned to chains longest-first onto the least loaded chain
// (cost = pixels x samples x (max depth + 1)), so small requests fill the GPU
// beside large ones. Frame parameters are baked into the captured launches;
// the graph is recaptured when the request list or the tuning changes.
// No reference counterpart (the reference renders one view per frame).
struct PbrtBatch : pbrt::Object {
  PbrtBatch() : Object(pbrt::Kind::Batch) {}
  ~PbrtBatch() override {
    drop();
    for (auto& r : reqs) {
      release(r.pipeline);
      release(r.accumulator);
      release(r.bmfr);
    }
  }
  std::vector<PbrtBatchRequest> reqs;
  PbrtBatchTuning tuning{4, 8, 8, 1};
  cudaGraphExec_t exec = nullptr;
  void drop() {
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
  }
};

namespace {

double request_cost(const PbrtBatchRequest& r) {
  return (double)r.pipeline->W * r.pipeline->H * (double)std::max<uint32_t>(r.spp, 1) *
         (double)(r.pipeline->max_depth + 1);
}

// Requests of one request's frames: set params, trace, accumulate,
// copy-to-back; then BMFR once.
int record_request(const PbrtBatchRequest& r, cudaStream_t s) {
  PbrtPipeline* pp = r.pipeline;
  const uint32_t spp = std::max<uint32_t>(r.spp, 1);
  int st = PBRT_OK;
  for (uint32_t k = 0; k < spp && !st; ++k) {
    PbrtPushConstants pc = r.pc;
    pc.frame_number = r.pc.frame_number + k;
    k_set_params<<<1, 1, 0, s>>>(pp->dev_fp, frame_params(pp, &pc));
    if ((st = check_launch("k_set_params"))) break;
    if ((st = record_frame(pp, s, nullptr))) break;
    if (r.accumulator) {
      if ((st = pbrt_accumulator_set_camera_matrices(r.accumulator, (int32_t)k, &r.camera, &r.camera))) break;
      if ((st = pbrt_accumulator_dispatch(r.accumulator, s))) break;
      PbrtIlluminationBuffer* acc_illu = nullptr;
      PbrtAccumulationBuffer* ab = nullptr;
      pbrt_accumulator_get_accumulated_illumination(r.accumulator, &acc_illu);
      pbrt_accumulator_get_accumulation_buffer(r.accumulator, &ab);
      if ((st = pbrt_accumulation_buffer_copy_to_back_images(ab, pp->gbuffer, acc_illu, s))) break;
    }
  }
  if (!st && r.bmfr) {
    PbrtPushConstants pc = r.pc;
    pc.frame_number = r.pc.frame_number + spp - 1;
    st = pbrt_bmfr_dispatch(r.bmfr, &pc, s);
  }
  return st;
}

int capture_batch(PbrtBatch* b) {
  const uint32_t nb = std::max<uint32_t>(1, std::min<uint32_t>(b->tuning.branches, (uint32_t)b->reqs.size()));
  std::vector<uint32_t> assign(b->reqs.size());
  std::vector<double> costs(b->reqs.size());
  for (size_t i = 0; i < b->reqs.size(); ++i) costs[i] = request_cost(b->reqs[i]);
  int st = pbrt_batch_plan(costs.data(), (uint32_t)costs.size(), nb, b->tuning.order, assign.data());
  if (st) return st;
  for (auto& r : b->reqs) {
    if ((st = pbrt_pipeline_set_launch(r.pipeline, (int32_t)b->tuning.trace_blocks_per_sm,
                                       (int32_t)b->tuning.shade_blocks_per_sm)))
      return st;
  }
  std::vector<cudaStream_t> br(nb, nullptr);
  std::vector<cudaEvent_t> ev(nb + 1, nullptr);
  cudaStream_t root = nullptr;
  auto cleanup = [&]() {
    for (auto s : br)
      if (s) cudaStreamDestroy(s);
    for (auto e : ev)
      if (e) cudaEventDestroy(e);
    if (root) cudaStreamDestroy(root);
  };
  cudaError_t e = cudaStreamCreateWithFlags(&root, cudaStreamNonBlocking);
  for (uint32_t i = 0; i < nb && e == cudaSuccess; ++i) e = cudaStreamCreateWithFlags(&br[i], cudaStreamNonBlocking);
  for (uint32_t i = 0; i <= nb && e == cudaSuccess; ++i) e = cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming);
  if (e != cudaSuccess) {
    cleanup();
    return cuda_fail(e, "batch streams");
  }
  cudaGraph_t graph = nullptr;
  e = cudaStreamBeginCapture(root, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) e = cudaEventRecord(ev[nb], root);
  for (uint32_t i = 0; i < nb && e == cudaSuccess; ++i) e = cudaStreamWaitEvent(br[i], ev[nb], 0);
  st = e == cudaSuccess ? PBRT_OK : cuda_fail(e, "batch fork");
  // order within a chain: as assigned (pbrt_batch_plan lists requests longest first)
  std::vector<uint32_t> order(b->reqs.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = (uint32_t)i;
  if (b->tuning.order == 1)
    std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) { return costs[x] > costs[y]; });
  for (uint32_t i : order) {
    if (st) break;
    st = record_request(b->reqs[i], br[assign[i]]);
  }
  for (uint32_t i = 0; i < nb && !st; ++i) {
    e = cudaEventRecord(ev[i], br[i]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(root, ev[i], 0);
    if (e != cudaSuccess) st = cuda_fail(e, "batch join");
  }
  cudaError_t e2 = cudaStreamEndCapture(root, &graph);
  if (!st && e2 != cudaSuccess) st = cuda_fail(e2, "end capture (batch)");
  if (!st) {
    e = cudaGraphInstantiate(&b->exec, graph, 0);
    if (e != cudaSuccess) st = cuda_fail(e, "graph instantiate (batch)");
  }
  if (graph) cudaGraphDestroy(graph);
  cleanup();
  return st;
}

}  // namespace

extern "C" {

PBRT_API int pbrt_batch_plan(const double* costs, uint32_t n, uint32_t branches, uint32_t order, uint32_t* assign) {
  if ((n && (!costs || !assign)) || branches == 0 || order > 1)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "batch plan: bad arguments");
  std::vector<uint32_t> idx(n);
  for (uint32_t i = 0; i < n; ++i) idx[i] = i;
  if (order == 1) std::stable_sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) { return costs[a] > costs[b]; });
  std::vector<double> load(branches, 0.0);
  for (uint32_t i : idx) {
    uint32_t best = 0;
    for (uint32_t k = 1; k < branches; ++k)
      if (load[k] < load[best]) best = k;
    assign[i] = best;
    load[best] += costs[i];
  }
  return PBRT_OK;
}

PBRT_API int pbrt_batch_create(PbrtBatch** out) {
  if (!out) return fail(PBRT_ERROR_INVALID_ARGUMENT, "batch create: null output");
  *out = new (std::nothrow) PbrtBatch();
  return *out ? PBRT_OK : fail(PBRT_ERROR_OUT_OF_MEMORY, "batch: host allocation");
}

PBRT_API int pbrt_batch_add(PbrtBatch* b, const PbrtBatchRequest* r) {
  if (!checked<PbrtBatch>(b, Kind::Batch) || !r || !checked<PbrtPipeline>(r->pipeline, Kind::Pipeline) ||
      (r->accumulator && !checked<PbrtAccumulator>(r->accumulator, Kind::Accumulator)) ||
      (r->bmfr && !checked<PbrtBMFR>(r->bmfr, Kind::BMFR)) || r->spp == 0 || r->spp > 4096)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "batch add: bad request");
  if (r->accumulator && !r->camera.has_proj)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "batch add: an accumulated request needs camera matrices with proj");
  for (const auto& q : b->reqs)
    if (q.pipeline == r->pipeline)
      return fail(PBRT_ERROR_INVALID_ARGUMENT, "batch add: a pipeline may appear in one request only");
  retain(r->pipeline);
  if (r->accumulator) retain(r->accumulator);
  if (r->bmfr) retain(r->bmfr);
  b->reqs.push_back(*r);
  b->drop();
  return PBRT_OK;
}

PBRT_API int pbrt_batch_size(const PbrtBatch* b, uint32_t* count) {
  if (!checked<const PbrtBatch>((void*)b, Kind::Batch) || !count) return fail(PBRT_ERROR_INVALID_ARGUMENT, "batch size");
  *count = (uint32_t)b->reqs.size();
  return PBRT_OK;
}

PBRT_API int pbrt_batch_set_tuning(PbrtBatch* b, const PbrtBatchTuning* t) {
  if (!checked<PbrtBatch>(b, Kind::Batch) || !t || t->branches == 0 || t->branches > 64 || t->trace_blocks_per_sm < 1 ||
      t->trace_blocks_per_sm > 16 || t->shade_blocks_per_sm < 1 || t->shade_blocks_per_sm > 16 || t->order > 1)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "batch tuning: out of range");
  b->tuning = *t;
  b->drop();
  return PBRT_OK;
}

PBRT_API int pbrt_batch_get_tuning(const PbrtBatch* b, PbrtBatchTuning* t) {
  if (!checked<const PbrtBatch>((void*)b, Kind::Batch) || !t) return fail(PBRT_ERROR_INVALID_ARGUMENT, "batch tuning");
  *t = b->tuning;
  return PBRT_OK;
}

PBRT_API int pbrt_batch_submit(PbrtBatch* b, pbrt_stream_t stream) {
  if (!checked<PbrtBatch>(b, Kind::Batch)) return fail(PBRT_ERROR_INVALID_ARGUMENT, "batch submit: not a batch");
  if (b->reqs.empty()) return PBRT_OK;
  if (!b->exec) {
    int st = capture_batch(b);
    if (st) return st;
  }
  PBRT_CUDA(cudaGraphLaunch(b->exec, stream));
  return PBRT_OK;
}

// Autotuner: times every candidate (chains x traversal CTAs/SM x shading
// CTAs/SM, longest-first order) on the batch itself -- one warm-up launch,
// then the median of `repeats` launches -- and keeps the fastest.
PBRT_API int pbrt_batch_autotune(PbrtBatch* b, pbrt_stream_t stream, int32_t repeats, PbrtBatchTuning* best_out,
                                 float* best_ms_out) {
  if (!checked<PbrtBatch>(b, Kind::Batch) || repeats < 1 || repeats > 16)
    return fail(PBRT_ERROR_INVALID_ARGUMENT, "batch autotune: bad arguments");
  if (b->reqs.empty()) return fail(PBRT_ERROR_INVALID_ARGUMENT, "batch autotune: empty batch");
  const uint32_t chains[] = {1, 2, 4, 8, 16};
  const uint32_t trace_bps[] = {4, 8};
  const uint32_t shade_bps[] = {4, 8};
  cudaEvent_t e0, e1;
  PBRT_CUDA(cudaEventCreate(&e0));
  PBRT_CUDA(cudaEventCreate(&e1));
  PbrtBatchTuning best = b->tuning;
  float best_ms = 1e30f;
  int st = PBRT_OK;
  for (uint32_t c : chains) {
    if (c > b->reqs.size() && c != 1) continue;
    for (uint32_t tb : trace_bps)
      for (uint32_t sb : shade_bps) {
        if (st) break;
        PbrtBatchTuning t{c, tb, sb, 1};
        if ((st = pbrt_batch_set_tuning(b, &t))) break;
        if ((st = pbrt_batch_submit(b, stream))) break;  // capture + warm-up
        std::vector<float> ms;
        for (int r = 0; r < repeats && !st; ++r) {
          cudaEventRecord(e0, stream);
          st = pbrt_batch_submit(b, stream);
          cudaEventRecord(e1, stream);
          cudaError_t e = cudaEventSynchronize(e1);
          if (!st && e != cudaSuccess) st = cuda_fail(e, "autotune timing");
          float m = 0.f;
          cudaEventElapsedTime(&m, e0, e1);
          ms.push_back(m);
        }
        if (st) break;
        std::sort(ms.begin(), ms.end());
        const float med = ms[ms.size() / 2];
        if (med < best_ms) {
          best_ms = med;
          best = t;
        }
      }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st) return st;
  if ((st = pbrt_batch_set_tuning(b, &best))) return st;
  if (best_out) *best_out = best;
  if (best_ms_out) *best_ms_out = best_ms;
  return PBRT_OK;
}

}  // extern "C"
