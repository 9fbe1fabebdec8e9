// Device BVH build: the fast-build alternative to the host's binned-SAH
// build (bvh_build.cpp), producing the same 8-wide Node8 layout and the same
// leaf-ordered triangle records, directly in device memory.
//
// The reference builds its acceleration structures on the device
// (vkCmdBuildAccelerationStructuresKHR through
// vsg::BuildAccelerationStructureTraversal, VulkanPBRT.cpp:365-367); Vulkan
// lets the caller trade trace speed for build speed
// (VK_BUILD_ACCELERATION_STRUCTURE_PREFER_FAST_BUILD_BIT_KHR). This is that
// trade: a linear BVH over 63-bit Morton codes of the triangle centroids
// (Karras, "Maximizing Parallelism in the Construction of BVHs, Octrees, and
// k-d Trees", HPG 2012), its boxes by one bottom-up pass, then a
// level-by-level collapse into 8-wide nodes (the SAH-optimal distribution
// of Ylitie, Karras & Laine 2017, its programme evaluated in the same
// bottom-up pass; or greedily, opening the child with the largest surface
// area until eight), leaves of at most three triangles, consecutive in
// Morton order. Closest hits do not depend on the tree (ties go to the
// lowest triangle key, the flattening index), so frames rendered over either
// build are bit-identical.
#include <cub/device/device_radix_sort.cuh>

#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "bvh.hpp"
#include "internal.hpp"
#include "lbvh.cuh"

namespace pbrt {
namespace lbvh {

constexpr int kLeafMax = 3;        // triangles a leaf slot holds (5-bit offsets, 3-bit counts)
constexpr int kReduceBlocks = 1024;
constexpr int kThreads = 256;

__device__ __forceinline__ void tri_box(const float* w, float lo[3], float hi[3]) {
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    lo[a] = fminf(fminf(w[a], w[3 + a]), w[6 + a]);
    hi[a] = fmaxf(fmaxf(w[a], w[3 + a]), w[6 + a]);
  }
}

// Centroids (the host build's 0.5 * (lo + hi)) and per-block centroid bounds.
__global__ void __launch_bounds__(kThreads) k_centroids(const float* __restrict__ world, int n,
                                                        float4* __restrict__ cent, float* __restrict__ part) {
  float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float lo[3], hi[3];
    tri_box(world + 9 * (size_t)i, lo, hi);
    float c[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      c[a] = 0.5f * (lo[a] + hi[a]);
      mn[a] = fminf(mn[a], c[a]);
      mx[a] = fmaxf(mx[a], c[a]);
    }
    cent[i] = make_float4(c[0], c[1], c[2], 0.f);
  }
  __shared__ float s[6][kThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    for (int o = 16; o; o >>= 1) {
      mn[a] = fminf(mn[a], __shfl_xor_sync(0xffffffffu, mn[a], o));
      mx[a] = fmaxf(mx[a], __shfl_xor_sync(0xffffffffu, mx[a], o));
    }
    if (lane == 0) {
      s[a][warp] = mn[a];
      s[3 + a][warp] = mx[a];
    }
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    const bool is_min = threadIdx.x < 3;
    float v = s[threadIdx.x][0];
    for (int w = 1; w < kThreads / 32; ++w) v = is_min ? fminf(v, s[threadIdx.x][w]) : fmaxf(v, s[threadIdx.x][w]);
    part[6 * blockIdx.x + threadIdx.x] = v;
  }
}

// Morton keys over the centroid bounds (one block folds the partial bounds).
__global__ void __launch_bounds__(kThreads) k_morton(const float4* __restrict__ cent, int n,
                                                     const float* __restrict__ part, int nparts,
                                                     uint64_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  __shared__ float cb[6];
  if (threadIdx.x < 6) {
    const bool is_min = threadIdx.x < 3;
    float v = part[threadIdx.x];
    for (int b = 1; b < nparts; ++b) v = is_min ? fminf(v, part[6 * b + threadIdx.x]) : fmaxf(v, part[6 * b + threadIdx.x]);
    cb[threadIdx.x] = v;
  }
  __syncthreads();
  const float kQ = 2097151.f;  // 2^21 - 1
  float sc[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float ext = cb[3 + a] - cb[a];
    sc[a] = ext > 0.f ? kQ / ext : 0.f;
  }
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 c = cent[i];
    const float cc[3] = {c.x, c.y, c.z};
    uint64_t q[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      float f = (cc[a] - cb[a]) * sc[a];
      f = fminf(fmaxf(f, 0.f), kQ);  // NaN -> 0
      q[a] = (uint64_t)f;
    }
    keys[i] = (spread21(q[0]) << 2) | (spread21(q[1]) << 1) | spread21(q[2]);
    vals[i] = (uint32_t)i;
  }
}

// Internal node i of the radix tree over n sorted keys (0 <= i < n - 1):
// its children (internal index, or n - 1 + leaf position), parent links and
// the range of sorted positions it covers.
__global__ void __launch_bounds__(kThreads) k_radix_tree(const uint64_t* __restrict__ k, int n, int* __restrict__ left,
                                                         int* __restrict__ right, int* __restrict__ parent,
                                                         int* __restrict__ first, int* __restrict__ last) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  int lc, rc, lo, hi;
  radix_node(k, n, i, &lc, &rc, &lo, &hi);
  left[i] = lc;
  right[i] = rc;
  parent[lc] = i;
  parent[rc] = i;
  first[i] = lo;
  last[i] = hi;
}

// The SAH-optimal collapse's dynamic programme (Ylitie, Karras & Laine,
// HPG 2017, section 3.1, as the host build runs it), per binary node m:
// cost[m][i-1] = the cheapest way to represent m's subtree as at most i
// slots of a wide node (i = 1..8); split[m][i-1] = k > 0: k slots to the
// left child, i - k to the right; 0: as with i - 1 slots; -1: one slot (a
// leaf of at most three triangles when leaf[m], else a wide node);
// wsplit[m] = the left share of the 8-slot distribution of m's own wide node.
struct WideDp {
  float* cost;       // [2n - 1][8]
  int8_t* split;     // [2n - 1][8]
  uint8_t* leaf;     // [2n - 1]
  uint8_t* wsplit;   // [2n - 1]
  float prim_cost;   // a triangle test against a node visit (1)
};

__device__ __forceinline__ float box_area(float4 a, float4 c) {
  const float dx = fmaxf(0.f, c.x - a.x), dy = fmaxf(0.f, c.y - a.y), dz = fmaxf(0.f, c.z - a.z);
  return 2.f * (dx * dy + dy * dz + dz * dx);
}

__device__ void dp_node(const WideDp& dp, int m, int l, int r, int count, float area) {
  constexpr float kInf = INFINITY;
  float cl[8], cr[8];
  const float4* pl = reinterpret_cast<const float4*>(dp.cost + 8 * (size_t)l);
  const float4* pr = reinterpret_cast<const float4*>(dp.cost + 8 * (size_t)r);
  const float4 l0 = __ldcg(pl), l1 = __ldcg(pl + 1), r0 = __ldcg(pr), r1 = __ldcg(pr + 1);
  cl[0] = l0.x; cl[1] = l0.y; cl[2] = l0.z; cl[3] = l0.w; cl[4] = l1.x; cl[5] = l1.y; cl[6] = l1.z; cl[7] = l1.w;
  cr[0] = r0.x; cr[1] = r0.y; cr[2] = r0.z; cr[3] = r0.w; cr[4] = r1.x; cr[5] = r1.y; cr[6] = r1.z; cr[7] = r1.w;
  float dist[9];
  int8_t arg[9];
#pragma unroll
  for (int j = 2; j <= 8; ++j) {
    dist[j] = kInf;
    arg[j] = 1;
#pragma unroll
    for (int k = 1; k < j; ++k) {
      const float v = cl[k - 1] + cr[j - k - 1];
      if (v < dist[j]) {
        dist[j] = v;
        arg[j] = (int8_t)k;
      }
    }
  }
  const float leafc = count <= kLeafMax ? area * dp.prim_cost * (float)count : kInf;
  const float internal = area + dist[8];
  float c[8];
  int8_t sp[8];
  c[0] = fminf(leafc, internal);
  sp[0] = -1;
#pragma unroll
  for (int i = 2; i <= 8; ++i) {
    if (dist[i] < c[i - 2]) {
      c[i - 1] = dist[i];
      sp[i - 1] = arg[i];
    } else {
      c[i - 1] = c[i - 2];
      sp[i - 1] = 0;
    }
  }
  float4* pc = reinterpret_cast<float4*>(dp.cost + 8 * (size_t)m);
  pc[0] = make_float4(c[0], c[1], c[2], c[3]);
  pc[1] = make_float4(c[4], c[5], c[6], c[7]);
#pragma unroll
  for (int i = 0; i < 8; ++i) dp.split[8 * (size_t)m + i] = sp[i];
  dp.leaf[m] = leafc <= internal ? 1 : 0;
  dp.wsplit[m] = (uint8_t)arg[8];
}

// Boxes (and, with dp.cost set, the collapse's programme), bottom-up: each
// leaf writes its triangle's box and climbs; of the two threads reaching a
// node, the second (which sees the first's results through L2) forms the
// node's and goes on.
__global__ void __launch_bounds__(kThreads) k_boxes(const float* __restrict__ world, const uint32_t* __restrict__ vals,
                                                    int n, const int* __restrict__ left, const int* __restrict__ right,
                                                    const int* __restrict__ parent, const int* __restrict__ first,
                                                    const int* __restrict__ last, float4* lo, float4* hi,
                                                    int* __restrict__ flag, WideDp dp) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float a[3], b[3];
  tri_box(world + 9 * (size_t)vals[i], a, b);
  const int leaf = n - 1 + i;
  const float4 bl = make_float4(a[0], a[1], a[2], 0.f), bh = make_float4(b[0], b[1], b[2], 0.f);
  lo[leaf] = bl;
  hi[leaf] = bh;
  if (dp.cost) {
    const float lc = box_area(bl, bh) * dp.prim_cost;
    float4* pc = reinterpret_cast<float4*>(dp.cost + 8 * (size_t)leaf);
    pc[0] = make_float4(lc, lc, lc, lc);
    pc[1] = make_float4(lc, lc, lc, lc);
    for (int k = 0; k < 8; ++k) dp.split[8 * (size_t)leaf + k] = -1;
    dp.leaf[leaf] = 1;
    dp.wsplit[leaf] = 1;
  }
  int node = parent[leaf];
  for (int guard = 0; node >= 0 && guard < n; ++guard) {
    __threadfence();
    if (atomicAdd(&flag[node], 1) == 0) return;
    __threadfence();
    const int l = left[node], r = right[node];
    const float4 l0 = __ldcg(&lo[l]), l1 = __ldcg(&hi[l]), r0 = __ldcg(&lo[r]), r1 = __ldcg(&hi[r]);
    const float4 nl = make_float4(fminf(l0.x, r0.x), fminf(l0.y, r0.y), fminf(l0.z, r0.z), 0.f);
    const float4 nh = make_float4(fmaxf(l1.x, r1.x), fmaxf(l1.y, r1.y), fmaxf(l1.z, r1.z), 0.f);
    lo[node] = nl;
    hi[node] = nh;
    if (dp.cost) dp_node(dp, node, l, r, last[node] - first[node] + 1, box_area(nl, nh));
    node = parent[node];
  }
}

struct Tree {
  int n;
  const int *left, *right, *first, *last;
  const float4 *lo, *hi;
  __device__ bool is_leaf(int b) const { return b >= n - 1; }
  __device__ int count(int b) const { return is_leaf(b) ? 1 : last[b] - first[b] + 1; }
  __device__ int pos(int b) const { return is_leaf(b) ? b - (n - 1) : first[b]; }
  __device__ bool leaf_slot(int b) const { return is_leaf(b) || count(b) <= kLeafMax; }
  __device__ float area(int b) const { return box_area(lo[b], hi[b]); }
};

struct Out {
  Node8* nodes;
  float4* tris;          // 3 a triangle slot: (v0 | key), (v1 | instance), (v2 | primitive)
  uint32_t* order;       // triangle slot -> flattening index
  unsigned* counters;    // [0] nodes, [1] triangle slots, [2] next-level items, [3] leaves, [4] error
  uint32_t node_cap;
};

__device__ __forceinline__ uint8_t exponent_for(double extent) {
  // smallest power of two s with extent / s <= 255, as the host build
  if (!(extent > 0.0)) return 1;
  int e;
  frexp(extent / 255.0, &e);
  return (uint8_t)min(254, max(1, e + 127));
}

// One level of the collapse: item = (binary node, its wide node's index).
__global__ void __launch_bounds__(128) k_collapse(Tree t, WideDp dp, const float* __restrict__ world,
                                                  const uint32_t* __restrict__ vals, const uint32_t* __restrict__ inst,
                                                  const uint32_t* __restrict__ prim, const uint2* __restrict__ items,
                                                  int count, uint2* __restrict__ next, Out o) {
  const int it = blockIdx.x * blockDim.x + threadIdx.x;
  if (it >= count) return;
  const int b = (int)items[it].x;
  const uint32_t out_index = items[it].y;
  int ch[8];
  int nch = 0;
  // a slot is a leaf: the programme's choice, else any subtree of <= 3 triangles
  auto is_leaf_slot = [&](int c) { return dp.cost ? (t.is_leaf(c) || dp.leaf[c] != 0) : t.leaf_slot(c); };
  // one leaf slot: the root when it is a leaf; any other wide node was made
  // for a subtree that is not one (with the programme, a subtree of <= 3
  // triangles can be cheaper as a wide node of several leaves)
  if (is_leaf_slot(b)) {
    ch[nch++] = b;
  } else if (dp.cost) {
    // the programme's eight-slot distribution (the host build's slots())
    int stn[8], stj[8], sp = 0;
    const int ws = dp.wsplit[b];
    stn[sp] = t.right[b];
    stj[sp++] = 8 - ws;
    stn[sp] = t.left[b];
    stj[sp++] = ws;
    while (sp > 0 && nch < 8) {
      --sp;
      const int m = stn[sp], j = stj[sp];
      const int s = (j == 1 || t.is_leaf(m)) ? -1 : dp.split[8 * (size_t)m + (j - 1)];
      if (s < 0) {
        ch[nch++] = m;
      } else if (s == 0) {
        stn[sp] = m;
        stj[sp++] = j - 1;
      } else if (sp + 2 <= 8) {
        stn[sp] = t.right[m];
        stj[sp++] = j - s;
        stn[sp] = t.left[m];
        stj[sp++] = s;
      } else {
        ch[nch++] = m;  // cannot happen: the entries' slot counts sum to at most 8
      }
    }
  } else {
    ch[nch++] = t.left[b];
    ch[nch++] = t.right[b];
    while (nch < 8) {
      int best = -1;
      float best_area = -1.f;
      for (int k = 0; k < nch; ++k) {
        if (t.leaf_slot(ch[k])) continue;
        const float a = t.area(ch[k]);
        if (a > best_area) {
          best_area = a;
          best = k;
        }
      }
      if (best < 0) break;
      const int c = ch[best];
      ch[best] = t.left[c];
      ch[nch++] = t.right[c];
    }
  }
  // octant slots around the node's centre (the host build's rule)
  const float4 nlo = t.lo[b], nhi = t.hi[b];
  const float pc[3] = {0.5f * (nlo.x + nhi.x), 0.5f * (nlo.y + nhi.y), 0.5f * (nlo.z + nhi.z)};
  int slot_child[8];
  unsigned used = 0, placed = 0;
  for (int round = 0; round < nch; ++round) {
    double best = -INFINITY;
    int bc = -1, bs = -1;
    for (int k = 0; k < nch; ++k) {
      if (placed >> k & 1u) continue;
      const float4 cl = t.lo[ch[k]], chh = t.hi[ch[k]];
      const double d0 = 0.5 * ((double)cl.x + chh.x) - pc[0];
      const double d1 = 0.5 * ((double)cl.y + chh.y) - pc[1];
      const double d2 = 0.5 * ((double)cl.z + chh.z) - pc[2];
      for (int s = 0; s < 8; ++s) {
        if (used >> s & 1u) continue;
        const double score = (s & 1 ? d0 : -d0) + (s & 2 ? d1 : -d1) + (s & 4 ? d2 : -d2);
        if (score > best || bc < 0) {
          best = score;
          bc = k;
          bs = s;
        }
      }
    }
    placed |= 1u << bc;
    used |= 1u << bs;
    slot_child[bs] = ch[bc];
  }
  int n_inner = 0, n_tris = 0;
  for (int s = 0; s < 8; ++s) {
    if (!(used >> s & 1u)) continue;
    if (is_leaf_slot(slot_child[s]))
      n_tris += t.count(slot_child[s]);
    else
      ++n_inner;
  }
  const uint32_t cbase = n_inner ? atomicAdd(&o.counters[0], (unsigned)n_inner) : 0u;
  const uint32_t tbase = n_tris ? atomicAdd(&o.counters[1], (unsigned)n_tris) : 0u;
  if ((n_inner && cbase + (uint32_t)n_inner > o.node_cap) || (n_tris && tbase + (uint32_t)n_tris > (uint32_t)t.n) ||
      n_tris > 31) {
    atomicExch(&o.counters[4], 1u);
    return;
  }
  Node8 nd;
  memset(&nd, 0, sizeof(nd));
  nd.px = nlo.x;
  nd.py = nlo.y;
  nd.pz = nlo.z;
  const float p[3] = {nlo.x, nlo.y, nlo.z};
  const double ext[3] = {(double)nhi.x - (double)nlo.x, (double)nhi.y - (double)nlo.y, (double)nhi.z - (double)nlo.z};
  uint8_t ex[3];
  float scale[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    ex[a] = exponent_for(ext[a]);
    scale[a] = ldexpf(1.0f, (int)ex[a] - 127);
  }
  nd.ex = ex[0];
  nd.ey = ex[1];
  nd.ez = ex[2];
  nd.child_base = cbase;
  nd.tri_base = tbase;
  int rank = 0, tri_off = 0, leaves = 0;
  for (int s = 0; s < 8; ++s) {
    if (!(used >> s & 1u)) continue;
    const int c = slot_child[s];
    const float4 cl = t.lo[c], chh = t.hi[c];
    const float clo[3] = {cl.x, cl.y, cl.z}, chi[3] = {chh.x, chh.y, chh.z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const double ql = floor(((double)clo[a] - p[a]) / scale[a]);
      const double qh = ceil(((double)chi[a] - p[a]) / scale[a]);
      nd.qlo[a][s] = (uint8_t)fmin(255.0, fmax(0.0, ql));
      nd.qhi[a][s] = (uint8_t)fmin(255.0, fmax(0.0, qh));
    }
    if (!is_leaf_slot(c)) {
      nd.imask |= (uint8_t)(1u << s);
      nd.meta[s] = 0x80;
      const unsigned q = atomicAdd(&o.counters[2], 1u);
      next[q] = make_uint2((uint32_t)c, cbase + (uint32_t)rank);
      ++rank;
    } else {
      const int cnt = t.count(c), p0 = t.pos(c);
      nd.meta[s] = (uint8_t)((cnt << 5) | tri_off);
      for (int k = 0; k < cnt; ++k) {
        const uint32_t src = vals[p0 + k];
        const uint32_t slot = tbase + (uint32_t)(tri_off + k);
        const float* w = world + 9 * (size_t)src;
        o.tris[3 * (size_t)slot + 0] = make_float4(w[0], w[1], w[2], __uint_as_float(src));
        o.tris[3 * (size_t)slot + 1] = make_float4(w[3], w[4], w[5], __uint_as_float(inst[src]));
        o.tris[3 * (size_t)slot + 2] = make_float4(w[6], w[7], w[8], __uint_as_float(prim[src]));
        o.order[slot] = src;
      }
      tri_off += cnt;
      ++leaves;
    }
  }
  if (leaves) atomicAdd(&o.counters[3], (unsigned)leaves);
  o.nodes[out_index] = nd;
}

// Device allocations of one build, freed together.
struct Arena {
  std::vector<void*> ptrs;
  ~Arena() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <class T> int get(T** p, size_t count) {
    *p = nullptr;
    cudaError_t e = cudaMalloc((void**)p, (count ? count : 1) * sizeof(T));
    if (e != cudaSuccess) return cuda_fail(e, "device BVH build: cudaMalloc");
    ptrs.push_back((void*)*p);
    return PBRT_OK;
  }
  void keep(void* p) {  // ownership leaves the arena
    for (void*& q : ptrs)
      if (q == p) q = nullptr;
  }
};

}  // namespace lbvh

int build_bvh8_device(const float* world_h, const uint32_t* inst_h, const uint32_t* prim_h, size_t n_, int max_depth,
                      Node8** nodes_out, float4** tris_out, Bvh8Stats* stats) {
  using namespace lbvh;
  *nodes_out = nullptr;
  *tris_out = nullptr;
  if (n_ == 0 || n_ > 0x7fffffffu) return fail(PBRT_ERROR_INVALID_ARGUMENT, "device BVH build: %zu triangles", n_);
  const auto t0 = std::chrono::steady_clock::now();
  const int n = (int)n_;
  Arena ar;
  float* world = nullptr;
  uint32_t *inst = nullptr, *prim = nullptr, *vals_in = nullptr, *vals = nullptr, *order = nullptr;
  uint64_t *keys_in = nullptr, *keys = nullptr;
  float4 *cent = nullptr, *lo = nullptr, *hi = nullptr, *tris = nullptr;
  float* part = nullptr;
  int *left = nullptr, *right = nullptr, *parent = nullptr, *first = nullptr, *last = nullptr, *flag = nullptr;
  uint2 *items_a = nullptr, *items_b = nullptr;
  unsigned* counters = nullptr;
  Node8* nodes = nullptr;
  const size_t nodes_total = 2 * (size_t)n - 1;
  int st = PBRT_OK;
  if (!st) st = ar.get(&world, 9 * (size_t)n);
  if (!st) st = ar.get(&inst, n);
  if (!st) st = ar.get(&prim, n);
  if (!st) st = ar.get(&cent, n);
  if (!st) st = ar.get(&part, 6 * kReduceBlocks);
  if (!st) st = ar.get(&keys_in, n);
  if (!st) st = ar.get(&keys, n);
  if (!st) st = ar.get(&vals_in, n);
  if (!st) st = ar.get(&vals, n);
  if (!st) st = ar.get(&left, n);
  if (!st) st = ar.get(&right, n);
  if (!st) st = ar.get(&first, n);
  if (!st) st = ar.get(&last, n);
  if (!st) st = ar.get(&flag, n);
  if (!st) st = ar.get(&parent, nodes_total);
  if (!st) st = ar.get(&lo, nodes_total);
  if (!st) st = ar.get(&hi, nodes_total);
  if (!st) st = ar.get(&items_a, n);
  if (!st) st = ar.get(&items_b, n);
  if (!st) st = ar.get(&counters, 8);
  if (!st) st = ar.get(&nodes, n);
  if (!st) st = ar.get(&tris, 3 * (size_t)n);
  if (!st) st = ar.get(&order, n);
  if (st) return st;
  PBRT_CUDA(cudaMemcpy(world, world_h, 9 * (size_t)n * sizeof(float), cudaMemcpyHostToDevice));
  PBRT_CUDA(cudaMemcpy(inst, inst_h, (size_t)n * sizeof(uint32_t), cudaMemcpyHostToDevice));
  PBRT_CUDA(cudaMemcpy(prim, prim_h, (size_t)n * sizeof(uint32_t), cudaMemcpyHostToDevice));
  const int nblk = (n + kThreads - 1) / kThreads;
  const int rblk = nblk < kReduceBlocks ? nblk : kReduceBlocks;
  k_centroids<<<rblk, kThreads>>>(world, n, cent, part);
  k_morton<<<rblk, kThreads>>>(cent, n, part, rblk, keys_in, vals_in);
  if ((st = check_launch("device BVH build: Morton keys"))) return st;
  size_t temp_bytes = 0;
  PBRT_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, temp_bytes, keys_in, keys, vals_in, vals, n, 0, 63));
  void* temp = nullptr;
  if ((st = ar.get((uint8_t**)&temp, temp_bytes))) return st;
  PBRT_CUDA(cub::DeviceRadixSort::SortPairs(temp, temp_bytes, keys_in, keys, vals_in, vals, n, 0, 63));
  PBRT_CUDA(cudaMemset(parent, 0xff, nodes_total * sizeof(int)));
  PBRT_CUDA(cudaMemset(flag, 0, (size_t)n * sizeof(int)));
  if (n > 1) k_radix_tree<<<(n - 1 + kThreads - 1) / kThreads, kThreads>>>(keys, n, left, right, parent, first, last);
  // the SAH-optimal collapse (default) or, with PBRT_BVH_COLLAPSE=greedy,
  // opening the largest child until eight -- the host build's two modes
  WideDp dp{nullptr, nullptr, nullptr, nullptr, 0.3f};
  const char* mode = std::getenv("PBRT_BVH_COLLAPSE");
  if (const char* pc = std::getenv("PBRT_BVH_PRIM_COST")) dp.prim_cost = (float)std::atof(pc);
  if (!(mode && std::strcmp(mode, "greedy") == 0)) {
    if (!st) st = ar.get(&dp.cost, 8 * nodes_total);
    if (!st) st = ar.get(&dp.split, 8 * nodes_total);
    if (!st) st = ar.get(&dp.leaf, nodes_total);
    if (!st) st = ar.get(&dp.wsplit, nodes_total);
    if (st) return st;
  }
  k_boxes<<<nblk, kThreads>>>(world, vals, n, left, right, parent, first, last, lo, hi, flag, dp);
  if ((st = check_launch("device BVH build: tree"))) return st;
  // collapse, one launch a level from the root (binary node 0: internal,
  // or the only leaf when n == 1) into wide node 0. The SAH cost does not
  // see the traversal stack: on a deep, unbalanced stretch of the linear
  // tree the programme can keep one inner slot a level, so a collapse that
  // runs past max_depth is redone greedily (which opens the largest child).
  Tree tr{n, left, right, first, last, lo, hi};
  Out o{nodes, tris, order, counters, (uint32_t)n};
  int levels = 0;
  for (int attempt = 0; attempt < 2; ++attempt) {
    const unsigned init[8] = {1u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
    PBRT_CUDA(cudaMemcpy(counters, init, sizeof(init), cudaMemcpyHostToDevice));
    const uint2 root = make_uint2(0u, 0u);
    PBRT_CUDA(cudaMemcpy(items_a, &root, sizeof(root), cudaMemcpyHostToDevice));
    int level_items = 1;
    levels = 0;
    bool too_deep = false;
    while (level_items > 0) {
      if (levels > max_depth) {
        too_deep = true;
        break;
      }
      PBRT_CUDA(cudaMemset(counters + 2, 0, sizeof(unsigned)));
      k_collapse<<<(level_items + 127) / 128, 128>>>(tr, dp, world, vals, inst, prim, items_a, level_items, items_b,
                                                     o);
      if ((st = check_launch("device BVH build: collapse"))) return st;
      unsigned nxt = 0;
      PBRT_CUDA(cudaMemcpy(&nxt, counters + 2, sizeof(unsigned), cudaMemcpyDeviceToHost));
      level_items = (int)nxt;
      std::swap(items_a, items_b);
      ++levels;
    }
    if (!too_deep) break;
    if (!dp.cost || attempt == 1)
      return fail(PBRT_ERROR_UNSUPPORTED, "device BVH build: depth above %d (the traversal stack)", max_depth);
    dp.cost = nullptr;  // greedy from here
  }
  unsigned c[8];
  PBRT_CUDA(cudaMemcpy(c, counters, sizeof(c), cudaMemcpyDeviceToHost));
  if (c[4] || c[1] != (unsigned)n || c[0] > (unsigned)n)
    return fail(PBRT_ERROR_CUDA, "device BVH build: inconsistent tree (%u nodes, %u of %d triangles)", c[0], c[1], n);
  // the nodes' exact size; the triangle records are handed over as they are
  Node8* exact = nullptr;
  PBRT_CUDA(cudaMalloc((void**)&exact, (size_t)c[0] * sizeof(Node8)));
  cudaError_t e = cudaMemcpy(exact, nodes, (size_t)c[0] * sizeof(Node8), cudaMemcpyDeviceToDevice);
  if (e != cudaSuccess) {
    cudaFree(exact);
    return cuda_fail(e, "device BVH build: node copy");
  }
  ar.keep(tris);
  *nodes_out = exact;
  *tris_out = tris;
  if (stats) {
    *stats = Bvh8Stats{};
    stats->nodes = c[0];
    stats->leaves = c[3];
    stats->tris = c[1];
    stats->depth = levels - 1;
    stats->build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  return PBRT_OK;
}

}  // namespace pbrt
