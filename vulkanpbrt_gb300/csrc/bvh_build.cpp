// Host BVH build: binned SAH binary tree, then collapse to Node8 (see bvh.hpp).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <future>
#include <limits>
#include <memory>
#include <thread>

#include "bvh.hpp"

namespace pbrt {
namespace {

constexpr int kMaxBins = 128;
int bins_from_env() {  // binned-SAH bins (PBRT_BVH_BINS, default 32)
  const char* e = std::getenv("PBRT_BVH_BINS");
  const int v = e ? std::atoi(e) : 32;
  return std::min(kMaxBins, std::max(4, v));
}
constexpr int kMaxLeaf = 3;
constexpr uint32_t kParallelCutoff = 1u << 15;

struct Box {
  float lo[3] = {std::numeric_limits<float>::infinity(), std::numeric_limits<float>::infinity(),
                 std::numeric_limits<float>::infinity()};
  float hi[3] = {-std::numeric_limits<float>::infinity(), -std::numeric_limits<float>::infinity(),
                 -std::numeric_limits<float>::infinity()};
  void grow(const Box& b) {
    for (int a = 0; a < 3; ++a) {
      lo[a] = std::min(lo[a], b.lo[a]);
      hi[a] = std::max(hi[a], b.hi[a]);
    }
  }
  void grow(const float* p) {
    for (int a = 0; a < 3; ++a) {
      lo[a] = std::min(lo[a], p[a]);
      hi[a] = std::max(hi[a], p[a]);
    }
  }
  double area() const {
    double d[3];
    for (int a = 0; a < 3; ++a) d[a] = std::max(0.0, (double)hi[a] - (double)lo[a]);
    return 2.0 * (d[0] * d[1] + d[1] * d[2] + d[2] * d[0]);
  }
  bool empty() const { return !(lo[0] <= hi[0]); }
};

struct BNode {
  Box box;
  int32_t left = -1, right = -1;  // children (internal) or -1 (leaf)
  uint32_t begin = 0, count = 0;  // leaf range in the index array
};

struct Builder {
  int kBins = bins_from_env();
  std::vector<Box> pbox;
  std::vector<float> cent;  // 3 per prim
  std::vector<uint32_t> idx;
  std::vector<BNode> nodes;
  std::atomic<uint32_t> next{0};
  // binary leaves: up to 3 triangles, or (with the SAH-optimal collapse)
  // single triangles, the collapse then choosing which subtrees of <= 3
  // triangles become leaves
  uint32_t binary_leaf = (uint32_t)kMaxLeaf;

  uint32_t alloc() { return next.fetch_add(1); }
  // ranges of at least kParallelScan primitives are scanned and binned in
  // scan_threads chunks
  static constexpr uint32_t kParallelScan = 1u << 17;
  const int scan_threads = std::max(1, std::min(16, (int)std::thread::hardware_concurrency()));

  // per-axis bins of a range of primitives: boxes and counts
  struct Bins {
    Box bb[3][kMaxBins];
    uint32_t bc[3][kMaxBins] = {};
    void merge(const Bins& o, int bins) {
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < bins; ++b) {
          bb[a][b].grow(o.bb[a][b]);
          bc[a][b] += o.bc[a][b];
        }
    }
  };
  void scan(uint32_t begin, uint32_t end, Box& box, Box& cb) const {
    for (uint32_t i = begin; i < end; ++i) {
      box.grow(pbox[idx[i]]);
      cb.grow(&cent[3 * idx[i]]);
    }
  }
  void bin(uint32_t begin, uint32_t end, const Box& cb, const float* k, Bins& out) const {
    for (uint32_t i = begin; i < end; ++i) {
      const uint32_t p = idx[i];
      for (int a = 0; a < 3; ++a) {
        if (!(k[a] > 0.f)) continue;
        const int b = std::min(kBins - 1, (int)((cent[3 * p + a] - cb.lo[a]) * k[a]));
        out.bb[a][b].grow(pbox[p]);
        out.bc[a][b]++;
      }
    }
  }

  void build(uint32_t ni, uint32_t begin, uint32_t count) {
    BNode& nd = nodes[ni];
    // The node's box and centroid box, then the bins of all three axes; a
    // large range in chunks on their own threads, merged in order (minima,
    // maxima and counts: the serial result)
    const int chunks = count >= kParallelScan ? scan_threads : 1;
    const uint32_t step = (count + (uint32_t)chunks - 1) / (uint32_t)chunks;
    Box box, cb;
    if (chunks == 1) {
      scan(begin, begin + count, box, cb);
    } else {
      std::vector<std::future<std::pair<Box, Box>>> f;
      for (int c = 0; c < chunks; ++c) {
        const uint32_t s = begin + std::min(count, (uint32_t)c * step), e = begin + std::min(count, (uint32_t)(c + 1) * step);
        f.push_back(std::async(std::launch::async, [=]() {
          Box bx, cx;
          scan(s, e, bx, cx);
          return std::make_pair(bx, cx);
        }));
      }
      for (auto& x : f) {
        const auto r = x.get();
        box.grow(r.first);
        cb.grow(r.second);
      }
    }
    nd.box = box;
    nd.begin = begin;
    nd.count = count;
    if (count <= binary_leaf) return;
    float kax[3];
    for (int a = 0; a < 3; ++a) {
      const float ext = cb.hi[a] - cb.lo[a];
      kax[a] = ext > 0.f ? (float)kBins / ext : 0.f;
    }
    Bins local;  // serial: on the stack (most nodes); large ranges merge into it
    Bins* bins = &local;
    if (chunks == 1) {
      bin(begin, begin + count, cb, kax, *bins);
    } else {
      std::vector<std::future<std::unique_ptr<Bins>>> f;
      for (int c = 0; c < chunks; ++c) {
        const uint32_t s = begin + std::min(count, (uint32_t)c * step), e = begin + std::min(count, (uint32_t)(c + 1) * step);
        f.push_back(std::async(std::launch::async, [=, &cb]() {
          std::unique_ptr<Bins> part(new Bins());
          bin(s, e, cb, kax, *part);
          return part;
        }));
      }
      for (auto& x : f) bins->merge(*x.get(), kBins);
    }
    // Binned SAH over all three axes.
    double best_cost = std::numeric_limits<double>::infinity();
    int best_axis = -1, best_split = -1;
    for (int a = 0; a < 3; ++a) {
      if (!(kax[a] > 0.f)) continue;
      const Box* bb = bins->bb[a];
      const uint32_t* bc = bins->bc[a];
      double ra[kMaxBins];
      uint32_t rc[kMaxBins];
      Box acc;
      uint32_t n = 0;
      for (int b = kBins - 1; b > 0; --b) {
        acc.grow(bb[b]);
        n += bc[b];
        ra[b] = acc.empty() ? 0.0 : acc.area();
        rc[b] = n;
      }
      Box lacc;
      uint32_t ln = 0;
      for (int b = 0; b < kBins - 1; ++b) {
        lacc.grow(bb[b]);
        ln += bc[b];
        if (ln == 0 || rc[b + 1] == 0) continue;
        double c = (lacc.empty() ? 0.0 : lacc.area()) * ln + ra[b + 1] * rc[b + 1];
        if (c < best_cost) {
          best_cost = c;
          best_axis = a;
          best_split = b;
        }
      }
    }
    uint32_t mid;
    if (best_axis < 0) {
      mid = begin + count / 2;  // identical centroids: split by index
    } else {
      float k = (float)kBins / (cb.hi[best_axis] - cb.lo[best_axis]);
      auto it = std::partition(idx.begin() + begin, idx.begin() + begin + count, [&](uint32_t p) {
        int b = std::min(kBins - 1, (int)((cent[3 * p + best_axis] - cb.lo[best_axis]) * k));
        return b <= best_split;
      });
      mid = (uint32_t)(it - idx.begin());
      if (mid == begin || mid == begin + count) mid = begin + count / 2;
    }
    uint32_t l = alloc(), r = alloc();
    nd.left = (int32_t)l;
    nd.right = (int32_t)r;
    uint32_t lc = mid - begin, rc = begin + count - mid;
    if (count > kParallelCutoff) {
      auto f = std::async(std::launch::async, [=]() { build(l, begin, lc); });
      build(r, mid, rc);
      f.get();
    } else {
      build(l, begin, lc);
      build(r, mid, rc);
    }
  }
};

// SAH-optimal collapse of the binary tree into 8-wide nodes (the dynamic
// programme of Ylitie, Karras & Laine, HPG 2017, section 3.1): for every
// binary node n and i = 1..8, cost[n][i] is the cheapest way to represent
// n's subtree as at most i child slots of a wide node, a slot being a leaf
// (<= 3 triangles, cost area x kPrim x count) or a wide node (cost
// area x kNode + its best 8-slot distribution).
struct WideDP {
  static constexpr float kNode = 1.0f;
  float kPrim = 0.3f;  // triangle test vs node visit cost (PBRT_BVH_PRIM_COST)
  static constexpr float kInf = std::numeric_limits<float>::infinity();
  const Builder& b;
  std::vector<float> cost;      // [node][9], index 1..8
  std::vector<int8_t> split;    // [node][9]: left share k of a distribution, 0 = take i - 1, -1 = single slot
  std::vector<uint8_t> is_leaf; // slot type when the node is one slot
  std::vector<int8_t> wide_split;  // left share of the 8-slot distribution of a wide node
  explicit WideDP(const Builder& bb) : b(bb) {}

  void solve(uint32_t root) {
    const size_t n = b.next.load();
    cost.assign(n * 9, kInf);
    split.assign(n * 9, -1);
    is_leaf.assign(n, 0);
    wide_split.assign(n, 1);
    post_order(root);
  }

  // children before parents; large subtrees on their own threads (a node's
  // values depend on its children's alone, so the result is the serial one)
  void post_order(uint32_t ni) {
    const BNode& nd = b.nodes[ni];
    if (nd.left >= 0) {
      if (nd.count > kParallelCutoff) {
        auto f = std::async(std::launch::async, [=]() { post_order((uint32_t)nd.left); });
        post_order((uint32_t)nd.right);
        f.get();
      } else {
        post_order((uint32_t)nd.left);
        post_order((uint32_t)nd.right);
      }
    }
    node(ni);
  }

  void node(uint32_t ni) {
    const BNode& nd = b.nodes[ni];
    float* c = &cost[9 * (size_t)ni];
    int8_t* sp = &split[9 * (size_t)ni];
    const float area = (float)nd.box.area();
    const float leafc = nd.count <= (uint32_t)kMaxLeaf ? area * kPrim * (float)nd.count : kInf;
    if (nd.left < 0) {
      for (int i = 1; i <= 8; ++i) c[i] = leafc;
      is_leaf[ni] = 1;
      return;
    }
    const float* cl = &cost[9 * (size_t)nd.left];
    const float* cr = &cost[9 * (size_t)nd.right];
    float dist[9];
    int8_t arg[9];
    for (int j = 2; j <= 8; ++j) {
      dist[j] = kInf;
      arg[j] = 1;
      for (int k = 1; k < j; ++k) {
        const float v = cl[k] + cr[j - k];
        if (v < dist[j]) {
          dist[j] = v;
          arg[j] = (int8_t)k;
        }
      }
    }
    const float internal = area * kNode + dist[8];
    is_leaf[ni] = leafc <= internal ? 1 : 0;
    c[1] = std::min(leafc, internal);
    sp[1] = -1;
    for (int i = 2; i <= 8; ++i) {
      if (dist[i] < c[i - 1]) {
        c[i] = dist[i];
        sp[i] = arg[i];
      } else {
        c[i] = c[i - 1];
        sp[i] = 0;
      }
    }
    wide_split[ni] = arg[8];
  }

  // the slots representing node ni with at most i of them
  void slots(uint32_t ni, int i, uint32_t* out, int& n) const {
    const int8_t s = split[9 * (size_t)ni + i];
    if (i == 1 || s < 0) {
      out[n++] = ni;
      return;
    }
    if (s == 0) {
      slots(ni, i - 1, out, n);
      return;
    }
    const BNode& nd = b.nodes[ni];
    slots((uint32_t)nd.left, s, out, n);
    slots((uint32_t)nd.right, i - s, out, n);
  }
  // children slots (at most 8) of the wide node made from binary node ni
  void children(uint32_t ni, uint32_t* out, int& n) const {
    const BNode& nd = b.nodes[ni];
    const int k = wide_split[ni];
    slots((uint32_t)nd.left, k, out, n);
    slots((uint32_t)nd.right, 8 - k, out, n);
  }
};

struct Collapser {
  const Builder& b;
  std::vector<Node8>& out;
  std::vector<uint32_t>& tri_order;
  Bvh8Stats st;
  const WideDP* dp = nullptr;  // SAH collapse (else: open the largest child)
  // The output is laid out depth first: a wide node's children block is
  // appended when the node is encoded, after its earlier siblings' whole
  // subtrees; its leaves' triangles likewise. wide_below[b] (wide nodes
  // under the one made from binary node b) gives every subtree its ranges
  // in advance, so subtrees are encoded on their own threads into the same
  // places.
  std::vector<uint32_t> wide_below;
  std::atomic<int> max_depth{0};
  std::atomic<size_t> leaves{0};

  bool leaf_slot(uint32_t c) const { return b.nodes[c].left < 0 || (dp && dp->is_leaf[c]); }

  static uint8_t exponent_for(double extent) {
    // smallest power of two s with extent / s <= 255 (extent taken in double)
    if (!(extent > 0.0)) return 1;  // 2^-126
    int e;
    std::frexp(extent / 255.0, &e);  // extent/255 = m * 2^e with m in [0.5, 1), so 2^e > extent/255
    return (uint8_t)std::min(254, std::max(1, e + 127));
  }

  // the child slots of the wide node made from binary node bnode
  int gather(uint32_t bnode, uint32_t* ch) const {
    // Open the largest child until 8 children (or only leaves remain).
    int nch = 0;
    const BNode& root = b.nodes[bnode];
    if (root.left < 0) {
      ch[nch++] = bnode;  // single leaf under this node
    } else if (dp) {
      dp->children(bnode, ch, nch);
    } else {
      ch[nch++] = (uint32_t)root.left;
      ch[nch++] = (uint32_t)root.right;
      while (nch < 8) {
        int best = -1;
        double best_area = -1.0;
        for (int i = 0; i < nch; ++i) {
          const BNode& c = b.nodes[ch[i]];
          if (c.left < 0) continue;
          double a = c.box.area();
          if (a > best_area) {
            best_area = a;
            best = i;
          }
        }
        if (best < 0) break;
        uint32_t open = ch[best];
        ch[best] = (uint32_t)b.nodes[open].left;
        ch[nch++] = (uint32_t)b.nodes[open].right;
      }
    }
    return nch;
  }

  uint32_t count_below(uint32_t bnode) {
    uint32_t ch[8];
    const int nch = gather(bnode, ch);
    uint32_t sum = 0;
    std::future<uint32_t> big[8];
    bool async_[8] = {false};
    for (int i = 0; i < nch; ++i) {
      if (leaf_slot(ch[i])) continue;
      if (b.nodes[ch[i]].count > kParallelCutoff) {
        const uint32_t c = ch[i];
        big[i] = std::async(std::launch::async, [this, c]() { return count_below(c); });
        async_[i] = true;
      } else {
        sum += 1 + count_below(ch[i]);
      }
    }
    for (int i = 0; i < nch; ++i)
      if (async_[i]) sum += 1 + big[i].get();
    wide_below[bnode] = sum;
    return sum;
  }

  // the wide node made from binary node bnode into out[out_index]; its
  // children block at child_base, its leaves' triangles from tri_base on
  void encode(uint32_t out_index, uint32_t bnode, int depth, uint32_t child_base, uint32_t tri_base) {
    for (int d = max_depth.load(); depth > d && !max_depth.compare_exchange_weak(d, depth);) {
    }
    uint32_t ch[8];
    const int nch = gather(bnode, ch);
    const BNode& root = b.nodes[bnode];
    // Leaves with more than 3 triangles (identical centroids beyond the leaf
    // size) cannot happen: build() splits them by index.
    const Box& nb = root.box;
    // Octant slot assignment around the node's centre.
    float pc[3];
    for (int a = 0; a < 3; ++a) pc[a] = 0.5f * (nb.lo[a] + nb.hi[a]);
    int slot_of[8];
    bool used[8] = {false};
    bool placed[8] = {false};
    // each child's score for each slot (its centre's offset along the slot's
    // octant direction), once; the rounds then take the best free pair
    double score_of[8][8];
    for (int i = 0; i < nch; ++i) {
      const Box& cbx = b.nodes[ch[i]].box;
      double d[3];
      for (int a = 0; a < 3; ++a) d[a] = 0.5 * ((double)cbx.lo[a] + cbx.hi[a]) - pc[a];
      for (int s = 0; s < 8; ++s)
        score_of[i][s] = (s & 1 ? d[0] : -d[0]) + (s & 2 ? d[1] : -d[1]) + (s & 4 ? d[2] : -d[2]);
    }
    for (int round = 0; round < nch; ++round) {
      double best = -std::numeric_limits<double>::infinity();
      int bc = -1, bs = -1;
      for (int i = 0; i < nch; ++i) {
        if (placed[i]) continue;
        for (int s = 0; s < 8; ++s) {
          if (used[s]) continue;
          const double score = score_of[i][s];
          if (score > best) {
            best = score;
            bc = i;
            bs = s;
          }
        }
      }
      placed[bc] = true;
      used[bs] = true;
      slot_of[bc] = bs;
    }
    uint32_t slot_child[8];
    bool slot_used[8] = {false};
    for (int i = 0; i < nch; ++i) {
      slot_child[slot_of[i]] = ch[i];
      slot_used[slot_of[i]] = true;
    }
    Node8 n;
    std::memset(&n, 0, sizeof(n));
    n.px = nb.lo[0];
    n.py = nb.lo[1];
    n.pz = nb.lo[2];
    uint8_t ex[3];
    float scale[3];
    for (int a = 0; a < 3; ++a) {
      ex[a] = exponent_for((double)nb.hi[a] - (double)nb.lo[a]);
      scale[a] = std::ldexp(1.0f, (int)ex[a] - 127);
    }
    n.ex = ex[0];
    n.ey = ex[1];
    n.ez = ex[2];
    const float p[3] = {n.px, n.py, n.pz};
    // internal children first (to allocate them consecutively), in slot order
    uint32_t inner[8];  // binary nodes of the internal children, slot order
    int ninner = 0;
    uint32_t tri_off = 0;
    n.tri_base = tri_base;
    for (int s = 0; s < 8; ++s) {
      if (!slot_used[s]) continue;
      const BNode& c = b.nodes[slot_child[s]];
      const bool is_leaf = leaf_slot(slot_child[s]);
      for (int a = 0; a < 3; ++a) {
        double lo = std::floor(((double)c.box.lo[a] - p[a]) / scale[a]);
        double hi = std::ceil(((double)c.box.hi[a] - p[a]) / scale[a]);
        n.qlo[a][s] = (uint8_t)std::min(255.0, std::max(0.0, lo));
        n.qhi[a][s] = (uint8_t)std::min(255.0, std::max(0.0, hi));
      }
      if (!is_leaf) {
        n.imask |= (uint8_t)(1u << s);
        n.meta[s] = 0x80;
        inner[ninner++] = slot_child[s];
      } else {
        n.meta[s] = (uint8_t)((c.count << 5) | tri_off);
        for (uint32_t k = 0; k < c.count; ++k) tri_order[tri_base + tri_off + k] = b.idx[c.begin + k];
        tri_off += c.count;
        leaves.fetch_add(1, std::memory_order_relaxed);
      }
    }
    n.child_base = child_base;
    out[out_index] = n;
    // each inner child's subtree: its block after the earlier siblings' subtrees
    uint32_t next_node = child_base + (uint32_t)ninner, next_tri = tri_base + tri_off;
    std::vector<std::future<void>> big;
    for (int i = 0; i < ninner; ++i) {
      const uint32_t c = inner[i], idx = child_base + (uint32_t)i, cb = next_node, tb = next_tri;
      if (b.nodes[c].count > kParallelCutoff)
        big.push_back(std::async(std::launch::async, [=]() { encode(idx, c, depth + 1, cb, tb); }));
      else
        encode(idx, c, depth + 1, cb, tb);
      next_node += wide_below[c];
      next_tri += b.nodes[c].count;
    }
    for (auto& f : big) f.get();
  }
};

}  // namespace

void build_bvh8(const float* v, size_t n, std::vector<Node8>& nodes, std::vector<uint32_t>& tri_order,
                Bvh8Stats* stats) {
  auto t0 = std::chrono::steady_clock::now();
  Builder b;
  b.pbox.resize(n);
  b.cent.resize(3 * n);
  b.idx.resize(n);
  for (size_t i = 0; i < n; ++i) {
    Box bx;
    bx.grow(v + 9 * i);
    bx.grow(v + 9 * i + 3);
    bx.grow(v + 9 * i + 6);
    b.pbox[i] = bx;
    for (int a = 0; a < 3; ++a) b.cent[3 * i + a] = 0.5f * (bx.lo[a] + bx.hi[a]);
    b.idx[i] = (uint32_t)i;
  }
  b.nodes.resize(std::max<size_t>(1, 2 * n));
  // PBRT_BVH_COLLAPSE=greedy: open the largest child until 8 (the default is
  // the SAH-optimal collapse)
  const char* mode = std::getenv("PBRT_BVH_COLLAPSE");
  const bool greedy = mode && std::strcmp(mode, "greedy") == 0;
  if (!greedy) {
    const char* bl = std::getenv("PBRT_BVH_BINARY_LEAF");
    b.binary_leaf = (uint32_t)std::min(kMaxLeaf, std::max(1, bl ? std::atoi(bl) : 1));
  }
  uint32_t root = b.alloc();
  b.build(root, 0, (uint32_t)n);
  nodes.clear();
  tri_order.clear();
  WideDP dp(b);
  if (const char* pc = std::getenv("PBRT_BVH_PRIM_COST")) dp.kPrim = (float)std::atof(pc);
  Collapser c{b, nodes, tri_order, {}};
  if (!greedy && b.nodes[root].left >= 0) {
    dp.solve(root);
    c.dp = &dp;
  }
  c.wide_below.assign(b.next.load(), 0);
  // the root is distributed over its children unless it is a single triangle leaf
  const uint32_t below = b.nodes[root].left < 0 ? 0u : c.count_below(root);
  nodes.resize(1 + (size_t)below);
  tri_order.resize(n);
  c.encode(0, root, 0, 1, 0);
  c.st.depth = c.max_depth.load();
  c.st.leaves = c.leaves.load();
  if (stats) {
    *stats = c.st;
    stats->nodes = nodes.size();
    stats->tris = tri_order.size();
    stats->build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
}

}  // namespace pbrt
