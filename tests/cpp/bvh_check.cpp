// Host check of the host BVH build (bvh_build.cpp): over random triangles
// (with duplicates and degenerate ones) the 8-wide tree covers every
// triangle exactly once, and every quantised child box (origin + 2^(e-127)
// x the 8-bit offsets) contains its whole subtree -- the conservative bounds
// the traversal relies on. Run under each collapse mode and binary leaf size
// the caller selects through the environment. Prints "ok" or the failure.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "bvh.hpp"

using pbrt::Node8;

struct Box {
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  void grow(const float* p) {
    for (int a = 0; a < 3; ++a) {
      lo[a] = std::fmin(lo[a], p[a]);
      hi[a] = std::fmax(hi[a], p[a]);
    }
  }
  void grow(const Box& b) {
    for (int a = 0; a < 3; ++a) {
      lo[a] = std::fmin(lo[a], b.lo[a]);
      hi[a] = std::fmax(hi[a], b.hi[a]);
    }
  }
};

static const std::vector<float>* g_v;
static const std::vector<Node8>* g_nodes;
static const std::vector<uint32_t>* g_order;
static std::vector<int> g_seen;
static int g_err = 0;

static Box walk(uint32_t ni, int depth) {
  const Node8& n = (*g_nodes)[ni];
  Box all;
  const float p[3] = {n.px, n.py, n.pz};
  const uint8_t e[3] = {n.ex, n.ey, n.ez};
  int inner = 0;
  for (int s = 0; s < 8; ++s) {
    if (n.meta[s] == 0) continue;
    Box cb;
    if (n.meta[s] == 0x80) {
      cb = walk(n.child_base + (uint32_t)inner++, depth + 1);
    } else {
      const int cnt = n.meta[s] >> 5, off = n.meta[s] & 31;
      for (int k = 0; k < cnt; ++k) {
        const uint32_t t = (*g_order)[n.tri_base + off + k];
        ++g_seen[t];
        for (int c = 0; c < 3; ++c) cb.grow(&(*g_v)[9 * (size_t)t + 3 * c]);
      }
    }
    for (int a = 0; a < 3; ++a) {
      const double sc = std::ldexp(1.0, (int)e[a] - 127);
      const double lo = p[a] + sc * n.qlo[a][s], hi = p[a] + sc * n.qhi[a][s];
      if (!(lo <= cb.lo[a] && cb.hi[a] <= hi)) {
        if (g_err++ < 5)
          std::printf("node %u slot %d axis %d: box [%g, %g] does not hold [%g, %g]\n", ni, s, a, lo, hi, cb.lo[a],
                      cb.hi[a]);
      }
    }
    all.grow(cb);
  }
  if ((n.imask != 0) != (inner > 0)) ++g_err;
  return all;
}

int main() {
  std::mt19937 rng(7);
  std::uniform_real_distribution<float> u(-50.f, 50.f), d(-0.5f, 0.5f);
  for (size_t ntri : {1u, 2u, 3u, 4u, 9u, 100u, 5000u, 60000u}) {
    std::vector<float> v(9 * ntri);
    for (size_t t = 0; t < ntri; ++t) {
      const float c[3] = {u(rng), u(rng), u(rng)};
      for (int k = 0; k < 9; ++k) v[9 * t + k] = c[k % 3] + d(rng);
      if (t % 17 == 5 && t >= 1)  // a duplicate of the previous triangle
        for (int k = 0; k < 9; ++k) v[9 * t + k] = v[9 * (t - 1) + k];
      if (t % 23 == 7)  // a degenerate one (a point)
        for (int k = 3; k < 9; ++k) v[9 * t + k] = v[9 * t + k % 3];
    }
    std::vector<Node8> nodes;
    std::vector<uint32_t> order;
    pbrt::Bvh8Stats st;
    pbrt::build_bvh8(v.data(), ntri, nodes, order, &st);
    g_v = &v;
    g_nodes = &nodes;
    g_order = &order;
    g_seen.assign(ntri, 0);
    walk(0, 0);
    for (size_t t = 0; t < ntri; ++t)
      if (g_seen[t] != 1) {
        if (g_err++ < 5) std::printf("%zu triangles: triangle %zu reached %d times\n", ntri, t, g_seen[t]);
      }
    if (order.size() != ntri || st.nodes != nodes.size()) ++g_err;
  }
  if (g_err) return 1;
  std::printf("ok\n");
  return 0;
}
