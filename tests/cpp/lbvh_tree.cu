// Host check of the device BVH build's radix tree (lbvh.cuh, the code the
// build's kernel runs): over sorted random 63-bit keys with runs of equal
// keys, every internal node's two children split its range of sorted
// positions exactly, node 0 spans all keys, and every other node has one
// parent (so the tree reaches each leaf once). Prints "ok" or the failure.
#include <algorithm>
#include <cstdio>
#include <random>
#include <vector>

#include "lbvh.cuh"

static int check(int n, unsigned seed, int dup_bits) {
  std::mt19937_64 rng(seed);
  std::vector<uint64_t> k(n);
  for (auto& v : k) v = (rng() >> 1) >> dup_bits << dup_bits;  // low bits cleared: equal keys
  std::sort(k.begin(), k.end());
  std::vector<int> L(n), R(n), lo(n), hi(n), parents(2 * n - 1, 0);
  for (int i = 0; i < n - 1; ++i) pbrt::lbvh::radix_node(k.data(), n, i, &L[i], &R[i], &lo[i], &hi[i]);
  auto range = [&](int c, int& a, int& b) {
    if (c >= n - 1) a = b = c - (n - 1);
    else a = lo[c], b = hi[c];
  };
  if (lo[0] != 0 || hi[0] != n - 1) {
    std::printf("n %d: root spans [%d, %d]\n", n, lo[0], hi[0]);
    return 1;
  }
  for (int i = 0; i < n - 1; ++i) {
    int la, lb, ra, rb;
    range(L[i], la, lb);
    range(R[i], ra, rb);
    if (la != lo[i] || rb != hi[i] || lb + 1 != ra || L[i] < 0 || R[i] < 0 || L[i] >= 2 * n - 1 || R[i] >= 2 * n - 1) {
      std::printf("n %d: node %d [%d, %d] -> [%d, %d] + [%d, %d]\n", n, i, lo[i], hi[i], la, lb, ra, rb);
      return 1;
    }
    ++parents[L[i]];
    ++parents[R[i]];
  }
  for (int c = 1; c < 2 * n - 1; ++c)
    if (parents[c] != 1) {
      std::printf("n %d: node %d has %d parents\n", n, c, parents[c]);
      return 1;
    }
  if (parents[0] != 0) return 1;
  return 0;
}

int main() {
  int bad = 0;
  for (int n : {2, 3, 4, 5, 7, 16, 100, 1000, 65537})
    for (int dup : {0, 40, 58, 63})  // 63: every key equal (the index orders the whole tree)
      bad |= check(n, 1234u + (unsigned)n, dup);
  // the Morton interleave: bit b of the axis value lands on bit 3b
  for (int b = 0; b < 21; ++b)
    if (pbrt::lbvh::spread21(1ull << b) != 1ull << (3 * b)) {
      std::printf("spread21: bit %d\n", b);
      bad = 1;
    }
  if (!bad) std::printf("ok\n");
  return bad;
}
