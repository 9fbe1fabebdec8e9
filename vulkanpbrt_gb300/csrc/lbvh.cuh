// The radix tree of the device BVH build (bvh_gpu.cu), as host/device
// functions so that the same code runs in the build's kernel and in host
// checks: Karras, "Maximizing Parallelism in the Construction of BVHs,
// Octrees, and k-d Trees" (HPG 2012), over 63-bit Morton keys sorted
// ascending, equal keys ordered by their index.
#pragma once
#include <stdint.h>

#include "device_common.cuh"

namespace pbrt {
namespace lbvh {

// 21-bit value -> bits at positions 3k (the "magic bits" interleave).
PBRT_HD uint64_t spread21(uint64_t v) {
  v &= 0x1fffffull;
  v = (v | v << 32) & 0x1f00000000ffffull;
  v = (v | v << 16) & 0x1f0000ff0000ffull;
  v = (v | v << 8) & 0x100f00f00f00f00full;
  v = (v | v << 4) & 0x10c30c30c30c30c3ull;
  v = (v | v << 2) & 0x1249249249249249ull;
  return v;
}

PBRT_HD int clz64(uint64_t v) {  // v != 0
#ifdef __CUDA_ARCH__
  return __clzll((long long)v);
#else
  return __builtin_clzll(v);
#endif
}
PBRT_HD int clz32(uint32_t v) {  // v != 0
#ifdef __CUDA_ARCH__
  return __clz((int)v);
#else
  return __builtin_clz(v);
#endif
}

// Length of the common prefix of sorted keys i and j (the index breaks ties),
// -1 outside [0, n); i != j.
PBRT_HD int delta(const uint64_t* k, long long n, long long i, long long j) {
  if (j < 0 || j >= n) return -1;
  const uint64_t a = k[i], b = k[j];
  if (a == b) return 64 + clz32((uint32_t)i ^ (uint32_t)j);
  return clz64(a ^ b);
}

// Internal node i (0 <= i < n - 1) of the tree over n >= 2 sorted keys: its
// children (an internal index, or n - 1 + a leaf's sorted position) and the
// range [lo, hi] of sorted positions it covers.
PBRT_HD void radix_node(const uint64_t* k, int n, int i, int* left, int* right, int* lo, int* hi) {
  const int d = delta(k, n, i, i + 1) - delta(k, n, i, i - 1) >= 0 ? 1 : -1;
  const int dmin = delta(k, n, i, (long long)i - d);
  long long lmax = 2;
  while (delta(k, n, i, i + lmax * d) > dmin) lmax <<= 1;  // ends once i + lmax * d leaves [0, n)
  long long l = 0;
  for (long long t = lmax >> 1; t >= 1; t >>= 1)
    if (delta(k, n, i, i + (l + t) * d) > dmin) l += t;
  const long long j = i + l * d;
  const int dnode = delta(k, n, i, j);
  long long s = 0;
  for (long long div = 2;; div <<= 1) {
    const long long t = (l + div - 1) / div;
    if (delta(k, n, i, i + (s + t) * d) > dnode) s += t;
    if (t == 1) break;
  }
  const int gamma = (int)(i + s * d + (d < 0 ? -1 : 0));
  *lo = (int)(i < j ? i : j);
  *hi = (int)(i < j ? j : i);
  *left = *lo == gamma ? n - 1 + gamma : gamma;
  *right = *hi == gamma + 1 ? n - 1 + gamma + 1 : gamma + 1;
}

}  // namespace lbvh
}  // namespace pbrt
