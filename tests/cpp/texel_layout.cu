// Host check of the texel pool's tiled layout (texture_tile_index in
// shading.cuh, the function the shading kernels and the upload's tiling
// kernel share): for many texture sizes every texel maps to its own slot
// inside the padded allocation the scene upload makes, (w + 3 & ~3) x
// (h + 1 & ~1) texels, and a bilinear footprint's 2 x 2 texels lie in 1.875
// 32-byte sectors on average (2.25 row-major). Prints "ok" or the failure.
#include <cstdio>
#include <set>
#include <vector>

#include "shading.cuh"

int main() {
  const unsigned sizes[][2] = {{1, 1}, {2, 1}, {1, 3}, {3, 5}, {4, 2}, {5, 3}, {13, 7}, {64, 64}, {100, 37}, {1024, 1024}};
  for (const auto& s : sizes) {
    const unsigned w = s[0], h = s[1];
    const size_t cap = (size_t)((w + 3) & ~3u) * ((h + 1) & ~1u);
    std::vector<unsigned char> seen(cap, 0);
    for (unsigned y = 0; y < h; ++y)
      for (unsigned x = 0; x < w; ++x) {
        const unsigned i = pbrt::texture_tile_index(w, x, y);
        if (i >= cap || seen[i]) {
          std::printf("texture %ux%u: texel (%u, %u) -> %u (%s)\n", w, h, x, y, i, i >= cap ? "out of range" : "twice");
          return 1;
        }
        seen[i] = 1;
      }
  }
  const unsigned w = 1024, h = 1024;
  double sectors = 0.0;
  size_t n = 0;
  for (unsigned y = 0; y + 1 < h; ++y)
    for (unsigned x = 0; x + 1 < w; ++x, ++n) {
      std::set<unsigned> s;
      for (unsigned k = 0; k < 4; ++k) s.insert(pbrt::texture_tile_index(w, x + (k & 1), y + (k >> 1)) >> 3);
      sectors += (double)s.size();
    }
  sectors /= (double)n;
  if (sectors < 1.86 || sectors > 1.89) {
    std::printf("bilinear footprint: %.4f sectors on average, expected 1.875\n", sectors);
    return 1;
  }
  std::printf("ok %.4f\n", sectors);
  return 0;
}
