// Procedural RGBA8 textures for the seeded synthetic scenes (no reference
// counterpart: the reference loads textures through assimp). Tileable value
// noise (hashed integer lattice, smoothstep interpolation, 5 octaves), on the
// host over all cores.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <thread>
#include <vector>

#include "internal.hpp"

namespace {

inline uint32_t mix32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

inline float lattice(uint32_t seed, int ix, int iy, int period) {
  ix = ((ix % period) + period) % period;
  iy = ((iy % period) + period) % period;
  uint32_t h = mix32(seed ^ mix32((uint32_t)ix * 0x9E3779B1u ^ mix32((uint32_t)iy + 0x632BE5ABu)));
  return (float)(h >> 8) * (1.0f / 16777216.0f);
}

inline float smooth(float t) { return t * t * (3.f - 2.f * t); }

// Tileable value noise at (u, v) in [0,1)^2 with `period` cells per side.
inline float value_noise(uint32_t seed, float u, float v, int period) {
  float x = u * (float)period, y = v * (float)period;
  int ix = (int)std::floor(x), iy = (int)std::floor(y);
  float fx = smooth(x - (float)ix), fy = smooth(y - (float)iy);
  float a = lattice(seed, ix, iy, period), b = lattice(seed, ix + 1, iy, period);
  float c = lattice(seed, ix, iy + 1, period), d = lattice(seed, ix + 1, iy + 1, period);
  float ab = a + (b - a) * fx, cd = c + (d - c) * fx;
  return ab + (cd - ab) * fy;
}

inline float fbm(uint32_t seed, float u, float v) {
  float s = 0.f, amp = 0.5f, norm = 0.f;
  int period = 4;
  for (int o = 0; o < 5; ++o) {
    s += amp * value_noise(seed + 0x1000193u * (uint32_t)o, u, v, period);
    norm += amp;
    amp *= 0.5f;
    period *= 2;
  }
  return s / norm;
}

inline uint8_t to_u8(float x) {
  x = std::min(std::max(x, 0.f), 1.f);
  return (uint8_t)std::floor(x * 255.f + 0.5f);
}

template <class F> void rows_parallel(int h, F f) {
  int n = (int)std::max(1u, std::thread::hardware_concurrency());
  n = std::min(n, std::max(1, h / 16));
  std::vector<std::thread> pool;
  for (int t = 0; t < n; ++t)
    pool.emplace_back([&, t]() {
      for (int y = t; y < h; y += n) f(y);
    });
  for (auto& th : pool) th.join();
}

}  // namespace

extern "C" {

// kind 0: albedo (rgb = colour * (0.55 + 0.45 * noise), stored sRGB-encoded
//         because the shaders linearise with pow(x, 2.2); a = 255, or holes
//         (a = 0) where a second noise field < 0.38 when alpha_mask != 0);
// kind 1: specular (rgb = colour, sRGB-encoded; a = roughness in
//         [rough_lo, rough_hi] from noise, linear);
// kind 2: tangent-space normal map from a noise height field.
PBRT_API int pbrt_synth_texture(uint64_t seed, uint32_t size, int32_t kind, const float* color, int32_t alpha_mask,
                                float rough_lo, float rough_hi, uint8_t* out_rgba) {
  if (!out_rgba || size == 0 || size > 16384 || kind < 0 || kind > 2 || (kind != 2 && !color))
    return pbrt::fail(PBRT_ERROR_INVALID_ARGUMENT, "pbrt_synth_texture: bad arguments");
  const int W = (int)size;
  const uint32_t s0 = (uint32_t)(seed ^ (seed >> 32)) * 0x9E3779B1u + 0x7F4A7C15u;
  const float inv = 1.f / (float)W;
  const float g = 1.f / 2.2f;
  if (kind == 2) {
    std::vector<float> hgt((size_t)W * W);
    rows_parallel(W, [&](int y) {
      for (int x = 0; x < W; ++x) hgt[(size_t)y * W + x] = fbm(s0, ((float)x + .5f) * inv, ((float)y + .5f) * inv);
    });
    const float strength = 0.02f * (float)W;
    rows_parallel(W, [&](int y) {
      for (int x = 0; x < W; ++x) {
        int xm = (x + W - 1) % W, xp = (x + 1) % W, ym = (y + W - 1) % W, yp = (y + 1) % W;
        float dx = (hgt[(size_t)y * W + xp] - hgt[(size_t)y * W + xm]) * 0.5f * strength;
        float dy = (hgt[(size_t)yp * W + x] - hgt[(size_t)ym * W + x]) * 0.5f * strength;
        float nx = -dx, ny = -dy, nz = 1.f;
        float l = std::sqrt(nx * nx + ny * ny + nz * nz);
        uint8_t* o = out_rgba + 4 * ((size_t)y * W + x);
        o[0] = to_u8(nx / l * .5f + .5f);
        o[1] = to_u8(ny / l * .5f + .5f);
        o[2] = to_u8(nz / l * .5f + .5f);
        o[3] = 255;
      }
    });
    return PBRT_OK;
  }
  rows_parallel(W, [&](int y) {
    for (int x = 0; x < W; ++x) {
      float u = ((float)x + .5f) * inv, v = ((float)y + .5f) * inv;
      uint8_t* o = out_rgba + 4 * ((size_t)y * W + x);
      if (kind == 0) {
        float n = fbm(s0, u, v), m = value_noise(s0 + 77u, u, v, 16);
        const float hue[3] = {m, 1.f - m, 0.5f};
        for (int c = 0; c < 3; ++c) {
          float t = 0.55f + 0.45f * (0.3f * hue[c] + 0.7f * n);
          o[c] = to_u8(std::pow(std::min(color[c] * t, 1.f), g));
        }
        o[3] = 255;
        if (alpha_mask && fbm(s0 ^ 0xA5A5A5A5u, u, v) < 0.38f) o[3] = 0;
      } else {
        for (int c = 0; c < 3; ++c) o[c] = to_u8(std::pow(std::min(color[c], 1.f), g));
        o[3] = to_u8(rough_lo + (rough_hi - rough_lo) * fbm(s0, u, v));
      }
    }
  });
  return PBRT_OK;
}

}  // extern "C"
