"""Procedural RGBA8 textures for the seeded synthetic scenes.

No reference counterpart: the reference loads its textures through assimp.
Tileable value noise (hashed integer lattice, smoothstep interpolation, five
octaves) in plain numpy FP32, one texture per call. Value noise is separable:
the lattice index and the smoothstep weight of a texel depend on its column
(x) or on its row (y) alone, so each octave interpolates the small lattice
along x once per lattice row and then along y once per texel -- the same
FP32 operations in the same order as a per-texel evaluation, at a few
array passes per octave. Pure numpy keeps scene generation free of the
native library, so the CPU restatement can build the same scenes.
"""
from __future__ import annotations

import numpy as np

KINDS = {"albedo": 0, "specular": 1, "normal": 2}
_M32 = np.uint64(0xFFFFFFFF)


def _u32(x) -> np.ndarray:
    return np.asarray(x, np.uint64) & _M32


def _mix32(x: np.ndarray) -> np.ndarray:
    """32-bit integer finaliser (xorshift-multiply); operands held in uint64."""
    x = _u32(x)
    x = x ^ (x >> np.uint64(16))
    x = (x * np.uint64(0x7FEB352D)) & _M32
    x = x ^ (x >> np.uint64(15))
    x = (x * np.uint64(0x846CA68B)) & _M32
    return x ^ (x >> np.uint64(16))


def _lattice(seed: int, period: int) -> np.ndarray:
    """[period, period] lattice values in [0, 1), indexed [iy, ix]."""
    i = np.arange(period, dtype=np.uint64)
    hx = (i * np.uint64(0x9E3779B1)) & _M32  # per ix
    hy = _mix32(i + np.uint64(0x632BE5AB))  # per iy
    h = _mix32(np.uint64(seed) ^ _mix32(hx[None, :] ^ hy[:, None]))
    return (h >> np.uint64(8)).astype(np.float32) * np.float32(1.0 / 16777216.0)


def _axis(coord: np.ndarray, period: int):
    """Per-column (or per-row) lattice cell, its neighbour and smoothstep weight."""
    x = coord * np.float32(period)
    i = np.floor(x)
    t = x - i
    w = t * t * (np.float32(3.0) - np.float32(2.0) * t)
    i = i.astype(np.int64)
    return i % period, (i + 1) % period, w


def value_noise(seed: int, u: np.ndarray, v: np.ndarray, period: int) -> np.ndarray:
    """Tileable value noise on the grid u (columns) x v (rows), both in [0,1)."""
    L = _lattice(seed & 0xFFFFFFFF, period)
    ix0, ix1, fx = _axis(u, period)
    iy0, iy1, fy = _axis(v, period)
    a = L[:, ix0]
    row = a + (L[:, ix1] - a) * fx[None, :]  # [period, W]: interpolated along x per lattice row
    ab = row[iy0]
    return ab + (row[iy1] - ab) * fy[:, None]


def fbm(seed: int, u: np.ndarray, v: np.ndarray) -> np.ndarray:
    s = np.zeros((len(v), len(u)), np.float32)
    amp, norm, period = np.float32(0.5), np.float32(0.0), 4
    for o in range(5):
        s = s + amp * value_noise((seed + 0x1000193 * o) & 0xFFFFFFFF, u, v, period)
        norm = norm + amp
        amp = amp * np.float32(0.5)
        period *= 2
    return s / norm


def _to_u8(x: np.ndarray) -> np.ndarray:
    x = np.minimum(np.maximum(x, np.float32(0.0)), np.float32(1.0))
    return np.floor(x * np.float32(255.0) + np.float32(0.5)).astype(np.uint8)


def synth_texture(seed: int, size: int, kind: str, color=(1.0, 1.0, 1.0), alpha_mask: bool = False,
                  rough_lo: float = 0.2, rough_hi: float = 0.8) -> np.ndarray:
    """One size x size RGBA8 texture.

    kind "albedo": rgb = colour * (0.55 + 0.45 * noise), stored sRGB-encoded
    (the shaders linearise with pow(x, 2.2)); a = 255, or 0 (holes) where a
    second noise field is below 0.38 when alpha_mask is set.
    kind "specular": rgb = colour (sRGB-encoded); a = roughness in
    [rough_lo, rough_hi] from noise, linear.
    kind "normal": tangent-space normal map of a noise height field.
    """
    if kind not in KINDS or not 0 < size <= 16384:
        raise ValueError(f"synth_texture: bad kind {kind!r} or size {size}")
    seed &= (1 << 64) - 1
    s0 = ((((seed ^ (seed >> 32)) & 0xFFFFFFFF) * 0x9E3779B1) + 0x7F4A7C15) & 0xFFFFFFFF
    W = int(size)
    inv = np.float32(1.0) / np.float32(W)
    c = (np.arange(W, dtype=np.float32) + np.float32(0.5)) * inv
    out = np.empty((W, W, 4), np.uint8)
    g = np.float32(1.0) / np.float32(2.2)
    if kind == "normal":
        h = fbm(s0, c, c)
        strength = np.float32(0.02) * np.float32(W)
        dx = (np.roll(h, -1, axis=1) - np.roll(h, 1, axis=1)) * np.float32(0.5) * strength
        dy = (np.roll(h, -1, axis=0) - np.roll(h, 1, axis=0)) * np.float32(0.5) * strength
        nx, ny = -dx, -dy
        nz = np.float32(1.0)
        ln = np.sqrt(nx * nx + ny * ny + nz * nz)
        out[..., 0] = _to_u8(nx / ln * np.float32(0.5) + np.float32(0.5))
        out[..., 1] = _to_u8(ny / ln * np.float32(0.5) + np.float32(0.5))
        out[..., 2] = _to_u8(nz / ln * np.float32(0.5) + np.float32(0.5))
        out[..., 3] = 255
        return out
    col = [np.float32(x) for x in color]
    if kind == "albedo":
        n = fbm(s0, c, c)
        m = value_noise((s0 + 77) & 0xFFFFFFFF, c, c, 16)
        hue = (m, np.float32(1.0) - m, np.float32(0.5))
        for ch in range(3):
            t = np.float32(0.55) + np.float32(0.45) * (np.float32(0.3) * hue[ch] + np.float32(0.7) * n)
            out[..., ch] = _to_u8(np.power(np.minimum(col[ch] * t, np.float32(1.0)), g))
        out[..., 3] = 255
        if alpha_mask:
            out[..., 3] = np.where(fbm(s0 ^ 0xA5A5A5A5, c, c) < np.float32(0.38), 0, 255).astype(np.uint8)
        return out
    for ch in range(3):
        out[..., ch] = _to_u8(np.power(np.minimum(col[ch], np.float32(1.0)), g))
    out[..., 3] = _to_u8(np.float32(rough_lo) + (np.float32(rough_hi) - np.float32(rough_lo)) * fbm(s0, c, c))
    return out
