"""Generates the known-answer vectors in this directory.

The reference ships no tests or golden data, so these vectors come from
independent numpy/pure-Python restatements of the reference's integer and
storage arithmetic (each function cites the shader line it follows). They pin
the C++ oracle and the CUDA kernels to the same bits.

    python tests/golden/make_golden.py      # rewrites kat_*.json
"""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
M32 = 0xFFFFFFFF


def bmfr_random(a: int) -> float:
    """shaders/bmfrGeneral.comp:103-113."""
    a &= M32
    a = ((a + 0x7ED55D16) + (a << 12)) & M32
    a = ((a ^ 0xC761C23C) ^ (a >> 19)) & M32
    a = ((a + 0x165667B1) + (a << 5)) & M32
    a = ((a + 0xD3A2646C) ^ (a << 9)) & M32
    a = ((a + 0xFD7046C5) + (a << 3)) & M32
    a = ((a ^ 0xB55A4F09) ^ (a >> 16)) & M32
    return float(np.float32(a) / np.float32(4294967295.0))


def wang_hash(seed: int) -> int:
    """shaders/random.glsl:73-80."""
    seed &= M32
    seed = (seed ^ 61) ^ (seed >> 16)
    seed = (seed * 9) & M32
    seed = seed ^ (seed >> 4)
    seed = (seed * 0x27D4EB2D) & M32
    seed = seed ^ (seed >> 15)
    return seed


def taus_step(z, s1, s2, s3, m):
    """shaders/random.glsl:16-20."""
    b = (((z << s1) & M32) ^ z) >> s2
    return (((z & m) << s3) & M32) ^ b


def rng_stream(x: int, y: int, frame: int, n: int) -> list[float]:
    """rEInit + n x randomNumber (shaders/random.glsl:38-47, 83-96)."""
    s = [wang_hash(x), wang_hash(y), wang_hash(frame), wang_hash(((x + y) & M32) * frame)]
    out = []
    for _ in range(n):
        s[0] = taus_step(s[0], 13, 19, 12, 4294967294)
        s[1] = taus_step(s[1], 2, 25, 4, 4294967288)
        s[2] = taus_step(s[2], 3, 11, 17, 4294967280)
        s[3] = (1664525 * s[3] + 1013904223) & M32
        u = s[0] ^ s[1] ^ s[2] ^ s[3]
        # 2.3283064365387e-10 * float(u): uint -> float, then an FP32 product
        out.append(float(np.float32(2.3283064365387e-10) * np.float32(u)))
    return out


def mirror(x: int, s: int) -> int:
    """shaders/bmfrGeneral.comp:93-97."""
    if x < 0:
        return abs(x) - 1
    if x >= s:
        return 2 * s - x - 1
    return x


def main():
    rng = np.random.default_rng(1234)
    ints = [0, 1, 2, 255, 65535, 0x7FFFFFFF, 0x80000000, M32] + [int(v) for v in rng.integers(0, 2**32, 64, dtype=np.uint64)]
    floats = [0.0, -0.0, 1.0, -1.0, 65504.0, 65519.0, 65520.0, 1e5, 6.1e-5, 6.0e-8, 3.0e-8, 2.9e-8, 1e-9, 1000.0,
              0.1, 1.0 / 3.0] + [float(v) for v in rng.normal(0, 10, 64).astype(np.float32)]
    half_bits = [int(np.float16(np.float32(f)).view(np.uint16)) for f in floats]
    kat = {
        "bmfr_random": {"in": ints, "out": [bmfr_random(a) for a in ints]},
        "f32_to_f16_bits": {"in": floats, "out": half_bits},
        "mirror": {"in": [[x, s] for s in (7, 32, 640) for x in (-40, -33, -1, 0, 5, 31, 32, 33, 639, 640, 700)],
                   "out": [mirror(x, s) for s in (7, 32, 640) for x in (-40, -33, -1, 0, 5, 31, 32, 33, 639, 640, 700)]},
        "wang_hash": {"in": ints, "out": [wang_hash(a) for a in ints]},
        "rng_stream": {"in": [[0, 0, 0], [1, 0, 0], [13, 7, 3], [639, 359, 1], [1919, 1079, 15]],
                       "out": [rng_stream(x, y, f, 12) for (x, y, f) in [[0, 0, 0], [1, 0, 0], [13, 7, 3], [639, 359, 1], [1919, 1079, 15]]]},
    }
    (HERE / "kat_integer.json").write_text(json.dumps(kat, indent=1))
    print("wrote", HERE / "kat_integer.json")


if __name__ == "__main__":
    main()
