"""Procedural scene textures (value noise), generated by the native library."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi

_abi.add_signatures({
    "pbrt_synth_texture": (C.c_int32, [C.c_uint64, C.c_uint32, C.c_int32, C.POINTER(C.c_float), C.c_int32, C.c_float,
                                       C.c_float, C.c_void_p]),
})

KINDS = {"albedo": 0, "specular": 1, "normal": 2}


def synth_texture(seed: int, size: int, kind: str, color=(1.0, 1.0, 1.0), alpha_mask: bool = False,
                  rough_lo: float = 0.2, rough_hi: float = 0.8) -> np.ndarray:
    out = np.empty((size, size, 4), np.uint8)
    col = (C.c_float * 3)(*[float(c) for c in color])
    _abi.check(_abi.lib().pbrt_synth_texture(C.c_uint64(seed & (2**64 - 1)), size, KINDS[kind], col, int(alpha_mask),
                                             rough_lo, rough_hi, out.ctypes.data_as(C.c_void_p)))
    return out
