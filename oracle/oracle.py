"""Oracle (test infrastructure only): ctypes front end of liboracle.so.

The CPU restatement of the reference shader math lives in the C++ files of
this directory; this module builds it (make) and exposes numpy wrappers.
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs use it,
as the checker -- never as the thing measured for the GPU path or shipped.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
_lib = None


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(str(LIB))
        _lib.oracle_bmfr_random.restype = C.c_float
        _lib.oracle_bmfr_random.argtypes = [C.c_uint32]
        _lib.oracle_f2h.restype = C.c_uint16
        _lib.oracle_f2h.argtypes = [C.c_float]
        _lib.oracle_h2f.restype = C.c_float
        _lib.oracle_h2f.argtypes = [C.c_uint16]
        _lib.oracle_mirror.restype = C.c_int
        _lib.oracle_mirror.argtypes = [C.c_int, C.c_int]
    return _lib


def _p(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"], "oracle arrays must be C-contiguous"
    return a.ctypes.data_as(C.c_void_p)


def _f32(m) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(m, dtype=np.float32).reshape(-1))


def threads_default() -> int:
    return int(os.environ.get("ORACLE_THREADS", "0"))


def accumulate(frame, separate, view, inverse_view, prev_view, prev_origin, src_rgba32f, depth, prev_depth, prev_spp,
               prev_output_f16, threads=None):
    """accumulator.comp; matrices column-major [16]. Returns (motion f16 [H,W,2], spp u8 [H,W], illum f16 [H,W,4])."""
    H, W = depth.shape
    motion = np.zeros((H, W, 2), np.float16)
    spp = np.zeros((H, W), np.uint8)
    illum = np.zeros((H, W, 4), np.float16)
    args = [np.ascontiguousarray(a) for a in (src_rgba32f.astype(np.float32), depth.astype(np.float32),
                                              prev_depth.astype(np.float32), prev_spp.astype(np.uint8),
                                              prev_output_f16.astype(np.float16))]
    mats = [_f32(m) for m in (view, inverse_view, prev_view, prev_origin)]
    rc = lib().oracle_accumulate(W, H, C.c_uint32(frame), int(separate), *[_p(m) for m in mats], *[_p(a) for a in args],
                                 _p(motion), _p(spp), _p(illum), threads_default() if threads is None else threads)
    assert rc == 0
    return motion, spp, illum


def bmfr_pre(bw, frame, position_type, inv_view, inv_proj, depth, normal, noisy_f16, threads=None):
    H, W = depth.shape
    gw, gh = W // bw + 2, H // bw + 2
    feats = np.zeros((13, gh * bw, gw * bw), np.float16)
    rc = lib().oracle_bmfr_pre(W, H, bw, C.c_uint32(frame), position_type, _p(_f32(inv_view)), _p(_f32(inv_proj)),
                               _p(np.ascontiguousarray(depth, np.float32)), _p(np.ascontiguousarray(normal, np.float32)),
                               _p(np.ascontiguousarray(noisy_f16, np.float16)), _p(feats),
                               threads_default() if threads is None else threads)
    assert rc == 0
    return feats


def bmfr_fit(W, H, bw, fit_threads, frame, feats, threads=None):
    gw, gh = W // bw + 2, H // bw + 2
    weights = np.zeros((30, gh, gw), np.float32)
    rc = lib().oracle_bmfr_fit(W, H, bw, fit_threads, C.c_uint32(frame), _p(np.ascontiguousarray(feats)), _p(weights),
                               threads_default() if threads is None else threads)
    assert rc == 0
    return weights


def bmfr_post(bw, frame, position_type, inv_view, inv_proj, depth, normal, albedo, motion_f16, spp, weights, denoised,
              threads=None):
    """Updates `denoised` (f16 [2,H,W,4]) in place; returns final BGRA8 [H,W,4]."""
    H, W = depth.shape
    final = np.zeros((H, W, 4), np.uint8)
    assert denoised.dtype == np.float16 and denoised.flags["C_CONTIGUOUS"]
    rc = lib().oracle_bmfr_post(W, H, bw, C.c_uint32(frame), position_type, _p(_f32(inv_view)), _p(_f32(inv_proj)),
                                _p(np.ascontiguousarray(depth, np.float32)), _p(np.ascontiguousarray(normal, np.float32)),
                                _p(np.ascontiguousarray(albedo, np.uint8)), _p(np.ascontiguousarray(motion_f16, np.float16)),
                                _p(np.ascontiguousarray(spp, np.uint8)), _p(np.ascontiguousarray(weights, np.float32)),
                                _p(denoised), _p(final), threads_default() if threads is None else threads)
    assert rc == 0
    return final


def bmfr(bw, fit_threads, frame, position_type, inv_view, inv_proj, depth, normal, albedo, noisy_f16, motion_f16, spp,
         denoised, threads=None):
    """bmfrPre -> bmfrFit -> bmfrPost. Returns (features, weights, final); `denoised` updated in place."""
    H, W = depth.shape
    feats = bmfr_pre(bw, frame, position_type, inv_view, inv_proj, depth, normal, noisy_f16, threads)
    weights = bmfr_fit(W, H, bw, fit_threads, frame, feats, threads)
    final = bmfr_post(bw, frame, position_type, inv_view, inv_proj, depth, normal, albedo, motion_f16, spp, weights,
                      denoised, threads)
    return feats, weights, final


def bfr(bw, bh, frame, depth, normal, albedo, motion_f16, spp, noisy_f16, denoised, threads=None):
    H, W = depth.shape
    final = np.zeros((H, W, 4), np.uint8)
    rc = lib().oracle_bfr(W, H, bw, bh, C.c_uint32(frame), _p(np.ascontiguousarray(depth, np.float32)),
                          _p(np.ascontiguousarray(normal, np.float32)), _p(np.ascontiguousarray(albedo, np.uint8)),
                          _p(np.ascontiguousarray(motion_f16, np.float16)), _p(np.ascontiguousarray(spp, np.uint8)),
                          _p(np.ascontiguousarray(noisy_f16, np.float16)), _p(denoised), _p(final),
                          threads_default() if threads is None else threads)
    assert rc == 0
    return final
