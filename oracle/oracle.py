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


def taa(frame, motion_f16, denoised_bgra, history, threads=None):
    """taa.comp with the reference's byte-copied history. Returns (final BGRA8 [H,W,4], next history [H,W,4])."""
    H, W = denoised_bgra.shape[:2]
    final = np.zeros((H, W, 4), np.uint8)
    nxt = np.zeros((H, W, 4), np.uint8)
    rc = lib().oracle_taa(W, H, C.c_uint32(frame), _p(np.ascontiguousarray(motion_f16, np.float16)),
                          _p(np.ascontiguousarray(denoised_bgra, np.uint8)), _p(np.ascontiguousarray(history, np.uint8)),
                          _p(final), _p(nxt), threads_default() if threads is None else threads)
    assert rc == 0
    return final, nxt


def bfr_blend(avg, avg_sq, den8, den16, den32, radius=2, threads=None):
    """bfrBlender.comp. avg / avg_sq: [H,W,4] float16 or float32; den*: [H,W,4] u8. Returns [H,W,4] u8."""
    H, W = den8.shape[:2]
    f32 = avg.dtype == np.float32
    dt = np.float32 if f32 else np.float16
    out = np.zeros((H, W, 4), np.uint8)
    rc = lib().oracle_bfr_blend(W, H, radius, int(f32), _p(np.ascontiguousarray(avg, dt)),
                                _p(np.ascontiguousarray(avg_sq, dt)), _p(np.ascontiguousarray(den8, np.uint8)),
                                _p(np.ascontiguousarray(den16, np.uint8)), _p(np.ascontiguousarray(den32, np.uint8)),
                                _p(out), threads_default() if threads is None else threads)
    assert rc == 0
    return out


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


# ---------------------------------------------------------------------------
# Path tracer


class OrcScene(C.Structure):
    _fields_ = [("mesh_count", C.c_uint32), ("mesh_vbase", C.c_void_p), ("mesh_ibase", C.c_void_p),
                ("mesh_tex", C.c_void_p), ("pos", C.c_void_p), ("nor", C.c_void_p), ("uv", C.c_void_p),
                ("idx", C.c_void_p), ("instance_count", C.c_uint32), ("inst_mat", C.c_void_p),
                ("inst_mesh", C.c_void_p), ("inst_stride", C.c_void_p), ("inst_opaque", C.c_void_p),
                ("inst_tri_count", C.c_void_p), ("materials", C.c_void_p), ("light_count", C.c_uint32),
                ("lights", C.c_void_p), ("texture_count", C.c_uint32), ("tex_offset", C.c_void_p),
                ("tex_w", C.c_void_p), ("tex_h", C.c_void_p), ("texels", C.c_void_p)]


class OracleScene:
    """A vulkanpbrt_gb300.scene.Scene packed into the oracle's plain arrays."""

    def __init__(self, scene):
        vb, ib, pos, nor, uv, idx = [], [], [], [], [], []
        nv = 0
        nw = 0
        for m in scene.meshes:
            vb.append(nv)
            ib.append(nw)
            pos.append(m.positions.reshape(-1))
            nor.append(m.normals.reshape(-1))
            uv.append(m.uvs.reshape(-1))
            if m.index_stride == 4:
                words = m.indices.astype(np.uint32)
            else:
                i16 = m.indices.astype(np.uint32)
                if len(i16) % 2:
                    i16 = np.append(i16, 0)
                words = (i16[0::2] | (i16[1::2] << 16)).astype(np.uint32)
                words = np.append(words, np.uint32(0))
            idx.append(words)
            nv += len(m.positions)
            nw += len(words)
        self.a = dict(
            mesh_vbase=np.array(vb, np.uint32), mesh_ibase=np.array(ib, np.uint32),
            mesh_tex=np.array(scene.mesh_textures, np.int32).reshape(-1),
            pos=np.concatenate(pos).astype(np.float32), nor=np.concatenate(nor).astype(np.float32),
            uv=np.concatenate(uv).astype(np.float32), idx=np.concatenate(idx).astype(np.uint32),
            inst_mat=np.concatenate([np.asarray(m, np.float32).T.reshape(16) for m in scene.instance_mats]),
            inst_mesh=np.array(scene.instance_mesh, np.int32),
            inst_stride=np.array([scene.meshes[m].index_stride for m in scene.instance_mesh], np.uint32),
            inst_opaque=scene.instance_opaque().astype(np.uint8),
            inst_tri_count=np.array([scene.meshes[m].tri_count for m in scene.instance_mesh], np.uint32),
            materials=np.stack(scene.materials).astype(np.float32).reshape(-1),
            lights=(np.stack(scene.lights) if scene.lights else np.zeros((1, 32), np.float32)).astype(np.float32).reshape(-1),
            tex_w=np.array([t.shape[1] for t in scene.textures], np.uint32),
            tex_h=np.array([t.shape[0] for t in scene.textures], np.uint32),
        )
        offs, acc = [], 0
        for t in scene.textures:
            offs.append(acc)
            acc += t.shape[0] * t.shape[1]
        self.a["tex_offset"] = np.array(offs, np.uint64)
        self.a["texels"] = np.concatenate([np.ascontiguousarray(t, np.uint8).reshape(-1) for t in scene.textures])
        for k, v in self.a.items():
            self.a[k] = np.ascontiguousarray(v)
        s = OrcScene()
        s.mesh_count = len(scene.meshes)
        s.instance_count = len(scene.instance_mesh)
        s.light_count = len(scene.lights)
        s.texture_count = len(scene.textures)
        for k, v in self.a.items():
            setattr(s, k, v.ctypes.data)
        self.c = s


def render(oscene: OracleScene, W, H, inv_view, inv_proj, frame=0, sample=0, min_depth=0, max_depth=2, light_mode=0,
           final_image=False, precision=32, frames=1, threads=None):
    """Returns dict(illum [H,W,4] f32, depth, normal [H,W,2], material, albedo [H,W,4] u8, hit_key [H,W] u32, rays)."""
    out = dict(illum=np.zeros((H, W, 4), np.float32), depth=np.zeros((H, W), np.float32),
               normal=np.zeros((H, W, 2), np.float32), material=np.zeros((H, W, 4), np.uint8),
               albedo=np.zeros((H, W, 4), np.uint8), hit_key=np.zeros((H, W), np.uint32))
    rays = np.zeros(3, np.uint64)
    rc = lib().oracle_render(C.byref(oscene.c), W, H, _p(_f32(inv_view)), _p(_f32(inv_proj)), C.c_uint32(frame),
                             C.c_uint32(sample), min_depth, max_depth, light_mode, int(final_image), precision, frames,
                             _p(out["illum"]), _p(out["depth"]), _p(out["normal"]), _p(out["material"]),
                             _p(out["albedo"]), _p(out["hit_key"]), _p(rays),
                             threads_default() if threads is None else threads)
    assert rc == 0
    out["rays"] = rays
    return out


def trace_rays(oscene: OracleScene, org_tmin: np.ndarray, dir_tmax: np.ndarray, any_hit=False, precision=64,
               threads=None) -> np.ndarray:
    n = len(org_tmin)
    hits = np.zeros((n, 4), np.float32)
    rc = lib().oracle_trace_rays(C.byref(oscene.c), _p(np.ascontiguousarray(org_tmin, np.float32)),
                                 _p(np.ascontiguousarray(dir_tmax, np.float32)), C.c_uint32(n), int(any_hit),
                                 _p(hits), precision, threads_default() if threads is None else threads)
    assert rc == 0
    return hits


def rng_stream(x, y, frame, n) -> np.ndarray:
    out = np.zeros(n, np.float32)
    lib().oracle_rng_stream(C.c_uint32(x), C.c_uint32(y), C.c_uint32(frame), n, _p(out))
    return out
