"""ctypes binding of libvulkanpbrt_gb300.so (declarations in include/vulkanpbrt_gb300.h).

The library is the product: there is no Python or CPU fallback. Loading fails
loudly when the shared object has not been built.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libvulkanpbrt_gb300.so"

PBRT_OK = 0
STATUS_NAMES = {
    -1: "PBRT_ERROR_INVALID_ARGUMENT",
    -2: "PBRT_ERROR_CUDA",
    -3: "PBRT_ERROR_OUT_OF_MEMORY",
    -4: "PBRT_ERROR_UNSUPPORTED",
    -5: "PBRT_ERROR_ABORTED",
    -6: "PBRT_ERROR_TIMEOUT",
}

# PbrtFormat -> (numpy/cuda typestr, channels)
FORMATS = {
    1: ("<f4", 1),  # R32_SFLOAT
    2: ("<f4", 2),  # R32G32_SFLOAT
    3: ("<f4", 4),  # R32G32B32A32_SFLOAT
    4: ("<f2", 1),  # R16_SFLOAT
    5: ("<f2", 2),  # R16G16_SFLOAT
    6: ("<f2", 4),  # R16G16B16A16_SFLOAT
    7: ("|u1", 1),  # R8_UNORM
    8: ("|u1", 4),  # R8G8B8A8_UNORM
    9: ("|u1", 4),  # B8G8R8A8_UNORM
    10: ("<u4", 1),  # R32_UINT
}


class PbrtError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class PbrtImage(C.Structure):
    _fields_ = [
        ("data", C.c_void_p),
        ("width", C.c_uint32),
        ("height", C.c_uint32),
        ("layers", C.c_uint32),
        ("format", C.c_int32),
        ("texel_bytes", C.c_uint32),
        ("row_bytes", C.c_size_t),
        ("layer_bytes", C.c_size_t),
    ]


class PbrtPushConstants(C.Structure):
    _fields_ = [
        ("view_inverse", C.c_float * 16),
        ("proj_inverse", C.c_float * 16),
        ("prev_view", C.c_float * 16),
        ("frame_number", C.c_uint32),
        ("sample_number", C.c_uint32),
    ]


class PbrtCameraMatrices(C.Structure):
    _fields_ = [
        ("view", C.c_float * 16),
        ("inv_view", C.c_float * 16),
        ("proj", C.c_float * 16),
        ("inv_proj", C.c_float * 16),
        ("has_proj", C.c_int32),
    ]


class PbrtAccumulationImages(C.Structure):
    _fields_ = [(n, PbrtImage) for n in ("prev_illu", "prev_illu_squared", "prev_depth", "prev_normal", "spp", "prev_spp", "motion")]


class PbrtBmfrNoAllocImages(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("depth", "normal", "albedo", "noisy", "motion", "spp", "denoised",
                                          "final_bgra")]


_lib = None

H = C.c_void_p
P = C.POINTER
u32, i32 = C.c_uint32, C.c_int32

_SIGS = {
    "pbrt_version": (C.c_char_p, []),
    "pbrt_last_error": (i32, [C.c_char_p, C.c_size_t]),
    "pbrt_retain": (i32, [H]),
    "pbrt_release": (i32, [H]),
    "pbrt_gbuffer_create": (i32, [u32, u32, P(H)]),
    "pbrt_gbuffer_images": (i32, [H, P(PbrtImage), P(PbrtImage), P(PbrtImage), P(PbrtImage)]),
    "pbrt_illumination_buffer_create": (i32, [i32, u32, u32, P(H)]),
    "pbrt_illumination_buffer_images": (i32, [H, P(PbrtImage), u32, P(u32)]),
    "pbrt_accumulation_buffer_create": (i32, [u32, u32, P(H)]),
    "pbrt_accumulation_buffer_images": (i32, [H, P(PbrtAccumulationImages)]),
    "pbrt_accumulation_buffer_copy_to_back_images": (i32, [H, H, H, H]),
    "pbrt_accumulator_create": (i32, [H, H, i32, i32, i32, P(H)]),
    "pbrt_accumulator_set_camera_matrices": (i32, [H, i32, P(PbrtCameraMatrices), P(PbrtCameraMatrices)]),
    "pbrt_accumulator_dispatch": (i32, [H, H]),
    "pbrt_accumulator_get_accumulated_illumination": (i32, [H, P(H)]),
    "pbrt_accumulator_get_accumulation_buffer": (i32, [H, P(H)]),
    "pbrt_bmfr_create": (i32, [u32, u32, u32, u32, H, H, H, u32, P(H)]),
    "pbrt_bmfr_set_options": (i32, [H, i32, i32]),
    "pbrt_bmfr_dispatch": (i32, [H, P(PbrtPushConstants), H]),
    "pbrt_bmfr_final_image": (i32, [H, P(PbrtImage)]),
    "pbrt_bmfr_images": (i32, [H, P(PbrtImage), P(PbrtImage)]),
    "pbrt_bmfr_fp64_block_count": (i32, [H, H, P(u32)]),
    "pbrt_bmfr_set_condition_limit": (i32, [H, C.c_float]),
    "pbrt_bmfr_condition_stats": (i32, [H, H, P(u32), P(C.c_float)]),
    "pbrt_bmfr_dispatch_noalloc": (i32, [u32, u32, u32, i32, P(PbrtBmfrNoAllocImages), P(PbrtPushConstants), H]),
    "pbrt_bfr_create": (i32, [u32, u32, u32, u32, H, H, H, P(H)]),
    "pbrt_bfr_dispatch": (i32, [H, P(PbrtPushConstants), H]),
    "pbrt_bfr_final_image": (i32, [H, P(PbrtImage)]),
    "pbrt_bfr_images": (i32, [H, P(PbrtImage)]),
    "pbrt_taa_create": (i32, [u32, u32, u32, u32, H, H, P(PbrtImage), P(H)]),
    "pbrt_taa_dispatch": (i32, [H, P(PbrtPushConstants), H]),
    "pbrt_taa_final_image": (i32, [H, P(PbrtImage)]),
    "pbrt_mesh_generate_normals": (i32, [H, u32, H, u32, u32, H]),
    "pbrt_mesh_fill_uvs": (i32, [u32, H, u32, u32, H]),
    "pbrt_image_upload": (i32, [P(PbrtImage), H, C.c_size_t, H]),
    "pbrt_image_download": (i32, [P(PbrtImage), H, C.c_size_t, H]),
    "pbrt_stream_synchronize": (i32, [H]),
    "pbrt_bfr_blender_create": (i32, [u32, u32, P(PbrtImage), P(PbrtImage), P(PbrtImage), P(PbrtImage), P(PbrtImage),
                                      u32, u32, u32, P(H)]),
    "pbrt_bfr_blender_dispatch": (i32, [H, H]),
    "pbrt_bfr_blender_final_image": (i32, [H, P(PbrtImage)]),
    "pbrt_format_convert": (i32, [P(PbrtImage), P(PbrtImage), H]),
}


def declared_symbols() -> list[str]:
    return list(_SIGS)


def lib() -> C.CDLL:
    """Load the native library (built by vulkanpbrt_gb300.build)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(
                f"{LIB_PATH.name} is not built: run `python -c 'import __graft_entry__ as g; g.build()'` "
                "(the CUDA path has no fallback)"
            )
        l = C.CDLL(str(LIB_PATH), mode=os.RTLD_NOW | os.RTLD_LOCAL)
        for name, (res, args) in _SIGS.items():
            fn = getattr(l, name)
            fn.restype = res
            fn.argtypes = args
        _lib = l
    return _lib


def add_signatures(sigs: dict) -> None:
    """Register further entry points (used by modules that extend the ABI)."""
    _SIGS.update(sigs)
    if _lib is not None:
        for name, (res, args) in sigs.items():
            fn = getattr(_lib, name)
            fn.restype = res
            fn.argtypes = args


def last_error() -> str:
    buf = C.create_string_buffer(1024)
    lib().pbrt_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(status: int) -> None:
    if status != PBRT_OK:
        raise PbrtError(status, last_error())


def stream_handle(stream) -> C.c_void_p:
    """cudaStream_t of a torch.cuda.Stream (or None for the legacy default stream)."""
    if stream is None:
        return C.c_void_p(0)
    if isinstance(stream, int):
        return C.c_void_p(stream)
    return C.c_void_p(stream.cuda_stream)
