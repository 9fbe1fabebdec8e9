"""Batched render requests over the pbrt_batch_* C ABI: many independent
renders (each its own PBRTPipeline -- scene, resolution, depth -- sample
count, and optional Accumulator and BMFR) in one CUDA graph launch, with an
autotuner for the number of concurrent chains and the tracer's launch shape.
No reference counterpart (the reference renders one view per frame)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from ._abi import PbrtCameraMatrices, PbrtPushConstants, check, lib, stream_handle
from .render_modules import Handle

H = C.c_void_p


class PbrtBatchRequest(C.Structure):
    _fields_ = [("pipeline", H), ("accumulator", H), ("bmfr", H), ("pc", PbrtPushConstants),
                ("camera", PbrtCameraMatrices), ("spp", C.c_uint32)]


class PbrtBatchTuning(C.Structure):
    _fields_ = [("branches", C.c_uint32), ("trace_blocks_per_sm", C.c_uint32), ("shade_blocks_per_sm", C.c_uint32),
                ("order", C.c_uint32)]

    def as_dict(self):
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


P = C.POINTER
_abi.add_signatures({
    "pbrt_pipeline_set_launch": (C.c_int32, [H, C.c_int32, C.c_int32]),
    "pbrt_batch_create": (C.c_int32, [P(H)]),
    "pbrt_batch_add": (C.c_int32, [H, P(PbrtBatchRequest)]),
    "pbrt_batch_size": (C.c_int32, [H, P(C.c_uint32)]),
    "pbrt_batch_set_tuning": (C.c_int32, [H, P(PbrtBatchTuning)]),
    "pbrt_batch_get_tuning": (C.c_int32, [H, P(PbrtBatchTuning)]),
    "pbrt_batch_submit": (C.c_int32, [H, H]),
    "pbrt_batch_autotune": (C.c_int32, [H, H, C.c_int32, P(PbrtBatchTuning), P(C.c_float)]),
    "pbrt_batch_plan": (C.c_int32, [P(C.c_double), C.c_uint32, C.c_uint32, C.c_uint32, P(C.c_uint32)]),
})


def plan(costs, branches: int, order: int = 1) -> np.ndarray:
    """The chain each request goes to (longest first onto the least loaded chain when order=1)."""
    c = np.ascontiguousarray(np.asarray(costs, dtype=np.float64))
    out = np.zeros(len(c), np.uint32)
    check(lib().pbrt_batch_plan(c.ctypes.data_as(P(C.c_double)), len(c), branches, order,
                                out.ctypes.data_as(P(C.c_uint32))))
    return out


class Batch(Handle):
    def __init__(self):
        h = C.c_void_p()
        check(lib().pbrt_batch_create(C.byref(h)))
        super().__init__(h)
        self._keep = []

    def add(self, pipeline, push_constants, spp: int = 1, accumulator=None, bmfr=None, camera=None) -> None:
        r = PbrtBatchRequest()
        r.pipeline = pipeline.ptr
        r.accumulator = accumulator.ptr if accumulator is not None else None
        r.bmfr = bmfr.ptr if bmfr is not None else None
        r.pc = push_constants.value
        if camera is not None:
            r.camera = camera.to_c()
        r.spp = spp
        check(lib().pbrt_batch_add(self.ptr, C.byref(r)))
        self._keep.append((pipeline, accumulator, bmfr))

    def __len__(self) -> int:
        n = C.c_uint32()
        check(lib().pbrt_batch_size(self.ptr, C.byref(n)))
        return n.value

    @property
    def tuning(self) -> dict:
        t = PbrtBatchTuning()
        check(lib().pbrt_batch_get_tuning(self.ptr, C.byref(t)))
        return t.as_dict()

    def set_tuning(self, branches=4, trace_blocks_per_sm=8, shade_blocks_per_sm=8, order=1) -> None:
        t = PbrtBatchTuning(branches, trace_blocks_per_sm, shade_blocks_per_sm, order)
        check(lib().pbrt_batch_set_tuning(self.ptr, C.byref(t)))

    def submit(self, stream=None) -> None:
        check(lib().pbrt_batch_submit(self.ptr, stream_handle(stream)))

    def autotune(self, repeats: int = 3, stream=None):
        t = PbrtBatchTuning()
        ms = C.c_float()
        check(lib().pbrt_batch_autotune(self.ptr, stream_handle(stream), repeats, C.byref(t), C.byref(ms)))
        return t.as_dict(), ms.value
