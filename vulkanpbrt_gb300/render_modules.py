"""Host-side mirror of VulkanPBRT's render modules over the C ABI.

Class and attribute names follow the reference (source/buffers/*.hpp,
source/renderModules/*.hpp): images are public attributes (here `Image`
views of device buffers the library owns, exportable to torch without a
copy), and `add_*_to_command_graph` records work into a `Commands` list that
`submit(stream)` replays each frame -- the reference records its command
graph once and resubmits it with updated push-constant values
(source/VulkanPBRT.cpp:397-505, 551-618).
"""
from __future__ import annotations

import ctypes as C
from typing import Callable, Optional

import numpy as np

from . import _abi
from ._abi import PbrtImage, check, lib, stream_handle


class Image:
    """A device image (PbrtImage view) owned by a library object."""

    def __init__(self, view: PbrtImage, owner: "Handle"):
        self.view = view
        self._owner = owner  # keeps the owning handle alive

    @property
    def width(self) -> int:
        return self.view.width

    @property
    def height(self) -> int:
        return self.view.height

    @property
    def layers(self) -> int:
        return self.view.layers

    @property
    def format(self) -> int:
        return self.view.format

    @property
    def shape(self) -> tuple:
        typestr, ch = _abi.FORMATS[self.view.format]
        if self.view.layers > 1:
            return (self.view.layers, self.view.height, self.view.width, ch)
        return (self.view.height, self.view.width, ch)

    @property
    def __cuda_array_interface__(self):
        typestr, _ = _abi.FORMATS[self.view.format]
        return {"version": 3, "shape": self.shape, "typestr": typestr, "data": (int(self.view.data), False), "strides": None}

    def tensor(self):
        """Zero-copy torch view of the device image (shape [layers,] H, W, C)."""
        import torch

        return torch.as_tensor(self, device="cuda")

    def nbytes(self) -> int:
        return self.view.layer_bytes * self.view.layers


class Handle:
    """Owns one reference to a library handle."""

    def __init__(self, ptr: C.c_void_p):
        self._ptr = ptr

    @property
    def ptr(self) -> C.c_void_p:
        return self._ptr

    def __del__(self):
        p = getattr(self, "_ptr", None)
        if p is not None and p.value:
            try:
                lib().pbrt_release(p)
            except Exception:
                pass
            self._ptr = C.c_void_p(0)

    @staticmethod
    def _borrowed(ptr: C.c_void_p) -> C.c_void_p:
        check(lib().pbrt_retain(ptr))
        return ptr


class Commands:
    """A recorded list of GPU work (the reference's vsg::Commands)."""

    def __init__(self):
        self._calls: list[Callable] = []

    def add(self, call: Callable) -> None:
        self._calls.append(call)

    def submit(self, stream=None) -> None:
        for call in self._calls:
            call(stream)


class PushConstants:
    """Mutable RayTracingPushConstants value (source/renderModules/PipelineStructs.hpp:6-13)."""

    def __init__(self, view_inverse=None, proj_inverse=None, prev_view=None, frame_number=0, sample_number=0):
        self.value = _abi.PbrtPushConstants()
        eye = np.eye(4, dtype=np.float32)
        self.set(view_inverse if view_inverse is not None else eye, proj_inverse if proj_inverse is not None else eye,
                 prev_view if prev_view is not None else eye, frame_number, sample_number)

    @staticmethod
    def _m(mat) -> np.ndarray:
        # Matrices are given as numpy [4,4] with m[row, col]; stored column-major.
        return np.asarray(mat, dtype=np.float32).T.reshape(16)

    def set(self, view_inverse=None, proj_inverse=None, prev_view=None, frame_number=None, sample_number=None):
        v = self.value
        if view_inverse is not None:
            v.view_inverse[:] = self._m(view_inverse).tolist()
        if proj_inverse is not None:
            v.proj_inverse[:] = self._m(proj_inverse).tolist()
        if prev_view is not None:
            v.prev_view[:] = self._m(prev_view).tolist()
        if frame_number is not None:
            v.frame_number = int(frame_number)
        if sample_number is not None:
            v.sample_number = int(sample_number)


class CameraMatrices:
    """CameraMatrices (source/io/RenderIO.hpp): view, inv_view, optional proj / inv_proj."""

    def __init__(self, view=None, inv_view=None, proj=None, inv_proj=None):
        self.view, self.inv_view, self.proj, self.inv_proj = view, inv_view, proj, inv_proj

    def to_c(self) -> _abi.PbrtCameraMatrices:
        c = _abi.PbrtCameraMatrices()
        eye = np.eye(4, dtype=np.float32)
        for name in ("view", "inv_view", "proj", "inv_proj"):
            m = getattr(self, name)
            getattr(c, name)[:] = PushConstants._m(m if m is not None else eye).tolist()
        c.has_proj = int(self.proj is not None and self.inv_proj is not None)
        return c


class GBuffer(Handle):
    """GBuffer (source/buffers/GBuffer.hpp): depth R32F, normal RG32F, material RGBA8, albedo RGBA8."""

    def __init__(self, width: int, height: int):
        h = C.c_void_p()
        check(lib().pbrt_gbuffer_create(width, height, C.byref(h)))
        super().__init__(h)
        self.width, self.height = width, height
        views = [PbrtImage() for _ in range(4)]
        check(lib().pbrt_gbuffer_images(h, *[C.byref(v) for v in views]))
        self.depth, self.normal, self.material, self.albedo = (Image(v, self) for v in views)


ILLUMINATION_TYPES = {
    "Final": 0,
    "FinalDemodulated": 1,
    "Demodulated": 2,
    "DemodulatedFloat": 3,
    "FinalFloat": 4,
}


class IlluminationBuffer(Handle):
    """IlluminationBuffer family (source/buffers/IlluminationBuffer.hpp)."""

    type_name = "DemodulatedFloat"

    def __init__(self, width: int, height: int, _ptr: Optional[C.c_void_p] = None):
        if _ptr is None:
            h = C.c_void_p()
            check(lib().pbrt_illumination_buffer_create(ILLUMINATION_TYPES[self.type_name], width, height, C.byref(h)))
        else:
            h = _ptr
        super().__init__(h)
        self.width, self.height = width, height
        views = (PbrtImage * 4)()
        n = C.c_uint32()
        check(lib().pbrt_illumination_buffer_images(h, views, 4, C.byref(n)))
        self.illumination_images = [Image(views[i], self) for i in range(n.value)]


class IlluminationBufferFinal(IlluminationBuffer):
    type_name = "Final"


class IlluminationBufferFinalDemodulated(IlluminationBuffer):
    type_name = "FinalDemodulated"


class IlluminationBufferDemodulated(IlluminationBuffer):
    type_name = "Demodulated"


class IlluminationBufferDemodulatedFloat(IlluminationBuffer):
    type_name = "DemodulatedFloat"


class IlluminationBufferFinalFloat(IlluminationBuffer):
    type_name = "FinalFloat"


class AccumulationBuffer(Handle):
    """AccumulationBuffer (source/buffers/AccumulationBuffer.hpp)."""

    def __init__(self, width: int, height: int, _ptr: Optional[C.c_void_p] = None):
        if _ptr is None:
            h = C.c_void_p()
            check(lib().pbrt_accumulation_buffer_create(width, height, C.byref(h)))
        else:
            h = _ptr
        super().__init__(h)
        self.width, self.height = width, height
        imgs = _abi.PbrtAccumulationImages()
        check(lib().pbrt_accumulation_buffer_images(h, C.byref(imgs)))
        for name in ("prev_illu", "prev_illu_squared", "prev_depth", "prev_normal", "spp", "prev_spp", "motion"):
            setattr(self, name, Image(getattr(imgs, name), self))

    def copy_to_back_images(self, commands: Commands, g_buffer: GBuffer, illumination_buffer: IlluminationBuffer):
        commands.add(lambda s: check(lib().pbrt_accumulation_buffer_copy_to_back_images(
            self.ptr, g_buffer.ptr, illumination_buffer.ptr, stream_handle(s))))


class Accumulator(Handle):
    """Accumulator (source/renderModules/Accumulator.hpp)."""

    def __init__(self, g_buffer: GBuffer, illumination_buffer: IlluminationBuffer, separate_matrices: bool = True,
                 work_width: int = 16, work_height: int = 16):
        h = C.c_void_p()
        check(lib().pbrt_accumulator_create(g_buffer.ptr, illumination_buffer.ptr, int(separate_matrices), work_width,
                                            work_height, C.byref(h)))
        super().__init__(h)
        self._inputs = (g_buffer, illumination_buffer)
        ib, ab = C.c_void_p(), C.c_void_p()
        check(lib().pbrt_accumulator_get_accumulated_illumination(h, C.byref(ib)))
        check(lib().pbrt_accumulator_get_accumulation_buffer(h, C.byref(ab)))
        self.accumulated_illumination = IlluminationBufferDemodulated(g_buffer.width, g_buffer.height,
                                                                     _ptr=Handle._borrowed(ib))
        self.accumulation_buffer = AccumulationBuffer(g_buffer.width, g_buffer.height, _ptr=Handle._borrowed(ab))

    def set_camera_matrices(self, frame_index: int, cur: CameraMatrices, prev: CameraMatrices) -> None:
        a, b = cur.to_c(), prev.to_c()
        check(lib().pbrt_accumulator_set_camera_matrices(self.ptr, frame_index, C.byref(a), C.byref(b)))

    def add_dispatch_to_command_graph(self, commands: Commands) -> None:
        commands.add(lambda s: check(lib().pbrt_accumulator_dispatch(self.ptr, stream_handle(s))))


class BMFR(Handle):
    """BMFR (source/renderModules/denoisers/BMFR.hpp)."""

    def __init__(self, width: int, height: int, work_width: int, work_height: int, g_buffer: GBuffer,
                 illu_buffer: IlluminationBuffer, acc_buffer: AccumulationBuffer, fitting_kernel: int = 256,
                 position_type: int = 0, fp64_resolve: bool = False):
        h = C.c_void_p()
        check(lib().pbrt_bmfr_create(width, height, work_width, work_height, g_buffer.ptr, illu_buffer.ptr,
                                     acc_buffer.ptr, fitting_kernel, C.byref(h)))
        super().__init__(h)
        self._inputs = (g_buffer, illu_buffer, acc_buffer)
        check(lib().pbrt_bmfr_set_options(h, position_type, int(fp64_resolve)))
        d, w, f = PbrtImage(), PbrtImage(), PbrtImage()
        check(lib().pbrt_bmfr_images(h, C.byref(d), C.byref(w)))
        check(lib().pbrt_bmfr_final_image(h, C.byref(f)))
        self.denoised, self.weights, self._final = Image(d, self), Image(w, self), Image(f, self)

    def compile(self, context=None) -> None:
        """Images are allocated at construction (vsg compiles them lazily)."""

    def update_image_layouts(self, context=None) -> None:
        """No layouts on CUDA: kept for interface parity."""

    def dispatch(self, push_constants: PushConstants, stream=None) -> None:
        check(lib().pbrt_bmfr_dispatch(self.ptr, C.byref(push_constants.value), stream_handle(stream)))

    def add_dispatch_to_command_graph(self, commands: Commands, push_constants: PushConstants) -> None:
        commands.add(lambda s: self.dispatch(push_constants, s))

    def get_final_descriptor_image(self) -> Image:
        return self._final

    def fp64_block_count(self, stream=None) -> int:
        n = C.c_uint32()
        check(lib().pbrt_bmfr_fp64_block_count(self.ptr, stream_handle(stream), C.byref(n)))
        return n.value

    def set_condition_limit(self, limit: float) -> None:
        """R-diagonal ratio above which a block is re-solved in FP64 (default 1e6)."""
        check(lib().pbrt_bmfr_set_condition_limit(self.ptr, float(limit)))

    def condition_stats(self, stream=None):
        """(blocks re-solved in FP64, largest R-diagonal ratio) of the last dispatch (needs fp64_resolve)."""
        n, r = C.c_uint32(), C.c_float()
        check(lib().pbrt_bmfr_condition_stats(self.ptr, stream_handle(stream), C.byref(n), C.byref(r)))
        return n.value, r.value


class BFR(Handle):
    """BFR (source/renderModules/denoisers/BFR.hpp)."""

    def __init__(self, width: int, height: int, work_width: int, work_height: int, g_buffer: GBuffer,
                 illu_buffer: IlluminationBuffer, acc_buffer: AccumulationBuffer):
        h = C.c_void_p()
        check(lib().pbrt_bfr_create(width, height, work_width, work_height, g_buffer.ptr, illu_buffer.ptr,
                                    acc_buffer.ptr, C.byref(h)))
        super().__init__(h)
        self._inputs = (g_buffer, illu_buffer, acc_buffer)
        d, f = PbrtImage(), PbrtImage()
        check(lib().pbrt_bfr_images(h, C.byref(d)))
        check(lib().pbrt_bfr_final_image(h, C.byref(f)))
        self.denoised, self._final = Image(d, self), Image(f, self)

    def compile(self, context=None) -> None:
        pass

    def update_image_layouts(self, context=None) -> None:
        pass

    def dispatch(self, push_constants: PushConstants, stream=None) -> None:
        check(lib().pbrt_bfr_dispatch(self.ptr, C.byref(push_constants.value), stream_handle(stream)))

    def add_dispatch_to_command_graph(self, commands: Commands, push_constants: PushConstants) -> None:
        commands.add(lambda s: self.dispatch(push_constants, s))

    def get_final_descriptor_image(self) -> Image:
        return self._final


class BFRBlender(Handle):
    """BFRBlender (source/renderModules/denoisers/BFRBlender.hpp): blends
    the final images of the 8x8, 16x16 and 32x32 denoisers by the local
    standard deviation of the average image."""

    def __init__(self, width: int, height: int, average_image: Image, average_squared_image: Image, denoised0: Image,
                 denoised1: Image, denoised2: Image, work_width: int = 16, work_height: int = 16,
                 filter_radius: int = 2):
        h = C.c_void_p()
        check(lib().pbrt_bfr_blender_create(width, height, C.byref(average_image.view),
                                            C.byref(average_squared_image.view), C.byref(denoised0.view),
                                            C.byref(denoised1.view), C.byref(denoised2.view), work_width, work_height,
                                            filter_radius, C.byref(h)))
        super().__init__(h)
        # the images' owners must outlive this object
        self._inputs = (average_image, average_squared_image, denoised0, denoised1, denoised2)
        f = PbrtImage()
        check(lib().pbrt_bfr_blender_final_image(h, C.byref(f)))
        self._final = Image(f, self)

    def compile(self, context=None) -> None:
        pass

    def update_image_layouts(self, context=None) -> None:
        pass

    def dispatch(self, stream=None) -> None:
        check(lib().pbrt_bfr_blender_dispatch(self.ptr, stream_handle(stream)))

    def add_dispatch_to_command_graph(self, commands: Commands) -> None:
        commands.add(lambda s: self.dispatch(s))

    def get_final_descriptor_image(self) -> Image:
        return self._final


class Taa(Handle):
    """Taa (source/renderModules/Taa.hpp): temporal anti-aliasing of a
    denoiser's final image with the accumulation buffer's motion vectors."""

    def __init__(self, width: int, height: int, work_width: int, work_height: int, g_buffer: GBuffer,
                 acc_buffer: AccumulationBuffer, denoised: Image):
        h = C.c_void_p()
        check(lib().pbrt_taa_create(width, height, work_width, work_height, g_buffer.ptr, acc_buffer.ptr,
                                    C.byref(denoised.view), C.byref(h)))
        super().__init__(h)
        self._inputs = (g_buffer, acc_buffer, denoised)  # the denoised image's owner must outlive this object
        f = PbrtImage()
        check(lib().pbrt_taa_final_image(h, C.byref(f)))
        self._final = Image(f, self)

    def compile(self, context=None) -> None:
        pass

    def update_image_layouts(self, context=None) -> None:
        pass

    def dispatch(self, push_constants: PushConstants, stream=None) -> None:
        check(lib().pbrt_taa_dispatch(self.ptr, C.byref(push_constants.value), stream_handle(stream)))

    def add_dispatch_to_command_graph(self, commands: Commands, push_constants: PushConstants) -> None:
        commands.add(lambda s: self.dispatch(push_constants, s))

    def get_final_descriptor_image(self) -> Image:
        return self._final


def format_convert(src: Image, dst: Image, stream=None) -> None:
    """FormatConverter (source/renderModules/FormatConverter.cpp): dst = src texel by texel."""
    check(lib().pbrt_format_convert(C.byref(src.view), C.byref(dst.view), stream_handle(stream)))
