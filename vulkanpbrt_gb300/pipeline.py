"""PBRTPipeline and scene upload over the C ABI (source/renderModules/PBRTPipeline.hpp)."""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _abi
from ._abi import PbrtImage, check, lib, stream_handle
from .render_modules import Commands, GBuffer, Handle, IlluminationBuffer, Image, PushConstants
from .scene import Scene


class PbrtMeshDesc(C.Structure):
    _fields_ = [("positions", C.c_void_p), ("normals", C.c_void_p), ("uvs", C.c_void_p), ("vertex_count", C.c_uint32),
                ("indices", C.c_void_p), ("index_count", C.c_uint32), ("index_stride", C.c_uint32)]


class PbrtObjectInstance(C.Structure):
    _fields_ = [("object_mat", C.c_float * 16), ("mesh_id", C.c_int32), ("index_stride", C.c_uint32),
                ("pad", C.c_int32 * 2)]


class PbrtTextureDesc(C.Structure):
    _fields_ = [("rgba8", C.c_void_p), ("width", C.c_uint32), ("height", C.c_uint32)]


class PbrtSceneDesc(C.Structure):
    _fields_ = [("mesh_count", C.c_uint32), ("meshes", C.POINTER(PbrtMeshDesc)), ("instance_count", C.c_uint32),
                ("instances", C.POINTER(PbrtObjectInstance)), ("instance_opaque", C.c_void_p),
                ("materials", C.c_void_p), ("light_count", C.c_uint32), ("lights", C.c_void_p),
                ("texture_count", C.c_uint32), ("textures", C.POINTER(PbrtTextureDesc)),
                ("mesh_textures", C.c_void_p)]


class PbrtSceneInfo(C.Structure):
    _fields_ = [("triangle_count", C.c_uint32), ("instance_count", C.c_uint32), ("bvh_nodes", C.c_uint32),
                ("bvh_depth", C.c_uint32), ("light_count", C.c_uint32), ("bvh_bytes", C.c_uint64),
                ("triangle_bytes", C.c_uint64), ("build_ms", C.c_double)]


class PbrtTraceStats(C.Structure):
    _fields_ = [("frames", C.c_uint64), ("primary_rays", C.c_uint64), ("extension_rays", C.c_uint64),
                ("shadow_rays", C.c_uint64), ("error_flags", C.c_uint32)]


class PbrtStageTimes(C.Structure):
    _fields_ = [("raygen_ms", C.c_float), ("trace_closest_ms", C.c_float), ("shade_ms", C.c_float),
                ("trace_shadow_ms", C.c_float), ("finalize_ms", C.c_float), ("closest_rays", C.c_uint64),
                ("shadow_rays", C.c_uint64), ("closest_nodes", C.c_uint64), ("closest_tris", C.c_uint64),
                ("shadow_nodes", C.c_uint64), ("shadow_tris", C.c_uint64), ("closest_launches", C.c_uint32)]


H, P = C.c_void_p, C.POINTER
_abi.add_signatures({
    "pbrt_scene_create": (C.c_int32, [P(PbrtSceneDesc), P(H)]),
    "pbrt_scene_create_ex": (C.c_int32, [P(PbrtSceneDesc), C.c_uint32, P(H)]),
    "pbrt_scene_info": (C.c_int32, [H, P(PbrtSceneInfo)]),
    "pbrt_scene_trace_rays": (C.c_int32, [H, H, H, C.c_uint32, C.c_int32, H, H, H]),
    "pbrt_pipeline_create": (C.c_int32, [H, H, H, C.c_int32, P(H)]),
    "pbrt_pipeline_set_config": (C.c_int32, [H, C.c_int32, C.c_int32, C.c_int32]),
    "pbrt_pipeline_trace": (C.c_int32, [H, P(_abi.PbrtPushConstants), H]),
    "pbrt_pipeline_stats": (C.c_int32, [H, H, P(PbrtTraceStats)]),
    "pbrt_pipeline_reset_stats": (C.c_int32, [H, H]),
    "pbrt_pipeline_debug_images": (C.c_int32, [H, P(PbrtImage)]),
    "pbrt_pipeline_profile": (C.c_int32, [H, P(_abi.PbrtPushConstants), H, P(PbrtStageTimes)]),
    "pbrt_pipeline_abort_flag": (C.c_int32, [H, P(P(C.c_uint32))]),
    "pbrt_pipeline_set_budget": (C.c_int32, [H, C.c_uint64]),
    "pbrt_pipeline_status": (C.c_int32, [H, H, P(C.c_int32)]),
    "pbrt_pipeline_set_schedule": (C.c_int32, [H, C.c_int32, C.c_int32]),
})


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def col_major16(m) -> list:
    return np.asarray(m, np.float32).T.reshape(16).tolist()


class SceneHandle(Handle):
    """The scene uploaded to HBM with its 8-wide BVH (RayTracingSceneDescriptorCreationVisitor output
    plus the acceleration-structure build).

    build: "fast_trace" (binned-SAH BVH built on the host, the default) or
    "fast_build" (linear BVH built on the device; lower quality, same hits)."""

    BUILDS = {"fast_trace": 0, "fast_build": 1}

    def __init__(self, scene: Scene, build: str = "fast_trace"):
        if build not in self.BUILDS:
            raise ValueError(f"build must be one of {sorted(self.BUILDS)}, not {build!r}")
        keep = []  # host arrays alive for the duration of the call

        def arr(a, dt):
            a = np.ascontiguousarray(a, dt)
            keep.append(a)
            return a

        meshes = (PbrtMeshDesc * len(scene.meshes))()
        for i, m in enumerate(scene.meshes):
            pos, nor, uv = arr(m.positions, np.float32), arr(m.normals, np.float32), arr(m.uvs, np.float32)
            idx = arr(m.indices, m.indices.dtype)
            meshes[i] = PbrtMeshDesc(_ptr(pos), _ptr(nor), _ptr(uv), len(pos), _ptr(idx), len(idx), m.index_stride)
        insts = (PbrtObjectInstance * len(scene.instance_mesh))()
        for i, (mid, mat) in enumerate(zip(scene.instance_mesh, scene.instance_mats)):
            insts[i].object_mat[:] = col_major16(mat)
            insts[i].mesh_id = mid
            insts[i].index_stride = scene.meshes[mid].index_stride
        opaque = arr(scene.instance_opaque().astype(np.uint8), np.uint8)
        mats = arr(np.stack(scene.materials), np.float32)
        lights = arr(np.stack(scene.lights) if scene.lights else np.zeros((1, 32), np.float32), np.float32)
        texs = (PbrtTextureDesc * len(scene.textures))()
        for i, t in enumerate(scene.textures):
            t = arr(t, np.uint8)
            texs[i] = PbrtTextureDesc(_ptr(t), t.shape[1], t.shape[0])
        mt = arr(np.array(scene.mesh_textures, np.int32), np.int32)
        d = PbrtSceneDesc(len(scene.meshes), meshes, len(insts), insts, _ptr(opaque), _ptr(mats), len(scene.lights),
                          _ptr(lights), len(scene.textures), texs, _ptr(mt))
        h = C.c_void_p()
        check(lib().pbrt_scene_create_ex(C.byref(d), self.BUILDS[build], C.byref(h)))
        super().__init__(h)
        self.scene = scene

    def info(self) -> PbrtSceneInfo:
        i = PbrtSceneInfo()
        check(lib().pbrt_scene_info(self.ptr, C.byref(i)))
        return i

    def trace_rays(self, origins_tmin, directions_tmax, any_hit: bool = False, stream=None):
        """Device float4 tensors [n,4] -> hits [n,4] (t, u, v, key bits)."""
        import torch

        n = origins_tmin.shape[0]
        hits = torch.empty((n, 4), dtype=torch.float32, device=origins_tmin.device)
        scratch = torch.empty(2, dtype=torch.int32, device=origins_tmin.device)
        check(lib().pbrt_scene_trace_rays(self.ptr, origins_tmin.data_ptr(), directions_tmax.data_ptr(), n,
                                          int(any_hit), hits.data_ptr(), scratch.data_ptr(), stream_handle(stream)))
        return hits


class PBRTPipeline(Handle):
    """PBRTPipeline (source/renderModules/PBRTPipeline.hpp:19-60)."""

    SAMPLE_SURFACE_STRENGTH, SAMPLE_LIGHT_STRENGTH, SAMPLE_UNIFORM = 0, 1, 2

    def __init__(self, scene: SceneHandle, g_buffer: Optional[GBuffer], illumination_buffer: IlluminationBuffer,
                 write_g_buffer: bool = True, max_recursion_depth: int = 2, min_recursion_depth: int = 0,
                 light_sampling_method: Optional[int] = None):
        h = C.c_void_p()
        check(lib().pbrt_pipeline_create(scene.ptr, g_buffer.ptr if g_buffer is not None else None,
                                          illumination_buffer.ptr, int(write_g_buffer), C.byref(h)))
        super().__init__(h)
        self._inputs = (scene, g_buffer, illumination_buffer)
        self.illumination_buffer = illumination_buffer
        if light_sampling_method is None:
            light_sampling_method = self.SAMPLE_UNIFORM if len(scene.scene.lights) > 800 else self.SAMPLE_SURFACE_STRENGTH
        self.light_sampling_method = light_sampling_method
        self.max_recursion_depth = max_recursion_depth
        self.min_recursion_depth = min_recursion_depth
        self._apply()
        k = PbrtImage()
        check(lib().pbrt_pipeline_debug_images(h, C.byref(k)))
        self.primary_hit_key = Image(k, self)

    def _apply(self):
        check(lib().pbrt_pipeline_set_config(self.ptr, self.light_sampling_method, self.min_recursion_depth,
                                             self.max_recursion_depth))

    def set_config(self, light_sampling_method=None, min_recursion_depth=None, max_recursion_depth=None):
        if light_sampling_method is not None:
            self.light_sampling_method = light_sampling_method
        if min_recursion_depth is not None:
            self.min_recursion_depth = min_recursion_depth
        if max_recursion_depth is not None:
            self.max_recursion_depth = max_recursion_depth
        self._apply()

    def compile(self, context=None) -> None:
        pass

    def update_image_layouts(self, context=None) -> None:
        pass

    def trace(self, push_constants: PushConstants, stream=None) -> None:
        check(lib().pbrt_pipeline_trace(self.ptr, C.byref(push_constants.value), stream_handle(stream)))

    def add_trace_rays_to_command_graph(self, commands: Commands, push_constants: PushConstants) -> None:
        commands.add(lambda s: self.trace(push_constants, s))

    def get_illumination_buffer(self) -> IlluminationBuffer:
        return self.illumination_buffer

    def stats(self, stream=None) -> PbrtTraceStats:
        s = PbrtTraceStats()
        check(lib().pbrt_pipeline_stats(self.ptr, stream_handle(stream), C.byref(s)))
        return s

    def profile(self, push_constants: PushConstants, stream=None) -> PbrtStageTimes:
        """One frame launched stage by stage with CUDA events (per-kernel times, BVH work counts)."""
        t = PbrtStageTimes()
        check(lib().pbrt_pipeline_profile(self.ptr, C.byref(push_constants.value), stream_handle(stream), C.byref(t)))
        return t

    def reset_stats(self, stream=None) -> None:
        check(lib().pbrt_pipeline_reset_stats(self.ptr, stream_handle(stream)))

    def abort_flag(self):
        """The pinned host word that stops frames while nonzero (ctypes uint32 view)."""
        if getattr(self, "_abort", None) is None:
            p = P(C.c_uint32)()
            check(lib().pbrt_pipeline_abort_flag(self.ptr, C.byref(p)))
            self._abort = p
        return self._abort

    def set_abort(self, on: bool) -> None:
        self.abort_flag()[0] = 1 if on else 0

    def set_launch(self, trace_blocks_per_sm: int = 8, shade_blocks_per_sm: int = 8) -> None:
        """Persistent traversal CTAs and shading CTAs per SM (1..16)."""
        check(lib().pbrt_pipeline_set_launch(self.ptr, trace_blocks_per_sm, shade_blocks_per_sm))

    def set_schedule(self, sort_rays: bool = False, merge_shadow: bool = True) -> None:
        """Frame schedule: ray sorting before traversal; shadow rays merged into the next bounce's launch."""
        check(lib().pbrt_pipeline_set_schedule(self.ptr, int(sort_rays), int(merge_shadow)))

    def set_budget(self, budget_ns: int) -> None:
        check(lib().pbrt_pipeline_set_budget(self.ptr, int(budget_ns)))

    def status(self, stream=None) -> int:
        """PBRT_OK, or PBRT_ERROR_ABORTED / PBRT_ERROR_TIMEOUT for a frame stopped since the last call."""
        st = C.c_int32()
        check(lib().pbrt_pipeline_status(self.ptr, stream_handle(stream), C.byref(st)))
        return st.value
