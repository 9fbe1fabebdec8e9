"""Offline replay I/O (source/io/RenderIO.hpp, RenderIO.cpp): recorded
G-buffers, illumination and camera matrices on disk, and their staging to
and from the device buffers.

* `MatrixIO` -- camera matrices as JSON ("amtOfFrames", "matrices" with
  view / invView [/ proj / invProj], column major; RenderIO.cpp:593-716) or
  the BMFR dataset's text format (16 numbers per frame, column major, the
  inverse computed on import).
* `GBufferIO`, `IlluminationBufferIO` -- per-frame OpenEXR files named by a
  printf pattern with the frame index (e.g. "depth_%d.exr"), read and
  written by `exr` (RenderIO.cpp:6-591). Conversions as the reference's:
  normals stored as cartesian RGBA (z = cos theta) and held as (theta, phi);
  albedo stored as float RGBA and held as 8-bit (x 255, truncated); depth
  stored as R32F or recovered from a position image; material and albedo
  exported as float (/ 255).
* `OfflineGBuffer`, `OfflineIllumination` -- host arrays of one frame plus a
  staging copy that `upload_to_*_command` / `download_from_*_command`
  record as host<->device copies into a `Commands` list, and
  `transfer_staging_data_from/to` fill or drain between frames
  (VulkanPBRT.cpp:568-605).

Deliberate differences from the reference: the position -> depth import
takes the camera position from column 3 of the inverse view matrix (the
export side's column, RenderIO.cpp:356), where the import reads column 2
(RenderIO.cpp:106), which holds the camera's z axis; frames are loaded on a
thread pool rather than one thread per frame; a missing file raises
FileNotFoundError instead of printing and leaving the frame empty.
"""
from __future__ import annotations

import ctypes as C
import json
import re
from concurrent.futures import ThreadPoolExecutor
from typing import List

import numpy as np

from . import exr
from ._abi import check, lib, stream_handle
from .render_modules import CameraMatrices, Commands, GBuffer, IlluminationBuffer

CameraMatricesVec = List[CameraMatrices]
_NUMBER = re.compile(r"[-+]?(\d+\.?\d*|\.\d+)([eE][-+]?\d+)?")


def _pool(n):
    return ThreadPoolExecutor(max_workers=max(1, min(16, n)))


# ---- camera matrices -------------------------------------------------------
def _from_col_major(vals) -> np.ndarray:
    return np.asarray(vals, np.float32).reshape(4, 4).T.copy()


def _to_col_major(m) -> list:
    return [float(v) for v in np.asarray(m, np.float32).T.reshape(16)]


class MatrixIO:
    @staticmethod
    def import_matrices(matrix_path: str) -> CameraMatricesVec:
        """RenderIO.cpp:593-659. JSON when the name ends in .json, else the
        BMFR text format: every whitespace-separated token that starts with
        a digit or '-' (after dropping a trailing ',' and a leading '{') is a
        number; each 16 numbers are one column-major view matrix."""
        with open(matrix_path) as f:
            text = f.read()
        out: CameraMatricesVec = []
        if matrix_path.endswith(".json"):
            js = json.loads(text)
            for i in range(int(js["amtOfFrames"])):
                m = js["matrices"][i]
                cm = CameraMatrices(_from_col_major(m["view"]), _from_col_major(m["invView"]))
                if m.get("type") == "ModelView+Projection":
                    cm.proj, cm.inv_proj = _from_col_major(m["proj"]), _from_col_major(m["invProj"])
                out.append(cm)
            return out
        vals = []
        for tok in text.split():
            if tok.endswith(","):
                tok = tok[:-1]
            if tok.startswith("{"):
                tok = tok[1:]
            if tok and (tok[0].isdigit() or tok[0] == "-"):
                num = _NUMBER.match(tok)  # std::stof: the longest numeric prefix
                if not num:
                    raise ValueError(f"{matrix_path}: cannot parse {tok!r}")
                vals.append(float(np.float32(float(num.group(0)))))
                if len(vals) == 16:
                    v = _from_col_major(vals)
                    out.append(CameraMatrices(v, np.linalg.inv(v.astype(np.float64)).astype(np.float32)))
                    vals = []
        return out

    @staticmethod
    def export_matrices(matrix_path: str, matrices: CameraMatricesVec) -> bool:
        """RenderIO.cpp:661-716 (JSON, 4-space indent)."""
        mats = []
        for m in matrices:
            has_proj = m.proj is not None
            obj = {"type": "ModelView+Projection" if has_proj else "ModelViewProjection", "storageType": "ColumnMajor",
                   "view": _to_col_major(m.view), "invView": _to_col_major(m.inv_view)}
            if has_proj:
                obj["proj"] = _to_col_major(m.proj)
                obj["invProj"] = _to_col_major(m.inv_proj)
            mats.append(obj)
        with open(matrix_path, "w") as f:
            f.write(json.dumps({"amtOfFrames": len(matrices), "matrices": mats}, indent=4))
        return True


# ---- conversions (RenderIO.cpp:166-391) ------------------------------------
def convert_normal_to_spherical(normals: np.ndarray) -> np.ndarray:
    """[H,W,4] cartesian -> [H,W,2] (acos z, atan2(y, x)), float32."""
    n = np.asarray(normals, np.float32)
    return np.stack([np.arccos(n[..., 2]), np.arctan2(n[..., 1], n[..., 0])], -1).astype(np.float32)


def spherical_to_cartesian(normals: np.ndarray) -> np.ndarray:
    n = np.asarray(normals, np.float32)
    th, ph = n[..., 0], n[..., 1]
    s = np.sin(th)
    return np.stack([np.cos(ph) * s, np.sin(ph) * s, np.cos(th), np.ones_like(th)], -1).astype(np.float32)


def compress_albedo(a: np.ndarray) -> np.ndarray:
    """float / half RGBA (x 255, truncated towards zero, clamped to [0, 255])
    or 32-bit unsigned RGBA (low byte) -> 8-bit RGBA."""
    a = np.asarray(a)
    if a.dtype == np.uint32:
        return (a & 0xFF).astype(np.uint8)
    v = a.astype(np.float32) * np.float32(255.0)
    return np.clip(np.trunc(np.nan_to_num(v)), 0, 255).astype(np.uint8)


def unorm_to_float(a: np.ndarray) -> np.ndarray:
    return np.asarray(a, np.float32) / np.float32(255.0)


def depth_to_position(depth: np.ndarray, m: CameraMatrices) -> np.ndarray:
    """RenderIO.cpp:337-370: camera position + depth x world direction of the
    pixel centre's ray ((x+.5)/W*2-1, (y+.5)/H*2-1)."""
    if m.proj is None:
        raise ValueError("depth_to_position needs camera matrices with a separate projection matrix")
    H, W = depth.shape
    x = (np.arange(W, dtype=np.float32) + np.float32(0.5)) / np.float32(W) * 2 - 1
    y = (np.arange(H, dtype=np.float32) + np.float32(0.5)) / np.float32(H) * 2 - 1
    px, py = np.meshgrid(x, y)
    ip = np.asarray(m.inv_proj, np.float32)
    iv = np.asarray(m.inv_view, np.float32)
    p = np.stack([px, py, np.ones_like(px), np.ones_like(px)], -1)
    d = p @ ip.T
    d[..., 3] = 0
    d = d / np.linalg.norm(d, axis=-1, keepdims=True)
    dirw = (d @ iv.T)[..., :3] * depth[..., None]
    pos = iv[:3, 3] + dirw
    return np.concatenate([pos, np.ones((H, W, 1), np.float32)], -1).astype(np.float32)


def position_to_depth(pos: np.ndarray, m: CameraMatrices) -> np.ndarray:
    """RenderIO.cpp:96-116 (camera position from the inverse view's column 3)."""
    iv = np.asarray(m.inv_view, np.float32)
    cam = iv[:, 3] / iv[3, 3]
    return np.linalg.norm(cam[:3] - np.asarray(pos, np.float32)[..., :3], axis=-1).astype(np.float32)


# ---- device staging --------------------------------------------------------
def _upload(img, arr: np.ndarray, stream) -> None:
    a = np.ascontiguousarray(arr)
    row = a.nbytes // img.height
    if a.nbytes != img.view.row_bytes * img.height:
        raise ValueError(f"host array of {a.nbytes} bytes does not fill a {img.width}x{img.height} image")
    check(lib().pbrt_image_upload(C.byref(img.view), a.ctypes.data_as(C.c_void_p), row, stream_handle(stream)))


def _download(img, arr: np.ndarray, stream) -> None:
    if not arr.flags["C_CONTIGUOUS"] or arr.nbytes != img.view.row_bytes * img.height:
        raise ValueError("download target must be a contiguous array of the image's size")
    check(lib().pbrt_image_download(C.byref(img.view), arr.ctypes.data_as(C.c_void_p), arr.nbytes // img.height,
                                    stream_handle(stream)))


def _sync(stream) -> None:
    check(lib().pbrt_stream_synchronize(stream_handle(stream)))


class OfflineGBuffer:
    """One frame of G-buffer data on the host (RenderIO.hpp:43-60): depth
    [H,W] f32, normal [H,W,2] f32 (theta, phi), material / albedo [H,W,4] u8."""

    def __init__(self, depth=None, normal=None, material=None, albedo=None):
        self.depth, self.normal, self.material, self.albedo = depth, normal, material, albedo
        self._staging = None

    def _stage(self, w, h):
        if self._staging is None:
            self._staging = OfflineGBuffer(np.zeros((h, w), np.float32), np.zeros((h, w, 2), np.float32),
                                           np.zeros((h, w, 4), np.uint8), np.zeros((h, w, 4), np.uint8))
        return self._staging

    def upload_to_g_buffer_command(self, g_buffer: GBuffer, commands: Commands, context=None) -> None:
        st = self._stage(g_buffer.width, g_buffer.height)

        def run(s):
            _upload(g_buffer.depth, st.depth, s)
            _upload(g_buffer.normal, st.normal, s)
            _upload(g_buffer.material, st.material, s)
            _upload(g_buffer.albedo, st.albedo, s)
            _sync(s)  # the staging arrays may be refilled once the copies are done

        commands.add(run)

    def download_from_g_buffer_command(self, g_buffer: GBuffer, commands: Commands, context=None) -> None:
        st = self._stage(g_buffer.width, g_buffer.height)

        def run(s):
            _download(g_buffer.depth, st.depth, s)
            _download(g_buffer.normal, st.normal, s)
            _download(g_buffer.material, st.material, s)
            _download(g_buffer.albedo, st.albedo, s)
            _sync(s)

        commands.add(run)

    def transfer_staging_data_from(self, other: "OfflineGBuffer") -> None:
        h, w = other.depth.shape
        st = self._stage(w, h)
        st.depth[...] = other.depth
        st.normal[...] = other.normal
        st.albedo[...] = other.albedo
        st.material[...] = other.material if other.material is not None else 0

    def transfer_staging_data_to(self, other: "OfflineGBuffer") -> None:
        st = self._staging
        if st is None:
            raise RuntimeError("this stager has not been added to a command list")
        other.depth, other.normal = st.depth.copy(), st.normal.copy()
        other.material, other.albedo = st.material.copy(), st.albedo.copy()


class OfflineIllumination:
    """One frame of illumination on the host: noisy [H,W,4] f16 or f32
    (RenderIO.hpp:83-100)."""

    def __init__(self, noisy=None):
        self.noisy = noisy
        self._staging = None

    def _stage(self, img):
        if self._staging is None:
            dt = np.float16 if img.view.texel_bytes == 8 else np.float32
            self._staging = np.zeros((img.height, img.width, 4), dt)
        return self._staging

    def upload_to_illumination_buffer_command(self, illu_buffer: IlluminationBuffer, commands: Commands,
                                              context=None) -> None:
        img = illu_buffer.illumination_images[0]
        st = self._stage(img)

        def run(s):
            _upload(img, st, s)
            _sync(s)

        commands.add(run)

    def download_from_illumination_buffer_command(self, illu_buffer: IlluminationBuffer, commands: Commands,
                                                  context=None) -> None:
        img = illu_buffer.illumination_images[0]
        st = self._stage(img)

        def run(s):
            _download(img, st, s)
            _sync(s)

        commands.add(run)

    def transfer_staging_data_from(self, other: "OfflineIllumination") -> None:
        if self._staging is None:
            raise RuntimeError("this stager has not been added to a command list")
        self._staging[...] = other.noisy

    def transfer_staging_data_to(self, other: "OfflineIllumination") -> None:
        if self._staging is None:
            raise RuntimeError("this stager has not been added to a command list")
        other.noisy = self._staging.copy()


def _name(fmt: str, f: int) -> str:
    return fmt % f


class GBufferIO:
    @staticmethod
    def import_g_buffer_depth(depth_format, normal_format, material_format, albedo_format, num_frames,
                              verbosity=1) -> List[OfflineGBuffer]:
        """RenderIO.cpp:6-72 (material_format is accepted and unused, as there)."""
        def one(f):
            d = exr.load(_name(depth_format, f))
            if d.ndim == 3:
                d = d[..., 0]
            n = convert_normal_to_spherical(exr.load(_name(normal_format, f)))
            a = compress_albedo(exr.load(_name(albedo_format, f)))
            return OfflineGBuffer(np.ascontiguousarray(d, np.float32), n, None, a)

        with _pool(num_frames) as ex:
            out = list(ex.map(one, range(num_frames)))
        if verbosity > 0:
            print(f"Loaded {num_frames} G-buffer frames")
        return out

    @staticmethod
    def import_g_buffer_position(position_format, normal_format, material_format, albedo_format,
                                 matrices: CameraMatricesVec, num_frames, verbosity=1) -> List[OfflineGBuffer]:
        """RenderIO.cpp:74-152: depth = distance of each position from the camera."""
        def one(f):
            pos = exr.load(_name(position_format, f))
            if pos.ndim != 3 or pos.shape[-1] != 4:
                raise exr.ExrError("unexpected position format (want RGBA)")
            d = position_to_depth(pos, matrices[f])
            n = convert_normal_to_spherical(exr.load(_name(normal_format, f)))
            a = compress_albedo(exr.load(_name(albedo_format, f)))
            return OfflineGBuffer(d, n, None, a)

        with _pool(num_frames) as ex:
            out = list(ex.map(one, range(num_frames)))
        if verbosity > 0:
            print(f"Loaded {num_frames} G-buffer frames")
        return out

    @staticmethod
    def export_g_buffer(position_format, depth_format, normal_format, material_format, albedo_format, num_frames,
                        g_buffers: List[OfflineGBuffer], matrices: CameraMatricesVec, verbosity=1,
                        compression="ZIP") -> bool:
        """RenderIO.cpp:213-320: every non-empty pattern is written."""
        def one(f):
            g = g_buffers[f]
            if depth_format:
                exr.save(_name(depth_format, f), np.asarray(g.depth, np.float32), compression)
            if position_format:
                exr.save(_name(position_format, f), depth_to_position(g.depth, matrices[f]), compression)
            if normal_format:
                exr.save(_name(normal_format, f), spherical_to_cartesian(g.normal), compression)
            if material_format:
                exr.save(_name(material_format, f), unorm_to_float(g.material), compression)
            if albedo_format:
                exr.save(_name(albedo_format, f), unorm_to_float(g.albedo), compression)

        with _pool(num_frames) as ex:
            list(ex.map(one, range(num_frames)))
        return True


class IlluminationBufferIO:
    @staticmethod
    def import_illumination(illumination_format, num_frames, verbosity=1) -> List[OfflineIllumination]:
        """RenderIO.cpp:521-560: RGBA as stored (half -> f16, float -> f32)."""
        def one(f):
            a = exr.load(_name(illumination_format, f))
            if a.ndim != 3 or a.shape[-1] != 4 or a.dtype not in (np.float16, np.float32):
                raise exr.ExrError("illumination images must be half or float RGBA")
            return OfflineIllumination(np.ascontiguousarray(a))

        with _pool(num_frames) as ex:
            return list(ex.map(one, range(num_frames)))

    @staticmethod
    def export_illumination(illumination_format, num_frames, illus: List[OfflineIllumination], verbosity=1,
                            compression="ZIP") -> bool:
        def one(f):
            exr.save(_name(illumination_format, f), np.asarray(illus[f].noisy), compression)

        with _pool(num_frames) as ex:
            list(ex.map(one, range(num_frames)))
        return True


def illumination_buffer_for(noisy: np.ndarray, width: int, height: int) -> IlluminationBuffer:
    """The buffer the reference creates for replayed illumination
    (VulkanPBRT.cpp:375-389): RGBA16F -> Demodulated, RGBA32F -> DemodulatedFloat."""
    from .render_modules import IlluminationBufferDemodulated, IlluminationBufferDemodulatedFloat

    if noisy.dtype == np.float16:
        return IlluminationBufferDemodulated(width, height)
    if noisy.dtype == np.float32:
        return IlluminationBufferDemodulatedFloat(width, height)
    raise ValueError("Offline illumination buffer image format not compatible")


__all__ = ["MatrixIO", "GBufferIO", "IlluminationBufferIO", "OfflineGBuffer", "OfflineIllumination", "CameraMatrices",
           "convert_normal_to_spherical", "spherical_to_cartesian", "compress_albedo", "unorm_to_float",
           "depth_to_position", "position_to_depth", "illumination_buffer_for"]
