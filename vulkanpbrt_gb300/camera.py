"""Camera matrices with vsg's conventions (column vectors, m[row, col]).

vsg::Perspective / vsg::LookAt as the reference's frame loop builds them
(source/VulkanPBRT.cpp:314-324): perspective() follows
external/vsg/include/vsg/maths/transform.h:148-156 (Vulkan clip space, y
flipped, depth 0..1), look_at() follows transform.h:169-183. Inverses are
taken in float64 and rounded to float32, as vsg's double-precision
Perspective/LookAt::inverse() results are.
"""
from __future__ import annotations

import math

import numpy as np


def perspective(fovy_degrees: float, aspect: float, z_near: float, z_far: float) -> np.ndarray:
    f = 1.0 / math.tan(math.radians(fovy_degrees) * 0.5)
    r = 1.0 / (z_near - z_far)
    m = np.zeros((4, 4), dtype=np.float64)
    m[0, 0] = f / aspect
    m[1, 1] = -f
    m[2, 2] = z_far * r
    m[3, 2] = -1.0
    m[2, 3] = z_far * z_near * r
    return m


def look_at(eye, center, up) -> np.ndarray:
    eye, center, up = (np.asarray(v, dtype=np.float64) for v in (eye, center, up))
    forward = center - eye
    forward /= np.linalg.norm(forward)
    up_n = up / np.linalg.norm(up)
    side = np.cross(forward, up_n)
    side /= np.linalg.norm(side)
    u = np.cross(side, forward)
    u /= np.linalg.norm(u)
    rot = np.eye(4)
    rot[0, :3] = side
    rot[1, :3] = u
    rot[2, :3] = -forward
    trans = np.eye(4)
    trans[:3, 3] = -eye
    return rot @ trans


class Camera:
    """A pinhole camera: view / projection matrices and their inverses (float32)."""

    def __init__(self, eye, center, up=(0.0, 0.0, 1.0), fovy_degrees=60.0, aspect=16 / 9, z_near=0.1, z_far=1000.0):
        self.view64 = look_at(eye, center, up)
        self.proj64 = perspective(fovy_degrees, aspect, z_near, z_far)
        self.view = self.view64.astype(np.float32)
        self.proj = self.proj64.astype(np.float32)
        self.inv_view = np.linalg.inv(self.view64).astype(np.float32)
        self.inv_proj = np.linalg.inv(self.proj64).astype(np.float32)


def default_camera(width: int, height: int) -> Camera:
    """The reference's default camera: eye (0,-3,1) -> (0,0,1), z up, 60 deg, near .1, far 1000."""
    return Camera((0.0, -3.0, 1.0), (0.0, 0.0, 1.0), (0.0, 0.0, 1.0), 60.0, width / height, 0.1, 1000.0)


def orbit_camera(width: int, height: int, frame: int, frames: int, radius=12.0, height_z=5.0, center=(0.0, 0.0, 1.0),
                 degrees_per_frame=None) -> Camera:
    """Camera on a circular orbit around `center` (the 16-frame orbit workload)."""
    step = degrees_per_frame if degrees_per_frame is not None else 360.0 / max(frames, 1) / 8.0
    a = math.radians(step * frame)
    eye = (center[0] + radius * math.sin(a), center[1] - radius * math.cos(a), height_z)
    return Camera(eye, center, (0.0, 0.0, 1.0), 60.0, width / height, 0.1, 1000.0)


def col_major(m: np.ndarray) -> np.ndarray:
    """float32 [16] column-major (GLSL / vsg::mat4 memory order)."""
    return np.ascontiguousarray(np.asarray(m, dtype=np.float32).T).reshape(16)


class CropCamera:
    """The pixels [x0, x0 + w) x [y0, y0 + h) of a full_w x full_h frame of
    `cam`, as a camera of its own: the inverse projection maps the crop's
    NDC onto that window of the full frame's NDC, so a w x h render of it
    matches the same pixels of the full render (same rays, same pixel
    footprint)."""

    def __init__(self, cam: Camera, full_w: int, full_h: int, x0: int, y0: int, w: int, h: int):
        s = np.eye(4)
        s[0, 0] = w / full_w
        s[1, 1] = h / full_h
        s[0, 3] = (2.0 * x0 + w) / full_w - 1.0
        s[1, 3] = (2.0 * y0 + h) / full_h - 1.0
        self.view64 = cam.view64
        self.proj64 = np.linalg.inv(s) @ cam.proj64
        self.view = cam.view
        self.inv_view = cam.inv_view
        self.proj = self.proj64.astype(np.float32)
        self.inv_proj = (np.linalg.inv(cam.proj64) @ s).astype(np.float32)
