"""Seeded synthetic denoiser inputs (the reference's offline replay input, made up).

The reference's denoiser-only mode replays recorded G-buffers and noisy
illumination (source/VulkanPBRT.cpp:104-115, source/io/RenderIO.cpp); that
dataset is not available, so this module ray-casts an analytic scene (a
ground plane and spheres) with numpy to make G-buffers with the same formats
-- depth R32F, spherical normal RG32F, albedo RGBA8 -- and a noisy,
demodulated 1-spp-like illumination image. Used for denoiser tests and the
denoiser-only benchmark; path-traced inputs come from PBRTPipeline.
"""
from __future__ import annotations

import numpy as np

from .camera import Camera, default_camera


def _normal_encode(n: np.ndarray) -> np.ndarray:
    th = np.arccos(np.clip(n[..., 2], -1.0, 1.0))
    ph = np.arctan2(n[..., 1], n[..., 0])
    return np.stack([th, ph], -1).astype(np.float32)


def gbuffer_scene(width: int, height: int, seed: int = 0, camera: Camera | None = None, spheres: int = 12,
                  noise: float = 0.6):
    """Returns dict(depth [H,W] f32, normal [H,W,2] f32, albedo [H,W,4] u8,
    noisy [H,W,4] f32 (demodulated), clean [H,W,4] f32, camera)."""
    rng = np.random.default_rng(seed)
    cam = camera or default_camera(width, height)
    ys, xs = np.mgrid[0:height, 0:width].astype(np.float64)
    clip = np.stack([(xs + 0.5) / width * 2 - 1, (ys + 0.5) / height * 2 - 1, np.ones_like(xs), np.ones_like(xs)], -1)
    inv_proj = np.linalg.inv(cam.proj64)
    inv_view = np.linalg.inv(cam.view64)
    d = clip @ inv_proj.T
    d = d[..., :3] / np.linalg.norm(d[..., :3], axis=-1, keepdims=True)
    dirs = d @ inv_view[:3, :3].T
    org = inv_view[:3, 3]
    t_best = np.full((height, width), 1e10)
    nrm = np.zeros((height, width, 3))
    nrm[..., :] = 1.0
    alb = np.zeros((height, width, 3))
    # ground plane z = 0
    with np.errstate(divide="ignore", invalid="ignore"):
        tp = -org[2] / dirs[..., 2]
    hit = (tp > 1e-3) & (tp < t_best)
    t_best = np.where(hit, tp, t_best)
    nrm[hit] = (0, 0, 1)
    p = org + dirs * tp[..., None]
    checker = ((np.floor(p[..., 0] * 2) + np.floor(p[..., 1] * 2)) % 2).astype(np.float64)
    alb[hit] = (0.3 + 0.4 * checker[hit, None]) * np.array([0.9, 0.85, 0.8])
    for _ in range(spheres):
        c = np.array([rng.uniform(-2.5, 2.5), rng.uniform(-1.0, 4.0), 0.0])
        r = rng.uniform(0.2, 0.8)
        c[2] = r
        col = rng.uniform(0.05, 1.0, 3)
        oc = org - c
        b = (dirs * oc).sum(-1)
        cc = (oc * oc).sum() - r * r
        disc = b * b - cc
        with np.errstate(invalid="ignore"):
            ts = -b - np.sqrt(np.maximum(disc, 0))
        hit = (disc > 0) & (ts > 1e-3) & (ts < t_best)
        t_best = np.where(hit, ts, t_best)
        ph = org + dirs * ts[..., None]
        nn = (ph - c) / r
        nrm[hit] = nn[hit]
        alb[hit] = col
    miss = t_best >= 1e10
    pos = org + dirs * t_best[..., None]
    depth = np.where(miss, np.linalg.norm(np.full(3, 1e10) - org), t_best).astype(np.float32)
    light = np.array([2.0, -1.0, 4.0])
    ldir = light - pos
    ldist = np.linalg.norm(ldir, axis=-1, keepdims=True)
    ldir = ldir / np.maximum(ldist, 1e-9)
    lam = np.clip((nrm * ldir).sum(-1), 0, None) * 12.0 / (ldist[..., 0] ** 2 + 1.0) + 0.15
    clean = np.repeat(lam[..., None], 3, -1)
    clean[miss] = 1e3
    noisy = clean * rng.gamma(1.0 / noise, noise, size=clean.shape)
    noisy[miss] = 1e3
    normal = _normal_encode(np.where(miss[..., None], np.ones(3), nrm))
    albedo = np.zeros((height, width, 4), np.uint8)
    albedo[..., :3] = np.clip(np.round(alb * 255), 0, 255).astype(np.uint8)
    albedo[..., 3] = 255
    rgba = lambda a: np.concatenate([a, np.ones(a.shape[:-1] + (1,))], -1).astype(np.float32)
    return dict(depth=depth, normal=normal, albedo=albedo, noisy=rgba(noisy), clean=rgba(clean), camera=cam)
