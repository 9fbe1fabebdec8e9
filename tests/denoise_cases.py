"""Shared set-up for the denoiser parity tests: the same seeded inputs go to
the CUDA path (through the C ABI) and to the CPU oracle."""
from __future__ import annotations

import numpy as np

REL_TOL = 1e-3  # BMFR/BFR output tolerance (relative), on RGBA16F values
ABS_FLOOR = 1e-4  # absolute floor for values near zero


def put(img, arr):
    import torch

    t = img.tensor()
    src = torch.from_numpy(np.ascontiguousarray(arr)).reshape(t.shape)
    t.copy_(src.to(t.device))


def get(img) -> np.ndarray:
    import torch

    torch.cuda.synchronize()
    return img.tensor().cpu().numpy()


def inputs(W, H, seed=0, frame=0):
    from vulkanpbrt_gb300 import synthetic

    s = synthetic.gbuffer_scene(W, H, seed=seed)
    rng = np.random.default_rng(seed + 100)
    noisy16 = s["noisy"].astype(np.float16)
    if frame == 0:
        motion = np.full((H, W, 2), -1, np.float16)
        spp = np.ones((H, W), np.uint8)
    else:
        ys, xs = np.mgrid[0:H, 0:W]
        uv = np.stack([(xs + 0.5) / W + rng.normal(0, 0.3 / W, (H, W)), (ys + 0.5) / H + rng.normal(0, 0.3 / H, (H, W))], -1)
        reject = rng.random((H, W)) < 0.1
        uv[reject] = -1
        motion = uv.astype(np.float16)
        spp = rng.integers(1, 40, (H, W)).astype(np.uint8)
    s.update(noisy16=noisy16, motion=motion, spp=spp)
    return s


def close_fraction(gpu, ref, rel=REL_TOL, floor=ABS_FLOOR):
    g = gpu.astype(np.float64)
    r = ref.astype(np.float64)
    ok = np.abs(g - r) <= rel * np.maximum(np.abs(g), np.abs(r)) + floor
    both_nan = np.isnan(g) & np.isnan(r)
    ok |= both_nan
    return ok.mean(), np.nanmax(np.abs(g - r) / (np.abs(r) + floor))


def stats(name, gpu, ref):
    frac, worst = close_fraction(gpu, ref)
    print(f"{name}: within {REL_TOL:g} rel: {frac * 100:.4f}%  worst rel {worst:.3g}")
    return frac
