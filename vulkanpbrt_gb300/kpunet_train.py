"""Training data and training loop of the kernel-predicting denoiser.

Every training pair comes from this library's own path tracer: a seeded
procedural scene (the instanced field of displaced icospheres and boxes, or
the Cornell-style box with spheres), a camera, and a window of a 1920x1080
frame rendered at 1 spp (several independent frames: the network inputs) and
at `target_spp` spp (the mean of that many frames of the demodulated
illumination: the target). The window is cut into square crops. Training
runs the network's own forward and backward kernels with Adam on FP32
master weights.

Usage (on a GPU):
    python -m vulkanpbrt_gb300.kpunet_train --out weights.npz
"""
from __future__ import annotations

import argparse
import json
import math
import time
from concurrent.futures import ThreadPoolExecutor

import numpy as np


def _scene(kind, seed, texture_size, instances):
    from . import scene as S

    if kind == "cornell":
        return S.cornell_spheres(seed=seed)
    return S.instanced_field(seed=seed, instances=instances, texture_size=texture_size)


def _camera(kind, sc, rng, full_w, full_h):
    from .camera import Camera

    if kind == "cornell":
        eye = (rng.uniform(-0.6, 0.6), rng.uniform(-3.4, -2.6), rng.uniform(0.7, 1.6))
        center = (rng.uniform(-0.3, 0.3), 0.0, rng.uniform(0.6, 1.2))
        return Camera(eye, center, aspect=full_w / full_h)
    c = np.asarray(sc.camera_center, np.float64)
    e0 = np.asarray(sc.camera_eye, np.float64)
    r = math.hypot(e0[0] - c[0], e0[1] - c[1]) * rng.uniform(0.35, 1.1)
    a = rng.uniform(0, 2 * math.pi)
    eye = (c[0] + r * math.cos(a), c[1] + r * math.sin(a), e0[2] * rng.uniform(0.3, 1.2))
    center = (c[0] + rng.uniform(-5, 5), c[1] + rng.uniform(-5, 5), c[2])
    return Camera(eye, center, aspect=full_w / full_h)


def render_views(views, window=1024, crop=256, full=(1920, 1080), inputs=16, target_spp=4096, max_depth=8,
                 min_depth=3, texture_size=256, instances=2000, device="cuda", log=print):
    """views: list of (kind, scene_seed, camera_seed). Returns a dict of device
    tensors with one entry per crop: illum [M, inputs, crop, crop, 4] f32,
    albedo [M, crop, crop, 4] u8, normal [M, crop, crop, 2] f32, depth
    [M, crop, crop] f32, target [M, crop, crop, 3] f32."""
    import torch

    from . import render_modules as R
    from .camera import CropCamera
    from .pipeline import PBRTPipeline, SceneHandle

    full_w, full_h = full
    per = (window // crop) ** 2
    M = len(views) * per
    dev = torch.device(device)
    out = {
        "illum": torch.empty((M, inputs, crop, crop, 4), dtype=torch.float32, device=dev),
        "albedo": torch.empty((M, crop, crop, 4), dtype=torch.uint8, device=dev),
        "normal": torch.empty((M, crop, crop, 2), dtype=torch.float32, device=dev),
        "depth": torch.empty((M, crop, crop), dtype=torch.float32, device=dev),
        "target": torch.empty((M, crop, crop, 3), dtype=torch.float32, device=dev),
    }
    g = R.GBuffer(window, window)
    illu = R.IlluminationBufferDemodulatedFloat(window, window)
    acc = torch.empty((window, window, 3), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    pc = R.PushConstants()
    cache = {}
    m = 0
    t0 = time.time()
    # the next scene is built on the host while the GPU traces the current one
    keys = list(dict.fromkeys((kind, sseed) for kind, sseed, _ in views))
    pool = ThreadPoolExecutor(1)
    pending = {}

    def want(i):
        if i < len(keys) and keys[i] not in pending:
            pending[keys[i]] = pool.submit(_scene, keys[i][0], keys[i][1], texture_size, instances)

    want(0)
    for vi, (kind, sseed, cseed) in enumerate(views):
        key = (kind, sseed)
        if key not in cache:
            cache.clear()
            want(keys.index(key))
            sc = pending.pop(key).result()
            want(keys.index(key) + 1)
            sh = SceneHandle(sc)
            pipe = PBRTPipeline(sh, g, illu, True, max_recursion_depth=max_depth, min_recursion_depth=min_depth)
            cache[key] = (sc, sh, pipe)
        sc, sh, pipe = cache[key]
        rng = np.random.default_rng(cseed)
        cam = _camera(kind, sc, rng, full_w, full_h)
        x0 = int(rng.integers(0, full_w - window + 1))
        y0 = int(rng.integers(0, full_h - window + 1))
        cc = CropCamera(cam, full_w, full_h, x0, y0, window, window)
        img = illu.illumination_images[0].tensor()
        frame_base = 1 + vi * (target_spp + inputs + 1)
        ins = []
        for k in range(inputs):
            pc.set(view_inverse=cc.inv_view, proj_inverse=cc.inv_proj, prev_view=cc.view,
                   frame_number=frame_base + k, sample_number=0)
            pipe.trace(pc, stream)
            ins.append(img.clone())
        albedo = g.albedo.tensor().clone()
        normal = g.normal.tensor().clone()
        depth = g.depth.tensor()[..., 0].clone()
        acc.zero_()
        for s in range(target_spp):
            pc.set(frame_number=frame_base + inputs + s)
            pipe.trace(pc, stream)
            acc += img[..., :3]
        target = (acc / target_spp).float()
        for cy in range(window // crop):
            for cx in range(window // crop):
                sl = (slice(cy * crop, (cy + 1) * crop), slice(cx * crop, (cx + 1) * crop))
                for k in range(inputs):
                    out["illum"][m, k] = ins[k][sl]
                out["albedo"][m] = albedo[sl]
                out["normal"][m] = normal[sl]
                out["depth"][m] = depth[sl]
                out["target"][m] = target[sl]
                m += 1
        if log and (vi % 5 == 0 or vi == len(views) - 1):
            torch.cuda.synchronize()
            log(f"view {vi + 1}/{len(views)} ({kind} seed {sseed}) {time.time() - t0:.1f} s")
    pool.shutdown()
    return out


def default_views(n_views, seed=1000, cornell_fraction=0.25, views_per_scene=2):
    """Scene seeds start at `seed` (the benchmark's scene, seed 0, is never trained on)."""
    rng = np.random.default_rng(seed)
    views = []
    for i in range(n_views):
        s = seed + i // views_per_scene
        kind = "cornell" if rng.random() < cornell_fraction else "field"
        views.append((kind, int(s), int(rng.integers(1 << 30))))
    views.sort(key=lambda v: (v[0], v[1]))
    return views


def augment(batch, rng):
    """Random flips and transposes of square crops (the network has no
    preferred orientation)."""
    if rng.random() < 0.5:
        batch = {k: v.flip(2 if k == "illum" else 1) for k, v in batch.items()}
    if rng.random() < 0.5:
        batch = {k: v.flip(3 if k == "illum" else 2) for k, v in batch.items()}
    if rng.random() < 0.5:
        batch = {k: (v.transpose(2, 3) if k == "illum" else v.transpose(1, 2)).contiguous() for k, v in batch.items()}
    return batch


SPP_CHOICES = (1, 1, 2, 4, 8, 16)  # samples averaged into one network input (1 spp twice as likely)


def train(net, data, steps, batch=16, lr=1e-4, seed=0, log_every=100, var_weight=0.1, log=print,
          lr_floor=0.1, kernel="umma", checkpoint=None, checkpoint_every=0):
    """Adam steps over random crops; each input is the mean of k of the
    crop's one-sample frames (k from SPP_CHOICES, with the matching samples-
    per-pixel channel, as the Accumulator's output carries it) -- so one
    network serves raw 1-spp and accumulated input. Cosine learning-rate
    decay to lr * lr_floor. kernel: the convolutions (forward, backward data
    and weights) on "mma" (mma.sync) or "umma" (tcgen05). With `checkpoint`
    (a path), the weights are saved there every `checkpoint_every` steps.
    Returns the loss history."""
    import torch

    from . import nn

    M, inputs, crop = data["illum"].shape[:3]
    dev = data["illum"].device
    ws = net.workspace(batch, crop, crop)
    rng = np.random.default_rng(seed)
    hist = []
    t0 = time.time()
    spp_u8 = torch.empty((batch, crop, crop), dtype=torch.uint8, device=dev)
    for it in range(steps):
        idx = rng.integers(0, M, batch)
        ill = []
        for j, m in enumerate(idx):
            k = min(int(rng.choice(SPP_CHOICES)), inputs)
            frames = torch.from_numpy(rng.permutation(inputs)[:k]).to(dev)
            ill.append(data["illum"][int(m)][frames].mean(0))
            spp_u8[j] = int(round(k / 256.0 * 255.0))  # the accumulator's R8 spp encoding
        ti = torch.from_numpy(idx).to(dev)
        b = {"illum": torch.stack(ill)[:, None], "albedo": data["albedo"][ti], "normal": data["normal"][ti],
             "depth": data["depth"][ti], "target": data["target"][ti], "spp": spp_u8}
        b = augment(b, rng)
        illum = b["illum"][:, 0].contiguous()
        nn.features(illum, b["albedo"].contiguous(), b["normal"].contiguous(), b["depth"].contiguous(), ws.feat,
                    ws.rad[0], spp=b["spp"].contiguous())
        cur = lr * (lr_floor + (1 - lr_floor) * 0.5 * (1 + math.cos(math.pi * it / max(steps, 1))))
        loss = ws.train_step(b["target"].contiguous(), b["albedo"].contiguous(), lr=cur, var_weight=var_weight,
                             kernel=kernel)
        if it % log_every == 0 or it == steps - 1:
            lv = loss.tolist()
            hist.append((it, lv[0], lv[1]))
            if log:
                log(f"step {it} relMSE {lv[0]:.5f} var {lv[1]:.4f} lr {cur:.2e} {time.time() - t0:.1f} s")
        if checkpoint and checkpoint_every and (it + 1) % checkpoint_every == 0 and it + 1 < steps:
            net.save(checkpoint)
    return hist


def main(argv=None):
    import torch

    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--views", type=int, default=24)
    ap.add_argument("--views-per-scene", type=int, default=2, help="views (windows) rendered from each seeded scene")
    ap.add_argument("--scene-seed", type=int, default=1000, help="first scene seed (the benchmark scene is seed 0)")
    ap.add_argument("--window", type=int, default=1024)
    ap.add_argument("--crop", type=int, default=256)
    ap.add_argument("--inputs", type=int, default=16)
    ap.add_argument("--target-spp", type=int, default=4096)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--lr", type=float, default=1e-4)
    ap.add_argument("--max-depth", type=int, default=8)
    ap.add_argument("--min-depth", type=int, default=3)
    ap.add_argument("--texture-size", type=int, default=256)
    ap.add_argument("--instances", type=int, default=2000)
    ap.add_argument("--init", default=None, help="start from these weights")
    ap.add_argument("--kernel", default="umma", choices=["mma", "umma"],
                    help="convolutions (forward and backward) on tcgen05 (default) or mma.sync")
    ap.add_argument("--out", required=True)
    ap.add_argument("--checkpoint-every", type=int, default=0, help="also save the weights to --out every N steps")
    ap.add_argument("--log", default=None)
    a = ap.parse_args(argv)

    from . import build

    build.build()
    from .kpunet import KPUNet

    dev = torch.device("cuda", 0)
    t0 = time.time()
    views = default_views(a.views, seed=a.scene_seed, views_per_scene=a.views_per_scene)
    data = render_views(views, a.window, a.crop, inputs=a.inputs, target_spp=a.target_spp, max_depth=a.max_depth,
                        min_depth=a.min_depth, texture_size=a.texture_size, instances=a.instances, device=dev)
    t_data = time.time() - t0
    net = KPUNet.load(a.init, dev) if a.init else KPUNet(dev, seed=0)
    t1 = time.time()
    hist = train(net, data, a.steps, a.batch, a.lr, kernel=a.kernel, checkpoint=a.out,
                 checkpoint_every=a.checkpoint_every)
    torch.cuda.synchronize()
    t_train = time.time() - t1
    net.save(a.out)
    rec = {"views": len(views), "scene_count": len({(k, s) for k, s, _ in views}), "window": a.window,
           "crops": int(data["illum"].shape[0]), "inputs_per_crop": a.inputs,
           "target_spp": a.target_spp, "steps": a.steps, "batch": a.batch, "lr": a.lr, "data_s": t_data,
           "train_s": t_train, "init": a.init, "kernel": a.kernel, "loss": hist, "scenes": sorted({(k, s) for k, s, _ in views})}
    if a.log:
        with open(a.log, "w") as f:
            json.dump(rec, f, indent=1)
    print(json.dumps({k: v for k, v in rec.items() if k not in ("loss", "scenes")}))


if __name__ == "__main__":
    main()
