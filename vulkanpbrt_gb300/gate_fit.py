"""Fitting the neural denoiser's learned tile gate (no reference counterpart).

The gate (pbrt_nn_gate_model) shows, per 32x32 tile, alpha * network +
(1 - alpha) * BMFR with alpha in {1, 0.75, 0.5, 0.25, 0}: four linear
functions of eight per-tile log features predict how much each blend
changes the tile's relative squared error against the network alone, and
the tile takes the lowest prediction below zero. This module makes the
training data and fits the predictions:

    python -m vulkanpbrt_gb300.gate_fit collect --out gate_data.npz   # GPU
    python -m vulkanpbrt_gb300.gate_fit fit gate_data.npz --out gate.json

collect renders held-out seeded instanced fields (never the benchmark's seed
0) through the benchmark's frame -- trace, accumulate, BMFR 32x32, the
network -- along the benchmark's 16-frame orbit and, at a few frames, the
features the gate kernel computes, plus the per-tile relMSE of the network,
of BMFR and of the three blends against a many-sample render of the same
camera (remodulated by the G-buffer albedo, as the benchmark measures). fit
is a ridge regression per blend of the error change on standardised
features, with the regularisation chosen by leave-one-scene-out error of
the resulting choice, written back as coefficients on the raw features.
"""
from __future__ import annotations

import argparse
import json
from pathlib import Path

import numpy as np

FEATURES = ["log mean exp(predicted log relative squared error)",
            "log mean squared final-image difference, network vs BMFR",
            "log mean samples per pixel", "log variance of log(1 + noisy luminance)", "log mean |d log depth|",
            "log (1 - |mean normal|)", "log mean noisy luminance", "log mean albedo"]
TILE = 32


def tile_features(var, nn_fin, bm_fin, spp, noisy, depth, nrm, alb8):
    """The gate kernel's eight per-tile features (torch, float64 inputs)."""
    import torch

    H, W = depth.shape
    th, tw = (H + TILE - 1) // TILE, (W + TILE - 1) // TILE

    def ts(x):
        xp = torch.nn.functional.pad(x[None, None], (0, tw * TILE - W, 0, th * TILE - H))
        return torch.nn.functional.avg_pool2d(xp, TILE, divisor_override=1).flatten()

    n = ts(torch.ones_like(depth))
    e = 1e-8
    f0 = torch.log(ts(torch.exp(var)) / n + e)
    d = (bm_fin[..., :3].double() - nn_fin[..., :3].double()) / 255.0
    f1 = torch.log(ts((d * d).mean(-1)) / n + e)
    f2 = torch.log(ts(spp) / n + e)
    lum = 0.2126 * noisy[..., 0] + 0.7152 * noisy[..., 1] + 0.0722 * noisy[..., 2]
    ll = torch.log1p(torch.clamp(lum, min=0))
    m1, m2 = ts(ll) / n, ts(ll * ll) / n
    f3 = torch.log(torch.clamp(m2 - m1 * m1, min=0) + e)
    ld = torch.log(torch.clamp(depth, 1e-3, 1e4))
    gx = torch.nn.functional.pad((ld[:, 1:] - ld[:, :-1]).abs(), (0, 1))
    gy = torch.nn.functional.pad((ld[1:] - ld[:-1]).abs(), (0, 0, 0, 1))
    f4 = torch.log(ts(gx + gy) / n + e)
    t_, p_ = nrm[..., 0], nrm[..., 1]
    mx, my, mz = ts(torch.sin(t_) * torch.cos(p_)) / n, ts(torch.sin(t_) * torch.sin(p_)) / n, ts(torch.cos(t_)) / n
    f5 = torch.log(torch.clamp(1 - torch.sqrt(mx * mx + my * my + mz * mz), min=0) + e)
    f6 = torch.log(ts(lum) / n + e)
    f7 = torch.log(ts(alb8[..., :3].double().mean(-1) / 255.0) / n + e)
    return torch.stack([f0, f1, f2, f3, f4, f5, f6, f7], 1), n


def collect(out: str, seeds=(21, 22, 23, 24, 25, 26), frames=(15, 30, 46), ref_spp=2048, width=1920, height=1080,
            weights=None):
    """Renders the training frames on cuda:0 and saves features and errors to `out` (.npz); `weights`: the
    network's .npz (default: the packaged weights)."""
    import sys

    import torch

    root = Path(__file__).resolve().parents[1]
    sys.path.insert(0, str(root))
    import bench  # the benchmark's orbit

    import vulkanpbrt_gb300 as vp
    from vulkanpbrt_gb300 import scene as S

    W, H = width, height
    stream = torch.cuda.current_stream()
    rec = {k: [] for k in ("err_nn", "err_b75", "err_b50", "err_b25", "err_bm", "f", "scene", "frame")}
    for si, seed in enumerate(seeds):
        sc = S.instanced_field(seed=seed)
        sh = vp.SceneHandle(sc)
        g = vp.GBuffer(W, H)
        illu = vp.IlluminationBufferDemodulatedFloat(W, H)
        pipe = vp.PBRTPipeline(sh, g, illu, True, max_recursion_depth=8, min_recursion_depth=3)
        accu = vp.Accumulator(g, illu, separate_matrices=True)
        acc_illu, abuf = accu.accumulated_illumination, accu.accumulation_buffer
        bm = vp.BMFR(W, H, 32, 32, g, acc_illu, abuf, 256)
        nd = vp.NeuralDenoiser(W, H, g, acc_illu, weights=weights, fallback=bm, threshold=1e30, tile=TILE,
                               acc_buffer=abuf, gate_model=None)  # the network alone
        pc = vp.PushConstants()
        prev = bench.orbit(sc, W, H, 0)
        hs = vp._abi.stream_handle(stream)
        for f in range(max(frames) + 1):
            cam = bench.orbit(sc, W, H, f)
            pc.set(view_inverse=cam.inv_view, proj_inverse=cam.inv_proj, prev_view=prev.view,
                   frame_number=f + 1000 * seed)
            accu.set_camera_matrices(f, vp.CameraMatrices(cam.view, cam.inv_view, cam.proj, cam.inv_proj),
                                     vp.CameraMatrices(prev.view, prev.inv_view))
            pipe.trace(pc, stream)
            vp.lib().pbrt_accumulator_dispatch(accu.ptr, hs)
            bm.dispatch(pc, stream)
            nd.dispatch(pc, stream)
            vp.lib().pbrt_accumulation_buffer_copy_to_back_images(abuf.ptr, g.ptr, acc_illu.ptr, hs)
            prev = cam
            if f not in frames:
                continue
            torch.cuda.synchronize()
            fn = pc.value.frame_number
            albedo = g.albedo.tensor()[..., :3].double() / 255.0
            nn_o = nd.denoised.tensor()[..., :3].double().clone()
            bm_o = bm.denoised.tensor()[(fn & 1) ^ 1][..., :3].double().clone()
            feats, npx = tile_features(nd.variance.tensor()[..., 0][:H, :W].double(),
                                       nd.get_final_descriptor_image().tensor(), bm.get_final_descriptor_image().tensor(),
                                       abuf.spp.tensor()[..., 0].double(),
                                       acc_illu.illumination_images[0].tensor()[..., :3].double(),
                                       g.depth.tensor()[..., 0].double(), g.normal.tensor().double(), g.albedo.tensor())
            img = illu.illumination_images[0].tensor()
            ref = torch.zeros_like(nn_o)
            for s_ in range(ref_spp):
                pc.set(frame_number=(1 << 24) + s_)
                pipe.trace(pc, stream)
                ref += img[..., :3]
            torch.cuda.synchronize()
            ref /= ref_spp
            pc.set(frame_number=fn)
            r = albedo * ref

            def err(v):
                e = (((albedo * v - r) ** 2) / (r * r + 0.01)).mean(-1)
                th, tw = (H + TILE - 1) // TILE, (W + TILE - 1) // TILE
                ep = torch.nn.functional.pad(e[None, None], (0, tw * TILE - W, 0, th * TILE - H))
                return torch.nn.functional.avg_pool2d(ep, TILE, divisor_override=1).flatten() / npx

            rec["err_nn"].append(err(nn_o).cpu().numpy())
            rec["err_bm"].append(err(bm_o).cpu().numpy())
            for a_, k_ in ((0.75, "err_b75"), (0.5, "err_b50"), (0.25, "err_b25")):
                rec[k_].append(err(a_ * nn_o + (1 - a_) * bm_o).cpu().numpy())
            rec["f"].append(feats.cpu().numpy())
            rec["scene"].append(np.full(feats.shape[0], si))
            rec["frame"].append(np.full(feats.shape[0], f))
            print(f"seed {seed} frame {f}: network {rec['err_nn'][-1].mean():.5f} BMFR {rec['err_bm'][-1].mean():.5f}",
                  flush=True)
    np.savez(out, **{k: np.concatenate(v) for k, v in rec.items()}, seeds=np.array(seeds), ref_spp=ref_spp)


BLENDS = ("err_b75", "err_b50", "err_b25", "err_bm")  # alpha 0.75, 0.5, 0.25, 0 on the network


def fit(data: str, out: str, lams=(0.1, 1.0, 10.0)):
    d = np.load(data)
    X, scene = d["f"], d["scene"]
    E = np.stack([d["err_nn"]] + [d[k] for k in BLENDS], 1)
    ok = np.isfinite(X).all(1) & np.isfinite(E).all(1)
    X, E, scene = X[ok], E[ok], scene[ok]

    def train(sel, lam):
        mu, sd = X[sel].mean(0), X[sel].std(0) + 1e-9
        A = np.concatenate([(X[sel] - mu) / sd, np.ones((int(sel.sum()), 1))], 1)
        coef = []
        for k in range(1, 5):
            b = np.linalg.solve(A.T @ A + lam * np.eye(9), A.T @ (E[sel, k] - E[sel, 0]))
            coef.append(np.concatenate([b[:8] / sd, [b[8] - (b[:8] * mu / sd).sum()]]))
        return np.stack(coef)

    def choose(C, Xs):
        pred = np.concatenate([np.zeros((len(Xs), 1)), Xs @ C[:, :8].T + C[:, 8]], 1)
        return pred.argmin(1)

    best = None
    for lam in lams:
        tot, picks = np.zeros(2), np.zeros(5)
        for s in np.unique(scene):
            te = scene == s
            ch = choose(train(scene != s, lam), X[te])
            tot += [E[te][np.arange(int(te.sum())), ch].sum(), E[te, 0].sum()]
            picks += np.bincount(ch, minlength=5)
        res = tot / len(E)
        print(f"ridge {lam}: leave-one-scene-out relMSE gated {res[0]:.5f}, network {res[1]:.5f}, "
              f"alpha 1/.75/.5/.25/0 on {np.round(picks / picks.sum(), 3).tolist()} of the tiles")
        if best is None or res[0] < best[1][0]:
            best = (lam, res, picks / picks.sum())
    lam, res, picks = best
    C = train(np.ones(len(E), bool), lam)
    doc = {"coef": [float(v) for v in C.reshape(-1)], "features": FEATURES,
           "data": "held-out seeded instanced fields (never the benchmark's seed 0), 1920x1080, depth 8 with Russian "
                   "roulette after bounce 3, the benchmark's 16-frame orbit with accumulation, BMFR 32x32 and the "
                   "network; 2040 tiles of 32x32 a frame; per-tile relMSE against a many-sample render of the same "
                   "camera, remodulated by the G-buffer albedo",
           "blends": "rows: alpha 0.75, 0.5, 0.25, 0 on the network (1 - alpha on BMFR); 8 weights, then the bias",
           "fit": {"tiles": int(len(E)), "scenes": int(len(np.unique(scene))), "ridge": lam,
                   "seeds": [int(v) for v in d["seeds"]] if "seeds" in d.files else None,
                   "reference_spp": int(d["ref_spp"]) if "ref_spp" in d.files else None,
                   "leave_one_scene_out": {"gated": float(res[0]), "network": float(res[1]),
                                           "alpha_share": [float(v) for v in picks]},
                   "per_tile_best_of_the_five": float(E.min(1).mean()), "bmfr": float(E[:, 4].mean())}}
    Path(out).write_text(json.dumps(doc, indent=1))
    return doc


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    sub = ap.add_subparsers(dest="cmd", required=True)
    c = sub.add_parser("collect")
    c.add_argument("--out", default="gate_data.npz")
    c.add_argument("--ref-spp", type=int, default=2048)
    c.add_argument("--weights", default=None, help="the network's .npz (default: the packaged weights)")
    f = sub.add_parser("fit")
    f.add_argument("data")
    f.add_argument("--out", default=str(Path(__file__).resolve().parent / "weights" / "gate.json"))
    a = ap.parse_args(argv)
    if a.cmd == "collect":
        collect(a.out, ref_spp=a.ref_spp, weights=a.weights)
    else:
        print(json.dumps(fit(a.data, a.out), indent=1))


if __name__ == "__main__":
    main()
