#!/usr/bin/env python
"""Benchmark of the per-frame path: 1080p denoised frames/s and Grays/s.

A step is one frame of the reference's per-frame command list
(source/VulkanPBRT.cpp:397-505): path-trace 1 spp (PBRTPipeline), temporal
accumulation (Accumulator), BMFR denoise, copy-to-back -- on the full-size
workload: 1920x1080, max depth 8 with Russian roulette after bounce 3, a
seeded ~1M-triangle scene of 2000 instanced displaced icospheres and boxes
(log-uniform scale .05-2) on a ground plane, per-mesh 1024^2 RGBA8
value-noise textures, 5% alpha-masked meshes, 8 point lights + 1 area light,
camera on a 16-frame orbit. Synthetic, seeded data stands in for the scenes
the reference loads (no dataset is available).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the reference algorithm's CPU implementation (the
project's C++ restatement; the reference's own shaders cannot run without a
Vulkan stack) on this host's cores, on a bounded sample of the same frame.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "1080p denoised fps and Grays/s: neural vs BMFR at equal relMSE to 4096 spp"
NODE_BYTES, TRI_BYTES = 80, 48  # Node8 and the 3-float4 triangle record


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=32)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--max-depth", type=int, default=8)
    ap.add_argument("--min-depth", type=int, default=3)
    ap.add_argument("--instances", type=int, default=2000)
    ap.add_argument("--texture-size", type=int, default=1024)
    ap.add_argument("--denoiser", default="neural", choices=["neural", "bmfr", "bfr"],
                    help="neural: U-Net with BMFR as variance-gate fallback (BMFR runs every frame)")
    ap.add_argument("--gate", default="learned", choices=["learned", "threshold"],
                    help="neural path: the learned tile gate (weights/gate.json) or the threshold rule")
    ap.add_argument("--gate-threshold", type=float, default=0.05,
                    help="neural path, threshold rule: tiles whose predicted relative squared error exceeds this "
                         "show BMFR")
    ap.add_argument("--weights", default=None, help="neural path: .npz of trained parameters (default: packaged)")
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-request batch measured after the frames")
    ap.add_argument("--ref-spp", type=int, default=4096, help="samples of the relMSE reference render (0: skip)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--sort-rays", action="store_true", help="sort extension / shadow rays before traversal")
    ap.add_argument("--separate-shadow", action="store_true",
                    help="trace shadow rays in their own launch (default: merged into the next bounce's launch)")
    ap.add_argument("--workload", default="frame1080p",
                    choices=["frame1080p", "batch64", "unet_layers", "full", "bvh_build"],
                    help="batch64: 64 uneven render requests in one graph launch; unet_layers: per-convolution "
                         "times of the U-Net; full: 4K 4 spp frames of a 4M-triangle scene (FP8 network, gate, "
                         "BMFR with the FP64 re-solve) beside 16 concurrent 1080p requests; bvh_build: host and "
                         "device BVH builds side by side (none of these is the headline line)")
    ap.add_argument("--bvh", default="fast_trace", choices=["fast_trace", "fast_build"],
                    help="BVH build of the workload's scenes: binned SAH on the host (fast_trace) or the linear "
                         "BVH built on the device (fast_build)")
    ap.add_argument("--frames", type=int, default=60, help="full: frames of the camera path")
    ap.add_argument("--relmse-frames", default="59", help="full: comma-separated frames whose relMSE is measured")
    ap.add_argument("--full-ref-spp", type=int, default=1024, help="full: samples of each 4K relMSE reference")
    ap.add_argument("--layers", default="", help="unet_layers: comma-separated layer names (default: all 18)")
    ap.add_argument("--kernels", default="bf16_tcgen05,bf16_mma,fp8_tcgen05,fp8_mma",
                    help="unet_layers: comma-separated subset of bf16_tcgen05,bf16_mma,fp8_tcgen05,fp8_mma")
    ap.add_argument("--reps", type=int, default=20, help="unet_layers: timed launches per layer and kernel")
    return ap.parse_args()


def max_over_ranks(ms: float, world: int, device=None) -> float:
    """The job's time for a timed region: the slowest rank's (all ranks call this)."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist

    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(world: int, steps: int, total_ms: float) -> float:
    """Whole-job frames per second: every rank renders `steps` frames (weak scaling)."""
    return world * steps / (total_ms / 1e3)


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def workload(args, seed_offset=0):
    from vulkanpbrt_gb300 import scene as S

    return S.instanced_field(seed=seed_offset, instances=args.instances, texture_size=args.texture_size)


def orbit(sc, W, H, f, frames=16):
    from vulkanpbrt_gb300.camera import Camera

    eye0 = np.array(sc.camera_eye, np.float64)
    c = np.array(sc.camera_center, np.float64)
    r = math.hypot(eye0[0] - c[0], eye0[1] - c[1])
    a0 = math.atan2(eye0[1] - c[1], eye0[0] - c[0])
    a = a0 + 2 * math.pi * (f % frames) / frames / 16.0  # a slow orbit: 1/16 turn over 16 frames
    eye = (c[0] + r * math.cos(a), c[1] + r * math.sin(a), eye0[2])
    return Camera(eye, sc.camera_center, aspect=W / H)


class ClockSampler:
    """nvidia-smi SM clocks and throttle reasons while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if len(r) > 4 + i and r[4 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_counters(kernel: str) -> dict:
    """Per-launch ncu figures of `kernel` from the committed summary (DRAM and
    L2 bytes, issue-slot use, lanes per instruction), if any."""
    p = ROOT / "profiles" / "ncu_traffic.json"
    if p.exists():
        d = json.loads(p.read_text()).get(kernel)
        if isinstance(d, dict):
            return d
    return {}


# ---------------------------------------------------------------------------
class CpuFrames:
    """The reference frame (source/VulkanPBRT.cpp:397-445: trace, accumulate,
    BMFR 32x32, copy to the back images) run by the CPU restatement at full
    resolution, FP32, on all host threads, over the same orbit as the GPU arm.
    Only the oracle's library is loaded: the scene comes from the numpy scene
    generator, and the orbit cameras from plain numpy."""

    def __init__(self, args, sc):
        from oracle import oracle as O

        self.O, self.args, self.sc = O, args, sc
        self.W, self.H = args.width, args.height
        self.os = O.OracleScene(sc)
        cam = orbit(sc, 8, 8, 0)
        from vulkanpbrt_gb300.camera import col_major

        self.col_major = col_major
        # builds and caches the oracle's BVH (not timed, like the GPU arm's scene build)
        O.render(self.os, 8, 8, col_major(cam.inv_view), col_major(cam.inv_proj), min_depth=args.min_depth,
                 max_depth=args.max_depth)
        W, H = self.W, self.H
        self.prev_depth = np.zeros((H, W), np.float32)
        self.prev_spp = np.zeros((H, W), np.uint8)
        self.prev_out = np.zeros((H, W, 4), np.float16)
        self.denoised = np.zeros((2, H, W, 4), np.float16)
        self.prev_cam = orbit(sc, W, H, 0)
        self.rays = 0.0
        self.trace_s = 0.0

    def frame(self, f: int) -> float:
        """Renders frame f; returns its wall time in seconds."""
        O, a, cm = self.O, self.args, self.col_major
        cam, prev = orbit(self.sc, self.W, self.H, f), self.prev_cam
        t0 = time.perf_counter()
        r = O.render(self.os, self.W, self.H, cm(cam.inv_view), cm(cam.inv_proj), frame=f, min_depth=a.min_depth,
                     max_depth=a.max_depth)
        t1 = time.perf_counter()
        prev_origin = np.linalg.inv(prev.view.astype(np.float64))[:3, 3].tolist() + [1.0]
        motion, spp, illum = O.accumulate(f, 1, cm(cam.inv_proj), cm(cam.inv_view), cm(prev.view), prev_origin,
                                          r["illum"], r["depth"], self.prev_depth, self.prev_spp, self.prev_out)
        O.bmfr(32, 256, f, 0, cm(cam.inv_view), cm(cam.inv_proj), r["depth"], r["normal"], r["albedo"], illum, motion,
               spp, self.denoised)
        t2 = time.perf_counter()
        # copy to the back images
        self.prev_depth, self.prev_spp, self.prev_out, self.prev_cam = r["depth"], spp, illum, cam
        self.rays += float(r["rays"].sum())
        self.trace_s += t1 - t0
        return t2 - t0


def cpu_baseline(args, sc, frames=3):
    """The CPU restatement on a bounded sample of the workload: `frames` full
    1920x1080 frames of the orbit (after one untimed frame), each traced,
    accumulated and BMFR-denoised exactly as the GPU arm's frame."""
    cf = CpuFrames(args, sc)
    cf.frame(0)
    cf.rays, cf.trace_s = 0.0, 0.0
    t = [cf.frame(1 + i) for i in range(frames)]
    per = float(np.mean(t))
    return {
        "value": 1.0 / per,
        "unit": "fps",
        "cores": os.cpu_count(),
        "kind": "port",
        "sample": f"{frames} full {args.width}x{args.height} frames of the same scene and orbit after one untimed "
                  f"frame: trace + accumulate + BMFR 32x32, FP32, all host threads (no extrapolation)",
        "grays_per_s": cf.rays / cf.trace_s / 1e9,
        "ms_per_frame": per * 1e3,
    }


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    sc = workload(args)
    cf = CpuFrames(args, sc)
    for f in range(args.warmup):
        cf.frame(f)
    cf.rays, cf.trace_s = 0.0, 0.0
    t0 = time.perf_counter()
    for i in range(args.steps):
        cf.frame(args.warmup + i)
    total = time.perf_counter() - t0
    per = total / args.steps
    line = {
        "metric": METRIC, "value": 1.0 / per, "unit": "fps", "impl": "reference", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": per * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
        "config": {"workload": "1080p 1spp depth8 RR>=3, 1M-tri instanced scene, 16-frame orbit: accumulate + BMFR "
                               "32x32 (the frame of the GPU arm's bmfr_path; the reference has no learned denoiser)",
                   "width": args.width, "height": args.height, "max_depth": args.max_depth,
                   "min_depth": args.min_depth, "instances": args.instances, "texture_size": args.texture_size,
                   "frames": f"{args.steps} full frames timed after {args.warmup} untimed (no sampling, "
                             f"no extrapolation)"},
        "cpu_baseline": {"value": 1.0 / per, "unit": "fps", "cores": os.cpu_count(), "kind": "port",
                         "sample": f"{args.steps} full {args.width}x{args.height} frames of the orbit, trace + "
                                   f"accumulate + BMFR 32x32, FP32, all host threads"},
        "e2e": {"value": 1.0 / per, "unit": "fps", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "grays_per_s": cf.rays / cf.trace_s / 1e9,
        "trace_ms_per_frame": cf.trace_s / args.steps * 1e3,
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# kernels of one neural dispatch: features, 2 radiance poolings, 4 encoder
# poolings, 18 convolutions, 3 heads, the gate and the compose
NEURAL_LAUNCHES = 1 + 2 + 4 + 18 + 3 + 1 + 1


def relmse_eval(args, vp, pipe, g, illu, bmfr, neural, pc, cams, stream, dev):
    """relMSE of the last frame's outputs against an args.ref_spp-sample render
    of the same camera (mean of the demodulated illumination; every image is
    remodulated by the G-buffer albedo first): the 1-spp input, BMFR (after
    the orbit's temporal accumulation) and the network (alone, and as shown:
    gated tiles from BMFR)."""
    import torch

    f = pc.value.frame_number
    img = illu.illumination_images[0].tensor()
    noisy = img[..., :3].double().clone()
    albedo = g.albedo.tensor()[..., :3].double() / 255.0
    out = {"reference_spp": args.ref_spp, "frame": int(f)}
    den = {"input_1spp": noisy}
    if bmfr is not None:
        den["bmfr"] = bmfr.denoised.tensor()[(f & 1) ^ 1][..., :3].double().clone()
    if neural is not None:
        coef = getattr(neural, "gate_coef", None)
        if coef is not None and bmfr is not None:
            # the learned gate: `denoised` is what the module shows (per-tile blends of the network and BMFR);
            # the network alone comes from one more dispatch with the gate off
            m = neural.fallback_mask.tensor()[..., 0].long()
            den["neural_gated"] = neural.denoised.tensor()[..., :3].double().clone()
            out["fallback_tiles"] = int((m > 0).sum().item())
            out["tiles"] = int(m.numel())
            out["gate_tiles_by_alpha"] = dict(zip(("1", "0.75", "0.5", "0.25", "0"),
                                                  torch.bincount(m.flatten(), minlength=5).tolist()))
            neural.set_gate_model(None)
            neural.set_fallback(bmfr, threshold=1e30, tile=neural.tile)
            neural.dispatch(pc, stream)
            torch.cuda.synchronize()
            den["neural"] = neural.denoised.tensor()[..., :3].double().clone()
            neural.set_precision(8)  # calibrated during the FP8 timing; the network alone
            neural.dispatch(pc, stream)
            torch.cuda.synchronize()
            den["neural_fp8"] = neural.denoised.tensor()[..., :3].double().clone()
            neural.set_precision(16)
            neural.set_fallback(bmfr, threshold=args.gate_threshold, tile=neural.tile)
            neural.set_gate_model(coef)
        else:
            nn_out = neural.denoised.tensor()[..., :3].double().clone()
            den["neural"] = nn_out
            if neural.fallback_mask is not None and bmfr is not None:
                m = neural.fallback_mask.tensor()[..., 0].bool()
                px = m.repeat_interleave(neural.tile, 0).repeat_interleave(neural.tile, 1)[:g.height, :g.width]
                den["neural_gated"] = torch.where(px[..., None], den["bmfr"], nn_out)
                out["fallback_tiles"] = int(m.sum().item())
                out["tiles"] = int(m.numel())
            neural.set_precision(8)  # calibrated during the FP8 timing
            neural.dispatch(pc, stream)
            torch.cuda.synchronize()
            den["neural_fp8"] = neural.denoised.tensor()[..., :3].double().clone()
            neural.set_precision(16)
    torch.cuda.synchronize()
    ref = torch.zeros_like(noisy)
    t0 = time.perf_counter()
    base = 1 << 24
    for s_ in range(args.ref_spp):
        pc.set(frame_number=base + s_)
        pipe.trace(pc, stream)
        ref += img[..., :3]
    torch.cuda.synchronize()
    out["reference_s"] = time.perf_counter() - t0
    ref /= args.ref_spp
    r = albedo * ref
    err = {}
    for k, v in den.items():
        e = ((albedo * v - r) ** 2) / (r * r + 0.01)
        err[k] = e.mean(-1)
        out[k] = float(e.mean().item())
    if neural is not None and bmfr is not None:
        out["gate"] = gate_analysis(neural, err["neural"], err["bmfr"], g.width, g.height)
    return out


def gate_analysis(neural, err_nn, err_bmfr, W, H, tile=32):
    """How well the error head ranks 32x32 tiles: per tile, the predicted
    relative squared error (mean exp of the head) against the measured
    relMSE of the network and of BMFR; the composite relMSE if tiles whose
    prediction exceeds each of several quantile thresholds showed BMFR."""
    import torch

    var = neural.variance.tensor()[..., 0][:H, :W].double().exp()
    th, tw = (H + tile - 1) // tile, (W + tile - 1) // tile
    ph, pw = th * tile - H, tw * tile - W

    def tiles(x):
        x = torch.nn.functional.pad(x[None, None], (0, pw, 0, ph))
        cnt = torch.nn.functional.pad(torch.ones_like(x[0, 0])[:H, :W][None, None], (0, pw, 0, ph))
        s = torch.nn.functional.avg_pool2d(x, tile, divisor_override=1)[0, 0]
        n = torch.nn.functional.avg_pool2d(cnt, tile, divisor_override=1)[0, 0]
        return (s / n).flatten(), n.flatten()

    pred, n = tiles(var)
    e_nn, _ = tiles(err_nn)
    e_bm, _ = tiles(err_bmfr)
    total = float(n.sum())
    res = {"tiles": int(pred.numel()),
           "corr_pred_vs_neural_err": float(torch.corrcoef(torch.stack([pred.log(), (e_nn + 1e-6).log()]))[0, 1]),
           "best_possible": float(((torch.minimum(e_nn, e_bm) * n).sum() / total).item()),
           "bmfr_better_tiles": int((e_bm < e_nn).sum().item())}
    sweep = {}
    for q in (0.5, 0.75, 0.9, 0.95, 0.99):
        thr = float(torch.quantile(pred, q).item())
        comp = torch.where(pred > thr, e_bm, e_nn)
        sweep[f"q{q}"] = {"threshold": thr, "relmse": float(((comp * n).sum() / total).item())}
    res["sweep"] = sweep
    return res


def run_gb300(args):
    import torch

    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from vulkanpbrt_gb300 import build as B

    B.build()
    import vulkanpbrt_gb300 as vp

    W, H = args.width, args.height
    sc = workload(args, seed_offset=0)  # every rank renders its own request stream of the same scene
    sh = vp.SceneHandle(sc, build=args.bvh)
    info = sh.info()
    g = vp.GBuffer(W, H)
    illu = vp.IlluminationBufferDemodulatedFloat(W, H)
    pipe = vp.PBRTPipeline(sh, g, illu, True, max_recursion_depth=args.max_depth, min_recursion_depth=args.min_depth)
    pipe.set_schedule(sort_rays=args.sort_rays, merge_shadow=not args.separate_shadow)
    accu = vp.Accumulator(g, illu, separate_matrices=True)
    acc_illu = accu.accumulated_illumination
    abuf = accu.accumulation_buffer
    if args.denoiser == "bfr":
        den = vp.BFR(W, H, 16, 16, g, acc_illu, abuf)
        bmfr = None
    else:
        bmfr = den = vp.BMFR(W, H, 32, 32, g, acc_illu, abuf, 256)
    neural = None
    if args.denoiser == "neural":
        # the network reads what BMFR reads: the accumulator's output and its sample counts
        neural = vp.NeuralDenoiser(W, H, g, acc_illu, weights=args.weights, fallback=bmfr,
                                   threshold=args.gate_threshold, tile=32, acc_buffer=abuf,
                                   gate_model="default" if args.gate == "learned" else None)
    pc = vp.PushConstants()
    stream = torch.cuda.current_stream(dev)
    cams = [orbit(sc, W, H, f) for f in range(16)]
    state = {"prev": cams[0]}

    def frame(f, use_neural=True):
        cam = cams[f % 16]
        prev = state["prev"]
        pc.set(view_inverse=cam.inv_view, proj_inverse=cam.inv_proj, prev_view=prev.view, frame_number=f)
        accu.set_camera_matrices(f, vp.CameraMatrices(cam.view, cam.inv_view, cam.proj, cam.inv_proj),
                                 vp.CameraMatrices(prev.view, prev.inv_view))
        s = stream
        pipe.trace(pc, s)
        vp.lib().pbrt_accumulator_dispatch(accu.ptr, vp._abi.stream_handle(s))
        den.dispatch(pc, s)
        if neural is not None and use_neural:
            neural.dispatch(pc, s)
        vp.lib().pbrt_accumulation_buffer_copy_to_back_images(abuf.ptr, g.ptr, acc_illu.ptr, vp._abi.stream_handle(s))
        state["prev"] = cam

    # warm-up (also builds the frame graph)
    for f in range(args.warmup):
        frame(f)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    st0 = pipe.stats(stream)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    tev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        ev[0].record(stream)
        for i in range(args.steps):
            f = args.warmup + i
            cam = cams[f % 16]
            prev = state["prev"]
            pc.set(view_inverse=cam.inv_view, proj_inverse=cam.inv_proj, prev_view=prev.view, frame_number=f)
            accu.set_camera_matrices(f, vp.CameraMatrices(cam.view, cam.inv_view, cam.proj, cam.inv_proj),
                                     vp.CameraMatrices(prev.view, prev.inv_view))
            tev[i][0].record(stream)
            pipe.trace(pc, stream)
            tev[i][1].record(stream)
            vp.lib().pbrt_accumulator_dispatch(accu.ptr, vp._abi.stream_handle(stream))
            den.dispatch(pc, stream)
            if neural is not None:
                neural.dispatch(pc, stream)
            vp.lib().pbrt_accumulation_buffer_copy_to_back_images(abuf.ptr, g.ptr, acc_illu.ptr,
                                                                  vp._abi.stream_handle(stream))
            state["prev"] = cam
        ev[1].record(stream)
        torch.cuda.synchronize()
    total_ms = ev[0].elapsed_time(ev[1])
    trace_ms = sum(a.elapsed_time(b) for a, b in tev)
    st1 = pipe.stats(stream)
    rays = (st1.primary_rays - st0.primary_rays) + (st1.extension_rays - st0.extension_rays) + \
        (st1.shadow_rays - st0.shadow_rays)
    total_ms = max_over_ranks(total_ms, world, dev)

    # ---- the same frames with FP8 (e4m3) convolutions, calibrated on the current frame
    fp8_ms, fp8_layers = None, None
    if neural is not None:
        neural.calibrate(stream)
        neural.set_precision(8)
        for f in range(2):
            frame(args.warmup + args.steps + f)
        torch.cuda.synchronize()
        ev[0].record(stream)
        for i in range(args.steps):
            frame(args.warmup + args.steps + 2 + i)
        ev[1].record(stream)
        torch.cuda.synchronize()
        fp8_ms = ev[0].elapsed_time(ev[1]) / args.steps
        fp8_neural_ms = _stage_ms(lambda: neural.dispatch(pc, stream), stream)
        fp8_layers = neural.fp8_layers()
        neural.set_precision(16)

    # ---- the BMFR-only path (no network) over the same frames, for the neural-vs-BMFR comparison
    bmfr_ms = None
    if neural is not None:
        for f in range(2):
            frame(args.warmup + args.steps + f, use_neural=False)
        torch.cuda.synchronize()
        ev[0].record(stream)
        for i in range(args.steps):
            frame(args.warmup + args.steps + 2 + i, use_neural=False)
        ev[1].record(stream)
        torch.cuda.synchronize()
        bmfr_ms = ev[0].elapsed_time(ev[1]) / args.steps

    # ---- end to end through the public API: frame + read-back of the final image every step
    final = (neural if neural is not None else den).get_final_descriptor_image().tensor()
    host = torch.empty(final.shape, dtype=final.dtype, pin_memory=True)
    for f in range(2):
        frame(args.warmup + args.steps + f)
        host.copy_(final, non_blocking=True)
    torch.cuda.synchronize()
    e2e_steps = args.steps
    t0 = time.perf_counter()
    for i in range(e2e_steps):
        frame(args.warmup + args.steps + 2 + i)
        host.copy_(final, non_blocking=True)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    # per-step host inputs: the push constants and two CameraMatrices, passed by value (kernel arguments)
    h2d = C.sizeof(vp._abi.PbrtPushConstants) + 2 * C.sizeof(vp._abi.PbrtCameraMatrices)
    d2h = final.numel() * final.element_size()

    # ---- per-kernel profile of one frame (roofline of the dominant kernel)
    prof = pipe.profile(pc, stream)
    stages = {"trace_closest": prof.trace_closest_ms, "shade": prof.shade_ms, "trace_shadow": prof.trace_shadow_ms,
              "raygen": prof.raygen_ms, "finalize": prof.finalize_ms}
    # denoiser / accumulator kernels timed alone
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    vp.lib().pbrt_accumulator_dispatch(accu.ptr, vp._abi.stream_handle(stream))
    e1.record(stream)
    torch.cuda.synchronize()
    stages["accumulate"] = e0.elapsed_time(e1)
    e0.record(stream)
    den.dispatch(pc, stream)
    e1.record(stream)
    torch.cuda.synchronize()
    stages["bfr" if args.denoiser == "bfr" else "bmfr"] = e0.elapsed_time(e1)
    if neural is not None:  # the network's graph launch, mean of 10 after the frames above
        stages["neural"] = _stage_ms(lambda: neural.dispatch(pc, stream), stream)
        stages["neural_fp8"] = fp8_neural_ms
    quality = None
    if args.ref_spp > 0 and rank == 0:
        quality = relmse_eval(args, vp, pipe, g, illu, bmfr, neural, pc, cams, stream, dev)
    # traversal launches trace closest-hit and shadow rays together (bounce k's
    # closest-hit rays with bounce k-1's shadow rays), so the roofline covers both
    closest_bytes = (prof.closest_nodes + prof.shadow_nodes) * NODE_BYTES + \
        (prof.closest_tris + prof.shadow_tris) * TRI_BYTES
    trav_ms = prof.trace_closest_ms + prof.trace_shadow_ms
    launches = max(1, prof.closest_launches + 1)
    per_launch_s = trav_ms / 1e3 / launches
    achieved = closest_bytes / launches / per_launch_s / 1e9
    peak, peak_kind = peaks()
    counters = profile_counters("k_traverse")
    traffic = counters.get("dram_bytes_per_launch")
    dominant = max(stages, key=stages.get)
    if rank == 0:
        steps = args.steps
        value = job_throughput(world, steps, total_ms)
        clocks = clk.summary()
        cpu = None
        if not args.no_cpu_baseline:
            try:
                cpu = cpu_baseline(args, sc)
            except Exception as e:  # the baseline must not sink the GPU line
                cpu = {"value": None, "unit": "fps", "cores": os.cpu_count(), "kind": "port", "sample": f"failed: {e}"}
        line = {
            "metric": METRIC,
            "value": value,
            "unit": "fps",
            "n_gpus": world,
            "steps": steps,
            "warmup": args.warmup,
            "ms_per_step": total_ms / steps,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32 tracer / bf16 network" if neural is not None else "f32",
            "data": "synthetic (seeded procedural scene; inputs larger than L2: 0.8 GB textures, 0.5 GB path state)",
            "config": {
                "workload": ("1080p 1spp depth8 RR>=3, 1M-tri instanced scene, 16-frame orbit: accumulate + BMFR 32x32"
                             + (" + kernel-predicting U-Net (BF16) with the learned per-tile BMFR fallback gate"
                                if neural is not None else "")),
                "width": W, "height": H, "max_depth": args.max_depth, "min_depth": args.min_depth,
                "triangles": int(info.triangle_count), "instances": int(info.instance_count),
                "lights": int(info.light_count), "texture_size": args.texture_size, "denoiser": args.denoiser, "gate": args.gate,
                "l2": "inputs larger than L2 (no flush)", "parallelism": f"replicas x{world}",
                "schedule": {"sort_rays": bool(args.sort_rays), "merge_shadow": not args.separate_shadow},
            },
            "grays_per_s": rays / (trace_ms / 1e3) / 1e9 * world,
            # the same queries over the traversal kernels' time alone (packet,
            # merged closest + shadow, last shadow launches of one profiled frame)
            "traversal_grays_per_s": (prof.closest_rays + prof.shadow_rays) / (trav_ms / 1e3) / 1e9 * world,
            "rays_per_frame": rays / steps,
            "trace_ms_per_frame": trace_ms / steps,
            "stage_ms": {k: round(v, 4) for k, v in stages.items()},
            "e2e": {"value": world * e2e_steps / e2e_s, "unit": "fps", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "roofline": {
                "kernel": "k_traverse (BVH8 traversal: closest-hit and shadow rays, merged launches)",
                "bound": "hbm",
                "achieved": achieved,
                "peak": peak,
                "unit": "GB/s",
                "frac": achieved / peak,
                "peak_source": peak_kind,
                "traffic": traffic,
                # the roof the traversal actually meets: instruction issue
                # (ncu, per launch of one frame's traversal); the BVH and most
                # triangle records stay in L2
                "issue_active_pct": counters.get("issue_active_pct"),
                "lanes_per_instruction": counters.get("lanes_per_instruction"),
                "l2_bytes_per_launch": counters.get("l2_bytes_per_launch"),
                "l2_pct_of_peak": counters.get("l2_pct_of_peak"),
                "counters_source": counters.get("source"),
                "bytes_per_ray": closest_bytes / max(1, prof.closest_rays + prof.shadow_rays),
                "nodes_per_ray": (prof.closest_nodes + prof.shadow_nodes) / max(1, prof.closest_rays + prof.shadow_rays),
                "tris_per_ray": (prof.closest_tris + prof.shadow_tris) / max(1, prof.closest_rays + prof.shadow_rays),
                "dominant_kernel": dominant,
            },
            "cpu_baseline": cpu,
            "clocks": clocks,
            "gpu_launches": steps * (3 + 5 * (args.max_depth + 1) + 1 + 2 + (NEURAL_LAUNCHES if neural else 0)),
            "bmfr_path": None if bmfr_ms is None else {"fps": world * 1e3 / bmfr_ms, "ms_per_step": bmfr_ms},
            "neural_fp8_path": None if fp8_ms is None else {"fps": world * 1e3 / fp8_ms, "ms_per_step": fp8_ms,
                                                            "e4m3_layers": [n for (n, *_), f in
                                                                            zip(_conv_table(), fp8_layers) if f]},
            "relmse": quality,
            "bvh": {"build": args.bvh, "nodes": int(info.bvh_nodes), "depth": int(info.bvh_depth),
                    "build_ms": info.build_ms},
        }
        if world == 1 and not args.no_batch:
            # the 64-request batch, measured here too (fixed tuning, 3 submits
            # after 1): BVH queries of requests of 10k-2M triangles each
            bl = batch64_measure(3, 1, tune=False, bvh=args.bvh)
            line["batch64"] = {k: bl[k] for k in ("ms_per_batch", "requests_per_s", "pixel_samples_per_s",
                                                  "grays_per_s", "tuning", "steps", "warmup")}
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


def batch_scene(rng, seed):
    """A Cornell-style box with icospheres, 10k-2M triangles (log-uniform)."""
    from vulkanpbrt_gb300 import scene as S

    tris = float(np.exp(rng.uniform(np.log(1e4), np.log(2e6))))
    if tris < 1e5:
        return S.cornell_spheres(seed=seed, spheres=max(1, int(tris / 1280)), subdiv=3)
    return S.cornell_spheres(seed=seed, spheres=max(1, int(tris / 20480)), subdiv=5)


# the autotuner's pick for the 64-request batch on a GB300 (python bench.py --workload batch64)
BATCH64_TUNING = dict(branches=16, trace_blocks_per_sm=4, shade_blocks_per_sm=8, order=1)


def run_batch(args):
    """64 independent requests (own scene of 10k-2M triangles, resolution
    log-uniform 256^2..1080p, 1/2/4/8/16 spp, depth 4-8, accumulator + BMFR
    each) in one graph launch; the autotuner picks the chain count and the
    tracer's launch shape."""
    print(json.dumps(batch64_measure(args.steps, args.warmup, tune=True, bvh=args.bvh)), flush=True)


def batch64_measure(steps, warmup, tune=True, bvh="fast_trace"):
    """The 64-request batch timed over `steps` submits after `warmup`; tune:
    run the autotuner first, else take BATCH64_TUNING; bvh: the scenes' BVH
    build. Returns the line."""
    import torch

    from vulkanpbrt_gb300 import build as B

    B.build()
    import vulkanpbrt_gb300 as vp
    from vulkanpbrt_gb300.camera import default_camera

    rng = np.random.default_rng(2024)
    reqs, keep, pixels_spp = [], [], 0
    t0 = time.perf_counter()
    for i in range(64):
        sc = batch_scene(rng, 5000 + i)
        sh = vp.SceneHandle(sc, build=bvh)
        side = float(np.exp(rng.uniform(np.log(256 * 256), np.log(1920 * 1080))))
        aspect = rng.uniform(1.0, 16 / 9)
        H = max(64, int(np.sqrt(side / aspect)) // 32 * 32)
        W = max(96, int(H * aspect) // 32 * 32)
        spp = int(rng.choice([1, 2, 4, 8, 16]))
        depth = int(rng.integers(4, 9))
        g = vp.GBuffer(W, H)
        illu = vp.IlluminationBufferDemodulatedFloat(W, H)
        pipe = vp.PBRTPipeline(sh, g, illu, True, max_recursion_depth=depth, min_recursion_depth=min(3, depth))
        acc = vp.Accumulator(g, illu, separate_matrices=True)
        bmfr = vp.BMFR(W, H, 32, 32, g, acc.accumulated_illumination, acc.accumulation_buffer, 256)
        cam = default_camera(W, H)
        pc = vp.PushConstants(view_inverse=cam.inv_view, proj_inverse=cam.inv_proj, prev_view=cam.view,
                              frame_number=1 + 100 * i)
        cm = vp.CameraMatrices(cam.view, cam.inv_view, cam.proj, cam.inv_proj)
        reqs.append(dict(pipe=pipe, pc=pc, spp=spp, acc=acc, bmfr=bmfr, cm=cm))
        keep.append((sc, sh, g, illu))
        pixels_spp += W * H * spp
    setup_s = time.perf_counter() - t0
    b = vp.Batch()
    for r in reqs:
        b.add(r["pipe"], r["pc"], spp=r["spp"], accumulator=r["acc"], bmfr=r["bmfr"], camera=r["cm"])
    stream = torch.cuda.current_stream()
    t1 = time.perf_counter()
    if tune:
        best, best_ms = b.autotune(repeats=3)
    else:
        b.set_tuning(**BATCH64_TUNING)
        best, best_ms = b.tuning, None
    tune_s = time.perf_counter() - t1
    for _ in range(warmup):
        b.submit()
    torch.cuda.synchronize()
    st0 = [r["pipe"].stats() for r in reqs]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        b.submit()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    st1 = [r["pipe"].stats() for r in reqs]
    rays = sum((a.primary_rays + a.extension_rays + a.shadow_rays) - (z.primary_rays + z.extension_rays + z.shadow_rays)
               for a, z in zip(st1, st0)) / steps
    return {"metric": "batched render requests (64 per graph launch)", "value": 1e3 / ms, "unit": "batches/s",
            "ms_per_batch": ms, "requests_per_s": 64e3 / ms, "pixel_samples_per_s": pixels_spp / ms * 1e3,
            "grays_per_s": rays / ms / 1e6, "rays_per_batch": rays, "tuning": best, "autotune_best_ms": best_ms,
            "setup_s": setup_s, "autotune_s": tune_s, "steps": steps, "warmup": warmup, "bvh": bvh,
            "config": {"requests": 64, "scenes": "own seeded scene each, 10k-2M tris (log-uniform)",
                       "resolution": "log-uniform 256^2..1080p", "spp": "uniform {1,2,4,8,16}", "depth": "4-8",
                       "denoiser": "accumulate + BMFR 32x32 per request"}}

def run_full(args):
    """The full chosen form: 3840x2160, 4 samples per pixel, max depth 8 with
    Russian roulette after bounce 3, a seeded ~4M-triangle instanced field
    with 32 lights, a 60-frame camera path; every frame traced 4 times (the
    samples averaged), accumulated, then BMFR 32x32 (FP64 re-solve on) and
    the kernel-predicting network in FP8 with the learned per-tile gate
    blending in BMFR; beside each
    4K frame, 16 independent 1080p requests (own seeded scene, 1 spp,
    accumulator + BMFR each) in one graph launch on a second stream. A step
    is one 4K frame plus one submission of the 16 requests. relMSE of the
    listed frames against an --full-ref-spp render of the same camera
    (remodulated by the G-buffer albedo), beside BMFR's."""
    import torch

    from vulkanpbrt_gb300 import build as B

    B.build()
    import vulkanpbrt_gb300 as vp
    from vulkanpbrt_gb300 import scene as S
    from vulkanpbrt_gb300.camera import default_camera

    W, H, spp = 3840, 2160, 4
    t0 = time.perf_counter()
    sc = S.instanced_field(seed=0, instances=8000, point_lights=30)
    sh = vp.SceneHandle(sc, build=args.bvh)
    info = sh.info()
    g = vp.GBuffer(W, H)
    illu = vp.IlluminationBufferDemodulatedFloat(W, H)
    pipe = vp.PBRTPipeline(sh, g, illu, True, max_recursion_depth=args.max_depth, min_recursion_depth=args.min_depth)
    accu = vp.Accumulator(g, illu, separate_matrices=True)
    abuf, acc_illu = accu.accumulation_buffer, accu.accumulated_illumination
    bmfr = vp.BMFR(W, H, 32, 32, g, acc_illu, abuf, 256, fp64_resolve=True)
    neural = vp.NeuralDenoiser(W, H, g, acc_illu, fallback=bmfr, threshold=args.gate_threshold, tile=32,
                               gate_model="default" if args.gate == "learned" else None,
                               acc_buffer=abuf)
    # the 16 concurrent 1080p requests
    rng = np.random.default_rng(77)
    batch, keep = vp.Batch(), []
    for i in range(16):
        rsc = batch_scene(rng, 9000 + i)
        rsh = vp.SceneHandle(rsc, build=args.bvh)
        rg, ri = vp.GBuffer(1920, 1080), vp.IlluminationBufferDemodulatedFloat(1920, 1080)
        rp = vp.PBRTPipeline(rsh, rg, ri, True, max_recursion_depth=args.max_depth, min_recursion_depth=args.min_depth)
        ra = vp.Accumulator(rg, ri, separate_matrices=True)
        rb = vp.BMFR(1920, 1080, 32, 32, rg, ra.accumulated_illumination, ra.accumulation_buffer, 256)
        cam = default_camera(1920, 1080)
        rpc = vp.PushConstants(view_inverse=cam.inv_view, proj_inverse=cam.inv_proj, prev_view=cam.view,
                               frame_number=1 + 37 * i)
        batch.add(rp, rpc, spp=1, accumulator=ra, bmfr=rb,
                  camera=vp.CameraMatrices(cam.view, cam.inv_view, cam.proj, cam.inv_proj))
        keep.append((rsc, rsh, rg, ri, rp, ra, rb, rpc))
    setup_s = time.perf_counter() - t0
    main_s = torch.cuda.current_stream()
    side_s = torch.cuda.Stream()
    pc = vp.PushConstants()
    pc_den = vp.PushConstants()  # the denoisers' frame number counts frames, not samples (BMFR's layer parity)
    cams = [orbit(sc, W, H, f, frames=args.frames) for f in range(args.frames)]
    state = {"prev": cams[0]}

    img = illu.illumination_images[0].tensor()
    sample_sum = torch.zeros_like(img)

    tr0, tr1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def frame(f, stream):
        # the frame's 4 samples are traced and averaged into the illumination
        # buffer, then accumulated once with the frame's own camera motion
        cam, prev = cams[f % args.frames], state["prev"]
        sh_ = vp._abi.stream_handle(stream)
        sample_sum.zero_()
        tr0.record(stream)
        for s_ in range(spp):
            pc.set(view_inverse=cam.inv_view, proj_inverse=cam.inv_proj, prev_view=prev.view,
                   frame_number=f * spp + s_)
            pipe.trace(pc, stream)
            sample_sum.add_(img)
        tr1.record(stream)
        img.copy_(sample_sum / spp)
        accu.set_camera_matrices(f, vp.CameraMatrices(cam.view, cam.inv_view, cam.proj, cam.inv_proj),
                                 vp.CameraMatrices(prev.view, prev.inv_view))
        vp.lib().pbrt_accumulator_dispatch(accu.ptr, sh_)
        pc_den.set(view_inverse=cam.inv_view, proj_inverse=cam.inv_proj, prev_view=prev.view, frame_number=f)
        bmfr.dispatch(pc_den, stream)
        neural.dispatch(pc_den, stream)
        vp.lib().pbrt_accumulation_buffer_copy_to_back_images(abuf.ptr, g.ptr, acc_illu.ptr, sh_)
        state["prev"] = cam

    # warm-up: graphs, autotune of the network's kernels, FP8 calibration
    frame(0, main_s)
    neural.calibrate(main_s)
    neural.set_precision(8)
    batch.submit(side_s)
    for f in range(1, 1 + max(1, args.warmup)):
        frame(f, main_s)
    torch.cuda.synchronize()
    measure = {int(x) for x in args.relmse_frames.split(",") if x}
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    req_pipes = [k[4] for k in keep]

    def queries(pipes):
        return sum(st.primary_rays + st.extension_rays + st.shadow_rays for st in (q.stats() for q in pipes))

    st0, req0 = queries([pipe]), queries(req_pipes)
    total_ms, trace_ms, ref_rays, per_frame, fp64_blocks, ratios, fallback = 0.0, 0.0, 0, [], [], [], []
    quality = []
    state["prev"] = cams[0]
    for f in range(args.frames):
        torch.cuda.synchronize()
        ev0.record(main_s)
        side_s.wait_event(ev0)
        batch.submit(side_s)
        frame(f, main_s)
        done = torch.cuda.Event()
        done.record(side_s)
        main_s.wait_event(done)
        ev1.record(main_s)
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1)
        total_ms += ms
        trace_ms += tr0.elapsed_time(tr1)
        per_frame.append(ms)
        n, r = bmfr.condition_stats(main_s)
        fp64_blocks.append(n)
        ratios.append(r)
        fallback.append(neural.fallback_tiles(main_s))
        if f in measure:  # outside the timed region; its reference renders' rays are not counted
            q0 = queries([pipe])
            quality.append(dict(frame=f, **full_relmse(args, vp, pipe, g, illu, bmfr, neural, pc, pc_den, main_s)))
            ref_rays += queries([pipe]) - q0
    rays = queries([pipe]) - st0 - ref_rays
    req_rays = queries(req_pipes) - req0
    line = {
        "metric": "4K 4spp denoised frames/s with 16 concurrent 1080p requests", "value": args.frames / (total_ms / 1e3),
        "unit": "fps", "frames": args.frames, "ms_per_step": total_ms / args.frames,
        "ms_per_step_max": max(per_frame), "requests_per_s": 16 * args.frames / (total_ms / 1e3),
        # BVH queries (primary + extension + shadow) of the 4K frames over the
        # 4K tracing time (its launches run beside the requests' stream), and
        # of the whole step (4K frames and requests) over the step time
        "grays_per_s_4k": rays / (trace_ms / 1e3) / 1e9,
        "grays_per_s_step": (rays + req_rays) / (total_ms / 1e3) / 1e9,
        "trace_ms_4k_per_frame": trace_ms / args.frames,
        "config": {"workload": "full chosen form", "width": W, "height": H, "spp": spp, "max_depth": args.max_depth,
                   "min_depth": args.min_depth, "triangles": int(info.triangle_count), "lights": int(info.light_count),
                   "instances": int(info.instance_count),
                   "network": "FP8 mode: e4m3 on the layers the calibration timed faster, BF16 on the others",
                   "e4m3_layers": [n for (n, *_), f in zip(_conv_table(), neural.fp8_layers()) if f],
                   "gate": ("learned per-tile blend of network and BMFR" if args.gate == "learned"
                            else f"variance threshold {args.gate_threshold}"),
                   "bmfr": "32x32, FP64 re-solve above R-ratio 1e6",
                   "requests": "16 x 1080p, 1 spp, accumulate + BMFR, own seeded scene each, one graph launch on a "
                               "second stream beside each 4K frame"},
        "fp64_blocks_per_frame_max": max(fp64_blocks), "largest_r_ratio": max(ratios),
        "fallback_tiles_per_frame": {"min": min(fallback), "max": max(fallback), "tiles": int(
            ((W + 31) // 32) * ((H + 31) // 32))},
        "relmse": quality, "setup_s": setup_s,
    }
    print(json.dumps(line), flush=True)


def full_relmse(args, vp, pipe, g, illu, bmfr, neural, pc, pc_den, stream):
    """relMSE of the current frame's outputs (network as shown with the gate,
    network alone, BMFR) against an --full-ref-spp render of the same camera."""
    import torch

    f = pc_den.value.frame_number
    albedo = g.albedo.tensor()[..., :3].double() / 255.0
    outs = {"bmfr": bmfr.denoised.tensor()[(f & 1) ^ 1][..., :3].double().clone(),
            "neural_gated": neural.denoised.tensor()[..., :3].double().clone()}  # as shown (learned gate)
    coef = neural.gate_coef
    neural.set_gate_model(None)
    neural.set_fallback(bmfr, threshold=1e30, tile=neural.tile)
    neural.dispatch(pc_den, stream)  # the network alone
    torch.cuda.synchronize()
    outs["neural"] = neural.denoised.tensor()[..., :3].double().clone()
    neural.set_fallback(bmfr, threshold=args.gate_threshold, tile=neural.tile)
    neural.set_gate_model(coef)
    img = illu.illumination_images[0].tensor()
    ref = torch.zeros_like(outs["bmfr"])
    for s_ in range(args.full_ref_spp):
        pc.set(frame_number=(1 << 24) + s_)
        pipe.trace(pc, stream)
        ref += img[..., :3]
    torch.cuda.synchronize()
    ref /= args.full_ref_spp
    r = albedo * ref
    res = {"reference_spp": args.full_ref_spp}
    for k, v in outs.items():
        res[k] = float((((albedo * v - r) ** 2) / (r * r + 0.01)).mean().item())
    return res


UNET_KERNELS = ("bf16_tcgen05", "bf16_mma", "fp8_tcgen05", "fp8_mma", "bf16_tcgen05_gather", "fp8_tcgen05_gather",
                "bf16_tcgen05_planes")


def _stage_ms(fn, stream, reps=10):
    """Mean device time of fn() on `stream` over `reps` back-to-back calls (CUDA events)."""
    import torch

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def _conv_table():
    from vulkanpbrt_gb300.kpunet import CONVS

    return CONVS


def _event_time_us(fn, reps):
    import torch

    for _ in range(3):
        fn()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps * 1e3


def unet_layer_times(width, height, reps, layers, kernels):
    """Per-convolution device times of the kernel-predicting U-Net: each of its
    18 3x3 convolutions (kpunet's layer table) timed alone with CUDA events on
    random BF16 inputs at its level of the padded frame, on the BF16 tcgen05
    kernels, the BF16 mma.sync kernel, the FP8 tcgen05 form and the FP8
    mma.sync kernel. Returns [(name, c1, c2, cout, level, {kernel: us or None})]."""
    import torch

    from vulkanpbrt_gb300 import build as B

    B.build()
    from vulkanpbrt_gb300 import nn
    from vulkanpbrt_gb300._abi import PbrtError
    from vulkanpbrt_gb300.kpunet import CONVS

    dev = torch.device("cuda:0")
    g = torch.Generator(device=dev).manual_seed(0)
    rows = []
    for name, (c1, c2), cout, lvl in CONVS:
        if layers and name not in layers:
            continue
        h, w = height >> lvl, width >> lvl
        x1 = torch.rand(1, h, w, c1, device=dev, generator=g).bfloat16()
        x2 = torch.rand(1, h // 2, w // 2, c2, device=dev, generator=g).bfloat16() if c2 else None
        cin = c1 + c2
        w32 = torch.randn(cout, 9, cin, device=dev, generator=g) * 0.05
        wb = w32.bfloat16()
        b = torch.zeros(cout, device=dev)
        xs = torch.ones(cin, device=dev)
        w8, ws = nn.quantize_weights_fp8(w32, xs)
        out = torch.empty(1, h, w, cout, device=dev, dtype=torch.bfloat16)
        run = {
            "bf16_tcgen05": lambda: nn.conv3x3_umma(x1, wb, b, x2=x2, relu=True, out=out),
            "bf16_mma": lambda: nn.conv3x3(x1, wb, b, x2=x2, relu=True, out=out),
            "fp8_tcgen05": lambda: nn.conv3x3_fp8(x1, w8, ws, xs, b, x2=x2, relu=True, out=out, kernel="umma"),
            "fp8_mma": lambda: nn.conv3x3_fp8(x1, w8, ws, xs, b, x2=x2, relu=True, out=out, kernel="mma"),
            # the upsampled second input gathered with cp.async instead of its TMA box
            "bf16_tcgen05_gather": lambda: nn.conv3x3_umma(x1, wb, b, x2=x2, relu=True, out=out, box=False),
            "fp8_tcgen05_gather": lambda: nn.conv3x3_fp8(x1, w8, ws, xs, b, x2=x2, relu=True, out=out, kernel="umma",
                                                         box=False),
            # the first input's halo as 8-channel planes instead of swizzled pixel rows
            "bf16_tcgen05_planes": lambda: nn.conv3x3_umma(x1, wb, b, x2=x2, relu=True, out=out, swizzle=False),
        }
        t = {}
        for k in UNET_KERNELS:
            swz = c1 in (16, 32) and not c2 and cout in (32, 48)  # the swizzled form applies
            if k not in kernels or (k.endswith("_gather") and not c2) or (k.endswith("_planes") and not swz):
                t[k] = None
                continue
            try:
                t[k] = _event_time_us(run[k], reps)
            except PbrtError:  # the FP8 tcgen05 form: weights and two input stages do not fit in shared memory
                t[k] = None
        rows.append((name, c1, c2, cout, lvl, t))
    if nn.umma_status():
        raise RuntimeError("a tcgen05 convolution reported a timed-out wait")
    return rows


def unet_head_times(width, height, reps):
    """Device time of each kernel-prediction head at its scale (inference
    outputs: the filtered, blended radiance and, at full scale, the error
    prediction) on random inputs. Returns [(name, channels, logits, scale, us)]."""
    import torch

    from vulkanpbrt_gb300 import nn
    from vulkanpbrt_gb300.kpunet import HEADS

    dev = torch.device("cuda:0")
    g = torch.Generator(device=dev).manual_seed(1)
    rows = []
    for name, _, c, k, s_ in HEADS:
        h, w = height >> s_, width >> s_
        F = torch.rand(1, h, w, c, device=dev, generator=g).bfloat16()
        Wh = torch.randn(k, c, device=dev, generator=g) * 0.1
        bh = torch.zeros(k, device=dev)
        R = torch.rand(1, h, w, 3, device=dev, generator=g)
        coarse = torch.rand(1, h // 2, w // 2, 3, device=dev, generator=g) if k > 25 else None
        out = torch.empty(1, h, w, 3, device=dev)
        var = torch.empty(1, h, w, device=dev) if k == 27 else None
        us = _event_time_us(lambda: nn.kp_head(F, Wh, bh, R, out, coarse=coarse, var=var), reps)
        rows.append((name, c, k, s_, us))
    return rows


def run_unet_layers(args):
    """Markdown table of per-convolution times (microseconds per launch) at
    --width x --height rounded up to the network's padded frame (multiples of
    16). Inputs are larger than L2 for the full-resolution layers only, so the
    deeper levels' times are L2-warm."""
    layers = [x for x in args.layers.split(",") if x]
    keys = [x for x in args.kernels.split(",") if x]
    bad = [k for k in keys if k not in UNET_KERNELS]
    if bad:
        raise SystemExit(f"unknown kernels {bad}; choose from {','.join(UNET_KERNELS)}")
    W, H = (args.width + 15) // 16 * 16, (args.height + 15) // 16 * 16
    rows = unet_layer_times(W, H, args.reps, layers, keys)
    print("| layer | c1+c2 -> cout | size | " + " | ".join(keys) + " |")
    print("|---|---|---|" + "---|" * len(keys))
    tot = {k: 0.0 for k in keys}
    for name, c1, c2, cout, lvl, t in rows:
        cells = []
        for k in keys:
            v = t[k]
            cells.append("-" if v is None else f"{v:.1f}")
            tot[k] += 0.0 if v is None else v
        print(f"| {name} | {c1}+{c2} -> {cout} | {W >> lvl}x{H >> lvl} | " + " | ".join(cells) + " |")
    print("| sum | | | " + " | ".join(f"{tot[k]:.1f}" for k in keys) + " |")
    heads = unet_head_times(W, H, args.reps)
    print("\n| head | channels -> logits | size | us |\n|---|---|---|---|")
    for name, c, k, s_, us in heads:
        print(f"| {name} | {c} -> {k} | {W >> s_}x{H >> s_} | {us:.1f} |")
    if "fp8_tcgen05" in keys and "fp8_mma" in keys:  # the FP8 path as dispatched: tcgen05 where it fits
        fp8_net = sum((t["fp8_tcgen05"] if t["fp8_tcgen05"] is not None else t["fp8_mma"]) or 0.0 for *_, t in rows)
        print(f"\nFP8 as dispatched (tcgen05 where it fits): {fp8_net:.1f} us")


def run_bvh_build(args):
    """The two BVH builds side by side -- FAST_TRACE (binned SAH on the host,
    SAH-optimal collapse; the default) and FAST_BUILD (linear BVH on the
    device, SAH-optimal or greedy collapse) -- on the benchmark scene and the full-form 4.3M-triangle scene:
    scene set-up and build time, tree size and depth, and what each tree
    costs a 1080p path-traced frame (frame ms by CUDA events over graph
    launches; traversal ms, nodes and triangles a ray from one profiled
    frame). Frames are bit-identical under both (tested)."""
    import torch

    from vulkanpbrt_gb300 import build as B

    B.build()
    import vulkanpbrt_gb300 as vp
    from vulkanpbrt_gb300 import scene as S

    W, H = args.width, args.height
    stream = torch.cuda.current_stream()
    scenes = {"bench_1M": lambda: workload(args),
              "full_4M": lambda: S.instanced_field(seed=0, instances=8000, point_lights=30)}
    out = {"metric": "BVH build ms and 1080p path-tracing ms: host binned SAH vs device linear BVH",
           "width": W, "height": H, "steps": args.steps, "scenes": {}}
    for name, make in scenes.items():
        sc = make()
        cams = [orbit(sc, W, H, f) for f in range(16)]
        rows = {}
        for label, build, collapse in (("fast_trace", "fast_trace", None), ("fast_build", "fast_build", None),
                                       ("fast_build_greedy", "fast_build", "greedy")):
            torch.cuda.synchronize()
            if collapse:
                os.environ["PBRT_BVH_COLLAPSE"] = collapse
            t0 = time.perf_counter()
            sh = vp.SceneHandle(sc, build=build)
            torch.cuda.synchronize()
            create_s = time.perf_counter() - t0
            os.environ.pop("PBRT_BVH_COLLAPSE", None)
            info = sh.info()
            g = vp.GBuffer(W, H)
            illu = vp.IlluminationBufferDemodulatedFloat(W, H)
            pipe = vp.PBRTPipeline(sh, g, illu, True, max_recursion_depth=args.max_depth,
                                   min_recursion_depth=args.min_depth)
            pc = vp.PushConstants()

            def set_cam(f):
                cam = cams[f % 16]
                pc.set(view_inverse=cam.inv_view, proj_inverse=cam.inv_proj, prev_view=cam.view, frame_number=f)

            for f in range(max(3, args.warmup)):
                set_cam(f)
                pipe.trace(pc, stream)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for f in range(args.steps):
                set_cam(f)
                pipe.trace(pc, stream)
            e1.record(stream)
            torch.cuda.synchronize()
            frame_ms = e0.elapsed_time(e1) / args.steps
            set_cam(5)
            t = pipe.profile(pc, stream)
            rays = t.closest_rays + t.shadow_rays
            rows[label] = {"scene_create_s": round(create_s, 3), "build_ms": round(info.build_ms, 1),
                           "nodes": int(info.bvh_nodes), "depth": int(info.bvh_depth),
                           "frame_ms": round(frame_ms, 3),
                           "traversal_ms": round(t.trace_closest_ms + t.trace_shadow_ms, 3),
                           "nodes_per_ray": round((t.closest_nodes + t.shadow_nodes) / max(1, rays), 2),
                           "tris_per_ray": round((t.closest_tris + t.shadow_tris) / max(1, rays), 2)}
            del pipe, g, illu, sh
            torch.cuda.synchronize()
        out["scenes"][name] = {"triangles": int(sc.tri_count), **rows}
    print(json.dumps(out))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "unet_layers":
        run_unet_layers(args)
    elif args.workload == "full":
        run_full(args)
    elif args.workload == "batch64":
        run_batch(args)
    elif args.workload == "bvh_build":
        run_bvh_build(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
