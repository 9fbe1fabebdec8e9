"""Per-convolution device times of the kernel-predicting U-Net at one frame
size: each of its 18 3x3 convolutions (the layer table of ``kpunet``) timed
alone with CUDA events on random BF16 inputs, on the BF16 tcgen05 kernels,
the BF16 mma.sync kernel, the FP8 tcgen05 form (kind::f8f6f4) and the FP8
mma.sync kernel. Prints a markdown table (microseconds per launch).

    python -m vulkanpbrt_gb300.layer_times [--width 1920] [--height 1088] [--reps 20]
        [--layers e0b,d0a] [--kernels fp8_tcgen05]

The frame is the network's padded frame (multiples of 16); inputs are
larger than L2 at 1080p for the full-resolution layers only, so the deeper
levels' times are L2-warm."""
from __future__ import annotations

import argparse


def _time(fn, reps):
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


KERNELS = ("bf16_tcgen05", "bf16_mma", "fp8_tcgen05", "fp8_mma")


def layer_times(width=1920, height=1088, reps=20, layers=None, kernels=KERNELS):
    """[(name, c1, c2, cout, level, {kernel: microseconds or None})] for every convolution (or those named
    in layers), on the kernels named in kernels."""
    import torch

    from . import nn
    from ._abi import PbrtError
    from .kpunet import CONVS

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
        }
        t = {}
        for k in KERNELS:
            if k not in kernels:
                t[k] = None
                continue
            try:
                t[k] = _time(run[k], reps)
            except PbrtError:  # the FP8 tcgen05 form: weights and two input stages do not fit in shared memory
                t[k] = None
        rows.append((name, c1, c2, cout, lvl, t))
    if nn.umma_status():
        raise RuntimeError("a tcgen05 convolution reported a timed-out wait")
    return rows


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1088)
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--layers", default="", help="comma-separated layer names (default: all 18)")
    ap.add_argument("--kernels", default=",".join(KERNELS), help="comma-separated subset of " + ",".join(KERNELS))
    a = ap.parse_args(argv)
    layers = [x for x in a.layers.split(",") if x]
    keys = [x for x in a.kernels.split(",") if x]
    bad = [k for k in keys if k not in KERNELS]
    if bad:
        ap.error(f"unknown kernels {bad}")
    rows = layer_times(a.width, a.height, a.reps, layers, keys)
    print(f"| layer | c1+c2 -> cout | size | " + " | ".join(keys) + " |")
    print("|---|---|---|" + "---|" * len(keys))
    tot = {k: 0.0 for k in keys}
    for name, c1, c2, cout, lvl, t in rows:
        cells = []
        for k in keys:
            v = t[k]
            cells.append("-" if v is None else f"{v:.1f}")
            tot[k] += 0.0 if v is None else v
        print(f"| {name} | {c1}+{c2} -> {cout} | {a.width >> lvl}x{a.height >> lvl} | " + " | ".join(cells) + " |")
    print("| sum | | | " + " | ".join(f"{tot[k]:.1f}" for k in keys) + " |")
    if "fp8_tcgen05" in keys and "fp8_mma" in keys:  # the FP8 path as dispatched: tcgen05 where it fits
        fp8_net = sum((t["fp8_tcgen05"] if t["fp8_tcgen05"] is not None else t["fp8_mma"]) or 0.0 for *_, t in rows)
        print(f"\nFP8 as dispatched (tcgen05 where it fits): {fp8_net:.1f} us")


if __name__ == "__main__":
    main()
