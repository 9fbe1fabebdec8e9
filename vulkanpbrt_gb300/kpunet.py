"""Kernel-predicting U-Net denoiser on this library's kernels.

Five levels with 32/48/64/96/128 channels, two 3x3 convolutions with ReLU
per level, 2x2 average pooling down and nearest upsampling fused into the
first decoder convolution (concat of the skip and the upsampled coarser
level). Heads at three scales (full, 1/2, 1/4) predict a softmax 5x5 kernel
that filters the noisy demodulated illumination of that scale (pooled for
the coarse ones); the two finer heads also predict the weight that blends
the upsampled coarser result in, and the full-scale head predicts the log
squared error of its pixel (the variance gate that hands tiles back to
BMFR). Inputs are the 1-spp G-buffer and illumination: 16 BF16 channels
(log1p radiance, albedo, normal, log1p depth / 8, samples per pixel, five
zero channels).

Activations and convolution weights are BF16 with FP32 accumulation; the
master weights, gradients and Adam moments are FP32 in one flat buffer each,
so one Adam launch updates everything. All buffers for one batch shape are
allocated once (``KPUNet.workspace``), so a training step or an inference
pass allocates nothing and can be captured in a CUDA graph.

No reference counterpart: the reference's denoisers are BMFR and BFR
(source/renderModules/BMFR.cpp, source/renderModules/BFR.cpp)."""
from __future__ import annotations

import numpy as np

from . import nn

LEVELS = (32, 48, 64, 96, 128)
IN_CH = 16
KP = 25

# (name, input channels (skip, upsampled), output channels); level index
ENCODER = [("e0a", (IN_CH, 0), 32, 0), ("e0b", (32, 0), 32, 0),
           ("e1a", (32, 0), 48, 1), ("e1b", (48, 0), 48, 1),
           ("e2a", (48, 0), 64, 2), ("e2b", (64, 0), 64, 2),
           ("e3a", (64, 0), 96, 3), ("e3b", (96, 0), 96, 3),
           ("e4a", (96, 0), 128, 4), ("e4b", (128, 0), 128, 4)]
DECODER = [("d3a", (96, 128), 96, 3), ("d3b", (96, 0), 96, 3),
           ("d2a", (64, 96), 64, 2), ("d2b", (64, 0), 64, 2),
           ("d1a", (48, 64), 48, 1), ("d1b", (48, 0), 48, 1),
           ("d0a", (32, 48), 32, 0), ("d0b", (32, 0), 32, 0)]
CONVS = ENCODER + DECODER
# (name, feature tensor, channels, logits, scale)
HEADS = [("h2", "d2", 64, KP, 2), ("h1", "d1", 48, KP + 1, 1), ("h0", "d0", 32, KP + 2, 0)]


def param_layout():
    """Offsets (in floats) of every parameter in the flat buffer: conv weights
    [cout][9][cin], conv biases [cout], head weights [k][c], head biases [k]."""
    off, lay = 0, {}
    for name, (c1, c2), cout, _ in CONVS:
        n = cout * 9 * (c1 + c2)
        lay[name + ".w"] = (off, (cout, 9, c1 + c2))
        off += n
    for name, (c1, c2), cout, _ in CONVS:
        lay[name + ".b"] = (off, (cout,))
        off += cout
    for name, _, c, k, _ in HEADS:
        lay[name + ".w"] = (off, (k, c))
        off += k * c
        lay[name + ".b"] = (off, (k,))
        off += k
    return lay, off


def init_params(seed=0):
    """He-normal convolution weights (zero for the padding input channels),
    zero biases, head weights of scale 1e-3 (close to a uniform 5x5 box
    filter and an even blend at the start)."""
    lay, total = param_layout()
    rng = np.random.default_rng(seed)
    p = np.zeros(total, np.float32)
    for name, (c1, c2), cout, _ in CONVS:
        off, shape = lay[name + ".w"]
        w = rng.standard_normal(shape).astype(np.float32) * np.sqrt(2.0 / (9 * (c1 + c2)))
        if name == "e0a":
            w[:, :, 11:] = 0.0
        p[off:off + w.size] = w.ravel()
    for name, _, c, k, _ in HEADS:
        off, shape = lay[name + ".w"]
        p[off:off + k * c] = (rng.standard_normal(shape) * 1e-3).astype(np.float32).ravel()
    return p


class KPUNet:
    """Parameters on the device plus forward / backward / Adam over them."""

    def __init__(self, device="cuda", params=None, seed=0):
        import torch

        self.device = torch.device(device)
        self.layout, self.n_params = param_layout()
        host = init_params(seed) if params is None else np.asarray(params, np.float32)
        if host.size != self.n_params:
            raise ValueError(f"KPUNet: expected {self.n_params} parameters, got {host.size}")
        self.w32 = torch.from_numpy(host.copy()).to(self.device)
        self.w16 = self.w32.to(torch.bfloat16)
        self.grad = torch.zeros_like(self.w32)
        self.m = torch.zeros_like(self.w32)
        self.v = torch.zeros_like(self.w32)
        self.step_count = 0
        self._flipped = {}
        self._flip_stamp = -1

    # ---- parameter views --------------------------------------------------
    def _view(self, buf, key):
        off, shape = self.layout[key]
        n = int(np.prod(shape))
        return buf[off:off + n].view(*shape)

    def conv_w(self, name):
        return self._view(self.w16, name + ".w")

    def conv_b(self, name):
        return self._view(self.w32, name + ".b")

    def flipped(self, name):
        if self._flip_stamp != self.step_count:
            for cname, (c1, c2), cout, _ in CONVS:
                if cname == "e0a":
                    continue
                if cname not in self._flipped:
                    import torch

                    self._flipped[cname] = torch.empty((c1 + c2, 9, cout), dtype=torch.bfloat16,
                                                       device=self.device)
                nn.flip_weights(self.conv_w(cname), self._flipped[cname])
            self._flip_stamp = self.step_count
        return self._flipped[name]

    def state_dict(self):
        return {"params": self.w32.detach().cpu().numpy(), "step": self.step_count}

    def save(self, path):
        np.savez_compressed(path, params=self.w32.detach().cpu().numpy(), step=np.int64(self.step_count),
                            levels=np.asarray(LEVELS))

    @classmethod
    def load(cls, path, device="cuda"):
        d = np.load(path)
        net = cls(device, params=d["params"])
        net.step_count = int(d["step"])
        return net

    # ---- workspace ----------------------------------------------------------
    def workspace(self, n, ph, pw, training=True):
        """All activation (and, for training, gradient) buffers for a batch of
        n padded images of ph x pw (multiples of 16)."""
        if ph % 16 or pw % 16:
            raise ValueError("KPUNet: padded sizes must be multiples of 16")
        return Workspace(self, n, ph, pw, training)


class Workspace:
    def __init__(self, net, n, ph, pw, training):
        import torch

        self.net, self.n, self.ph, self.pw, self.training = net, n, ph, pw, training
        dev = net.device
        bf, f32 = torch.bfloat16, torch.float32

        def t(level, c, dtype=bf):
            return torch.empty((n, ph >> level, pw >> level, c), dtype=dtype, device=dev)

        self.feat = t(0, IN_CH)
        self.act = {}
        for name, _, cout, lvl in CONVS:
            self.act[name] = t(lvl, cout)
        self.pool = {1: t(1, 32), 2: t(2, 48), 3: t(3, 64), 4: t(4, 96)}
        self.rad = {0: t(0, 3, f32), 1: t(1, 3, f32), 2: t(2, 3, f32)}
        self.out = {s: t(s, 3, f32) for s in (0, 1, 2)}
        self.var = torch.empty((n, ph, pw), dtype=f32, device=dev)
        self.loss = torch.zeros(2, dtype=f32, device=dev)
        if training:
            self.kw = {s: t(s, KP, f32) for s in (0, 1, 2)}
            self.filt = {s: t(s, 3, f32) for s in (0, 1, 2)}
            self.alpha = {s: torch.empty((n, ph >> s, pw >> s), dtype=f32, device=dev) for s in (0, 1)}
            self.gact = {name: t(lvl, cout, f32) for name, _, cout, lvl in CONVS}
            self.gpool = {1: t(1, 32, f32), 2: t(2, 48, f32), 3: t(3, 64, f32), 4: t(4, 96, f32)}
            self.gout = {s: t(s, 3, f32) for s in (0, 1, 2)}
            self.gvar = torch.empty((n, ph, pw), dtype=f32, device=dev)
            # scratch sized for the largest use (level 0); _scratch picks the shape
            self.gmask = t(0, 32, bf)  # ReLU-masked BF16 gradient of a convolution output
            self.gcat = t(0, 80, f32)  # gradient of a concatenated input (d0a: 32 + 48 channels)
            self._gmask_flat = self.gmask.view(-1)
            self._gcat_flat = self.gcat.view(-1)

    def _scratch(self, flat, level, c):
        n = self.n * (self.ph >> level) * (self.pw >> level) * c
        return flat[:n].view(self.n, self.ph >> level, self.pw >> level, c)

    # ---- forward ------------------------------------------------------------
    def set_input(self, illum, albedo, normal, depth, spp=None):
        nn.features(illum, albedo, normal, depth, self.feat, self.rad[0], spp=spp)

    def forward(self, kernel="mma"):
        """kernel: "mma" (warp-level mma.sync convolutions, the training path), "umma" (tcgen05), or a
        list with one per convolution (layer order of CONVS; "umma_planes": tcgen05 with the first
        input's halo as 8-channel planes, the same bits as "umma")."""
        import functools

        net, a = self.net, self.act
        kinds = list(kernel) if isinstance(kernel, (list, tuple)) else [kernel] * len(CONVS)
        conv = {"mma": nn.conv3x3, "umma": nn.conv3x3_umma,
                "umma_planes": functools.partial(nn.conv3x3_umma, swizzle=False)}
        layer = {name: conv[k] for (name, _, _, _), k in zip(CONVS, kinds)}
        nn.avgpool2(self.rad[0], self.rad[1])
        nn.avgpool2(self.rad[1], self.rad[2])
        x = self.feat
        for name, (c1, c2), cout, lvl in ENCODER:
            if name.endswith("a") and lvl > 0:
                nn.avgpool2(x, self.pool[lvl])
                x = self.pool[lvl]
            layer[name](x, net.conv_w(name), net.conv_b(name), relu=True, out=a[name])
            x = a[name]
        skips = {0: a["e0b"], 1: a["e1b"], 2: a["e2b"], 3: a["e3b"]}
        for name, (c1, c2), cout, lvl in DECODER:
            if name.endswith("a"):
                layer[name](skips[lvl], net.conv_w(name), net.conv_b(name), x2=x, relu=True, out=a[name])
            else:
                layer[name](x, net.conv_w(name), net.conv_b(name), relu=True, out=a[name])
            x = a[name]
        tr = self.training
        for hname, fname, c, k, s in HEADS:
            coarse = self.out[s + 1] if s < 2 else None
            nn.kp_head(a[fname + "b"], net._view(net.w32, hname + ".w"), net._view(net.w32, hname + ".b"),
                       self.rad[s], self.out[s], coarse=coarse,
                       kw=self.kw[s] if tr else None, filt=self.filt[s] if tr else None,
                       alpha=self.alpha[s] if (tr and coarse is not None) else None,
                       var=self.var if s == 0 else None)
        return self.out[0]

    # ---- loss and backward --------------------------------------------------
    def loss_and_grad(self, target, albedo, var_weight=0.1, kernel="mma"):
        """relMSE (plus the variance head's loss) into self.loss; gradients into net.grad."""
        self.loss.zero_()
        nn.relmse_loss(self.out[0], target, albedo, self.gout[0], self.loss, var=self.var, dvar=self.gvar,
                       var_weight=var_weight)
        self.backward(kernel)

    def _dgrad(self, gm, name, out32, kernel):
        """Gradient of a convolution's input: gm convolved with the flipped weights, FP32 out."""
        if kernel == "umma":
            nn.conv3x3_umma_f32(gm, self.net.flipped(name), out32)
        else:
            nn.conv3x3(gm, self.net.flipped(name), None, out32=out32, store_bf16=False)

    def backward(self, kernel="mma"):
        """kernel: the backward-data and backward-weight convolutions on "mma" (mma.sync) or "umma"
        (tcgen05)."""
        net, a, g = self.net, self.act, self.gact
        G = net.grad
        for t in list(g.values()) + list(self.gpool.values()) + [self.gout[1], self.gout[2]]:
            t.zero_()
        # heads, fine to coarse
        for hname, fname, c, k, s in reversed(HEADS):
            coarse = self.out[s + 1] if s < 2 else None
            nn.kp_head_bwd(a[fname + "b"], net._view(net.w32, hname + ".w"), net._view(net.w32, hname + ".b"),
                           self.rad[s], self.kw[s], self.filt[s], self.gout[s], g[fname + "b"],
                           net._view(G, hname + ".w"), net._view(G, hname + ".b"), coarse=coarse,
                           alpha=self.alpha[s] if coarse is not None else None,
                           dvar=self.gvar if s == 0 else None,
                           dcoarse=self.gout[s + 1] if coarse is not None else None)
        # decoder, coarse gradient flows fine -> coarse
        skip_of = {3: "e3b", 2: "e2b", 1: "e1b", 0: "e0b"}
        up_of = {3: "e4b", 2: "d3b", 1: "d2b", 0: "d1b"}
        for name, (c1, c2), cout, lvl in reversed(DECODER):
            gm = self._scratch(self._gmask_flat, lvl, cout)
            nn.relu_bwd(g[name], a[name], gm, db=net._view(G, name + ".b"))
            if name.endswith("b"):
                prev = name[:-1] + "a"
                nn.conv3x3_wgrad(gm, a[prev], net._view(G, name + ".w"), kernel=kernel)
                self._dgrad(gm, name, g[prev], kernel)
            else:
                sk, up = skip_of[lvl], up_of[lvl]
                nn.conv3x3_wgrad(gm, a[sk], net._view(G, name + ".w"), x2=a[up], kernel=kernel)
                gc = self._scratch(self._gcat_flat, lvl, c1 + c2)
                self._dgrad(gm, name, gc, kernel)
                nn.split_upsum(gc, c1, g[sk], g[up])
        # encoder
        for name, (c1, c2), cout, lvl in reversed(ENCODER):
            gm = self._scratch(self._gmask_flat, lvl, cout)
            nn.relu_bwd(g[name], a[name], gm, db=net._view(G, name + ".b"))
            if name.endswith("b"):
                prev = name[:-1] + "a"
                nn.conv3x3_wgrad(gm, a[prev], net._view(G, name + ".w"), kernel=kernel)
                self._dgrad(gm, name, g[prev], kernel)
            elif lvl > 0:
                xin = self.pool[lvl]
                nn.conv3x3_wgrad(gm, xin, net._view(G, name + ".w"), kernel=kernel)
                self._dgrad(gm, name, self.gpool[lvl], kernel)
                nn.avgpool2_bwd_add(self.gpool[lvl], g["e%db" % (lvl - 1)])
            else:
                nn.conv3x3_wgrad(gm, self.feat, net._view(G, name + ".w"), kernel=kernel)

    def train_step(self, target, albedo, lr=1e-4, var_weight=0.1, kernel="mma"):
        """One Adam step; kernel "umma" runs every convolution (forward, backward data and weights) on tcgen05."""
        net = self.net
        self.forward(kernel)
        net.grad.zero_()
        self.loss_and_grad(target, albedo, var_weight, kernel)
        net.step_count += 1
        nn.adam(net.w32, net.grad, net.m, net.v, net.step_count, lr=lr, w_bf16=net.w16)
        return self.loss


def main(argv=None):
    """Times the network's forward pass on random inputs:
    python -m vulkanpbrt_gb300.kpunet [--height 1088 --width 1920 --iters 10];
    with --train, Adam training steps instead (random inputs and targets,
    default batch 16 of 256x256, the training kernels)."""
    import argparse
    import json

    import torch

    ap = argparse.ArgumentParser(description="time the kernel-predicting U-Net forward pass or training step")
    ap.add_argument("--height", type=int, default=None, help="default 1088 (forward), 256 (--train)")
    ap.add_argument("--width", type=int, default=None, help="default 1920 (forward), 256 (--train)")
    ap.add_argument("--batch", type=int, default=None, help="default 1 (forward), 16 (--train)")
    ap.add_argument("--iters", type=int, default=10)
    ap.add_argument("--kernel", default="mma", choices=["mma", "umma"], help="convolutions: mma.sync or tcgen05")
    ap.add_argument("--train", action="store_true", help="time training steps (forward, loss, backward, Adam)")
    a = ap.parse_args(argv)
    h = a.height or (256 if a.train else 1088)
    w = a.width or (256 if a.train else 1920)
    n = a.batch or (16 if a.train else 1)
    from . import build

    build.build()
    dev = torch.device("cuda", 0)
    net = KPUNet(dev, seed=0)
    ws = net.workspace(n, h, w, training=a.train)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if a.train:
        g = torch.Generator(device=dev).manual_seed(0)
        illum = torch.rand(n, h, w, 4, device=dev, generator=g) ** 3 * 6
        albedo = torch.randint(20, 256, (n, h, w, 4), device=dev, generator=g, dtype=torch.uint8)
        normal = torch.rand(n, h, w, 2, device=dev, generator=g) * 3
        depth = torch.rand(n, h, w, device=dev, generator=g) * 30
        target = illum[..., :3].contiguous()
        ws.set_input(illum, albedo, normal, depth)
        ws.train_step(target, albedo, kernel=a.kernel)  # warm-up
        torch.cuda.synchronize()
        e0.record()
        for _ in range(a.iters):
            ws.train_step(target, albedo, kernel=a.kernel)
        e1.record()
        torch.cuda.synchronize()
        print(json.dumps({"train_step_ms": e0.elapsed_time(e1) / a.iters, "batch": n, "height": h, "width": w,
                          "kernel": a.kernel}))
        return
    ws.feat.normal_()
    ws.rad[0].uniform_()
    ws.forward(a.kernel)  # warm-up
    torch.cuda.synchronize()
    e0.record()
    for _ in range(a.iters):
        ws.forward(a.kernel)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / a.iters
    flop = sum(2 * 9 * (c1 + c2) * co * (h >> l) * (w >> l) for _, (c1, c2), co, l in CONVS) * n
    print(json.dumps({"forward_ms": ms, "conv_tflops_per_s": flop / ms / 1e9, "pixels": h * w * n}))


if __name__ == "__main__":
    main()
