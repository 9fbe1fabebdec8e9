"""Plain PyTorch FP32 (CPU) restatement of the kernel-predicting U-Net, its
loss and its input features: the floating-point reference the GPU kernels'
forward values and gradients are checked against. Activations are rounded
to BF16 where the GPU stores them in BF16, so the two differ only by
accumulation order and by the BF16 rounding of gradients."""
from __future__ import annotations

import numpy as np
import torch
import torch.nn.functional as F

from vulkanpbrt_gb300 import kpunet as K


def bf16(x):
    return x.to(torch.bfloat16).to(torch.float32)


def decode_normal(th, ph):
    st = torch.sin(th)
    return torch.stack([torch.cos(ph) * st, torch.sin(ph) * st, torch.cos(th)], -1)


def features(illum, albedo, normal, depth, ph, pw, spp=None):
    """illum [N,h,w,4] f32, albedo [N,h,w,4] u8, normal [N,h,w,2], depth [N,h,w], spp [N,h,w] u8 (1/256 steps)
    -> feat [N,ph,pw,16], rad (clamped to [0, 10])."""
    n, h, w = illum.shape[:3]
    yi = torch.clamp(torch.arange(ph), max=h - 1)
    xi = torch.clamp(torch.arange(pw), max=w - 1)

    def pad(t):
        return t[:, yi][:, :, xi]

    c = pad(illum[..., :3].float()).clamp(0, 10)
    a = pad(albedo[..., :3].float()) / 255.0
    nrm = decode_normal(pad(normal[..., 0]), pad(normal[..., 1]))
    d = torch.log1p(pad(depth).clamp_min(0)) * 0.125
    s = (torch.full((n, ph, pw), 1.0 / 16) if spp is None
         else (pad(spp.float()) / 255.0 * 256.0).clamp(max=16.0) / 16.0)
    f = torch.cat([torch.log1p(c), a, nrm, d[..., None], s[..., None], torch.zeros(n, ph, pw, 5)], -1)
    return bf16(f), c


def conv(x, w, b, relu=True):
    """x [N,H,W,C], w [cout, 9, cin] -> [N,H,W,cout]."""
    cout, _, cin = w.shape
    wt = w.reshape(cout, 3, 3, cin).permute(0, 3, 1, 2)
    y = F.conv2d(x.permute(0, 3, 1, 2), wt, b, padding=1).permute(0, 2, 3, 1)
    return torch.relu(y) if relu else y


def pool(x):
    return F.avg_pool2d(x.permute(0, 3, 1, 2), 2).permute(0, 2, 3, 1)


def up(x):
    return x.repeat_interleave(2, 1).repeat_interleave(2, 2)


def head(Fm, Wh, bh, R, coarse):
    lg = Fm @ Wh.t() + bh
    kw = torch.softmax(lg[..., :K.KP], -1)
    n, h, w, _ = R.shape
    Rp = F.pad(R.permute(0, 3, 1, 2), (2, 2, 2, 2), mode="replicate")
    patches = F.unfold(Rp, 5).view(n, 3, 25, h, w).permute(0, 3, 4, 1, 2)  # [n,h,w,3,25] (dy major, dx minor)
    filt = (patches * kw[..., None, :]).sum(-1)
    out = filt
    if coarse is not None:
        al = torch.sigmoid(lg[..., K.KP])
        out = (1 - al[..., None]) * filt + al[..., None] * up(coarse)
    var = lg[..., -1]
    return out, var


def params_dict(flat):
    lay, _ = K.param_layout()
    return {k: flat[o:o + int(np.prod(s))].view(*s) for k, (o, s) in lay.items()}


def forward(flat, feat, rad, rounding=True):
    """flat: FP32 master parameters (leaf tensor). Returns out0, var. With
    rounding=False nothing is rounded to BF16 (for finite differences)."""
    p = params_dict(flat)
    rnd = bf16 if rounding else (lambda t: t)

    def cw(name):
        return rnd(p[name + ".w"])

    a = {}
    x = feat
    for name, _, _, lvl in K.ENCODER:
        if name.endswith("a") and lvl > 0:
            x = rnd(pool(x))
        a[name] = rnd(conv(x, cw(name), p[name + ".b"]))
        x = a[name]
    skips = {0: a["e0b"], 1: a["e1b"], 2: a["e2b"], 3: a["e3b"]}
    for name, _, _, lvl in K.DECODER:
        inp = torch.cat([skips[lvl], up(x)], -1) if name.endswith("a") else x
        a[name] = rnd(conv(inp, cw(name), p[name + ".b"]))
        x = a[name]
    R = {0: rad}
    R[1] = pool(R[0])
    R[2] = pool(R[1])
    out = {}
    var = None
    for hname, fname, c, k, s in K.HEADS:
        o, v = head(a[fname + "b"], p[hname + ".w"], p[hname + ".b"], R[s], out.get(s + 1))
        out[s] = o
        if s == 0:
            var = v
    return out[0], var


def loss(out, var, target, albedo, var_weight=0.1):
    A = albedo[..., :3].float() / 255.0
    n, h, w = target.shape[:3]
    o = out[:, :h, :w]
    r = A * target
    e = (A * o - r) ** 2 / (r * r + 0.01)
    l_main = e.mean()
    tgt = torch.log(e.sum(-1).detach() / 3.0 + 1e-4)
    l_var = ((var[:, :h, :w] - tgt) ** 2).mean()
    return l_main, l_var, l_main + var_weight * l_var
