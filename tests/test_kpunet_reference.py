"""CPU checks of the neural denoiser's host side: the parameter layout, and
the PyTorch restatement's gradients against central finite differences in
FP64 (so the reference the GPU gradients are checked against is itself
right)."""
import numpy as np
import torch

from tests import kpunet_reference as ref
from vulkanpbrt_gb300 import kpunet as K


def test_parameter_layout_is_dense_and_ordered():
    lay, total = K.param_layout()
    spans = sorted((o, o + int(np.prod(s))) for o, s in lay.values())
    assert spans[0][0] == 0 and spans[-1][1] == total
    for (a0, a1), (b0, b1) in zip(spans, spans[1:]):
        assert a1 == b0
    assert lay["d3a.w"][1] == (96, 9, 96 + 128)
    assert lay["h0.w"][1] == (K.KP + 2, 32)
    p = K.init_params(0)
    assert p.size == total and np.isfinite(p).all()
    off, shape = lay["e0a.w"]
    assert not p[off:off + int(np.prod(shape))].reshape(shape)[:, :, 11:].any()


def test_reference_gradient_matches_finite_differences():
    torch.manual_seed(0)
    n, h, w = 1, 16, 16
    feat = torch.rand(n, h, w, K.IN_CH, dtype=torch.float64)
    rad = torch.rand(n, h, w, 3, dtype=torch.float64) * 2
    target = torch.rand(n, h, w, 3, dtype=torch.float64)
    albedo = torch.randint(30, 256, (n, h, w, 4), dtype=torch.uint8)
    rng = np.random.default_rng(3)
    p = K.init_params(2).astype(np.float64)
    lay, _ = K.param_layout()
    for key, (off, shape) in lay.items():
        if key.startswith("h") and key.endswith(".w"):
            p[off:off + int(np.prod(shape))] = rng.standard_normal(int(np.prod(shape))) * 0.2
    flat = torch.from_numpy(p).requires_grad_(True)

    # the variance head regresses on a detached target: hold it at the base point
    with torch.no_grad():
        o0, _ = ref.forward(flat, feat, rad, rounding=False)
        A = albedo[..., :3].double() / 255.0
        e0 = (A * o0 - A * target) ** 2 / ((A * target) ** 2 + 0.01)
        vt = torch.log(e0.sum(-1) / 3.0 + 1e-4)

    def objective(f):
        o, v = ref.forward(f, feat, rad, rounding=False)
        return ref.loss(o, v, target, albedo, 0.1)[0] + 0.1 * ((v - vt) ** 2).mean()

    o, v = ref.forward(flat, feat, rad, rounding=False)
    ref.loss(o, v, target, albedo, 0.1)[2].backward()
    g = flat.grad.numpy()
    idx = []
    for key in ("e0a.w", "e4b.w", "d3a.w", "d0b.b", "h0.w", "h1.b", "h2.w"):
        off, shape = lay[key]
        size = int(np.prod(shape))
        cand = off + rng.choice(size, 3, replace=False)
        idx.extend(int(i) for i in cand if key != "e0a.w" or (i - off) % K.IN_CH < 11)
    eps = 1e-6
    for i in idx:
        fp = flat.detach().clone()
        fm = flat.detach().clone()
        fp[i] += eps
        fm[i] -= eps
        fd = (objective(fp) - objective(fm)).item() / (2 * eps)
        assert abs(fd - g[i]) <= 1e-5 * max(1.0, abs(fd)) + 1e-9, (i, fd, g[i])
