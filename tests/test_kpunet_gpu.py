"""The whole kernel-predicting U-Net on the GPU kernels against the plain
PyTorch FP32 CPU restatement in tests/kpunet_reference.py: forward values,
the loss, and the gradient of every parameter tensor (the gradient check of
the training path), then a short training run that must lower the loss.

Tolerances: outputs and losses within 2e-2 relative (BF16 activations
rounded at the same points, FP32 accumulation in a different order); each
parameter gradient within 6e-2 relative L2 error and cosine similarity above
0.995 (the GPU also rounds the ReLU-masked gradients to BF16). Checked with
the forward and backward-data convolutions on mma.sync and on tcgen05."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _net_inputs(n, h, w, seed):
    import torch

    g = torch.Generator().manual_seed(seed)
    illum = torch.rand(n, h, w, 4, generator=g) ** 3 * 6.0
    albedo = torch.randint(20, 256, (n, h, w, 4), generator=g, dtype=torch.uint8)
    normal = torch.rand(n, h, w, 2, generator=g) * torch.tensor([3.14159, 6.28318])
    depth = torch.rand(n, h, w, generator=g) * 30.0
    target = torch.nn.functional.avg_pool2d(illum[..., :3].permute(0, 3, 1, 2), 5, 1, 2,
                                            count_include_pad=False).permute(0, 2, 3, 1).contiguous()
    return illum, albedo, normal, depth, target


def _params(seed):
    from vulkanpbrt_gb300 import kpunet as K

    p = K.init_params(seed)
    lay, _ = K.param_layout()
    rng = np.random.default_rng(seed + 1)
    for key, (off, shape) in lay.items():  # heads large enough that every layer gets a real gradient
        if key.startswith("h") and key.endswith(".w"):
            p[off:off + int(np.prod(shape))] = rng.standard_normal(int(np.prod(shape))).astype(np.float32) * 0.2
        if key.endswith(".b") and not key.startswith("h"):
            p[off:off + shape[0]] = rng.standard_normal(shape[0]).astype(np.float32) * 0.05
    return p


@pytest.mark.parametrize("kernel", ["mma", "umma"])
def test_forward_loss_and_gradients_match_reference(cuda, kernel):
    import torch

    from tests import kpunet_reference as ref
    from vulkanpbrt_gb300 import kpunet as K

    n, h, w = 2, 32, 48
    illum, albedo, normal, depth, target = _net_inputs(n, h, w, 3)
    p = _params(4)
    net = K.KPUNet(cuda, params=p)
    ws = net.workspace(n, h, w)
    ws.set_input(illum.to(cuda), albedo.to(cuda), normal.to(cuda), depth.to(cuda))
    out = ws.forward(kernel)
    net.grad.zero_()
    ws.loss_and_grad(target.to(cuda), albedo.to(cuda), var_weight=0.1, kernel=kernel)
    torch.cuda.synchronize()

    feat, rad = ref.features(illum, albedo, normal, depth, h, w)
    flat = torch.from_numpy(p.copy()).requires_grad_(True)
    o_ref, v_ref = ref.forward(flat, feat, rad)
    lm, lv, total = ref.loss(o_ref, v_ref, target, albedo, 0.1)
    total.backward()

    scale = o_ref.abs().max().item()
    assert (out.cpu() - o_ref.detach()).abs().max().item() < 2e-2 * scale
    assert (ws.var.cpu() - v_ref.detach()).abs().max().item() < 2e-2 * (v_ref.abs().max().item() + 1)
    lg = ws.loss.cpu()
    assert abs(lg[0].item() - lm.item()) < 2e-2 * lm.item()
    assert abs(lg[1].item() - lv.item()) < 2e-2 * lv.item()

    gg = net.grad.cpu()
    worst = []
    for key, (off, shape) in net.layout.items():
        size = int(np.prod(shape))
        a = gg[off:off + size].double()
        b = flat.grad[off:off + size].double()
        rel = ((a - b).norm() / (b.norm() + 1e-30)).item()
        cos = (a @ b / (a.norm() * b.norm() + 1e-30)).item()
        worst.append((rel, cos, key))
        assert rel < 6e-2 and cos > 0.995, (key, rel, cos)
    worst.sort(reverse=True)
    print("largest gradient errors:", worst[:4])


def test_training_lowers_the_loss(cuda):
    import torch

    from vulkanpbrt_gb300 import kpunet as K

    n, h, w = 4, 64, 64
    illum, albedo, normal, depth, target = _net_inputs(n, h, w, 11)
    net = K.KPUNet(cuda, seed=1)
    ws = net.workspace(n, h, w)
    ws.set_input(illum.to(cuda), albedo.to(cuda), normal.to(cuda), depth.to(cuda))
    t, a = target.to(cuda), albedo.to(cuda)
    losses = []
    for _ in range(60):
        losses.append(ws.train_step(t, a, lr=1e-3)[0].item())
    torch.cuda.synchronize()
    print("loss first/last", losses[0], losses[-1])
    assert np.isfinite(losses).all()
    assert losses[-1] < 0.7 * losses[0]
