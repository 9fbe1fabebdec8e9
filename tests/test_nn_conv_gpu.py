"""Tensor-core convolution kernels of the neural denoiser against torch's FP32
conv2d on the same BF16-rounded operands (the floating-point reference for
these kernels). Tolerance, relative to the output scale: 1e-4 for FP32
outputs (FP32 accumulation of BF16 products), 4e-3 (one BF16 ulp) where the
output is stored as BF16."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ref_conv(x1, w, bias, x2=None):
    import torch
    import torch.nn.functional as F

    x = x1.float()
    if x2 is not None:
        up = x2.float().repeat_interleave(2, 1).repeat_interleave(2, 2)
        x = torch.cat([x, up], -1)
    wt = w.float().reshape(w.shape[0], 3, 3, -1).permute(0, 3, 1, 2)  # [co, ci, ky, kx]
    y = F.conv2d(x.permute(0, 3, 1, 2).cpu(), wt.cpu(), bias.float().cpu() if bias is not None else None, padding=1)
    return y.permute(0, 2, 3, 1)


def _close(got, want, tol=4e-3):
    scale = want.abs().max().item() + 1e-6
    err = (got.float().cpu() - want.float().cpu()).abs().max().item()
    return err / scale, err <= tol * scale


@pytest.mark.parametrize("kernel", ["halo", "halo4x2", "kstep"])
@pytest.mark.parametrize("n,h,w,c1,c2,cout", [(2, 24, 40, 16, 0, 32), (1, 32, 32, 32, 0, 48), (1, 16, 48, 48, 32, 48),
                                             (2, 20, 36, 64, 0, 160), (1, 18, 34, 96, 128, 96),
                                             (1, 10, 22, 48, 64, 48), (1, 12, 16, 32, 48, 32),
                                             (1, 8, 16, 128, 0, 128), (1, 9, 17, 16, 0, 64),
                                             (2, 33, 47, 32, 0, 16), (1, 18, 30, 16, 16, 48)])
def test_conv3x3_forward(cuda, n, h, w, c1, c2, cout, kernel):
    import torch

    from vulkanpbrt_gb300 import nn

    g = torch.Generator().manual_seed(n * 100 + c1 + c2 + cout)
    x1 = torch.randn(n, h, w, c1, generator=g).bfloat16().to(cuda)
    x2 = torch.randn(n, h // 2, w // 2, c2, generator=g).bfloat16().to(cuda) if c2 else None
    wt = (torch.randn(cout, 9, c1 + c2, generator=g) * 0.1).bfloat16().to(cuda)
    b = torch.randn(cout, generator=g).float().to(cuda)
    y32 = torch.empty(n, h, w, cout, device=cuda)
    y = nn.conv3x3(x1, wt, b, x2=x2, relu=False, out32=y32, kernel=kernel)
    torch.cuda.synchronize()
    ref = _ref_conv(x1, wt, b, x2)
    rel, ok = _close(y32, ref, 1e-4)
    print(f"forward fp32 epilogue rel err {rel:.2e}")
    assert ok
    rel, ok = _close(y, ref, 4e-3)
    assert ok
    yr = nn.conv3x3(x1, wt, b, x2=x2, relu=True, kernel=kernel)
    torch.cuda.synchronize()
    assert _close(yr, ref.clamp_min(0), 4e-3)[1]


@pytest.mark.parametrize("wkernel", ["mma", "umma"])
@pytest.mark.parametrize("n,h,w,cin,cout", [(2, 24, 40, 16, 32), (1, 32, 32, 48, 64), (2, 16, 24, 64, 32),
                                             (1, 18, 34, 224, 96), (2, 64, 96, 32, 32), (1, 20, 36, 128, 128)])
def test_conv3x3_backward_data_and_weight(cuda, n, h, w, cin, cout, wkernel):
    """Backward data (the forward kernel on the flipped weights) and backward
    weights (wkernel: the mma.sync or the tcgen05 kernel)."""
    import torch
    import torch.nn.functional as F

    from vulkanpbrt_gb300 import nn

    g = torch.Generator().manual_seed(7 + cin + cout)
    x = torch.randn(n, h, w, cin, generator=g).bfloat16()
    wt = (torch.randn(cout, 9, cin, generator=g) * 0.1).bfloat16()
    dy = torch.randn(n, h, w, cout, generator=g).bfloat16()
    # reference gradients in FP32 from the BF16-rounded operands
    xr = x.float().permute(0, 3, 1, 2).clone().requires_grad_(True)
    wr = wt.float().reshape(cout, 3, 3, cin).permute(0, 3, 1, 2).clone().requires_grad_(True)
    yr = F.conv2d(xr, wr, padding=1)
    yr.backward(dy.float().permute(0, 3, 1, 2))
    dx_ref = xr.grad.permute(0, 2, 3, 1)
    dw_ref = wr.grad.permute(0, 2, 3, 1).reshape(cout, 9, cin)
    # backward data: forward kernel on flipped weights
    wflip = nn.flip_weights(wt.to(cuda))
    dx = torch.empty(n, h, w, cin, device=cuda)
    nn.conv3x3(dy.to(cuda), wflip, None, out32=dx)
    dw = torch.zeros(cout, 9, cin, device=cuda)
    nn.conv3x3_wgrad(dy.to(cuda), x.to(cuda), dw, kernel=wkernel)
    torch.cuda.synchronize()
    assert nn.umma_status() == 0
    rel, ok = _close(dx, dx_ref, 1e-4)
    print(f"dgrad rel err {rel:.2e}")
    assert ok
    rel, ok = _close(dw, dw_ref, 1e-4)
    print(f"wgrad rel err {rel:.2e}")
    assert ok


@pytest.mark.parametrize("n,h,w,cin,cout", [(2, 24, 40, 16, 32), (1, 32, 32, 48, 64), (2, 16, 24, 64, 32),
                                             (1, 18, 34, 224, 96), (1, 9, 17, 128, 128), (1, 40, 24, 80, 32)])
def test_conv3x3_dgrad_tcgen05(cuda, n, h, w, cin, cout):
    """Backward data on tcgen05 (pbrt_nn_conv3x3_umma_f32: dY with the flipped
    weights, FP32 out, the input channels in slices that fit in shared memory:
    224 in four, 128 from 128 in three) against torch's FP32 gradient."""
    import torch
    import torch.nn.functional as F

    from vulkanpbrt_gb300 import nn

    g = torch.Generator().manual_seed(17 + cin + cout + h)
    wt = (torch.randn(cout, 9, cin, generator=g) * 0.1).bfloat16()
    dy = torch.randn(n, h, w, cout, generator=g).bfloat16()
    xr = torch.zeros(n, cin, h, w, requires_grad=True)
    wr = wt.float().reshape(cout, 3, 3, cin).permute(0, 3, 1, 2)
    F.conv2d(xr, wr, padding=1).backward(dy.float().permute(0, 3, 1, 2))
    dx_ref = xr.grad.permute(0, 2, 3, 1)
    wflip = nn.flip_weights(wt.to(cuda))
    dx = torch.full((n, h, w, cin), float("nan"), device=cuda)
    nn.conv3x3_umma_f32(dy.to(cuda), wflip, dx)
    assert nn.umma_status() == 0
    rel, ok = _close(dx, dx_ref, 1e-4)
    print(f"tcgen05 dgrad rel err {rel:.2e}")
    assert ok


@pytest.mark.parametrize("wkernel", ["mma", "umma"])
def test_conv3x3_wgrad_with_upsampled_concat(cuda, wkernel):
    import torch
    import torch.nn.functional as F

    from vulkanpbrt_gb300 import nn

    n, h, w, c1, c2, cout = 2, 16, 24, 32, 48, 32
    g = torch.Generator().manual_seed(3)
    x1 = torch.randn(n, h, w, c1, generator=g).bfloat16()
    x2 = torch.randn(n, h // 2, w // 2, c2, generator=g).bfloat16()
    dy = torch.randn(n, h, w, cout, generator=g).bfloat16()
    up = x2.float().repeat_interleave(2, 1).repeat_interleave(2, 2)
    xc = torch.cat([x1.float(), up], -1).permute(0, 3, 1, 2)
    wr = torch.zeros(cout, c1 + c2, 3, 3, requires_grad=True)
    F.conv2d(xc, wr, padding=1).backward(dy.float().permute(0, 3, 1, 2))
    dw_ref = wr.grad.permute(0, 2, 3, 1).reshape(cout, 9, c1 + c2)
    dw = torch.zeros(cout, 9, c1 + c2, device=cuda)
    nn.conv3x3_wgrad(dy.to(cuda), x1.to(cuda), dw, x2=x2.to(cuda), kernel=wkernel)
    torch.cuda.synchronize()
    assert nn.umma_status() == 0
    assert _close(dw, dw_ref, 1e-4)[1]
