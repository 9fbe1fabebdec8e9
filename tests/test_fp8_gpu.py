"""FP8 (e4m3) inference path of the neural denoiser: the FP8 convolution
against a plain PyTorch FP32 convolution of the same e4m3-quantised operands
(one BF16 ulp, 4e-3 of the output scale), the weight quantiser against
torch's own e4m3 rounding (byte-exact), and the calibrated FP8 network
against the BF16 network on the same frame."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,h,w,c1,c2,cout", [(1, 24, 40, 16, 0, 32), (2, 16, 32, 48, 64, 48), (1, 20, 36, 96, 128, 96),
                                             (1, 9, 17, 32, 0, 128)])
def test_conv3x3_fp8_matches_quantised_reference(cuda, n, h, w, c1, c2, cout):
    import torch
    import torch.nn.functional as F

    from vulkanpbrt_gb300 import nn

    g = torch.Generator().manual_seed(c1 + c2 + cout)
    x1 = (torch.randn(n, h, w, c1, generator=g).abs() * 3).bfloat16()
    x2 = (torch.randn(n, h // 2, w // 2, c2, generator=g).abs()).bfloat16() if c2 else None
    cin = c1 + c2
    w32 = torch.randn(cout, 9, cin, generator=g) * 0.1
    bias = torch.randn(cout, generator=g)
    up = x2.float().repeat_interleave(2, 1).repeat_interleave(2, 2) if c2 else None
    xc = torch.cat([x1.float(), up], -1) if c2 else x1.float()
    amax = xc.abs().amax((0, 1, 2))
    xs = torch.where(amax > 0, amax / 448.0, torch.ones_like(amax))
    # device-side quantisation and convolution
    amax_d = torch.zeros(c1, device=cuda)
    nn.channel_amax(x1.to(cuda), amax_d)
    assert torch.equal(amax_d.cpu(), x1.float().abs().amax((0, 1, 2)))
    w8, ws = nn.quantize_weights_fp8(w32.to(cuda), xs.to(cuda))
    y = nn.conv3x3_fp8(x1.to(cuda), w8, ws, (1.0 / xs).to(cuda), bias.to(cuda), x2=x2.to(cuda) if c2 else None)
    torch.cuda.synchronize()
    # reference: the same e4m3 operands in FP32
    wsc = (w32 * xs).abs().amax((1, 2)) / 448.0
    w8_ref = (w32 * xs / wsc[:, None, None]).to(torch.float8_e4m3fn)
    assert torch.equal(w8.cpu(), w8_ref.view(torch.uint8))
    assert torch.allclose(ws.cpu(), wsc, rtol=1e-6)
    xq = (xc * (1.0 / xs)).to(torch.float8_e4m3fn).float()
    wt = w8_ref.float().reshape(cout, 3, 3, cin).permute(0, 3, 1, 2)
    ref = F.conv2d(xq.permute(0, 3, 1, 2), wt, padding=1).permute(0, 2, 3, 1) * wsc + bias
    scale = ref.abs().max().item()
    err = (y.float().cpu() - ref).abs().max().item()
    print(f"fp8 conv max err / scale = {err / scale:.2e}")
    assert err <= 4e-3 * scale


def test_fp8_network_close_to_bf16(cuda):
    import torch

    import vulkanpbrt_gb300 as vp
    from tests.test_neural_gpu import _params, _random_frame
    from vulkanpbrt_gb300.neural import NeuralDenoiser

    W, H = 256, 160
    g = vp.GBuffer(W, H)
    illu = vp.IlluminationBufferDemodulatedFloat(W, H)
    _random_frame(g, illu, 7)
    nd = NeuralDenoiser(W, H, g, illu, weights=_params(5))
    nd.dispatch()
    torch.cuda.synchronize()
    bf = nd.denoised.tensor().clone()
    with pytest.raises(vp.PbrtError):
        nd.set_precision(8)  # not calibrated yet
    nd.calibrate()
    nd.set_precision(8)
    nd.dispatch()
    torch.cuda.synchronize()
    f8 = nd.denoised.tensor().clone()
    assert torch.isfinite(f8).all()
    rel = (((f8[..., :3] - bf[..., :3]) ** 2) / (bf[..., :3] ** 2 + 0.01)).mean().item()
    print(f"relMSE(FP8 network, BF16 network) = {rel:.3e}")
    assert rel < 2e-2
    nd.set_precision(16)
    nd.dispatch()
    torch.cuda.synchronize()
    assert torch.equal(nd.denoised.tensor(), bf)
