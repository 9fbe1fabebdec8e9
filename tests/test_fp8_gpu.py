"""FP8 (e4m3) inference path of the neural denoiser: the FP8 convolutions
(the tcgen05 kind::f8f6f4 form and the mma.sync kernel) against a plain
PyTorch FP32 convolution of the same e4m3-quantised operands (one BF16 ulp,
4e-3 of the output scale), the fused pooling of the tcgen05 form against the
stand-alone pooling kernel (bit-exact), the weight quantiser against
torch's own e4m3 rounding (byte-exact), and the calibrated FP8 network
against the BF16 network on the same frame."""
import pytest

pytestmark = pytest.mark.gpu


def _fp8_case(n, h, w, c1, c2, cout):
    """Seeded inputs, device-quantised weights and the FP32 reference convolution of the same e4m3 operands."""
    import torch
    import torch.nn.functional as F

    from vulkanpbrt_gb300 import nn

    cuda = torch.device("cuda:0")
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
    w8, ws = nn.quantize_weights_fp8(w32.to(cuda), xs.to(cuda))
    wsc = (w32 * xs).abs().amax((1, 2)) / 448.0
    w8_ref = (w32 * xs / wsc[:, None, None]).to(torch.float8_e4m3fn)
    assert torch.equal(w8.cpu(), w8_ref.view(torch.uint8))
    assert torch.allclose(ws.cpu(), wsc, rtol=1e-6)
    xq = (xc * (1.0 / xs)).to(torch.float8_e4m3fn).float()
    wt = w8_ref.float().reshape(cout, 3, 3, cin).permute(0, 3, 1, 2)
    ref = F.conv2d(xq.permute(0, 3, 1, 2).to(cuda), wt.to(cuda), padding=1).permute(0, 2, 3, 1).cpu() * wsc + bias
    args = dict(x1=x1.to(cuda), w8=w8, wscale=ws, inv_xscale=(1.0 / xs).to(cuda), bias=bias.to(cuda),
                x2=x2.to(cuda) if c2 else None)
    return args, ref


def _check(y, ref, what):
    scale = ref.abs().max().item()
    err = (y.float().cpu() - ref).abs().max().item()
    print(f"{what}: fp8 conv max err / scale = {err / scale:.2e}")
    assert err <= 4e-3 * scale


@pytest.mark.parametrize("kernel", ["auto", "mma"])
@pytest.mark.parametrize("n,h,w,c1,c2,cout", [(1, 24, 40, 16, 0, 32), (2, 16, 32, 48, 64, 48), (1, 20, 36, 96, 128, 96),
                                             (1, 9, 17, 32, 0, 128)])
def test_conv3x3_fp8_matches_quantised_reference(cuda, n, h, w, c1, c2, cout, kernel):
    import torch

    from vulkanpbrt_gb300 import nn

    x1 = (torch.randn(n, h, w, c1, generator=torch.Generator().manual_seed(c1 + c2 + cout)).abs() * 3).bfloat16()
    amax_d = torch.zeros(c1, device=cuda)
    nn.channel_amax(x1.to(cuda), amax_d)
    assert torch.equal(amax_d.cpu(), x1.float().abs().amax((0, 1, 2)))
    args, ref = _fp8_case(n, h, w, c1, c2, cout)
    y = nn.conv3x3_fp8(**args, kernel=kernel)
    torch.cuda.synchronize()
    _check(y, ref, kernel)


# the tcgen05 form alone: the padded 16-channel input, the upsampled second
# input, Cout 128, 160 input channels (two stages in 204 KB of shared
# memory), and a frame of more tiles than resident CTAs (every input stage
# and accumulator buffer reused several times)
@pytest.mark.parametrize("n,h,w,c1,c2,cout", [(1, 24, 40, 16, 0, 32), (2, 32, 64, 48, 64, 48), (1, 9, 17, 32, 0, 128),
                                             (1, 40, 24, 80, 0, 96), (1, 48, 64, 64, 96, 64),
                                             (4, 256, 256, 32, 0, 32)])
def test_conv3x3_fp8_umma(cuda, n, h, w, c1, c2, cout):
    import torch

    from vulkanpbrt_gb300 import nn

    args, ref = _fp8_case(n, h, w, c1, c2, cout)
    y = nn.conv3x3_fp8(**args, kernel="umma")
    assert nn.umma_status() == 0
    _check(y, ref, "umma")
    if c2:  # the upsampled input's TMA box and its cp.async gathers: the same bits
        y_g = nn.conv3x3_fp8(**args, kernel="umma", box=False)
        assert nn.umma_status() == 0
        assert torch.equal(y, y_g)
    # the same operands on the mma.sync kernel: the two agree to the BF16 rounding of the output
    y_mma = nn.conv3x3_fp8(**args, kernel="mma")
    torch.cuda.synchronize()
    d = (y.float() - y_mma.float()).abs().max().item()
    assert d <= 8e-3 * ref.abs().max().item()


def test_conv3x3_fp8_umma_full_frame(cuda):
    """The decoder's full-resolution concatenated layer (32 + 48 -> 32) at
    1088x1920: the FP8 form with two stages and two CTAs an SM."""
    import torch

    from vulkanpbrt_gb300 import nn

    args, ref = _fp8_case(1, 1088, 1920, 32, 48, 32)
    y = nn.conv3x3_fp8(**args, kernel="umma")
    assert nn.umma_status() == 0
    _check(y, ref, "umma full frame")


def test_conv3x3_fp8_fallback_records_no_error(cuda):
    """A layer the tcgen05 form does not take (224 input channels) runs on
    the mma.sync kernel without leaving an error message behind."""
    import torch

    import vulkanpbrt_gb300 as vp
    from vulkanpbrt_gb300 import nn
    from vulkanpbrt_gb300._abi import last_error

    bad = torch.zeros(1, 4, 4, 8, dtype=torch.bfloat16, device=cuda)  # 8 channels: rejected
    w8 = torch.zeros(16, 9, 8, dtype=torch.uint8, device=cuda)
    one = torch.ones(16, device=cuda)
    with pytest.raises(vp.PbrtError):
        nn.conv3x3_fp8(bad, w8, one, one[:8])
    msg = last_error()
    assert "bad arguments" in msg
    args, ref = _fp8_case(1, 20, 36, 96, 128, 96)
    y = nn.conv3x3_fp8(**args)
    torch.cuda.synchronize()
    _check(y, ref, "auto (mma.sync)")
    assert last_error() == msg


def test_conv3x3_fp8_umma_pooled(cuda):
    import torch

    from vulkanpbrt_gb300 import nn

    args, _ = _fp8_case(2, 64, 48, 32, 0, 48)
    y0 = nn.conv3x3_fp8(**args, relu=True, kernel="umma")
    y, pooled = nn.conv3x3_fp8(**args, relu=True, pooled=True)
    assert nn.umma_status() == 0
    assert torch.equal(y, y0)
    assert torch.equal(pooled, nn.avgpool2(y, torch.empty_like(pooled)))
    import vulkanpbrt_gb300 as vp

    a2, _ = _fp8_case(1, 24, 40, 16, 0, 32)  # a frame that does not divide into 16 x 8 tiles
    with pytest.raises(vp.PbrtError):
        nn.conv3x3_fp8(**a2, pooled=True)


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
    mixed = nd.fp8_layers()
    assert not mixed[0]
    nd.set_fp8_layers([False] + [True] * 17)  # every layer but the first in e4m3
    nd.set_precision(8)
    nd.dispatch()
    torch.cuda.synchronize()
    f8 = nd.denoised.tensor().clone()
    assert torch.isfinite(f8).all()
    rel = (((f8[..., :3] - bf[..., :3]) ** 2) / (bf[..., :3] ** 2 + 0.01)).mean().item()
    print(f"relMSE(FP8 network, BF16 network) = {rel:.3e}; calibration's e4m3 layers {mixed}")
    assert rel < 2e-2
    with pytest.raises(vp.PbrtError):
        nd.set_fp8_layers([True] * 18)  # the first convolution stays BF16
    nd.set_fp8_layers([False] * 18)  # no e4m3 layer: the BF16 network's bits
    nd.dispatch()
    torch.cuda.synchronize()
    assert torch.equal(nd.denoised.tensor(), bf)
    nd.set_fp8_layers(mixed)
    nd.set_precision(16)
    nd.dispatch()
    torch.cuda.synchronize()
    assert torch.equal(nd.denoised.tensor(), bf)
