"""The tcgen05 convolutions (accumulator in tensor memory; the per-tile
form, and the persistent form with its input halo from a TMA load or from
cp.async gathers; the warp-specialised form with the first input's halo as
swizzled whole-pixel rows or 8-channel planes, and the upsampled second
input from a TMA load of its half-resolution box or from cp.async gathers)
against torch's FP32 conv2d on the same BF16 operands:
within one BF16 ulp (4e-3) of the output scale, no error flag from their
bounded waits. Larger images exercise the persistent form's tile loop."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,h,w,c1,c2,cout", [(1, 16, 8, 16, 0, 32), (2, 24, 40, 16, 0, 32), (1, 32, 32, 32, 0, 48),
                                             (1, 16, 48, 48, 32, 48), (1, 20, 36, 64, 0, 64),
                                             (1, 18, 34, 96, 128, 96), (1, 9, 17, 128, 0, 128),
                                             (1, 34, 46, 32, 48, 32), (2, 136, 240, 32, 48, 32),
                                             (2, 128, 256, 48, 64, 48),
                                             (1, 128, 200, 16, 0, 32)])
@pytest.mark.parametrize("mode", ["ws", "ws_planes", "ws_nobox", "ws_gather", "tma", "persistent", "tile"])
def test_conv3x3_umma_forward(cuda, n, h, w, c1, c2, cout, mode):
    import torch

    from tests.test_nn_conv_gpu import _close, _ref_conv
    from vulkanpbrt_gb300 import nn

    g = torch.Generator().manual_seed(n * 100 + c1 + c2 + cout + h)
    x1 = torch.randn(n, h, w, c1, generator=g).bfloat16().to(cuda)
    x2 = torch.randn(n, h // 2, w // 2, c2, generator=g).bfloat16().to(cuda) if c2 else None
    wt = (torch.randn(cout, 9, c1 + c2, generator=g) * 0.1).bfloat16().to(cuda)
    b = torch.randn(cout, generator=g).float().to(cuda)
    kw = dict(persistent=mode != "tile", tma=mode in ("ws", "ws_planes", "ws_nobox", "tma"),
              specialised=mode.startswith("ws"), box=mode != "ws_nobox", swizzle=mode != "ws_planes")
    y = nn.conv3x3_umma(x1, wt, b, x2=x2, relu=False, **kw)
    yr = nn.conv3x3_umma(x1, wt, b, x2=x2, relu=True, **kw)
    assert nn.umma_status() == 0
    ref = _ref_conv(x1, wt, b, x2)
    rel, ok = _close(y, ref, 4e-3)
    print(f"umma conv rel err {rel:.2e}")
    assert ok
    assert _close(yr, ref.clamp_min(0), 4e-3)[1]
    if mode == "ws":
        # the first input's halo as swizzled pixel rows (default) or as
        # 8-channel planes: the same operands, MMAs and order, the same bits
        assert torch.equal(y, nn.conv3x3_umma(x1, wt, b, x2=x2, relu=False, **dict(kw, swizzle=False)))


@pytest.mark.parametrize("c1,c2", [(32, 48), (32, 0)])
def test_conv3x3_umma_full_frame(cuda, c1, c2):
    """The full-resolution decoder / encoder shapes at 1088x1920, where the
    warp-specialised form trades stages for resident CTAs (two stages: two
    CTAs an SM with the upsampled input, four without)."""
    import torch

    from tests.test_nn_conv_gpu import _close, _ref_conv
    from vulkanpbrt_gb300 import nn

    g = torch.Generator(device=cuda).manual_seed(c1 + c2)
    h, w, cout = 1088, 1920, 32
    x1 = torch.randn(1, h, w, c1, device=cuda, generator=g).bfloat16()
    x2 = torch.randn(1, h // 2, w // 2, c2, device=cuda, generator=g).bfloat16() if c2 else None
    wt = (torch.randn(cout, 9, c1 + c2, device=cuda, generator=g) * 0.1).bfloat16()
    b = torch.randn(cout, device=cuda, generator=g)
    y = nn.conv3x3_umma(x1, wt, b, x2=x2)
    assert nn.umma_status() == 0
    rel, ok = _close(y, _ref_conv(x1, wt, b, x2), 4e-3)
    print(f"full-frame umma conv rel err {rel:.2e}")
    assert ok
    if c2:  # the upsampled input's TMA box and its cp.async gathers: the same bits
        assert torch.equal(y, nn.conv3x3_umma(x1, wt, b, x2=x2, box=False))
    # swizzled pixel rows against 8-channel planes for the first input: the same bits
    assert torch.equal(y, nn.conv3x3_umma(x1, wt, b, x2=x2, swizzle=False))


@pytest.mark.parametrize("n,h,w,c1,cout", [(1, 32, 48, 16, 32), (2, 64, 40, 32, 48), (1, 48, 64, 48, 64),
                                          (1, 272, 480, 48, 64)])
def test_conv3x3_umma_pooled(cuda, n, h, w, c1, cout):
    """The warp-specialised convolution with the next level's 2x2 average
    pooling in its epilogue: the same output bits as without it, and the
    same pooled bits as the stand-alone pooling kernel on that output."""
    import torch

    from vulkanpbrt_gb300 import nn

    g = torch.Generator().manual_seed(h + w + c1)
    x1 = torch.randn(n, h, w, c1, generator=g).bfloat16().to(cuda)
    wt = (torch.randn(cout, 9, c1, generator=g) * 0.1).bfloat16().to(cuda)
    b = torch.randn(cout, generator=g).float().to(cuda)
    y, pooled = nn.conv3x3_umma_pooled(x1, wt, b, relu=True)
    y_plain = nn.conv3x3_umma(x1, wt, b, relu=True)
    p_ref = torch.empty_like(pooled)
    nn.avgpool2(y_plain, p_ref)
    torch.cuda.synchronize()
    assert nn.umma_status() == 0
    assert torch.equal(y, y_plain)
    assert torch.equal(pooled, p_ref)
    y_pl, pooled_pl = nn.conv3x3_umma_pooled(x1, wt, b, relu=True, swizzle=False)
    assert torch.equal(y, y_pl) and torch.equal(pooled, pooled_pl)
