"""FP32 helper kernels of the neural denoiser against plain PyTorch FP32 on the
CPU: input features, pooling and its backward, the ReLU/bias backward, the
concat/upsample backward, the kernel-prediction heads (forward and
backward), the relMSE loss, Adam and the final composition. Tolerances are
written per test: 1e-5 relative for exact FP32 restatements, 1e-4 where the
summation order differs, one BF16 ulp (8e-3) for BF16 outputs."""
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a = a.detach().float().cpu()
    b = b.detach().float().cpu()
    return (a - b).abs().max().item() / (b.abs().max().item() + 1e-12)


def _inputs(n, h, w, seed=0):
    import torch

    g = torch.Generator().manual_seed(seed)
    illum = torch.rand(n, h, w, 4, generator=g) * 4.0
    illum[..., 0] -= 0.5  # a few negatives (clamped)
    albedo = torch.randint(0, 256, (n, h, w, 4), generator=g, dtype=torch.uint8)
    normal = torch.rand(n, h, w, 2, generator=g) * torch.tensor([3.14159, 6.28318])
    depth = torch.rand(n, h, w, generator=g) * 50.0
    return illum, albedo, normal, depth


def test_features_match_reference(cuda):
    import torch

    from tests import kpunet_reference as ref
    from vulkanpbrt_gb300 import nn

    n, h, w, ph, pw = 2, 27, 41, 32, 48
    illum, albedo, normal, depth = _inputs(n, h, w)
    feat = torch.empty(n, ph, pw, 16, dtype=torch.bfloat16, device=cuda)
    rad = torch.empty(n, ph, pw, 3, device=cuda)
    nn.features(illum.to(cuda), albedo.to(cuda), normal.to(cuda), depth.to(cuda), feat, rad)
    # half-precision illumination input too
    feat16 = torch.empty_like(feat)
    rad16 = torch.empty_like(rad)
    nn.features(illum.half().to(cuda), albedo.to(cuda), normal.to(cuda), depth.to(cuda), feat16, rad16)
    torch.cuda.synchronize()
    f_ref, r_ref = ref.features(illum, albedo, normal, depth, ph, pw)
    assert _rel(rad, r_ref) < 1e-6
    assert (feat.float().cpu() - f_ref).abs().max().item() < 8e-3 * 4
    assert _rel(rad16, ref.features(illum.half().float(), albedo, normal, depth, ph, pw)[1]) < 1e-6


def test_pool_relu_split_backward(cuda):
    import torch

    from tests import kpunet_reference as ref
    from vulkanpbrt_gb300 import nn

    g = torch.Generator().manual_seed(1)
    n, h, w, c1, c2 = 2, 16, 24, 32, 48
    x = torch.randn(n, h, w, c1, generator=g)
    xb = x.bfloat16()
    y = torch.empty(n, h // 2, w // 2, c1, dtype=torch.bfloat16, device=cuda)
    nn.avgpool2(xb.to(cuda), y)
    y32 = torch.empty(n, h // 2, w // 2, c1, device=cuda)
    nn.avgpool2(x.to(cuda), y32)
    dy = torch.randn(n, h // 2, w // 2, c1, generator=g)
    dx = torch.ones(n, h, w, c1, device=cuda)
    nn.avgpool2_bwd_add(dy.to(cuda), dx)
    # relu backward with bias gradient
    ya = torch.randn(n, h, w, c1, generator=g).bfloat16()
    dya = torch.randn(n, h, w, c1, generator=g)
    gm = torch.empty(n, h, w, c1, dtype=torch.bfloat16, device=cuda)
    db = torch.zeros(c1, device=cuda)
    nn.relu_bwd(dya.to(cuda), ya.to(cuda), gm, db)
    # concat / upsample backward
    dcat = torch.randn(n, h, w, c1 + c2, generator=g)
    dx1 = torch.zeros(n, h, w, c1, device=cuda)
    dx2 = torch.zeros(n, h // 2, w // 2, c2, device=cuda)
    nn.split_upsum(dcat.to(cuda), c1, dx1, dx2)
    torch.cuda.synchronize()
    assert _rel(y, ref.pool(xb.float())) < 8e-3
    assert _rel(y32, ref.pool(x)) < 1e-6
    xr = torch.zeros(n, h, w, c1, requires_grad=True)
    ref.pool(xr).backward(dy)
    assert _rel(dx, xr.grad + 1) < 1e-6
    gm_ref = (dya * (ya.float() > 0)).bfloat16()
    assert torch.equal(gm.cpu(), gm_ref)
    assert _rel(db, gm_ref.float().sum((0, 1, 2))) < 1e-4
    x1r = torch.zeros(n, h, w, c1, requires_grad=True)
    x2r = torch.zeros(n, h // 2, w // 2, c2, requires_grad=True)
    torch.cat([x1r, ref.up(x2r)], -1).backward(dcat)
    assert _rel(dx1, x1r.grad) < 1e-6 and _rel(dx2, x2r.grad) < 1e-5


@pytest.mark.parametrize("c", [48, 96, 128])
def test_relu_backward_channel_groups(cuda, c):
    """ReLU backward at the network's other widths (8-channel groups: 6, 12,
    16 a pixel) over more pixels than one block's first pass."""
    import torch

    from vulkanpbrt_gb300 import nn

    g = torch.Generator().manual_seed(c)
    n, h, w = 1, 96, 160
    ya = torch.randn(n, h, w, c, generator=g).bfloat16()
    dya = torch.randn(n, h, w, c, generator=g)
    gm = torch.empty(n, h, w, c, dtype=torch.bfloat16, device=cuda)
    db = torch.zeros(c, device=cuda)
    nn.relu_bwd(dya.to(cuda), ya.to(cuda), gm, db)
    torch.cuda.synchronize()
    gm_ref = (dya * (ya.float() > 0)).bfloat16()
    assert torch.equal(gm.cpu(), gm_ref)
    assert _rel(db, gm_ref.float().sum((0, 1, 2))) < 1e-4


@pytest.mark.parametrize("n,h,w", [(2, 12, 20), (1, 10, 14)])
@pytest.mark.parametrize("scale,k,c", [(2, 25, 64), (1, 26, 48), (0, 27, 32)])
def test_kp_head_forward_backward(cuda, scale, k, c, n, h, w):
    """The heads (forward: the 1x1 convolution on the tensor cores with the
    weights split in three BF16 parts, 16 pixels a warp, a partial last group
    at 10x14) against the FP32 restatement."""
    import torch

    from tests import kpunet_reference as ref
    from vulkanpbrt_gb300 import nn

    g = torch.Generator().manual_seed(10 + k + h)
    Fm = torch.randn(n, h, w, c, generator=g).bfloat16()
    Wh = torch.randn(k, c, generator=g) * 0.3
    bh = torch.randn(k, generator=g) * 0.1
    R = torch.rand(n, h, w, 3, generator=g) * 3
    coarse = torch.rand(n, h // 2, w // 2, 3, generator=g) if k > 25 else None
    dout = torch.randn(n, h, w, 3, generator=g)
    dvar = torch.randn(n, h, w, generator=g) if k == 27 else None
    dev = {t: None if v is None else v.to(cuda) for t, v in dict(F=Fm, W=Wh, b=bh, R=R, c=coarse, do=dout,
                                                                dv=dvar).items()}
    out = torch.empty(n, h, w, 3, device=cuda)
    kw = torch.empty(n, h, w, 25, device=cuda)
    filt = torch.empty(n, h, w, 3, device=cuda)
    alpha = torch.empty(n, h, w, device=cuda) if coarse is not None else None
    var = torch.empty(n, h, w, device=cuda) if k == 27 else None
    nn.kp_head(dev["F"], dev["W"], dev["b"], dev["R"], out, coarse=dev["c"], kw=kw, filt=filt, alpha=alpha, var=var)
    dF = torch.zeros(n, h, w, c, device=cuda)
    dW = torch.zeros(k, c, device=cuda)
    db = torch.zeros(k, device=cuda)
    dc = torch.zeros(n, h // 2, w // 2, 3, device=cuda) if coarse is not None else None
    nn.kp_head_bwd(dev["F"], dev["W"], dev["b"], dev["R"], kw, filt, dev["do"], dF, dW, db, coarse=dev["c"],
                   alpha=alpha, dvar=dev["dv"], dcoarse=dc)
    torch.cuda.synchronize()
    Fr = Fm.float().requires_grad_(True)
    Wr = Wh.clone().requires_grad_(True)
    br = bh.clone().requires_grad_(True)
    cr = coarse.clone().requires_grad_(True) if coarse is not None else None
    o_ref, v_ref = ref.head(Fr, Wr, br, R, cr)
    assert _rel(out, o_ref) < 1e-5
    if var is not None:
        assert _rel(var, v_ref) < 1e-5
    obj = (o_ref * dout).sum() + ((v_ref * dvar).sum() if dvar is not None else 0)
    obj.backward()
    assert _rel(dF, Fr.grad) < 1e-4
    assert _rel(dW, Wr.grad) < 1e-4
    assert _rel(db, br.grad) < 1e-4
    if coarse is not None:
        assert _rel(dc, cr.grad) < 1e-5


def test_relmse_loss_and_gradient(cuda):
    import torch

    from tests import kpunet_reference as ref
    from vulkanpbrt_gb300 import nn

    g = torch.Generator().manual_seed(5)
    n, h, w, ph, pw = 2, 27, 41, 32, 48
    out = torch.rand(n, ph, pw, 3, generator=g) * 2
    var = torch.randn(n, ph, pw, generator=g)
    target = torch.rand(n, h, w, 3, generator=g) * 2
    albedo = torch.randint(0, 256, (n, h, w, 4), generator=g, dtype=torch.uint8)
    dout = torch.empty(n, ph, pw, 3, device=cuda)
    dvar = torch.empty(n, ph, pw, device=cuda)
    loss = torch.zeros(2, device=cuda)
    nn.relmse_loss(out.to(cuda), target.to(cuda), albedo.to(cuda), dout, loss, var=var.to(cuda), dvar=dvar,
                   var_weight=0.1)
    torch.cuda.synchronize()
    o = out.clone().requires_grad_(True)
    v = var.clone().requires_grad_(True)
    lm, lv, total = ref.loss(o, v, target, albedo, 0.1)
    total.backward()
    lc = loss.cpu()
    assert abs(lc[0].item() - lm.item()) <= 1e-5 * lm.item()
    assert abs(lc[1].item() - lv.item()) <= 1e-4 * lv.item()
    assert _rel(dout, o.grad) < 1e-5
    assert _rel(dvar, v.grad) < 1e-4


def test_adam_step(cuda):
    import torch

    g = torch.Generator().manual_seed(2)
    from vulkanpbrt_gb300 import nn

    n = 10007
    w = torch.randn(n, generator=g)
    m = torch.randn(n, generator=g) * 0.01
    v = torch.rand(n, generator=g) * 0.01
    grad = torch.randn(n, generator=g)
    wd, md, vd = w.to(cuda), m.to(cuda), v.to(cuda)
    w16 = torch.empty(n, dtype=torch.bfloat16, device=cuda)
    nn.adam(wd, grad.to(cuda), md, vd, 7, lr=1e-3, w_bf16=w16)
    torch.cuda.synchronize()
    b1, b2 = torch.tensor(0.9), torch.tensor(0.999)  # FP32 constants, as the kernel has them
    m2 = b1 * m + (1 - b1) * grad
    v2 = b2 * v + (1 - b2) * grad * grad
    w2 = w - 1e-3 * (m2 / (1 - b1 ** 7)) / ((v2 / (1 - b2 ** 7)).sqrt() + 1e-8)
    assert _rel(md, m2) < 1e-6 and _rel(vd, v2) < 1e-6, (_rel(md, m2), _rel(vd, v2))
    assert (wd.cpu() - w2).abs().max().item() < 1e-6
    assert torch.equal(w16.cpu(), wd.cpu().bfloat16())


def test_compose_and_variance_gate(cuda):
    import torch

    from vulkanpbrt_gb300 import nn

    g = torch.Generator().manual_seed(9)
    h, w, ph, pw, tile = 70, 100, 80, 112, 32
    out = torch.rand(ph, pw, 3, generator=g) * 2
    albedo = torch.randint(0, 256, (h, w, 4), generator=g, dtype=torch.uint8)
    fallback = torch.randint(0, 256, (h, w, 4), generator=g, dtype=torch.uint8)
    var = torch.full((ph, pw), -9.0)
    var[:32, 32:64] = 3.0        # tile (1, 0): mean exp(3) > 1
    var[64:70, 96:100] = 4.0     # tile (3, 2), partial 6 x 4 tile: over the threshold only if edges count
    var[70:, :] = 50.0           # padding rows: must not count
    tiles_x, tiles_y = (w + tile - 1) // tile, (h + tile - 1) // tile
    mask = torch.zeros(tiles_x * tiles_y, dtype=torch.uint8, device=cuda)
    count = torch.zeros(1, dtype=torch.int32, device=cuda)
    nn.gate(var.to(cuda), w, h, 1.0, tile, mask, count)
    final = torch.empty(h, w, 4, dtype=torch.uint8, device=cuda)
    den = torch.empty(h, w, 4, device=cuda)
    nn.compose(out.to(cuda), albedo.to(cuda), final, mask=mask, tile=tile, fallback=fallback.to(cuda), denoised=den)
    torch.cuda.synchronize()
    want = torch.zeros(tiles_y, tiles_x, dtype=torch.uint8)
    for ty in range(tiles_y):
        for tx in range(tiles_x):
            blk = var[ty * tile:min(h, (ty + 1) * tile), tx * tile:min(w, (tx + 1) * tile)]
            want[ty, tx] = int(blk.exp().mean().item() > 1.0)
    assert torch.equal(mask.cpu().view(tiles_y, tiles_x), want)
    assert int(count.item()) == int(want.sum())
    A = albedo[..., :3].float() / 255 + 1e-6
    t = (A * out[:h, :w]).clamp_min(0).pow(0.454545).clamp(0, 1)
    bgra = torch.floor(t * 255 + 0.5).to(torch.uint8).flip(-1)
    gate_px = want.repeat_interleave(tile, 0).repeat_interleave(tile, 1)[:h, :w].bool()
    fc = final.cpu()
    assert torch.equal(fc[gate_px], fallback[gate_px])
    assert (fc[~gate_px][:, :3].int() - bgra[~gate_px].int()).abs().max().item() <= 1
    assert _rel(den[..., :3], out[:h, :w]) < 1e-6
