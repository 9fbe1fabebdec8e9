"""The learned tile gate of the neural denoiser against a float64 PyTorch
restatement of its features and score (no reference counterpart: the
specification's per-tile fallback from the network to BMFR).

Per 32x32 tile the kernel forms eight log features (predicted error, the
network / BMFR final-image difference, samples, noisy log-luminance
variance, depth gradient, normal spread, luminance, albedo) and a linear
score; checked: every tile whose restated score is clear of zero (|s| >
0.05) gets the same decision, the fallback count is the mask's sum, the
tiles handed to BMFR show BMFR's final pixels and the others the network's,
and a bias of +/-1000 sends all / no tiles to BMFR.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

T = 32


def _tile_sum(x, H, W):
    import torch

    th, tw = (H + T - 1) // T, (W + T - 1) // T
    xp = torch.nn.functional.pad(x[None, None], (0, tw * T - W, 0, th * T - H))
    return torch.nn.functional.avg_pool2d(xp, T, divisor_override=1).flatten()


def gate_features(var, nn_fin, bm_fin, spp, noisy, depth, nrm, alb8):
    """The kernel's eight tile features (pbrt_nn_gate_model), float64."""
    import torch

    H, W = depth.shape
    n = _tile_sum(torch.ones_like(depth), H, W)
    ts = lambda x: _tile_sum(x, H, W) / n  # noqa: E731
    e = 1e-8
    f0 = torch.log(ts(torch.exp(var)) + e)
    d = (bm_fin[..., :3].double() - nn_fin[..., :3].double()) / 255.0
    f1 = torch.log(ts((d * d).mean(-1)) + e)
    f2 = torch.log(ts(spp) + e)
    lum = 0.2126 * noisy[..., 0] + 0.7152 * noisy[..., 1] + 0.0722 * noisy[..., 2]
    ll = torch.log1p(torch.clamp(lum, min=0))
    m1, m2 = ts(ll), ts(ll * ll)
    f3 = torch.log(torch.clamp(m2 - m1 * m1, min=0) + e)
    ld = torch.log(torch.clamp(depth, 1e-3, 1e4))
    gx = torch.nn.functional.pad((ld[:, 1:] - ld[:, :-1]).abs(), (0, 1))
    gy = torch.nn.functional.pad((ld[1:] - ld[:-1]).abs(), (0, 0, 0, 1))
    f4 = torch.log(ts(gx + gy) + e)
    t_, p_ = nrm[..., 0], nrm[..., 1]
    mx, my, mz = ts(torch.sin(t_) * torch.cos(p_)), ts(torch.sin(t_) * torch.sin(p_)), ts(torch.cos(t_))
    f5 = torch.log(torch.clamp(1 - torch.sqrt(mx * mx + my * my + mz * mz), min=0) + e)
    f6 = torch.log(ts(lum) + e)
    f7 = torch.log(ts(alb8[..., :3].double().mean(-1) / 255.0) + e)
    return torch.stack([f0, f1, f2, f3, f4, f5, f6, f7], 1)


def test_learned_gate_matches_restatement(cuda):
    import torch

    import vulkanpbrt_gb300 as vp
    from vulkanpbrt_gb300 import scene as S
    from vulkanpbrt_gb300.camera import Camera
    from vulkanpbrt_gb300.neural import gate_coefficients

    sc = S.instanced_field(seed=8, instances=150, unique_meshes=12, texture_size=64, radius=8.0)
    W, H = 512, 288
    cam = Camera(sc.camera_eye, sc.camera_center, aspect=W / H)
    sh = vp.SceneHandle(sc)
    g = vp.GBuffer(W, H)
    illu = vp.IlluminationBufferDemodulatedFloat(W, H)
    pipe = vp.PBRTPipeline(sh, g, illu, True, max_recursion_depth=6, min_recursion_depth=3)
    accu = vp.Accumulator(g, illu, separate_matrices=True)
    acc_illu, abuf = accu.accumulated_illumination, accu.accumulation_buffer
    bm = vp.BMFR(W, H, 32, 32, g, acc_illu, abuf, 256)
    coef = gate_coefficients()
    nd = vp.NeuralDenoiser(W, H, g, acc_illu, fallback=bm, tile=T, acc_buffer=abuf, gate_model=coef)
    cm = vp.CameraMatrices(cam.view, cam.inv_view, cam.proj, cam.inv_proj)
    for f in range(3):
        pc = vp.PushConstants(view_inverse=cam.inv_view, proj_inverse=cam.inv_proj, prev_view=cam.view, frame_number=f)
        accu.set_camera_matrices(f, cm, vp.CameraMatrices(cam.view, cam.inv_view))
        pipe.trace(pc)
        vp.lib().pbrt_accumulator_dispatch(accu.ptr, None)
        bm.dispatch(pc)
        nd.dispatch(pc)
        if f < 2:
            vp.lib().pbrt_accumulation_buffer_copy_to_back_images(abuf.ptr, g.ptr, acc_illu.ptr, None)
    torch.cuda.synchronize()
    gated = nd.get_final_descriptor_image().tensor().clone()
    mask = nd.fallback_mask.tensor()[..., 0].clone().flatten().bool()
    count = nd.fallback_tiles()
    bm_fin = bm.get_final_descriptor_image().tensor().clone()
    # the network alone (no tile handed over): the gate's input image
    nd.set_gate_model(np.array([0.0] * 8 + [-1e3], np.float32))
    nd.dispatch(pc)
    torch.cuda.synchronize()
    assert nd.fallback_tiles() == 0
    nn_fin = nd.get_final_descriptor_image().tensor().clone()
    feats = gate_features(nd.variance.tensor()[..., 0][:H, :W].double(), nn_fin, bm_fin,
                          abuf.spp.tensor()[..., 0].double(), acc_illu.illumination_images[0].tensor()[..., :3].double(),
                          g.depth.tensor()[..., 0].double(), g.normal.tensor().double(), g.albedo.tensor())
    score = feats @ torch.from_numpy(coef[:8].astype(np.float64)).to(feats.device) + float(coef[8])
    clear = score.abs() > 0.05
    print(f"gate: {int(mask.sum())} of {mask.numel()} tiles to BMFR; scores {score.min():.3f}..{score.max():.3f}; "
          f"{int(clear.sum())} clear of zero")
    assert count == int(mask.sum())
    assert bool(((score > 0) == mask)[clear].all())
    th, tw = (H + T - 1) // T, (W + T - 1) // T
    px = mask.reshape(th, tw).repeat_interleave(T, 0).repeat_interleave(T, 1)[:H, :W]
    assert torch.equal(gated[px], bm_fin[px])
    assert torch.equal(gated[~px], nn_fin[~px])
    # all tiles
    nd.set_gate_model(np.array([0.0] * 8 + [1e3], np.float32))
    nd.dispatch(pc)
    torch.cuda.synchronize()
    assert nd.fallback_tiles() == th * tw
    assert torch.equal(nd.get_final_descriptor_image().tensor(), bm_fin)
