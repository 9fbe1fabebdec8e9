"""The learned tile gate of the neural denoiser against a float64 PyTorch
restatement (no reference counterpart: the specification's per-tile
fallback from the network to BMFR, here a choice of blend).

Per 32x32 tile the kernel forms eight log features (predicted error, the
network / BMFR final-image difference, samples, noisy log-luminance
variance, depth gradient, normal spread, luminance, albedo) and four linear
predictions of the error change of showing alpha * network + (1 - alpha) *
BMFR (alpha 0.75, 0.5, 0.25, 0); the tile takes the lowest prediction below
zero, else the network. Checked: the same choice on every tile whose two
best predictions are clear of each other; the count of blended tiles; the
blended tiles' denoised values (the FP32 blend of the network output and
BMFR's denoised layer of this frame) and final pixels (BMFR's own pixels at
alpha 0, else the blend remodulated and tone mapped within 1 LSB); the
other tiles unchanged; a model that always predicts alpha 0 shows BMFR's
final image exactly.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

T = 32


def _frame(vp, sc, W, H, gate_model):
    import torch

    from vulkanpbrt_gb300.camera import Camera

    cam = Camera(sc.camera_eye, sc.camera_center, aspect=W / H)
    sh = vp.SceneHandle(sc)
    g = vp.GBuffer(W, H)
    illu = vp.IlluminationBufferDemodulatedFloat(W, H)
    pipe = vp.PBRTPipeline(sh, g, illu, True, max_recursion_depth=6, min_recursion_depth=3)
    accu = vp.Accumulator(g, illu, separate_matrices=True)
    acc_illu, abuf = accu.accumulated_illumination, accu.accumulation_buffer
    bm = vp.BMFR(W, H, 32, 32, g, acc_illu, abuf, 256)
    nd = vp.NeuralDenoiser(W, H, g, acc_illu, fallback=bm, tile=T, acc_buffer=abuf, gate_model=gate_model)
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
    return dict(g=g, acc_illu=acc_illu, abuf=abuf, bm=bm, nd=nd, pc=pc, keep=(sh, pipe, accu, illu))


def test_learned_gate_matches_restatement(cuda):
    import torch

    import vulkanpbrt_gb300 as vp
    from vulkanpbrt_gb300 import scene as S
    from vulkanpbrt_gb300.gate_fit import tile_features
    from vulkanpbrt_gb300.neural import gate_coefficients

    sc = S.instanced_field(seed=8, instances=150, unique_meshes=12, texture_size=64, radius=8.0)
    W, H = 512, 288
    coef = gate_coefficients()
    assert coef.shape == (36,)
    r = _frame(vp, sc, W, H, coef)
    g, bm, nd, abuf, acc_illu, pc = r["g"], r["bm"], r["nd"], r["abuf"], r["acc_illu"], r["pc"]
    gated_fin = nd.get_final_descriptor_image().tensor().clone()
    gated_den = nd.denoised.tensor()[..., :3].clone()
    mask = nd.fallback_mask.tensor()[..., 0].clone().flatten().long()
    count = nd.fallback_tiles()
    bm_fin = bm.get_final_descriptor_image().tensor().clone()
    bm_den = bm.denoised.tensor()[(pc.value.frame_number & 1) ^ 1][..., :3].float()
    # the network alone: the gate's inputs
    nd.set_gate_model(None)
    nd.set_fallback(bm, threshold=1e30, tile=T)
    nd.dispatch(pc)
    torch.cuda.synchronize()
    nn_fin = nd.get_final_descriptor_image().tensor().clone()
    nn_den = nd.denoised.tensor()[..., :3].clone()
    feats, _ = tile_features(nd.variance.tensor()[..., 0][:H, :W].double(), nn_fin, bm_fin,
                             abuf.spp.tensor()[..., 0].double(), acc_illu.illumination_images[0].tensor()[..., :3].double(),
                             g.depth.tensor()[..., 0].double(), g.normal.tensor().double(), g.albedo.tensor())
    C = torch.from_numpy(coef.reshape(4, 9).astype(np.float64)).to(feats.device)
    pred = torch.cat([torch.zeros_like(feats[:, :1]), feats @ C[:, :8].T + C[:, 8]], 1)
    srt = pred.sort(1).values
    clear = (srt[:, 1] - srt[:, 0]) > 1e-4 * pred.abs().max()
    choice = pred.argmin(1)
    print(f"gate: tiles per alpha 1/.75/.5/.25/0: {torch.bincount(mask, minlength=5).tolist()}; "
          f"{int(clear.sum())} of {mask.numel()} clear")
    assert count == int((mask > 0).sum())
    assert bool((choice == mask)[clear].all())
    th, tw = (H + T - 1) // T, (W + T - 1) // T
    per_px = mask.reshape(th, tw).repeat_interleave(T, 0).repeat_interleave(T, 1)[:H, :W]
    alpha = (1.0 - 0.25 * per_px.float())[..., None]
    blend = nn_den * alpha + bm_den * (1 - alpha)
    keep = per_px == 0
    assert torch.equal(gated_fin[keep], nn_fin[keep]) and torch.equal(gated_den[keep], nn_den[keep])
    assert torch.allclose(gated_den[~keep], blend[~keep], rtol=1e-6, atol=1e-6)
    full = per_px == 4
    assert torch.equal(gated_fin[full], bm_fin[full])
    part = (per_px > 0) & (per_px < 4)
    a = g.albedo.tensor()[..., :3].float() / 255.0 + 1e-6
    tm = torch.clamp(torch.clamp(a * blend, min=0) ** 0.454545, 0, 1)
    want = torch.floor(tm * 255.0 + 0.5)[..., [2, 1, 0]]
    assert (gated_fin[..., :3][part].float() - want[part]).abs().max().item() <= 1.0


def test_gate_always_bmfr_shows_bmfr(cuda):
    import torch

    import vulkanpbrt_gb300 as vp
    from vulkanpbrt_gb300 import scene as S

    sc = S.instanced_field(seed=9, instances=80, unique_meshes=8, texture_size=64, radius=8.0)
    W, H = 320, 192
    always = np.zeros(36, np.float32)
    always[8::9] = [1.0, 1.0, 1.0, -1.0]  # only alpha 0 predicts an error drop
    r = _frame(vp, sc, W, H, always)
    nd, bm = r["nd"], r["bm"]
    assert nd.fallback_tiles() == ((W + T - 1) // T) * ((H + T - 1) // T)
    assert int(nd.fallback_mask.tensor().min()) == 4
    assert torch.equal(nd.get_final_descriptor_image().tensor(), bm.get_final_descriptor_image().tensor())
