"""The neural denoiser render module (pbrt_neural_*): its graph-captured
native forward pass against the training-side forward of the same network
(same kernels, so bit-identical), the variance gate at its extremes, and the
ablation: on a held-out view the trained network must beat BMFR on the same
1-spp frame, the untrained network and the raw 1-spp input, in relMSE
against a many-sample render."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _random_frame(g, illu, seed):
    import torch

    gen = torch.Generator().manual_seed(seed)
    H, W = g.height, g.width
    g.depth.tensor().copy_(torch.rand(H, W, 1, generator=gen) * 20)
    nrm = torch.rand(H, W, 2, generator=gen) * torch.tensor([3.14159, 6.28318])
    g.normal.tensor().copy_(nrm)
    g.albedo.tensor().copy_(torch.randint(10, 256, (H, W, 4), generator=gen, dtype=torch.uint8))
    illu.illumination_images[0].tensor().copy_(torch.rand(H, W, 4, generator=gen) ** 4 * 8)


def _params(seed):
    from vulkanpbrt_gb300 import kpunet as K

    p = K.init_params(seed)
    lay, _ = K.param_layout()
    rng = np.random.default_rng(seed)
    for key, (off, shape) in lay.items():
        if key.startswith("h") and key.endswith(".w"):
            p[off:off + int(np.prod(shape))] = rng.standard_normal(int(np.prod(shape))).astype(np.float32) * 0.2
    return p


def test_native_forward_equals_training_forward(cuda):
    import torch

    import vulkanpbrt_gb300 as vp
    from vulkanpbrt_gb300 import kpunet as K
    from vulkanpbrt_gb300.neural import NeuralDenoiser, param_count

    W, H = 200, 120
    assert param_count() == K.param_layout()[1]
    g = vp.GBuffer(W, H)
    illu = vp.IlluminationBufferDemodulatedFloat(W, H)
    _random_frame(g, illu, 1)
    p = _params(3)
    nd = NeuralDenoiser(W, H, g, illu, weights=p)
    nd.dispatch()  # tunes the per-layer kernel choice, then captures the graph
    nd.dispatch()  # graph replay
    torch.cuda.synchronize()
    got = nd.denoised.tensor()[..., :3].cpu()
    kinds = nd.conv_kernels()
    net = K.KPUNet(cuda, params=p)
    ws = net.workspace(1, 128, 208, training=False)
    ws.set_input(illu.illumination_images[0].tensor()[None], g.albedo.tensor()[None], g.normal.tensor()[None],
                 g.depth.tensor()[None, ..., 0])
    want = ws.forward(kinds)[0, :H, :W].cpu()
    torch.cuda.synchronize()
    assert torch.equal(got, want)
    # a fixed choice: every layer on the tcgen05 kernel (swizzled or plane
    # halos), then every layer on mma.sync
    for kind in ("umma", "umma_planes", "mma"):
        nd.set_conv_kernels([kind] * 18)
        nd.dispatch()
        torch.cuda.synchronize()
        assert torch.equal(nd.denoised.tensor()[..., :3].cpu(), ws.forward(kind)[0, :H, :W].cpu())
    assert torch.isfinite(got).all()


def test_variance_gate_extremes(cuda):
    import torch

    import vulkanpbrt_gb300 as vp
    from vulkanpbrt_gb300.neural import NeuralDenoiser

    W, H = 200, 120
    g = vp.GBuffer(W, H)
    illu = vp.IlluminationBufferDemodulatedFloat(W, H)
    _random_frame(g, illu, 2)
    acc = vp.AccumulationBuffer(W, H)
    bmfr = vp.BMFR(W, H, 32, 32, g, illu, acc, 256)
    pc = vp.PushConstants()
    bmfr.dispatch(pc)
    # the threshold rule on the predicted error (the learned gate is off)
    nd = NeuralDenoiser(W, H, g, illu, weights=_params(4), fallback=bmfr, threshold=-1.0, tile=32, gate_model=None)
    nd.dispatch()
    torch.cuda.synchronize()
    tiles = ((W + 31) // 32) * ((H + 31) // 32)
    assert nd.fallback_tiles() == tiles
    assert torch.equal(nd.get_final_descriptor_image().tensor().cpu(), bmfr.get_final_descriptor_image().tensor().cpu())
    assert int(nd.fallback_mask.tensor().sum()) == tiles
    nd.set_fallback(bmfr, threshold=1e30, tile=32)
    nd.dispatch()
    torch.cuda.synchronize()
    assert nd.fallback_tiles() == 0
    plain = NeuralDenoiser(W, H, g, illu, weights=_params(4))
    plain.set_conv_kernels(nd.conv_kernels())  # the same per-layer kernels, so the same bits
    plain.dispatch()
    torch.cuda.synchronize()
    assert torch.equal(nd.get_final_descriptor_image().tensor().cpu(), plain.get_final_descriptor_image().tensor().cpu())


def relmse(x, ref, albedo):
    """mean of (A x - A r)^2 / ((A r)^2 + 0.01) over pixels and channels (A: the G-buffer albedo)."""
    A = albedo[..., :3].double() / 255.0
    r = A * ref[..., :3].double()
    return (((A * x[..., :3].double() - r) ** 2) / (r * r + 0.01)).mean().item()


def test_trained_network_beats_bmfr_and_untrained(cuda):
    """Ablation on a view no training pair came from (the benchmark scene,
    seed 0): 256 x 256 window of a 1080p frame, 1 spp, reference 1024 spp."""
    import torch

    import vulkanpbrt_gb300 as vp
    from vulkanpbrt_gb300 import kpunet as K
    from vulkanpbrt_gb300 import scene as S
    from vulkanpbrt_gb300.camera import Camera, CropCamera
    from vulkanpbrt_gb300.neural import WEIGHTS, NeuralDenoiser

    if not WEIGHTS.exists():
        pytest.skip("no trained weights in the package")
    W = H = 256
    sc = S.instanced_field(seed=0, texture_size=256)
    sh = vp.SceneHandle(sc)
    g = vp.GBuffer(W, H)
    illu = vp.IlluminationBufferDemodulatedFloat(W, H)
    pipe = vp.PBRTPipeline(sh, g, illu, True, max_recursion_depth=8, min_recursion_depth=3)
    cam = Camera(sc.camera_eye, sc.camera_center, aspect=1920 / 1080)
    cc = CropCamera(cam, 1920, 1080, 832, 412, W, H)
    pc = vp.PushConstants()
    pc.set(view_inverse=cc.inv_view, proj_inverse=cc.inv_proj, prev_view=cc.view, frame_number=0)
    pipe.trace(pc)
    img = illu.illumination_images[0].tensor()
    noisy = img.clone()
    acc = vp.AccumulationBuffer(W, H)
    bmfr = vp.BMFR(W, H, 32, 32, g, illu, acc, 256)
    bmfr.dispatch(pc)
    trained = NeuralDenoiser(W, H, g, illu)
    trained.dispatch()
    untrained = NeuralDenoiser(W, H, g, illu, weights=K.init_params(0))
    untrained.dispatch()
    torch.cuda.synchronize()
    den_bmfr = bmfr.denoised.tensor()[1].float().clone()  # frame 0 writes layer 1
    den_nn = trained.denoised.tensor().clone()
    den_un = untrained.denoised.tensor().clone()
    albedo = g.albedo.tensor().clone()
    ref = torch.zeros(H, W, 3, dtype=torch.float64, device=cuda)
    spp = 1024
    for s in range(spp):
        pc.set(frame_number=1 + s)
        pipe.trace(pc)
        ref += img[..., :3]
    ref /= spp
    r = {k: relmse(v, ref, albedo) for k, v in
         {"1spp": noisy, "bmfr": den_bmfr, "untrained": den_un, "trained": den_nn}.items()}
    # the same comparison on the accumulator's output after 8 static frames
    accu = vp.Accumulator(g, illu, separate_matrices=True)
    acc_illu, abuf = accu.accumulated_illumination, accu.accumulation_buffer
    bmfr8 = vp.BMFR(W, H, 32, 32, g, acc_illu, abuf, 256)
    nn8 = NeuralDenoiser(W, H, g, acc_illu, acc_buffer=abuf)
    cm = vp.CameraMatrices(cam.view, cam.inv_view, cc.proj, cc.inv_proj)
    for f in range(8):
        pc.set(frame_number=5000 + f)
        pipe.trace(pc)
        accu.set_camera_matrices(f, cm, cm)
        vp.lib().pbrt_accumulator_dispatch(accu.ptr, None)
        bmfr8.dispatch(pc)
        nn8.dispatch()
        vp.lib().pbrt_accumulation_buffer_copy_to_back_images(abuf.ptr, g.ptr, acc_illu.ptr, None)
    torch.cuda.synchronize()
    r["bmfr_8frames"] = relmse(bmfr8.denoised.tensor()[(5007 & 1) ^ 1].float(), ref, albedo)
    r["trained_8frames"] = relmse(nn8.denoised.tensor(), ref, albedo)
    r["accumulated_8frames"] = relmse(acc_illu.illumination_images[0].tensor().float(), ref, albedo)
    nn8.calibrate()
    nn8.set_precision(8)
    nn8.dispatch()
    torch.cuda.synchronize()
    r["trained_8frames_fp8"] = relmse(nn8.denoised.tensor(), ref, albedo)
    print("relMSE vs 1024 spp:", r)
    assert r["trained_8frames_fp8"] < 1.25 * r["trained_8frames"] + 1e-3
    assert r["trained"] < r["bmfr"]
    assert r["trained"] < r["untrained"]
    assert r["trained"] < r["1spp"]
    assert r["trained_8frames"] < r["bmfr_8frames"]
