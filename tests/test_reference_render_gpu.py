"""Pins the many-sample GPU render that relMSE is measured against: on a
crop of the 640x360 Cornell-box frame (depth 4, no Russian roulette), the
mean of 4096 one-sample GPU frames of the demodulated illumination is
compared with the FP64 CPU oracle's 4096-sample mean over the same RNG
streams (same frame numbers, same pixels). The two estimators are the same,
so their relMSE is far below the relMSE between any denoiser and either of
them; the tolerance is 1e-3."""
import numpy as np
import pytest

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


def test_gpu_4096spp_mean_matches_fp64_oracle(cuda, oracle):
    import torch

    import vulkanpbrt_gb300 as vp
    from vulkanpbrt_gb300 import scene as S
    from vulkanpbrt_gb300.camera import CropCamera, col_major, default_camera

    sc = S.cornell_spheres(seed=1)
    full = default_camera(640, 360)
    W, H, spp, f0 = 48, 32, 4096, 11
    cam = CropCamera(full, 640, 360, 300, 170, W, H)
    sh = vp.SceneHandle(sc)
    g = vp.GBuffer(W, H)
    illu = vp.IlluminationBufferDemodulatedFloat(W, H)
    pipe = vp.PBRTPipeline(sh, g, illu, True, max_recursion_depth=4, min_recursion_depth=4)
    pc = vp.PushConstants(view_inverse=cam.inv_view, proj_inverse=cam.inv_proj, prev_view=cam.view, frame_number=f0)
    img = illu.illumination_images[0].tensor()
    acc = torch.zeros(H, W, 3, dtype=torch.float64, device=cuda)
    for s in range(spp):
        pc.set(frame_number=f0 + s)
        pipe.trace(pc)
        acc += img[..., :3]
    gpu = (acc / spp).cpu().numpy()
    albedo = g.albedo.tensor()[..., :3].cpu().numpy().astype(np.float64) / 255.0
    ref = oracle.render(oracle.OracleScene(sc), W, H, col_major(cam.inv_view), col_major(cam.inv_proj), frame=f0,
                        min_depth=4, max_depth=4, precision=64, frames=spp)
    r = albedo * ref["illum"][..., :3].astype(np.float64)
    x = albedo * gpu
    rel = float((((x - r) ** 2) / (r * r + 0.01)).mean())
    noisy = img[..., :3].cpu().numpy().astype(np.float64) * albedo
    rel_1spp = float((((noisy - r) ** 2) / (r * r + 0.01)).mean())
    print(f"relMSE(GPU {spp} spp, FP64 oracle {spp} spp) = {rel:.3e}; one GPU sample: {rel_1spp:.3e}")
    assert rel < 1e-3
    assert rel < 1e-2 * rel_1spp
