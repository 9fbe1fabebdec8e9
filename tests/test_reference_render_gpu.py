"""Pins the many-sample GPU render that relMSE is measured against: on a
crop of the 640x360 Cornell-box frame (depth 4, no Russian roulette), the
mean of 4096 one-sample GPU frames of the demodulated illumination is
compared with the FP64 CPU oracle's 4096-sample mean over the same RNG
streams (same frame numbers, same pixels). The two estimators are the same,
so their relMSE is far below the relMSE between any denoiser and either of
them; the tolerance is 1e-3. The second test does the same on a crop of the
benchmark's own scene at its depth and Russian roulette."""
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


def test_benchmark_scene_1024spp_mean_matches_fp64_oracle(cuda, oracle):
    """The same pinning on the benchmark's own scene and settings: a 32x24
    crop of the 1080p frame of the instanced field (seed 0: 2002 instances,
    1024^2 textures, 10 lights), depth 8 with Russian roulette after bounce
    3, camera of the benchmark's orbit; 1024 one-sample GPU frames against
    the FP64 oracle's 1024-sample mean over the same RNG streams."""
    import sys
    from pathlib import Path

    import torch

    import vulkanpbrt_gb300 as vp
    from vulkanpbrt_gb300 import scene as S
    from vulkanpbrt_gb300.camera import CropCamera, col_major

    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    import bench

    sc = S.instanced_field(seed=0)
    W, H, spp, f0 = 32, 24, 1024, 40
    full = bench.orbit(sc, 1920, 1080, 7)
    cam = CropCamera(full, 1920, 1080, 940, 560, W, H)
    sh = vp.SceneHandle(sc)
    g = vp.GBuffer(W, H)
    illu = vp.IlluminationBufferDemodulatedFloat(W, H)
    pipe = vp.PBRTPipeline(sh, g, illu, True, max_recursion_depth=8, min_recursion_depth=3)
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
                        min_depth=3, max_depth=8, precision=64, frames=spp)
    r = albedo * ref["illum"][..., :3].astype(np.float64)
    x = albedo * gpu
    rel = float((((x - r) ** 2) / (r * r + 0.01)).mean())
    noisy = img[..., :3].cpu().numpy().astype(np.float64) * albedo
    rel_1spp = float((((noisy - r) ** 2) / (r * r + 0.01)).mean())
    print(f"benchmark scene: relMSE(GPU {spp} spp, FP64 oracle {spp} spp) = {rel:.3e}; one GPU sample: {rel_1spp:.3e}")
    assert rel < 1e-3
    assert rel < 1e-2 * rel_1spp
