"""Taa and FormatConverter against the oracle's restatement of
shaders/taa.comp and shaders/formatConverter.comp: bit-exact (integer
outputs from the same FP32 arithmetic), over several frames so the history
(the byte-copied previous final image) feeds back."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_taa_matches_oracle_over_frames(cuda, oracle):
    import torch

    import vulkanpbrt_gb300 as vp

    W, H = 203, 117
    g = vp.GBuffer(W, H)
    acc = vp.AccumulationBuffer(W, H)
    illu = vp.IlluminationBufferDemodulatedFloat(W, H)
    bmfr = vp.BMFR(W, H, 32, 32, g, illu, acc, 256)  # owner of a B8G8R8A8 final image the TAA reads
    den = bmfr.get_final_descriptor_image()
    taa = vp.Taa(W, H, 16, 16, g, acc, den)
    rng = np.random.default_rng(4)
    hist = np.zeros((H, W, 4), np.uint8)
    pc = vp.PushConstants()
    for frame in range(4):
        img = rng.integers(0, 256, (H, W, 4), dtype=np.uint8)
        if frame:  # a smooth field plus noise, so some history samples fall inside the clamp box
            img = (0.7 * prev + 0.3 * img).astype(np.uint8)
        prev = img
        uv = np.stack(np.meshgrid((np.arange(W) + 0.5 + rng.uniform(-2, 2)) / W,
                                  (np.arange(H) + 0.5 + rng.uniform(-2, 2)) / H), -1)
        uv[rng.random((H, W)) < 0.05] = -1.0  # disoccluded pixels
        motion = uv.astype(np.float16)
        den.tensor().copy_(torch.from_numpy(img))
        acc.motion.tensor().copy_(torch.from_numpy(motion))
        pc.set(frame_number=frame)
        taa.dispatch(pc)
        torch.cuda.synchronize()
        got = taa.get_final_descriptor_image().tensor().cpu().numpy()
        want, hist = oracle.taa(frame, motion, img, hist)
        assert np.array_equal(got, want), (frame, int((got != want).any(-1).sum()))


def test_format_convert(cuda):
    import torch

    import vulkanpbrt_gb300 as vp

    W, H = 70, 33
    illu = vp.IlluminationBufferFinalFloat(W, H)  # RGBA32F
    g = vp.GBuffer(W, H)  # albedo: R8G8B8A8
    src = torch.rand(H, W, 4, generator=torch.Generator().manual_seed(1)) * 1.2 - 0.1
    illu.illumination_images[0].tensor().copy_(src)
    vp.format_convert(illu.illumination_images[0], g.albedo)
    torch.cuda.synchronize()
    want = torch.floor(src.clamp(0, 1) * 255 + 0.5).to(torch.uint8)
    assert torch.equal(g.albedo.tensor().cpu(), want)
