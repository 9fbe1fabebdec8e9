"""The allocation-free BMFR entry point against the regular one.

pbrt_bmfr_dispatch_noalloc serves callers that cannot allocate device memory
themselves -- an engine that owns the memory budget and passes a plugin only
its images, per-frame code that must not trigger cudaMalloc's device-wide
synchronisation, code running while its stream is captured. It runs the same
BMFR kernel on caller-provided images with its scratch in a fixed array
inside the library. This file is collected last on purpose; it must pass
alone in a fresh process as well as after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from denoise_cases import close_fraction, get, inputs, put

pytestmark = pytest.mark.gpu


def _noalloc(vp, W, H, bw, s_dev, den, fin, pc, position_type=0):
    from vulkanpbrt_gb300._abi import PbrtBmfrNoAllocImages, check, lib

    im = PbrtBmfrNoAllocImages(*[t.data_ptr() for t in (s_dev["depth"], s_dev["normal"], s_dev["albedo"],
                                                        s_dev["noisy"], s_dev["motion"], s_dev["spp"], den, fin)])
    check(lib().pbrt_bmfr_dispatch_noalloc(W, H, bw, position_type, C.byref(im), C.byref(pc.value), None))


# block size, fitting threads of the allocating BMFR, POSITION_TYPE (0: the
# reference's default screen-space position feature; 1, 2: world-space forms)
@pytest.mark.parametrize("bw,fk,ptype", [(32, 256, 0), (16, 256, 0), (8, 64, 0), (32, 256, 1), (32, 256, 2)])
def test_noalloc_matches_allocating_bmfr_on_two_calls(cuda, bw, fk, ptype):
    import torch

    import vulkanpbrt_gb300 as vp

    W, H = 320, 180
    g = vp.GBuffer(W, H)
    illu = vp.IlluminationBufferDemodulated(W, H)
    acc = vp.AccumulationBuffer(W, H)
    ref = vp.BMFR(W, H, bw, bw, g, illu, acc, fk, position_type=ptype)
    den = torch.zeros((2, H, W, 4), dtype=torch.float16, device=cuda)
    fin = torch.zeros((H, W, 4), dtype=torch.uint8, device=cuda)
    for frame in (0, 1):  # two calls in a row: the second reads the first's denoised layer
        s = inputs(W, H, seed=41, frame=frame)
        for img, key in ((g.depth, "depth"), (g.normal, "normal"), (g.albedo, "albedo"), (acc.motion, "motion"),
                         (acc.spp, "spp")):
            put(img, s[key])
        put(illu.illumination_images[0], s["noisy16"])
        cam = s["camera"]
        pc = vp.PushConstants(view_inverse=cam.inv_view, proj_inverse=cam.inv_proj, prev_view=cam.view,
                              frame_number=frame)
        ref.dispatch(pc)
        s_dev = {
            "depth": torch.from_numpy(s["depth"]).to(cuda),
            "normal": torch.from_numpy(s["normal"]).to(cuda),
            "albedo": torch.from_numpy(s["albedo"]).to(cuda),
            "noisy": torch.from_numpy(s["noisy16"]).to(cuda),
            "motion": torch.from_numpy(s["motion"]).to(cuda),
            "spp": torch.from_numpy(s["spp"]).to(cuda),
        }
        _noalloc(vp, W, H, bw, s_dev, den, fin, pc, ptype)
        torch.cuda.synchronize()
        want_den = get(ref.denoised)
        want_fin = get(ref.get_final_descriptor_image())
        got_den = den.cpu().numpy()
        frac, worst = close_fraction(got_den, want_den)
        assert frac == 1.0, f"frame {frame}: {frac} within tolerance (worst rel {worst})"
        assert np.abs(fin.cpu().numpy().astype(int) - want_fin.astype(int)).max() <= 1


def test_noalloc_rejects_grids_beyond_its_scratch(cuda):
    import torch

    import vulkanpbrt_gb300 as vp
    from vulkanpbrt_gb300._abi import PbrtBmfrNoAllocImages, PbrtError, check, lib

    W, H = 1920, 1080  # 8x8 blocks: 242 x 137 = 33154 blocks > 16384
    buf = torch.zeros(16, dtype=torch.uint8, device=cuda)
    p = buf.data_ptr()
    im = PbrtBmfrNoAllocImages(p, p, p, p, p, p, p, p)
    pc = vp.PushConstants()
    with pytest.raises(PbrtError, match="fixed maximum"):
        check(lib().pbrt_bmfr_dispatch_noalloc(W, H, 8, 0, C.byref(im), C.byref(pc.value), None))


def test_noalloc_rejects_misaligned_images(cuda):
    import torch

    import vulkanpbrt_gb300 as vp
    from vulkanpbrt_gb300._abi import PbrtBmfrNoAllocImages, PbrtError, check, lib

    W, H = 320, 180
    buf = torch.zeros(W * H * 16 + 64, dtype=torch.uint8, device=cuda)
    p = buf.data_ptr()
    pc = vp.PushConstants()
    for field, off in (("noisy", 4), ("denoised", 2), ("normal", 4), ("depth", 2), ("final_bgra", 1)):
        im = PbrtBmfrNoAllocImages(p, p, p, p, p, p, p, p)
        setattr(im, field, p + off)
        with pytest.raises(PbrtError, match=f"{field} pointer .* aligned"):
            check(lib().pbrt_bmfr_dispatch_noalloc(W, H, 32, 0, C.byref(im), C.byref(pc.value), None))
