"""BFRBlender (shaders/bfrBlender.comp) and the X8X16X32 denoiser
configurations of source/util/DenoiserUtils.cpp against the oracle:
bit-exact (8-bit outputs of the same unfused FP32 arithmetic) on random
inputs, and on a traced, accumulated frame through add_denoiser_to_commands
for both BFR and BMFR, where the blend of the three GPU denoisers' final
images must equal the oracle's blend of those same images."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("illu_type,radius", [("Demodulated", 2), ("FinalFloat", 1), ("Demodulated", 3)])
def test_blender_matches_oracle_random(cuda, oracle, illu_type, radius):
    import torch

    import vulkanpbrt_gb300 as vp
    from vulkanpbrt_gb300.render_modules import IlluminationBufferDemodulated, IlluminationBufferFinalFloat

    W, H = 211, 97
    cls = IlluminationBufferDemodulated if illu_type == "Demodulated" else IlluminationBufferFinalFloat
    a, b = cls(W, H), cls(W, H)
    g = vp.GBuffer(W, H)
    acc = vp.AccumulationBuffer(W, H)
    owner = vp.IlluminationBufferDemodulatedFloat(W, H)
    dens = [vp.BFR(W, H, bs, bs, g, owner, acc) for bs in (8, 16, 32)]  # owners of B8G8R8A8 final images
    rng = np.random.default_rng(radius)
    avg_img, sq_img = a.illumination_images[0], b.illumination_images[0]
    dt = np.float16 if illu_type == "Demodulated" else np.float32
    avg = (rng.random((H, W, 4)) ** 3 * 2).astype(dt)
    sq = (avg.astype(np.float32) ** 2 * rng.uniform(0.5, 3.0, (H, W, 1))).astype(dt)
    sq[rng.random((H, W)) < 0.1] = 0  # negative variances: NaN deviation -> the 8x8 result
    avg[10:40, 10:60] = 0  # zero deviation inside -> the 32x32 result
    sq[10:40, 10:60] = 0
    avg[50:90, 100:160] = 0  # deviation 0.5 inside -> the 16x16 result
    sq[50:90, 100:160] = 0.5
    avg_img.tensor().copy_(torch.from_numpy(avg))
    sq_img.tensor().copy_(torch.from_numpy(sq))
    bytes_ = []
    for d in dens:
        x = rng.integers(0, 256, (H, W, 4), dtype=np.uint8)
        d.get_final_descriptor_image().tensor().copy_(torch.from_numpy(x))
        bytes_.append(x)
    bl = vp.BFRBlender(W, H, avg_img, sq_img, *(d.get_final_descriptor_image() for d in dens), filter_radius=radius)
    bl.dispatch()
    torch.cuda.synchronize()
    got = bl.get_final_descriptor_image().tensor().cpu().numpy()
    want = oracle.bfr_blend(avg, sq, *bytes_, radius=radius)
    assert np.array_equal(got, want), int((got != want).any(-1).sum())
    # every branch of the blend is exercised
    sel = [np.mean((got[..., :3] == x[..., :3]).all(-1)) for x in bytes_]
    assert min(sel) > 0.01, sel


def _traced_accumulated(vp, W, H, frames):
    from vulkanpbrt_gb300 import scene as S
    from vulkanpbrt_gb300.camera import Camera

    sc = S.cornell_spheres(seed=2)
    sh = vp.SceneHandle(sc)
    g = vp.GBuffer(W, H)
    illu = vp.IlluminationBufferDemodulatedFloat(W, H)
    pipe = vp.PBRTPipeline(sh, g, illu, True, max_recursion_depth=4, min_recursion_depth=4)
    cam = Camera(sc.camera_eye, sc.camera_center, aspect=W / H)
    accu = vp.Accumulator(g, illu, separate_matrices=True)
    pc = vp.PushConstants(view_inverse=cam.inv_view, proj_inverse=cam.inv_proj, prev_view=cam.view)
    cm = vp.CameraMatrices(cam.view, cam.inv_view, cam.proj, cam.inv_proj)
    return sh, g, illu, pipe, accu, pc, cm


@pytest.mark.parametrize("kind", ["BFR", "BMFR"])
def test_x8x16x32_through_denoiser_utils(cuda, oracle, kind):
    import torch

    import vulkanpbrt_gb300 as vp
    from vulkanpbrt_gb300.denoiser_utils import DenoisingBlockSize, DenoisingType

    W, H = 160, 96
    sh, g, illu, pipe, accu, pc, cm = _traced_accumulated(vp, W, H, 3)
    acc_illu, abuf = accu.accumulated_illumination, accu.accumulation_buffer
    cmds = vp.Commands()
    final = vp.add_denoiser_to_commands(DenoisingType[kind], DenoisingBlockSize.X8X16X32, cmds, None, W, H, pc, g,
                                        acc_illu, abuf)
    single = vp.Commands()
    final32 = vp.add_denoiser_to_commands(DenoisingType[kind], DenoisingBlockSize.X32, single, None, W, H, pc, g,
                                          acc_illu, abuf)
    for f in range(3):
        pc.set(frame_number=f)
        pipe.trace(pc)
        accu.set_camera_matrices(f, cm, cm)
        vp.lib().pbrt_accumulator_dispatch(accu.ptr, None)
        cmds.submit()
        single.submit()
        vp.lib().pbrt_accumulation_buffer_copy_to_back_images(abuf.ptr, g.ptr, acc_illu.ptr, None)
    torch.cuda.synchronize()
    got = final.tensor().cpu().numpy()
    blender = final._owner
    ins = blender._inputs
    avg, sq = (ins[0].tensor().cpu().numpy(), ins[1].tensor().cpu().numpy())
    dens = [im.tensor().cpu().numpy() for im in ins[2:]]
    want = oracle.bfr_blend(avg, sq, *dens, radius=2)
    assert np.array_equal(got, want), int((got != want).any(-1).sum())
    # the 32x32 member of the blend and a lone X32 denoiser see the same inputs
    assert np.array_equal(dens[2], final32.tensor().cpu().numpy())
    assert got[..., :3].mean() > 1.0
