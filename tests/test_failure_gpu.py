"""Failure handling of the tracer without a GPU fault: a frame budget that
runs out and a host abort flag both stop the frame early (no more rays
taken, nothing shaded), the host reads the reason from pbrt_pipeline_status,
and the same pipeline then renders a normal frame bit-identical to one from
a pipeline that never stopped. Nothing here waits on a flag that is never
set: the kernels only poll."""
import pytest

pytestmark = pytest.mark.gpu


def _setup(W=320, H=180):
    import vulkanpbrt_gb300 as vp
    from vulkanpbrt_gb300 import scene as S
    from vulkanpbrt_gb300.camera import default_camera

    sc = S.cornell_spheres(seed=3)
    sh = vp.SceneHandle(sc)
    g = vp.GBuffer(W, H)
    illu = vp.IlluminationBufferDemodulatedFloat(W, H)
    pipe = vp.PBRTPipeline(sh, g, illu, True, max_recursion_depth=4, min_recursion_depth=4)
    cam = default_camera(W, H)
    pc = vp.PushConstants()
    pc.set(view_inverse=cam.inv_view, proj_inverse=cam.inv_proj, prev_view=cam.view, frame_number=7)
    return vp, pipe, illu, pc


def test_budget_and_abort_stop_the_frame_and_recover(cuda):
    import torch

    vp, pipe, illu, pc = _setup()
    img = illu.illumination_images[0].tensor()
    # a normal frame first
    pipe.trace(pc)
    assert pipe.status() == 0
    good = img.clone()
    stats0 = pipe.stats()

    # budget of 1 ns: the first poll stops the frame
    pipe.set_budget(1)
    pipe.trace(pc)
    assert pipe.status() == -6  # PBRT_ERROR_TIMEOUT
    stats1 = pipe.stats()
    assert pipe.status() == 0  # cleared by the previous read
    torch.cuda.synchronize()
    assert torch.isfinite(img).all()
    full_rays = stats0.extension_rays + stats0.shadow_rays
    assert (stats1.extension_rays + stats1.shadow_rays) - full_rays < full_rays  # stopped early

    # abort flag set before the frame: stops at the first poll
    pipe.set_budget(0)
    pipe.set_abort(True)
    pipe.trace(pc)
    assert pipe.status() == -5  # PBRT_ERROR_ABORTED
    pipe.set_abort(False)

    # the pipeline is still usable and renders the same frame as before
    pipe.trace(pc)
    assert pipe.status() == 0
    torch.cuda.synchronize()
    assert torch.equal(img, good)


def test_generous_budget_changes_nothing(cuda):
    import torch

    vp, pipe, illu, pc = _setup()
    img = illu.illumination_images[0].tensor()
    pipe.trace(pc)
    ref = img.clone()
    pipe.set_budget(10 ** 10)  # 10 s
    pipe.trace(pc)
    assert pipe.status() == 0
    torch.cuda.synchronize()
    assert torch.equal(img, ref)
