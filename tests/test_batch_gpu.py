"""Batched requests: a batch of uneven requests (two scenes, five
resolutions, 1-4 samples, some accumulated and denoised with BMFR) rendered
in one graph launch gives, request by request, bit-identical images to the
same requests rendered one after another through the per-module calls --
for the default tuning, for a single chain, and for the tuning the
autotuner picks."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SPECS = [  # (scene, width, height, spp, denoise)
    (0, 96, 64, 1, False), (1, 160, 90, 2, True), (0, 200, 120, 4, True), (1, 64, 64, 3, False),
    (0, 128, 128, 2, True),
]


def _objects(vp, scenes, seed_frame=5):
    from vulkanpbrt_gb300.camera import Camera

    objs = []
    for i, (si, W, H, spp, den) in enumerate(SPECS):
        sc, sh = scenes[si]
        g = vp.GBuffer(W, H)
        illu = vp.IlluminationBufferDemodulatedFloat(W, H)
        pipe = vp.PBRTPipeline(sh, g, illu, True, max_recursion_depth=3 + (i % 2), min_recursion_depth=2)
        cam = Camera(sc.camera_eye, sc.camera_center, aspect=W / H)
        pc = vp.PushConstants(view_inverse=cam.inv_view, proj_inverse=cam.inv_proj, prev_view=cam.view,
                              frame_number=seed_frame + 100 * i)
        cm = vp.CameraMatrices(cam.view, cam.inv_view, cam.proj, cam.inv_proj)
        acc = bmfr = None
        if den:
            acc = vp.Accumulator(g, illu, separate_matrices=True)
            bmfr = vp.BMFR(W, H, 32, 32, g, acc.accumulated_illumination, acc.accumulation_buffer, 256)
        objs.append(dict(g=g, illu=illu, pipe=pipe, pc=pc, cm=cm, acc=acc, bmfr=bmfr, spp=spp))
    return objs


def _outputs(objs):
    import torch

    torch.cuda.synchronize()
    out = []
    for o in objs:
        d = {"illum": o["illu"].illumination_images[0].tensor().cpu().clone(),
             "albedo": o["g"].albedo.tensor().cpu().clone()}
        if o["bmfr"] is not None:
            d["final"] = o["bmfr"].get_final_descriptor_image().tensor().cpu().clone()
        out.append(d)
    return out


def _sequential(vp, objs):
    for o in objs:
        f0 = o["pc"].value.frame_number
        for k in range(o["spp"]):
            o["pc"].set(frame_number=f0 + k)
            o["pipe"].trace(o["pc"])
            if o["acc"] is not None:
                o["acc"].set_camera_matrices(k, o["cm"], o["cm"])
                vp.lib().pbrt_accumulator_dispatch(o["acc"].ptr, None)
                vp.lib().pbrt_accumulation_buffer_copy_to_back_images(
                    o["acc"].accumulation_buffer.ptr, o["g"].ptr, o["acc"].accumulated_illumination.ptr, None)
        o["pc"].set(frame_number=f0 + o["spp"] - 1)
        if o["bmfr"] is not None:
            o["bmfr"].dispatch(o["pc"])
        o["pc"].set(frame_number=f0)


def _batch(vp, objs, **tuning):
    b = vp.Batch()
    for o in objs:
        b.add(o["pipe"], o["pc"], spp=o["spp"], accumulator=o["acc"], bmfr=o["bmfr"], camera=o["cm"])
    if tuning:
        b.set_tuning(**tuning)
    return b


def _same(a, b):
    for x, y in zip(a, b):
        for k in x:
            assert np.array_equal(x[k].numpy(), y[k].numpy()), k


def test_batch_matches_sequential(cuda):
    import vulkanpbrt_gb300 as vp
    from vulkanpbrt_gb300 import scene as S

    scenes = []
    for seed in (2, 3):
        sc = S.cornell_spheres(seed=seed)
        scenes.append((sc, vp.SceneHandle(sc)))
    ref_objs = _objects(vp, scenes)
    _sequential(vp, ref_objs)
    ref = _outputs(ref_objs)
    for tuning in ({}, {"branches": 1, "trace_blocks_per_sm": 4, "shade_blocks_per_sm": 4, "order": 0}):
        objs = _objects(vp, scenes)
        b = _batch(vp, objs, **tuning)
        assert len(b) == len(SPECS)
        b.submit()
        _same(_outputs(objs), ref)
    # autotuned: every candidate is launched on the same objects, so compare after a fresh set
    objs = _objects(vp, scenes)
    b = _batch(vp, objs)
    best, ms = b.autotune(repeats=1)
    assert best["branches"] in (1, 2, 4, 8) and ms > 0
    objs2 = _objects(vp, scenes)
    b2 = _batch(vp, objs2, **best)
    b2.submit()
    _same(_outputs(objs2), ref)
