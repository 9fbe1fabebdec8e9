"""CUDA path tracer (PBRTPipeline) against the CPU oracle.

Tolerances (from the project's parity targets):
  * primary / random-ray hit ids bit-exact against the FP64 oracle for rays
    whose FP64 hit lies more than 1e-5 (barycentric) from a triangle edge;
  * per-pixel demodulated radiance within 1e-4 relative of the FP32 oracle
    (same RNG streams) on >= 99.8% of pixels -- the rest are paths that took
    a different branch after a last-bit difference (the shading kernel's
    hardware sin/cos/exp2/rsqrt vs the host libm, FMA contraction), which
    then differ entirely;
  * G-buffer depth within 1e-5 relative, albedo / material bytes within 1.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MISS = 0xFFFFFFFF
# pixels whose demodulated radiance must lie within 1e-4 (relative) of the
# FP32 oracle's: the parity the shaders' 1e-4 tolerance asks for, less the
# paths that branch differently after a last-bit difference
RADIANCE_FRACTION = 0.998


def _cam(sc, W, H):
    from vulkanpbrt_gb300.camera import Camera

    return Camera(sc.camera_eye, sc.camera_center, aspect=W / H)


def _render_gpu(vp, sh, W, H, cam, frame=0, min_depth=4, max_depth=4, light_mode=None):
    import torch

    g = vp.GBuffer(W, H)
    illu = vp.IlluminationBufferDemodulatedFloat(W, H)
    pipe = vp.PBRTPipeline(sh, g, illu, True, max_recursion_depth=max_depth, min_recursion_depth=min_depth,
                           light_sampling_method=light_mode)
    pc = vp.PushConstants(view_inverse=cam.inv_view, proj_inverse=cam.inv_proj, prev_view=cam.view, frame_number=frame)
    pipe.trace(pc)
    torch.cuda.synchronize()
    out = dict(illum=illu.illumination_images[0].tensor().cpu().numpy(),
               depth=g.depth.tensor().cpu().numpy()[..., 0], normal=g.normal.tensor().cpu().numpy(),
               albedo=g.albedo.tensor().cpu().numpy(), material=g.material.tensor().cpu().numpy(),
               hit_key=pipe.primary_hit_key.tensor().cpu().numpy()[..., 0].view(np.uint32), stats=pipe.stats())
    return out, pipe


def _rel_ok(a, b, rel, floor=1e-6):
    a = a.astype(np.float64)
    b = b.astype(np.float64)
    return np.abs(a - b) <= rel * np.maximum(np.abs(a), np.abs(b)) + floor


@pytest.fixture(scope="module")
def cornell():
    from vulkanpbrt_gb300 import scene as S

    return S.cornell_spheres(seed=1)


def test_random_ray_hits_match_fp64_oracle(cuda, oracle, cornell):
    import torch

    import vulkanpbrt_gb300 as vp

    sh = vp.SceneHandle(cornell)
    rng = np.random.default_rng(5)
    n = 200000
    org = np.stack([rng.uniform(-1.5, 1.5, n), rng.uniform(-3.5, 1.5, n), rng.uniform(0.05, 2.5, n),
                    np.full(n, 1e-3)], -1).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    dirs = np.concatenate([d, np.full((n, 1), 1e4)], -1).astype(np.float32)
    for any_hit in (False, True):
        hits = sh.trace_rays(torch.from_numpy(org).cuda(), torch.from_numpy(dirs).cuda(), any_hit=any_hit).cpu().numpy()
        gkey = hits[:, 3].view(np.uint32)
        os_ = oracle.OracleScene(cornell)
        ref = oracle.trace_rays(os_, org, dirs, any_hit=any_hit, precision=64)
        rkey = ref[:, 3].view(np.uint32)
        if any_hit:
            # inside a closed box every ray is occluded
            assert (gkey != MISS).all() and (rkey != MISS).all()
            continue
        u, v = ref[:, 1].astype(np.float64), ref[:, 2].astype(np.float64)
        far_from_edge = np.minimum(np.minimum(u, v), 1 - u - v) > 1e-5
        same = gkey == rkey
        print(f"random rays: {same.mean() * 100:.4f}% identical hit ids; away from edges "
              f"{same[far_from_edge].mean() * 100:.5f}% of {far_from_edge.sum()}")
        assert same[far_from_edge].all()
        t_ok = _rel_ok(hits[:, 0], ref[:, 0], 1e-5)
        assert t_ok[far_from_edge].mean() > 0.9999


def test_cornell_frame_matches_fp32_oracle(cuda, oracle, cornell):
    import vulkanpbrt_gb300 as vp
    from vulkanpbrt_gb300.camera import col_major

    W, H = 320, 180
    cam = _cam(cornell, W, H)
    sh = vp.SceneHandle(cornell)
    gpu, pipe = _render_gpu(vp, sh, W, H, cam, frame=3)
    ref = oracle.render(oracle.OracleScene(cornell), W, H, col_major(cam.inv_view), col_major(cam.inv_proj), frame=3,
                        min_depth=4, max_depth=4)
    keys = (gpu["hit_key"] == ref["hit_key"]).mean()
    print(f"primary hit ids identical: {keys * 100:.4f}%")
    assert keys >= 0.999
    ok = _rel_ok(gpu["illum"][..., :3], ref["illum"][..., :3], 1e-4).all(-1)
    print(f"radiance within 1e-4: {ok.mean() * 100:.3f}%; mean gpu {gpu['illum'][..., :3].mean():.5f} "
          f"oracle {ref['illum'][..., :3].mean():.5f}")
    assert ok.mean() >= RADIANCE_FRACTION
    assert abs(gpu["illum"][..., :3].mean() / ref["illum"][..., :3].mean() - 1) < 5e-3
    assert _rel_ok(gpu["depth"], ref["depth"], 1e-5).mean() >= 0.999
    assert (np.abs(gpu["albedo"].astype(int) - ref["albedo"].astype(int)) <= 1).mean() >= 0.999
    assert (gpu["material"] == ref["material"]).mean() >= 0.999
    nrm = np.abs(gpu["normal"] - ref["normal"]) <= 1e-4
    assert nrm.mean() >= 0.999
    st = gpu["stats"]
    print("rays gpu", st.primary_rays, st.extension_rays, st.shadow_rays, "oracle", ref["rays"])
    assert st.primary_rays == W * H and st.error_flags == 0
    assert abs(st.extension_rays / ref["rays"][1] - 1) < 0.01
    assert abs(st.shadow_rays / ref["rays"][2] - 1) < 0.01


@pytest.mark.parametrize("light_mode", [1, 2])
def test_light_sampling_modes(cuda, oracle, cornell, light_mode):
    import vulkanpbrt_gb300 as vp
    from vulkanpbrt_gb300.camera import col_major

    W, H = 160, 96
    cam = _cam(cornell, W, H)
    sh = vp.SceneHandle(cornell)
    gpu, _ = _render_gpu(vp, sh, W, H, cam, frame=1, min_depth=1, max_depth=3, light_mode=light_mode)
    ref = oracle.render(oracle.OracleScene(cornell), W, H, col_major(cam.inv_view), col_major(cam.inv_proj), frame=1,
                        min_depth=1, max_depth=3, light_mode=light_mode)
    ok = _rel_ok(gpu["illum"][..., :3], ref["illum"][..., :3], 1e-4).all(-1)
    print(f"light mode {light_mode}: {ok.mean() * 100:.3f}% within 1e-4")
    assert ok.mean() >= RADIANCE_FRACTION


def test_textured_instanced_scene_with_alpha_and_roulette(cuda, oracle):
    """The instanced-field workload at small size: textures (normal, specular,
    alpha-masked diffuse), u16 and u32 indices, point + area lights, Russian
    roulette from bounce 1."""
    import vulkanpbrt_gb300 as vp
    from vulkanpbrt_gb300 import scene as S
    from vulkanpbrt_gb300.camera import col_major

    sc = S.instanced_field(seed=3, instances=120, unique_meshes=12, texture_size=64, alpha_fraction=0.5, radius=8.0)
    W, H = 256, 144
    cam = _cam(sc, W, H)
    sh = vp.SceneHandle(sc)
    assert sh.info().triangle_count == sc.tri_count
    gpu, _ = _render_gpu(vp, sh, W, H, cam, frame=2, min_depth=1, max_depth=5)
    ref = oracle.render(oracle.OracleScene(sc), W, H, col_major(cam.inv_view), col_major(cam.inv_proj), frame=2,
                        min_depth=1, max_depth=5)
    keys = (gpu["hit_key"] == ref["hit_key"]).mean()
    ok = _rel_ok(gpu["illum"][..., :3], ref["illum"][..., :3], 1e-4).all(-1)
    print(f"instanced: hit ids {keys * 100:.4f}%, radiance within 1e-4 {ok.mean() * 100:.3f}%")
    assert keys >= 0.999
    assert ok.mean() >= RADIANCE_FRACTION


def _compare_frame(gpu, ref, W, H, label, fraction=None):
    keys = (gpu["hit_key"] == ref["hit_key"]).mean()
    ok = _rel_ok(gpu["illum"][..., :3], ref["illum"][..., :3], 1e-4).all(-1)
    st = gpu["stats"]
    print(f"{label}: primary hit ids {keys * 100:.4f}% identical, radiance within 1e-4 {ok.mean() * 100:.3f}%, "
          f"mean gpu {gpu['illum'][..., :3].mean():.5f} oracle {ref['illum'][..., :3].mean():.5f}; rays gpu "
          f"{st.primary_rays} {st.extension_rays} {st.shadow_rays} oracle {ref['rays'].tolist()}")
    assert st.primary_rays == W * H and st.error_flags == 0
    assert keys >= 0.999
    assert ok.mean() >= (RADIANCE_FRACTION if fraction is None else fraction)
    # the pixels outside the tolerance are other samples of the same estimator: the means agree
    assert abs(gpu["illum"][..., :3].mean() / ref["illum"][..., :3].mean() - 1) < 1e-3
    assert abs(st.extension_rays / ref["rays"][1] - 1) < 0.01
    assert abs(st.shadow_rays / ref["rays"][2] - 1) < 0.01
    return ok.mean()


def test_transmissive_materials_match_fp32_oracle(cuda, oracle):
    """illum 7 (transmission, IOR 1.5): the Fresnel-chosen refraction branch
    of sampleBRDF (shaders/sampling.glsl:35, 51-72), the transmissive-depth
    loop rule that does not count bounces through glass
    (shaders/ptRaygen.rgen:69) and the cosine factor of 1 for illum 7
    (shaders/lighting.glsl:272), against the FP32 oracle."""
    import vulkanpbrt_gb300 as vp
    from vulkanpbrt_gb300 import scene as S
    from vulkanpbrt_gb300.camera import col_major

    sc = S.cornell_spheres(seed=4)
    glass = 0
    for mid in range(3, len(sc.meshes) - 1):  # walls 0-2, spheres, then the light
        if mid % 2 == 1:
            sc.materials[mid] = S.material(diffuse=(0, 0, 0), specular=(0.04, 0.04, 0.04), roughness=0.05, ior=1.5,
                                           transmittance=(0.95, 0.9, 0.85), illum=7)
            glass += 1
    assert glass >= 3
    W, H = 320, 180
    cam = _cam(sc, W, H)
    sh = vp.SceneHandle(sc)
    gpu, _ = _render_gpu(vp, sh, W, H, cam, frame=5, min_depth=8, max_depth=8)
    ref = oracle.render(oracle.OracleScene(sc), W, H, col_major(cam.inv_view), col_major(cam.inv_proj), frame=5,
                        min_depth=8, max_depth=8)
    # glass paths run up to 10 extra bounces (transmissive bounces do not
    # count towards the depth), each another chance for a last-bit
    # difference to send the path elsewhere
    _compare_frame(gpu, ref, W, H, "transmissive spheres", fraction=0.98)
    # the glass spheres are visible: their refracted paths carry light
    assert gpu["illum"][..., :3].mean() > 0


def test_benchmark_frame_matches_fp32_oracle(cuda, oracle):
    """The timed workload itself: the seeded 1.06M-triangle instanced field
    (seed 0, 2000 instances, 196 textures of 1024^2, 5% alpha-masked meshes,
    8 point lights and an area light), 1920x1080, depth 8 with Russian
    roulette after bounce 3, the orbit's first camera -- every pixel of the
    GPU frame against the FP32 oracle's."""
    import vulkanpbrt_gb300 as vp
    from vulkanpbrt_gb300 import scene as S
    from vulkanpbrt_gb300.camera import col_major

    sc = S.instanced_field(seed=0)
    W, H = 1920, 1080
    cam = _cam(sc, W, H)
    sh = vp.SceneHandle(sc)
    assert sh.info().triangle_count == sc.tri_count > 1_000_000
    gpu, _ = _render_gpu(vp, sh, W, H, cam, frame=9, min_depth=3, max_depth=8)
    ref = oracle.render(oracle.OracleScene(sc), W, H, col_major(cam.inv_view), col_major(cam.inv_proj), frame=9,
                        min_depth=3, max_depth=8)
    # depth 8 and 1024^2 normal-mapped textures: longer paths than the
    # small scenes, so more of them branch after a last-bit difference
    _compare_frame(gpu, ref, W, H, "benchmark frame 1080p", fraction=0.995)
    assert _rel_ok(gpu["depth"], ref["depth"], 1e-5).mean() >= 0.999
    assert (np.abs(gpu["albedo"].astype(int) - ref["albedo"].astype(int)) <= 1).mean() >= 0.999


def test_frame_schedules_give_identical_frames(cuda):
    """The ray-sorting and shadow-merging schedule options change only the
    order in which rays are traced: every schedule renders the same frame,
    bit for bit, with the same ray counts."""
    import torch

    import vulkanpbrt_gb300 as vp
    from vulkanpbrt_gb300 import scene as S

    sc = S.instanced_field(seed=5, instances=150, unique_meshes=12, texture_size=64, alpha_fraction=0.3, radius=8.0)
    W, H = 256, 144
    cam = _cam(sc, W, H)
    sh = vp.SceneHandle(sc)
    g = vp.GBuffer(W, H)
    illu = vp.IlluminationBufferDemodulatedFloat(W, H)
    pipe = vp.PBRTPipeline(sh, g, illu, True, max_recursion_depth=6, min_recursion_depth=1)
    pc = vp.PushConstants(view_inverse=cam.inv_view, proj_inverse=cam.inv_proj, prev_view=cam.view, frame_number=4)
    frames = {}
    for sort_rays, merge in ((False, True), (True, True), (False, False), (True, False)):
        pipe.set_schedule(sort_rays=sort_rays, merge_shadow=merge)
        pipe.reset_stats()
        pipe.trace(pc)
        torch.cuda.synchronize()
        st = pipe.stats()
        frames[(sort_rays, merge)] = (illu.illumination_images[0].tensor().cpu().numpy().copy(),
                                      g.depth.tensor().cpu().numpy().copy(), g.albedo.tensor().cpu().numpy().copy(),
                                      (st.primary_rays, st.extension_rays, st.shadow_rays, st.error_flags))
    base = frames[(False, True)]
    assert base[3][1] > 0 and base[3][2] > 0 and base[3][3] == 0
    for key, f in frames.items():
        for a, b in zip(f[:3], base[:3]):
            np.testing.assert_array_equal(a, b, err_msg=str(key))
        assert f[3] == base[3], key
