"""Device BVH build (pbrt_scene_create_ex with PBRT_BUILD_PREFER_FAST_BUILD)
against the host build (binned SAH, the default).

The closest hit does not depend on the tree: every triangle the ray could hit
is tested, and ties go to the lowest triangle key (the flattening index). So
closest-hit results (t, u, v, key) and whole rendered frames must be
bit-identical under the two builds; an any-hit (shadow) query stops at the
first occluder the traversal order meets, so there the answer -- occluded or
not, all a shadow ray uses -- must agree. Covered: alpha-tested instances,
duplicate triangles (equal Morton codes) and the smallest trees (1-5
triangles: a root that is itself a leaf).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _tri_scene(ntri, seed, duplicates=0):
    from vulkanpbrt_gb300 import scene as S

    rng = np.random.default_rng(seed)
    c = rng.uniform(-1, 1, (ntri, 1, 3))
    pos = (c + rng.uniform(-0.3, 0.3, (ntri, 3, 3))).reshape(-1, 3)
    if duplicates:
        pos = np.concatenate([pos, np.repeat(pos[:3], duplicates, axis=0)])  # copies of triangle 0
    pos = pos.astype(np.float32)
    nv = len(pos)
    mesh = S.Mesh(pos, np.tile(np.float32([0, 0, 1]), (nv, 1)), np.zeros((nv, 2), np.float32),
                  np.arange(nv, dtype=np.uint32))
    sc = S.Scene()
    mid = sc.add_mesh(mesh, S.material(diffuse=(0.5, 0.5, 0.5)))
    sc.add_instance(mid, np.eye(4))
    sc.lights.append(S.packed_light(S.LIGHT_POINT, (0, 0, 3)))
    sc.finalize_lights()
    return sc


def _rays(n, seed, lo=-1.5, hi=1.5):
    import torch

    rng = np.random.default_rng(seed)
    org = np.concatenate([rng.uniform(lo, hi, (n, 3)), np.full((n, 1), 1e-4)], -1).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    dirs = np.concatenate([d, np.full((n, 1), 1e30)], -1).astype(np.float32)
    return torch.from_numpy(org).cuda(), torch.from_numpy(dirs).cuda()


def _hits(sh, org, dirs, any_hit):
    h = sh.trace_rays(org, dirs, any_hit=any_hit).cpu().numpy().view(np.uint32)
    return (h[:, 3] != 0xFFFFFFFF) if any_hit else h  # any-hit: occluded or not


def _both(sc):
    import vulkanpbrt_gb300 as vp

    return vp.SceneHandle(sc), vp.SceneHandle(sc, build="fast_build")


@pytest.mark.parametrize("ntri", [1, 2, 3, 4, 5, 17, 1000, 50000])
def test_random_triangles_hit_the_same(cuda, ntri):
    host, dev = _both(_tri_scene(ntri, seed=ntri))
    info = dev.info()
    assert info.triangle_count == ntri and info.bvh_nodes >= 1
    org, dirs = _rays(20000, seed=7)
    for any_hit in (False, True):
        a, b = _hits(host, org, dirs, any_hit), _hits(dev, org, dirs, any_hit)
        bad = int((a != b).reshape(len(a), -1).any(-1).sum())
        assert bad == 0, f"{ntri} triangles, any_hit={any_hit}: {bad} rays differ"
    hit = _hits(dev, org, dirs, False)[:, 3] != 0xFFFFFFFF
    assert hit.any()


def test_duplicate_triangles_tie_to_the_lowest_key(cuda):
    """60 copies of one triangle: equal centroids, equal Morton codes (the
    radix tree splits them by index) and exact t ties."""
    host, dev = _both(_tri_scene(200, seed=3, duplicates=60))
    org, dirs = _rays(20000, seed=11)
    for any_hit in (False, True):
        assert np.array_equal(_hits(host, org, dirs, any_hit), _hits(dev, org, dirs, any_hit))


@pytest.mark.parametrize("collapse", ["sah", "greedy", "sah_triangle_cost_1"])
def test_instanced_alpha_scene_hits_the_same(cuda, collapse, monkeypatch):
    from vulkanpbrt_gb300 import scene as S

    if collapse == "greedy":
        monkeypatch.setenv("PBRT_BVH_COLLAPSE", "greedy")  # both builds: open the largest child until eight
    if collapse == "sah_triangle_cost_1":
        # triangles as dear as node visits: subtrees of 2-3 triangles become
        # wide nodes of single-triangle leaves where that is cheaper
        monkeypatch.setenv("PBRT_BVH_PRIM_COST", "1.0")

    sc = S.instanced_field(seed=3, instances=120, unique_meshes=12, texture_size=64, alpha_fraction=0.5, radius=8.0)
    host, dev = _both(sc)
    hi, di = host.info(), dev.info()
    assert hi.triangle_count == di.triangle_count == sc.tri_count
    print(f"instanced field ({collapse} collapse), {sc.tri_count} triangles: host {hi.bvh_nodes} nodes depth {hi.bvh_depth} "
          f"{hi.build_ms:.1f} ms; device {di.bvh_nodes} nodes depth {di.bvh_depth} {di.build_ms:.1f} ms")
    org, dirs = _rays(200000, seed=5, lo=-8.0, hi=8.0)
    for any_hit in (False, True):
        a, b = _hits(host, org, dirs, any_hit), _hits(dev, org, dirs, any_hit)
        bad = int((a != b).reshape(len(a), -1).any(-1).sum())
        assert bad == 0, f"any_hit={any_hit}: {bad} rays differ"


def _frame(vp, sh, sc, W, H, frame):
    import torch

    from vulkanpbrt_gb300.camera import Camera

    cam = Camera(sc.camera_eye, sc.camera_center, aspect=W / H)
    g = vp.GBuffer(W, H)
    illu = vp.IlluminationBufferDemodulatedFloat(W, H)
    pipe = vp.PBRTPipeline(sh, g, illu, True, max_recursion_depth=6, min_recursion_depth=1)
    pc = vp.PushConstants(view_inverse=cam.inv_view, proj_inverse=cam.inv_proj, prev_view=cam.view,
                          frame_number=frame)
    pipe.trace(pc)
    torch.cuda.synchronize()
    return [illu.illumination_images[0].tensor().cpu().numpy(), g.depth.tensor().cpu().numpy(),
            g.normal.tensor().cpu().numpy(), g.albedo.tensor().cpu().numpy(), g.material.tensor().cpu().numpy()]


@pytest.mark.parametrize("which", ["cornell", "instanced"])
def test_frames_are_bit_identical(cuda, which):
    import vulkanpbrt_gb300 as vp
    from vulkanpbrt_gb300 import scene as S

    if which == "cornell":
        sc = S.cornell_spheres(seed=1)
    else:
        sc = S.instanced_field(seed=3, instances=120, unique_meshes=12, texture_size=64, alpha_fraction=0.5,
                               radius=8.0)
    host, dev = _both(sc)
    W, H = 256, 144
    for frame in (0, 3):
        a, b = _frame(vp, host, sc, W, H, frame), _frame(vp, dev, sc, W, H, frame)
        for x, y in zip(a, b):
            assert np.array_equal(np.ascontiguousarray(x).view(np.uint8), np.ascontiguousarray(y).view(np.uint8))
