"""Scenes loaded from Wavefront OBJ/MTL (generated normals, flipped uvs,
an emissive mesh as area lights, a PNG texture) and a scene without lights
(the visitor's default directional light) traced on the GPU against the
FP32 oracle on the same scene data, same RNG streams."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _box_obj(tmp_path, with_lamp=True):
    from tests.test_scene_import import _png

    _png(tmp_path / "checker.png", (np.indices((8, 8)).sum(0) % 2 * 180 + 40)[..., None].repeat(3, -1).astype(np.uint8),
         2)
    mtl = ("newmtl white\nKd 0.75 0.75 0.75\nmap_Kd checker.png\n"
           "newmtl red\nKd 0.7 0.1 0.1\nKs 0.3 0.3 0.3\nNs 40\n"
           "newmtl green\nKd 0.1 0.7 0.1\n")
    if with_lamp:
        mtl += "newmtl lamp\nKd 0 0 0\nKe 15 15 15\n"
    (tmp_path / "box.mtl").write_text(mtl)
    v = [(-1, -1, 0), (1, -1, 0), (1, 1, 0), (-1, 1, 0), (-1, -1, 2), (1, -1, 2), (1, 1, 2), (-1, 1, 2)]
    lines = ["mtllib box.mtl"] + [f"v {x} {y} {z}" for x, y, z in v]
    lines += ["vt 0 0", "vt 4 0", "vt 4 4", "vt 0 4"]
    lines += ["usemtl white", "f 1/1 2/2 3/3 4/4", "f 5/1 8/4 7/3 6/2", "f 3/1 7/2 8/3 4/4",
              "usemtl red", "f 1 4 8 5", "usemtl green", "f 2 6 7 3"]
    n = len(v)
    # a low-poly sphere without normals: generated (flat) normals
    k = 0
    for i in range(6):
        for j in range(8):
            th0, th1 = np.pi * i / 6, np.pi * (i + 1) / 6
            ph0, ph1 = 2 * np.pi * j / 8, 2 * np.pi * (j + 1) / 8
            quad = [(th0, ph0), (th1, ph0), (th1, ph1), (th0, ph1)]
            for th, ph in quad:
                lines.append(f"v {0.3 + 0.35 * np.sin(th) * np.cos(ph):.6f} {0.2 + 0.35 * np.sin(th) * np.sin(ph):.6f} "
                             f"{0.5 + 0.35 * np.cos(th):.6f}")
            lines.append(f"f {n + k + 1} {n + k + 2} {n + k + 3} {n + k + 4}")
            k += 4
    lines.insert(lines.index("usemtl red"), "o sphere")
    if with_lamp:
        n2 = n + k
        lines += [f"v {x} {y} 1.98" for x, y in ((-0.3, -0.3), (0.3, -0.3), (0.3, 0.3), (-0.3, 0.3))]
        lines += ["o lamp", "usemtl lamp", f"f {n2 + 1} {n2 + 4} {n2 + 3} {n2 + 2}"]
    (tmp_path / "box.obj").write_text("\n".join(lines) + "\n")
    return tmp_path / "box.obj"


@pytest.mark.parametrize("with_lamp", [True, False])
def test_obj_scene_frame_matches_oracle(cuda, oracle, tmp_path, with_lamp):
    import torch

    import vulkanpbrt_gb300 as vp
    from vulkanpbrt_gb300.camera import Camera, col_major
    from vulkanpbrt_gb300.scene_import import load_obj

    sc = load_obj(_box_obj(tmp_path, with_lamp))
    assert len(sc.lights) == (2 if with_lamp else 1)
    if not with_lamp:
        assert sc.lights[0][3] == 1  # the default directional light
    W, H = 160, 96
    cam = Camera((0.0, -3.2, 1.0), (0.0, 0.0, 1.0), aspect=W / H)
    sh = vp.SceneHandle(sc)
    g = vp.GBuffer(W, H)
    illu = vp.IlluminationBufferDemodulatedFloat(W, H)
    pipe = vp.PBRTPipeline(sh, g, illu, True, max_recursion_depth=4, min_recursion_depth=4)
    pc = vp.PushConstants(view_inverse=cam.inv_view, proj_inverse=cam.inv_proj, prev_view=cam.view, frame_number=5)
    pipe.trace(pc)
    torch.cuda.synchronize()
    gpu = illu.illumination_images[0].tensor().cpu().numpy()[..., :3].astype(np.float64)
    ref = oracle.render(oracle.OracleScene(sc), W, H, col_major(cam.inv_view), col_major(cam.inv_proj), frame=5,
                        min_depth=4, max_depth=4)["illum"][..., :3].astype(np.float64)
    ok = np.abs(gpu - ref) <= 1e-4 * np.maximum(np.abs(gpu), np.abs(ref)) + 1e-6
    print(f"OBJ scene (lamp={with_lamp}): {ok.all(-1).mean() * 100:.3f}% of pixels within 1e-4; mean {gpu.mean():.4f}")
    assert ok.all(-1).mean() >= 0.98
    assert gpu.mean() > 1e-3 and abs(gpu.mean() / ref.mean() - 1) < 5e-3
