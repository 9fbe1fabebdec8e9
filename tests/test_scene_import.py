"""Scene ingestion on the CPU: the visitor's mesh preparation
(source/scene/RayTracingVisitor.cpp:52-166) against a float32 restatement
written here in vsg's operation order, its material and default-light
rules, the PNG / PPM decoders against files encoded here with every PNG
row filter, and the OBJ/MTL loader."""
import struct
import zlib

import numpy as np
import pytest

f32 = np.float32


def _normals_py(pos, idx, init):
    nor = init.astype(np.float32).copy()
    ws = np.zeros(len(pos), np.float32)
    for t in range(len(idx) // 3):
        ia, ib, ic = (int(i) for i in idx[3 * t:3 * t + 3])
        a, b, c = pos[ia], pos[ib], pos[ic]
        l, r = b - a, c - a
        fn = np.array([l[1] * r[2] - r[1] * l[2], l[2] * r[0] - r[2] * l[0], l[0] * r[1] - r[0] * l[1]], np.float32)
        w = f32(np.sqrt(f32(f32(fn[0] * fn[0] + fn[1] * fn[1]) + fn[2] * fn[2])))
        with np.errstate(divide="ignore", invalid="ignore"):
            fn = fn * (f32(1) / w)
            for k in (ia, ib, ic):
                nw = f32(w + ws[k])
                nor[k] = nor[k] * (ws[k] / nw) + fn * (w / nw)
                ws[k] = nw
    return nor


@pytest.mark.parametrize("dtype", [np.uint16, np.uint32])
def test_generated_normals_match_restatement(native_lib, dtype):
    from vulkanpbrt_gb300.scene_import import generate_normals

    rng = np.random.default_rng(1)
    pos = rng.standard_normal((40, 3)).astype(np.float32)
    idx = np.concatenate([rng.choice(36, 3, replace=False) for _ in range(30)]).astype(dtype)  # 36..39 unreferenced
    init = np.zeros((40, 3), np.float32)
    init[37] = (0.0, 0.0, 5.0)
    got = generate_normals(pos, idx, init)
    want = _normals_py(pos, idx, init)
    assert np.array_equal(got, want) and np.isfinite(got).all()
    assert np.array_equal(got[37], [0, 0, 5])  # kept
    assert not np.allclose(np.linalg.norm(got[:36], axis=1), 1.0)  # not normalised, as in the reference


def test_degenerate_triangle_gives_nan_as_the_reference(native_lib):
    from vulkanpbrt_gb300.scene_import import generate_normals

    pos = np.array([[0, 0, 0], [1, 0, 0], [2, 0, 0], [0, 1, 0]], np.float32)
    nor = generate_normals(pos, np.array([0, 1, 2, 0, 1, 3], np.uint16))
    assert np.isnan(nor[2]).all() and np.isnan(nor[0]).all()  # 0/0 weights on the collinear triangle


def test_uv_fill_and_prepare_mesh(native_lib):
    from vulkanpbrt_gb300.scene_import import fill_uvs, prepare_mesh

    uv = fill_uvs(5, np.array([0, 1, 2, 2, 3, 0], np.uint32))
    assert uv.tolist() == [[1, 0], [0, 1], [0, 0], [0, 1], [0, 0]]
    pos = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    m = prepare_mesh(pos, np.zeros((3, 3), np.float32), None, np.array([0, 1, 2], np.int64))
    assert m.indices.dtype == np.uint16 and np.allclose(m.normals, [[0, 0, 1]] * 3)
    assert m.uvs.tolist() == [[0, 0], [0, 1], [1, 0]]
    given = np.array([[0, 0, 1], [0, 0, 0], [0, 0, 0]], np.float32)  # first normal non-zero: kept as given
    assert np.array_equal(prepare_mesh(pos, given, np.zeros((3, 2)), np.array([0, 1, 2])).normals, given)


def test_materials_and_default_light():
    from vulkanpbrt_gb300.scene import Scene
    from vulkanpbrt_gb300.scene_import import default_light, is_emissive, pbr_material, phong_material

    m = phong_material(diffuse=(0.5, 0.25, 1, 1), shininess=30.0, transmissive=(1, 1, 0.5), emissive=(0, 0, 0.1, 1))
    assert m[3] == np.sqrt(f32(2) / f32(32)) and m[15] == 7.0 and tuple(m[4:7]) == (0.5, 0.25, 1.0)
    assert is_emissive(m) and not is_emissive(phong_material())
    p = pbr_material(base_color=(0.2, 0.3, 0.4, 1), roughness=0.7, index_of_refraction=1.5, category_id=9)
    assert p[3] == f32(0.7) and p[7] == f32(1.5) and p[15] == 0 and p[20:21].view(np.uint32)[0] == 9
    l = default_light()
    assert l[3] == 1 and abs(np.linalg.norm(l[12:15]) - 1) < 1e-6 and l[28] == 0.5 and l[24:27].sum() == 0
    sc = Scene()
    sc.finalize_lights()
    assert len(sc.lights) == 1 and sc.lights[0][31] == 12.0  # inclusive strength 2*3 + 2*3


def _png(path, rgba, ctype=6, filters=(0, 1, 2, 3, 4), palette=None, trns=None):
    h, w = rgba.shape[:2]
    px = rgba.astype(np.int32)
    bpp = px.shape[2]
    rows = px.reshape(h, -1)
    raw = bytearray()
    prev = np.zeros(w * bpp, np.int32)
    for y in range(h):
        ft = filters[y % len(filters)]
        cur = rows[y]
        left = np.concatenate([np.zeros(bpp, np.int32), cur[:-bpp]])
        upleft = np.concatenate([np.zeros(bpp, np.int32), prev[:-bpp]])
        if ft == 0:
            f = cur
        elif ft == 1:
            f = cur - left
        elif ft == 2:
            f = cur - prev
        elif ft == 3:
            f = cur - (left + prev) // 2
        else:
            pr = []
            for a, b, c in zip(left, prev, upleft):
                p = a + b - c
                pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                pr.append(a if pa <= pb and pa <= pc else (b if pb <= pc else c))
            f = cur - np.array(pr, np.int32)
        raw.append(ft)
        raw += (f & 0xFF).astype(np.uint8).tobytes()
        prev = cur

    def chunk(t, b):
        return struct.pack(">I", len(b)) + t + b + struct.pack(">I", zlib.crc32(t + b) & 0xFFFFFFFF)

    data = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0))
    if palette is not None:
        data += chunk(b"PLTE", palette.astype(np.uint8).tobytes())
    if trns is not None:
        data += chunk(b"tRNS", trns.astype(np.uint8).tobytes())
    data += chunk(b"IDAT", zlib.compress(bytes(raw))) + chunk(b"IEND", b"")
    path.write_bytes(data)


def test_png_and_ppm_decoders(tmp_path):
    from vulkanpbrt_gb300.scene_import import load_image

    rng = np.random.default_rng(4)
    rgba = rng.integers(0, 256, (7, 5, 4), dtype=np.uint8)
    _png(tmp_path / "a.png", rgba, 6)
    assert np.array_equal(load_image(tmp_path / "a.png"), rgba)
    _png(tmp_path / "b.png", rgba[..., :3], 2)
    assert np.array_equal(load_image(tmp_path / "b.png")[..., :3], rgba[..., :3])
    _png(tmp_path / "g.png", rgba[..., :1], 0)
    g = load_image(tmp_path / "g.png")
    assert np.array_equal(g[..., 0], rgba[..., 0]) and np.array_equal(g[..., 2], rgba[..., 0]) and (g[..., 3] == 255).all()
    pal = rng.integers(0, 256, (6, 3))
    ind = rng.integers(0, 6, (7, 5, 1), dtype=np.uint8)
    _png(tmp_path / "p.png", ind, 3, palette=pal, trns=np.array([0, 128]))
    p = load_image(tmp_path / "p.png")
    assert np.array_equal(p[..., :3], pal[ind[..., 0]]) and p[..., 3][ind[..., 0] == 1].max(initial=128) == 128
    (tmp_path / "c.ppm").write_bytes(b"P6\n# comment\n5 7\n255\n" + rgba[..., :3].tobytes())
    c = load_image(tmp_path / "c.ppm")
    assert np.array_equal(c[..., :3], rgba[..., :3]) and (c[..., 3] == 255).all()


def test_obj_loader(tmp_path, native_lib):
    from vulkanpbrt_gb300.scene_import import load_obj

    _png(tmp_path / "tex.png", np.full((2, 2, 4), 200, np.uint8))
    (tmp_path / "m.mtl").write_text(
        "newmtl white\nKd 0.8 0.8 0.8\nKs 0.5 0.5 0.5\nNs 0.001\nmap_Kd tex.png\n"
        "newmtl lamp\nKd 0 0 0\nKe 10 9 8\n")
    (tmp_path / "s.obj").write_text(
        "mtllib m.mtl\n"
        "v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nv 0 0 1\n"
        "vt 0 0\nvt 1 0\nvt 1 1\nvt 0 1\n"
        "usemtl white\n"
        "f 1/1 2/2 3/3 4/4\n"  # a quad, no normals
        "f -5/1 -4/2 -1/4\n"  # relative indices
        "o lamp\nusemtl lamp\n"
        "f 1 2 5\n")
    sc = load_obj(tmp_path / "s.obj")
    assert len(sc.meshes) == 2 and len(sc.instance_mesh) == 2
    quad = sc.meshes[0]
    assert quad.tri_count == 3 and quad.indices.dtype == np.uint16 and len(quad.positions) == 9
    assert np.allclose(quad.uvs[:4], [[0, 1], [1, 1], [1, 0], [0, 1]])  # v flipped, fan (1,2,3), (1,3,4)
    assert np.allclose(quad.normals[:6], [[0, 0, 1]] * 6)  # per-face normals
    white = sc.materials[0]
    assert white[8:11].sum() == 0 and white[3] == 1.0  # Ns < 0.01: no specular, shininess 0
    assert sc.mesh_textures[0][0] != 0 and sc.textures[sc.mesh_textures[0][0]].shape == (2, 2, 4)
    lamp = sc.lights
    assert len(lamp) == 1 and lamp[0][3] == 5 and tuple(lamp[0][16:19]) == (10, 9, 8)  # one area light
    with pytest.raises(OSError):
        (tmp_path / "m.mtl").write_text("newmtl white\nmap_Kd missing.png\n")
        load_obj(tmp_path / "s.obj")
    assert load_obj(tmp_path / "s.obj", missing_textures="white").mesh_textures[0][0] == 0
