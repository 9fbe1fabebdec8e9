"""Offline replay I/O on the CPU: the OpenEXR codec against hand-assembled
files and known answers of the format's byte preprocessing (so the reader
is not only checked against this library's writer), round trips over every
supported compression and pixel type, the camera-matrix formats of
source/io/RenderIO.cpp:593-716, and the G-buffer conversions of
RenderIO.cpp:166-370."""
import json
import struct

import numpy as np
import pytest

from vulkanpbrt_gb300 import exr


def _attr(name, typ, payload):
    return name.encode() + b"\0" + typ.encode() + b"\0" + struct.pack("<i", len(payload)) + payload


def test_reader_on_hand_assembled_file(tmp_path):
    """2 x 3 image, channels G (half) and R (float), uncompressed, one
    scanline per chunk, chunks written in decreasing y order."""
    W, H = 3, 2
    g = np.array([[0.5, -2.0, 65504.0], [1.0, 0.25, -0.0]], np.float16)
    r = np.array([[1.5, 2.5, 3.5], [-4.0, 1e-30, 7.0]], np.float32)
    chl = b"G\0" + struct.pack("<iB3xii", 1, 0, 1, 1) + b"R\0" + struct.pack("<iB3xii", 2, 0, 1, 1) + b"\0"
    hdr = struct.pack("<ii", 20000630, 2) + _attr("channels", "chlist", chl) + _attr("compression", "compression", b"\0")
    hdr += _attr("dataWindow", "box2i", struct.pack("<iiii", 10, 20, 12, 21)) + b"\0"
    chunks = [struct.pack("<ii", 20 + y, 3 * 2 + 3 * 4) + g[y].tobytes() + r[y].tobytes() for y in range(H)]
    offs = [len(hdr) + 16 + len(chunks[1]), len(hdr) + 16]  # line 0's chunk is stored second
    data = hdr + struct.pack("<2Q", *offs) + chunks[1] + chunks[0]
    p = tmp_path / "hand.exr"
    p.write_bytes(data)
    ch = exr.read(p)
    assert set(ch) == {"G", "R"} and ch["G"].dtype == np.float16 and ch["R"].dtype == np.float32
    assert np.array_equal(ch["G"], g) and np.array_equal(ch["R"], r)
    two = exr.load(p)  # two channels -> [H, W, 2] (R, G)
    assert two.shape == (H, W, 2) and np.array_equal(two[..., 0], r) and np.array_equal(two[..., 1], g)


def test_zip_and_rle_preprocessing_known_answers():
    # even bytes then odd bytes, then deltas + 128 (mod 256)
    pre = exr._split_predict(bytes([1, 2, 3, 4, 5]))
    assert pre.tolist() == [1, 130, 130, 125, 130]
    assert exr._unpredict_merge(pre) == bytes([1, 2, 3, 4, 5])
    enc = exr._rle_encode(np.array([7, 7, 7, 7, 1, 2], np.uint8))
    assert enc == bytes([3, 7, 0xFE, 1, 2])
    assert exr._rle_decode(enc, 6).tolist() == [7, 7, 7, 7, 1, 2]
    with pytest.raises(exr.ExrError):
        exr._rle_decode(enc, 7)


@pytest.mark.parametrize("compression", ["NONE", "RLE", "ZIPS", "ZIP"])
@pytest.mark.parametrize("dtype", [np.float16, np.float32, np.uint32])
def test_round_trip(tmp_path, compression, dtype):
    rng = np.random.default_rng(3)
    H, W = 37, 21  # not a multiple of ZIP's 16 lines per chunk
    smooth = np.add.outer(np.arange(H), np.arange(W)) % 7  # compressible
    if dtype == np.uint32:
        chans = {c: (smooth * 1000 + rng.integers(0, 3, (H, W))).astype(np.uint32) for c in "RGBA"}
    else:
        chans = {c: (smooth + rng.standard_normal((H, W)) * (c == "B")).astype(dtype) for c in "RGBA"}
    p = tmp_path / "x.exr"
    exr.write(p, chans, compression)
    back = exr.read(p)
    for c in "RGBA":
        assert back[c].dtype == chans[c].dtype and np.array_equal(back[c].view(np.uint8), chans[c].view(np.uint8))
    raw = p.read_bytes()
    assert raw[:4] == struct.pack("<i", 20000630) and b"channels\0chlist\0" in raw
    assert raw[raw.index(b"compression\0compression\0") + 28] == exr.COMPRESSION[compression]
    img = exr.load(p)
    assert img.shape == (H, W, 4)


def test_load_save_shapes(tmp_path):
    rng = np.random.default_rng(5)
    for a in (rng.random((5, 6)).astype(np.float32), rng.random((5, 6, 2)).astype(np.float32),
              rng.random((5, 6, 4)).astype(np.float16)):
        exr.save(tmp_path / "a.exr", a)
        b = exr.load(tmp_path / "a.exr")
        assert b.dtype == a.dtype and np.array_equal(a, b)
    exr.write(tmp_path / "rgb.exr", {c: np.full((2, 2), 0.5, np.float32) for c in "RGB"})
    assert np.array_equal(exr.load(tmp_path / "rgb.exr")[..., 3], np.ones((2, 2), np.float32))
    with pytest.raises(exr.ExrError):
        exr.write(tmp_path / "p.exr", {"R": np.zeros((2, 2), np.float32)}, "PIZ")


def test_matrix_io_json_and_text(tmp_path):
    from vulkanpbrt_gb300.camera import Camera
    from vulkanpbrt_gb300.render_io import MatrixIO
    from vulkanpbrt_gb300.render_modules import CameraMatrices

    cams = [Camera((i, -3.0, 1.0), (0.0, 0.0, 1.0)) for i in range(3)]
    mats = [CameraMatrices(c.view, c.inv_view, c.proj, c.inv_proj) for c in cams[:2]]
    mats.append(CameraMatrices(cams[2].view, cams[2].inv_view))
    p = str(tmp_path / "m.json")
    MatrixIO.export_matrices(p, mats)
    js = json.loads(open(p).read())
    assert js["amtOfFrames"] == 3 and js["matrices"][0]["storageType"] == "ColumnMajor"
    assert js["matrices"][0]["type"] == "ModelView+Projection" and js["matrices"][2]["type"] == "ModelViewProjection"
    # column major: the translation sits in elements 12..14
    assert js["matrices"][0]["invView"][12:15] == [float(v) for v in cams[0].inv_view[:3, 3]]
    back = MatrixIO.import_matrices(p)
    for a, b in zip(mats, back):
        assert np.array_equal(a.view, b.view) and np.array_equal(a.inv_view, b.inv_view)
        assert (a.proj is None) == (b.proj is None)
        if a.proj is not None:
            assert np.array_equal(a.proj, b.proj) and np.array_equal(a.inv_proj, b.inv_proj)
    # the BMFR dataset's text format: braces, commas, column major
    m = np.arange(16, dtype=np.float32).reshape(4, 4) + np.eye(4, dtype=np.float32) * 20
    cols = ", ".join(str(float(v)) for v in m.T.reshape(16))
    tp = tmp_path / "cams.txt"
    # every token that starts with a digit or '-' is a number, labels included
    tp.write_text("camera:\n{" + cols + "}\ncamera:\n{" + cols.replace("1.0,", "-1.0,", 1) + "}\n")
    t = MatrixIO.import_matrices(str(tp))
    assert len(t) == 2 and np.array_equal(t[0].view, m) and t[0].proj is None
    assert np.allclose(t[0].inv_view @ m, np.eye(4), atol=1e-5)
    assert t[1].view[0, 1] == -1.0  # the fifth number: column 1, row 0


def test_gbuffer_conversions():
    from vulkanpbrt_gb300.camera import Camera
    from vulkanpbrt_gb300.render_io import (compress_albedo, convert_normal_to_spherical, depth_to_position,
                                            position_to_depth, spherical_to_cartesian, unorm_to_float)
    from vulkanpbrt_gb300.render_modules import CameraMatrices

    rng = np.random.default_rng(2)
    sph = np.stack([rng.uniform(0.01, 3.13, (6, 7)), rng.uniform(-3.1, 3.1, (6, 7))], -1).astype(np.float32)
    back = convert_normal_to_spherical(spherical_to_cartesian(sph))
    assert np.abs(back - sph).max() < 2e-3 and spherical_to_cartesian(sph)[..., 3].min() == 1.0
    a = np.array([0.0, 0.999, 1.0, 0.5, -0.2, 1.7], np.float32)
    assert compress_albedo(a).tolist() == [0, 254, 255, 127, 0, 255]
    assert compress_albedo(np.array([258, 7], np.uint32)).tolist() == [2, 7]
    assert np.array_equal(compress_albedo(unorm_to_float(np.arange(256, dtype=np.uint8))), np.arange(256))
    cam = Camera((1.0, -4.0, 2.0), (0.0, 0.0, 1.0), aspect=7 / 6)
    m = CameraMatrices(cam.view, cam.inv_view, cam.proj, cam.inv_proj)
    depth = rng.uniform(1.0, 30.0, (6, 7)).astype(np.float32)
    pos = depth_to_position(depth, m)
    assert pos.shape == (6, 7, 4) and np.abs(position_to_depth(pos, m) - depth).max() < 1e-4 * depth.max()
    with pytest.raises(ValueError):
        depth_to_position(depth, CameraMatrices(cam.view, cam.inv_view))
