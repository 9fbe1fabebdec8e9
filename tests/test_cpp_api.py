"""The C++ render-module layer (include/vulkanpbrt_gb300.hpp): the reference's
classes (PBRTPipeline, GBuffer, IlluminationBuffer*, AccumulationBuffer,
Accumulator, BMFR, ...) as header-only C++ over the C ABI, compiled with g++
into tests/cpp/render_frame.cpp.

CPU: the header compiles warning-free; ref_ptr counts references; recorded
commands read the push constants current at submit time; construction
errors arrive as vkpbrt::Exception with the C ABI's status and message.
GPU: the C++ program records the reference's frame (trace, accumulate, BMFR
32x32, copy to the back images) once and submits it for three frames; its
illumination and final image equal, bit for bit, the same frames rendered
through the Python render modules.
"""
import shutil
import struct
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
LIBDIR = ROOT / "vulkanpbrt_gb300"


@pytest.fixture(scope="module")
def cpp_driver(native_lib, tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    exe = tmp_path_factory.mktemp("cpp") / "render_frame"
    cmd = [gxx, "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I", str(ROOT / "include"),
           str(ROOT / "tests" / "cpp" / "render_frame.cpp"), "-L", str(LIBDIR), "-l:libvulkanpbrt_gb300.so",
           f"-Wl,-rpath,{LIBDIR}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_cpp_layer_host_semantics(cpp_driver):
    r = subprocess.run([str(cpp_driver), "errors"], capture_output=True, text=True, timeout=120)
    print(r.stdout, r.stderr)
    assert r.returncode == 0, r.stderr
    assert "errors: ok" in r.stdout
    assert "bad GBuffer" in r.stdout and "bad scene" in r.stdout


def _write_scene(path, sc, max_depth, min_depth):
    from vulkanpbrt_gb300.pipeline import PbrtObjectInstance, col_major16

    with open(path, "wb") as f:
        f.write(b"PBRTSCN1")
        f.write(struct.pack("<I", len(sc.meshes)))
        for m in sc.meshes:
            idx = np.ascontiguousarray(m.indices)
            f.write(struct.pack("<III", len(m.positions), len(idx), m.index_stride))
            for a in (m.positions, m.normals, m.uvs):
                f.write(np.ascontiguousarray(a, np.float32).tobytes())
            b = idx.astype(np.uint16 if m.index_stride == 2 else np.uint32).tobytes()
            f.write(b + b"\0" * (-len(b) % 4))
        f.write(struct.pack("<I", len(sc.instance_mesh)))
        for mid, mat in zip(sc.instance_mesh, sc.instance_mats):
            inst = PbrtObjectInstance()
            inst.object_mat[:] = col_major16(mat)
            inst.mesh_id = mid
            inst.index_stride = sc.meshes[mid].index_stride
            f.write(bytes(inst))
        op = sc.instance_opaque().astype(np.uint8).tobytes()
        f.write(op + b"\0" * (-len(op) % 4))
        f.write(np.stack(sc.materials).astype(np.float32).tobytes())
        f.write(struct.pack("<I", len(sc.lights)))
        if sc.lights:
            f.write(np.stack(sc.lights).astype(np.float32).tobytes())
        f.write(struct.pack("<I", len(sc.textures)))
        for t in sc.textures:
            f.write(struct.pack("<II", t.shape[1], t.shape[0]))
            f.write(np.ascontiguousarray(t, np.uint8).tobytes())
        f.write(np.array(sc.mesh_textures, np.int32).tobytes())
        f.write(struct.pack("<II", max_depth, min_depth))


@pytest.mark.gpu
def test_cpp_frame_equals_python_render_modules(cuda, cpp_driver, tmp_path):
    import torch

    import vulkanpbrt_gb300 as vp
    from vulkanpbrt_gb300 import scene as S
    from vulkanpbrt_gb300.camera import Camera

    W, H, depth, min_depth = 320, 192, 5, 2
    sc = S.cornell_spheres(seed=6)
    scene_file, frames_file = tmp_path / "scene.bin", tmp_path / "frames.bin"
    _write_scene(scene_file, sc, depth, min_depth)
    cams = [Camera((0.05 * k, -3.0, 1.0), sc.camera_center, aspect=W / H) for k in range(3)]
    frames = []
    for f, cam in enumerate(cams):
        prev = cams[max(0, f - 1)]
        pc = vp.PushConstants(view_inverse=cam.inv_view, proj_inverse=cam.inv_proj, prev_view=prev.view,
                              frame_number=f)
        cur = vp.CameraMatrices(cam.view, cam.inv_view, cam.proj, cam.inv_proj)
        prv = vp.CameraMatrices(prev.view, prev.inv_view)
        frames.append((pc, cur, prv))
    with open(frames_file, "wb") as fh:
        fh.write(struct.pack("<III", W, H, len(frames)))
        for pc, cur, prv in frames:
            fh.write(bytes(pc.value))
            fh.write(bytes(cur.to_c()))
            fh.write(bytes(prv.to_c()))
    out = tmp_path / "cpp"
    r = subprocess.run([str(cpp_driver), "frame", str(scene_file), str(frames_file), str(out)], capture_output=True,
                       text=True, timeout=600)
    print(r.stdout, r.stderr)
    assert r.returncode == 0, r.stderr

    # the same frames through the Python render modules
    sh = vp.SceneHandle(sc)
    g = vp.GBuffer(W, H)
    illu = vp.IlluminationBufferDemodulatedFloat(W, H)
    pipe = vp.PBRTPipeline(sh, g, illu, True, max_recursion_depth=depth, min_recursion_depth=min_depth)
    accu = vp.Accumulator(g, illu, separate_matrices=True)
    bm = vp.BMFR(W, H, 32, 32, g, accu.accumulated_illumination, accu.accumulation_buffer, 256)
    for pc, cur, prv in frames:
        accu.set_camera_matrices(pc.value.frame_number, cur, prv)
        pipe.trace(pc)
        vp.lib().pbrt_accumulator_dispatch(accu.ptr, None)
        bm.dispatch(pc)
        vp.lib().pbrt_accumulation_buffer_copy_to_back_images(accu.accumulation_buffer.ptr, g.ptr,
                                                              accu.accumulated_illumination.ptr, None)
    torch.cuda.synchronize()
    want_il = illu.illumination_images[0].tensor().cpu().numpy()
    want_fin = bm.get_final_descriptor_image().tensor().cpu().numpy()
    got_il = np.fromfile(str(out) + ".illum", np.float32).reshape(want_il.shape)
    got_fin = np.fromfile(str(out) + ".final", np.uint8).reshape(want_fin.shape)
    assert got_il[..., :3].sum() > 0
    np.testing.assert_array_equal(got_il, want_il)
    np.testing.assert_array_equal(got_fin, want_fin)
