"""The C-ABI library loads and exports every symbol the public headers declare (no GPU needed)."""
import ctypes
import re

from conftest import ROOT


def declared_entry_points():
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = h.read_text()
        names += re.findall(r"PBRT_API\s+[\w\s\*]+?\b(pbrt_\w+)\s*\(", text)
    return names


def test_header_declares_entry_points():
    names = declared_entry_points()
    assert len(names) >= 26
    assert len(set(names)) == len(names)


def test_library_exports_every_declared_symbol(native_lib):
    missing = [n for n in declared_entry_points() if not hasattr(native_lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_python_binding_covers_header(native_lib):
    import vulkanpbrt_gb300._abi as abi

    bound = set(abi.declared_symbols())
    missing = [n for n in declared_entry_points() if n not in bound]
    assert not missing, f"declared in include/ but not bound in _abi.py: {missing}"


def test_version_and_error_plumbing(native_lib):
    import vulkanpbrt_gb300 as vp
    from vulkanpbrt_gb300._abi import PbrtError, check, last_error

    assert b"sm_103a" in native_lib.pbrt_version()
    # Invalid arguments are rejected on the host, before any CUDA call.
    h = ctypes.c_void_p()
    rc = native_lib.pbrt_gbuffer_create(0, 10, ctypes.byref(h))
    assert rc == -1 and "bad size" in last_error()
    rc = native_lib.pbrt_illumination_buffer_create(17, 8, 8, ctypes.byref(h))
    assert rc == -1 and "unknown type" in last_error()
    rc = native_lib.pbrt_bmfr_set_options(None, 0, 0)
    assert rc == -1
    # the scene build's flags: FAST_TRACE (0) or FAST_BUILD (1), nothing else
    from vulkanpbrt_gb300.pipeline import PbrtSceneDesc

    desc = PbrtSceneDesc()
    rc = native_lib.pbrt_scene_create_ex(ctypes.byref(desc), 2, ctypes.byref(h))
    assert rc == -1 and "build flags" in last_error()
    rc = native_lib.pbrt_scene_create_ex(ctypes.byref(desc), 1, ctypes.byref(h))
    assert rc == -1 and "needs meshes" in last_error() and not h.value
    try:
        check(-4)
    except PbrtError as e:
        assert e.status == -4
    assert native_lib.pbrt_release(None) == 0
