"""The host BVH build's 8-wide tree checked on the host (no GPU): every
triangle is reached exactly once and every quantised child box contains its
whole subtree (tests/cpp/bvh_check.cpp, compiled with bvh_build.cpp), for
both collapse modes and both binary leaf sizes."""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not available")
    exe = tmp_path_factory.mktemp("bvh") / "bvh_check"
    csrc = ROOT / "vulkanpbrt_gb300" / "csrc"
    cmd = [nvcc, "-std=c++17", "-O2", "-x", "cu", "-I", str(csrc), str(ROOT / "tests" / "cpp" / "bvh_check.cpp"),
           str(csrc / "bvh_build.cpp"), "-o", str(exe), "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


@pytest.mark.parametrize("collapse,binary_leaf", [("sah", "1"), ("sah", "3"), ("greedy", "3")])
def test_tree_holds_every_triangle_once_in_conservative_boxes(checker, collapse, binary_leaf):
    env = dict(os.environ, PBRT_BVH_BINARY_LEAF=binary_leaf)
    if collapse == "greedy":
        env["PBRT_BVH_COLLAPSE"] = "greedy"
    else:
        env.pop("PBRT_BVH_COLLAPSE", None)
    out = subprocess.run([str(checker)], capture_output=True, text=True, timeout=300, env=env)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout + out.stderr
