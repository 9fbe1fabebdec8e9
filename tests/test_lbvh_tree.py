"""The device BVH build's radix tree (vulkanpbrt_gb300/csrc/lbvh.cuh, the
functions its kernel calls), checked on the host (no GPU): compiled by nvcc
into tests/cpp/lbvh_tree.cu, which builds the tree over sorted random keys
with runs of equal keys and checks that every internal node's children split
its range exactly and every node but the root has one parent."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_radix_tree_partitions_every_range(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not available")
    exe = tmp_path / "lbvh_tree"
    cmd = [nvcc, "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a",
           "-I", str(ROOT / "vulkanpbrt_gb300" / "csrc"), str(ROOT / "tests" / "cpp" / "lbvh_tree.cu"), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout + out.stderr
