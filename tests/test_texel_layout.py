"""The texel pool's tiled layout, checked on the host (no GPU): the
index function the shading kernels and the upload's tiling kernel share is
compiled by nvcc into a host program (tests/cpp/texel_layout.cu) that
checks it is one-to-one into the padded allocation and that a bilinear
footprint touches 1.875 sectors on average."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_texel_tiles_are_one_to_one_and_sector_aligned(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not available")
    exe = tmp_path / "texel_layout"
    cmd = [nvcc, "-std=c++17", "-O1", "--expt-relaxed-constexpr", "-gencode", "arch=compute_103a,code=sm_103a",
           "-I", str(ROOT / "vulkanpbrt_gb300" / "csrc"), "-I", str(ROOT / "include"),
           str(ROOT / "tests" / "cpp" / "texel_layout.cu"), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and out.stdout.startswith("ok"), out.stdout + out.stderr
