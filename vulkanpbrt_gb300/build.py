"""Build recipe for the native library libvulkanpbrt_gb300.so (sm_103a).

Every CUDA translation unit under csrc/ is compiled with nvcc for
``arch=compute_103a,code=sm_103a`` in parallel and linked, with the CUDA
runtime static, into a shared library next to this file. Host code is built
with FP contraction off so host-side float math gives the same bits on x86_64
and aarch64.
"""
from __future__ import annotations

import concurrent.futures
import os
import platform
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libvulkanpbrt_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = [
    "-O3",
    "-std=c++17",
    "-lineinfo",
    "--expt-relaxed-constexpr",
    "-Xcompiler",
    "-fPIC",
    "-Xcompiler",
    "-ffp-contract=off",
    "-Xcompiler",
    "-fvisibility=hidden",
]
# Per-file extra flags. The denoiser kernels restate the shaders' unfused
# FP32 arithmetic.
EXTRA = {
    "denoise.cu": ["-fmad=false"],
    "taa.cu": ["-fmad=false"],
    "blend.cu": ["-fmad=false"],
}


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found; the CUDA 13 toolkit is required to build libvulkanpbrt_gb300.so")
    return path


def sources() -> list[Path]:
    return sorted(p for p in CSRC.iterdir() if p.suffix in (".cu", ".cpp"))


def _compile(src: Path, verbose: bool) -> Path:
    obj = BUILD / (src.name + ".o")
    deps = [src] + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.hpp")) + [PKG.parent / "include" / "vulkanpbrt_gb300.h"]
    if obj.exists() and all(obj.stat().st_mtime >= d.stat().st_mtime for d in deps if d.exists()):
        return obj
    cmd = [nvcc(), *ARCH, *COMMON, *EXTRA.get(src.name, []), "-c", str(src), "-o", str(obj)]
    if src.suffix == ".cpp":
        cmd = [nvcc(), *COMMON, "-x", "cu", *ARCH, "-c", str(src), "-o", str(obj)]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stdout}\n{res.stderr}")
    if verbose and res.stderr:
        print(res.stderr, file=sys.stderr)
    return obj


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compile every csrc translation unit for sm_103a and link the library."""
    BUILD.mkdir(exist_ok=True)
    stamp = BUILD / "ARCH"
    if not stamp.exists() or stamp.read_text().strip() != platform.machine():
        force = True  # objects from another host architecture
        if LIB.exists():
            LIB.unlink()
    if force:
        for o in BUILD.glob("*.o"):
            o.unlink()
    srcs = sources()
    with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if LIB.exists() and all(LIB.stat().st_mtime >= o.stat().st_mtime for o in objs):
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *map(str, objs), "-lpthread"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    stamp.write_text(platform.machine())
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
