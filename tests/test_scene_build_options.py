"""Host-side checks of the scene build choice (no GPU): the Python handle's
`build` argument and the benchmark's `--bvh` option reject unknown values
before any device work; the C entry point's flag check is in test_abi."""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_scene_handle_rejects_unknown_build():
    import vulkanpbrt_gb300 as vp
    from vulkanpbrt_gb300 import scene as S

    sc = S.cornell_spheres(seed=1, spheres=1, subdiv=1)
    import re

    hdr = (ROOT / "include" / "vulkanpbrt_gb300.h").read_text()
    flags = dict((k.lower(), int(v)) for k, v in re.findall(r"PBRT_BUILD_PREFER_(FAST_\w+) = (\d+)", hdr))
    assert vp.SceneHandle.BUILDS == flags  # {"fast_trace": 0, "fast_build": 1}, as the C header
    with pytest.raises(ValueError, match="build must be one of"):
        vp.SceneHandle(sc, build="sah")


def test_bench_rejects_unknown_bvh(monkeypatch):
    sys.path.insert(0, str(ROOT))
    import bench

    monkeypatch.setattr(sys, "argv", ["bench.py", "--workload", "bvh_build", "--bvh", "lbvh"])
    with pytest.raises(SystemExit):
        bench.parse()
    monkeypatch.setattr(sys, "argv", ["bench.py", "--workload", "bvh_build", "--bvh", "fast_build"])
    a = bench.parse()
    assert a.workload == "bvh_build" and a.bvh == "fast_build"
