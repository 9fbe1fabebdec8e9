"""The benchmark's own arm on a small frame (640x352, 200 instances, 64^2
textures): one JSON line with every key of the benchmark contract and the
additions this benchmark reports (roofline with the traversal's counters,
clocks, launch count, stage times, relMSE of the network, BMFR and the
gated output against a many-sample render, the FP8 mode's layers), both
denoisers well below the 1-sample input, the frame's device-timed rate and its
end-to-end rate within a sane ratio, and the native library loaded."""
import json
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]


def test_bench_json_line(cuda):
    argv = ["bench.py", "--steps", "4", "--warmup", "3", "--width", "640", "--height", "352", "--instances", "200",
            "--texture-size", "64", "--ref-spp", "256", "--no-cpu-baseline", "--no-batch"]
    code = ("import runpy, sys; sys.argv = %r; runpy.run_path('bench.py', run_name='__main__'); "
            "print('MAPS', sorted({l.split()[-1] for l in open('/proc/self/maps') if '.so' in l}))" % argv)
    out = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert out.returncode == 0, out.stderr[-3000:]
    lines = [ln for ln in out.stdout.strip().splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "e2e", "roofline", "clocks", "gpu_launches", "stage_ms",
              "relmse", "grays_per_s", "traversal_grays_per_s", "bmfr_path", "neural_fp8_path"):
        assert k in d, k
    assert d["n_gpus"] == 1 and d["steps"] == 4 and d["warmup"] == 3 and d["unit"] == "fps" and d["value"] > 0
    e = d["e2e"]
    assert e["unit"] == "fps" and e["h2d_bytes_per_step"] > 0 and e["d2h_bytes_per_step"] == 640 * 352 * 4
    assert 0.3 < e["value"] / d["value"] < 1.2
    r = d["roofline"]
    assert r["bound"] == "hbm" and r["unit"] == "GB/s" and 0 < r["frac"] < 2 and r["achieved"] > 0
    for k in ("trace_closest", "shade", "accumulate", "bmfr", "neural", "neural_fp8"):
        assert d["stage_ms"][k] > 0, k
    q = d["relmse"]
    assert max(q["neural"], q["bmfr"]) < q["input_1spp"] and q["neural"] < 1.25 * q["bmfr"]
    assert q["neural_gated"] > 0 and 0 <= q["fallback_tiles"] <= q["tiles"]
    assert isinstance(d["neural_fp8_path"]["e4m3_layers"], list)
    assert d["gpu_launches"] > 0 and d["grays_per_s"] > 0
    maps = [ln for ln in out.stdout.splitlines() if ln.startswith("MAPS")][0]
    ours = [p for p in eval(maps[5:]) if p.startswith(str(ROOT))]
    assert str(ROOT / "vulkanpbrt_gb300" / "libvulkanpbrt_gb300.so") in ours, ours
