"""The benchmark's reference arm (the CPU restatement of the path, timed on
the host cores) on a small frame: one JSON line with the keys the
benchmark contract names, `impl` = reference, a `cpu_baseline` describing
the run and an `e2e` entry without host-device copies; the arm loads the
oracle's library and no other library of this repository. CPU only."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_json_line():
    argv = ["bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0", "--width", "160", "--height", "96",
            "--instances", "20", "--texture-size", "64"]
    code = ("import runpy, sys; sys.argv = %r; runpy.run_path('bench.py', run_name='__main__'); "
            "print('MAPS', sorted({l.split()[-1] for l in open('/proc/self/maps') if '.so' in l}))" % argv)
    out = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.strip().splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["n_gpus"] == 1 and d["steps"] == 1
    assert d["value"] > 0 and d["unit"] == "fps" and d["higher_is_better"] is True
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["width"] == 160 and d["config"]["height"] == 96
    maps = [ln for ln in out.stdout.splitlines() if ln.startswith("MAPS")][0]
    ours = [p for p in eval(maps[5:]) if p.startswith(str(ROOT))]
    assert ours == [str(ROOT / "oracle" / "_build" / "liboracle.so")], ours
