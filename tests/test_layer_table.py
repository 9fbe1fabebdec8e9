"""The U-Net's layer table in Python (`kpunet.CONVS`, used by training and
by the benchmark's per-layer timing) against the native network's table
(`kConvs` in csrc/neural.cu), and the timing workload's argument checks.
CPU only."""
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_python_layer_table_matches_native():
    from vulkanpbrt_gb300.kpunet import CONVS

    src = (ROOT / "vulkanpbrt_gb300" / "csrc" / "neural.cu").read_text()
    body = src[src.index("constexpr ConvSpec kConvs[]"):]
    body = body[:body.index("};")]
    native = [(m[0], int(m[1]), int(m[2]), int(m[3]), int(m[4]))
              for m in re.findall(r'\{"(\w+)",\s*(\d+),\s*(\d+),\s*(\d+),\s*(\d+)\}', body)]
    assert len(native) == 18
    assert native == [(name, c1, c2, cout, lvl) for name, (c1, c2), cout, lvl in CONVS]


def test_unet_layer_workload_rejects_unknown_kernels(monkeypatch):
    import sys

    sys.path.insert(0, str(ROOT))
    import bench

    monkeypatch.setattr(sys, "argv", ["bench.py", "--workload", "unet_layers", "--kernels", "bf16_tcgen05,int4"])
    with pytest.raises(SystemExit, match="unknown kernels"):
        bench.main()
