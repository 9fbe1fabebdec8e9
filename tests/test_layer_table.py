"""The U-Net's layer table in Python (`kpunet.CONVS`, used by training and
by the per-layer timing tool) against the native network's table
(`kConvs` in csrc/neural.cu), and the timing tool's argument checks. CPU
only."""
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


def test_layer_times_rejects_unknown_kernels():
    from vulkanpbrt_gb300 import layer_times

    with pytest.raises(SystemExit):
        layer_times.main(["--kernels", "bf16_tcgen05,int4"])
