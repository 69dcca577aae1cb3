"""The tensor-core primitives (fortnet_gb300/csrc/tc.cuh) in isolation: one BF16 tcgen05.mma
product with FP32 accumulation in tensor memory for K-major and MN-major operands in the
library's core-matrix layout, against an FP64 product of the same values (tests/cpp/tc_probe.cu).
"""

import os
import subprocess

import pytest

from fortnet_gb300 import build as B

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_tcgen05_bf16_products_match_fp64(tmp_path):
    exe = str(tmp_path / "tc_probe")
    cmd = [B.nvcc_path(), *B.ARCH, "-O2", "-std=c++17", "-o", exe,
           os.path.join(HERE, "cpp", "tc_probe.cu")]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    res = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    print(res.stdout)
    lines = [l.split() for l in res.stdout.strip().splitlines()]
    assert len(lines) == 4, res.stdout + res.stderr
    for a_mn, b_mn, err, dmax, status in lines:
        assert int(status) == 0, f"mbarrier wait gave up (a_mn={a_mn}, b_mn={b_mn})"
        assert float(err) <= 1e-5 * float(dmax), (a_mn, b_mn, err)
    assert res.returncode == 0
