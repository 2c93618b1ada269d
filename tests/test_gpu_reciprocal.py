"""The triangle test's reciprocal without a division (nbd::rcp_newton): for every float in the
range it is used on, the same bits as the correctly rounded 1 / det the reference arithmetic
prescribes (raytracing_sw.wgsl:64, the Moller-Trumbore inv_det).  Exhaustive: ~1.28G inputs,
about a second on the GPU."""
import os
import subprocess

import pytest

from nbounce_gb300 import build as B

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def test_rcp_newton_matches_correctly_rounded_division_everywhere(tmp_path):
    exe = str(tmp_path / "rcp_newton_check")
    src = os.path.join(HERE, "rcp_newton_check.cu")
    flags = list(B.NVCC_FLAGS)
    i = flags.index("-fPIC")  # the library's flags, less the shared-object one
    del flags[i - 1:i + 1]
    subprocess.run([B.nvcc(), *B.ARCH, *flags, src, "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches=0" in r.stdout, r.stdout
