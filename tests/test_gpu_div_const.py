"""Division by a per-scene constant (div_const, the pair kernels' q = 2d / r) against
the IEEE division, bit for bit, on every float in the range the kernels use, for
64 divisors.  Built with the library's own nvcc flags."""
import os
import subprocess

import pytest

from twoscalesplit_gb300 import build

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def test_division_by_a_constant_equals_ieee_division(tmp_path):
    exe = str(tmp_path / "div_const")
    subprocess.check_call([build.nvcc(), *build.flags(), os.path.join(HERE, "cuda", "div_const.cu"), "-o", exe])
    out = subprocess.check_output([exe], timeout=300).decode()
    assert out.strip().splitlines()[-1].startswith("mismatches 0 of"), out
