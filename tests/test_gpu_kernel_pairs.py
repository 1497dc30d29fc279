"""The packed kernel pairs (both scales' cubic spline and gradient as float2 pairs,
used by the single-scene gathers) against the scalar kernels, bit for bit, on
4M random distances per radius.  Built with the library's own nvcc flags."""
import os
import subprocess

import pytest

from twoscalesplit_gb300 import build

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def probe(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("pairs") / "kernel_pairs")
    subprocess.check_call([build.nvcc(), *build.flags(), os.path.join(HERE, "cuda", "kernel_pairs.cu"), "-o", exe])
    return exe


@pytest.mark.parametrize("r", ["0.001132", "0.0667", "0.016", "0.0004"])
def test_packed_kernel_pairs_equal_scalar_kernels(probe, r):
    out = subprocess.check_output([probe, r], timeout=120).decode()
    assert out.strip().startswith("mismatches 0 of"), out
