"""The division by a per-scene constant (tss_device.cuh: recip_split on the host,
div_const on the device) checked in exact rational arithmetic on the CPU:
recip_split's yh is the correctly rounded reciprocal RN(1/b) for every divisor
tested, and div_const's four steps -- q0 = fma(a, yh, a*yl), r = fma(-q0, b, a),
q = fma(r, yh, q0), each rounded once to FP32 -- give RN(a/b) for seeded samples of
a in the kernels' range (0 <= a <= 4b) and beyond.  The GPU test
(test_gpu_div_const.py) runs the same comparison against the hardware division on
every float in range."""
import math
import os
import struct
import subprocess
from fractions import Fraction

import numpy as np
import pytest

from twoscalesplit_gb300 import build

HERE = os.path.dirname(os.path.abspath(__file__))


def rn32(x):
    """x (a Fraction) rounded to the nearest FP32 value, ties to even (subnormals
    included: below 2^-126 the spacing is 2^-149)."""
    if x == 0:
        return 0.0
    s = -1 if x < 0 else 1
    x = abs(x)
    e = math.floor(math.log2(x.numerator) - math.log2(x.denominator))
    while Fraction(2) ** e > x:
        e -= 1
    while Fraction(2) ** (e + 1) <= x:
        e += 1
    assert e <= 127
    e = max(e, -126)
    m = x / Fraction(2) ** (e - 23)  # in [2^23, 2^24) for normal results
    q, r = divmod(m.numerator, m.denominator)
    if 2 * r > m.denominator or (2 * r == m.denominator and q % 2 == 1):
        q += 1
    return s * float(Fraction(q) * Fraction(2) ** (e - 23))


def f32(v):
    return struct.unpack("f", struct.pack("f", v))[0]


def div_const(a, b, yh, yl):
    fa, fb, fyh, fyl = (Fraction(v) for v in (a, b, yh, yl))
    q0 = rn32(fa * fyh + Fraction(rn32(fa * fyl)))
    r = rn32(-Fraction(q0) * fb + fa)
    return rn32(Fraction(r) * fyh + Fraction(q0))


@pytest.fixture(scope="module")
def splits(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("recip") / "recip_split_host")
    subprocess.check_call([build.nvcc(), *build.flags(), os.path.join(HERE, "cuda", "recip_split_host.cu"), "-o", exe])
    rng = np.random.default_rng(11)
    bs = [0.001132, 0.000566, 0.0667, 0.03335, 0.016, 0.008, 0.0004, 0.0002, 1.0, 3.0, 0.1, 0.7, 2.0 ** -40,
          2.0 ** 40, 12345.678] + list(np.exp2(rng.uniform(-40, 40, 200)))
    bs = [f32(float(b)) for b in bs]
    out = subprocess.check_output([exe], input="".join(f"{b.hex()}\n" for b in bs).encode(), timeout=60).decode()
    rows = [tuple(float.fromhex(t) for t in line.split()) for line in out.split("\n") if line.strip()]
    assert len(rows) == len(bs)
    return rows


def test_reciprocal_split_is_the_correctly_rounded_reciprocal(splits):
    for b, yh, yl in splits:
        assert yh == rn32(1 / Fraction(b)), (b.hex(), yh.hex())
        # yl carries the rest of 1/b to FP32 precision of its own
        rest = 1 / Fraction(b) - Fraction(yh)
        assert abs(Fraction(yl) - rest) <= abs(rest) * Fraction(1, 2 ** 23), b.hex()


def test_division_steps_give_the_correctly_rounded_quotient(splits):
    rng = np.random.default_rng(5)
    checked = 0
    for b, yh, yl in splits:
        # a = 2d for pair distances d in [0, r] (a <= 4b for both radii), a few ulps
        # around the q = 1 and q = 2 branch points, and a wide log-uniform range
        a_vals = list(rng.uniform(0.0, 4.0 * b, 60))
        for q in (0.5, 1.0, 2.0, 4.0):
            c = f32(q * b)
            a_vals += [c, np.nextafter(np.float32(c), np.float32(0)), np.nextafter(np.float32(c), np.float32(1e38))]
        a_vals += list(b * np.exp2(rng.uniform(-60, 4, 20)))
        for a in a_vals:
            a = f32(float(a))
            if a != 0 and abs(a) < 2.0 ** -75:
                continue
            got = div_const(a, b, yh, yl)
            want = rn32(Fraction(a) / Fraction(b))
            assert got == want, (a.hex(), b.hex(), got, want)
            checked += 1
    assert checked > 15000


def test_cell_coordinates_of_tiny_offsets_truncate_to_zero(splits):
    """The grid coordinates use the same steps (cell_quot).  Below |a| = 2^-75 they
    may leave the normal range, but the quotient stays far below 1 in magnitude,
    so its truncation -- the cell index -- is 0, as the IEEE quotient's is."""
    rng = np.random.default_rng(9)
    for b, yh, yl in splits[::5]:
        for a in list(np.exp2(rng.uniform(-149, -75, 40))) + [2.0 ** -149, 2.0 ** -76]:
            a = f32(float(a))
            for sa in (a, -a):
                got = div_const(sa, b, yh, yl)
                want = rn32(Fraction(sa) / Fraction(b))
                assert abs(got) < 2.0 ** -30 and int(got) == int(want) == 0, (sa, b)


def cell_quot(a, b, yh, yl):
    """tss_device.cuh cell_quot: finite offsets through the division steps,
    infinite and NaN ones passed through."""
    return div_const(a, b, yh, yl) if math.isfinite(a) else a


def test_cell_coordinates_beyond_the_exhaustive_range(splits):
    """Grid coordinates between 2^20 and 2^31 cells (past the GPU test's exhaustive
    range; the clamp to the grid only reads them there) truncate as the IEEE
    quotient does, and infinite or NaN offsets give the division's own result."""
    rng = np.random.default_rng(13)
    for b, yh, yl in splits[::3]:
        for a in b * np.exp2(rng.uniform(20, 31, 25)):
            for sa in (f32(float(a)), -f32(float(a))):
                got = cell_quot(sa, b, yh, yl)
                assert got == rn32(Fraction(sa) / Fraction(b)), (sa, b)
        assert cell_quot(math.inf, b, yh, yl) == math.inf
        assert cell_quot(-math.inf, b, yh, yl) == -math.inf
        assert math.isnan(cell_quot(math.nan, b, yh, yl))
