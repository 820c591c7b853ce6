"""The constants of the exact mode's float-float paths (csrc/swe_device.cuh),
re-derived here with 60-digit decimal arithmetic: the 2^(j/64) table of
exp_ff (hi = nearest float, lo = nearest float to the rest, pair within
2^-47), the three-part split of ln2/64 (first two parts with at most 11
significant bits, so k times them is exact for |k| < 2^13), 64/ln2, the
Taylor coefficients, and the split of the double 0.3 used by drag_factor."""
import math
import re
from decimal import Decimal, getcontext
from pathlib import Path

import numpy as np

SRC = (Path(__file__).resolve().parents[1] / "simplewinderosion_gb300" / "csrc" / "swe_device.cuh").read_text()
getcontext().prec = 60
LN2 = Decimal(2).ln()


def f32(bits: int) -> float:
    return float(np.uint32(bits).view(np.float32))


def nearest_f32(d: Decimal) -> float:
    return float(np.float32(float(d)))


def table(name: str) -> list[int]:
    body = re.search(name + r"\[64\] = \{(.*?)\};", SRC, re.S).group(1)
    vals = [int(v, 16) for v in re.findall(r"0x[0-9a-f]{8}", body)]
    assert len(vals) == 64
    return vals


def sig_bits(x: float) -> int:
    m, _ = math.frexp(abs(x))
    n = 0
    while m != int(m):
        m *= 2
        n += 1
    return n


def test_exp2_table():
    hi, lo = table("kExp2TabHi"), table("kExp2TabLo")
    for j in range(64):
        t = (Decimal(j) / 64 * LN2).exp()
        assert f32(hi[j]) == nearest_f32(t), j
        assert f32(lo[j]) == nearest_f32(t - Decimal(f32(hi[j]))), j
        assert abs(t - Decimal(f32(hi[j])) - Decimal(f32(lo[j]))) < t * Decimal(2) ** -47


def test_reduction_constants():
    c1, c2, c3 = f32(0x3C318000), f32(0xB65E8000), f32(0xAE02E308)
    assert sig_bits(c1) <= 11 and sig_bits(c2) <= 11
    c = LN2 / 64
    assert c3 == nearest_f32(c - Decimal(c1) - Decimal(c2))
    # |k| <= 8125 on -87 <= x <= 88: the split's error times k stays below 2^-46
    assert abs(c - Decimal(c1) - Decimal(c2) - Decimal(c3)) * 8192 < Decimal(2) ** -46
    assert f32(0x42B8AA3B) == nearest_f32(64 / LN2)
    for bits, v in ((0x3C088889, 1 / 120), (0x3D2AAAAB, 1 / 24), (0x3E2AAAAB, 1 / 6)):
        assert f32(bits) == float(np.float32(v))
    for pat in ("0x3c318000u", "0xb65e8000u", "0xae02e308u", "0x42b8aa3bu", "0x3c088889u", "0x3d2aaaabu",
                "0x3e2aaaabu"):
        assert pat in SRC


def test_drag_split_of_double_point_three():
    d = Decimal(0.3)  # the double nearest 0.3, exactly
    dhi, dlo = f32(0x3E99999A), f32(0xB24CCCCD)
    assert dhi == nearest_f32(d) and dlo == nearest_f32(d - Decimal(dhi))
    assert abs(d - Decimal(dhi) - Decimal(dlo)) < Decimal(2) ** -52
    assert "0x3e99999au" in SRC and "0xb24ccccdu" in SRC
