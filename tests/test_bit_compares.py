"""The integer-pipe comparisons and scalings of the momentum kernels
(curvib_old_gb300/csrc/kernels_momentum.cu: visc_blocked, gt_01, lt_01,
scale_down), restated here on 64-bit patterns and checked against the FP64
operations they stand for on the values where the two could part: signed
zeros, subnormals, the constants' neighbours, infinities and NaNs of both
signs."""
import math
import struct

import numpy as np

B01, B05, B7 = 0x3FB999999999999A, 0x3FE0000000000000, 0x401C000000000000
BINF, BNEGINF = 0x7FF0000000000000, -0x10000000000000  # 0xFFF0000000000000 as int64


def bits(x):
    return struct.unpack("<q", struct.pack("<d", x))[0]


def from_bits(b):
    return struct.unpack("<d", struct.pack("<q", b))[0]


def visc_blocked(v):
    b = bits(v)
    return B05 < b < B7


def gt_01(v):
    b = bits(v)
    return B01 < b <= BINF


def lt_01(v):
    b = bits(v)
    return b < B01 and not (BNEGINF < b < 0)


def scale_down(x, k):
    b = bits(x)
    e = (b >> 52) & 0x7FF
    if k < e < 0x7FF:
        return from_bits(b - (k << 52))
    if b & 0x7FFFFFFFFFFFFFFF == 0:
        return x
    return x * (0.5 if k == 1 else 0.25)


def _values():
    nan_neg = from_bits(-0x7FFFFFFFFFFFF)  # a NaN with the sign bit
    base = [0.0, -0.0, 5e-324, -5e-324, 2.2250738585072014e-308, -2.2250738585072014e-308, 1e-310, -1e-310,
            0.1, 0.5, 7.0, 1.0, 3.0, 1.2, 1e300, 1.7976931348623157e308, math.inf, -math.inf, math.nan, nan_neg]
    out = []
    for v in base:
        out.append(v)
        if math.isfinite(v):
            out += [math.nextafter(v, math.inf), math.nextafter(v, -math.inf), -v]
    return [float(v) for v in out]


def test_compares_match_fp64():
    for v in _values():
        assert visc_blocked(v) == (v > 0.5 and v < 7.0), v
        assert gt_01(v) == (v > 0.1), v
        assert lt_01(v) == (v < 0.1), v


def test_scalings_match_fp64():
    for v in _values():
        for k, f in ((1, 0.5), (2, 0.25)):
            want, got = np.float64(v) * np.float64(f), scale_down(v, k)
            if math.isnan(want):
                assert math.isnan(got)
            else:
                assert bits(got) == bits(float(want)), (v, k)
