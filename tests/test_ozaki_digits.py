"""The digit split of the FP64 tensor-core GEMM (digits6 in csrc/ozgemm.cu),
restated step by step with Python integers: from the double's bits, a value
v with |v| < 2^e becomes six balanced base-256 digits of v 2^(8 - e) rounded
to 2^-40, each exact in BF16 (|d0| <= 256, |d1..d5| <= 128), and the level
sums of 96 digit products stay below 2^24."""
import struct

import numpy as np


def digits6(v: float, e: int):
    bits = struct.unpack("<Q", struct.pack("<d", v))[0]
    hi, lo = bits >> 32, bits & 0xFFFFFFFF
    E = (hi >> 20) & 0x7FF
    xl = xh = 0
    if E != 0:
        M = (((hi & 0xFFFFF) | 0x100000) << 32) | lo
        rs = 1075 - 48 + e - E
        assert rs >= 5
        if rs < 63:
            X = (M + (1 << (rs - 1))) >> rs
            xl, xh = X & 0xFFFFFF, X >> 24
    g = [0] * 6
    t = xl
    for i in (5, 4, 3):
        g[i] = ((t + 128) & 255) - 128
        t = (t + 128) >> 8
    u = xh + t
    for i in (2, 1):
        g[i] = ((u + 128) & 255) - 128
        u = (u + 128) >> 8
    g[0] = u
    return [-x for x in g] if bits >> 63 else g


def row_exp(values):
    m = max((struct.unpack("<Q", struct.pack("<d", abs(x)))[0] >> 52) & 0x7FF for x in values)
    return 0 if m == 0 else min(m, 2046) - 1022


def test_digits_reconstruct_and_stay_in_bf16_range():
    rng = np.random.default_rng(3)
    for trial in range(40):
        row = rng.standard_normal(64) * 10.0 ** rng.uniform(-30, 30)
        row[rng.integers(0, 64, 4)] *= 10.0 ** rng.uniform(-12, 0, 4)
        e = row_exp(row)
        assert np.max(np.abs(row)) < 2.0 ** e
        for v in row:
            d = digits6(float(v), e)
            assert abs(d[0]) <= 256 and all(abs(x) <= 128 for x in d[1:])
            got = sum(x * 2.0 ** (-8 * i) for i, x in enumerate(d))
            exact = float(v) * 2.0 ** (8 - e)
            # rounding to 2^-40 of the scaled value (|value| < 256)
            assert abs(got - exact) <= 2.0 ** -41 * (1 + 1e-12)


def test_level_sums_below_2_24():
    """Worst case of one level over a 96-deep group: digits at their bounds."""
    d_max = [256, 128, 128, 128, 128, 128]
    for level in range(6):
        per_k = sum(d_max[i] * d_max[level - i] for i in range(level + 1))
        assert 96 * per_k < 2 ** 24
