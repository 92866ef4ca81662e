"""The two FP32 splits behind the tensor-core kernels, restated in NumPy.

1. The filter's three-term BF16 split (k_split3 in csrc/spmm_umma.cu):
   v0 = bf16(v), v1 = bf16(v - v0), v2 = bf16(v - v0 - v1).  For normal FP32
   values v = v0 + v1 + v2 exactly, |v1| <= 2^-8 |v|, |v2| <= 2^-17 |v|, and
   the three products of order 3 that the FP32 degrees leave out (v1w2,
   v2w1, v2w2) stay below 2^-24 of |v w| together.
2. The exact integer slicing of the contraction engine (slice8 in
   csrc/tgemm.cu): with max |v| < 2^e over a group, x = v 2^(8-e) becomes
   a0 + a1/256 + a2/65536 with integers |a0| <= 256, |a1|, |a2| <= 128, the
   rounding below 2^-17 on that grid, and every level sum of slice products
   over a group of 192 values of K is an integer below 2^24 (exact in an FP32
   accumulator)."""
import numpy as np


def bf16(x):
    """Round FP32 to BF16 (nearest, ties to even), returned as FP32."""
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return (r.astype(np.uint32) << 16).view(np.float32)


def split3(v):
    v = np.asarray(v, np.float32)
    h0 = bf16(v)
    r1 = (v - h0).astype(np.float32)
    h1 = bf16(r1)
    h2 = bf16((r1 - h1).astype(np.float32))
    return h0, h1, h2


def random_fp32(rng, n):
    v = rng.uniform(1, 2, n) * 2.0 ** rng.integers(-30, 30, n)
    return (v * np.where(rng.random(n) < 0.5, -1, 1)).astype(np.float32)


def test_three_term_bf16_split_bounds():
    rng = np.random.default_rng(11)
    v, w = random_fp32(rng, 1 << 20), random_fp32(rng, 1 << 20)
    h0, h1, h2 = split3(v)
    g0, g1, g2 = split3(w)
    a, b = np.abs(v.astype(np.float64)), np.abs(w.astype(np.float64))
    assert np.array_equal(h0.astype(np.float64) + h1 + h2, v.astype(np.float64))
    assert np.all(np.abs(h1) <= 2.0 ** -8 * a)
    assert np.all(np.abs(h2) <= 2.0 ** -17 * a)
    # every term is a BF16 value: 8 significant bits
    for h in (h0, h1, h2):
        assert np.array_equal(bf16(h), h)
    dropped = (np.abs(h1.astype(np.float64) * g2) + np.abs(h2.astype(np.float64) * g1)
               + np.abs(h2.astype(np.float64) * g2))
    assert np.all(dropped <= 2.0 ** -24 * a * b)


def grid_exp(amax):
    return 0 if amax == 0 else int(np.frexp(np.float32(amax))[1])


def slice3(v, e):
    """slice8's arithmetic, in FP32 as the kernel does it."""
    x = (np.asarray(v, np.float32) * np.float32(2.0 ** (8 - e))).astype(np.float32)
    a0 = np.rint(x).astype(np.float32)
    r = ((x - a0) * np.float32(256)).astype(np.float32)
    a1 = np.rint(r).astype(np.float32)
    a2 = np.rint(((r - a1) * np.float32(256)).astype(np.float32)).astype(np.float32)
    return x, a0, a1, a2


def test_integer_slices_and_level_sums():
    rng = np.random.default_rng(12)
    for trial in range(50):
        g = random_fp32(rng, 192) * np.float32(10.0 ** rng.uniform(-3, 3))
        g[rng.integers(0, 192, 8)] = 0.0
        e = grid_exp(np.abs(g).max())
        assert np.abs(g).max() < 2.0 ** e
        x, a0, a1, a2 = slice3(g, e)
        assert np.abs(a0).max() <= 256 and np.abs(a1).max() <= 128 and np.abs(a2).max() <= 128
        for a in (a0, a1, a2):              # integers of at most 9 bits: exact in BF16
            assert np.array_equal(np.rint(a), a) and np.array_equal(bf16(a), a)
        rec = a0.astype(np.float64) + a1 / 256.0 + a2 / 65536.0
        assert np.abs(rec - x.astype(np.float64)).max() <= 2.0 ** -17
    # worst case of each level over 192 values of K, slices at their bounds
    m = [256, 128, 128]
    levels = [m[0] * m[0], 2 * m[0] * m[1], 2 * m[0] * m[2] + m[1] * m[1], 2 * m[1] * m[2]]
    assert all(192 * lv < 2 ** 24 for lv in levels)


def test_sliced_dot_products_match_exact_sums():
    """A 192-deep dot product through the slices: level sums are exact
    integers, and the result differs from the exact sum only by the slicing's
    rounding (2^-17 of the grid on each operand, so 2^-24 of 2^(ea + eb)
    per term) and the dropped a2 b2 level (2^-34 of 2^(ea + eb) per term)."""
    rng = np.random.default_rng(13)
    for trial in range(50):
        a = random_fp32(rng, 192) * np.float32(10.0 ** rng.uniform(-3, 3))
        b = random_fp32(rng, 192) * np.float32(10.0 ** rng.uniform(-3, 3))
        ea, eb = grid_exp(np.abs(a).max()), grid_exp(np.abs(b).max())
        _, p0, p1, p2 = slice3(a, ea)
        _, q0, q1, q2 = slice3(b, eb)
        P = [p.astype(np.int64) for p in (p0, p1, p2)]
        Q = [q.astype(np.int64) for q in (q0, q1, q2)]
        S = [int(np.dot(P[0], Q[0])), int(np.dot(P[0], Q[1]) + np.dot(P[1], Q[0])),
             int(np.dot(P[0], Q[2]) + np.dot(P[1], Q[1]) + np.dot(P[2], Q[0])),
             int(np.dot(P[1], Q[2]) + np.dot(P[2], Q[1]))]
        assert all(abs(s) < 2 ** 24 for s in S)
        got = (S[0] + S[1] / 256.0 + S[2] / 65536.0 + S[3] / 16777216.0) * 2.0 ** (ea + eb - 16)
        exact = float(np.dot(a.astype(np.float64), b.astype(np.float64)))
        bound = 192 * 2.0 ** (ea + eb - 16) * (2 * 256 * 2.0 ** -17 + 2.0 ** -32 * 128 * 128 + 2.0 ** -34)
        assert abs(got - exact) <= bound
