"""The double-FP32 multiply-add that the FP64-data GEMMs use on the FP32 pipe
(f2_fma in csrc/ttg_internal.cuh), restated step by step in NumPy float32:
the value split, the error-free product, the two-sum and the lazily
normalised accumulator keep about 2^-47 relative accuracy over long sums,
far beyond FP32 and close to FP64."""
import numpy as np

f32 = np.float32


def to_f2(x):
    h = np.float32(x)
    return h, np.float32(x - np.float64(h))


def fmaf(a, b, c):
    # a*b is exact in float64 (24 + 24 significant bits); one rounding to float32
    return np.float32(np.float64(a) * np.float64(b) + np.float64(c))


def f2_fma(acc, a, b):
    ah, al = a
    bh, bl = b
    p = f32(ah * bh)
    e = fmaf(ah, bh, -p)
    e = fmaf(ah, bl, e)
    e = fmaf(al, bh, e)
    s = f32(acc[0] + p)
    v = f32(s - acc[0])
    t = f32(f32(acc[0] - f32(s - v)) + f32(p - v))
    return s, f32(acc[1] + f32(t + e))


def test_df64_dot_products_reach_double_accuracy():
    rng = np.random.default_rng(5)
    worst = 0.0
    for trial in range(6):
        K = 4096
        x = rng.standard_normal(K) * np.exp(rng.uniform(-3, 3, K))
        y = rng.standard_normal(K)
        acc = (f32(0.0), f32(0.0))
        for i in range(K):
            acc = f2_fma(acc, to_f2(x[i]), to_f2(y[i]))
        got = np.float64(acc[0]) + np.float64(acc[1])
        ref = float(np.sum(np.longdouble(x) * np.longdouble(y)))
        scale = float(np.sum(np.abs(x * y)))
        worst = max(worst, abs(got - ref) / scale)
    # FP32 accumulation would give ~1e-7 here; the double-FP32 sum stays near 1e-14
    assert worst < 2.0 ** -40, worst


def f2_renorm(acc):
    s = f32(acc[0] + acc[1])
    return s, f32(acc[1] - f32(s - acc[0]))


def long_sums(n_terms, renorm_every):
    """16 sums of n_terms positive products (a Gram diagonal's shape), all
    advanced together; returns the worst error relative to the sum."""
    rng = np.random.default_rng(11)
    x = rng.standard_normal((n_terms, 16))
    xh = x.astype(f32)
    xl = (x - xh.astype(np.float64)).astype(f32)
    acc = (np.zeros(16, f32), np.zeros(16, f32))
    for i in range(n_terms):
        acc = f2_fma(acc, (xh[i], xl[i]), (xh[i], xl[i]))
        if renorm_every and (i + 1) % renorm_every == 0:
            acc = f2_renorm(acc)
    got = acc[0].astype(np.float64) + acc[1].astype(np.float64)
    ref = np.sum(x.astype(np.longdouble) ** 2, axis=0).astype(np.float64)
    return float(np.max(np.abs(got - ref) / ref))


def test_renormalised_accumulator_keeps_long_sums_accurate():
    """The GEMM loops fold lo into hi every 16 steps (f2_renorm).  Without it,
    lo grows like the square root of the number of steps and its own FP32
    rounding sets the error: 8e-11 relative over 100,000 terms, growing
    linearly, which made a 512,000-row Gram matrix indefinite by more than
    1e-8 after unit scaling.  With it the error is a random walk of 2^-48
    steps: 1e-12 over 100,000 terms."""
    plain = long_sums(100_000, 0)
    folded = long_sums(100_000, 16)
    assert folded < 5e-12, folded
    assert plain > 20 * folded, (plain, folded)
