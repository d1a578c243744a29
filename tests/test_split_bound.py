"""The split-precision scheme's exactness bound, on the CPU.

The digit cut is restated here in numpy integer arithmetic (the kernels do
the same on the FP64 bit pattern): a row scaled by 2^-e so that |x| < 1/2,
rounded to X = round(x 2^(ws - e)) and split from the bottom into balanced
base-2^w digits.  With w = 6 and s = 9 every digit lies in [-32, 32], so a
digit product is at most 2^10 and diagonal d (d + 1 products per k) sums to at
most (d + 1) 2^21 over a 2048-wide K segment: at most 2^24, where fp32
accumulation is still exact, for every d <= 7.  Checked on operands built to
reach the bound (all digits at their extremes, one sign), on random operands,
and with fp32 accumulation emulated in 16-wide steps as the tensor pipe adds
them.
"""
import numpy as np
import pytest

W, S, KSEG = 6, 9, 2048


def cut(x):
    """Digits [S][n] (a_0 first) and the exponent of one row, as the kernels cut it."""
    m = float(np.abs(x).max())
    e = (int(np.frexp(m)[1]) if m > 0 else 0) + 1      # |x| < 2^(e-1)
    X = [int(v) for v in np.round(np.ldexp(x, W * S - e))]
    half, mask = 1 << (W - 1), (1 << W) - 1
    digits = []
    for _ in range(S - 1):
        a = [((v + half) & mask) - half for v in X]
        X = [(v - d) >> W for v, d in zip(X, a)]
        digits.append(a)
    digits.append(X)
    return np.array(digits[::-1], dtype=np.int64), e


def reconstruct(d):
    v = np.zeros(d.shape[1], dtype=object)
    for p in range(S):
        v = v * (1 << W) + d[p].astype(object)
    return v


def diag_sums(da, db):
    """Exact integer sum over k of every diagonal d = p + q < S."""
    return [int(sum((da[p] * db[d - p]).sum() for p in range(d + 1))) for d in range(S)]


def fp32_sums(da, db):
    """The same sums accumulated in fp32, 16 products of a diagonal per step."""
    out = []
    for d in range(S):
        prod = sum(da[p] * db[d - p] for p in range(d + 1)).astype(np.float64)
        acc = np.float32(0.0)
        for k0 in range(0, prod.size, 16):
            acc = np.float32(acc + np.float32(prod[k0:k0 + 16].sum()))
        out.append(int(acc))
    return out


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_digits_in_range_and_exact(seed):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(512) * np.exp(rng.uniform(-30, 30))
    d, e = cut(x)
    assert np.abs(d).max() <= 1 << (W - 1)
    # the digits reproduce the fixed-point integers exactly
    X = [int(v) for v in np.round(np.ldexp(x, W * S - e))]
    assert list(reconstruct(d)) == X


def test_worst_case_diagonals_stay_within_fp32_integers():
    # every digit of both operands at +32 (the bound), one K segment
    da = np.full((S, KSEG), 1 << (W - 1), dtype=np.int64)
    sums = diag_sums(da, da)
    for dd in range(S - 1):  # d <= 7
        assert sums[dd] == (dd + 1) * (1 << 10) * KSEG <= 1 << 24
    assert sums[S - 1] > 1 << 24  # the last diagonal (weight 2^-48) may round
    assert fp32_sums(da, da)[:S - 1] == sums[:S - 1]


@pytest.mark.parametrize("kind", ["one_sign", "random"])
def test_fp32_accumulation_exact_within_a_segment(kind):
    rng = np.random.default_rng(5)
    if kind == "one_sign":
        a, b = rng.uniform(0.5, 1.0, KSEG), rng.uniform(0.5, 1.0, KSEG)
    else:
        a, b = rng.standard_normal(KSEG), rng.standard_normal(KSEG)
    da, _ = cut(a)
    db, _ = cut(b)
    exact, f32 = diag_sums(da, db), fp32_sums(da, db)
    assert f32[:S - 1] == exact[:S - 1]


def test_one_segment_is_not_enough_beyond_2048():
    # the reason for K segments: digits of one sign near their bound (as in
    # rows of equal-signed values with aligned digits) over 11008 elements
    # drive the diagonals past 2^24 within a single accumulation, where fp32
    # sums are no longer exact ...
    rng = np.random.default_rng(7)
    da = rng.integers(16, 33, size=(S, 11008)).astype(np.int64)
    exact = diag_sums(da, da)
    assert max(exact[:S - 1]) > 1 << 24
    assert fp32_sums(da, da)[:S - 1] != exact[:S - 1]
    # ... while each 2048-wide segment stays exact
    for k0 in range(0, 11008, KSEG):
        seg = da[:, k0:k0 + KSEG]
        assert fp32_sums(seg, seg)[:S - 1] == diag_sums(seg, seg)[:S - 1]
