"""The split-precision GEMM alone on chosen operands (gi_probe_split_gemm).

Within one launch each diagonal of digit products is summed in fp32, exact
while the sum stays below 2^24; with w = 6 that holds for any operands up to
K = 2048, so longer K runs as 2048-wide segments whose FP64 results are
added.  The hardest case for that bound is operands of one sign with every
leading digit near its maximum: all-positive rows of length 11008 put the
leading diagonal's sum above 2^25, where unsegmented fp32 sums would lose
about 5e-7 relative.  Checked here against FP64 dot products, on every
kernel (GI_SPLIT_FORCE), with ragged K and rows.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KINDS = ["9:64", "6:64", "7:64", "8:64"]  # 9: the 2-SM pair (cta_group::2)
PLAIN = ["0:64", "1:64", "2:64"]


def rel_err(got, want):
    return float(np.abs(got - want).max() / np.abs(want).max())


@pytest.mark.parametrize("K", [11008, 4160, 2048])
def test_one_sign_operands_long_k(pkg, K):
    rng = np.random.default_rng(K)
    A = rng.uniform(0.5, 1.0, (200, K))
    B = rng.uniform(0.5, 1.0, (72, K))
    want = A @ B.T
    got = pkg.split_gemm(A, B)
    # FP64 dot products of one-signed terms: relative error ~ sqrt(K) 2^-53
    assert rel_err(got, want) <= 1e-13, rel_err(got, want)


@pytest.mark.parametrize("layout,force", [("grouped", k) for k in KINDS] +
                         [("plain", k) for k in PLAIN])
def test_every_kernel_two_segments(pkg, monkeypatch, layout, force):
    monkeypatch.setenv("GI_SPLIT_LAYOUT", layout)
    monkeypatch.setenv("GI_SPLIT_FORCE", force)
    rng = np.random.default_rng(7)
    K = 2048 + 64 * 3 - 17  # two segments, the last ragged (K padded to 64)
    A = rng.uniform(0.25, 1.0, (300, K))
    B = rng.standard_normal((130, K)) + 1.5
    want = A @ B.T
    got = pkg.split_gemm(A, B)
    assert rel_err(got, want) <= 1e-13, rel_err(got, want)


def test_mixed_signs_and_scales(pkg):
    """Rows spanning 1e-8..1 (per-row exponents) and mixed signs."""
    rng = np.random.default_rng(3)
    K = 6000
    A = rng.standard_normal((130, K)) * np.exp(rng.uniform(np.log(1e-8), 0.0, (130, 1)))
    B = rng.standard_normal((257, K))
    want = A @ B.T
    got = pkg.split_gemm(A, B)
    row = np.abs(got - want).max(axis=1) / (np.abs(A).sum(axis=1) * np.abs(B).max())
    assert row.max() <= 1e-15
