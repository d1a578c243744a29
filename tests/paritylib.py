"""Helpers shared by the GPU parity tests: line-set comparison against the oracle."""
import numpy as np

KEYS = ("jI", "gammaI", "recI", "jF", "gammaF", "recF")


def sort_lines(a):
    return a[np.lexsort(tuple(a[k] for k in reversed(KEYS)))]


def compare(got, ref, rtol_S=1e-11, cond_floor=1e-4, norm_tol=1e-13):
    """Identical line selection and per-line accuracy.

    Returns a dict of error statistics.  Every line must satisfy the
    normwise bound |t_gpu - t_ref| <= norm_tol * max|t| over the job; lines
    whose moment is not tiny (|t| >= cond_floor * max|t|) must also satisfy
    the componentwise bound |S_gpu - S_ref| <= rtol_S * S_ref.  Lines below
    cond_floor lose relative accuracy to cancellation in any FP64 evaluation
    order, so for them the normwise bound is the meaningful one.
    """
    assert len(got) == len(ref), (len(got), len(ref))
    g, r = sort_lines(got), sort_lines(ref)
    for k in KEYS:
        assert np.array_equal(g[k], r[k]), f"line selection differs in {k}"
    out = {"n": len(r)}
    if len(r) == 0:
        return out
    assert np.array_equal(g["nu"], r["nu"])
    tmax = np.abs(r["t"]).max()
    dt = np.abs(g["t"] - r["t"]).max(axis=1)
    out["norm_err"] = float(dt.max() / tmax)
    assert out["norm_err"] <= norm_tol, out
    tl = np.sqrt(np.maximum(r["S"], 0))
    big = np.abs(r["t"]).max(axis=1) >= cond_floor * tmax
    relS = np.abs(g["S"] - r["S"]) / np.where(r["S"] > 0, r["S"], 1.0)
    out["rel_S_max_wellcond"] = float(relS[big].max()) if big.any() else 0.0
    out["rel_S_p99"] = float(np.quantile(relS, 0.99))
    out["rel_S_max_all"] = float(relS.max())
    out["frac_wellcond"] = float(big.mean())
    assert out["rel_S_max_wellcond"] <= rtol_S, out
    for f in ("A", "I"):
        rel = np.abs(g[f] - r[f]) / np.where(np.abs(r[f]) > 0, np.abs(r[f]), 1.0)
        out[f"rel_{f}_max_wellcond"] = float(rel[big].max()) if big.any() else 0.0
        assert out[f"rel_{f}_max_wellcond"] <= rtol_S * 10, (f, out)
    del tl
    return out
