"""Helpers shared by the GPU parity tests: line-set comparison against the oracle."""
import numpy as np

KEYS = ("jI", "gammaI", "recI", "jF", "gammaF", "recF")
# the intensity threshold of the workloads (cm/molecule); parity is judged on
# every line above it
THRESH_I = 1e-30


def sort_lines(a):
    return a[np.lexsort(tuple(a[k] for k in reversed(KEYS)))]


def with_threshold(prob, thresh=THRESH_I):
    """The workloads' intensity threshold on a synthetic problem."""
    prob.params.thresh_intensity = thresh
    return prob


def compare(got, ref, rtol_S=1e-11, norm_tol=1e-13):
    """Identical line selection and per-line accuracy on every line.

    Both sides apply the job's thresholds, so every line compared is a line
    above the intensity threshold.  Each must satisfy
    |S_gpu - S_ref| <= rtol_S * S_ref, and the same relative bound holds for
    A and I (both are S times exact per-line factors).  The oracle evaluates
    in double-double, so the bound measures the engine, also on lines whose
    transition moment cancels far below its terms.  The normwise transition
    moment error |t_gpu - t_ref| <= norm_tol * max|t| is reported and checked
    too.  Returns error statistics.
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
    relS = np.abs(g["S"] - r["S"]) / np.abs(r["S"])
    worst = int(np.argmax(relS))
    out["rel_S_max"] = float(relS[worst])
    out["rel_S_p99"] = float(np.quantile(relS, 0.99))
    out["worst_t_over_max"] = float(np.abs(r["t"][worst]).max() / tmax)
    for f in ("A", "I"):
        rel = np.abs(g[f] - r[f]) / np.abs(r[f])
        out[f"rel_{f}_max"] = float(rel.max())
    assert out["norm_err"] <= norm_tol, out
    assert out["rel_S_max"] <= rtol_S, out
    assert out["rel_A_max"] <= rtol_S and out["rel_I_max"] <= rtol_S, out
    return out
