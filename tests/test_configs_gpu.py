"""The precision and batched workloads at their full sizes, through a
size-independent property: on the same job the split-precision path selects
exactly the lines of the FP64 GPU path and agrees with it to <= 1e-10 in S
(lines whose transition moment is at least 1e-4 of the largest; below that
both orders of evaluation lose digits to cancellation).  Every final block is
full size; the initial levels are the lowest few of each block (energy window),
which keeps the FP64 reference run short.

* c2v_precision: J = 20 -> 21, Nvib = 5000 with a log-uniform dipole
  (magnitudes 1e-8..1, the case that stresses the digit count), ~26k
  functions per symmetry, 2000 vectors per block.
* c3v_batched: the two largest J of the tetratomic C3v job (J = 39, 40,
  blocks up to 81k functions for E), 1500 vectors per block.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def keyed_sorted(pkg, eng):
    k = pkg.keyed(eng.lines(), eng.levels())
    return np.sort(k, order=["jI", "gammaI", "recI", "jF", "gammaF", "recF"])


def split_vs_fp64(pkg, prob, n_lower):
    e = np.sort(np.concatenate([b.energies[:n_lower] for b in prob.blocks.values()]))
    p = prob.params
    p.erange_lower = (0.0, float(e[n_lower - 1]))
    out = {}
    with pkg.Engine(0) as eng:
        eng.load(prob, precision=pkg.GI_PREC_FP64)
        for name, prec in (("fp64", pkg.GI_PREC_FP64), ("split", pkg.GI_PREC_SPLIT)):
            eng.set_params(p, precision=prec)
            eng.run()
            out[name] = keyed_sorted(pkg, eng)
    a, b = out["fp64"], out["split"]
    for f in ("jI", "gammaI", "recI", "jF", "gammaF", "recF"):
        assert np.array_equal(a[f], b[f])
    t = np.abs(a["t"]).max(axis=1)
    ok = t >= 1e-4 * t.max()
    rel = np.abs(b["S"] - a["S"]) / np.abs(a["S"])
    return len(a), float(rel[ok].max()), float(np.abs(b["t"] - a["t"]).max() / np.abs(a["t"]).max())


def test_precision_workload_full_size(pkg, synth):
    prob = synth.workload("c2v_precision", seed=3)
    n, rel, norm = split_vs_fp64(pkg, prob, 12)
    print("c2v_precision lines", n, "max rel err S", rel, "normwise", norm)
    assert n > 10000
    assert rel <= 1e-10 and norm <= 1e-12


def test_batched_workload_largest_blocks(pkg, synth):
    prob = synth.workload("c3v_batched", seed=4, jlist=[39, 40])
    n, rel, norm = split_vs_fp64(pkg, prob, 6)
    print("c3v_batched lines", n, "max rel err S", rel, "normwise", norm)
    assert n > 5000
    assert rel <= 1e-10 and norm <= 1e-12
