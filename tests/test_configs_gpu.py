"""The named workloads at their full sizes against the CPU oracle (the
double-double checker), line by line: identical line selection, and relative
error in S, A and I of at most 1e-11 (FP64 path) and 1e-10 (split path) on
every line above the intensity threshold of 1e-30 cm/molecule.

Each case is one reference run (J, J+1) of the workload with every final
level and the lowest few initial levels (the lower energy window), which keeps
the oracle's share of the test to seconds:

* c2v_plain: J = 9 -> 10, Nvib = 2000, 1000 vectors per block, 8 initial levels.
* c2v_precision: J = 20 -> 21, Nvib = 5000 with a log-uniform dipole
  (magnitudes 1e-8..1, the case that stresses the digit count), ~26k
  functions per symmetry, 2000 vectors per block, 2 initial levels.
* c3v_batched: the two largest J of the tetratomic C3v job (J = 39, 40, blocks
  up to 81k functions for E), 1500 vectors per block, 2 initial levels.
"""
import os

import numpy as np
import pytest

from paritylib import compare, with_threshold

pytestmark = pytest.mark.gpu

CASES = {"c2v_plain": ((9, 10), 8), "c2v_precision": ((20, 21), 2),
         "c3v_batched": ((39, 40), 2)}


@pytest.fixture(scope="module")
def samples(synth, oracle):
    cache = {}

    def get(name):
        if name not in cache:
            (j0, j1), nlow = CASES[name]
            prob = with_threshold(synth.workload(name, seed=5, jlist=[j0, j1]))
            e = np.sort(np.concatenate([b.energies for b in prob.blocks.values()]))
            prob.params.erange_lower = (prob.params.erange_lower[0], float(e[nlow - 1]))
            ref = oracle.run_pair(prob, (j0, j1), nthreads=os.cpu_count() or 1)
            cache.clear()  # one workload's arrays at a time
            cache[name] = (prob, ref)
        return cache[name]
    return get


@pytest.mark.parametrize("precision", ["fp64", "split"])
@pytest.mark.parametrize("name", list(CASES))
def test_workload_sample_matches_oracle(pkg, samples, name, precision):
    prob, ref = samples(name)
    prec = pkg.GI_PREC_SPLIT if precision == "split" else pkg.GI_PREC_FP64
    with pkg.Engine(0) as eng:
        eng.load(prob, precision=prec)
        eng.set_refine(1 << 20)  # doubtful lines re-evaluated exactly
        eng.run()
        got = pkg.keyed(eng.lines(), eng.levels())
        st = eng.stats()
    tol = 1e-10 if precision == "split" else 1e-11
    res = compare(got, ref, rtol_S=tol, norm_tol=tol / 10)
    print(name, precision, res, "doubtful", st["nlines_doubtful"], "refined",
          st["nlines_refined"])
    assert res["n"] > 1000
