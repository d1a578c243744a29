"""Where the reference sources were compiled here (oracle/_ref), compare the
oracle with the reference's own functions on fresh random inputs."""
import ctypes as C

import numpy as np
import pytest


@pytest.fixture(scope="module")
def ref(oracle):
    if not oracle.ref_available():
        pytest.skip("reference pin library not built (reference sources absent)")
    return oracle.ref()


def test_threej_large_jmax(oracle, ref):
    jmax = 60
    a = oracle.threej_table(jmax)
    b = np.zeros_like(a)
    ref.ref_precompute_threej(jmax, oracle.ptr(b, oracle.f64p))
    assert np.array_equal(a, b)


@pytest.mark.parametrize("seed", [21, 22])
def test_half_ls_random(oracle, synth, ref, seed):
    prob = synth.make_c3v(seed, 14, [2, 3, 4], nvec_max=3)
    N = prob.N
    rec = prob.mu.reshape(3, N, N)
    flip = np.ascontiguousarray(np.transpose(rec, (0, 2, 1))).reshape(-1)
    tj = oracle.threej_table(4)
    dg = np.array(prob.degen, np.int32)
    rng = np.random.default_rng(seed)
    for jI in (2, 3, 4):
        for jF in (jI - 1, jI, jI + 1):
            if jF not in prob.bases:
                continue
            bI, bF = prob.bases[jI], prob.bases[jF]
            vp = rng.standard_normal(bI.Maxcontracts)
            keep = oracle.Keep()
            oI, oF = oracle.make_basis(bI, keep), oracle.make_basis(bF, keep)
            theirs = np.zeros(bF.Maxcontracts)
            ref.ref_half_ls_flipped(C.byref(oI), C.byref(oF), prob.nrep, oracle.ptr(dg, oracle.i32p),
                                    N, oracle.ptr(flip, oracle.f64p), 4, oracle.ptr(tj, oracle.f64p),
                                    oracle.ptr(vp, oracle.f64p), oracle.ptr(theirs, oracle.f64p))
            mine = oracle.half_ls(bI, bF, N, prob.mu, 4, vp)
            assert np.abs(mine - theirs).max() <= 1e-14 * np.abs(theirs).max()
