"""The CPU oracle against fixtures produced by the reference's own code
(tests/golden/make_golden.py): its 3j table, its kernels run on the CPU, its
dipole reader and its filters."""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import GOLDEN


def test_threej_bit_exact(oracle):
    ref = np.load(os.path.join(GOLDEN, "threej_ref_j24.npy"))
    mine = oracle.threej_table(24)
    assert np.array_equal(mine, ref)


def test_three_j_known_values(oracle):
    L = oracle.lib()
    # TROVE phase convention: three_j(2,1,2,1,0,-1)
    assert abs(L.or_three_j(2, 1, 2, 1, 0, -1) - 0.18257418583505522) < 1e-15
    # selection rules give exact zeros
    assert L.or_three_j(1, 1, 3, 0, 0, 0) == 0.0
    assert L.or_three_j(2, 1, 2, 1, 1, -1) == 0.0
    # orthogonality: sum_{k1,k2} (j1 j2 j3; k1 k2 -k3)^2 = 1/(2j3+1)
    for j1, j3 in [(3, 3), (5, 4), (7, 8)]:
        for k3 in range(-j3, j3 + 1):
            s = sum(L.or_three_j(j1, 1, j3, k1, k3 - k1, -k3) ** 2 for k1 in range(-j1, j1 + 1))
            assert abs(s - 1.0 / (2 * j3 + 1)) < 1e-13


@pytest.mark.parametrize("name", ["c2v", "c3v"])
def test_kernels_match_reference(oracle, synth, name):
    prob = synth.load(os.path.join(GOLDEN, f"{name}_problem.npz"))
    fx = np.load(os.path.join(GOLDEN, f"{name}_kernels.npz"))
    N = prob.N
    # read_dipole_flipped: flipped[f + i*N + c*N^2] = record mu_c(i, f)
    flip = fx["flipped_dipole"].reshape(3, N, N)  # [c][i][f]
    rec = prob.mu.reshape(3, N, N)                 # [c][f][i] (record i + f*N)
    assert np.array_equal(flip, np.transpose(rec, (0, 2, 1)))
    for (J, g), blk in sorted(prob.blocks.items()):
        if blk.nvec == 0:
            continue
        for d in range(prob.degen[g]):
            mine = oracle.correlate(prob.bases[J], prob.nrep, prob.degen, d, g, blk.vecs[0])
            np.testing.assert_allclose(mine, fx[f"corr_{J}_{g}_{d}"], rtol=0, atol=1e-15)
    js = prob.jlist
    for jI in js:
        for jF in js:
            if abs(jI - jF) > 1:
                continue
            ref = fx[f"hls_{jI}_{jF}"]
            mine = oracle.half_ls(prob.bases[jI], prob.bases[jF], N, prob.mu, max(js),
                                  fx[f"hls_in_{jI}_{jF}"])
            scale = np.abs(ref).max()
            assert np.abs(mine - ref).max() <= 1e-14 * scale


@pytest.mark.parametrize("name", ["c2v", "c3v"])
def test_filters_match_reference(oracle, synth, name):
    fx = np.load(os.path.join(GOLDEN, f"{name}_filters.npz"))
    prob = synth.load(os.path.join(GOLDEN, f"{name}_problem.npz"))
    if name == "c3v":
        prob.params.reduced = True
    nm = prob.params.nmodes
    keep = oracle.Keep()
    js = fx["jvals"]
    job = oracle.make_job(prob, (int(js[0]), int(js[1])), keep)
    job.erange_lower[:] = list(fx["erange_lower"])
    job.erange_upper[:] = list(fx["erange_upper"])
    job.freq_window[:] = list(fx["freq_window"])
    ql = keep(np.ascontiguousarray(fx["quanta_lower"], np.int32))
    qu = keep(np.ascontiguousarray(fx["quanta_upper"], np.int32))
    job.quanta_lower = oracle.ptr(ql, oracle.i32p)
    job.quanta_upper = oracle.ptr(qu, oracle.i32p)
    L = oracle.lib()
    igp = np.zeros(prob.nrep, np.int32)
    rows = fx["rows"]
    n = 0
    for row in rows:
        jI, gI, EI = int(row[0]), int(row[1]), row[2]
        qI = np.ascontiguousarray(row[3:4 + nm], np.int32)
        o = 4 + nm
        jF, gF, EF = int(row[o]), int(row[o + 1]), row[o + 2]
        qF = np.ascontiguousarray(row[o + 3:o + 4 + nm], np.int32)
        want = row[o + 4 + nm:].astype(np.int32)
        got = np.zeros(3, np.int32)
        L.or_filter_pair(C.byref(job), jI, EI, gI, oracle.ptr(qI, oracle.i32p), jF, EF, gF,
                         oracle.ptr(qF, oracle.i32p), oracle.ptr(got, oracle.i32p),
                         oracle.ptr(igp, oracle.i32p))
        assert np.array_equal(got, want), (row, got, want)
        n += int(want[2])
    assert np.array_equal(igp, fx["igamma_pair"])
    assert n > 3  # the fixture exercises accepted pairs too


def test_degeneracy_filter_matches_reference(oracle, synth):
    tab = np.load(os.path.join(GOLDEN, "degeneracy_filter.npy"))
    probs = {}
    for name in ("c2v", "c3v"):
        probs[name] = synth.load(os.path.join(GOLDEN, f"{name}_problem.npz"))
    L = oracle.lib()
    for sym, red, gI, gF, dI, dF, want in tab:
        prob = probs["c2v" if sym == 1 else "c3v"]
        prob.params.reduced = bool(red)
        keep = oracle.Keep()
        job = oracle.make_job(prob, (prob.jlist[0], prob.jlist[-1]), keep)
        assert L.or_degeneracy_filter(C.byref(job), int(gI), int(gF), int(dI), int(dF)) == want
