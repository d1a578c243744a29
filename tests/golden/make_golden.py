"""Regenerates the golden fixtures of tests/golden from the reference itself.

Runs only where the reference sources exist (it builds oracle/_ref/libref.so
from them via oracle/build_ref.sh): the reference's own precompute_threej,
device_correlate_vectors and device_compute_1st_half_ls_flipped_dipole
(kernel bodies run on the CPU), read_dipole_flipped and its filters.  The
fixtures hold the exact inputs next to the reference outputs, so the tests
need neither the reference nor bit-identical input generation.

    python tests/golden/make_golden.py
"""
import ctypes as C
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), "..", ".."))
sys.path.insert(0, ROOT)
import __graft_entry__ as G  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def write_extfield(path, N, mu):
    """j0_extfield.chk as TROVE writes it: Fortran sequential records."""
    def rec(f, payload: bytes):
        n = np.array([len(payload)], np.uint32).tobytes()
        f.write(n + payload + n)
    with open(path, "wb") as f:
        rec(f, b"Start external field")
        rec(f, np.array([N], np.int32).tobytes())
        for c in range(3):
            rec(f, np.array([c + 1], np.int32).tobytes())
            rec(f, np.ascontiguousarray(mu[c], np.float64).tobytes())
        rec(f, b"End external field  ")


def kernel_fixture(prob, name, R, O):
    synth = sys.modules["gpu_intensities_gb300.synth"]
    nrep = prob.nrep
    dg = np.array(prob.degen, np.int32)
    N = prob.N
    js = prob.jlist
    jmax = max(js)
    with tempfile.TemporaryDirectory() as td:
        write_extfield(os.path.join(td, "j0_extfield.chk"), N, prob.mu)
        flip = np.zeros(3 * N * N)
        n = R.ref_read_dipole_flipped(td.encode(), N, O.ptr(flip, O.f64p))
        assert n == 3 * N * N
    tj = np.zeros((jmax + 1) ** 2 * 9)
    R.ref_precompute_threej(jmax, O.ptr(tj, O.f64p))
    out = {}
    rng = np.random.default_rng(11)
    for (J, g), blk in sorted(prob.blocks.items()):
        if blk.nvec == 0:
            continue
        keep = O.Keep()
        ob = O.make_basis(prob.bases[J], keep)
        v = np.ascontiguousarray(blk.vecs[0])
        for d in range(prob.degen[g]):
            res = np.zeros(prob.bases[J].Maxcontracts)
            R.ref_correlate(C.byref(ob), nrep, O.ptr(dg, O.i32p), d, g, O.ptr(v, O.f64p),
                            O.ptr(res, O.f64p))
            out[f"corr_{J}_{g}_{d}"] = res
    for jI in js:
        for jF in js:
            if abs(jI - jF) > 1:
                continue
            bI, bF = prob.bases[jI], prob.bases[jF]
            vp = rng.standard_normal(bI.Maxcontracts)
            keep = O.Keep()
            oI, oF = O.make_basis(bI, keep), O.make_basis(bF, keep)
            res = np.zeros(bF.Maxcontracts)
            R.ref_half_ls_flipped(C.byref(oI), C.byref(oF), nrep, O.ptr(dg, O.i32p), N,
                                  O.ptr(flip, O.f64p), jmax, O.ptr(tj, O.f64p), O.ptr(vp, O.f64p),
                                  O.ptr(res, O.f64p))
            out[f"hls_in_{jI}_{jF}"] = vp
            out[f"hls_{jI}_{jF}"] = res
    out["flipped_dipole"] = flip
    synth.save(prob, os.path.join(HERE, f"{name}_problem.npz"))
    np.savez_compressed(os.path.join(HERE, f"{name}_kernels.npz"), **out)


def filter_fixture(prob, name, R, O):
    """Random level pairs through the reference's filters."""
    rng = np.random.default_rng(5)
    p = prob.params
    js = prob.jlist
    rows = []
    keep = O.Keep()
    job = O.make_job(prob, (js[0], js[-1]), keep)
    # tight windows so that every branch of the filters is exercised
    job.erange_lower[:] = [100.0, 9000.0]
    job.erange_upper[:] = [500.0, 15000.0]
    job.freq_window[:] = [-2000.0, 6000.0]
    ql = np.array([[1] * p.nmodes, [5] * p.nmodes], np.int32).reshape(-1)
    qu = np.array([[0] * p.nmodes, [6] * p.nmodes], np.int32).reshape(-1)
    job.quanta_lower = O.ptr(keep(ql), O.i32p)
    job.quanta_upper = O.ptr(keep(qu), O.i32p)
    igp = np.zeros(prob.nrep, np.int32)
    for _ in range(4000):
        jI, jF = int(rng.choice(js)), int(rng.choice(js))
        gI, gF = int(rng.integers(prob.nrep)), int(rng.integers(prob.nrep))
        EI, EF = float(rng.uniform(0, 16000)), float(rng.uniform(0, 16000))
        qI = rng.integers(0, 8, p.nmodes + 1).astype(np.int32)
        qF = rng.integers(0, 8, p.nmodes + 1).astype(np.int32)
        o = np.zeros(3, np.int32)
        R.ref_filters(C.byref(job), jI, EI, gI, O.ptr(qI, O.i32p), jF, EF, gF, O.ptr(qF, O.i32p),
                      O.ptr(o, O.i32p), O.ptr(igp, O.i32p))
        rows.append((jI, gI, EI, *qI, jF, gF, EF, *qF, *o))
    arr = np.array(rows, dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, f"{name}_filters.npz"), rows=arr, igamma_pair=igp,
                        erange_lower=np.array([100.0, 9000.0]),
                        erange_upper=np.array([500.0, 15000.0]),
                        freq_window=np.array([-2000.0, 6000.0]), quanta_lower=ql,
                        quanta_upper=qu, jvals=np.array([js[0], js[-1]]))


def trove_fixture(prob, name, O):
    """A small TROVE job (files as the reference reads them) and what the
    reference's own readers make of it: bset_contr_factory + correlate_index
    per J and read_eigenvalues."""
    synth = sys.modules["gpu_intensities_gb300.synth"]
    d = os.path.join(HERE, f"trove_{name}")
    deck = synth.write_trove(prob, d)
    with open(os.path.join(d, "job.inp"), "w") as f:
        f.write(deck)
    out = {}
    for J in prob.jlist:
        b = O.ref_trove_basis(d, J, prob.degen)
        for key in ("k", "ktau", "iroot", "icontr2icase", "Nsym", "Ntotal", "dims"):
            out[f"basis{J}_{key}"] = b[key]
        for g, r in enumerate(b["repres"]):
            out[f"basis{J}_repres{g}"] = r
    js = prob.jlist
    lv = O.ref_trove_levels(d, (js[0], js[-1]), prob.sym_type, prob.degen,
                            prob.params.nmodes, 1, prob.params.ZPE, (-1e300, 1e300),
                            prob.params.gns, max(b.Maxcontracts for b in prob.bases.values()))
    out["levels"] = lv
    np.savez_compressed(os.path.join(HERE, f"trove_{name}_ref.npz"), **out)


def main():
    G.build()
    G.load_package()
    from gpu_intensities_gb300 import synth
    O = G.load_oracle()
    if not O.ref_available():
        sys.exit("oracle/_ref/libref.so not built: the reference sources are required")
    R = O.ref()
    tj = np.zeros(25 * 25 * 9)
    R.ref_precompute_threej(24, O.ptr(tj, O.f64p))
    np.save(os.path.join(HERE, "threej_ref_j24.npy"), tj)
    c2v = synth.make_c2v(3, 12, [0, 1, 2, 3], nvec_max=5, name="golden_c2v")
    c3v = synth.make_c3v(4, 10, [1, 2, 3], nvec_max=5, name="golden_c3v")
    kernel_fixture(c2v, "c2v", R, O)
    kernel_fixture(c3v, "c3v", R, O)
    filter_fixture(c2v, "c2v", R, O)
    c3r = synth.make_c3v(4, 10, [1, 2, 3], nvec_max=5, reduced=True)
    filter_fixture(c3r, "c3v", R, O)
    degen = []
    for prob, nm in ((c2v, "c2v"), (c3r, "c3v_reduced"), (c3v, "c3v")):
        keep = O.Keep()
        job = O.make_job(prob, (prob.jlist[0], prob.jlist[-1]), keep)
        for gI in range(prob.nrep):
            for gF in range(prob.nrep):
                for dI in range(2):
                    for dF in range(2):
                        degen.append((prob.sym_type, int(prob.params.reduced), gI, gF, dI, dF,
                                      R.ref_degeneracy_filter(C.byref(job), gI, gF, dI, dF)))
    np.save(os.path.join(HERE, "degeneracy_filter.npy"), np.array(degen, np.int32))
    trove_fixture(synth.make_c3v(6, 12, [0, 1], nvec_max=3), "c3v", O)
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
