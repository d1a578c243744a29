"""ctypes binding to the CPU oracle (liboracle.so) and, where it was built, to
the reference-compiled pin library (_ref/libref.so).

Test infrastructure only: imported by tests/, the smoke check and the
CPU-baseline leg of bench.py, always as the checker.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Dict, List, Optional, Tuple

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libref.so")

i32p = C.POINTER(C.c_int32)
f64p = C.POINTER(C.c_double)


class or_basis(C.Structure):
    _fields_ = [("jval", C.c_int), ("Maxcontracts", C.c_int), ("Maxsymcoeffs", C.c_int),
                ("max_deg_size", C.c_int), ("mat_size", C.c_int),
                ("icontr2icase", i32p), ("iroot_correlat_j0", i32p), ("k", i32p),
                ("ktau", i32p), ("Nsym", i32p), ("Ntotal", i32p),
                ("repres", C.POINTER(f64p))]


class or_block(C.Structure):
    _fields_ = [("nsize", C.c_int), ("nvec", C.c_int), ("vecs", f64p), ("energies", f64p),
                ("quanta", i32p)]


class or_job(C.Structure):
    _fields_ = [("sym_type", C.c_int), ("nrep", C.c_int), ("degen", i32p), ("nmodes", C.c_int),
                ("ZPE", C.c_double), ("erange_lower", C.c_double * 2),
                ("erange_upper", C.c_double * 2), ("freq_window", C.c_double * 2),
                ("jvals", C.c_int * 2), ("q_stat", C.c_double), ("temperature", C.c_double),
                ("gns", f64p), ("isym_pairs", i32p), ("reduced", C.c_int),
                ("quanta_lower", i32p), ("quanta_upper", i32p),
                ("thresh_linestrength", C.c_double), ("thresh_intensity", C.c_double),
                ("N", C.c_int), ("mu", f64p), ("basis", or_basis * 2),
                ("blocks", C.POINTER(or_block)), ("nthreads", C.c_int), ("precise", C.c_int)]


LINE_DTYPE = np.dtype([("jI", np.int32), ("gammaI", np.int32), ("recI", np.int32),
                       ("jF", np.int32), ("gammaF", np.int32), ("recF", np.int32),
                       ("ndegI", np.int32), ("ndegF", np.int32),
                       ("nu", np.float64), ("S", np.float64), ("A", np.float64),
                       ("I", np.float64), ("t", np.float64, (4,)),
                       ("Elow", np.float64), ("Eup", np.float64)])


class or_line(C.Structure):
    _fields_ = [("jI", C.c_int32), ("gammaI", C.c_int32), ("recI", C.c_int32),
                ("jF", C.c_int32), ("gammaF", C.c_int32), ("recF", C.c_int32),
                ("ndegI", C.c_int32), ("ndegF", C.c_int32),
                ("nu", C.c_double), ("S", C.c_double), ("A", C.c_double), ("I", C.c_double),
                ("t", C.c_double * 4), ("Elow", C.c_double), ("Eup", C.c_double)]


assert C.sizeof(or_line) == LINE_DTYPE.itemsize

_lib = None
_ref = None


def build():
    """Compile liboracle.so (and the reference pin where its sources exist)."""
    import subprocess
    subprocess.check_call(["make", "-s", "-C", HERE])
    # the recipe finds the reference sources itself and skips when they are absent
    subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh")])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.or_three_j.restype = C.c_double
        L.or_three_j.argtypes = [C.c_int] * 6
        L.or_fakt.restype = C.c_double
        L.or_fakt.argtypes = [C.c_double]
        L.or_precompute_threej.argtypes = [C.c_int, f64p]
        L.or_compute_ijterms.argtypes = [C.POINTER(or_basis), C.c_int, i32p]
        L.or_correlate.argtypes = [C.POINTER(or_basis), i32p, C.c_int, i32p, C.c_int, C.c_int,
                                   f64p, f64p]
        L.or_half_ls.argtypes = [C.POINTER(or_basis), C.POINTER(or_basis), C.c_int, f64p, f64p,
                                 C.c_int, f64p, f64p]
        L.or_dot.restype = C.c_double
        L.or_dot.argtypes = [f64p, f64p, C.c_int]
        L.or_run.restype = C.c_int
        L.or_run.argtypes = [C.POINTER(or_job), C.POINTER(C.POINTER(or_line)),
                             C.POINTER(C.c_size_t)]
        L.or_free.argtypes = [C.c_void_p]
        L.or_resolve_zpe.restype = C.c_double
        L.or_resolve_zpe.argtypes = [C.POINTER(or_job)]
        L.or_filter_pair.argtypes = [C.POINTER(or_job), C.c_int, C.c_double, C.c_int, i32p,
                                     C.c_int, C.c_double, C.c_int, i32p, i32p, i32p]
        L.or_degeneracy_filter.argtypes = [C.POINTER(or_job), C.c_int, C.c_int, C.c_int, C.c_int]
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_PATH)


def ref():
    """The reference-compiled pin library (only where it was built)."""
    global _ref
    if _ref is None:
        R = C.CDLL(REF_PATH)
        R.ref_three_j.restype = C.c_double
        R.ref_three_j.argtypes = [C.c_int] * 6
        R.ref_fakt.restype = C.c_double
        R.ref_fakt.argtypes = [C.c_double]
        R.ref_precompute_threej.argtypes = [C.c_int, f64p]
        R.ref_compute_ijterms.argtypes = [C.POINTER(or_basis), C.c_int, i32p]
        R.ref_correlate.argtypes = [C.POINTER(or_basis), C.c_int, i32p, C.c_int, C.c_int, f64p,
                                    f64p]
        R.ref_half_ls_flipped.argtypes = [C.POINTER(or_basis), C.POINTER(or_basis), C.c_int, i32p,
                                          C.c_int, f64p, C.c_int, f64p, f64p, f64p]
        R.ref_read_dipole_flipped.restype = C.c_int
        R.ref_read_dipole_flipped.argtypes = [C.c_char_p, C.c_int, f64p]
        R.ref_filters.argtypes = [C.POINTER(or_job), C.c_int, C.c_double, C.c_int, i32p, C.c_int,
                                  C.c_double, C.c_int, i32p, i32p, i32p]
        R.ref_degeneracy_filter.restype = C.c_int
        R.ref_degeneracy_filter.argtypes = [C.POINTER(or_job), C.c_int, C.c_int, C.c_int, C.c_int]
        R.ref_read_quanta.restype = C.c_int
        R.ref_read_quanta.argtypes = [C.c_char_p, C.c_int, C.c_int, i32p, i32p, i32p, i32p, i32p,
                                      i32p, i32p, i32p, C.POINTER(f64p)]
        R.ref_read_levels.restype = C.c_int
        R.ref_read_levels.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int, i32p,
                                      C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, f64p,
                                      C.c_int, C.c_int, C.c_void_p]
        _ref = R
    return _ref


REF_LEVEL = np.dtype([("jval", np.int32), ("igamma", np.int32), ("ilevel", np.int32),
                      ("ndeg", np.int32), ("irec0", np.int32), ("irec1", np.int32),
                      ("krot", np.int32), ("taurot", np.int32), ("energy", np.float64),
                      ("quanta", np.int32, (17,)), ("normal", np.int32, (17,)),
                      ("cgamma", np.int32, (17,))], align=True)  # the C struct's padding


def ref_trove_basis(directory: str, J: int, degen) -> dict:
    """The reference's bset_contr_factory + correlate_index on TROVE files."""
    R = ref()
    nrep = len(degen)
    dg = np.asarray(degen, np.int32)
    dims = np.zeros(5, np.int32)
    nt = np.zeros(nrep, np.int32)
    R.ref_read_quanta(directory.encode(), J, nrep, ptr(dg, i32p), ptr(dims, i32p), None, None,
                      None, None, None, ptr(nt, i32p), None)
    D, ncase, _, mat, _ = (int(x) for x in dims)
    out = {"k": np.zeros(D, np.int32), "ktau": np.zeros(D, np.int32),
           "iroot": np.zeros(D, np.int32), "icontr2icase": np.zeros(2 * D, np.int32),
           "Nsym": np.zeros(nrep * ncase, np.int32), "Ntotal": nt,
           "repres": [np.zeros(int(nt[g]) * degen[g] * mat) for g in range(nrep)],
           "dims": dims}
    rp = (f64p * nrep)(*[ptr(r, f64p) for r in out["repres"]])
    R.ref_read_quanta(directory.encode(), J, nrep, ptr(dg, i32p), ptr(dims, i32p),
                      ptr(out["k"], i32p), ptr(out["ktau"], i32p), ptr(out["iroot"], i32p),
                      ptr(out["icontr2icase"], i32p), ptr(out["Nsym"], i32p), ptr(nt, i32p), rp)
    return out


def ref_trove_levels(directory: str, jvals, sym_type: int, degen, nmodes: int, nclasses: int,
                     zpe: float, erange, gns, maxcontracts: int, cap: int = 100000) -> np.ndarray:
    """The reference's read_eigenvalues over the descr files of (j0, j1)."""
    R = ref()
    dg = np.asarray(degen, np.int32)
    g = np.asarray(gns, np.float64)
    out = np.zeros(cap, REF_LEVEL)
    n = R.ref_read_levels(directory.encode(), jvals[0], jvals[1], sym_type, len(degen),
                          ptr(dg, i32p), nmodes, nclasses, zpe, erange[0], erange[1],
                          ptr(g, f64p), maxcontracts, cap, out.ctypes.data)
    return out[:n]


def ptr(a: np.ndarray, t):
    return a.ctypes.data_as(t)


class Keep:
    """Holds numpy buffers alive while ctypes structs point at them."""

    def __init__(self):
        self.items = []

    def __call__(self, a):
        self.items.append(a)
        return a


def make_basis(b, keep: Keep) -> or_basis:
    ob = or_basis()
    ob.jval = b.jval
    ob.Maxcontracts = b.Maxcontracts
    ob.Maxsymcoeffs = b.Maxsymcoeffs
    ob.max_deg_size = b.max_deg_size
    ob.mat_size = b.mat_size
    for name in ("icontr2icase", "iroot_correlat_j0", "k", "ktau", "Nsym", "Ntotal"):
        a = keep(np.ascontiguousarray(getattr(b, name), dtype=np.int32))
        setattr(ob, name, ptr(a, i32p))
    arr = (f64p * len(b.repres))()
    for g, r in enumerate(b.repres):
        rr = keep(np.ascontiguousarray(r, dtype=np.float64))
        arr[g] = ptr(rr, f64p)
    keep(arr)
    ob.repres = C.cast(arr, C.POINTER(f64p))
    return ob


def make_job(prob, jvals: Tuple[int, int], keep: Keep, zpe: Optional[float] = None,
             nthreads: int = 0, precise: bool = True) -> or_job:
    """An or_job for one reference run over jvals = (jvals[0], jvals[1])."""
    p = prob.params
    j = or_job()
    j.sym_type = prob.sym_type
    j.nrep = prob.nrep
    j.degen = ptr(keep(np.array(prob.degen, np.int32)), i32p)
    j.nmodes = p.nmodes
    j.ZPE = p.ZPE if zpe is None else zpe
    j.erange_lower[:] = list(p.erange_lower)
    j.erange_upper[:] = list(p.erange_upper)
    j.freq_window[:] = list(p.freq_window)
    j.jvals[:] = list(jvals)
    j.q_stat = p.q_stat
    j.temperature = p.temperature
    j.gns = ptr(keep(np.array(p.gns, np.float64)), f64p)
    j.isym_pairs = ptr(keep(np.array(p.isym_pairs, np.int32)), i32p)
    j.reduced = int(p.reduced)
    ql, qu = p.windows()
    j.quanta_lower = ptr(keep(np.ascontiguousarray(ql.reshape(-1), np.int32)), i32p)
    j.quanta_upper = ptr(keep(np.ascontiguousarray(qu.reshape(-1), np.int32)), i32p)
    j.thresh_linestrength = p.thresh_linestrength
    j.thresh_intensity = p.thresh_intensity
    j.N = prob.N
    mu = keep(np.ascontiguousarray(prob.mu, np.float64))
    j.mu = ptr(mu, f64p)
    for i in range(2):
        j.basis[i] = make_basis(prob.bases[jvals[i]], keep)
    blocks = (or_block * (2 * prob.nrep))()
    for i in range(2):
        for g in range(prob.nrep):
            b = prob.blocks[(jvals[i], g)]
            ob = blocks[i + 2 * g]
            ob.nsize = b.nsize
            ob.nvec = b.nvec
            v = keep(np.ascontiguousarray(b.vecs, np.float64))
            e = keep(np.ascontiguousarray(b.energies, np.float64))
            q = keep(np.ascontiguousarray(b.quanta, np.int32))
            ob.vecs = ptr(v, f64p)
            ob.energies = ptr(e, f64p)
            ob.quanta = ptr(q, i32p)
    keep(blocks)
    j.blocks = C.cast(blocks, C.POINTER(or_block))
    j.nthreads = nthreads
    j.precise = int(precise)
    return j


def run_pair(prob, jvals: Tuple[int, int], zpe: Optional[float] = None,
             nthreads: int = 0, precise: bool = True) -> np.ndarray:
    """Lines of one reference run over (jvals[0], jvals[1]); precise=False runs
    the reference's plain FP64 arithmetic (the timed CPU port) instead of the
    double-double checker."""
    L = lib()
    keep = Keep()
    job = make_job(prob, jvals, keep, zpe, nthreads, precise)
    out = C.POINTER(or_line)()
    n = C.c_size_t(0)
    rc = L.or_run(C.byref(job), C.byref(out), C.byref(n))
    if rc != 0:
        raise RuntimeError(f"or_run failed: {rc}")
    arr = np.empty(n.value, dtype=LINE_DTYPE)
    if n.value:
        C.memmove(arr.ctypes.data, out, n.value * LINE_DTYPE.itemsize)
    L.or_free(out)
    return arr


def resolve_zpe(prob) -> float:
    """The ZPE a run starting at J=min(J) resolves (J=0, Gamma=0 records)."""
    js = prob.jlist
    keep = Keep()
    job = make_job(prob, (js[0], js[1] if len(js) > 1 else js[0]), keep)
    return float(lib().or_resolve_zpe(C.byref(job)))


def run_all(prob, nthreads: int = 0, precise: bool = True) -> np.ndarray:
    """All lines of a multi-J job as the union of consecutive reference runs
    (J, J+1) for J = Jmin .. Jmax-1, with the ZPE resolved once and passed
    explicitly to every run, exactly as a user chains the reference."""
    js = prob.jlist
    zpe = resolve_zpe(prob)
    parts = [run_pair(prob, (js[i], js[i + 1]), zpe, nthreads, precise)
             for i in range(len(js) - 1)]
    return np.concatenate(parts) if parts else np.empty(0, LINE_DTYPE)


def threej_table(jmax: int) -> np.ndarray:
    out = np.zeros((jmax + 1) ** 2 * 9, np.float64)
    lib().or_precompute_threej(jmax, ptr(out, f64p))
    return out


def ijterms(b, nrep: int) -> np.ndarray:
    keep = Keep()
    ob = make_basis(b, keep)
    out = np.zeros(b.Maxsymcoeffs * nrep, np.int32)
    lib().or_compute_ijterms(C.byref(ob), nrep, ptr(out, i32p))
    return out


def correlate(b, nrep: int, degen, ideg: int, gamma: int, vsym: np.ndarray) -> np.ndarray:
    keep = Keep()
    ob = make_basis(b, keep)
    ijt = ijterms(b, nrep)
    dg = np.array(degen, np.int32)
    out = np.zeros(b.Maxcontracts, np.float64)
    v = np.ascontiguousarray(vsym, np.float64)
    lib().or_correlate(C.byref(ob), ptr(ijt, i32p), nrep, ptr(dg, i32p), ideg, gamma,
                       ptr(v, f64p), ptr(out, f64p))
    return out


def half_ls(bI, bF, N: int, mu: np.ndarray, jmax: int, vprim: np.ndarray) -> np.ndarray:
    keep = Keep()
    oI = make_basis(bI, keep)
    oF = make_basis(bF, keep)
    tj = threej_table(jmax)
    m = np.ascontiguousarray(mu, np.float64)
    v = np.ascontiguousarray(vprim, np.float64)
    out = np.zeros(bF.Maxcontracts, np.float64)
    lib().or_half_ls(C.byref(oI), C.byref(oF), N, ptr(m, f64p), ptr(tj, f64p), jmax,
                     ptr(v, f64p), ptr(out, f64p))
    return out
