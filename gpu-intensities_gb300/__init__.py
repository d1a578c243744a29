"""GB300 line-intensity engine: Python host mirror of the C ABI (include/gi.h).

The engine replaces the reference's intensity step (``main.x < job.inp``:
``dipole_initialise_cpu`` + ``dipole_do_intensities_async_omp``,
cuda_host.cu:837-1506).  This module binds ``libgi.so`` with ctypes and
offers the same job model: a symmetry group, the INTENSITY parameters, the
vibrational dipole, per-J basis tables and per-(J, Gamma) eigenvector blocks
in; lines (S, A_if, I(T), transition moments) and the level table out.

There is no CPU fallback: every call goes through the CUDA library, and an
``Engine`` cannot be created without it.
"""
from __future__ import annotations

import ctypes as C
import os
import re
from typing import Dict, Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgi.so")
HEADER = os.path.join(HERE, os.pardir, "include", "gi.h")
HEADERS = [os.path.join(HERE, os.pardir, "include", h) for h in ("gi.h", "gi_probe.h")]

GI_OK, GI_ERR_ARG, GI_ERR_CUDA, GI_ERR_NOMEM, GI_ERR_STATE, GI_ERR_BUDGET, GI_ERR_NOTFOUND, \
    GI_ERR_DEVICE = range(8)
GI_PREC_FP64, GI_PREC_SPLIT = 0, 1
GI_RUN_LINES_ON_DEVICE = 1
GI_RUN_PHASE_TIMING = 2
GI_RUN_GRAPH = 4
GI_RUN_COMPACT_LINES = 8
PHASES = ("correlate", "halfls_gemm", "stencil", "final_gemm", "epilogue", "slice")
GI_MAX_REP, GI_MAX_MODES = 8, 16

i32p = C.POINTER(C.c_int32)
f64p = C.POINTER(C.c_double)


class gi_params(C.Structure):
    _fields_ = [("temperature", C.c_double), ("q_stat", C.c_double), ("ZPE", C.c_double),
                ("erange_lower", C.c_double * 2), ("erange_upper", C.c_double * 2),
                ("freq_window", C.c_double * 2), ("gns", C.c_double * GI_MAX_REP),
                ("isym_pairs", C.c_int32 * GI_MAX_REP), ("nmodes", C.c_int32),
                ("quanta_lower", (C.c_int32 * GI_MAX_MODES) * 2),
                ("quanta_upper", (C.c_int32 * GI_MAX_MODES) * 2),
                ("reduced", C.c_int32), ("precision", C.c_int32), ("split_slices", C.c_int32),
                ("reserved", C.c_int32), ("thresh_linestrength", C.c_double),
                ("thresh_intensity", C.c_double)]


LINE_DTYPE = np.dtype([("level_i", np.int32), ("level_f", np.int32), ("ndeg_i", np.int32),
                       ("ndeg_f", np.int32), ("nu", np.float64), ("S", np.float64),
                       ("A", np.float64), ("I", np.float64), ("t", np.float64, (4,))])
LEVEL_DTYPE = np.dtype([("J", np.int32), ("gamma", np.int32), ("rec", np.int32),
                        ("ndeg", np.int32), ("krot", np.int32), ("taurot", np.int32),
                        ("energy", np.float64)])
# gi_line_compact: the 40-byte record of GI_RUN_COMPACT_LINES
LINE_COMPACT_DTYPE = np.dtype([("level_i", np.int32), ("level_f", np.int32), ("nu", np.float64),
                               ("S", np.float64), ("A", np.float64), ("I", np.float64)])


class gi_stats(C.Structure):
    _fields_ = [("nlines", C.c_int64), ("nlines_filtered", C.c_int64),
                ("npairs_checked", C.c_int64),
                ("nblock_pairs", C.c_int32), ("nlevels", C.c_int32), ("zpe", C.c_double),
                ("seconds_total", C.c_double), ("seconds_gpu", C.c_double),
                ("flops_halfls", C.c_double), ("flops_final", C.c_double),
                ("flops_tensor", C.c_double), ("bytes_correlate", C.c_double),
                ("seconds_phase", C.c_double * 6), ("launches_phase", C.c_int32 * 6),
                ("kernel_launches", C.c_int32), ("reserved", C.c_int32),
                ("nlines_doubtful", C.c_int64), ("nlines_handed", C.c_int64),
                ("nlines_refined", C.c_int64)]


class gi_serve_config(C.Structure):
    _fields_ = [("slots", C.c_int32), ("flags", C.c_int32),
                ("hbm_budget_bytes", C.c_size_t), ("slot_workspace_bytes", C.c_size_t)]


class gi_job_info(C.Structure):
    _fields_ = [("state", C.c_int32), ("status", C.c_int32), ("nlines", C.c_int64),
                ("nlines_filtered", C.c_int64), ("seconds_queued", C.c_double),
                ("seconds_latency", C.c_double), ("seconds_gpu", C.c_double)]


class gi_serve_stats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("completed", C.c_int64), ("failed", C.c_int64),
                ("lines", C.c_int64), ("lines_filtered", C.c_int64),
                ("evictions", C.c_int64), ("restores", C.c_int64),
                ("queued", C.c_int32), ("running", C.c_int32),
                ("latency_p50", C.c_double), ("latency_p99", C.c_double),
                ("latency_mean", C.c_double), ("latency_max", C.c_double),
                ("queue_p50", C.c_double), ("queue_p99", C.c_double),
                ("resident_bytes", C.c_size_t), ("peak_resident_bytes", C.c_size_t),
                ("budget_bytes", C.c_size_t), ("slot_workspace_bytes", C.c_size_t),
                ("slots", C.c_int32), ("reserved", C.c_int32),
                ("zcache_hits", C.c_int64), ("zcache_misses", C.c_int64),
                ("zcache_evictions", C.c_int64), ("zcache_bytes", C.c_size_t)]


GI_JOB_QUEUED, GI_JOB_RUNNING, GI_JOB_DONE, GI_JOB_FAILED = range(4)
GI_TROVE_MAXQ = 17
GI_TROVE_ALL_J = 1
GI_TROVE_STREAM_DIPOLE = 2
GI_DIPOLE_BORROW = 1


class gi_deck(C.Structure):
    _fields_ = [("sym_type", C.c_int32), ("nmodes", C.c_int32), ("jvals", C.c_int32 * 2),
                ("params", gi_params)]


class gi_line_text(C.Structure):
    """The fields of one printed line (gi_format_line_text)."""
    _fields_ = [("jF", C.c_int32), ("jI", C.c_int32), ("krotF", C.c_int32), ("krotI", C.c_int32),
                ("ilevelF", C.c_int32), ("ilevelI", C.c_int32), ("nclasses", C.c_int32),
                ("nmodes", C.c_int32), ("ndegF", C.c_int32), ("ndegI", C.c_int32),
                ("symF", C.c_char_p), ("symI", C.c_char_p),
                ("cgF", C.c_char_p * GI_TROVE_MAXQ), ("cgI", C.c_char_p * GI_TROVE_MAXQ),
                ("quantaF", C.c_int32 * GI_TROVE_MAXQ), ("quantaI", C.c_int32 * GI_TROVE_MAXQ),
                ("normalF", C.c_int32 * GI_TROVE_MAXQ), ("normalI", C.c_int32 * GI_TROVE_MAXQ),
                ("eF", C.c_double), ("eI", C.c_double), ("nu", C.c_double), ("S", C.c_double),
                ("A", C.c_double), ("I", C.c_double), ("t", C.c_double * 4)]


def format_line_text(f: dict) -> str:
    """One printed line from explicit fields (host code, no GPU): labels
    cgF/cgI for classes 0..nclasses, quanta/normal with index 0 unused."""
    x = gi_line_text()
    for k in ("jF", "jI", "krotF", "krotI", "ilevelF", "ilevelI", "ndegF", "ndegI"):
        setattr(x, k, int(f[k]))
    x.nclasses, x.nmodes = len(f["cgF"]) - 1, len(f["quantaF"]) - 1
    keep = [str(v).encode() for v in [f["symF"], f["symI"]] + list(f["cgF"]) + list(f["cgI"])]
    x.symF, x.symI = keep[0], keep[1]
    for i, v in enumerate(f["cgF"]):
        x.cgF[i] = str(v).encode()
    for i, v in enumerate(f["cgI"]):
        x.cgI[i] = str(v).encode()
    for k in ("quantaF", "quantaI", "normalF", "normalI"):
        arr = getattr(x, k)
        for i, v in enumerate(f[k]):
            arr[i] = int(v)
    for k in ("eF", "eI", "nu", "S", "A", "I"):
        setattr(x, k, float(f[k]))
    for i, v in enumerate(f["t"]):
        x.t[i] = float(v)
    L = lib()
    used = C.c_size_t(0)
    buf = C.create_string_buffer(4096)
    st = L.gi_format_line_text(C.byref(x), buf, len(buf), C.byref(used))
    if st != GI_OK:
        raise GiError(st, "gi_format_line_text")
    return buf.value.decode()


class gi_trove_level(C.Structure):
    _fields_ = [("irec", C.c_int32 * 2), ("ilevel", C.c_int32), ("ndeg", C.c_int32),
                ("krot", C.c_int32), ("taurot", C.c_int32), ("large_coef", C.c_int32),
                ("reserved", C.c_int32), ("energy", C.c_double),
                ("quanta", C.c_int32 * GI_TROVE_MAXQ), ("cgamma", C.c_int32 * GI_TROVE_MAXQ),
                ("normal", C.c_int32 * GI_TROVE_MAXQ)]


class GiError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"gi status {status}: {msg}")
        self.status = status


_lib = None


def header_functions():
    """Names of the entry points the headers in include/ declare."""
    text = "".join(open(h).read() for h in HEADERS)
    return sorted(set(re.findall(r"^\s*(?:gi_status|const char\*)\s+(gi_\w+)\s*\(", text, re.M)))


def build(verbose: bool = False) -> str:
    """Compile libgi.so in-tree for sm_103a (nvcc)."""
    import subprocess
    cmd = ["make", "-C", HERE, f"-j{min(8, os.cpu_count() or 1)}"]
    if not verbose:
        cmd.insert(1, "-s")
    subprocess.check_call(cmd)
    return LIB_PATH


def lib():
    """Load libgi.so; raises if the CUDA library has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"libgi.so not built ({LIB_PATH}); run build() first")
        L = C.CDLL(LIB_PATH)
        L.gi_create.argtypes = [C.POINTER(C.c_void_p), C.c_int, C.c_size_t]
        L.gi_destroy.argtypes = [C.c_void_p]
        L.gi_set_stream.argtypes = [C.c_void_p, C.c_void_p]
        L.gi_set_tuning.argtypes = [C.c_void_p, C.c_int, C.c_char_p]
        L.gi_last_error.restype = C.c_char_p
        L.gi_last_error.argtypes = [C.c_void_p]
        L.gi_status_string.restype = C.c_char_p
        L.gi_status_string.argtypes = [C.c_int]
        L.gi_set_symmetry.argtypes = [C.c_void_p, C.c_int]
        L.gi_set_params.argtypes = [C.c_void_p, C.POINTER(gi_params)]
        L.gi_set_dipole.argtypes = [C.c_void_p, C.c_int, f64p]
        L.gi_set_dipole_flipped.argtypes = [C.c_void_p, C.c_int, f64p]
        L.gi_set_dipole_streamed.argtypes = [C.c_void_p, C.c_int, f64p, C.c_int, C.c_int]
        L.gi_dipole_panel_rows.argtypes = [C.c_void_p]
        L.gi_set_basis.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                   i32p, i32p, i32p, i32p, i32p, i32p, C.POINTER(f64p)]
        L.gi_set_threej.argtypes = [C.c_void_p, C.c_int, f64p]
        L.gi_set_block.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, f64p, f64p,
                                   i32p]
        L.gi_set_block_device.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                          C.c_void_p, f64p, i32p]
        L.gi_run.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int64)]
        L.gi_set_refine.argtypes = [C.c_void_p, C.c_int64]
        L.gi_run_shard.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int64)]
        L.gi_deck_parse.argtypes = [C.c_char_p, C.POINTER(gi_deck), C.c_char_p, C.c_size_t]
        L.gi_trove_read_basis.argtypes = [C.c_char_p, C.c_int, C.c_int, i32p, i32p, i32p, i32p,
                                          i32p, i32p, i32p, C.POINTER(f64p), C.c_char_p,
                                          C.c_size_t]
        L.gi_trove_read_dipole.argtypes = [C.c_char_p, C.c_int, f64p, C.c_char_p, C.c_size_t]
        L.gi_trove_read_levels.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                           C.c_int, i32p, i32p, C.POINTER(gi_trove_level),
                                           C.c_int32, C.c_char_p, C.c_size_t]
        L.gi_load_trove.argtypes = [C.c_void_p, C.c_char_p, C.POINTER(gi_deck), C.c_int]
        L.gi_format_line_text.argtypes = [C.c_void_p, C.c_char_p, C.c_size_t, C.c_void_p]
        L.gi_format_lines.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.c_char_p, C.c_size_t,
                                      C.POINTER(C.c_size_t)]
        L.gi_partition_function.argtypes = [C.c_void_p, C.c_double, f64p]
        L.gi_serve_start.argtypes = [C.c_void_p, C.POINTER(gi_serve_config)]
        L.gi_serve_stop.argtypes = [C.c_void_p]
        L.gi_submit.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                C.POINTER(C.c_uint64)]
        L.gi_job_wait.argtypes = [C.c_void_p, C.c_uint64, C.c_double, C.POINTER(gi_job_info)]
        L.gi_job_lines.argtypes = [C.c_void_p, C.c_uint64, C.c_int64, C.c_int64, C.c_void_p]
        L.gi_job_release.argtypes = [C.c_void_p, C.c_uint64]
        L.gi_serve_get_stats.argtypes = [C.c_void_p, C.POINTER(gi_serve_stats)]
        L.gi_serve_reset_stats.argtypes = [C.c_void_p]
        L.gi_get_lines.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.c_void_p]
        L.gi_sort_lines.argtypes = [C.c_void_p]
        L.gi_get_lines_compact.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.c_void_p]
        L.gi_num_levels.argtypes = [C.c_void_p, C.POINTER(C.c_int32)]
        L.gi_get_levels.argtypes = [C.c_void_p, C.c_int32, C.c_void_p]
        L.gi_get_stats.argtypes = [C.c_void_p, C.POINTER(gi_stats)]
        L.gi_half_ls.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, f64p, f64p]
        L.gi_measure_fp64_peak.argtypes = [C.c_int, f64p]
        L.gi_probe_split_gemm.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, f64p, f64p,
                                          f64p]
        L.gi_half_ls_noalloc.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                         C.c_void_p, C.c_void_p, C.c_void_p]
        for name in header_functions():
            if name not in ("gi_last_error", "gi_status_string"):
                getattr(L, name).restype = C.c_int
        _lib = L
    return _lib


def measure_fp64_peak(device: int = 0) -> float:
    """FP64 DMMA peak of the device in TFLOP/s (gi_measure_fp64_peak)."""
    v = C.c_double(0.0)
    st = lib().gi_measure_fp64_peak(device, C.byref(v))
    if st != GI_OK:
        raise GiError(st, "gi_measure_fp64_peak failed")
    return v.value


def split_gemm(A: np.ndarray, B: np.ndarray, slices: int = 0, device: int = 0) -> np.ndarray:
    """A @ B.T through the split-precision GEMM alone (gi_probe_split_gemm)."""
    a = np.ascontiguousarray(A, np.float64)
    b = np.ascontiguousarray(B, np.float64)
    M, K = a.shape
    N = b.shape[0]
    if b.shape[1] != K:
        raise ValueError("A and B must have the same number of columns")
    out = np.empty((N, M), np.float64)
    st = lib().gi_probe_split_gemm(device, slices, M, N, K, _p(a, f64p), _p(b, f64p),
                                   _p(out, f64p))
    if st != GI_OK:
        raise GiError(st, "gi_probe_split_gemm failed")
    return out.T


def _p(a: np.ndarray, t):
    return a.ctypes.data_as(t)


def make_params(p, precision: int = GI_PREC_FP64, split_slices: int = 0) -> gi_params:
    """gi_params from a synth.Params-like object."""
    g = gi_params()
    g.temperature = p.temperature
    g.q_stat = p.q_stat
    g.ZPE = p.ZPE
    g.erange_lower[:] = list(p.erange_lower)
    g.erange_upper[:] = list(p.erange_upper)
    g.freq_window[:] = list(p.freq_window)
    for i, v in enumerate(p.gns):
        g.gns[i] = v
    for i, v in enumerate(p.isym_pairs):
        g.isym_pairs[i] = v
    g.nmodes = p.nmodes
    ql, qu = p.windows()
    for r in range(2):
        for m in range(p.nmodes):
            g.quanta_lower[r][m] = int(ql[r, m])
            g.quanta_upper[r][m] = int(qu[r, m])
    g.reduced = int(p.reduced)
    g.precision = precision
    g.split_slices = split_slices
    g.thresh_linestrength = p.thresh_linestrength
    g.thresh_intensity = p.thresh_intensity
    return g


def _host_err(st: int, err) -> None:
    if st != GI_OK:
        raise GiError(st, err.value.decode(errors="replace"))


def parse_deck(text: str) -> gi_deck:
    """The reference's input deck (gi_deck_parse), host only."""
    d = gi_deck()
    err = C.create_string_buffer(512)
    _host_err(lib().gi_deck_parse(text.encode(), C.byref(d), err, 512), err)
    return d


def trove_read_basis(directory: str, J: int, sym_type: int, nrep: int, degen) -> Dict:
    """j0eigen_quanta<J>.chk (with J=0's for the root correlation), host only."""
    L = lib()
    err = C.create_string_buffer(512)
    dims = np.zeros(6, np.int32)
    d = directory.encode()
    _host_err(L.gi_trove_read_basis(d, J, sym_type, _p(dims, i32p), None, None, None, None, None,
                                    None, None, err, 512), err)
    D, ncase, maxdeg, mat, ncls, N = (int(x) for x in dims)
    out = {"D": D, "ncase": ncase, "max_deg_size": maxdeg, "mat_size": mat, "nclasses": ncls,
           "N": N, "k": np.zeros(D, np.int32), "ktau": np.zeros(D, np.int32),
           "iroot": np.zeros(D, np.int32), "icontr2icase": np.zeros(2 * D, np.int32),
           "Nsym": np.zeros(nrep * ncase, np.int32), "Ntotal": np.zeros(nrep, np.int32)}
    # sizes of repres need Ntotal: a second call fills it, a third the tables
    _host_err(L.gi_trove_read_basis(d, J, sym_type, _p(dims, i32p), None, None, None, None, None,
                                    _p(out["Ntotal"], i32p), None, err, 512), err)
    out["repres"] = [np.zeros(int(out["Ntotal"][g]) * degen[g] * mat, np.float64)
                     for g in range(nrep)]
    rp = (f64p * nrep)(*[_p(r, f64p) for r in out["repres"]])
    _host_err(L.gi_trove_read_basis(d, J, sym_type, _p(dims, i32p), _p(out["k"], i32p),
                                    _p(out["ktau"], i32p), _p(out["iroot"], i32p),
                                    _p(out["icontr2icase"], i32p), _p(out["Nsym"], i32p),
                                    _p(out["Ntotal"], i32p), rp, err, 512), err)
    return out


def trove_read_dipole(directory: str, N: int) -> np.ndarray:
    mu = np.zeros(3 * N * N, np.float64)
    err = C.create_string_buffer(512)
    _host_err(lib().gi_trove_read_dipole(directory.encode(), N, _p(mu, f64p), err, 512), err)
    return mu.reshape(3, N * N)


def trove_read_levels(directory: str, J: int, gamma: int, sym_type: int, nmodes: int,
                      nclasses: int):
    """Levels of j0eigen_descr<J>_<gamma+1>.chk and its basis dimension."""
    L = lib()
    err = C.create_string_buffer(512)
    n, dim = C.c_int32(0), C.c_int32(0)
    d = directory.encode()
    _host_err(L.gi_trove_read_levels(d, J, gamma, sym_type, nmodes, nclasses, C.byref(n),
                                     C.byref(dim), None, 0, err, 512), err)
    out = (gi_trove_level * max(n.value, 1))()
    _host_err(L.gi_trove_read_levels(d, J, gamma, sym_type, nmodes, nclasses, C.byref(n),
                                     C.byref(dim), out, n.value, err, 512), err)
    return list(out)[:n.value], dim.value


class Engine:
    """One GPU context of the line-intensity engine (gi_create/gi_destroy)."""

    def __init__(self, device: int = 0, hbm_budget: int = 0):
        self._L = lib()
        h = C.c_void_p()
        st = self._L.gi_create(C.byref(h), device, hbm_budget)
        if st != GI_OK:
            raise GiError(st, "gi_create failed (no usable CUDA device?)")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._L.gi_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _ck(self, st: int):
        if st != GI_OK:
            msg = self._L.gi_last_error(self._h).decode(errors="replace")
            raise GiError(st, msg)

    # inputs --------------------------------------------------------------
    def set_stream(self, stream: int | None):
        """Order the engine's device work on a caller's cudaStream_t (an int
        handle, e.g. torch.cuda.Stream().cuda_stream); None: its own stream."""
        self._ck(self._L.gi_set_stream(self._h, C.c_void_p(stream or None)))

    def set_tuning(self, mode: int, path: Optional[str] = None):
        """Split GEMM autotuner: mode 1 times the candidate launch configurations
        on the first GEMM of each new shape class; path keeps the table on disk."""
        self._ck(self._L.gi_set_tuning(self._h, mode, path.encode() if path else None))

    def set_refine(self, max_lines: int):
        """Re-evaluate up to max_lines doubtful lines per run exactly
        (gi_set_refine); lines next to a threshold are always re-evaluated."""
        self._ck(self._L.gi_set_refine(self._h, int(max_lines)))

    def set_symmetry(self, sym_type: int):
        self._ck(self._L.gi_set_symmetry(self._h, sym_type))

    def set_params(self, params, precision: int = GI_PREC_FP64, split_slices: int = 0):
        self._params = make_params(params, precision, split_slices)
        self._ck(self._L.gi_set_params(self._h, C.byref(self._params)))

    def set_dipole(self, N: int, mu: np.ndarray):
        m = np.ascontiguousarray(mu, np.float64).reshape(-1)
        if m.size != 3 * N * N:
            raise ValueError("mu must hold 3*N*N doubles")
        self._ck(self._L.gi_set_dipole(self._h, N, _p(m, f64p)))

    def set_dipole_flipped(self, N: int, dip: np.ndarray):
        """Dipole in the reference's flipped layout: dip[c][i][f] = mu_c(i, f)."""
        m = np.ascontiguousarray(dip, np.float64).reshape(-1)
        if m.size != 3 * N * N:
            raise ValueError("dip must hold 3*N*N doubles")
        self._ck(self._L.gi_set_dipole_flipped(self._h, N, _p(m, f64p)))

    def set_dipole_streamed(self, N: int, mu: np.ndarray, panel_rows: int = 0,
                            borrow: bool = False):
        """Dipole kept in host memory and streamed through the device in panels
        of `panel_rows` rows f (0: the engine's default).  With borrow=True the
        engine page-locks and reads this array (kept alive by the Engine)."""
        m = np.ascontiguousarray(mu, np.float64).reshape(-1)
        if m.size != 3 * N * N:
            raise ValueError("mu must hold 3*N*N doubles")
        self._ck(self._L.gi_set_dipole_streamed(self._h, N, _p(m, f64p), panel_rows,
                                                GI_DIPOLE_BORROW if borrow else 0))
        self._borrowed = m if borrow else None

    @property
    def dipole_panel_rows(self) -> int:
        """Rows per panel of a streamed dipole; 0 when the dipole is resident."""
        return int(self._L.gi_dipole_panel_rows(self._h))

    def set_basis(self, b):
        arrs = [np.ascontiguousarray(getattr(b, n), np.int32) for n in
                ("icontr2icase", "iroot_correlat_j0", "k", "ktau", "Nsym", "Ntotal")]
        reps = [np.ascontiguousarray(r, np.float64) for r in b.repres]
        rp = (f64p * len(reps))(*[_p(r, f64p) for r in reps])
        self._ck(self._L.gi_set_basis(self._h, b.jval, b.Maxcontracts, b.Maxsymcoeffs,
                                      b.max_deg_size, b.mat_size,
                                      *[_p(a, i32p) for a in arrs], rp))

    def set_threej(self, jmax: int, table: np.ndarray):
        t = np.ascontiguousarray(table, np.float64)
        self._ck(self._L.gi_set_threej(self._h, jmax, _p(t, f64p)))

    def set_block(self, J: int, gamma: int, vecs: np.ndarray, energies: np.ndarray,
                  quanta: np.ndarray):
        v = np.ascontiguousarray(vecs, np.float64)
        e = np.ascontiguousarray(energies, np.float64)
        q = np.ascontiguousarray(quanta, np.int32)
        nvec, nsize = v.shape
        self._ck(self._L.gi_set_block(self._h, J, gamma, nsize, nvec, _p(v, f64p), _p(e, f64p),
                                      _p(q, i32p)))

    def set_block_device(self, J: int, gamma: int, vecs_dev_ptr: int, nvec: int, nsize: int,
                         energies: np.ndarray, quanta: np.ndarray):
        """Block whose vectors are already in device memory ([nvec][nsize] doubles)."""
        e = np.ascontiguousarray(energies, np.float64)
        q = np.ascontiguousarray(quanta, np.int32)
        self._ck(self._L.gi_set_block_device(self._h, J, gamma, nsize, nvec,
                                             C.c_void_p(vecs_dev_ptr), _p(e, f64p), _p(q, i32p)))

    def load(self, prob, precision: int = GI_PREC_FP64, split_slices: int = 0,
             panel_rows: Optional[int] = None):
        """Hand a synth.Problem (or any object with the same fields) to the engine;
        panel_rows (not None) streams the dipole from host memory in panels."""
        self.set_symmetry(prob.sym_type)
        self.set_params(prob.params, precision, split_slices)
        if panel_rows is None:
            self.set_dipole(prob.N, prob.mu)
        else:
            self.set_dipole_streamed(prob.N, prob.mu, panel_rows)
        for J in sorted(prob.bases):
            self.set_basis(prob.bases[J])
        for (J, g), b in sorted(prob.blocks.items()):
            self.set_block(J, g, b.vecs, b.energies, b.quanta)

    # run -----------------------------------------------------------------
    def run(self, lines_on_device: bool = False, phase_timing: bool = False,
            graph: bool = False, shard: int = 0, nshards: int = 1, compact: bool = False) -> int:
        """gi_run, or with nshards > 1 gi_run_shard: the initial levels at
        positions l % nshards == shard of the level table.  compact: the
        lines come back to host memory as 40-byte records (lines_compact)."""
        n = C.c_int64(0)
        flags = (GI_RUN_LINES_ON_DEVICE if lines_on_device else 0) | \
            (GI_RUN_PHASE_TIMING if phase_timing else 0) | (GI_RUN_GRAPH if graph else 0) | \
            (GI_RUN_COMPACT_LINES if compact else 0)
        if nshards > 1:
            self._ck(self._L.gi_run_shard(self._h, flags, shard, nshards, C.byref(n)))
        else:
            self._ck(self._L.gi_run(self._h, flags, C.byref(n)))
        return int(n.value)

    def lines(self, offset: int = 0, count: Optional[int] = None) -> np.ndarray:
        total = self.stats()["nlines"]
        if count is None:
            count = total - offset
        out = np.empty(count, LINE_DTYPE)
        if count:
            self._ck(self._L.gi_get_lines(self._h, offset, count, out.ctypes.data))
        return out

    def lines_compact(self, offset: int = 0, count: Optional[int] = None) -> np.ndarray:
        """The last run's lines as gi_line_compact records."""
        total = self.stats()["nlines"]
        if count is None:
            count = total - offset
        out = np.empty(count, LINE_COMPACT_DTYPE)
        if count:
            self._ck(self._L.gi_get_lines_compact(self._h, offset, count, out.ctypes.data))
        return out

    def sort_lines(self):
        """Order the last run's lines by (initial level, final level)."""
        self._ck(self._L.gi_sort_lines(self._h))

    def levels(self) -> np.ndarray:
        n = C.c_int32(0)
        self._ck(self._L.gi_num_levels(self._h, C.byref(n)))
        out = np.empty(n.value, LEVEL_DTYPE)
        if n.value:
            self._ck(self._L.gi_get_levels(self._h, n.value, out.ctypes.data))
        return out

    def stats(self) -> Dict[str, float]:
        s = gi_stats()
        self._ck(self._L.gi_get_stats(self._h, C.byref(s)))
        out = {f: getattr(s, f) for f, _ in gi_stats._fields_
               if f not in ("reserved", "seconds_phase", "launches_phase")}
        out["seconds_phase"] = dict(zip(PHASES, list(s.seconds_phase)))
        out["launches_phase"] = dict(zip(PHASES, list(s.launches_phase)))
        return out

    # TROVE jobs and the reference's line list ---------------------------------
    def load_trove(self, directory: str, deck, all_j: bool = False,
                   stream_dipole: bool = False):
        d = parse_deck(deck) if isinstance(deck, str) else deck
        flags = (GI_TROVE_ALL_J if all_j else 0) | (GI_TROVE_STREAM_DIPOLE if stream_dipole else 0)
        self._ck(self._L.gi_load_trove(self._h, directory.encode(), C.byref(d), flags))
        self._deck = d

    def format_lines(self, offset: int = 0, count: Optional[int] = None) -> str:
        if count is None:
            count = self.stats()["nlines"] - offset
        used = C.c_size_t(0)
        self._ck(self._L.gi_format_lines(self._h, offset, count, None, 0, C.byref(used)))
        buf = C.create_string_buffer(used.value + 1)
        self._ck(self._L.gi_format_lines(self._h, offset, count, buf, used.value + 1,
                                         C.byref(used)))
        return buf.value.decode()

    def partition_function(self, temperature: float) -> float:
        q = C.c_double(0.0)
        self._ck(self._L.gi_partition_function(self._h, temperature, C.byref(q)))
        return q.value

    # serving ---------------------------------------------------------------
    def serve_start(self, slots: int = 3, budget: int = 0, slot_workspace: int = 0,
                    zcache: bool = True):
        cfg = gi_serve_config(slots, 0 if zcache else 1, budget, slot_workspace)
        self._ck(self._L.gi_serve_start(self._h, C.byref(cfg)))

    def serve_stop(self):
        self._ck(self._L.gi_serve_stop(self._h))

    def submit(self, jI: int, gammaI: int, jF: int, gammaF: int) -> int:
        i = C.c_uint64(0)
        self._ck(self._L.gi_submit(self._h, jI, gammaI, jF, gammaF, C.byref(i)))
        return int(i.value)

    def wait(self, job: int, timeout: float = -1.0, check: bool = True) -> Dict[str, float]:
        info = gi_job_info()
        st = self._L.gi_job_wait(self._h, job, timeout, C.byref(info))
        if check:
            self._ck(st)
        return {f: getattr(info, f) for f, _ in gi_job_info._fields_}

    def job_lines(self, job: int, release: bool = True) -> np.ndarray:
        n = self.wait(job)["nlines"]
        out = np.empty(n, LINE_DTYPE)
        if n:
            self._ck(self._L.gi_job_lines(self._h, job, 0, n, out.ctypes.data))
        if release:
            self._ck(self._L.gi_job_release(self._h, job))
        return out

    def release(self, job: int):
        """Forget a finished job and its lines (gi_job_release)."""
        self._ck(self._L.gi_job_release(self._h, job))

    def serve_stats(self) -> Dict[str, float]:
        s = gi_serve_stats()
        self._ck(self._L.gi_serve_get_stats(self._h, C.byref(s)))
        return {f: getattr(s, f) for f, _ in gi_serve_stats._fields_ if f != "reserved"}

    def serve_reset_stats(self):
        self._ck(self._L.gi_serve_reset_stats(self._h))

    def half_ls(self, jI: int, gammaI: int, ideg: int, jF: int, vsym: np.ndarray,
                D_F: int) -> np.ndarray:
        v = np.ascontiguousarray(vsym, np.float64)
        out = np.zeros(D_F, np.float64)
        self._ck(self._L.gi_half_ls(self._h, jI, gammaI, ideg, jF, _p(v, f64p), _p(out, f64p)))
        return out


def keyed(lines: np.ndarray, levels: np.ndarray) -> np.ndarray:
    """Engine lines with (J, gamma, record) keys of both levels attached."""
    li = levels[lines["level_i"]]
    lf = levels[lines["level_f"]]
    out = np.empty(len(lines), dtype=[("jI", np.int32), ("gammaI", np.int32), ("recI", np.int32),
                                      ("jF", np.int32), ("gammaF", np.int32), ("recF", np.int32),
                                      ("nu", np.float64), ("S", np.float64), ("A", np.float64),
                                      ("I", np.float64), ("t", np.float64, (4,))])
    out["jI"], out["gammaI"], out["recI"] = li["J"], li["gamma"], li["rec"]
    out["jF"], out["gammaF"], out["recF"] = lf["J"], lf["gamma"], lf["rec"]
    for f in ("nu", "S", "A", "I", "t"):
        out[f] = lines[f]
    return out
