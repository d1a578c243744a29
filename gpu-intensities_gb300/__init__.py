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


class gi_stats(C.Structure):
    _fields_ = [("nlines", C.c_int64), ("nlines_filtered", C.c_int64),
                ("npairs_checked", C.c_int64),
                ("nblock_pairs", C.c_int32), ("nlevels", C.c_int32), ("zpe", C.c_double),
                ("seconds_total", C.c_double), ("seconds_gpu", C.c_double),
                ("flops_halfls", C.c_double), ("flops_final", C.c_double),
                ("flops_tensor", C.c_double), ("bytes_correlate", C.c_double),
                ("seconds_phase", C.c_double * 6), ("launches_phase", C.c_int32 * 6),
                ("kernel_launches", C.c_int32), ("reserved", C.c_int32)]


class gi_serve_config(C.Structure):
    _fields_ = [("slots", C.c_int32), ("reserved", C.c_int32),
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
                ("slots", C.c_int32), ("reserved", C.c_int32)]


GI_JOB_QUEUED, GI_JOB_RUNNING, GI_JOB_DONE, GI_JOB_FAILED = range(4)


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
        L.gi_set_basis.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                   i32p, i32p, i32p, i32p, i32p, i32p, C.POINTER(f64p)]
        L.gi_set_threej.argtypes = [C.c_void_p, C.c_int, f64p]
        L.gi_set_block.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, f64p, f64p,
                                   i32p]
        L.gi_set_block_device.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                          C.c_void_p, f64p, i32p]
        L.gi_run.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int64)]
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
        L.gi_num_levels.argtypes = [C.c_void_p, C.POINTER(C.c_int32)]
        L.gi_get_levels.argtypes = [C.c_void_p, C.c_int32, C.c_void_p]
        L.gi_get_stats.argtypes = [C.c_void_p, C.POINTER(gi_stats)]
        L.gi_half_ls.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, f64p, f64p]
        L.gi_measure_fp64_peak.argtypes = [C.c_int, f64p]
        L.gi_measure_mma_cycles.argtypes = [C.c_int, C.c_int, f64p]
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


def measure_mma_cycles(device: int = 0, n: int = 128) -> float:
    """Cycles of one bf16 tcgen05 MMA (M=128, K=16) of width n (gi_measure_mma_cycles)."""
    v = C.c_double(0.0)
    st = lib().gi_measure_mma_cycles(device, n, C.byref(v))
    if st != GI_OK:
        raise GiError(st, "gi_measure_mma_cycles failed")
    return v.value


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

    def load(self, prob, precision: int = GI_PREC_FP64, split_slices: int = 0):
        """Hand a synth.Problem (or any object with the same fields) to the engine."""
        self.set_symmetry(prob.sym_type)
        self.set_params(prob.params, precision, split_slices)
        self.set_dipole(prob.N, prob.mu)
        for J in sorted(prob.bases):
            self.set_basis(prob.bases[J])
        for (J, g), b in sorted(prob.blocks.items()):
            self.set_block(J, g, b.vecs, b.energies, b.quanta)

    # run -----------------------------------------------------------------
    def run(self, lines_on_device: bool = False, phase_timing: bool = False,
            graph: bool = False) -> int:
        n = C.c_int64(0)
        flags = (GI_RUN_LINES_ON_DEVICE if lines_on_device else 0) | \
            (GI_RUN_PHASE_TIMING if phase_timing else 0) | (GI_RUN_GRAPH if graph else 0)
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

    # serving ---------------------------------------------------------------
    def serve_start(self, slots: int = 3, budget: int = 0, slot_workspace: int = 0):
        cfg = gi_serve_config(slots, 0, budget, slot_workspace)
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
