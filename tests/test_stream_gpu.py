"""A dipole streamed from host memory in panels of rows f (the reference's
split-dipole path for dipoles above 5 GiB: read_dipole_flipped_blocks,
trove_functions.cpp:207-310; do_1st_half_ls_blocks, cuda_host.cu:783-817).

Each panel's GEMM produces its own rows of Z = mu^T Y with the resident
GEMM's per-element reduction (and, on the split path, the same per-row digit
exponents), so every result must be BIT-IDENTICAL to the resident dipole's:
lines of every precision, one panel or many, ragged last panels, a borrowed
(page-locked) caller array, repeated runs reusing the staging panels, the
single-vector half line strength, the allocation-free entry point and a
TROVE job loaded with its dipole streamed.
"""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

FIELDS = ("jI", "gammaI", "recI", "jF", "gammaF", "recF")


def keyed(pkg, eng):
    k = pkg.keyed(eng.lines(), eng.levels())
    return np.sort(k, order=list(FIELDS))


def run_lines(pkg, prob, precision, panel_rows=None, runs=1, **kw):
    with pkg.Engine(0) as eng:
        eng.load(prob, precision=precision, panel_rows=panel_rows)
        if panel_rows is not None:
            assert eng.dipole_panel_rows == min(panel_rows, prob.N) or panel_rows == 0
        out = []
        for _ in range(runs):
            eng.run(**kw)
            out.append((keyed(pkg, eng), eng.stats()))
        return out


def assert_same(a, b):
    assert len(a) == len(b)
    for f in a.dtype.names:
        assert np.array_equal(a[f], b[f]), f


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("panel", [0, 37, 128, 10000])
def test_streamed_lines_identical(pkg, synth, precision, panel):
    """One panel (10000 > N), the default (0), a 128-row tile and a ragged
    37-row panel: the same lines, bit for bit."""
    prob = synth.make_c3v(51, 150, [0, 1, 2, 3], nvec_max=10)
    (ref, st_r), = run_lines(pkg, prob, precision)
    (got, st_s), = run_lines(pkg, prob, precision, panel_rows=panel)
    assert len(ref) > 200
    assert_same(ref, got)
    npanel = -(-prob.N // min(panel or prob.N, prob.N))
    gemms = st_r["launches_phase"]["halfls_gemm"]
    assert st_s["launches_phase"]["halfls_gemm"] == gemms * npanel


def test_streamed_repeated_runs_and_graph_flag(pkg, synth):
    """Staging panels reused across runs (the copy of a run's first panel waits
    for the previous run's last reader); GI_RUN_GRAPH runs eagerly."""
    prob = synth.make_c2v(52, 120, [0, 1, 2], nvec_max=8)
    (ref, _), = run_lines(pkg, prob, 1)
    outs = run_lines(pkg, prob, 1, panel_rows=50, runs=3, graph=True)
    for got, _ in outs:
        assert_same(ref, got)


def test_borrowed_dipole(pkg, synth):
    prob = synth.make_c2v(53, 90, [0, 1, 2], nvec_max=6)
    (ref, _), = run_lines(pkg, prob, 1)
    with pkg.Engine(0) as eng:
        eng.load(prob, precision=1)
        mu = np.array(prob.mu, np.float64).reshape(-1)
        eng.set_dipole_streamed(prob.N, mu, panel_rows=40, borrow=True)
        eng.run()
        assert_same(ref, keyed(pkg, eng))
        # back to a resident dipole: the borrowed array is released
        eng.set_dipole(prob.N, prob.mu)
        assert eng.dipole_panel_rows == 0
        eng.run()
        assert_same(ref, keyed(pkg, eng))


def test_streamed_half_ls_and_noalloc(pkg, synth):
    torch = pytest.importorskip("torch")
    prob = synth.make_c3v(54, 60, [1, 2], nvec_max=3)
    stream = torch.cuda.current_stream().cuda_stream
    with pkg.Engine(0) as res, pkg.Engine(0) as stm:
        res.load(prob)
        stm.load(prob, panel_rows=16)
        n = 0
        for (jI, gI), blk in sorted(prob.blocks.items()):
            if blk.nvec == 0:
                continue
            vdev = torch.from_numpy(np.ascontiguousarray(blk.vecs[0])).to("cuda")
            for jF in prob.jlist:
                DF = prob.bases[jF].Maxcontracts
                for d in range(prob.degen[gI]):
                    want = res.half_ls(jI, gI, d, jF, blk.vecs[0], DF)
                    got = stm.half_ls(jI, gI, d, jF, blk.vecs[0], DF)
                    assert np.array_equal(want, got)
                    out = torch.full((DF,), float("nan"), dtype=torch.float64, device="cuda")
                    st = pkg.lib().gi_half_ls_noalloc(
                        stm._h, jI, gI, d, jF, C.c_void_p(vdev.data_ptr()),
                        C.c_void_p(out.data_ptr()), C.c_void_p(stream))
                    assert st == pkg.GI_OK, pkg.lib().gi_last_error(stm._h)
                    torch.cuda.synchronize()
                    assert np.array_equal(out.cpu().numpy(), want)
                    n += 1
        assert n > 4


def test_streamed_dipole_cannot_be_served(pkg, synth):
    prob = synth.make_c2v(55, 40, [0, 1], nvec_max=3)
    with pkg.Engine(0) as eng:
        eng.load(prob, panel_rows=16)
        with pytest.raises(pkg.GiError, match="resident dipole"):
            eng.serve_start(slots=1)


def test_trove_job_with_streamed_dipole(pkg):
    d = os.path.join(GOLDEN, "trove_c3v")
    deck = open(os.path.join(d, "job.inp")).read()
    out = []
    for stream_dipole in (False, True):
        with pkg.Engine(0) as eng:
            eng.load_trove(d, deck, stream_dipole=stream_dipole)
            assert (eng.dipole_panel_rows > 0) == stream_dipole
            eng.run()
            out.append(keyed(pkg, eng))
    assert len(out[0]) > 10
    assert_same(out[0], out[1])


def test_precision_workload_streamed(pkg, synth):
    """Full-size c2v_precision job (Nvib = 5000, K = 5000) with its dipole in
    four panels of 1280 rows (the last ragged): identical to the resident run
    on the split path."""
    prob = synth.workload("c2v_precision", seed=3)
    e = np.sort(np.concatenate([b.energies[:8] for b in prob.blocks.values()]))
    prob.params.erange_lower = (0.0, float(e[7]))
    (ref, _), = run_lines(pkg, prob, 1)
    (got, st), = run_lines(pkg, prob, 1, panel_rows=1280)
    assert len(ref) > 5000
    assert_same(ref, got)
