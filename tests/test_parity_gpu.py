"""Engine (CUDA, through the C ABI) against the CPU oracle: identical line
selection and per-line accuracy in FP64 (relative 1e-11 in S, A and I on
every line above the workloads' intensity threshold)."""
import numpy as np
import pytest

from paritylib import compare, with_threshold

pytestmark = pytest.mark.gpu


def run_engine(pkg, prob, refine=1 << 20, **kw):
    """One job; doubtful lines (moments cancelled far below their columns)
    re-evaluated exactly, up to `refine` per run."""
    with pkg.Engine(0) as eng:
        eng.load(prob, **kw)
        eng.set_refine(refine)
        eng.run()
        return pkg.keyed(eng.lines(), eng.levels()), eng.stats(), eng.levels()


@pytest.mark.parametrize("case", ["c2v", "c3v", "c3v_reduced"])
def test_lines_match_oracle(pkg, synth, oracle, case):
    if case == "c2v":
        prob = synth.make_c2v(11, 30, [0, 1, 2, 3], nvec_max=8)
    else:
        prob = synth.make_c3v(12, 24, [0, 1, 2, 3], nvec_max=8, reduced=case.endswith("reduced"))
    with_threshold(prob)
    got, st, _ = run_engine(pkg, prob)
    ref = oracle.run_all(prob)
    res = compare(got, ref)
    assert res["n"] > 100
    print(case, res, st["kernel_launches"])


def test_small_workload_full(pkg, synth, oracle):
    """Every eigenvector of the CPU-sized workload (N=200, J=0..2)."""
    prob = with_threshold(synth.workload("c2v_small", seed=1))
    got, st, _ = run_engine(pkg, prob)
    ref = oracle.run_all(prob)
    res = compare(got, ref)
    assert res["n"] > 50000
    print(res)


@pytest.mark.parametrize("precision", [0, 1])
def test_half_ls_matches_oracle(pkg, synth, oracle, precision):
    """gi_half_ls on the FP64 path and on the split path (the narrow digit GEMM
    with K split over the SMs), normwise within 1e-13 of the oracle."""
    for prob in (synth.make_c2v(3, 16, [1, 2, 3], nvec_max=3),
                 synth.make_c3v(4, 14, [1, 2, 3], nvec_max=3),
                 synth.make_c2v(8, 700, [4, 5], nvec_max=2)):
        with pkg.Engine(0) as eng:
            eng.load(prob, precision=precision)
            for (jI, gI), blk in sorted(prob.blocks.items()):
                if blk.nvec == 0:
                    continue
                for jF in prob.jlist:
                    if abs(jF - jI) > 1:
                        continue
                    for d in range(prob.degen[gI]):
                        vprim = oracle.correlate(prob.bases[jI], prob.nrep, prob.degen, d, gI,
                                                 blk.vecs[0])
                        want = oracle.half_ls(prob.bases[jI], prob.bases[jF], prob.N, prob.mu,
                                              max(prob.jlist), vprim)
                        got = eng.half_ls(jI, gI, d, jF, blk.vecs[0], prob.bases[jF].Maxcontracts)
                        assert np.abs(got - want).max() <= 1e-13 * np.abs(want).max()


def test_empty_and_filtered(pkg, synth, oracle):
    prob = with_threshold(synth.make_c2v(5, 20, [0, 1, 2], nvec_max=6))
    # an empty block and a symmetry switched off by its spin weight
    b = prob.blocks[(1, 2)]
    prob.blocks[(1, 2)] = synth.Block(1, 2, b.vecs[:0], b.energies[:0], b.quanta[:0])
    prob.params.gns = (1.0, 1.0, 0.0, 0.0)
    got, _, _ = run_engine(pkg, prob)
    ref = oracle.run_all(prob)
    compare(got, ref)
    assert len(ref) > 0 and np.all(ref["gammaI"] < 2)
    # windows that select nothing
    prob.params.erange_lower = (1e8, 2e8)
    got, _, _ = run_engine(pkg, prob)
    assert len(got) == 0 and len(oracle.run_all(prob)) == 0


def test_windows_thresholds_zpe(pkg, synth, oracle):
    prob = synth.make_c2v(6, 24, [0, 1, 2], nvec_max=10)
    p = prob.params
    p.ZPE = -1.0                      # taken from the first J=0, A1 record
    p.freq_window = (-3000.0, 8000.0)  # emission and absorption
    p.erange_lower = (0.0, 9000.0)
    p.erange_upper = (500.0, 19000.0)
    p.quanta_lower = np.array([[0, 1, 0], [7, 6, 7]], np.int32)
    p.quanta_upper = np.array([[1, 0, 0], [7, 7, 5]], np.int32)
    p.thresh_intensity = 1e-24
    p.thresh_linestrength = 1e-3
    got, st, _ = run_engine(pkg, prob)
    ref = oracle.run_all(prob)
    compare(got, ref)
    assert abs(st["zpe"] - prob.blocks[(0, 0)].energies[0]) == 0.0
    assert (ref["nu"] < 0).any() and len(ref) > 50


def test_errors_are_reported(pkg, synth):
    with pkg.Engine(0) as eng:
        with pytest.raises(pkg.GiError) as e:
            eng.run()
        assert e.value.status == pkg.GI_ERR_STATE
        prob = synth.make_c2v(1, 10, [0, 1], nvec_max=3)
        eng.set_symmetry(prob.sym_type)
        b = prob.bases[1]
        bad = synth.Basis(**{**b.__dict__, "Ntotal": b.Ntotal + 1})
        with pytest.raises(pkg.GiError) as e:
            eng.set_basis(bad)
        assert e.value.status == pkg.GI_ERR_ARG
        with pytest.raises(pkg.GiError):
            eng.set_symmetry(9)


def test_flipped_dipole_layout(pkg, synth):
    """gi_set_dipole_flipped (the reference's in-memory layout) = gi_set_dipole."""
    prob = synth.make_c2v(31, 30, [0, 1, 2], nvec_max=6)
    got = []
    for flipped in (False, True):
        with pkg.Engine(0) as eng:
            eng.load(prob)
            if flipped:
                N = prob.N
                eng.set_dipole_flipped(N, prob.mu.reshape(3, N, N).transpose(0, 2, 1))
            eng.run()
            got.append(np.sort(eng.lines(), order=["level_i", "level_f"]))
    assert len(got[0]) > 50
    assert np.array_equal(got[0]["S"], got[1]["S"])


@pytest.mark.parametrize("precision", [0, 1])
def test_graph_replay_matches_eager(pkg, synth, precision):
    """GI_RUN_GRAPH: captured once, replayed while the plan is unchanged,
    recaptured when it changes; every run equals the eager launch sequence."""
    prob = synth.make_c3v(41, 30, [0, 1, 2, 3], nvec_max=10)

    def lines(eng, **kw):
        eng.run(**kw)
        return np.sort(eng.lines(), order=["level_i", "level_f"]), eng.stats()

    with pkg.Engine(0) as eng:
        eng.load(prob, precision=precision)
        lines(eng)  # the first run also cuts the final blocks' digit planes
        eager, st_e = lines(eng)
        for _ in range(3):  # capture, then two replays
            g, st_g = lines(eng, graph=True)
            assert np.array_equal(g, eager)
            assert st_g["kernel_launches"] == st_e["kernel_launches"]
        # a new threshold changes the epilogue's arguments: recapture
        p = prob.params
        p.thresh_intensity = 1e-24
        eng.set_params(p, precision=precision)
        eager2, _ = lines(eng)
        g2, _ = lines(eng, graph=True)
        assert len(eager2) < len(eager)
        assert np.array_equal(g2, eager2)
        # new vectors of the same shape (same device arrays): replay reads them
        blk = prob.blocks[(2, 0)]
        eng.set_block(2, 0, -blk.vecs, blk.energies, blk.quanta)
        eager3, _ = lines(eng)
        g3, _ = lines(eng, graph=True)
        assert np.array_equal(g3, eager3)


@pytest.mark.parametrize("budget", [0, 48 << 20])
def test_host_readback_equals_device_lines(pkg, synth, budget):
    """Lines read back to host memory while the run goes on (a copy per final
    block, after its epilogues) equal the device-resident lines, eager and
    replayed, in one round or many (a small HBM budget)."""
    prob = synth.make_c3v(42, 40, [0, 1, 2, 3], nvec_max=12)
    with pkg.Engine(0, hbm_budget=budget) as eng:
        eng.load(prob, precision=1)
        eng.run(lines_on_device=True)
        ref = np.sort(eng.lines(), order=["level_i", "level_f"])
        assert len(ref) > 500
        for graph in (False, True, True):
            n = eng.run(lines_on_device=False, graph=graph)
            assert n == len(ref)
            assert np.array_equal(np.sort(eng.lines(), order=["level_i", "level_f"]), ref)


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("which", ["S", "I"])
def test_threshold_guard_band(pkg, synth, oracle, precision, which):
    """A threshold placed 2e-15 (relative, a few units of rounding) from a
    line's S or I, on either side: closer than the GEMM paths' error, so
    without the guard band the keep decision would follow rounding.  The
    engine re-evaluates lines that close to a threshold exactly before the
    keep decision, so its selection is the oracle's (double-double) one, on
    the FP64 and the split path."""
    prob = with_threshold(synth.make_c2v(21, 30, [0, 1, 2], nvec_max=8))
    ref = oracle.run_all(prob)
    assert len(ref) > 100
    key = "S" if which == "S" else "I"
    picks = np.argsort(ref[key])[[len(ref) // 5, len(ref) // 2, 4 * len(ref) // 5]]
    for idx in picks:
        for side in (-1.0, 1.0):
            v = float(ref[key][idx]) * (1.0 + side * 2e-15)
            if which == "S":
                prob.params.thresh_linestrength = v
            else:
                prob.params.thresh_intensity = v / 6.0221415e23
            want = oracle.run_all(prob)
            got, st, _ = run_engine(pkg, prob, refine=0, precision=precision)
            assert st["nlines_handed"] >= 1
            compare(got, want, rtol_S=1e-10 if precision else 1e-11,
                    norm_tol=1e-12 if precision else 1e-13)
        prob.params.thresh_linestrength = 0.0
        with_threshold(prob)


@pytest.mark.parametrize("precision", [0, 1])
def test_half_ls_repeated_calls_replay_a_graph(pkg, synth, precision):
    """The second call of a gi_half_ls shape is captured into a CUDA graph and
    later calls replay it: every call gives, bit for bit, what a first (eager)
    call on the same vector gives, also after the shape changed in between."""
    prob = synth.make_c3v(4, 14, [1, 2], nvec_max=4)
    DF = prob.bases[2].Maxcontracts
    blk = prob.blocks[(1, 2)]
    order = [(0, 1), (1, 1), (2, 1), (3, 0), (0, 1), (3, 1), (1, 0), (2, 1)]
    with pkg.Engine(0) as eng:
        eng.load(prob, precision=precision)
        got = [eng.half_ls(1, 2, d, 2, blk.vecs[i], DF) for i, d in order]
    for (i, d), g in zip(order, got):
        with pkg.Engine(0) as fresh:
            fresh.load(prob, precision=precision)
            want = fresh.half_ls(1, 2, d, 2, blk.vecs[i], DF)
        assert np.array_equal(g, want), (i, d)
