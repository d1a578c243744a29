"""Split-precision path (bf16 digit GEMMs on tcgen05) against the CPU oracle:
identical line selection and <= 1e-10 relative error in S, A and I on every
line above the workloads' intensity threshold."""
import numpy as np
import pytest

from paritylib import compare, with_threshold

pytestmark = pytest.mark.gpu


def run(pkg, prob, slices=0, refine=1 << 20):
    with pkg.Engine(0) as eng:
        eng.load(prob, precision=pkg.GI_PREC_SPLIT, split_slices=slices)
        eng.set_refine(refine)
        eng.run()
        return pkg.keyed(eng.lines(), eng.levels()), eng.stats()


@pytest.mark.parametrize("case", ["c2v", "c3v", "c3v_reduced"])
def test_split_matches_oracle(pkg, synth, oracle, case):
    if case == "c2v":
        prob = synth.make_c2v(11, 30, [0, 1, 2, 3], nvec_max=8)
    else:
        prob = synth.make_c3v(12, 24, [0, 1, 2, 3], nvec_max=8, reduced=case.endswith("reduced"))
    with_threshold(prob)
    got, st = run(pkg, prob)
    res = compare(got, oracle.run_all(prob), rtol_S=1e-10, norm_tol=1e-12)
    assert st["flops_tensor"] > 0
    print(case, res)


def test_split_small_workload(pkg, synth, oracle):
    prob = with_threshold(synth.workload("c2v_small", seed=1))
    got, st = run(pkg, prob)
    res = compare(got, oracle.run_all(prob), rtol_S=1e-10, norm_tol=1e-12)
    print(res, st["seconds_gpu"])


@pytest.mark.parametrize("slices", [6, 9, 10])
def test_split_slice_counts(pkg, synth, oracle, slices):
    prob = with_threshold(synth.make_c2v(4, 40, [0, 1, 2], nvec_max=10))
    got, _ = run(pkg, prob, slices)
    ref = oracle.run_all(prob)
    tol = {6: 1e-6, 9: 1e-10, 10: 1e-10}[slices]
    res = compare(got, ref, rtol_S=tol, norm_tol=tol / 100)
    print(slices, res)


def test_autotuner_table_and_results(pkg, synth, tmp_path, monkeypatch):
    """gi_set_tuning(1, path): every GEMM shape class gets a timed choice in the
    table file, and the tuned run's lines agree with the default ones.  The
    final-state GEMMs go through the tuner when they run one launch per final
    block (GI_SPLIT_PERSIST=0)."""
    monkeypatch.setenv("GI_SPLIT_PERSIST", "0")
    prob = synth.make_c2v(51, 64, [0, 1, 2, 3], nvec_max=24)
    path = str(tmp_path / "tune.txt")
    with pkg.Engine(0) as eng:
        eng.load(prob, precision=1)
        eng.run()
        ref = np.sort(eng.lines(), order=["level_i", "level_f"])
        eng.set_tuning(1, path)
        eng.run()
        got = np.sort(eng.lines(), order=["level_i", "level_f"])
    rows = [l.split() for l in open(path).read().splitlines()]
    assert len(rows) >= 2 and all(len(r) == 8 for r in rows)
    assert all(r[5] in ("6", "7", "8", "9") for r in rows)  # the grouped layout's kernels
    assert np.array_equal(got[["level_i", "level_f"]], ref[["level_i", "level_f"]])
    assert np.allclose(got["S"], ref["S"], rtol=1e-12, atol=0)


@pytest.mark.parametrize("config", ["grouped/9:64", "grouped/9:1", "plain/0:64", "plain/1:16",
                                    "plain/1:128", "plain/1:1", "plain/2:32", "grouped/6:64",
                                    "grouped/6:1", "grouped/7:32", "grouped/8:64"])
def test_every_split_kernel_matches_oracle(pkg, synth, oracle, monkeypatch, config):
    """Each launch configuration the autotuner can pick (one-pass, two-pass at
    either split point, the grouped-layout kernels and their 2-SM pair form,
    several L2 groups), pinned
    with GI_SPLIT_FORCE on its digit layout.  Row and column tile counts are
    odd here, so tiles past the edge run too."""
    layout, force = config.split("/")
    monkeypatch.setenv("GI_SPLIT_LAYOUT", layout)
    monkeypatch.setenv("GI_SPLIT_FORCE", force)
    prob = with_threshold(synth.make_c3v(13, 40, [0, 1, 2, 3], nvec_max=20))
    got, _ = run(pkg, prob)
    res = compare(got, oracle.run_all(prob), rtol_S=1e-10, norm_tol=1e-12)
    print(config, res)


@pytest.mark.parametrize("config", ["grouped/9:64", "plain/0:64", "plain/1:64", "plain/2:64",
                                    "grouped/6:64", "grouped/7:64", "grouped/8:64"])
def test_every_split_kernel_large_k(pkg, synth, monkeypatch, config):
    """Each configuration at contraction lengths of 1216 (half line strength)
    to ~2100 (final states), where the exact integer diagonal sums reach the
    int64 range, against the FP64 GPU path on the same job."""
    layout, force = config.split("/")
    prob = with_threshold(synth.make_c2v(61, 1200, [0, 1, 2, 3], nvec_max=12))
    with pkg.Engine(0) as eng:
        eng.load(prob, precision=pkg.GI_PREC_FP64)
        eng.set_refine(1 << 20)
        eng.run()
        want = pkg.keyed(eng.lines(), eng.levels())
    monkeypatch.setenv("GI_SPLIT_LAYOUT", layout)
    monkeypatch.setenv("GI_SPLIT_FORCE", force)
    got, _ = run(pkg, prob)
    res = compare(got, want, rtol_S=1e-10, norm_tol=1e-12)
    print(config, res)


@pytest.mark.parametrize("case,budget", [("c3v", 0), ("c3v", 24 << 20), ("c2v_large_k", 0),
                                         ("c3v_many_blocks", 0)])
def test_persistent_grouped_final_gemm(pkg, synth, monkeypatch, case, budget):
    """The final-state GEMMs of all final blocks of a round in one persistent
    launch (a work list of uneven tiles, K segments inside the kernel) give the
    same lines, bit for bit, as one launch per block: in one round or many
    (small HBM budget), and with final blocks of ~2100 functions (two K
    segments per tile)."""
    if case == "c3v":
        prob = synth.make_c3v(71, 40, [0, 1, 2, 3, 4], nvec_max=30)
    elif case == "c2v_large_k":
        prob = synth.make_c2v(61, 1200, [0, 1, 2, 3], nvec_max=12)
    else:  # 63 final blocks in one round: groups split at the launch's 44 problems
        prob = synth.make_c3v(72, 24, list(range(21)), nvec_max=6)
    out = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("GI_SPLIT_PERSIST", mode)
        with pkg.Engine(0, hbm_budget=budget) as eng:
            eng.load(prob, precision=1)
            eng.run(phase_timing=True)
            st = eng.stats()
            out[mode] = (pkg.keyed(eng.lines(), eng.levels()), st["launches_phase"]["final_gemm"])
    (a, la), (b, lb) = out["0"], out["1"]
    order = ["jI", "gammaI", "recI", "jF", "gammaF", "recF"]
    a, b = np.sort(a, order=order), np.sort(b, order=order)
    assert len(a) > 1000 and lb < la
    for f in a.dtype.names:
        assert np.array_equal(a[f], b[f]), f


@pytest.mark.parametrize("case,budget,thresh", [("c3v", 0, 0.0), ("c3v", 24 << 20, 1e-30),
                                                ("c2v_large_k", 0, 1e-30),
                                                ("c3v_many_blocks", 0, 0.0),
                                                ("c3v_reduced", 0, 1e-30)])
def test_fused_epilogue_matches_separate(pkg, synth, monkeypatch, case, budget, thresh):
    """The S/A/I epilogue formed by the persistent final GEMM's epilogue warps
    on the last K segment gives the lines of the separate epilogue launches,
    bit for bit (every field), with fewer launches: one round or many, two K
    segments per tile, groups split at the launch's problem limit, degenerate
    symmetries with the reduced combination rule; with graph replay too."""
    if case.startswith("c3v") and case != "c3v_many_blocks":
        prob = synth.make_c3v(71, 40, [0, 1, 2, 3, 4], nvec_max=30,
                              reduced=case.endswith("reduced"))
    elif case == "c2v_large_k":
        prob = synth.make_c2v(61, 1200, [0, 1, 2, 3], nvec_max=12)
    else:
        prob = synth.make_c3v(72, 24, list(range(21)), nvec_max=6)
    prob.params.thresh_intensity = thresh
    out = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("GI_SPLIT_FUSED_EPI", mode)
        with pkg.Engine(0, hbm_budget=budget) as eng:
            eng.load(prob, precision=1)
            eng.run()
            st = eng.stats()
            lines = pkg.keyed(eng.lines(), eng.levels())
            eng.run(graph=True)
            eng.run(graph=True)  # a replay
            again = pkg.keyed(eng.lines(), eng.levels())
        out[mode] = (lines, again, st)
    order = ["jI", "gammaI", "recI", "jF", "gammaF", "recF"]
    (a, a2, sa), (b, b2, sb) = out["0"], out["1"]
    a, b = np.sort(a, order=order), np.sort(b, order=order)
    b2 = np.sort(b2, order=order)
    assert len(a) > 1000 and sb["kernel_launches"] < sa["kernel_launches"]
    assert sb["nlines_filtered"] == sa["nlines_filtered"]
    for f in a.dtype.names:
        assert np.array_equal(a[f], b[f]), f
        assert np.array_equal(b[f], b2[f]), f
