"""The small kernels of a run as work lists: every unit's Y digit rows of a
round, every H build, every H column norm and every H slice of a group of
final blocks in one launch each.  The lines are bit for bit those of one
launch per item (GI_BATCH_SMALL=0), on both paths, in one round and in many,
with graph replay, and the run takes fewer launches."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ORDER = ["level_i", "level_f"]


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("case,budget", [("c3v", 0), ("c3v", 24 << 20), ("c2v_large_k", 0),
                                         ("c3v_many_blocks", 0)])
def test_batched_small_launches_match(pkg, synth, monkeypatch, precision, case, budget):
    if case == "c3v":
        prob = synth.make_c3v(71, 40, [0, 1, 2, 3, 4], nvec_max=30)
    elif case == "c2v_large_k":
        prob = synth.make_c2v(61, 1200, [0, 1, 2, 3], nvec_max=12)
    else:
        prob = synth.make_c3v(72, 24, list(range(21)), nvec_max=6)
    prob.params.thresh_intensity = 1e-30
    out = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("GI_BATCH_SMALL", mode)
        with pkg.Engine(0, hbm_budget=budget) as eng:
            eng.load(prob, precision=precision)
            eng.set_refine(1 << 20)
            eng.run()
            st = eng.stats()
            lines = np.sort(eng.lines(), order=ORDER)
            eng.run(graph=True)
            eng.run(graph=True)  # a replay
            again = np.sort(eng.lines(), order=ORDER)
        out[mode] = (lines, again, st)
    (a, a2, sa), (b, b2, sb) = out["0"], out["1"]
    assert len(a) > 1000
    assert sb["kernel_launches"] < sa["kernel_launches"]
    for f in a.dtype.names:
        assert np.array_equal(a[f], b[f]), f
        assert np.array_equal(b[f], b2[f]), f
        assert np.array_equal(a[f], a2[f]), f
