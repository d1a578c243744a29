"""GI_RUN_COMPACT_LINES: the 40-byte records that a run reads back carry
exactly the fields of the full records, line for line in the same order: on
both precision paths, through a graph replay and a shard, after the exact
re-evaluation has patched the list (a threshold a few units of rounding from
a line) and after gi_sort_lines.  gi_get_lines still returns the full records
of a compact run."""
import numpy as np
import pytest

from paritylib import with_threshold

pytestmark = pytest.mark.gpu

FIELDS = ("level_i", "level_f", "nu", "S", "A", "I")


def same(comp, full):
    assert len(comp) == len(full)
    for f in FIELDS:
        assert np.array_equal(comp[f], full[f]), f


def by_pair(x):
    return np.sort(x, order=["level_i", "level_f"])


@pytest.mark.parametrize("precision", [0, 1])
def test_compact_lines_equal_full(pkg, synth, precision):
    prob = with_threshold(synth.make_c3v(31, 30, [0, 1, 2, 3], nvec_max=12))
    with pkg.Engine(0) as eng:
        eng.load(prob, precision=precision)
        eng.run()
        full = eng.lines()
        assert len(full) > 1000
        n = eng.run(compact=True)
        comp = eng.lines_compact()
        assert n == len(full) and comp.dtype.itemsize == 40
        same(comp, eng.lines())                 # the same run's full records, same order
        same(by_pair(comp), by_pair(full))      # and the plain run's values
        eng.sort_lines()
        same(eng.lines_compact(), eng.lines())
        same(eng.lines_compact(), by_pair(full))
        for _ in range(2):                      # capture, then replay
            eng.run(compact=True, graph=True)
            same(eng.lines_compact(), eng.lines())
            same(by_pair(eng.lines_compact()), by_pair(full))
        eng.run(compact=True, shard=1, nshards=3)
        part = eng.lines_compact()
        same(part, eng.lines())
        eng.run(shard=1, nshards=3)
        same(by_pair(part), by_pair(eng.lines()))


@pytest.mark.parametrize("precision", [0, 1])
def test_compact_lines_after_exact_reevaluation(pkg, synth, precision):
    prob = with_threshold(synth.make_c2v(21, 30, [0, 1, 2], nvec_max=8))
    with pkg.Engine(0) as eng:
        eng.load(prob, precision=precision)
        eng.run()
        base = eng.lines()
        picks = np.argsort(base["S"])[[len(base) // 4, len(base) // 2]]
        for idx in picks:
            for side in (-1.0, 1.0):
                prob.params.thresh_linestrength = float(base["S"][idx]) * (1.0 + side * 2e-15)
                eng.set_params(prob.params, precision=precision)
                eng.run()
                want = eng.lines()
                eng.run(compact=True)
                assert eng.stats()["nlines_handed"] >= 1
                comp = eng.lines_compact()
                same(comp, eng.lines())
                same(by_pair(comp), by_pair(want))
