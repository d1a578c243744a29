"""TROVE jobs on the GPU: gi_load_trove gives the same lines as handing the
same job over in memory; the reference's line list format; the partition
function; the gi_main process-level drop-in."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KEY = ["level_i", "level_f"]


def lines_of(eng, pkg):
    k = pkg.keyed(eng.lines(), eng.levels())
    return np.sort(k, order=["jI", "gammaI", "recI", "jF", "gammaF", "recF"])


@pytest.mark.parametrize("sym", ["c2v", "c3v"])
@pytest.mark.parametrize("precision", [0, 1])
def test_trove_load_equals_in_memory_job(pkg, synth, tmp_path, sym, precision):
    prob = (synth.make_c2v(31, 24, [0, 1, 2, 3], nvec_max=8) if sym == "c2v"
            else synth.make_c3v(31, 21, [0, 1, 2, 3], nvec_max=8))
    deck = synth.write_trove(prob, str(tmp_path))
    with pkg.Engine(0) as eng:
        eng.load(prob, precision=precision)
        eng.run()
        want = lines_of(eng, pkg)
    with pkg.Engine(0) as eng:
        d = pkg.parse_deck(deck)
        d.params.precision = precision
        eng.load_trove(str(tmp_path), d, all_j=True)
        eng.run()
        got = lines_of(eng, pkg)
    assert len(want) > 100
    for f in ("jI", "gammaI", "recI", "jF", "gammaF", "recF"):
        assert np.array_equal(got[f], want[f])
    assert np.array_equal(got["S"], want["S"]) and np.array_equal(got["t"], want["t"])


def test_line_list_format_and_partition_function(pkg, synth, tmp_path):
    prob = synth.make_c3v(32, 21, [0, 1, 2], nvec_max=6)
    deck = synth.write_trove(prob, str(tmp_path))
    with pkg.Engine(0) as eng:
        eng.load_trove(str(tmp_path), deck, all_j=True)
        n = eng.run()
        text = eng.format_lines()
        lines = eng.lines()
        levels = eng.levels()
        q = eng.partition_function(500.0)
    rows = text.splitlines()
    assert len(rows) == n > 20
    labels = ["A1", "A2", "E"]
    for row, ln in zip(rows, lines):
        LF, LI = levels[ln["level_f"]], levels[ln["level_i"]]
        tok = row.split()
        # jF gF <- jI gI branch EF <- EI nu ...
        assert int(tok[0]) == LF["J"] and tok[1] == labels[LF["gamma"]]
        assert tok[2] == "<-" and int(tok[3]) == LI["J"] and tok[4] == labels[LI["gamma"]]
        assert tok[5] == {0: "Q", 1: "R", -1: "P"}[int(LF["J"]) - int(LI["J"])]
        assert float(tok[6]) == pytest.approx(LF["energy"], abs=6e-5)
        assert float(tok[9]) == pytest.approx(abs(ln["nu"]), abs=6e-5)
        nd = ln["ndeg_i"] * ln["ndeg_f"]
        vals = [float(x) for x in tok[-nd:]]
        want_t = [ln["t"][dI + 2 * dF] for dF in range(ln["ndeg_f"]) for dI in range(ln["ndeg_i"])]
        assert vals == pytest.approx(want_t, rel=1e-8, abs=1e-300)
        s_a_i = [float(x) for x in row.split(")")[4].split()[:3]]
        assert s_a_i == pytest.approx([ln["S"], ln["A"], ln["I"]], rel=1e-7)
    beta = 6.62606896e-27 * 2.99792458e10 / (1.380658e-16 * 500.0)
    want_q = sum(prob.params.gns[g] * (2 * J + 1) * prob.degen[g] * np.exp(-e * beta).sum()
                 for (J, g), b in prob.blocks.items() for e in [b.energies])
    assert q == pytest.approx(want_q, rel=1e-12)


def test_gi_main_process(pkg, synth, tmp_path):
    exe = os.path.join(os.path.dirname(pkg.LIB_PATH), "gi_main")
    if not os.path.exists(exe):
        pytest.skip("gi_main not built")
    prob = synth.make_c2v(33, 20, [0, 1], nvec_max=5)
    deck = synth.write_trove(prob, str(tmp_path))
    out = subprocess.run([exe, str(tmp_path)], input=deck.encode(), capture_output=True,
                         check=True).stdout.decode()
    head, _, body = out.partition("\n\n\n")
    assert head.startswith("Linestrength S(f<-i)")
    with pkg.Engine(0) as eng:
        eng.load_trove(str(tmp_path), deck)
        eng.run()
        eng.sort_lines()  # gi_main prints in (initial, final) level order
        assert body == eng.format_lines()
        ln = eng.lines()
    assert len(body.splitlines()) > 10
    key = ln["level_i"].astype(np.int64) * (1 << 32) + ln["level_f"]
    assert np.all(np.diff(key) > 0)


def test_computed_partition_function_in_the_run(pkg, synth):
    """q_stat <= 0: the run divides by the partition function of the loaded
    levels, as if that value had been given."""
    prob = synth.make_c2v(34, 24, [0, 1, 2], nvec_max=6)
    with pkg.Engine(0) as eng:
        eng.load(prob)
        q = eng.partition_function(prob.params.temperature)
        p = prob.params
        p.q_stat = q
        eng.set_params(p)
        eng.run()
        want = np.sort(eng.lines(), order=KEY)
        p.q_stat = 0.0
        eng.set_params(p)
        eng.run()
        got = np.sort(eng.lines(), order=KEY)
    assert len(want) > 50
    assert np.array_equal(got["I"], want["I"]) and np.array_equal(got["S"], want["S"])
