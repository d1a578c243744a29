"""Serving loop: pair jobs, continuous batching over several streams, block
residency under a budget, latency statistics.

The lines of a pair job are the lines of that block pair in a full gi_run
(same filters, ZPE and J range); a job gives the same lines alone and in a mix
of concurrent jobs; evicting blocks to pinned host and bringing them back
changes nothing.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KEY = ("jI", "gammaI", "recI", "jF", "gammaF", "recF")


def pair_jobs(prob):
    """Every (J, Gamma) -> (J', Gamma') block pair with |dJ| <= 1."""
    keys = sorted(prob.blocks)
    return [(jI, gI, jF, gF) for (jI, gI) in keys for (jF, gF) in keys if abs(jI - jF) <= 1]


def job_keyed(lines, job):
    jI, gI, jF, gF = job
    out = np.empty(len(lines), dtype=[("jI", np.int32), ("gammaI", np.int32),
                                      ("recI", np.int32), ("jF", np.int32),
                                      ("gammaF", np.int32), ("recF", np.int32),
                                      ("S", np.float64), ("A", np.float64), ("I", np.float64),
                                      ("nu", np.float64)])
    out["jI"], out["gammaI"], out["jF"], out["gammaF"] = jI, gI, jF, gF
    out["recI"], out["recF"] = lines["level_i"], lines["level_f"]
    for f in ("S", "A", "I", "nu"):
        out[f] = lines[f]
    return out


def as_dict(arr):
    return {tuple(int(r[k]) for k in KEY): (r["S"], r["A"], r["I"], r["nu"]) for r in arr}


def serve_all(pkg, prob, jobs, precision, slots=3, budget=0, slot_ws=0, order=None,
              zcache=True):
    with pkg.Engine(0) as eng:
        eng.load(prob, precision=precision)
        eng.serve_start(slots=slots, budget=budget, slot_workspace=slot_ws, zcache=zcache)
        ids = [eng.submit(*j) for j in (order or jobs)]
        res = {}
        for j, i in zip(order or jobs, ids):
            res[j] = eng.job_lines(i)
        st = eng.serve_stats()
        eng.serve_stop()
    return res, st


def assert_same(a, b, rtol):
    assert a.keys() == b.keys()
    for k, va in a.items():
        vb = b[k]
        for x, y in zip(va, vb):
            assert abs(x - y) <= rtol * max(abs(x), abs(y)) + 1e-300, (k, va, vb)


@pytest.mark.parametrize("precision", [0, 1])
def test_pair_jobs_cover_the_full_run(pkg, synth, precision):
    prob = synth.make_c2v(21, 40, [0, 1, 2, 3], nvec_max=10)
    with pkg.Engine(0) as eng:
        eng.load(prob, precision=precision)
        eng.run()
        full = as_dict(pkg.keyed(eng.lines(), eng.levels()))
    jobs = pair_jobs(prob)
    res, st = serve_all(pkg, prob, jobs, precision)
    got = {}
    for j, lines in res.items():
        got.update(as_dict(job_keyed(lines, j)))
    assert st["completed"] == len(jobs) and st["failed"] == 0
    assert len(full) > 500
    assert_same(got, full, 1e-13)


def test_same_alone_and_in_the_mix(pkg, synth):
    prob = synth.make_c3v(22, 36, [0, 1, 2, 3], nvec_max=12)
    jobs = pair_jobs(prob)
    rng = np.random.default_rng(5)
    order = [jobs[i] for i in rng.permutation(len(jobs))]
    res, st = serve_all(pkg, prob, jobs, 1, slots=4, order=order)
    assert st["completed"] == len(jobs)
    assert 0 < st["latency_p50"] <= st["latency_p99"] <= st["latency_max"]
    # the jobs with the most lines (E blocks included), each run alone
    probes = sorted(jobs, key=lambda j: -len(res[j]))[:3]
    for probe in probes:
        alone, _ = serve_all(pkg, prob, [probe], 1, slots=1)
        a = as_dict(job_keyed(alone[probe], probe))
        b = as_dict(job_keyed(res[probe], probe))
        assert len(a) > 0
        assert_same(a, b, 1e-13)


def test_eviction_to_host_keeps_results(pkg, synth):
    prob = synth.make_c2v(23, 48, [0, 1, 2, 3, 4], nvec_max=40)
    jobs = pair_jobs(prob)
    big, st_big = serve_all(pkg, prob, jobs, 1, slots=2, zcache=False)
    assert st_big["evictions"] == 0
    blk = max(b.vecs.nbytes for b in prob.blocks.values())
    slot_ws = 8 << 20
    # room for the slot workspaces and a few blocks (with their digit planes)
    budget = 2 * slot_ws + 40 * blk
    small, st = serve_all(pkg, prob, jobs, 1, slots=2, budget=budget, slot_ws=slot_ws,
                          zcache=False)
    assert st["evictions"] > 0 and st["restores"] > 0
    assert st["peak_resident_bytes"] <= budget - 2 * slot_ws
    for j in jobs:
        assert_same(as_dict(job_keyed(small[j], j)), as_dict(job_keyed(big[j], j)), 0.0)


def test_job_larger_than_budget_fails_cleanly(pkg, synth):
    prob = synth.make_c2v(24, 48, [0, 1, 2], nvec_max=40)
    slot_ws = 1 << 20
    with pkg.Engine(0) as eng:
        eng.load(prob, precision=1)
        eng.serve_start(slots=1, budget=slot_ws + (4 << 10), slot_workspace=slot_ws)
        i = eng.submit(1, 0, 2, 1)
        info = eng.wait(i, check=False)
        assert info["state"] == pkg.GI_JOB_FAILED
        assert info["status"] == pkg.GI_ERR_BUDGET
        eng.serve_stop()


@pytest.mark.parametrize("precision", [0, 1])
def test_zcache_shares_initial_blocks(pkg, synth, precision):
    """Jobs that start from the same initial block reuse its cached half line
    strength: the lines are bit for bit those of jobs that compute it, with a
    cache large enough for every block and with one so small that entries are
    evicted and recomputed."""
    prob = synth.make_c3v(25, 36, [0, 1, 2, 3], nvec_max=12)
    jobs = [j for j in pair_jobs(prob) if j[3] == prob.partner(j[1])]
    plain, st0 = serve_all(pkg, prob, jobs, precision, slots=3, zcache=False)
    cached, st = serve_all(pkg, prob, jobs, precision, slots=3)
    assert st0["zcache_hits"] == 0
    assert st["zcache_hits"] > 0 and st["zcache_misses"] > 0
    assert st["zcache_hits"] + st["zcache_misses"] <= len(jobs)
    for j in jobs:
        assert np.array_equal(np.sort(cached[j], order=["level_i", "level_f"]),
                              np.sort(plain[j], order=["level_i", "level_f"]))
    slot_ws = 8 << 20
    # room for the slot workspaces and a few final blocks with their digit
    # planes and cached Z: entries and blocks take turns
    tight, st2 = serve_all(pkg, prob, jobs, precision, slots=2, budget=2 * slot_ws + (1 << 20),
                           slot_ws=slot_ws)
    assert st2["zcache_evictions"] > 0 or st2["evictions"] > 0
    for j in jobs:
        assert np.array_equal(np.sort(tight[j], order=["level_i", "level_f"]),
                              np.sort(plain[j], order=["level_i", "level_f"]))
