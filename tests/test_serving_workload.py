"""The serving workload's generators (host code): the block pool draws each
block's vector count log-uniform in its range, and the job stream draws
valid pair jobs (the initial block's selection partner, |dJ| <= 1, non-empty
blocks, the reference's rule against the (Jmin, Jmin) pair) with Poisson
inter-arrival gaps at the stated rate."""
import numpy as np


def test_pool_and_job_stream(synth):
    base = synth.make_c3v(3, 30, list(range(6)), nvec_max=4)
    pool = synth.serving_pool(base, seed=2, nvec_range=(5.0, 40.0), ecut=1e9)
    assert set(pool.blocks) == {(J, g) for J in base.bases for g in range(base.nrep)}
    counts = np.array([b.nvec for b in pool.blocks.values()])
    sizes = np.array([b.nsize for b in pool.blocks.values()])
    assert counts.min() >= 1 and counts.max() <= 40
    assert np.all(counts <= np.maximum(sizes, 1))
    jobs, gaps = synth.serving_jobs(pool, seed=3, njobs=4000, rate=200.0,
                                    dims=(float(sizes[sizes > 0].min()), float(sizes.max())))
    assert len(jobs) == 4000 and len(gaps) == 4000
    jmin = min(pool.jlist)
    for J, g, jF, gF in jobs:
        assert gF == pool.partner(g) and abs(jF - J) <= 1
        assert pool.blocks[(J, g)].nvec > 0 and pool.blocks[(jF, gF)].nvec > 0
        assert J + jF >= 1 and not (J == jmin and jF == jmin)
    # Poisson arrivals: exponential gaps with mean 1/rate
    assert abs(gaps.mean() * 200.0 - 1.0) < 0.08
    assert abs(gaps.std() / gaps.mean() - 1.0) < 0.1
    # initial blocks of many sizes (log-uniform in dimension)
    assert len({(J, g) for J, g, _, _ in jobs}) >= len(pool.blocks) // 2
