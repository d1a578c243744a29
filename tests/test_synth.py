"""Invariants of the synthetic inputs and of their persistence."""
import numpy as np
import pytest


@pytest.mark.parametrize("maker", ["c2v", "c3v"])
def test_basis_and_block_invariants(synth, maker):
    prob = synth.make_c2v(1, 16, [0, 1, 2, 3], nvec_max=6) if maker == "c2v" else \
        synth.make_c3v(2, 12, [0, 1, 2, 3], nvec_max=6)
    N = prob.N
    mu = prob.mu.reshape(3, N, N)
    assert np.allclose(mu[0], mu[0].T) and np.allclose(mu[2], mu[2].T)
    assert np.allclose(mu[1], -mu[1].T)
    for J, b in prob.bases.items():
        assert b.Maxcontracts == (2 * J + 1) * N
        assert int(b.Ntotal.sum() * 1) <= b.Maxcontracts
        degs = np.array(prob.degen)
        assert int((b.Ntotal * degs).sum()) == b.Maxcontracts
        assert set(np.unique(b.k)) <= set(range(J + 1))
        assert np.all(b.ktau >> 1 == b.k)
    for (J, g), blk in prob.blocks.items():
        assert blk.nsize == prob.bases[J].Ntotal[g]
        G = blk.vecs @ blk.vecs.T
        assert np.allclose(G, np.eye(blk.nvec), atol=1e-12)
        assert np.all(np.diff(blk.energies) >= 0)


def test_save_load_roundtrip(synth, tmp_path):
    prob = synth.make_c3v(5, 10, [1, 2], nvec_max=4, reduced=True)
    p = tmp_path / "p.npz"
    synth.save(prob, str(p))
    q = synth.load(str(p))
    assert q.sym_type == prob.sym_type and q.N == prob.N
    assert np.array_equal(q.mu, prob.mu)
    assert q.params.reduced and q.params.gns == prob.params.gns
    for J in prob.bases:
        assert np.array_equal(q.bases[J].icontr2icase, prob.bases[J].icontr2icase)
        for a, b in zip(q.bases[J].repres, prob.bases[J].repres):
            assert np.array_equal(a, b)
    for k in prob.blocks:
        assert np.array_equal(q.blocks[k].vecs, prob.blocks[k].vecs)
