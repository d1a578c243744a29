"""TROVE job files and the input deck (host code, no GPU).

The readers are held to what the reference's own readers (bset_contr_factory,
correlate_index, read_eigenvalues, read_dipole_flipped) make of the same
files: through the committed fixture tests/golden/trove_c3v (written by
synth.write_trove, parsed by the reference in make_golden.py), and on fresh
files where the reference pin library exists.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN


def basis_equal(got, want_basis, nrep, degen):
    assert np.array_equal(got["k"], want_basis.k)
    assert np.array_equal(got["ktau"], want_basis.ktau)
    assert np.array_equal(got["iroot"], want_basis.iroot_correlat_j0)
    assert np.array_equal(got["icontr2icase"], want_basis.icontr2icase)
    assert np.array_equal(got["Nsym"], want_basis.Nsym)
    assert np.array_equal(got["Ntotal"], want_basis.Ntotal)
    for g in range(nrep):  # the generator keeps one zero for an empty symmetry
        n = int(want_basis.Ntotal[g]) * degen[g] * want_basis.mat_size
        assert np.array_equal(got["repres"][g], np.asarray(want_basis.repres[g])[:n])


@pytest.mark.parametrize("sym", ["c2v", "c3v"])
def test_round_trip_of_a_synthetic_job(pkg, synth, tmp_path, sym):
    prob = (synth.make_c2v(7, 16, [0, 1, 2], nvec_max=4) if sym == "c2v"
            else synth.make_c3v(7, 15, [0, 1, 2], nvec_max=4))
    d = str(tmp_path)
    deck = synth.write_trove(prob, d)
    for J in prob.jlist:
        got = pkg.trove_read_basis(d, J, prob.sym_type, prob.nrep, prob.degen)
        assert got["N"] == prob.N and got["nclasses"] == 1
        basis_equal(got, prob.bases[J], prob.nrep, prob.degen)
    assert np.array_equal(pkg.trove_read_dipole(d, prob.N), prob.mu.reshape(3, -1))
    nm = prob.params.nmodes
    for (J, g), blk in prob.blocks.items():
        lv, dim = pkg.trove_read_levels(d, J, g, prob.sym_type, nm, 1)
        assert dim == blk.nsize and len(lv) == blk.nvec
        assert np.array_equal([x.energy for x in lv], blk.energies)
        assert np.array_equal(np.array([list(x.quanta)[:nm + 1] for x in lv],
                                       np.int32).reshape(-1, nm + 1), blk.quanta)
        assert all(x.ndeg == prob.degen[g] and x.irec[0] == i * x.ndeg + 1
                   for i, x in enumerate(lv))
    d2 = pkg.parse_deck(deck)
    p = prob.params
    assert (d2.sym_type, d2.nmodes, list(d2.jvals)) == (prob.sym_type, nm,
                                                         [prob.jlist[0], prob.jlist[-1]])
    assert d2.params.temperature == p.temperature and d2.params.q_stat == p.q_stat
    assert list(d2.params.gns)[:prob.nrep] == list(p.gns)[:prob.nrep]
    assert list(d2.params.isym_pairs)[:prob.nrep] == list(p.isym_pairs)[:prob.nrep]
    assert tuple(d2.params.erange_lower) == tuple(p.erange_lower)
    assert tuple(d2.params.freq_window) == tuple(p.freq_window)


def test_deck_keywords(pkg):
    deck = """
    NMODES 3
    SYMGROUP C3V(M)
    INTENSITY
      temperature 500.0
      qstat 12.5
      zpe -1
      J 4, 5
      freq-window  -0.1, 8000.0
      energy low -0.1, 6000.0, upper -0.1, 9000.0
      gns 2.0 2.0 4.0
      selection (rules) 1 1 2
      thresh_line 1e-8
      V 2 lower 0 4 upper 1 9
      symmetry reduced
    end
    """
    d = pkg.parse_deck(deck)
    p = d.params
    assert (d.sym_type, d.nmodes, list(d.jvals)) == (2, 3, [4, 5])
    assert (p.temperature, p.q_stat, p.ZPE) == (500.0, 12.5, -1.0)
    assert tuple(p.freq_window) == (-0.1, 8000.0)
    assert tuple(p.erange_lower) == (-0.1, 6000.0) and tuple(p.erange_upper) == (-0.1, 9000.0)
    assert list(p.gns)[:3] == [2.0, 2.0, 4.0] and list(p.isym_pairs)[:3] == [1, 1, 2]
    assert p.thresh_linestrength == 1e-8 and p.reduced == 1
    assert (p.quanta_lower[0][1], p.quanta_lower[1][1]) == (0, 4)
    assert (p.quanta_upper[0][1], p.quanta_upper[1][1]) == (1, 9)
    with pytest.raises(pkg.GiError):
        pkg.parse_deck("SYMGROUP C7V(M)\n")


def test_reader_errors(pkg, synth, tmp_path):
    prob = synth.make_c2v(8, 10, [0, 1], nvec_max=2)
    d = str(tmp_path)
    synth.write_trove(prob, d)
    with pytest.raises(pkg.GiError, match="cannot open"):
        pkg.trove_read_basis(d, 5, prob.sym_type, prob.nrep, prob.degen)
    with pytest.raises(pkg.GiError, match="N=10"):
        pkg.trove_read_dipole(d, 11)
    path = os.path.join(d, "j0eigen_quanta1.chk")
    text = open(path).read()
    open(path, "w").write(text.replace("Start Primitive basis set", "Start primitive basis"))
    with pytest.raises(pkg.GiError, match="bad header"):
        pkg.trove_read_basis(d, 1, prob.sym_type, prob.nrep, prob.degen)
    raw = bytearray(open(os.path.join(d, "j0_extfield.chk"), "rb").read())
    raw[4:9] = b"Stop "
    open(os.path.join(d, "j0_extfield.chk"), "wb").write(bytes(raw))
    with pytest.raises(pkg.GiError, match="bogus header"):
        pkg.trove_read_dipole(d, 10)


def levels_as_set(levels, sym_type):
    return {(int(x["jval"]), int(x["igamma"]), int(x["ilevel"])):
            (float(x["energy"]), int(x["irec0"]), int(x["krot"]), int(x["taurot"]),
             tuple(int(q) for q in x["quanta"][:7]), tuple(int(q) for q in x["normal"][:7]))
            for x in levels}


def ours_as_set(pkg, d, js, sym_type, nrep, nmodes):
    out = {}
    for J in js:
        for g in range(nrep):
            lv, _ = pkg.trove_read_levels(d, J, g, sym_type, nmodes, 1)
            for x in lv:
                out[(J, g, x.ilevel)] = (x.energy, x.irec[0], x.krot, x.taurot,
                                         tuple(list(x.quanta)[:7]), tuple(list(x.normal)[:7]))
    return out


def test_golden_fixture_parsed_as_the_reference_parses_it(pkg, synth):
    d = os.path.join(GOLDEN, "trove_c3v")
    ref = np.load(os.path.join(GOLDEN, "trove_c3v_ref.npz"))
    sym, nrep, degen = 2, 3, [1, 1, 2]
    deck = pkg.parse_deck(open(os.path.join(d, "job.inp")).read())
    js = sorted({int(k[5:].split("_")[0]) for k in ref.files if k.startswith("basis")})
    for J in js:
        got = pkg.trove_read_basis(d, J, sym, nrep, degen)
        for key in ("k", "ktau", "iroot", "icontr2icase", "Nsym", "Ntotal"):
            assert np.array_equal(got[key], ref[f"basis{J}_{key}"]), (J, key)
        for g in range(nrep):
            assert np.array_equal(got["repres"][g], ref[f"basis{J}_repres{g}"])
    want = levels_as_set(ref["levels"], sym)
    got = ours_as_set(pkg, d, js, sym, nrep, deck.nmodes)
    assert got == want and len(got) > 10


def test_live_reference_readers(pkg, synth, oracle, tmp_path):
    if not oracle.ref_available():
        pytest.skip("reference pin library not built (reference sources absent)")
    prob = synth.make_c2v(9, 14, [0, 1, 2], nvec_max=3)
    d = str(tmp_path)
    synth.write_trove(prob, d)
    for J in prob.jlist:
        got = pkg.trove_read_basis(d, J, prob.sym_type, prob.nrep, prob.degen)
        want = oracle.ref_trove_basis(d, J, prob.degen)
        for key in ("k", "ktau", "iroot", "icontr2icase", "Nsym", "Ntotal"):
            assert np.array_equal(got[key], want[key]), (J, key)
    # read_eigenvalues reads exactly two J values (the deck's jvals)
    lv = oracle.ref_trove_levels(d, (1, 2), prob.sym_type, prob.degen, prob.params.nmodes, 1,
                                 0.0, (-1e300, 1e300), prob.params.gns,
                                 max(b.Maxcontracts for b in prob.bases.values()))
    assert ours_as_set(pkg, d, [1, 2], prob.sym_type, prob.nrep, prob.params.nmodes) == \
        levels_as_set(lv, prob.sym_type)
    N = prob.N
    flip = np.zeros(3 * N * N)
    oracle.ref().ref_read_dipole_flipped(d.encode(), N, oracle.ptr(flip, oracle.f64p))
    ours = pkg.trove_read_dipole(d, N).reshape(3, N, N)
    assert np.array_equal(np.transpose(ours, (0, 2, 1)).reshape(-1), flip)
