"""gi_half_ls_noalloc: the half line strength for callers that cannot allocate
device memory at the point of the call (a serving loop whose HBM is fully
reserved by its admission budget, a framework or eigensolver that owns device
memory through its own pool, latency-sensitive code that cannot take the
implicit synchronisation of cudaMalloc/cudaFree).  The caller owns the input
and output device buffers; the scratch is a fixed array inside the library.

Checked through the C ABI against the allocating gi_half_ls, on two calls in
a row, with the tolerance of the other half-line-strength tests; and the
size limit is checked to fail with a clear error.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def call_noalloc(pkg, eng, jI, gI, ideg, jF, vsym_dev, out_dev, stream):
    return pkg.lib().gi_half_ls_noalloc(eng._h, jI, gI, ideg, jF, C.c_void_p(vsym_dev.data_ptr()),
                                        C.c_void_p(out_dev.data_ptr()), C.c_void_p(stream))


def test_noalloc_matches_half_ls_twice(pkg, synth):
    torch = pytest.importorskip("torch")
    stream = torch.cuda.current_stream().cuda_stream
    cases = 0
    for prob in (synth.make_c2v(3, 16, [1, 2, 3], nvec_max=3),
                 synth.make_c3v(4, 14, [1, 2, 3], nvec_max=3)):
        with pkg.Engine(0) as eng:
            eng.load(prob)
            for (jI, gI), blk in sorted(prob.blocks.items()):
                if blk.nvec == 0:
                    continue
                vdev = torch.from_numpy(np.ascontiguousarray(blk.vecs[0])).to("cuda")
                for jF in prob.jlist:
                    if abs(jF - jI) > 1:
                        continue
                    DF = prob.bases[jF].Maxcontracts
                    for d in range(prob.degen[gI]):
                        want = eng.half_ls(jI, gI, d, jF, blk.vecs[0], DF)
                        outs = [torch.full((DF,), float("nan"), dtype=torch.float64,
                                           device="cuda") for _ in range(2)]
                        for out in outs:  # two calls in a row on one stream
                            st = call_noalloc(pkg, eng, jI, gI, d, jF, vdev, out, stream)
                            assert st == pkg.GI_OK, pkg.lib().gi_last_error(eng._h)
                        torch.cuda.synchronize()
                        tol = 1e-13 * np.abs(want).max()
                        for out in outs:
                            got = out.cpu().numpy()
                            assert np.abs(got - want).max() <= tol
                        cases += 1
    assert cases > 20


def test_noalloc_rejects_sizes_beyond_scratch(pkg, synth):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(2)
    N = 2000  # row stride 2048
    vib = synth._c2v_vib_syms(rng, N)
    big = synth.make_c2v_basis(128, vib, rng)  # 257 (k, tau) slots: 257 * 2048 > 2^19
    p = synth.Params()
    with pkg.Engine(0) as eng:
        eng.set_symmetry(synth.SYM_C2V)
        eng.set_params(p)
        eng.set_dipole(N, synth.make_dipole(rng, N))
        eng.set_basis(big)
        vdev = torch.zeros(int(big.Ntotal[0]), dtype=torch.float64, device="cuda")
        out = torch.zeros(big.Maxcontracts, dtype=torch.float64, device="cuda")
        st = call_noalloc(pkg, eng, 128, 0, 0, 128, vdev, out,
                          torch.cuda.current_stream().cuda_stream)
        assert st == pkg.GI_ERR_ARG
        assert b"beyond the fixed scratch" in pkg.lib().gi_last_error(eng._h)


def test_noalloc_captured_in_a_graph(pkg, synth):
    """The call issues only device work on the caller's stream (no host copy,
    no synchronisation), so after a first call on the device it can be
    captured into a CUDA graph: a replay after the input vector changed gives
    that vector's half line strength, bit for bit the direct call's."""
    torch = pytest.importorskip("torch")
    prob = synth.make_c3v(4, 14, [1, 2], nvec_max=3)
    with pkg.Engine(0) as eng:
        eng.load(prob)
        jI, gI = 1, 2  # E: the second degenerate component below
        blk = prob.blocks[(jI, gI)]
        jF = jI + 1
        DF = prob.bases[jF].Maxcontracts
        d = prob.degen[gI] - 1
        s = torch.cuda.Stream()
        vdev = torch.from_numpy(np.ascontiguousarray(blk.vecs[0])).to("cuda")
        out = torch.zeros(DF, dtype=torch.float64, device="cuda")
        direct = torch.zeros_like(out)
        with torch.cuda.stream(s):
            assert call_noalloc(pkg, eng, jI, gI, d, jF, vdev, out, s.cuda_stream) == pkg.GI_OK
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            st = call_noalloc(pkg, eng, jI, gI, d, jF, vdev, out, s.cuda_stream)
        assert st == pkg.GI_OK, pkg.lib().gi_last_error(eng._h)
        vdev.copy_(torch.from_numpy(np.ascontiguousarray(blk.vecs[1])))
        g.replay()
        torch.cuda.synchronize()
        with torch.cuda.stream(s):
            assert call_noalloc(pkg, eng, jI, gI, d, jF, vdev, direct, s.cuda_stream) == pkg.GI_OK
        torch.cuda.synchronize()
        assert torch.equal(out, direct)
        want = eng.half_ls(jI, gI, d, jF, blk.vecs[1], DF)
        assert np.abs(out.cpu().numpy() - want).max() <= 1e-13 * np.abs(want).max()
