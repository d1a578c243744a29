"""Seeded synthetic inputs for the line-intensity path.

The reference reads TROVE checkpoints (basis tables, dipole, level records,
eigenvectors).  None ship with it, so every workload here is generated from a
seed with the shapes, sizes and value distributions of the named workloads:

* ``c2v_small``   triatomic C2v, J=0..2, Nvib=200, all eigenvectors (CPU-sized)
* ``c2v_plain``   triatomic C2v, J=0..10, Nvib=2000, lowest 1000 vectors per
                  (J, Gamma) under 15000 cm^-1 (the throughput workload)
* ``c2v_precision`` C2v, J=20,21, Nvib=5000, ~26k per Gamma (the J>0 bases
                  built on the lowest 2500 J=0 functions), 2000 vectors,
                  dipole magnitudes log-uniform 1e-8..1
* ``c3v_batched`` tetratomic C3v (A1, A2, E), Nvib=3000, J=0..40 (blocks up
                  to ~60k), <=1500 vectors under 12000 cm^-1, T=500 K
* serving     ``serving_pool`` / ``serving_jobs``: the c3v_batched bases with
                  100..2000 vectors per block (log-uniform), pair jobs with
                  initial block sizes log-uniform in 500..80k, Poisson arrivals

The contracted basis is the product form TROVE produces for a rigid-rotor
factor: for each J the "cases" are (k, vibrational function) with
k = 0..J, and the degenerate components ("lambda") enumerate tau (and, for
C3v, the components of a degenerate vibrational function).  The tables carry
exactly the meaning of the reference's ``TO_bset_contrT`` fields
(trove_objects.h:88-111): ``icontr2icase``, ``iroot_correlat_j0``, ``k``,
``ktau = 2k+tau``, per-symmetry ``N``/``Ntotal``/``repres``.  Eigenvectors are
the Q factor of a thin QR of a Gaussian ``nsize x nvec`` matrix (the same
distribution as the first ``nvec`` columns of a full Haar QR).
"""
from __future__ import annotations

import dataclasses
from concurrent.futures import ThreadPoolExecutor
from typing import Dict, List, Optional, Tuple

import numpy as np

# Symmetry groups as the reference's input deck knows them (fields.cpp:11-115).
SYM_C2V, SYM_C3V, SYM_D3H = 1, 2, 3
SYM_INFO = {
    SYM_C2V: dict(name="C2V(M)", degen=[1, 1, 1, 1], labels=["A1", "A2", "B1", "B2"]),
    SYM_C3V: dict(name="C3V(M)", degen=[1, 1, 2], labels=["A1", "A2", "E"]),
    SYM_D3H: dict(name="D3H(M)", degen=[1, 1, 2, 1, 1, 2],
                  labels=["A1'", "A2'", "E'", 'A1"', 'A2"', 'E"']),
}


@dataclasses.dataclass
class Basis:
    """Per-J contracted basis tables (mirrors TO_bset_contrT)."""
    jval: int
    Maxcontracts: int
    Maxsymcoeffs: int
    max_deg_size: int
    mat_size: int
    icontr2icase: np.ndarray      # int32 [2*D]
    iroot_correlat_j0: np.ndarray  # int32 [D]
    k: np.ndarray                  # int32 [D]
    ktau: np.ndarray               # int32 [D]
    Nsym: np.ndarray               # int32 [nrep*Maxsymcoeffs], N[g + icase*nrep]
    Ntotal: np.ndarray             # int32 [nrep]
    repres: List[np.ndarray]       # per g: float64 [Ntotal*degen*mat_size]

    def nsize(self, g: int) -> int:
        return int(self.Ntotal[g])


@dataclasses.dataclass
class Block:
    """One (J, Gamma) eigenvector block: vectors in record order."""
    J: int
    gamma: int
    vecs: np.ndarray      # float64 [nvec, nsize]
    energies: np.ndarray  # float64 [nvec], ascending
    quanta: np.ndarray    # int32 [nvec, nmodes+1]; quanta[:,0] = rotational index

    @property
    def nsize(self) -> int:
        return int(self.vecs.shape[1])

    @property
    def nvec(self) -> int:
        return int(self.vecs.shape[0])


@dataclasses.dataclass
class Params:
    """The intensity block of the input deck (fields.cpp:145-234)."""
    temperature: float = 296.0
    q_stat: float = 1.0
    ZPE: float = 0.0
    erange_lower: Tuple[float, float] = (0.0, 1.0e9)
    erange_upper: Tuple[float, float] = (0.0, 1.0e9)
    freq_window: Tuple[float, float] = (0.0, 1.0e9)
    gns: Tuple[float, ...] = (1.0, 1.0, 3.0, 3.0)
    isym_pairs: Tuple[int, ...] = (1, 1, 2, 2)
    reduced: bool = False
    nmodes: int = 3
    quanta_lower: Optional[np.ndarray] = None  # int32 [2, nmodes]: rows (min, max)
    quanta_upper: Optional[np.ndarray] = None
    thresh_linestrength: float = 0.0
    thresh_intensity: float = 0.0             # cm/molecule

    def windows(self):
        wide = np.array([[0] * self.nmodes, [1 << 30] * self.nmodes], dtype=np.int32)
        ql = wide if self.quanta_lower is None else np.asarray(self.quanta_lower, np.int32)
        qu = wide if self.quanta_upper is None else np.asarray(self.quanta_upper, np.int32)
        return ql, qu


@dataclasses.dataclass
class Problem:
    sym_type: int
    N: int
    mu: np.ndarray                      # float64 [3, N*N], mu_c(i,f) at [c, i + f*N]
    bases: Dict[int, Basis]
    blocks: Dict[Tuple[int, int], Block]
    params: Params
    name: str = ""

    @property
    def nrep(self) -> int:
        return len(SYM_INFO[self.sym_type]["degen"])

    @property
    def degen(self) -> List[int]:
        return SYM_INFO[self.sym_type]["degen"]

    @property
    def jlist(self) -> List[int]:
        return sorted(self.bases)

    def partner(self, g: int) -> int:
        """The symmetry a level of symmetry g can reach (find_igamma_pair,
        trove_functions.cpp:1041-1072): the other irrep of its isym_pairs
        class, or g itself when it is alone in its class."""
        for h in range(len(self.params.isym_pairs)):
            if h != g and self.params.isym_pairs[h] == self.params.isym_pairs[g]:
                return h
        return g

    def pair_jobs(self) -> List[Tuple[int, int, int, int]]:
        """Block pairs (jI, gI, jF, gF) that can carry lines: |dJ| <= 1 and
        gF the partner of gI, both blocks present with vectors."""
        out = []
        for (jI, gI), bI in sorted(self.blocks.items()):
            gF = self.partner(gI)
            for jF in (jI - 1, jI, jI + 1):
                bF = self.blocks.get((jF, gF))
                if bI.nvec and bF is not None and bF.nvec:
                    out.append((jI, gI, jF, gF))
        return out

    def nlines_upper_bound(self) -> int:
        n = 0
        for (jI, gI), bI in self.blocks.items():
            for (jF, gF), bF in self.blocks.items():
                if abs(jF - jI) <= 1 and self.params.isym_pairs[gI] == self.params.isym_pairs[gF] and gI != gF:
                    n += bI.nvec * bF.nvec
        return n


# ---------------------------------------------------------------- dipole
def make_dipole(rng: np.random.Generator, N: int, kind: str = "decay") -> np.ndarray:
    """mu_x, mu_z symmetric and mu_y antisymmetric, in Debye.

    kind="decay": N(0,1) * exp(-|i-j|/10); kind="loguniform": magnitudes
    log-uniform in [1e-8, 1] with random signs.
    """
    i = np.arange(N)
    mu = np.empty((3, N * N), dtype=np.float64)
    for c in range(3):
        if kind == "decay":
            a = rng.standard_normal((N, N)) * np.exp(-np.abs(i[:, None] - i[None, :]) / 10.0)
        else:
            mag = 10.0 ** rng.uniform(-8.0, 0.0, size=(N, N))
            a = mag * rng.choice([-1.0, 1.0], size=(N, N))
        if c == 1:
            a = np.triu(a, 1)
            a = a - a.T
        else:
            a = np.triu(a)
            a = a + np.triu(a, 1).T
        # record order: element (i, f) at i + f*N  (column-major)
        mu[c] = a.reshape(-1, order="F")
    return mu


# ---------------------------------------------------------------- C2v basis
def _c2v_vib_syms(rng: np.random.Generator, N: int) -> np.ndarray:
    # vibrational functions of a C2v triatomic are A1 (00) or B2 (11)
    return np.where(rng.random(N) < 0.5, 0, 3).astype(np.int32)


def _c2v_rot_bits(k: int, tau: int) -> int:
    # C2v(M) irreps as (C2, sigma) character bits: A1=00, A2=01, B1=10, B2=11
    return ((k & 1) << 1) | ((tau ^ (k & 1)) & 1)


def make_c2v_basis(J: int, vib_sym: np.ndarray, rng: np.random.Generator,
                   signs: bool = True) -> Basis:
    """Product basis (k, v) x tau for C2v; every primitive root carries one irrep."""
    N = len(vib_sym)
    nrep = 4
    cases = []  # (k, v, [taus])
    for k in range(J + 1):
        taus = [J % 2] if k == 0 else [0, 1]
        for v in range(N):
            cases.append((k, v, taus))
    ncase = len(cases)
    D = sum(len(c[2]) for c in cases)
    icontr2icase = np.empty(2 * D, np.int32)
    iroot = np.empty(D, np.int32)
    kk = np.empty(D, np.int32)
    ktau = np.empty(D, np.int32)
    Nsym = np.zeros(nrep * ncase, np.int32)
    root_sym = np.empty(D, np.int32)
    r = 0
    for ic, (k, v, taus) in enumerate(cases):
        for il, tau in enumerate(taus):
            icontr2icase[r] = ic
            icontr2icase[r + D] = il
            iroot[r] = v
            kk[r] = k
            ktau[r] = 2 * k + tau
            g = int(vib_sym[v]) ^ _c2v_rot_bits(k, tau)
            root_sym[r] = g
            Nsym[g + ic * nrep] += 1
            r += 1
    mat = 1 if J == 0 else 2
    Ntotal = np.array([int(Nsym[g::nrep].sum()) for g in range(nrep)], np.int32)
    repres = [np.zeros(max(int(Ntotal[g]), 1) * 1 * mat, np.float64) for g in range(nrep)]
    ptr = [0] * nrep
    r = 0
    for ic, (k, v, taus) in enumerate(cases):
        for il, tau in enumerate(taus):
            g = int(root_sym[r])
            s = ptr[g]
            ptr[g] += 1
            val = float(rng.choice([-1.0, 1.0])) if signs else 1.0
            repres[g][s + 0 * int(Ntotal[g]) + il * 1 * int(Ntotal[g])] = val
            r += 1
    return Basis(J, D, ncase, mat, mat, icontr2icase, iroot, kk, ktau, Nsym, Ntotal, repres)


# ---------------------------------------------------------------- C3v basis
def _random_orthogonal(rng: np.random.Generator, n: int) -> np.ndarray:
    q, r = np.linalg.qr(rng.standard_normal((n, n)))
    return q * np.sign(np.diag(r))[None, :]


def make_c3v_basis(J: int, vib_kind: List[int], rng: np.random.Generator) -> Basis:
    """Product basis for C3v(M): irreps A1=0, A2=1, E=2 (degen 2).

    vib_kind[v] gives the vibrational "class" of function v: 0 (A1), 1 (A2)
    or (2, comp) pairs for the two components of an E function (two
    consecutive J=0 indices).  Rotational factor per k: k=0 one function
    (A1 or A2 by J parity); k>0 with k%3==0 an A1+A2 pair; else an E pair.
    Each case (k, vib level) has lambda = (tau, vib component); its space is
    split into irreps by a random orthogonal matrix, as a symmetrisation
    (repres) would.
    """
    nrep, degen = 3, [1, 1, 2]
    # vibrational levels: list of lists of J=0 indices
    levels = []
    v = 0
    while v < len(vib_kind):
        if vib_kind[v] == 2:
            levels.append(("E", [v, v + 1]))
            v += 2
        else:
            levels.append(("A1" if vib_kind[v] == 0 else "A2", [v]))
            v += 1
    cases = []
    for k in range(J + 1):
        if k == 0:
            rot = ("A1" if J % 2 == 0 else "A2", [J % 2])
        elif k % 3 == 0:
            rot = ("A1A2", [0, 1])
        else:
            rot = ("E", [0, 1])
        for vk, vidx in levels:
            cases.append((k, rot, vk, vidx))

    def decompose(rk: str, vk: str) -> List[int]:
        # multiset of irreps in rot x vib (as irreps, E counted once)
        def irr(x):
            return {"A1": [0], "A2": [1], "E": [2], "A1A2": [0, 1]}[x]
        out = []
        for a in irr(rk):
            for b in irr(vk):
                if a == 2 and b == 2:
                    out += [0, 1, 2]
                elif a == 2 or b == 2:
                    out += [2]
                else:
                    out += [a ^ b]  # A1=0, A2=1 multiply by xor
        return out

    ncase = len(cases)
    rows_i2c, rows_lam, iroot, kk, ktau = [], [], [], [], []
    Nsym = np.zeros(nrep * ncase, np.int32)
    case_info = []
    for ic, (k, (rk, taus), vk, vidx) in enumerate(cases):
        lam = [(tau, vi) for tau in taus for vi in vidx]
        for il, (tau, vi) in enumerate(lam):
            rows_i2c.append(ic)
            rows_lam.append(il)
            iroot.append(vi)
            kk.append(k)
            ktau.append(2 * k + tau)
        irreps = decompose(rk, vk)
        assert sum(degen[g] for g in irreps) == len(lam)
        for g in irreps:
            Nsym[g + ic * nrep] += 1
        case_info.append((len(lam), irreps))
    D = len(iroot)
    mat = max(n for n, _ in case_info)
    Ntotal = np.array([int(Nsym[g::nrep].sum()) for g in range(nrep)], np.int32)
    repres = [np.zeros(max(int(Ntotal[g]), 1) * degen[g] * mat, np.float64) for g in range(nrep)]
    ptr = [0] * nrep
    for ic, (nl, irreps) in enumerate(case_info):
        Q = _random_orthogonal(rng, nl)  # rows: symmetrised components, cols: lambda
        row = 0
        # symmetrised functions of a case are stored per irrep in ascending g
        for g in range(nrep):
            cnt = Nsym[g + ic * nrep]
            for _ in range(cnt):
                s = ptr[g]
                ptr[g] += 1
                Nt = int(Ntotal[g])
                for d in range(degen[g]):
                    for il in range(nl):
                        repres[g][s + d * Nt + il * degen[g] * Nt] = Q[row, il]
                    row += 1
        assert row == nl
    icontr2icase = np.array(rows_i2c + rows_lam, np.int32)
    return Basis(J, D, ncase, mat, mat, icontr2icase, np.array(iroot, np.int32),
                 np.array(kk, np.int32), np.array(ktau, np.int32), Nsym, Ntotal, repres)


# ---------------------------------------------------------------- blocks
def make_block(rng: np.random.Generator, J: int, g: int, nsize: int, nmodes: int,
               nvec_max: Optional[int] = None, ecut: Optional[float] = None,
               emax: float = 20000.0, qr_limit: int = 20_000_000) -> Block:
    e = np.sort(rng.uniform(0.0, emax, size=nsize))
    if ecut is not None:
        e = e[e < ecut]
    nvec = len(e) if nvec_max is None else min(nvec_max, len(e))
    e = e[:nvec].copy()
    if nvec > 0 and nsize * nvec <= qr_limit:
        q, r = np.linalg.qr(rng.standard_normal((nsize, nvec)))
        vecs = np.ascontiguousarray((q * np.sign(np.diag(r))[None, :]).T)
    elif nvec > 0:
        # large blocks: unit Gaussian vectors (nearly orthogonal at these sizes;
        # a QR would take minutes and changes nothing the intensity path sees),
        # drawn in row bands by generators spawned from this block's seed, on
        # threads (numpy releases the GIL while it fills an array)
        vecs = np.empty((nvec, nsize))
        seeds = np.random.SeedSequence(int(rng.integers(1 << 62))).spawn(8)
        bands = np.array_split(np.arange(nvec), len(seeds))

        def fill(k):
            rows = bands[k]
            if len(rows):
                g = np.random.default_rng(seeds[k])
                g.standard_normal(out=vecs[rows[0]:rows[-1] + 1])
                vecs[rows[0]:rows[-1] + 1] /= np.linalg.norm(vecs[rows[0]:rows[-1] + 1], axis=1,
                                                             keepdims=True)

        with ThreadPoolExecutor(len(seeds)) as ex:
            list(ex.map(fill, range(len(seeds))))
    else:
        vecs = np.zeros((0, nsize))
    quanta = np.zeros((nvec, nmodes + 1), np.int32)
    quanta[:, 0] = rng.integers(0, 2 * J + 1, size=nvec)
    quanta[:, 1:] = rng.integers(0, 8, size=(nvec, nmodes))
    return Block(J, g, vecs, e, quanta)


def partition_function(blocks: Dict[Tuple[int, int], Block], gns, T: float, zpe: float) -> float:
    """Q = sum g_ns (2J+1) exp(-beta (E - ZPE)) over the supplied levels (FP64)."""
    planck, vellgt, boltz = 6.62606896e-27, 2.99792458e10, 1.380658e-16
    beta = planck * vellgt / (boltz * T)
    q = 0.0
    for (J, g), b in sorted(blocks.items()):
        q += gns[g] * (2 * J + 1) * float(np.sum(np.exp(-(b.energies - zpe) * beta)))
    return q


def make_c2v(seed: int, N: int, jlist: List[int], nvec_max: Optional[int] = None,
             ecut: Optional[float] = None, dipole: str = "decay", nsize_scale: float = 1.0,
             T: float = 296.0, zpe: float = 0.0, name: str = "") -> Problem:
    rng = np.random.default_rng(seed)
    mu = make_dipole(rng, N, dipole)
    vib = _c2v_vib_syms(rng, N)
    bases, blocks = {}, {}
    # nsize_scale < 1: the J > 0 bases use the lowest part of the J = 0
    # functions, as a contracted TROVE basis truncated by energy does
    M = max(1, int(round(N * nsize_scale)))
    for J in jlist:
        b = make_c2v_basis(J, vib if J == 0 else vib[:M], rng)
        bases[J] = b
        for g in range(4):
            nsize = int(b.Ntotal[g])
            blocks[(J, g)] = make_block(rng, J, g, nsize, 3, nvec_max, ecut)
    gns = (1.0, 1.0, 3.0, 3.0)
    p = Params(temperature=T, ZPE=zpe, gns=gns, isym_pairs=(1, 1, 2, 2), nmodes=3,
               freq_window=(0.0, 25000.0), erange_lower=(0.0, 20000.0),
               erange_upper=(0.0, 20000.0))
    p.q_stat = partition_function(blocks, gns, T, 0.0 if zpe < 0 else zpe)
    return Problem(SYM_C2V, N, mu, bases, blocks, p, name=name)


def make_c3v(seed: int, N: int, jlist: List[int], nvec_max: Optional[int] = None,
             ecut: Optional[float] = None, T: float = 500.0, reduced: bool = False,
             name: str = "") -> Problem:
    rng = np.random.default_rng(seed)
    mu = make_dipole(rng, N, "decay")
    kinds: List[int] = []
    while len(kinds) < N:
        x = rng.random()
        if x < 0.5 and len(kinds) + 2 <= N:
            kinds += [2, 2]
        elif x < 0.8:
            kinds.append(0)
        else:
            kinds.append(1)
    bases, blocks = {}, {}
    for J in jlist:
        b = make_c3v_basis(J, kinds, rng)
        bases[J] = b
        for g in range(3):
            blocks[(J, g)] = make_block(rng, J, g, int(b.Ntotal[g]), 6, nvec_max, ecut,
                                        emax=12000.0 * 4 / 3)
    gns = (2.0, 2.0, 2.0)
    # C3v(M) selection: A1 <-> A2, E <-> E
    p = Params(temperature=T, gns=gns, isym_pairs=(1, 1, 2), nmodes=6, reduced=reduced,
               freq_window=(0.0, 20000.0), erange_lower=(0.0, 12000.0),
               erange_upper=(0.0, 16000.0))
    p.q_stat = partition_function(blocks, gns, T, 0.0)
    return Problem(SYM_C3V, N, mu, bases, blocks, p, name=name)


# ---------------------------------------------------------------- named workloads
def workload(name: str, seed: int = 1, **kw) -> Problem:
    """Build one of the named workloads (sizes in the module docstring)."""
    if name == "c2v_small":
        kw.setdefault("N", 200)
        return make_c2v(seed, kw.pop("N"), kw.pop("jlist", [0, 1, 2]), name=name, **kw)
    if name == "c2v_plain":
        return make_c2v(seed, kw.pop("N", 2000), kw.pop("jlist", list(range(11))),
                        nvec_max=kw.pop("nvec_max", 1000), ecut=kw.pop("ecut", 15000.0),
                        name=name, **kw)
    if name == "c3v_small":
        return make_c3v(seed, kw.pop("N", 60), kw.pop("jlist", [0, 1, 2, 3]), name=name, **kw)
    if name == "c2v_precision":
        # one large pair J = 20 -> 21, Nvib = 5000, ~26k functions per Gamma,
        # 2000 vectors per block, dipole magnitudes log-uniform in [1e-8, 1]
        return make_c2v(seed, kw.pop("N", 5000), kw.pop("jlist", [20, 21]),
                        nvec_max=kw.pop("nvec_max", 2000), dipole="loguniform",
                        nsize_scale=kw.pop("nsize_scale", 0.5), name=name, **kw)
    if name == "c3v_batched":
        # tetratomic C3v, Nvib = 3000, blocks up to ~60k functions (J = 40),
        # up to 1500 vectors under 12000 cm^-1, T = 500 K; jlist selects J
        return make_c3v(seed, kw.pop("N", 3000), kw.pop("jlist", list(range(41))),
                        nvec_max=kw.pop("nvec_max", 1500), ecut=kw.pop("ecut", 12000.0),
                        name=name, **kw)
    raise KeyError(name)


# ---------------------------------------------------------------- serving
def serving_pool(prob: Problem, seed: int = 5, nvec_range: Tuple[float, float] = (100.0, 2000.0),
                 ecut: float = 12000.0) -> Problem:
    """The block pool of the serving workload: every (J, Gamma) block of a
    batched C3v problem's bases (the same dipole, bases and parameters), each
    with its own vector count drawn log-uniform in nvec_range (at most the
    levels under ecut), as unit Gaussian vectors."""
    rng = np.random.default_rng(seed)
    blocks = {}
    lo, hi = np.log(nvec_range[0]), np.log(nvec_range[1])
    for J in sorted(prob.bases):
        b = prob.bases[J]
        for g in range(len(b.Ntotal)):
            nmax = int(round(np.exp(rng.uniform(lo, hi))))
            blocks[(J, g)] = make_block(rng, J, g, int(b.Ntotal[g]), prob.params.nmodes, nmax,
                                        ecut, emax=ecut * 4 / 3, qr_limit=0)
    return Problem(prob.sym_type, prob.N, prob.mu, prob.bases, blocks, prob.params,
                   name=prob.name + "_serving_pool")


def serving_jobs(pool: Problem, seed: int = 6, njobs: int = 10000, rate: float = 200.0,
                 dims: Tuple[float, float] = (500.0, 80000.0)):
    """Pair jobs (J, Gamma) -> (J', Gamma') of the serving workload: the
    initial block's dimension drawn log-uniform in `dims` (the pool block of
    the nearest size), Gamma' its selection partner, J' uniform among the J-1,
    J, J+1 that carry lines; and Poisson inter-arrival gaps at `rate` jobs/s."""
    rng = np.random.default_rng(seed)
    keys = sorted(k for k, b in pool.blocks.items() if b.nvec > 0)
    logsz = np.log(np.array([pool.blocks[k].nsize for k in keys], dtype=np.float64))
    jmin = min(pool.jlist)
    jobs = []
    while len(jobs) < njobs:
        d = rng.uniform(np.log(dims[0]), np.log(dims[1]))
        J, g = keys[int(np.argmin(np.abs(logsz - d)))]
        gF = pool.partner(g)
        cands = [jF for jF in (J - 1, J, J + 1)
                 if (jF, gF) in pool.blocks and pool.blocks[(jF, gF)].nvec > 0 and J + jF >= 1
                 and not (J == jmin and jF == jmin)]
        if not cands:
            continue
        jobs.append((J, g, int(cands[rng.integers(len(cands))]), gF))
    gaps = rng.exponential(1.0 / rate, size=njobs)
    return jobs, gaps


# ---------------------------------------------------------------- persistence
def save(prob: Problem, path: str) -> None:
    """Write a Problem to one .npz file (no pickling)."""
    d = {"sym_type": prob.sym_type, "N": prob.N, "mu": prob.mu, "name": prob.name}
    p = prob.params
    for f in dataclasses.fields(Params):
        v = getattr(p, f.name)
        if v is not None:
            d["param_" + f.name] = np.asarray(v)
    for J, b in prob.bases.items():
        for f in dataclasses.fields(Basis):
            if f.name == "repres":
                for g, r in enumerate(b.repres):
                    d[f"basis{J}_repres{g}"] = r
            else:
                d[f"basis{J}_{f.name}"] = np.asarray(getattr(b, f.name))
    for (J, g), b in prob.blocks.items():
        d[f"block{J}_{g}_vecs"] = b.vecs
        d[f"block{J}_{g}_energies"] = b.energies
        d[f"block{J}_{g}_quanta"] = b.quanta
    np.savez_compressed(path, **d)


def load(path: str) -> Problem:
    z = np.load(path)
    sym = int(z["sym_type"])
    nrep = len(SYM_INFO[sym]["degen"])
    kw = {}
    for f in dataclasses.fields(Params):
        key = "param_" + f.name
        if key in z:
            v = z[key]
            kw[f.name] = (tuple(v.tolist()) if v.ndim == 1 else v) if v.ndim else v.item()
    params = Params(**kw)
    bases, blocks = {}, {}
    Js = sorted({int(k[5:].split("_")[0]) for k in z.files if k.startswith("basis")})
    for J in Js:
        vals = {}
        for f in dataclasses.fields(Basis):
            if f.name == "repres":
                vals["repres"] = [z[f"basis{J}_repres{g}"] for g in range(nrep)]
            else:
                a = z[f"basis{J}_{f.name}"]
                vals[f.name] = int(a) if a.ndim == 0 else a
        bases[J] = Basis(**vals)
    for k in z.files:
        if k.startswith("block") and k.endswith("_vecs"):
            J, g = map(int, k[5:-5].split("_"))
            blocks[(J, g)] = Block(J, g, z[k], z[f"block{J}_{g}_energies"],
                                   z[f"block{J}_{g}_quanta"])
    return Problem(sym, int(z["N"]), z["mu"], bases, blocks, params, name=str(z["name"]))


# ---------------------------------------------------------------- TROVE files
def _fortran_record(f, payload: bytes) -> None:
    n = np.int32(len(payload)).tobytes()
    f.write(n)
    f.write(payload)
    f.write(n)


def write_trove(prob: Problem, directory: str, thresh_linestrength: float = 0.0) -> str:
    """Write a Problem as the TROVE checkpoints the reference reads and return
    the matching input deck text.

    Files (formats as the reference's readers parse them): j0_extfield.chk
    (Fortran records, trove_functions.cpp:113-205), j0eigen_quanta<J>.chk
    (trove_functions.cpp:401-679), j0eigen_descr<J>_<G>.chk and
    j0eigen_vectors<J>_<G>.chk (trove_functions.cpp:1075-1429,
    cuda_host.cu:1196).  The contracted basis is written with one vibrational
    class: a case's class label is the J=0 case its roots correlate with and a
    lambda's label the J=0 lambda, so correlate_index recovers
    iroot_correlat_j0; every case is its own rotational level and
    rot_index(case, lambda) carries (J, k, tau) of that root.  Every level of a
    block is written once per degenerate component (records ndeg*i + ideg).
    """
    import os
    if 0 not in prob.bases:
        raise ValueError("a TROVE job needs the J=0 basis")
    os.makedirs(directory, exist_ok=True)
    info = SYM_INFO[prob.sym_type]
    degen, labels = info["degen"], info["labels"]
    nrep = len(degen)
    b0 = prob.bases[0]
    D0 = b0.Maxcontracts
    c0 = np.asarray(b0.icontr2icase[:D0])
    l0 = np.asarray(b0.icontr2icase[D0:])
    for J, b in sorted(prob.bases.items()):
        D = b.Maxcontracts
        cases = np.asarray(b.icontr2icase[:D])
        lams = np.asarray(b.icontr2icase[D:])
        ncase = b.Maxsymcoeffs
        ir = np.asarray(b.iroot_correlat_j0)
        vib_case = np.full(ncase, -1)
        lines = ["Start Primitive basis set",
                 f"{ncase:8d}{b.max_deg_size:8d}{D:8d}{1:8d}"]
        rot = []
        r = 0
        for c in range(ncase):
            roots = np.nonzero(cases == c)[0]
            if len(roots) == 0:
                raise ValueError(f"J={J}: case {c} has no roots")
            vc = set(int(c0[ir[x]]) for x in roots)
            if len(vc) != 1:
                raise ValueError(f"J={J}: case {c} correlates with several J=0 cases")
            vib_case[c] = vc.pop()
            lines.append(f"{len(roots):8d}{c + 1:6d}{vib_case[c] + 1:6d}")
            for x in roots:
                if x != r:
                    raise ValueError(f"J={J}: roots are not ordered by case and lambda")
                lam = int(lams[x])
                lines.append(f"{x + 1:8d}{lam + 1:6d}{int(l0[ir[x]]) + 1:6d}")
                rot.append((c, lam, int(b.k[x]), int(b.ktau[x]) & 1))
                r += 1
        lines.append(f"{ncase:8d}{b.max_deg_size:8d}")
        for c, lam, k, tau in rot:
            lines.append(f"{c + 1:8d}{lam + 1:8d}{J:8d}{k:8d}{tau:8d}")
        lines += ["End Primitive basis set", "Start irreducible transformation",
                  f"{b.mat_size:8d}", "".join(f"{int(n):8d}" for n in b.Ntotal)]
        Nsym = np.asarray(b.Nsym)
        for g in range(nrep):
            for c in range(ncase):
                lines.append(f"{int(Nsym[g + c * nrep]):8d}")
            nt, dg = int(b.Ntotal[g]), degen[g]
            rep = np.asarray(b.repres[g], np.float64)
            for s in range(nt):
                for d in range(dg):
                    lines.append(" ".join(repr(float(rep[s + d * nt + i * nt * dg]))
                                          for i in range(b.mat_size)))
        lines.append("End irreducible transformation")
        with open(os.path.join(directory, f"j0eigen_quanta{J}.chk"), "w") as f:
            f.write("\n".join(lines) + "\n")
    N = prob.N
    with open(os.path.join(directory, "j0_extfield.chk"), "wb") as f:
        _fortran_record(f, b"Start external field")
        _fortran_record(f, np.int32(N).tobytes())
        mu = np.asarray(prob.mu, np.float64).reshape(3, N * N)
        for c in range(3):
            _fortran_record(f, np.int32(c + 1).tobytes())
            _fortran_record(f, mu[c].tobytes())
        _fortran_record(f, b"End external field")
    nq = prob.params.nmodes + 1
    for (J, g), blk in sorted(prob.blocks.items()):
        dg = degen[g]
        lines = [f"fingerprint J={J} gamma={labels[g]}", "Start Quantum numbers and energies",
                 "   irec gamma ilevel ideg energy quanta", "",
                 f"{blk.nvec * dg:8d}{blk.nsize:8d}"]
        for i in range(blk.nvec):
            q = " ".join(str(int(x)) for x in blk.quanta[i, :nq])
            for ideg in range(1, dg + 1):
                lines.append(f"{i * dg + ideg:8d}{g + 1:4d}{i + 1:8d}{ideg:4d} "
                             f"{repr(float(blk.energies[i]))} {q} 1 {g + 1} {g + 1} {q}")
        lines.append("End Quantum numbers and energies")
        with open(os.path.join(directory, f"j0eigen_descr{J}_{g + 1}.chk"), "w") as f:
            f.write("\n".join(lines) + "\n")
        with open(os.path.join(directory, f"j0eigen_vectors{J}_{g + 1}.chk"), "wb") as f:
            v = np.ascontiguousarray(blk.vecs, np.float64)
            for i in range(blk.nvec):
                for _ in range(dg):
                    f.write(v[i].tobytes())
    p = prob.params
    js = sorted(prob.bases)
    ql, qu = p.windows()
    deck = [f"NMODES {p.nmodes}", f"SYMGROUP {info['name']}", "INTENSITY",
            f"  TEMPERATURE {p.temperature!r}", f"  QSTAT {p.q_stat!r}", f"  ZPE {p.ZPE!r}",
            f"  J {js[0]}, {js[-1]}",
            f"  FREQ-WINDOW {p.freq_window[0]!r} {p.freq_window[1]!r}",
            f"  ENERGY LOW {p.erange_lower[0]!r} {p.erange_lower[1]!r}, "
            f"UPPER {p.erange_upper[0]!r} {p.erange_upper[1]!r}",
            "  GNS " + " ".join(repr(float(x)) for x in p.gns[:nrep]),
            "  SELECTION (pairs) " + " ".join(str(int(x)) for x in p.isym_pairs[:nrep]),
            f"  THRESH_LINE {thresh_linestrength!r}"]
    for m in range(p.nmodes):
        deck.append(f"  V {m + 1} lower {int(ql[0][m])} {int(ql[1][m])} "
                    f"upper {int(qu[0][m])} {int(qu[1][m])}")
    if p.reduced:
        deck.append("  SYMMETRY REDUCED")
    deck.append("END")
    return "\n".join(deck) + "\n"
