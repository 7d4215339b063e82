"""Seeded synthetic NEVPT2 problems with the shapes and value distributions of
the benchmark configurations.

A problem is: a CAS(n) determinant expansion with Gaussian coefficients
(orthonormalised across roots), its exact spin-free 1-4-RDMs in the
reference's layouts (``ro4`` packed as in src/indices_norm.F90 / ord8), and
density-fitted integrals ``(pq|rs) = sum_Q B[Q,pq] B[Q,rs]`` stored as the
reference's Cholesky array ``cholesky_array(Q, norb(norb+1)/2)``
(src/ijkl_utils.F90:637-688), with ``B ~ N(0, (0.05 exp(-|p-q|/8))^2)``
symmetric in pq.  The one-electron integrals are chosen so that the core and
virtual Fock operators rebuilt by the NEVPT2 stage (src/qdnevpt.F:369-698)
equal a target Fock matrix whose diagonal holds sorted uniform orbital
energies (inactive [-2,-0.5], active [-0.5,0.5], virtual [0.5,5]) and whose
off-diagonal elements are normal with standard deviation 1e-3, symmetric:
``h1 = F_target - G_core - G_act[gamma_1 of root 1]``.

The RDMs come from the in-tree OpenMP generator ``librdmgen.so``.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
_LIB = None


def _rdmgen():
    global _LIB
    if _LIB is None:
        path = _PKG / "librdmgen.so"
        if not path.exists():
            from . import build
            build.build_rdmgen()
        lib = ctypes.CDLL(str(path))
        u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
        f64p = ctypes.POINTER(ctypes.c_double)
        lib.rdmgen_dense.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_long, u32p, u32p, f64p, ctypes.c_int,
                                     ctypes.c_int, f64p, ctypes.c_long, ctypes.c_long]
        lib.rdmgen_dense.restype = ctypes.c_int
        lib.rdmgen_ro4.argtypes = [ctypes.c_int, ctypes.c_long, u32p, u32p, f64p, ctypes.c_int, f64p]
        lib.rdmgen_ro4.restype = ctypes.c_int
        _LIB = lib
    return _LIB


def _dptr(a: np.ndarray, offset: int = 0):
    return ctypes.cast(a.ctypes.data + 8 * offset, ctypes.POINTER(ctypes.c_double))


def nwords(n: int) -> int:
    return n * (n + 1) * (n + 2) * (n + 3) // 24


def npair(norb: int) -> int:
    return norb * (norb + 1) // 2


def tri(i: int, j: int) -> int:
    """1-based lower-triangle index indice(i,j) of the reference."""
    mx, mn = max(i, j), min(i, j)
    return mx * (mx - 1) // 2 + mn


def strings(n: int, k: int) -> np.ndarray:
    """All n-bit masks with k bits set, in colex (= numeric) order."""
    out = [m for m in range(1 << n) if bin(m).count("1") == k]
    return np.array(out, dtype=np.uint32)


@dataclass
class Problem:
    nact: int
    nele: int
    ncore: int
    nvirt: int
    metat: int
    nchovec: int
    seed: int
    amask: np.ndarray
    bmask: np.ndarray
    coef: np.ndarray          # (ndet, metat) Fortran order
    dal: np.ndarray           # (M,n,n)
    taa: np.ndarray           # (M,n,n,n,n)
    daaa: np.ndarray          # (M,n^6)
    ro4: np.ndarray | None    # (W,n,n,n,n,M)
    oneint: np.ndarray        # (norb(norb+1)/2,)
    chol: np.ndarray          # (Q, npair) Fortran order
    eps: np.ndarray           # target orbital energies (norb,)
    energies: np.ndarray = field(default_factory=lambda: np.zeros(1))
    # transition 1-3-RDMs (daoff, daaoff, ro3off) of every root pair, metat > 1
    trdm: tuple | None = None

    @property
    def norb(self) -> int:
        return self.ncore + self.nact + self.nvirt

    @property
    def ndet(self) -> int:
        return int(self.amask.size)

    @property
    def nwords(self) -> int:
        return nwords(self.nact)


def _dets(n: int, na: int, nb: int, ndet: int | None, rng: np.random.Generator):
    sa, sb = strings(n, na), strings(n, nb)
    full = sa.size * sb.size
    if ndet is None or ndet >= full:
        idx = np.arange(full, dtype=np.int64)
    else:
        idx = np.sort(rng.choice(full, size=ndet, replace=False).astype(np.int64))
    return sa[idx // sb.size].copy(), sb[idx % sb.size].copy()


def _chol(norb: int, Q: int, rng: np.random.Generator) -> np.ndarray:
    """cholesky_array(Q, npair): column indice(p,q) holds B[:, p, q]."""
    P = npair(norb)
    L = np.empty((Q, P), order="F")
    col = 0
    for p in range(1, norb + 1):
        q = np.arange(1, p + 1)
        sd = 0.05 * np.exp(-np.abs(p - q) / 8.0)
        L[:, col:col + p] = rng.standard_normal((Q, p)) * sd[None, :]
        col += p
    return L


def _dense_B(L: np.ndarray, norb: int, rows: slice) -> np.ndarray:
    """Dense B[Q-chunk, p, q] from the packed columns."""
    Lc = L[rows, :]
    B = np.empty((Lc.shape[0], norb, norb))
    col = 0
    for p in range(norb):
        B[:, p, : p + 1] = Lc[:, col:col + p + 1]
        B[:, : p + 1, p] = Lc[:, col:col + p + 1]
        col += p + 1
    return B


def fock_two_electron(L: np.ndarray, norb: int, ncore: int, nact: int, gamma1: np.ndarray) -> np.ndarray:
    """G_core + G_act of the reference's core/virtual Fock operators:
    sum_k [2(pq|kk) - (pk|kq)] + sum_ab g_ba [(pq|ab) - 1/2 (pb|aq)]."""
    Q = L.shape[0]
    G = np.zeros((norb, norb))
    act = slice(ncore, ncore + nact)
    for q0 in range(0, Q, 64):
        B = _dense_B(L, norb, slice(q0, min(Q, q0 + 64)))
        x = B.shape[0]
        Jc = np.einsum("xkk->x", B[:, :ncore, :ncore])
        # gamma1[a,b] = <E_ab>; the reference multiplies (pq|ab) by da(b,a)
        Ja = np.einsum("xab,ba->x", B[:, act, act], gamma1)
        # Coulomb parts: sum_x B[x] (2 Jc[x] + Ja[x]) as one matrix-vector product
        G += ((2.0 * Jc + Ja) @ B.reshape(x, norb * norb)).reshape(norb, norb)
        # exchange parts as batched GEMMs: sum_x B[x][:, k] B[x][k, :] and B[x][:, act] gamma1 B[x][act, :]
        Bk = np.ascontiguousarray(B[:, :, :ncore])
        G -= np.matmul(Bk, np.ascontiguousarray(B[:, :ncore, :])).sum(axis=0)
        Bg = np.matmul(np.ascontiguousarray(B[:, :, act]), gamma1)
        G -= 0.5 * np.matmul(Bg, np.ascontiguousarray(B[:, act, :])).sum(axis=0)
    return G


def make_problem(nact: int, nele: int, ncore: int, nvirt: int, metat: int = 1, ndet: int | None = None,
                 seed: int = 20261203, nchovec: int | None = None, with_ro4: bool = True,
                 with_trdm: bool = False) -> Problem:
    """Build one seeded problem.  ``ndet=None`` takes the full CAS space."""
    if nact > 16:
        raise ValueError("nact <= 16")
    rng = np.random.Generator(np.random.PCG64(seed))
    na = nele - nele // 2
    nb = nele // 2
    amask, bmask = _dets(nact, na, nb, ndet, rng)
    nd = amask.size
    C = rng.standard_normal((nd, metat))
    Qm, _ = np.linalg.qr(C)
    coef = np.asfortranarray(Qm[:, :metat] * np.sign(np.diag(_)[:metat])[None, :])
    n = nact
    dal, taa, daaa, ro4 = rdms(n, amask, bmask, coef, with_ro4)
    norb = ncore + nact + nvirt
    Q = nchovec if nchovec is not None else 4 * norb
    chol = _chol(norb, Q, rng)
    eps = np.concatenate([np.sort(rng.uniform(-2.0, -0.5, ncore)), np.sort(rng.uniform(-0.5, 0.5, nact)),
                          np.sort(rng.uniform(0.5, 5.0, nvirt))])
    off = rng.normal(0.0, 1e-3, (norb, norb))
    F = np.diag(eps) + np.triu(off, 1) + np.triu(off, 1).T
    G = fock_two_electron(chol, norb, ncore, nact, dal[0])
    h1 = F - G
    oneint = np.array([h1[p, q] for p in range(norb) for q in range(p + 1)])
    trdm = transition_rdms(n, amask, bmask, coef) if (with_trdm and metat > 1) else None
    return Problem(nact=n, nele=nele, ncore=ncore, nvirt=nvirt, metat=metat, nchovec=Q, seed=seed, amask=amask,
                   bmask=bmask, coef=coef, dal=dal, taa=taa, daaa=daaa, ro4=ro4, oneint=oneint, chol=chol, eps=eps,
                   energies=np.zeros(metat), trdm=trdm)


def rdms(n: int, amask, bmask, coef, with_ro4: bool = True):
    """Exact (dal, taa, daaa, ro4) of every root of a CI expansion."""
    lib = _rdmgen()
    coef = np.asfortranarray(coef, dtype=np.float64)
    nd, metat = coef.shape
    amask = np.ascontiguousarray(amask, dtype=np.uint32)
    bmask = np.ascontiguousarray(bmask, dtype=np.uint32)
    dal = np.zeros((metat,) + (n,) * 2, order="F")
    taa = np.zeros((metat,) + (n,) * 4, order="F")
    daaa = np.zeros((metat,) + (n,) * 6, order="F")
    for s in range(metat):
        for k, arr in ((1, dal), (2, taa), (3, daaa)):
            if lib.rdmgen_dense(n, k, nd, amask, bmask, _dptr(coef), s, s, _dptr(arr), metat, s):
                raise RuntimeError("rdmgen_dense failed")
    ro4 = None
    if with_ro4:
        W = nwords(n)
        ro4 = np.zeros((W,) + (n,) * 4 + (metat,), order="F")
        for s in range(metat):
            if lib.rdmgen_ro4(n, nd, amask, bmask, _dptr(coef), s, _dptr(ro4, W * n**4 * s)):
                raise RuntimeError("rdmgen_ro4 failed")
    return dal, taa, daaa, ro4


def rdms_device(n: int, amask, bmask, coef, with_ro4: bool = True, transition: bool = False, ctx=None,
                device: str = "cuda:0"):
    """The outputs of ``rdms`` (and, with transition=True, of
    ``transition_rdms`` as a fifth item) computed on the GPU by the library's
    RDM builder (nvpt_rdm_dense_d / nvpt_rofour_d), returned as host arrays."""
    import torch

    from ._native import Context, ptr
    ctx = ctx or Context(torch.device(device).index or 0)
    dev = torch.device(device)
    coef = np.asfortranarray(coef, dtype=np.float64)
    nd, M = coef.shape
    am = torch.from_numpy(np.ascontiguousarray(amask, dtype=np.uint32).view(np.int32)).to(dev)
    bm = torch.from_numpy(np.ascontiguousarray(bmask, dtype=np.uint32).view(np.int32)).to(dev)
    cf = torch.from_numpy(coef.ravel(order="F").copy()).to(dev)
    z = lambda k: torch.zeros(k, dtype=torch.float64, device=dev)
    outs = [z(M * n ** (2 * k)) for k in (1, 2, 3)]
    for s in range(M):
        for k, o in zip((1, 2, 3), outs):
            ctx.call("nvpt_rdm_dense_d", n, k, nd, ptr(am), ptr(bm), ptr(cf), M, s, s, ptr(o), M, s, None)
    ro4 = None
    W = nwords(n)
    if with_ro4:
        r4 = z(W * n**4 * M)
        for s in range(M):
            ctx.call("nvpt_rofour_d", n, nd, ptr(am), ptr(bm), ptr(cf), M, s, ctypes.c_void_p(r4.data_ptr() + 8 * W * n**4 * s),
                     None)
    tr = None
    if transition and M > 1:
        P = M * (M - 1) // 2
        tr_d = [z(P * n ** (2 * k)) for k in (1, 2, 3)]
        for big in range(M):
            for small in range(big):
                kp = big * (big - 1) // 2 + small
                for k, o in zip((1, 2, 3), tr_d):
                    ctx.call("nvpt_rdm_dense_d", n, k, nd, ptr(am), ptr(bm), ptr(cf), M, small, big, ptr(o), P, kp,
                             None)
    ctx.synchronize()
    host = lambda t, shape: t.cpu().numpy().reshape(shape, order="F")
    dal, taa, daaa = (host(o, (M,) + (n,) * (2 * k)) for k, o in zip((1, 2, 3), outs))
    if with_ro4:
        ro4 = host(r4, (W,) + (n,) * 4 + (M,))
    if transition and M > 1:
        P = M * (M - 1) // 2
        tr = [host(o, (P,) + (n,) * (2 * k)) for k, o in zip((1, 2, 3), tr_d)]
    return (dal, taa, daaa, ro4, tr) if transition else (dal, taa, daaa, ro4)


def transition_rdms(n: int, amask, bmask, coef):
    """Transition 1-3-RDMs for every root pair (big > small), stored at pair
    index big*(big-1)/2 + small (the reference's iroot > jroot loop,
    src/koopro4QD.F90:433) with bra = the smaller root:
    daoff[k,i,j] = <Psi_small| E_ij |Psi_big>, and likewise for 2 and 3."""
    lib = _rdmgen()
    coef = np.asfortranarray(coef, dtype=np.float64)
    nd, metat = coef.shape
    P = metat * (metat - 1) // 2
    amask = np.ascontiguousarray(amask, dtype=np.uint32)
    bmask = np.ascontiguousarray(bmask, dtype=np.uint32)
    out = [np.zeros((P,) + (n,) * (2 * k), order="F") for k in (1, 2, 3)]
    for big in range(metat):
        for small in range(big):
            kpair = big * (big - 1) // 2 + small
            for k, arr in zip((1, 2, 3), out):
                if lib.rdmgen_dense(n, k, nd, amask, bmask, _dptr(coef), small, big, _dptr(arr), P, kpair):
                    raise RuntimeError("rdmgen_dense failed")
    return out


def with_ci(p: Problem, amask, bmask, coef) -> Problem:
    """Same integrals, different CI expansion (RDMs recomputed)."""
    dal, taa, daaa, ro4 = rdms(p.nact, amask, bmask, coef, with_ro4=p.ro4 is not None)
    coef = np.asfortranarray(coef)
    return Problem(nact=p.nact, nele=p.nele, ncore=p.ncore, nvirt=p.nvirt, metat=coef.shape[1], nchovec=p.nchovec,
                   seed=p.seed, amask=np.asarray(amask, np.uint32), bmask=np.asarray(bmask, np.uint32), coef=coef,
                   dal=dal, taa=taa, daaa=daaa, ro4=ro4, oneint=p.oneint, chol=p.chol, eps=p.eps,
                   energies=np.zeros(coef.shape[1]))


# Benchmark configurations: (nact, nele, ncore, nvirt, metat, ndet)
CONFIGS = {
    "cas8": dict(nact=8, nele=8, ncore=10, nvirt=40, metat=1, ndet=None, seed=20261203 + 1),
    "cas14": dict(nact=14, nele=14, ncore=20, nvirt=150, metat=1, ndet=50_000, seed=20261203 + 2),
    # a mid-size case for single-kernel profiler captures (slab buffers above L2, a few GB in all)
    "cas10": dict(nact=10, nele=10, ncore=10, nvirt=40, metat=1, ndet=20_000, seed=20261203 + 10),
    "cas16_qd4": dict(nact=16, nele=16, ncore=30, nvirt=250, metat=4, ndet=100_000, seed=20261203 + 5),
}


def config_problem(name: str, **over) -> Problem:
    kw = dict(CONFIGS[name])
    kw.setdefault("with_trdm", kw["metat"] > 1)
    kw.update(over)
    return make_problem(**kw)


BATCH_SEED = 20261203 * 100


def batch_problems(count: int = 64, seed: int = BATCH_SEED, first: int = 0):
    """The batched configuration: ``count`` independent problems, problem p
    seeded with seed + p: active size uniform in {6, 8, 10, 12} at half
    filling, 3 roots, inactive orbitals uniform in [5, 20], virtual orbitals
    uniform in [30, 120], the full CAS space when it has at most 20,000
    determinants (else 20,000 drawn uniformly: within the configuration's
    bound of 100,000, and it keeps the host-side generator of 64 problems
    within minutes), transition RDMs of the 3 root pairs."""
    out = []
    for pid in range(first, first + count):
        r = np.random.default_rng(seed + pid)
        n = int(r.choice([6, 8, 10, 12]))
        nc = int(r.integers(5, 21))
        nv = int(r.integers(30, 121))
        full = math.comb(n, n // 2) ** 2
        out.append(make_problem(n, n, nc, nv, metat=3, ndet=None if full <= 20_000 else 20_000, seed=seed + pid,
                                with_trdm=True))
    return out


def orbital_irreps(nish, nash, nssh) -> np.ndarray:
    """itsym of src/infsym.F90:38-69: irrep (1-based) of every orbital,
    inactive irrep by irrep, then active, then secondary."""
    out = []
    for cnt in (nish, nash, nssh):
        for r, k in enumerate(cnt):
            out += [r + 1] * int(k)
    return np.array(out, dtype=np.int64)


def symmetric_chol(itsym, nchovec: int, rng: np.random.Generator) -> np.ndarray:
    """DF vectors that respect point-group symmetry: vector Q carries one
    irrep and L[Q, pq] vanishes unless irrep(p) x irrep(q) is that irrep, so
    (pq|rs) vanishes unless irrep(pq) = irrep(rs)."""
    itsym = np.asarray(itsym)
    norb = itsym.size
    gq = rng.integers(0, int(itsym.max()), nchovec)
    L = np.zeros((nchovec, npair(norb)), order="F")
    col = 0
    for p in range(norb):
        for q in range(p + 1):
            sd = 0.05 * np.exp(-abs(p - q) / 8.0)
            L[:, col] = np.where(gq == ((itsym[p] - 1) ^ (itsym[q] - 1)), rng.standard_normal(nchovec) * sd, 0.0)
            col += 1
    return L


def make_sym_problem(nish, nash, nssh, nele: int, metat: int = 1, ndet: int | None = None, seed: int = 7,
                     irrep: int = 1) -> Problem:
    """A problem with point-group symmetry: determinants of one total irrep
    (product of the irreps of every occupied active spin orbital), so the
    RDMs vanish exactly where symmetry forbids them; symmetric DF integrals
    and a one-electron operator coupling only orbitals of equal irrep.
    Problem.chol holds the DF vectors (the twoint list is built from them)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    itsym = orbital_irreps(nish, nash, nssh)
    ncore, nact = int(sum(nish)), int(sum(nash))
    nvirt = itsym.size - ncore - nact
    asym = itsym[ncore:ncore + nact] - 1
    na, nb = nele - nele // 2, nele // 2

    def irr(mask):
        g = 0
        for k in range(nact):
            if mask >> k & 1:
                g ^= int(asym[k])
        return g

    sa, sb = strings(nact, na), strings(nact, nb)
    ga = np.array([irr(int(m)) for m in sa]), np.array([irr(int(m)) for m in sb])
    pairs = [(i, j) for i in range(sa.size) for j in range(sb.size) if (ga[0][i] ^ ga[1][j]) == irrep - 1]
    if ndet is not None and ndet < len(pairs):
        pick = np.sort(rng.choice(len(pairs), size=ndet, replace=False))
        pairs = [pairs[k] for k in pick]
    amask = np.array([sa[i] for i, _ in pairs], dtype=np.uint32)
    bmask = np.array([sb[j] for _, j in pairs], dtype=np.uint32)
    C = rng.standard_normal((amask.size, metat))
    Qm, R = np.linalg.qr(C)
    coef = np.asfortranarray(Qm[:, :metat] * np.sign(np.diag(R)[:metat])[None, :])
    dal, taa, daaa, ro4 = rdms(nact, amask, bmask, coef, True)
    norb = itsym.size
    chol = symmetric_chol(itsym, 4 * norb, rng)
    eps = np.concatenate([np.sort(rng.uniform(-2.0, -0.5, ncore)), np.sort(rng.uniform(-0.5, 0.5, nact)),
                          np.sort(rng.uniform(0.5, 5.0, nvirt))])
    off = rng.normal(0.0, 1e-3, (norb, norb)) * (itsym[:, None] == itsym[None, :])
    F = np.diag(eps) + np.triu(off, 1) + np.triu(off, 1).T
    h1 = F - fock_two_electron(chol, norb, ncore, nact, dal[0])
    oneint = np.array([h1[p, q] for p in range(norb) for q in range(p + 1)])
    return Problem(nact=nact, nele=nele, ncore=ncore, nvirt=nvirt, metat=metat, nchovec=chol.shape[0], seed=seed,
                   amask=amask, bmask=bmask, coef=coef, dal=dal, taa=taa, daaa=daaa, ro4=ro4, oneint=oneint,
                   chol=chol, eps=eps, energies=np.zeros(metat))
