"""Host-side mirror of the reference's stage 2 (QDnevpt2.x): the per-state
SC/PC-NEVPT2 loop of src/qdnevpt.F:858-993 on the GPU through
``nvpt_qdnevpt``, plus the metat x metat effective-Hamiltonian step of
:1010-1230 (dgeev, ascending sort, and the Hermitisation of
hermitian_heff, :8089-8183) on the host.

Inputs use the nevpt.h5 dataset names and the reference's array shapes in
numpy Fortran order (state index first).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from ._native import Context, ptr
from .koopro import context

CLASSES = ["(0)", "(+1)", "(-1)", "(+2)", "(-2)", "(+1)'", "(-1)'", "(0)'"]
P = ctypes.c_void_p
I64 = ctypes.c_int64


class _In(ctypes.Structure):
    _fields_ = [("ncore", I64), ("nact", I64), ("nvirt", I64), ("metat", I64), ("nchovec", I64),
                ("thr_lindep", ctypes.c_double), ("no_pc", I64), ("class_mask", I64), ("frozen", P),
                ("oneint", P), ("cholesky_array", P), ("rdm1", P), ("rdm2", P), ("rdm3", P), ("hrdm2", P),
                ("ipko1", P), ("eako1", P), ("ipko2", P), ("eako2", P), ("gk0pa", P), ("gk0pd", P), ("gk0pf", P),
                ("amat_ip", P), ("amat_ea", P), ("bmat_ip", P), ("bmat_ea", P), ("cmat_ip", P), ("cmat_ea", P),
                ("dmat_ip", P), ("dmat_ea", P), ("trdm1", P), ("trdm2", P), ("trdm3", P)]


class _Out(ctypes.Structure):
    _fields_ = [("e2mpp", P), ("psimpp", P), ("e2enp", P), ("psienep", P), ("e2mp", P), ("e2en", P),
                ("psimp", P), ("psien", P), ("epsnew", P), ("nnew", P), ("rhoir", P), ("rhoid", P), ("rhodr", P)]


@dataclass
class Stage2Energies:
    e2mpp: np.ndarray
    psimpp: np.ndarray
    e2enp: np.ndarray
    psienep: np.ndarray
    e2mp: np.ndarray
    e2en: np.ndarray
    psimp: np.ndarray
    psien: np.ndarray
    epsnew: np.ndarray
    nnew: np.ndarray
    # first-order density blocks (rho1st=True): (ncore,nvirt,M), (ncore,nact,M), (nact,nvirt,M)
    rhoir: np.ndarray | None = None
    rhoid: np.ndarray | None = None
    rhodr: np.ndarray | None = None


_BOUND = False


def _bind(ctx: Context):
    global _BOUND
    if not _BOUND:
        for name in ("nvpt_qdnevpt",):
            fn = getattr(ctx._lib, name)
            fn.argtypes = [P, ctypes.POINTER(_In), ctypes.POINTER(_Out)]
            fn.restype = ctypes.c_int
        fn = ctx._lib.nvpt_qdnevpt_d
        fn.argtypes = [P, ctypes.POINTER(_In), ctypes.POINTER(_Out), P]
        fn.restype = ctypes.c_int
        _BOUND = True


def _f(a):
    if a is None:
        return None
    a = np.asarray(a, dtype=np.float64)
    return a if a.flags.f_contiguous else np.asfortranarray(a)


def qdnevpt(problem, koop: dict, transition=None, thr_lindep: float = 1e-6, class_mask: int = 0xFF,
            no_pc: bool = False, frozen=None, rho1st: bool = False) -> Stage2Energies:
    """Per-state loop of src/qdnevpt.F:858-993 on the GPU.  ``koop`` holds
    the stage-1 datasets by their nevpt.h5 names; ``transition`` the
    (1-TRDM, 2-TRDM, 3-TRDM) arrays when metat > 1; ``rho1st`` (.NATORB)
    also returns the first-order density blocks of the PC classes."""
    ctx = context()
    _bind(ctx)
    p = problem
    M, n = p.metat, p.nact
    if transition is None and M > 1:
        transition = getattr(p, "trdm", None)
    keep = []

    def h(a):
        a = _f(a)
        keep.append(a)
        return ptr(a)

    g = lambda k: h(koop[k])
    fr = None
    if frozen is not None:
        fm = np.zeros(p.norb, np.uint8)
        fm[list(frozen)] = 1
        keep.append(fm)
        fr = ptr(fm)
    inp = _In(p.ncore, n, p.nvirt, M, p.chol.shape[0], thr_lindep, int(no_pc), class_mask, fr, h(p.oneint),
              h(p.chol), g("1-RDM"), g("2-RDM"), g("3-RDM"), g("2-HRDM"), g("1-IPKO"), g("1-EAKO"), g("2-IPKO"),
              g("2-EAKO"), g("gk0pa"), g("gk0pd"), g("gk0pf"), g("amatIP"), g("amatEA"), g("bmatIP"), g("bmatEA"),
              g("cmatIP"), g("cmatEA"), g("dmatIP"), g("dmatEA"),
              *(h(t) for t in (transition if transition is not None else (None, None, None))))
    res = Stage2Energies(*(np.zeros((8, M), order="F") for _ in range(4)), np.zeros((M, M), order="F"),
                         np.zeros((M, M), order="F"), np.zeros(M), np.zeros(M), np.zeros((p.norb, M), order="F"),
                         np.zeros((10, M), np.int64, order="F"))
    if rho1st:
        nc, nv = p.ncore, p.nvirt
        res.rhoir = np.zeros((nc, nv, M), order="F")
        res.rhoid = np.zeros((nc, n, M), order="F")
        res.rhodr = np.zeros((n, nv, M), order="F")
    names = ("e2mpp", "psimpp", "e2enp", "psienep", "e2mp", "e2en", "psimp", "psien", "epsnew", "nnew", "rhoir",
             "rhoid", "rhodr")
    out = _Out(*(ptr(getattr(res, k)) for k in names))
    ctx.check(ctx._lib.nvpt_qdnevpt(ctx.handle, ctypes.byref(inp), ctypes.byref(out)), "nvpt_qdnevpt")
    return res


def natural_orbitals(res: Stage2Energies, dal, ncore: int, nact: int, nvirt: int):
    """src/qdnevpt.F:1240-1411 (.NATORB) on the host: each state's density in
    the canonical orbitals (2 on the inactive diagonal, the 1-RDM on the
    active block, the PC classes' first-order blocks off the diagonal,
    symmetric) and its natural occupation numbers (dsyev, then the
    reference's order_eigvalvec, :1484: descending magnitude, a later value of
    equal magnitude first).  Returns (rho (norb, norb, M), occupations (norb, M))."""
    if res.rhoir is None:
        raise ValueError("run qdnevpt(..., rho1st=True) first")
    M = res.rhoir.shape[2]
    norb = ncore + nact + nvirt
    c, a, v = slice(0, ncore), slice(ncore, ncore + nact), slice(ncore + nact, norb)
    rho = np.zeros((norb, norb, M))
    occ = np.zeros((norb, M))
    for s in range(M):
        R = rho[:, :, s]
        R[a, a] = np.asarray(dal)[s]
        R[np.arange(ncore), np.arange(ncore)] = 2.0
        for blk, rs, cs in ((res.rhoir, c, v), (res.rhodr, a, v), (res.rhoid, c, a)):
            R[rs, cs] = blk[:, :, s]
            R[cs, rs] = blk[:, :, s].T
        w = np.linalg.eigvalsh(np.tril(R) + np.tril(R, -1).T)
        for i in range(norb - 1):
            imin = i
            for j in range(i + 1, norb):
                if abs(w[j]) >= abs(w[imin]):
                    imin = j
            w[i], w[imin] = w[imin], w[i]
        occ[:, s] = w
    return rho, occ


@dataclass
class EffectiveHamiltonian:
    """What src/qdnevpt.F:1046-1126 and hermitian_heff (:8089-8183) leave
    behind for one of SC or PC.

    heff       Heff = e2 + diag(E), the non-Hermitian matrix given to dgeev
    wr, wi     its eigenvalues (real, imaginary parts), ascending in wr
    vr, vl     right / left eigenvectors in dgeev's real storage, same order
    heff_herm  the Hermitised Heff~ = C' diag(wr) C'^T with C' = vr S^-1/2 and
               S = vr^T vr (the reference copies it back over e2mp / e2en)
    evc_herm   eigenvectors of Heff~ (dsyev('V','U'), columns)
    w_herm     eigenvalues of Heff~, ascending (stored in psimp / psien)
    For one state (skip_effective_ham, src/qdnevpt.F:192) nothing is
    diagonalised: heff_herm = heff, w_herm = its diagonal."""
    heff: np.ndarray
    wr: np.ndarray
    wi: np.ndarray
    vr: np.ndarray
    vl: np.ndarray
    heff_herm: np.ndarray
    evc_herm: np.ndarray
    w_herm: np.ndarray


def _exchange_sort(wr, wi, vr, vl):
    """The reference's reordering after dgeev (src/qdnevpt.F:1069-1089):
    for i < j, swap eigenpairs i and j whenever wr(j) < wr(i)."""
    wr, wi, vr, vl = wr.copy(), wi.copy(), vr.copy(), vl.copy()
    m = wr.size
    for i in range(m):
        for j in range(i + 1, m):
            if wr[j] < wr[i]:
                wr[[i, j]] = wr[[j, i]]
                wi[[i, j]] = wi[[j, i]]
                vr[:, [i, j]] = vr[:, [j, i]]
                vl[:, [i, j]] = vl[:, [j, i]]
    return wr, wi, vr, vl


def hermitian_heff(vr: np.ndarray, wr: np.ndarray):
    """src/qdnevpt.F:8089-8183 (eq. 19 of JCP 121, 4043 (2004)): the
    similarity transform that makes Heff Hermitian.  S = vr^T vr; S^-1/2 from
    the eigenpairs of S (rtmatinv, :8305-8345); C' = vr S^-1/2;
    Heff~ = C' diag(wr) C'^T; then Heff~ is diagonalised (dsyev('V','U')).
    Returns (Heff~, its eigenvectors, its eigenvalues)."""
    vr = np.asarray(vr, dtype=np.float64)
    S = vr.T @ vr
    ev, G = np.linalg.eigh(S, UPLO="U")
    S_mhalf = (G / np.sqrt(ev)[None, :]) @ G.T
    Cp = vr @ S_mhalf
    H = (Cp * np.asarray(wr, dtype=np.float64)[None, :]) @ Cp.T
    w, evc = np.linalg.eigh(H, UPLO="U")
    return H, evc, w


def effective_hamiltonian(e2: np.ndarray, energies: np.ndarray) -> EffectiveHamiltonian:
    """src/qdnevpt.F:1046-1126 for one of SC (e2mp) or PC (e2en): add the
    reference energies to the diagonal, diagonalise the non-Hermitian Heff
    with LAPACK dgeev (left and right eigenvectors), reorder ascending by the
    real parts as the reference does, and Hermitise (hermitian_heff)."""
    from scipy.linalg import lapack

    H = np.array(e2, dtype=np.float64) + np.diag(np.asarray(energies, dtype=np.float64))
    m = H.shape[0]
    if m == 1:
        one = np.ones((1, 1))
        return EffectiveHamiltonian(H, H.diagonal().copy(), np.zeros(1), one, one.copy(), H.copy(), one.copy(),
                                    H.diagonal().copy())
    wr, wi, vl, vr, info = lapack.dgeev(np.asfortranarray(H), compute_vl=1, compute_vr=1)
    if info != 0:
        raise RuntimeError(f"dgeev failed (info={info})")
    wr, wi, vr, vl = _exchange_sort(wr, wi, vr, vl)
    Hh, evc, w = hermitian_heff(vr, wr)
    return EffectiveHamiltonian(H, wr, wi, vr, vl, Hh, evc, w)
