"""Host-side mirror of the reference's stage-1 subroutines (koopro4QD.x).

Each function has the name, argument meaning and array layout of the Fortran
subroutine it replaces (numpy arrays in Fortran order with the reference's
shapes: state index first, ro4 state last) and runs on the GPU through the C
ABI.  Results the reference writes to nevpt.h5 are returned as arrays keyed
by their dataset names.
"""
from __future__ import annotations

import numpy as np

from ._native import Context, ptr

_ctx: Context | None = None


def context() -> Context:
    global _ctx
    if _ctx is None:
        _ctx = Context(0)
    return _ctx


FP64, SPLIT = 0, 1


class precision:
    """Context manager selecting the contraction precision of the shared
    context (nvpt_set_precision): ``with koopro.precision(koopro.SPLIT): ...``."""

    def __init__(self, mode: int, ctx: Context | None = None):
        self.mode, self.ctx = mode, ctx

    def __enter__(self):
        c = self.ctx or context()
        self.prev = int(c._lib.nvpt_get_precision(c.handle))
        c.call("nvpt_set_precision", self.mode)
        return c

    def __exit__(self, *exc):
        (self.ctx or context()).call("nvpt_set_precision", self.prev)
        return False


def _f(a) -> np.ndarray:
    a = np.asarray(a, dtype=np.float64)
    return a if a.flags.f_contiguous else np.asfortranarray(a)


def _z(*shape) -> np.ndarray:
    return np.zeros(shape, order="F")


def nwords(nact: int) -> int:
    return int(context()._lib.nvpt_nwords(nact))


def ord8(nact: int, tuples) -> tuple[np.ndarray, np.ndarray]:
    """src/ord_utils.F90:71 ord8 on the device for an (N,8) array of 1-based
    tuples; returns ((N,8) sorted key + partner, (N,) lindice)."""
    t = np.ascontiguousarray(tuples, dtype=np.int64).reshape(-1, 8)
    out = np.zeros_like(t)
    lind = np.zeros(t.shape[0], np.int64)
    context().call("nvpt_ord8", nact, t.shape[0], ptr(t), ptr(out), ptr(lind))
    return out, lind


def ord9(nact: int, tuples) -> tuple[np.ndarray, np.ndarray]:
    """src/ord_utils.F90:16 ord9 on the device (same conventions as ord8)."""
    t = np.ascontiguousarray(tuples, dtype=np.int64).reshape(-1, 8)
    out = np.zeros_like(t)
    lind = np.zeros(t.shape[0], np.int64)
    context().call("nvpt_ord9", nact, t.shape[0], ptr(t), ptr(out), ptr(lind))
    return out, lind


def bro3(ro4, nact: int, nele: int, metat: int) -> np.ndarray:
    """src/koopro4QD.F90:4881 bro3 -> daaa(metat, n^6)."""
    out = _z(metat, *(nact,) * 6)
    context().call("nvpt_bro3", ptr(_f(ro4)), ptr(out), nact, nele, metat)
    return out


def bro2(daaa, nact: int, nele: int, metat: int) -> np.ndarray:
    out = _z(metat, *(nact,) * 4)
    context().call("nvpt_bro2", ptr(_f(daaa)), ptr(out), nact, nele, metat)
    return out


def bro1(taa, nact: int, nele: int, metat: int) -> np.ndarray:
    out = _z(metat, nact, nact)
    context().call("nvpt_bro1", ptr(_f(taa)), ptr(out), nact, nele, metat)
    return out


def get_aj_atwo(nact: int, ncore: int, norb: int, oneint, cholesky_array):
    """src/koopro4QD.F90:3900 get_aj_atwo on the Cholesky integral path."""
    atwo = _z(nact, nact, nact, nact)
    aj = np.zeros(norb * (norb + 1) // 2)
    L = _f(cholesky_array)
    context().call("nvpt_get_aj_atwo", ptr(atwo), nact, ncore, norb, ptr(aj), ptr(_f(oneint)), ptr(L), L.shape[0])
    return atwo, aj


def koop_matrices_ctl(metat: int, nact: int, ncore: int, atwo, daaa, taa, dal, f, aj, ctx: Context | None = None) -> dict:
    """src/koop_matrices.F90:16 koop_matrices_ctl.  ``f`` is updated in place.
    On a context with symmetry tables (SymmetryIntegrals) koop2E's irrep
    screen applies."""
    n, M = nact, metat
    out = {"1-IPKO": _z(M, n, n), "1-EAKO": _z(M, n, n), "2-HRDM": _z(M, n, n, n, n), "2-IPKO": _z(M, n, n, n, n),
           "2-EAKO": _z(M, n, n, n, n), "gk0pa": _z(M, n, n, n, n), "gk0pd": _z(M, n, n, n, n), "gk0pf": _z(M, n, n)}
    (ctx or context()).call("nvpt_koop_matrices_ctl", M, n, ncore, ptr(_f(atwo)), ptr(_f(daaa)), ptr(_f(taa)), ptr(_f(dal)),
                   ptr(f), ptr(_f(aj)), *[ptr(out[k]) for k in ("1-IPKO", "1-EAKO", "2-HRDM", "2-IPKO", "2-EAKO",
                                                               "gk0pa", "gk0pd", "gk0pf")])
    return out


def bamat(atwo, ro4, daaa, taa, dal, nact: int, ncore: int, f, aj, norb: int, metat: int, nsym: int = 1,
          ctx: Context | None = None):
    """src/koopro4QD.F90:3974 bamat -> (amat "amatIP", atmat "amatEA").
    nsym > 1 (the symmetry-screened branch) needs a context with the
    matching symmetry tables (SymmetryIntegrals.ctx)."""
    amat, atmat = _z(metat, *(nact,) * 6), _z(metat, *(nact,) * 6)
    (ctx or context()).call("nvpt_bamat", ptr(amat), ptr(atmat), ptr(_f(atwo)), ptr(_f(ro4)), ptr(_f(daaa)), ptr(_f(taa)),
                   ptr(_f(dal)), nact, ncore, ptr(f), ptr(_f(aj)), norb, metat, nsym)
    return amat, atmat


def bbmat(atwo, daaa, taa, dal, nact: int, ncore: int, f, aj, metat: int):
    b, bt = _z(metat, *(nact,) * 4), _z(metat, *(nact,) * 4)
    context().call("nvpt_bbmat", ptr(_f(atwo)), ptr(b), ptr(bt), ptr(_f(daaa)), ptr(_f(taa)), ptr(_f(dal)), nact,
                   ncore, ptr(f), ptr(_f(aj)), metat)
    return b, bt


def bcmat(atwo, daaa, taa, dal, nact: int, ncore: int, f, aj, metat: int):
    c, ct = _z(metat, *(nact,) * 4), _z(metat, *(nact,) * 4)
    context().call("nvpt_bcmat", ptr(_f(atwo)), ptr(c), ptr(ct), ptr(_f(daaa)), ptr(_f(taa)), ptr(_f(dal)), nact,
                   ncore, ptr(f), ptr(_f(aj)), metat)
    return c, ct


def bdmat(atwo, taa, dal, nact: int, ncore: int, f, aj, metat: int):
    d, dt = _z(metat, nact, nact), _z(metat, nact, nact)
    context().call("nvpt_bdmat", ptr(_f(atwo)), ptr(d), ptr(dt), ptr(_f(taa)), ptr(_f(dal)), nact, ncore, ptr(f),
                   ptr(_f(aj)), metat)
    return d, dt


class SymmetryIntegrals:
    """The non-Cholesky integral path with point-group symmetry
    (src/ijkl_utils.F90:209-262 readint): the irrep and addressing tables of
    initialize_infsym / determine_n2int / reijkl, built on the device by
    ``nvpt_ijkl_init`` for the inactive/active/secondary counts per irrep,
    and the symmetry-packed integral list ``twoint`` resident with them."""

    KEYS = ("its", "itsym", "num", "indic", "jndic", "ndeb", "nad", "kt")

    def __init__(self, nish, nash, nssh, ctx: Context | None = None):
        # a context of its own unless one is given: the tables are that
        # context's integral state and switch on the symmetry screens of
        # koop_matrices_ctl and bamat on it
        self.ctx = ctx or Context(0)
        self.nsym = len(nish)
        c = [np.ascontiguousarray(x, dtype=np.int64) for x in (nish, nash, nssh)]
        ni4 = np.zeros(1, np.int64)
        self.ctx.call("nvpt_ijkl_init", self.nsym, ptr(c[0]), ptr(c[1]), ptr(c[2]), ptr(ni4))
        self.ni4 = int(ni4[0])
        self.norb = int(sum(int(x.sum()) for x in c))

    def tables(self) -> dict:
        ns, no = self.nsym, self.norb
        npair, nj = no * (no + 1) // 2, ns * (ns + 1) // 2
        t = {"its": np.zeros((ns, ns), np.int64, order="F"), "itsym": np.zeros(no, np.int64),
             "num": np.zeros(npair, np.int64), "indic": np.zeros(npair, np.int64),
             "jndic": np.zeros(npair, np.int64), "ndeb": np.zeros(ns, np.int64), "nad": np.zeros(nj, np.int64),
             "kt": np.zeros(nj, np.int64)}
        self.ctx.call("nvpt_ijkl_tables", *[ptr(t[k]) for k in self.KEYS])
        t["ni4"] = self.ni4
        return t

    def set_twoint(self, twoint) -> None:
        tw = np.ascontiguousarray(twoint, dtype=np.float64)
        if tw.size != self.ni4:
            raise ValueError(f"twoint must hold ni4 = {self.ni4} integrals")
        self.ctx.call("nvpt_ijkl_set_twoint", ptr(tw))

    def ai(self, ijkl) -> np.ndarray:
        """src/ijkl_utils.F90:690 ai_twoint for an (N,4) array of 1-based indices."""
        q = np.ascontiguousarray(ijkl, dtype=np.int64).reshape(-1, 4)
        out = np.zeros(q.shape[0])
        self.ctx.call("nvpt_ai_twoint", q.shape[0], ptr(q), ptr(out))
        return out

    def get_aj_atwo(self, nact: int, ncore: int, oneint):
        """src/koopro4QD.F90:3900 get_aj_atwo on this integral path."""
        atwo = _z(nact, nact, nact, nact)
        aj = np.zeros(self.norb * (self.norb + 1) // 2)
        self.ctx.call("nvpt_get_aj_atwo_twoint", ptr(atwo), nact, ncore, self.norb, ptr(aj), ptr(_f(oneint)))
        return atwo, aj


def koopro4QD(problem) -> dict:
    """Stage 1 of one problem, in the reference driver's order
    (src/koopro4QD.F90:270-423): bro3/bro2/bro1 from the packed 4-RDM,
    get_aj_atwo, koop_matrices_ctl, bamat, bbmat, bcmat, bdmat."""
    p = problem
    n, M, nc, norb = p.nact, p.metat, p.ncore, p.norb
    daaa = bro3(p.ro4, n, p.nele, M)
    taa = bro2(daaa, n, p.nele, M)
    dal = bro1(taa, n, p.nele, M)
    atwo, aj = get_aj_atwo(n, nc, norb, p.oneint, p.chol)
    f = np.zeros(norb * (norb + 1) // 2)
    out = koop_matrices_ctl(M, n, nc, atwo, daaa, taa, dal, f, aj)
    out.update({"3-RDM": daaa, "2-RDM": taa, "1-RDM": dal, "atwo": atwo, "aj": aj})
    out["amatIP"], out["amatEA"] = bamat(atwo, p.ro4, daaa, taa, dal, n, nc, f, aj, norb, M)
    out["bmatIP"], out["bmatEA"] = bbmat(atwo, daaa, taa, dal, n, nc, f, aj, M)
    out["cmatIP"], out["cmatEA"] = bcmat(atwo, daaa, taa, dal, n, nc, f, aj, M)
    out["dmatIP"], out["dmatEA"] = bdmat(atwo, taa, dal, n, nc, f, aj, M)
    return out


def permute_4rdm(ro4, labels, values):
    """src/rdm_utils.F90:236 permute_4rdm over a QCMaquis label/value list
    (as hdf5_read_rdm_from_resfile applies it): ``ro4`` (W,n,n,n,n) of one
    state, Fortran order, updated in place; ``labels`` (nentries, 8) 0-based."""
    n = ro4.shape[1]
    lab = np.ascontiguousarray(labels, dtype=np.int32)
    val = np.ascontiguousarray(values, dtype=np.float64)
    if not ro4.flags.f_contiguous:
        raise ValueError("ro4 must be Fortran-contiguous")
    context().call("nvpt_permute_4rdm", ptr(ro4), n, ptr(lab), ptr(val), val.size)
    return ro4


def permute_3rdm(rdm3, labels, values, trans: bool = False, state: int = 0):
    """src/rdm_utils.F90:470 permute_3rdm into ``rdm3`` -- (M,n,n,n,n,n,n)
    Fortran order (state ``state``) or (n,)*6 -- in place; ``labels``
    (nentries, 6) 0-based."""
    if not rdm3.flags.f_contiguous:
        raise ValueError("rdm3 must be Fortran-contiguous")
    if rdm3.ndim == 7:
        ld, n = rdm3.shape[0], rdm3.shape[1]
        flat = rdm3.reshape(-1, order="F")
        base = flat[state:]
    else:
        ld, n = 1, rdm3.shape[0]
        base = rdm3.reshape(-1, order="F")
    lab = np.ascontiguousarray(labels, dtype=np.int32)
    val = np.ascontiguousarray(values, dtype=np.float64)
    # the host entry stages ld * n^6 elements from the pointer: hand it a
    # buffer of exactly that extent
    tmp = np.zeros(ld * n**6)
    tmp[: base.size] = base
    context().call("nvpt_permute_3rdm", ptr(tmp), ld, n, ptr(lab), ptr(val), val.size, int(trans))
    base[:] = tmp[: base.size]
    return rdm3

