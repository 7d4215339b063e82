"""ctypes front end of the CPU oracle (oracle/nvpt2_oracle.c).

TEST INFRASTRUCTURE ONLY: the oracle the CUDA library is compared against,
and the scalar CPU baseline of the benchmark.  Arrays use the reference's
Fortran shapes in numpy Fortran order (state first; ro4 state last).
"""
from __future__ import annotations

import ctypes
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"
_lib = None
I64 = ctypes.c_int64


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < (HERE / "nvpt2_oracle.c").stat().st_mtime:
            build()
        L = ctypes.CDLL(str(LIB_PATH))
        P = ctypes.c_void_p
        L.orc_nwords.argtypes = [I64]; L.orc_nwords.restype = I64
        L.orc_index_tables.argtypes = [I64, P, P, P, P]
        L.orc_ord.argtypes = [I64, ctypes.c_int, I64, P, P]
        L.orc_bro3.argtypes = [P, P, I64, I64, I64]
        L.orc_bro2.argtypes = [P, P, I64, I64, I64]
        L.orc_bro1.argtypes = [P, P, I64, I64, I64]
        L.orc_ai.argtypes = [P, I64, I64, I64, I64, I64]; L.orc_ai.restype = ctypes.c_double
        L.orc_get_aj_atwo.argtypes = [P, P, I64, I64, I64, I64, P, P]
        L.orc_koop_matrices_ctl.argtypes = [I64, I64, I64] + [P] * 14
        L.orc_permute_4rdm.argtypes = [P, I64, P, P, I64]; L.orc_permute_4rdm.restype = ctypes.c_int
        L.orc_permute_3rdm.argtypes = [P, I64, I64, P, P, I64, ctypes.c_int]
        L.orc_permute_3rdm.restype = ctypes.c_int
        L.orc_fdiff_F.argtypes = [P, I64, I64, P]
        L.orc_bamat.argtypes = [P] * 7 + [I64, I64, P, P, I64, I64]
        L.orc_bamat_slabs.argtypes = [P] * 7 + [I64, I64, P, P, I64, I64]
        L.orc_koop_matrices_ctl_sym.argtypes = [I64, I64, I64] + [P] * 15
        L.orc_bamat_sym.argtypes = [P] * 7 + [I64, I64, P, P, I64, P]
        L.orc_bro3_touched.argtypes = [I64]
        L.orc_bro3_touched.restype = I64
        L.orc_bamat_slab_list.argtypes = [P] * 7 + [I64, I64, P, P, I64, P, I64]
        L.orc_bbmat.argtypes = [P] * 6 + [I64, I64, P, P, I64]
        L.orc_bcmat.argtypes = [P] * 6 + [I64, I64, P, P, I64]
        L.orc_bdmat.argtypes = [P] * 5 + [I64, I64, P, P, I64]
        L.orc_fdiff.argtypes = [P, P, P, P, I64, I64, P]
        L.orc_eeee_at.argtypes = [P, P, P, P, I64, I64, P, I64]; L.orc_eeee_at.restype = ctypes.c_double
        L.orc_eee2_at.argtypes = [P, P, P, I64, I64, P, I64]; L.orc_eee2_at.restype = ctypes.c_double
        L.orc_num_threads.restype = ctypes.c_int
        L.orc_ijkl_tables.argtypes = [I64, P, P, P, I64] + [P] * 8
        L.orc_ijkl_tables.restype = I64
        L.orc_ai_twoint_list.argtypes = [P] * 7 + [I64, P, P]
        L.orc_get_aj_atwo_twoint.argtypes = [P] * 8 + [I64, I64, I64, P, P]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def _chk(a, dtype=np.float64):
    assert a.dtype == dtype and (a.flags.f_contiguous or a.ndim <= 1), "expected Fortran-ordered array"
    return a


def zeros(*shape):
    return np.zeros(shape, order="F")


def nwords(n):
    return int(lib().orc_nwords(n))


def index_tables(n):
    lindi, lindj, lindk = (np.zeros(n, np.int64) for _ in range(3))
    normind = np.zeros((n,) * 4, np.int64, order="F")
    lib().orc_index_tables(n, _p(lindi), _p(lindj), _p(lindk), _p(normind))
    return lindi, lindj, lindk, normind


def ord_tuples(n, which, tuples):
    t = np.ascontiguousarray(tuples, dtype=np.int64)
    out = np.zeros_like(t)
    lib().orc_ord(n, which, t.shape[0], _p(t), _p(out))
    return out


def bro3(ro4, nact, nele, metat):
    out = zeros(metat, *(nact,) * 6)
    lib().orc_bro3(_p(_chk(ro4)), _p(out), nact, nele, metat)
    return out


def bro3_touched(nact):
    """Distinct packed 4-RDM entries bro3 reads per state."""
    return int(lib().orc_bro3_touched(nact))


def bro2(daaa, nact, nele, metat):
    out = zeros(metat, *(nact,) * 4)
    lib().orc_bro2(_p(_chk(daaa)), _p(out), nact, nele, metat)
    return out


def bro1(taa, nact, nele, metat):
    out = zeros(metat, nact, nact)
    lib().orc_bro1(_p(_chk(taa)), _p(out), nact, nele, metat)
    return out


def get_aj_atwo(oneint, chol, nact, ncore, norb):
    atwo = zeros(nact, nact, nact, nact)
    aj = np.zeros(norb * (norb + 1) // 2)
    lib().orc_get_aj_atwo(_p(oneint), _p(_chk(chol)), chol.shape[0], nact, ncore, norb, _p(atwo), _p(aj))
    return atwo, aj


def koop_matrices_ctl(metat, nact, ncore, atwo, daaa, taa, dal, f, aj):
    n, M = nact, metat
    out = dict(ipko1=zeros(M, n, n), eako1=zeros(M, n, n), hrdm2=zeros(M, n, n, n, n), ipko2=zeros(M, n, n, n, n),
               eako2=zeros(M, n, n, n, n), gk0pa=zeros(M, n, n, n, n), gk0pd=zeros(M, n, n, n, n),
               gk0pf=zeros(M, n, n))
    lib().orc_koop_matrices_ctl(M, n, ncore, _p(atwo), _p(daaa), _p(taa), _p(dal), _p(f), _p(aj),
                                *[_p(out[k]) for k in ("ipko1", "eako1", "hrdm2", "ipko2", "eako2", "gk0pa",
                                                       "gk0pd", "gk0pf")])
    return out


def koop_matrices_ctl_sym(metat, nact, ncore, atwo, daaa, taa, dal, f, aj, asym):
    """koop_matrices_ctl with the its() screen of koop2E (koop_matrices.F90:289-351);
    asym = irreps (1-based) of the active orbitals."""
    n, M = nact, metat
    out = dict(ipko1=zeros(M, n, n), eako1=zeros(M, n, n), hrdm2=zeros(M, n, n, n, n), ipko2=zeros(M, n, n, n, n),
               eako2=zeros(M, n, n, n, n), gk0pa=zeros(M, n, n, n, n), gk0pd=zeros(M, n, n, n, n),
               gk0pf=zeros(M, n, n))
    sy = np.ascontiguousarray(asym, dtype=np.int64)
    lib().orc_koop_matrices_ctl_sym(M, n, ncore, _p(atwo), _p(daaa), _p(taa), _p(dal), _p(f), _p(aj),
                                    *[_p(out[k]) for k in ("ipko1", "eako1", "hrdm2", "ipko2", "eako2", "gk0pa",
                                                           "gk0pd", "gk0pf")], _p(sy))
    return out


def bamat_sym(atwo, ro4, daaa, taa, dal, nact, ncore, f, aj, metat, asym):
    """The symmetry-screened bamat branch (koopro4QD.F90:4105-4228)."""
    amat, atmat = zeros(metat, *(nact,) * 6), zeros(metat, *(nact,) * 6)
    sy = np.ascontiguousarray(asym, dtype=np.int64)
    lib().orc_bamat_sym(_p(amat), _p(atmat), _p(atwo), _p(ro4), _p(daaa), _p(taa), _p(dal), nact, ncore, _p(f),
                        _p(aj), metat, _p(sy))
    return amat, atmat


def fdiff_F(gk0pf, nact, metat):
    out = np.zeros(metat)
    lib().orc_fdiff_F(_p(gk0pf), nact, metat, _p(out))
    return out


def bamat(atwo, ro4, daaa, taa, dal, nact, ncore, f, aj, norb, metat):
    amat, atmat = zeros(metat, *(nact,) * 6), zeros(metat, *(nact,) * 6)
    lib().orc_bamat(_p(amat), _p(atmat), _p(atwo), _p(ro4), _p(daaa), _p(taa), _p(dal), nact, ncore, _p(f), _p(aj),
                    norb, metat)
    return amat, atmat


def bamat_slabs(atwo, ro4, daaa, taa, dal, nact, ncore, f, aj, metat, nslab):
    amat, atmat = zeros(metat, *(nact,) * 6), zeros(metat, *(nact,) * 6)
    lib().orc_bamat_slabs(_p(amat), _p(atmat), _p(atwo), _p(ro4), _p(daaa), _p(taa), _p(dal), nact, ncore, _p(f),
                          _p(aj), metat, nslab)
    return amat, atmat


def bamat_slab_list(atwo, ro4, daaa, taa, dal, nact, ncore, f, aj, metat, slabs):
    """amat/atmat whose elements (s, ap, *, cp, a, *, c) are exact for the
    0-based slabs (a-1) n + (c-1) listed; other elements are zero."""
    amat, atmat = zeros(metat, *(nact,) * 6), zeros(metat, *(nact,) * 6)
    sl = np.ascontiguousarray(slabs, dtype=np.int64)
    lib().orc_bamat_slab_list(_p(amat), _p(atmat), _p(atwo), _p(ro4), _p(daaa), _p(taa), _p(dal), nact, ncore,
                              _p(f), _p(aj), metat, _p(sl), sl.size)
    return amat, atmat


def slab_mask(nact, slabs):
    """Boolean mask over (ap,bp,cp,a,b,c) (Fortran order, no state index) of
    the elements the listed slabs determine."""
    n = nact
    m = np.zeros((n,) * 6, dtype=bool, order="F")
    for sl in slabs:
        a, c = divmod(int(sl), n)
        m[:, :, :, a, :, c] = True
    return m


def bbmat(atwo, daaa, taa, dal, nact, ncore, f, aj, metat):
    b, bt = zeros(metat, *(nact,) * 4), zeros(metat, *(nact,) * 4)
    lib().orc_bbmat(_p(atwo), _p(b), _p(bt), _p(daaa), _p(taa), _p(dal), nact, ncore, _p(f), _p(aj), metat)
    return b, bt


def bcmat(atwo, daaa, taa, dal, nact, ncore, f, aj, metat):
    c, ct = zeros(metat, *(nact,) * 4), zeros(metat, *(nact,) * 4)
    lib().orc_bcmat(_p(atwo), _p(c), _p(ct), _p(daaa), _p(taa), _p(dal), nact, ncore, _p(f), _p(aj), metat)
    return c, ct


def bdmat(atwo, taa, dal, nact, ncore, f, aj, metat):
    d, dt = zeros(metat, nact, nact), zeros(metat, nact, nact)
    lib().orc_bdmat(_p(atwo), _p(d), _p(dt), _p(taa), _p(dal), nact, ncore, _p(f), _p(aj), metat)
    return d, dt


def fdiff(bmat, cmat, btmat, ctmat, nact, metat):
    out = np.zeros(2 * metat)
    lib().orc_fdiff(_p(bmat), _p(cmat), _p(btmat), _p(ctmat), nact, metat, _p(out))
    return out[:metat], out[metat:]


def eeee_at(ro4, daaa, taa, dal, nact, metat, idx8, s):
    i = np.ascontiguousarray(idx8, np.int64)
    return lib().orc_eeee_at(_p(ro4), _p(daaa), _p(taa), _p(dal), nact, metat, _p(i), s)


def eee2_at(daaa, taa, dal, nact, metat, idx6, s):
    i = np.ascontiguousarray(idx6, np.int64)
    return lib().orc_eee2_at(_p(daaa), _p(taa), _p(dal), nact, metat, _p(i), s)


def num_threads():
    return int(lib().orc_num_threads())


def stage1(problem):
    """Full oracle stage 1 of one problem; returns a dict of every dataset."""
    p = problem
    n, M, nc, norb = p.nact, p.metat, p.ncore, p.norb
    atwo, aj = get_aj_atwo(p.oneint, p.chol, n, nc, norb)
    f = np.zeros(norb * (norb + 1) // 2)
    out = koop_matrices_ctl(M, n, nc, atwo, p.daaa, p.taa, p.dal, f, aj)
    out["atwo"], out["aj"] = atwo, aj
    if p.ro4 is not None:
        out["amatIP"], out["amatEA"] = bamat(atwo, p.ro4, p.daaa, p.taa, p.dal, n, nc, f, aj, norb, M)
    out["bmatIP"], out["bmatEA"] = bbmat(atwo, p.daaa, p.taa, p.dal, n, nc, f, aj, M)
    out["cmatIP"], out["cmatEA"] = bcmat(atwo, p.daaa, p.taa, p.dal, n, nc, f, aj, M)
    out["dmatIP"], out["dmatEA"] = bdmat(atwo, p.taa, p.dal, n, nc, f, aj, M)
    return out


def permute_4rdm(ro4, labels, values):
    """rdm_utils.F90:236 permute_4rdm over a label list, sequentially (C)."""
    lab = np.ascontiguousarray(labels, dtype=np.int32)
    val = np.ascontiguousarray(values, dtype=np.float64)
    assert ro4.flags.f_contiguous
    bad = lib().orc_permute_4rdm(_p(ro4), ro4.shape[1], _p(lab), _p(val), val.size)
    return ro4, bad


def permute_3rdm(flat, ld, n, labels, values, trans=False):
    """rdm_utils.F90:470 permute_3rdm into a flat buffer with element stride ld."""
    lab = np.ascontiguousarray(labels, dtype=np.int32)
    val = np.ascontiguousarray(values, dtype=np.float64)
    bad = lib().orc_permute_3rdm(_p(flat), ld, n, _p(lab), _p(val), val.size, int(trans))
    return flat, bad



# ---------------------------------------------------------------------------
# Symmetry-packed two-electron integrals (infsym.F90, ijkl_utils.F90)

def ijkl_tables(nish, nash, nssh):
    """initialize_infsym + reijkl + determine_n2int: dict of the int64 tables
    (1-based values) and ni4."""
    nsym = len(nish)
    norb = int(sum(nish) + sum(nash) + sum(nssh))
    npair = norb * (norb + 1) // 2
    c = [np.ascontiguousarray(x, dtype=np.int64) for x in (nish, nash, nssh)]
    t = {"its": np.zeros((nsym, nsym), np.int64, order="F"), "itsym": np.zeros(norb, np.int64),
         "num": np.zeros(npair, np.int64), "indic": np.zeros(npair, np.int64), "jndic": np.zeros(npair, np.int64),
         "ndeb": np.zeros(nsym, np.int64), "nad": np.zeros(nsym * (nsym + 1) // 2, np.int64),
         "kt": np.zeros(nsym * (nsym + 1) // 2, np.int64)}
    ni4 = lib().orc_ijkl_tables(nsym, _p(c[0]), _p(c[1]), _p(c[2]), norb,
                                *[_p(t[k]) for k in ("its", "itsym", "num", "indic", "jndic", "ndeb", "nad", "kt")])
    t["ni4"] = int(ni4)
    return t


def _tab_ptrs(t, twoint):
    return [_p(t[k]) for k in ("num", "indic", "jndic", "ndeb", "nad", "kt")] + [_p(twoint)]


def ai_twoint(t, twoint, ijkl):
    q = np.ascontiguousarray(ijkl, dtype=np.int64).reshape(-1, 4)
    out = np.zeros(q.shape[0])
    lib().orc_ai_twoint_list(*_tab_ptrs(t, twoint), q.shape[0], _p(q), _p(out))
    return out


def get_aj_atwo_twoint(t, twoint, oneint, nact, ncore, norb):
    atwo = zeros(nact, nact, nact, nact)
    aj = np.zeros(norb * (norb + 1) // 2)
    lib().orc_get_aj_atwo_twoint(*_tab_ptrs(t, twoint), _p(np.ascontiguousarray(oneint)), nact, ncore, norb,
                                 _p(atwo), _p(aj))
    return atwo, aj


def pack_twoint(t, chol):
    """twoint in the reference's layout from a Cholesky/DF array whose
    vectors respect the symmetry ((ij|kl) = sum_Q L[Q,ij] L[Q,kl] vanishes
    unless indic(ij) == indic(kl)): per pair irrep r, the lower triangle of
    the Gram matrix of its pairs (ranked by jndic), row by row, at ndeb(r)."""
    L = np.asarray(chol)
    tw = np.zeros(t["ni4"])
    for r in range(1, len(t["ndeb"]) + 1):
        pairs = np.nonzero(t["indic"] == r)[0]
        pairs = pairs[np.argsort(t["jndic"][pairs])]
        if pairs.size == 0:
            continue
        G = L[:, pairs].T @ L[:, pairs]
        a, b = np.tril_indices(pairs.size)
        tw[t["ndeb"][r - 1] + a * (a + 1) // 2 + b] = G[a, b]
    return tw


def symmetric_chol(itsym, nchovec, rng):
    """A DF array L(Q, norb(norb+1)/2) with one irrep per vector: L[Q, pq] is
    nonzero only when irrep(p) x irrep(q) equals vector Q's irrep (values
    N(0, (0.05 exp(-|p-q|/8))^2) like the C1 generator)."""
    itsym = np.asarray(itsym)
    norb = itsym.size
    nsym = int(itsym.max())
    gq = rng.integers(0, nsym, nchovec)
    L = np.zeros((nchovec, norb * (norb + 1) // 2), order="F")
    col = 0
    for p in range(norb):
        for q in range(p + 1):
            sd = 0.05 * np.exp(-abs(p - q) / 8.0)
            pr = (itsym[p] - 1) ^ (itsym[q] - 1)
            L[:, col] = np.where(gq == pr, rng.standard_normal(nchovec) * sd, 0.0)
            col += 1
    return L
