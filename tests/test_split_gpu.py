"""Split-precision (Ozaki digits on tcgen05) products against FP64.

Bounds follow the scheme: every product x*a carries an error below
2^-60 * 2^(E_i + F_j), E_i / F_j the row / column exponents (at most twice the
row / column maximum), so a K-term dot product is within K * 2^-58 *
max|X_i| * max|A_j|.  The energy criterion is the path's: split-mode NEVPT2
energies within 1e-7 Eh of FP64, per class and in total.
"""
import numpy as np
import pytest

from nevpt2_gb300 import koopro, synth
from nevpt2_gb300._native import NvptError, ptr

pytestmark = pytest.mark.gpu


def _split_gemm(A, B):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    m, k = A.shape
    n = B.shape[1]
    tA = torch.from_numpy(np.ascontiguousarray(A)).to(dev)
    tB = torch.from_numpy(np.ascontiguousarray(B)).to(dev)
    tC = torch.full((m, n), float("nan"), dtype=torch.float64, device=dev)
    ctx = koopro.context()
    ctx.call("nvpt_dgemm_split_d", m, n, k, ptr(tA), ptr(tB), ptr(tC), None)
    ctx.synchronize()
    return tC.cpu().numpy()


def _bound(A, B):
    """Split error bound plus the rounding of the FP64 reference A @ B itself
    (|fl(A B) - A B| <= K u |A| |B|)."""
    k = A.shape[1]
    split = k * 2.0**-58 * np.abs(A).max(axis=1)[:, None] * np.abs(B).max(axis=0)[None, :]
    return split + k * 2.0**-53 * (np.abs(A) @ np.abs(B))


@pytest.mark.parametrize("m,k,n", [(128, 16, 16), (300, 100, 14), (1000, 2744, 14), (257, 4096, 16), (5, 33, 1)])
def test_split_gemm_within_ozaki_bound(m, k, n):
    rng = np.random.default_rng(m * 7 + k)
    A = rng.standard_normal((m, k))
    B = rng.standard_normal((k, n)) * 0.05
    C = _split_gemm(A, B)
    ref = A @ B
    assert np.isfinite(C).all()
    err = np.abs(C - ref)
    assert (err <= _bound(A, B)).all()
    # typical error is far below the worst-case bound
    assert err.max() <= 1e-14 * np.abs(ref).max()


def test_split_gemm_exact_on_small_integers():
    rng = np.random.default_rng(5)
    A = rng.integers(-63, 64, (256, 512)).astype(np.float64)
    B = rng.integers(-63, 64, (512, 16)).astype(np.float64)
    assert np.array_equal(_split_gemm(A, B), A @ B)


def test_split_gemm_mixed_row_scales_and_zero_rows():
    rng = np.random.default_rng(9)
    A = rng.standard_normal((384, 700)) * (10.0 ** rng.uniform(-8, 3, 384))[:, None]
    A[17] = 0.0
    A[200, :350] = 0.0
    B = rng.standard_normal((700, 12))
    C = _split_gemm(A, B)
    ref = A @ B
    assert (np.abs(C - ref) <= _bound(A, B)).all()
    assert (C[17] == 0.0).all()


def test_split_gemm_rejects_out_of_range_shapes():
    ctx = koopro.context()
    with pytest.raises(NvptError) as e:
        ctx.call("nvpt_dgemm_split_d", 4, 17, 8, None, None, None, None)
    assert e.value.status == 1
    x = np.zeros(1)
    with pytest.raises(NvptError):
        ctx.call("nvpt_dgemm_split_d", 4, 16, 4097, ptr(x), ptr(x), ptr(x), None)


@pytest.mark.parametrize("n,ne,metat,ndet", [(6, 6, 2, None), (8, 8, 1, 3000)])
def test_bamat_split_matches_fp64(n, ne, metat, ndet):
    p = synth.make_problem(n, ne, 3, 5, metat=metat, ndet=ndet, seed=90 + n)
    koop = koopro.koopro4QD(p)
    args = lambda: (koop["atwo"], p.ro4, p.daaa, p.taa, p.dal, n, p.ncore,
                    np.zeros(p.norb * (p.norb + 1) // 2), koop["aj"], p.norb, metat)
    ref = koopro.bamat(*args())
    with koopro.precision(koopro.SPLIT):
        got = koopro.bamat(*args())
    for g, r in zip(got, ref):
        assert np.abs(g - r).max() <= 1e-12 * np.abs(r).max()


def test_split_energies_within_1e7_of_fp64():
    from nevpt2_gb300 import qdnevpt as gq
    p = synth.config_problem("cas8")
    e64 = gq.qdnevpt(p, koopro.koopro4QD(p))
    with koopro.precision(koopro.SPLIT):
        koop = koopro.koopro4QD(p)
        esp = gq.qdnevpt(p, koop)
    assert np.abs(esp.e2mpp - e64.e2mpp).max() <= 1e-7
    assert np.abs(esp.e2enp - e64.e2enp).max() <= 1e-7
    assert abs(esp.e2mp[0, 0] - e64.e2mp[0, 0]) <= 1e-7
    assert abs(esp.e2en[0, 0] - e64.e2en[0, 0]) <= 1e-7
    assert np.array_equal(esp.nnew, e64.nnew)


# ---------------------------------------------------------------- general products
def _split_ex(A, B, ta=False, tb=False, alpha=1.0, beta=0.0, C0=None):
    """Row-major C = alpha op(A) op(B) + beta C0 through nvpt_dgemm_split_ex_d."""
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    m = A.shape[1] if ta else A.shape[0]
    k = A.shape[0] if ta else A.shape[1]
    n = B.shape[0] if tb else B.shape[1]
    tA = torch.from_numpy(np.ascontiguousarray(A)).to(dev)
    tB = torch.from_numpy(np.ascontiguousarray(B)).to(dev)
    tC = (torch.from_numpy(np.ascontiguousarray(C0)).to(dev) if C0 is not None
          else torch.full((m, n), float("nan"), dtype=torch.float64, device=dev))
    ctx = koopro.context()
    ctx.call("nvpt_dgemm_split_ex_d", int(ta), int(tb), m, n, k, alpha, ptr(tA), A.shape[1], ptr(tB), B.shape[1],
             beta, ptr(tC), n, None)
    ctx.synchronize()
    return tC.cpu().numpy()


def _bound_ex(X, Y):
    """Per-term error 2^-59 max|X_i| max|Y_j| plus the FP64 reference's own rounding."""
    k = X.shape[1]
    split = k * 2.0**-59 * np.abs(X).max(axis=1)[:, None] * np.abs(Y).max(axis=0)[None, :]
    return split + k * 2.0**-53 * (np.abs(X) @ np.abs(Y))


@pytest.mark.parametrize("m,n,k,ta,tb", [(128, 32, 64, False, False), (300, 77, 1184, False, False),
                                         (257, 500, 100, True, False), (1000, 1000, 4096, False, True),
                                         (33, 5, 3000, True, True), (7, 1, 1, False, False),
                                         (640, 96, 1537, False, False), (30, 700, 1184, False, False),
                                         (40, 512, 512, True, True)])
def test_split_ex_within_bound(m, n, k, ta, tb):
    rng = np.random.default_rng(m + 3 * n + 7 * k)
    A = rng.standard_normal((k, m) if ta else (m, k))
    B = rng.standard_normal((n, k) if tb else (k, n)) * 0.05
    X = A.T if ta else A
    Y = B.T if tb else B
    C = _split_ex(A, B, ta, tb)
    ref = X @ Y
    assert np.isfinite(C).all()
    err = np.abs(C - ref)
    assert (err <= _bound_ex(X, Y)).all()
    assert err.max() <= 1e-14 * np.abs(ref).max()


def test_split_ex_exact_on_small_integers():
    rng = np.random.default_rng(15)
    A = rng.integers(-63, 64, (256, 2000)).astype(np.float64)
    B = rng.integers(-63, 64, (2000, 96)).astype(np.float64)
    assert np.array_equal(_split_ex(A, B), A @ B)


def test_split_ex_alpha_beta_scales_and_zero_rows():
    rng = np.random.default_rng(16)
    A = rng.standard_normal((384, 700)) * (10.0 ** rng.uniform(-8, 3, 384))[:, None]
    A[17] = 0.0
    B = rng.standard_normal((700, 200)) * (10.0 ** rng.uniform(-4, 4, 200))[None, :]
    C0 = rng.standard_normal((384, 200))
    C = _split_ex(A, B, alpha=-0.5, beta=1.0, C0=C0)
    ref = -0.5 * (A @ B) + C0
    assert (np.abs(C - ref) <= 0.5 * _bound_ex(A, B) + 2.0**-52 * np.abs(ref)).all()
    assert np.array_equal(C[17], C0[17])


def test_split_ex_rejects_bad_arguments():
    ctx = koopro.context()
    x = np.zeros(1)
    with pytest.raises(NvptError) as e:
        ctx.call("nvpt_dgemm_split_ex_d", 0, 0, 4, 4, 4, 3.0, ptr(x), 4, ptr(x), 4, 0.0, ptr(x), 4, None)
    assert e.value.status == 1
    with pytest.raises(NvptError):
        ctx.call("nvpt_dgemm_split_ex_d", 0, 0, 4, 4, 4, 1.0, ptr(x), 3, ptr(x), 4, 0.0, ptr(x), 4, None)
