"""The mathematics of the resolvent route of the order-n^3 PC pencils (CPU).

The reference forms, per external label with shift s, sum_mu r_mu^2 / (w_mu + s)
over the eigenpairs of the orthonormalised Koopmans problem (metric S kept
whole, Koopmans matrix K), with r = C^T z and C the PC coefficients.  The device
evaluates the same sums as z^T (K + s S)^-1 z through S = U^T U,
K~ = U^-T K U^-1 = Q T Q^T and Gaussian elimination with partial pivoting on
the tridiagonal T + s.  This test restates both in numpy/scipy on random
pencils, including shifts next to an eigenvalue (near-singular denominators)
and the cross terms of two right-hand sides, and checks that they agree.
"""
import numpy as np
import pytest

linalg = pytest.importorskip("scipy.linalg")


def _tridiag_solve(d, e, s, y):
    """(T + s I) x = y with row interchanges, as the device kernel does it."""
    n = d.size
    wb, wc, wd, wy = (np.zeros(n) for _ in range(4))
    b, c = d[0] + s, (e[0] if n > 1 else 0.0)
    yy = y[0]
    for i in range(n - 1):
        a1, b1 = e[i], d[i + 1] + s
        c1 = e[i + 1] if i + 2 < n else 0.0
        y1 = y[i + 1]
        if abs(b) >= abs(a1):
            f = a1 / b
            wb[i], wc[i], wd[i], wy[i] = b, c, 0.0, yy
            b, c, yy = b1 - f * c, c1, y1 - f * yy
        else:
            f = b / a1
            wb[i], wc[i], wd[i], wy[i] = a1, b1, c1, y1
            b, c, yy = c - f * b1, -f * c1, yy - f * y1
    wb[n - 1], wy[n - 1] = b, yy
    x = np.zeros(n)
    x[n - 1] = yy / b
    for i in range(n - 2, -1, -1):
        x[i] = (wy[i] - wc[i] * x[i + 1] - (wd[i] * x[i + 2] if i + 2 < n else 0.0)) / wb[i]
    return x


def _pencil(n, seed):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, n))
    S = X @ X.T / n + 0.1 * np.eye(n)  # metric: positive definite
    Y = rng.standard_normal((n, n))
    K = (Y + Y.T) / 2                  # Koopmans matrix: symmetric, indefinite
    return S, K, rng


@pytest.mark.parametrize("n", [5, 40, 120])
def test_resolvent_sums_equal_the_eigenpair_sums(n):
    S, K, rng = _pencil(n, n)
    w, V = linalg.eigh(K, S)            # K v = w S v, V^T S V = I (the PC coefficients)
    U = np.linalg.cholesky(S).T         # S = U^T U
    Kt = linalg.solve_triangular(U, linalg.solve_triangular(U, K, trans="T").T, trans="T").T
    Kt = (Kt + Kt.T) / 2
    T, Q = linalg.hessenberg(Kt, calc_q=True)  # symmetric Hessenberg = tridiagonal
    d, e = np.diag(T).copy(), np.diag(T, -1).copy()
    z1, z2 = rng.standard_normal(n), rng.standard_normal(n)
    shifts = [0.37, -w[n // 2] + 1e-7, -w[0] - 0.5]  # ordinary, next to an eigenvalue, below the spectrum
    for s in shifts:
        r1, r2 = V.T @ z1, V.T @ z2
        ref_e = np.sum(r1 * r1 / (w + s))
        ref_psi = np.sum(r1 * r1 / (w + s) ** 2)
        ref_x = np.sum(r2 * r1 / (w + s))
        y1 = Q.T @ linalg.solve_triangular(U, z1, trans="T")
        y2 = Q.T @ linalg.solve_triangular(U, z2, trans="T")
        x = _tridiag_solve(d, e, s, y1)
        # both evaluations carry rounding errors of order eps * cond(K + s S) relative
        # to the sums of absolute terms; cond is large next to an eigenvalue
        cond = np.abs(w + s).max() / np.abs(w + s).min() * np.linalg.cond(S)
        tol = 1e3 * np.finfo(float).eps * cond
        assert abs(y1 @ x - ref_e) <= tol * np.sum(np.abs(r1 * r1 / (w + s)))
        assert abs(x @ x - ref_psi) <= 2 * tol * np.sum(r1 * r1 / (w + s) ** 2)
        assert abs(y2 @ x - ref_x) <= tol * np.sum(np.abs(r2 * r1 / (w + s)))


def test_tridiagonal_solver_pivots():
    rng = np.random.default_rng(3)
    n = 60
    d = rng.standard_normal(n) * 1e-3   # small diagonal: the elimination must interchange rows
    e = rng.standard_normal(n - 1)
    T = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
    y = rng.standard_normal(n)
    x = _tridiag_solve(d, e, 0.0, y)
    assert np.abs(T @ x - y).max() <= 1e-10 * np.abs(T).max() * np.abs(x).max()


def _to_band(A, b):
    """Dense symmetric A -> band form of half-bandwidth b by block Householder
    (two-sided QR of each panel below the band); returns the band matrix and
    the panel transforms (row offset, orthogonal factor)."""
    A = A.copy()
    n = A.shape[0]
    Qs = []
    for k in range(0, n - b, b):
        Qp, _ = np.linalg.qr(A[k + b:, k:k + b], mode="complete")
        A[k + b:, :] = Qp.T @ A[k + b:, :]
        A[:, k + b:] = A[:, k + b:] @ Qp
        Qs.append((k + b, Qp))
    return A, Qs


def test_band_route_resolvents_equal_the_eigenpair_sums():
    """The next step's route: resolvents on the band form (banded LU with
    partial pivoting), no reduction to tridiagonal."""
    rng = np.random.default_rng(11)
    n, b = 150, 12
    X = rng.standard_normal((n, n))
    A = (X + X.T) / 2
    Bm, Qs = _to_band(A, b)
    assert np.abs(np.tril(Bm, -b - 1)).max() <= 1e-13 * np.abs(A).max()
    w, V = np.linalg.eigh(A)
    z = rng.standard_normal(n)
    y = z.copy()
    for k, Qp in Qs:
        y[k:] = Qp.T @ y[k:]
    for s in (0.3, -w[7] + 1e-6):
        ref = np.sum((V.T @ z) ** 2 / (w + s))
        M = Bm + s * np.eye(n)
        ab = np.zeros((3 * b + 1, n))  # LAPACK general band storage with room for the pivoting fill
        for j in range(n):
            for i in range(max(0, j - b), min(n, j + b + 1)):
                ab[2 * b + i - j, j] = M[i, j]
        _, _, x, info = linalg.lapack.dgbsv(b, b, ab, y)
        assert info == 0
        cond = np.abs(w + s).max() / np.abs(w + s).min()
        assert abs(y @ x - ref) <= 1e3 * np.finfo(float).eps * cond * np.sum(np.abs((V.T @ z) ** 2 / (w + s)))
