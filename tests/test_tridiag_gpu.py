"""Device Householder tridiagonalisation (nvpt_sytrd_d): the building block of
the order-n^3 PC pencils.  Checked against LAPACK-free invariants: the
eigenvalues of T are those of A, and the reflectors rebuild A = Q T Q^T."""
import numpy as np
import pytest

from nevpt2_gb300 import koopro
from nevpt2_gb300._native import ptr

pytestmark = pytest.mark.gpu


def _sytrd(A):
    torch = pytest.importorskip("torch")
    n = A.shape[0]
    dev = torch.device("cuda:0")
    tA = torch.from_numpy(np.asfortranarray(A).ravel(order="F").copy()).to(dev)
    d = torch.zeros(n, dtype=torch.float64, device=dev)
    e = torch.zeros(max(n, 1), dtype=torch.float64, device=dev)
    tau = torch.zeros(max(n, 1), dtype=torch.float64, device=dev)
    ctx = koopro.context()
    ctx.call("nvpt_sytrd_d", n, ptr(tA), ptr(d), ptr(e), ptr(tau), None)
    ctx.synchronize()
    return (tA.cpu().numpy().reshape((n, n), order="F"), d.cpu().numpy(), e.cpu().numpy()[:n - 1],
            tau.cpu().numpy()[:n - 1])


def _sym(n, seed):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, n))
    return (X + X.T) / 2


@pytest.mark.parametrize("n", [1, 2, 3, 33, 300, 512, 777])
def test_sytrd_keeps_the_eigenvalues(n):
    linalg = pytest.importorskip("scipy.linalg")
    A = _sym(n, n)
    _, d, e, _ = _sytrd(A)
    w = linalg.eigh_tridiagonal(d, e, eigvals_only=True) if n > 1 else d
    ref = np.linalg.eigvalsh(A)
    assert np.abs(np.sort(w) - ref).max() <= 50 * n * 2.2e-16 * np.abs(ref).max()


@pytest.mark.parametrize("n", [40, 130])
def test_sytrd_reflectors_rebuild_the_matrix(n):
    A = _sym(n, 7 + n)
    Af, d, e, tau = _sytrd(A)
    assert np.array_equal(np.diag(Af), d)
    assert np.array_equal(np.diag(Af, -1), e)
    Q = np.eye(n)
    for i in range(n - 1):  # Q = H_0 H_1 ... H_{n-2}
        v = np.zeros(n)
        v[i + 1] = 1.0
        v[i + 2:] = Af[i + 2:, i]
        Q = Q - tau[i] * np.outer(Q @ v, v)
    T = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
    assert np.abs(Q @ T @ Q.T - A).max() <= 1e-13 * n * np.abs(A).max()
    assert np.abs(Q.T @ Q - np.eye(n)).max() <= 1e-13 * n


def test_barrier_timeout_reports_and_the_context_recovers():
    """A grid-barrier wait that runs out of polls makes the kernel return and
    the call report NVPT_ETIMEDOUT; the context stays usable.  The limit of
    one poll makes every CTA that is not the last to arrive give up."""
    torch = pytest.importorskip("torch")
    from nevpt2_gb300._native import Context, NvptError
    n = 512
    A = _sym(n, 5)
    dev = torch.device("cuda:0")
    ctx = Context(0)
    d = torch.zeros(n, dtype=torch.float64, device=dev)
    e = torch.zeros(n, dtype=torch.float64, device=dev)
    tau = torch.zeros(n, dtype=torch.float64, device=dev)
    ctx.call("nvpt_set_wait_limit", 1)
    statuses = []
    for _ in range(3):
        tA = torch.from_numpy(A.ravel(order="F").copy()).to(dev)
        try:
            ctx.call("nvpt_sytrd_d", n, ptr(tA), ptr(d), ptr(e), ptr(tau), None)
            ctx.synchronize()
            statuses.append(0)
        except NvptError as err:
            statuses.append(err.status)
            if err.status == 5:
                break
    assert statuses[-1] == 5, statuses
    ctx.call("nvpt_set_wait_limit", 0)
    tA = torch.from_numpy(A.ravel(order="F").copy()).to(dev)
    ctx.call("nvpt_sytrd_d", n, ptr(tA), ptr(d), ptr(e), ptr(tau), None)
    ctx.synchronize()
    linalg = pytest.importorskip("scipy.linalg")
    w = linalg.eigh_tridiagonal(d.cpu().numpy(), e.cpu().numpy()[:n - 1], eigvals_only=True)
    ref = np.linalg.eigvalsh(A)
    assert np.abs(np.sort(w) - ref).max() <= 50 * n * 2.2e-16 * np.abs(ref).max()
    ctx.close()
