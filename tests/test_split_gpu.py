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
