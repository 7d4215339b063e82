"""Symmetry-packed two-electron integrals (src/infsym.F90:16-69,
src/ijkl_utils.F90:111-207,690-756): the device tables bit-exact against the
oracle's restatement, ai_twoint lookups bit-exact, get_aj_atwo on this path
against the oracle and against the Cholesky path on the same integrals.
The CPU tests pin the oracle itself: C1 tables reduce to the plain
triangular index, and packing a symmetric DF integral set into twoint and
looking it up again returns every integral (0 where symmetry forbids it)."""
import numpy as np
import pytest

from oracle import oracle as orc

CASES = [  # (nish, nash, nssh) per irrep
    ([3], [4], [5]),
    ([2, 1], [3, 2], [4, 3]),
    ([2, 0, 1, 1], [2, 1, 1, 2], [3, 2, 2, 1]),
    ([1, 1, 0, 1, 1, 0, 1, 0], [1, 2, 1, 0, 1, 1, 0, 1], [2, 1, 2, 1, 1, 2, 1, 1]),
]


def _all_quads(norb, rng, k=4000):
    return rng.integers(1, norb + 1, (k, 4)).astype(np.int64)


def _dense(chol, norb):
    P = chol.shape[1]
    G = chol.T @ chol
    idx = np.zeros((norb, norb), np.int64)
    for p in range(norb):
        for q in range(norb):
            a, b = max(p, q) + 1, min(p, q) + 1
            idx[p, q] = a * (a - 1) // 2 + b - 1
    return G, idx


@pytest.mark.parametrize("case", range(len(CASES)))
def test_oracle_tables_and_roundtrip(case):
    nish, nash, nssh = CASES[case]
    t = orc.ijkl_tables(nish, nash, nssh)
    norb = len(t["itsym"])
    npair = norb * (norb + 1) // 2
    np.testing.assert_array_equal(t["num"], np.arange(npair) * (np.arange(npair) + 1) // 2)
    for r in range(1, len(nish) + 1):  # jndic ranks the pairs of each irrep 1..nos
        ranks = t["jndic"][t["indic"] == r]
        np.testing.assert_array_equal(ranks, np.arange(1, ranks.size + 1))
    rng = np.random.default_rng(case)
    chol = orc.symmetric_chol(t["itsym"], 3 * norb, rng)
    tw = orc.pack_twoint(t, chol)
    G, idx = _dense(chol, norb)
    q = _all_quads(norb, rng)
    got = orc.ai_twoint(t, tw, q)
    want = G[idx[q[:, 0] - 1, q[:, 1] - 1], idx[q[:, 2] - 1, q[:, 3] - 1]]
    np.testing.assert_allclose(got, want, rtol=1e-14, atol=1e-17)
    if len(nish) > 1:
        sym = (t["itsym"][q[:, 0] - 1] - 1) ^ (t["itsym"][q[:, 1] - 1] - 1) ^ \
              (t["itsym"][q[:, 2] - 1] - 1) ^ (t["itsym"][q[:, 3] - 1] - 1)
        assert np.all(got[sym != 0] == 0.0) and np.any(sym != 0)


def test_c1_tables_are_the_triangular_index():
    t = orc.ijkl_tables([2], [3], [4])
    npair = 9 * 10 // 2
    assert t["ni4"] == npair * (npair + 1) // 2
    np.testing.assert_array_equal(t["jndic"], np.arange(1, npair + 1))
    assert list(t["nad"]) == [1] and list(t["kt"]) == [1] and list(t["ndeb"]) == [0]


@pytest.mark.gpu
@pytest.mark.parametrize("case", range(len(CASES)))
def test_device_tables_bit_exact(gpu_ctx, case):
    from nevpt2_gb300 import koopro
    nish, nash, nssh = CASES[case]
    si = koopro.SymmetryIntegrals(nish, nash, nssh)
    got = si.tables()
    ref = orc.ijkl_tables(nish, nash, nssh)
    for k in koopro.SymmetryIntegrals.KEYS:
        np.testing.assert_array_equal(got[k], ref[k], err_msg=k)
    assert got["ni4"] == ref["ni4"]


@pytest.mark.gpu
def test_device_tables_bit_exact_large(gpu_ctx):
    from nevpt2_gb300 import koopro
    rng = np.random.default_rng(3)
    c = [list(rng.integers(0, 40, 8)) for _ in range(3)]
    si = koopro.SymmetryIntegrals(*c)
    got, ref = si.tables(), orc.ijkl_tables(*c)
    for k in koopro.SymmetryIntegrals.KEYS:
        np.testing.assert_array_equal(got[k], ref[k], err_msg=k)


@pytest.mark.gpu
@pytest.mark.parametrize("case", range(len(CASES)))
def test_ai_twoint_and_get_aj_atwo(gpu_ctx, case):
    from nevpt2_gb300 import koopro
    nish, nash, nssh = CASES[case]
    si = koopro.SymmetryIntegrals(nish, nash, nssh)
    t = orc.ijkl_tables(nish, nash, nssh)
    norb = si.norb
    rng = np.random.default_rng(10 + case)
    chol = orc.symmetric_chol(t["itsym"], 3 * norb, rng)
    tw = orc.pack_twoint(t, chol)
    si.set_twoint(tw)
    q = _all_quads(norb, rng)
    np.testing.assert_array_equal(si.ai(q), orc.ai_twoint(t, tw, q))
    ncore, nact = int(sum(nish)), int(sum(nash))
    oneint = rng.standard_normal(norb * (norb + 1) // 2)
    atwo, aj = si.get_aj_atwo(nact, ncore, oneint)
    ratwo, raj = orc.get_aj_atwo_twoint(t, tw, oneint, nact, ncore, norb)
    np.testing.assert_array_equal(atwo, ratwo)
    np.testing.assert_allclose(aj, raj, rtol=0, atol=1e-15)
    # the same integrals through the Cholesky path (C1 addressing)
    catwo, caj = koopro.get_aj_atwo(nact, ncore, norb, oneint, np.asfortranarray(chol))
    np.testing.assert_allclose(atwo, catwo, rtol=0, atol=1e-15)
    np.testing.assert_allclose(aj, caj, rtol=0, atol=1e-14)


@pytest.mark.gpu
def test_init_rejects_bad_counts(gpu_ctx):
    from nevpt2_gb300 import _native, koopro
    with pytest.raises(_native.NvptError) as e:
        koopro.SymmetryIntegrals([1, 1, 1], [1, 1, 1], [1, 1, 1])
    assert e.value.status == 1
    si = koopro.SymmetryIntegrals([1, 1], [1, 1], [1, 1])
    with pytest.raises(_native.NvptError):
        si.ai(np.array([[1, 1, 1, 7]]))  # twoint not set yet


# ------------------------------------------- symmetry-screened Koopmans builders
SYM = [([1, 1], [2, 2], [2, 2], 4, 1), ([1, 0, 1, 0], [2, 1, 2, 1], [1, 1, 1, 1], 6, 2)]


def _sym_inputs(case):
    from nevpt2_gb300 import synth
    nish, nash, nssh, ne, M = case
    p = synth.make_sym_problem(nish, nash, nssh, ne, metat=M, seed=5)
    t = orc.ijkl_tables(nish, nash, nssh)
    tw = orc.pack_twoint(t, p.chol)
    asym = t["itsym"][p.ncore:p.ncore + p.nact]
    return p, t, tw, asym


@pytest.mark.parametrize("case", range(len(SYM)))
def test_oracle_screened_branches_equal_c1_on_symmetric_inputs(case):
    """The terms the reference's symmetry branches skip vanish on symmetric
    inputs: the screened and the C1 loops agree (CPU, oracle)."""
    p, t, tw, asym = _sym_inputs(SYM[case])
    n, nc, M = p.nact, p.ncore, p.metat
    atwo, aj = orc.get_aj_atwo_twoint(t, tw, p.oneint, n, nc, p.norb)
    f1, f2 = np.zeros_like(aj), np.zeros_like(aj)
    a = orc.koop_matrices_ctl(M, n, nc, atwo, p.daaa, p.taa, p.dal, f1, aj)
    b = orc.koop_matrices_ctl_sym(M, n, nc, atwo, p.daaa, p.taa, p.dal, f2, aj, asym)
    for k in ("ipko2", "eako2"):
        assert np.abs(a[k] - b[k]).max() <= 1e-12 * max(np.abs(a[k]).max(), 1.0)
    A, At = orc.bamat(atwo, p.ro4, p.daaa, p.taa, p.dal, n, nc, f1, aj, p.norb, M)
    B, Bt = orc.bamat_sym(atwo, p.ro4, p.daaa, p.taa, p.dal, n, nc, f2, aj, M, asym)
    assert np.abs(A - B).max() <= 1e-12 * np.abs(A).max()
    assert np.abs(At - Bt).max() <= 1e-12 * np.abs(At).max()


@pytest.mark.gpu
@pytest.mark.parametrize("case", range(len(SYM)))
def test_symmetry_screened_builders_against_oracle(gpu_ctx, case):
    from conftest import rel_err
    from nevpt2_gb300 import _native, koopro
    p, t, tw, asym = _sym_inputs(SYM[case])
    nish, nash, nssh = SYM[case][:3]
    n, nc, M = p.nact, p.ncore, p.metat
    si = koopro.SymmetryIntegrals(nish, nash, nssh)
    si.set_twoint(tw)
    atwo, aj = si.get_aj_atwo(n, nc, p.oneint)
    ratwo, raj = orc.get_aj_atwo_twoint(t, tw, p.oneint, n, nc, p.norb)
    f, rf = np.zeros_like(aj), np.zeros_like(aj)
    got = koopro.koop_matrices_ctl(M, n, nc, atwo, p.daaa, p.taa, p.dal, f, aj, ctx=si.ctx)
    ref = orc.koop_matrices_ctl_sym(M, n, nc, ratwo, p.daaa, p.taa, p.dal, rf, raj, asym)
    for k, rk in (("2-IPKO", "ipko2"), ("2-EAKO", "eako2"), ("1-IPKO", "ipko1"), ("gk0pa", "gk0pa")):
        assert rel_err(got[k], ref[rk]) < 1e-10, k
    A, At = koopro.bamat(atwo, p.ro4, p.daaa, p.taa, p.dal, n, nc, f, aj, p.norb, M, nsym=len(nish), ctx=si.ctx)
    R, Rt = orc.bamat_sym(ratwo, p.ro4, p.daaa, p.taa, p.dal, n, nc, rf, raj, M, asym)
    assert rel_err(A, R) < 1e-10 and rel_err(At, Rt) < 1e-10
    # elements the reference never assigns are exactly zero
    irr = asym - 1
    tot = np.zeros((n,) * 6, dtype=np.int64)
    for ax in range(6):
        sh = [1] * 6
        sh[ax] = n
        tot = tot ^ irr.reshape(sh)
    assert np.all(A[:, tot != 0] == 0.0) and np.all(At[:, tot != 0] == 0.0)
    # without the tables the symmetry branch is refused
    with pytest.raises(_native.NvptError) as e:
        koopro.bamat(atwo, p.ro4, p.daaa, p.taa, p.dal, n, nc, f, aj, p.norb, M, nsym=len(nish))
    assert e.value.status == 4
