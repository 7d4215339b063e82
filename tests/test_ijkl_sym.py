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
