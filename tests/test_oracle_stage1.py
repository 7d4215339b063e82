"""The oracle against the reference's own run-time invariants and the
committed golden fixtures."""
import numpy as np
import pytest

from conftest import load_golden, rel_err
from nevpt2_gb300 import synth
from oracle import bruteforce as bf
from oracle import oracle as orc


def _golden_problem(g):
    n, ne, nc, nv = (int(g[k]) for k in ("nact", "nele", "ncore", "nvirt"))
    p = synth.make_problem(n, ne, nc, nv, metat=1, seed=1)
    p = synth.with_ci(p, g["amask"], g["bmask"], g["coef"])
    p.oneint = g["oneint"]
    p.chol = np.asfortranarray(g["chol"])
    return p


@pytest.mark.parametrize("name", ["stage1_cas44", "stage1_cas54_m2"])
def test_oracle_reproduces_golden(name):
    g = load_golden(name)
    p = _golden_problem(g)
    o = orc.stage1(p)
    for k, v in o.items():
        assert rel_err(v, g["out_" + k]) < 1e-12, k


@pytest.mark.parametrize("name", ["stage1_cas44", "stage1_cas54_m2"])
def test_fdiff_and_fdiff_F_vanish_on_eigenstates(name):
    """src/koopro4QD.F90:5053 fdiff (B == C^T) and src/koop_matrices.F90:591
    fdiff_F (F == 0), thresholds 1e-7 in the reference."""
    g = load_golden(name)
    n, M = int(g["nact"]), int(g["metat"])
    ip, ea = orc.fdiff(g["out_bmatIP"], g["out_cmatIP"], g["out_bmatEA"], g["out_cmatEA"], n, M)
    assert ip.max() < 1e-12 and ea.max() < 1e-12
    assert orc.fdiff_F(g["out_gk0pf"], n, M).max() < 1e-12


def test_golden_cas_is_an_eigenstate():
    g = load_golden("stage1_cas44")
    p = _golden_problem(g)
    atwo, aj = orc.get_aj_atwo(p.oneint, p.chol, p.nact, p.ncore, p.norb)
    n, nc = p.nact, p.ncore
    h = np.array([[aj[synth.tri(a + nc + 1, b + nc + 1) - 1] for b in range(n)] for a in range(n)])
    _, _, C, E = bf.casci(n, 2, 2, h, np.asarray(atwo), nroots=1)
    assert abs(E[0] - g["casci_energies"][0]) < 1e-12
    assert abs(abs(C[:, 0] @ g["coef"][:, 0]) - 1.0) < 1e-12


def test_aj_atwo_against_dense_integrals():
    p = synth.make_problem(4, 4, 3, 3, seed=2)
    atwo, aj = orc.get_aj_atwo(p.oneint, p.chol, 4, 3, p.norb)
    B = synth._dense_B(p.chol, p.norb, slice(0, p.chol.shape[0]))
    eri = np.einsum("xpq,xrs->pqrs", B, B)
    act = slice(3, 7)
    np.testing.assert_allclose(atwo, eri[act, act, act, act], atol=1e-14)
    h = np.zeros((p.norb, p.norb))
    k = 0
    for i in range(p.norb):
        for j in range(i + 1):
            h[i, j] = h[j, i] = p.oneint[k]
            k += 1
    core = slice(0, 3)
    heff = h + 2 * np.einsum("pqkk->pq", eri[:, :, core, core]) - np.einsum("pkkq->pq", eri[:, core, core, :])
    for a in range(3, 7):
        for b in range(a, 7):
            assert abs(aj[synth.tri(a + 1, b + 1) - 1] - heff[a, b]) < 1e-13
