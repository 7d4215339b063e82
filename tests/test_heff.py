"""QD effective Hamiltonian (src/qdnevpt.F:1046-1126, hermitian_heff
:8089-8183): the host mirror against the oracle's element-loop restatement,
plus the properties the Hermitisation guarantees (CPU only)."""
import numpy as np
import pytest

from nevpt2_gb300 import qdnevpt as gq
from oracle import qdnevpt_oracle as q


def _heff(rng, m, asym):
    a = rng.standard_normal((m, m)) * 1e-2
    h = 0.5 * (a + a.T) + asym * rng.standard_normal((m, m)) * 1e-3
    return h + np.diag(np.sort(rng.uniform(-1.0, 1.0, m)))


@pytest.mark.parametrize("m,seed", [(2, 1), (3, 2), (4, 3), (6, 4)])
def test_mirror_matches_oracle(m, seed):
    rng = np.random.default_rng(seed)
    e2 = _heff(rng, m, 1.0)
    E = rng.uniform(-100.0, -99.0, m)
    h = gq.effective_hamiltonian(e2, E)
    wr, wi, vr, Hh, evc, w = q.heff_qd(e2, E)
    np.testing.assert_allclose(h.wr, wr, rtol=0, atol=1e-12)
    np.testing.assert_array_equal(h.wi, wi)
    np.testing.assert_allclose(np.abs(h.vr), np.abs(vr), rtol=0, atol=1e-12)
    np.testing.assert_allclose(h.heff_herm, Hh, rtol=0, atol=1e-11)
    np.testing.assert_allclose(h.w_herm, w, rtol=0, atol=1e-11)
    np.testing.assert_allclose(np.abs(h.evc_herm), np.abs(evc), rtol=0, atol=1e-9)


@pytest.mark.parametrize("m", [2, 4, 5])
def test_hermitisation_properties(m):
    rng = np.random.default_rng(10 + m)
    e2 = _heff(rng, m, 1.0)
    h = gq.effective_hamiltonian(e2, np.zeros(m))
    assert np.all(np.diff(h.wr) >= 0)
    np.testing.assert_allclose(h.heff_herm, h.heff_herm.T, rtol=0, atol=1e-14)
    # a similarity transform: the spectrum is kept
    np.testing.assert_allclose(h.w_herm, np.sort(np.linalg.eigvals(h.heff).real), rtol=0, atol=1e-12)
    # the Loewdin-orthonormalised right eigenvectors diagonalise Heff~
    S = h.vr.T @ h.vr
    ev, G = np.linalg.eigh(S)
    Cp = h.vr @ (G / np.sqrt(ev)) @ G.T
    np.testing.assert_allclose(Cp.T @ Cp, np.eye(m), rtol=0, atol=1e-12)
    np.testing.assert_allclose(Cp.T @ h.heff_herm @ Cp, np.diag(h.wr), rtol=0, atol=1e-12)


def test_symmetric_heff_is_left_unchanged():
    rng = np.random.default_rng(5)
    e2 = _heff(rng, 4, 0.0)
    h = gq.effective_hamiltonian(e2, np.zeros(4))
    np.testing.assert_allclose(h.heff_herm, h.heff, rtol=0, atol=1e-13)


def test_single_state_skips_the_diagonalisation():
    h = gq.effective_hamiltonian(np.array([[-0.25]]), np.array([-100.0]))
    assert h.w_herm[0] == -100.25 and h.heff_herm[0, 0] == -100.25
