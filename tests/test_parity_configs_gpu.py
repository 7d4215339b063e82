"""The CUDA path against the oracle on the benchmark's own configurations,
through the C ABI (host-pointer entry points).

* CAS(8,8), 10 inactive / 40 virtual, 4900 determinants: stage 1 and stage 2
  in full (per-class SC/PC energies and norms, nnew exact).
* CAS(14,14), 20 / 150, 50,000 determinants: every stage-1 builder in full
  except bamat, which is compared on 16 sampled (a,c) slabs (the oracle's
  slab-restricted loop gives those slabs' elements exactly); stage 2 in full
  on the GPU's Koopmans matrices.
* CAS(16,16), 30 / 250, 4 roots of 100,000 determinants: every stage-1
  builder in full except bamat, which is compared on sampled slabs of two
  states.

Tolerances: Koopmans matrices <= 1e-10 relative to the largest element of
each array (per state for the sampled bamat elements); nnew exact; norms
<= 1e-9 absolute or 1e-9 relative; energies <= 1e-9 Eh absolute or 1e-9
relative.  The relative part is for these random-CI workloads: their
wavefunctions are not eigenstates of the active Hamiltonian, so some PC
denominators w + de nearly vanish and single classes reach 10-100 Eh
(CAS(14,14): (-1)' PC = -66.4 Eh), where one rounding of the inputs moves
the energy by more than 1e-9 Eh; the oracle's eigenvector route and the
device's resolvent route then agree to about 1e-10 relative.
"""
import numpy as np
import pytest

from conftest import rel_err
from nevpt2_gb300 import koopro, synth
from nevpt2_gb300 import qdnevpt as gq
from oracle import oracle as orc
from oracle import qdnevpt_oracle as q

pytestmark = pytest.mark.gpu
TOL = 1e-10
ETOL = 1e-9
ERTOL = 1e-9
NORM_RTOL = 1e-9
DSETS = {"1-IPKO": "ipko1", "1-EAKO": "eako1", "2-HRDM": "hrdm2", "2-IPKO": "ipko2", "2-EAKO": "eako2",
         "gk0pa": "gk0pa", "gk0pd": "gk0pd", "gk0pf": "gk0pf"}
SLOTS = {(1, "p"): 0, (2, "p"): 1, (3, "a"): 2, (3, "b"): 3, (4, "a"): 4, (4, "b"): 5, (5, "p"): 6, (6, "p"): 7,
         (7, "p"): 8}


def _oracle_stage1_but_bamat(p):
    """Every stage-1 dataset of the oracle except amatIP/amatEA."""
    n, M, nc, norb = p.nact, p.metat, p.ncore, p.norb
    atwo, aj = orc.get_aj_atwo(p.oneint, p.chol, n, nc, norb)
    f = np.zeros(norb * (norb + 1) // 2)
    out = orc.koop_matrices_ctl(M, n, nc, atwo, p.daaa, p.taa, p.dal, f, aj)
    out["bmatIP"], out["bmatEA"] = orc.bbmat(atwo, p.daaa, p.taa, p.dal, n, nc, f, aj, M)
    out["cmatIP"], out["cmatEA"] = orc.bcmat(atwo, p.daaa, p.taa, p.dal, n, nc, f, aj, M)
    out["dmatIP"], out["dmatEA"] = orc.bdmat(atwo, p.taa, p.dal, n, nc, f, aj, M)
    out["daaa"] = orc.bro3(p.ro4, n, p.nele, M)
    out["atwo"], out["aj"] = atwo, aj
    return out


def _check_builders(got, ref, M):
    assert rel_err(got["3-RDM"], ref["daaa"]) < 1e-13
    assert rel_err(got["atwo"], ref["atwo"]) < 1e-13
    for k, v in got.items():
        if k in ("3-RDM", "2-RDM", "1-RDM", "atwo", "aj", "amatIP", "amatEA"):
            continue
        r = ref[DSETS.get(k, k)]
        for s in range(M):
            assert rel_err(v[s], r[s]) < TOL, (k, s, rel_err(v[s], r[s]))


def _check_bamat_slabs(p, got, slabs, states):
    """amat/atmat of the listed 0-based (a,c) slabs against the oracle's
    slab-restricted bamat, state by state."""
    n = p.nact
    atwo, aj = orc.get_aj_atwo(p.oneint, p.chol, n, p.ncore, p.norb)
    mask = orc.slab_mask(n, slabs)
    for s in states:
        f = np.zeros(p.norb * (p.norb + 1) // 2)
        sl = lambda a: np.asfortranarray(a[s:s + 1])
        ro4 = np.asfortranarray(p.ro4[..., s:s + 1])
        A, At = orc.bamat_slab_list(atwo, ro4, sl(p.daaa), sl(p.taa), sl(p.dal), n, p.ncore, f, aj, 1, slabs)
        for name, ref in (("amatIP", A[0]), ("amatEA", At[0])):
            g = got[name][s]
            scale = max(float(np.abs(g).max()), 1e-2)
            err = float(np.abs(g[mask] - ref[mask]).max()) / scale
            assert err < TOL, (name, s, err)


def _stage2_compare(p, koop, transition=None):
    """nvpt_qdnevpt against the oracle's stage 2, both fed the same Koopmans
    matrices (the GPU's FP64 stage-1 results)."""
    o = {k: v for k, v in koop.items()}
    o["1-RDM"], o["2-RDM"], o["3-RDM"] = p.dal, p.taa, p.daaa
    got = gq.qdnevpt(p, o, transition=transition)
    ref = q.qdnevpt(q.inputs_from(p, o, transition=None if transition is None else
                                  tuple(list(t) for t in transition)))
    for name in ("e2mpp", "psimpp", "e2enp", "psienep", "e2mp", "e2en", "psimp", "psien"):
        rtol = NORM_RTOL if name.startswith("psi") else ERTOL
        np.testing.assert_allclose(getattr(got, name), getattr(ref, name), rtol=rtol, atol=ETOL, err_msg=name)
    for s in range(p.metat):
        for key, slot in SLOTS.items():
            cls, part = key
            rk = (cls, s) if part == "p" else (cls, s, part)
            if rk in ref.nnew:
                assert got.nnew[slot, s] == ref.nnew[rk], (key, s)
    np.testing.assert_allclose(got.epsnew, np.column_stack([ref.epsnew[:, s] for s in range(p.metat)]), rtol=0,
                               atol=1e-11)
    return got, ref


def test_cas8_config_stage1_and_stage2_in_full(gpu_ctx):
    """CAS(8,8), 4900 determinants, 10 inactive / 40 virtual orbitals."""
    p = synth.config_problem("cas8")
    got = koopro.koopro4QD(p)
    ref = orc.stage1(p)
    for k, v in got.items():
        if k in ("3-RDM", "2-RDM", "1-RDM", "aj"):
            continue
        assert rel_err(v, ref[DSETS.get(k, k)]) < TOL, k
    _stage2_compare(p, got)


@pytest.fixture(scope="module")
def cas14():
    p = synth.config_problem("cas14")
    return p, koopro.koopro4QD(p)


def test_cas14_config_stage1_builders_in_full(gpu_ctx, cas14):
    p, got = cas14
    _check_builders(got, _oracle_stage1_but_bamat(p), 1)


def test_cas14_config_bamat_on_sampled_slabs(gpu_ctx, cas14):
    p, got = cas14
    n = p.nact
    rng = np.random.default_rng(14)
    slabs = sorted(set(int(x) for x in rng.choice(n * n, 16, replace=False)) | {0, n * n - 1})
    _check_bamat_slabs(p, got, slabs, [0])


def test_cas14_config_stage2_in_full(gpu_ctx, cas14):
    p, got = cas14
    _stage2_compare(p, got)


def test_cas16_qd4_config_stage1_builders_and_sampled_bamat(gpu_ctx):
    """CAS(16,16), 4 roots of 100,000 determinants, 30 / 250."""
    p = synth.config_problem("cas16_qd4")
    got = koopro.koopro4QD(p)
    _check_builders(got, _oracle_stage1_but_bamat(p), p.metat)
    n = p.nact
    _check_bamat_slabs(p, got, [0, 5 * n + 9, n * n - 1], [0])
    _check_bamat_slabs(p, got, [3 * n + 14, 11 * n + 2], [3])
