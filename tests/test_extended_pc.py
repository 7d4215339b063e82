"""The extended-precision (+2) PC evaluation (oracle/extended_pc.py) against
the oracle's eigenpair route (src/qdnevpt.F:2804-3010) on small problems."""
import numpy as np
import pytest

from nevpt2_gb300 import synth
from oracle import extended_pc as X
from oracle import qdnevpt_oracle as q


def test_batched_elimination_solves():
    rng = np.random.default_rng(3)
    A = rng.standard_normal((5, 12, 12))
    b = rng.standard_normal((5, 12))
    x = X.solve_batched(A, b)
    for k in range(5):
        np.testing.assert_allclose(A[k] @ x[k], b[k], rtol=0, atol=1e-12)
    xl = X.solve_batched(A.astype(np.longdouble), b.astype(np.longdouble))
    np.testing.assert_allclose(xl.astype(np.float64), x, rtol=1e-12, atol=1e-13)


@pytest.mark.parametrize("n,ne,nc,nv,M,seed", [(4, 4, 3, 4, 1, 5), (5, 4, 4, 5, 1, 6), (6, 6, 5, 8, 2, 7)])
def test_resolvent_form_equals_eigenpair_route(n, ne, nc, nv, M, seed):
    p = synth.make_problem(n, ne, nc, nv, metat=M, seed=seed, with_ro4=False)
    inp = X.stage2_inputs(p)
    r = q.qdnevpt(inp, classes=[3])
    B, h = q.dense_B(inp.chol, inp.norb), q.unpack_tri(inp.oneint, inp.norb)
    for s in range(M):
        st = q._State(inp, s, B, h)
        e64 = X.plus2_pc_energy(inp, st, s, np.float64)
        eld = X.plus2_pc_energy(inp, st, s, np.longdouble)
        assert abs(e64 - r.e2enp[3, s]) < 1e-12
        assert abs(float(eld) - r.e2enp[3, s]) < 1e-12


def test_sensitivity_of_a_well_conditioned_class_is_at_rounding_level():
    p = synth.make_problem(5, 4, 4, 5, metat=1, seed=6, with_ro4=False)
    inp = X.stage2_inputs(p)
    B, h = q.dense_B(inp.chol, inp.norb), q.unpack_tri(inp.oneint, inp.norb)
    st = q._State(inp, 0, B, h)
    e0 = X.plus2_pc_energy(inp, st, 0, np.float64, lapack=True)
    sens = X.sensitivity(inp, st, 0)
    assert set(sens) == {"eps_one_rounding", "eako2_one_rounding", "hrdm_one_rounding", "eako2_one_rounding_of_max"}
    for v in sens.values():
        assert 0.0 <= v < 1e-12 * max(1.0, abs(e0))
    # the inputs are restored
    assert X.plus2_pc_energy(inp, st, 0, np.float64, lapack=True) == e0
