"""Stage-1 CUDA kernels against the oracle (through the C ABI).

Tolerances: integers bit-exact; FP64 Koopmans matrices <= 1e-10 relative to
the largest element of each array (the reference's own FP64 sums use OpenMP
atomics, so only tolerance-based parity is meaningful)."""
import itertools

import numpy as np
import pytest

from conftest import load_golden, rel_err
from nevpt2_gb300 import _native, koopro, synth
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
TOL = 1e-10


def test_ord8_bit_exact_all_tuples(gpu_ctx):
    n = 4
    t = np.array(list(itertools.product(range(1, n + 1), repeat=8)), dtype=np.int64)
    got, lind = koopro.ord8(n, t)
    ref = orc.ord_tuples(n, 8, t)
    np.testing.assert_array_equal(got, ref)
    lindi, lindj, lindk, _ = orc.index_tables(n)
    want = lindi[ref[:, 0] - 1] + lindj[ref[:, 1] - 1] + lindk[ref[:, 2] - 1] + ref[:, 3]
    np.testing.assert_array_equal(lind, want)


def test_ord8_bit_exact_n16_sample(gpu_ctx):
    rng = np.random.default_rng(1)
    t = rng.integers(1, 17, (200000, 8)).astype(np.int64)
    t[::3, 4:] = t[::3, :4][:, ::-1]  # many ties and equal multisets
    got, _ = koopro.ord8(16, t)
    np.testing.assert_array_equal(got, orc.ord_tuples(16, 8, t))


def test_ord9_bit_exact_all_tuples_and_n16_sample(gpu_ctx):
    n = 4
    t = np.array(list(itertools.product(range(1, n + 1), repeat=8)), dtype=np.int64)
    got, lind = koopro.ord9(n, t)
    ref = orc.ord_tuples(n, 9, t)
    np.testing.assert_array_equal(got, ref)
    lindi, lindj, lindk, _ = orc.index_tables(n)
    np.testing.assert_array_equal(lind, lindi[ref[:, 0] - 1] + lindj[ref[:, 1] - 1] + lindk[ref[:, 2] - 1] + ref[:, 3])
    rng = np.random.default_rng(2)
    t = rng.integers(1, 17, (100000, 8)).astype(np.int64)
    t[::2, 4:] = t[::2, :4][:, ::-1]
    got, _ = koopro.ord9(16, t)
    np.testing.assert_array_equal(got, orc.ord_tuples(16, 9, t))


@pytest.mark.parametrize("n,ne,metat,ndet", [(6, 6, 2, None), (8, 8, 1, None), (7, 5, 1, 200)])
def test_bro_chain(gpu_ctx, n, ne, metat, ndet):
    p = synth.make_problem(n, ne, 2, 3, metat=metat, ndet=ndet, seed=31)
    d3 = koopro.bro3(p.ro4, n, ne, metat)
    assert rel_err(d3, orc.bro3(p.ro4, n, ne, metat)) < 1e-13
    d2 = koopro.bro2(d3, n, ne, metat)
    assert rel_err(d2, orc.bro2(d3, n, ne, metat)) < 1e-13
    d1 = koopro.bro1(d2, n, ne, metat)
    assert rel_err(d1, orc.bro1(d2, n, ne, metat)) < 1e-13
    for s in range(metat):
        assert abs(np.trace(d1[s]) - ne) < 1e-11


def test_get_aj_atwo(gpu_ctx):
    p = synth.make_problem(6, 6, 5, 9, seed=4)
    atwo, aj = koopro.get_aj_atwo(6, 5, p.norb, p.oneint, p.chol)
    ratwo, raj = orc.get_aj_atwo(p.oneint, p.chol, 6, 5, p.norb)
    assert rel_err(atwo, ratwo) < 1e-13
    assert rel_err(aj, raj) < 1e-13


def _check_stage1(p, names=None):
    o = koopro.koopro4QD(p)
    r = orc.stage1(p)
    mapping = {"1-IPKO": "ipko1", "1-EAKO": "eako1", "2-HRDM": "hrdm2", "2-IPKO": "ipko2", "2-EAKO": "eako2",
               "gk0pa": "gk0pa", "gk0pd": "gk0pd", "gk0pf": "gk0pf"}
    for k, v in o.items():
        if k in ("3-RDM", "2-RDM", "1-RDM"):
            continue
        rk = mapping.get(k, k)
        if names and k not in names:
            continue
        assert rel_err(v, r[rk]) < TOL, (k, rel_err(v, r[rk]))


def test_stage1_random_ci_n6_two_states(gpu_ctx):
    _check_stage1(synth.make_problem(6, 6, 3, 4, metat=2, seed=7))


def test_stage1_open_shell_no_core(gpu_ctx):
    _check_stage1(synth.make_problem(5, 5, 0, 4, metat=1, seed=8))


@pytest.mark.parametrize("name", ["stage1_cas44", "stage1_cas54_m2"])
def test_stage1_golden(gpu_ctx, name):
    g = load_golden(name)
    n, ne, nc, nv = (int(g[k]) for k in ("nact", "nele", "ncore", "nvirt"))
    p = synth.with_ci(synth.make_problem(n, ne, nc, nv, seed=1), g["amask"], g["bmask"], g["coef"])
    p.oneint, p.chol = g["oneint"], np.asfortranarray(g["chol"])
    o = koopro.koopro4QD(p)
    for k, v in o.items():
        key = {"1-IPKO": "ipko1", "1-EAKO": "eako1", "2-HRDM": "hrdm2", "2-IPKO": "ipko2", "2-EAKO": "eako2"}.get(k, k)
        if "out_" + key in g:
            assert rel_err(v, g["out_" + key]) < TOL, k
    ip, ea = orc.fdiff(o["bmatIP"], o["cmatIP"], o["bmatEA"], o["cmatEA"], n, p.metat)
    assert ip.max() < 1e-11 and ea.max() < 1e-11
    assert orc.fdiff_F(o["gk0pf"], n, p.metat).max() < 1e-11


def test_stage1_cas8_config(gpu_ctx):
    """CAS(8,8), 4900 determinants, 10 inactive / 40 virtual orbitals."""
    _check_stage1(synth.config_problem("cas8"))


def test_f_scratch_is_overwritten_like_the_reference(gpu_ctx):
    p = synth.make_problem(5, 4, 2, 3, seed=3)
    atwo, aj = orc.get_aj_atwo(p.oneint, p.chol, 5, 2, p.norb)
    f_gpu = np.full(p.norb * (p.norb + 1) // 2, 7.0)
    f_ref = f_gpu.copy()
    koopro.bbmat(atwo, p.daaa, p.taa, p.dal, 5, 2, f_gpu, aj, 1)
    orc.bbmat(atwo, p.daaa, p.taa, p.dal, 5, 2, f_ref, aj, 1)
    np.testing.assert_allclose(f_gpu, f_ref, rtol=0, atol=1e-14)
    assert f_gpu[0] == 7.0  # outside the active triangle: untouched


def test_error_statuses(gpu_ctx):
    p = synth.make_problem(4, 4, 1, 2, seed=3)
    with pytest.raises(_native.NvptError) as e:
        koopro.bro3(p.ro4, 4, 3, 1)
    assert e.value.status == 1
    atwo, aj = orc.get_aj_atwo(p.oneint, p.chol, 4, 1, p.norb)
    f = np.zeros(p.norb * (p.norb + 1) // 2)
    with pytest.raises(_native.NvptError) as e:
        koopro.bamat(atwo, p.ro4, p.daaa, p.taa, p.dal, 4, 1, f, aj, p.norb, 1, nsym=2)
    assert e.value.status == 4
    with pytest.raises(_native.NvptError) as e:
        koopro.bro1(np.zeros((1,) + (17,) * 4, order="F"), 17, 5, 1)
    assert e.value.status == 1


def test_launch_counter_moves(gpu_ctx):
    before = gpu_ctx.launches
    p = synth.make_problem(4, 4, 1, 2, seed=3)
    koopro.bro3(p.ro4, 4, 4, 1)
    assert gpu_ctx.launches == before + 2  # bro3: the case-A pass and the transpose-add
