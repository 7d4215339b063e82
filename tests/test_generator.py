"""Exact RDM generator: brute-force check and the partial-trace chain
(src/koopro4QD.F90:4881-5049 bro3/bro2/bro1)."""
import itertools

import numpy as np
import pytest

from nevpt2_gb300 import synth
from oracle import bruteforce as bf
from oracle import oracle as orc


@pytest.mark.parametrize("n,ne,ndet", [(3, 2, None), (4, 4, None), (4, 3, None), (5, 4, 40)])
def test_dense_rdms_match_bruteforce(n, ne, ndet):
    p = synth.make_problem(n, ne, 1, 2, metat=1, ndet=ndet, seed=3 + n)
    c = p.coef[:, 0]
    for k, arr in ((1, p.dal), (2, p.taa), (3, p.daaa)):
        ref = bf.spinfree_rdm(n, p.amask, p.bmask, c, c, k)
        assert np.abs(arr[0] - ref).max() < 1e-13


def test_packed_ro4_matches_bruteforce():
    n = 4
    p = synth.make_problem(n, 4, 1, 2, metat=1, seed=9)
    c = p.coef[:, 0]
    g4 = bf.spinfree_rdm(n, p.amask, p.bmask, c, c, 4)
    worst = 0.0
    for K in itertools.product(range(1, n + 1), repeat=4):
        if list(K) != sorted(K, reverse=True):
            continue
        ind = bf.lindice(*K)
        for L in itertools.product(range(1, n + 1), repeat=4):
            if bf.normind(*L) > ind:
                continue
            worst = max(worst, abs(p.ro4[(ind - 1,) + tuple(x - 1 for x in L) + (0,)] -
                                   g4[tuple(x - 1 for x in K) + tuple(x - 1 for x in L)]))
    assert worst < 1e-13


@pytest.mark.parametrize("n,ne,metat", [(5, 5, 1), (6, 6, 2)])
def test_partial_trace_chain_and_trace(n, ne, metat):
    p = synth.make_problem(n, ne, 1, 2, metat=metat, seed=21)
    d3 = orc.bro3(p.ro4, n, ne, metat)
    d2 = orc.bro2(p.daaa, n, ne, metat)
    d1 = orc.bro1(p.taa, n, ne, metat)
    assert np.abs(d3 - p.daaa).max() < 1e-13
    assert np.abs(d2 - p.taa).max() < 1e-13
    assert np.abs(d1 - p.dal).max() < 1e-13
    for s in range(metat):
        assert abs(np.trace(p.dal[s]) - ne) < 1e-12


def test_hermiticity_of_state_rdms():
    p = synth.make_problem(5, 4, 1, 2, metat=1, seed=4)
    n = 5
    np.testing.assert_allclose(p.dal[0], p.dal[0].T, atol=1e-14)
    t = p.taa[0]
    np.testing.assert_allclose(t, t.transpose(2, 3, 0, 1), atol=1e-14)
    d = p.daaa[0]
    np.testing.assert_allclose(d, d.transpose(3, 4, 5, 0, 1, 2), atol=1e-14)
    assert n == 5


def test_accessors_match_bruteforce_e_products():
    """eee2/eeee (src/eexx_functions.F90:25-94) equal <E E E (E)> products."""
    n = 4
    p = synth.make_problem(n, 4, 1, 2, metat=1, seed=13)
    rng = np.random.default_rng(0)
    c = p.coef[:, 0]
    for _ in range(40):
        idx = rng.integers(1, n + 1, 8)
        idx[2] = idx[1] if rng.random() < 0.4 else idx[2]
        idx[4] = idx[3] if rng.random() < 0.4 else idx[4]
        ref = bf.expect_e_product(n, p.amask, p.bmask, c, [(idx[0] - 1, idx[1] - 1), (idx[2] - 1, idx[3] - 1),
                                                           (idx[4] - 1, idx[5] - 1), (idx[6] - 1, idx[7] - 1)])
        got = orc.eeee_at(p.ro4, p.daaa, p.taa, p.dal, n, 1, idx, 1)
        assert abs(got - ref) < 1e-12
        ref3 = bf.expect_e_product(n, p.amask, p.bmask, c, [(idx[0] - 1, idx[1] - 1), (idx[2] - 1, idx[3] - 1),
                                                            (idx[4] - 1, idx[5] - 1)])
        got3 = orc.eee2_at(p.daaa, p.taa, p.dal, n, 1, idx[:6], 1)
        assert abs(got3 - ref3) < 1e-12
