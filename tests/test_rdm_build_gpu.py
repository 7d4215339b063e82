"""The device RDM builder (nvpt_rdm_dense_d, nvpt_rofour_d: the role of the
reference's rofour/ro3/ro2/ro1 and *off builders, src/koopro4QD.F90:921-3013)
against explicit second quantisation (oracle/bruteforce.py) on small
expansions and against the host generator at larger ones.  Tolerance 1e-13
absolute (the sums run in another order)."""
import itertools

import numpy as np
import pytest

from nevpt2_gb300 import synth
from oracle import bruteforce as bf

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,ne,ndet,metat", [(4, 4, None, 1), (5, 4, 40, 2), (3, 2, None, 2)])
def test_device_rdms_match_bruteforce(gpu_ctx, n, ne, ndet, metat):
    p = synth.make_problem(n, ne, 1, 2, metat=metat, ndet=ndet, seed=3 + n)
    dal, taa, daaa, ro4, tr = synth.rdms_device(n, p.amask, p.bmask, p.coef, transition=True, ctx=gpu_ctx)
    for s in range(metat):
        c = p.coef[:, s]
        for k, arr in ((1, dal), (2, taa), (3, daaa)):
            assert np.abs(arr[s] - bf.spinfree_rdm(n, p.amask, p.bmask, c, c, k)).max() < 1e-13
    if metat > 1:
        c0, c1 = p.coef[:, 0], p.coef[:, 1]
        for k, arr in zip((1, 2, 3), tr):
            assert np.abs(arr[0] - bf.spinfree_rdm(n, p.amask, p.bmask, c0, c1, k)).max() < 1e-13
    if ne >= 4:
        g4 = bf.spinfree_rdm(n, p.amask, p.bmask, p.coef[:, 0], p.coef[:, 0], 4)
        worst = 0.0
        for K in itertools.product(range(1, n + 1), repeat=4):
            if list(K) != sorted(K, reverse=True):
                continue
            ind = bf.lindice(*K)
            for L in itertools.product(range(1, n + 1), repeat=4):
                if bf.normind(*L) > ind:
                    continue
                worst = max(worst, abs(ro4[(ind - 1,) + tuple(x - 1 for x in L) + (0,)] -
                                       g4[tuple(x - 1 for x in K) + tuple(x - 1 for x in L)]))
        assert worst < 1e-13


@pytest.mark.parametrize("n,ndet,metat", [(8, 2000, 2), (12, 3000, 1)])
def test_device_rdms_match_host_generator(gpu_ctx, n, ndet, metat):
    p = synth.make_problem(n, n, 1, 2, metat=metat, ndet=ndet, seed=50 + n, with_trdm=metat > 1)
    dal, taa, daaa, ro4, tr = synth.rdms_device(n, p.amask, p.bmask, p.coef, transition=True, ctx=gpu_ctx)
    for got, ref in ((dal, p.dal), (taa, p.taa), (daaa, p.daaa), (ro4, p.ro4)):
        assert np.abs(got - ref).max() < 1e-13
    if metat > 1:
        for got, ref in zip(tr, p.trdm):
            assert np.abs(got - ref).max() < 1e-13
