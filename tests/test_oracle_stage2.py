"""Stage-2 oracle: the vectorised restatement against the literal
loop-by-loop transliteration, and the reference's own invariants."""
import numpy as np
import pytest

from nevpt2_gb300 import synth
from oracle import oracle as orc
from oracle import qdnevpt_loops as ql
from oracle import qdnevpt_oracle as q

KOOP_NAMES = {"ipko1": "1-IPKO", "eako1": "1-EAKO", "hrdm2": "2-HRDM", "ipko2": "2-IPKO", "eako2": "2-EAKO"}


def stage2_inputs(p, thr=1e-6):
    o = {KOOP_NAMES.get(k, k): v for k, v in orc.stage1(p).items()}
    tr = None
    if p.metat > 1:
        tr = tuple(list(t) for t in synth.transition_rdms(p.nact, p.amask, p.bmask, p.coef))
    return q.inputs_from(p, o, thr_lindep=thr, transition=tr)


@pytest.mark.parametrize("n,ne,nc,nv,M,seed", [(3, 2, 2, 3, 1, 5), (4, 4, 2, 3, 1, 6), (3, 3, 2, 2, 2, 7),
                                             (4, 4, 1, 2, 2, 8), (3, 4, 0, 2, 1, 9)])
def test_vectorised_matches_literal_loops(n, ne, nc, nv, M, seed):
    inp = stage2_inputs(synth.make_problem(n, ne, nc, nv, metat=M, seed=seed))
    rv = q.qdnevpt(inp)
    rl = ql.qdnevpt_loops(inp)
    for name in ("e2mpp", "psimpp", "e2enp", "psienep", "e2mp", "e2en", "psimp", "psien"):
        np.testing.assert_allclose(getattr(rv, name), getattr(rl, name), rtol=0, atol=1e-12, err_msg=name)


def test_class0_sc_equals_pc_and_totals():
    inp = stage2_inputs(synth.make_problem(5, 4, 3, 4, metat=1, seed=3))
    r = q.qdnevpt(inp)
    assert r.e2mpp[0, 0] == r.e2enp[0, 0]
    assert abs(r.e2mp[0, 0] - r.e2mpp[:, 0].sum()) < 1e-13
    assert abs(r.e2en[0, 0] - r.e2enp[:, 0].sum()) < 1e-13
    assert abs(r.psien[0] - r.psienep[:, 0].sum()) < 1e-13


def test_pc_metric_ranks_are_integers_and_bounded():
    inp = stage2_inputs(synth.make_problem(4, 4, 2, 3, metat=1, seed=11))
    r = q.qdnevpt(inp)
    n = 4
    bounds = {1: n, 2: n, 7: 2 * n * n, 6: n ** 3, 5: n ** 3}
    for key, v in r.nnew.items():
        cls = key[0]
        if cls in bounds:
            assert 0 < v <= bounds[cls]


def test_fock_spectrum_is_the_target():
    """The generator's h1 makes the rebuilt core/virtual Fock operators of
    root 1 reproduce the target orbital energies up to the N(0,1e-3)
    off-diagonal coupling."""
    p = synth.make_problem(4, 4, 3, 5, metat=1, seed=2)
    inp = stage2_inputs(p)
    r = q.qdnevpt(inp, classes=())
    core = slice(0, 3)
    virt = slice(7, 12)
    assert np.abs(r.epsnew[core, 0] - p.eps[core]).max() < 1e-2
    assert np.abs(r.epsnew[virt, 0] - p.eps[virt]).max() < 1e-2
