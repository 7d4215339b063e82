"""The batched configuration (nevpt2_gb300.batch): four of its 64 problems
(CAS(6,6), CAS(8,8) and two CAS(10,10), 3 roots each, uneven inactive and
virtual spaces) run through the batch runner with two workers, then each is
checked against the oracle the way the benchmark configurations are:
stage-1 builders in full, bamat on sampled slabs, stage 2 on the same
Koopmans matrices.  Tolerances as in test_parity_configs_gpu."""
import numpy as np
import pytest

import test_parity_configs_gpu as cfg
from nevpt2_gb300 import synth

pytestmark = pytest.mark.gpu
PICK = [1, 2, 4, 5]  # of the first eight problems: nact 8, 10, 10, 6


@pytest.fixture(scope="module")
def batch():
    from nevpt2_gb300.batch import Batch
    sel = [synth.batch_problems(1, first=i)[0] for i in PICK]
    b = Batch(sel, workers=2)
    out = b.run()
    return b, sel, out


def test_batch_runs_every_problem(gpu_ctx, batch):
    b, sel, out = batch
    assert sorted(out) == list(range(len(sel)))
    assert sorted({p.nact for p in sel}) == [6, 8, 10]


@pytest.mark.parametrize("k", range(len(PICK)))
def test_batch_problem_against_oracle(gpu_ctx, batch, k):
    b, sel, out = batch
    p = sel[k]
    pipe = b.pipes[k]
    got = {name: pipe.result(name) for name in pipe.out}
    got["3-RDM"] = pipe.daaa.cpu().numpy().reshape((p.metat,) + (p.nact,) * 6, order="F")
    got["atwo"] = pipe.atwo.cpu().numpy().reshape((p.nact,) * 4, order="F")
    cfg._check_builders(got, cfg._oracle_stage1_but_bamat(p), p.metat)
    n = p.nact
    cfg._check_bamat_slabs(p, got, [0, n + 3, n * n - 1], [0, 2])
    e = out[k]
    koop = {name: got[name] for name in pipe.out}
    koop["1-RDM"], koop["2-RDM"], koop["3-RDM"] = p.dal, p.taa, p.daaa
    from oracle import qdnevpt_oracle as q
    ref = q.qdnevpt(q.inputs_from(p, koop, transition=tuple(list(t) for t in p.trdm)))
    for name in ("e2mpp", "psimpp", "e2enp", "psienep", "e2mp", "e2en"):
        rtol = cfg.NORM_RTOL if name.startswith("psi") else cfg.ERTOL
        np.testing.assert_allclose(getattr(e, name), getattr(ref, name), rtol=rtol, atol=cfg.ETOL, err_msg=name)
