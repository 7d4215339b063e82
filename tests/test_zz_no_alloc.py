"""nvpt_bamat_static_d (the A-matrix builder whose scratch is a fixed device
array) against nvpt_bamat_d on the same device inputs, through the C ABI.

Collected last so it runs both alone and after every other GPU test.
"""
import ctypes

import numpy as np
import pytest

from nevpt2_gb300 import synth
from nevpt2_gb300._native import Context, NvptError, ptr

pytestmark = pytest.mark.gpu

TOL = 1e-12  # relative to the array's largest element; only the summation order differs


def _inputs(p, torch, dev):
    flat = lambda a: torch.from_numpy(np.ascontiguousarray(np.asarray(a).reshape(-1, order="F"))).to(dev)
    n, M, nc = p.nact, p.metat, p.ncore
    ctx = Context(0)
    z = lambda k: torch.zeros(k, dtype=torch.float64, device=dev)
    d = {"ro4": flat(p.ro4), "daaa": flat(p.daaa), "taa": flat(p.taa), "dal": flat(p.dal),
         "oneint": flat(p.oneint), "chol": flat(p.chol), "atwo": z(n**4)}
    npair = p.norb * (p.norb + 1) // 2
    d["aj"] = z(npair)
    ctx.call("nvpt_get_aj_atwo_d", ptr(d["atwo"]), n, nc, p.norb, ptr(d["aj"]), ptr(d["oneint"]), ptr(d["chol"]),
             p.nchovec, None)
    return ctx, d, npair


def _bamat(ctx, name, p, d, npair, torch, dev):
    n, M = p.nact, p.metat
    amat = torch.full((M * n**6,), float("nan"), dtype=torch.float64, device=dev)
    atmat = torch.full((M * n**6,), float("nan"), dtype=torch.float64, device=dev)
    f = torch.zeros(npair, dtype=torch.float64, device=dev)
    ctx.call(name, ptr(amat), ptr(atmat), ptr(d["atwo"]), ptr(d["ro4"]), ptr(d["daaa"]), ptr(d["taa"]),
             ptr(d["dal"]), n, p.ncore, ptr(f), ptr(d["aj"]), p.norb, M, 1, None)
    ctx.synchronize()
    return amat.cpu().numpy(), atmat.cpu().numpy(), f.cpu().numpy()


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("n,ne,nc,nv,metat,ndet", [(6, 6, 3, 4, 2, None), (8, 8, 4, 5, 1, 2000), (4, 4, 2, 3, 1, None)])
def test_static_scratch_matches_allocating_entry(n, ne, nc, nv, metat, ndet):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    p = synth.make_problem(n, ne, nc, nv, metat=metat, ndet=ndet, seed=77 + n)
    ctx, d, npair = _inputs(p, torch, dev)
    ref_a, ref_at, ref_f = _bamat(ctx, "nvpt_bamat_d", p, d, npair, torch, dev)
    # two calls in a row: the second sees the scratch the first left behind
    for _ in range(2):
        a, at, f = _bamat(ctx, "nvpt_bamat_static_d", p, d, npair, torch, dev)
        assert np.isfinite(a).all() and np.isfinite(at).all()
        assert _rel(a, ref_a) <= TOL
        assert _rel(at, ref_at) <= TOL
        assert np.array_equal(f, ref_f)
    ctx.close()


def test_static_scratch_rejects_nact_above_limit():
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    ctx = Context(0)
    x = torch.zeros(8, dtype=torch.float64, device=dev)
    with pytest.raises(NvptError) as e:
        ctx.call("nvpt_bamat_static_d", ptr(x), ptr(x), ptr(x), ptr(x), ptr(x), ptr(x), ptr(x), 9, 1, ptr(x), ptr(x),
                 20, 1, 1, None)
    assert e.value.status == 1 and "static scratch limit of 8" in str(e.value)
    ctx.close()
