"""nvpt_bamat_static_d (the A-matrix builder whose scratch is a fixed device
array) against nvpt_bamat_d on the same device inputs, through the C ABI.

The entry exists for callers that cannot allocate device memory while a
Koopmans pass runs, so besides the results the test checks that a call takes
nothing from the device: the default memory pool's used-memory high-water
mark (what cudaMallocAsync draws on) stays at its level before the calls, the
pool reserves nothing new, and the device's free memory (cudaMalloc) does not
move across a call.

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


def _outputs(p, torch, dev):
    n, M = p.nact, p.metat
    amat = torch.full((M * n**6,), float("nan"), dtype=torch.float64, device=dev)
    atmat = torch.full((M * n**6,), float("nan"), dtype=torch.float64, device=dev)
    f = torch.zeros(p.norb * (p.norb + 1) // 2, dtype=torch.float64, device=dev)
    return amat, atmat, f


def _bamat(ctx, name, p, d, out):
    amat, atmat, f = out
    ctx.call(name, ptr(amat), ptr(atmat), ptr(d["atwo"]), ptr(d["ro4"]), ptr(d["daaa"]), ptr(d["taa"]),
             ptr(d["dal"]), p.nact, p.ncore, ptr(f), ptr(d["aj"]), p.norb, p.metat, 1, None)
    ctx.synchronize()
    return amat.cpu().numpy(), atmat.cpu().numpy(), f.cpu().numpy()


class _DevMem:
    """Driver-level view of device memory: the default pool's attributes
    (CU_MEMPOOL_ATTR_RESERVED_MEM_CURRENT = 5, USED_MEM_CURRENT = 7,
    USED_MEM_HIGH = 8) and cuMemGetInfo."""

    def __init__(self, device):
        self.cu = ctypes.CDLL("libcuda.so.1")
        self.pool = ctypes.c_void_p()
        dev = ctypes.c_int()
        assert self.cu.cuDeviceGet(ctypes.byref(dev), device) == 0
        assert self.cu.cuDeviceGetDefaultMemPool(ctypes.byref(self.pool), dev) == 0

    def attr(self, a):
        v = ctypes.c_uint64()
        assert self.cu.cuMemPoolGetAttribute(self.pool, a, ctypes.byref(v)) == 0
        return v.value

    def reset_high(self):
        z = ctypes.c_uint64(0)
        assert self.cu.cuMemPoolSetAttribute(self.pool, 8, ctypes.byref(z)) == 0

    def free_bytes(self):
        free, total = ctypes.c_size_t(), ctypes.c_size_t()
        assert self.cu.cuMemGetInfo_v2(ctypes.byref(free), ctypes.byref(total)) == 0
        return free.value


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("n,ne,nc,nv,metat,ndet", [(6, 6, 3, 4, 2, None), (8, 8, 4, 5, 1, 2000), (4, 4, 2, 3, 1, None)])
def test_static_scratch_matches_allocating_entry(n, ne, nc, nv, metat, ndet):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    p = synth.make_problem(n, ne, nc, nv, metat=metat, ndet=ndet, seed=77 + n)
    ctx, d, npair = _inputs(p, torch, dev)
    ref_a, ref_at, ref_f = _bamat(ctx, "nvpt_bamat_d", p, d, _outputs(p, torch, dev))
    out = _outputs(p, torch, dev)
    torch.cuda.synchronize()
    mem = _DevMem(0)
    mem.reset_high()
    used0, reserved0 = mem.attr(7), mem.attr(5)
    # two calls in a row: the second sees the scratch the first left behind
    for call in range(2):
        free0 = mem.free_bytes()
        a, at, f = _bamat(ctx, "nvpt_bamat_static_d", p, d, out)
        if call == 1:  # the first call may load the library's module on this device
            assert mem.free_bytes() == free0, "the no-allocation entry took device memory"
        assert np.isfinite(a).all() and np.isfinite(at).all()
        assert _rel(a, ref_a) <= TOL
        assert _rel(at, ref_at) <= TOL
        assert np.array_equal(f, ref_f)
        out[0].fill_(float("nan"))
        out[1].fill_(float("nan"))
    assert mem.attr(8) <= used0, "the no-allocation entry drew on the stream-ordered memory pool"
    assert mem.attr(5) <= reserved0
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
