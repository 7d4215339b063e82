"""Device-resident stage-1 pipeline.

Keeps every input and output of the Koopmans stage on the GPU (torch tensors
are used only as device allocations) and runs the reference driver's sequence
of builders (src/koopro4QD.F90:270-423) through the ``_d`` entry points of
the C ABI on one CUDA stream.
"""
from __future__ import annotations

import numpy as np
import torch

from ._native import Context, ptr


def _dev(a: np.ndarray, device) -> torch.Tensor:
    """Device copy of a Fortran-ordered array, flattened in Fortran order."""
    flat = np.asarray(a).reshape(-1, order="F")
    return torch.from_numpy(np.ascontiguousarray(flat)).to(device)


class Stage1:
    """All stage-1 buffers of one problem, resident on ``device``."""

    OUTPUTS_N2 = ("1-IPKO", "1-EAKO", "gk0pf", "dmatIP", "dmatEA")
    OUTPUTS_N4 = ("2-HRDM", "2-IPKO", "2-EAKO", "gk0pa", "gk0pd", "bmatIP", "bmatEA", "cmatIP", "cmatEA")
    OUTPUTS_N6 = ("amatIP", "amatEA")

    def __init__(self, problem, ctx: Context | None = None, device: str = "cuda:0"):
        p = problem
        self.p = p
        self.ctx = ctx or Context(torch.device(device).index or 0)
        self.device = torch.device(device)
        n, M = p.nact, p.metat
        self.ro4 = _dev(p.ro4, self.device)
        self.oneint = _dev(p.oneint, self.device)
        self.chol = _dev(p.chol, self.device)
        z = lambda k: torch.zeros(k, dtype=torch.float64, device=self.device)
        self.daaa, self.taa, self.dal = z(M * n**6), z(M * n**4), z(M * n**2)
        self.atwo = z(n**4)
        npair = p.norb * (p.norb + 1) // 2
        self.aj, self.f = z(npair), z(npair)
        self.out = {}
        for k in self.OUTPUTS_N2:
            self.out[k] = z(M * n**2)
        for k in self.OUTPUTS_N4:
            self.out[k] = z(M * n**4)
        for k in self.OUTPUTS_N6:
            self.out[k] = z(M * n**6)
        # transition RDMs of the root pairs (quasi-degenerate stage 2)
        self.trdm = tuple(_dev(t, self.device) for t in p.trdm) if (M > 1 and p.trdm is not None) else None

    def run(self, stream: torch.cuda.Stream | None = None) -> None:
        """Enqueue the whole stage on ``stream`` (default: torch's current)."""
        p, c, o = self.p, self.ctx, self.out
        st = ptr_stream(stream or torch.cuda.current_stream(self.device))
        n, M, nc, norb, ne = p.nact, p.metat, p.ncore, p.norb, p.nele
        c.call("nvpt_bro3_d", ptr(self.ro4), ptr(self.daaa), n, ne, M, st)
        c.call("nvpt_bro2_d", ptr(self.daaa), ptr(self.taa), n, ne, M, st)
        c.call("nvpt_bro1_d", ptr(self.taa), ptr(self.dal), n, ne, M, st)
        c.call("nvpt_get_aj_atwo_d", ptr(self.atwo), n, nc, norb, ptr(self.aj), ptr(self.oneint), ptr(self.chol),
               p.nchovec, st)
        c.call("nvpt_koop_matrices_ctl_d", M, n, nc, ptr(self.atwo), ptr(self.daaa), ptr(self.taa), ptr(self.dal),
               ptr(self.f), ptr(self.aj), *[ptr(o[k]) for k in ("1-IPKO", "1-EAKO", "2-HRDM", "2-IPKO", "2-EAKO",
                                                                 "gk0pa", "gk0pd", "gk0pf")], st)
        c.call("nvpt_bamat_d", ptr(o["amatIP"]), ptr(o["amatEA"]), ptr(self.atwo), ptr(self.ro4), ptr(self.daaa),
               ptr(self.taa), ptr(self.dal), n, nc, ptr(self.f), ptr(self.aj), norb, M, 1, st)
        c.call("nvpt_bbmat_d", ptr(self.atwo), ptr(o["bmatIP"]), ptr(o["bmatEA"]), ptr(self.daaa), ptr(self.taa),
               ptr(self.dal), n, nc, ptr(self.f), ptr(self.aj), M, st)
        c.call("nvpt_bcmat_d", ptr(self.atwo), ptr(o["cmatIP"]), ptr(o["cmatEA"]), ptr(self.daaa), ptr(self.taa),
               ptr(self.dal), n, nc, ptr(self.f), ptr(self.aj), M, st)
        c.call("nvpt_bdmat_d", ptr(self.atwo), ptr(o["dmatIP"]), ptr(o["dmatEA"]), ptr(self.taa), ptr(self.dal), n,
               nc, ptr(self.f), ptr(self.aj), M, st)

    def stage2(self, stream: torch.cuda.Stream | None = None, thr_lindep: float = 1e-6, class_mask: int = 0xFF):
        """Run the NEVPT2 energy stage on the resident stage-1 outputs
        (nvpt_qdnevpt_d), with the resident transition RDMs when metat > 1."""
        import ctypes

        from . import qdnevpt as gq
        p, o = self.p, self.out
        if p.metat > 1 and self.trdm is None:
            raise ValueError("a multi-state problem needs its transition RDMs (Problem.trdm)")
        gq._bind(self.ctx)
        st = ptr_stream(stream or torch.cuda.current_stream(self.device))
        inp = gq._In(p.ncore, p.nact, p.nvirt, p.metat, p.chol.shape[0], thr_lindep, 0, class_mask, None,
                     ptr(self.oneint), ptr(self.chol), ptr(self.dal), ptr(self.taa), ptr(self.daaa), ptr(o["2-HRDM"]),
                     ptr(o["1-IPKO"]), ptr(o["1-EAKO"]), ptr(o["2-IPKO"]), ptr(o["2-EAKO"]), ptr(o["gk0pa"]),
                     ptr(o["gk0pd"]), ptr(o["gk0pf"]), ptr(o["amatIP"]), ptr(o["amatEA"]), ptr(o["bmatIP"]),
                     ptr(o["bmatEA"]), ptr(o["cmatIP"]), ptr(o["cmatEA"]), ptr(o["dmatIP"]), ptr(o["dmatEA"]),
                     *((ptr(t) for t in self.trdm) if self.trdm is not None else (None, None, None)))
        M = p.metat
        res = gq.Stage2Energies(*(np.zeros((8, M), order="F") for _ in range(4)), np.zeros((M, M), order="F"),
                                np.zeros((M, M), order="F"), np.zeros(M), np.zeros(M),
                                np.zeros((p.norb, M), order="F"), np.zeros((10, M), np.int64, order="F"))
        out = gq._Out(*(ptr(getattr(res, k)) for k in ("e2mpp", "psimpp", "e2enp", "psienep", "e2mp", "e2en",
                                                         "psimp", "psien", "epsnew", "nnew")))
        self.ctx.check(self.ctx._lib.nvpt_qdnevpt_d(self.ctx.handle, ctypes.byref(inp), ctypes.byref(out), st),
                       "nvpt_qdnevpt_d")
        return res

    def result(self, name: str) -> np.ndarray:
        n, M = self.p.nact, self.p.metat
        t = self.out[name].cpu().numpy()
        k = {**{x: 2 for x in self.OUTPUTS_N2}, **{x: 4 for x in self.OUTPUTS_N4}, **{x: 6 for x in self.OUTPUTS_N6}}[name]
        return t.reshape((M,) + (n,) * k, order="F")


def ptr_stream(stream: torch.cuda.Stream):
    import ctypes
    return ctypes.c_void_p(stream.cuda_stream)
