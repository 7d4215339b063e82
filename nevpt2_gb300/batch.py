"""Batched quasi-degenerate NEVPT2 over many independent problems of uneven
size (the reference runs koopro4QD_driver + qdnevpt once per problem,
src/koopro4QD.F90:270-423 and src/qdnevpt.F:858-993; here a batch of them
shares one GPU).

Every problem keeps its stage-1 inputs and outputs resident in HBM
(``pipeline.Stage1``).  A pool of workers, each with its own context (CUDA
stream) and host thread, takes problems from a shared queue, largest first,
and runs stage 1 and stage 2 back to back on its stream; the problems of
different workers overlap on the GPU, and inside a problem the states and
perturber classes already run on their own streams.  The number of workers is
a schedule parameter chosen by ``tune_workers`` (timed on a sample of the
batch); kernel launch parameters are tuned by the library
(``nvpt_set_autotune``)."""
from __future__ import annotations

import threading
import time

import torch

from ._native import Context
from .pipeline import Stage1


class Batch:
    def __init__(self, problems, device: str = "cuda:0", workers: int = 4):
        self.problems = list(problems)
        self.device = torch.device(device)
        self.ctxs: list[Context] = []
        self.streams: list[torch.cuda.Stream] = []
        self._ensure_workers(workers)
        self.workers = workers
        # resident buffers per problem, bound to worker contexts at run time
        self.pipes = [Stage1(p, ctx=self.ctxs[0], device=device) for p in self.problems]
        # largest problems first (n^9 stage 1, n^3-order pencils in stage 2)
        self.order = sorted(range(len(self.problems)), key=lambda i: -self._cost(self.problems[i]))

    @staticmethod
    def _cost(p) -> float:
        return p.metat * (p.nact ** 9 + 2.0 * p.nact ** 9 + (p.ncore + p.nvirt) * p.nact ** 6)

    def _ensure_workers(self, k: int) -> None:
        while len(self.ctxs) < k:
            self.ctxs.append(Context(self.device.index or 0))
            self.streams.append(torch.cuda.Stream(self.device))

    def set_precision(self, mode: int) -> None:
        for c in self.ctxs:
            c.call("nvpt_set_precision", mode)

    def run(self, subset=None, workers: int | None = None):
        """Stage 1 + stage 2 of every problem (or of ``subset``, indices);
        returns {problem index: Stage2Energies}."""
        k = workers or self.workers
        self._ensure_workers(k)
        todo = [i for i in self.order if subset is None or i in set(subset)]
        lock = threading.Lock()
        out, errors = {}, []

        def worker(w: int):
            ctx, st = self.ctxs[w], self.streams[w]
            torch.cuda.set_device(self.device)
            while True:
                with lock:
                    if not todo or errors:
                        return
                    i = todo.pop(0)
                try:
                    pipe = self.pipes[i]
                    pipe.ctx = ctx
                    with torch.cuda.stream(st):
                        pipe.run(st)
                        e = pipe.stage2(st)
                    with lock:
                        out[i] = e
                except Exception as ex:  # surfaced after the join
                    with lock:
                        errors.append(ex)
                    return

        th = [threading.Thread(target=worker, args=(w,)) for w in range(k)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        if errors:
            raise errors[0]
        torch.cuda.synchronize(self.device)
        return out

    def tune_workers(self, candidates=(1, 2, 4, 8), sample: int = 8) -> dict:
        """Schedule tuning: time the first ``sample`` problems of the batch
        order at each worker count and keep the fastest."""
        sub = self.order[:sample]
        self.run(sub, workers=max(candidates))  # warm: kernel tuning, module loads, handle pools
        times = {}
        for k in candidates:
            torch.cuda.synchronize(self.device)
            t0 = time.perf_counter()
            self.run(sub, workers=k)
            times[k] = time.perf_counter() - t0
        self.workers = min(times, key=times.get)
        return {"workers": self.workers, "sample_problems": len(sub),
                "seconds_per_candidate": {str(k): round(v, 4) for k, v in times.items()}}
