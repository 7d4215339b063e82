"""Regenerates the committed golden fixtures of tests/golden/.

The reference (qcscine/nevpt2) ships no tests, sample inputs or outputs, so
these fixtures are produced by the CPU oracle of this repository on seeded
problems whose RDMs are checked against a brute-force second-quantised
evaluation, and whose CI vectors are CASCI eigenstates of the active
Hamiltonian (the reference's run-time invariants fdiff / fdiff_F hold on
them).  They pin the oracle and the CUDA path against regressions.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import itertools
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from nevpt2_gb300 import synth  # noqa: E402
from oracle import bruteforce as bf  # noqa: E402
from oracle import oracle as orc  # noqa: E402

OUT = Path(__file__).resolve().parent


def casci_problem(n, ne, nc, nv, nroots, seed):
    p = synth.make_problem(n, ne, nc, nv, metat=1, seed=seed)
    atwo, aj = orc.get_aj_atwo(p.oneint, p.chol, n, nc, p.norb)
    h = np.array([[aj[synth.tri(a + nc + 1, b + nc + 1) - 1] for b in range(n)] for a in range(n)])
    am, bm, C, E = bf.casci(n, ne - ne // 2, ne // 2, h, np.asarray(atwo), nroots=nroots)
    return synth.with_ci(p, am, bm, C), E


def index_maps():
    n = 4
    tuples = np.array(list(itertools.product(range(1, n + 1), repeat=8)), dtype=np.int64)
    rng = np.random.default_rng(5)
    sel = tuples[rng.choice(len(tuples), 8000, replace=False)]
    o8 = orc.ord_tuples(n, 8, sel)
    o9 = orc.ord_tuples(n, 9, sel)
    lindi, lindj, lindk, normind = orc.index_tables(5)
    np.savez_compressed(OUT / "index_maps.npz", tuples=sel.astype(np.int8), ord8=o8.astype(np.int8),
                        ord9=o9.astype(np.int8), lindi=lindi, lindj=lindj, lindk=lindk,
                        normind5=normind)


def stage1_case(name, n, ne, nc, nv, nroots, seed):
    p, E = casci_problem(n, ne, nc, nv, nroots, seed)
    o = orc.stage1(p)
    d = dict(nact=n, nele=ne, ncore=nc, nvirt=nv, metat=p.metat, amask=p.amask, bmask=p.bmask, coef=p.coef,
             oneint=p.oneint, chol=p.chol, casci_energies=E)
    for k, v in o.items():
        d["out_" + k] = v
    np.savez_compressed(OUT / f"{name}.npz", **d)


if __name__ == "__main__":
    index_maps()
    stage1_case("stage1_cas44", 4, 4, 2, 3, 1, 101)
    stage1_case("stage1_cas54_m2", 5, 4, 1, 3, 2, 102)
    print("written:", sorted(p.name for p in OUT.glob("*.npz")))
