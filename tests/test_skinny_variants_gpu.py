"""Each variant of the FP64 slab product behind bamat (DFMA register blocks
of 2 or 4 rows per thread, DMMA tensor-core fragments) against the oracle's
bamat.  A variant is fixed per process by NVPT_SKINNY_VARIANT, so each runs
in a child process.  Tolerance 1e-10 relative to the array's largest
element."""
import os
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]

CHILD = r"""
import sys, numpy as np
sys.path.insert(0, {root!r})
from nevpt2_gb300 import koopro, synth
from oracle import oracle as orc
p = synth.make_problem(7, 6, 2, 3, metat=2, ndet=600, seed=17)
atwo, aj = orc.get_aj_atwo(p.oneint, p.chol, 7, 2, p.norb)
f = np.zeros(p.norb * (p.norb + 1) // 2)
A, At = orc.bamat(atwo, p.ro4, p.daaa, p.taa, p.dal, 7, 2, f, aj, p.norb, 2)
g = np.zeros_like(f)
B, Bt = koopro.bamat(atwo, p.ro4, p.daaa, p.taa, p.dal, 7, 2, g, aj, p.norb, 2)
print(max(np.abs(A - B).max() / np.abs(A).max(), np.abs(At - Bt).max() / np.abs(At).max()))
"""


@pytest.mark.parametrize("variant", ["1", "2", "4"])
def test_skinny_variant_against_oracle(variant):
    env = dict(os.environ, NVPT_SKINNY_VARIANT=variant)
    r = subprocess.run([sys.executable, "-c", CHILD.format(root=str(ROOT))], env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert float(r.stdout.strip().splitlines()[-1]) < 1e-10
