"""First-order density and natural occupations (.NATORB, src/qdnevpt.F:
1240-1467): the PC classes' density blocks -- rhoir from (0'), rhoid from
(+1'), rhodr from (-1') -- on the device against the oracle's restatement of
the reference loops (e20pcont :4854-4975, e21pcont :5113-5191, e2m1pcont
:5326-5411), on the eigenpair route (small metrics) and on the resolvent route
of the order-n^3 pencils, where they become z^T (K + sig S)^-1 g_d sums over
extra right-hand sides.  Tolerance 1e-10 absolute or 1e-9 relative.

The blocks are in the canonical orbitals, whose signs are the eigensolver's
choice (cuSOLVER on the device, LAPACK in the oracle): a flipped orbital flips
its row or column of the density.  So the blocks are compared in magnitude,
and the natural occupations of the assembled density -- which do not depend
on those signs but do on every other sign -- as numbers."""
import numpy as np
import pytest

from nevpt2_gb300 import qdnevpt as gq
from nevpt2_gb300 import synth
from oracle import oracle as orc
from oracle import qdnevpt_oracle as q

pytestmark = pytest.mark.gpu
KOOP = {"ipko1": "1-IPKO", "eako1": "1-EAKO", "hrdm2": "2-HRDM", "ipko2": "2-IPKO", "eako2": "2-EAKO"}


def _both(p, mask=0xFF, frozen=None):
    o = {KOOP.get(k, k): v for k, v in orc.stage1(p).items()}
    o["1-RDM"], o["2-RDM"], o["3-RDM"] = p.dal, p.taa, p.daaa
    tr = synth.transition_rdms(p.nact, p.amask, p.bmask, p.coef) if p.metat > 1 else None
    inp = q.inputs_from(p, o, transition=None if tr is None else tuple(list(t) for t in tr))
    if frozen:
        inp.frozen = tuple(frozen)
    ref = q.qdnevpt(inp, classes=[k for k in range(8) if mask >> k & 1])
    got = gq.qdnevpt(p, o, transition=tr, class_mask=mask, frozen=frozen, rho1st=True)
    return ref, got


def _close(a, b, what):
    np.testing.assert_allclose(a, b, rtol=1e-9, atol=1e-10, err_msg=what)


def _close_magnitudes(got, ref, what):
    """Equal magnitudes; the signs are checked through the natural
    occupations of the assembled density (see _occupations), which change if
    the blocks' signs are not those of one flip per canonical orbital."""
    _close(np.abs(got), np.abs(ref), what + " (magnitudes)")


def _occupations(p, got, ref):
    rho, occ = gq.natural_orbitals(got, p.dal, p.ncore, p.nact, p.nvirt)
    rr = q.first_order_density(ref, [p.dal[s] for s in range(p.metat)], p.ncore, p.nact, p.nvirt)
    for s in range(p.metat):
        _close(occ[:, s], q.natural_occupations(rr[:, :, s]), "occupations")
        assert abs(occ[:, s].sum() - (2 * p.ncore + np.trace(p.dal[s]))) < 1e-10  # trace kept


@pytest.mark.parametrize("metat", [1, 2])
def test_density_blocks_eigenpair_route(gpu_ctx, metat):
    p = synth.make_problem(4, 4, 3, 5, metat=metat, seed=90 + metat)
    ref, got = _both(p)
    _close_magnitudes(got.rhoir, ref.rhoir, "rhoir")
    _close_magnitudes(got.rhoid, ref.rhoid, "rhoid")
    _close_magnitudes(got.rhodr, ref.rhodr, "rhodr")
    assert np.abs(got.rhoid).max() > 0 and np.abs(got.rhodr).max() > 0 and np.abs(got.rhoir).max() > 0
    _occupations(p, got, ref)


@pytest.mark.parametrize("metat", [1, 2])
def test_density_blocks_resolvent_route(gpu_ctx, metat):
    """n = 8: the (+-1') metrics have order 512 and take the resolvent route."""
    p = synth.make_problem(8, 8, 4, 12, metat=metat, ndet=None if metat == 1 else 2000, seed=70 + metat)
    ref, got = _both(p, mask=0x60)
    for s in range(metat):
        assert got.nnew[6, s] == 512 and got.nnew[7, s] == 512
    _close_magnitudes(got.rhoid, ref.rhoid, "rhoid")
    _close_magnitudes(got.rhodr, ref.rhodr, "rhodr")
    _occupations(p, got, ref)


def test_density_with_frozen_core(gpu_ctx):
    p = synth.make_problem(4, 4, 3, 4, metat=1, seed=12)
    ref, got = _both(p, frozen=[0])
    _close_magnitudes(got.rhoir, ref.rhoir, "rhoir")
    _close_magnitudes(got.rhoid, ref.rhoid, "rhoid")
    _occupations(p, got, ref)
    assert np.all(got.rhoir[0] == 0.0) and np.all(got.rhoid[0] == 0.0)
