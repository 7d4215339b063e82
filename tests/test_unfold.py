"""QCMaquis label/value unfolding (src/rdm_utils.F90:236-511): the oracle's
restatement on hand-checked cases (CPU) and the GPU kernels against it, bit
for bit, including the overwrite order of colliding images (GPU)."""
import numpy as np
import pytest

from oracle import oracle as orc
from oracle.bruteforce import normind
from nevpt2_gb300 import synth


def _w(n):
    return n * (n + 1) * (n + 2) * (n + 3) // 24


def _ro4(n, fill=np.nan):
    return np.full((_w(n), n, n, n, n), fill, order="F")


def test_oracle_case5_default_single_image():
    n = 4
    ro4 = _ro4(n)
    # i,j,k,l all different (case 5), m,n,o,p generic -> one image
    orc.permute_4rdm(ro4, np.array([[3, 2, 1, 0, 0, 1, 3, 2]]), np.array([0.25]))
    written = np.argwhere(~np.isnan(ro4))
    assert len(written) == 1
    ind = normind(4, 3, 2, 1) - 1
    assert tuple(written[0]) == (ind, 0, 1, 3, 2) and ro4[ind, 0, 1, 3, 2] == 0.25


def test_oracle_case1_weights_and_threshold():
    n = 3
    ro4 = _ro4(n, 0.0)
    # i=j, k=l, m=n, o=p: 2 images of val and 4 of -val/2
    orc.permute_4rdm(ro4, np.array([[1, 1, 2, 2, 0, 0, 2, 2]]), np.array([2.0]))
    ind = normind(2, 2, 3, 3) - 1
    blk = ro4[ind]
    assert blk[0, 0, 2, 2] == 2.0 and blk[2, 2, 0, 0] == 2.0
    for a, b, c, d in [(0, 2, 2, 0), (0, 2, 0, 2), (2, 0, 0, 2), (2, 0, 2, 0)]:
        assert blk[a, b, c, d] == -1.0
    assert np.count_nonzero(ro4) == 6
    # below the 1e-12 threshold nothing is written
    ro4b = _ro4(n, 0.0)
    orc.permute_4rdm(ro4b, np.array([[1, 1, 2, 2, 0, 0, 2, 2]]), np.array([9e-13]))
    assert not ro4b.any()


def test_oracle_3rdm_negation_and_transition():
    n = 3
    r = np.zeros(n**6)
    orc.permute_3rdm(r, 1, n, np.array([[0, 1, 2, 2, 0, 1]]), np.array([0.5]), trans=False)
    a = r.reshape((n,) * 6, order="F")
    assert a[0, 1, 2, 2, 0, 1] == -0.5 and a[2, 0, 1, 0, 1, 2] == -0.5  # image and transpose image
    assert np.count_nonzero(r) == 12
    t = np.zeros(n**6)
    orc.permute_3rdm(t, 1, n, np.array([[0, 1, 2, 2, 0, 1]]), np.array([0.5]), trans=True)
    assert np.count_nonzero(t) == 6 and t.reshape((n,) * 6, order="F")[0, 1, 2, 2, 0, 1] == 0.5
    # i = j = k is skipped
    s = np.zeros(n**6)
    orc.permute_3rdm(s, 1, n, np.array([[1, 1, 1, 0, 2, 1]]), np.array([0.5]))
    assert not s.any()


def test_oracle_later_entry_overwrites():
    n = 3
    ro4 = _ro4(n, 0.0)
    lab = np.array([[2, 1, 0, 0, 0, 1, 2, 1], [2, 1, 0, 0, 0, 1, 2, 1]])
    orc.permute_4rdm(ro4, lab, np.array([1.0, 3.0]))
    assert set(np.unique(ro4[ro4 != 0])) <= {3.0}


# ----------------------------------------------------------------- GPU
def _labels(rng, n, k, ne):
    lab = rng.integers(0, n, (ne, k)).astype(np.int32)
    # plenty of coinciding indices: the case tables branch on them
    eq = rng.random((ne, k)) < 0.3
    lab[eq] = lab[np.nonzero(eq)[0], 0]
    return lab


@pytest.mark.gpu
@pytest.mark.parametrize("n,ne", [(3, 4000), (4, 20000), (8, 200000)])
def test_gpu_unfold4_matches_oracle_bitwise(n, ne):
    from nevpt2_gb300 import koopro
    rng = np.random.default_rng(n * 31 + ne)
    lab = _labels(rng, n, 8, ne)
    val = rng.standard_normal(ne)
    val[rng.random(ne) < 0.05] = 1e-13  # below the threshold
    ref, bad = orc.permute_4rdm(_ro4(n, -7.0), lab, val)
    assert bad == 0
    got = koopro.permute_4rdm(_ro4(n, -7.0), lab, val)
    assert np.array_equal(got, ref)


@pytest.mark.gpu
@pytest.mark.parametrize("trans", [False, True])
def test_gpu_unfold3_strided_matches_oracle_bitwise(trans):
    from nevpt2_gb300 import koopro
    n, M, ne = 5, 3, 30000
    rng = np.random.default_rng(11 + trans)
    lab = _labels(rng, n, 6, ne)
    val = rng.standard_normal(ne)
    base = rng.standard_normal((M,) + (n,) * 6)
    daaa = np.asfortranarray(base)
    ref = np.asfortranarray(base.copy()).reshape(-1, order="F").copy()
    orc.permute_3rdm(ref[1:], M, n, lab, val, trans=trans)
    got = koopro.permute_3rdm(daaa, lab, val, trans=trans, state=1)
    assert np.array_equal(got.reshape(-1, order="F"), ref)


@pytest.mark.gpu
def test_gpu_unfold_rejects_out_of_range_labels():
    from nevpt2_gb300 import koopro
    from nevpt2_gb300._native import NvptError
    with pytest.raises(NvptError) as e:
        koopro.permute_4rdm(_ro4(3), np.array([[0, 0, 0, 0, 0, 0, 0, 3]]), np.array([1.0]))
    assert e.value.status == 1
