"""The dataset container that stands in for HDF5 (nvpt_h5c_*), the
QCMaquis label/value readers on it (src/rdm_utils.F90:69-227,522-614) and
the nevpt.h5 hand-off from stage 1 to stage 2 across a file."""
import numpy as np
import pytest

from nevpt2_gb300 import h5c
from nevpt2_gb300._native import NvptError
from oracle import oracle as orc


def test_roundtrip_types_shapes_and_replace(tmp_path):
    f = tmp_path / "nevpt.h5"
    rng = np.random.default_rng(0)
    a = np.asfortranarray(rng.standard_normal((2, 3, 4)))
    b = np.arange(12, dtype=np.int32).reshape(3, 4)
    c = np.arange(5, dtype=np.int64)
    h5c.write(f, "amatIP", a, append=False)
    h5c.write(f, "/spectrum/results/fourptdm/labels_num", b)
    h5c.write(f, "c", c)
    np.testing.assert_array_equal(h5c.read(f, "amatIP"), a)
    np.testing.assert_array_equal(h5c.read(f, "/spectrum/results/fourptdm/labels_num"), b)
    assert h5c.read(f, "c").dtype == np.int64 and h5c.info(f, "amatIP") == (np.dtype(np.float64), (2, 3, 4))
    h5c.write(f, "amatIP", 2 * a)  # a later dataset of the same name replaces the earlier one
    np.testing.assert_array_equal(h5c.read(f, "amatIP"), 2 * a)
    with pytest.raises(NvptError) as e:
        h5c.read(f, "missing")
    assert e.value.status == 1
    with pytest.raises(NvptError) as e:
        h5c.read(tmp_path / "nofile", "x")
    assert e.value.status == 6
    (tmp_path / "junk").write_bytes(b"not a container")
    with pytest.raises(NvptError) as e:
        h5c.read(tmp_path / "junk", "x")
    assert e.value.status == 6


# ----------------------------------------------------------------- GPU
def _labels(rng, n, k, ne):
    lab = rng.integers(0, n, (ne, k)).astype(np.int32)
    eq = rng.random((ne, k)) < 0.3
    lab[eq] = lab[np.nonzero(eq)[0], 0]
    return lab


@pytest.mark.gpu
def test_read_4rdm_from_resfile_matches_oracle(gpu_ctx, tmp_path):
    n, ne = 6, 20000
    rng = np.random.default_rng(1)
    lab, val = _labels(rng, n, 8, ne), rng.standard_normal(ne)
    f = tmp_path / "result.h5"
    h5c.write_qcmaquis_rdm(f, 4, lab, val)
    W = n * (n + 1) * (n + 2) * (n + 3) // 24
    got = np.zeros((W, n, n, n, n), order="F")
    assert h5c.read_rdm_from_resfile(gpu_ctx, f, 4, got, n) == ne
    ref, _ = orc.permute_4rdm(np.zeros((W, n, n, n, n), order="F"), lab, val)
    np.testing.assert_array_equal(got, ref)


@pytest.mark.gpu
@pytest.mark.parametrize("trans", [False, True])
def test_read_distributed_3rdm_matches_oracle(gpu_ctx, tmp_path, trans):
    n, ne = 5, 9000
    rng = np.random.default_rng(2 + trans)
    lab, val = _labels(rng, n, 6, ne), rng.standard_normal(ne)
    cuts = [0, 2500, 6000, ne]
    for i in range(3):  # three worker directories, one without a result file
        d = tmp_path / f"part{i}"
        d.mkdir()
        h5c.write_qcmaquis_rdm(d / "res.h5", 3, lab[cuts[i]:cuts[i + 1]], val[cuts[i]:cuts[i + 1]], trans=trans)
    (tmp_path / "part3").mkdir()
    got = np.zeros(n**6)
    h5c.read_distributed_rdm(gpu_ctx, tmp_path, "res.h5", 3, got, n, ne, trans=trans)
    ref, _ = orc.permute_3rdm(np.zeros(n**6), 1, n, lab, val, trans=trans)
    np.testing.assert_array_equal(got, ref)
    with pytest.raises(NvptError) as e:  # the reference stops on a count mismatch
        h5c.read_distributed_rdm(gpu_ctx, tmp_path, "res.h5", 3, np.zeros(n**6), n, ne + 1, trans=trans)
    assert e.value.status == 1 and "Mismatch" in str(e.value)


@pytest.mark.gpu
def test_wrong_label_rank_is_rejected(gpu_ctx, tmp_path):
    f = tmp_path / "r.h5"
    h5c.write_qcmaquis_rdm(f, 3, np.zeros((4, 6), np.int32), np.ones(4))
    h5c.write(f, "/spectrum/results/fourptdm/labels_num", np.zeros((6, 4), np.int32))
    h5c.write(f, "/spectrum/results/fourptdm/mean/value", np.ones(4))
    with pytest.raises(NvptError) as e:
        h5c.read_rdm_from_resfile(gpu_ctx, f, 4, np.zeros((15, 2, 2, 2, 2), order="F"), 2)
    assert "8 indices" in str(e.value)


@pytest.mark.gpu
def test_nevpt_h5_handoff_between_stages(gpu_ctx, tmp_path):
    """Stage 1 writes nevpt.h5, stage 2 reads it back (as when the two run as
    separate processes): the energies equal those of the in-memory hand-off."""
    from nevpt2_gb300 import koopro, synth
    from nevpt2_gb300 import qdnevpt as gq
    p = synth.make_problem(5, 4, 3, 6, metat=2, seed=21, with_trdm=True)
    koop = koopro.koopro4QD(p)
    direct = gq.qdnevpt(p, koop, transition=p.trdm)
    f = tmp_path / "nevpt.h5"
    h5c.write_nevpt_h5(f, koop, transition=p.trdm)
    back, tr = h5c.read_nevpt_h5(f)
    for k in h5c.NEVPT_H5_STAGE1:
        np.testing.assert_array_equal(back[k], koop[k])
    again = gq.qdnevpt(p, back, transition=tr)
    # (the device tridiagonalisation sums with atomics: equal to rounding)
    for name in ("e2mpp", "e2enp", "e2mp", "e2en", "psimp", "psien"):
        np.testing.assert_allclose(getattr(again, name), getattr(direct, name), rtol=1e-12, atol=1e-13)
