"""Files of the path in the library's dataset container (include/nvpt2.h,
nvpt_h5c_*), which stands in for HDF5 where libhdf5 is absent: nevpt.h5,
the hand-off from stage 1 (src/koopro4QD.F90:305,369-418,473-477) to stage 2
(src/qdnevpt.F:792-853), and the QCMaquis result files whose 3-/4-RDM
label/value lists src/rdm_utils.F90:69-227 reads.  Arrays are stored with
their Fortran-order shapes and HDF5 dataset names."""
from __future__ import annotations

import ctypes
import os

import numpy as np

from ._native import NvptError, lib, ptr

_TYPES = {np.dtype(np.int32): 1, np.dtype(np.int64): 2, np.dtype(np.float64): 3}
_DTYPES = {v: k for k, v in _TYPES.items()}

# Stage-1 datasets of nevpt.h5 (src/koopro4QD.F90:305,369-418,473-477)
NEVPT_H5_STAGE1 = ("1-RDM", "2-RDM", "3-RDM", "1-IPKO", "1-EAKO", "2-HRDM", "2-IPKO", "2-EAKO", "gk0pa", "gk0pd",
                   "gk0pf", "amatIP", "amatEA", "bmatIP", "bmatEA", "cmatIP", "cmatEA", "dmatIP", "dmatEA")
NEVPT_H5_TRDM = ("1-TRDM", "2-TRDM", "3-TRDM")


def _chk(status: int, what: str) -> None:
    if status != 0:
        raise NvptError(status, what, "")


def write(path, name: str, a, append: bool = True) -> None:
    a = np.asarray(a)
    if a.dtype not in _TYPES:
        a = a.astype(np.float64)
    a = np.asfortranarray(a)
    dims = np.array(a.shape, dtype=np.int64)
    _chk(lib().nvpt_h5c_write(os.fsencode(path), name.encode(), _TYPES[a.dtype], a.ndim, ptr(dims), ptr(a),
                              int(append)), f"nvpt_h5c_write({name})")


def info(path, name: str):
    t, r = ctypes.c_int(), ctypes.c_int()
    dims = np.zeros(8, np.int64)
    _chk(lib().nvpt_h5c_info(os.fsencode(path), name.encode(), ctypes.byref(t), ctypes.byref(r), ptr(dims)),
         f"nvpt_h5c_info({name})")
    return _DTYPES[t.value], tuple(int(x) for x in dims[:r.value])


def read(path, name: str) -> np.ndarray:
    dt, shape = info(path, name)
    out = np.zeros(shape, dtype=dt, order="F")
    _chk(lib().nvpt_h5c_read(os.fsencode(path), name.encode(), ptr(out), out.nbytes), f"nvpt_h5c_read({name})")
    return out


def write_nevpt_h5(path, datasets: dict, transition=None) -> None:
    """Stage-1 results (keys = nevpt.h5 dataset names) and, for QD runs, the
    transition RDMs "1-TRDM".."3-TRDM" into a fresh file."""
    first = True
    for k in NEVPT_H5_STAGE1:
        if k in datasets:
            write(path, k, datasets[k], append=not first)
            first = False
    if transition is not None:
        for k, t in zip(NEVPT_H5_TRDM, transition):
            write(path, k, t)


def read_nevpt_h5(path) -> tuple[dict, tuple | None]:
    """(stage-1 datasets, transition RDMs or None) as written above."""
    out = {}
    for k in NEVPT_H5_STAGE1:
        try:
            out[k] = read(path, k)
        except NvptError:
            pass
    tr = []
    for k in NEVPT_H5_TRDM:
        try:
            tr.append(read(path, k))
        except NvptError:
            break
    return out, (tuple(tr) if len(tr) == 3 else None)


def write_qcmaquis_rdm(path, which: int, labels, values, trans: bool = False) -> None:
    """A QCMaquis result file with one RDM's label/value lists: labels
    (nentries, 8 or 6), 0-based, stored as labels_num (int32, (rank,
    nentries)); values as mean/value."""
    root = ("/spectrum/results/fourptdm" if which == 4 else
            "/spectrum/results/transition_threeptdm" if trans else "/spectrum/results/threeptdm")
    lab = np.ascontiguousarray(labels, dtype=np.int32)
    write(path, root + "/labels_num", lab.T, append=False)  # (rank, nentries) Fortran = label-major rows
    write(path, root + "/mean/value", np.asarray(values, dtype=np.float64))


def read_rdm_from_resfile(ctx, path, which: int, rdm: np.ndarray, nact: int, trans: bool = False, ld: int = 1) -> int:
    """src/rdm_utils.F90:69 on a container file, unfolding on the GPU into
    ``rdm`` (Fortran-ordered host array, updated in place)."""
    n = ctypes.c_int64()
    ctx.call("nvpt_read_rdm_from_resfile", os.fsencode(path), which, int(trans), ptr(rdm), ld, nact, ctypes.byref(n))
    return int(n.value)


def read_distributed_rdm(ctx, directory, result_name: str, which: int, rdm: np.ndarray, nact: int,
                         total_elements: int, trans: bool = False, ld: int = 1) -> None:
    """src/rdm_utils.F90:522 read_distributed_rdm on container files."""
    ctx.call("nvpt_read_distributed_rdm", os.fsencode(directory), result_name.encode(), which, int(trans), ptr(rdm),
             ld, nact, total_elements)
