"""Loader for the in-tree CUDA library ``libnvpt2.so`` (C ABI in include/nvpt2.h).

There is no CPU fallback: if the library is missing or no GPU is visible the
calls raise.
"""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libnvpt2.so"
HEADER = PKG.parent / "include" / "nvpt2.h"

I64 = ctypes.c_int64
P = ctypes.c_void_p

_lib = None


class NvptError(RuntimeError):
    def __init__(self, status: int, what: str, detail: str):
        super().__init__(f"{what} failed with status {status} ({STATUS.get(status, '?')}): {detail}")
        self.status = status


STATUS = {0: "NVPT_OK", 1: "NVPT_EINVAL", 2: "NVPT_ECUDA", 3: "NVPT_ENOMEM", 4: "NVPT_ENOTSUP", 5: "NVPT_ETIMEDOUT", 6: "NVPT_EIO"}


def header_prototypes() -> dict[str, list[str]]:
    """Every function include/nvpt2.h declares -> its parameter types."""
    txt = HEADER.read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    out = {}
    for m in re.finditer(r"\b(nvpt_\w+)\s*\(([^;{]*?)\)\s*;", txt, flags=re.S):
        params = [" ".join(x.split()) for x in m.group(2).split(",") if x.strip() and x.strip() != "void"]
        out[m.group(1)] = [re.sub(r"\s*\b\w+$", "", x) if not x.endswith("*") else x for x in params]
    return out


def header_functions() -> list[str]:
    """Every function name include/nvpt2.h declares."""
    return sorted(header_prototypes())


_SIGS = {
    "nvpt_create": ([ctypes.POINTER(P), ctypes.c_int], ctypes.c_int),
    "nvpt_destroy": ([P], ctypes.c_int),
    "nvpt_synchronize": ([P], ctypes.c_int),
    "nvpt_last_error": ([P], ctypes.c_char_p),
    "nvpt_status_string": ([ctypes.c_int], ctypes.c_char_p),
    "nvpt_launch_count": ([P], I64),
    "nvpt_nwords": ([I64], I64),
    "nvpt_ord8": ([P, I64, I64, P, P, P], ctypes.c_int),
    "nvpt_ord9": ([P, I64, I64, P, P, P], ctypes.c_int),
    "nvpt_bro3": ([P, P, P, I64, I64, I64], ctypes.c_int),
    "nvpt_bro2": ([P, P, P, I64, I64, I64], ctypes.c_int),
    "nvpt_bro1": ([P, P, P, I64, I64, I64], ctypes.c_int),
    "nvpt_get_aj_atwo": ([P, P, I64, I64, I64, P, P, P, I64], ctypes.c_int),
    "nvpt_koop_matrices_ctl": ([P, I64, I64, I64] + [P] * 14, ctypes.c_int),
    "nvpt_bamat": ([P] + [P] * 7 + [I64, I64, P, P, I64, I64, I64], ctypes.c_int),
    "nvpt_bbmat": ([P] + [P] * 6 + [I64, I64, P, P, I64], ctypes.c_int),
    "nvpt_bcmat": ([P] + [P] * 6 + [I64, I64, P, P, I64], ctypes.c_int),
    "nvpt_bdmat": ([P] + [P] * 5 + [I64, I64, P, P, I64], ctypes.c_int),
    "nvpt_bro3_d": ([P, P, P, I64, I64, I64, P], ctypes.c_int),
    "nvpt_bro2_d": ([P, P, P, I64, I64, I64, P], ctypes.c_int),
    "nvpt_bro1_d": ([P, P, P, I64, I64, I64, P], ctypes.c_int),
    "nvpt_get_aj_atwo_d": ([P, P, I64, I64, I64, P, P, P, I64, P], ctypes.c_int),
    "nvpt_koop_matrices_ctl_d": ([P, I64, I64, I64] + [P] * 14 + [P], ctypes.c_int),
    "nvpt_bamat_d": ([P] + [P] * 7 + [I64, I64, P, P, I64, I64, I64, P], ctypes.c_int),
    "nvpt_bamat_static_d": ([P] + [P] * 7 + [I64, I64, P, P, I64, I64, I64, P], ctypes.c_int),
    "nvpt_permute_4rdm": ([P, P, I64, P, P, I64], ctypes.c_int),
    "nvpt_permute_3rdm": ([P, P, I64, I64, P, P, I64, ctypes.c_int], ctypes.c_int),
    "nvpt_permute_4rdm_d": ([P, P, I64, P, P, I64, P], ctypes.c_int),
    "nvpt_permute_3rdm_d": ([P, P, I64, I64, P, P, I64, ctypes.c_int, P], ctypes.c_int),
    "nvpt_set_precision": ([P, ctypes.c_int], ctypes.c_int),
    "nvpt_get_precision": ([P], ctypes.c_int),
    "nvpt_dgemm_split_d": ([P, I64, I64, I64, P, P, P, P], ctypes.c_int),
    "nvpt_sytrd_d": ([P, I64, P, P, P, P, P], ctypes.c_int),
    "nvpt_dgemm_split_ex_d": ([P, ctypes.c_int, ctypes.c_int, I64, I64, I64, ctypes.c_double, P, I64, P, I64,
                               ctypes.c_double, P, I64, P], ctypes.c_int),
    "nvpt_set_profiling": ([P, ctypes.c_int], ctypes.c_int),
    "nvpt_profile_read": ([P, ctypes.c_char_p, P, P, P], ctypes.c_int),
    "nvpt_bbmat_d": ([P] + [P] * 6 + [I64, I64, P, P, I64, P], ctypes.c_int),
    "nvpt_bcmat_d": ([P] + [P] * 6 + [I64, I64, P, P, I64, P], ctypes.c_int),
    "nvpt_bdmat_d": ([P] + [P] * 5 + [I64, I64, P, P, I64, P], ctypes.c_int),
    "nvpt_set_autotune": ([P, ctypes.c_int], ctypes.c_int),
    "nvpt_set_wait_limit": ([P, I64], ctypes.c_int),
    "nvpt_set_pc_route": ([P, ctypes.c_int], ctypes.c_int),
    "nvpt_autotune_report": ([P, ctypes.c_char_p, I64], I64),
    "nvpt_h5c_write": ([ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int, P, P, ctypes.c_int],
                       ctypes.c_int),
    "nvpt_h5c_info": ([ctypes.c_char_p, ctypes.c_char_p, P, P, P], ctypes.c_int),
    "nvpt_h5c_read": ([ctypes.c_char_p, ctypes.c_char_p, P, I64], ctypes.c_int),
    "nvpt_h5c_list_dir": ([ctypes.c_char_p, ctypes.c_char_p, I64], ctypes.c_int),
    "nvpt_read_rdm_from_resfile": ([P, ctypes.c_char_p, ctypes.c_int, ctypes.c_int, P, I64, I64, P], ctypes.c_int),
    "nvpt_read_distributed_rdm": ([P, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int, P, I64, I64,
                                   I64], ctypes.c_int),
    "nvpt_rdm_dense_d": ([P, I64, I64, I64, P, P, P, I64, I64, I64, P, I64, I64, P], ctypes.c_int),
    "nvpt_rofour_d": ([P, I64, I64, P, P, P, I64, I64, P, P], ctypes.c_int),
    "nvpt_ijkl_init": ([P, I64, P, P, P, P], ctypes.c_int),
    "nvpt_ijkl_tables": ([P] + [P] * 8, ctypes.c_int),
    "nvpt_ijkl_set_twoint": ([P, P], ctypes.c_int),
    "nvpt_ai_twoint": ([P, I64, P, P], ctypes.c_int),
    "nvpt_get_aj_atwo_twoint": ([P, P, I64, I64, I64, P, P], ctypes.c_int),
    "nvpt_get_aj_atwo_twoint_d": ([P, P, I64, I64, I64, P, P, P], ctypes.c_int),
    # stage 2: struct pointers (nevpt2_gb300.qdnevpt rebinds them with typed structs)
    "nvpt_qdnevpt": ([P, P, P], ctypes.c_int),
    "nvpt_qdnevpt_d": ([P, P, P, P], ctypes.c_int),
}


def lib():
    """Load libnvpt2.so (building it if the tree has no copy yet)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            from . import build
            build.build_cuda()
        L = ctypes.CDLL(str(LIB_PATH))
        for name, (args, res) in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def ptr(a) -> P | None:
    """Address of a numpy array or a torch tensor (host or device)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return P(a.ctypes.data)
    return P(a.data_ptr())


class Context:
    """Owns one nvpt_context (a CUDA device and stream)."""

    def __init__(self, device: int = 0):
        self._lib = lib()
        h = P()
        st = self._lib.nvpt_create(ctypes.byref(h), device)
        if st != 0:
            raise NvptError(st, "nvpt_create", "no usable CUDA device (the library has no CPU fallback)")
        self.handle = h

    def check(self, status: int, what: str) -> None:
        if status != 0:
            detail = self._lib.nvpt_last_error(self.handle)
            raise NvptError(status, what, detail.decode() if detail else "")

    def call(self, name: str, *args) -> None:
        self.check(getattr(self._lib, name)(self.handle, *args), name)

    def synchronize(self) -> None:
        self.call("nvpt_synchronize")

    def autotune(self, on: bool = True) -> None:
        """nvpt_set_autotune: tune the launch parameters of new shapes."""
        self.call("nvpt_set_autotune", 1 if on else 0)

    def pc_route(self, mode: int) -> None:
        """nvpt_set_pc_route: 0 = resolvents for the order-n^3 (+-1') pencils
        only (default), 1 = for every PC class whose metric is kept whole."""
        self.call("nvpt_set_pc_route", int(mode))

    def autotune_report(self) -> dict:
        """The tuned choices (nvpt_autotune_report) as a dict."""
        import json
        n = int(self._lib.nvpt_autotune_report(self.handle, None, 0))
        buf = ctypes.create_string_buffer(n)
        self._lib.nvpt_autotune_report(self.handle, buf, n)
        return json.loads(buf.value.decode() or "{}")

    @property
    def launches(self) -> int:
        return int(self._lib.nvpt_launch_count(self.handle))

    def close(self) -> None:
        if getattr(self, "handle", None):
            self._lib.nvpt_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
