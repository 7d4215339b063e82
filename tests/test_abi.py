"""The C ABI library loads here (no GPU needed) and exports every symbol the
header declares."""
import ctypes
import subprocess

import pytest

from nevpt2_gb300 import _native, build


def test_library_builds_and_exports_header_symbols():
    path = build.build_cuda()
    lib = ctypes.CDLL(str(path))
    names = _native.header_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) <= set(_native._SIGS), set(names) - set(_native._SIGS)


def test_pure_host_entry_points():
    lib = _native.lib()
    assert lib.nvpt_nwords(16) == 3876
    assert lib.nvpt_status_string(0) == b"ok"
    assert lib.nvpt_status_string(4) == b"unsupported configuration"


def test_exports_are_c_symbols():
    out = subprocess.run(["nm", "-D", "--defined-only", str(_native.LIB_PATH)], capture_output=True, text=True).stdout
    for n in _native.header_functions():
        assert f" T {n}\n" in out, n


def test_ctypes_signatures_match_header():
    """Each ctypes prototype has the header's arity, with int64_t where the
    header says int64_t and pointers where it says pointers."""
    import ctypes as C
    protos = _native.header_prototypes()
    for name, params in protos.items():
        args, _ = _native._SIGS[name]
        assert len(args) == len(params), (name, len(args), len(params))
        for a, p in zip(args, params):
            if "*" in p:
                assert a in (C.c_void_p,) or getattr(a, "_type_", None) is not None, (name, p, a)
            elif p.startswith("int64_t"):
                assert a is C.c_int64, (name, p, a)
            elif p.startswith("int"):
                assert a is C.c_int, (name, p, a)
