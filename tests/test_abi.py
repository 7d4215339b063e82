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


def test_struct_layouts_match_header(tmp_path):
    """ctypes mirrors of the stage-2 structs agree with the C compiler's
    layout of include/nvpt2.h."""
    import ctypes as C

    from nevpt2_gb300 import qdnevpt as gq
    src = tmp_path / "layout.c"
    fields_in = [f for f, _ in gq._In._fields_]
    fields_out = [f for f, _ in gq._Out._fields_]
    body = "\n".join([f'printf("in {f} %zu\\n", offsetof(nvpt_qdnevpt_in, {f}));' for f in fields_in] +
                     [f'printf("out {f} %zu\\n", offsetof(nvpt_qdnevpt_out, {f}));' for f in fields_out])
    src.write_text(f'#include <stdio.h>\n#include <stddef.h>\n#include "nvpt2.h"\nint main(void){{\n'
                   f'printf("size_in %zu\\nsize_out %zu\\n", sizeof(nvpt_qdnevpt_in), sizeof(nvpt_qdnevpt_out));\n'
                   f'{body}\nreturn 0;}}\n')
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", str(_native.HEADER.parent), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {" ".join(l.split()[:-1]): int(l.split()[-1]) for l in out if l.strip()}
    assert got["size_in"] == C.sizeof(gq._In)
    assert got["size_out"] == C.sizeof(gq._Out)
    for f in fields_in:
        assert got[f"in {f}"] == getattr(gq._In, f).offset, f
    for f in fields_out:
        assert got[f"out {f}"] == getattr(gq._Out, f).offset, f
