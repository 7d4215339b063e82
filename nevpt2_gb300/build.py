"""Build recipe for the in-tree native libraries.

* ``libnvpt2.so``  - the CUDA library behind include/nvpt2.h, sm_103a only.
* ``librdmgen.so`` - host (OpenMP) generator of exact RDMs for synthetic inputs.

Both land next to this file so that the Python layer loads them from the
source tree.  ``nvcc`` cross-compiles for sm_103a without a GPU.
"""
from __future__ import annotations

import hashlib
import os
import platform
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"

CUDA_SOURCES = ["capi.cu", "koop_kernels.cu", "bamat.cu", "bamat_gemm.cu", "s2_tensor.cu", "tridiag.cu", "qdnevpt.cu", "ozaki.cu", "ozaki_wide.cu", "rdm_unfold.cu", "ijkl_sym.cu", "tuner.cu", "container.cpp", "rdm_build.cu"]
CUDA_HEADERS = ["eexx.cuh", "nvpt2_internal.h", "s2_tensor.cuh", "ozaki.cuh", "oz_ptx.cuh", "tuner.h"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libnvpt2.so")
    return cand


def _tool_version(tool: str) -> str:
    r = subprocess.run([tool, "--version"], capture_output=True, text=True)
    return r.stdout.strip()


def _stamp(deps: list[Path], tool: str, flags: list[str]) -> str:
    """What a library was built from: this machine's architecture and host
    name, the compiler's version, the flags, and the sources' contents."""
    h = hashlib.sha256()
    for part in (platform.machine(), platform.node(), _tool_version(tool), " ".join(flags)):
        h.update(part.encode() + b"\0")
    for d in deps:
        h.update(d.name.encode() + b"\0" + d.read_bytes())
    return h.hexdigest()


def _stale(target: Path, stamp: str) -> bool:
    """A library is rebuilt unless it exists with a stamp file that matches:
    a binary built elsewhere (another machine, compiler or source state) is
    never reused."""
    sfile = target.with_name(target.name + ".stamp")
    if not target.exists() or not sfile.exists():
        return True
    return sfile.read_text().strip() != stamp


def _write_stamp(target: Path, stamp: str) -> None:
    target.with_name(target.name + ".stamp").write_text(stamp + "\n")


def build_cuda(force: bool = False, verbose: bool = False) -> Path:
    out = PKG / "libnvpt2.so"
    deps = [CSRC / s for s in CUDA_SOURCES + CUDA_HEADERS] + [INCLUDE / "nvpt2.h"]
    nvcc = _nvcc()
    flags = [GENCODE, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
             f"-I{INCLUDE}", f"-I{CSRC}"]
    stamp = _stamp(deps, nvcc, flags)
    if not force and not _stale(out, stamp):
        return out
    objdir = PKG / "_build"
    objdir.mkdir(exist_ok=True)
    procs = []
    objs = []
    for src in CUDA_SOURCES:
        obj = objdir / (Path(src).stem + ".o")
        objs.append(obj)
        cmd = [nvcc, *flags, "-c", str(CSRC / src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    for cmd, p in procs:
        txt, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError(f"nvcc failed ({' '.join(cmd)}):\n{txt}")
        if verbose and txt:
            print(txt)
    tmp = out.with_suffix(".so.tmp")
    cmd = [nvcc, GENCODE, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart", "-lcublas", "-lcusolver"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {r.stdout}\n{r.stderr}")
    os.replace(tmp, out)
    _write_stamp(out, stamp)
    return out


def build_rdmgen(force: bool = False) -> Path:
    out = PKG / "librdmgen.so"
    src = CSRC / "rdmgen.cpp"
    flags = ["-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared"]
    stamp = _stamp([src], "g++", flags)
    if not force and not _stale(out, stamp):
        return out
    tmp = out.with_suffix(".so.tmp")
    cmd = ["g++", *flags, str(src), "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"g++ failed: {r.stdout}\n{r.stderr}")
    os.replace(tmp, out)
    _write_stamp(out, stamp)
    return out


def build_oracle(force: bool = False) -> Path:
    """The CPU oracle (test infrastructure, oracle/Makefile), rebuilt under
    the same stamp rule as the product libraries."""
    odir = PKG.parent / "oracle"
    out = odir / "_build" / "liboracle.so"
    stamp = _stamp([odir / "nvpt2_oracle.c", odir / "Makefile"], "gcc", [])
    if not force and not _stale(out, stamp):
        return out
    subprocess.run(["make", "-s", "-B", "-C", str(odir)], check=True)
    _write_stamp(out, stamp)
    return out


def build_all(force: bool = False, verbose: bool = False) -> None:
    build_rdmgen(force)
    build_cuda(force, verbose)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv, verbose="-v" in sys.argv)
