"""Build recipe for the GB300 MPFA-O library and the CPU oracle.

``build_library()`` compiles the C++ host code and the CUDA kernels with nvcc
for sm_103a into ``tdycore_gb300/_lib/libtdycore_gb300.so`` (in-tree, static
CUDA runtime, so the shared object only needs the driver).  ``build_oracle()``
compiles the C restatement used by the tests into ``oracle/_build``.
Translation units compile in parallel; objects are rebuilt only when a source
or header is newer.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "_lib"
LIB = LIBDIR / "libtdycore_gb300.so"
ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "_build" / "libmpfao_oracle.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O3", "--expt-relaxed-constexpr"]
SOURCES = ["tdy_mesh.cpp", "tdy_setup.cpp", "tdy_api.cpp", "tdy_kernels.cu", "tdy_setup_kernels.cu", "tdy_solver.cu"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build tdycore_gb300")


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def _headers():
    return list(CSRC.glob("*.h")) + list((ROOT / "include").glob("*.h"))


def build_library(verbose: bool = False) -> Path:
    nvcc = _nvcc()
    objdir = LIBDIR / "obj"
    objdir.mkdir(parents=True, exist_ok=True)
    headers = _headers()
    procs = []
    objs = []
    for src in SOURCES:
        s = CSRC / src
        o = objdir / (src + ".o")
        objs.append(o)
        if not _stale(o, [s] + headers):
            continue
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-I", str(ROOT / "include"), "-c", str(s), "-o", str(o)]
        if src.endswith(".cpp"):
            cmd[1:1] = ["-x", "c++"]
        if verbose:
            print(" ".join(cmd))
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    failed = []
    for src, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append(f"--- {src}\n{out}")
        elif verbose and out.strip():
            print(out)
    if failed:
        raise RuntimeError("nvcc failed:\n" + "\n".join(failed))
    if _stale(LIB, objs):
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
        subprocess.run(cmd, check=True, capture_output=not verbose)
        os.replace(tmp, LIB)
    return LIB


def build_oracle(verbose: bool = False) -> Path:
    src = ORACLE_DIR / "mpfao_oracle.c"
    hdr = ORACLE_DIR / "mpfao_oracle.h"
    ORACLE_LIB.parent.mkdir(parents=True, exist_ok=True)
    if _stale(ORACLE_LIB, [src, hdr]):
        cc = os.environ.get("CC", "gcc")
        tmp = ORACLE_LIB.with_suffix(".so.tmp")
        cmd = [cc, "-O2", "-fPIC", "-shared", "-fopenmp", "-std=c99", "-o", str(tmp), str(src), "-lm"]
        if verbose:
            print(" ".join(cmd))
        subprocess.run(cmd, check=True, capture_output=not verbose)
        os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


if __name__ == "__main__":
    print(build_library(verbose=True))
    print(build_oracle(verbose=True))
