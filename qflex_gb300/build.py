"""Builds libqflex_gb300.so (host C++ + sm_103a CUDA kernels) in-tree.

    python -m qflex_gb300.build          # or: from qflex_gb300.build import build

Every translation unit compiles in parallel with nvcc for
``-gencode arch=compute_103a,code=sm_103a``; the CUDA runtime is linked
statically so the library needs only the driver at run time.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libqflex_gb300.so"
CLI = PKG / "qflex"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found; the CUDA toolkit is required to build qflex_gb300")


def _sources():
    return sorted(list(CSRC.glob("*.cpp")) + list(CSRC.glob("*.cu")))


def _compile(src: Path, nvcc: str) -> Path:
    obj = BUILD / (src.name + ".o")
    deps = [src] + list(CSRC.glob("*.h")) + [PKG.parent / "include" / "qflex_gb300.h"]
    if obj.exists() and obj.stat().st_mtime >= max(d.stat().st_mtime for d in deps if d.exists()):
        return obj
    flags = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", str(CSRC), "-I", str(PKG.parent / "include")]
    if src.suffix == ".cu":
        flags += ARCH + ["-lineinfo", "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]
    cmd = [nvcc, *flags, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False) -> Path:
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, nvcc), srcs))
    newest = max(o.stat().st_mtime for o in objs)
    if not LIB.exists() or LIB.stat().st_mtime < newest:
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc, *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *map(str, objs), "-lpthread", "-ldl", "-lrt"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    cli_src = PKG / "cli" / "qflex_cli.cpp"
    if not CLI.exists() or CLI.stat().st_mtime < max(LIB.stat().st_mtime, cli_src.stat().st_mtime):
        cmd = ["g++", "-O2", "-std=c++17", "-I", str(PKG.parent / "include"), str(cli_src),
               "-L", str(PKG), "-lqflex_gb300", "-Wl,-rpath,$ORIGIN", "-o", str(CLI)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"CLI build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(f"built {LIB} and {CLI}")
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
