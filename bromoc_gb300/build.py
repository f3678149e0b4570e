"""Build libbromoc_gpu.so in-tree for sm_103a.

Each translation unit compiles in parallel (one nvcc per file, one -gencode),
then one link step.  Objects go to bromoc_gb300/_build/; the library lands
beside this file.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
SRC = PKG / "csrc"
OBJ = PKG / "_build"
LIB = PKG / "libbromoc_gpu.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
UNITS = ["api.cu", "energy.cu", "fields.cu", "dyn.cu", "gcmc.cu", "probe.cu", "noalloc.cu", "batch.cu", "adjoint.cu", "loop.cu", "cells.cu", "mc.cu", "nucl.cu", "analysis.cu", "mmij.cu", "tables.cpp"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"),
                 "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    OBJ.mkdir(exist_ok=True)
    headers = list(SRC.glob("*.cuh")) + list(SRC.glob("*.h")) + \
        [PKG.parent / "include" / "bromoc_gpu.h"]
    nv = nvcc()
    procs, objs = [], []
    for u in UNITS:
        src = SRC / u
        obj = OBJ / (u + ".o")
        objs.append(obj)
        if not force and not _stale(obj, [src] + headers):
            continue
        cmd = [nv, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler",
               "-fPIC", "-c", str(src), "-o", str(obj)]
        if u.endswith(".cu"):
            cmd += ["-Xptxas", "-v"] if verbose else []
        else:
            cmd += ["-x", "c++"]
        procs.append((u, subprocess.Popen(cmd, stdout=subprocess.PIPE,
                                          stderr=subprocess.STDOUT)))
    failed = []
    for u, p in procs:
        out, _ = p.communicate()
        if verbose or p.returncode:
            sys.stderr.write(out.decode())
        if p.returncode:
            failed.append(u)
    if failed:
        raise RuntimeError(f"nvcc failed for {failed}")
    if force or procs or _stale(LIB, objs):
        cmd = [nv, *ARCH, "-shared", "-o", str(LIB), *map(str, objs)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
