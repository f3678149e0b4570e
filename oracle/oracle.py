"""ORACLE -- test infrastructure only.  ctypes loader of the CPU FP64
restatement (oracle/build/liboracle.so, built by oracle/Makefile).  Imported
by tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py;
never by the product.  Parity with the reference's own outputs is unpinned:
the Fortran reference cannot be built here (see ref_state.h)."""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

from bromoc_gb300 import abi

HERE = Path(__file__).resolve().parent
PREFIX = "bromoc_ref"
_libs = {}


def build(quiet: bool = True) -> None:
    r = subprocess.run(["make", "-C", str(HERE), "-j4"], capture_output=True,
                       text=True)
    if r.returncode:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)


def load(omp: bool = False) -> C.CDLL:
    name = "liboracle_omp.so" if omp else "liboracle.so"
    if name not in _libs:
        path = HERE / "build" / name
        if not path.exists():
            build()
        lib = C.CDLL(str(path))
        abi.declare(lib, PREFIX)
        lib.bromoc_ref_create.argtypes = [C.c_int32, C.POINTER(C.c_void_p)]
        lib.bromoc_ref_threads.restype = C.c_int
        lib.bromoc_ref_set_threads.argtypes = [C.c_int32]
        lib.bromoc_ref_set_threads.restype = C.c_int
        lib.bromoc_ref_philox.argtypes = [C.POINTER(C.c_uint32)] * 3
        lib.bromoc_ref_philox.restype = None
        lib.bromoc_ref_bd_gauss.argtypes = [C.c_uint64, C.c_uint64, C.c_uint32,
                                            C.c_int32]
        lib.bromoc_ref_bd_gauss.restype = C.c_double
        lib.bromoc_ref_gcmc_uniform.argtypes = [C.c_uint64, C.c_uint64,
                                                C.c_uint32, C.c_uint32]
        lib.bromoc_ref_gcmc_uniform.restype = C.c_double
        lib.bromoc_ref_squarespline.argtypes = [
            C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double),
            C.POINTER(C.c_double), C.c_double, C.c_double, C.c_double]
        lib.bromoc_ref_squarespline.restype = None
        _libs[name] = lib
    return _libs[name]


def create(capacity: int = 23000, omp: bool = False) -> abi.Engine:
    lib = load(omp)
    h = C.c_void_p()
    rc = lib.bromoc_ref_create(capacity, C.byref(h))
    if rc != abi.OK:
        raise abi.BromocError(rc, "bromoc_ref_create")
    return abi.Engine(lib, PREFIX, h, capacity)


def efpot_from_knots(r, u, fct, qchr):
    return abi.efpot_from_knots(load(), PREFIX, r, u, fct, qchr)


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    load().bromoc_ref_philox(c, k, o)
    return list(o)


def bd_gauss(seed, step, slot, comp):
    return load().bromoc_ref_bd_gauss(seed, step, slot, comp)


def gcmc_uniform(seed, cycle, attempt, draw):
    return load().bromoc_ref_gcmc_uniform(seed, cycle, attempt, draw)
