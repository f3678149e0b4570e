"""Loader of the in-tree libbromoc_gpu.so (no fallback: a missing library or a
missing GPU is an error)."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from . import abi

LIB_PATH = Path(__file__).resolve().parent / "libbromoc_gpu.so"
PREFIX = "bromoc_gpu"
_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'`")
        lib = C.CDLL(str(LIB_PATH))
        abi.declare(lib, PREFIX)
        lib.bromoc_gpu_create.argtypes = [C.c_int32, C.c_int32, C.c_void_p,
                                          C.POINTER(C.c_void_p)]
        lib.bromoc_gpu_abi_version.restype = C.c_int
        _lib = lib
    return _lib


def create(capacity: int = 23000, precision: int = abi.FP64,
           stream: int | None = None) -> abi.Engine:
    """New device context; `stream` is a cudaStream_t handle (e.g.
    torch.cuda.current_stream().cuda_stream) or None for a private stream."""
    lib = load()
    h = C.c_void_p()
    rc = lib.bromoc_gpu_create(capacity, precision,
                               C.c_void_p(stream) if stream else None,
                               C.byref(h))
    if rc != abi.OK:
        raise abi.BromocError(rc, "bromoc_gpu_create failed (is a GPU present?)")
    return abi.Engine(lib, PREFIX, h, capacity)


def efpot_from_knots(r, u, fct, qchr):
    return abi.efpot_from_knots(load(), PREFIX, r, u, fct, qchr)
