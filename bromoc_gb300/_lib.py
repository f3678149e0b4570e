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
        d, i32 = C.POINTER(C.c_double), C.POINTER(C.c_int32)
        lib.bromoc_gpu_simul_cycles_host.argtypes = [
            C.c_void_p, C.c_uint32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
            C.c_uint64, C.c_uint64, i32, C.c_int32, C.c_int32, C.c_void_p,
            C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, d]
        lib.bromoc_gpu_simul_cycles_host.restype = C.c_int
        lib.bromoc_gpu_bd_steps_host.argtypes = [
            C.c_void_p, C.c_uint32, C.c_int32, C.c_int32, C.c_uint64,
            C.c_uint64, C.c_int32, C.c_int32, C.c_int32, d, d, d, i32, d]
        lib.bromoc_gpu_bd_steps_host.restype = C.c_int
        lib.bromoc_gpu_launch_count.argtypes = [C.c_void_p]
        lib.bromoc_gpu_launch_count.restype = C.c_int64
        lib.bromoc_gpu_kernel_timing.argtypes = [C.c_void_p, C.c_int32]
        lib.bromoc_gpu_kernel_timing.restype = C.c_int
        lib.bromoc_gpu_live_count_async.argtypes = [C.c_void_p, C.c_void_p]
        lib.bromoc_gpu_live_count_async.restype = C.c_int
        lib.bromoc_gpu_set_fused_bd.argtypes = [C.c_void_p, C.c_int32]
        lib.bromoc_gpu_set_fused_bd.restype = C.c_int
        lib.bromoc_gpu_kernel_time.argtypes = [C.c_void_p, C.c_int32, d,
                                               C.POINTER(C.c_int64)]
        lib.bromoc_gpu_kernel_time.restype = C.c_int
        lib.bromoc_gpu_fp32_peak.argtypes = [C.c_void_p, d]
        lib.bromoc_gpu_fp32_peak.restype = C.c_int
        i64p = C.POINTER(C.c_int64)
        for name, args in (
                ("set_profiles", [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                  C.c_double, C.c_int32]),
                ("accum_profiles", [C.c_void_p]),
                ("get_profiles", [C.c_void_p, d, d, d, i32, i32]),
                ("traj_header", [C.c_int32, C.c_int32, C.c_char_p, C.c_void_p, C.c_int64,
                                 i64p]),
                ("traj_frame", [C.c_void_p, C.c_double, C.c_void_p, C.c_int64, i64p])):
            f = getattr(lib, "bromoc_gpu_" + name)
            f.argtypes = args
            f.restype = C.c_int
        vp = C.c_void_p
        for name, args in (
                ("create", [vp, C.c_int32, i32, C.POINTER(vp)]),
                ("destroy", [vp]),
                ("set_systems", [vp, vp]),
                ("set_particles", [vp, C.c_int32, C.c_int32, d, d, d, i32]),
                ("get_particles", [vp, C.c_int32, i32, d, d, d]),
                ("bd_steps", [vp, C.c_uint32, C.c_int32, C.POINTER(C.c_uint64),
                              C.c_uint64, d]),
                ("energy", [vp, C.c_uint32, d, d]),
                ("offset", [vp, C.c_int32]),
                ("slots", [vp]),
                ("set_buffers", [vp, C.c_int32, C.POINTER(abi.Buffers), i32]),
                ("grand", [vp, C.c_uint32, C.c_int32, C.POINTER(C.c_uint64), C.c_uint64, d]),
                ("count", [vp]),
                ("get_buffers", [vp, C.c_int32, i32, i32, i32, i32, i32])):
            f = getattr(lib, "bromoc_batch_" + name)
            f.argtypes = args
            f.restype = C.c_int
        u64 = C.c_uint64
        for name, args in (
                ("create", [vp, C.c_int32, C.c_int32, C.POINTER(vp)]),
                ("destroy", [vp]),
                ("set_particles", [vp, C.c_int32, d, d, d, i32]),
                ("forward", [vp, C.c_int32, C.c_int32, u64, u64, C.c_int32, C.c_double,
                             C.c_double, C.c_double, d]),
                ("backward", [vp, d, d, d]),
                ("get_particles", [vp, C.c_int32, d, d, d])):
            f = getattr(lib, "bromoc_adj_" + name)
            f.argtypes = args
            f.restype = C.c_int
        lib.bromoc_adj_last_error.argtypes = [vp]
        lib.bromoc_adj_last_error.restype = C.c_char_p
        lib.bromoc_batch_last_error.argtypes = [vp]
        lib.bromoc_batch_last_error.restype = C.c_char_p
        lib.bromoc_batch_launch_count.argtypes = [vp]
        lib.bromoc_batch_launch_count.restype = C.c_int64
        lib.bromoc_batch_graph_launches.argtypes = [vp]
        lib.bromoc_batch_graph_launches.restype = C.c_int64
        lib.bromoc_batch_set_graph.argtypes = [vp, C.c_int32]
        lib.bromoc_batch_set_graph.restype = C.c_int
        lib.bromoc_batch_tuning.argtypes = [vp, i32, i32, d]
        lib.bromoc_batch_tuning.restype = C.c_int
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


K_PAIRS, K_RFCROSS, K_FIELDS, K_ASSEMBLE, K_LOOP, K_GRAND = 0, 1, 2, 3, 4, 5


def live_count_async(eng: abi.Engine, dst_ptr: int) -> None:
    """Enqueue a copy of the live particle count to the pinned int32 at
    dst_ptr; it holds the value once the context's stream has synchronised."""
    eng._chk(load().bromoc_gpu_live_count_async(eng.h, C.c_void_p(dst_ptr)),
             "live_count_async")


def set_fused_bd(eng: abi.Engine, on: bool) -> None:
    """FP32 bd_steps as one cooperative launch (on, the default) or one
    launch per kernel and step (off); the trajectories agree."""
    eng._chk(load().bromoc_gpu_set_fused_bd(eng.h, int(on)), "set_fused_bd")


def kernel_timing(eng: abi.Engine, on: bool) -> None:
    eng._chk(load().bromoc_gpu_kernel_timing(eng.h, int(on)), "kernel_timing")


def kernel_time(eng: abi.Engine, which: int):
    """(total ms, timed launches) of one kernel family since timing on."""
    ms, n = C.c_double(0.0), C.c_int64(0)
    eng._chk(load().bromoc_gpu_kernel_time(eng.h, which, C.byref(ms),
                                           C.byref(n)), "kernel_time")
    return ms.value, n.value


def launch_count(eng: abi.Engine) -> int:
    return int(load().bromoc_gpu_launch_count(eng.h))


def fp32_peak(stream: int | None = None) -> float:
    t = C.c_double(0.0)
    rc = load().bromoc_gpu_fp32_peak(C.c_void_p(stream) if stream else None,
                                     C.byref(t))
    if rc != abi.OK:
        raise abi.BromocError(rc, "bromoc_gpu_fp32_peak")
    return t.value
