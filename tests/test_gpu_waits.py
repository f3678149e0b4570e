"""The bounded waits of the cooperative kernels (the fused BD loop, GRAND):
a wait whose arrival never comes gives up after its poll limit, records the
barrier flag in the device error word and lets the kernel return, so the
host reads a status instead of hanging and the context stays usable.  The
wait is made to run out on purpose (one block never arrives), with a short
poll limit; the same wait with the arrival made ends without the flag."""
import ctypes as C
import time

import numpy as np
import pytest

from bromoc_gb300 import abi

from . import systems

pytestmark = pytest.mark.gpu
BARRIER_FLAG = 16


def _selftest(lib, spins, arrive):
    f = lib.bromoc_gpu_wait_selftest
    f.argtypes = [C.c_int32, C.c_int32, C.POINTER(C.c_int32)]
    f.restype = C.c_int
    err = C.c_int32(-1)
    t0 = time.perf_counter()
    rc = f(spins, arrive, C.byref(err))
    return rc, err.value, time.perf_counter() - t0


def test_wait_runs_out_and_reports(gpu_lib):
    lib = gpu_lib.load()
    rc, err, dt = _selftest(lib, 1 << 12, 0)
    assert rc == abi.OK
    assert err & BARRIER_FLAG, err
    assert dt < 5.0


def test_wait_with_arrival_succeeds(gpu_lib):
    lib = gpu_lib.load()
    rc, err, _ = _selftest(lib, 1 << 22, 1)
    assert rc == abi.OK and err == 0, err


def test_device_usable_after_expired_wait(gpu_lib, oracle_mod):
    lib = gpu_lib.load()
    assert _selftest(lib, 1 << 10, 0)[1] & BARRIER_FLAG
    spec = systems.pairs(precision=abi.FP64)
    g = gpu_lib.create(256, abi.FP64)
    o = oracle_mod.create(256)
    spec.push(g)
    spec.push(o)
    tg, fg, _ = g.energy(abi.M_ALL, forces=True)
    to, fo, _ = o.energy(abi.M_ALL, forces=True)
    assert np.linalg.norm(fg - fo) <= 1e-10 * np.linalg.norm(fo)
    assert abs(tg["ener"] - to["ener"]) <= 1e-10 * max(1.0, abs(to["ener"]))


def test_context_destroyed_before_its_dependents(gpu_lib):
    """A context destroyed while a replica batch and an adjoint engine still
    borrow it: they are flagged, refuse further work with an error, and
    their own destroy touches nothing of the gone context."""
    import ctypes as C
    from bromoc_gb300.adjoint import Adjoint
    from bromoc_gb300.batch import Batch
    lib = gpu_lib.load()
    spec = systems.pairs(precision=abi.FP32)
    proto = gpu_lib.create(256, abi.FP32)
    spec.push(proto)
    b = Batch(proto, [len(spec.x)])
    adj_spec = systems.efpot_all(precision=abi.FP32)
    proto2 = gpu_lib.create(256, abi.FP32)
    adj_spec.push(proto2)
    adj = Adjoint(proto2, 256, abi.FP32)
    # destroy the contexts behind the dependents' backs (the C ABI)
    lib.bromoc_gpu_destroy(proto.h)
    proto.h = None
    lib.bromoc_gpu_destroy(proto2.h)
    proto2.h = None
    with pytest.raises(abi.BromocError) as e:
        b.set_particles(0, spec.x, spec.y, spec.z, spec.typei)
    assert e.value.code == abi.E_STATE
    with pytest.raises(abi.BromocError):
        adj.set_particles(adj_spec.x, adj_spec.y, adj_spec.z, adj_spec.typei)
    b.close()
    adj.close()
    # the device is still fine
    g = gpu_lib.create(256, abi.FP64)
    spec.push(g)
    g.energy()
