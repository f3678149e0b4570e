"""The host-array cycle entry point (bromoc_gpu_simul_cycles_host: upload the
caller's arrays, run ncycle x (GRAND attempts + BD steps), write the arrays
back with the new count, one wait at the end) against the same calls made one
by one through the context: positions, types, buffer tags, the count, the
last cycle's energies and the GCMC counters must agree bit for bit.  Also the
BD-only entry (bromoc_gpu_bd_steps_host) on an FP32 context, and the error
path: a rejected upload leaves the context usable."""
import ctypes as C

import numpy as np
import pytest

from bromoc_gb300 import _lib, abi

from . import systems

pytestmark = pytest.mark.gpu
CAP = 4000
NGCMC, NBD, SEED = 6, 4, 4242


def _host_arrays(g, kind):
    """Capacity-sized host copies of g's particles ("pageable" numpy or
    "pinned" torch buffers, the form a caller in a timed loop would use)."""
    x, y, z, t, ib = g.get_particles()
    n = len(x)
    out = {}
    for k, a, dt in (("x", x, np.float64), ("y", y, np.float64), ("z", z, np.float64),
                     ("t", t, np.int32), ("ib", ib, np.int32)):
        if kind == "pinned":
            import torch
            buf = torch.zeros(CAP, dtype=torch.float64 if dt == np.float64 else torch.int32,
                              pin_memory=True).numpy()
        else:
            buf = np.zeros(CAP, dt)
        buf[:n] = a
        out[k] = buf
    return out, n


def _cycles(g, spec, a, ntot, ncycle, cycle0, eterms=None):
    lib = _lib.load()
    n = C.c_int32(ntot)
    rc = lib.bromoc_gpu_simul_cycles_host(
        g.h, abi.M_ALL, abi.DYN0, ncycle, NGCMC, NBD, SEED, cycle0, C.byref(n),
        spec.nsites, spec.nfix, a["x"].ctypes.data, a["y"].ctypes.data, a["z"].ctypes.data,
        a["t"].ctypes.data, a["ib"].ctypes.data,
        None if eterms is None else eterms.ctypes.data_as(C.POINTER(C.c_double)))
    return rc, n.value


def _stepwise(g, ncycle, cycle0):
    e = None
    for c in range(ncycle):
        cyc = cycle0 + c
        g.grand(NGCMC, SEED, cyc, dener=False)
        e = g.bd_steps(NBD, seed=SEED, step0=(cyc - 1) * NBD, energies=c + 1 == ncycle)
        g.count()  # simul1.f90:462
    return e


def _same(a, n, g):
    x, y, z, t, ib = g.get_particles()
    assert n == len(x)
    for k, want in (("x", x), ("y", y), ("z", z), ("t", t), ("ib", ib)):
        np.testing.assert_array_equal(a[k][:n], want, err_msg=k)


@pytest.mark.parametrize("precision", [abi.FP32, abi.FP64])
@pytest.mark.parametrize("kind", ["pageable", "pinned"])
def test_simul_cycles_host_matches_stepwise(gpu_lib, precision, kind):
    spec = systems.gcmc(precision=precision)
    a_eng = gpu_lib.create(CAP, precision)
    b_eng = gpu_lib.create(CAP, precision)
    spec.push(a_eng)
    spec.push(b_eng)
    arrs, n = _host_arrays(b_eng, kind)
    counts = []
    for ncycle, cycle0 in ((3, 1), (1, 4), (5, 5)):
        e = np.zeros(abi.NTERMS)
        rc, n = _cycles(a_eng, spec, arrs, n, ncycle, cycle0, e)
        assert rc == 0, _lib.load().bromoc_gpu_last_error(a_eng.h)
        want = _stepwise(b_eng, ncycle, cycle0)
        _same(arrs, n, b_eng)
        assert dict(zip(abi.TERM_NAMES, e.tolist())) == want
        counts.append(n)
    for u, v in zip(a_eng.get_buffers(), b_eng.get_buffers()):
        np.testing.assert_array_equal(u, v)
    assert len(set(counts)) > 1 or counts[0] != len(spec.x)  # GCMC changed the count


def test_simul_cycles_host_rejects_and_recovers(gpu_lib):
    spec = systems.gcmc(precision=abi.FP32)
    g = gpu_lib.create(CAP, abi.FP32)
    spec.push(g)
    arrs, n = _host_arrays(g, "pageable")
    bad = {k: v.copy() for k, v in arrs.items()}
    bad["t"][n - 1] = 0  # not an ion type
    rc, _ = _cycles(g, spec, bad, n, 2, 1)
    assert rc == abi.E_ARG
    rc, n2 = _cycles(g, spec, arrs, n, 2, 1)
    assert rc == 0
    ref = gpu_lib.create(CAP, abi.FP32)
    spec.push(ref)
    _stepwise(ref, 2, 1)
    _same(arrs, n2, ref)


def test_bd_steps_host_fp32_matches_context(gpu_lib):
    spec = systems.maps(precision=abi.FP32)
    g = gpu_lib.create(CAP, abi.FP32)
    ref = gpu_lib.create(CAP, abi.FP32)
    spec.push(g)
    spec.push(ref)
    x, y, z = spec.x.copy(), spec.y.copy(), spec.z.copy()
    t = np.ascontiguousarray(spec.typei, np.int32)
    e = np.zeros(abi.NTERMS)
    P = lambda v, ct: v.ctypes.data_as(C.POINTER(ct))
    for step0 in (0, 5):
        rc = g.lib.bromoc_gpu_bd_steps_host(
            g.h, abi.M_ALL, abi.DYN0, 5, 99, step0, len(x), spec.nsites, spec.nfix,
            P(x, C.c_double), P(y, C.c_double), P(z, C.c_double), P(t, C.c_int32),
            P(e, C.c_double))
        assert rc == 0
        want = ref.bd_steps(5, seed=99, step0=step0)
        assert dict(zip(abi.TERM_NAMES, e.tolist())) == want
    xr, yr, zr = ref.get_particles()[:3]
    np.testing.assert_array_equal(np.stack([x, y, z]), np.stack([xr, yr, zr]))
