"""bromoc_gpu_pair_energy_static: the pair energy/force entry point for
callers that cannot allocate device memory while they run (their memory is
reserved up front, or owned by another runtime's allocator).  Its scratch is
a static device array, so this file checks it through the C ABI against the
context path (bromoc_gpu_energy with the nonbond mask) on two calls in a row
-- the second call must not see the first call's leftovers -- and checks
that a system above its 4096-ion limit is refused.

Collected last on purpose (file name), so a failure here stops a -x run only
after every other test has run; it passes alone in a fresh process too."""
import ctypes as C

import numpy as np
import pytest

from bromoc_gb300 import abi

from . import systems

pytestmark = pytest.mark.gpu

TOL = {abi.FP64: 1e-10, abi.FP32: 1e-5}


def _declare(lib):
    d = C.c_void_p
    lib.bromoc_gpu_pair_energy_static.argtypes = [
        C.c_void_p, C.c_int32, C.c_int32, d, d, d, d, d, d, d, d]
    lib.bromoc_gpu_pair_energy_static.restype = C.c_int


def _static_call(lib, eng, x, y, z, t, nfix):
    import torch
    dev = torch.device("cuda")
    xs = [torch.from_numpy(np.ascontiguousarray(a, np.float64)).to(dev)
          for a in (x, y, z)]
    ts = torch.from_numpy(np.ascontiguousarray(t, np.int32)).to(dev)
    n = len(x)
    fo = [torch.full((max(n, 1),), np.nan, dtype=torch.float64, device=dev)
          for _ in range(3)]
    eo = torch.full((4,), np.nan, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    rc = lib.bromoc_gpu_pair_energy_static(
        eng.h, n, nfix, xs[0].data_ptr(), xs[1].data_ptr(), xs[2].data_ptr(),
        ts.data_ptr(), fo[0].data_ptr(), fo[1].data_ptr(), fo[2].data_ptr(),
        eo.data_ptr())
    torch.cuda.synchronize()
    return rc, np.stack([f.cpu().numpy()[:n] for f in fo], 1), eo.cpu().numpy()


def _check(lib, spec, eng):
    spec.push(eng)
    ref, fref, _ = eng.energy(abi.M_NONBOND, forces=True)
    rc, f, e = _static_call(lib, eng, spec.x, spec.y, spec.z, spec.typei, spec.nfix)
    assert rc == abi.OK, lib.bromoc_gpu_last_error(eng.h)
    tol = TOL[spec.precision]
    np.testing.assert_allclose(f, fref, rtol=0,
                               atol=tol * max(1.0, np.abs(fref).max()))
    eref = np.array([ref["eelec"], ref["evdw"], ref["esrpmf"], ref["eefpot"]])
    np.testing.assert_allclose(e, eref, rtol=0,
                               atol=tol * max(1.0, np.abs(eref).sum()))


@pytest.mark.parametrize("prec", [abi.FP64, abi.FP32])
def test_static_scratch_matches_context_path(gpu_lib, prec):
    lib = gpu_lib.load()
    _declare(lib)
    eng = gpu_lib.create(5000, prec)
    # first call: a larger bulk system, SRPMF and tabulated pairs
    a = systems.efpot_ions(n_per=180, L=60.0, seed=31, precision=prec)
    _check(lib, a, eng)
    # second call in a row: fewer ions, some fixed -- any stale scratch from
    # the first call would show up in the forces or the energies
    b = systems.pairs(n_per=40, L=36.0, seed=32, precision=prec)
    b.nfix = 5
    _check(lib, b, eng)


@pytest.mark.parametrize("prec", [abi.FP64, abi.FP32])
def test_static_scratch_chunk_packing(gpu_lib, prec):
    """Sizes that pack several source tiles into one chunk: about 2100 ions
    (two tiles per chunk, a ragged last chunk) and the 4096-ion limit (all
    16 chunks of the scratch), both with fixed ions."""
    from bromoc_gb300 import synth
    lib = gpu_lib.load()
    _declare(lib)
    eng = gpu_lib.create(4200, prec)
    for n_per, L, nfix in ((1050, 72.0, 7), (2048, 84.0, 33)):
        s = synth.bulk_kcl(seed=40 + n_per, n_per=n_per, L=L, srpmf=True,
                           precision=prec)
        s.nfix = nfix
        _check(lib, s, eng)


def test_static_scratch_empty(gpu_lib):
    """No ions: the energies come back as zeros, whatever the output
    buffer held before."""
    lib = gpu_lib.load()
    _declare(lib)
    eng = gpu_lib.create(64, abi.FP64)
    systems.pairs(n_per=10).push(eng)
    rc, _, e = _static_call(lib, eng, np.zeros(0), np.zeros(0), np.zeros(0),
                            np.zeros(0, np.int32), 0)
    assert rc == abi.OK
    np.testing.assert_array_equal(e, np.zeros(4))


def test_static_scratch_rejects_oversize(gpu_lib):
    lib = gpu_lib.load()
    _declare(lib)
    eng = gpu_lib.create(5000, abi.FP64)
    systems.pairs(n_per=10).push(eng)
    n = 4097
    rc = lib.bromoc_gpu_pair_energy_static(eng.h, n, 0, 1, 1, 1, 1, 1, 1, 1, 1)
    assert rc == abi.E_CAPACITY
    assert b"4096" in lib.bromoc_gpu_last_error(eng.h)
