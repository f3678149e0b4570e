"""COUNT on the device (k_count) and whole cycles GRAND + BD + COUNT against
the oracle: buffer tags, type signs and nat exactly, ntotat exactly, and the
positions; the simulation loop entry runs COUNT every cycle itself."""
import numpy as np
import pytest

from bromoc_gb300 import abi

from . import systems

pytestmark = pytest.mark.gpu
CAP = 4000


@pytest.mark.parametrize("prec", [abi.FP64, abi.FP32])
def test_cycles_with_count(gpu_lib, oracle_mod, prec):
    spec = systems.gcmc(precision=prec)
    g = gpu_lib.create(CAP, prec)
    o = oracle_mod.create(CAP)
    spec.push(g)
    spec.push(o)
    tol = 1e-9 if prec == abi.FP64 else 1e-5
    for cyc in range(1, 7):
        g.grand(4, 31, cyc, dener=False)
        o.grand(4, 31, cyc)
        g.bd_steps(5, 31, (cyc - 1) * 5, energies=False)
        o.bd_steps(5, 31, (cyc - 1) * 5)
        g.count()
        o.count()
        xg, yg, zg, tg, ig = g.get_particles()
        xo, yo, zo, to, io = o.get_particles()
        assert len(xg) == len(xo), cyc
        np.testing.assert_array_equal(tg, to)
        np.testing.assert_array_equal(ig, io)
        for a, b in ((xg, xo), (yg, yo), (zg, zo)):
            assert np.abs(a - b).max() <= tol
        for a, b in zip(g.get_buffers()[:3], o.get_buffers()[:3]):
            np.testing.assert_array_equal(a, b)
        np.testing.assert_array_equal(g.ntotat(), o.ntotat())


def test_count_tags_ions_that_drift_into_a_buffer(gpu_lib, oracle_mod):
    spec = systems.gcmc(precision=abi.FP64)
    g = gpu_lib.create(CAP, abi.FP64)
    o = oracle_mod.create(CAP)
    spec.push(g)
    spec.push(o)
    x, y, z, t, ib = g.get_particles()
    ib = np.zeros_like(ib)  # stale tags: COUNT rebuilds them from positions
    g.set_particles(x, y, z, np.abs(t), spec.nsites, spec.nfix, ib)
    o.set_particles(x, y, z, np.abs(t), spec.nsites, spec.nfix, ib)
    g.count()
    o.count()
    np.testing.assert_array_equal(g.get_particles()[4], o.get_particles()[4])
    np.testing.assert_array_equal(g.get_particles()[3], o.get_particles()[3])
    np.testing.assert_array_equal(g.get_buffers()[0], o.get_buffers()[0])
    assert g.get_buffers()[0].sum() > 0
