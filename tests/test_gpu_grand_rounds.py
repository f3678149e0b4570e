"""GRAND settles its attempts in rounds: the pair terms of up to eight
attempts are summed together in the state at the start of the round, and
the attempts after an accepted move are corrected with trial-trial terms
or, for a deletion whose target may have moved, proposed again in a new
round.  These cases drive that logic: buffers far from equilibrium (most
insertions, or most deletions, accepted), a single buffer (every deletion
after an accepted move shares its buffer), mixed buffers, and call sizes
from one attempt to several rounds.  The oracle settles one attempt at a
time; counters, histograms, types, buffer tags and slot order must agree
exactly, the energy sums to FP64 rounding, positions to the FP32 records'
precision.  Between calls the particles take BD steps (in FP32 mode the
oracle restarts from the device's positions, the FP32 step being within
its own tolerance of the FP64 one)."""
import numpy as np
import pytest

from bromoc_gb300 import abi

from . import systems

pytestmark = pytest.mark.gpu
CAP = 2000


def _spec(kind, precision):
    s = systems.gcmc(nions=60, precision=precision)
    if kind == "dense":
        for b in s.buffers:
            b["conc"] = 20.0
    elif kind == "dilute":
        for b in s.buffers:
            b["conc"] = 0.005
    elif kind == "one_buffer":
        s.buffers = [dict(s.buffers[0], conc=8.0)]
    elif kind == "mixed":
        for b, c in zip(s.buffers, (12.0, 0.01, 0.01, 12.0)):
            b["conc"] = c
    s.count()
    return s


@pytest.mark.parametrize("precision", [abi.FP64, abi.FP32])
@pytest.mark.parametrize("kind", ["dense", "dilute", "one_buffer", "mixed"])
def test_rounds_match_sequential_oracle(gpu_lib, oracle_mod, kind, precision):
    spec = _spec(kind, precision)
    g = gpu_lib.create(CAP, precision)
    spec.push(g)
    o = oracle_mod.create(CAP)
    spec.push(o)
    cyc = 0
    for ngcmc in (1, 3, 8, 13, 24, 5):
        for _ in range(3):
            cyc += 1
            dg = g.grand(ngcmc, 777, cyc)
            do = o.grand(ngcmc, 777, cyc)
            assert abs(dg - do) <= 1e-8 * max(1.0, abs(do)), (ngcmc, cyc, dg, do)
        g.bd_steps(2, seed=3, step0=2 * cyc, energies=False)
        if precision == abi.FP32:  # FP32 steps stay ~1e-7 A from FP64 ones: restart
            x, y, z, t, ib = g.get_particles()  # the oracle from the device's state
            o.set_particles(x, y, z, t, nsites=spec.nsites, nfix=spec.nfix, ibuffer=ib)
        else:
            o.bd_steps(2, seed=3, step0=2 * cyc, energies=False)
    for x, y in zip(g.get_buffers(), o.get_buffers()):
        np.testing.assert_array_equal(x, y)
    _, nins, nrem, _ = o.get_buffers()
    assert nins.sum() + nrem.sum() >= 20  # many accepted moves, many corrected sums
    xg, yg, zg, tg, ibg = g.get_particles()
    xo, yo, zo, to, ibo = o.get_particles()
    np.testing.assert_array_equal(tg, to)
    np.testing.assert_array_equal(ibg, ibo)
    tol = 1e-7 if precision == abi.FP32 else 1e-9
    np.testing.assert_allclose(np.stack([xg, yg, zg]), np.stack([xo, yo, zo]), atol=tol)


@pytest.mark.parametrize("precision", [abi.FP64, abi.FP32])
def test_rounds_with_sites(gpu_lib, oracle_mod, precision):
    """Fixed DNA sites among the particles: the O(N) sums take the ion-site
    laws (tabulated) for them; buffers at both ends of the box."""
    spec = systems.dna(precision=precision)
    spec.buffers = [dict(ion="K", conc=1.0, lzmin=-0.5 * spec.lz, lzmax=-0.5 * spec.lz + 10.0),
                    dict(ion="Cl", conc=1.0, lzmin=0.5 * spec.lz - 10.0, lzmax=0.5 * spec.lz)]
    spec.count()
    g = gpu_lib.create(CAP, precision)
    spec.push(g)
    o = oracle_mod.create(CAP)
    spec.push(o)
    for cyc in range(1, 7):
        dg, do = g.grand(6, 17, cyc), o.grand(6, 17, cyc)
        assert abs(dg - do) <= 1e-8 * max(1.0, abs(do)), (cyc, dg, do)
    for x, y in zip(g.get_buffers(), o.get_buffers()):
        np.testing.assert_array_equal(x, y)
    pg, po = g.get_particles(), o.get_particles()
    np.testing.assert_array_equal(pg[3], po[3])
    np.testing.assert_array_equal(pg[4], po[4])
    np.testing.assert_allclose(np.stack(pg[:3]), np.stack(po[:3]), atol=1e-9)
