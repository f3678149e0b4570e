"""METROPOLIS (metropolis.f90:31-55, move.f90:19-45) on the device against
the oracle's restatement, and the oracle pinned by the reference's own
bookkeeping: ener += enew - eold after every accepted move, so the summed
change equals the change of the total ENERGY (on a system without SRPMF,
whose taper ENERGY and INTERACT compute differently in the reference)."""
import numpy as np
import pytest

from bromoc_gb300 import abi

from . import systems


def test_oracle_energy_bookkeeping(oracle_mod):
    spec = systems.maps(precision=abi.FP64, srpmf=False)
    o = oracle_mod.create(256)
    spec.push(o)
    e0 = o.energy(abi.M_ALL, forces=False)[0]["ener"]
    na, d = o.metropolis(200, 2.0, seed=17, cycle=1)
    e1 = o.energy(abi.M_ALL, forces=False)[0]["ener"]
    assert 0 < na < 200
    assert abs((e1 - e0) - d) <= 1e-8 * max(1.0, abs(e0))


def test_oracle_moves_stay_inside(oracle_mod):
    spec = systems.pairs(precision=abi.FP64)
    o = oracle_mod.create(256)
    spec.push(o)
    o.metropolis(300, 3.0, seed=5, cycle=2)
    x, y, z = o.get_particles()[:3]
    h = 0.5 * spec.lx
    assert np.abs(np.stack([x, y, z])).max() <= h


@pytest.mark.gpu
@pytest.mark.parametrize("family", ["maps_trln", "pairs", "dna", "efpot"])
@pytest.mark.parametrize("prec", [abi.FP64, abi.FP32])
def test_metropolis_matches_oracle(gpu_lib, oracle_mod, family, prec):
    spec = systems.all_families()[family](precision=prec)
    if spec.nfix:
        pytest.skip("fixed ions are refused")
    g = gpu_lib.create(256, prec)
    o = oracle_mod.create(256)
    spec.push(g)
    spec.push(o)
    for cyc in (1, 2):
        ng, dg = g.metropolis(40, 1.5, seed=99, cycle=cyc)
        no, do = o.metropolis(40, 1.5, seed=99, cycle=cyc)
        assert ng == no, (cyc, ng, no)
        assert abs(dg - do) <= 1e-8 * max(1.0, abs(do)), (cyc, dg, do)
    pg = np.stack(g.get_particles()[:3], 1)
    po = np.stack(o.get_particles()[:3], 1)
    assert np.abs(pg - po).max() <= (1e-10 if prec == abi.FP64 else 1e-9)
    # a BD step after the moves starts from the moved positions
    g.bd_steps(1, seed=3, step0=0, energies=False)
    o.bd_steps(1, seed=3, step0=0, energies=False)
    pg = np.stack(g.get_particles()[:3], 1)
    po = np.stack(o.get_particles()[:3], 1)
    assert np.abs(pg - po).max() <= (1e-10 if prec == abi.FP64 else 1e-5)


@pytest.mark.gpu
def test_metropolis_refuses_fixed_ions(gpu_lib):
    spec = systems.maps(precision=abi.FP64, nfix=4)
    g = gpu_lib.create(256, abi.FP64)
    spec.push(g)
    with pytest.raises(abi.BromocError) as e:
        g.metropolis(5, 1.0, seed=1, cycle=1)
    assert e.value.code == abi.E_STATE
