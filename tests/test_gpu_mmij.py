"""The MMIJ reaction field on the GPU against the oracle (rect_rf1/rf0,
sphe_rf1/rf0): ENERGY and forces run in test_gpu_parity's family sweep;
here INTERACT of present ions, insertion trials and sites, BD steps,
METROPOLIS, the mask and GRAND's refusal."""
import numpy as np
import pytest

from bromoc_gb300 import abi

from . import systems

pytestmark = pytest.mark.gpu
CAP = 4000


def _engines(spec, gpu_lib, oracle_mod):
    g = gpu_lib.create(CAP, spec.precision)
    o = oracle_mod.create(CAP)
    spec.push(g)
    spec.push(o)
    return g, o


@pytest.mark.parametrize("shape", ["rect", "sphere"])
@pytest.mark.parametrize("prec", [abi.FP64, abi.FP32])
def test_interact(gpu_lib, oracle_mod, shape, prec):
    spec = systems.mmij(shape, precision=prec)
    g, o = _engines(spec, gpu_lib, oracle_mod)
    n = len(spec.x)
    for mask in (abi.M_MMIJ, abi.M_ALL):
        for j in list(range(0, n, 7)):
            it = abs(int(spec.typei[j]))
            a = g.interact(spec.x[j], spec.y[j], spec.z[j], it, j + 1, mask)
            b = o.interact(spec.x[j], spec.y[j], spec.z[j], it, j + 1, mask)
            assert abs(a - b) <= 1e-9 * max(1.0, abs(b)), (j, a, b)
        rng = np.random.default_rng(3)
        for _ in range(6):  # insertion trials inside and outside the region
            pnt = rng.uniform(-12.0, 12.0, 3)
            it = spec.nold + 1 + int(rng.integers(0, spec.nion))
            a = g.interact(*pnt, it, n + 1, mask)
            b = o.interact(*pnt, it, n + 1, mask)
            assert abs(a - b) <= 1e-9 * max(1.0, abs(b)), (pnt, a, b)


@pytest.mark.parametrize("shape", ["rect", "sphere"])
def test_bd_steps(gpu_lib, oracle_mod, shape):
    spec = systems.mmij(shape, precision=abi.FP64)
    g, o = _engines(spec, gpu_lib, oracle_mod)
    eg = g.bd_steps(5, seed=8, step0=0)
    eo = o.bd_steps(5, seed=8, step0=0)
    pg = np.stack(g.get_particles()[:3], 1)
    po = np.stack(o.get_particles()[:3], 1)
    assert np.abs(pg - po).max() <= 1e-8
    assert abs(eg["egsbpb"] - eo["egsbpb"]) <= 1e-9 * max(1.0, abs(eo["egsbpb"]))


def test_fp32_bd_steps_skip_the_fused_loop(gpu_lib, oracle_mod):
    """FP32 steps of a system with the reaction field run per kernel (the
    fused loop has no MMIJ term) and land within 1e-5 A of the oracle."""
    spec = systems.mmij("rect", precision=abi.FP32)
    g, o = _engines(spec, gpu_lib, oracle_mod)
    g.bd_steps(3, seed=8, step0=0, energies=False)
    o.bd_steps(3, seed=8, step0=0)
    pg = np.stack(g.get_particles()[:3], 1)
    po = np.stack(o.get_particles()[:3], 1)
    assert np.abs(pg - po).max() <= 1e-5


def test_mask_and_grand(gpu_lib, oracle_mod):
    spec = systems.mmij("rect", precision=abi.FP64)
    g, o = _engines(spec, gpu_lib, oracle_mod)
    off = abi.M_ALL & ~abi.M_MMIJ
    tg = g.energy(off)[0]
    to = o.energy(off)[0]
    assert tg["egsbpb"] == 0.0 and abs(tg["ener"] - to["ener"]) <= 1e-10 * abs(to["ener"])
    spec_b = systems.mmij("rect", precision=abi.FP64, buffers=True)
    gb = gpu_lib.create(CAP, abi.FP64)
    spec_b.push(gb)
    with pytest.raises(abi.BromocError) as e:
        gb.grand(2, seed=1, cycle=1)
    assert e.value.code == abi.E_STATE and "MMIJ" in str(e.value)
    gb.grand(2, seed=1, cycle=1, terms=abi.M_ALL & ~abi.M_MMIJ)  # without the term it runs


def test_metropolis_with_the_reaction_field(gpu_lib, oracle_mod):
    spec = systems.mmij("rect", precision=abi.FP64)
    g, o = _engines(spec, gpu_lib, oracle_mod)
    ag, dg = g.metropolis(20, 0.8, seed=5, cycle=1)
    ao, do = o.metropolis(20, 0.8, seed=5, cycle=1)
    assert ag == ao
    assert abs(dg - do) <= 1e-8 * max(1.0, abs(do))
