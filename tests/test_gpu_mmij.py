"""The MMIJ reaction field on the GPU against the oracle (rect_rf1/rf0,
sphe_rf1/rf0): ENERGY and forces run in test_gpu_parity's family sweep;
here INTERACT of present ions, insertion trials and sites, BD steps,
METROPOLIS, GRAND and the mask."""
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


def test_mask(gpu_lib, oracle_mod):
    spec = systems.mmij("rect", precision=abi.FP64)
    g, o = _engines(spec, gpu_lib, oracle_mod)
    off = abi.M_ALL & ~abi.M_MMIJ
    tg = g.energy(off)[0]
    to = o.energy(off)[0]
    assert tg["egsbpb"] == 0.0 and abs(tg["ener"] - to["ener"]) <= 1e-10 * abs(to["ener"])


def _compare_gcmc(g, o, atol):
    ng, nig, nrg, prg = g.get_buffers()
    no, nio, nro, pro = o.get_buffers()
    np.testing.assert_array_equal(ng, no)
    np.testing.assert_array_equal(nig, nio)
    np.testing.assert_array_equal(nrg, nro)
    np.testing.assert_array_equal(prg, pro)
    assert nig.sum() + nrg.sum() > 0
    xg, yg, zg, tg, ibg = g.get_particles()
    xo, yo, zo, to, ibo = o.get_particles()
    np.testing.assert_array_equal(tg, to)
    np.testing.assert_array_equal(ibg, ibo)
    np.testing.assert_allclose(np.stack([xg, yg, zg]), np.stack([xo, yo, zo]), atol=atol)


@pytest.mark.parametrize("shape", ["rect", "sphere"])
@pytest.mark.parametrize("prec", [abi.FP64, abi.FP32])
def test_grand_with_the_reaction_field(gpu_lib, oracle_mod, shape, prec):
    """GRAND with the MMIJ term (the attempts one after another through
    INTERACT): the oracle's insertions and deletions, counters and
    histogram exact, its energy sums, the same particles after BD steps and
    COUNT between the calls."""
    spec = systems.mmij(shape, precision=prec, buffers=True)
    g, o = _engines(spec, gpu_lib, oracle_mod)
    # FP32 BD steps between the calls leave the positions ~1e-6 A from the
    # oracle's, and the energy sums follow
    tol = 1e-8 if prec == abi.FP64 else 1e-5
    for cyc in range(1, 9):
        dg = g.grand(6, 4242, cyc)
        do = o.grand(6, 4242, cyc)
        assert abs(dg - do) <= tol * max(1.0, abs(do)), (cyc, dg, do)
        g.bd_steps(2, seed=7, step0=2 * cyc, energies=False)
        o.bd_steps(2, seed=7, step0=2 * cyc)
        g.count()
        o.count()
    _compare_gcmc(g, o, 1e-7 if prec == abi.FP64 else 1e-5)


def test_grand_one_by_one_makes_the_round_kernels_moves(gpu_lib):
    """With a zero MMIJ matrix the term vanishes: GRAND one attempt after
    another (MMIJ on) and the round kernel (MMIJ masked out) make the same
    moves from the same draws."""
    spec = systems.mmij("rect", precision=abi.FP64, buffers=True)
    spec.mmij = dict(spec.mmij, mmij=np.zeros_like(spec.mmij["mmij"]))
    a = gpu_lib.create(CAP, abi.FP64)
    b = gpu_lib.create(CAP, abi.FP64)
    spec.push(a)
    spec.push(b)
    for cyc in range(1, 9):
        da = a.grand(6, 99, cyc)
        db = b.grand(6, 99, cyc, terms=abi.M_ALL & ~abi.M_MMIJ)
        assert abs(da - db) <= 1e-9 * max(1.0, abs(db)), (cyc, da, db)
        a.bd_steps(2, seed=3, step0=2 * cyc, energies=False)
        b.bd_steps(2, seed=3, step0=2 * cyc, energies=False)
        a.count()
        b.count()
    _compare_gcmc(a, b, 0.0)


def test_metropolis_with_the_reaction_field(gpu_lib, oracle_mod):
    spec = systems.mmij("rect", precision=abi.FP64)
    g, o = _engines(spec, gpu_lib, oracle_mod)
    ag, dg = g.metropolis(20, 0.8, seed=5, cycle=1)
    ao, do = o.metropolis(20, 0.8, seed=5, cycle=1)
    assert ag == ao
    assert abs(dg - do) <= 1e-8 * max(1.0, abs(do))
