"""Parity with the FP64 oracle at the sizes the measured workloads run.

The small systems of test_gpu_parity.py leave the paths that only large
systems take unchecked: the pair tile's single-chain loop (more than 96 ion
tiles, i.e. over 3072 ions), the 120x120x180 maps, the ssDNA system with
about 5000 ions, and batch replicas of thousands of ions.  Each is compared
here with the CPU restatement of the reference on the same inputs.

Force tolerances as in test_gpu_parity.py: FP32 within 1e-5 of the oracle
as a whole and per particle against max(|F_i|, RMS |F|).
"""
import copy

import numpy as np
import pytest

from bromoc_gb300 import abi, synth

from .test_gpu_parity import FP32_TOL, FP64_TOL, energy_err
from .test_gpu_parity import force_err as scale_force_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pore_maps():
    return synth.pore_maps(seed=103)


def _pair(spec, gpu_lib, oracle_mod, prec, cap):
    s = copy.copy(spec)
    s.precision = prec
    g = gpu_lib.create(cap, prec)
    o = oracle_mod.create(cap)
    s.push(g)
    s.push(o)
    return g, o


@pytest.mark.parametrize("nions", [4000, 8000])
def test_pore_single_chain_tile(gpu_lib, oracle_mod, pore_maps, nions):
    """Pore with 4000 / 8000 ions (125 / 250 ion tiles: the tile's one-chain
    loop), every term on, FP32 against the FP64 oracle; FP64 to rounding."""
    spec = synth.pore(seed=3, nions=nions, maps=pore_maps, precision=abi.FP32,
                      buffers=False)
    o = oracle_mod.create(nions + 16)
    spec.push(o)
    to, fo, wo = o.energy(abi.M_ALL, forces=True)
    for prec, tol in ((abi.FP32, FP32_TOL), (abi.FP64, FP64_TOL)):
        s = copy.copy(spec)
        s.precision = prec
        g = gpu_lib.create(nions + 16, prec)
        s.push(g)
        tg, fg, wg = g.energy(abi.M_ALL, forces=True)
        glob, worst = scale_force_err(fg, fo)
        assert glob <= tol and worst <= tol, (prec, glob, worst)
        assert energy_err(tg, to) <= tol, (prec, tg, to)
        np.testing.assert_array_equal(wg, wo)


def test_pore_full_size_cycle(gpu_lib, oracle_mod):
    """The measured nanopore cycle at full size (2000 ions, 120x120x180
    maps, four GCMC buffers): ENERGY in FP64 and FP32, one FP32 BD step, and
    four GRAND(4) calls with every counter exact, against the oracle."""
    spec = synth.pore(seed=3, nions=2000, maps=synth.pore_maps(seed=102),
                      precision=abi.FP32, buffers=True)
    cap = 2400
    for prec, tol in ((abi.FP64, FP64_TOL), (abi.FP32, FP32_TOL)):
        g, o = _pair(spec, gpu_lib, oracle_mod, prec, cap)
        tg, fg, _ = g.energy(abi.M_ALL, forces=True)
        to, fo, _ = o.energy(abi.M_ALL, forces=True)
        glob, worst = scale_force_err(fg, fo)
        assert glob <= tol and worst <= tol, (prec, glob, worst)
        assert energy_err(tg, to) <= tol
    g, o = _pair(spec, gpu_lib, oracle_mod, abi.FP32, cap)
    g.bd_steps(1, seed=5, step0=0, energies=False)
    o.bd_steps(1, seed=5, step0=0, energies=False)
    pg = np.stack(g.get_particles()[:3], 1)
    po = np.stack(o.get_particles()[:3], 1)
    assert np.abs(pg - po).max() <= 1e-5
    g, o = _pair(spec, gpu_lib, oracle_mod, abi.FP32, cap)
    for cyc in range(1, 5):
        dg, do = g.grand(4, 1234, cyc), o.grand(4, 1234, cyc)
        assert abs(dg - do) <= 1e-8 * max(1.0, abs(do)), (cyc, dg, do)
    for a, b in zip(g.get_buffers(), o.get_buffers()):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(g.get_particles()[3], o.get_particles()[3])


@pytest.mark.parametrize("prec", [abi.FP64, abi.FP32])
def test_ssdna_full_size_energy(gpu_lib, oracle_mod, pore_maps, prec):
    """ssDNA (40 nt x 3 sites, tabulated ion-site laws) through the pore
    with about 5000 ions: ENERGY and forces."""
    spec = synth.ssdna(seed=4, nions=5000, nnuc=40, maps=pore_maps, precision=prec)
    g, o = _pair(spec, gpu_lib, oracle_mod, prec, len(spec.x) + 16)
    tg, fg, wg = g.energy(abi.M_ALL, forces=True)
    to, fo, wo = o.energy(abi.M_ALL, forces=True)
    tol = FP64_TOL if prec == abi.FP64 else FP32_TOL
    glob, worst = scale_force_err(fg, fo)
    assert glob <= tol and worst <= tol, (glob, worst)
    assert energy_err(tg, to) <= tol
    np.testing.assert_array_equal(wg, wo)


def test_batch_large_replicas(gpu_lib, oracle_mod):
    """Replicas of 3000 and 8000 ions (the batch's single-chain tiles) and a
    small one, as the batched workload builds them (bulk KCl at 1 M in cube
    boxes sharing the pore maps): each against the oracle."""
    from bromoc_gb300.batch import Batch
    maps = synth.pore_maps(seed=102)
    spec = synth.pore(seed=3, nions=2000, maps=maps, precision=abi.FP32, buffers=False)
    rng = np.random.default_rng(8)
    counts = [3000, 8000, 250]
    reps = []
    for n in counts:
        L = (n / (2.0 * 6.02214e-4)) ** (1.0 / 3.0)
        h = 0.5 * L - 0.5
        p = synth.jittered_lattice(rng, n, -h, h, ok=synth.outside_pore_slab)
        s = copy.copy(spec)
        s.lx = s.ly = s.lz = float(L)
        s.x, s.y, s.z = p[:, 0].copy(), p[:, 1].copy(), p[:, 2].copy()
        s.typei = np.array([1, 2] * (n // 2), np.int32)
        reps.append(s)
    proto = gpu_lib.create(2064, abi.FP32)
    spec.push(proto)
    b = Batch(proto, counts)
    b.set_systems([s.system_struct() for s in reps])
    for r, s in enumerate(reps):
        b.set_particles(r, s.x, s.y, s.z, s.typei)
    et, f = b.energy(abi.M_ALL, forces=True)
    for r, s in enumerate(reps):
        o = oracle_mod.create(len(s.x) + 16)
        s.push(o)
        to, fo, _ = o.energy(abi.M_ALL, forces=True)
        off = b.offset(r)
        glob, worst = scale_force_err(f[off:off + len(s.x)], fo)
        assert glob <= FP32_TOL and worst <= FP32_TOL, (counts[r], glob, worst)
        tb = {k: et[r, i] for i, k in enumerate(abi.TERM_NAMES)}
        assert energy_err(tb, to) <= FP32_TOL, (counts[r], tb, to)


def _walled(shape, prec, seed=17):
    """Bulk KCl in a sphere (radius 15 A) or an elliptic cylinder (semi-axes
    14 and 11 A, 40 A long), half of the ions within 0.25 A of the wall so
    that BD moves cross it and fixcoor (fixcoor.f90:19-68) acts."""
    rng = np.random.default_rng(seed)
    s = synth.bulk_kcl(seed=seed, n_per=4, L=30.0, srpmf=True, precision=prec)
    s.shape = shape
    pts = []
    if shape == abi.SPHERE:
        s.rsphe = 15.0
        while len(pts) < 48:
            u = rng.normal(size=3)
            u /= np.linalg.norm(u)
            r = 14.75 + 0.25 * rng.random() if len(pts) % 2 == 0 else 12.0 * rng.random() ** (1 / 3)
            q = r * u
            if all(np.sum((q - a) ** 2) >= 9.0 for a in pts):
                pts.append(q)
    else:
        s.lx, s.ly, s.lz = 28.0, 22.0, 40.0
        while len(pts) < 48:
            t = rng.uniform(0, 2 * np.pi)
            if len(pts) % 3 == 0:  # next to the curved wall
                f = 0.985 + 0.015 * rng.random()
                q = np.array([14.0 * f * np.cos(t), 11.0 * f * np.sin(t), rng.uniform(-19, 19)])
            elif len(pts) % 3 == 1:  # next to an end cap
                f = 0.8 * np.sqrt(rng.random())
                q = np.array([14.0 * f * np.cos(t), 11.0 * f * np.sin(t),
                              np.sign(rng.random() - 0.5) * (19.75 + 0.25 * rng.random())])
            else:
                f = 0.8 * np.sqrt(rng.random())
                q = np.array([14.0 * f * np.cos(t), 11.0 * f * np.sin(t), rng.uniform(-15, 15)])
            if all(np.sum((q - a) ** 2) >= 9.0 for a in pts):
                pts.append(q)
    p = np.array(pts)
    s.x, s.y, s.z = p[:, 0].copy(), p[:, 1].copy(), p[:, 2].copy()
    s.typei = np.array([1, 2] * 24, np.int32)
    return s


@pytest.mark.parametrize("shape", [abi.SPHERE, abi.ECYL])
@pytest.mark.parametrize("prec", [abi.FP64, abi.FP32])
def test_fixcoor_walls(gpu_lib, oracle_mod, shape, prec):
    """BD steps in a sphere (reflection through the wall) and an elliptic
    cylinder (radial pull-back, clamped ends): positions against the oracle
    after each of 20 steps, and the walls actually acted."""
    spec = _walled(shape, prec)
    g, o = _pair(spec, gpu_lib, oracle_mod, prec, 64)
    tol = 1e-10 if prec == abi.FP64 else 1e-5
    hit = 0
    for k in range(20):
        g.bd_steps(1, seed=91, step0=k, energies=False)
        o.bd_steps(1, seed=91, step0=k, energies=False)
        pg = np.stack(g.get_particles()[:3], 1)
        po = np.stack(o.get_particles()[:3], 1)
        assert np.abs(pg - po).max() <= tol * (k + 1), (k, np.abs(pg - po).max())
        if shape == abi.SPHERE:
            hit += int(np.sum(np.linalg.norm(po, axis=1) > 14.9))
        else:
            ex = (po[:, 0] / 14.0) ** 2 + (po[:, 1] / 11.0) ** 2
            hit += int(np.sum(ex > 0.999) + np.sum(np.abs(po[:, 2]) >= 19.999))
    assert hit > 0
