"""Parity of the CUDA path (through the C ABI) with the CPU FP64 oracle.

Tolerances: FP64 mode reproduces the oracle to summation-order rounding
(1e-10 relative); FP32 pair arithmetic must give forces within 1e-5 relative
of the FP64 oracle, as a whole (||dF|| / ||F||) and particle by particle
against max(|F_i|, RMS |F|).  The floor is there because an FP32 r^2 rounds
at a few 1e-7, which the contact pairs' r^-14 law turns into ~1e-6 of their
force: a particle whose contact forces nearly cancel cannot reach 1e-5 of
its own small net force.
Integer outputs (warning counters, GCMC counters, crossing counts, particle
counts) must match exactly.
"""
import numpy as np
import pytest

from bromoc_gb300 import abi

from . import systems

pytestmark = pytest.mark.gpu
CAP = 4000
FP64_TOL = 1e-10
FP32_TOL = 1e-5


def _engines(spec, gpu_lib, oracle_mod, cap=CAP):
    g = gpu_lib.create(cap, spec.precision)
    o = oracle_mod.create(cap)
    spec.push(g)
    spec.push(o)
    return g, o


def force_err(fg, fo):
    """(global relative error, worst per-particle error against
    max(|F_i|, RMS |F|))."""
    d = np.linalg.norm(fg - fo, axis=1)
    n = np.linalg.norm(fo, axis=1)
    floor = max(np.sqrt(np.mean(n * n)), 1e-300)
    glob = np.linalg.norm(fg - fo) / max(np.linalg.norm(fo), 1e-300)
    return glob, float((d / np.maximum(n, floor)).max())


def energy_err(tg, to):
    scale = max(1.0, sum(abs(v) for k, v in to.items() if k != "ener"))
    return max(abs(tg[k] - to[k]) for k in to) / scale


@pytest.mark.parametrize("family", list(systems.all_families()))
@pytest.mark.parametrize("prec", [abi.FP64, abi.FP32])
def test_energy_forces(gpu_lib, oracle_mod, family, prec):
    spec = systems.all_families()[family](precision=prec)
    g, o = _engines(spec, gpu_lib, oracle_mod)
    tg, fg, wg = g.energy(abi.M_ALL, forces=True)
    to, fo, wo = o.energy(abi.M_ALL, forces=True)
    tol = FP64_TOL if prec == abi.FP64 else FP32_TOL
    glob, worst = force_err(fg, fo)
    assert glob <= tol and worst <= tol, (family, glob, worst)
    etol = FP64_TOL if prec == abi.FP64 else 1e-5
    assert energy_err(tg, to) <= etol, (tg, to)
    np.testing.assert_array_equal(wg, wo)


@pytest.mark.parametrize("mask", [abi.M_NONBOND, abi.M_MEMB, abi.M_PHIX,
                                  abi.M_PHIV, abi.M_RFPAR, 0])
def test_term_masks(gpu_lib, oracle_mod, mask):
    """ENERGY keyword masks (shell_simul.f90:1428-1465) switch terms off."""
    spec = systems.maps(precision=abi.FP64)
    g, o = _engines(spec, gpu_lib, oracle_mod)
    tg, fg, _ = g.energy(mask, forces=True)
    to, fo, _ = o.energy(mask, forces=True)
    assert energy_err(tg, to) <= FP64_TOL
    if np.linalg.norm(fo) > 0:
        assert force_err(fg, fo)[0] <= FP64_TOL
    else:
        assert np.abs(fg).max() == 0.0


def test_rfpar_zero_cells(gpu_lib, oracle_mod):
    """Zero gsrfen cells trigger the reference's early exit of the gather
    loop (rfpar.f90:121) identically on both sides."""
    from bromoc_gb300 import synth
    maps = synth.pore_maps(seed=21, nclx=28, ncly=28, nclz=40, radius=6.0,
                           slab=10.0, zero_mouth=True)
    spec = synth.pore(seed=22, nions=90, maps=maps, radius=6.0, slab=10.0,
                      precision=abi.FP64, buffers=False)
    g, o = _engines(spec, gpu_lib, oracle_mod)
    tg, fg, _ = g.energy(abi.M_RFPAR, forces=True)
    to, fo, _ = o.energy(abi.M_RFPAR, forces=True)
    assert energy_err(tg, to) <= FP64_TOL
    assert force_err(fg, fo)[0] <= FP64_TOL


@pytest.mark.parametrize("family", ["pairs", "efpot", "maps_trln",
                                    "maps_spln", "dna"])
def test_interact(gpu_lib, oracle_mod, family):
    """INTERACT of existing particles (deletion trials) and of insertion
    trials at fresh points, FP64 on both sides."""
    spec = systems.all_families()[family](precision=abi.FP64)
    g, o = _engines(spec, gpu_lib, oracle_mod)
    rng = np.random.default_rng(1)
    n = len(spec.x)
    for j in list(range(spec.nsites, n, max(1, n // 12))):
        it = abs(int(spec.typei[j]))
        a = g.interact(spec.x[j], spec.y[j], spec.z[j], it, j + 1)
        b = o.interact(spec.x[j], spec.y[j], spec.z[j], it, j + 1)
        assert abs(a - b) <= FP64_TOL * max(1.0, abs(b)), (j, a, b)
    half = 0.5 * np.array([spec.lx, spec.ly, spec.lz]) - 1.0
    for _ in range(8):
        p = rng.uniform(-half, half)
        it = spec.nold + 1 + int(rng.integers(0, spec.nion))
        a = g.interact(*p, it, n + 1)
        b = o.interact(*p, it, n + 1)
        assert abs(a - b) <= FP64_TOL * max(1.0, abs(b)), (p, a, b)


@pytest.mark.parametrize("family", ["pairs", "maps_trln", "maps_spln", "dna", "dna_duplex"])
def test_bd_steps(gpu_lib, oracle_mod, family):
    """ENERGY + DYNAMICS: identical Philox noise on both sides, so positions
    agree to rounding after one step and stay close over ten."""
    spec = systems.all_families()[family](precision=abi.FP64)
    g, o = _engines(spec, gpu_lib, oracle_mod)
    g.bd_steps(1, seed=2024, step0=0)
    o.bd_steps(1, seed=2024, step0=0)
    pg = np.stack(g.get_particles()[:3], 1)
    po = np.stack(o.get_particles()[:3], 1)
    assert np.abs(pg - po).max() <= 1e-10
    g.bd_steps(9, seed=2024, step0=1)
    o.bd_steps(9, seed=2024, step0=1)
    pg = np.stack(g.get_particles()[:3], 1)
    po = np.stack(o.get_particles()[:3], 1)
    assert np.abs(pg - po).max() <= 1e-7


@pytest.mark.parametrize("family", ["pairs", "maps_trln", "efpot"])
def test_bd_step_fp32(gpu_lib, oracle_mod, family):
    """FP32 pair path + single-precision Box-Muller: one BD step lands within
    1e-5 A of the FP64 oracle (force error 1e-5 relative times D dt / kT,
    plus ~1e-7 relative noise error)."""
    spec = systems.all_families()[family](precision=abi.FP32)
    g, o = _engines(spec, gpu_lib, oracle_mod)
    g.bd_steps(1, seed=77, step0=3)
    o.bd_steps(1, seed=77, step0=3)
    pg = np.stack(g.get_particles()[:3], 1)
    po = np.stack(o.get_particles()[:3], 1)
    assert np.abs(pg - po).max() <= 1e-5


@pytest.mark.parametrize("variant", [abi.DYN1, abi.DYN2, abi.DYN3])
def test_dynamics_variants(gpu_lib, oracle_mod, variant):
    """dynamics1 (z-switch D), dynamics2 (spline D(z)), dynamics3 (DNA
    proximity D) plus countions crossing counters."""
    spec = systems.dna(precision=abi.FP64) if variant == abi.DYN3 else \
        systems.maps(precision=abi.FP64)
    nt = spec.ntype
    if variant == abi.DYN1:
        spec.diffusion = dict(plength2=5.0, pcenter=0.0,
                              ampl3=np.full(nt, 0.3), p3=np.full(nt, 2.0))
    elif variant == abi.DYN2:
        xs = np.linspace(-20, 20, 9)
        ys = 0.6 + 0.4 * np.cos(xs / 8.0)
        b = -0.05 * np.sin(xs / 8.0)
        spec.diffusion = dict(spline=(xs, ys, b, np.zeros(9), np.zeros(9)))
    spec.qcountion = True
    spec.zcont = np.array([-6.0, 0.0, 6.0])
    g, o = _engines(spec, gpu_lib, oracle_mod)
    for k in range(5):
        g.energy(abi.M_ALL, forces=True)
        o.energy(abi.M_ALL, forces=True)
        g.dynamics(variant, 555, k)
        o.dynamics(variant, 555, k)
    pg = np.stack(g.get_particles()[:3], 1)
    po = np.stack(o.get_particles()[:3], 1)
    assert np.abs(pg - po).max() <= 1e-8
    for a, b in zip(g.get_countions(), o.get_countions()):
        np.testing.assert_array_equal(a, b)
    if variant == abi.DYN3:
        np.testing.assert_allclose(g.get_dids(), o.get_dids(), atol=1e-10)


def test_gcmc_chain(gpu_lib, oracle_mod):
    """GRAND on the device: the same insertions and deletions as the oracle
    (integer counters exact), the same particle arrays after compaction."""
    spec = systems.gcmc(precision=abi.FP64)
    g, o = _engines(spec, gpu_lib, oracle_mod)
    for cyc in range(1, 16):
        dg = g.grand(6, 4242, cyc)
        do = o.grand(6, 4242, cyc)
        assert abs(dg - do) <= 1e-8 * max(1.0, abs(do))
        g.bd_steps(2, seed=7, step0=2 * cyc)
        o.bd_steps(2, seed=7, step0=2 * cyc)
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
    np.testing.assert_allclose(np.stack([xg, yg, zg]), np.stack([xo, yo, zo]),
                               atol=1e-7)


def test_bd_steps_host_dropin(gpu_lib, oracle_mod):
    """The host-array entry point that replaces simul1's BD loop."""
    import ctypes as C
    spec = systems.pairs(precision=abi.FP64)
    g, o = _engines(spec, gpu_lib, oracle_mod)
    x, y, z = spec.x.copy(), spec.y.copy(), spec.z.copy()
    t = spec.typei.copy()
    e = np.zeros(abi.NTERMS)
    P = lambda a, ct: a.ctypes.data_as(C.POINTER(ct))
    rc = g.lib.bromoc_gpu_bd_steps_host(
        g.h, abi.M_ALL, abi.DYN0, 3, 99, 0, len(x), 0, 0, P(x, C.c_double),
        P(y, C.c_double), P(z, C.c_double), P(t, C.c_int32), P(e, C.c_double))
    assert rc == 0
    o.bd_steps(3, seed=99, step0=0)
    po = np.stack(o.get_particles()[:3], 1)
    assert np.abs(np.stack([x, y, z], 1) - po).max() <= 1e-9


def test_deterministic(gpu_lib):
    """Fixed-order reductions: two runs are bit-identical."""
    spec = systems.maps(precision=abi.FP32)
    out = []
    for _ in range(2):
        g = gpu_lib.create(CAP, spec.precision)
        spec.push(g)
        g.bd_steps(5, seed=3, step0=0)
        out.append(np.stack(g.get_particles()[:3], 1))
    np.testing.assert_array_equal(out[0], out[1])


def test_capacity_error(gpu_lib):
    """Insertion beyond capacity is reported, not a crash."""
    spec = systems.gcmc(nions=30, precision=abi.FP64)
    g = gpu_lib.create(len(spec.x) + 2, spec.precision)
    spec.push(g)
    with pytest.raises(abi.BromocError) as ei:
        for cyc in range(1, 400):
            g.grand(10, 11, cyc)  # syncs and checks the device error flags
    assert ei.value.code == abi.E_CAPACITY
    # the context stays usable after the error
    g.energy()


def test_full_size_fp32_vs_fp64(gpu_lib):
    """Pore workload at full size (2000 ions, 120x120x180 maps): FP32 pairs
    against the GPU's own FP64 path, and Newton's third law of the pair
    forces (sum zero) in FP64."""
    from bromoc_gb300 import synth
    s64 = synth.pore(seed=3, nions=2000, precision=abi.FP64, buffers=False)
    g64 = gpu_lib.create(CAP, abi.FP64)
    s64.push(g64)
    t64, f64, _ = g64.energy(abi.M_ALL, forces=True)
    g32 = gpu_lib.create(CAP, abi.FP32)
    s64.push(g32)
    t32, f32, _ = g32.energy(abi.M_ALL, forces=True)
    glob, worst = force_err(f32, f64)
    assert glob <= FP32_TOL, glob
    _, fnb, _ = g64.energy(abi.M_NONBOND, forces=True)
    assert np.abs(fnb.sum(0)).max() <= 1e-9 * np.abs(fnb).sum()
