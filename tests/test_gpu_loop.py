"""Fused BD loop (a run of FP32 BD steps as one cooperative launch, loop.cu)
against the per-kernel path (fields, Newton-3 pair kernel, assembly per
step) on the same system, seed and steps.  The loop runs the same force
terms in the same summation order with the same noise, so positions, types,
GCMC and crossing counters must agree bit for bit; the energies of the last
step (formed on the per-kernel path in both) must agree as well.  The FP64
oracle anchors the fused trajectory within the FP32 tolerance of one step."""
import numpy as np
import pytest

from bromoc_gb300 import _lib, abi, synth

from . import systems

pytestmark = pytest.mark.gpu
CAP = 8000
# systems without sites: the fused loop's domain
FAMILIES = ["pairs", "pairs_nosrpmf", "efpot", "maps_trln", "maps_spln", "maps_fixed",
            "gcmc", "efpot_all"]


def _spec(name):
    if name == "efpot_all":
        return systems.efpot_all(precision=abi.FP32)
    if name == "gcmc":
        return systems.gcmc(precision=abi.FP32)
    return systems.all_families()[name](precision=abi.FP32)


def _engine(gpu_lib, spec, fused, cap=CAP):
    g = gpu_lib.create(cap, abi.FP32)
    spec.push(g)
    _lib.set_fused_bd(g, fused)
    return g


def _state(g):
    x, y, z, t, ib = g.get_particles()
    return np.stack([x, y, z], 1), t, ib


def _same(ga, gb):
    pa, ta, iba = _state(ga)
    pb, tb, ibb = _state(gb)
    np.testing.assert_array_equal(ta, tb)
    np.testing.assert_array_equal(iba, ibb)
    assert np.array_equal(pa, pb), np.abs(pa - pb).max()
    return pa


@pytest.mark.parametrize("family", FAMILIES)
def test_loop_matches_per_kernel_steps(gpu_lib, family):
    spec = _spec(family)
    assert spec.nsites == 0
    a = _engine(gpu_lib, spec, True)
    b = _engine(gpu_lib, spec, False)
    ea = a.bd_steps(12, seed=31, step0=5)           # 11 fused + 1 with energies
    eb = b.bd_steps(12, seed=31, step0=5)
    assert ea == eb
    a.bd_steps(7, seed=31, step0=17, energies=False)  # 7 fused
    b.bd_steps(7, seed=31, step0=17, energies=False)
    a.bd_steps(1, seed=31, step0=24, energies=False)  # a single fused step
    b.bd_steps(1, seed=31, step0=24, energies=False)
    _same(a, b)
    # an energy call checks the device error word (no barrier gave up)
    ta, fa, _ = a.energy(abi.M_ALL, forces=True)
    tb, fb, _ = b.energy(abi.M_ALL, forces=True)
    np.testing.assert_array_equal(fa, fb)
    assert ta == tb


def test_loop_one_step_near_oracle(gpu_lib, oracle_mod):
    spec = systems.maps(precision=abi.FP32)
    g = _engine(gpu_lib, spec, True)
    o = oracle_mod.create(CAP)
    spec.push(o)
    g.bd_steps(1, seed=77, step0=3, energies=False)
    o.bd_steps(1, seed=77, step0=3, energies=False)
    pg = _state(g)[0]
    po = np.stack(o.get_particles()[:3], 1)
    assert np.abs(pg - po).max() <= 1e-5


@pytest.mark.parametrize("variant", [abi.DYN1, abi.DYN2])
def test_loop_diffusion_models_and_crossings(gpu_lib, variant):
    spec = systems.maps(precision=abi.FP32)
    nt = spec.ntype
    if variant == abi.DYN1:
        spec.diffusion = dict(plength2=5.0, pcenter=0.0,
                              ampl3=np.full(nt, 0.3), p3=np.full(nt, 2.0))
    else:
        xs = np.linspace(-20, 20, 9)
        ys = 0.6 + 0.4 * np.cos(xs / 8.0)
        b = -0.05 * np.sin(xs / 8.0)
        spec.diffusion = dict(spline=(xs, ys, b, np.zeros(9), np.zeros(9)))
    spec.qcountion = True
    spec.zcont = np.array([-6.0, 0.0, 6.0])
    a = _engine(gpu_lib, spec, True)
    b = _engine(gpu_lib, spec, False)
    a.bd_steps(20, seed=555, step0=0, variant=variant, energies=False)
    b.bd_steps(20, seed=555, step0=0, variant=variant, energies=False)
    _same(a, b)
    for x, y in zip(a.get_countions(), b.get_countions()):
        np.testing.assert_array_equal(x, y)
    assert sum(int(c.sum()) for c in a.get_countions()) > 0


def test_loop_with_gcmc_cycles(gpu_lib):
    spec = systems.gcmc(precision=abi.FP32)
    a = _engine(gpu_lib, spec, True)
    b = _engine(gpu_lib, spec, False)
    for cyc in range(1, 11):
        assert a.grand(6, 4242, cyc) == b.grand(6, 4242, cyc)
        a.bd_steps(4, seed=7, step0=4 * cyc, energies=False)
        b.bd_steps(4, seed=7, step0=4 * cyc, energies=False)
    _same(a, b)
    for x, y in zip(a.get_buffers(), b.get_buffers()):
        np.testing.assert_array_equal(x, y)


@pytest.mark.parametrize("nions", [2000, 6000])
def test_loop_pore_sizes(gpu_lib, nions):
    """The nanopore workload and a size with several tile pairs per warp
    (6000 ions: 188 tiles, 17,766 tile pairs over at most 2,432 warps)."""
    spec = synth.pore(nions=nions, precision=abi.FP32)
    a = _engine(gpu_lib, spec, True)
    b = _engine(gpu_lib, spec, False)
    a.bd_steps(6, seed=2, step0=0, energies=False)
    b.bd_steps(6, seed=2, step0=0, energies=False)
    p = _same(a, b)
    assert np.isfinite(p).all()
    ta, _, _ = a.energy(abi.M_ALL, forces=False)
    tb, _, _ = b.energy(abi.M_ALL, forces=False)
    assert ta == tb


def test_live_count_async(gpu_lib):
    """The count copied on the stream without a wait equals the synchronous
    read, cycle by cycle through GRAND."""
    import ctypes as C
    spec = systems.gcmc(precision=abi.FP32)
    g = _engine(gpu_lib, spec, True)
    got = (C.c_int32 * 8)()
    want = []
    for cyc in range(1, 9):
        g.grand(6, 99, cyc, dener=False)
        _lib.live_count_async(g, C.addressof(got) + 4 * (cyc - 1))
        g.bd_steps(2, seed=5, step0=2 * cyc, energies=False)
        want.append(g.live_ntot())
    assert list(got) == want


def test_fp32_grand_on_records_matches_oracle(gpu_lib, oracle_mod):
    """FP32 mode runs GRAND on the float-float records (no conversion
    kernels): the same insertions and deletions as the FP64 oracle, counter
    for counter, with energy sums and positions equal to within the records'
    ~48-bit precision; interleaved BD steps keep the records authoritative."""
    spec = systems.gcmc(precision=abi.FP32)
    g = _engine(gpu_lib, spec, True)
    o = oracle_mod.create(CAP)
    spec.push(o)
    for cyc in range(1, 13):
        dg = g.grand(6, 4242, cyc)
        do = o.grand(6, 4242, cyc)
        assert abs(dg - do) <= 1e-8 * max(1.0, abs(do)), (cyc, dg, do)
    for x, y in zip(g.get_buffers(), o.get_buffers()):
        np.testing.assert_array_equal(x, y)
    xg, yg, zg, tg, ibg = g.get_particles()
    xo, yo, zo, to, ibo = o.get_particles()
    np.testing.assert_array_equal(tg, to)
    np.testing.assert_array_equal(ibg, ibo)
    np.testing.assert_allclose(np.stack([xg, yg, zg]), np.stack([xo, yo, zo]), atol=1e-10)
    # records stay current through a BD run and a further GRAND call
    g.bd_steps(3, seed=8, step0=0, energies=False)
    n0 = g.live_ntot()
    g.grand(6, 4242, 13)
    p = _state(g)[0]
    assert np.isfinite(p).all() and abs(g.live_ntot() - n0) <= 6
