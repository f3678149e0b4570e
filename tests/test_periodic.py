"""Extension mode of the bulk configuration (no counterpart in the
reference): a periodic box in which ion pairs interact through the nearest
image when closer than a plain cutoff, with every move wrapped into the box.

CPU tests pin the oracle's switch: TEST's central-difference forces, the
nearest-image geometry and the wrap.  GPU tests compare the CUDA path with
the oracle in that mode: FP64 to summation order, FP32 within the FP32
tolerance, BD trajectories across the faces, the fused loop against the
per-kernel steps, INTERACT, and the entry points that refuse the mode."""
import numpy as np
import pytest

from bromoc_gb300 import abi, synth

from .test_oracle import _fd_forces

CAP = 2000
RCUT, L = 20.0, 60.0


def _spec(precision=abi.FP64, n_per=130, seed=21):
    return synth.bulk_kcl(seed=seed, n_per=n_per, L=L, srpmf=True, precision=precision,
                          periodic_rcut=RCUT)


def _min_image(d):
    return d - L * np.rint(d / L)


def _far_from_cutoff(spec, idx, margin):
    """Particles none of whose nearest-image pair distances lies within
    margin of the cutoff (a central difference across it sees the jump)."""
    p = np.stack([spec.x, spec.y, spec.z], 1)
    keep = []
    for i in idx:
        d = np.linalg.norm(_min_image(p - p[i]), axis=1)
        d[i] = 0.0
        if not np.any(np.abs(d - RCUT) < margin):
            keep.append(i)
    return keep


def test_oracle_fd_forces_periodic(oracle_mod):
    spec = _spec()
    eng = oracle_mod.create(CAP).load(spec)
    _, f, _ = eng.energy(abi.M_ALL, forces=True)
    p = np.stack([spec.x, spec.y, spec.z], 1)
    # ions near the faces first: their forces come through the images
    order = np.argsort(-np.abs(p).max(1))
    idx = _far_from_cutoff(spec, order[:60], 5e-3)[:25]
    fd = _fd_forces(eng, spec, abi.M_ALL, idx=idx)
    for i, v in fd.items():
        assert np.abs(v - f[i]).max() <= 1e-3, (i, v, f[i])


def test_oracle_nearest_image_pair(oracle_mod):
    """Two ions 4 A apart through the x faces have the energy of the same
    pair 4 A apart in the middle of the box."""
    a = _spec(n_per=1)
    a.x = np.array([0.5 * L - 2.0, -0.5 * L + 2.0])
    a.y = np.zeros(2)
    a.z = np.zeros(2)
    b = _spec(n_per=1)
    b.x = np.array([-2.0, 2.0])
    b.y = np.zeros(2)
    b.z = np.zeros(2)
    ea = oracle_mod.create(16).load(a).energy(abi.M_ALL, forces=False)[0]
    eb = oracle_mod.create(16).load(b).energy(abi.M_ALL, forces=False)[0]
    assert ea["ener"] != 0.0
    assert abs(ea["ener"] - eb["ener"]) <= 1e-12 * abs(eb["ener"])


def test_oracle_moves_wrap(oracle_mod):
    spec = _spec()
    eng = oracle_mod.create(CAP).load(spec)
    p0 = np.stack([spec.x, spec.y, spec.z], 1)
    eng.bd_steps(200, seed=3, step0=0, energies=False)
    p = np.stack(eng.get_particles()[:3], 1)
    assert (p >= -0.5 * L).all() and (p < 0.5 * L).all()
    # a hard-walled box clamps at the faces; here some ions crossed them
    jump = np.abs(p - p0).max(1)
    assert (jump > 0.5 * L).any()


@pytest.mark.gpu
class TestGpuPeriodic:
    def _pair(self, gpu_lib, oracle_mod, precision, at_face=False):
        spec = _spec(precision=precision)
        if at_face:  # six ions 0.05 A inside the +x face: they cross it soon
            far = np.argsort(-spec.x)[:6]
            spec.x[far] = 0.5 * L - 0.05
        g = gpu_lib.create(CAP, precision)
        spec.push(g)
        o = oracle_mod.create(CAP)
        spec.push(o)
        return spec, g, o

    def test_energy_forces_fp64(self, gpu_lib, oracle_mod):
        _, g, o = self._pair(gpu_lib, oracle_mod, abi.FP64)
        tg, fg, _ = g.energy(abi.M_ALL, forces=True)
        to, fo, _ = o.energy(abi.M_ALL, forces=True)
        scale = max(1.0, sum(abs(v) for k, v in to.items() if k != "ener"))
        assert max(abs(tg[k] - to[k]) for k in to) / scale <= 1e-10
        assert np.linalg.norm(fg - fo) / np.linalg.norm(fo) <= 1e-10

    def test_energy_forces_fp32(self, gpu_lib, oracle_mod):
        from .test_gpu_parity import FP32_TOL, energy_err, force_err
        _, g, o = self._pair(gpu_lib, oracle_mod, abi.FP32)
        tg, fg, _ = g.energy(abi.M_ALL, forces=True)
        to, fo, _ = o.energy(abi.M_ALL, forces=True)
        glob, worst = force_err(fg, fo)
        assert glob <= FP32_TOL and worst <= 10 * FP32_TOL, (glob, worst)
        assert energy_err(tg, to) <= 1e-5

    def test_bd_trajectory_fp64(self, gpu_lib, oracle_mod):
        spec, g, o = self._pair(gpu_lib, oracle_mod, abi.FP64, at_face=True)
        g.bd_steps(40, seed=9, step0=0, energies=False)
        o.bd_steps(40, seed=9, step0=0, energies=False)
        pg = np.stack(g.get_particles()[:3], 1)
        po = np.stack(o.get_particles()[:3], 1)
        assert np.abs(pg - po).max() <= 1e-8
        p0 = np.stack([spec.x, spec.y, spec.z], 1)
        assert (np.abs(pg - p0).max(1) > 0.5 * L).any()  # some ions wrapped

    def test_fused_loop_matches_per_kernel(self, gpu_lib):
        from bromoc_gb300 import _lib
        spec = _spec(precision=abi.FP32)
        a = gpu_lib.create(CAP, abi.FP32)
        b = gpu_lib.create(CAP, abi.FP32)
        spec.push(a)
        spec.push(b)
        _lib.set_fused_bd(b, False)
        a.bd_steps(60, seed=4, step0=0, energies=False)
        b.bd_steps(60, seed=4, step0=0, energies=False)
        pa = np.stack(a.get_particles()[:3], 1)
        pb = np.stack(b.get_particles()[:3], 1)
        assert np.array_equal(pa, pb)
        assert (pa >= -0.5 * L).all() and (pa < 0.5 * L).all()

    def test_fp32_one_step_near_oracle(self, gpu_lib, oracle_mod):
        _, g, o = self._pair(gpu_lib, oracle_mod, abi.FP32)
        g.bd_steps(1, seed=2, step0=0, energies=False)
        o.bd_steps(1, seed=2, step0=0, energies=False)
        pg = np.stack(g.get_particles()[:3], 1)
        po = np.stack(o.get_particles()[:3], 1)
        d = np.abs(_min_image(pg - po)).max()
        assert d <= 1e-5

    def test_interact(self, gpu_lib, oracle_mod):
        spec, g, o = self._pair(gpu_lib, oracle_mod, abi.FP64)
        n = len(spec.x)
        for j in range(0, n, 37):
            it = abs(int(spec.typei[j]))
            a = g.interact(spec.x[j], spec.y[j], spec.z[j], it, j + 1)
            b = o.interact(spec.x[j], spec.y[j], spec.z[j], it, j + 1)
            assert abs(a - b) <= 1e-10 * max(1.0, abs(b)), (j, a, b)
        for p in ([0.5 * L - 0.2, 0.0, 0.0], [-0.5 * L + 0.1, 0.5 * L - 0.1, 3.0]):
            a = g.interact(*p, 1, n + 1)
            b = o.interact(*p, 1, n + 1)
            assert abs(a - b) <= 1e-10 * max(1.0, abs(b)), (p, a, b)

    @pytest.mark.parametrize("precision", [abi.FP64, abi.FP32])
    def test_grand_nearest_image(self, gpu_lib, oracle_mod, precision):
        """GRAND in the extension mode: ΔE through the nearest image within
        the cutoff (float-float in the GPU kernel), the same attempts and
        outcomes as the oracle."""
        spec = _spec(precision=precision, n_per=60)
        spec.buffers = [dict(ion="K", conc=1.5, lzmin=-0.5 * L, lzmax=0.5 * L),
                        dict(ion="Cl", conc=0.5, lzmin=-0.5 * L, lzmax=0.5 * L)]
        spec.count()
        g = gpu_lib.create(CAP, precision)
        spec.push(g)
        o = oracle_mod.create(CAP)
        spec.push(o)
        for cyc in range(1, 7):
            dg, do = g.grand(8, 31, cyc), o.grand(8, 31, cyc)
            assert abs(dg - do) <= 1e-8 * max(1.0, abs(do)), (cyc, dg, do)
        for x, y in zip(g.get_buffers(), o.get_buffers()):
            np.testing.assert_array_equal(x, y)
        _, nins, nrem, _ = o.get_buffers()
        assert nins.sum() + nrem.sum() > 0
        pg, po = g.get_particles(), o.get_particles()
        np.testing.assert_array_equal(pg[3], po[3])
        np.testing.assert_array_equal(pg[4], po[4])
        np.testing.assert_allclose(np.stack(pg[:3]), np.stack(po[:3]), atol=1e-9)

    def test_refusals(self, gpu_lib):
        sph = synth.bulk_kcl(n_per=4, L=30.0)
        sph.shape = abi.SPHERE
        sph.rsphe = 14.0
        g = gpu_lib.create(64, abi.FP64)
        sph.push(g)
        with pytest.raises(abi.BromocError):
            g.call("set_periodic", 1, 10.0)
        from bromoc_gb300.batch import Batch
        proto = gpu_lib.create(64, abi.FP32)
        _spec(precision=abi.FP32, n_per=8).push(proto)
        with pytest.raises(abi.BromocError):
            Batch(proto, [10, 20])
