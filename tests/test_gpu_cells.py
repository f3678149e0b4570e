"""The cell list of the periodic extension mode (FP32): parity with the
oracle's all-pairs cutoff sum at 600 ions (5 cells along each edge) and
20,000 ions at 1 M KCl (12 cells along each edge, beyond the all-pairs
tile's 8192 ions), BD steps across the faces, and run-to-run equality (the
cells' ion lists are sorted, so every run sums in one order)."""
import numpy as np
import pytest

from bromoc_gb300 import abi, synth

from .test_gpu_parity import FP32_TOL, energy_err, force_err

pytestmark = pytest.mark.gpu


def _box(n, L, rc, seed, precision=abi.FP32):
    """n ions of 1:1 KCl on a jittered lattice in a periodic cube of edge L,
    3 A apart across the faces too."""
    rng = np.random.default_rng(seed)
    s = synth.bulk_kcl(seed=seed, n_per=1, L=L, srpmf=True, precision=precision,
                       periodic_rcut=rc)
    h = 0.5 * L - 1.5
    p = synth.jittered_lattice(rng, n, -h, h)
    s.x, s.y, s.z = p[:, 0].copy(), p[:, 1].copy(), p[:, 2].copy()
    s.typei = np.array([1, 2] * (n // 2), np.int32)
    return s


CASES = {"600": (600, 80.0, 15.0), "20000": (20000, (20000 / 1.2044e-3) ** (1 / 3), 20.0)}


@pytest.mark.parametrize("case", list(CASES))
def test_cells_energy_forces(gpu_lib, oracle_mod, case):
    n, L, rc = CASES[case]
    assert int(L / (rc * 1.0001)) >= 4  # the cell path, not the all-pairs tile
    spec = _box(n, L, rc, seed=31)
    g = gpu_lib.create(n + 16, abi.FP32)
    o = oracle_mod.create(n + 16)
    spec.push(g)
    spec.push(o)
    tg, fg, _ = g.energy(abi.M_ALL, forces=True)
    to, fo, _ = o.energy(abi.M_ALL, forces=True)
    glob, worst = force_err(fg, fo)
    assert glob <= FP32_TOL and worst <= FP32_TOL, (glob, worst)
    assert energy_err(tg, to) <= FP32_TOL, (tg, to)


def test_cells_bd_steps_across_faces(gpu_lib, oracle_mod):
    n, L, rc = CASES["600"]
    spec = _box(n, L, rc, seed=32)
    g = gpu_lib.create(n + 16, abi.FP32)
    o = oracle_mod.create(n + 16)
    spec.push(g)
    spec.push(o)
    for k in range(20):
        g.bd_steps(1, seed=11, step0=k, energies=False)
        o.bd_steps(1, seed=11, step0=k, energies=False)
    pg = np.stack(g.get_particles()[:3], 1)
    po = np.stack(o.get_particles()[:3], 1)
    d = pg - po
    d -= L * np.rint(d / L)  # an ion right at a face may sit on either side
    assert np.abs(d).max() <= 20 * 1e-5
    assert (po >= -0.5 * L).all() and (po < 0.5 * L).all()


def test_cells_deterministic(gpu_lib):
    n, L, rc = CASES["600"]
    spec = _box(n, L, rc, seed=33)
    out = []
    for _ in range(2):
        g = gpu_lib.create(n + 16, abi.FP32)
        spec.push(g)
        g.bd_steps(5, seed=4, step0=0, energies=False)
        out.append(np.stack(g.get_particles()[:3], 1))
    np.testing.assert_array_equal(out[0], out[1])
