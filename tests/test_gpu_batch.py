"""Replica batches (bromoc_batch_*): uneven replicas sharing one prototype's
tables and maps give, replica by replica, the FP64 oracle's energies and
forces within the FP32 tolerance, and exactly the BD step of a single
context with the same seed."""
import numpy as np
import pytest

from bromoc_gb300 import abi, synth
from bromoc_gb300.batch import Batch

from . import systems
from .test_gpu_parity import FP32_TOL, energy_err, force_err

pytestmark = pytest.mark.gpu
CAP = 2000
SIZES = [5, 33, 64, 97, 150]


def _replica(r, n):
    s = synth.pore(seed=200 + r, nions=n, maps=systems.small_maps(), radius=6.0,
                   slab=10.0, precision=abi.FP32, rfpar=True, buffers=False,
                   membrane=False)
    if r == 3:  # its own, smaller box: positions scaled into it
        f = 0.8
        s.lx, s.ly = s.lx * f, s.ly * f
        s.x, s.y = s.x * f, s.y * f
    return s


@pytest.fixture(scope="module")
def setup(gpu_lib):
    proto_spec = _replica(99, 20)
    proto = gpu_lib.create(CAP, abi.FP32)
    proto_spec.push(proto)
    reps = [_replica(r, n) for r, n in enumerate(SIZES)]
    b = Batch(proto, SIZES)
    b.set_systems([s.system_struct() for s in reps])
    for r, s in enumerate(reps):
        b.set_particles(r, s.x, s.y, s.z, s.typei)
    return proto, reps, b


def test_batch_energy_forces(setup, oracle_mod):
    _, reps, b = setup
    et, f = b.energy(abi.M_ALL, forces=True)
    for r, s in enumerate(reps):
        o = oracle_mod.create(CAP)
        s.push(o)
        to, fo, _ = o.energy(abi.M_ALL, forces=True)
        off = b.offset(r)
        fb = f[off:off + len(s.x)]
        glob, worst = force_err(fb, fo)
        assert glob <= FP32_TOL and worst <= FP32_TOL, (r, glob, worst)
        tb = {k: et[r, i] for i, k in enumerate(abi.TERM_NAMES)}
        assert energy_err(tb, to) <= 1e-5, (r, tb, to)


def test_batch_bd_step_matches_single(setup, gpu_lib):
    _, reps, b = setup
    seeds = [1000 + 17 * r for r in range(len(reps))]
    b.bd_steps(1, seeds, step0=5)
    for r, s in enumerate(reps):
        g = gpu_lib.create(CAP, abi.FP32)
        s.push(g)
        g.bd_steps(1, seed=seeds[r], step0=5)
        xs, ys, zs = g.get_particles()[:3]
        xb, yb, zb = b.get_particles(r, len(s.x))
        # the batch runs the single context's pair tile, assembly and move
        # on the replica's slots: the same positions bit for bit
        d = np.abs(np.stack([xb - xs, yb - ys, zb - zs])).max()
        assert d == 0.0, (r, d)


def test_batch_rejects_bad_input(setup):
    _, reps, b = setup
    with pytest.raises(abi.BromocError):
        b.set_particles(0, np.zeros(10), np.zeros(10), np.zeros(10), np.ones(10, np.int32))
    with pytest.raises(abi.BromocError):
        b.set_particles(len(SIZES), np.zeros(1), np.zeros(1), np.zeros(1),
                        np.ones(1, np.int32))
