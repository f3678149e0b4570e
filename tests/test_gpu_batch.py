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


def _uneven_batch(gpu_lib, sizes, seed=300):
    proto_spec = _replica(99, 20)
    proto = gpu_lib.create(CAP, abi.FP32)
    proto_spec.push(proto)
    reps = []
    for r, n in enumerate(sizes):
        if n < 500:
            reps.append(_replica(seed + r, n))
            continue
        # a bulk cube at 1 M for the larger replicas
        s = _replica(seed + r, 20)
        L = (n / (2.0 * 6.02214e-4)) ** (1.0 / 3.0)
        p = synth.jittered_lattice(np.random.default_rng(seed + r), n, -0.5 * L + 0.5,
                                   0.5 * L - 0.5)
        s.lx = s.ly = s.lz = float(L)
        s.x, s.y, s.z = p[:, 0].copy(), p[:, 1].copy(), p[:, 2].copy()
        s.typei = np.array([1, 2] * (n // 2), np.int32)
        reps.append(s)
    b = Batch(proto, sizes)
    b.set_systems([s.system_struct() for s in reps])
    for r, s in enumerate(reps):
        b.set_particles(r, s.x, s.y, s.z, s.typei)
    return proto, reps, b


def test_graph_replay_matches_launches(gpu_lib):
    """Runs replayed from the captured graph (several calls, changing step0
    and seeds) and the same runs launched one by one agree bit for bit;
    the graph is captured once per step count and replayed."""
    sizes = [40, 150, 1100, 70]
    out = []
    for graph in (True, False):
        _, reps, b = _uneven_batch(gpu_lib, sizes)
        b.set_graph(graph)
        for call in range(3):
            seeds = [500 + 13 * r + call for r in range(len(sizes))]
            b.bd_steps(2, seeds, step0=10 * call)
        if graph:
            assert b.graph_launches() == 3
        out.append([np.stack(b.get_particles(r, sizes[r])) for r in range(len(sizes))])
    for a, c in zip(*out):
        np.testing.assert_array_equal(a, c)


def test_autotuner_chooses_per_bucket(gpu_lib):
    sizes = [40, 1100, 60]
    _, _, b = _uneven_batch(gpu_lib, sizes)
    w, n, ms = b.tuning()
    assert (w == 0).all()  # nothing tuned before the first step
    b.bd_steps(1, [1, 2, 3], step0=0)
    w, n, ms = b.tuning()
    assert n[0] > 0 and n[1] > 0 and n[2] == 0
    for k in range(3):
        if n[k]:
            assert w[k] in (2, 4, 8) and (ms[k] > 0).all()
            assert ms[k][[2, 4, 8].index(w[k])] == ms[k].min()
        else:
            assert w[k] == 0
