"""GCMC inside a replica batch (bromoc_batch_grand / bromoc_batch_count):
each replica, cycle after cycle of GRAND + BD + COUNT, against the FP64
oracle holding that replica with the replica's seed -- GCMC counters, buffer
tags and signed types exactly, positions within FP32 BD rounding."""
import numpy as np
import pytest

from bromoc_gb300 import _lib, abi, synth
from bromoc_gb300.batch import Batch

from . import systems

pytestmark = pytest.mark.gpu


def _replicas():
    maps = systems.small_maps()
    out = []
    for k, n in enumerate((40, 75, 110)):
        s = synth.pore(seed=60 + k, nions=n, maps=maps, radius=6.0, slab=10.0,
                       precision=abi.FP32, buffers=True, membrane=False)
        s.count()
        out.append(s)
    return out


def test_batch_grand_cycles_match_the_oracle(gpu_lib, oracle_mod):
    reps = _replicas()
    proto = _lib.create(400, abi.FP32)
    reps[0].push(proto)
    caps = [len(s.x) + 40 for s in reps]
    b = Batch(proto, caps)
    b.set_systems([s.system_struct() for s in reps])
    oracles = []
    for r, s in enumerate(reps):
        b.set_particles(r, s.x, s.y, s.z, s.typei)
        b.set_buffers(r, s.buffer_params(), s.ibuffer)
        o = oracle_mod.create(caps[r])
        s.push(o)
        oracles.append(o)
    seeds = np.array([101, 202, 303], np.uint64)
    nb = len(reps[0].buffers)
    moved = 0
    for cyc in range(1, 6):
        dg = b.grand(4, seeds, cyc)
        b.bd_steps(4, seeds, (cyc - 1) * 4)
        b.count()
        for r, o in enumerate(oracles):
            do = o.grand(4, int(seeds[r]), cyc)
            o.bd_steps(4, int(seeds[r]), (cyc - 1) * 4)
            o.count()
            assert abs(dg[r] - do) <= 1e-6 * max(1.0, abs(do)), (cyc, r, dg[r], do)
            xo, yo, zo, to, io = o.get_particles()
            nat, nin, nrm, tg, ig = b.get_buffers(r, nb, caps[r])
            nato, nino, nrmo, _ = o.get_buffers()
            np.testing.assert_array_equal(nat, nato)
            np.testing.assert_array_equal(nin, nino)
            np.testing.assert_array_equal(nrm, nrmo)
            np.testing.assert_array_equal(tg, to)
            np.testing.assert_array_equal(ig, io)
            x, y, z = b.get_particles(r, caps[r])
            assert len(x) == len(xo)
            assert max(np.abs(x - xo).max(), np.abs(y - yo).max(), np.abs(z - zo).max()) <= 2e-4
            moved += int(nin.sum() + nrm.sum())
    assert moved > 0  # the attempts did insert and delete


def test_batch_grand_needs_buffers(gpu_lib):
    reps = _replicas()
    proto = _lib.create(400, abi.FP32)
    reps[0].push(proto)
    b = Batch(proto, [200, 200, 200])
    b.set_systems([s.system_struct() for s in reps])
    for r, s in enumerate(reps):
        b.set_particles(r, s.x, s.y, s.z, s.typei)
    with pytest.raises(abi.BromocError) as e:
        b.grand(2, np.array([1, 2, 3], np.uint64), 1)
    assert e.value.code == abi.E_STATE
