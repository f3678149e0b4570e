"""Named small workloads of the hot path, each a few calls on cuda:0, for
kernel captures with ncu (the summaries under profiles/ give the exact
command lines):

  python -m bromoc_gb300.cases pairs N     FP32 ENERGY (forces) of an N-ion
                                           pore with the 120x120x180 maps,
                                           3 calls: k_fields_warp_f32,
                                           k_pairs32n, k_assemble_tiles
  python -m bromoc_gb300.cases loop        the nanopore workload (2000 ions,
                                           4 GCMC buffers): 4 cycles of
                                           GRAND(4) + a 10-step k_bd_loop +
                                           COUNT
  python -m bromoc_gb300.cases cells N     FP32 BD steps of N ions of 1 M KCl
                                           in a periodic cube, 20 A cutoff
                                           (the cell-list kernels), 3 steps
  python -m bromoc_gb300.cases batch       the bench's replica batch (256 bulk
                                           KCl replicas, 1.08 M ions): 3 BD steps
  python -m bromoc_gb300.cases adjoint N   the adjoint engine on N ions of 1 M
                                           KCl with tabulated laws: a 20-step
                                           forward (RDF deposit) and backward
  python -m bromoc_gb300.cases ssdna       FP32 BD steps of 40 nt x 3 free sites
                                           with their bonded terms and ~5000
                                           ions in the 120x120x180 pore maps,
                                           3 steps (per-kernel path)
"""
from __future__ import annotations

import sys

import numpy as np

from . import _lib, abi, synth


def pairs(n: int):
    s = synth.pore(seed=3, nions=n, maps=synth.pore_maps(seed=103), precision=abi.FP32,
                   buffers=False)
    g = _lib.create(n + 16, abi.FP32)
    s.push(g)
    for _ in range(3):
        g.energy(abi.M_ALL, forces=True)


def loop():
    s = synth.pore(seed=3, nions=2000, maps=synth.pore_maps(seed=102), precision=abi.FP32,
                   buffers=True)
    g = _lib.create(2400, abi.FP32)
    s.push(g)
    for c in range(4):
        g.grand(4, 1234, c + 1, dener=False)
        g.bd_steps(10, seed=1234, step0=10 * c, energies=False)
        g.count()
    g.live_ntot()


def cells(n: int):
    L = (n / 1.2044e-3) ** (1.0 / 3.0)
    rng = np.random.default_rng(5)
    s = synth.bulk_kcl(seed=5, n_per=1, L=L, srpmf=True, precision=abi.FP32,
                       periodic_rcut=20.0)
    p = synth.jittered_lattice(rng, n, -0.5 * L + 1.5, 0.5 * L - 1.5)
    s.x, s.y, s.z = p[:, 0].copy(), p[:, 1].copy(), p[:, 2].copy()
    s.typei = np.array([1, 2] * (n // 2), np.int32)
    g = _lib.create(n + 16, abi.FP32)
    s.push(g)
    for k in range(3):
        g.bd_steps(1, seed=7, step0=k, energies=False)
    g.live_ntot()


def ssdna():
    s = synth.ssdna(seed=4, nions=5000, nnuc=40, maps=synth.pore_maps(seed=102),
                    precision=abi.FP32, bonded=True, free=True)
    g = _lib.create(len(s.x) + 16, abi.FP32)
    s.push(g)
    for k in range(3):
        g.bd_steps(1, seed=7, step0=k, energies=False)
    g.live_ntot()


def adjoint(n: int):
    from .adjoint import Adjoint, RdfLoss
    rng = np.random.default_rng(7)
    L = (n / (2 * 6.02214e-4)) ** (1.0 / 3.0)
    spec = synth.bulk_kcl(seed=7, n_per=2, L=L, precision=abi.FP32)
    p = synth.jittered_lattice(rng, n, -0.5 * L + 0.5, 0.5 * L - 0.5)
    spec.x, spec.y, spec.z = p[:, 0].copy(), p[:, 1].copy(), p[:, 2].copy()
    spec.typei = np.array([1, 2] * (n // 2), np.int32)
    spec.efpot_res = 0.05
    for key, (sg, ep) in ((("K", "K"), (3.1, 0.09)), (("K", "Cl"), (3.6, 0.11)),
                          (("Cl", "Cl"), (4.0, 0.15))):
        spec.efpot_knots[key] = synth.efpot_knots(rng, sg, ep, r0=1.05, r1=16.0, res=0.05)
    proto = _lib.create(n + 64, abi.FP32)
    spec.push(proto)
    adj = Adjoint(proto, n, abi.FP32)
    adj.set_particles(spec.x, spec.y, spec.z, spec.typei)
    nbins, r0, dr, sig, steps = 150, 0.05, 0.1, 0.1, 20
    rb = r0 + dr * np.arange(nbins)
    loss = RdfLoss(2, [n // 2] * 2, L ** 3, steps, rb, np.ones((3, nbins)))
    hist = adj.forward(steps, 10, 11, 0, nbins, r0, dr, sig, 3)
    _, dl = loss.loss_grad(hist)
    pt = spec.pair_tables()
    adj.backward(dl, int(pt["cnt"]), int(pt["ntc"]))
    adj.close()


def batch(nrep: int = 256):
    """256 bulk KCl replicas, N uniform in [200, 8000], sharing the pore maps:
    3 tuned, graph-replayed BD steps (the bench's batch workload)."""
    from .batch import Batch
    spec = synth.pore(seed=3, nions=2000, maps=synth.pore_maps(seed=102), precision=abi.FP32,
                      buffers=False)
    counts, edges, parts = synth.batch_replicas(nrep=nrep)
    systems = []
    for L in edges:
        sy = spec.system_struct()
        sy.lx = sy.ly = sy.lz = float(L)
        sy.cx = sy.cy = sy.cz = 0.0
        systems.append(sy)
    proto = _lib.create(2064, abi.FP32)
    spec.push(proto)
    b = Batch(proto, counts)
    b.set_systems(systems)
    for r, (x, y, z, t) in enumerate(parts):
        b.set_particles(r, x, y, z, t)
    seeds = np.arange(nrep, dtype=np.uint64) + 1234
    for k in range(3):
        b.bd_steps(1, seeds, k)
    b.close()


def main(argv):
    what = argv[1] if len(argv) > 1 else "loop"
    if what == "batch":
        batch()
    elif what == "adjoint":
        adjoint(int(argv[2]) if len(argv) > 2 else 4096)
    elif what == "pairs":
        pairs(int(argv[2]) if len(argv) > 2 else 8000)
    elif what == "cells":
        cells(int(argv[2]) if len(argv) > 2 else 20000)
    elif what == "loop":
        loop()
    elif what == "ssdna":
        ssdna()
    else:
        raise SystemExit(f"unknown case {what!r}: pairs N | loop | cells N | ssdna")
    print("ok")


if __name__ == "__main__":
    main(sys.argv)
