#!/usr/bin/env python
"""particle-steps/s of the cg-gcmc-bd inner loop on GB300.

Workload (the nanopore system with grid maps): 120x120x180 maps at 1 A
(static field = 1 V drop + seeded Gaussians, RFPAR Born-like wall penalty,
repulsion slab with a 10 A pore, repwalls layers), ~2000 K+/Cl- ions with
Coulomb/cdie 80 + LJ + SRPMF pairs, four GCMC buffers (1 M) at both ends.
One bench step = one simul1 cycle: GRAND with 4 attempts, then 10 BD steps
(ENERGY forces + dynamics0).  GPU arm: pair laws and the BD update in FP32
(float-float positions, compensated force sums); the GCMC acceptance ΔE in
float-float on the FP32 pipe (about 48 bits; the FP64 formula where float's
range does not hold), not FP64.  The CPU arm is FP64 throughout.  Energy
totals are not formed in the timed BD steps (forces only), as simul1 forms
them only at its print steps.  Synthetic inputs (the reference ships no maps
or decks).

The line also carries "batched": 256 bulk KCl replicas of 200-8000 ions
(1 M, cube boxes, the same maps) advanced by the replica-batch engine, timed
against the plain path run replica by replica through one context; and
"adjoint": the gradient of a smoothed-RDF loss over a 2000-step segment of
4096 ions with respect to 3x300 EFPOT knots (forward + adjoint times).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

N > 1 (torchrun): replicas only -- every rank advances its own replica (its
own seed), no data-path collective; value = all ranks' particle-steps / the
slowest rank's time.  --impl reference times the CPU restatement of the
reference routines (the Fortran reference cannot be built here) on the
host cores, rank 0 only.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import re
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

from bromoc_gb300 import abi, replicas, synth  # noqa: E402

METRIC = ("particle-steps/s, 1 GB300: plain vs batched+adjoint, force rel err "
          "≤1e-5 vs FP64")
NGCMC, NBD = 4, 10
NIONS = 2000
SEED = 1234
L2_FLUSH_BYTES = 256 << 20  # > 129 MB L2
PAIR_FLOP = 38              # LJ + Coulomb pair, algorithmic FLOP per pair
RF_FLOP = 32                # RFPAR cross term, FLOP per unordered pair


def workload(rank: int = 0, precision=abi.FP32):
    maps = synth.pore_maps(seed=102)
    spec = synth.pore(seed=replicas.replica_seed(3, rank), nions=NIONS, maps=maps,
                      precision=precision, buffers=True)
    return spec


def config_dict():
    return {"workload": f"nanopore-{NIONS}: 120x120x180 maps (phix, phiv+repwalls, "
                        "rfpar), K+/Cl- Coulomb+LJ+SRPMF, 4 GCMC buffers",
            "step": f"one cycle = GRAND({NGCMC} attempts) + {NBD} BD steps + COUNT",
            "nions": NIONS, "grid": [120, 120, 180], "ngcmc": NGCMC, "nbd": NBD,
            "pairs": "all pairs (no cutoff); arithmetic per arm under 'precision'",
            "energy_totals": "not formed in the timed BD steps (forces only)",
            "l2": "flushed between timed steps (256 MB write outside the events)"}


PRECISION_GPU = {"pairs": "FP32 arithmetic, float-float positions, compensated FP32 "
                          "force sums",
                 "gcmc_dE": "float-float on the FP32 pipe (~2^-47 per operation); "
                            "FP64 formula where float's range does not hold",
                 "energy_totals": "FP64 sums of FP32 block partials"}
PRECISION_CPU = {"pairs": "FP64", "gcmc_dE": "FP64", "energy_totals": "FP64"}


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
BATCH_NREP = 256


def batch_measure(sh, flush, steps=10, warm=3, plain_steps=3):
    """Batched replicas (256 bulk KCl systems, N uniform in [200, 8000], 1 M,
    cube boxes, the nanopore maps) against the plain path launched replica
    by replica through one context; CUDA events on the shared stream, L2
    flushed before every timed launch outside the events."""
    import torch
    from bromoc_gb300 import _lib
    from bromoc_gb300.batch import Batch
    spec = synth.pore(seed=3, nions=NIONS, maps=synth.pore_maps(seed=102),
                      precision=abi.FP32, buffers=False)
    counts, edges, parts = synth.batch_replicas(nrep=BATCH_NREP)
    systems = []
    for L in edges:
        sy = spec.system_struct()
        sy.lx = sy.ly = sy.lz = float(L)
        sy.cx = sy.cy = sy.cz = 0.0
        systems.append(sy)
    proto = _lib.create(NIONS + 64, abi.FP32, sh)
    spec.push(proto)
    b = Batch(proto, counts)
    b.set_systems(systems)
    for r, (x, y, z, t) in enumerate(parts):
        b.set_particles(r, x, y, z, t)
    seeds = np.arange(BATCH_NREP, dtype=np.uint64) + SEED
    stream = torch.cuda.current_stream()
    b.bd_steps(warm, seeds, 0)
    torch.cuda.synchronize()
    l0 = b.launch_count()
    tb = 0.0
    for k in range(steps):
        flush.zero_()
        a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        b.bd_steps(1, seeds, warm + k)
        e.record(stream)
        torch.cuda.synchronize()
        tb += a.elapsed_time(e)
    launches = b.launch_count() - l0
    nions = int(counts.sum())
    value = nions * steps / (tb * 1e-3)
    tw, tn, tms = b.tuning()
    graph_calls = b.graph_launches()
    b.close()
    # plain path, replica by replica
    g = _lib.create(int(counts.max()) + 64, abi.FP32, sh)
    spec.push(g)
    tp = 0.0
    tp_rep = np.zeros(len(parts))
    for r, (x, y, z, t) in enumerate(parts):
        g.call("set_system", C.byref(systems[r]))
        g.set_particles(x, y, z, t)
        g.bd_steps(1, int(seeds[r]), 0, energies=False)
        torch.cuda.synchronize()
        flush.zero_()
        a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        g.bd_steps(plain_steps, int(seeds[r]), 1, energies=False)
        e.record(stream)
        torch.cuda.synchronize()
        tp_rep[r] = a.elapsed_time(e)
        tp += tp_rep[r]
    plain = nions * plain_steps / (tp * 1e-3)
    del g
    # per size bucket: the bucket's replicas as a batch of their own against
    # the same replicas on the plain path (times above)
    buckets = []
    for k, (lo, hi) in enumerate(((0, 999), (1000, 4000), (4001, 1 << 30))):
        sel = [r for r in range(len(counts)) if lo <= counts[r] <= hi]
        if not sel:
            continue
        sb = Batch(proto, [int(counts[r]) for r in sel])
        sb.set_systems([systems[r] for r in sel])
        for j, r in enumerate(sel):
            sb.set_particles(j, *parts[r])
        sseeds = seeds[sel]
        sb.bd_steps(warm, sseeds, 0)
        torch.cuda.synchronize()
        ts = 0.0
        for kk in range(steps):
            flush.zero_()
            a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            sb.bd_steps(1, sseeds, warm + kk)
            e.record(stream)
            torch.cuda.synchronize()
            ts += a.elapsed_time(e)
        nb_ions = int(counts[sel].sum())
        bv = nb_ions * steps / (ts * 1e-3)
        pv = nb_ions * plain_steps / (tp_rep[sel].sum() * 1e-3)
        buckets.append({"ions_range": [lo, min(hi, 8000)], "replicas": len(sel),
                        "ions": nb_ions, "batch": bv, "plain_per_replica": pv,
                        "speedup": bv / pv, "pair_warps_chosen": int(sb.tuning()[0][k])})
        sb.close()
    del proto
    return {"workload": f"{BATCH_NREP} bulk KCl replicas, N uniform in [200, 8000] "
                        f"({nions} ions), 1 M, cube boxes, shared 120x120x180 maps, "
                        "ENERGY (Coulomb+LJ+SRPMF, fields, RFPAR) + dynamics0, FP32",
            "value": value, "unit": "particle-steps/s", "ms_per_step": tb / steps,
            "steps": steps, "gpu_launches": launches,
            "plain_per_replica": {"value": plain, "ms_per_step": tp / plain_steps,
                                  "steps": plain_steps},
            "speedup_vs_plain": value / plain,
            "graph": {"calls_replayed": graph_calls,
                      "note": "each bd_steps call: one CUDA-graph launch (seed and step "
                              "uploads, then per step the field pass and, per size bucket, "
                              "the pair and assembly launches)"},
            "autotuner": {"buckets": ["<1000", "1000-4000", ">4000"],
                          "pair_warps_per_block": [int(v) for v in tw],
                          "pair_items": [int(v) for v in tn],
                          "pair_pass_ms_by_warps_2_4_8": [[float(x) for x in row] for row in tms]},
            "per_bucket": buckets}


def pair_scaling(sh, peak_fp32, sizes=(2000, 4000, 8000), reps=10):
    """The Newton-3 pair kernel alone on larger pores (the same maps and
    laws), where the tile pairs outnumber the warps: its FP32 roofline
    without the latency floor of the 2000-ion step.  CUDA events around
    each launch (the library's kernel timers), after three warm-up calls."""
    from bromoc_gb300 import _lib
    maps = synth.pore_maps(seed=102)
    out = []
    for n in sizes:
        spec = synth.pore(seed=3, nions=n, maps=maps, precision=abi.FP32, buffers=False)
        g = _lib.create(n + 64, abi.FP32, sh)
        spec.push(g)
        for _ in range(3):
            g.energy(abi.M_ALL, forces=True)
        _lib.kernel_timing(g, True)
        for _ in range(reps):
            g.energy(abi.M_ALL, forces=True)
        ms, nl = _lib.kernel_time(g, _lib.K_PAIRS)
        _lib.kernel_timing(g, False)
        n_ion = g.live_ntot()
        pairs = n_ion * (n_ion - 1) / 2
        t = ms / nl * 1e-3
        a = (PAIR_FLOP + RF_FLOP) * pairs / t / 1e12
        row = {"ions": n_ion, "launch_us": t * 1e6, "achieved_tflops": a,
               "frac": a / peak_fp32}
        traffic, prof = profile_traffic(f"k_pairs32n/{n}")
        if traffic is not None:
            row["traffic"] = traffic
            row["traffic_source"] = prof
        out.append(row)
        del g
    return out


BULK_STEPS = 2000


def bulk_measure(sh, steps=BULK_STEPS):
    """The bulk configuration: 130 K+ and 130 Cl- in a 60 A cube, FP64,
    dt 0.02 ps; reference semantics (hard walls, all pairs) and the
    extension mode (periodic, 20 A cutoff).  GPU: `steps` BD steps per call
    (ENERGY forces + dynamics0), CUDA events on the shared stream after
    warm-up.  CPU: the oracle restatement, one thread, a bounded sample of
    the same steps."""
    import torch
    from bromoc_gb300 import _lib
    from oracle import oracle
    out = {"workload": "bulk KCl: 130 K+ / 130 Cl- (1 M), 60 A cube, FP64, dt 0.02 ps"}
    stream = torch.cuda.current_stream()
    for mode, rc in (("hard_walls", None), ("periodic_rc20", 20.0)):
        spec = synth.bulk_kcl(seed=SEED, n_per=130, L=60.0, srpmf=True, precision=abi.FP64,
                              periodic_rcut=rc)
        g = _lib.create(300, abi.FP64, sh)
        spec.push(g)
        g.bd_steps(50, SEED, 0, energies=False)
        a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(stream)
        g.bd_steps(steps, SEED, 50, energies=False)
        e.record(stream)
        torch.cuda.synchronize()
        ms = a.elapsed_time(e)
        lib = oracle.load(omp=True)
        lib.bromoc_ref_set_threads(1)
        o = oracle.create(300, omp=True)
        spec.push(o)
        ncpu, t0 = 0, time.perf_counter()
        while time.perf_counter() - t0 < 2.0:
            o.bd_steps(20, SEED, ncpu, energies=False)
            ncpu += 20
        dt = time.perf_counter() - t0
        lib.bromoc_ref_set_threads(int(os.cpu_count() or 1))
        out[mode] = {"value": 260 * steps / (ms * 1e-3), "unit": "particle-steps/s",
                     "ms_per_bd_step": ms / steps, "steps": steps,
                     "cpu_one_thread": {"value": 260 * ncpu / dt, "steps": ncpu,
                                        "kind": "port"}}
        del g
    return out


SSDNA_STEPS = 200


def ssdna_measure(sh, steps=SSDNA_STEPS):
    """The ssDNA configuration: 40 nt x 3 sites (free, with their bonded and
    Go-like terms) in the 120x120x180 pore maps with ~5000 K+/Cl-, FP32
    pairs, dynamics0 / dynamics0nuc.  GPU: `steps` BD steps (ENERGY forces +
    move, one launch per kernel and step: the fused loop takes systems
    without sites), CUDA events after warm-up.  Error: forces of one ENERGY
    against the FP64 oracle.  CPU: the oracle on all host threads, a bounded
    sample of the same steps."""
    import torch
    from bromoc_gb300 import _lib
    from oracle import oracle
    spec = synth.ssdna(seed=4, nions=5000, nnuc=40, maps=synth.pore_maps(seed=102),
                       precision=abi.FP32, bonded=True, free=True)
    n = len(spec.x)
    g = _lib.create(n + 16, abi.FP32, sh)
    spec.push(g)
    o = oracle.create(n + 16)
    spec.push(o)
    tg, fg, _ = g.energy(abi.M_ALL, forces=True)
    to, fo, _ = o.energy(abi.M_ALL, forces=True)
    fe, fw = _force_errs(np.asarray(fg)[:n], np.asarray(fo)[:n])
    err = {"force_rel_err": fe, "force_worst_particle": fw,
           "energy_rel_err": _energy_err(tg, to)}
    del o
    stream = torch.cuda.current_stream()
    g.bd_steps(10, SEED, 0, energies=False)
    a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(stream)
    g.bd_steps(steps, SEED, 10, energies=False)
    e.record(stream)
    torch.cuda.synchronize()
    ms = a.elapsed_time(e)
    oc = oracle.create(n + 16, omp=True)
    spec.push(oc)
    ncpu, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < 3.0:
        oc.bd_steps(2, SEED, ncpu, energies=False)
        ncpu += 2
    dt = time.perf_counter() - t0
    return {"workload": f"ssDNA: 40 nt x 3 free sites (bonded + Go-like terms) in the "
                        f"120x120x180 pore maps, {n - spec.nsites} K+/Cl-, FP32 pairs",
            "particles": n, "sites": spec.nsites, "terms": spec.nucl.counts(),
            "value": n * steps / (ms * 1e-3), "unit": "particle-steps/s",
            "ms_per_bd_step": ms / steps, "steps": steps,
            "oracle_error": err,
            "cpu": {"value": n * ncpu / dt, "steps": ncpu, "cores": int(os.cpu_count() or 1),
                    "kind": "port"}}


ADJ_N, ADJ_STEPS, ADJ_CKPT = 4096, 2000, 100


def adjoint_measure(sh):
    """Adjoint of a frozen-noise BD segment (4096 ions at 1 M KCl, all three
    ion-ion laws tabulated on 300 knots each, 2000 steps, checkpoints every
    100): forward (with the smoothed-RDF histogram, 0.05-15 A, sigma 0.1 A)
    and backward (recomputation + adjoint), FP32 pair arithmetic, FP64
    gradient accumulators; CUDA events on the shared stream."""
    import torch
    from bromoc_gb300 import _lib
    from bromoc_gb300.adjoint import Adjoint, RdfLoss, knot_gradient, knot_jacobians
    rng = np.random.default_rng(SEED + 5)
    L = (ADJ_N / (2 * 6.02214e-4)) ** (1.0 / 3.0)
    spec = synth.bulk_kcl(seed=SEED, n_per=2, L=L, precision=abi.FP32)
    h = 0.5 * L - 0.5
    p = synth.jittered_lattice(rng, ADJ_N, -h, h)
    spec.x, spec.y, spec.z = p[:, 0].copy(), p[:, 1].copy(), p[:, 2].copy()
    spec.typei = np.array([1, 2] * (ADJ_N // 2), np.int32)
    spec.efpot_res = 0.05
    for key, (sg, ep) in ((("K", "K"), (3.1, 0.09)), (("K", "Cl"), (3.6, 0.11)),
                          (("Cl", "Cl"), (4.0, 0.15))):
        spec.efpot_knots[key] = synth.efpot_knots(rng, sg, ep, r0=1.05, r1=16.0, res=0.05)
    proto = _lib.create(ADJ_N + 64, abi.FP32, sh)
    spec.push(proto)
    adj = Adjoint(proto, ADJ_N, abi.FP32)
    adj.set_particles(spec.x, spec.y, spec.z, spec.typei)
    nbins, r0, dr, sig = 150, 0.05, 0.1, 0.1
    rb = r0 + dr * np.arange(nbins)
    loss = RdfLoss(2, [ADJ_N // 2] * 2, L ** 3, ADJ_STEPS, rb, np.ones((3, nbins)))
    fd = adjoint_fd_check(sh, spec, (nbins, r0, dr, sig))
    fd += adjoint_fd_check(sh, spec, (nbins, r0, dr, sig), steps=200)
    stream = torch.cuda.current_stream()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    torch.cuda.synchronize()
    ev[0].record(stream)
    hist = adj.forward(ADJ_STEPS, ADJ_CKPT, SEED, 0, nbins, r0, dr, sig, 3)
    ev[1].record(stream)
    value, dl = loss.loss_grad(hist)
    pt = spec.pair_tables()
    g_ep, g_sc = adj.backward(dl, int(pt["cnt"]), int(pt["ntc"]))
    ev[2].record(stream)
    torch.cuda.synchronize()
    t_f, t_b = ev[0].elapsed_time(ev[1]), ev[1].elapsed_time(ev[2])
    grads = knot_gradient(knot_jacobians(spec, proto.efpot_from_knots), g_ep, g_sc)
    adj.close()
    return {"workload": f"{ADJ_N} ions, 1 M KCl, 3x300 EFPOT knots, {ADJ_STEPS}-step "
                        f"frozen-noise segment, checkpoints every {ADJ_CKPT}, smoothed RDF "
                        "0.05-15 A (sigma 0.1 A), FP32 pairs, FP64 gradient accumulators",
            "forward_ms": t_f, "backward_ms": t_b,
            "value": ADJ_N * ADJ_STEPS / ((t_f + t_b) * 1e-3),
            "unit": "particle-steps/s (forward + adjoint)",
            "loss": value,
            "knot_grad_norm": float(np.sqrt(sum(np.sum(g * g) for g in grads.values()))),
            "fd_check": fd}


def adjoint_fd_check(sh, spec, hist_args, steps=None, hs=(3e-5, 1e-4, 3e-4)):
    """The segment's knot gradients against central differences of the
    same frozen-noise loss, untimed: for the K-K and K-Cl knot the loss
    feels most, the FP64 adjoint, the FP32 adjoint, and the difference
    quotients of FP64 forward runs at each step h (kcal/mol).  Clamp and
    wall events and the tables' piece boundaries make the loss piecewise
    smooth; over long segments they put a scatter of a few 1e-4 into the
    difference quotients themselves (fd_spread: their range over hs,
    relative), so the same check also runs on the first 200 steps."""
    import copy
    from bromoc_gb300 import _lib
    from bromoc_gb300.adjoint import Adjoint, RdfLoss, knot_gradient, knot_jacobians
    nbins, r0, dr, sig = hist_args
    steps = steps or ADJ_STEPS
    L = float(spec.lx)
    loss = RdfLoss(2, [ADJ_N // 2] * 2, L ** 3, steps, r0 + dr * np.arange(nbins),
                   np.ones((3, nbins)))
    grads, runs = {}, {}
    for prec in (abi.FP64, abi.FP32):
        s = copy.copy(spec)
        s.efpot_knots = dict(spec.efpot_knots)
        s.precision = prec
        proto = _lib.create(ADJ_N + 64, prec, sh)
        s.push(proto)
        adj = Adjoint(proto, ADJ_N, prec)

        def run(s=s, proto=proto, adj=adj):
            s.push(proto)
            adj.set_particles(s.x, s.y, s.z, s.typei)
            return adj.forward(steps, ADJ_CKPT, SEED, 0, nbins, r0, dr, sig, 3)

        _, dl = loss.loss_grad(run())
        pt = s.pair_tables()
        g_ep, g_sc = adj.backward(dl, int(pt["cnt"]), int(pt["ntc"]))
        grads[prec] = knot_gradient(knot_jacobians(s, proto.efpot_from_knots), g_ep, g_sc)
        runs[prec] = (s, run, adj, proto)
    s64, run64, _, _ = runs[abi.FP64]
    out = []
    for key in (("K", "K"), ("K", "Cl")):
        g64 = grads[abi.FP64][key]
        m = int(np.argmax(np.abs(g64)))
        r, u0 = s64.efpot_knots[key]
        u0 = np.asarray(u0, float)
        fds = []
        for h in hs:
            vals = []
            for sgn in (1, -1):
                u = u0.copy()
                u[m] += sgn * h
                s64.efpot_knots[key] = (r, u)
                vals.append(loss.loss_grad(run64())[0])
            fds.append((vals[0] - vals[1]) / (2 * h))
        s64.efpot_knots[key] = (r, u0)
        g32 = float(grads[abi.FP32][key][m])
        fd = fds[list(hs).index(1e-4)]
        out.append({"pair": "-".join(key), "knot_r": float(r[m]), "steps": steps,
                    "adjoint_fp64": float(g64[m]), "adjoint_fp32": g32,
                    "central_difference": fd, "h": 1e-4,
                    "central_difference_by_h": {f"{h:g}": v for h, v in zip(hs, fds)},
                    "fd_spread": (max(fds) - min(fds)) / abs(np.mean(fds)),
                    "rel_err_fp64_vs_fd": abs(float(g64[m]) - fd) / abs(fd),
                    "rel_err_fp32_vs_fd": abs(g32 - fd) / abs(fd),
                    "rel_err_fp32_vs_fp64": abs(g32 - float(g64[m])) / abs(float(g64[m]))})
    for _, _, adj, _ in runs.values():
        adj.close()
    return out


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return json.loads(p.read_text()), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def profile_traffic(kernel: str):
    """DRAM bytes per launch of `kernel` from the committed ncu summary."""
    for f in sorted((ROOT / "profiles").glob("*.md")):
        txt = f.read_text()
        m = re.search(r"^traffic_bytes_per_launch\[%s\]:\s*([0-9.eE+]+)" % re.escape(kernel),
                      txt, re.M)
        if m:
            return float(m.group(1)), f.name
    return None, None


def oracle_baseline(steps_budget_s: float, nthreads: int | None = None):
    """The CPU restatement (OpenMP build) on the same workload for a bounded
    sample: whole cycles until the time budget is spent; nthreads: OpenMP
    threads (default: all the host's)."""
    from oracle import oracle
    lib = oracle.load(omp=True)
    lib.bromoc_ref_set_threads(int(nthreads or os.cpu_count() or 1))
    spec = workload(0, precision=abi.FP64)
    eng = oracle.create(23000, omp=True)
    spec.push(eng)
    cores = lib.bromoc_ref_threads()
    done_ps, cyc, t0 = 0, 0, time.perf_counter()
    while True:
        cyc += 1
        eng.grand(NGCMC, SEED, cyc)
        n = eng.live_ntot()
        eng.bd_steps(NBD, SEED, (cyc - 1) * NBD)
        eng.count()
        done_ps += NBD * (n - spec.nsites - spec.nfix)
        if time.perf_counter() - t0 >= steps_budget_s:
            break
    dt = time.perf_counter() - t0
    lib.bromoc_ref_set_threads(int(os.cpu_count() or 1))
    return {"value": done_ps / dt, "unit": "particle-steps/s", "cores": cores,
            "kind": "port",
            "sample": f"{cyc} cycles ({cyc * NBD} BD steps, {cyc * NGCMC} GCMC "
                      f"attempts) of the same workload, FP64, {dt:.1f} s"}


def _force_errs(fg, fo):
    d = np.linalg.norm(fg - fo, axis=1)
    n = np.linalg.norm(fo, axis=1)
    floor = max(float(np.sqrt(np.mean(n * n))), 1e-300)
    return (float(np.linalg.norm(fg - fo) / max(np.linalg.norm(fo), 1e-300)),
            float((d / np.maximum(n, floor)).max()))


def _energy_err(tg, to):
    scale = max(1.0, sum(abs(v) for k, v in to.items() if k != "ener"))
    return float(max(abs(tg[k] - to[k]) for k in to) / scale)


def oracle_checks(sh, batch_parts):
    """The FP64 oracle as the checker of each timed form, on the timed
    workloads' own inputs (untimed):
      plain   : ENERGY of the nanopore workload, FP32 GPU against the oracle;
      grand   : four GRAND(4) calls from the workload's state: the float-float
                ΔE against the oracle's FP64 ΔE, and whether every counter
                and particle type agrees;
      batched : three replicas of the batch (smallest, median, largest).
    Force errors: ||dF|| / ||F|| and the worst particle against
    max(|F_i|, RMS |F|); energy: the worst term relative to the sum of the
    terms' magnitudes."""
    from bromoc_gb300 import _lib
    from bromoc_gb300.batch import Batch
    from oracle import oracle
    out = {}
    spec = workload(0, precision=abi.FP32)
    g = _lib.create(23000, abi.FP32, sh)
    o = oracle.create(23000)
    spec.push(g)
    spec.push(o)
    tg, fg, _ = g.energy(abi.M_ALL, forces=True)
    to, fo, _ = o.energy(abi.M_ALL, forces=True)
    fgl, fwo = _force_errs(fg, fo)
    out["plain"] = {"force_rel_err": fgl, "force_worst_particle": fwo,
                    "energy_rel_err": _energy_err(tg, to), "ions": len(fo)}
    derr = 0.0
    for cyc in range(1, 5):
        dg, do = g.grand(NGCMC, SEED, cyc), o.grand(NGCMC, SEED, cyc)
        derr = max(derr, abs(dg - do) / max(1.0, abs(do)))
    same = all((a == b).all() for a, b in zip(g.get_buffers(), o.get_buffers()))
    same = same and bool((g.get_particles()[3] == o.get_particles()[3]).all())
    out["grand"] = {"dE_rel_err": derr, "counters_equal": same, "calls": 4}
    del g, o
    counts, edges, parts = batch_parts
    pick = [int(np.argmin(counts)), int(np.argsort(counts)[len(counts) // 2]),
            int(np.argmax(counts))]
    proto_spec = synth.pore(seed=3, nions=NIONS, maps=synth.pore_maps(seed=102),
                            precision=abi.FP32, buffers=False)
    proto = _lib.create(NIONS + 64, abi.FP32, sh)
    proto_spec.push(proto)
    sub = [int(counts[r]) for r in pick]
    b = Batch(proto, sub)
    reps = []
    for r in pick:
        s = synth.pore(seed=3, nions=NIONS, maps=synth.pore_maps(seed=102),
                       precision=abi.FP32, buffers=False)
        s.lx = s.ly = s.lz = float(edges[r])
        x, y, z, t = parts[r]
        s.x, s.y, s.z, s.typei = x, y, z, t
        reps.append(s)
    b.set_systems([s.system_struct() for s in reps])
    for k, s in enumerate(reps):
        b.set_particles(k, s.x, s.y, s.z, s.typei)
    et, f = b.energy(abi.M_ALL, forces=True)
    worst = {"force_rel_err": 0.0, "force_worst_particle": 0.0, "energy_rel_err": 0.0}
    for k, s in enumerate(reps):
        o = oracle.create(len(s.x) + 16)
        s.push(o)
        to, fo, _ = o.energy(abi.M_ALL, forces=True)
        off = b.offset(k)
        fgl, fwo = _force_errs(f[off:off + len(s.x)], fo)
        tb = {kk: et[k, i] for i, kk in enumerate(abi.TERM_NAMES)}
        worst["force_rel_err"] = max(worst["force_rel_err"], fgl)
        worst["force_worst_particle"] = max(worst["force_worst_particle"], fwo)
        worst["energy_rel_err"] = max(worst["energy_rel_err"], _energy_err(tb, to))
    worst["replicas"] = sub
    out["batched"] = worst
    b.close()
    return out


# ---------------------------------------------------------------------------
def run_reference(args, rank, world):
    if rank != 0:
        return
    budget = float(os.environ.get("BROMOC_REF_STEP_S", "3.0"))
    from oracle import oracle
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    spec = workload(0, precision=abi.FP64)
    eng = oracle.create(23000, omp=True)
    spec.push(eng)
    cores = oracle.load(omp=True).bromoc_ref_threads()

    def one_cycle(cyc):
        eng.grand(NGCMC, SEED, cyc)
        n = eng.live_ntot()
        eng.bd_steps(NBD, SEED, (cyc - 1) * NBD)
        eng.count()
        return NBD * (n - spec.nsites - spec.nfix)

    for c in range(1, args.warmup + 1):
        one_cycle(c)
    tot_ps, t0 = 0, time.perf_counter()
    for c in range(args.warmup + 1, args.warmup + args.steps + 1):
        tot_ps += one_cycle(c)
    dt = time.perf_counter() - t0
    v = tot_ps / dt
    line = {"metric": METRIC, "value": v, "unit": "particle-steps/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": config_dict(), "impl": "reference",
            "precision": PRECISION_CPU,
            "cpu_baseline": {"value": v, "unit": "particle-steps/s",
                             "cores": cores, "kind": "port",
                             "sample": f"{args.steps} full cycles of the workload "
                                       "(CPU FP64 restatement, OpenMP)"},
            "e2e": {"value": v, "unit": "particle-steps/s",
                    "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
def run_gpu(args, rank, world, local_rank):
    import torch
    from bromoc_gb300 import _lib
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    # a stream of our own: torch's default (legacy) stream does not order
    # with the library's non-blocking streams, so the contexts adopt this one
    # and every event and the L2 flush are recorded on it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sh = stream.cuda_stream

    spec = workload(rank, precision=abi.FP32)
    eng = _lib.create(23000, abi.FP32, sh)
    spec.push(eng)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    nfix = spec.nsites + spec.nfix

    def step(cyc):
        eng.grand(NGCMC, SEED, cyc, dener=False)
        eng.bd_steps(NBD, SEED, (cyc - 1) * NBD, energies=False)
        eng.count()

    for c in range(1, args.warmup + 1):
        step(c)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    # the mobile count of each cycle (after its GRAND) is copied to pinned
    # memory on the stream, so the host never waits inside the loop
    counts = torch.zeros(args.steps, dtype=torch.int32, pin_memory=True)
    l0 = _lib.launch_count(eng)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local_rank) as clk:
        w0 = time.perf_counter()
        for k in range(args.steps):
            cyc = args.warmup + 1 + k
            flush.zero_()
            ev[k][0].record(stream)
            eng.grand(NGCMC, SEED, cyc, dener=False)
            _lib.live_count_async(eng, counts.data_ptr() + 4 * k)
            eng.bd_steps(NBD, SEED, (cyc - 1) * NBD, energies=False)
            eng.count()
            ev[k][1].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - w0
    nmob = [int(c) - nfix for c in counts.tolist()]
    launches = _lib.launch_count(eng) - l0
    t_ms = sum(a.elapsed_time(b) for a, b in ev)
    ps = NBD * sum(nmob)
    tmax, ps = replicas.aggregate(t_ms, ps, device="cuda")
    value = ps / (tmax * 1e-3)
    # per-kernel CUDA-event timing in a separate pass after the timed region
    # (the event records would perturb it), same workload and step sequence
    # (a) as timed: the BD steps of a cycle are one fused loop launch;
    # (b) the same steps one launch per kernel and step, for the per-kernel
    #     breakdown and the pair kernel's own roofline
    ktsteps = min(args.steps, 10)
    cyc_k = args.warmup + args.steps + 1

    def timed_kernels(cyc0):
        _lib.kernel_timing(eng, True)
        for k in range(ktsteps):
            flush.zero_()
            step(cyc0 + k)
        torch.cuda.synchronize()
        out = {name: _lib.kernel_time(eng, k) for name, k in
               (("pairs", _lib.K_PAIRS), ("rfcross", _lib.K_RFCROSS),
                ("fields", _lib.K_FIELDS), ("assemble", _lib.K_ASSEMBLE),
                ("bd_loop", _lib.K_LOOP), ("grand", _lib.K_GRAND))}
        _lib.kernel_timing(eng, False)
        return {k: v for k, v in out.items() if v[1] > 0}

    kt = timed_kernels(cyc_k)
    _lib.set_fused_bd(eng, False)
    kt_split = timed_kernels(cyc_k + ktsteps)
    _lib.set_fused_bd(eng, True)
    ktsteps *= 2

    # e2e through the host-array C ABI entry point (pinned host buffers)
    cap = 23000
    pin = {k: torch.empty(cap, dtype=dt, pin_memory=True)
           for k, dt in (("x", torch.float64), ("y", torch.float64),
                         ("z", torch.float64), ("t", torch.int32),
                         ("ib", torch.int32))}
    x, y, z, t, ib = eng.get_particles()
    n0 = len(x)
    for k, a in (("x", x), ("y", y), ("z", z), ("t", t), ("ib", ib)):
        pin[k][:n0] = torch.from_numpy(np.ascontiguousarray(a))
    ntot = C.c_int32(n0)
    lib = _lib.load()
    e2e_steps = max(3, args.steps // 2)
    h2d = d2h = 0
    e2e_ps = 0
    cyc0 = args.warmup + args.steps + ktsteps + 1
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        n_before = ntot.value
        rc = lib.bromoc_gpu_simul_cycles_host(
            eng.h, abi.M_ALL, abi.DYN0, 1, NGCMC, NBD, SEED, cyc0 + k,
            C.byref(ntot), spec.nsites, spec.nfix, pin["x"].data_ptr(),
            pin["y"].data_ptr(), pin["z"].data_ptr(), pin["t"].data_ptr(),
            pin["ib"].data_ptr(), None)
        if rc:
            raise abi.BromocError(rc, lib.bromoc_gpu_last_error(eng.h).decode())
        h2d += n_before * (3 * 8 + 4 + 4)
        d2h += ntot.value * (3 * 8 + 4 + 4)
        e2e_ps += NBD * (n_before - nfix)
    e2e_dt = time.perf_counter() - t0
    e2e_val = e2e_ps / e2e_dt

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    # roofline of the dominant kernel (by measured time share)
    peak_fp32 = _lib.fp32_peak(sh)
    peaks, src = measured_peaks()
    tot_k = sum(v[0] for v in kt.values()) or 1.0
    dom = max(kt, key=lambda k: kt[k][0])
    n_ion = statistics.mean(nmob) + spec.nfix
    pairs = n_ion * (n_ion - 1) / 2
    per = PAIR_FLOP + RF_FLOP
    pair_roof = None
    if "pairs" in kt_split:
        ms, nl = kt_split["pairs"]
        a = per * pairs / (ms / nl * 1e-3) / 1e12
        pair_roof = {"kernel": "k_pairs32n (one launch per BD step)", "achieved": a,
                     "unit": "TFLOP/s", "frac": a / peak_fp32, "launch_ms": ms / nl}
    gathers = None
    if "fields" in kt_split:
        # single-particle terms: 8 static-field corners (32 B), 8 repulsion
        # corners (8 B), 2 x 8 RFPAR corners (64 B) and the records (48 B)
        ms, nl = kt_split["fields"]
        nbytes = n_ion * (32 + 8 + 64 + 48)
        a = nbytes / (ms / nl * 1e-3) / 1e9
        gathers = {"kernel": "k_fields_warp_f32 (grid gathers, one launch per BD step)",
                   "achieved": a, "unit": "GB/s", "peak": peaks["hbm_gbs"],
                   "peak_source": src + " HBM copy bandwidth (the maps are L2-resident)",
                   "frac": a / peaks["hbm_gbs"], "launch_ms": ms / nl,
                   "algorithmic": f"152 B per particle x {n_ion:.0f} particles",
                   "bound": "latency (cell search, then one round of gathers per particle)"}
    if dom == "bd_loop":
        # one launch runs the NBD steps of a cycle: the pair work of each
        # step (ion-ion law + RFPAR cross term of every unordered pair) is
        # the algorithmic FLOP count; maps, assembly and moves ride along
        ms, nl = kt[dom]
        achieved = per * pairs * NBD / (ms / nl * 1e-3) / 1e12
        traffic, prof = profile_traffic("k_bd_loop")
        roof = {"kernel": "k_bd_loop",
                "bound": "fp32", "achieved": achieved, "peak": peak_fp32,
                "unit": "TFLOP/s", "frac": achieved / peak_fp32,
                "traffic": traffic,
                "peak_source": "FP32 FMA probe kernel measured in this run "
                               "(MEASURED_PEAKS.json has no FP32 figure)",
                "algorithmic": f"{per} FLOP x N(N-1)/2 unordered pairs x {NBD} BD "
                               f"steps per launch, N = {n_ion:.0f} ions",
                "launch_ms": ms / nl, "share": kt[dom][0] / tot_k,
                "pair_kernel_unfused": pair_roof, "gathers": gathers}
    elif dom == "pairs":
        # the FP32 pair kernel evaluates the ion-ion law and the RFPAR cross
        # term of every pair in one pass
        per = PAIR_FLOP + RF_FLOP
        ms, nl = kt[dom]
        achieved = per * pairs / (ms / nl * 1e-3) / 1e12
        traffic, prof = profile_traffic("k_pairs32n")
        roof = {"kernel": "k_pairs32n",
                "bound": "fp32", "achieved": achieved, "peak": peak_fp32,
                "unit": "TFLOP/s", "frac": achieved / peak_fp32,
                "traffic": traffic,
                "peak_source": "FP32 FMA probe kernel measured in this run "
                               "(MEASURED_PEAKS.json has no FP32 figure)",
                "algorithmic": f"{per} FLOP x N(N-1)/2 unordered pairs, N = "
                               f"{n_ion:.0f} ions",
                "launch_ms": ms / nl, "share": kt[dom][0] / tot_k}
    else:
        ms, nl = kt[dom]
        nbytes = n_ion * (32 + 8 + 64 + 48) if dom == "fields" else n_ion * 200
        achieved = nbytes / (ms / nl * 1e-3) / 1e9
        roof = {"kernel": dom, "bound": "hbm", "achieved": achieved,
                "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"], "traffic": None,
                "peak_source": src, "launch_ms": ms / nl,
                "share": kt[dom][0] / tot_k}
    scaling_pairs = pair_scaling(sh, peak_fp32)
    batched = batch_measure(sh, flush)
    adjoint = adjoint_measure(sh)
    bulk_kcl260 = bulk_measure(sh)
    ssdna40 = ssdna_measure(sh)
    # the oracle leg: CPU baselines, then the oracle as the checker
    budget = float(os.environ.get("BROMOC_CPU_SAMPLE_S", "15"))
    cpu = oracle_baseline(budget)
    cpu_mono = oracle_baseline(max(1.0, budget / 2), nthreads=1)
    checks = oracle_checks(sh, synth.batch_replicas(nrep=BATCH_NREP))
    clocks = clk.summary()
    line = {"metric": METRIC, "value": value, "unit": "particle-steps/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": tmax / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": config_dict(),
            "precision": PRECISION_GPU,
            "oracle_error": checks,
            "roofline": roof,
            "kernel_ms": {k: {"total_ms": v[0], "launches": v[1],
                              "share": v[0] / tot_k} for k, v in kt.items()},
            "kernel_ms_unfused": {k: {"total_ms": v[0], "launches": v[1]}
                                  for k, v in kt_split.items()},
            "cpu_baseline": cpu,
            "cpu_baseline_mono": cpu_mono,
            "e2e": {"value": e2e_val, "unit": "particle-steps/s",
                    "h2d_bytes_per_step": h2d // e2e_steps,
                    "d2h_bytes_per_step": d2h // e2e_steps,
                    "steps": e2e_steps,
                    "path": "bromoc_gpu_simul_cycles_host, pinned host arrays"},
            "gpu_launches": launches,
            "pair_kernel_scaling": scaling_pairs,
            "batched": batched,
            "adjoint": adjoint,
            "bulk_kcl260": bulk_kcl260,
            "ssdna40": ssdna40,
            "wall_s": wall, "clocks": clocks}
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus)))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1 and "RANK" not in os.environ:
        raise SystemExit("--gpus N > 1 must be launched with torchrun")
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_gpu(args, rank, world, local)


if __name__ == "__main__":
    main()
