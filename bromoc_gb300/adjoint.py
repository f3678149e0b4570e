"""Adjoint of a BD segment with respect to tabulated effective potentials
(bromoc_adj_* in include/bromoc_gpu.h), the smoothed-RDF loss it is used
with, and a torch.autograd.Function for inverse-Monte-Carlo-style fitting of
the knot values of the EFPOT tables.

Loss chain: knots U -> table parameters (p1, p2, p3 per piece; core and tail
constants), linear through the table builder -> BD segment (device) ->
Gaussian-smoothed pair-distance histogram H_b -> RDF g(r_b) -> loss(g).  The device gives dL/d(table) from dL/dH; the builder's Jacobian,
taken once per knot grid, maps it onto the knots.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib, abi
from .deck import SystemSpec, nindex


class Adjoint:
    """Device engine of the segment and its adjoint (one system)."""

    def __init__(self, proto: abi.Engine, capacity: int, precision: int = abi.FP32):
        self.lib = _lib.load()
        self.proto = proto
        h = C.c_void_p()
        rc = self.lib.bromoc_adj_create(proto.h, capacity, precision, C.byref(h))
        if rc != abi.OK:
            raise abi.BromocError(rc, self.lib.bromoc_gpu_last_error(proto.h).decode())
        self.h = h
        self.n = 0
        abi.register_dependent(self, proto)

    def _chk(self, rc, what):
        if rc != abi.OK:
            raise abi.BromocError(rc, f"{what}: {self.lib.bromoc_adj_last_error(self.h).decode()}")

    def close(self):
        if getattr(self, "h", None):
            self.lib.bromoc_adj_destroy(self.h)
            self.h = None
            abi.unregister_dependent(self, self.proto)

    def __del__(self):
        if abi.shutting_down():
            return
        try:
            self.close()
        except Exception:
            pass

    def set_particles(self, x, y, z, typei):
        x, y, z = (np.ascontiguousarray(a, np.float64) for a in (x, y, z))
        t = np.ascontiguousarray(typei, np.int32)
        dp = C.POINTER(C.c_double)
        self._chk(self.lib.bromoc_adj_set_particles(
            self.h, len(x), x.ctypes.data_as(dp), y.ctypes.data_as(dp), z.ctypes.data_as(dp),
            t.ctypes.data_as(C.POINTER(C.c_int32))), "set_particles")
        self.n = len(x)

    def forward(self, nsteps, ckpt, seed, step0, nbins, r0, dr, sigma, ntp):
        hist = np.zeros((ntp, nbins))
        self._chk(self.lib.bromoc_adj_forward(
            self.h, nsteps, ckpt, seed, step0, nbins, r0, dr, sigma,
            hist.ctypes.data_as(C.POINTER(C.c_double))), "forward")
        return hist

    def backward(self, dl_dhist, cnt, ntc):
        s = np.ascontiguousarray(dl_dhist, np.float64)
        g_ep = np.zeros((max(cnt, 1), 3))
        g_sc = np.zeros((ntc, 3))
        dp = C.POINTER(C.c_double)
        self._chk(self.lib.bromoc_adj_backward(
            self.h, s.ctypes.data_as(dp), g_ep.ctypes.data_as(dp), g_sc.ctypes.data_as(dp)),
            "backward")
        return g_ep, g_sc

    def get_particles(self, which=1):
        x, y, z = (np.zeros(self.n) for _ in range(3))
        dp = C.POINTER(C.c_double)
        self._chk(self.lib.bromoc_adj_get_particles(
            self.h, which, x.ctypes.data_as(dp), y.ctypes.data_as(dp), z.ctypes.data_as(dp)),
            "get_particles")
        return x, y, z


class RdfLoss:
    """RDF of each ion-type pair at the bin centres r_b from the smoothed
    histogram: g(r_b) = H_b / (T npair 4 pi r_b^2 / V), and the loss
    sum w (g - g_target)^2."""

    def __init__(self, nt, counts, volume, nsteps, rbins, target, weight=None):
        self.ntp = nt * (nt + 1) // 2
        self.norm = np.zeros((self.ntp, len(rbins)))
        k = 0
        for a in range(nt):
            for b in range(a, nt):
                npair = counts[a] * (counts[a] - 1) / 2 if a == b else counts[a] * counts[b]
                self.norm[k] = nsteps * npair * 4.0 * np.pi * rbins ** 2 / volume
                k += 1
        self.target = np.asarray(target, float).reshape(self.ntp, len(rbins))
        self.w = np.ones_like(self.target) if weight is None else np.asarray(weight, float)

    def rdf(self, hist):
        return hist / self.norm

    def loss_grad(self, hist):
        """(loss, dL/dhist)"""
        g = self.rdf(hist)
        r = g - self.target
        loss = float(np.sum(self.w * r * r))
        dl = (2.0 * self.w * r) / self.norm
        return loss, dl


def knot_jacobians(spec: SystemSpec, builder):
    """Per tabulated pair (a, b): the 0-based pair index, its first piece,
    and d(ep rows, sc) / d(knot values) -- the builder is linear in the knot
    values for fixed knot positions, so unit steps give exact columns."""
    out = {}
    ndna, nion = spec.ndna, spec.nion
    fct = spec.pair_tables()["fct"]
    qchr = spec.pair_tables()["qchr"]
    first = 0
    for (a, b), (r, u) in spec.efpot_knots.items():
        k = nindex(spec.ctype(a), spec.ctype(b), ndna, nion) - 1
        u = np.asarray(u, float)
        base_ep, base_sc = (np.asarray(v, float) for v in builder(r, u, fct[k], bool(qchr[k]))[:2])
        cols = []
        for m in range(len(u)):
            du = np.zeros_like(u)
            du[m] = 1.0
            ep, sc = (np.asarray(v, float) for v in builder(r, u + du, fct[k], bool(qchr[k]))[:2])
            cols.append(np.concatenate([(ep - base_ep).ravel(), sc - base_sc]))
        out[(a, b)] = dict(index=k, first=first, n=len(r), J=np.stack(cols, 1))
        first += len(r)
    return out


def knot_gradient(jac, g_ep, g_sc):
    """dL/d(knot values) per tabulated pair from dL/d(table parameters)."""
    grads = {}
    for key, j in jac.items():
        rows = g_ep[j["first"]:j["first"] + j["n"]].ravel()
        grads[key] = j["J"].T @ np.concatenate([rows, g_sc[j["index"]]])
    return grads


def make_autograd(spec: SystemSpec, proto: abi.Engine, adj: Adjoint, loss: RdfLoss,
                  segment: dict):
    """torch.autograd.Function over the knot values of spec.efpot_knots (one
    tensor per pair, in their order): forward pushes the tables, runs the
    segment and returns the loss; backward runs the adjoint."""
    import torch
    keys = list(spec.efpot_knots)
    jac = knot_jacobians(spec, proto.efpot_from_knots)
    nt = spec.nion

    class SegmentLoss(torch.autograd.Function):
        @staticmethod
        def forward(ctx, *knots):
            for key, u in zip(keys, knots):
                r = spec.efpot_knots[key][0]
                spec.efpot_knots[key] = (r, u.detach().cpu().double().numpy())
            spec.push(proto)
            adj.set_particles(spec.x, spec.y, spec.z, spec.typei)
            hist = adj.forward(segment["nsteps"], segment["ckpt"], segment["seed"],
                               segment.get("step0", 0), segment["nbins"], segment["r0"],
                               segment["dr"], segment["sigma"], nt * (nt + 1) // 2)
            value, dl = loss.loss_grad(hist)
            ctx.dl = dl
            return torch.tensor(value, dtype=torch.float64)

        @staticmethod
        def backward(ctx, grad_out):
            pt = spec.pair_tables()
            g_ep, g_sc = adj.backward(ctx.dl, int(pt["cnt"]), int(pt["ntc"]))
            grads = knot_gradient(jac, g_ep, g_sc)
            return tuple(grad_out * torch.tensor(grads[k], dtype=torch.float64) for k in keys)

    return SegmentLoss
