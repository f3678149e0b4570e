"""Restatement of imc-macro's covariance Jacobian -- test infrastructure, a
check oracle for the adjoint of a BD segment (never called by the product).

imc-macro (Lyubartsev's inverse Monte Carlo) samples configurations of the
equilibrium ensemble and, per sample, counts the pairs in each bin a of the
tabulated potential, S_a; it accumulates sum S_a and sum S_a S_b
(`correl`, imc-macro/src/imc-macro.f90:1187-1255, cors and corp at
:1240-1252) and forms cross(a,b) = <S_a S_b> - <S_a><S_b> (:788-793).  With
the energy U = sum_b V_b S_b, cross is -1/beta times the Jacobian
d<S_a>/dV_b, which the program solves against the RDF error (:803-813).

The same identity holds for any observable A and any parameter theta of
the potential: d<A>/dtheta = -beta (<A dU/dtheta> - <A><dU/dtheta>).  Here A
is the Gaussian-smoothed pair histogram the adjoint differentiates, and
theta are the knot values of the EFPOT tables: the table builder is linear
in them, so dU/dU_k is the sum over pairs of the table's basis function for
knot k -- (1, r, r^2) of the pair's quadratic piece, 1/r^12 and 1 in the
core, 1/r^6 in the tail (polynom.f90:197-230), mapped through the builder's
Jacobian.  The time-averaged adjoint gradient over long frozen-noise
segments estimates the same equilibrium derivative.
"""
from __future__ import annotations

import numpy as np


def pair_distances(x, y, z, typei, nion):
    """All ion pairs i < j of one configuration: distances and the pair-type
    index (0-based over a <= b of the 1-based ion types, a-major)."""
    p = np.stack([x, y, z], 1)
    t = np.abs(np.asarray(typei)) - 1
    i, j = np.triu_indices(len(p), 1)
    r = np.linalg.norm(p[i] - p[j], axis=1)
    a, b = np.minimum(t[i], t[j]), np.maximum(t[i], t[j])
    tp = a * nion - a * (a - 1) // 2 + (b - a)
    return r, tp


def smoothed_histogram(r, tp, ntp, nbins, r0, dr, sigma):
    """sum over pairs of K(r_b - r), K the normalised Gaussian of width
    sigma cut at 5 sigma, per pair type and bin centre r_b = r0 + b dr."""
    rb = r0 + dr * np.arange(nbins)
    u = (rb[None, :] - r[:, None]) / sigma
    k = np.exp(-0.5 * u * u) / (np.sqrt(2 * np.pi) * sigma)
    k[np.abs(u) > 5.0] = 0.0
    h = np.zeros((ntp, nbins))
    np.add.at(h, tp, k)
    return h


def table_basis(r, ep, sc, dm2, dmi, res):
    """Per pair at distance r: the rows of the table parameters it reads
    (piece rows 3i..3i+2 of ep, then core a, core b, tail a at 3n..3n+2) and
    dU/d(row), as efp64 evaluates U (polynom.f90:197-230)."""
    n = len(ep)
    x2 = r * r
    rows = np.zeros((len(r), 3), np.int64)
    vals = np.zeros((len(r), 3))
    core = x2 < dm2[0]
    tail = x2 > dm2[1]
    mid = ~(core | tail)
    rows[core] = [3 * n, 3 * n + 1, 3 * n + 1]
    vals[core, 0] = 1.0 / x2[core] ** 6
    vals[core, 1] = 1.0
    rows[tail] = [3 * n + 2, 3 * n + 2, 3 * n + 2]
    vals[tail, 0] = 1.0 / x2[tail] ** 3
    i = np.clip(((r[mid] - dmi) * (1.0 / res)).astype(np.int64), 0, n - 1)
    rows[mid] = np.stack([3 * i, 3 * i + 1, 3 * i + 2], 1)
    vals[mid] = np.stack([np.ones_like(r[mid]), r[mid], r[mid] ** 2], 1)
    return rows, vals


def knot_derivative(r, rows, vals, jac):
    """dU/dU_k for the pairs of one type: sum over pairs of the basis rows
    through the builder's Jacobian jac[row, k]."""
    acc = np.zeros(jac.shape[0])
    np.add.at(acc, rows.ravel(), vals.ravel())
    return acc @ jac


def covariance_jacobian(a, d, beta):
    """-beta (<A D> - <A><D>) from per-sample observables a[s, m] and
    parameter derivatives d[s, k] (imc-macro.f90:788-793 with the sums of
    correl, :1240-1252, normalised by the sample count)."""
    a = np.asarray(a, float)
    d = np.asarray(d, float)
    ns = len(a)
    cross = a.T @ d / ns - np.outer(a.mean(0), d.mean(0))
    return -beta * cross
