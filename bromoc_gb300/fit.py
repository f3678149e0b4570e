"""Inverse-Monte-Carlo-style fitting of tabulated effective potentials.

imc-macro's update loop (imc-macro/src/imc-macro.f90:720-813) iterates:
simulate, compare the pair correlations with the reference RDF, solve the
covariance system for a potential correction (damped by its regularisation
parameter regp, each change capped at dpotm), update the tables, repeat.
This driver keeps that loop but takes the correction's direction from the
segment adjoint: the exact gradient of a frozen-noise BD segment's smoothed
RDF loss with respect to the EFPOT knot values, obtained through the
torch.autograd.Function of adjoint.make_autograd.  Each iteration steps
the knots against the gradient, scaled so that no knot moves more than
`dpotm` kcal/mol, and halves the step while the loss does not decrease (a
backtracking line search on the frozen-noise objective).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import abi
from .adjoint import Adjoint, RdfLoss, make_autograd
from .deck import SystemSpec


@dataclass
class FitHistory:
    loss: list = field(default_factory=list)      # loss after each accepted step
    step: list = field(default_factory=list)      # largest knot change of the step
    grad_norm: list = field(default_factory=list)


def fit_knots(spec: SystemSpec, proto: abi.Engine, adj: Adjoint, loss: RdfLoss,
              segment: dict, iters: int = 8, dpotm: float = 0.05, keys=None,
              max_halvings: int = 6) -> FitHistory:
    """Fit spec.efpot_knots (all pairs, or `keys`) to loss's target RDF.

    segment: nsteps, ckpt, seed, nbins, r0, dr, sigma (as Adjoint.forward);
    the same frozen noise every iteration.  Returns the loss history (the
    first entry is the starting loss); spec.efpot_knots holds the fitted
    values afterwards, and proto the matching tables."""
    import torch
    all_keys = list(spec.efpot_knots)
    keys = all_keys if keys is None else list(keys)
    Seg = make_autograd(spec, proto, adj, loss, segment)

    def tensors():
        return [torch.tensor(np.asarray(spec.efpot_knots[k][1], float), dtype=torch.float64,
                             requires_grad=k in keys) for k in all_keys]

    hist = FitHistory()
    knots = tensors()
    value = Seg.apply(*knots)
    hist.loss.append(value.item())
    scale = dpotm
    for _ in range(iters):
        # the adjoint runs on the segment of the last forward call: `value`'s
        value.backward()
        grads = {k: t.grad.numpy().copy() for k, t in zip(all_keys, knots) if k in keys}
        gmax = max(np.abs(g).max() for g in grads.values())
        hist.grad_norm.append(float(np.sqrt(sum(np.sum(g * g) for g in grads.values()))))
        if gmax == 0.0:
            break
        base = {k: np.asarray(spec.efpot_knots[k][1], float).copy() for k in all_keys}
        accepted = False
        for _h in range(max_halvings + 1):
            for k in keys:
                r = spec.efpot_knots[k][0]
                spec.efpot_knots[k] = (r, base[k] - scale * grads[k] / gmax)
            knots = tensors()
            trial = Seg.apply(*knots)
            if trial.item() < hist.loss[-1]:
                accepted = True
                break
            scale *= 0.5
        if not accepted:
            for k in all_keys:
                spec.efpot_knots[k] = (spec.efpot_knots[k][0], base[k])
            break
        hist.loss.append(trial.item())
        hist.step.append(scale)
        value = trial
        scale = min(2.0 * scale, dpotm)
    spec.push(proto)
    return hist
