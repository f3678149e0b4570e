"""The torch.autograd.Function over the EFPOT knots (adjoint.make_autograd)
and the inverse-Monte-Carlo-style fitting driver (fit.fit_knots) built on
it."""
import numpy as np
import pytest

from bromoc_gb300 import abi
from bromoc_gb300.adjoint import Adjoint, RdfLoss, knot_gradient, knot_jacobians, make_autograd
from bromoc_gb300.fit import fit_knots

from . import systems

pytestmark = pytest.mark.gpu
CAP = 256
SEG = dict(nsteps=30, ckpt=10, seed=9, step0=0, nbins=24, r0=2.5, dr=0.25, sigma=0.1)


def _setup(gpu_lib, precision, target=None):
    spec = systems.efpot_all(precision=precision)
    proto = gpu_lib.create(CAP, precision)
    spec.push(proto)
    adj = Adjoint(proto, CAP, precision)
    adj.set_particles(spec.x, spec.y, spec.z, spec.typei)
    nt = spec.nion
    counts = [int(np.sum(np.abs(spec.typei) == t)) for t in range(1, nt + 1)]
    rb = SEG["r0"] + SEG["dr"] * np.arange(SEG["nbins"])
    tgt = np.ones((nt * (nt + 1) // 2, len(rb))) if target is None else target
    loss = RdfLoss(nt, counts, spec.lx * spec.ly * spec.lz, SEG["nsteps"], rb, tgt)
    return spec, proto, adj, loss


def _hist(spec, proto, adj, loss):
    spec.push(proto)
    adj.set_particles(spec.x, spec.y, spec.z, spec.typei)
    return adj.forward(SEG["nsteps"], SEG["ckpt"], SEG["seed"], SEG["step0"], SEG["nbins"],
                       SEG["r0"], SEG["dr"], SEG["sigma"], loss.ntp)


def test_autograd_matches_adjoint_and_differences(gpu_lib):
    """The Function's gradients equal the adjoint's knot gradients, and the
    two largest components of each pair agree with central differences of
    the Function's own forward (FP64, h = 1e-5 kcal/mol, within 1e-4 of
    the pair's largest component)."""
    import torch
    spec, proto, adj, loss = _setup(gpu_lib, abi.FP64)
    keys = list(spec.efpot_knots)
    Seg = make_autograd(spec, proto, adj, loss, SEG)
    knots = [torch.tensor(np.asarray(spec.efpot_knots[k][1], float), dtype=torch.float64,
                          requires_grad=True) for k in keys]
    value = Seg.apply(*knots)
    value.backward()
    hist = _hist(spec, proto, adj, loss)
    v2, dl = loss.loss_grad(hist)
    assert value.item() == v2
    pt = spec.pair_tables()
    g_ep, g_sc = adj.backward(dl, int(pt["cnt"]), int(pt["ntc"]))
    direct = knot_gradient(knot_jacobians(spec, proto.efpot_from_knots), g_ep, g_sc)
    h = 1e-5
    for k, t in zip(keys, knots):
        g = t.grad.numpy()
        np.testing.assert_allclose(g, direct[k], rtol=1e-12, atol=1e-14 * np.abs(direct[k]).max())
        for m in np.argsort(-np.abs(g))[:2]:
            vals = []
            for sgn in (1, -1):
                kk = [x.detach().clone() for x in knots]
                kk[keys.index(k)][m] += sgn * h
                vals.append(Seg.apply(*kk).item())
            fd = (vals[0] - vals[1]) / (2 * h)
            assert abs(fd - g[m]) <= 1e-4 * np.abs(g).max(), (k, m, fd, g[m])


def test_fit_lowers_the_loss(gpu_lib):
    """Target: the smoothed RDF of the same segment with the K-Cl well made
    0.3 kcal/mol deeper around 4 A.  Fitting the K-Cl knots from the
    unperturbed values must cut the loss at least fourfold within eight
    iterations, every accepted step lowering it."""
    spec, proto, adj, loss0 = _setup(gpu_lib, abi.FP64)
    r, u = spec.efpot_knots[("K", "Cl")]
    u0 = np.array(u, float)
    spec.efpot_knots[("K", "Cl")] = (r, u0 - 0.3 * np.exp(-((np.asarray(r) - 4.0) / 0.7) ** 2))
    target = loss0.rdf(_hist(spec, proto, adj, loss0))
    spec.efpot_knots[("K", "Cl")] = (r, u0)
    _, proto, adj, loss = _setup(gpu_lib, abi.FP64, target=target)
    spec.push(proto)
    hist = fit_knots(spec, proto, adj, loss, SEG, iters=8, dpotm=0.1, keys=[("K", "Cl")])
    assert len(hist.loss) >= 3, hist
    assert all(b < a for a, b in zip(hist.loss, hist.loss[1:]))
    assert hist.loss[-1] <= 0.25 * hist.loss[0], hist.loss
