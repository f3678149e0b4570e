"""Adjoint of a BD segment (bromoc_adj_*): gradients of a smoothed-RDF loss
with respect to the EFPOT knot values against central finite differences of
the same loss (FP64 arithmetic), FP32 against FP64, independence of the
checkpoint interval, and the adjoint engine's forward step against the main
engine's FP32 BD step."""
import numpy as np
import pytest

from bromoc_gb300 import abi
from bromoc_gb300.adjoint import Adjoint, RdfLoss, knot_gradient, knot_jacobians

from . import systems

pytestmark = pytest.mark.gpu
CAP = 256
SEG = dict(nsteps=20, ckpt=5, seed=5, step0=0, nbins=21, r0=3.0, dr=0.25, sigma=0.1)


def _setup(gpu_lib, precision):
    spec = systems.efpot_all(precision=precision)
    proto = gpu_lib.create(CAP, precision)
    spec.push(proto)
    adj = Adjoint(proto, CAP, precision)
    adj.set_particles(spec.x, spec.y, spec.z, spec.typei)
    nt = spec.nion
    counts = [int(np.sum(np.abs(spec.typei) == t)) for t in range(1, nt + 1)]
    rb = SEG["r0"] + SEG["dr"] * np.arange(SEG["nbins"])
    loss = RdfLoss(nt, counts, spec.lx * spec.ly * spec.lz, SEG["nsteps"], rb,
                   np.ones((nt * (nt + 1) // 2, len(rb))))
    return spec, proto, adj, loss


def _run(spec, proto, adj, loss):
    spec.push(proto)
    adj.set_particles(spec.x, spec.y, spec.z, spec.typei)
    return adj.forward(SEG["nsteps"], SEG["ckpt"], SEG["seed"], SEG["step0"], SEG["nbins"],
                       SEG["r0"], SEG["dr"], SEG["sigma"], loss.ntp)


def _grad(spec, proto, adj, loss, ckpt=None):
    seg = dict(SEG, ckpt=ckpt or SEG["ckpt"])
    spec.push(proto)
    adj.set_particles(spec.x, spec.y, spec.z, spec.typei)
    hist = adj.forward(seg["nsteps"], seg["ckpt"], seg["seed"], seg["step0"], seg["nbins"],
                       seg["r0"], seg["dr"], seg["sigma"], loss.ntp)
    value, dl = loss.loss_grad(hist)
    pt = spec.pair_tables()
    g_ep, g_sc = adj.backward(dl, int(pt["cnt"]), int(pt["ntc"]))
    jac = knot_jacobians(spec, proto.efpot_from_knots)
    return value, knot_gradient(jac, g_ep, g_sc)


def _central_differences(spec, proto, adj, loss, picks, h=1e-5):
    """FP64 central differences of the loss at the given knots {key: [m]}."""
    out = {}
    for key, ms in picks.items():
        r, u0 = spec.efpot_knots[key]
        u0 = np.array(u0)
        for m in ms:
            vals = []
            for sgn in (1, -1):
                u = u0.copy()
                u[m] += sgn * h
                spec.efpot_knots[key] = (r, u)
                vals.append(loss.loss_grad(_run(spec, proto, adj, loss))[0])
            spec.efpot_knots[key] = (r, u0)
            out[key, int(m)] = (vals[0] - vals[1]) / (2 * h)
    return out


def test_adjoint_matches_finite_differences(gpu_lib):
    """Central differences with h = 1e-5 kcal/mol, FP64 arithmetic.  The
    tables keep the reference's knot-spacing quirk (fixdy), which leaves
    ~1e-5 jumps of U and U' at piece boundaries; a trajectory whose pair
    crosses a boundary at a different step in the +h and -h runs picks one
    up, so steps of 1e-4 mix in such events, while at 1e-5 the two agree to
    ~1e-7.  The knots the loss feels most: each within 1e-5 of its own
    value; two random knots (gradients possibly near zero): within 1e-5 of
    the largest component."""
    spec, proto, adj, loss = _setup(gpu_lib, abi.FP64)
    value, grads = _grad(spec, proto, adj, loss)
    rng = np.random.default_rng(0)
    big = {k: list(np.argsort(-np.abs(grads[k]))[:6]) for k in spec.efpot_knots}
    rnd = {k: list(rng.integers(0, len(spec.efpot_knots[k][1]), 2)) for k in spec.efpot_knots}
    fd = _central_differences(spec, proto, adj, loss, big)
    for (key, m), v in fd.items():
        assert abs(v - grads[key][m]) <= 1e-5 * abs(grads[key][m]), (key, m, v, grads[key][m])
    fd = _central_differences(spec, proto, adj, loss, rnd)
    for (key, m), v in fd.items():
        scale = max(np.abs(grads[key]).max(), 1e-30)
        assert abs(v - grads[key][m]) <= 1e-5 * scale, (key, m, v, grads[key][m])


def test_adjoint_fp32_matches_finite_differences(gpu_lib):
    """The FP32 adjoint (FP32 pairs, FP64 accumulators) against FP64 central
    differences (h = 1e-5) at the knots the loss feels most: each within
    1e-4 of its own value."""
    spec64, proto64, adj64, loss64 = _setup(gpu_lib, abi.FP64)
    _, g64 = _grad(spec64, proto64, adj64, loss64)
    spec32, proto32, adj32, loss32 = _setup(gpu_lib, abi.FP32)
    _, g32 = _grad(spec32, proto32, adj32, loss32)
    big = {k: list(np.argsort(-np.abs(g64[k]))[:6]) for k in spec64.efpot_knots}
    fd = _central_differences(spec64, proto64, adj64, loss64, big)
    for (key, m), v in fd.items():
        assert abs(g32[key][m] - v) <= 1e-4 * abs(v), (key, m, g32[key][m], v)


def test_adjoint_fp32_close_to_fp64(gpu_lib):
    spec64, proto64, adj64, loss64 = _setup(gpu_lib, abi.FP64)
    _, g64 = _grad(spec64, proto64, adj64, loss64)
    spec32, proto32, adj32, loss32 = _setup(gpu_lib, abi.FP32)
    _, g32 = _grad(spec32, proto32, adj32, loss32)
    for key in g64:
        err = np.linalg.norm(g32[key] - g64[key]) / np.linalg.norm(g64[key])
        assert err <= 1e-3, (key, err)


def test_checkpoint_interval_does_not_change_the_gradient(gpu_lib):
    spec, proto, adj, loss = _setup(gpu_lib, abi.FP64)
    v1, g1 = _grad(spec, proto, adj, loss, ckpt=5)
    v2, g2 = _grad(spec, proto, adj, loss, ckpt=20)
    assert v1 == v2
    for key in g1:
        np.testing.assert_allclose(g1[key], g2[key], rtol=1e-10,
                                   atol=1e-12 * np.abs(g1[key]).max())


def test_adjoint_forward_matches_engine(gpu_lib):
    spec, proto, adj, loss = _setup(gpu_lib, abi.FP32)
    adj.forward(1, 1, 5, 3, SEG["nbins"], SEG["r0"], SEG["dr"], SEG["sigma"], loss.ntp)
    xa = np.stack(adj.get_particles(1), 1)
    g = gpu_lib.create(CAP, abi.FP32)
    spec.push(g)
    g.bd_steps(1, seed=5, step0=3)
    xg = np.stack(g.get_particles()[:3], 1)
    assert np.abs(xa - xg).max() <= 1e-5
