"""The adjoint of BD segments against imc-macro's covariance Jacobian, as a
statistical test.

imc-macro's update (imc-macro.f90:788-793 with the sums of correl,
:1187-1255) rests on d<A>/dtheta = -beta cov(A, dU/dtheta) over the
equilibrium ensemble (oracle/imc.py).  A frozen-noise segment's adjoint
gives the pathwise derivative of the segment average A_T with the start x0
held fixed; for segments started from the equilibrium ensemble the same
derivative is the average of that pathwise part plus the response of the
starting ensemble, -beta cov(A_T, dU/dtheta(x0)) over the segments (the
score of the start).  So

    E[adjoint] - beta cov(A_T, dU/dtheta(x0)) = -beta cov(A, dU/dtheta)

for any segment length; the pathwise part alone falls short by what the
start carries (about half here).  System: 64 neutral particles with the
three tabulated K/Cl short-range laws (no charges, so the pair kinetics are
fast and the run equilibrates in the time the test takes), A the smoothed
K-Cl pair count over 3-6 A, theta the K-Cl knot values over 3-6 A (their
sum).  Both sides are estimated from one equilibrium BD run: covariance
samples along it, segment starts every 2000 steps; standard errors from
the segments (adjoint side) and from batches between segment starts
(covariance side)."""
import numpy as np
import pytest

from bromoc_gb300 import abi
from bromoc_gb300.adjoint import Adjoint, knot_gradient, knot_jacobians
from oracle import imc

from . import systems

pytestmark = pytest.mark.gpu
NBINS, R0, DR, SIG = 13, 3.0, 0.25, 0.1
KCL = 1            # the (K, Cl) type pair
T, NSEG, GAP, EVERY, EQ = 1000, 96, 2000, 20, 20000


def test_adjoint_plus_start_response_equals_covariance_jacobian(gpu_lib):
    spec = systems.efpot_all(precision=abi.FP32)
    spec.ion_cg = [0.0, 0.0]
    beta = 1.0 / (0.0019872041 * spec.temp)
    nt = spec.nion
    ntp = nt * (nt + 1) // 2
    w = np.zeros((ntp, NBINS))
    w[KCL] = 1.0
    g = gpu_lib.create(256, abi.FP32)
    spec.push(g)
    adj = Adjoint(g, 256, abi.FP32)
    jac = knot_jacobians(spec, g.efpot_from_knots)
    J = jac[("K", "Cl")]["J"]
    rk, uk = spec.efpot_knots[("K", "Cl")]
    pt = spec.pair_tables()
    k = jac[("K", "Cl")]["index"]
    ep, sc, dm2, dmi = g.efpot_from_knots(rk, np.asarray(uk, float), pt["fct"][k],
                                          bool(pt["qchr"][k]))
    sel = (np.asarray(rk) >= 3.0) & (np.asarray(rk) <= 6.0)

    def sample(x, y, z, t):  # A and sum over the window of dU/dtheta_k
        r, tp = imc.pair_distances(x, y, z, t, nt)
        a = float(np.sum(imc.smoothed_histogram(r, tp, ntp, NBINS, R0, DR, SIG) * w))
        rr = r[tp == KCL]
        rows, vals = imc.table_basis(rr, ep, sc, dm2, dmi, spec.efpot_res)
        return a, float(imc.knot_derivative(rr, rows, vals, J)[sel].sum())

    g.bd_steps(EQ, seed=101, step0=0, energies=False)
    step = EQ
    a_s, d_s, cov_b = [], [], []
    adj_w, seg_a, d0 = [], [], []
    for s in range(NSEG):
        x, y, z, ti, _ = g.get_particles()
        d0.append(sample(x, y, z, ti)[1])
        adj.set_particles(x, y, z, ti)
        hist = adj.forward(T, 100, 1000 + s, 0, NBINS, R0, DR, SIG, ntp)
        seg_a.append(float(np.sum(hist * w)) / T)
        g_ep, g_sc = adj.backward(w / T, int(pt["cnt"]), int(pt["ntc"]))
        adj_w.append(float(knot_gradient(jac, g_ep, g_sc)[("K", "Cl")][sel].sum()))
        ab, db = [], []
        for _ in range(GAP // EVERY):
            g.bd_steps(EVERY, seed=101, step0=step, energies=False)
            step += EVERY
            a, d = sample(*g.get_particles()[:4])
            ab.append(a)
            db.append(d)
        a_s += ab
        d_s += db
        cov_b.append(-beta * np.cov(ab, db)[0, 1])
    adj.close()
    adj_w, seg_a, d0 = np.array(adj_w), np.array(seg_a), np.array(d0)
    # per segment: pathwise part + its share of the start's response
    z = adj_w - beta * (seg_a - seg_a.mean()) * (d0 - d0.mean()) * NSEG / (NSEG - 1)
    total, total_se = z.mean(), z.std(ddof=1) / np.sqrt(NSEG)
    cov = -beta * np.cov(a_s, d_s)[0, 1]
    cov_se = np.std(cov_b, ddof=1) / np.sqrt(NSEG)
    assert abs(cov) > 10 * cov_se, (cov, cov_se)
    assert abs(total - cov) <= 3.0 * np.hypot(total_se, cov_se), (total, total_se, cov, cov_se,
                                                                   adj_w.mean())
