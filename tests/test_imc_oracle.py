"""The covariance-Jacobian restatement of imc-macro (oracle/imc.py) against
an exact derivative.  One ion pair with the Boltzmann density
p(r) ~ r^2 exp(-beta u(r)) on [2.8, 9.5] A, u an EFPOT table built from
knots by the oracle's table builder: d<A>/dU_k by central differences of
<A> by quadrature (the table rebuilt from shifted knots) against
-beta cov(A, dU/dU_k) over Monte Carlo samples of p(r), with dU/dU_k from
the restated table basis and the builder's Jacobian.  A is the smoothed
first-shell pair histogram the adjoint's tests use."""
import numpy as np

from bromoc_gb300 import synth
from oracle import imc

RES, BETA = 0.05, 1.0 / 0.5961612495806317
NB, R0, DR, SIG = 41, 2.5, 0.2, 0.15


def _knots():
    return synth.efpot_knots(np.random.default_rng(3), 3.6, 0.11, r0=2.5, r1=10.0)


def _table(oracle_mod, r, u):
    ep, sc, dm2, dmi = oracle_mod.efpot_from_knots(r, u, 0.0, False)
    return np.asarray(ep), np.asarray(sc), np.asarray(dm2), float(dmi)


def _u_direct(r, ep, sc, dm2, dmi):
    """efp64 written out pair by pair (polynom.f90:197-230), no fct tail."""
    out = np.empty_like(r)
    for m, x in enumerate(r):
        x2 = x * x
        if x2 < dm2[0]:
            out[m] = sc[0] / x2 ** 6 + sc[1]
        elif x2 > dm2[1]:
            out[m] = sc[2] / x2 ** 3
        else:
            i = min(max(int((x - dmi) * (1.0 / RES)), 0), len(ep) - 1)  # as efp64: times 1/res
            out[m] = ep[i, 0] + x * (ep[i, 1] + x * ep[i, 2])
    return out


def _observable(r):
    rb = R0 + DR * np.arange(NB)
    w = ((rb >= 3.0) & (rb <= 6.0)).astype(float)
    u = (rb[None, :] - r[:, None]) / SIG
    k = np.exp(-0.5 * u * u) / (np.sqrt(2 * np.pi) * SIG)
    k[np.abs(u) > 5.0] = 0.0
    return k @ w


def _mean_a(oracle_mod, rk, uk, grid):
    ep, sc, dm2, dmi = _table(oracle_mod, rk, uk)
    p = grid ** 2 * np.exp(-BETA * _u_direct(grid, ep, sc, dm2, dmi))
    return np.trapezoid(_observable(grid) * p, grid) / np.trapezoid(p, grid)


def _jacobian(oracle_mod, rk, uk):
    """d(ep rows, sc) / d(knot values) by unit steps (the builder is linear)."""
    ep0, sc0, _, _ = _table(oracle_mod, rk, uk)
    base = np.concatenate([ep0.ravel(), sc0])
    cols = []
    for m in range(len(uk)):
        du = np.zeros_like(uk)
        du[m] = 1.0
        ep, sc, _, _ = _table(oracle_mod, rk, uk + du)
        cols.append(np.concatenate([ep.ravel(), sc]) - base)
    return np.stack(cols, 1)


def test_table_basis_reproduces_the_law(oracle_mod):
    rk, uk = _knots()
    ep, sc, dm2, dmi = _table(oracle_mod, rk, uk)
    r = np.linspace(2.0, 12.0, 2001)
    rows, vals = imc.table_basis(r, ep, sc, dm2, dmi, RES)
    params = np.concatenate([ep.ravel(), sc])
    u = np.sum(params[rows] * vals, 1)
    np.testing.assert_allclose(u, _u_direct(r, ep, sc, dm2, dmi), rtol=1e-12, atol=1e-12)


def test_covariance_jacobian_matches_exact_derivative(oracle_mod):
    rk, uk = _knots()
    uk = np.asarray(uk, float)
    grid = np.linspace(2.8, 9.5, 40001)
    ep, sc, dm2, dmi = _table(oracle_mod, rk, uk)
    # samples of p(r) by inverse CDF on the grid
    p = grid ** 2 * np.exp(-BETA * _u_direct(grid, ep, sc, dm2, dmi))
    cdf = np.concatenate([[0.0], np.cumsum(0.5 * (p[1:] + p[:-1]) * np.diff(grid))])
    cdf /= cdf[-1]
    rs = np.interp(np.random.default_rng(11).random(400000), cdf, grid)
    a = _observable(rs)
    jac = _jacobian(oracle_mod, rk, uk)
    ks = [k for k in range(len(uk)) if 2.9 <= rk[k] <= 6.5][::6]
    rows, vals = imc.table_basis(rs, ep, sc, dm2, dmi, RES)
    jk = jac[:, ks]  # the knots checked
    d = sum(vals[:, j:j + 1] * jk[rows[:, j]] for j in range(3))
    # one pair per sample: knot_derivative of a single pair is the same row
    np.testing.assert_allclose(imc.knot_derivative(rs[:1], rows[:1], vals[:1], jk), d[0])
    g = imc.covariance_jacobian(a[:, None], d, BETA)[0]
    h = 1e-3
    exact = []
    for k in ks:
        up, dn = uk.copy(), uk.copy()
        up[k] += h
        dn[k] -= h
        exact.append((_mean_a(oracle_mod, rk, up, grid) - _mean_a(oracle_mod, rk, dn, grid)) / (2 * h))
    exact = np.array(exact)
    scale = np.abs(exact).max()
    assert scale > 0.0
    assert np.abs(g - exact).max() <= 0.05 * scale, np.c_[g, exact]
