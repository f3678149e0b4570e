"""The oracle pinned against the reference's own known-answer procedures.

The reference ships no golden vectors; its built-in checks are the TEST
command (central finite-difference forces vs analytic forces, absolute
tolerance 1e-3 kcal/mol/A, delta 5e-4 A; testfirst.f90:35-85) and the
ENERGY == 1/2 sum INTERACT consistency print (shell_simul.f90:2688-2696).
These tests run those procedures on the CPU restatement, plus the published
Philox4x32-10 known-answer vectors of its noise stream.
"""
import math

import numpy as np
import pytest

from bromoc_gb300 import abi

from . import systems

CAP = 2000


def _fd_forces(eng, spec, mask, delta=5e-4, idx=None):
    """testfirst.f90:35-62: central differences of ENERGY per coordinate."""
    x, y, z, t = spec.x.copy(), spec.y.copy(), spec.z.copy(), spec.typei.copy()
    n = len(x)
    idx = range(n) if idx is None else idx
    out = {}
    for i in idx:
        row = []
        for arr in (x, y, z):
            v = arr[i]
            arr[i] = v - delta
            eng.set_particles(x, y, z, t, spec.nsites, spec.nfix, spec.ibuffer)
            em = eng.energy(mask, forces=False)[0]["ener"]
            arr[i] = v + delta
            eng.set_particles(x, y, z, t, spec.nsites, spec.nfix, spec.ibuffer)
            ep = eng.energy(mask, forces=False)[0]["ener"]
            arr[i] = v
            row.append(-(ep - em) / (2 * delta))
        out[i] = np.array(row)
    eng.set_particles(x, y, z, t, spec.nsites, spec.nfix, spec.ibuffer)
    return out


def _near_grid_plane(spec, p, tol=2e-3):
    """Particles within tol of a grid plane: the reference drops force
    components there (rsmall gating, staticf1.f90:95-103), so TEST would flag
    them too."""
    if spec.phix is None:
        return np.zeros(len(p), bool)
    g = spec.phix[0]
    t = np.array([0.5 * (g["nclx"] - 1), 0.5 * (g["ncly"] - 1),
                  0.5 * (g["nclz"] - 1)]) * g["dcel"]
    u = (p + t) / g["dcel"]
    frac = np.abs(u - np.round(u))
    return (frac < tol / g["dcel"] + 1e-9).any(1)


def test_philox_known_answers(oracle_mod):
    # Random123 kat_vectors, philox4x32 with 10 rounds
    assert oracle_mod.philox([0, 0, 0, 0], [0, 0]) == \
        [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    assert oracle_mod.philox([0xffffffff] * 4, [0xffffffff] * 2) == \
        [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]
    assert oracle_mod.philox([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344],
                             [0xa4093822, 0x299f31d0]) == \
        [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]


def test_noise_moments(oracle_mod):
    g = np.array([oracle_mod.bd_gauss(1234, s, k, c) for s in range(40)
                  for k in range(250) for c in range(3)])
    assert abs(g.mean()) < 0.02 and abs(g.var() - 1.0) < 0.03
    u = np.array([oracle_mod.gcmc_uniform(99, 3, a, d) for a in range(100)
                  for d in range(50)])
    assert 0.0 <= u.min() and u.max() < 1.0 and abs(u.mean() - 0.5) < 0.01


def _near_table_knot(spec, p, delta=5e-4):
    """Particles with a tabulated pair whose distance lies within 2 delta of
    a knot.  The reference's table is continuous in value only to ~1e-5
    kcal/mol at its knots (fixdy's per-piece curvature correction,
    polynom.f90:104-111), which a central difference across a knot reads as
    a force error of jump/(2 delta); inside one quadratic piece the central
    difference is exact."""
    if not spec.efpot_knots:
        return np.zeros(len(p), bool)
    pt = spec.pair_tables()
    from bromoc_gb300.deck import nindex
    t2 = np.array([spec.nwtype()[abs(int(t)) - 1] if i >= spec.nsites
                   else spec.site_types[i] for i, t in enumerate(spec.typei)])
    bad = np.zeros(len(p), bool)
    for i in range(len(p)):
        r = np.sqrt(((p - p[i]) ** 2).sum(1))
        for j in np.nonzero((r > 0) & (r < 25.0))[0]:
            if i < spec.nsites and j < spec.nsites:
                continue
            k = nindex(t2[i], t2[j], spec.ndna, spec.nion) - 1
            if not pt["qefpot"][k]:
                continue
            u = (r[j] - pt["dmi"][k]) / pt["res"]
            if abs(u - round(u)) * pt["res"] < 2 * delta:
                bad[i] = bad[j] = True
    return bad


@pytest.mark.parametrize("family", ["pairs", "efpot", "maps_trln", "maps_spln",
                                   "dna"])
def test_fd_forces_match_analytic(oracle_mod, family):
    """TEST (testfirst.f90): analytic forces within 1e-3 kcal/mol/A of the
    central differences of ENERGY (relative 1e-5 for the stiff 1e3 kcal/mol
    repulsion walls)."""
    spec = systems.all_families()[family]()
    eng = oracle_mod.create(CAP).load(spec)
    _, f, _ = eng.energy(abi.M_ALL, forces=True)
    p = np.stack([spec.x, spec.y, spec.z], 1)
    skip = _near_grid_plane(spec, p) | _near_table_knot(spec, p)
    # DNA sites held by FIXSITE still get forces; only mobile ions and free
    # sites are compared (fixed ions have no force by construction).
    idx = [i for i in range(spec.nsites + spec.nfix, len(p)) if not skip[i]][:40]
    fd = _fd_forces(eng, spec, abi.M_ALL, idx=idx)
    for i, v in fd.items():
        tol = max(1e-3, 1e-5 * np.abs(f[i]).max())
        assert np.abs(v - f[i]).max() <= tol, (family, i, v, f[i])


def _taper_correction(spec, eng):
    """1/2 sum INTERACT - ENERGY for SRPMF pairs inside the taper zone:
    interact.f90:200 uses e*exp(-k(r-x)) - y where energy.mono.f90:154-158
    uses e*(exp(-k(r-x)) - y); the difference per pair is y*(e - 1)."""
    pt = spec.pair_tables()
    p = np.stack([spec.x, spec.y, spec.z], 1)
    t2 = np.array([spec.nwtype()[abs(int(t)) - 1] for t in spec.typei])
    from bromoc_gb300.deck import nindex
    corr = 0.0
    n = len(p)
    for i in range(n):
        for j in range(i + 1, n):
            k = nindex(t2[i], t2[j], spec.ndna, spec.nion) - 1
            if not pt["qsrpmf"][k] or pt["qefpot"][k]:
                continue
            r = math.sqrt(((p[i] - p[j]) ** 2).sum())
            if r * r > pt["rth"] or r < pt["srpx"]:
                continue
            c0, c1, c2, c3, c4 = pt["c"][:, k]
            e = c0 * math.exp((c1 - r) * c2) * math.cos(c3 * math.pi * (c1 - r)) + \
                c4 * (c1 / r) ** 6
            corr += pt["srpy"] * (e - 1.0)
    return corr


@pytest.mark.parametrize("family", ["pairs_nosrpmf", "pairs", "efpot"])
def test_energy_equals_half_sum_interact(oracle_mod, family):
    """shell_simul.f90:2688-2696 for the pair terms, with the reference's
    SRPMF taper difference between ENERGY and INTERACT accounted for."""
    spec = systems.all_families()[family]()
    eng = oracle_mod.create(CAP).load(spec)
    e = eng.energy(abi.M_NONBOND, forces=False)[0]["ener"]
    tot = sum(eng.interact(spec.x[i], spec.y[i], spec.z[i],
                           abs(int(spec.typei[i])), i + 1, abi.M_NONBOND)
              for i in range(len(spec.x)))
    expect = e + _taper_correction(spec, eng)
    assert abs(0.5 * tot - expect) <= 1e-10 * max(1.0, abs(e)), (0.5 * tot, e)


def test_table_builder_matches(oracle_mod, gpu_lib):
    """The product's host-side table builder reproduces splinepot.f90."""
    rng = np.random.default_rng(3)
    from bromoc_gb300 import synth
    for qchr, fct in ((0, 0.0), (1, -4.15)):
        r, u = synth.efpot_knots(rng, 3.5, 0.12, r0=2.0, r1=15.0, res=0.05)
        a = gpu_lib.efpot_from_knots(r, u, fct, qchr)
        b = oracle_mod.efpot_from_knots(r, u, fct, qchr)
        np.testing.assert_allclose(a[0], b[0], rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(a[1], b[1], rtol=1e-13)
        np.testing.assert_allclose(a[2], b[2], rtol=1e-15)
        assert a[3] == b[3]


def test_table_reproduces_knots(oracle_mod):
    """The quadratic pieces pass through the first and last knots and are
    continuous at interior knots up to the small jumps left by fixdy's
    per-piece curvature correction (polynom.f90:104-111): |b| res / 2 with
    b = 2 (y_n - y_n') / (x_n - x_1)."""
    rng = np.random.default_rng(4)
    from bromoc_gb300 import synth
    r, u = synth.efpot_knots(rng, 3.5, 0.12, r0=2.0, r1=15.0, res=0.05)
    ep, sc3, dm2, dmi = oracle_mod.efpot_from_knots(r, u, 0.0, 0)
    vals = ep[:, 0] + r * (ep[:, 1] + r * ep[:, 2])
    assert abs(vals[-1] - u[-1]) < 1e-9 and abs(vals[0] - u[0]) < 1e-9
    left = ep[:-1, 0] + r[1:] * (ep[:-1, 1] + r[1:] * ep[:-1, 2])
    jumps = np.abs(left - vals[1:])
    assert jumps.max() < 1e-5 * (np.abs(u).max() + 1.0)
    # the table follows the data to within its local curvature
    assert np.abs(vals - u).max() < 0.05 * (np.abs(u).max() + 1)


def test_repwalls_literal(oracle_mod):
    """The vectorised layering equals a literal loop restatement of
    repwalls.f90:38-65 on a small grid."""
    from bromoc_gb300 import synth
    rng = np.random.default_rng(5)
    nx, ny, nz = 9, 10, 11
    a = np.zeros((nx, ny, nz), np.int8)
    a[1:8, 2:9, 1:10] = 1
    a[rng.random(a.shape) < 0.03] = 0
    got = synth.repwalls(a.reshape(-1), (nx, ny, nz), walls=126).reshape(nx, ny, nz)
    ref = a.astype(int).copy()
    for n in range(1, 127):
        t = ref.copy()
        ck = 0
        for i in range(n, nx - n):
            for j in range(n, ny - n):
                for k in range(n, nz - n):
                    if ref[i, j, k] == n:
                        ck += 1
                        if ref[i - 1:i + 2, j - 1:j + 2, k - 1:k + 2].sum() == 27 * n:
                            t[i, j, k] = n + 1
        ref = t
        if ck == 0:
            break
    np.testing.assert_array_equal(got, ref)


def test_nindex_table(oracle_mod):
    """Packed pair indices cover 1..ntc exactly once over unordered pairs
    with at least one ion type (nindex.f90)."""
    from bromoc_gb300.deck import nindex
    for ndna, nion in ((0, 2), (0, 5), (2, 2), (6, 3)):
        seen = []
        nt = ndna + nion
        for i in range(1, nt + 1):
            for j in range(i, nt + 1):
                if j <= ndna:
                    continue
                seen.append(nindex(i, j, ndna, nion))
                assert nindex(i, j, ndna, nion) == nindex(j, i, ndna, nion)
        ntc = (nt + ndna + 1) * nion // 2
        assert sorted(seen) == list(range(1, ntc + 1))


def test_bd_step_noise_and_clamp(oracle_mod):
    """dynamics0 with zero forces moves each mobile ion by exactly
    sqrt(2 D dt) * (the Philox Box-Muller Gaussians of its slot), then clamps
    into the box (fixcoor.f90)."""
    spec = systems.pairs(n_per=10, L=32.0)
    eng = oracle_mod.create(CAP).load(spec)
    eng.energy(0, forces=True)  # no terms: zero forces
    eng.dynamics(abi.DYN0, 77, 5)
    x, y, z, t, _ = eng.get_particles()
    for i in range(len(x)):
        D = spec.ion_diff[abs(int(spec.typei[i])) - 1]
        a = math.sqrt(2 * spec.dt * D)
        g = [oracle_mod.bd_gauss(77, 5, i, c) for c in range(3)]
        exp = np.clip(np.array([spec.x[i], spec.y[i], spec.z[i]]) + a * np.array(g),
                      -16.0, 16.0)
        np.testing.assert_allclose([x[i], y[i], z[i]], exp, rtol=0, atol=1e-13)


def test_gcmc_chain_bookkeeping(oracle_mod):
    """GRAND keeps ntot = sites + fixed + sum(nat) and every mobile ion's
    ibuffer consistent with the counters (grand.f90:63-110)."""
    spec = systems.gcmc(nions=60)
    eng = oracle_mod.create(CAP).load(spec)
    for cyc in range(1, 30):
        eng.grand(8, 4242, cyc)
    nat, nin, nrm, prob = eng.get_buffers()
    x, y, z, t, ib = eng.get_particles()
    assert nin.sum() + nrm.sum() > 0
    counts = np.bincount(ib, minlength=len(nat) + 1)[1:]
    np.testing.assert_array_equal(counts, nat)
    assert prob.sum() == 29 * 8 * len(nat)
