"""Seeded synthetic systems standing in for the benchmark workloads.

The reference ships no PB maps, effective-potential tables or input decks, so
each workload is generated from a seed with the stated shapes and sizes:

  bulk_kcl : 130 K+ / 130 Cl- in a 60 A box, hard walls, FP64 (bulk 1 M KCl)
  pore     : 120x120x180 maps at 1 A (static field = 1 V drop + Gaussians,
             RFPAR Born-like wall penalty, repulsion slab with a 10 A pore),
             ~2000 ions, GCMC buffers at both ends
  ssdna    : 40 nt x 3 sites (base, S, P) along the pore axis plus ~5000 ions
             with tabulated ion-site effective potentials
"""
from __future__ import annotations

import math

import numpy as np

from . import abi, nucleotides
from .deck import CELEC, SystemSpec

# KCl parameters of the bulk workload
K_PARAMS = dict(q=1.0, sigma=3.14, eps=0.087, D=0.196)
CL_PARAMS = dict(q=-1.0, sigma=4.04, eps=0.15, D=0.203)
# SRPMF coefficients for K+/Cl- pairs (the reference manual's POT/CLA example,
# cg-gcmc-bd/doc/bromoc.doc:565-570)
SRPMF_KCL = {("K", "K"): (-0.60, 4.40, 0.90, 0.80, 0.25),
             ("Cl", "Cl"): (-0.50, 4.90, 0.90, 0.80, 0.25),
             ("K", "Cl"): (-3.70, 2.90, 0.90, 0.75, 0.00)}
MOLAR = 6.0221412927e23 * 1e-27  # ions per A^3 at 1 mol/L


def place(rng, n, lo, hi, dmin=3.0, ok=None, existing=None, max_tries=200000):
    """Uniform positions in [lo, hi) with a minimum separation, rejecting
    points where ok(p) is False."""
    lo, hi = np.asarray(lo, float), np.asarray(hi, float)
    pts = [] if existing is None else list(existing)
    cell = dmin
    grid = {}

    def key(p):
        return tuple((p // cell).astype(int))

    for p in pts:
        grid.setdefault(key(p), []).append(p)
    out = []
    tries = 0
    while len(out) < n:
        tries += 1
        if tries > max_tries + 50 * n:
            raise RuntimeError("could not place particles")
        p = lo + (hi - lo) * rng.random(3)
        if ok is not None and not ok(p):
            continue
        k = key(p)
        clash = False
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    for q in grid.get((k[0] + dx, k[1] + dy, k[2] + dz), ()):
                        if np.sum((p - q) ** 2) < dmin * dmin:
                            clash = True
                            break
                    if clash:
                        break
                if clash:
                    break
            if clash:
                break
        if clash:
            continue
        grid.setdefault(k, []).append(p)
        out.append(p)
    return np.array(out)


def _kcl_types(spec: SystemSpec):
    spec.ion_names = ["K", "Cl"]
    spec.ion_cg = [K_PARAMS["q"], CL_PARAMS["q"]]
    spec.ion_diff = [K_PARAMS["D"], CL_PARAMS["D"]]
    spec.lj_eps.update(K=K_PARAMS["eps"], Cl=CL_PARAMS["eps"])
    spec.lj_sigma.update(K=K_PARAMS["sigma"], Cl=CL_PARAMS["sigma"])


def jittered_lattice(rng, n, lo, hi, dmin=3.0, ok=None):
    """n positions in [lo, hi)^3 at least dmin apart, vectorised: a random
    subset of the sites of a cubic lattice (spacing a >= dmin), each moved
    uniformly within +-(a - dmin)/2 of its site; ok(points) -> bool mask
    drops sites (the lattice is refined until n sites remain)."""
    lo, hi = float(lo), float(hi)
    m = int(np.ceil(n ** (1.0 / 3.0)))
    while True:
        a = (hi - lo) / m
        if a < dmin:
            raise ValueError("box too small for n particles at this separation")
        sites = rng.permutation(m ** 3)
        ijk = np.stack(np.unravel_index(sites, (m, m, m)), 1).astype(float)
        p = lo + (ijk + 0.5) * a + (a - dmin) * (rng.random((len(sites), 3)) - 0.5)
        if ok is not None:
            p = p[ok(p)]
        if len(p) >= n:
            return p[:n]
        m += 1


def outside_pore_slab(p, radius=10.0, slab=30.0, half_xy=59.5):
    """Mask of points not inside the solid slab of pore_maps' geometry."""
    rho = np.hypot(p[:, 0], p[:, 1])
    inside_map = (np.abs(p[:, 0]) <= half_xy) & (np.abs(p[:, 1]) <= half_xy)
    return ~(inside_map & (np.abs(p[:, 2]) <= 0.5 * slab + 1.0) & (rho >= radius - 1.0))


def batch_replicas(seed=4, nrep=256, nmin=200, nmax=8000, conc=1.0):
    """Replica set of uneven bulk KCl systems at conc (M of salt, so
    2 conc 6.022e-4 ions per A^3): counts uniform in [nmin, nmax], cube boxes
    of edge (N / (2 conc 6.022e-4))^(1/3) centred at the origin, positions
    on a jittered lattice (3 A minimum separation).
    Returns (counts, edges, list of (x, y, z, typei))."""
    rng = np.random.default_rng(seed)
    counts = rng.integers(nmin, nmax + 1, nrep)
    counts += counts % 2  # equal K+ and Cl-
    edges = (counts / (2.0 * conc * 6.02214e-4)) ** (1.0 / 3.0)
    parts = []
    for n, L in zip(counts, edges):
        h = 0.5 * L - 0.5
        p = jittered_lattice(rng, int(n), -h, h, ok=outside_pore_slab)
        t = np.array([1, 2] * (int(n) // 2), np.int32)
        parts.append((p[:, 0].copy(), p[:, 1].copy(), p[:, 2].copy(), t))
    return counts.astype(int), edges, parts


def bulk_kcl(seed=1, n_per=130, L=60.0, srpmf=False, precision=abi.FP64, periodic_rcut=None):
    """Bulk KCl: 2*n_per ions in an L^3 box with hard walls, or (periodic_rcut,
    the extension mode) periodic with that pair cutoff; the ions then keep
    1.5 A from the faces, so no two images start closer than 3 A."""
    rng = np.random.default_rng(seed)
    s = SystemSpec(shape=abi.BOX, lx=L, ly=L, lz=L, temp=300.0, cdie=80.0,
                   dt=0.02, bdmax=1.0, precision=precision)
    _kcl_types(s)
    if srpmf:
        s.srpmf.update(SRPMF_KCL)
        s.srpmf_rth = 8.0
    s.periodic_rcut = periodic_rcut
    h = 0.5 * L - (1.5 if periodic_rcut is not None else 0.5)
    p = place(rng, 2 * n_per, [-h] * 3, [h] * 3)
    s.x, s.y, s.z = p[:, 0].copy(), p[:, 1].copy(), p[:, 2].copy()
    s.typei = np.array([1] * n_per + [2] * n_per, np.int32)
    return s


def repwalls(phiv: np.ndarray, shape, walls: int = 126) -> np.ndarray:
    """Layer closed repulsive bodies: a cell of value n whose 27 neighbours
    all equal n becomes n+1 (repwalls.f90:40-64), until no cell equals n."""
    nx, ny, nz = shape
    a = phiv.reshape(shape).astype(np.int16)
    for n in range(1, walls + 1):
        if nx - 2 * n <= 0 or ny - 2 * n <= 0 or nz - 2 * n <= 0:
            break
        core = a[n:nx - n, n:ny - n, n:nz - n]
        mask = core == n
        if not mask.any():
            break
        allsame = np.ones_like(mask)
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    allsame &= a[n + dx:nx - n + dx, n + dy:ny - n + dy,
                                 n + dz:nz - n + dz] == n
        t = a.copy()
        t[n:nx - n, n:ny - n, n:nz - n][mask & allsame] = n + 1
        a = t
    return a.reshape(-1).astype(np.int8)


def pore_maps(seed=2, nclx=120, ncly=120, nclz=180, dcel=1.0, radius=10.0,
              slab=30.0, volt=1.0, rf_amp=2.0, greff=3.0, zero_mouth=False):
    """Static field, repulsion and RFPAR grids of a cylindrical pore through
    a slab centred at the origin; z fastest, x slowest."""
    rng = np.random.default_rng(seed)
    tx, ty, tz = 0.5 * (nclx - 1) * dcel, 0.5 * (ncly - 1) * dcel, 0.5 * (nclz - 1) * dcel
    xs = np.arange(nclx) * dcel - tx
    ys = np.arange(ncly) * dcel - ty
    zs = np.arange(nclz) * dcel - tz
    X, Y, Z = np.meshgrid(xs, ys, zs, indexing="ij")
    rho = np.sqrt(X * X + Y * Y)
    h = 0.5 * slab
    # static field in the map's units (phi * celec * q = kcal/mol)
    v = volt * 23.060548 / CELEC  # 1 V in kcal/mol/e, over celec
    phi = np.where(Z < -h, 0.5 * v, np.where(Z > h, -0.5 * v, -v * Z / slab))
    for _ in range(12):
        c = rng.uniform([-tx, -ty, -tz], [tx, ty, tz])
        a = rng.uniform(-0.1, 0.1) * v
        w = rng.uniform(4.0, 10.0)
        phi = phi + a * np.exp(-((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2) / (2 * w * w))
    # inaccessible region: the slab outside the pore
    solid = (np.abs(Z) <= h) & (rho >= radius)
    phiv = repwalls(solid.astype(np.int8).reshape(-1), (nclx, ncly, nclz))
    # RFPAR: 1/2 celec q^2 srfe^2 = rf_amp / d, d = distance to the walls
    # (pore wall inside the slab, slab faces outside it); nonzero everywhere
    # unless zero_mouth, which zeroes the grid above and below the pore mouth
    # to exercise the reference's early exit on zero gsrfen values
    d_pore = np.where(np.abs(Z) <= h, radius - rho, np.inf)
    d_slab = np.where(np.abs(Z) > h, np.abs(Z) - h, np.inf)
    d = np.clip(np.minimum(d_pore, d_slab), 1.0, None)
    d = np.where(solid, 1.0, d)
    if zero_mouth:
        d = np.where((np.abs(Z) > h) & (rho < radius), np.inf, d)
    srfe = np.sqrt(2.0 * rf_amp / (CELEC * d))
    grid = dict(nclx=nclx, ncly=ncly, nclz=nclz, dcel=dcel, xbcen=0.0,
                ybcen=0.0, zbcen=0.0)
    return (grid, phi.astype(np.float32).reshape(-1), phiv,
            srfe.astype(np.float32).reshape(-1),
            np.full(nclx * ncly * nclz, greff, np.float32))


def pore(seed=3, nions=2000, maps=None, nclx=120, ncly=120, nclz=180,
         radius=10.0, slab=30.0, precision=abi.FP32, rfpar=True, buffers=True,
         membrane=False, trilinear=True, srpmf=True):
    """Nanopore system: ~nions KCl in the map box, GCMC buffers at both ends."""
    rng = np.random.default_rng(seed)
    if maps is None:
        maps = pore_maps(seed + 100, nclx, ncly, nclz, radius=radius, slab=slab)
    grid, phix, phiv, gsrfen, greff = maps
    tx = 0.5 * (grid["nclx"] - 1) * grid["dcel"]
    tz = 0.5 * (grid["nclz"] - 1) * grid["dcel"]
    Lxy, Lz = 2 * tx - 2.0, 2 * tz - 2.0
    s = SystemSpec(shape=abi.BOX, lx=Lxy, ly=Lxy, lz=Lz, temp=300.0,
                   cdie=80.0, dt=0.02, bdmax=1.0, precision=precision)
    _kcl_types(s)
    if srpmf:
        s.srpmf.update(SRPMF_KCL)
        s.srpmf_rth = 8.0
    s.phix = (grid, phix)
    s.phiv = (grid, phiv, dict(svdw=1000.0, vzmin=-tz, vzmax=tz,
                               trilinear=trilinear))
    if rfpar:
        s.rfpar = (grid, gsrfen, greff, 1.5, None)
    h = 0.5 * slab
    if membrane:
        s.ionic = 1.0
        s.membrane = dict(thick=slab, zmemb=0.0, epsm=2.0, pore=True,
                          types={n: dict(amplmemb=50.0, pmemb=2.0,
                                         amplpore=50.0, ppore=1.0,
                                         radi=radius) for n in ("K", "Cl")})

    def ok(p):
        return not (abs(p[2]) <= h + 1.0 and math.hypot(p[0], p[1]) >= radius - 1.0)

    half = 0.5 * Lxy - 0.5
    p = place(rng, nions, [-half, -half, -0.5 * Lz + 0.5],
              [half, half, 0.5 * Lz - 0.5], ok=ok)
    s.x, s.y, s.z = p[:, 0].copy(), p[:, 1].copy(), p[:, 2].copy()
    s.typei = np.array([1, 2] * (nions // 2) + [1] * (nions % 2), np.int32)
    if buffers:
        zb = 0.5 * Lz
        for name in ("K", "Cl"):
            s.buffers.append(dict(ion=name, conc=1.0, lzmin=-zb, lzmax=-zb + 20.0))
            s.buffers.append(dict(ion=name, conc=1.0, lzmin=zb - 20.0, lzmax=zb))
        s.count()
    return s


def efpot_knots(rng, sigma, eps, r0=2.0, r1=20.0, res=0.05):
    """LJ plus a damped oscillation A exp(-r/lam) cos(2 pi r / ell) sampled
    at res from r0 to r1 (kcal/mol)."""
    r = r0 + res * np.arange(int(round((r1 - r0) / res)) + 1)
    A = rng.uniform(0.3, 1.0)
    lam = rng.uniform(2.0, 4.0)
    ell = rng.uniform(2.5, 3.5)
    s6 = (sigma / r) ** 6
    u = 4 * eps * (s6 * s6 - s6) + A * np.exp(-r / lam) * np.cos(2 * np.pi * r / ell)
    return r, u


def ssdna(seed=4, nions=5000, nnuc=40, maps=None, precision=abi.FP32, bonded=False,
          free=False, **kw):
    """Single-stranded DNA (base, S, P per nucleotide, the site order of
    bonds.f90) along the pore axis, immersed in KCl; ion-site pairs use
    tabulated potentials.  bonded: the bonded and Go-like terms of the strand
    (nucleotides.build_topology on the initial coordinates as the native
    structure); free: the sites move (else FIXSITE)."""
    rng = np.random.default_rng(seed)
    s = pore(seed=seed + 7, nions=nions, maps=maps, precision=precision,
             buffers=False, **kw)
    s.site_type_names = ["S", "P", "Ab", "Tb", "Cb", "Gb"]
    s.lj_eps.update(S=0.2, P=0.2, Ab=0.2, Tb=0.2, Cb=0.2, Gb=0.2)
    s.lj_sigma.update(S=4.0, P=4.0, Ab=4.0, Tb=4.0, Cb=4.0, Gb=4.0)
    bases = rng.integers(3, 7, size=nnuc)
    types, pos = [], []
    z0 = -0.5 * nnuc * 3.4
    for k in range(nnuc):
        z = z0 + 3.4 * k
        ang = 0.6 * k
        types += [int(bases[k]), 1, 2]
        pos += [(2.0 * math.cos(ang + 0.5), 2.0 * math.sin(ang + 0.5), z + 1.2),
                (5.5 * math.cos(ang + 0.3), 5.5 * math.sin(ang + 0.3), z + 1.0),
                (8.0 * math.cos(ang), 8.0 * math.sin(ang), z)]
    pos = np.array(pos)
    s.site_types = np.array(types, np.int32)
    s.site_free = np.full(len(types), 1 if free else 0, np.uint8)
    if bonded:
        names = [s.site_type_names[t - 1] for t in types]
        s.nucl = nucleotides.build_topology(
            names, np.ones(len(types), np.int32), pos,
            fctn=CELEC * s.cgnuc ** 2 / s.cdie)
    # drop ions overlapping the strand
    ions = np.stack([s.x, s.y, s.z], 1)
    d2 = ((ions[:, None, :] - pos[None, :, :]) ** 2).sum(-1).min(1)
    keep = d2 > 9.0
    # ion types follow the site types (types 1..nold are the DNA ones)
    t = s.typei[keep] + len(s.site_type_names)
    ions = ions[keep]
    s.x = np.concatenate([pos[:, 0], ions[:, 0]])
    s.y = np.concatenate([pos[:, 1], ions[:, 1]])
    s.z = np.concatenate([pos[:, 2], ions[:, 2]])
    s.typei = np.concatenate([np.zeros(len(types), np.int32), t]).astype(np.int32)
    s.efpot_res = 0.05
    for site in s.site_type_names:
        for ion, prm in (("K", K_PARAMS), ("Cl", CL_PARAMS)):
            sig = 0.5 * (4.0 + prm["sigma"])
            s.efpot_knots[(site, ion)] = efpot_knots(rng, sig, math.sqrt(0.2 * prm["eps"]))
    return s


def mmij_rect(seed=12, npol=(4, 4, 5), half=(9.0, 9.0, 14.0), rfscal=1.0, scale=2e-3):
    """A RECTBOX MMIJ reaction field: every basis order up to npol - 1 along
    each axis (the order pnpio.f writes, z fastest), a symmetric matrix with
    a negative diagonal (a reaction field lowers the self energy), over the
    region |x| <= half[0], ..."""
    rng = np.random.default_rng(seed)
    lx, ly, lz = np.meshgrid(*(np.arange(n) for n in npol), indexing="ij")
    nt = int(np.prod(npol))
    a = rng.normal(0.0, scale, (nt, nt))
    m = 0.5 * (a + a.T) - np.diag(np.abs(rng.normal(4 * scale, scale, nt)))
    return dict(shape=abi.BOX, npol=tuple(npol), lstp=(lx.ravel(), ly.ravel(), lz.ravel()),
                region=((-half[0], half[0]), (-half[1], half[1]), (-half[2], half[2])),
                rfscal=rfscal, mmij=m)


def mmij_sphere(seed=13, nmpol=5, srdist=12.0, scale=2e-3):
    """A SPHERE MMIJ reaction field of nmpol multipole orders inside radius
    srdist (symmetric matrix, negative diagonal)."""
    rng = np.random.default_rng(seed)
    nt = nmpol * nmpol
    a = rng.normal(0.0, scale, (nt, nt))
    m = 0.5 * (a + a.T) - np.diag(np.abs(rng.normal(4 * scale, scale, nt)))
    return dict(shape=abi.SPHERE, nmpol=nmpol, srdist=srdist, mmij=m)
