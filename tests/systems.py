"""Small seeded systems exercising each term family of the hot path; shared by
the CPU oracle tests and the GPU parity tests."""
from __future__ import annotations

import numpy as np

from bromoc_gb300 import abi, nucleotides, synth
from bromoc_gb300.deck import CELEC, SystemSpec

_MAPS = {}


def small_maps(nclx=28, ncly=28, nclz=40, radius=6.0, slab=10.0):
    key = (nclx, ncly, nclz, radius, slab)
    if key not in _MAPS:
        _MAPS[key] = synth.pore_maps(seed=11, nclx=nclx, ncly=ncly, nclz=nclz,
                                     radius=radius, slab=slab)
    return _MAPS[key]


def pairs(n_per=24, L=32.0, srpmf=True, seed=5, precision=abi.FP64):
    return synth.bulk_kcl(seed=seed, n_per=n_per, L=L, srpmf=srpmf,
                          precision=precision)


def periodic_kcl(n_per=40, L=36.0, seed=11, precision=abi.FP64, rcut=15.0):
    """Bulk KCl in the extension mode: periodic box, 15 A pair cutoff."""
    return synth.bulk_kcl(seed=seed, n_per=n_per, L=L, srpmf=True, precision=precision,
                          periodic_rcut=rcut)


def efpot_ions(n_per=24, L=32.0, seed=6, precision=abi.FP64):
    """Bulk KCl whose K-Cl and Cl-Cl pairs use tabulated potentials."""
    s = pairs(n_per, L, srpmf=True, seed=seed, precision=precision)
    rng = np.random.default_rng(seed)
    s.efpot_res = 0.05
    s.efpot_knots[("K", "Cl")] = synth.efpot_knots(rng, 3.6, 0.11, r0=2.5, r1=12.0)
    s.efpot_knots[("Cl", "Cl")] = synth.efpot_knots(rng, 4.0, 0.15, r0=2.5, r1=12.0)
    return s


def maps(nions=80, seed=7, trilinear=True, membrane=True, rfpar=True,
         buffers=False, precision=abi.FP64, nfix=0, srpmf=True):
    s = synth.pore(seed=seed, nions=nions, maps=small_maps(), radius=6.0,
                   slab=10.0, precision=precision, rfpar=rfpar,
                   buffers=buffers, membrane=membrane, trilinear=trilinear,
                   srpmf=srpmf)
    s.nfix = nfix
    if buffers:
        s.count()
    return s


def dna(nions=80, nnuc=5, seed=8, precision=abi.FP64, free=True, bonded=True,
        jitter=0.25):
    """ssDNA in the small pore with its bonded and Go-like terms; the sites are
    moved off the native structure by `jitter` A so every term carries force."""
    s = synth.ssdna(seed=seed, nions=nions, nnuc=nnuc, maps=small_maps(),
                    precision=precision, radius=6.0, slab=10.0, bonded=bonded)
    if free:
        s.site_free = np.ones(len(s.site_types), np.uint8)
    if jitter:
        ns = len(s.site_types)
        d = np.random.default_rng(seed + 100).normal(0.0, jitter, (ns, 3))
        s.x[:ns] += d[:, 0]
        s.y[:ns] += d[:, 1]
        s.z[:ns] += d[:, 2]
    s.diffusion = dict(diffcutoff=6.0, diff0=0.05, beta=2.93)
    return s


def dna_duplex(nions=60, nbp=6, seed=21, precision=abi.FP64, qdeby=2):
    """Two complementary strands side by side in the small pore: base pairs,
    inter-strand solvent terms, Debye-Hueckel P-P terms (hybrid: screened
    only with both sites outside the system), an applied force and CONTRANS
    springs on a site and on each strand's centre."""
    s = synth.pore(seed=seed, nions=nions, maps=small_maps(), radius=6.0, slab=10.0,
                   precision=precision, buffers=False, rfpar=False)
    s.site_type_names = ["S", "P", "Ab", "Tb", "Cb", "Gb"]
    s.lj_eps.update(S=0.2, P=0.2, Ab=0.2, Tb=0.2, Cb=0.2, Gb=0.2)
    s.lj_sigma.update(S=4.0, P=4.0, Ab=4.0, Tb=4.0, Cb=4.0, Gb=4.0)
    rng = np.random.default_rng(seed)
    seq = rng.integers(3, 7, size=nbp)
    comp = {3: 4, 4: 3, 5: 6, 6: 5}
    types, pos, strand = [], [], []
    for st, (xs, bases) in enumerate(((-1.0, seq), (1.0, [comp[int(b)] for b in seq[::-1]]))):
        for k, b in enumerate(bases):
            z = -0.5 * nbp * 3.4 + 3.4 * k
            types += [int(b), 1, 2]
            pos += [(xs * 2.4, 0.3 * k, z), (xs * 4.2, 0.4 * k, z + 0.9),
                    (xs * 8.2, 0.2 * k, z + 2.1)]
            strand += [st + 1] * 3
    pos = np.array(pos)
    names = [s.site_type_names[t - 1] for t in types]
    ns = len(types)
    topo = nucleotides.build_topology(
        names, strand, pos, fctn=CELEC * s.cgnuc ** 2 / s.cdie, kappa=9.6, qdeby=qdeby,
        qsolv=True, epsolv=0.35, scalepairing=1.3)
    topo.apfor = [(2, (0.3, -0.2, 0.5))]
    half = ns // 2
    topo.contrans = [(0, (0.4, 0.0, 0.7), (0.1, 0.0, -0.2)), (5, (0.0, 1.2, 0.0), (0.0, 0.5, 0.0))]
    topo.contr_second = (0.2, 0.0, 0.3)
    topo.qunsplit = True
    topo.nsites1st = half
    s.nucl = topo
    s.site_types = np.array(types, np.int32)
    s.site_free = np.ones(ns, np.uint8)
    s.site_free[7] = 0
    d = rng.normal(0.0, 0.25, (ns, 3))
    pos = pos + d
    ions = np.stack([s.x, s.y, s.z], 1)
    keep = ((ions[:, None, :] - pos[None, :, :]) ** 2).sum(-1).min(1) > 9.0
    t = s.typei[keep] + len(s.site_type_names)
    ions = ions[keep]
    s.x = np.concatenate([pos[:, 0], ions[:, 0]])
    s.y = np.concatenate([pos[:, 1], ions[:, 1]])
    s.z = np.concatenate([pos[:, 2], ions[:, 2]])
    s.typei = np.concatenate([np.zeros(ns, np.int32), t]).astype(np.int32)
    s.efpot_res = 0.05
    for site in s.site_type_names:
        for ion, prm in (("K", synth.K_PARAMS), ("Cl", synth.CL_PARAMS)):
            sig = 0.5 * (4.0 + prm["sigma"])
            s.efpot_knots[(site, ion)] = synth.efpot_knots(rng, sig, 0.3)
    s.diffusion = dict(diffcutoff=6.0, diff0=0.05, beta=2.93)
    return s


def mmij(shape="rect", nions=80, seed=14, precision=abi.FP64, buffers=False):
    """The small pore (fields, RFPAR off) with an MMIJ reaction field over a
    region that holds part of the ions."""
    s = synth.pore(seed=seed, nions=nions, maps=small_maps(), radius=6.0, slab=10.0,
                   precision=precision, buffers=buffers, rfpar=False)
    if buffers:
        s.count()
    s.mmij = (synth.mmij_rect(seed=seed, half=(9.0, 9.0, 12.0), rfscal=1.5) if shape == "rect"
              else synth.mmij_sphere(seed=seed, nmpol=5, srdist=11.0))
    return s


def gcmc(nions=60, seed=9, precision=abi.FP64):
    s = maps(nions=nions, seed=seed, buffers=True, precision=precision,
             membrane=False)
    return s


def all_families():
    """name -> builder for the energy parity sweep."""
    return {
        "pairs": lambda **k: pairs(**k),
        "pairs_nosrpmf": lambda **k: pairs(srpmf=False, **k),
        "efpot": lambda **k: efpot_ions(**k),
        "maps_trln": lambda **k: maps(trilinear=True, **k),
        "maps_spln": lambda **k: maps(trilinear=False, **k),
        "maps_fixed": lambda **k: maps(nfix=6, **k),
        "dna": lambda **k: dna(**k),
        "dna_duplex": lambda **k: dna_duplex(**k),
        "mmij_rect": lambda **k: mmij("rect", **k),
        "mmij_sphere": lambda **k: mmij("sphere", **k),
    }


def make_pair(spec: SystemSpec, gpu_create, oracle_create, cap=4000):
    """The same spec loaded into a GPU engine and an oracle engine."""
    g = gpu_create(cap, spec.precision)
    o = oracle_create(cap)
    spec.push(g)
    spec.push(o)
    return g, o


def efpot_all(n_per=32, L=30.0, seed=13, precision=abi.FP64, r1=10.0):
    """Bulk KCl whose three ion-ion laws are all tabulated (the adjoint's
    system)."""
    s = pairs(n_per, L, srpmf=False, seed=seed, precision=precision)
    rng = np.random.default_rng(seed)
    s.efpot_res = 0.05
    s.efpot_knots[("K", "K")] = synth.efpot_knots(rng, 3.1, 0.09, r0=2.5, r1=r1)
    s.efpot_knots[("K", "Cl")] = synth.efpot_knots(rng, 3.6, 0.11, r0=2.5, r1=r1)
    s.efpot_knots[("Cl", "Cl")] = synth.efpot_knots(rng, 4.0, 0.15, r0=2.5, r1=r1)
    return s
