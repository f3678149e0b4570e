"""Small seeded systems exercising each term family of the hot path; shared by
the CPU oracle tests and the GPU parity tests."""
from __future__ import annotations

import numpy as np

from bromoc_gb300 import abi, synth
from bromoc_gb300.deck import SystemSpec

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


def dna(nions=80, nnuc=5, seed=8, precision=abi.FP64, free=True):
    s = synth.ssdna(seed=seed, nions=nions, nnuc=nnuc, maps=small_maps(),
                    precision=precision, radius=6.0, slab=10.0)
    if free:
        s.site_free = np.ones(len(s.site_types), np.uint8)
    s.diffusion = dict(diffcutoff=6.0, diff0=0.05, beta=2.93)
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
