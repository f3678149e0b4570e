"""DNA bonded and Go-like terms on the CPU: the list builder's selection rules,
and the oracle's forces against central differences of its own ENERGY (the
reference's TEST procedure, testfirst.f90:35-62) on a two-strand system that
holds every term kind."""
from __future__ import annotations

import numpy as np
import pytest

from bromoc_gb300 import abi, nucleotides

from . import systems


def test_topology_rules_single_strand():
    """bonds.f90 / angles.f90 / dihedral.f90 on base-S-P x 3 (sites 1..9)."""
    names = ["Ab", "S", "P", "Cb", "S", "P", "Gb", "S", "P"]
    pos = np.random.default_rng(1).normal(0.0, 5.0, (9, 3))
    t = nucleotides.build_topology(names, [1] * 9, pos)
    assert [b[0] for b in t.bonds] == [(1, 2), (2, 3), (3, 5), (4, 5), (5, 6), (6, 8),
                                       (7, 8), (8, 9)]
    assert [a[0] for a in t.angles] == [(1, 2, 3), (2, 3, 5), (3, 5, 4), (3, 5, 6), (4, 5, 6),
                                        (5, 6, 8), (6, 8, 7), (6, 8, 9), (7, 8, 9)]
    assert [d[0] for d in t.dihes] == [(1, 2, 3, 5), (2, 3, 5, 4), (2, 3, 5, 6), (3, 5, 6, 8),
                                       (4, 5, 6, 8), (5, 6, 8, 7), (5, 6, 8, 9)]
    # natural values are the native geometry's
    (i, j), d0 = t.bonds[2]
    assert d0 == pytest.approx(np.linalg.norm(pos[j - 1] - pos[i - 1]))
    # every unbonded pair lands in exactly one of stack / bp / ex
    npairs = 9 * 8 // 2 - len(t.bonds)
    assert len(t.stacks) + len(t.bps) + len(t.exs) == npairs
    # P-P electrostatics skip pairs of a bond angle (3-6 by 3-5-6, 6-9 by 6-8-9)
    assert t.qqs == [(9, 3)]


def test_topology_pairs_and_solvent():
    s = systems.dna_duplex()
    t = s.nucl
    c = t.counts()
    assert c["bp"] > 0 and c["solv"] > 0 and c["stack"] > 0 and c["ex"] > 0
    gc = [b for b in t.bps if b[2]]
    assert all(b[1] == 2.8694 for b in gc)
    assert all(b[1] == 2.9002 for b in t.bps if not b[2])


def _fd(eng, spec, mask, sites, h=1e-5):
    x, y, z, ty = spec.x.copy(), spec.y.copy(), spec.z.copy(), spec.typei.copy()
    out = {}
    for i in sites:
        row = []
        for arr in (x, y, z):
            v = arr[i]
            e = []
            for d in (-h, h):
                arr[i] = v + d
                eng.set_particles(x, y, z, ty, spec.nsites, spec.nfix)
                e.append(eng.energy(mask, forces=False)[0]["ener"])
            arr[i] = v
            row.append(-(e[1] - e[0]) / (2 * h))
        out[i] = np.array(row)
    eng.set_particles(x, y, z, ty, spec.nsites, spec.nfix)
    return out


def _sites_only(spec):
    ns = spec.nsites
    sp = type("Sites", (), {})()
    sp.x, sp.y, sp.z = spec.x[:ns].copy(), spec.y[:ns].copy(), spec.z[:ns].copy()
    sp.typei, sp.nsites, sp.nfix = spec.typei[:ns].copy(), ns, 0
    return sp


@pytest.mark.parametrize("qdeby", [0, 1, 2])
def test_oracle_site_forces_are_energy_gradients(oracle_mod, qdeby):
    """Every kind but the bond angle (next test): forces on the free sites
    against central differences, with the ions and their ion-site terms."""
    spec = systems.dna_duplex(qdeby=qdeby)
    o = oracle_mod.create(4000)
    spec.push(o)
    mask = abi.M_BOND | abi.M_NONBOND
    t, _, _ = o.energy(mask, forces=True)
    for k in ("ebond", "eang", "edihe", "estack", "ebp", "eex", "eqq", "esolv", "econ"):
        assert t[k] != 0.0, k
    spec.nucl.angles = []
    spec.nucl.apfor = []  # a constant force has no energy
    spec.push(o)
    _, f, _ = o.energy(mask, forces=True)
    free = [i for i in range(spec.nsites) if spec.site_free[i]]
    fd = _fd(o, spec, mask, free)
    scale = np.abs(f[:spec.nsites]).max()
    for i in free:
        assert np.abs(fd[i] - f[i]).max() <= 2e-6 * scale, (i, fd[i], f[i])


def test_oracle_angle_force_is_the_references(oracle_mod):
    """energy.mono.f90:255-273 gives the end sites of a bond angle the force
    de r_other (de = 1400 eps dtheta / (|r1||r2| sin theta)), without the
    -cos(theta) r_own / |r_own|^2 part of the gradient: the difference from
    central differences lies along the site's own arm, and the vertex takes
    minus the sum."""
    spec = systems.dna_duplex()
    full = spec.nucl
    sp = _sites_only(spec)
    for (a, b, c), th0 in full.angles[:6]:
        t = nucleotides.Topology(epsnuc=full.epsnuc)
        t.angles = [((a, b, c), th0)]
        spec.nucl = t
        o = oracle_mod.create(4000)
        spec.push(o)
        o.set_particles(sp.x, sp.y, sp.z, sp.typei, sp.nsites, 0)
        _, f, _ = o.energy(abi.M_BOND, forces=True)
        fd = _fd(o, sp, abi.M_BOND, [a - 1, c - 1])
        P = np.stack([sp.x, sp.y, sp.z], 1)
        for end, own in ((a, P[a - 1] - P[b - 1]), (c, P[c - 1] - P[b - 1])):
            if not spec.site_free[end - 1]:
                continue
            d = f[end - 1] - fd[end - 1]
            u = own / np.linalg.norm(own)
            perp = d - np.dot(d, u) * u
            assert np.abs(perp).max() <= 1e-6 * np.abs(f[end - 1]).max(), (a, b, c, end)
        if spec.site_free[[a - 1, b - 1, c - 1]].all():
            assert np.allclose(f[b - 1], -(f[a - 1] + f[c - 1]), rtol=0, atol=1e-12)
    spec.nucl = full


def test_oracle_interact_of_a_site_is_its_terms(oracle_mod):
    """INTERACT(site j) with the bonded mask equals ENERGY of a topology that
    keeps only the terms naming j (no ions, no fields)."""
    spec = systems.dna_duplex()
    spec.nucl.scalepairing = 1.0  # INTERACT's base pairs carry no pairing scale
    ns = spec.nsites
    full = spec.nucl
    for j in (1, 5, 11, ns):
        only = nucleotides.Topology(
            epsnuc=full.epsnuc, scalepairing=1.0, fctn=full.fctn, kappa=full.kappa,
            qdeby=full.qdeby, qsolv=full.qsolv, epsolv=full.epsolv)
        only.bonds = [b for b in full.bonds if j in b[0]]
        only.angles = [a for a in full.angles if j in a[0]]
        only.dihes = [d for d in full.dihes if j in d[0]]
        only.stacks = [b for b in full.stacks if j in b[0]]
        only.bps = [b for b in full.bps if j in b[0]]
        only.exs = [b for b in full.exs if j in b[0]]
        only.qqs = [b for b in full.qqs if j in b]
        only.solvs = [b for b in full.solvs if j in b]
        for mask in (abi.M_BOND, abi.M_NONBOND, abi.M_BOND | abi.M_NONBOND):
            o = oracle_mod.create(4000)
            spec.nucl = full
            spec.push(o)
            o.set_particles(spec.x[:ns], spec.y[:ns], spec.z[:ns], spec.typei[:ns], ns, 0)
            de = o.interact(spec.x[j - 1], spec.y[j - 1], spec.z[j - 1], 0, j, mask)
            spec.nucl = only
            o2 = oracle_mod.create(4000)
            spec.push(o2)
            o2.set_particles(spec.x[:ns], spec.y[:ns], spec.z[:ns], spec.typei[:ns], ns, 0)
            t, _, _ = o2.energy(mask, forces=False)
            e = sum(t[k] for k in ("ebond", "eang", "edihe", "estack", "ebp", "eex", "eqq",
                                   "esolv"))
            assert de == pytest.approx(e, rel=1e-12, abs=1e-12), (j, mask)
        spec.nucl = full


def test_oracle_rejects_bad_lists(oracle_mod):
    spec = systems.dna_duplex()
    o = oracle_mod.create(4000)
    spec.push(o)
    bad = systems.dna_duplex().nucl
    bad.bonds = bad.bonds + [((1, spec.nsites + 1), 3.0)]
    with pytest.raises(abi.BromocError):
        o.set_nucleotides(bad)
