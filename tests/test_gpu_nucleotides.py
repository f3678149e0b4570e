"""DNA bonded and Go-like terms on the GPU against the oracle: INTERACT of
sites, the bonded/non-bonded masks, FP32 BD steps with moving sites, and the
boundary's argument checks.  (ENERGY and FP64 BD parity of the DNA systems
run in test_gpu_parity's family sweeps.)"""
import numpy as np
import pytest

from bromoc_gb300 import abi

from . import systems

pytestmark = pytest.mark.gpu
CAP = 4000
NUC_TERMS = ("ebond", "eang", "edihe", "estack", "ebp", "eex", "eqq", "esolv", "econ")


def _engines(spec, gpu_lib, oracle_mod):
    g = gpu_lib.create(CAP, spec.precision)
    o = oracle_mod.create(CAP)
    spec.push(g)
    spec.push(o)
    return g, o


@pytest.mark.parametrize("prec", [abi.FP64, abi.FP32])
@pytest.mark.parametrize("mask", [abi.M_BOND, abi.M_NONBOND, abi.M_ALL])
def test_interact_sites(gpu_lib, oracle_mod, prec, mask):
    """INTERACT of every site (interact.f90:211-334 plus its ion-site and
    field terms), FP64 on both sides.  A site's sum holds ~100 terms of
    either sign (LJ-like contacts, ion-site tables) summed in another order
    on each side: 1e-9 of max(1, |dE|)."""
    spec = systems.dna_duplex(precision=prec)
    g, o = _engines(spec, gpu_lib, oracle_mod)
    for j in range(1, spec.nsites + 1):
        a = g.interact(spec.x[j - 1], spec.y[j - 1], spec.z[j - 1], 0, j, mask)
        b = o.interact(spec.x[j - 1], spec.y[j - 1], spec.z[j - 1], 0, j, mask)
        assert abs(a - b) <= 1e-9 * max(1.0, abs(b)), (j, a, b)


@pytest.mark.parametrize("prec", [abi.FP64, abi.FP32])
@pytest.mark.parametrize("mask", [abi.M_BOND, abi.M_NONBOND, abi.M_BOND | abi.M_PHIX, 0])
def test_masks(gpu_lib, oracle_mod, prec, mask):
    """Qnobond / Qnonbond switch the bonded and the Go-like kinds; APFOR and
    CONTRANS act under every mask (energy.mono.f90:504-581)."""
    spec = systems.dna_duplex(precision=prec)
    g, o = _engines(spec, gpu_lib, oracle_mod)
    tg, fg, _ = g.energy(mask, forces=True)
    to, fo, _ = o.energy(mask, forces=True)
    for k in NUC_TERMS:  # FP64 in both modes
        assert abs(tg[k] - to[k]) <= 1e-10 * max(1.0, abs(to[k])), (k, tg[k], to[k])
    etol = 1e-10 if prec == abi.FP64 else 1e-5  # ener holds the FP32 pair/field terms
    assert abs(tg["ener"] - to["ener"]) <= etol * max(1.0, abs(to["ener"]))
    ns = spec.nsites
    scale = max(np.abs(fo[:ns]).max(), 1e-300)
    tol = 1e-10 if prec == abi.FP64 else 1e-5
    assert np.abs(fg[:ns] - fo[:ns]).max() <= tol * scale


@pytest.mark.parametrize("family", ["dna", "dna_duplex"])
def test_bd_steps_fp32_moving_sites(gpu_lib, oracle_mod, family):
    """FP32 ENERGY + DYNAMICS with free sites: positions of sites and ions
    within 1e-5 A of the FP64 oracle after one step, energies of the DNA
    terms within 1e-8 relative after five."""
    spec = systems.all_families()[family](precision=abi.FP32)
    g, o = _engines(spec, gpu_lib, oracle_mod)
    g.bd_steps(1, seed=77, step0=0, energies=False)
    o.bd_steps(1, seed=77, step0=0)
    pg = np.stack(g.get_particles()[:3], 1)
    po = np.stack(o.get_particles()[:3], 1)
    assert np.abs(pg - po).max() <= 1e-5
    moved = np.abs(po[:spec.nsites] - np.stack([spec.x, spec.y, spec.z], 1)[:spec.nsites])
    assert moved.max() > 1e-3  # the sites do move
    eg = g.bd_steps(4, seed=77, step0=1)
    eo = o.bd_steps(4, seed=77, step0=1)
    for k in NUC_TERMS:
        assert abs(eg[k] - eo[k]) <= 1e-6 * max(1.0, abs(eo[k])), (k, eg[k], eo[k])


def test_set_sites_clears_the_lists(gpu_lib, oracle_mod):
    spec = systems.dna_duplex()
    g, o = _engines(spec, gpu_lib, oracle_mod)
    assert g.energy(abi.M_ALL)[0]["ebond"] != 0.0
    nucl = spec.nucl
    spec.nucl = None
    spec.push(g)
    spec.push(o)
    tg = g.energy(abi.M_ALL)[0]
    to = o.energy(abi.M_ALL)[0]
    assert all(tg[k] == 0.0 for k in NUC_TERMS)
    assert abs(tg["ener"] - to["ener"]) <= 1e-10 * abs(to["ener"])
    spec.nucl = nucl


def test_bad_lists_are_refused(gpu_lib):
    spec = systems.dna_duplex()
    g = gpu_lib.create(CAP, abi.FP64)
    spec.push(g)
    bad = systems.dna_duplex().nucl
    bad.dihes = bad.dihes + [((1, 2, 3, spec.nsites + 5), 0.0)]
    with pytest.raises(abi.BromocError) as e:
        g.set_nucleotides(bad)
    assert e.value.code == abi.E_ARG
    bad = systems.dna_duplex().nucl
    bad.contrans = [(spec.nsites + 1, (1.0, 0.0, 0.0), (0.0, 0.0, 0.0))]
    with pytest.raises(abi.BromocError):
        g.set_nucleotides(bad)
    # the context still works and has no lists
    assert g.energy(abi.M_ALL)[0]["ebond"] == 0.0


@pytest.mark.parametrize("prec", [abi.FP64, abi.FP32])
def test_notrans_recentres_the_sites(gpu_lib, oracle_mod, prec):
    """NOTRAN (simul1.f90:380-385): after every BD step the sites' centre
    along x and z is back at the given values; positions match the oracle."""
    spec = systems.dna_duplex(precision=prec)
    spec.nucl.notrans = (0.5, None, -1.25)
    g, o = _engines(spec, gpu_lib, oracle_mod)
    g.bd_steps(3, seed=12, step0=0, energies=False)
    o.bd_steps(3, seed=12, step0=0)
    pg = np.stack(g.get_particles()[:3], 1)
    po = np.stack(o.get_particles()[:3], 1)
    tol = 1e-9 if prec == abi.FP64 else 1e-5
    assert np.abs(pg - po).max() <= tol
    ns = spec.nsites
    c = pg[:ns].mean(0)
    assert abs(c[0] - 0.5) <= 1e-6 and abs(c[2] + 1.25) <= 1e-6
    assert abs(c[1] - np.asarray(spec.y[:ns]).mean()) > 1e-6  # y is left free
