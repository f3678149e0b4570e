"""Golden vectors (tests/golden/golden.npz, made by tests/golden/make_golden.py
from the FP64 restatement): the oracle still reproduces them on this machine
(CPU), and the FP64 GPU path reproduces them to summation-order rounding
(GPU).  Integer outputs must match exactly."""
from pathlib import Path

import numpy as np
import pytest

from bromoc_gb300 import abi

from .golden import make_golden as mg

GOLD = np.load(Path(__file__).parent / "golden" / "golden.npz")
FAMILIES = ["pairs", "efpot", "maps_trln", "maps_spln", "dna", "dna_duplex", "periodic"]


def _scale(a):
    return max(np.abs(a).max(), 1e-300)


def _check(name, rec, tol_e, tol_f, tol_x):
    g = {k.split("/")[1]: GOLD[k] for k in GOLD.files if k.startswith(name + "/")}
    assert np.abs(rec["terms"] - g["terms"]).max() <= tol_e * max(1.0, _scale(g["terms"])), name
    assert np.abs(rec["forces"] - g["forces"]).max() <= tol_f * _scale(g["forces"]), name
    np.testing.assert_array_equal(rec["warn"], g["warn"])
    assert np.abs(rec["pos2"] - g["pos2"]).max() <= tol_x, name


@pytest.mark.parametrize("name", FAMILIES)
def test_oracle_reproduces_golden(oracle_mod, name):
    rec = mg.record(mg.families()[name])
    _check(name, rec, 1e-12, 1e-12, 1e-12)


def test_oracle_gcmc_golden(oracle_mod):
    rec = mg.record_gcmc()
    for k, v in rec.items():
        np.testing.assert_array_equal(v, GOLD["gcmc/" + k])


def _record_gpu(gpu_lib, spec):
    g = gpu_lib.create(mg.CAP, abi.FP64)
    spec.push(g)
    terms, f, warn = g.energy(abi.M_ALL, forces=True)
    g.bd_steps(2, seed=mg.SEED, step0=mg.STEP0)
    x, y, z = g.get_particles()[:3]
    return dict(terms=np.array([terms[k] for k in abi.TERM_NAMES]), forces=f,
                warn=np.asarray(warn), pos2=np.stack([x, y, z], 1))


@pytest.mark.gpu
@pytest.mark.parametrize("name", FAMILIES)
def test_gpu_fp64_matches_golden(gpu_lib, name):
    _check(name, _record_gpu(gpu_lib, mg.families()[name]), 1e-10, 1e-10, 1e-9)


@pytest.mark.gpu
def test_gpu_gcmc_golden(gpu_lib):
    spec = mg.systems.gcmc()
    g = gpu_lib.create(mg.CAP, abi.FP64)
    spec.push(g)
    for cyc in range(1, 6):
        g.grand(4, mg.SEED, cyc)
    nat, nins, nrem, _ = g.get_buffers()
    np.testing.assert_array_equal(nat, GOLD["gcmc/nat"])
    np.testing.assert_array_equal(nins, GOLD["gcmc/ninsert"])
    np.testing.assert_array_equal(nrem, GOLD["gcmc/nremove"])
    assert len(g.get_particles()[0]) == int(GOLD["gcmc/ntot"][0])
