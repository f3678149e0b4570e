"""Generate the golden vectors of tests/golden/golden.npz.

The reference (Fortran) cannot be built or imported here and ships no golden
vectors, so these come from the FP64 CPU restatement in oracle/ on the seeded
systems of tests/systems.py (the last of them in the periodic extension mode):
for each term family the ENERGY terms (BROMOC_NTERMS of them) and the forces, the positions after
two BD steps with the injected Philox noise, and
for the GCMC system the buffer counters and particle count after five GRAND
calls.  They pin the restatement (and, through the GPU tests, the FP64 GPU
path) against later changes.

    python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from bromoc_gb300 import abi  # noqa: E402
from oracle import oracle  # noqa: E402
from tests import systems  # noqa: E402

CAP = 4000
SEED, STEP0 = 31, 7


def families():
    return {
        "pairs": systems.pairs(),
        "efpot": systems.efpot_ions(),
        "maps_trln": systems.maps(),
        "maps_spln": systems.maps(trilinear=False),
        "dna": systems.dna(),
        "dna_duplex": systems.dna_duplex(),
        "periodic": systems.periodic_kcl(),
    }


def record(spec):
    o = oracle.create(CAP)
    spec.push(o)
    terms, f, warn = o.energy(abi.M_ALL, forces=True)
    o.bd_steps(2, seed=SEED, step0=STEP0)
    x, y, z = o.get_particles()[:3]
    return dict(terms=np.array([terms[k] for k in abi.TERM_NAMES]), forces=f,
                warn=np.asarray(warn), pos2=np.stack([x, y, z], 1))


def record_gcmc():
    spec = systems.gcmc()
    o = oracle.create(CAP)
    spec.push(o)
    for cyc in range(1, 6):
        o.grand(4, SEED, cyc)
    nat, nins, nrem, _ = o.get_buffers()
    x = o.get_particles()[0]
    return dict(nat=np.asarray(nat), ninsert=np.asarray(nins), nremove=np.asarray(nrem),
                ntot=np.array([len(x)]))


def main():
    oracle.build()
    out = {}
    for name, spec in families().items():
        for k, v in record(spec).items():
            out[f"{name}/{k}"] = v
    for k, v in record_gcmc().items():
        out[f"gcmc/{k}"] = v
    np.savez_compressed(Path(__file__).with_name("golden.npz"), **out)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    main()
