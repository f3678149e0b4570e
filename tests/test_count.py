"""COUNT (count.f90) in the oracle: buffer membership, nat and type signs
equal the deck-time count of the same positions (SystemSpec.count), and
ntotat grows by nat at every call."""
import numpy as np

from bromoc_gb300 import abi

from . import systems


def test_oracle_count_matches_the_deck_count(oracle_mod):
    spec = systems.gcmc(precision=abi.FP64)
    o = oracle_mod.create(4000)
    spec.push(o)
    # scramble the buffer tags and signs, then let COUNT restore them
    t0 = spec.typei.copy()
    o.set_particles(spec.x, spec.y, spec.z, np.abs(t0), spec.nsites, spec.nfix,
                    np.zeros(len(t0), np.int32))
    nt0 = o.ntotat().copy()
    o.count()
    nat_deck = spec.count()
    x, y, z, t, ib = o.get_particles()
    np.testing.assert_array_equal(ib, spec.ibuffer)
    np.testing.assert_array_equal(t, spec.typei)
    nat = o.get_buffers()[0]
    np.testing.assert_array_equal(nat, nat_deck)
    np.testing.assert_array_equal(o.ntotat(), nt0 + np.asarray(nat_deck))
