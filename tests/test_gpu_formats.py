"""Device-side analysis and trajectory frames against CPU restatements:
rho(z), rho_DNA(z) and the RDF counts of simul1.f90:476-509 (exact), and
.btr frames (wrttraj.f90) whose coordinates are the single-precision
roundings of the positions."""
import numpy as np
import pytest

from bromoc_gb300 import abi, formats
from oracle import analysis

from . import systems

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [abi.FP64, abi.FP32])
def test_profiles_count_like_the_reference(gpu_lib, prec):
    spec = systems.dna(nions=120, precision=prec)
    g = gpu_lib.create(4000, prec)
    spec.push(g)
    prof = formats.Profiles(g, rho=True, rdna=True, gr=True, igr=spec.nsites + 3, dr=0.25,
                            npoints=400)
    acc = {}
    typtyp = np.asarray(spec.site_types)
    for c in range(4):
        g.bd_steps(5, seed=11, step0=5 * c, energies=False)
        prof.accumulate()
        x, y, z, t, _ = g.get_particles()
        analysis.accumulate(acc, x, y, z, t, spec.nsites, spec.nfix, spec.nold, typtyp,
                            lz=spec.lz, cz=spec.cz, npoints=400, rho=True, rdna=True,
                            gr=True, igr=spec.nsites + 3, dr=0.25)
    got = prof.get()
    nz = got["nzmax"]
    assert nz == analysis.profile_bins(spec.lz, spec.cz, 400)[2]
    r = acc["rho"]
    np.testing.assert_array_equal(got["rho"][:r.shape[0]], r)
    np.testing.assert_array_equal(got["rdna"][:acc["rdna"].shape[0]], acc["rdna"])
    np.testing.assert_array_equal(got["gr"][:acc["gr"].shape[0]], acc["gr"])
    assert got["irmax"] == acc["irmax"]
    assert got["rho"].sum() == 4 * (len(spec.x) - spec.nsites - spec.nfix)


def test_traj_frames_round_trip(gpu_lib, tmp_path):
    spec = systems.dna(nions=90, precision=abi.FP32)
    g = gpu_lib.create(4000, abi.FP32)
    spec.push(g)
    names = list(spec.site_type_names) + list(spec.ion_names)
    with formats.TrajWriter(tmp_path / "run.btr", 3, names) as w:
        for k in range(3):
            g.bd_steps(4, seed=5, step0=4 * k, energies=False)
            w.write(g, runtime=(k + 1) * 4 * spec.dt)
            x, y, z, t, _ = g.get_particles()
            last = np.stack([x, y, z], 1), t
    nframe, got_names, frames = formats.read_btr(tmp_path / "run.btr")
    assert nframe == 3 and got_names == [n[:4] for n in names]
    f = frames[-1]
    assert f.runtime == pytest.approx(12 * spec.dt)
    np.testing.assert_array_equal(f.xyz, last[0].astype(np.float32))
    nw = spec.nwtype()
    expect = np.concatenate([spec.site_types, nw[np.abs(last[1][spec.nsites:]) - 1]])
    np.testing.assert_array_equal(f.types, expect)
