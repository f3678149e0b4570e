"""File formats on the CPU: PB/PNP maps and MMIJ files written and read back
(pnpio.f SAVGD1/2/3, readphi.f90, readmmij.f90), and the .btr header the
library forms (simul1.f90:283-287) read back as rdf-bromoc.f90 reads it."""
import struct

import numpy as np
import pytest

from bromoc_gb300 import formats


def test_map_round_trip(tmp_path):
    g = dict(nclx=5, ncly=4, nclz=3, dcel=0.5, xbcen=1.0, ybcen=-2.0, zbcen=0.25)
    v = np.random.default_rng(1).normal(size=60).astype(np.float32)
    formats.write_map(tmp_path / "phix.bin", g, v, params=(80.0, 2.0, 0.1, 25.0, -12.5, 2.0),
                      prftr=2.0)
    m = formats.read_map(tmp_path / "phix.bin")
    assert m.grid == g
    assert m.params == (80.0, 2.0, 0.1, 25.0, -12.5, 2.0)
    np.testing.assert_array_equal(m.values[0], np.float32(2.0) * v)
    raw = (tmp_path / "phix.bin").read_bytes()
    # first record: 3 x int32 + 4 x real*8 = 44 bytes between its markers
    assert struct.unpack_from("<i", raw, 0)[0] == 44
    assert struct.unpack_from("<i", raw, 48)[0] == 44


def test_rfpar_map_has_two_value_records(tmp_path):
    g = dict(nclx=3, ncly=3, nclz=3, dcel=1.0, xbcen=0.0, ybcen=0.0, zbcen=0.0)
    a, b = np.arange(27, dtype=np.float32), -np.arange(27, dtype=np.float32)
    formats.write_map(tmp_path / "rf.bin", g, [a, b], params=(2.1,) * 6)
    m = formats.read_map(tmp_path / "rf.bin")
    assert len(m.values) == 2
    np.testing.assert_array_equal(m.values[1], b)


def test_mmij_round_trip_mirrors_the_lower_triangle(tmp_path):
    npol = (2, 2, 3)
    nt = 12
    lx, ly, lz = np.meshgrid(range(2), range(2), range(3), indexing="ij")
    m = np.random.default_rng(2).normal(size=(nt, nt))
    formats.write_mmij(tmp_path / "mmij.bin", npol, (lx.ravel(), ly.ravel(), lz.ravel()), m)
    shape, n, lstp, mm = formats.read_mmij(tmp_path / "mmij.bin")
    assert shape == "RECTBOX " and tuple(n) == npol
    np.testing.assert_array_equal(lstp[2], lz.ravel())
    iu = np.triu_indices(nt)
    np.testing.assert_array_equal(mm[iu], m[iu])
    np.testing.assert_array_equal(mm, mm.T)


def test_btr_header_and_a_frame_read_back(tmp_path):
    head = formats.traj_header(3, ["S", "P", "Ab", "K", "Cl"])
    assert len(head) == 12 + 12 + 8 + 20
    # a frame as the device packs it (60 + 16 n bytes)
    n = 4
    xyz = np.random.default_rng(3).normal(size=(n, 3)).astype(np.float32)
    fr = (formats._record(struct.pack("<d", 12.5)) + formats._record(struct.pack("<i", n)) +
          formats._record(np.array([1, 2, 4, 5], "<i4").tobytes()) +
          b"".join(formats._record(xyz[:, k].astype("<f4").tobytes()) for k in range(3)))
    assert len(fr) == 60 + 16 * n
    (tmp_path / "t.btr").write_bytes(head + fr)
    nframe, names, frames = formats.read_btr(tmp_path / "t.btr")
    assert nframe == 3 and names == ["S", "P", "Ab", "K", "Cl"]
    assert frames[0].runtime == 12.5
    np.testing.assert_array_equal(frames[0].types, [1, 2, 4, 5])
    np.testing.assert_array_equal(frames[0].xyz, xyz)


def test_mismatched_markers_are_caught(tmp_path):
    bad = struct.pack("<i", 4) + struct.pack("<i", 7) + struct.pack("<i", 5)
    (tmp_path / "bad.btr").write_bytes(bad)
    with pytest.raises(ValueError):
        formats.read_btr(tmp_path / "bad.btr")
