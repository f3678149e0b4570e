"""File formats around the hot path, and the per-cycle analysis.

- `.btr` trajectories (simul1.f90:283-287, wrttraj.f90:33-38; the reader
  tools/src/rdf-bromoc.f90:93-200): gfortran unformatted sequential records,
  each framed by 4-byte length markers.  Header: nframe, nttyp, atnam2
  (character*4 each); frame: runtime (real*8), ntot, typtyp(1:ntot), and x,
  y, z rounded to real*4.  `TrajWriter` appends frames that the library packs
  on the device (bromoc_gpu_traj_frame); `read_btr` reads a file back.
- PB/PNP map files (pb-pnp/src/pnpio.f:489-508 SAVGD1, read by
  cg-gcmc-bd/src/readphi.f90:19-52): (nclx, ncly, nclz, dcel, xbcen, ybcen,
  zbcen), (epsw, epsp, conc, tmemb, zmemb, epsm), then the nclx*ncly*nclz
  real*4 values (z fastest).  RFPAR maps (SAVGD3) carry two value records
  and the ion radius six times in the second record.
- MMIJ files (pnpio.f SAVGD2, read by readmmij.f90): shape (character*8),
  then for RECTBOX (xnpol, ynpol, znpol), lstpx, lstpy, lstpz and mij(ntpol^2).
- `Profiles`: the device-side rho(z), rho_DNA(z) and RDF sums of
  simul1.f90:476-509 (bromoc_gpu_set/accum/get_profiles).
"""
from __future__ import annotations

import ctypes as C
import struct
from dataclasses import dataclass

import numpy as np

from . import _lib, abi


# ---- gfortran unformatted sequential records --------------------------------
def _record(payload: bytes) -> bytes:
    n = struct.pack("<i", len(payload))
    return n + payload + n


def _records(buf: bytes):
    """Yield the payloads of consecutive records; a marker mismatch raises."""
    off = 0
    while off < len(buf):
        (n,) = struct.unpack_from("<i", buf, off)
        end = off + 4 + n
        (m,) = struct.unpack_from("<i", buf, end)
        if m != n:
            raise ValueError(f"record markers {n} and {m} differ at byte {off}")
        yield buf[off + 4:end]
        off = end + 4


# ---- .btr trajectories ----------------------------------------------------------
def traj_header(nframe: int, names) -> bytes:
    """Header records of a .btr file (simul1.f90:283-287)."""
    at = b"".join(n.encode()[:4].ljust(4) for n in names)
    n = C.c_int64(0)
    lib = _lib.load()
    rc = lib.bromoc_gpu_traj_header(nframe, len(names), at, None, 0, C.byref(n))
    if rc != abi.OK:
        raise abi.BromocError(rc, "bromoc_gpu_traj_header")
    buf = C.create_string_buffer(n.value)
    rc = lib.bromoc_gpu_traj_header(nframe, len(names), at, buf, n.value, C.byref(n))
    if rc != abi.OK:
        raise abi.BromocError(rc, "bromoc_gpu_traj_header")
    return buf.raw[:n.value]


def traj_frame(eng: abi.Engine, runtime: float) -> bytes:
    """One .btr frame of the context's current state, packed on the device."""
    lib = _lib.load()
    n = C.c_int64(0)
    eng._chk(lib.bromoc_gpu_traj_frame(eng.h, runtime, None, 0, C.byref(n)), "traj_frame")
    buf = C.create_string_buffer(n.value)
    eng._chk(lib.bromoc_gpu_traj_frame(eng.h, runtime, buf, n.value, C.byref(n)), "traj_frame")
    return buf.raw[:n.value]


class TrajWriter:
    """Writes a .btr file: the header at open, one frame per write()."""

    def __init__(self, path, nframe: int, names):
        self.f = open(path, "wb")
        self.f.write(traj_header(nframe, names))

    def write(self, eng: abi.Engine, runtime: float) -> None:
        self.f.write(traj_frame(eng, runtime))

    def close(self) -> None:
        self.f.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


@dataclass
class Frame:
    runtime: float
    types: np.ndarray
    xyz: np.ndarray  # [ntot, 3] float32


def read_btr(path):
    """(nframe, names, frames) of a .btr file, read the way
    tools/src/rdf-bromoc.f90:93-200 reads it."""
    recs = _records(open(path, "rb").read())
    (nframe,) = struct.unpack("<i", next(recs))
    (nttyp,) = struct.unpack("<i", next(recs))
    at = next(recs)
    names = [at[4 * k:4 * k + 4].decode().rstrip() for k in range(nttyp)]
    frames = []
    for r in recs:
        (runtime,) = struct.unpack("<d", r)
        (n,) = struct.unpack("<i", next(recs))
        types = np.frombuffer(next(recs), "<i4").copy()
        xyz = np.stack([np.frombuffer(next(recs), "<f4") for _ in range(3)], 1)
        assert len(types) == n
        frames.append(Frame(runtime, types, xyz))
    return nframe, names, frames


# ---- PB/PNP maps -----------------------------------------------------------------
@dataclass
class MapFile:
    grid: dict                  # nclx, ncly, nclz, dcel, xbcen, ybcen, zbcen
    params: tuple               # (epsw, epsp, conc, tmemb, zmemb, epsm) or 6 x radion
    values: list                # one float32 array per value record


def write_map(path, grid: dict, values, params=(80.0, 1.0, 0.0, 0.0, 0.0, 1.0),
              prftr: float = 1.0) -> None:
    """SAVGD1 (one value record, prftr * values) or, with a list of two
    arrays, SAVGD3 (the RFPAR map pair)."""
    vals = values if isinstance(values, (list, tuple)) else [values]
    head = struct.pack("<3i4d", grid["nclx"], grid["ncly"], grid["nclz"], grid["dcel"],
                       grid["xbcen"], grid["ybcen"], grid["zbcen"])
    out = [_record(head), _record(struct.pack("<6d", *params))]
    n3 = grid["nclx"] * grid["ncly"] * grid["nclz"]
    for v in vals:
        v = np.asarray(v, np.float32).reshape(-1)
        if v.size != n3:
            raise ValueError(f"map holds {v.size} values, grid {n3}")
        out.append(_record((np.float32(prftr) * v).astype("<f4").tobytes()))
    with open(path, "wb") as f:
        f.write(b"".join(out))


def read_map(path) -> MapFile:
    """readphi.f90:43-52 (and readrfpar's two-record form)."""
    recs = list(_records(open(path, "rb").read()))
    nclx, ncly, nclz, dcel, xb, yb, zb = struct.unpack("<3i4d", recs[0])
    grid = dict(nclx=nclx, ncly=ncly, nclz=nclz, dcel=dcel, xbcen=xb, ybcen=yb, zbcen=zb)
    params = struct.unpack("<6d", recs[1])
    vals = [np.frombuffer(r, "<f4").copy() for r in recs[2:]]
    return MapFile(grid, params, vals)


def write_mmij(path, npol, lstp, mij) -> None:
    """SAVGD2 for a RECTBOX basis: npol = (xnpol, ynpol, znpol), lstp =
    (lstpx, lstpy, lstpz), mij the ntpol x ntpol matrix (row-major)."""
    ntpol = int(np.prod(npol))
    mij = np.asarray(mij, np.float64).reshape(-1)
    if mij.size != ntpol * ntpol:
        raise ValueError("mij must hold ntpol^2 values")
    out = [_record(b"RECTBOX "), _record(struct.pack("<3i", *npol))]
    for l in lstp:
        out.append(_record(np.asarray(l, "<i4").tobytes()))
    out.append(_record(mij.astype("<f8").tobytes()))
    with open(path, "wb") as f:
        f.write(b"".join(out))


def read_mmij(path):
    """readmmij.f90 (RECTBOX): (shape, npol, (lstpx, lstpy, lstpz), mij) with
    the lower triangle mirrored from the upper one as readmmij does."""
    recs = list(_records(open(path, "rb").read()))
    shape = recs[0].decode()
    if shape != "RECTBOX ":
        raise ValueError(f"MMIJ shape {shape!r}: RECTBOX files only")
    npol = struct.unpack("<3i", recs[1])
    ntpol = int(np.prod(npol))
    lstp = tuple(np.frombuffer(recs[k], "<i4").copy() for k in (2, 3, 4))
    m = np.frombuffer(recs[5], "<f8").copy().reshape(ntpol, ntpol)
    iu = np.triu_indices(ntpol, 1)
    m[(iu[1], iu[0])] = m[iu]  # mmij(ij) = mmij(ji) for i > j
    return shape, npol, lstp, m


# ---- per-cycle profiles ------------------------------------------------------------
class Profiles:
    """rho(z) of the ions, rho(z) of the DNA sites and the RDF around one
    particle, summed on the device once per accumulate() (simul1.f90:476-509)."""

    def __init__(self, eng: abi.Engine, rho=True, rdna=False, gr=False, igr=1, dr=0.1,
                 npoints=1000):
        self.eng, self.npoints = eng, npoints
        self.lib = _lib.load()
        eng._chk(self.lib.bromoc_gpu_set_profiles(eng.h, int(rho), int(rdna), int(gr), igr,
                                                  dr, npoints), "set_profiles")

    def accumulate(self) -> None:
        self.eng._chk(self.lib.bromoc_gpu_accum_profiles(self.eng.h), "accum_profiles")

    def get(self):
        """dict rho [ntype-nold, nzmax], rdna [ndna, nzmax], gr [ntype-nold,
        npoints], nzmax, irmax."""
        e = self.eng
        nion = e.ntype - e.nold
        nz = C.c_int32(0)
        e._chk(self.lib.bromoc_gpu_get_profiles(e.h, None, None, None, C.byref(nz), None),
               "get_profiles")
        rho = np.zeros((max(nion, 1), max(nz.value, 1)))
        rdna = np.zeros((max(e.ndna, 1), max(nz.value, 1)))
        gr = np.zeros((max(nion, 1), self.npoints))
        irmax = C.c_int32(0)
        d = C.POINTER(C.c_double)
        e._chk(self.lib.bromoc_gpu_get_profiles(
            e.h, rho.ctypes.data_as(d), rdna.ctypes.data_as(d), gr.ctypes.data_as(d),
            C.byref(nz), C.byref(irmax)), "get_profiles")
        return dict(rho=rho, rdna=rdna, gr=gr, nzmax=nz.value, irmax=irmax.value)
