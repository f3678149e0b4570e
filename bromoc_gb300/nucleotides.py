"""DNA bonded and Go-like term lists (the NUCLEOTIDES section's setup).

`build_topology` applies the selection rules of the reference's list
builders to a strand description (site names, strand numbers, native
coordinates):
  bonds.f90:37-110     base-S, S-P (same strand), P-S(next) (same strand)
  angles.f90:30-145    base-S-P, S-P-S(next), P-S(next)-base(next),
                       P-S(next)-P(next)
  dihedral.f90:16-150  base-S-P-S(next), S-P-S(next)-base(next),
                       S-P-S(next)-P(next), P-S(next)-P(next)-S(next+1)
  go_qq.f90:30-100     every non-bonded pair: a native contact (same strand,
                       native distance under 9 A), a base pair (G-C or A-T),
                       or excluded volume; P-P electrostatics outside bond
                       angles; S-S solvent terms between strands
The natural lengths, angles and torsions are measured on the native
coordinates themselves, as native_structure.f90 measures them on its ideal
B-DNA (so the native structure has zero bonded energy).  Site order along
a strand is base, S, P per nucleotide, the order bonds.f90 accepts.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import abi
from .abi import ptr

BASES = ("Ab", "Tb", "Cb", "Gb")
PAIRS = {("Gb", "Cb"), ("Cb", "Gb"), ("Ab", "Tb"), ("Tb", "Ab")}


def angbond(r1, r2) -> float:
    """angbond.f90: angle between r1 and r2."""
    c = float(np.dot(r1, r2)) / (math.sqrt(float(np.dot(r1, r1))) *
                                 math.sqrt(float(np.dot(r2, r2))))
    return math.acos(c)


def angdih(r1, r2, r3) -> float:
    """angdih.f90: torsion of the bond vectors r1, r2, r3."""
    n1 = np.cross(r1, r2)
    n2 = np.cross(r2, r3)
    return math.atan2(math.sqrt(float(np.dot(r2, r2))) * float(np.dot(r1, n2)),
                      float(np.dot(n1, n2)))


@dataclass
class Topology:
    epsnuc: float = 0.184          # shell_simul.f90:161
    scalepairing: float = 1.0
    fctn: float = 0.0              # celec cgnuc^2 / cdie
    kappa: float = 0.0
    qdeby: int = 0
    qsolv: bool = False
    epsolv: float = 0.0
    bonds: list = field(default_factory=list)    # ((i, j), d0), 1-based
    angles: list = field(default_factory=list)   # ((i, j, k), theta0)
    dihes: list = field(default_factory=list)    # ((i, j, k, l), phi0)
    stacks: list = field(default_factory=list)   # ((i, j), sigma)
    bps: list = field(default_factory=list)      # ((i, j), sigma, gc)
    exs: list = field(default_factory=list)      # ((i, j), sigma)
    qqs: list = field(default_factory=list)      # (i, j)
    solvs: list = field(default_factory=list)    # (i, j)
    apfor: list = field(default_factory=list)    # (site, (fx, fy, fz))
    contrans: list = field(default_factory=list)  # (site or 0, (kx, ky, kz), (x, y, z))
    contr_second: tuple = (0.0, 0.0, 0.0)        # anchor of the second strand's centre
    qunsplit: bool = False
    nsites1st: int = 0
    notrans: tuple = (None, None, None)          # NOTRAN centre per axis, None = off

    def counts(self) -> dict:
        return {"bond": len(self.bonds), "angle": len(self.angles), "dihe": len(self.dihes),
                "stack": len(self.stacks), "bp": len(self.bps), "ex": len(self.exs),
                "qq": len(self.qqs), "solv": len(self.solvs)}

    def struct(self):
        """(bromoc_nucleotides, arrays to keep alive during the call)."""
        keep = []

        def arr(v, dt, width=None):
            a = np.ascontiguousarray(np.asarray(v, dt).reshape(-1) if len(v) else
                                     np.zeros(1, dt))
            keep.append(a)
            return a

        def sites(lst, width):
            return arr([s for t in lst for s in (t[0] if width else t)], np.int32)

        b = sites(self.bonds, 2)
        a = sites(self.angles, 3)
        d = sites(self.dihes, 4)
        st = sites(self.stacks, 2)
        bp = sites(self.bps, 2)
        ex = sites(self.exs, 2)
        qq = arr([s for t in self.qqs for s in t], np.int32)
        sv = arr([s for t in self.solvs for s in t], np.int32)
        ct = self.contrans
        csn = arr([c[0] for c in ct], np.int32)
        kk = [arr([c[1][m] for c in ct], np.float64) for m in range(3)]
        anchors = [arr([c[2][m] for c in ct] + [self.contr_second[m]], np.float64)
                   for m in range(3)]
        s = abi.Nucleotides(
            epsnuc=self.epsnuc, scalepairing=self.scalepairing, fctn=self.fctn,
            kappa=self.kappa, qdeby=self.qdeby, qsolv=int(self.qsolv), epsolv=self.epsolv,
            nbond=len(self.bonds), sitebond=ptr(b, C.c_int32),
            distbond=ptr(arr([t[1] for t in self.bonds], np.float64), C.c_double),
            nangle=len(self.angles), siteangle=ptr(a, C.c_int32),
            valangle=ptr(arr([t[1] for t in self.angles], np.float64), C.c_double),
            ndihe=len(self.dihes), sitedihe=ptr(d, C.c_int32),
            valdihe=ptr(arr([t[1] for t in self.dihes], np.float64), C.c_double),
            nstack=len(self.stacks), sitestack=ptr(st, C.c_int32),
            sgstack=ptr(arr([t[1] for t in self.stacks], np.float64), C.c_double),
            nbp=len(self.bps), sitebp=ptr(bp, C.c_int32),
            sgbp=ptr(arr([t[1] for t in self.bps], np.float64), C.c_double),
            bpgc=ptr(arr([int(t[2]) for t in self.bps], np.uint8), C.c_uint8),
            nex=len(self.exs), siteex=ptr(ex, C.c_int32),
            sgex=ptr(arr([t[1] for t in self.exs], np.float64), C.c_double),
            nqq=len(self.qqs), siteqq=ptr(qq, C.c_int32),
            nsolv=len(self.solvs), siteslv=ptr(sv, C.c_int32),
            afn=len(self.apfor), sn=ptr(arr([t[0] for t in self.apfor], np.int32), C.c_int32),
            af=ptr(arr([t[1] for t in self.apfor], np.float64), C.c_double),
            ctn=len(ct), csn=ptr(csn, C.c_int32),
            kx=ptr(kk[0], C.c_double), ky=ptr(kk[1], C.c_double), kz=ptr(kk[2], C.c_double),
            contrx=ptr(anchors[0], C.c_double), contry=ptr(anchors[1], C.c_double),
            contrz=ptr(anchors[2], C.c_double),
            qunsplit=int(self.qunsplit), nsites1st=self.nsites1st)
        for a in range(3):
            s.qnotr[a] = int(self.notrans[a] is not None)
            s.notr[a] = float(self.notrans[a] or 0.0)
        return s, keep


def build_topology(names, strand, pos, *, epsnuc=0.184, fctn=0.0, kappa=0.0, qdeby=0,
                   qsolv=False, epsolv=0.0, scalepairing=1.0) -> Topology:
    """Term lists of a DNA described by site names ('Ab','Tb','Cb','Gb','S','P'),
    strand numbers and native coordinates [nsites, 3], by the reference's
    selection rules (module docstring).  Sites are 1-based in the lists."""
    names = [str(n) for n in names]
    strand = [int(s) for s in strand]
    pos = np.asarray(pos, np.float64)
    ns = len(names)
    t = Topology(epsnuc=epsnuc, fctn=fctn, kappa=kappa, qdeby=qdeby, qsolv=qsolv,
                 epsolv=epsolv, scalepairing=scalepairing)
    nm = [""] + names          # 1-based views
    sd = [0] + strand
    P = np.vstack([np.zeros(3), pos])
    bonded, angled = set(), set()

    def key(i, j):
        return (min(i, j), max(i, j))

    def dist(i, j):
        return float(np.linalg.norm(P[j] - P[i]))

    def bond(i, j):
        t.bonds.append(((i, j), dist(i, j)))
        bonded.add(key(i, j))

    def angle(i, j, k):  # j is the vertex
        t.angles.append(((i, j, k), angbond(P[i] - P[j], P[k] - P[j])))
        angled.update({key(i, j), key(i, k), key(j, k)})

    def dihe(i, j, k, l):
        t.dihes.append(((i, j, k, l), angdih(P[j] - P[i], P[k] - P[j], P[l] - P[k])))

    def isbase(i):
        return 1 <= i <= ns and nm[i] in BASES

    for i in range(1, ns):  # bonds.f90
        if isbase(i):
            bond(i, i + 1)
        elif nm[i] == "S":
            if sd[i] == sd[i + 1]:
                bond(i, i + 1)
        elif i + 2 <= ns and sd[i] == sd[i + 2]:
            bond(i, i + 2)
    for i in range(1, ns - 1):  # angles.f90
        if isbase(i):
            if sd[i] == sd[i + 2]:
                angle(i, i + 1, i + 2)
        elif nm[i] == "S":
            if i + 3 <= ns and sd[i] == sd[i + 3]:
                angle(i, i + 1, i + 3)
        else:
            n2, n3 = nm[i + 1], nm[i + 2]
            # Fortran precedence: Ab .or. Tb .or. Cb .or. (Gb .and. S)
            if n2 in ("Ab", "Tb", "Cb") or (n2 == "Gb" and n3 == "S"):
                angle(i, i + 2, i + 1)
            if i + 3 <= ns and sd[i] == sd[i + 3]:
                angle(i, i + 2, i + 3)
    for i in range(1, ns - 2):  # dihedral.f90
        if isbase(i):
            if i + 4 <= ns and sd[i] == sd[i + 4]:
                dihe(i, i + 1, i + 2, i + 4)
        elif nm[i] == "S":
            if sd[i] == sd[i + 3]:
                n2, n3 = nm[i + 1], nm[i + 2]
                # Fortran precedence: (P .and. Ab) .or. Tb .or. Cb .or. Gb
                if (n2 == "P" and n3 == "Ab") or n3 in ("Tb", "Cb", "Gb"):
                    dihe(i, i + 1, i + 3, i + 2)
            if i + 4 <= ns and sd[i] == sd[i + 4]:
                if nm[i + 1] == "P" and nm[i + 3] == "S" and nm[i + 4] == "P":
                    dihe(i, i + 1, i + 3, i + 4)
        else:
            if i + 5 <= ns and sd[i] == sd[i + 5]:
                if nm[i + 2] == "S" and nm[i + 3] == "P" and nm[i + 5] == "S":
                    dihe(i, i + 2, i + 3, i + 5)
    for i in range(2, ns + 1):  # go_qq.f90
        for j in range(1, i):
            if key(i, j) not in bonded:
                dij = dist(i, j)
                if sd[i] == sd[j] and dij - 9.0 < 0.0 and abs(dij - 9.0) >= 1e-4:
                    t.stacks.append(((i, j), dij))
                elif (nm[i], nm[j]) in PAIRS:
                    gc = nm[i] in ("Gb", "Cb")
                    t.bps.append(((i, j), 2.8694 if gc else 2.9002, gc))
                else:
                    both_bases = nm[i] not in ("P", "S") and nm[j] not in ("P", "S")
                    t.exs.append(((i, j), 1.0 if both_bases else 6.86))
                if key(i, j) not in angled and nm[i] == "P" and nm[j] == "P":
                    t.qqs.append((i, j))
            if qsolv and sd[i] != sd[j] and nm[i] == "S" and nm[j] == "S":
                t.solvs.append((i, j))
    return t
