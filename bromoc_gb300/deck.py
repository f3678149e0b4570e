"""Deck-time setup: the parameter derivations of cg-gcmc-bd's input deck.

`SystemSpec` collects what the reference's keyword interpreter leaves in its
modules (shell_simul.f90) and pushes it through the C ABI.  Each builder
method names the deck section it mirrors.  Physical constants are those of
constamod.f90:71-85.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import abi
from .abi import ptr

# constamod.f90:71-85 (2010 CODATA as in the reference)
PI = 3.14159265358979323846264338327950288419716939937510
KBOLTZ = 1.380648813e-23
ANGSTROM = 1e-10
LITER = 1e-3
AVOGADRO = 6.0221412927e23
KCAL = 4184.0
KCALMOL = KCAL / AVOGADRO
COULOMB = 1.60217656535e-19
EPERMIT = 8.854187817620e-12
CELEC = COULOMB ** 2 / (4.0 * PI * EPERMIT * KCALMOL * ANGSTROM)
CONST_KAPPA = EPERMIT * KBOLTZ * 1.0e17 / (2.0 * AVOGADRO * COULOMB ** 2)


def nindex(itype: int, jtype: int, ndna: int, nion: int) -> int:
    """Packed pair index of two combined types (nindex.f90:19-35)."""
    if itype > jtype:
        maxi, mini = itype - ndna, jtype
    else:
        maxi, mini = jtype - ndna, itype
    if mini > ndna:
        return maxi * (maxi - 1) // 2 + mini - ndna + ndna * nion
    return (mini - 1) * nion + maxi


@dataclass
class SystemSpec:
    # SYSTEM
    shape: int = abi.BOX
    lx: float = 0.0
    ly: float = 0.0
    lz: float = 0.0
    cx: float = 0.0
    cy: float = 0.0
    cz: float = 0.0
    rsphe: float = 0.0
    temp: float = 300.0
    cdie: float = 80.0
    ionic: float = 0.0
    volt: float = 0.0
    dt: float = 0.02
    bdmax: float = 1.0
    qcountion: bool = False
    # types: combined types = DNA site types (1..ndna) + ion types
    site_type_names: list = field(default_factory=list)
    ion_names: list = field(default_factory=list)
    ion_cg: list = field(default_factory=list)
    ion_diff: list = field(default_factory=list)
    cgnuc: float = -1.0
    # per-combined-type LJ singles (LJSIN) and per-pair overrides (LJPAR)
    lj_eps: dict = field(default_factory=dict)
    lj_sigma: dict = field(default_factory=dict)
    lj_pair: dict = field(default_factory=dict)   # (a, b) -> (eps, sigma)
    srpmf: dict = field(default_factory=dict)     # (a, b) -> (c0..c4)
    srpmf_rth: float | None = None
    # extension mode (no counterpart in the reference): minimum-image periodic
    # box with a plain cutoff on ion pairs (Angstrom); None = hard walls
    periodic_rcut: float | None = None
    efpot_knots: dict = field(default_factory=dict)  # (a, b) -> (r[], U[])
    efpot_res: float = 0.1
    # sites
    site_types: np.ndarray | None = None    # [nsites] combined type 1..ndna
    site_free: np.ndarray | None = None
    nucl: object = None           # nucleotides.Topology: bonded and Go-like terms
    mmij: dict | None = None      # MMIJ reaction field (abi.Engine.set_mmij)
    # maps
    phix: tuple | None = None     # (grid dict, float32[n])
    phiv: tuple | None = None     # (grid dict, int8[nmaps*n], opts dict)
    rfpar: tuple | None = None    # (grid dict, gsrfen, greff, reffac, map)
    membrane: dict | None = None
    diffusion: dict | None = None
    zcont: np.ndarray | None = None
    buffers: list = field(default_factory=list)
    precision: int = abi.FP64
    # particles
    x: np.ndarray | None = None
    y: np.ndarray | None = None
    z: np.ndarray | None = None
    typei: np.ndarray | None = None
    ibuffer: np.ndarray | None = None
    nfix: int = 0

    # ---- derived -----------------------------------------------------------
    @property
    def ndna(self) -> int:
        return len(self.site_type_names)

    @property
    def nold(self) -> int:
        return self.ndna

    @property
    def nion(self) -> int:
        return len(self.ion_names)

    @property
    def ntype(self) -> int:
        return self.nold + self.nion

    @property
    def nttyp(self) -> int:
        return self.ndna + self.nion

    @property
    def ntc(self) -> int:
        return (self.nttyp + self.ndna + 1) * self.nion // 2

    @property
    def nsites(self) -> int:
        return 0 if self.site_types is None else len(self.site_types)

    @property
    def ntot(self) -> int:
        return 0 if self.x is None else len(self.x)

    @property
    def kbt(self) -> float:
        return KBOLTZ * self.temp / KCALMOL  # shell_simul.f90:865

    def type_names(self):
        return list(self.site_type_names) + list(self.ion_names)

    def ctype(self, name: str) -> int:
        """1-based combined type of a name (atnam2)."""
        return self.type_names().index(name) + 1

    def ion_type(self, name: str) -> int:
        """1-based ion type (typei value) of an ion name (atnam)."""
        return self.nold + self.ion_names.index(name) + 1

    def nwtype(self) -> np.ndarray:
        nw = np.zeros(self.ntype, np.int32)
        for k in range(self.nion):
            nw[self.nold + k] = self.ndna + k + 1  # reasig.f90:303-307
        return nw

    def cg2(self) -> np.ndarray:
        """Charge per combined type (shell_simul.f90:601-607)."""
        c = np.zeros(self.nttyp)
        if self.ndna > 1:
            c[1] = self.cgnuc  # type 2 is 'P'
        for k, q in enumerate(self.ion_cg):
            c[self.ndna + k] = q
        return c

    def pair_tables(self):
        """fct/LJ/SRPMF/EFPOT tables by packed pair index (1-based)."""
        ntc, ndna, nion, nt = self.ntc, self.ndna, self.nion, self.nttyp
        names = self.type_names()
        qchr = np.zeros(ntc, np.uint8)
        qlj = np.zeros(ntc, np.uint8)
        qsr = np.zeros(ntc, np.uint8)
        qef = np.zeros(ntc, np.uint8)
        fct = np.zeros(ntc)
        epp4 = np.zeros(ntc)
        sgp2 = np.zeros(ntc)
        cc = np.zeros((5, ntc))
        cg2 = self.cg2()
        for i in range(1, nt + 1):
            for j in range(i, nt + 1):
                if j <= ndna:
                    continue
                k = nindex(i, j, ndna, nion) - 1
                # PARTICLES / SYSTEM: shell_simul.f90:610-622, 920-934
                if cg2[i - 1] != 0.0 and cg2[j - 1] != 0.0:
                    fct[k] = CELEC * cg2[i - 1] * cg2[j - 1] / self.cdie
                    qchr[k] = 1
                # LJSIN: shell_simul.f90:1118-1131
                ei, si = self.lj_eps.get(names[i - 1], 0.0), self.lj_sigma.get(names[i - 1], 0.0)
                ej, sj = self.lj_eps.get(names[j - 1], 0.0), self.lj_sigma.get(names[j - 1], 0.0)
                if ei > 0 and si > 0 and ej > 0 and sj > 0:
                    epp4[k] = 4.0 * math.sqrt(ei * ej)
                    sgp2[k] = (0.5 * (si + sj)) ** 2
                    qlj[k] = 1
                # LJPAR overrides: shell_simul.f90:1171-1194
                lp = self.lj_pair.get((names[i - 1], names[j - 1])) or \
                    self.lj_pair.get((names[j - 1], names[i - 1]))
                if lp is not None and lp[0] > 0 and lp[1] > 0:
                    epp4[k] = 4.0 * lp[0]
                    sgp2[k] = lp[1] ** 2
                    qlj[k] = 1
                # SRPMF: shell_simul.f90:1671-1767 (c2 stored inverted)
                sp = self.srpmf.get((names[i - 1], names[j - 1])) or \
                    self.srpmf.get((names[j - 1], names[i - 1]))
                if sp is not None and sp[2] != 0.0:
                    cc[:, k] = sp
                    cc[2, k] = 1.0 / sp[2]
                    qsr[k] = 1
        rth_in = 8.0 if self.srpmf_rth is None else self.srpmf_rth
        srpx = rth_in - 0.5
        srpk = 6.90775527898 / 0.5
        srpy = 0.001
        rth = rth_in ** 2
        # EFPOT read: shell_simul.f90:1810-1839, 1861-1867
        sc = np.zeros((ntc, 3))
        dm2 = np.zeros((ntc, 2))
        dmi = np.zeros(ntc)
        nxi = np.zeros(ntc, np.int32)
        eps_list = []
        cnt = 0
        for (a, b), (r, u) in self.efpot_knots.items():
            k = nindex(self.ctype(a), self.ctype(b), ndna, nion) - 1
            qef[k] = 1
            ep, sc3, d2, d1 = self.build_efpot(r, u, fct[k], bool(qchr[k]))
            nxi[k] = cnt + 1
            cnt += len(r)
            eps_list.append(ep)
            sc[k], dm2[k], dmi[k] = sc3, d2, d1
        ep_all = np.concatenate(eps_list) if eps_list else np.zeros((1, 3))
        return dict(ntc=ntc, qchr=qchr, qlj=qlj, qsrpmf=qsr, qefpot=qef,
                    fct=fct, epp4=epp4, sgp2=sgp2, c=cc, rth=rth, srpx=srpx,
                    srpk=srpk, srpy=srpy, cnt=max(cnt, 1),
                    ep=np.ascontiguousarray(ep_all), sc=sc, dm2=dm2, dmi=dmi,
                    nxi=nxi, res=self.efpot_res)

    # effective-potential table builder; push() sets it to the target
    # engine's own (splinepot.f90 semantics)
    _builder = None

    def build_efpot(self, r, u, fct, qchr):
        if self._builder is None:
            from . import _lib
            return _lib.efpot_from_knots(r, u, fct, qchr)
        return self._builder(r, u, fct, qchr)

    def system_struct(self) -> "abi.System":
        """The SYSTEM + SIMUL scalars as the C struct (bromoc_system)."""
        return abi.System(shape=self.shape, qcountion=int(self.qcountion),
                          lx=self.lx, ly=self.ly, lz=self.lz, cx=self.cx,
                          cy=self.cy, cz=self.cz, rsphe=self.rsphe,
                          temp=self.temp, kbt=self.kbt, cdie=self.cdie,
                          dt=self.dt, bdmax=self.bdmax)

    # ---- push into an engine ------------------------------------------------
    def push(self, eng: "abi.Engine"):
        keep = []

        def k(a):
            keep.append(a)
            return a

        nt, ntype = self.nttyp, self.ntype
        eng.nttyp, eng.ntype, eng.nold = nt, ntype, self.nold
        eng.ndna = self.ndna
        self._builder = eng.efpot_from_knots
        sysd = self.system_struct()
        eng.call("set_system", C.byref(sysd))
        if self.periodic_rcut is not None:
            eng.call("set_periodic", 1, float(self.periodic_rcut))
        cg = np.zeros(ntype)
        dif = np.zeros(ntype)
        for i in range(self.nion):
            cg[self.nold + i] = self.ion_cg[i]
            dif[self.nold + i] = self.ion_diff[i]
        nw = k(self.nwtype())
        cg, dif = k(cg), k(dif)
        t = abi.Types(ntype=ntype, nold=self.nold, nttyp=nt, ndna=self.ndna,
                      nwtype=ptr(nw, C.c_int32), cg=ptr(cg, C.c_double),
                      diffusion=ptr(dif, C.c_double))
        eng.call("set_types", C.byref(t))
        pt = self.pair_tables()
        for key in ("qchr", "qlj", "qsrpmf", "qefpot", "fct", "epp4", "sgp2",
                    "ep", "sc", "dm2", "dmi", "nxi"):
            pt[key] = k(np.ascontiguousarray(pt[key]))
        cc = [k(np.ascontiguousarray(pt["c"][m])) for m in range(5)]
        p = abi.Pairs(ntc=pt["ntc"], qchr=ptr(pt["qchr"], C.c_uint8),
                      qlj=ptr(pt["qlj"], C.c_uint8),
                      qsrpmf=ptr(pt["qsrpmf"], C.c_uint8),
                      qefpot=ptr(pt["qefpot"], C.c_uint8),
                      fct=ptr(pt["fct"], C.c_double),
                      epp4=ptr(pt["epp4"], C.c_double),
                      sgp2=ptr(pt["sgp2"], C.c_double),
                      c0=ptr(cc[0], C.c_double), c1=ptr(cc[1], C.c_double),
                      c2=ptr(cc[2], C.c_double), c3=ptr(cc[3], C.c_double),
                      c4=ptr(cc[4], C.c_double), rth=pt["rth"],
                      srpx=pt["srpx"], srpk=pt["srpk"], srpy=pt["srpy"],
                      cnt=pt["cnt"], ep=ptr(pt["ep"], C.c_double),
                      sc=ptr(pt["sc"], C.c_double),
                      dm2=ptr(pt["dm2"], C.c_double),
                      dmi=ptr(pt["dmi"], C.c_double),
                      nxi=ptr(pt["nxi"], C.c_int32), res=pt["res"])
        eng.call("set_pairs", C.byref(p))
        ns = self.nsites
        st = k(np.ascontiguousarray(self.site_types if ns else np.zeros(1), np.int32))
        sq = np.zeros(max(ns, 1))
        if ns:
            sq[:ns] = np.where(st == 2, self.cgnuc, 0.0)  # 'P' sites carry cgnuc
        sq = k(sq)
        sf = k(np.ascontiguousarray(self.site_free if ns and self.site_free is not None
                                    else np.ones(max(ns, 1)), np.uint8))
        sites = abi.Sites(nsites=ns, typtyp=ptr(st, C.c_int32),
                          charge=ptr(sq, C.c_double), stfree=ptr(sf, C.c_uint8),
                          phiv_map=None)
        eng.call("set_sites", C.byref(sites))
        if ns and self.nucl is not None:
            eng.set_nucleotides(self.nucl)
        if self.mmij is not None:
            eng.set_mmij(self.mmij)
        if self.phix is not None:
            g, data = self.phix
            data = k(np.ascontiguousarray(data, np.float32))
            eng.call("set_phix", C.byref(abi.Grid(**g)), ptr(data, C.c_float))
        if self.phiv is not None:
            g, data, o = self.phiv
            data = k(np.ascontiguousarray(data, np.int8))
            mot = o.get("map_of_type")
            mot = None if mot is None else k(np.ascontiguousarray(mot, np.int32))
            scal = o.get("scal")
            scal = None if scal is None else k(np.ascontiguousarray(scal, np.float64))
            opts = abi.PhivOpts(nmaps=o.get("nmaps", 1),
                                trilinear=int(o.get("trilinear", True)),
                                nmcden=int(o.get("nmcden", False)),
                                svdw=o["svdw"], vzmin=o["vzmin"],
                                vzmax=o["vzmax"], thold8=o.get("thold8", 8.0),
                                thold27=o.get("thold27", 27.0),
                                map_of_type=ptr(mot, C.c_int32),
                                scal=ptr(scal, C.c_double))
            eng.call("set_phiv", C.byref(abi.Grid(**g)), ptr(data, C.c_int8),
                     C.byref(opts))
        if self.rfpar is not None:
            g, gs, gr, reffac, mot = self.rfpar
            gs = k(np.ascontiguousarray(gs, np.float32))
            gr = k(np.ascontiguousarray(gr, np.float32))
            nmaps = 1 if mot is None else int(np.max(mot)) + 1
            mot = None if mot is None else k(np.ascontiguousarray(mot, np.int32))
            eng.call("set_rfpar", C.byref(abi.Grid(**g)), nmaps,
                     ptr(gs, C.c_float), ptr(gr, C.c_float), float(reffac),
                     ptr(mot, C.c_int32))
        if self.membrane is not None:
            m = self.membrane_params()
            arrs = {n: k(np.ascontiguousarray(m[n], np.float64))
                    for n in ("ampl1", "p1", "ampl2", "p2", "rcylinder")}
            mm = abi.Membrane(qpore=int(m["qpore"]), voltage=m["voltage"],
                              afact=m["afact"], ikappa=m["ikappa"],
                              ceps=m["ceps"], zmemb1=m["zmemb1"],
                              zmemb2=m["zmemb2"],
                              **{n: ptr(a, C.c_double) for n, a in arrs.items()})
            eng.call("set_membrane", C.byref(mm))
        d = self.diffusion or {}
        a3 = k(np.ascontiguousarray(d.get("ampl3", np.zeros(ntype)), np.float64))
        p3 = k(np.ascontiguousarray(d.get("p3", np.ones(ntype)), np.float64))
        sp = d.get("spline")
        if sp is not None:
            sp = [k(np.ascontiguousarray(v, np.float64)) for v in sp]
        diffnuc = d.get("diffnuc", 0.1)
        dd = abi.Diffusion(plength2=d.get("plength2", 0.0),
                           pcenter=d.get("pcenter", 0.0),
                           ampl3=ptr(a3, C.c_double), p3=ptr(p3, C.c_double),
                           nspline=0 if sp is None else len(sp[0]),
                           xs=None if sp is None else ptr(sp[0], C.c_double),
                           ys=None if sp is None else ptr(sp[1], C.c_double),
                           b=None if sp is None else ptr(sp[2], C.c_double),
                           c=None if sp is None else ptr(sp[3], C.c_double),
                           d=None if sp is None else ptr(sp[4], C.c_double),
                           diff0=d.get("diff0", 0.101),
                           ibeta=1.0 / d.get("beta", 2.93),
                           diffcutoff=d.get("diffcutoff", 0.0),
                           fact0n1=diffnuc * self.kbt * self.dt,
                           fact0n2=math.sqrt(2.0 * self.dt * diffnuc),
                           qdnafree=int(d.get("dnafree", False)))
        eng.call("set_diffusion", C.byref(dd))
        if self.zcont is not None:
            zc = k(np.ascontiguousarray(self.zcont, np.float64))
            eng.call("set_countions", len(zc), ptr(zc, C.c_double))
            eng.cntpts = len(zc)
        if self.buffers:
            bf = self.buffer_params()
            arrs = {n: k(np.ascontiguousarray(v)) for n, v in bf.items()}
            bb = abi.Buffers(nbuffer=len(self.buffers),
                             ibfftyp=ptr(arrs["ibfftyp"], C.c_int32),
                             avnum=ptr(arrs["avnum"], C.c_double),
                             mu=ptr(arrs["mu"], C.c_double),
                             kb=ptr(arrs["kb"], C.c_double),
                             lzmin=ptr(arrs["lzmin"], C.c_double),
                             lzmax=ptr(arrs["lzmax"], C.c_double),
                             rmin=ptr(arrs["rmin"], C.c_double),
                             rmax=ptr(arrs["rmax"], C.c_double),
                             qbufferbias=ptr(arrs["qbufferbias"], C.c_uint8),
                             nat=ptr(arrs["nat"], C.c_int32),
                             ntotat=ptr(arrs["ntotat"], C.c_int32))
            eng.call("set_buffers", C.byref(bb))
            eng.nbuffer = len(self.buffers)
        if self.x is not None:
            eng.set_particles(self.x, self.y, self.z, self.typei, self.nsites,
                              self.nfix, self.ibuffer)
        eng._keep = keep

    # ---- MEMBRANE: shell_simul.f90:1563-1669 ------------------------------
    def membrane_params(self):
        m = self.membrane
        nt = self.nttyp
        thick2 = 0.5 * m["thick"]
        zmemb = m.get("zmemb", 0.0)
        epsm = m.get("epsm", 2.0)
        voltage = self.volt * COULOMB / KCALMOL  # shell_simul.f90:852
        kappa = math.sqrt(CONST_KAPPA * self.cdie * self.temp / self.ionic)
        ikappa = 1.0 / kappa
        afact = epsm * voltage / (2.0 * epsm + self.cdie * ikappa * m["thick"])
        ampl1 = np.zeros(nt)
        p1 = np.ones((nt, 2))
        ampl2 = np.zeros(nt)
        p2 = np.ones((nt, 2))
        rcyl = np.ones(nt)
        for name, v in m["types"].items():
            t = self.ctype(name) - 1
            ampl1[t] = v.get("amplmemb", 0.0)
            p1[t] = (v.get("pmemb", 1.0), 1.0 / v.get("pmemb", 1.0))
            if m.get("pore"):
                ampl2[t] = v.get("amplpore", 0.0)
                p2[t] = (v.get("ppore", 1.0), 1.0 / v.get("ppore", 1.0))
                rcyl[t] = v.get("radi", 1.0)
        return dict(qpore=bool(m.get("pore")), voltage=voltage, afact=afact,
                    ikappa=ikappa, ceps=self.cdie / epsm,
                    zmemb1=-thick2 + zmemb, zmemb2=thick2 + zmemb, ampl1=ampl1,
                    p1=p1.reshape(-1), ampl2=ampl2, p2=p2.reshape(-1),
                    rcylinder=rcyl)

    # ---- BUFFERS: shell_simul.f90:949-1083 --------------------------------
    def buffer_params(self):
        nb = len(self.buffers)
        out = {n: np.zeros(nb) for n in ("avnum", "mu", "kb", "lzmin", "lzmax",
                                          "rmin", "rmax")}
        out["ibfftyp"] = np.zeros(nb, np.int32)
        out["qbufferbias"] = np.zeros(nb, np.uint8)
        out["nat"] = np.zeros(nb, np.int32)
        out["ntotat"] = np.zeros(nb, np.int32)
        lz2m, lz2p = self.cz - 0.5 * self.lz, self.cz + 0.5 * self.lz
        for ib, b in enumerate(self.buffers):
            it = self.ion_type(b["ion"])
            out["ibfftyp"][ib] = it
            lzmin, lzmax = b.get("lzmin", lz2m), b.get("lzmax", lz2p)
            out["lzmin"][ib], out["lzmax"][ib] = lzmin, lzmax
            if self.shape == abi.ECYL:
                vol = 0.25 * PI * self.lx * self.ly * (lzmax - lzmin)
            elif self.shape == abi.BOX:
                vol = self.lx * self.ly * (lzmax - lzmin)
            else:
                raise NotImplementedError("spherical buffers")
            dens = b.get("conc", 0.0) * (AVOGADRO / LITER) * ANGSTROM ** 3
            avnum = b.get("aver", dens * vol)
            out["avnum"][ib] = avnum
            q = self.ion_cg[self.ion_names.index(b["ion"])]
            out["mu"][ib] = b.get("mu", 0.0) + q * b.get("volt", 0.0) * COULOMB / KCALMOL
            out["kb"][ib] = b.get("kb", 0.0)
            out["qbufferbias"][ib] = int(b.get("bufferbias", False))
            out["nat"][ib] = b.get("nat", 0)
            # simul1.f90:332-336: ntotat starts from nint(avnum)
            out["ntotat"][ib] = int(math.floor(avnum + 0.5))
        return out

    def count(self):
        """COUNT (count.f90:19-95) for box/ecyl systems: ibuffer, nat, sign."""
        n = self.ntot
        ib = np.zeros(n, np.int32)
        nat = [0] * len(self.buffers)
        bp = self.buffer_params() if self.buffers else None
        for i in range(self.nsites + self.nfix, n):
            it = abs(int(self.typei[i]))
            for b in range(len(self.buffers)):
                if it == bp["ibfftyp"][b] and bp["lzmin"][b] <= self.z[i] <= bp["lzmax"][b]:
                    ib[i] = b + 1
                    nat[b] += 1
                    self.typei[i] = -it if self.z[i] < self.cz else it
                    break
        self.ibuffer = ib
        for b, v in enumerate(nat):
            self.buffers[b]["nat"] = v
        return nat
