"""ctypes mirror of include/bromoc_gpu.h.

The structs and the engine wrapper are shared by every library that exports
the bromoc ABI shape (`<prefix>_create`, `<prefix>_set_system`, ...).  The
product library is libbromoc_gpu.so with prefix ``bromoc_gpu``.
"""
from __future__ import annotations

import atexit
import ctypes as C
import weakref

import numpy as np

OK = 0
E_ARG, E_STATE, E_CUDA, E_CAPACITY, E_NOMEM, E_DEVICE = 1, 2, 3, 4, 5, 6

TERM_NAMES = ("ener", "eelec", "evdw", "esrpmf", "eefpot", "eqqmx", "evdwmx",
              "esrpmfmx", "eefpotmx", "ememb", "egsbpa", "egsbpb", "evdwgd",
              "erfpar", "ebond", "eang", "edihe", "estack", "ebp", "eex", "eqq",
              "esolv", "econ")
NTERMS = len(TERM_NAMES)

M_NONBOND, M_MEMB, M_PHIX, M_PHIV, M_RFPAR, M_BOND, M_MMIJ = 1, 2, 4, 8, 16, 32, 64
M_ALL = 0x7F
BOX, SPHERE, ECYL = 0, 1, 2
FP64, FP32 = 0, 1
DYN0, DYN1, DYN2, DYN3 = 0, 1, 2, 3

_d = C.POINTER(C.c_double)
_f = C.POINTER(C.c_float)
_i = C.POINTER(C.c_int32)
_u8 = C.POINTER(C.c_uint8)
_i8 = C.POINTER(C.c_int8)


class System(C.Structure):
    _fields_ = [("shape", C.c_int32), ("qcountion", C.c_int32),
                ("lx", C.c_double), ("ly", C.c_double), ("lz", C.c_double),
                ("cx", C.c_double), ("cy", C.c_double), ("cz", C.c_double),
                ("rsphe", C.c_double), ("temp", C.c_double),
                ("kbt", C.c_double), ("cdie", C.c_double),
                ("dt", C.c_double), ("bdmax", C.c_double)]


class Types(C.Structure):
    _fields_ = [("ntype", C.c_int32), ("nold", C.c_int32),
                ("nttyp", C.c_int32), ("ndna", C.c_int32),
                ("nwtype", _i), ("cg", _d), ("diffusion", _d)]


class Pairs(C.Structure):
    _fields_ = [("ntc", C.c_int32),
                ("qchr", _u8), ("qlj", _u8), ("qsrpmf", _u8), ("qefpot", _u8),
                ("fct", _d), ("epp4", _d), ("sgp2", _d),
                ("c0", _d), ("c1", _d), ("c2", _d), ("c3", _d), ("c4", _d),
                ("rth", C.c_double), ("srpx", C.c_double),
                ("srpk", C.c_double), ("srpy", C.c_double),
                ("cnt", C.c_int32), ("ep", _d), ("sc", _d), ("dm2", _d),
                ("dmi", _d), ("nxi", _i), ("res", C.c_double)]


class Sites(C.Structure):
    _fields_ = [("nsites", C.c_int32), ("typtyp", _i), ("charge", _d),
                ("stfree", _u8), ("phiv_map", _i)]


class Nucleotides(C.Structure):
    _fields_ = [("epsnuc", C.c_double), ("scalepairing", C.c_double),
                ("fctn", C.c_double), ("kappa", C.c_double),
                ("qdeby", C.c_int32), ("qsolv", C.c_int32), ("epsolv", C.c_double),
                ("nbond", C.c_int32), ("sitebond", _i), ("distbond", _d),
                ("nangle", C.c_int32), ("siteangle", _i), ("valangle", _d),
                ("ndihe", C.c_int32), ("sitedihe", _i), ("valdihe", _d),
                ("nstack", C.c_int32), ("sitestack", _i), ("sgstack", _d),
                ("nbp", C.c_int32), ("sitebp", _i), ("sgbp", _d), ("bpgc", _u8),
                ("nex", C.c_int32), ("siteex", _i), ("sgex", _d),
                ("nqq", C.c_int32), ("siteqq", _i),
                ("nsolv", C.c_int32), ("siteslv", _i),
                ("afn", C.c_int32), ("sn", _i), ("af", _d),
                ("ctn", C.c_int32), ("csn", _i),
                ("kx", _d), ("ky", _d), ("kz", _d),
                ("contrx", _d), ("contry", _d), ("contrz", _d),
                ("qunsplit", C.c_int32), ("nsites1st", C.c_int32),
                ("qnotr", C.c_int32 * 3), ("notr", C.c_double * 3)]


class Mmij(C.Structure):
    _fields_ = [("shape", C.c_int32), ("xnpol", C.c_int32), ("ynpol", C.c_int32),
                ("znpol", C.c_int32), ("lstpx", _i), ("lstpy", _i), ("lstpz", _i),
                ("rbxmin", C.c_double), ("rbxmax", C.c_double), ("rbymin", C.c_double),
                ("rbymax", C.c_double), ("rbzmin", C.c_double), ("rbzmax", C.c_double),
                ("rfscal", C.c_double), ("nmpol", C.c_int32), ("srdist", C.c_double),
                ("mmij", _d)]


class Grid(C.Structure):
    _fields_ = [("nclx", C.c_int32), ("ncly", C.c_int32), ("nclz", C.c_int32),
                ("dcel", C.c_double), ("xbcen", C.c_double),
                ("ybcen", C.c_double), ("zbcen", C.c_double)]


class PhivOpts(C.Structure):
    _fields_ = [("nmaps", C.c_int32), ("trilinear", C.c_int32),
                ("nmcden", C.c_int32), ("svdw", C.c_double),
                ("vzmin", C.c_double), ("vzmax", C.c_double),
                ("thold8", C.c_double), ("thold27", C.c_double),
                ("map_of_type", _i), ("scal", _d)]


class Membrane(C.Structure):
    _fields_ = [("qpore", C.c_int32), ("voltage", C.c_double),
                ("afact", C.c_double), ("ikappa", C.c_double),
                ("ceps", C.c_double), ("zmemb1", C.c_double),
                ("zmemb2", C.c_double), ("ampl1", _d), ("p1", _d),
                ("ampl2", _d), ("p2", _d), ("rcylinder", _d)]


class Diffusion(C.Structure):
    _fields_ = [("plength2", C.c_double), ("pcenter", C.c_double),
                ("ampl3", _d), ("p3", _d), ("nspline", C.c_int32),
                ("xs", _d), ("ys", _d), ("b", _d), ("c", _d), ("d", _d),
                ("diff0", C.c_double), ("ibeta", C.c_double),
                ("diffcutoff", C.c_double), ("fact0n1", C.c_double),
                ("fact0n2", C.c_double), ("qdnafree", C.c_int32)]


class Buffers(C.Structure):
    _fields_ = [("nbuffer", C.c_int32), ("ibfftyp", _i), ("avnum", _d),
                ("mu", _d), ("kb", _d), ("lzmin", _d), ("lzmax", _d),
                ("rmin", _d), ("rmax", _d), ("qbufferbias", _u8),
                ("nat", _i), ("ntotat", _i)]


def ptr(a, ctype):
    """ctypes pointer to a contiguous numpy array (None passes NULL)."""
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(ctype))


def declare(lib: C.CDLL, prefix: str) -> None:
    """Attach argtypes/restype for every ABI entry point under `prefix`."""
    vp = C.c_void_p
    sig = {
        "create": None,  # differs between the product and the oracle
        "destroy": [vp],
        "set_system": [vp, C.POINTER(System)],
        "set_types": [vp, C.POINTER(Types)],
        "set_pairs": [vp, C.POINTER(Pairs)],
        "set_sites": [vp, C.POINTER(Sites)],
        "set_nucleotides": [vp, C.POINTER(Nucleotides)],
        "set_mmij": [vp, C.POINTER(Mmij)],
        "set_phix": [vp, C.POINTER(Grid), _f],
        "set_phiv": [vp, C.POINTER(Grid), _i8, C.POINTER(PhivOpts)],
        "set_rfpar": [vp, C.POINTER(Grid), C.c_int32, _f, _f, C.c_double, _i],
        "set_membrane": [vp, C.POINTER(Membrane)],
        "set_diffusion": [vp, C.POINTER(Diffusion)],
        "set_countions": [vp, C.c_int32, _d],
        "set_periodic": [vp, C.c_int32, C.c_double],
        "set_buffers": [vp, C.POINTER(Buffers)],
        "set_particles": [vp, C.c_int32, C.c_int32, C.c_int32, _d, _d, _d, _i,
                          _i],
        "get_particles": [vp, _i, _d, _d, _d, _i, _i],
        "energy": [vp, C.c_uint32, C.c_int32, _d, _d, _d, _d, _i],
        "interact": [vp, C.c_uint32, C.c_double, C.c_double, C.c_double,
                     C.c_int32, C.c_int32, _d],
        "dynamics": [vp, C.c_int32, C.c_uint64, C.c_uint64],
        "bd_steps": [vp, C.c_uint32, C.c_int32, C.c_int32, C.c_uint64,
                     C.c_uint64, _d],
        "grand": [vp, C.c_uint32, C.c_int32, C.c_uint64, C.c_uint64, _d],
        "metropolis": [vp, C.c_uint32, C.c_int32, C.c_double, C.c_uint64, C.c_uint64, _i,
                       _d],
        "get_buffers": [vp, _i, _i, _i, _i],
        "get_countions": [vp, _i, _i],
        "get_dids": [vp, _d],
        "count": [vp],
        "get_ntotat": [vp, _i],
        "efpot_from_knots": [C.c_int32, _d, _d, C.c_double, C.c_int32, _d, _d,
                             _d, _d],
    }
    for name, args in sig.items():
        fn = getattr(lib, f"{prefix}_{name}")
        fn.restype = C.c_int
        if args is not None:
            fn.argtypes = args
    last = getattr(lib, f"{prefix}_last_error")
    last.restype = C.c_char_p
    last.argtypes = [vp]


class BromocError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"status {code}: {msg}")
        self.code = code


# Contexts must be destroyed before the CUDA runtime linked into the library
# tears itself down at process exit: Python's atexit hooks run first.
_LIVE = weakref.WeakSet()
# objects that borrow a context (replica batches, adjoint engines): closed
# before any context, since their teardown uses the context's stream
_DEPENDENTS = weakref.WeakSet()
_SHUTDOWN = False


def register_dependent(obj, owner=None) -> None:
    """obj borrows owner's context (its stream and tables).  The owner holds
    it strongly and closes it before destroying the context: a garbage
    collection may finalize the two in either order (and clears weak
    references first), so the order cannot rest on weak references.  obj
    removes itself from the owner when it closes (unregister_dependent)."""
    _DEPENDENTS.add(obj)
    if owner is not None:
        owner._dependents.add(obj)


def unregister_dependent(obj, owner) -> None:
    if owner is not None:
        owner._dependents.discard(obj)


def shutting_down() -> bool:
    return _SHUTDOWN


@atexit.register
def _close_all():
    global _SHUTDOWN
    for group in (_DEPENDENTS, _LIVE):
        for obj in list(group):
            try:
                obj.close()
            except Exception:
                pass
    _SHUTDOWN = True


class Engine:
    """One context of a library exporting the bromoc ABI.

    The methods mirror the reference's subroutine surface: energy() is
    ENERGY, interact() is INTERACT, dynamics() is DYNAMICSn, grand() is GRAND.
    """

    def __init__(self, lib: C.CDLL, prefix: str, handle: C.c_void_p,
                 capacity: int):
        self.lib, self.prefix, self.h, self.capacity = lib, prefix, handle, capacity
        self._keep = []  # arrays referenced by structs during a call
        self.ntot = 0
        self.nsites = 0
        self.nfix = 0
        self.nttyp = 0
        self.ntype = 0
        self.nold = 0
        self.ndna = 0
        self.nbuffer = 0
        self.cntpts = 0
        self._dependents = set()
        _LIVE.add(self)

    def _fn(self, name):
        return getattr(self.lib, f"{self.prefix}_{name}")

    def _chk(self, rc: int, what: str):
        if rc != OK:
            msg = self._fn("last_error")(self.h)
            raise BromocError(rc, f"{self.prefix}_{what}: "
                              f"{msg.decode() if msg else ''}")

    def close(self):
        if self.h:
            for dep in list(getattr(self, "_dependents", ())):
                dep.close()
            self._fn("destroy")(self.h)
            self.h = None

    def __del__(self):
        if _SHUTDOWN:
            return
        try:
            self.close()
        except Exception:
            pass

    # -- module state -----------------------------------------------------
    def load(self, spec) -> "Engine":
        """Push a SystemSpec (bromoc_gb300.deck) into the context."""
        spec.push(self)
        return self

    def call(self, name, *args):
        self._chk(self._fn(name)(self.h, *args), name)

    def set_nucleotides(self, topo) -> None:
        """DNA bonded and Go-like term lists (a bromoc_gb300.nucleotides.Topology,
        or None to clear them)."""
        if topo is None:
            self._chk(self._fn("set_nucleotides")(self.h, None), "set_nucleotides")
            return
        st, keep = topo.struct()
        self._keep = keep
        self._chk(self._fn("set_nucleotides")(self.h, C.byref(st)), "set_nucleotides")
        self._keep = []

    def set_mmij(self, mm) -> None:
        """MMIJ reaction field from a dict (shape, npol + lstp + region + rfscal
        for RECTBOX, or nmpol + srdist for SPHERE, and mmij), or None."""
        if mm is None:
            self._chk(self._fn("set_mmij")(self.h, None), "set_mmij")
            return
        keep = []

        def arr(v, dt):
            a = np.ascontiguousarray(v, dt)
            keep.append(a)
            return a

        m = arr(np.asarray(mm["mmij"], np.float64).reshape(-1), np.float64)
        st = Mmij(shape=mm["shape"], mmij=ptr(m, C.c_double), rfscal=mm.get("rfscal", 1.0))
        if mm["shape"] == BOX:
            st.xnpol, st.ynpol, st.znpol = mm["npol"]
            lx, ly, lz = (arr(v, np.int32) for v in mm["lstp"])
            st.lstpx, st.lstpy, st.lstpz = (ptr(v, C.c_int32) for v in (lx, ly, lz))
            (st.rbxmin, st.rbxmax), (st.rbymin, st.rbymax), (st.rbzmin, st.rbzmax) = mm["region"]
        else:
            st.nmpol, st.srdist = mm["nmpol"], mm["srdist"]
        self._chk(self._fn("set_mmij")(self.h, C.byref(st)), "set_mmij")

    # -- particles ------------------------------------------------------------
    def set_particles(self, x, y, z, typei, nsites=0, nfix=0, ibuffer=None):
        x = np.ascontiguousarray(x, np.float64)
        y = np.ascontiguousarray(y, np.float64)
        z = np.ascontiguousarray(z, np.float64)
        typei = np.ascontiguousarray(typei, np.int32)
        ib = None if ibuffer is None else np.ascontiguousarray(ibuffer, np.int32)
        n = len(x)
        self._chk(self._fn("set_particles")(
            self.h, n, nsites, nfix, ptr(x, C.c_double), ptr(y, C.c_double),
            ptr(z, C.c_double), ptr(typei, C.c_int32), ptr(ib, C.c_int32)),
            "set_particles")
        self.ntot, self.nsites, self.nfix = n, nsites, nfix

    def get_particles(self):
        n = C.c_int32(0)
        cap = self.capacity
        x, y, z = (np.zeros(cap) for _ in range(3))
        t = np.zeros(cap, np.int32)
        ib = np.zeros(cap, np.int32)
        self._chk(self._fn("get_particles")(
            self.h, C.byref(n), ptr(x, C.c_double), ptr(y, C.c_double),
            ptr(z, C.c_double), ptr(t, C.c_int32), ptr(ib, C.c_int32)),
            "get_particles")
        k = n.value
        self.ntot = k
        return x[:k], y[:k], z[:k], t[:k], ib[:k]

    def live_ntot(self) -> int:
        """Current particle count (GCMC changes it on the device)."""
        n = C.c_int32(0)
        self._chk(self._fn("get_particles")(self.h, C.byref(n), None, None,
                                            None, None, None), "get_particles")
        self.ntot = n.value
        return n.value

    # -- hot path -----------------------------------------------------------
    def energy(self, terms=M_ALL, forces=True):
        # capacity-sized outputs: the live ntot may exceed the last upload
        cap = self.capacity
        fx, fy, fz = np.zeros(cap), np.zeros(cap), np.zeros(cap)
        e = np.zeros(NTERMS)
        warn = np.zeros(max(self.nttyp, 1), np.int32)
        self._chk(self._fn("energy")(
            self.h, terms, 1 if forces else 0, ptr(fx, C.c_double),
            ptr(fy, C.c_double), ptr(fz, C.c_double), ptr(e, C.c_double),
            ptr(warn, C.c_int32)), "energy")
        n = self.live_ntot()
        terms_d = dict(zip(TERM_NAMES, e.tolist()))
        f = np.stack([fx[:n], fy[:n], fz[:n]], 1) if forces else None
        return terms_d, f, warn

    def interact(self, xj, yj, zj, jtype, j, terms=M_ALL):
        d = C.c_double(0.0)
        self._chk(self._fn("interact")(self.h, terms, xj, yj, zj, jtype, j,
                                       C.byref(d)), "interact")
        return d.value

    def dynamics(self, variant, seed, step):
        self._chk(self._fn("dynamics")(self.h, variant, seed, step), "dynamics")

    def bd_steps(self, nsteps, seed, step0=0, variant=DYN0, terms=M_ALL,
                 energies=True):
        """nsteps BD steps; with energies, the terms at the last step's
        starting configuration (else None, and no energy is formed)."""
        e = np.zeros(NTERMS)
        self._chk(self._fn("bd_steps")(self.h, terms, variant, nsteps, seed,
                                       step0, ptr(e, C.c_double) if energies else None),
                  "bd_steps")
        return dict(zip(TERM_NAMES, e.tolist())) if energies else None

    def grand(self, ngcmc, seed, cycle, terms=M_ALL, dener=True):
        """ngcmc GCMC attempts; with dener, waits for them and returns the
        sum of the attempts' energy changes (else returns None at once)."""
        d = C.c_double(0.0)
        self._chk(self._fn("grand")(self.h, terms, ngcmc, seed, cycle,
                                    C.byref(d) if dener else None), "grand")
        return d.value if dener else None

    def count(self) -> None:
        """COUNT (count.f90): buffer membership, nat, ntotat from positions."""
        self._chk(self._fn("count")(self.h), "count")

    def ntotat(self):
        v = np.zeros(max(self.nbuffer, 1), np.int32)
        self._chk(self._fn("get_ntotat")(self.h, ptr(v, C.c_int32)), "get_ntotat")
        return v[:self.nbuffer]

    def metropolis(self, nmcm, mcmax, seed, cycle, terms=M_ALL):
        """METROPOLIS: nmcm moves -> (accepted moves, summed energy change)."""
        na = C.c_int32(0)
        d = C.c_double(0.0)
        self._chk(self._fn("metropolis")(self.h, terms, nmcm, mcmax, seed, cycle,
                                         C.byref(na), C.byref(d)), "metropolis")
        return na.value, d.value

    def get_buffers(self):
        nb = self.nbuffer
        nat, nin, nrm = (np.zeros(nb, np.int32) for _ in range(3))
        prob = np.zeros(nb * (self.capacity + 1), np.int32)
        self._chk(self._fn("get_buffers")(self.h, ptr(nat, C.c_int32),
                                          ptr(nin, C.c_int32),
                                          ptr(nrm, C.c_int32),
                                          ptr(prob, C.c_int32)), "get_buffers")
        return nat, nin, nrm, prob.reshape(nb, self.capacity + 1)

    def get_countions(self):
        n = max((self.ntype - self.nold) * self.cntpts, 1)
        nf, nb = np.zeros(n, np.int32), np.zeros(n, np.int32)
        self._chk(self._fn("get_countions")(self.h, ptr(nf, C.c_int32),
                                            ptr(nb, C.c_int32)),
                  "get_countions")
        return nf, nb

    def get_dids(self):
        d = np.zeros(5 * max(self.capacity, 1))
        self._chk(self._fn("get_dids")(self.h, ptr(d, C.c_double)), "get_dids")
        return d.reshape(-1, 5)[: self.live_ntot()]

    def efpot_from_knots(self, xx, yy, fct, qchr):
        return efpot_from_knots(self.lib, self.prefix, xx, yy, fct, qchr)


def efpot_from_knots(lib, prefix, xx, yy, fct, qchr):
    """splinepot (splinepot.f90:19-96) for one pair -> (ep[n,3], sc3, dm2, dmi)."""
    xx = np.ascontiguousarray(xx, np.float64)
    yy = np.ascontiguousarray(yy, np.float64)
    n = len(xx)
    ep = np.zeros((n, 3))
    sc3 = np.zeros(3)
    dm2 = np.zeros(2)
    dmi = np.zeros(1)
    rc = getattr(lib, f"{prefix}_efpot_from_knots")(
        n, ptr(xx, C.c_double), ptr(yy, C.c_double), float(fct), int(qchr),
        ptr(ep, C.c_double), ptr(sc3, C.c_double), ptr(dm2, C.c_double),
        ptr(dmi, C.c_double))
    if rc != OK:
        raise BromocError(rc, f"{prefix}_efpot_from_knots")
    return ep, sc3, dm2, float(dmi[0])
