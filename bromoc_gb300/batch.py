"""Python face of the replica-batch C ABI (bromoc_batch_* in
include/bromoc_gpu.h): many independent ion systems sharing one FP32
prototype context's types, pair laws and grid maps."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib, abi


class Batch:
    def __init__(self, proto: abi.Engine, capacities):
        self.lib = _lib.load()
        self.proto = proto  # keeps the prototype alive as long as the batch
        caps = np.ascontiguousarray(capacities, dtype=np.int32)
        self.nrep = len(caps)
        h = C.c_void_p()
        rc = self.lib.bromoc_batch_create(
            proto.h, self.nrep, caps.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(h))
        if rc != abi.OK:
            raise abi.BromocError(rc, self.lib.bromoc_gpu_last_error(proto.h).decode())
        self.h = h
        abi.register_dependent(self, proto)

    def _chk(self, rc, what):
        if rc != abi.OK:
            raise abi.BromocError(
                rc, f"{what}: {self.lib.bromoc_batch_last_error(self.h).decode()}")

    def close(self):
        if getattr(self, "h", None):
            self.lib.bromoc_batch_destroy(self.h)
            self.h = None
            abi.unregister_dependent(self, self.proto)

    def __del__(self):
        if abi.shutting_down():
            return
        try:
            self.close()
        except Exception:
            pass

    def set_systems(self, systems):
        """systems: one abi.System (the ctypes bromoc_system) per replica."""
        arr = (abi.System * self.nrep)(*systems)
        self._chk(self.lib.bromoc_batch_set_systems(self.h, C.cast(arr, C.c_void_p)),
                  "set_systems")

    def set_particles(self, r, x, y, z, typei):
        x, y, z = (np.ascontiguousarray(a, np.float64) for a in (x, y, z))
        t = np.ascontiguousarray(typei, np.int32)
        dp = C.POINTER(C.c_double)
        self._chk(self.lib.bromoc_batch_set_particles(
            self.h, r, len(x), x.ctypes.data_as(dp), y.ctypes.data_as(dp),
            z.ctypes.data_as(dp), t.ctypes.data_as(C.POINTER(C.c_int32))), "set_particles")

    def get_particles(self, r, nmax):
        x, y, z = (np.zeros(nmax) for _ in range(3))
        n = C.c_int32(0)
        dp = C.POINTER(C.c_double)
        self._chk(self.lib.bromoc_batch_get_particles(
            self.h, r, C.byref(n), x.ctypes.data_as(dp), y.ctypes.data_as(dp),
            z.ctypes.data_as(dp)), "get_particles")
        return x[:n.value], y[:n.value], z[:n.value]

    def bd_steps(self, nsteps, seeds, step0=0, terms=abi.M_ALL, energies=False):
        s = np.ascontiguousarray(seeds, np.uint64)
        et = np.zeros((self.nrep, abi.NTERMS)) if energies else None
        self._chk(self.lib.bromoc_batch_bd_steps(
            self.h, terms, nsteps, s.ctypes.data_as(C.POINTER(C.c_uint64)), step0,
            et.ctypes.data_as(C.POINTER(C.c_double)) if et is not None else None), "bd_steps")
        return et

    def energy(self, terms=abi.M_ALL, forces=True):
        et = np.zeros((self.nrep, abi.NTERMS))
        nsl = self.lib.bromoc_batch_slots(self.h)
        f = np.zeros((nsl, 3)) if forces else None
        dp = C.POINTER(C.c_double)
        self._chk(self.lib.bromoc_batch_energy(
            self.h, terms, f.ctypes.data_as(dp) if f is not None else None,
            et.ctypes.data_as(dp)), "energy")
        return et, f

    def set_buffers(self, r, buffers: dict, ibuffer):
        """GCMC buffers of replica r (keys of bromoc_buffers, per buffer:
        ibfftyp, avnum, mu, kb, lzmin, lzmax, rmin, rmax, qbufferbias, nat,
        ntotat) and the buffer of each of its ions (0 none)."""
        keep = []

        def arr(k, dt):
            a = np.ascontiguousarray(buffers[k], dt)
            keep.append(a)
            return a.ctypes.data_as(C.POINTER(C.c_int32 if dt == np.int32 else
                                              (C.c_uint8 if dt == np.uint8 else C.c_double)))

        nb = len(buffers["ibfftyp"])
        st = abi.Buffers(nbuffer=nb, ibfftyp=arr("ibfftyp", np.int32), avnum=arr("avnum", np.float64),
                         mu=arr("mu", np.float64), kb=arr("kb", np.float64),
                         lzmin=arr("lzmin", np.float64), lzmax=arr("lzmax", np.float64),
                         rmin=arr("rmin", np.float64), rmax=arr("rmax", np.float64),
                         qbufferbias=arr("qbufferbias", np.uint8), nat=arr("nat", np.int32),
                         ntotat=arr("ntotat", np.int32))
        ib = np.ascontiguousarray(ibuffer, np.int32)
        self._chk(self.lib.bromoc_batch_set_buffers(
            self.h, r, C.byref(st), ib.ctypes.data_as(C.POINTER(C.c_int32))), "set_buffers")

    def grand(self, ngcmc, seeds, cycle, terms=abi.M_ALL):
        """ngcmc GCMC attempts on every replica; returns each replica's summed
        energy change of its accepted moves."""
        s = np.ascontiguousarray(seeds, np.uint64)
        d = np.zeros(self.nrep)
        self._chk(self.lib.bromoc_batch_grand(
            self.h, terms, ngcmc, s.ctypes.data_as(C.POINTER(C.c_uint64)), cycle,
            d.ctypes.data_as(C.POINTER(C.c_double))), "grand")
        return d

    def count(self):
        self._chk(self.lib.bromoc_batch_count(self.h), "count")

    def get_buffers(self, r, nbuffer, nmax):
        """(nat, ninsert, nremove, typei[n], ibuffer[n]) of replica r."""
        ip = C.POINTER(C.c_int32)
        nat, nin, nrm = (np.zeros(nbuffer, np.int32) for _ in range(3))
        t = np.zeros(nmax, np.int32)
        ib = np.zeros(nmax, np.int32)
        self._chk(self.lib.bromoc_batch_get_buffers(
            self.h, r, nat.ctypes.data_as(ip), nin.ctypes.data_as(ip), nrm.ctypes.data_as(ip),
            t.ctypes.data_as(ip), ib.ctypes.data_as(ip)), "get_buffers")
        n = len(self.get_particles(r, nmax)[0])
        return nat, nin, nrm, t[:n], ib[:n]

    def set_graph(self, on: bool):
        """Replay runs of BD steps from a captured CUDA graph (on, the
        default) or launch them one by one; the trajectories agree."""
        self._chk(self.lib.bromoc_batch_set_graph(self.h, int(on)), "set_graph")

    def tuning(self):
        """The autotuner's state per size bucket (< 1000, 1000-4000, > 4000
        ions): chosen pair-kernel warps per block (0: not tuned or empty),
        tile pairs, and the measured ms of a pair pass per candidate
        (2, 4, 8 warps)."""
        w = np.zeros(3, np.int32)
        n = np.zeros(3, np.int32)
        ms = np.zeros(9)
        self._chk(self.lib.bromoc_batch_tuning(self.h, w.ctypes.data_as(C.POINTER(C.c_int32)),
                                               n.ctypes.data_as(C.POINTER(C.c_int32)),
                                               ms.ctypes.data_as(C.POINTER(C.c_double))),
                  "tuning")
        return w, n, ms.reshape(3, 3)

    def graph_launches(self):
        return int(self.lib.bromoc_batch_graph_launches(self.h))

    def offset(self, r):
        return self.lib.bromoc_batch_offset(self.h, r)

    def launch_count(self):
        return self.lib.bromoc_batch_launch_count(self.h)
