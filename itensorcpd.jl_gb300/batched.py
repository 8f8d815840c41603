"""Batched small decompositions on the device (libcpals ``cpals_batch_*``).

Many independent order-3 CP-ALS problems of uneven shape and rank run together: one
persistent kernel launch per ALS sweep, every tensor with its own FitCheck.  This replaces a
host loop of ``decompose(A, rank)`` calls (decompose.jl:1-30) for small tensors.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L


class BatchEngine:
    """Device handle for a batch of order-3 tensors (dims: list of 3-tuples, ranks: list)."""

    def __init__(self, dims, ranks, ref_norms, device=0):
        self.lib = L.load()
        self.dims = [tuple(int(x) for x in d) for d in dims]
        self.ranks = [int(r) for r in ranks]
        if len(self.dims) != len(self.ranks) or len(self.dims) != len(ref_norms):
            raise ValueError("dims, ranks and ref_norms must have one entry per tensor")
        self.count = len(self.dims)
        d = np.ascontiguousarray(np.asarray(self.dims, dtype=np.int64).reshape(-1))
        r = np.ascontiguousarray(np.asarray(self.ranks, dtype=np.int64))
        nrm = np.ascontiguousarray(np.asarray(ref_norms, dtype=np.float64))
        h = C.c_void_p()
        L.check(self.lib.cpals_batch_create(C.byref(h), int(device), self.count, L.i64ptr(d), L.i64ptr(r),
                                            L.dptr(nrm)), "cpals_batch_create")
        self.h = h
        self._foffs = []
        off = 0
        for dd, rr in zip(self.dims, self.ranks):
            self._foffs.append(off)
            off += (sum(dd) + 1) * rr
        self._ftotal = off

    def close(self):
        if getattr(self, "h", None):
            self.lib.cpals_batch_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_tensors(self, tensors):
        buf = np.concatenate([np.asarray(T, dtype=np.float32).reshape(-1, order="F") for T in tensors])
        self.set_tensors_concat(buf)

    def set_tensors_concat(self, buf):
        """The tensors already concatenated column-major in one FP32 host buffer (pinned for
        the fastest copy)."""
        if buf.dtype != np.float32 or not buf.flags.c_contiguous:
            raise TypeError("expected one contiguous float32 buffer")
        L.check(self.lib.cpals_batch_set_tensors(self.h, buf.ctypes.data_as(C.POINTER(C.c_float))),
                "cpals_batch_set_tensors")
        self._tensors_keep = buf

    def set_norms(self, ref_norms):
        """New reference norms, one per tensor (with new tensors of the same shapes)."""
        nrm = np.ascontiguousarray(np.asarray(ref_norms, dtype=np.float64))
        if nrm.size != self.count:
            raise ValueError("one norm per tensor")
        L.check(self.lib.cpals_batch_set_norms(self.h, L.dptr(nrm)), "cpals_batch_set_norms")

    def pack_factors(self, factors, lams):
        buf = np.empty(self._ftotal, dtype=np.float64)
        for t, (F, lam) in enumerate(zip(factors, lams)):
            parts = [np.asarray(f, dtype=np.float64).reshape(-1, order="F") for f in F]
            parts.append(np.asarray(lam, dtype=np.float64))
            v = np.concatenate(parts)
            buf[self._foffs[t]:self._foffs[t] + v.size] = v
        return buf

    def unpack_factors(self, buf):
        out = []
        for t, (dd, R) in enumerate(zip(self.dims, self.ranks)):
            o = self._foffs[t]
            F = []
            for I in dd:
                F.append(np.reshape(buf[o:o + I * R], (I, R), order="F").copy())
                o += I * R
            out.append((F, buf[o:o + R].copy()))
        return out

    def set_factors(self, factors, lams):
        buf = self.pack_factors(factors, lams)
        L.check(self.lib.cpals_batch_set_factors(self.h, L.dptr(buf)), "cpals_batch_set_factors")
        self._factors_keep = buf
        return buf

    def get_factors(self):
        buf = np.empty(self._ftotal, dtype=np.float64)
        L.check(self.lib.cpals_batch_get_factors(self.h, L.dptr(buf)), "cpals_batch_get_factors")
        return self.unpack_factors(buf)

    def set_factors_concat(self, buf):
        """The factors already packed (pack_factors' layout: per tensor F_0, F_1, F_2
        column-major, then lambda) in one FP64 host buffer."""
        if buf.dtype != np.float64 or not buf.flags.c_contiguous or buf.size != self._ftotal:
            raise TypeError("expected one contiguous float64 buffer of the packed factors' size")
        L.check(self.lib.cpals_batch_set_factors(self.h, L.dptr(buf)), "cpals_batch_set_factors")
        self._factors_keep = buf

    def get_factors_concat(self, out=None):
        """The factors into one FP64 host buffer in pack_factors' layout (unpack_factors splits it)."""
        if out is None:
            out = np.empty(self._ftotal, dtype=np.float64)
        elif out.dtype != np.float64 or not out.flags.c_contiguous or out.size != self._ftotal:
            raise TypeError("expected one contiguous float64 buffer of the packed factors' size")
        L.check(self.lib.cpals_batch_get_factors(self.h, L.dptr(out)), "cpals_batch_get_factors")
        return out

    def set_threads(self, threads):
        L.check(self.lib.cpals_batch_set_threads(self.h, int(threads)), "cpals_batch_set_threads")

    def set_sweeps_per_launch(self, k):
        """0 (default): optimize runs every tensor to its own stop in one launch; k >= 1: k
        sweeps per launch, the active count polled between launches.  Same results."""
        L.check(self.lib.cpals_batch_set_sweeps_per_launch(self.h, int(k)), "cpals_batch_set_sweeps_per_launch")

    def autotune(self, factors, lams, sweeps=2):
        buf = self.pack_factors(factors, lams)
        nt = C.c_int()
        ms = np.zeros(3)
        L.check(self.lib.cpals_batch_autotune(self.h, L.dptr(buf), int(sweeps), C.byref(nt), L.dptr(ms)),
                "cpals_batch_autotune")
        self._factors_keep = buf
        return int(nt.value), {128: ms[0], 256: ms[1], 512: ms[2]}

    def schedule(self):
        """The launch schedule in use: a list of per-class dicts (tensors, largest extent, largest
        rank, threads, CTAs per SM, microseconds alone) and the split schedule's autotune time."""
        n = C.c_int()
        info = np.zeros(6 * 4, dtype=np.int64)
        ms = C.c_double()
        L.check(self.lib.cpals_batch_schedule(self.h, C.byref(n), L.i64ptr(info), C.byref(ms)), "cpals_batch_schedule")
        keys = ("tensors", "max_extent", "max_rank", "threads", "ctas_per_sm", "us_alone")
        classes = [dict(zip(keys, (int(x) for x in info[6 * i:6 * i + 6]))) for i in range(n.value)]
        return classes, float(ms.value)

    def optimize(self, tol=1e-5, max_iter=200):
        """FitCheck(tol, max_iter) per tensor; returns (sweeps, fits, flags, kernel launches)."""
        sweeps = np.zeros(self.count, dtype=np.int32)
        fits = np.zeros(self.count)
        flags = np.zeros(self.count, dtype=np.int32)
        launches = C.c_int64()
        L.check(self.lib.cpals_batch_optimize(self.h, float(tol), int(max_iter),
                                              sweeps.ctypes.data_as(C.POINTER(C.c_int)), L.dptr(fits),
                                              flags.ctypes.data_as(C.POINTER(C.c_int)), C.byref(launches)),
                "cpals_batch_optimize")
        return sweeps, fits, flags, int(launches.value)
