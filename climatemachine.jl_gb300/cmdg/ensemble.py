"""Ensembles of mixed-precision models advanced together on one GPU.

``Ensemble(members)`` wraps ``cmdg_batch_*``.  Two kernel families advance
the inviscid members: "per_order" (members grouped by polynomial order,
every LSRK54 stage of a group one launch of a tile-walking kernel, the groups
independent stream branches of one CUDA graph per call) and "persistent"
(one launch per stage of one kernel over tiles of every order, whose CTA
size sets each order's elements per CTA pass and nodes per thread).  LES
members (a turbulence closure) take their gradient and viscous stage kernels
on a branch of their own.  ``autotune`` times both families and keeps the
faster one with its tiling.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from ._lib import call
from .dgmodel import DGModel, _stream


class Ensemble:
    def __init__(self, members: list[DGModel]):
        if not members:
            raise ValueError("an ensemble needs members")
        self.members = list(members)
        arr = (ctypes.c_void_p * len(members))(*[m.h for m in members])
        h = ctypes.c_void_p()
        call("cmdg_batch_create", arr, len(members), ctypes.byref(h))
        self.h = h

    def __del__(self):
        if getattr(self, "h", None) and _lib._lib is not None:
            _lib._lib.cmdg_batch_destroy(self.h)
            self.h = None

    def _ptrs(self, Qs, dQs):
        n = len(self.members)
        if len(Qs) != n or len(dQs) != n:
            raise ValueError("one state and one register per member")
        q = (ctypes.c_void_p * n)(*[Q.data_ptr() for Q in Qs])
        d = (ctypes.c_void_p * n)(*[dQ.data_ptr() for dQ in dQs])
        return q, d

    def lsrk54_step(self, Qs, dQs, dts, nsteps=1):
        q, d = self._ptrs(Qs, dQs)
        dt = (ctypes.c_double * len(self.members))(*[float(x) for x in dts])
        call("cmdg_batch_lsrk54_step", self.h, q, d, dt, int(nsteps), _stream())

    def set_tiling(self, tile_elems=1, grid_ctas=-1, N=0):
        """Tiling of the members of order N (0 = all): elements per tile and
        grid (-1 = one CTA per tile, 0 = one wave of resident CTAs)."""
        call("cmdg_batch_set_tiling", self.h, int(N), int(tile_elems), int(grid_ctas))

    def get_tiling(self):
        """{N: (tile_elems, grid_ctas)} for N = 3, 4, 5."""
        out = {}
        for N in (3, 4, 5):
            a, b = ctypes.c_int(), ctypes.c_int()
            call("cmdg_batch_get_tiling", self.h, N, ctypes.byref(a), ctypes.byref(b))
            out[N] = (a.value, b.value)
        return out

    FAMILIES = {"per_order": 0, "persistent": 1}

    def set_kernel(self, family="per_order", cta_threads=128, tile_elems=2, grid_ctas=0):
        """Kernel family; for "persistent", its CTA size (128 or 256 threads),
        elements per tile and grid (-1 = one CTA per tile, 0 = one wave of
        resident CTAs)."""
        call("cmdg_batch_set_kernel", self.h, self.FAMILIES[family], int(cta_threads), int(tile_elems),
             int(grid_ctas))

    def get_kernel(self):
        f, c, t, g = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        call("cmdg_batch_get_kernel", self.h, ctypes.byref(f), ctypes.byref(c), ctypes.byref(t), ctypes.byref(g))
        return {v: k for k, v in self.FAMILIES.items()}[f.value], c.value, t.value, g.value

    def autotune(self, Qs, dQs, reps=5):
        """Times both families and keeps the faster.  Returns the ms per
        stage launch of every candidate -- {3, 4, 5: the 10 per-order
        tilings, "persistent": the 16 persistent candidates (CTA size 128
        then 256, tile_elems 1, 2, 4, 8, grid one CTA per tile / one wave),
        "per_order": the whole per-order family} -- and the choice: the
        per-order tilings and {"kernel": get_kernel()}."""
        q, d = self._ptrs(Qs, dQs)
        ms = (ctypes.c_double * 64)()
        n = ctypes.c_int()
        call("cmdg_batch_autotune", self.h, q, d, int(reps), ms, 64, ctypes.byref(n), _stream())
        v = list(ms)[: n.value]
        per = {N: v[i * 10:(i + 1) * 10] for i, N in enumerate((3, 4, 5))}
        per["persistent"] = v[30:46]
        per["per_order"] = v[46]
        choice = self.get_tiling()
        choice["kernel"] = self.get_kernel()
        return per, choice
