"""Ensembles of mixed-precision models advanced together on one GPU.

``Ensemble(members)`` wraps ``cmdg_batch_*``: members are grouped by
polynomial order, every LSRK54 stage of a group is one launch of a
tile-walking kernel, the groups run as independent stream branches of one
CUDA graph per call, and ``autotune`` picks each order's tiling.
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

    def autotune(self, Qs, dQs, reps=5):
        q, d = self._ptrs(Qs, dQs)
        ms = (ctypes.c_double * 64)()
        n = ctypes.c_int()
        call("cmdg_batch_autotune", self.h, q, d, int(reps), ms, 64, ctypes.byref(n), _stream())
        per = {N: list(ms)[i * n.value:(i + 1) * n.value] for i, N in enumerate((3, 4, 5))}
        return per, self.get_tiling()
