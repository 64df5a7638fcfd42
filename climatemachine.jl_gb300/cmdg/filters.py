"""Filters applied to a state between steps (src/Numerics/Mesh/Filters.jl).

    filt = ExponentialFilter(grid, Nc=0, s=32)      # CutoffFilter(grid, Nc), BoydVandevenFilter(grid, Nc, s)
    apply_(Q, (0, 4), dg, filt, direction="vertical")  # Filters.apply!(Q, target, grid, filter; direction)
    apply_(Q, (0,), dg, TMARFilter())

``Nc`` may be one order for every direction or a (horizontal, vertical)
pair, as in the reference.  The matrices are ``spectral_filter_matrix``
(``cmdg_filter_matrix``); the GPU applies them in place
(``cmdg_apply_filter``, ``cmdg_apply_tmar``).
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from ._lib import call
from .dgmodel import _dptr, _stream

KINDS = {"exponential": 0, "cutoff": 1, "boyd_vandeven": 2}
DIRECTIONS = {"every": 0, "horizontal": 1, "vertical": 2}


def filter_matrix(N: int, kind: str, Nc: int, s: int = 32, alpha: float | None = None) -> np.ndarray:
    """spectral_filter_matrix (Filters.jl:114-128): W[i, n], row i = output node."""
    if alpha is None:
        alpha = -math.log(np.finfo(np.float64).eps)
    W = np.zeros((N + 1, N + 1))
    call("cmdg_filter_matrix", int(N), KINDS[kind], int(Nc), int(s), float(alpha), ctypes.c_void_p(W.ctypes.data))
    return W


class _Spectral:
    kind = None

    def __init__(self, grid, Nc, s=32, alpha=None):
        Nc = (Nc, Nc) if isinstance(Nc, int) else tuple(Nc)
        self.Nc, self.s = Nc, s
        self.filter_matrices = (filter_matrix(grid.N, self.kind, Nc[0], s, alpha),
                                filter_matrix(grid.N, self.kind, Nc[1], s, alpha))


class ExponentialFilter(_Spectral):
    """ExponentialFilter(grid, Nc=0, s=32, alpha=-log(eps)) (Filters.jl:172-213)."""
    kind = "exponential"

    def __init__(self, grid, Nc=0, s=32, alpha=None):
        super().__init__(grid, Nc, s, alpha)


class CutoffFilter(_Spectral):
    """CutoffFilter(grid, Nc=N): zeroes the Legendre modes >= Nc (Filters.jl:275-306)."""
    kind = "cutoff"

    def __init__(self, grid, Nc=None):
        super().__init__(grid, grid.N if Nc is None else Nc)


class BoydVandevenFilter(_Spectral):
    """BoydVandevenFilter(grid, Nc=0, s=32) (Filters.jl:231-269)."""
    kind = "boyd_vandeven"

    def __init__(self, grid, Nc=0, s=32):
        super().__init__(grid, Nc, s)


class MassPreservingCutoffFilter:
    """MassPreservingCutoffFilter(grid, Nc=N) (Filters.jl:309-345): zeroes the
    Legendre modes >= Nc and restores each element's mass-weighted integral
    after each directional pass (for meshes with a non-constant Jacobian).
    The matrices are modified_filter_matrix with sigma = 0: the cutoff
    matrix, or the identity for Nc > N."""

    def __init__(self, grid, Nc=None):
        Nc = grid.N if Nc is None else Nc
        Nc = (Nc, Nc) if isinstance(Nc, int) else tuple(Nc)
        self.Nc = Nc
        self.filter_matrices = tuple(np.eye(grid.N + 1) if c > grid.N else filter_matrix(grid.N, "cutoff", c)
                                     for c in Nc)


class TMARFilter:
    """Truncation and mass-aware rescaling (Filters.jl:369-407)."""


def apply_(Q, target, dg, filt, direction: str = "every"):
    """Filters.apply!(Q, target, grid, filter; direction) on a model's state
    (FP64, or the FP32 perturbation of a mixed model)."""
    fields = tuple(range(5)) if target is None or target == slice(None) else tuple(int(f) for f in target)
    arr = (ctypes.c_int * len(fields))(*fields)
    if isinstance(filt, TMARFilter):
        call("cmdg_apply_tmar", dg.h, _dptr(Q), arr, len(fields), _stream())
        return Q
    if isinstance(filt, MassPreservingCutoffFilter):
        Wh = np.ascontiguousarray(filt.filter_matrices[0])
        Wv = np.ascontiguousarray(filt.filter_matrices[1])
        call("cmdg_apply_mp_filter", dg.h, _dptr(Q), ctypes.c_void_p(Wh.ctypes.data), ctypes.c_void_p(Wv.ctypes.data),
             DIRECTIONS[direction], arr, len(fields), _stream())
        return Q
    Wh = np.ascontiguousarray(filt.filter_matrices[0])
    Wv = np.ascontiguousarray(filt.filter_matrices[1])
    call("cmdg_apply_filter", dg.h, _dptr(Q), ctypes.c_void_p(Wh.ctypes.data), ctypes.c_void_p(Wv.ctypes.data),
         DIRECTIONS[direction], arr, len(fields), _stream())
    return Q
