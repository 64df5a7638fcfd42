"""LSRK54CarpenterKennedy, ARK2GiraldoKellyConstantinescu and solve! over
the GPU kernels.

Mirrors src/Numerics/ODESolvers/LowStorageRungeKuttaMethod.jl:26-62,102-158,
293-327, src/Numerics/ODESolvers/AdditiveRungeKuttaMethod.jl:413-538,
839-897 and src/Numerics/ODESolvers/ODESolvers.jl:49-158.  An LSRK54 step is
five fused DG-tendency + stage-update kernels issued by ``cmdg_lsrk54_step``;
runs of equal steps are issued as one call, which the library captures as a
CUDA graph.  An ARK2 step is three explicit tendencies and two column-LU
solves of the vertical linear model (``cmdg_hevi_step``).
"""
from __future__ import annotations

import math
from fractions import Fraction

import ctypes

import torch

from . import _lib
from ._lib import call

# Carpenter & Kennedy (1994) 2N-storage coefficients
RKA = tuple(float(x) for x in (Fraction(0), Fraction(-567301805773, 1357537059087),
                               Fraction(-2404267990393, 2016746695238), Fraction(-3550918686646, 2091501179385),
                               Fraction(-1275806237668, 842570457699)))
RKB = tuple(float(x) for x in (Fraction(1432997174477, 9575080441755), Fraction(5161836677717, 13612068292357),
                               Fraction(1720146321549, 2090206949498), Fraction(3134564353537, 4481467310338),
                               Fraction(2277821191437, 14882151754819)))
RKC = tuple(float(x) for x in (Fraction(0), Fraction(1432997174477, 9575080441755),
                               Fraction(2526269341429, 6820363962896), Fraction(2006345519317, 3224310063776),
                               Fraction(2802321613138, 2924317926251)))


class LSRK54CarpenterKennedy:
    """LowStorageRungeKutta2N with the LSRK54 coefficients; owns the FP64 RK
    register dQ (zero-filled, as ``fill!(dQ, 0)`` in the reference)."""

    def __init__(self, rhs, Q: torch.Tensor, dt: float = 0.0, t0: float = 0.0):
        self.rhs = rhs
        self.dt = float(dt)
        self.t = float(t0)
        self.steps = 0
        self.dQ = torch.zeros(Q.shape, dtype=torch.float64, device=Q.device)

    def gettime(self):
        return self.t

    def getdt(self):
        return self.dt


class ManyColumnLU:
    """ManyColumnLU() (src/Numerics/SystemSolvers/columnwise_lu_solver.jl:14):
    one banded LU factorization, without pivoting, per vertical node line."""


class SingleColumnLU:
    """SingleColumnLU() (columnwise_lu_solver.jl:17-23): one banded LU (the
    first column's) for every column; the library refuses it unless all
    column matrices agree (an affine brick, for instance)."""


class LowStorageVariant:
    """LowStorageVariant() of the additive Runge-Kutta schemes."""


class LinearBackwardEulerSolver:
    """LinearBackwardEulerSolver(solver; isadjustable, preconditioner_update_freq)
    (src/Numerics/ODESolvers/BackwardEulerSolvers.jl).  The column LU is
    factored once for the solver's dt."""

    def __init__(self, solver, isadjustable: bool = False, preconditioner_update_freq: int = -1):
        if not isinstance(solver, (ManyColumnLU, SingleColumnLU)):
            raise ValueError("the GPU backward Euler solver is ManyColumnLU() or SingleColumnLU()")
        self.solver = solver
        self.isadjustable = isadjustable
        self.preconditioner_update_freq = preconditioner_update_freq


class ARK2GiraldoKellyConstantinescu:
    """ARK2GiraldoKellyConstantinescu(F, L, backward_euler_solver, Q; dt, t0,
    split_explicit_implicit, variant = LowStorageVariant(), paperversion)
    (AdditiveRungeKuttaMethod.jl:839-897): F the full DGModel (or
    remainder_DGModel(dg, (lineardg,)) with split_explicit_implicit=True),
    L the vertical linear DGModel of the same model.  Q is the FP64 state;
    with a mixed-precision dg the explicit tendencies run on its FP32
    perturbation (the stage algebra and the column solve stay FP64)."""

    def __init__(self, F, L, backward_euler_solver, Q: torch.Tensor, dt: float = None, t0: float = 0.0,
                 split_explicit_implicit: bool = False, variant=None, paperversion: bool = False):
        from .dgmodel import DGModel, RemainderDGModel

        if dt is None:
            raise ValueError("dt is required")
        if variant is not None and not isinstance(variant, LowStorageVariant):
            raise ValueError("the GPU ARK2 scheme runs the LowStorageVariant")
        if not isinstance(backward_euler_solver, LinearBackwardEulerSolver):
            raise ValueError("backward_euler_solver must be a LinearBackwardEulerSolver(ManyColumnLU() or "
                             "SingleColumnLU())")
        if not (isinstance(L, DGModel) and L.is_linear):
            raise ValueError("L must be the vertical linear DGModel")
        dg = L.parent
        if split_explicit_implicit:
            if not (isinstance(F, RemainderDGModel) and F.main is dg):
                raise ValueError("split_explicit_implicit=True takes F = remainder_DGModel(dg, (lineardg,))")
        elif F is not dg:
            raise ValueError("F must be the DGModel whose linear model L is")
        if Q.dtype != torch.float64:
            raise ValueError("the ARK2 scheme advances FP64 states")
        self.rhs, self.rhs_implicit = F, L
        self.dg = dg
        self.dt = float(dt)
        self.t = float(t0)
        self.steps = 0
        self.split_explicit_implicit = bool(split_explicit_implicit)
        h = ctypes.c_void_p()
        self.single_column = isinstance(backward_euler_solver.solver, SingleColumnLU)
        call("cmdg_hevi_create", dg.h, self.dt, int(self.split_explicit_implicit), int(paperversion),
             int(self.single_column), ctypes.byref(h))
        self.h = h
        alpha, bw, nline = ctypes.c_double(), ctypes.c_int(), ctypes.c_int64()
        call("cmdg_hevi_info", h, ctypes.byref(alpha), ctypes.byref(bw), ctypes.byref(nline))
        self.alpha, self.bandwidth, self.nline = alpha.value, bw.value, nline.value

    def __del__(self):
        if getattr(self, "h", None) and _lib._lib is not None:
            _lib._lib.cmdg_hevi_destroy(self.h)
            self.h = None

    def gettime(self):
        return self.t

    def getdt(self):
        return self.dt

    def backward_euler_solve(self, Q: torch.Tensor, Qhat: torch.Tensor) -> torch.Tensor:
        """besolver!(Q, Qhat, alpha): Q = Qhat + alpha L(Q), alpha = dt (1 - 1/sqrt(2))."""
        from .dgmodel import _dptr, _stream

        call("cmdg_hevi_solve", self.h, _dptr(Q), _dptr(Qhat), _stream())
        return Q


def dostep_(Q, solver, p, time, nsteps: int = 1, dt: float | None = None):
    """dostep!(Q, solver, p, time): nsteps steps of size dt (fused LSRK54
    stage kernels, or ARK2 steps with the column LU)."""
    if isinstance(solver, ARK2GiraldoKellyConstantinescu):
        from .dgmodel import _dptr, _stream

        if dt is not None and dt != solver.dt:
            raise ValueError("the ARK2 column LU is factored for the solver's dt; a different step size needs a new solver")
        call("cmdg_hevi_step", solver.h, _dptr(Q), float(time), int(nsteps), _stream())
        return
    solver.rhs.lsrk54_step(Q, solver.dQ, time, solver.dt if dt is None else dt, nsteps)


def solve_(Q, solver, param=None, *, timeend: float = math.inf, adjustfinalstep: bool = True,
           numberofsteps: int = 0, callbacks=()):
    """solve!(Q, solver; timeend, adjustfinalstep, numberofsteps, callbacks).

    The step sequence (including the shortened final step) is the
    reference's; without callbacks, equal steps are issued in one batch.
    Each callback is called as ``cb(solver, Q)`` after every step and may
    return a positive value to stop.
    """
    if not (math.isfinite(timeend) or numberofsteps > 0):
        raise ValueError("timeend or numberofsteps must be given")
    time = solver.t
    dt = solver.dt
    step = 0
    plan = []  # (dt, count)
    while time < timeend:
        step += 1
        h = dt
        final = False
        if adjustfinalstep and time + h > timeend:
            h = timeend - time
            final = True
        if h <= 0:
            raise ValueError("non-positive time step")
        if plan and plan[-1][0] == h and not callbacks:
            plan[-1][1] += 1
        else:
            plan.append([h, 1])
        time = timeend if final else time + h
        if callbacks:
            dostep_(Q, solver, param, solver.t, 1, h)
            solver.t = time
            solver.steps = step
            stop = False
            for cb in callbacks:
                v = cb(solver, Q)
                if v is not None and v > 0:
                    stop = True
            if stop:
                return solver.t
            plan.clear()
        if step == numberofsteps:
            break
    if not callbacks:
        t = solver.t
        for h, count in plan:
            dostep_(Q, solver, param, t, count, h)
            t += h * count
        solver.t = time
        solver.steps = step
    return solver.t
