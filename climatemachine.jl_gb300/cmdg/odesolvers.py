"""LSRK54CarpenterKennedy and solve! over the fused GPU stage kernels.

Mirrors src/Numerics/ODESolvers/LowStorageRungeKuttaMethod.jl:26-62,102-158,
293-327 and src/Numerics/ODESolvers/ODESolvers.jl:49-158.  A step is five
fused DG-tendency + stage-update kernels issued by ``cmdg_lsrk54_step``;
runs of equal steps are issued as one call, which the library captures as a
CUDA graph.
"""
from __future__ import annotations

import math
from fractions import Fraction

import torch

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


def dostep_(Q, solver: LSRK54CarpenterKennedy, p, time, nsteps: int = 1, dt: float | None = None):
    """dostep!(Q, lsrk, p, time): nsteps fused LSRK54 steps of size dt."""
    solver.rhs.lsrk54_step(Q, solver.dQ, time, solver.dt if dt is None else dt, nsteps)


def solve_(Q, solver: LSRK54CarpenterKennedy, param=None, *, timeend: float = math.inf, adjustfinalstep: bool = True,
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
