"""cmdg — GB300-native DG tendency + LSRK54 engine for the dry AtmosModel.

Host-side mirror of ClimateMachine.jl's BalanceLaw / DGModel / ODESolvers API
for the DG spectral-element hot path, backed by libcmdg.so (hand-written CUDA
for sm_103a behind a C ABI, include/cmdg.h).  Names follow the reference:

    grid  = BrickGrid(N, ne, lo, hi, periodicity=...)        # BrickTopology + Grid
    model = AtmosModel(orientation="flat", ref_state=HydrostaticState(...), ...)
    dg    = DGModel(model, grid, numerical_flux="rusanov", precision="fp64")
    Q     = dg.init_ode_state(initial_condition)
    dg(dQ, Q, None, t)                                        # dQ = dQ/dt(Q)
    lsrk  = LSRK54CarpenterKennedy(dg, Q, dt=dt, t0=0.0)
    solve_(Q, lsrk, timeend=...)                              # solve!(Q, lsrk; timeend)
"""
from .atmos import (EARTH, AtmosModel, HydrostaticState, DryAdiabaticProfile, IsothermalProfile, DryBiharmonic,
                    AtmosAcousticGravityLinearModel)
from .dgmodel import (DGModel, BrickGrid, CubedShellGrid, ArraysGrid, euclidean_distance, weightedsum, norm,
                      remainder_DGModel, brick_element_order)
from .odesolvers import (LSRK54CarpenterKennedy, ARK2GiraldoKellyConstantinescu, LinearBackwardEulerSolver,
                         ManyColumnLU, SingleColumnLU, LowStorageVariant, solve_, dostep_)
from ._lib import CmdgError, load as load_library
from .ensemble import Ensemble
from . import checkpoint, filters, partition

__all__ = [
    "EARTH", "AtmosModel", "HydrostaticState", "DryBiharmonic", "DryAdiabaticProfile", "IsothermalProfile", "DGModel", "BrickGrid", "CubedShellGrid", "ArraysGrid",
    "euclidean_distance", "weightedsum", "norm", "LSRK54CarpenterKennedy", "solve_", "dostep_", "CmdgError",
    "load_library", "Ensemble", "AtmosAcousticGravityLinearModel", "remainder_DGModel",
    "ARK2GiraldoKellyConstantinescu", "LinearBackwardEulerSolver", "ManyColumnLU", "SingleColumnLU",
    "LowStorageVariant", "brick_element_order",
]
