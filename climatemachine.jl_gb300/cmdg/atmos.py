"""Dry AtmosModel configuration (the model side of the BalanceLaw plugin).

Mirrors the constructor surface of ``AtmosModel{FT}(AtmosLESConfigType,
AtmosPhysics{FT}(param_set; ref_state, turbulence, moisture); orientation,
source)`` (src/Atmos/Model/AtmosModel.jl:154-375) for the subset the GPU
path implements: DryModel moisture, TotalEnergyModel, Compressible, Rusanov
or central first-order flux, Gravity() source, HydrostaticState reference
state, NoOrientation, FlatOrientation or SphericalOrientation,
ConstantDynamicViscosity or SmagorinskyLilly turbulence, DryBiharmonic
hyperdiffusion, and the AtmosAcousticGravityLinearModel of HEVI stepping.

The planet constants are CLIMAParameters.jl 0.2.0's Earth values.
"""
from __future__ import annotations

from dataclasses import dataclass, field

from ._lib import AtmosParams

_R_D = 8.3144598 / 28.97e-3   # gas_constant / molmass_dryair
_KAPPA_D = 2 / 7
_CP_D = _R_D / _KAPPA_D
EARTH = dict(R_d=_R_D, cp_d=_CP_D, cv_d=_CP_D - _R_D, T_0=273.16, grav=9.81, MSLP=1.01325e5, inv_Pr_turb=3.0,
             C_smag=0.21, planet_radius=6.371e6)


@dataclass
class IsothermalProfile:
    """Thermodynamics.TemperatureProfiles.IsothermalProfile(T_virt)."""
    T_virt: float = 285.0


@dataclass
class DryAdiabaticProfile:
    """Thermodynamics.TemperatureProfiles.DryAdiabaticProfile(T_surface, T_min_ref)."""
    T_surface: float = 300.0
    T_min_ref: float = 0.0


@dataclass
class HydrostaticState:
    """HydrostaticState(profile; subtract_off) (src/Atmos/Model/ref_state.jl:36-60)."""
    profile: object = field(default_factory=DryAdiabaticProfile)
    subtract_off: bool = True


@dataclass
class DryBiharmonic:
    """DryBiharmonic(tau_timescale) horizontal hyperdiffusion
    (src/Common/TurbulenceClosures/TurbulenceClosures.jl:793-848):
    nu_4 = (Delta_h / 2)^4 / 2 / tau acting on u_h and h_tot."""
    tau_timescale: float = 8 * 3600.0


@dataclass
class AtmosModel:
    orientation: str = "none"            # "none" | "flat" | "sphere"
    ref_state: HydrostaticState | None = None
    gravity: bool = False                # source = (Gravity(),)
    turbulence: str = "none"             # "none" | "constant" | "smagorinsky"
    rho_nu: float = 0.0
    with_divergence: bool = False
    C_smag: float = EARTH["C_smag"]
    hyperdiffusion: DryBiharmonic | None = None   # None = NoHyperDiffusion()
    constants: dict = field(default_factory=lambda: dict(EARTH))

    def c_params(self, numerical_flux: str) -> AtmosParams:
        p = AtmosParams()
        for k in ("R_d", "cp_d", "cv_d", "T_0", "grav", "MSLP", "inv_Pr_turb", "planet_radius"):
            setattr(p, k, float(self.constants[k]))
        p.numflux = {"rusanov": 0, "central": 1}[numerical_flux]
        p.orientation = {"none": 0, "flat": 1, "sphere": 2}[self.orientation]
        p.gravity = int(self.gravity)
        rs = self.ref_state
        p.ref_state = int(rs is not None)
        p.subtract_off = int(rs.subtract_off) if rs is not None else 1
        if rs is not None and isinstance(rs.profile, IsothermalProfile):
            p.profile, p.T_surface, p.T_min = 0, rs.profile.T_virt, 0.0
        elif rs is not None:
            p.profile, p.T_surface, p.T_min = 1, rs.profile.T_surface, rs.profile.T_min_ref
        else:
            p.profile, p.T_surface, p.T_min = 1, 300.0, 0.0
        p.turbulence = {"none": 0, "constant": 1, "smagorinsky": 2}[self.turbulence]
        p.rho_nu = self.rho_nu
        p.with_divergence = int(self.with_divergence)
        p.C_smag = self.C_smag
        hd = self.hyperdiffusion
        p.hyperdiffusion = 0 if hd is None else 1
        p.tau_hyper = 0.0 if hd is None else float(hd.tau_timescale)
        return p


@dataclass
class AtmosAcousticGravityLinearModel:
    """AtmosAcousticGravityLinearModel(atmos) (src/Atmos/Model/linear.jl:
    242-262): the acoustic and gravity terms of the dry AtmosModel linearized
    about its hydrostatic reference state -- fluxes rho u, p_L I and
    (rhoe_ref + p_ref) / rho_ref rho u with
    p_L = rho R_d T_0 + R_d / cv_d (rhoe - rho Phi), source -rho grad Phi,
    wavespeed the reference sound speed.  Discretized by a DGModel in
    VerticalDirection that shares the atmos model's auxiliary state."""
    atmos: AtmosModel

    def __post_init__(self):
        if self.atmos.ref_state is None:
            raise ValueError("AtmosAcousticGravityLinearModel needs a model with a reference state")
