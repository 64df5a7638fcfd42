"""The algebra the mixed HEVI remainder kernel relies on, checked in FP64 on
the host: for dry air and the vertical AtmosAcousticGravityLinearModel
(src/Atmos/Model/linear.jl:103-190; PhaseDry pressure as in the stage
kernels), the flux differences F - F_L written without large cancelling
terms equal the differences of the two fluxes evaluated separately.

  p - p_L = -(R_d/cv_d) ke,   ke = |rho u|^2 / (2 rho)
  (rhoe + p)/rho - (rhoe_ref + p_ref)/rho_ref
        = ((rhoe' + p') rho_ref - (rhoe_ref + p_ref) rho') / (rho rho_ref)

with p = rho R_d T_0 + (R_d/cv_d)(rhoe - ke - rho Phi) and the linearised
p_L = rho R_d T_0 + (R_d/cv_d)(rhoe - rho Phi); primes are the
perturbations about the reference state.
"""
import numpy as np

from cmdg import EARTH

R_D, CV_D, T_0 = EARTH["R_d"], EARTH["cv_d"], EARTH["T_0"]
KV = R_D / CV_D


def pressure(rho, rhou, rhoe, phi):
    ke = 0.5 * np.sum(rhou * rhou, axis=0) / rho
    return rho * R_D * T_0 + KV * (rhoe - ke - rho * phi)


def linear_pressure(rho, rhoe, phi):
    return rho * R_D * T_0 + KV * (rhoe - rho * phi)


def test_remainder_flux_identities():
    rng = np.random.default_rng(17)
    n = 10000
    phi = rng.uniform(0, 9.81 * 3e4, n)                      # geopotential up to 30 km
    T_ref = rng.uniform(200.0, 300.0, n)
    rho_ref = rng.uniform(0.02, 1.3, n)
    p_ref = rho_ref * R_D * T_ref
    rhoe_ref = rho_ref * (CV_D * (T_ref - T_0) + phi)
    # perturbations: density, momentum, energy
    drho = rho_ref * rng.uniform(-1e-2, 1e-2, n)
    rhou = rng.uniform(-30, 30, (3, n)) * (rho_ref + drho)
    drhoe = rhoe_ref * rng.uniform(-1e-2, 1e-2, n) + rng.uniform(-1e3, 1e3, n)
    rho, rhoe = rho_ref + drho, rhoe_ref + drhoe
    ke = 0.5 * np.sum(rhou * rhou, axis=0) / rho

    p = pressure(rho, rhou, rhoe, phi)
    pL = linear_pressure(rho, rhoe, phi)
    assert np.allclose(p - pL, -KV * ke, rtol=1e-9, atol=1e-9 * np.abs(p).max())

    # the reference state's own pressure: p(q_ref) = p_L(q_ref) = p_ref
    assert np.allclose(pressure(rho_ref, 0 * rhou, rhoe_ref, phi), p_ref, rtol=1e-12)
    # p' as the mixed kernels form it: (R/cv)(rhoe' - ke) + rho' (R T_0 - (R/cv) Phi)
    dp = KV * (drhoe - ke) + drho * (R_D * T_0 - KV * phi)
    assert np.allclose(p - p_ref, dp, rtol=1e-9, atol=1e-9 * np.abs(p).max())

    href = rhoe_ref + p_ref
    direct = (rhoe + p) / rho - href / rho_ref
    written = ((drhoe + dp) * rho_ref - href * drho) / (rho * rho_ref)
    scale = np.abs(href / rho_ref).max()
    assert np.allclose(direct, written, rtol=0, atol=1e-12 * scale)
    # the energy flux differences along a direction: u (rhoe + p) - H_L rho u
    H_L = href / rho_ref
    for d in range(3):
        Fe, FLe = rhou[d] * (rhoe + p) / rho, H_L * rhou[d]
        assert np.allclose(Fe - FLe, rhou[d] * written, rtol=0, atol=1e-10 * np.abs(Fe).max())
