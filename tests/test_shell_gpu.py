"""Cubed-shell (GCM) path: the curvilinear stage kernel against the oracle.

* geometry: node coordinates and mass matrix equal the oracle's
  (StackedCubedSphereTopology + equiangular warp + curl-invariant metrics);
* FP64 tendency (Rusanov and central) within 1e-9 of the oracle, N = 3, 4;
* discrete hydrostatic balance of the GCM rest state on the GPU
  (test/Atmos/Model/discrete_hydrostatic_balance.jl: <= 100 eps after 100 s);
* mixed precision: tendency within 1e-4 and 100 LSRK54 steps within 1e-5 of
  the FP64 oracle; the full GCM workload (6 x 12 x 12 x 6 elements, N = 4,
  30 km lid) within 1e-5 of the GPU FP64 run after 200 steps;
* compensated sums and the Courant time step against the oracle;
* ConstantDynamicViscosity (with and without divergence) on the shell: the
  FP64 tendency within 1e-9 (its viscous part within 1e-8 of its own scale),
  FP64 LSRK54 steps within 1e-10, the mixed tendency within 1e-4 and 20
  mixed steps within 1e-5 of the FP64 oracle;
* SmagorinskyLilly on the shell (FP64): tendency within 1e-9 (viscous part
  1e-8), steps within 1e-10; mixed precision refused.
"""
import math

import numpy as np
import pytest
import torch

import cmdg
import oracle as O
from cmdg import workloads

pytestmark = pytest.mark.gpu

R = O.EARTH["planet_radius"]


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g

    g.build()
    torch.cuda.set_device(0)


def shell_pair(N, nh, nv, precision="fp64", numflux="rusanov", subtract_off=True, H=30e3, noise=True):
    om = O.OracleModel(N, shell=dict(nhorz=nh, nvert=nv, r_inner=R, r_outer=R + H), numflux=numflux,
                       orientation="sphere", gravity=True, ref_state=True, subtract_off=subtract_off,
                       profile="isothermal", T_surface=285.0)
    dg = workloads.gcm_shell_model(nhorz=nh, nvert=nv, N=N, H=H, precision=precision, numerical_flux=numflux,
                                   subtract_off=subtract_off)
    Q0 = workloads.gcm_initial_state(dg.grid.coordinates(), seed=5)
    if noise:
        rng = np.random.default_rng(3)
        Q0[:, 1:4] += rng.uniform(-0.5, 0.5, size=Q0[:, 1:4].shape)
    return om, dg, Q0


def rel_max(got, ref):
    out = []
    for s in range(5):
        sl = slice(1, 4) if 1 <= s <= 3 else slice(s, s + 1)
        out.append(np.abs(got[:, s] - ref[:, s]).max() / np.abs(ref[:, sl]).max())
    return np.array(out)


def field_rel(om, got, ref):
    err, nrm = om.field_l2(got, ref)
    err = np.array([err[0], np.sqrt(np.sum(err[1:4] ** 2)), err[4]])
    nrm = np.array([nrm[0], np.sqrt(np.sum(nrm[1:4] ** 2)), nrm[4]])
    return err / nrm


def test_shell_geometry_matches_oracle():
    om, dg, _ = shell_pair(4, 3, 2)
    vg = om.vgeo
    xyz = dg.grid.coordinates()
    assert np.abs(xyz - vg[:, 12:15]).max() < 1e-8 * R
    M = dg.grid.mass()
    assert np.abs(M / vg[:, 9] - 1).max() < 1e-10


@pytest.mark.parametrize("numflux", ["rusanov", "central"])
@pytest.mark.parametrize("N", [3, 4])
def test_shell_fp64_tendency_matches_oracle(N, numflux):
    om, dg, Q0 = shell_pair(N, 2, 3, numflux=numflux)
    ref = om.tendency(Q0)
    Q = dg.init_ode_state(Q0)
    dQ = dg.new_state(torch.float64)
    dg(dQ, Q, None, 0.0)
    err = rel_max(dQ.cpu().numpy(), ref)
    assert (err < 1e-9).all(), err
    assert dg.status_word() == 0


def test_shell_gcm_rest_state_stays_balanced_on_gpu():
    # GCM configuration of discrete_hydrostatic_balance.jl: 3 x 3 horizontal
    # elements per panel, 3 vertical, 50 km lid, N = 4, central flux,
    # subtract_off = false, IsothermalProfile, 100 s at Courant 0.1
    dg = workloads.gcm_shell_model(nhorz=3, nvert=3, N=4, H=50e3, numerical_flux="central", subtract_off=False,
                                   T_ref=290.0)
    ref = dg.reference_state()
    Q0 = np.zeros((dg.grid.nelem, 5, dg.grid.Np))
    Q0[:, 0] = ref[:, 0]
    Q0[:, 4] = ref[:, 1]
    Q = dg.init_ode_state(Q0)
    dt = dg.courant_dt(Q, 0.1)
    nsteps = math.ceil(100.0 / dt)
    lsrk = cmdg.LSRK54CarpenterKennedy(dg, Q, dt=100.0 / nsteps)
    cmdg.dostep_(Q, lsrk, None, 0.0, nsteps=nsteps)
    Qg = torch.from_numpy(Q0).cuda()
    err = cmdg.euclidean_distance(dg, Q, Qg) / cmdg.norm(dg, Qg)
    assert err <= 100 * np.finfo(np.float64).eps, err


@pytest.mark.parametrize("N", [3, 4])
def test_shell_mixed_tendency_close_to_oracle(N):
    om, dg, Q0 = shell_pair(N, 2, 3, precision="mixed")
    ref = om.tendency(Q0)
    Qp = dg.init_ode_state(Q0)
    dQ = dg.new_state(torch.float64)
    dg(dQ, Qp, None, 0.0)
    got = dQ.cpu().numpy()
    err = [np.linalg.norm(got[:, s] - ref[:, s]) / np.linalg.norm(ref[:, s]) for s in range(5)]
    assert max(err) < 1e-4, err


def test_shell_mixed_100_steps_within_1e5_of_fp64_oracle():
    om, dg, Q0 = shell_pair(4, 3, 3, precision="mixed", noise=False)
    dt = om.courant_dt(Q0, 0.4)
    Qo, _ = om.lsrk54(Q0.copy(), dt, 100)
    Qp = dg.init_ode_state(Q0)
    lsrk = cmdg.LSRK54CarpenterKennedy(dg, Qp, dt=dt)
    cmdg.dostep_(Qp, lsrk, None, 0.0, nsteps=100)
    rel = field_rel(om, dg.from_perturbation(Qp).cpu().numpy(), Qo)
    assert (rel < 1e-5).all(), rel
    assert dg.status_word() == 0


def test_shell_sums_and_courant_match_oracle():
    om, dg, Q0 = shell_pair(3, 2, 2)
    Q = dg.init_ode_state(Q0)
    sums = dg.weighted_sums(Q, (0, 4))
    assert sums[0] == pytest.approx(om.weightedsum(Q0, 0), rel=1e-13)
    assert sums[1] == pytest.approx(om.weightedsum(Q0, 4), rel=1e-13)
    assert dg.courant_dt(Q, 0.4) == pytest.approx(om.courant_dt(Q0, 0.4), rel=1e-10)


def test_gcm_workload_mixed_200_steps_within_1e5_of_fp64():
    """The GCM workload: 6 x 12 x 12 x 6 elements, N = 4, 30 km lid,
    isothermal 285 K, seeded zonal wind and 1 K anomaly; mixed vs FP64 on the
    GPU after 200 LSRK54 steps at CFL 0.4."""
    d64 = workloads.gcm_shell_model(precision="fp64")
    dmx = workloads.gcm_shell_model(precision="mixed")
    Q0 = workloads.gcm_initial_state(d64.grid.coordinates())
    Q64 = d64.init_ode_state(Q0)
    dt = d64.courant_dt(Q64, 0.4)
    l64 = cmdg.LSRK54CarpenterKennedy(d64, Q64, dt=dt)
    cmdg.dostep_(Q64, l64, None, 0.0, nsteps=200)
    Qp = dmx.init_ode_state(Q0)
    lmx = cmdg.LSRK54CarpenterKennedy(dmx, Qp, dt=dt)
    cmdg.dostep_(Qp, lmx, None, 0.0, nsteps=200)
    got = dmx.from_perturbation(Qp)
    M = torch.from_numpy(d64.grid.mass()).cuda()
    rel = []
    for sl in (slice(0, 1), slice(1, 4), slice(4, 5)):
        err = torch.sqrt((M[:, None] * (got[:, sl] - Q64[:, sl]) ** 2).sum())
        ref = torch.sqrt((M[:, None] * Q64[:, sl] ** 2).sum())
        rel.append(float(err / ref))
    assert max(rel) < 1e-5, rel
    assert d64.status_word() == 0 and dmx.status_word() == 0


def smag_pair(N, nh, nv, H=30e3, precision="fp64"):
    """SmagorinskyLilly on the cubed shell: oracle and GPU models and a
    sheared, stratified initial state."""
    om = O.OracleModel(N, shell=dict(nhorz=nh, nvert=nv, r_inner=R, r_outer=R + H), orientation="sphere",
                       gravity=True, ref_state=True, profile="isothermal", T_surface=285.0, turbulence="smagorinsky")
    grid = cmdg.CubedShellGrid(N, nh, nv, R, R + H)
    model = cmdg.AtmosModel(orientation="sphere", gravity=True,
                            ref_state=cmdg.HydrostaticState(cmdg.IsothermalProfile(285.0)), turbulence="smagorinsky")
    dg = cmdg.DGModel(model, grid, precision=precision)
    Q0 = workloads.gcm_initial_state(grid.coordinates(), seed=6)
    rng = np.random.default_rng(9)
    Q0[:, 1:4] += rng.uniform(-3, 3, size=Q0[:, 1:4].shape)
    return om, dg, Q0


@pytest.mark.parametrize("N", [3, 4])
def test_shell_smagorinsky_fp64_matches_oracle(N):
    """SmagorinskyLilly on the shell (grad theta_v for N^2, khat = grad Phi / g
    per node, length scale per node): the tendency within 1e-9, its viscous
    part within 1e-8 of its own scale, and 5 LSRK54 steps within 1e-10."""
    om, dg, Q0 = smag_pair(N, 2, 3)
    ref = om.tendency(Q0)
    om0, _, _ = shell_pair(N, 2, 3, noise=False)
    inv = om0.tendency(Q0)
    Q = dg.init_ode_state(Q0)
    dQ = dg.new_state(torch.float64)
    dg(dQ, Q, None, 0.0)
    got = dQ.cpu().numpy()
    assert rel_max(got, ref).max() < 1e-9
    vref, vgot = ref - inv, got - inv
    for sl in (slice(1, 4), slice(4, 5)):
        assert np.abs(vgot[:, sl] - vref[:, sl]).max() < 1e-8 * np.abs(vref[:, sl]).max()
    # the isotropic length scale 2 / (cbrt(det dxi/dx) N) is ~2e5 m on these
    # 5000 km x 10 km elements: the explicit diffusive limit is far below the
    # acoustic Courant step, so the steps use dt = 0.02 s
    Qs0 = workloads.gcm_initial_state(dg.grid.coordinates(), seed=6)
    dt = 0.02
    Qo, _ = om.lsrk54(Qs0.copy(), dt, 5)
    Qs = dg.init_ode_state(Qs0)
    lsrk = cmdg.LSRK54CarpenterKennedy(dg, Qs, dt=dt)
    cmdg.dostep_(Qs, lsrk, None, 0.0, 5)
    assert np.isfinite(Qo).all()
    assert rel_max(Qs.cpu().numpy(), Qo).max() < 1e-10


@pytest.mark.parametrize("N", [3, 4])
def test_shell_smagorinsky_mixed_close_to_oracle(N):
    """SmagorinskyLilly on the shell in mixed precision: the gradient pass
    differentiates the perturbations h' and theta_v' (formed without
    cancellation against the reference), the stage kernel adds the
    FP64-computed gradients of h_ref and theta_v_ref.  One tendency within
    1e-4 (relative L2 per field) and 20 LSRK54 steps within 1e-5 (relative
    L2 per field group) of the FP64 oracle."""
    om, dg, Q0 = smag_pair(N, 2, 3, precision="mixed")
    ref = om.tendency(Q0)
    Q = dg.init_ode_state(Q0)
    dQ = dg.new_state(torch.float64)
    dg(dQ, Q, None, 0.0)
    got = dQ.cpu().numpy()
    err = [np.linalg.norm(got[:, s] - ref[:, s]) / np.linalg.norm(ref[:, s]) for s in range(5)]
    assert max(err) < 1e-4, err
    # the explicit diffusive limit of these elements (see the FP64 test):
    # dt = 0.02 s, from the GCM state without the velocity noise (the noise's
    # node-to-node shear raises the Smagorinsky viscosity past the explicit
    # limit of any practical dt, and the oracle's own run blows up)
    dt = 0.02
    Qs0 = workloads.gcm_initial_state(dg.grid.coordinates(), seed=6)
    Qo, _ = om.lsrk54(Qs0.copy(), dt, 20)
    Q = dg.init_ode_state(Qs0)
    lsrk = cmdg.LSRK54CarpenterKennedy(dg, Q, dt=dt)
    cmdg.dostep_(Q, lsrk, None, 0.0, 20)
    assert np.isfinite(Qo).all()
    err = field_rel(om, dg.from_perturbation(Q).cpu().numpy(), Qo)
    assert err.max() < 1e-5, err
    assert dg.status_word() == 0


def visc_pair(N, nh, nv, precision="fp64", with_divergence=False, rho_nu=2e4, H=30e3):
    """ConstantDynamicViscosity on the cubed shell: oracle and GPU models and a
    sheared initial state (the GCM state plus seeded velocity noise)."""
    om = O.OracleModel(N, shell=dict(nhorz=nh, nvert=nv, r_inner=R, r_outer=R + H), orientation="sphere",
                       gravity=True, ref_state=True, profile="isothermal", T_surface=285.0, turbulence="constant",
                       rho_nu=rho_nu, with_divergence=with_divergence)
    grid = cmdg.CubedShellGrid(N, nh, nv, R, R + H)
    model = cmdg.AtmosModel(orientation="sphere", gravity=True,
                            ref_state=cmdg.HydrostaticState(cmdg.IsothermalProfile(285.0)), turbulence="constant",
                            rho_nu=rho_nu, with_divergence=with_divergence)
    dg = cmdg.DGModel(model, grid, precision=precision)
    Q0 = workloads.gcm_initial_state(grid.coordinates(), seed=5)
    rng = np.random.default_rng(8)
    Q0[:, 1:4] += rng.uniform(-3, 3, size=Q0[:, 1:4].shape)
    return om, dg, Q0


@pytest.mark.parametrize("with_divergence", [False, True])
@pytest.mark.parametrize("N", [3, 4])
def test_shell_viscous_fp64_tendency_matches_oracle(N, with_divergence):
    """The viscous part (tendency minus the inviscid model's) to 1e-8 of its
    own scale, the whole tendency to 1e-9 of the field scale."""
    om, dg, Q0 = visc_pair(N, 2, 3, with_divergence=with_divergence)
    ref = om.tendency(Q0)
    om0, dg0, _ = shell_pair(N, 2, 3, noise=False)
    inv = om0.tendency(Q0)
    Q = dg.init_ode_state(Q0)
    dQ = dg.new_state(torch.float64)
    dg(dQ, Q, None, 0.0)
    got = dQ.cpu().numpy()
    assert rel_max(got, ref).max() < 1e-9
    vref, vgot = ref - inv, got - inv
    for sl in (slice(1, 4), slice(4, 5)):
        assert np.abs(vgot[:, sl] - vref[:, sl]).max() < 1e-8 * np.abs(vref[:, sl]).max()
    assert np.abs(vref[:, 1:4]).max() > 1e-6 * np.abs(ref[:, 1:4]).max()  # the viscous part is present


def test_shell_viscous_mixed_close_to_oracle():
    # constant rho nu: nu = rho nu / rho grows to the lid, so the stepped runs
    # keep it small enough for the explicit diffusive limit at Courant 0.4
    om, dg, Q0 = visc_pair(4, 2, 3, precision="mixed", rho_nu=20.0)
    ref = om.tendency(Q0)
    Q = dg.init_ode_state(Q0)
    dQ = torch.zeros(Q.shape, dtype=torch.float64, device=Q.device)
    dg(dQ, Q, None, 0.0)
    got = dQ.cpu().numpy()
    err = [np.linalg.norm(got[:, s] - ref[:, s]) / np.linalg.norm(ref[:, s]) for s in range(5)]
    assert max(err) < 1e-4, err
    # 20 LSRK54 steps: relative L2 per field group within 1e-5 of the FP64 oracle
    dt = om.courant_dt(Q0, 0.4)
    Qo, _ = om.lsrk54(Q0.copy(), dt, 20)
    lsrk = cmdg.LSRK54CarpenterKennedy(dg, Q, dt=dt)
    cmdg.dostep_(Q, lsrk, None, 0.0, 20)
    err = field_rel(om, dg.from_perturbation(Q).cpu().numpy(), Qo)
    assert err.max() < 1e-5, err


def test_shell_viscous_fp64_steps_match_oracle():
    om, dg, Q0 = visc_pair(3, 2, 2, rho_nu=20.0)
    dt = om.courant_dt(Q0, 0.4)
    Qo, _ = om.lsrk54(Q0.copy(), dt, 5)
    Q = dg.init_ode_state(Q0)
    lsrk = cmdg.LSRK54CarpenterKennedy(dg, Q, dt=dt)
    cmdg.dostep_(Q, lsrk, None, 0.0, 5)
    assert rel_max(Q.cpu().numpy(), Qo).max() < 1e-10
