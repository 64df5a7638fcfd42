"""GPU parity of DryBiharmonic hyperdiffusion (the gradient, laplacian and
gradient-of-laplacian passes and the hyperdiffusive second-order fluxes)
against the oracle, whose passes reproduce the reference's golden errors of
test/Numerics/DGMethods/advection_diffusion/periodic_3D_hyperdiffusion.jl.

Bounds: FP64 <= 1e-10 of the field scale (the hyperdiffusive state scaled per
GradientLaplacian state as a 3-vector; momentum scaled as a vector); mixed
precision relative L2 <= 1e-3 for the hyperdiffusive state (three derivatives
of the FP32 perturbation h' amplify its rounding), <= 1e-4 for one tendency
and <= 1e-5 for the state after steps.
"""
import numpy as np
import pytest
import torch

import cmdg
import oracle as O

pytestmark = pytest.mark.gpu

TOL64 = 1e-10
L = 2500.0
TAU = 60.0  # short enough that the hyperdiffusive flux is a sizeable part of the tendency


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g

    g.build()
    torch.cuda.set_device(0)


def pair(turb="none", N=4, ne=(3, 2, 4), precision="fp64", profile="dry_adiabatic", direction="every", **kw):
    phys = dict(orientation="flat", gravity=True, ref_state=True, profile=profile,
                T_surface=300.0 if profile == "dry_adiabatic" else 285.0, T_min=0.0, turbulence=turb,
                hyperdiffusion="dry_biharmonic", tau_hyper=TAU, hyper_direction=direction)
    phys.update(kw)
    om = O.OracleModel(N, ne, (0, 0, 0), (L, L, L), periodic=(1, 1, 0), **phys)
    grid = cmdg.BrickGrid(N, ne, (0, 0, 0), (L, L, L), periodicity=(True, True, False),
                          boundary=((0, 0), (0, 0), (1, 2)))
    prof = cmdg.DryAdiabaticProfile(300.0, 0.0) if profile == "dry_adiabatic" else cmdg.IsothermalProfile(285.0)
    model = cmdg.AtmosModel(orientation="flat", gravity=True, ref_state=cmdg.HydrostaticState(prof),
                            turbulence=turb, rho_nu=kw.get("rho_nu", 0.0),
                            hyperdiffusion=cmdg.DryBiharmonic(TAU))
    dg = cmdg.DGModel(model, grid, precision=precision, diffusion_direction=direction)
    Q0 = om.init_bubble(rc=900.0, xc=1100.0, yc=1300.0, zc=800.0)
    rng = np.random.default_rng(29)
    Q0[:, 1:4] += rng.uniform(-3, 3, size=Q0[:, 1:4].shape)
    return om, dg, Q0


# GPU word 3 c + d (c = u, v, h_tot) <- oracle word 3 s + d (s = u_h[0..2], h_tot)
ORACLE_WORDS = [0, 1, 2, 3, 4, 5, 9, 10, 11]


def rel_groups(got, ref, groups):
    out = []
    for g in groups:
        sl = slice(g[0], g[-1] + 1)
        scale = np.abs(ref[:, sl]).max()
        out.append(np.abs(got[:, sl] - ref[:, sl]).max() / (scale if scale > 0 else 1.0))
    return np.array(out)


@pytest.mark.parametrize("direction", ["every", "horizontal"])
@pytest.mark.parametrize("N", [2, 3, 4, 5])
def test_fp64_hyperdiffusive_state_matches_oracle(N, direction):
    om, dg, Q0 = pair(N=N, direction=direction)
    ref, _ = om.hyper_pass(Q0)
    ref = ref[:, ORACLE_WORDS]
    got = dg.hyperdiffusive_state(dg.init_ode_state(Q0)).cpu().numpy()
    err = rel_groups(got, ref, [(0, 1, 2), (3, 4, 5), (6, 7, 8)])
    assert (err < TOL64).all(), err
    # u_h has no vertical component on a flat brick
    assert np.abs(om.hyper_pass(Q0)[0][:, 6:9]).max() <= 1e-12 * np.abs(ref[:, 0:6]).max()


CASES = [("none", {}), ("constant", dict(rho_nu=60.0)), ("smagorinsky", {})]


@pytest.mark.parametrize("N", [3, 4, 5])
@pytest.mark.parametrize("turb,kw", CASES)
def test_fp64_hyperdiffusive_tendency_matches_oracle(turb, kw, N):
    om, dg, Q0 = pair(turb, N=N, **kw)
    ref = om.tendency(Q0)
    dQ = dg.new_state(torch.float64)
    dg(dQ, dg.init_ode_state(Q0), None, 0.0)
    err = rel_groups(dQ.cpu().numpy(), ref, [(0,), (1, 2, 3), (4,)])
    assert (err < TOL64).all(), err


@pytest.mark.parametrize("N", [3, 4])
def test_fp64_horizontal_hyperdiffusive_tendency_matches_oracle(N):
    om, dg, Q0 = pair(N=N, direction="horizontal")
    ref = om.tendency(Q0)
    dQ = dg.new_state(torch.float64)
    dg(dQ, dg.init_ode_state(Q0), None, 0.0)
    err = rel_groups(dQ.cpu().numpy(), ref, [(0,), (1, 2, 3), (4,)])
    assert (err < TOL64).all(), err


def test_hyperdiffusion_is_a_sizeable_part_of_the_tendency():
    """The parity cases exercise the hyperdiffusive fluxes: they change the
    momentum tendency by more than 1 % of its scale and the energy tendency
    (dominated by the advection of rho e + p) by more than 0.05 %, well above
    the 1e-10 parity bound."""
    om, dg, Q0 = pair()
    with_h = om.tendency(Q0)
    om0 = O.OracleModel(4, (3, 2, 4), (0, 0, 0), (L, L, L), periodic=(1, 1, 0), orientation="flat", gravity=True,
                        ref_state=True, profile="dry_adiabatic", T_surface=300.0, T_min=0.0)
    without = om0.tendency(Q0)
    for sl, frac in ((slice(1, 4), 1e-2), (slice(4, 5), 5e-4)):
        assert np.abs(with_h[:, sl] - without[:, sl]).max() > frac * np.abs(with_h[:, sl]).max()


@pytest.mark.parametrize("turb,kw", CASES[:2])
def test_fp64_hyperdiffusive_steps_match_oracle(turb, kw):
    om, dg, Q0 = pair(turb, ne=(3, 3, 3), **kw)
    dt = 0.25 * om.courant_dt(Q0, 0.4)
    Qo, _ = om.lsrk54(Q0.copy(), dt, 5)
    Q = dg.init_ode_state(Q0)
    lsrk = cmdg.LSRK54CarpenterKennedy(dg, Q, dt=dt)
    cmdg.dostep_(Q, lsrk, None, 0.0, nsteps=5)
    err = rel_groups(Q.cpu().numpy(), Qo, [(0,), (1, 2, 3), (4,)])
    assert (err < TOL64).all(), err


@pytest.mark.parametrize("profile,direction", [("dry_adiabatic", "every"), ("isothermal", "every"),
                                               ("isothermal", "horizontal")])
def test_mixed_hyperdiffusion_close_to_fp64_oracle(profile, direction):
    om, dg, Q0 = pair(ne=(4, 3, 4), precision="mixed", profile=profile, direction=direction)
    Qp = dg.init_ode_state(Q0)
    ref_h = om.hyper_pass(Q0)[0][:, ORACLE_WORDS]
    got_h = dg.hyperdiffusive_state(Qp).cpu().numpy()
    for sl in (slice(0, 3), slice(3, 6), slice(6, 9)):
        e = np.linalg.norm(got_h[:, sl] - ref_h[:, sl]) / np.linalg.norm(ref_h[:, sl])
        assert e < 1e-3, (sl, e)
    ref = om.tendency(Q0)
    dQ = dg.new_state(torch.float64)
    dg(dQ, Qp, None, 0.0)
    got = dQ.cpu().numpy()
    errs = [np.linalg.norm(got[:, sl] - ref[:, sl]) / np.linalg.norm(ref[:, sl])
            for sl in (slice(0, 1), slice(1, 4), slice(4, 5))]
    assert max(errs) < 1e-4, errs
    dt = 0.25 * om.courant_dt(Q0, 0.4)
    Qo, _ = om.lsrk54(Q0.copy(), dt, 30)
    lsrk = cmdg.LSRK54CarpenterKennedy(dg, Qp, dt=dt)
    cmdg.dostep_(Qp, lsrk, None, 0.0, nsteps=30)
    err, refn = om.field_l2(dg.from_perturbation(Qp).cpu().numpy(), Qo)
    err = np.array([err[0], np.sqrt(np.sum(err[1:4] ** 2)), err[4]])
    refn = np.array([refn[0], np.sqrt(np.sum(refn[1:4] ** 2)), refn[4]])
    assert (err / refn < 1e-5).all(), err / refn


def test_hyperdiffusion_configuration_errors():
    grid = cmdg.BrickGrid(3, (2, 2, 2), (0, 0, 0), (L, L, L), periodicity=(True, True, False),
                          boundary=((0, 0), (0, 0), (1, 2)))
    with pytest.raises(cmdg.CmdgError, match="FlatOrientation"):
        cmdg.DGModel(cmdg.AtmosModel(hyperdiffusion=cmdg.DryBiharmonic(100.0)), grid)
    with pytest.raises(cmdg.CmdgError, match="tau_timescale"):
        cmdg.DGModel(cmdg.AtmosModel(orientation="flat", hyperdiffusion=cmdg.DryBiharmonic(0.0)), grid)
    shell = cmdg.CubedShellGrid(3, 2, 2, r_inner=6.371e6, r_outer=6.371e6 + 30e3)
    with pytest.raises(cmdg.CmdgError, match="SphericalOrientation"):
        cmdg.DGModel(cmdg.AtmosModel(orientation="none", hyperdiffusion=cmdg.DryBiharmonic(100.0)), shell)


# ---------------------------------------------------------------- cubed shell
R_EARTH = O.EARTH["planet_radius"]
TAU_GCM = 3600.0


def shell_pair(N=4, nh=2, nv=3, precision="fp64", H=30e3):
    from cmdg import workloads

    om = O.OracleModel(N, shell=dict(nhorz=nh, nvert=nv, r_inner=R_EARTH, r_outer=R_EARTH + H),
                       orientation="sphere", gravity=True, ref_state=True, profile="isothermal", T_surface=285.0,
                       hyperdiffusion="dry_biharmonic", tau_hyper=TAU_GCM, hyper_direction="horizontal")
    dg = workloads.gcm_shell_model(nhorz=nh, nvert=nv, N=N, H=H, precision=precision, tau_hyper=TAU_GCM)
    Q0 = workloads.gcm_initial_state(dg.grid.coordinates(), seed=5)
    rng = np.random.default_rng(7)
    Q0[:, 1:4] += rng.uniform(-0.5, 0.5, size=Q0[:, 1:4].shape)
    return om, dg, Q0


@pytest.mark.parametrize("N", [3, 4])
def test_shell_fp64_hyperdiffusive_state_matches_oracle(N):
    om, dg, Q0 = shell_pair(N=N)
    ref, _ = om.hyper_pass(Q0)
    got = dg.hyperdiffusive_state(dg.init_ode_state(Q0)).cpu().numpy()
    err = rel_groups(got, ref, [(0, 1, 2, 3, 4, 5, 6, 7, 8), (9, 10, 11)])
    assert (err < 1e-9).all(), err


@pytest.mark.parametrize("N", [3, 4])
def test_shell_fp64_hyperdiffusive_tendency_matches_oracle(N):
    om, dg, Q0 = shell_pair(N=N)
    ref = om.tendency(Q0)
    dQ = dg.new_state(torch.float64)
    dg(dQ, dg.init_ode_state(Q0), None, 0.0)
    err = rel_groups(dQ.cpu().numpy(), ref, [(0,), (1, 2, 3), (4,)])
    assert (err < 1e-9).all(), err
    # the hyperdiffusive part is a sizeable part of the momentum tendency
    om0 = O.OracleModel(N, shell=dict(nhorz=2, nvert=3, r_inner=R_EARTH, r_outer=R_EARTH + 30e3),
                        orientation="sphere", gravity=True, ref_state=True, profile="isothermal", T_surface=285.0)
    without = om0.tendency(Q0)
    assert np.abs(ref[:, 1:4] - without[:, 1:4]).max() > 1e-2 * np.abs(ref[:, 1:4]).max()


def test_shell_mixed_hyperdiffusion_close_to_fp64_oracle():
    om, dg, Q0 = shell_pair(precision="mixed")
    Qp = dg.init_ode_state(Q0)
    ref_h = om.hyper_pass(Q0)[0]
    got_h = dg.hyperdiffusive_state(Qp).cpu().numpy()
    for sl in (slice(0, 9), slice(9, 12)):
        e = np.linalg.norm(got_h[:, sl] - ref_h[:, sl]) / np.linalg.norm(ref_h[:, sl])
        assert e < 1e-3, (sl, e)
    ref = om.tendency(Q0)
    dQ = dg.new_state(torch.float64)
    dg(dQ, Qp, None, 0.0)
    got = dQ.cpu().numpy()
    errs = [np.linalg.norm(got[:, sl] - ref[:, sl]) / np.linalg.norm(ref[:, sl])
            for sl in (slice(0, 1), slice(1, 4), slice(4, 5))]
    assert max(errs) < 1e-4, errs
    dt = om.courant_dt(Q0, 0.4)
    Qo, _ = om.lsrk54(Q0.copy(), dt, 30)
    lsrk = cmdg.LSRK54CarpenterKennedy(dg, Qp, dt=dt)
    cmdg.dostep_(Qp, lsrk, None, 0.0, nsteps=30)
    err, refn = om.field_l2(dg.from_perturbation(Qp).cpu().numpy(), Qo)
    err = np.array([err[0], np.sqrt(np.sum(err[1:4] ** 2)), err[4]])
    refn = np.array([refn[0], np.sqrt(np.sum(refn[1:4] ** 2)), refn[4]])
    assert (err / refn < 1e-5).all(), err / refn
