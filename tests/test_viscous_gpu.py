"""GPU parity of the diffusive passes (gradient flux, second-order fluxes)
against the oracle, for ConstantDynamicViscosity (with and without the
divergence term) and SmagorinskyLilly.

Bounds: FP64 <= 1e-10 of the field scale (gradient-flux groups grad h_tot, S
and N^2 scaled as vectors; momentum scaled as a vector); mixed precision
relative L2 <= 1e-4 for one tendency and <= 1e-5 for the state after steps.
"""
import numpy as np
import pytest
import torch

import cmdg
import oracle as O

pytestmark = pytest.mark.gpu

TOL64 = 1e-10
L = 2500.0


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g

    g.build()
    torch.cuda.set_device(0)


def pair(turb, N=4, ne=(3, 2, 4), precision="fp64", **kw):
    phys = dict(orientation="flat", gravity=True, ref_state=True, profile="dry_adiabatic", T_surface=300.0,
                T_min=0.0, turbulence=turb)
    phys.update(kw)
    om = O.OracleModel(N, ne, (0, 0, 0), (L, L, L), periodic=(1, 1, 0), **phys)
    grid = cmdg.BrickGrid(N, ne, (0, 0, 0), (L, L, L), periodicity=(True, True, False),
                          boundary=((0, 0), (0, 0), (1, 2)))
    model = cmdg.AtmosModel(orientation="flat", gravity=True,
                            ref_state=cmdg.HydrostaticState(cmdg.DryAdiabaticProfile(300.0, 0.0)),
                            turbulence=turb, rho_nu=kw.get("rho_nu", 0.0),
                            with_divergence=kw.get("with_divergence", False))
    dg = cmdg.DGModel(model, grid, precision=precision)
    Q0 = om.init_bubble(rc=900.0, xc=1100.0, yc=1300.0, zc=800.0)
    rng = np.random.default_rng(23)
    Q0[:, 1:4] += rng.uniform(-3, 3, size=Q0[:, 1:4].shape)
    return om, dg, Q0


def rel_groups(got, ref, groups):
    out = []
    for g in groups:
        sl = slice(g[0], g[-1] + 1)
        scale = np.abs(ref[:, sl]).max()
        out.append(np.abs(got[:, sl] - ref[:, sl]).max() / (scale if scale > 0 else 1.0))
    return np.array(out)


CASES = [("constant", dict(rho_nu=60.0)), ("constant", dict(rho_nu=60.0, with_divergence=True)),
         ("smagorinsky", {})]


@pytest.mark.parametrize("turb,kw", CASES)
def test_fp64_gradient_flux_matches_oracle(turb, kw):
    om, dg, Q0 = pair(turb, **kw)
    ref = om.gradient_pass(Q0)
    got = dg.gradient_flux(dg.init_ode_state(Q0)).cpu().numpy()
    groups = [(0, 1, 2), (3, 4, 5, 6, 7, 8)] + ([(9,)] if turb == "smagorinsky" else [])
    err = rel_groups(got[:, : ref.shape[1]], ref, groups)
    assert (err < TOL64).all(), err


@pytest.mark.parametrize("N", [3, 4, 5])
@pytest.mark.parametrize("turb,kw", CASES)
def test_fp64_viscous_tendency_matches_oracle(turb, kw, N):
    om, dg, Q0 = pair(turb, N=N, **kw)
    ref = om.tendency(Q0)
    dQ = dg.new_state(torch.float64)
    dg(dQ, dg.init_ode_state(Q0), None, 0.0)
    err = rel_groups(dQ.cpu().numpy(), ref, [(0,), (1, 2, 3), (4,)])
    assert (err < TOL64).all(), err


@pytest.mark.parametrize("turb,kw", CASES)
def test_fp64_viscous_steps_match_oracle(turb, kw):
    om, dg, Q0 = pair(turb, ne=(3, 3, 3), **kw)
    dt = 0.5 * om.courant_dt(Q0, 0.4)
    Qo, _ = om.lsrk54(Q0.copy(), dt, 5)
    Q = dg.init_ode_state(Q0)
    lsrk = cmdg.LSRK54CarpenterKennedy(dg, Q, dt=dt)
    cmdg.dostep_(Q, lsrk, None, 0.0, nsteps=5)
    err = rel_groups(Q.cpu().numpy(), Qo, [(0,), (1, 2, 3), (4,)])
    assert (err < TOL64).all(), err


@pytest.mark.parametrize("turb,kw", CASES)
def test_mixed_viscous_close_to_fp64_oracle(turb, kw):
    om, dg, Q0 = pair(turb, ne=(4, 3, 4), precision="mixed", **kw)
    ref = om.tendency(Q0)
    dQ = dg.new_state(torch.float64)
    Qp = dg.init_ode_state(Q0)
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


def test_les_workload_mixed_100_steps_within_1e5_of_fp64():
    """The Smagorinsky LES workload: 32 x 32 x 16 elements, N = 4, stable
    stratification N_bv = 0.01 1/s, seeded divergence-free k^-5/3 velocity of
    rms 1 m/s; mixed vs FP64 on the GPU after 100 LSRK54 steps at CFL 0.4."""
    from cmdg import workloads

    d64 = workloads.les_model(precision="fp64")
    dmx = workloads.les_model(precision="mixed")
    Q0 = workloads.les_initial_state(d64.grid.coordinates())
    Qa = d64.init_ode_state(Q0)
    dt = d64.courant_dt(Qa, 0.4)
    Qb = dmx.init_ode_state(Q0)
    cmdg.dostep_(Qa, cmdg.LSRK54CarpenterKennedy(d64, Qa, dt=dt), None, 0.0, nsteps=100)
    cmdg.dostep_(Qb, cmdg.LSRK54CarpenterKennedy(dmx, Qb, dt=dt), None, 0.0, nsteps=100)
    got = dmx.from_perturbation(Qb)
    M = torch.from_numpy(d64.grid.mass()).cuda()
    rel = []
    for sl in (slice(0, 1), slice(1, 4), slice(4, 5)):
        err = torch.sqrt((M[:, None] * (got[:, sl] - Qa[:, sl]) ** 2).sum())
        rel.append(float(err / torch.sqrt((M[:, None] * Qa[:, sl] ** 2).sum())))
    assert max(rel) < 1e-5, rel
    assert d64.status_word() == 0 and dmx.status_word() == 0
