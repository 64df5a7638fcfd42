"""HEVI stepping on the GPU against the oracle and the reference's golden value.

* the vertical AtmosAcousticGravityLinearModel tendency (lineardg) on the
  cubed shell and on a wall-bounded brick, N = 2..5, within 1e-10 of the
  oracle per field (alpha / beta forms included; the momentum tendency is the
  small difference of the linearized pressure gradient and gravity, so its
  rounding is that of the larger terms);
* the column-LU backward Euler solve besolver!(Q, Qhat, alpha) against the
  oracle's band LU (1e-9), and its defining property Q - alpha L(Q) = Qhat
  checked with the GPU's own linear operator (1e-10);
* ARK2GiraldoKellyConstantinescu steps (full and split explicit parts)
  within 1e-9 of the oracle (per field, relative to the field's maximum;
  1e-8 for the momentum, an acoustic residual of cancelling terms);
* the acoustic wave of test/Numerics/DGMethods/Euler/acousticwave_1d_imex.jl
  (N = 5, 10 x 10 x 6 x 5 cubed-shell elements, 36 ARK2 steps of 100 s with
  ManyColumnLU and a vertical exponential filter of order 18): the norm of
  the state after one hour against the reference's golden value;
* the same with the explicit tendency on a mixed model's FP32 perturbation:
  the golden norm to 1e-9; rho, rhoe within 1e-6 and the momentum within
  5e-5 of the FP64 run;
* on a mesh from the reference's own grid arrays (stacks found from
  vmap+ / elemtobndy): linear tendency and ARK2 steps against the oracle;
* SingleColumnLU on an affine brick equals ManyColumnLU and is refused on
  the cubed shell;
* configuration errors (periodic columns, no reference state) are refused.
"""
import math

import numpy as np
import pytest
import torch

import cmdg
import oracle as O
from cmdg import workloads
from cmdg.filters import ExponentialFilter, apply_

pytestmark = pytest.mark.gpu

R = O.EARTH["planet_radius"]
GOLDEN_ACOUSTIC_WAVE = 9.5073452847149594e13  # acousticwave_1d_imex.jl, expected_result[Float64]


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g

    g.build()
    torch.cuda.set_device(0)


def shell_pair(N, nh, nv, H=10e3):
    om = O.OracleModel(N, shell=dict(nhorz=nh, nvert=nv, r_inner=R, r_outer=R + H), orientation="sphere",
                       gravity=True, ref_state=True, profile="isothermal", T_surface=300.0)
    dg = workloads.acoustic_wave_model(nhorz=nh, nvert=nv, N=N, H=H)
    Q0 = workloads.acoustic_wave_state(dg.grid.coordinates(), dg.reference_state()[:, 2], H=H)
    return om, dg, Q0


def brick_pair(N, ne=(2, 2, 4), L=(2000.0, 2000.0, 4000.0)):
    om = O.OracleModel(N, ne, (0, 0, 0), L, periodic=(1, 1, 0), orientation="flat", gravity=True, ref_state=True,
                       profile="dry_adiabatic", T_surface=300.0, T_min=0.0)
    grid = cmdg.BrickGrid(N, ne, (0, 0, 0), L, periodicity=(True, True, False))
    model = cmdg.AtmosModel(orientation="flat", gravity=True,
                            ref_state=cmdg.HydrostaticState(cmdg.DryAdiabaticProfile(300.0, 0.0)))
    dg = cmdg.DGModel(model, grid)
    Q0 = om.init_bubble(rc=600.0, xc=L[0] / 2, yc=L[1] / 2, zc=L[2] / 3)
    rng = np.random.default_rng(7)
    Q0[:, 1:4] += rng.uniform(-1, 1, size=Q0[:, 1:4].shape)
    return om, dg, Q0


def linear_dg(dg):
    return cmdg.DGModel(cmdg.AtmosAcousticGravityLinearModel(dg.balance_law), dg.grid, direction="vertical",
                        state_auxiliary=dg)


def rel_fields(got, ref):
    out = []
    for s in range(5):
        sl = slice(1, 4) if 1 <= s <= 3 else slice(s, s + 1)
        scale = max(np.abs(ref[:, sl]).max(), 1e-300)
        out.append(np.abs(got[:, s] - ref[:, s]).max() / scale)
    return np.array(out)


@pytest.mark.parametrize("N", [2, 3, 4, 5])
def test_shell_linear_tendency_matches_oracle(N):
    om, dg, Q0 = shell_pair(N, 2, 3)
    rng = np.random.default_rng(N)
    Q0[:, 1:4] += rng.uniform(-2, 2, size=Q0[:, 1:4].shape)
    ref = om.linear_tendency(Q0)
    lin = linear_dg(dg)
    Q = dg.init_ode_state(Q0)
    dQ = dg.new_state(torch.float64)
    lin(dQ, Q, None, 0.0)
    err = rel_fields(dQ.cpu().numpy(), ref)
    assert err.max() < 1e-10, err
    # alpha / beta form: dQ = 0.5 L(Q) - 2 dQ
    ref2 = om.linear_tendency(Q0, alpha=0.5, beta=-2.0, dQ=ref.copy())
    lin(dQ, Q, None, 0.0, alpha=0.5, beta=-2.0)
    err = rel_fields(dQ.cpu().numpy(), ref2)
    assert err.max() < 1e-10, err


@pytest.mark.parametrize("N", [2, 4])
def test_brick_linear_tendency_matches_oracle(N):
    om, dg, Q0 = brick_pair(N)
    ref = om.linear_tendency(Q0)
    lin = linear_dg(dg)
    Q = dg.init_ode_state(Q0)
    dQ = dg.new_state(torch.float64)
    lin(dQ, Q, None, 0.0)
    err = rel_fields(dQ.cpu().numpy(), ref)
    assert err.max() < 1e-10, err


def test_column_lu_solve_matches_oracle_and_inverts_the_operator():
    om, dg, Q0 = shell_pair(4, 2, 4)
    dt = 50.0
    ohv = O.OracleHevi(om, dt)
    lin = linear_dg(dg)
    ark = cmdg.ARK2GiraldoKellyConstantinescu(dg, lin, cmdg.LinearBackwardEulerSolver(cmdg.ManyColumnLU()),
                                              dg.init_ode_state(Q0), dt=dt)
    assert ark.alpha == pytest.approx(ohv.alpha, rel=1e-15)
    assert ark.bandwidth == ohv.bandwidth == 5 * 5 - 1
    rng = np.random.default_rng(11)
    Qhat0 = Q0 + rng.uniform(-1e-3, 1e-3, size=Q0.shape) * np.abs(Q0).max(axis=2, keepdims=True)
    Qhat0[:, 1:4] = rng.uniform(-1, 1, size=Qhat0[:, 1:4].shape)
    ref = ohv.solve(Qhat0)
    Qhat = dg.init_ode_state(Qhat0)
    Q = dg.new_state(torch.float64)
    ark.backward_euler_solve(Q, Qhat)
    got = Q.cpu().numpy()
    assert rel_fields(got, ref).max() < 1e-9
    # Q - alpha L(Q) = Qhat with the GPU's own operator
    LQ = dg.new_state(torch.float64)
    lin(LQ, Q, None, 0.0)
    res = (Q - ark.alpha * LQ - Qhat).cpu().numpy()
    assert rel_fields(res + Qhat0, Qhat0).max() < 1e-10
    # in place (Q aliases Qhat)
    ark.backward_euler_solve(Qhat, Qhat)
    assert torch.equal(Qhat, Q)


@pytest.mark.parametrize("split", [False, True])
def test_ark2_steps_match_oracle(split):
    om, dg, Q0 = shell_pair(3, 3, 3)
    dt = 60.0
    ohv = O.OracleHevi(om, dt, split_explicit_implicit=split)
    ref = ohv.step(Q0.copy(), 3)
    lin = linear_dg(dg)
    F = cmdg.remainder_DGModel(dg, (lin,)) if split else dg
    Q = dg.init_ode_state(Q0)
    ark = cmdg.ARK2GiraldoKellyConstantinescu(F, lin, cmdg.LinearBackwardEulerSolver(cmdg.ManyColumnLU()), Q,
                                              dt=dt, split_explicit_implicit=split)
    cmdg.dostep_(Q, ark, None, 0.0, 3)
    got = Q.cpu().numpy()
    dev = got - Q0
    refdev = ref - Q0
    err = rel_fields(got, ref)
    # rho, rhoe to 1e-9; the momentum is a small acoustic residual of large
    # cancelling pressure-gradient and gravity terms (the remainder f - l of
    # the split form subtracts two of them), so its rounding is held to 1e-8
    assert err[[0, 4]].max() < 1e-9 and err[1:4].max() < 1e-8, err
    # the change over the steps (what the scheme computes) to 1e-7 of its size
    for s in (0, 4):
        assert np.abs(dev[:, s] - refdev[:, s]).max() < 1e-7 * np.abs(refdev[:, s]).max()


def test_brick_ark2_steps_match_oracle():
    om, dg, Q0 = brick_pair(3)
    dt = 0.5
    ohv = O.OracleHevi(om, dt)
    ref = ohv.step(Q0.copy(), 4)
    lin = linear_dg(dg)
    Q = dg.init_ode_state(Q0)
    ark = cmdg.ARK2GiraldoKellyConstantinescu(dg, lin, cmdg.LinearBackwardEulerSolver(cmdg.ManyColumnLU()), Q,
                                              dt=dt)
    cmdg.dostep_(Q, ark, None, 0.0, 4)
    assert rel_fields(Q.cpu().numpy(), ref).max() < 1e-9


def test_single_column_lu_on_an_affine_brick():
    """SingleColumnLU (one factorization for every node column) on a brick,
    whose column matrices agree: the same steps as ManyColumnLU to rounding
    and as the oracle; refused on the cubed shell, whose columns differ."""
    om, dg, Q0 = brick_pair(3)
    dt = 0.5
    lin = linear_dg(dg)
    out = []
    for solver in (cmdg.ManyColumnLU(), cmdg.SingleColumnLU()):
        Q = dg.init_ode_state(Q0)
        ark = cmdg.ARK2GiraldoKellyConstantinescu(dg, lin, cmdg.LinearBackwardEulerSolver(solver), Q, dt=dt)
        cmdg.dostep_(Q, ark, None, 0.0, 4)
        out.append(Q.cpu().numpy())
    assert rel_fields(out[1], out[0]).max() < 1e-12
    ref = O.OracleHevi(om, dt).step(Q0.copy(), 4)
    assert rel_fields(out[1], ref).max() < 1e-9
    _, dgs, Qs0 = shell_pair(3, 2, 2)
    lins = linear_dg(dgs)
    with pytest.raises(cmdg.CmdgError):
        cmdg.ARK2GiraldoKellyConstantinescu(dgs, lins, cmdg.LinearBackwardEulerSolver(cmdg.SingleColumnLU()),
                                            dgs.init_ode_state(Qs0), dt=10.0)


@pytest.mark.parametrize("split", [False, True])
def test_acoustic_wave_hevi_golden(split):
    """acousticwave_1d_imex.jl (Float64): ||Q|| after one hour.  The reference
    compares at rtol sqrt(eps); its model also carries a passive tracer
    rho chi = 1, whose weighted norm (the square root of the shell volume) is
    3e-10 of ||Q|| and below that tolerance -- the golden value agrees with
    the norm of the five dry fields, which is what is compared here."""
    dg = workloads.acoustic_wave_model()
    dt, nsteps = workloads.acoustic_wave_dt()
    assert (dt, nsteps) == (100.0, 36)
    Q0 = workloads.acoustic_wave_state(dg.grid.coordinates(), dg.reference_state()[:, 2])
    Q = dg.init_ode_state(Q0)
    lin = linear_dg(dg)
    F = cmdg.remainder_DGModel(dg, (lin,)) if split else dg
    ark = cmdg.ARK2GiraldoKellyConstantinescu(F, lin, cmdg.LinearBackwardEulerSolver(cmdg.ManyColumnLU()), Q,
                                              dt=dt, split_explicit_implicit=split)
    filt = ExponentialFilter(dg.grid, 0, 18)

    def cbfilter(solver, Q):
        apply_(Q, (0, 1, 2, 3, 4), dg, filt, direction="vertical")

    cmdg.solve_(Q, ark, numberofsteps=nsteps, adjustfinalstep=False, callbacks=(cbfilter,))
    assert ark.steps == nsteps
    n = cmdg.norm(dg, Q)
    assert abs(n / GOLDEN_ACOUSTIC_WAVE - 1) < 1e-11, n


@pytest.mark.parametrize("split", [False, True])
def test_mixed_explicit_part_acoustic_wave_golden(split):
    """HEVI with the explicit tendency of a mixed model: on the cubed shell the
    fused remainder kernel forms f - l on the FP32 perturbation and the FP64
    linear kernel adds l of the FP64 perturbation (split: f - l(Q) = (f -
    l)(q') - l(q_ref)).  The one-hour acoustic wave keeps the golden norm to
    1e-9 (the reference's own check is rtol sqrt(eps) = 1.5e-8) and stays
    within 1e-7 (rho, rho e) and 1e-5 (momentum) of the FP64 run (relative
    L2 per field group)."""
    dt, nsteps = workloads.acoustic_wave_dt()
    out = {}
    for precision in ("fp64", "mixed"):
        dg = workloads.acoustic_wave_model(precision=precision)
        Q0 = workloads.acoustic_wave_state(dg.grid.coordinates(), dg.reference_state()[:, 2])
        Q = torch.from_numpy(Q0).to("cuda")
        lin = linear_dg(dg)
        F = cmdg.remainder_DGModel(dg, (lin,)) if split else dg
        ark = cmdg.ARK2GiraldoKellyConstantinescu(F, lin, cmdg.LinearBackwardEulerSolver(cmdg.ManyColumnLU()), Q,
                                                  dt=dt, split_explicit_implicit=split)
        filt = ExponentialFilter(dg.grid, 0, 18)

        def cbfilter(solver, Q, dg=dg, filt=filt):
            apply_(Q, (0, 1, 2, 3, 4), dg, filt, direction="vertical")

        # the filter of a mixed model acts on its FP32 perturbation: filter a
        # FP64 model's copy of the state instead, so both runs filter alike
        if precision == "mixed":
            dg64 = workloads.acoustic_wave_model()

            def cbfilter(solver, Q, dg64=dg64, filt=filt):  # noqa: F811
                apply_(Q, (0, 1, 2, 3, 4), dg64, filt, direction="vertical")

        cmdg.solve_(Q, ark, numberofsteps=nsteps, adjustfinalstep=False, callbacks=(cbfilter,))
        out[precision] = (dg, Q)
    dg64, Q64 = out["fp64"]
    n = cmdg.norm(dg64, out["mixed"][1])
    assert abs(n / GOLDEN_ACOUSTIC_WAVE - 1) < 1e-9, n
    a, b = out["mixed"][1].cpu().numpy(), Q64.cpu().numpy()
    M = dg64.grid.mass()
    rel = []
    for sl in (slice(0, 1), slice(1, 4), slice(4, 5)):
        err = math.sqrt(float(np.sum((a[:, sl] - b[:, sl]) ** 2 * M[:, None, :])))
        rel.append(err / math.sqrt(float(np.sum(b[:, sl] ** 2 * M[:, None, :]))))
    assert rel[0] < 1e-7 and rel[1] < 1e-5 and rel[2] < 1e-7, rel


def test_hevi_on_the_reference_grid_arrays():
    """The oracle's own vgeo, vmap+ and elemtobndy of a stacked cubed shell and
    its aux values (cmdg_mesh_create_arrays + cmdg_model_set_reference): the
    stacks are found from the arrays, the linear tendency and three ARK2
    steps match the oracle."""
    N, H = 3, 10e3
    om = O.OracleModel(N, shell=dict(nhorz=2, nvert=3, r_inner=R, r_outer=R + H), orientation="sphere",
                       gravity=True, ref_state=True, profile="isothermal", T_surface=300.0)
    a, A = om.aux, O.AUX
    aux7 = np.stack([a[:, A["Phi"]], a[:, A["gPhi"]], a[:, A["gPhi"] + 1], a[:, A["gPhi"] + 2], a[:, A["rho_ref"]],
                     a[:, A["rhoe_ref"]], a[:, A["p_ref"]]], axis=1)
    grid = cmdg.ArraysGrid(N, om.vgeo, om.vmapP + 1, om.elemtobndy)
    model = cmdg.AtmosModel(orientation="sphere", gravity=True,
                            ref_state=cmdg.HydrostaticState(cmdg.IsothermalProfile(300.0)))
    dg = cmdg.DGModel(model, grid)
    lin = linear_dg(dg)
    Q0 = workloads.acoustic_wave_state(om.vgeo[:, 12:15], a[:, A["p_ref"]], H=H)
    Q = dg.init_ode_state(Q0)
    dQ = dg.new_state(torch.float64)
    with pytest.raises(cmdg.CmdgError):  # the reference state is not set yet
        lin(dQ, Q, None, 0.0)
    dg.set_reference(aux7)
    rng = np.random.default_rng(12)
    Qn = Q0.copy()
    Qn[:, 1:4] += rng.uniform(-2, 2, size=Qn[:, 1:4].shape)
    lin(dQ, dg.init_ode_state(Qn), None, 0.0)
    assert rel_fields(dQ.cpu().numpy(), om.linear_tendency(Qn)).max() < 1e-10
    dt = 60.0
    ref = O.OracleHevi(om, dt).step(Q0.copy(), 3)
    ark = cmdg.ARK2GiraldoKellyConstantinescu(dg, lin, cmdg.LinearBackwardEulerSolver(cmdg.ManyColumnLU()), Q,
                                              dt=dt)
    cmdg.dostep_(Q, ark, None, 0.0, 3)
    err = rel_fields(Q.cpu().numpy(), ref)
    assert err[[0, 4]].max() < 1e-9 and err[1:4].max() < 1e-8, err


def test_hevi_configuration_errors():
    # periodic columns have no wall-bounded stacks
    grid = cmdg.BrickGrid(3, (2, 2, 2), (0, 0, 0), (1000.0, 1000.0, 1000.0), periodicity=(True, True, True))
    model = cmdg.AtmosModel(orientation="flat", gravity=True, ref_state=cmdg.HydrostaticState())
    dgp = cmdg.DGModel(model, grid)
    lin = linear_dg(dgp)
    Q = dgp.new_state()
    with pytest.raises(cmdg.CmdgError):
        cmdg.ARK2GiraldoKellyConstantinescu(dgp, lin, cmdg.LinearBackwardEulerSolver(cmdg.ManyColumnLU()), Q, dt=1.0)
    # no reference state
    with pytest.raises(ValueError):
        cmdg.AtmosAcousticGravityLinearModel(cmdg.AtmosModel())
