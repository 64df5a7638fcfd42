"""Meshes given by the reference's own grid arrays (cmdg_mesh_create_arrays
+ cmdg_model_set_reference): the oracle's vgeo, vmap+ and elemtobndy -- in
the layouts of src/Numerics/Mesh/Grids.jl:76-125, 559-638 -- and its aux
values (Phi, grad Phi, rho_ref, rhoe_ref, p_ref) feed the GPU model, which
then reproduces the oracle's tendency and steps on a periodic brick, a
walled brick with gravity and a hydrostatic reference state, and the cubed
shell (arbitrary face orientations through the facing-node table).

Bounds as in the other parity tests: FP64 <= 1e-10 (bricks) / 1e-9 (shell)
of the field scale; mixed precision <= 1e-4 for one tendency and <= 1e-5
relative L2 after steps.  Also the turbulence closures on grid arrays, and
the manufactured-solution Navier-Stokes golden error of mms_bc_atmos.jl
reproduced on the GPU (cmdg_model_set_mms)."""
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


def aux7(om):
    a = om.aux
    A = O.AUX
    return np.stack([a[:, A["Phi"]], a[:, A["gPhi"]], a[:, A["gPhi"] + 1], a[:, A["gPhi"] + 2], a[:, A["rho_ref"]],
                     a[:, A["rhoe_ref"]], a[:, A["p_ref"]]], axis=1)


def arrays_model(om, N, model, numflux="rusanov", precision="fp64", set_ref=True):
    grid = cmdg.ArraysGrid(N, om.vgeo, om.vmapP + 1, om.elemtobndy)
    dg = cmdg.DGModel(model, grid, numerical_flux=numflux, precision=precision)
    if set_ref:
        dg.set_reference(aux7(om))
    return dg


def rel_max(got, ref):
    out = []
    for s in range(5):
        sl = slice(1, 4) if 1 <= s <= 3 else slice(s, s + 1)
        out.append(np.abs(got[:, s] - ref[:, s]).max() / np.abs(ref[:, sl]).max())
    return np.array(out)


def cases(kind, N, precision="fp64"):
    if kind == "vortex":
        L = 1 / 20
        om = O.OracleModel(N, (3, 2, 4), (-L,) * 3, (L,) * 3, periodic=(1, 1, 1))
        Q0 = om.init_vortex(0.0)
        return om, arrays_model(om, N, cmdg.AtmosModel(), precision=precision, set_ref=False), Q0, 1e-10
    if kind == "bubble":
        Lb = 2500.0
        om = O.OracleModel(N, (3, 2, 4), (0, 0, 0), (Lb, Lb, Lb), periodic=(1, 1, 0), orientation="flat",
                           gravity=True, ref_state=True, profile="dry_adiabatic", T_surface=300.0, T_min=0.0)
        model = cmdg.AtmosModel(orientation="flat", gravity=True,
                                ref_state=cmdg.HydrostaticState(cmdg.DryAdiabaticProfile(300.0, 0.0)))
        Q0 = om.init_bubble(rc=900.0, xc=1100.0, yc=1300.0, zc=800.0)
        Q0[:, 1:4] += np.random.default_rng(11).uniform(-2, 2, size=Q0[:, 1:4].shape)
        return om, arrays_model(om, N, model, precision=precision), Q0, 1e-10
    om = O.OracleModel(N, shell=dict(nhorz=2, nvert=3, r_inner=R, r_outer=R + 30e3), orientation="sphere",
                       gravity=True, ref_state=True, profile="isothermal", T_surface=285.0)
    model = cmdg.AtmosModel(orientation="sphere", gravity=True,
                            ref_state=cmdg.HydrostaticState(cmdg.IsothermalProfile(285.0)))
    Q0 = workloads.gcm_initial_state(om.aux[:, 0:3], seed=5)
    Q0[:, 1:4] += np.random.default_rng(3).uniform(-0.5, 0.5, size=Q0[:, 1:4].shape)
    return om, arrays_model(om, N, model, precision=precision), Q0, 1e-9


@pytest.mark.parametrize("N", [3, 4])
@pytest.mark.parametrize("kind", ["vortex", "bubble", "shell"])
def test_fp64_tendency_on_grid_arrays_matches_oracle(kind, N):
    om, dg, Q0, tol = cases(kind, N)
    ref = om.tendency(Q0)
    dQ = dg.new_state(torch.float64)
    dg(dQ, dg.init_ode_state(Q0), None, 0.0)
    err = rel_max(dQ.cpu().numpy(), ref)
    assert (err < tol).all(), err
    assert np.allclose(dg.grid.coordinates(), om.aux[:, 0:3], rtol=0, atol=1e-9 * np.abs(om.aux[:, 0:3]).max())


@pytest.mark.parametrize("kind", ["bubble", "shell"])
def test_fp64_steps_on_grid_arrays_match_oracle(kind):
    om, dg, Q0, tol = cases(kind, 4)
    dt = 0.5 * om.courant_dt(Q0, 0.4)
    assert dg.courant_dt(dg.init_ode_state(Q0), 0.4) == pytest.approx(om.courant_dt(Q0, 0.4), rel=1e-12)
    Qo, _ = om.lsrk54(Q0.copy(), dt, 5)
    Q = dg.init_ode_state(Q0)
    cmdg.dostep_(Q, cmdg.LSRK54CarpenterKennedy(dg, Q, dt=dt), None, 0.0, nsteps=5)
    err = rel_max(Q.cpu().numpy(), Qo)
    assert (err < tol).all(), err


@pytest.mark.parametrize("kind", ["bubble", "shell"])
def test_mixed_on_grid_arrays_close_to_fp64_oracle(kind):
    om, dg, Q0, _ = cases(kind, 4, precision="mixed")
    ref = om.tendency(Q0)
    Qp = dg.init_ode_state(Q0)
    dQ = dg.new_state(torch.float64)
    dg(dQ, Qp, None, 0.0)
    got = dQ.cpu().numpy()
    errs = [np.linalg.norm(got[:, sl] - ref[:, sl]) / np.linalg.norm(ref[:, sl])
            for sl in (slice(0, 1), slice(1, 4), slice(4, 5))]
    assert max(errs) < 1e-4, errs
    dt = om.courant_dt(Q0, 0.4)
    Qo, _ = om.lsrk54(Q0.copy(), dt, 30)
    cmdg.dostep_(Qp, cmdg.LSRK54CarpenterKennedy(dg, Qp, dt=dt), None, 0.0, nsteps=30)
    err, refn = om.field_l2(dg.from_perturbation(Qp).cpu().numpy(), Qo)
    err = np.array([err[0], np.sqrt(np.sum(err[1:4] ** 2)), err[4]])
    refn = np.array([refn[0], np.sqrt(np.sum(refn[1:4] ** 2)), refn[4]])
    assert (err / refn < 1e-5).all(), err / refn
    assert dg.status_word() == 0


def test_grid_arrays_errors():
    om, dg, Q0, _ = cases("bubble", 3)
    grid = cmdg.ArraysGrid(3, om.vgeo, om.vmapP + 1, om.elemtobndy)
    model = cmdg.AtmosModel(orientation="flat", gravity=True,
                            ref_state=cmdg.HydrostaticState(cmdg.DryAdiabaticProfile(300.0, 0.0)))
    dg2 = cmdg.DGModel(model, grid)
    dQ = dg2.new_state(torch.float64)
    with pytest.raises(cmdg.CmdgError, match="set_reference"):
        dg2(dQ, dg2.init_ode_state(Q0), None, 0.0)
    bad = om.vmapP + 1
    e_int = int(np.nonzero((om.elemtobndy == 0).all(axis=1))[0][0])
    bad[e_int, 0, 3] = bad[e_int, 1, 3]  # one node of face 1 faces another element
    with pytest.raises(cmdg.CmdgError, match="different elements"):
        cmdg.ArraysGrid(3, om.vgeo, bad, om.elemtobndy)
    bad2 = om.vmapP + 1
    bad2[0, 0, 0] = 10**12
    with pytest.raises(cmdg.CmdgError, match="out of range"):
        cmdg.ArraysGrid(3, om.vgeo, bad2, om.elemtobndy)


def viscous_case(kind, turb, N, precision="fp64"):
    """Closures on grid arrays: the warped (curvilinear) brick of the
    manufactured-solution test (mms_bc_atmos.jl mesh warp, walls on all
    sides, NoOrientation) or the cubed shell, with the oracle's own arrays."""
    rng = np.random.default_rng(21)
    if kind == "warped":
        om = O.OracleModel(N, (3, 3, 3), (0, 0, 0), (1, 1, 1), periodic=(0, 0, 0), warp=1, turbulence="constant",
                           rho_nu=0.01, with_divergence=True)
        model = cmdg.AtmosModel(turbulence="constant", rho_nu=0.01, with_divergence=True)
        xyz = om.aux[:, 0:3]
        Q0 = om.state()
        Q0[:, 0] = 1 + 0.1 * np.sin(2 * xyz[:, 0]) * np.cos(3 * xyz[:, 1])
        Q0[:, 1:4] = rng.uniform(-0.3, 0.3, size=Q0[:, 1:4].shape)
        Q0[:, 4] = 2.5e5 + 1e3 * np.cos(xyz[:, 2])
        return om, arrays_model(om, N, model, precision=precision, set_ref=False), Q0
    kw = dict(turbulence=turb) if turb == "smagorinsky" else dict(turbulence=turb, rho_nu=2e3)
    om = O.OracleModel(N, shell=dict(nhorz=2, nvert=3, r_inner=R, r_outer=R + 30e3), orientation="sphere",
                       gravity=True, ref_state=True, profile="isothermal", T_surface=285.0, **kw)
    model = cmdg.AtmosModel(orientation="sphere", gravity=True,
                            ref_state=cmdg.HydrostaticState(cmdg.IsothermalProfile(285.0)), **kw)
    Q0 = workloads.gcm_initial_state(om.aux[:, 0:3], seed=5)
    Q0[:, 1:4] += rng.uniform(-2, 2, size=Q0[:, 1:4].shape)
    return om, arrays_model(om, N, model, precision=precision), Q0


@pytest.mark.parametrize("kind,turb", [("warped", "constant"), ("shell", "constant"), ("shell", "smagorinsky")])
def test_closures_on_grid_arrays_match_oracle(kind, turb):
    """ConstantDynamicViscosity / SmagorinskyLilly on grid-arrays meshes
    (FP64): the tendency within 1e-9 of the field scale."""
    om, dg, Q0 = viscous_case(kind, turb, 3)
    ref = om.tendency(Q0)
    dQ = dg.new_state(torch.float64)
    dg(dQ, dg.init_ode_state(Q0), None, 0.0)
    err = rel_max(dQ.cpu().numpy(), ref)
    assert (err < 1e-9).all(), err


@pytest.mark.parametrize("kind,turb", [("warped", "constant"), ("shell", "constant"), ("shell", "smagorinsky")])
def test_closures_on_grid_arrays_mixed_close_to_oracle(kind, turb):
    """The closures on grid-arrays meshes in mixed precision: the gradient
    pass differentiates the perturbations h' and theta_v' about the caller's
    reference state, and the FP64 gradients of the reference parts (computed
    when the reference state is set) join them in the stage kernel.  One
    tendency within 1e-4 and 5 LSRK54 steps within 1e-5 of the FP64 oracle
    (relative L2 per field group: rho, momentum as a vector, rho e), as on
    the bricks.  The warped unit cube has no reference state, so its mixed
    form is FP32 about zero: the pressure gradient of rho e ~ 2.5e5 carries
    FP32's rounding of the full pressure into momentum (~2e-5 after the 5
    steps), and its stepped bar is 5e-5."""
    om, dg, Q0 = viscous_case(kind, turb, 3, precision="mixed")
    ref = om.tendency(Q0)
    Q = dg.init_ode_state(Q0)
    dQ = dg.new_state(torch.float64)
    dg(dQ, Q, None, 0.0)
    got = dQ.cpu().numpy()
    err = [np.linalg.norm(got[:, sl] - ref[:, sl]) / np.linalg.norm(ref[:, sl])
           for sl in (slice(0, 1), slice(1, 4), slice(4, 5))]
    assert max(err) < 1e-4, err
    if kind == "shell":
        # dt = 0.02 s, under the explicit diffusive limit of these 5000 km x
        # 10 km elements, from the GCM state without the velocity noise (its
        # node-to-node shear raises the Smagorinsky viscosity past the limit)
        dt = 0.02
        Q0 = workloads.gcm_initial_state(om.aux[:, 0:3], seed=5)
        Q = dg.init_ode_state(Q0)
    else:
        dt = 0.25 * om.courant_dt(Q0, 0.4)
    Qo, _ = om.lsrk54(Q0.copy(), dt, 5)
    assert np.isfinite(Qo).all()
    cmdg.dostep_(Q, cmdg.LSRK54CarpenterKennedy(dg, Q, dt=dt), None, 0.0, nsteps=5)
    err, nrm = om.field_l2(dg.from_perturbation(Q).cpu().numpy(), Qo)
    err = np.array([err[0], np.sqrt(np.sum(err[1:4] ** 2)), err[4]])
    nrm = np.array([nrm[0], np.sqrt(np.sum(nrm[1:4] ** 2)), nrm[4]])
    assert (err / nrm < (5e-5 if kind == "warped" else 1e-5)).all(), err / nrm
    assert dg.status_word() == 0


def test_mms_navier_stokes_golden_on_gpu():
    """mms_bc_atmos.jl, 3D, level 1, on the GPU: the oracle's warped [0, 1]^3
    brick (4^3 elements, N = 4) as grid arrays, ConstantDynamicViscosity(1/100,
    WithDivergence), T_0 = 0, the manufactured source and the exact state as
    the InitStateBC wall state (cmdg_model_set_mms) refreshed at every stage
    time, total_specific_enthalpy := 0; 800 LSRK54 steps to t = 1 driven from
    the host.  The weighted L2 distance to the exact solution reproduces the
    reference's golden value (its check is rtol sqrt(eps)).  The source and
    state come from tests/golden/mms_functions.py (generated from the
    symbolic derivation by tests/golden/make_mms_functions.py)."""
    import importlib.util
    import math
    import os
    from fractions import Fraction as Fr

    spec = importlib.util.spec_from_file_location(
        "mms_functions", os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "mms_functions.py"))
    G = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(G)
    om = O.OracleModel(4, (4, 4, 4), (0, 0, 0), (1, 1, 1), periodic=(0, 0, 0), bc_lo=(1, 1, 1), bc_hi=(1, 1, 1),
                       warp=1, mms=True, T_0=0.0, turbulence="constant", rho_nu=0.01, with_divergence=True)
    grid = cmdg.ArraysGrid(4, om.vgeo, om.vmapP + 1, om.elemtobndy)
    consts = dict(cmdg.EARTH)
    consts["T_0"] = 0.0
    dg = cmdg.DGModel(cmdg.AtmosModel(turbulence="constant", rho_nu=0.01, with_divergence=True, constants=consts),
                      grid)
    X = grid.coordinates()

    def ev(f, tt):
        return np.ascontiguousarray(np.stack(np.broadcast_arrays(*f(tt, X[:, 0], X[:, 1], X[:, 2])), axis=1))

    src = torch.zeros((grid.nelem, 5, grid.Np), dtype=torch.float64, device="cuda")
    wall = torch.zeros_like(src)
    dg.set_mms(src, wall, zero_enthalpy=True)
    A = [float(a) for a in (Fr(0), Fr(-567301805773, 1357537059087), Fr(-2404267990393, 2016746695238),
                            Fr(-3550918686646, 2091501179385), Fr(-1275806237668, 842570457699))]
    B = [float(b) for b in (Fr(1432997174477, 9575080441755), Fr(5161836677717, 13612068292357),
                            Fr(1720146321549, 2090206949498), Fr(3134564353537, 4481467310338),
                            Fr(2277821191437, 14882151754819))]
    C = [float(c) for c in (Fr(0), Fr(1432997174477, 9575080441755), Fr(2526269341429, 6820363962896),
                            Fr(2006345519317, 3224310063776), Fr(2802321613138, 2924317926251))]
    nsteps = math.ceil(1 / (5e-3 / 4))
    dt = 1 / nsteps
    Q = torch.from_numpy(ev(G.q, 0.0)).cuda()
    dQ = torch.zeros_like(Q)
    for step in range(nsteps):
        t0 = step * dt
        for s in range(5):
            ts = t0 + C[s] * dt
            src.copy_(torch.from_numpy(ev(G.source, ts)))
            wall.copy_(torch.from_numpy(ev(G.q, ts)))
            dg(dQ, Q, None, ts, alpha=1.0, beta=1.0)
            Q.add_(dQ, alpha=B[s] * dt)
            dQ.mul_(A[(s + 1) % 5])
    err = cmdg.euclidean_distance(dg, Q, ev(G.q, 1.0))
    assert err == pytest.approx(3.3983777728925593e-02, rel=1e-9), err
    assert dg.status_word() == 0


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_bubble_through_reference_ordered_arrays_matches_brick_path(precision):
    """The rising bubble as a Julia caller runs it: the brick's grid arrays in
    BrickTopology's Hilbert element order (workloads.brick_grid_arrays) with
    Phi = g z and the library's hydrostatic reference state, through
    cmdg_mesh_create_arrays.  Against the generated brick (stacked order,
    FP64), element by element through the permutation: FP64 tendency and
    5 LSRK54 steps within 1e-10 of the field scale; mixed tendency within
    1e-4 and 20 steps within 1e-5 (relative L2 per field group)."""
    ne, L = (4, 3, 5), 2500.0
    dga, perm, xyz = workloads.bubble_arrays_model(ne=ne, N=4, L=L, precision=precision)
    dgb = workloads.bubble_model(ne=ne, N=4, L=L, precision="fp64")
    xb = dgb.grid.coordinates()
    assert np.abs(xyz - xb[perm]).max() < 1e-9 * L
    Qb0 = workloads.rising_bubble(xb, theta0=300.0, amp=2.0, rc=500.0, center=(1250.0, 1250.0, 800.0))
    Qb0[:, 1:4] += np.random.default_rng(4).uniform(-1, 1, size=Qb0[:, 1:4].shape)
    Qa0 = np.ascontiguousarray(Qb0[perm])
    Qa, Qb = dga.init_ode_state(Qa0), dgb.init_ode_state(Qb0)
    Ta, Tb = dga.new_state(torch.float64), dgb.new_state(torch.float64)
    dga(Ta, Qa, None, 0.0)
    dgb(Tb, Qb, None, 0.0)
    ta, tb = Ta.cpu().numpy(), Tb.cpu().numpy()[perm]
    groups = (slice(0, 1), slice(1, 4), slice(4, 5))
    dt = dgb.courant_dt(Qb, 0.4)
    if precision == "fp64":
        assert (rel_max(ta, tb) < 1e-10).all(), rel_max(ta, tb)
        nsteps, tol = 5, None
    else:
        err = [np.linalg.norm(ta[:, g] - tb[:, g]) / np.linalg.norm(tb[:, g]) for g in groups]
        assert max(err) < 1e-4, err
        nsteps, tol = 20, 1e-5
    cmdg.dostep_(Qa, cmdg.LSRK54CarpenterKennedy(dga, Qa, dt=dt), None, 0.0, nsteps=nsteps)
    cmdg.dostep_(Qb, cmdg.LSRK54CarpenterKennedy(dgb, Qb, dt=dt), None, 0.0, nsteps=nsteps)
    qa, qb = dga.full_state(Qa).cpu().numpy(), Qb.cpu().numpy()[perm]
    if tol is None:
        assert (rel_max(qa, qb) < 1e-10).all(), rel_max(qa, qb)
    else:
        M = dgb.grid.mass()[perm]
        err = [np.sqrt(np.sum((qa[:, g] - qb[:, g]) ** 2 * M[:, None])) / np.sqrt(np.sum(qb[:, g] ** 2 * M[:, None]))
               for g in groups]
        assert max(err) < tol, err
    assert dga.status_word() == 0


def test_mixed_filter_on_grid_arrays_close_to_fp64():
    """A mixed-precision spectral filter on a mesh from grid arrays (the cubed
    shell's arrays): the FP32 perturbation filtered plus the per-node FP64
    change of the reference state, within 1e-6 (relative to each field
    group's scale) of the FP64 model's filter of the full state."""
    from cmdg import filters

    om, dg64, Q0, _ = cases("shell", 4)
    _, dgm, _, _ = cases("shell", 4, precision="mixed")
    filt = filters.ExponentialFilter(dg64.grid, 0, 18)
    Q = dg64.init_ode_state(Q0)
    filters.apply_(Q, (0, 1, 2, 3, 4), dg64, filt, "every")
    Qp = dgm.init_ode_state(Q0)
    filters.apply_(Qp, (0, 1, 2, 3, 4), dgm, filt, "every")
    got, ref = dgm.from_perturbation(Qp).cpu().numpy(), Q.cpu().numpy()
    for sl in (slice(0, 1), slice(1, 4), slice(4, 5)):
        assert np.abs(got[:, sl] - ref[:, sl]).max() <= 1e-6 * np.abs(ref[:, sl]).max()
