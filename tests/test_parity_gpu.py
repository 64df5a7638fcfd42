"""GPU parity of the fused DG tendency / LSRK54 kernels against the oracle.

Every case feeds the same seeded FP64 state to the oracle (CPU restatement of
the reference) and to libcmdg.so through the C ABI, and compares:

  * FP64 tendency: max |gpu - oracle| / max |oracle| per field <= 1e-10
    (reassociated sums of O(1e5)-sized fluxes; the reference's own CPU/GPU
    check allows sqrt(eps), mms_bc_atmos.jl:152)
  * FP64 LSRK54 steps: the same bound on the state after K steps
  * mixed precision: relative L2 per field against the FP64 oracle
    (<= 1e-5 after the run, the stated target)
"""
import math

import numpy as np
import pytest
import torch

import cmdg
import oracle as O
from cmdg import workloads

pytestmark = pytest.mark.gpu

TOL64 = 1e-10
# stage-kernel configurations: one CTA per element, a resident wave walking
# the elements, one thread per vertical line of nodes
KERNELS = {"node": ("node", -1), "persistent": ("node", 0), "column": ("column", 0), "lines": ("lines", -1)}


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g

    g.build()
    torch.cuda.set_device(0)


def rel_max(got, ref):
    """max |got - ref| per field, relative to the field's largest magnitude;
    the three momentum components are scaled together as one vector field
    (a component that is zero up to noise, like rho*w in the vortex, is a
    difference of O(p) terms and carries their rounding)."""
    out = []
    for s in range(5):
        sl = slice(1, 4) if 1 <= s <= 3 else slice(s, s + 1)
        scale = np.abs(ref[:, sl]).max()
        out.append(np.abs(got[:, s] - ref[:, s]).max() / (scale if scale > 0 else 1.0))
    return np.array(out)


def make_pair(kind, N, ne, numflux="rusanov", precision="fp64"):
    if kind == "vortex":
        L = 1 / 20
        om = O.OracleModel(N, ne, (-L,) * 3, (L,) * 3, periodic=(1, 1, 1), numflux=numflux)
        grid = cmdg.BrickGrid(N, ne, (-L,) * 3, (L,) * 3, periodicity=(True, True, True))
        model = cmdg.AtmosModel()
        dg = cmdg.DGModel(model, grid, numerical_flux=numflux, precision=precision)
        Q0 = om.init_vortex(0.0)
        rng = np.random.default_rng(7)
        Q0 += rng.uniform(-1e-6, 1e-6, size=Q0.shape)
    else:
        Lb = 2500.0
        om = O.OracleModel(N, ne, (0, 0, 0), (Lb, Lb, Lb), periodic=(1, 1, 0), numflux=numflux, orientation="flat",
                           gravity=True, ref_state=True, profile="dry_adiabatic", T_surface=300.0, T_min=0.0)
        dg = workloads.bubble_model(ne=ne, N=N, L=Lb, precision=precision, numerical_flux=numflux)
        Q0 = om.init_bubble(rc=900.0, xc=1100.0, yc=1300.0, zc=800.0)
        rng = np.random.default_rng(11)
        Q0[:, 1:4] += rng.uniform(-2, 2, size=Q0[:, 1:4].shape)
    return om, dg, Q0


@pytest.mark.parametrize("kernel", ["node", "lines"])
@pytest.mark.parametrize("N", [2, 3, 4, 5])
@pytest.mark.parametrize("kind", ["vortex", "bubble"])
def test_fp64_tendency_matches_oracle(kind, N, kernel):
    om, dg, Q0 = make_pair(kind, N, (3, 2, 4))
    dg.set_kernel(*KERNELS[kernel])
    ref = om.tendency(Q0)
    Q = dg.init_ode_state(Q0)
    dQ = dg.new_state(torch.float64)
    dg(dQ, Q, None, 0.0)
    err = rel_max(dQ.cpu().numpy(), ref)
    assert (err < TOL64).all(), err


@pytest.mark.parametrize("kernel", ["node", "lines"])
def test_fp64_central_flux_and_alpha_beta(kernel):
    om, dg, Q0 = make_pair("bubble", 4, (2, 3, 3), numflux="central")
    dg.set_kernel(*KERNELS[kernel])
    prev = np.random.default_rng(3).standard_normal(Q0.shape)
    ref = om.tendency(Q0, alpha=0.7, beta=-1.3, dQ=prev.copy())
    Q = dg.init_ode_state(Q0)
    dQ = torch.from_numpy(prev.copy()).cuda()
    dg(dQ, Q, None, 0.0, alpha=0.7, beta=-1.3)
    err = rel_max(dQ.cpu().numpy(), ref)
    assert (err < TOL64).all(), err


@pytest.mark.parametrize("kernel", ["node", "lines"])
@pytest.mark.parametrize("kind", ["vortex", "bubble"])
def test_fp64_lsrk54_steps_match_oracle(kind, kernel):
    om, dg, Q0 = make_pair(kind, 4, (3, 3, 3))
    dg.set_kernel(*KERNELS[kernel])
    dt = 0.5 * om.courant_dt(Q0, 0.4)
    Qo, dQo = om.lsrk54(Q0.copy(), dt, 7)
    Q = dg.init_ode_state(Q0)
    lsrk = cmdg.LSRK54CarpenterKennedy(dg, Q, dt=dt)
    cmdg.dostep_(Q, lsrk, None, 0.0, nsteps=4)
    # A_1 = 0: a step never reads what the register held before it
    lsrk.dQ.fill_(1.0e30)
    cmdg.dostep_(Q, lsrk, None, 0.0, nsteps=3)
    got = Q.cpu().numpy()
    err = rel_max(got, Qo)
    assert (err < TOL64).all(), err


def test_isentropic_vortex_golden_through_gpu():
    """The reference's golden FP64 error (isentropicvortex.jl:105) via libcmdg."""
    L = 1 / 20
    ne = (5, 5, 1)
    grid = cmdg.BrickGrid(4, ne, (-L,) * 3, (L,) * 3)
    dg = cmdg.DGModel(cmdg.AtmosModel(), grid)
    xyz = grid.coordinates()
    Q = dg.init_ode_state(workloads.isentropic_vortex(xyz, 0.0))
    c = cmdg.EARTH
    timeend = 2 * L / 10 / 150
    dt = (2 * L / 5) / math.sqrt(c["cp_d"] / c["cv_d"] * c["R_d"] * 300.0) / 16
    dt = timeend / math.ceil(timeend / dt)
    lsrk = cmdg.LSRK54CarpenterKennedy(dg, Q, dt=dt)
    cmdg.solve_(Q, lsrk, timeend=timeend)
    err = cmdg.euclidean_distance(dg, Q, workloads.isentropic_vortex(xyz, timeend))
    assert err == pytest.approx(3.7918869862613858e00, rel=1e-10)


def test_c1_vortex_configuration_matches_oracle():
    """The plain CPU-runnable configuration as stated: periodic [0, 10]^3,
    4 x 4 x 4 elements, N = 4, dry Euler without gravity or viscosity,
    Rusanov, an isentropic vortex of strength 5 and radius 1 advected
    diagonally at Mach 0.5 with 1e-6 seeded noise; one tendency and then 10
    LSRK54 steps at CFL 0.4, FP64 GPU against the FP64 oracle."""
    ne, N = (4, 4, 4), 4
    om = O.OracleModel(N, ne, (0, 0, 0), (10, 10, 10), periodic=(1, 1, 1))
    grid = cmdg.BrickGrid(N, ne, (0, 0, 0), (10, 10, 10), periodicity=(True, True, True))
    dg = cmdg.DGModel(cmdg.AtmosModel(), grid)
    Q0 = workloads.c1_vortex_state(grid.coordinates())
    ref = om.tendency(Q0)
    Q = dg.init_ode_state(Q0)
    dQ = dg.new_state(torch.float64)
    dg(dQ, Q, None, 0.0)
    err = rel_max(dQ.cpu().numpy(), ref)
    assert (err < TOL64).all(), err
    dt = om.courant_dt(Q0, 0.4)
    assert dg.courant_dt(Q, 0.4) == pytest.approx(dt, rel=1e-12)
    Qo, _ = om.lsrk54(Q0.copy(), dt, 10)
    lsrk = cmdg.LSRK54CarpenterKennedy(dg, Q, dt=dt)
    cmdg.dostep_(Q, lsrk, None, 0.0, nsteps=10)
    err = rel_max(Q.cpu().numpy(), Qo)
    assert (err < TOL64).all(), err
    assert np.isfinite(Qo).all() and dg.status_word() == 0


@pytest.mark.parametrize("kernel", ["node", "persistent", "column", "lines"])
@pytest.mark.parametrize("N", [3, 4, 5])
def test_mixed_tendency_close_to_oracle(kernel, N):
    om, dg, Q0 = make_pair("bubble", N, (3, 3, 4), precision="mixed")
    dg.set_kernel(*KERNELS[kernel])
    ref = om.tendency(Q0)
    Qp = dg.init_ode_state(Q0)
    dQ = dg.new_state(torch.float64)
    dg(dQ, Qp, None, 0.0)
    got = dQ.cpu().numpy()
    err = [np.linalg.norm(got[:, s] - ref[:, s]) / np.linalg.norm(ref[:, s]) for s in range(5)]
    assert max(err) < 1e-4, err


@pytest.mark.parametrize("kernel", ["node", "persistent", "column", "lines"])
def test_mixed_bubble_100_steps_within_1e5_of_fp64_oracle(kernel):
    om, dg, Q0 = make_pair("bubble", 4, (4, 4, 4), precision="mixed")
    dg.set_kernel(*KERNELS[kernel])
    dt = om.courant_dt(Q0, 0.4)
    Qo, _ = om.lsrk54(Q0.copy(), dt, 100)
    Qp = dg.init_ode_state(Q0)
    lsrk = cmdg.LSRK54CarpenterKennedy(dg, Qp, dt=dt)
    cmdg.dostep_(Qp, lsrk, None, 0.0, nsteps=100)
    got = dg.from_perturbation(Qp).cpu().numpy()
    err, ref = om.field_l2(got, Qo)
    rel = err / ref
    assert (rel < 1e-5).all(), rel
    # conservation of mass through the compensated sums
    m_gpu = dg.weighted_sums(Qp, (0,))[0]
    assert m_gpu == pytest.approx(om.weightedsum(Qo, 0), rel=1e-9)


def test_weighted_sums_and_courant_match_oracle():
    om, dg, Q0 = make_pair("bubble", 3, (2, 2, 3))
    Q = dg.init_ode_state(Q0)
    sums = dg.weighted_sums(Q, (0, 4))
    assert sums[0] == pytest.approx(om.weightedsum(Q0, 0), rel=1e-14)
    assert sums[1] == pytest.approx(om.weightedsum(Q0, 4), rel=1e-14)
    assert dg.courant_dt(Q, 0.4) == pytest.approx(om.courant_dt(Q0, 0.4), rel=1e-12)


def test_fp64_discrete_hydrostatic_balance_central():
    H = 50e3
    grid = cmdg.BrickGrid(4, (3, 3, 3), (0, 0, 0), (H, H, H), periodicity=(True, True, False),
                          boundary=((0, 0), (0, 0), (1, 2)))
    model = cmdg.AtmosModel(orientation="flat", gravity=True,
                            ref_state=cmdg.HydrostaticState(cmdg.IsothermalProfile(285.0), subtract_off=False))
    dg = cmdg.DGModel(model, grid, numerical_flux="central")
    ref = dg.reference_state()
    Q0 = np.zeros((grid.nelem, 5, grid.Np))
    Q0[:, 0] = ref[:, 0]
    Q0[:, 4] = ref[:, 1]
    Q = dg.init_ode_state(Q0)
    dt = dg.courant_dt(Q, 0.1)
    lsrk = cmdg.LSRK54CarpenterKennedy(dg, Q, dt=dt)
    cmdg.solve_(Q, lsrk, timeend=100.0)
    err = cmdg.euclidean_distance(dg, Q, Q0) / cmdg.norm(dg, torch.from_numpy(Q0).cuda())
    assert err <= 100 * np.finfo(np.float64).eps


def test_nonfinite_state_sets_status_word_without_fault():
    om, dg, Q0 = make_pair("vortex", 3, (2, 2, 2))
    Q0[0, 0, 5] = np.nan
    Q = dg.init_ode_state(Q0)
    dQ = dg.new_state(torch.float64)
    dg(dQ, Q, None, 0.0)
    torch.cuda.synchronize()
    assert dg.status_word() & 1
    assert dg.status_word() == 0  # reading clears it


def test_fp64_steps_are_bitwise_deterministic():
    om, dg, Q0 = make_pair("bubble", 4, (3, 3, 3))
    outs = []
    for _ in range(2):
        Q = dg.init_ode_state(Q0)
        lsrk = cmdg.LSRK54CarpenterKennedy(dg, Q, dt=0.05)
        cmdg.dostep_(Q, lsrk, None, 0.0, nsteps=3)
        outs.append(Q.cpu().numpy())
    assert np.array_equal(outs[0], outs[1])


@pytest.mark.parametrize("kind", ["vortex", "bubble"])
def test_mixed_kernels_agree_and_autotune_keeps_results(kind):
    """Both stage-kernel families give the same mixed-precision steps up to
    FP32 reassociation, and the autotuner only changes speed."""
    om, dg, Q0 = make_pair(kind, 4, (5, 4, 6), precision="mixed")
    dt = 0.5 * om.courant_dt(Q0, 0.4)
    outs = {}
    for kernel in ("node", "persistent", "column", "lines"):
        dg.set_kernel(*KERNELS[kernel])
        Qp = dg.init_ode_state(Q0)
        lsrk = cmdg.LSRK54CarpenterKennedy(dg, Qp, dt=dt)
        cmdg.dostep_(Qp, lsrk, None, 0.0, nsteps=5)
        outs[kernel] = dg.from_perturbation(Qp).cpu().numpy()
    for other in ("persistent", "column", "lines"):
        err, ref = om.field_l2(outs["node"], outs[other])
        # momentum as one vector field (rho*w of the vortex is noise-sized)
        err = np.array([err[0], np.sqrt(np.sum(err[1:4] ** 2)), err[4]])
        ref = np.array([ref[0], np.sqrt(np.sum(ref[1:4] ** 2)), ref[4]])
        assert (err / ref < 1e-6).all(), (other, err / ref)
    ms, choice = dg.autotune(reps=3)
    # node (resident wave, one CTA per element), lines, column, and clusters
    # of 2 (z) elements: the 5 x 4 x 6 brick is odd in x
    assert len(ms) == 5 and all(m > 0 for m in ms)
    assert choice[0] in ("node", "column", "lines", "cluster")
    assert dg.status_word() == 0


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("grid", [0, 7])
def test_persistent_kernel_bitwise_equals_one_cta_per_element(precision, grid):
    """The persistent kernel stages each element's state and RK register
    with bulk copies into a two-buffer ring (plain loads for an element whose
    16-byte-aligned window would leave the array, e.g. the last of 27) and
    computes exactly what the one-CTA-per-element kernel computes, for a
    resident wave (grid 0) and for 7 CTAs walking ~4 elements each."""
    om, dg, Q0 = make_pair("bubble", 4, (3, 3, 3), precision=precision)
    outs, tends = [], []
    for kernel in (("node", -1), ("node", grid)):
        dg.set_kernel(*kernel)
        Q = dg.init_ode_state(Q0)
        lsrk = cmdg.LSRK54CarpenterKennedy(dg, Q, dt=0.05)
        cmdg.dostep_(Q, lsrk, None, 0.0, nsteps=3)
        outs.append(Q.cpu().numpy())
        dQ = torch.ones(Q.shape, dtype=torch.float64, device=Q.device)
        dg(dQ, Q, None, 0.0, 0.5, 0.25)  # tendency with the register read (beta != 0)
        tends.append(dQ.cpu().numpy())
    assert np.array_equal(outs[0], outs[1])
    assert np.array_equal(tends[0], tends[1])
    assert dg.status_word() == 0


@pytest.mark.parametrize("ne", [(3, 3, 3), (1, 1, 3), (1, 1, 1), (5, 1, 1)])
def test_host_state_steps_equal_device_steps(ne):
    """cmdg_lsrk54_step_mixed_host (the state in pinned host memory, copied
    over the host link in element chunks that overlap the conversions)
    gives the same bits as converting on the device and stepping, also on
    meshes with fewer elements than chunks or a count the chunks do not
    divide; pageable memory is refused; a step count of zero converts and
    copies back only."""
    import ctypes

    from cmdg import _lib

    om, dg, Q0 = make_pair("bubble", 4, ne, precision="mixed")
    h0 = torch.from_numpy(Q0.copy()).pin_memory()
    Qz = dg.new_state(torch.float32)
    dQz = torch.zeros(h0.shape, dtype=torch.float64, device="cuda")
    dg.lsrk54_step_host(h0, Qz, dQz, 0.0, 0.05, 0)
    torch.cuda.synchronize()
    assert torch.equal(h0, dg.from_perturbation(dg.init_ode_state(Q0)).cpu())
    dt = 0.05
    Qp = dg.init_ode_state(Q0)
    dQ = torch.zeros(Qp.shape, dtype=torch.float64, device=Qp.device)
    dg.lsrk54_step(Qp, dQ, 0.0, dt, 3)
    ref = dg.from_perturbation(Qp).cpu()
    h = torch.from_numpy(Q0.copy()).pin_memory()
    Qp2 = dg.new_state(torch.float32)
    dQ2 = torch.zeros(Qp.shape, dtype=torch.float64, device=Qp.device)
    dg.lsrk54_step_host(h, Qp2, dQ2, 0.0, dt, 3)
    torch.cuda.synchronize()
    assert torch.equal(h, ref)
    pageable = np.ascontiguousarray(Q0.copy())
    with pytest.raises(_lib.CmdgError, match="page-locked"):
        _lib.call("cmdg_lsrk54_step_mixed_host", dg.h, ctypes.c_void_p(pageable.ctypes.data),
                  ctypes.c_void_p(Qp2.data_ptr()), ctypes.c_void_p(dQ2.data_ptr()), 0.0, dt, 1, None)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_stacked_brick_topology_order_runs_reference_ordered_states(precision):
    """A brick mesh numbered like the reference's StackedBrickTopology (columns
    along the 2D Hilbert curve) takes a state in the reference's element
    order directly: its tendency and steps are those of the library's
    stacked order, element for element, bit for bit."""
    ne, L = (5, 4, 3), 2500.0
    lo, hi = (0.0, 0.0, 0.0), (L, L, L)
    grid_ref = cmdg.BrickGrid(4, ne, lo, hi, periodicity=(True, True, False), topology="stacked_brick")
    model = workloads.bubble_model(ne=ne, N=4, L=L, precision=precision).balance_law
    dg_ref = cmdg.DGModel(model, grid_ref, precision=precision)
    dg_lib = workloads.bubble_model(ne=ne, N=4, L=L, precision=precision)
    perm = cmdg.brick_element_order(ne, lo, hi, "stacked_brick")
    xyz = dg_lib.grid.coordinates()
    assert np.array_equal(grid_ref.coordinates(), xyz[perm])
    Q0 = workloads.rising_bubble(xyz, rc=900.0, center=(1100.0, 1300.0, 900.0))
    Q0[:, 1:4] += np.random.default_rng(4).uniform(-1, 1, size=Q0[:, 1:4].shape)
    Ql, Qr = dg_lib.init_ode_state(Q0), dg_ref.init_ode_state(Q0[perm])
    Tl, Tr = dg_lib.new_state(torch.float64), dg_ref.new_state(torch.float64)
    dg_lib(Tl, Ql, None, 0.0)
    dg_ref(Tr, Qr, None, 0.0)
    assert torch.equal(Tr, Tl[torch.from_numpy(perm).cuda()])
    dt = dg_lib.courant_dt(Ql, 0.4)
    for dg, Q in ((dg_lib, Ql), (dg_ref, Qr)):
        cmdg.dostep_(Q, cmdg.LSRK54CarpenterKennedy(dg, Q, dt=dt), None, 0.0, nsteps=3)
    assert torch.equal(Qr, Ql[torch.from_numpy(perm).cuda()])


@pytest.mark.parametrize("kernel", ["node", "persistent", "lines"])
@pytest.mark.parametrize("kind,ne", [("vortex", (2, 1, 1)), ("bubble", (1, 1, 1)), ("bubble", (1, 3, 1)),
                                     ("bubble", (2, 1, 2))])
def test_degenerate_meshes_match_oracle(kind, ne, kernel):
    """Edge cases of the connectivity: an element that is its own neighbour
    across periodic faces (one element in a direction), a column of one
    element between the two walls, and a single element with walls on top
    and bottom and itself on every side face.  (A single fully periodic
    vortex element is left out: its tendency is a near-cancellation of
    O(p / dx) terms and FP64 reassociation alone moves it by ~4e-9 of its
    scale.)  FP64 tendency and 3 LSRK54
    steps within 1e-10 of the field scale; on the bubble (which has a
    reference state) the mixed tendency within 1e-4 (relative L2 per field
    group).  The vortex has no reference state, so its mixed form is FP32
    about zero and its tendency, small next to p ~ 1e5, carries FP32
    rounding of p."""
    om, dg, Q0 = make_pair(kind, 3, ne)
    dg.set_kernel(*KERNELS[kernel])
    ref = om.tendency(Q0)
    Q = dg.init_ode_state(Q0)
    dQ = dg.new_state(torch.float64)
    dg(dQ, Q, None, 0.0)
    err = rel_max(dQ.cpu().numpy(), ref)
    assert (err < TOL64).all(), err
    dt = 0.5 * om.courant_dt(Q0, 0.4)
    Qo, _ = om.lsrk54(Q0.copy(), dt, 3)
    cmdg.dostep_(Q, cmdg.LSRK54CarpenterKennedy(dg, Q, dt=dt), None, 0.0, nsteps=3)
    err = rel_max(Q.cpu().numpy(), Qo)
    assert (err < TOL64).all(), err
    assert dg.status_word() == 0
    if kind != "bubble":
        return
    _, dgm, _ = make_pair(kind, 3, ne, precision="mixed")
    dgm.set_kernel(*KERNELS[kernel])
    dQm = dgm.new_state(torch.float64)
    dgm(dQm, dgm.init_ode_state(Q0), None, 0.0)
    got = dQm.cpu().numpy()
    errs = [np.linalg.norm(got[:, sl] - ref[:, sl]) / np.linalg.norm(ref[:, sl])
            for sl in (slice(0, 1), slice(1, 4), slice(4, 5))]
    assert max(errs) < 1e-4, errs
    assert dgm.status_word() == 0


@pytest.mark.parametrize("cl", [2, 4, 8])
@pytest.mark.parametrize("N", [2, 3, 4, 5])
@pytest.mark.parametrize("kind", ["vortex", "bubble"])
def test_cluster_kernel_matches_oracle(kind, N, cl):
    """The node kernel in thread-block clusters of 2, 4 or 8 adjacent
    elements, whose shared faces read the neighbour's staged state and flux
    from its CTA's shared memory: FP64 tendency and 3 LSRK54 steps within
    1e-10 of the oracle; mixed tendency and 3 steps within 1e-6 (relative L2
    per field group) of the one-CTA-per-element mixed kernel."""
    ne = (4, 2, 4)
    om, dg, Q0 = make_pair(kind, N, ne)
    dg.set_kernel("cluster", cl)
    assert dg.get_kernel() == ("cluster", cl)
    ref = om.tendency(Q0)
    Q = dg.init_ode_state(Q0)
    dQ = dg.new_state(torch.float64)
    dg(dQ, Q, None, 0.0)
    err = rel_max(dQ.cpu().numpy(), ref)
    assert (err < TOL64).all(), err
    dt = 0.5 * om.courant_dt(Q0, 0.4)
    Qo, _ = om.lsrk54(Q0.copy(), dt, 3)
    cmdg.dostep_(Q, cmdg.LSRK54CarpenterKennedy(dg, Q, dt=dt), None, 0.0, nsteps=3)
    err = rel_max(Q.cpu().numpy(), Qo)
    assert (err < TOL64).all(), err
    assert dg.status_word() == 0
    if kind != "bubble":
        return
    out = {}
    for k in ("node", "cluster"):
        _, dgm, _ = make_pair(kind, N, ne, precision="mixed")
        dgm.set_kernel(*(KERNELS["node"] if k == "node" else ("cluster", cl)))
        Qm = dgm.init_ode_state(Q0)
        T = dgm.new_state(torch.float64)
        dgm(T, Qm, None, 0.0)
        cmdg.dostep_(Qm, cmdg.LSRK54CarpenterKennedy(dgm, Qm, dt=dt), None, 0.0, nsteps=3)
        out[k] = (T.cpu().numpy(), dgm.from_perturbation(Qm).cpu().numpy())
        assert dgm.status_word() == 0
    for a, b in zip(out["cluster"], out["node"]):
        for sl in (slice(0, 1), slice(1, 4), slice(4, 5)):
            assert np.linalg.norm(a[:, sl] - b[:, sl]) <= 1e-6 * np.linalg.norm(b[:, sl])


def test_cluster_kernel_refuses_odd_counts():
    om, dg, Q0 = make_pair("bubble", 3, (3, 2, 4))
    with pytest.raises(cmdg.CmdgError, match="even element counts"):
        dg.set_kernel("cluster", 4)
    dg.set_kernel("cluster", 2)  # z only: 4 is even
