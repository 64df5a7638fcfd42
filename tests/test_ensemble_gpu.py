"""Ensembles: the batch kernel advances members of uneven size and order as
the single-model kernel does (the same per-element arithmetic), the
graph-captured steps repeat, every tiling gives bitwise-equal results, and a
member stays within 1e-5 of the FP64 oracle."""
import numpy as np
import pytest
import torch

import cmdg
import oracle as O
from cmdg import workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g

    g.build()
    torch.cuda.set_device(0)


def members(n=5, seed=3):
    specs = workloads.bubble_ensemble_specs(n=n, seed=seed)
    # small members keep the test quick, orders 3, 4 and 5 all present
    for i, s in enumerate(specs):
        s["ne"] = (2 + i % 3, 3, 2 + (i * 7) % 4)
        s["N"] = 3 + i % 3
    return specs


def test_ensemble_matches_single_model_steps():
    specs = members()
    pairs = [workloads.bubble_member(s) for s in specs]
    dgs = [p[0] for p in pairs]
    dts = [0.6 * dg.courant_dt(dg.init_ode_state(Q0), 0.4) for dg, Q0 in pairs]
    # sequential reference: the same node-kernel body, one CTA per element
    ref = []
    for (dg, Q0), dt in zip(pairs, dts):
        dg.set_kernel("node", -1)
        Q = dg.init_ode_state(Q0)
        lsrk = cmdg.LSRK54CarpenterKennedy(dg, Q, dt=dt)
        cmdg.dostep_(Q, lsrk, None, 0.0, nsteps=3)
        ref.append(Q.cpu().numpy())
    ens = cmdg.Ensemble(dgs)
    Qs = [dg.init_ode_state(Q0) for dg, Q0 in pairs]
    dQs = [torch.zeros(Q.shape, dtype=torch.float64, device="cuda") for Q in Qs]
    ens.lsrk54_step(Qs, dQs, dts, nsteps=1)
    ens.lsrk54_step(Qs, dQs, dts, nsteps=2)  # a second graph
    # the same FP32 element arithmetic: equal up to the compiler's FMA
    # contraction choices in the two kernels' instantiations
    for Q, r in zip(Qs, ref):
        got = Q.cpu().numpy()
        scale = np.abs(r).max(axis=(0, 2), keepdims=True)
        assert (np.abs(got - r) <= 1e-6 * scale).all()
    assert all(dg.status_word() == 0 for dg in dgs)


def test_ensemble_autotune_and_tilings_keep_results():
    """Every tiling runs the same kernel per order, so results are bitwise equal."""
    specs = members(n=4, seed=9)
    pairs = [workloads.bubble_member(s) for s in specs]
    dgs = [p[0] for p in pairs]
    dts = [0.5 * dg.courant_dt(dg.init_ode_state(Q0), 0.4) for dg, Q0 in pairs]
    outs = []
    for tiling in [(1, -1), (4, 0), (16, 7), None]:
        ens = cmdg.Ensemble(dgs)
        Qs = [dg.init_ode_state(Q0) for dg, Q0 in pairs]
        dQs = [torch.zeros(Q.shape, dtype=torch.float64, device="cuda") for Q in Qs]
        if tiling is None:
            ms, choice = ens.autotune(Qs, dQs, reps=2)
            for N in (3, 4, 5):
                assert len(ms[N]) == 10 and all(m > 0 for m in ms[N])
                assert choice[N][0] in (1, 2, 4, 8, 16) and choice[N][1] in (-1, 0)
            assert len(ms["persistent"]) == 16 and all(m > 0 for m in ms["persistent"]) and ms["per_order"] > 0
            assert choice["kernel"][0] in ("per_order", "persistent")
            ens.set_kernel("per_order")  # the per-order tilings chosen above, compared bitwise below
        else:
            ens.set_tiling(*tiling)
            assert ens.get_tiling()[4] == tiling
        ens.lsrk54_step(Qs, dQs, dts, nsteps=2)
        outs.append([Q.cpu().numpy() for Q in Qs])
    for other in outs[1:]:
        for a, b in zip(outs[0], other):
            assert np.array_equal(a, b)
    assert all(dg.status_word() == 0 for dg in dgs)


def test_persistent_ensemble_kernel_matches_per_order_launches():
    """The persistent kernel (one launch per stage over tiles of every order,
    one CTA shape: 128 or 256 threads, so each order runs its own number of
    elements per CTA pass and nodes per thread) advances every member as the
    per-order kernels do, up to FP32 reassociation (the two kernels sum the
    same terms in different orders), for every tiling, and its results do not
    depend on the tiling within one CTA size."""
    specs = members(n=6, seed=5)
    pairs = [workloads.bubble_member(s) for s in specs]
    dgs = [p[0] for p in pairs]
    dts = [0.5 * dg.courant_dt(dg.init_ode_state(Q0), 0.4) for dg, Q0 in pairs]

    def run(kernel):
        ens = cmdg.Ensemble(dgs)
        ens.set_kernel(*kernel)
        Qs = [dg.init_ode_state(Q0) for dg, Q0 in pairs]
        dQs = [torch.zeros(Q.shape, dtype=torch.float64, device="cuda") for Q in Qs]
        ens.lsrk54_step(Qs, dQs, dts, nsteps=3)
        return [dg.from_perturbation(Q).cpu().numpy() for dg, Q in zip(dgs, Qs)]

    def rel_l2(a, r, M):
        # relative L2 (mass-weighted) per field group: rho, momentum, rho e
        out = []
        for sl in (slice(0, 1), slice(1, 4), slice(4, 5)):
            out.append(np.sqrt(np.sum((a[:, sl] - r[:, sl]) ** 2 * M[:, None])) /
                       np.sqrt(np.sum(r[:, sl] ** 2 * M[:, None])))
        return np.array(out)

    ref = run(("per_order",))
    for threads in (128, 256):
        outs = [run(("persistent", threads, tile, grid)) for tile, grid in ((1, -1), (4, 0), (8, 5))]
        for other in outs[1:]:
            for a, b in zip(outs[0], other):
                assert np.array_equal(a, b)
        for dg, a, r in zip(dgs, outs[0], ref):
            err = rel_l2(a, r, dg.grid.mass())
            assert (err < 1e-6).all(), (threads, err)
    assert all(dg.status_word() == 0 for dg in dgs)


def test_ensemble_member_close_to_fp64_oracle():
    spec = dict(ne=(3, 3, 3), N=4, amp=2.5, rc=700.0, center=(1250.0, 1250.0, 900.0))
    dg, Q0 = workloads.bubble_member(spec)
    L = 2500.0
    om = O.OracleModel(4, spec["ne"], (0, 0, 0), (L, L, L), periodic=(1, 1, 0), orientation="flat", gravity=True,
                       ref_state=True, profile="dry_adiabatic", T_surface=300.0, T_min=0.0)
    dt = om.courant_dt(Q0, 0.4)
    Qo, _ = om.lsrk54(Q0.copy(), dt, 50)
    for kernel in (("per_order",), ("persistent", 128, 2, 0), ("persistent", 256, 2, 0)):
        ens = cmdg.Ensemble([dg])
        ens.set_kernel(*kernel)
        Q = dg.init_ode_state(Q0)
        dQ = torch.zeros(Q.shape, dtype=torch.float64, device="cuda")
        ens.lsrk54_step([Q], [dQ], [dt], nsteps=50)
        err, ref = om.field_l2(dg.from_perturbation(Q).cpu().numpy(), Qo)
        err = np.array([err[0], np.sqrt(np.sum(err[1:4] ** 2)), err[4]])
        ref = np.array([ref[0], np.sqrt(np.sum(ref[1:4] ** 2)), ref[4]])
        assert (err / ref < 1e-5).all(), (kernel, err / ref)


def test_les_ensemble_matches_single_models_and_stays_near_the_oracle():
    """A batch of LES members (mixed SmagorinskyLilly, as in the 16-member LES
    configuration, at a size the oracle steps quickly): a batched member's
    steps equal its single-model steps bit for bit (the same gradient pass
    and viscous stage kernel per stage), and a batched member stays within
    1e-5 (relative L2 per field group) of the FP64 oracle after 100 steps."""
    Lx, ne, nmem = (800.0, 800.0, 600.0), (4, 4, 3), 3
    dgs = [workloads.les_model(ne=ne, N=4, L=Lx, precision="mixed") for _ in range(nmem)]
    Q0s = [workloads.les_initial_state(dgs[0].grid.coordinates(), L=Lx, seed=s) for s in range(1, nmem + 1)]
    dt = min(dg.courant_dt(dg.init_ode_state(Q0), 0.4) for dg, Q0 in zip(dgs, Q0s))
    ens = cmdg.Ensemble(dgs)
    Qs = [dg.init_ode_state(Q0) for dg, Q0 in zip(dgs, Q0s)]
    dQs = [torch.zeros(Q.shape, dtype=torch.float64, device="cuda") for Q in Qs]
    for _ in range(2):
        ens.lsrk54_step(Qs, dQs, [dt] * nmem, nsteps=50)  # one graph, replayed
    single = workloads.les_model(ne=ne, N=4, L=Lx, precision="mixed")
    Q = single.init_ode_state(Q0s[0])
    cmdg.dostep_(Q, cmdg.LSRK54CarpenterKennedy(single, Q, dt=dt), None, 0.0, nsteps=100)
    assert torch.equal(Qs[0], Q)
    om = O.OracleModel(4, ne, (0, 0, 0), Lx, periodic=(1, 1, 0), orientation="flat", gravity=True, ref_state=True,
                       profile="dry_adiabatic", T_surface=300.0, T_min=0.0, turbulence="smagorinsky")
    Qo, _ = om.lsrk54(Q0s[1].copy(), dt, 100)
    err, refn = om.field_l2(dgs[1].from_perturbation(Qs[1]).cpu().numpy(), Qo)
    err = np.array([err[0], np.sqrt(np.sum(err[1:4] ** 2)), err[4]])
    refn = np.array([refn[0], np.sqrt(np.sum(refn[1:4] ** 2)), refn[4]])
    assert (err / refn < 1e-5).all(), err / refn
    assert all(dg.status_word() == 0 for dg in dgs)
