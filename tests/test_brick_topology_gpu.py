"""Generated brick meshes numbered in BrickTopology's order: every element
along the 3D Hilbert curve through the element centroids
(src/Numerics/Mesh/Topologies.jl:470-545, BrickMesh.partition in
src/Numerics/Mesh/BrickMesh.jl:531-627), so a column's elements are not
contiguous.  The kernels read an element's vertical index from its neighbour
row, so such a mesh must step a state given in the reference's element order
exactly as the library's stacked order steps the same state permuted: the
tendency and the LSRK54 steps bit for bit for every stage kernel, the
filters bit for bit, the weighted sums to double-double rounding, and the
Courant dt, coordinates and reference state equal after the permutation.
HEVI, whose column solves need contiguous columns, refuses the mesh.
"""
import numpy as np
import pytest
import torch

import cmdg
from cmdg import workloads
from cmdg.filters import CutoffFilter, ExponentialFilter, MassPreservingCutoffFilter, TMARFilter, apply_

pytestmark = pytest.mark.gpu

L = 2500.0
LO, HI = (0.0, 0.0, 0.0), (L, L, L)
BUBBLE_BC = dict(periodicity=(True, True, False), boundary=((0, 0), (0, 0), (1, 2)))


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g

    g.build()
    torch.cuda.set_device(0)


def pair(builder, ne, N=4, precision="fp64", hi=HI, **kw):
    """(library-order model, BrickTopology-order model, perm) of one
    configuration; perm[e_ref] = the library index of reference element e_ref."""
    dg_lib = builder(ne=ne, N=N, precision=precision, **kw)
    grid = cmdg.BrickGrid(N, ne, LO, hi, topology="brick", **BUBBLE_BC)
    dg_ref = cmdg.DGModel(dg_lib.balance_law, grid, precision=precision)
    perm = cmdg.brick_element_order(ne, LO, hi, "brick")
    return dg_lib, dg_ref, perm


def bubble_state(xyz, seed=4):
    Q0 = workloads.rising_bubble(xyz, rc=900.0, center=(1100.0, 1300.0, 900.0))
    Q0[:, 1:4] += np.random.default_rng(seed).uniform(-1, 1, size=Q0[:, 1:4].shape)
    return Q0


def test_brick_order_is_not_stacked():
    """The case this file covers: BrickTopology splits columns."""
    ne = (4, 4, 4)
    perm = cmdg.brick_element_order(ne, LO, HI, "brick")
    nz = ne[2]
    contiguous = all((perm[h * nz:(h + 1) * nz] == perm[h * nz] + np.arange(nz)).all() for h in range(16))
    assert not contiguous


# every stage kernel in both precisions (the column kernel is built for the mixed form only)
@pytest.mark.parametrize("precision,kernel", [(p, k) for p in ("fp64", "mixed")
                                              for k in ("node", "persistent", "lines", "column", "cluster")
                                              if not (k == "column" and p == "fp64")])
def test_bubble_in_brick_order_matches_library_order(precision, kernel):
    ne = (4, 2, 4)
    dg_lib, dg_ref, perm = pair(workloads.bubble_model, ne, precision=precision)
    kinds = {"node": ("node", -1), "persistent": ("node", 0), "lines": ("lines", -1), "column": ("column", 0),
             "cluster": ("cluster", 8)}
    for dg in (dg_lib, dg_ref):
        dg.set_kernel(*kinds[kernel])
    xyz = dg_lib.grid.coordinates()
    assert np.array_equal(dg_ref.grid.coordinates(), xyz[perm])
    assert np.array_equal(dg_ref.reference_state(), dg_lib.reference_state()[perm])
    Q0 = bubble_state(xyz)
    Ql, Qr = dg_lib.init_ode_state(Q0), dg_ref.init_ode_state(Q0[perm])
    P = torch.from_numpy(perm).cuda()
    assert torch.equal(Qr, Ql[P])
    Tl, Tr = dg_lib.new_state(torch.float64), dg_ref.new_state(torch.float64)
    dg_lib(Tl, Ql, None, 0.0)
    dg_ref(Tr, Qr, None, 0.0)
    assert torch.equal(Tr, Tl[P])
    dt = dg_lib.courant_dt(Ql, 0.4)
    assert dg_ref.courant_dt(Qr, 0.4) == dt
    for dg, Q in ((dg_lib, Ql), (dg_ref, Qr)):
        cmdg.dostep_(Q, cmdg.LSRK54CarpenterKennedy(dg, Q, dt=dt), None, 0.0, nsteps=3)
    assert torch.equal(Qr, Ql[P])
    assert torch.equal(dg_ref.from_perturbation(Qr) if precision == "mixed" else Qr,
                       (dg_lib.from_perturbation(Ql) if precision == "mixed" else Ql)[P])
    sl, sr = dg_lib.weighted_sums(Ql), dg_ref.weighted_sums(Qr)
    assert np.allclose(sr, sl, rtol=1e-15, atol=0)
    assert dg_lib.status_word() == 0 and dg_ref.status_word() == 0


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("N,ne", [(2, (3, 1, 5)), (3, (1, 3, 2)), (5, (2, 2, 1)), (3, (5, 4, 3))])
def test_other_orders_and_degenerate_bricks_in_brick_order(N, ne, precision):
    """Orders 2, 3 and 5, and bricks with one element in a direction (an
    element that is its own periodic neighbour, a single element between
    the two walls): tendency and steps bit for bit after the permutation."""
    dg_lib, dg_ref, perm = pair(workloads.bubble_model, ne, N=N, precision=precision)
    P = torch.from_numpy(perm).cuda()
    Q0 = bubble_state(dg_lib.grid.coordinates(), seed=N)
    Ql, Qr = dg_lib.init_ode_state(Q0), dg_ref.init_ode_state(Q0[perm])
    Tl, Tr = dg_lib.new_state(torch.float64), dg_ref.new_state(torch.float64)
    dg_lib(Tl, Ql, None, 0.0)
    dg_ref(Tr, Qr, None, 0.0)
    assert torch.equal(Tr, Tl[P])
    dt = dg_lib.courant_dt(Ql, 0.4)
    for dg, Q in ((dg_lib, Ql), (dg_ref, Qr)):
        cmdg.dostep_(Q, cmdg.LSRK54CarpenterKennedy(dg, Q, dt=dt), None, 0.0, nsteps=2)
    assert torch.equal(Qr, Ql[P])
    assert dg_lib.status_word() == 0 and dg_ref.status_word() == 0


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("case", ["les", "hyper"])
def test_viscous_and_hyperdiffusive_models_in_brick_order(case, precision):
    """SmagorinskyLilly (gradient + viscous stage kernels) and DryBiharmonic
    (the three hyperdiffusion passes) read the vertical index of an element
    and of its neighbours in every pass."""
    ne = (3, 2, 4)
    if case == "les":
        Lx = (3200.0, 3200.0, 1600.0)
        dg_lib, dg_ref, perm = pair(workloads.les_model, ne, precision=precision, hi=Lx, L=Lx)
        Q0 = workloads.les_initial_state(dg_lib.grid.coordinates(), L=Lx, seed=3)
    else:
        dg_lib, dg_ref, perm = pair(workloads.hyper_bubble_model, ne, precision=precision)
        Q0 = bubble_state(dg_lib.grid.coordinates(), seed=5)
    P = torch.from_numpy(perm).cuda()
    Ql, Qr = dg_lib.init_ode_state(Q0), dg_ref.init_ode_state(Q0[perm])
    Tl, Tr = dg_lib.new_state(torch.float64), dg_ref.new_state(torch.float64)
    dg_lib(Tl, Ql, None, 0.0)
    dg_ref(Tr, Qr, None, 0.0)
    assert torch.equal(Tr, Tl[P])
    dt = 0.5 * dg_lib.courant_dt(Ql, 0.4)
    for dg, Q in ((dg_lib, Ql), (dg_ref, Qr)):
        cmdg.dostep_(Q, cmdg.LSRK54CarpenterKennedy(dg, Q, dt=dt), None, 0.0, nsteps=2)
    assert torch.equal(Qr, Ql[P])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("filt,direction", [("exponential", "vertical"), ("cutoff", "every"), ("tmar", "every"),
                                            ("mp", "every")])
def test_filters_in_brick_order(filt, direction, precision):
    """The spectral filters (the mixed form's per-level FP64 correction
    W q_ref - q_ref), the mass-preserving cutoff filter and TMAR."""
    ne = (3, 3, 4)
    N = 4
    dg_lib, dg_ref, perm = pair(workloads.bubble_model, ne, N=N, precision=precision)
    P = torch.from_numpy(perm).cuda()
    Q0 = bubble_state(dg_lib.grid.coordinates(), seed=8)
    if filt == "tmar":
        Q0[:, 1:4] = np.random.default_rng(3).uniform(-1, 1, size=Q0[:, 1:4].shape)
    make = {"exponential": lambda g: ExponentialFilter(g, 0, 8), "cutoff": lambda g: CutoffFilter(g, 2),
            "tmar": lambda g: TMARFilter(), "mp": lambda g: MassPreservingCutoffFilter(g, 2)}[filt]
    target = (1, 2, 3) if filt == "tmar" else None
    Ql, Qr = dg_lib.init_ode_state(Q0), dg_ref.init_ode_state(Q0[perm])
    apply_(Ql, target, dg_lib, make(dg_lib.grid), direction)
    apply_(Qr, target, dg_ref, make(dg_ref.grid), direction)
    torch.cuda.synchronize()
    assert torch.equal(Qr, Ql[P])


def test_hevi_refuses_brick_order():
    """The ARK2 column solves need each column's elements contiguous."""
    dg_lib, dg_ref, _ = pair(workloads.bubble_model, (2, 2, 3), N=3)
    lin = cmdg.DGModel(cmdg.AtmosAcousticGravityLinearModel(dg_ref.balance_law), dg_ref.grid, direction="vertical",
                       state_auxiliary=dg_ref)
    Q = dg_ref.init_ode_state(bubble_state(dg_ref.grid.coordinates()))
    with pytest.raises(cmdg.CmdgError, match="column order"):
        cmdg.ARK2GiraldoKellyConstantinescu(dg_ref, lin, cmdg.LinearBackwardEulerSolver(cmdg.ManyColumnLU()), Q,
                                            dt=1.0)
