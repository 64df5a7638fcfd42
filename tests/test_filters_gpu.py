"""GPU filters against the oracle: spectral filters (exponential, cutoff,
Boyd-Vandeven; every, horizontal, vertical direction; field subsets) on the
FP64 state within 1e-13 and on the mixed-precision perturbation within 1e-6
(bricks and the cubed shell),
the CutoffFilter known answer, TMAR, and the MassPreservingCutoffFilter
(oracle parity on bricks and on the cubed shell, mass kept per field, the
vertical exponential filter on the shell)."""
import numpy as np
import pytest
import torch

import cmdg
import oracle as O
from cmdg import filters, workloads

pytestmark = pytest.mark.gpu
L = 2500.0


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g

    g.build()
    torch.cuda.set_device(0)


def pair(N=4, ne=(3, 2, 4), precision="fp64"):
    om = O.OracleModel(N, ne, (0, 0, 0), (L, L, L), periodic=(1, 1, 0), orientation="flat", gravity=True,
                       ref_state=True, profile="dry_adiabatic", T_surface=300.0, T_min=0.0)
    dg = workloads.bubble_model(ne=ne, N=N, L=L, precision=precision)
    Q0 = om.init_bubble(rc=900.0, xc=1100.0, yc=1300.0, zc=800.0)
    rng = np.random.default_rng(9)
    Q0[:, 1:4] += rng.uniform(-3, 3, size=Q0[:, 1:4].shape)
    return om, dg, Q0


def rel(got, ref):
    out = []
    for sl in (slice(0, 1), slice(1, 4), slice(4, 5)):
        out.append(np.abs(got[:, sl] - ref[:, sl]).max() / np.abs(ref[:, sl]).max())
    return np.array(out)


CASES = [("exponential", (0, 0), 32, "every", (0, 1, 2, 3, 4)), ("cutoff", (3, 2), 0, "vertical", (0, 4)),
         ("boyd_vandeven", (1, 1), 8, "horizontal", (1, 2, 3)), ("exponential", (2, 1), 4, "every", (0, 3, 4))]


@pytest.mark.parametrize("kind,Nc,s,direction,fields", CASES)
def test_fp64_spectral_filter_matches_oracle(kind, Nc, s, direction, fields):
    om, dg, Q0 = pair()
    cls = {"exponential": filters.ExponentialFilter, "cutoff": filters.CutoffFilter,
           "boyd_vandeven": filters.BoydVandevenFilter}[kind]
    filt = cls(dg.grid, Nc) if kind == "cutoff" else cls(dg.grid, Nc, s)
    Q = dg.init_ode_state(Q0)
    filters.apply_(Q, fields, dg, filt, direction)
    ref = O.apply_filter(om, Q0.copy(), filt.filter_matrices[0], filt.filter_matrices[1], direction, fields)
    assert (rel(Q.cpu().numpy(), ref) < 1e-13).all()


@pytest.mark.parametrize("kind,Nc,s,direction,fields", CASES)
def test_mixed_spectral_filter_close_to_fp64_oracle(kind, Nc, s, direction, fields):
    om, dg, Q0 = pair(precision="mixed")
    cls = {"exponential": filters.ExponentialFilter, "cutoff": filters.CutoffFilter,
           "boyd_vandeven": filters.BoydVandevenFilter}[kind]
    filt = cls(dg.grid, Nc) if kind == "cutoff" else cls(dg.grid, Nc, s)
    Qp = dg.init_ode_state(Q0)
    filters.apply_(Qp, fields, dg, filt, direction)
    ref = O.apply_filter(om, Q0.copy(), filt.filter_matrices[0], filt.filter_matrices[1], direction, fields)
    got = dg.from_perturbation(Qp).cpu().numpy()
    assert (rel(got, ref) < 1e-6).all(), rel(got, ref)


def test_cutoff_known_answer_on_gpu():
    grid = cmdg.BrickGrid(3, (2, 1, 2), (-1, -1, -1), (1, 1, 1))
    dg = cmdg.DGModel(cmdg.AtmosModel(), grid)
    xyz = grid.coordinates()
    lo, hi = xyz.min(axis=2, keepdims=True), xyz.max(axis=2, keepdims=True)
    r = 2 * (xyz - lo) / (hi - lo) - 1
    x, y, z = r[:, 0], r[:, 1], r[:, 2]
    low = 1 + 4 * x * y + 5 * z + 6 * z * x
    hh = (3 * x**2 - 1) / 2 * (5 * y**3 - 3 * y) / 2 + (5 * x**3 - 3 * x) / 2 + (3 * y**2 - 1) / 2
    hv = (5 * z**3 - 3 * z) / 2 * y
    Q = torch.from_numpy(np.stack([low + hh + hv] * 5, axis=1)).cuda()
    filters.apply_(Q, (0, 1, 2, 3, 4), dg, filters.CutoffFilter(grid, 2), "every")
    assert np.abs(Q.cpu().numpy() - low[:, None, :]).max() < 1e-12


def test_tmar_matches_oracle():
    om, dg, Q0 = pair()
    Q0[:, 3] = np.random.default_rng(1).normal(0.2, 1.0, size=Q0[:, 3].shape)  # a field with negative values
    Q = dg.init_ode_state(Q0)
    filters.apply_(Q, (3,), dg, filters.TMARFilter())
    ref = O.apply_tmar(om, Q0.copy(), (3,))
    got = Q.cpu().numpy()
    assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()
    assert (got[:, 3] >= 0).all()


@pytest.mark.parametrize("direction", ["every", "horizontal", "vertical"])
def test_mass_preserving_cutoff_matches_oracle_on_brick(direction):
    om, dg, Q0 = pair()
    filt = filters.MassPreservingCutoffFilter(dg.grid, 2)
    Q = dg.init_ode_state(Q0)
    filters.apply_(Q, (0, 1, 4), dg, filt, direction)
    ref = O.apply_mp_filter(om, Q0.copy(), filt.filter_matrices[0], filt.filter_matrices[1], direction, (0, 1, 4))
    assert rel(Q.cpu().numpy(), ref).max() < 1e-13


def shell_pair(N=4):
    R = O.EARTH["planet_radius"]
    om = O.OracleModel(N, shell=dict(nhorz=2, nvert=2, r_inner=R, r_outer=R + 30e3), orientation="sphere",
                       gravity=True, ref_state=True, profile="isothermal", T_surface=285.0)
    dg = workloads.gcm_shell_model(nhorz=2, nvert=2, N=N)
    Q0 = workloads.gcm_initial_state(dg.grid.coordinates(), seed=3)
    return om, dg, Q0


def test_mass_preserving_cutoff_on_the_shell_matches_oracle_and_keeps_mass():
    om, dg, Q0 = shell_pair()
    filt = filters.MassPreservingCutoffFilter(dg.grid, 2)
    Q = dg.init_ode_state(Q0)
    before = dg.weighted_sums(Q, (0, 1, 2, 3, 4))
    filters.apply_(Q, (0, 1, 2, 3, 4), dg, filt, "every")
    after = dg.weighted_sums(Q, (0, 1, 2, 3, 4))
    ref = O.apply_mp_filter(om, Q0.copy(), filt.filter_matrices[0], filt.filter_matrices[1], "every")
    assert rel(Q.cpu().numpy(), ref).max() < 1e-12
    for b, a in zip(before, after):
        # compensated sums over 41k nodes of a field whose sum cancels partly
        assert abs(a - b) <= 1e-11 * max(abs(b), 1.0)
    # the plain cutoff filter changes the weighted sums on the curved mesh
    Qc = dg.init_ode_state(Q0)
    filters.apply_(Qc, (0, 4), dg, filters.CutoffFilter(dg.grid, 2), "every")
    c = dg.weighted_sums(Qc, (0, 4))
    assert abs(c[0] - before[0]) > 1e-9 * abs(before[0])


def test_fp64_filters_run_on_the_shell():
    om, dg, Q0 = shell_pair(5)
    filt = filters.ExponentialFilter(dg.grid, 0, 18)
    Q = dg.init_ode_state(Q0)
    filters.apply_(Q, (0, 1, 2, 3, 4), dg, filt, "vertical")
    ref = O.apply_filter(om, Q0.copy(), filt.filter_matrices[0], filt.filter_matrices[1], "vertical")
    assert rel(Q.cpu().numpy(), ref).max() < 1e-13


@pytest.mark.parametrize("mesh", ["brick", "shell"])
def test_mass_preserving_cutoff_on_mixed_models(mesh):
    """A mixed model's perturbation filtered through an FP64 copy of its full
    state: within 1e-6 (relative to each field group's scale) of the oracle's
    FP64 filter, and the mass of every field kept to FP32 rounding of the
    perturbation."""
    if mesh == "brick":
        om, dgm, Q0 = pair(precision="mixed")
    else:
        om, _, Q0 = shell_pair()
        dgm = workloads.gcm_shell_model(nhorz=2, nvert=2, N=4, precision="mixed")
    filt = filters.MassPreservingCutoffFilter(dgm.grid, 2)
    Qp = dgm.init_ode_state(Q0)
    filters.apply_(Qp, (0, 1, 2, 3, 4), dgm, filt, "every")
    ref = O.apply_mp_filter(om, Q0.copy(), filt.filter_matrices[0], filt.filter_matrices[1], "every")
    got = dgm.from_perturbation(Qp).cpu().numpy()
    assert (rel(got, ref) < 1e-6).all(), rel(got, ref)
    assert dgm.status_word() == 0


@pytest.mark.parametrize("kind,direction", [("exponential", "vertical"), ("exponential", "every"),
                                            ("cutoff", "horizontal"), ("boyd_vandeven", "every")])
def test_mixed_filters_on_the_shell_close_to_fp64_oracle(kind, direction):
    """Mixed-precision filters on the cubed shell, whose reference density
    varies along a level: the FP32 perturbation is filtered and the FP64
    change of the reference state under the same filter, W q_ref - q_ref, is
    added per node.  Within 1e-6 of the oracle's FP64 filter of the full state."""
    om, _, Q0 = shell_pair()
    dg = workloads.gcm_shell_model(nhorz=2, nvert=2, N=4, precision="mixed")
    filt = {"exponential": lambda g: filters.ExponentialFilter(g, 0, 18),
            "cutoff": lambda g: filters.CutoffFilter(g, 2),
            "boyd_vandeven": lambda g: filters.BoydVandevenFilter(g, 1, 8)}[kind](dg.grid)
    Qp = dg.init_ode_state(Q0)
    filters.apply_(Qp, (0, 1, 2, 3, 4), dg, filt, direction)
    ref = O.apply_filter(om, Q0.copy(), filt.filter_matrices[0], filt.filter_matrices[1], direction)
    got = dg.from_perturbation(Qp).cpu().numpy()
    assert (rel(got, ref) < 1e-6).all(), rel(got, ref)
