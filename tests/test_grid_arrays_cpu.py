"""The brick grid arrays a Julia caller would pass to cmdg_mesh_create_arrays
(cmdg.workloads.brick_grid_arrays), on the CPU.

In the library's stacked element order they must equal the oracle's
restatement of the reference's DiscontinuousSpectralElementGrid arrays
(src/Numerics/Mesh/Grids.jl:76-125, 559-638): vgeo to 1e-12 of each
field's scale (the curl-invariant metric terms carry DG rounding), vmap+ and
elemtobndy exactly.  In BrickTopology's Hilbert order they must be the same
grid renumbered: every element's vgeo is its stacked twin's, and every face
node's vmap+ names a node at the same physical position (modulo the
periodic shifts) on the element across the face, or the node itself on a
wall.
"""
import numpy as np
import pytest

import oracle as O
from cmdg import workloads


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g

    g.build_library()


CASES = [
    (3, (3, 2, 4), (0.0, 0.0, 0.0), (2500.0, 2000.0, 3000.0), (1, 1, 0)),
    (4, (2, 3, 2), (-1.0, 0.5, 2.0), (3.0, 4.0, 5.0), (0, 1, 1)),
    (2, (1, 2, 3), (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (1, 0, 0)),
]


@pytest.mark.parametrize("N,ne,lo,hi,periodic", CASES)
def test_stacked_arrays_equal_the_oracles(N, ne, lo, hi, periodic):
    om = O.OracleModel(N, ne, lo, hi, periodic=periodic)
    vgeo, vmap, bndy, perm = workloads.brick_grid_arrays(N, ne, lo, hi, [bool(p) for p in periodic],
                                                         ((1, 2), (1, 2), (1, 2)), topology="library")
    assert np.array_equal(perm, np.arange(len(perm)))
    assert np.array_equal(vmap, om.vmapP + 1)
    assert np.array_equal(bndy, om.elemtobndy)
    scale = np.abs(om.vgeo).max(axis=(0, 2))
    scale[:9] = scale[:9].max()  # the curl-invariant off-diagonal metric terms are rounding-sized
    # the oracle fills the metric terms, M, MI and the coordinates (MH and
    # JcV, which no kernel of the path reads, it leaves at zero)
    for f in list(range(11)) + [12, 13, 14]:
        # the curl-invariant metric terms carry the rounding of their DG derivatives
        assert np.abs(vgeo[:, f] - om.vgeo[:, f]).max() <= 1e-12 * scale[f], f


@pytest.mark.parametrize("topology", ["brick", "stacked_brick"])
@pytest.mark.parametrize("N,ne,lo,hi,periodic", CASES)
def test_reference_ordered_arrays_are_the_same_grid(N, ne, lo, hi, periodic, topology):
    per = [bool(p) for p in periodic]
    bc = ((1, 2), (1, 2), (1, 2))
    g0, m0, b0, _ = workloads.brick_grid_arrays(N, ne, lo, hi, per, bc, topology="library")
    vgeo, vmap, bndy, perm = workloads.brick_grid_arrays(N, ne, lo, hi, per, bc, topology=topology)
    assert sorted(perm.tolist()) == list(range(len(perm)))
    assert np.array_equal(vgeo, g0[perm])
    assert np.array_equal(bndy, b0[perm])
    Np = vgeo.shape[2]
    X = vgeo[:, 12:15, :].transpose(0, 2, 1).reshape(-1, 3)     # node coordinates by global index
    period = np.asarray(hi, dtype=np.float64) - np.asarray(lo, dtype=np.float64)
    Nq = N + 1
    p = np.arange(Np).reshape(Nq, Nq, Nq)
    fmask = [p[:, :, 0].ravel(), p[:, :, N].ravel(), p[:, 0, :].ravel(), p[:, N, :].ravel(),
             p[0, :, :].ravel(), p[N, :, :].ravel()]
    tol = 1e-12 * np.abs(X).max()
    for f in range(6):
        own = (Np * np.arange(len(perm))[:, None] + fmask[f][None, :]).ravel()
        across = (vmap[:, f, :] - 1).ravel()
        d = X[across] - X[own]
        for c in range(3):
            if per[c]:
                d[:, c] -= period[c] * np.round(d[:, c] / period[c])
        assert np.abs(d).max() <= tol, f
        wall = np.repeat(bndy[:, f] != 0, fmask[f].size)
        assert np.array_equal(across[wall], own[wall])
        assert not np.any(across[~wall] // Np == own[~wall] // Np) or min(ne) == 1
