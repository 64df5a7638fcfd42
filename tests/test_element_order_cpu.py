"""Element orders of the reference's brick topologies, on the CPU.

BrickTopology numbers a brick's elements along the Hilbert curve through
their centroids (src/Numerics/Mesh/BrickMesh.jl:531-627), and
StackedBrickTopology numbers the columns of its horizontal base that way with
each column contiguous (src/Numerics/Mesh/Topologies.jl:632-715).  The
library's cmdg_brick_element_order (host code, no GPU) must give the same
permutation as the oracle's restatement, which is pinned to the reference's
hilbertcode / centroidtocode known answers (tests/test_oracle_pins.py); and a
state laid out in the reference's order must come back to the library's
stacked order bit for bit.
"""
import random

import numpy as np
import pytest

import cmdg
import oracle as O

BRICKS = [
    ((4, 3, 2), (0, 0, 0), (1, 1, 1)),
    ((20, 20, 20), (0, 0, 0), (2500, 2500, 2500)),   # the rising bubble
    ((32, 32, 16), (0, 0, 0), (3200, 3200, 1600)),   # the LES
    ((5, 7, 3), (-1, 0, 2), (3, 10, 5)),             # range points that are not dyadic
    ((1, 6, 2), (0, 0, 0), (1, 1, 1)),               # a zero extent of the centroids
    ((8, 8, 1), (0, 0, 0), (1, 1, 1)),
]


@pytest.fixture(scope="module", autouse=True)
def _built():
    import __graft_entry__ as g

    g.build_library()


def _random_bricks(n, seed=3):
    rng = random.Random(seed)
    out = []
    for _ in range(n):
        ne = tuple(rng.randint(1, 9) for _ in range(3))
        lo = tuple(rng.uniform(-5, 5) for _ in range(3))
        hi = tuple(a + rng.uniform(0.1, 20) for a in lo)
        out.append((ne, lo, hi))
    return out


@pytest.mark.parametrize("topology", ["brick", "stacked_brick"])
@pytest.mark.parametrize("ne,lo,hi", BRICKS + _random_bricks(6))
def test_library_order_equals_the_reference_restatement(ne, lo, hi, topology):
    got = cmdg.brick_element_order(ne, lo, hi, topology)
    ref = O.reference_element_order(ne, lo, hi, topology)
    assert np.array_equal(got, ref)
    assert sorted(got.tolist()) == list(range(int(np.prod(ne))))


@pytest.mark.parametrize("topology", ["brick", "stacked_brick"])
def test_reference_ordered_state_maps_back_bitwise(topology):
    ne, lo, hi = (6, 5, 4), (0.0, 0.0, 0.0), (2500.0, 2500.0, 1000.0)
    nelem, Np = int(np.prod(ne)), 125
    Q_lib = np.random.default_rng(9).standard_normal((nelem, 5, Np))
    # the reference's layout, from the oracle's restatement of its order
    perm_ref = O.reference_element_order(ne, lo, hi, topology)
    Q_ref = Q_lib[perm_ref]
    # back to the library's stacked order with the library's permutation
    perm = cmdg.brick_element_order(ne, lo, hi, topology)
    back = np.empty_like(Q_ref)
    back[perm] = Q_ref
    assert np.array_equal(back, Q_lib)


def test_stacked_brick_order_keeps_columns_contiguous():
    ne = (7, 3, 5)
    perm = cmdg.brick_element_order(ne, (0, 0, 0), (1, 1, 1), "stacked_brick")
    nz = ne[2]
    for h in range(ne[0] * ne[1]):
        col = perm[h * nz:(h + 1) * nz]
        assert (col == col[0] + np.arange(nz)).all() and col[0] % nz == 0
