"""Filter matrices and filter application on CPU.

Pins: the reference's golden ExponentialFilter matrices
(test/Numerics/Mesh/filter.jl, extracted by tests/golden/make_filter_golden.py)
reproduced by the oracle; the library's host-side matrices equal the
oracle's; the CutoffFilter known-answer test of the same file (Legendre
polynomials: modes of degree >= Nc disappear in the filtered directions)."""
import json
import os

import numpy as np
import pytest

import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))


def test_oracle_reproduces_golden_exponential_filter_matrices():
    gold = json.load(open(os.path.join(HERE, "golden", "filter_matrices.json")))
    assert len(gold) == 2
    for g in gold:
        W = O.filter_matrix(g["N"], "exponential", g["Nc"], g["s"])
        assert np.abs(W - np.array(g["W"])).max() < 1e-14


@pytest.mark.parametrize("kind", ["exponential", "cutoff", "boyd_vandeven"])
def test_library_filter_matrices_equal_oracle(kind):
    from cmdg import filters

    for N in range(1, 8):
        for Nc in range(0, N + 1):
            for s in (4, 32):
                W = filters.filter_matrix(N, kind, Nc, s)
                ref = O.filter_matrix(N, kind, Nc, s)
                assert np.abs(W - ref).max() < 1e-13, (N, Nc, s)


def legendre_fields(xyz):
    l0 = lambda r: np.ones_like(r)
    l1 = lambda r: r
    l2 = lambda r: (3 * r**2 - 1) / 2
    l3 = lambda r: (5 * r**3 - 3 * r) / 2
    x, y, z = xyz[:, 0], xyz[:, 1], xyz[:, 2]
    low = l0(x) * l0(y) + 4 * l1(x) * l1(y) + 5 * l1(z) + 6 * l1(z) * l1(x)
    high_h = l2(x) * l3(y) + l3(x) + l2(y)
    high_v = l3(z) * l1(y)
    return low, high_h, high_v


@pytest.mark.parametrize("direction", ["every", "horizontal", "vertical"])
def test_oracle_cutoff_filter_known_answer(direction):
    om = O.OracleModel(3, (2, 1, 2), (-1, -1, -1), (1, 1, 1), periodic=(1, 1, 1))
    xyz = om.vgeo[:, 12:15]
    # element-local coordinates in [-1, 1] (the polynomials live on each element)
    lo = xyz.min(axis=2, keepdims=True)
    hi = xyz.max(axis=2, keepdims=True)
    r = 2 * (xyz - lo) / (hi - lo) - 1
    low, hh, hv = legendre_fields(r)
    Q = np.stack([low + hh + hv] * 5, axis=1)
    W = O.filter_matrix(3, "cutoff", 2)
    O.apply_filter(om, Q, W, W, direction, fields=(0, 2, 4))
    keep = {"every": low, "horizontal": low + hv, "vertical": low + hh}[direction]
    for s in (0, 2, 4):
        assert np.abs(Q[:, s] - keep).max() < 1e-12
    for s in (1, 3):
        assert np.abs(Q[:, s] - (low + hh + hv)).max() == 0


@pytest.mark.parametrize("direction", ["every", "horizontal", "vertical"])
def test_oracle_mass_preserving_cutoff_known_answer(direction):
    """filter.jl "Mass Preserving Cutoff filter application": on an affine
    element the removed Legendre modes carry no mass, so the result is the
    cutoff result (N = 3, Nc = 2, fields 1 and 3 of 4 in the reference)."""
    om = O.OracleModel(3, (1, 1, 1), (-1, -1, -1), (1, 1, 1), periodic=(1, 1, 1))
    low, hh, hv = legendre_fields(om.vgeo[:, 12:15])
    Q = np.stack([low + hh + hv] * 5, axis=1)
    W = O.filter_matrix(3, "cutoff", 2)
    O.apply_mp_filter(om, Q, W, W, direction, fields=(0, 2))
    keep = {"every": low, "horizontal": low + hv, "vertical": low + hh}[direction]
    for s in (0, 2):
        assert np.abs(Q[:, s] - keep).max() < 1e-12
    for s in (1, 3, 4):
        assert np.abs(Q[:, s] - (low + hh + hv)).max() == 0


def test_oracle_mass_preserving_cutoff_keeps_mass_on_the_shell():
    """filter.jl "MassPreservingCutoffFilter on the sphere": on the cubed shell
    (non-constant Jacobian, radii 1 and 1.2) the mass-preserving filter keeps
    every field's weighted sum, the plain cutoff filter does not."""
    om = O.OracleModel(4, shell=dict(nhorz=1, nvert=1, r_inner=1.0, r_outer=1.2))
    xyz = om.vgeo[:, 12:15]
    low, hh, hv = legendre_fields(xyz)
    x, y = xyz[:, 0], xyz[:, 1]
    # fields without the shell's symmetries (their per-element losses must not cancel)
    Q0 = np.stack([low + hh + hv + 3 * x, np.exp(1.5 * x + 0.5 * y), (x + 2) ** 4 * (y + 1.5) ** 2, low, hh], axis=1)
    W = O.filter_matrix(4, "cutoff", 2)
    fields = (0, 1, 2)
    Q = Q0.copy()
    O.apply_mp_filter(om, Q, W, W, "every", fields=fields)
    Qc = Q0.copy()
    O.apply_filter(om, Qc, W, W, "every", fields=fields)
    for s in fields:
        before = om.weightedsum(Q0, s)
        assert abs(om.weightedsum(Q, s) - before) <= 1e-13 * abs(before) + 1e-15
        assert abs(om.weightedsum(Qc, s) - before) > 1e-8 * abs(before)
