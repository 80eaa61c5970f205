"""The de Rham map and its quadrature in the oracle, against the reference's
own laws (CPU only).

- The Grundmann-Moeller rule of degree d integrates every barycentric monomial
  of degree <= d exactly (simplicial/src/atlas/quadrature.rs:30-82): the mean of
  prod lambda_i^a_i over a k-simplex is k! prod a_i! / (k + |a|)!.
- R d = d R, Stokes' theorem (derham/src/project.rs, test
  derham_map_is_cochain_map), for polynomial forms whose integrands the rule
  integrates exactly, on jittered Kuhn meshes.
- R of a constant form is the tangent-blade sum of every simplex.
"""
import itertools
import math

import numpy as np
import pytest


@pytest.mark.parametrize("k", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("degree", [0, 1, 2, 3, 4, 5, 7])
def test_gm_rule_is_exact_to_its_degree(oracle, k, degree):
    """quadrature.rs:184-235: exact on every barycentric monomial up to the
    degree asked for; weights and each node's barycentric coordinates sum to 1."""
    bary, w = oracle.gm_rule(k, degree)
    assert abs(w.sum() - 1.0) < 1e-14
    assert np.abs(bary.sum(axis=1) - 1.0).max() < 1e-12
    for total in range(degree + 1):
        for a in itertools.product(range(total + 1), repeat=k + 1):
            if sum(a) != total:
                continue
            got = float(np.sum(w * np.prod(bary ** np.array(a), axis=1)))
            want = math.factorial(k) * np.prod([math.factorial(x) for x in a]) / math.factorial(k + total)
            assert abs(got - want) <= 1e-13 * max(1.0, want), (k, degree, a)


def _mesh(oracle, dim, nb, seed=3):
    cx, coords = oracle.cartesian_unit(dim, nb)
    return cx, oracle.jitter_coords(coords, nb, seed, 0.1)


def test_derham_map_is_a_cochain_map_2d(oracle):
    """w = x^2 y (0-form): dw = (2xy, x^2). w = (x y, x^2 + y) (1-form):
    dw = (2x - x) dx^dy."""
    cx, coords = _mesh(oracle, 2, 5)
    wc = oracle.WhitneyComplex(cx, cx.edge_lengths_sq(coords))
    f0 = lambda p: (p[:, 0] ** 2 * p[:, 1])[:, None]
    df0 = lambda p: np.stack([2 * p[:, 0] * p[:, 1], p[:, 0] ** 2], 1)
    r0 = oracle.derham_map(cx, coords, 0, f0, 3)
    r1 = oracle.derham_map(cx, coords, 1, df0, 3)
    assert np.abs(wc.dif(0) @ r0 - r1).max() < 1e-13
    f1 = lambda p: np.stack([p[:, 0] * p[:, 1], p[:, 0] ** 2 + p[:, 1]], 1)
    df1 = lambda p: (2 * p[:, 0] - p[:, 0])[:, None]
    r1 = oracle.derham_map(cx, coords, 1, f1, 3)
    r2 = oracle.derham_map(cx, coords, 2, df1, 3)
    assert np.abs(wc.dif(1) @ r1 - r2).max() < 1e-13


def test_derham_map_is_a_cochain_map_3d(oracle):
    """w = (y z, x^2, x y) on dx, dy, dz: dw = (dQ/dx - dP/dy) dxdy + (dR/dx - dP/dz) dxdz
    + (dR/dy - dQ/dz) dydz, colex order dx^dy, dx^dz, dy^dz."""
    cx, coords = _mesh(oracle, 3, 3)
    wc = oracle.WhitneyComplex(cx, cx.edge_lengths_sq(coords))
    f1 = lambda p: np.stack([p[:, 1] * p[:, 2], p[:, 0] ** 2, p[:, 0] * p[:, 1]], 1)
    df1 = lambda p: np.stack([2 * p[:, 0] - p[:, 2], p[:, 1] - p[:, 1], p[:, 0] - 0 * p[:, 0]], 1)
    r1 = oracle.derham_map(cx, coords, 1, f1, 3)
    r2 = oracle.derham_map(cx, coords, 2, df1, 3)
    assert np.abs(wc.dif(1) @ r1 - r2).max() < 1e-13


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_constant_forms_integrate_to_the_tangent_blade(oracle, dim):
    from test_oracle_golden import derham_constant

    cx, coords = _mesh(oracle, dim, 3)
    for k in range(dim + 1):
        ncomp = math.comb(dim, k)
        r = oracle.derham_map(cx, coords, k, lambda p: np.ones((len(p), ncomp)), 1)
        # itertools (lexicographic) and colex agree on the subsets of <= 3 axes
        assert np.abs(r - derham_constant(cx, coords, k)).max() < 1e-14
