"""The oracle's source load (SourceForm::element, formoniq/src/operators.rs:598-635,
summed by assemble_vector, galerkin.rs:279-312) pinned by the reference's own
laws: the load of a Whitney form is a column of the mass matrix
(galerkin.rs:334-371), a constant scalar source gives the P1 load vol/(n+1)
(the source of tests/hodge_theory.rs:168-180), and a flat constant k-form gives
M_k times its de Rham cochain (Whitney forms reproduce constants)."""
import math

import numpy as np
import pytest


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_load_of_a_whitney_form_is_a_mass_column(oracle, dim):
    cx, coords = oracle.cartesian_unit(dim, 2)
    lengths = cx.edge_lengths_sq(coords)
    wc = oracle.WhitneyComplex(cx, lengths)
    bary, _ = oracle.gm_rule(dim, 4)
    for k in range(dim + 1):
        nd = cx.nsimplices(k)
        basis = np.zeros(nd)
        basis[nd // 2] = 1.0
        vals = oracle.whitney_interpolant_values(cx, k, basis, bary)
        load = oracle.source_form(cx, lengths, k, vals, degree=4)
        assert rel(load, wc.mass(k) @ basis) < 1e-13, k
        # u^T load is the L2 pairing of u with the Whitney form (the reference's check)
        u = (np.arange(nd) % 7) - 3.0
        assert abs(u @ load - u @ (wc.mass(k) @ basis)) < 1e-12
        # and the load is not the de Rham cochain of the same field
        assert np.linalg.norm(load - basis) > 1e-9


@pytest.mark.parametrize("dim", [1, 2, 3, 4])
def test_constant_scalar_load(oracle, dim):
    nb = 2 if dim == 4 else 3
    cx, coords = oracle.cartesian_unit(dim, nb)
    coords = oracle.jitter_coords(coords, nb, seed=4, amplitude=0.1)
    lengths = cx.edge_lengths_sq(coords)
    _, w = oracle.gm_rule(dim, 1)
    load = oracle.source_form(cx, lengths, 0, np.ones((cx.ncells(), len(w), 1)), degree=1)
    _, _, _, vol, _ = cx.cell_metrics(lengths)
    want = np.zeros(cx.nsimplices(0))
    np.add.at(want, cx.simplices(dim).ravel(), np.repeat(vol / (dim + 1), dim + 1))
    assert rel(load, want) < 1e-14


@pytest.mark.parametrize("dim", [2, 3])
def test_flat_constant_form_load_is_mass_times_derham(oracle, dim):
    nb = 3
    cx, coords = oracle.cartesian_unit(dim, nb)
    coords = oracle.jitter_coords(coords, nb, seed=3, amplitude=0.1)
    lengths = cx.edge_lengths_sq(coords)
    wc = oracle.WhitneyComplex(cx, lengths)
    for k in range(1, dim + 1):
        ncomp = math.comb(dim, k)
        comp = np.arange(1, ncomp + 1, dtype=float)
        _, w = oracle.gm_rule(dim, 2)
        vals = np.broadcast_to(comp, (cx.ncells(), len(w), ncomp)).copy()
        load = oracle.source_form(cx, lengths, k, vals, degree=2, coords=coords)
        rw = oracle.derham_map(cx, coords, k, lambda x: np.broadcast_to(comp, (len(x), ncomp)), degree=1)
        assert rel(load, wc.mass(k) @ rw) < 1e-13, k


def test_relative_load_is_the_restriction(oracle):
    cx, coords = oracle.cartesian_unit(2, 3)
    lengths = cx.edge_lengths_sq(coords)
    _, w = oracle.gm_rule(2, 3)
    vals = np.random.default_rng(1).standard_normal((cx.ncells(), len(w), 2))
    full = oracle.source_form(cx, lengths, 1, vals, degree=3)
    rel_ = oracle.source_form(cx, lengths, 1, vals, degree=3, relative=True)
    assert np.array_equal(rel_, full[cx.interior(1)])
