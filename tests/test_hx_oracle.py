"""The HX-multigrid preconditioner's CPU restatement (oracle/hx_oracle.py).

Mirrors the reference's own checks of the structure: formoniq/src/hx.rs tests
(hx_cg_matches_the_direct_solve, hx_multigrid_matches_the_direct_solve),
formoniq/src/multigrid.rs tests (mg_cg_matches_the_direct_solve,
mg_cg_iterations_are_mesh_independent, galerkin_coarse_matches_reassembly), the
definition of vector_nodal_prolongation (hx.rs:89-125), iterative/src/aux_space.rs
(combiner_is_self_adjoint) and iterative/src/multigrid.rs
(vcycle_contracts_uniformly_in_h).
"""
import math

import numpy as np
import pytest
import scipy.sparse.linalg as spla

import hx_oracle as hxo


def make(oracle, dim, nbox, relative=False, seed=7, jitter=0.1):
    cx, coords = oracle.cartesian_unit(dim, nbox)
    coords = oracle.jitter_coords(coords, nbox, seed, jitter)
    lengths = cx.edge_lengths_sq(coords)
    return cx, lengths, oracle.WhitneyComplex(cx, lengths, relative=relative)


def pcg(A, apply_b, rhs, rtol=1e-10, maxit=2000):
    """krylov::cg (iterative/src/krylov.rs:48-95): stops on ||r|| / ||b||."""
    x = np.zeros_like(rhs)
    r = rhs.copy()
    z = apply_b(r)
    p = z.copy()
    rz = r @ z
    bn = np.linalg.norm(rhs)
    for it in range(1, maxit + 1):
        ap = A @ p
        alpha = rz / (p @ ap)
        x += alpha * p
        r -= alpha * ap
        if np.linalg.norm(r) <= rtol * bn:
            return x, it
        z = apply_b(r)
        rz_new = r @ z
        p = z + (rz_new / rz) * p
        rz = rz_new
    return x, maxit


@pytest.mark.parametrize("dim,nf", [(1, 7), (2, 6), (2, 5), (3, 4), (3, 5), (4, 3)])
@pytest.mark.parametrize("relative", [False, True])
def test_prolongation_reproduces_linear_functions(dim, nf, relative):
    nc = (nf + 1) // 2
    P = hxo.lattice_prolongation(dim, nf, nc, relative)
    rng = np.random.default_rng(dim * 10 + nf)
    g = rng.normal(size=dim)

    def nodal(nbox):
        vals = []
        for v in range((nbox + 1) ** dim):
            c = hxo.lattice_coords(v, dim, nbox)
            if hxo.node_index(c, dim, nbox, relative) < 0:
                continue
            x = np.array(c) / nbox
            # linear, vanishing on the boundary when relative (a bubble is not linear:
            # use the product form only for the absolute lattice)
            vals.append(g @ x + 0.3 if not relative else np.prod(x * (1 - x)))
        return np.array(vals)

    if not relative:
        np.testing.assert_allclose(P @ nodal(nc), nodal(nf), atol=1e-13)
        np.testing.assert_allclose(np.asarray(P.sum(axis=1)).ravel(), 1.0, atol=1e-14)
    else:
        assert P.shape == (max(nf - 1, 0) ** dim, max(nc - 1, 0) ** dim)
        assert (P.data > 0).all() and (np.asarray(P.sum(axis=1)).ravel() <= 1 + 1e-14).all()


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_vector_nodal_is_the_references_on_the_unit_box(oracle, dim):
    """hx.rs:89-125 restated from the mesh's true coordinates: entry
    (sigma, I * nvertices + a) = <e_I, tau_sigma> / (k+1)! for every vertex a of
    the k-simplex sigma, tau_sigma the ambient tangent blade (colex minors of
    the edge vectors from sigma's first vertex). On the unjittered unit box N = 2
    the lattice frame (per-axis RMS axis-edge length) is the true one, and the
    oracle's Pi_k equals it up to its node-major column order."""
    nbox = 2
    cx, coords = oracle.cartesian_unit(dim, nbox)
    lengths = cx.edge_lengths_sq(coords)
    h = hxo.lattice_spacing(cx, lengths, dim, nbox)
    np.testing.assert_allclose(h, 1.0 / nbox, rtol=1e-15)
    nv = cx.nsimplices(0)
    for k in range(1, dim + 1):
        subsets = hxo.colex_subsets(dim, k)
        simp = cx.simplices(k)
        want = np.zeros((len(simp), len(subsets) * nv))
        for row, s in enumerate(simp):
            e = (coords[s[1:]] - coords[s[0]]).T  # ambient x k
            for comp, sub in enumerate(subsets):
                value = np.linalg.det(e[sub, :]) / math.factorial(k + 1)
                for a in s:
                    want[row, comp * nv + a] = value
        got = hxo.vector_nodal(cx, k, dim, nbox, False, h).toarray()
        ncomp = len(subsets)
        perm = [(c % ncomp) * nv + c // ncomp for c in range(got.shape[1])]  # node-major -> I-major
        reordered = np.zeros_like(want)
        reordered[:, perm] = got
        np.testing.assert_allclose(reordered, want, rtol=0, atol=1e-14)


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("relative", [False, True])
def test_galerkin_coarse_matches_reassembly(oracle, dim, relative):
    """multigrid.rs:250-281 on the lattice levels: on the unjittered unit box
    the Kuhn mesh of 2N refines the one of N, so the reference's refinement
    tower and this lattice coarsening give the same levels there, and P^T A_f P
    of the grade-0 hdif_gram equals the operator reassembled on the coarse mesh
    (relative Frobenius 1e-10)."""
    nc, nf = 2, 4

    def hdif0(nbox):
        cx, coords = oracle.cartesian_unit(dim, nbox)
        return oracle.WhitneyComplex(cx, cx.edge_lengths_sq(coords), relative=relative).hdif_gram(0).toarray()

    P = hxo.lattice_prolongation(dim, nf, nc, relative)
    galerkin = P.T @ hdif0(nf) @ P
    want = hdif0(nc)
    assert np.linalg.norm(galerkin - want) < 1e-10 * np.linalg.norm(want)


@pytest.mark.parametrize("dim", [2, 3])
def test_vcycle_contracts_uniformly(oracle, dim):
    rates = []
    for nbox in ([32, 64] if dim == 2 else [8, 16]):
        cx, lengths, wc = make(oracle, dim, nbox)
        mg = hxo.NodalMultigrid(wc.hdif_gram(0), dim, nbox, False)
        assert len(mg.A) >= 2  # a real hierarchy, not the coarse solve alone
        A = wc.hdif_gram(0)
        b = A @ np.sin(np.arange(A.shape[0]) + 1.0)
        x = np.zeros_like(b)
        prev = np.linalg.norm(b)
        for _ in range(4):
            x += mg.apply((b - A @ x)[:, None])[:, 0]
            cur = np.linalg.norm(b - A @ x)
            rate = cur / prev
            prev = cur
        rates.append(rate)
    assert max(rates) < 0.35, rates


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("relative", [False, True])
def test_hx_is_self_adjoint(oracle, dim, relative):
    cx, lengths, wc = make(oracle, dim, 4, relative=relative)
    hx = hxo.HxPreconditioner(wc, cx, lengths, 4, relative)
    rng = np.random.default_rng(3)
    for j in range(dim + 1):
        n = wc.ndofs(j)
        r, s = rng.normal(size=n), rng.normal(size=n)
        a, b = hx.apply(j, r) @ s, r @ hx.apply(j, s)
        assert abs(a - b) <= 1e-12 * max(abs(a), 1.0), (j, a, b)
        assert hx.apply(j, r) @ r > 0


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("relative", [False, True])
def test_hx_cg_matches_the_direct_solve(oracle, dim, relative):
    nbox = 4
    cx, lengths, wc = make(oracle, dim, nbox, relative=relative)
    hx = hxo.HxPreconditioner(wc, cx, lengths, nbox, relative)
    for j in range(1, dim + 1):
        A = wc.hdif_gram(j).tocsc()
        n = A.shape[0]
        rhs = np.cos(np.arange(n) ** 2 + 1.0)
        x, its = pcg(A, lambda r: hx.apply(j, r), rhs)
        assert its < 200
        assert np.linalg.norm(x - spla.spsolve(A, rhs)) < 1e-7 * max(1.0, np.linalg.norm(x))


def test_hx_cg_iterations_are_mesh_independent(oracle):
    its = {}
    for nbox in (4, 8, 16):
        cx, lengths, wc = make(oracle, 2, nbox)
        hx = hxo.HxPreconditioner(wc, cx, lengths, nbox, False)
        A = wc.hdif_gram(1)
        rhs = np.log(np.arange(A.shape[0]) + 2.0)
        _, its[nbox] = pcg(A, lambda r: hx.apply(1, r), rhs)
        _, plain = pcg(A, lambda r: r / A.diagonal(), rhs, maxit=20000)
        its[(nbox, "jacobi")] = plain
    assert its[16] <= its[4] + 8, its
    assert its[16] * 3 < its[(16, "jacobi")], its
