"""The de Rham map on the GPU (fq_derham_nodes / fq_derham_reduce) against the
oracle's restatement of derham/src/project.rs:53-96, and the load of the
configuration-1 source problem, M_1 R f, against the oracle's."""
import math

import numpy as np
import pytest

import formoniq_gb300 as fq

pytestmark = pytest.mark.gpu

TOL = 1e-13


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def setup(oracle, ctx, dim, nb, seed=5):
    import torch

    cx, coords = oracle.cartesian_unit(dim, nb)
    coords = oracle.jitter_coords(coords, nb, seed, 0.1)
    mesh = fq.Mesh.kuhn_cube(ctx, dim, nb)
    mesh.set_lengths_sq(cx.edge_lengths_sq(coords))
    return cx, coords, mesh, torch.tensor(coords, device="cuda")


def poly_form(xp, p, k, ncomp):
    """A polynomial k-form of degree <= 3 with distinct components (xp: numpy or torch)."""
    cols = []
    for c in range(ncomp):
        a = p[:, c % p.shape[1]]
        b = p[:, (c + 1) % p.shape[1]]
        cols.append(1.0 + (c + 1) * a * b - 0.5 * a ** 3 + 0.25 * c * b)
    return xp.stack(cols, 1)


@pytest.mark.parametrize("dim,nb", [(2, 5), (3, 3), (4, 2)])
def test_derham_map_matches_oracle(oracle, ctx, dim, nb):
    import torch

    cx, coords, mesh, dcoords = setup(oracle, ctx, dim, nb)
    for k in range(dim + 1):
        ncomp = math.comb(dim, k)
        for degree in (1, 3, 5):
            want = oracle.derham_map(cx, coords, k, lambda p: poly_form(np, p, k, ncomp), degree)
            got = fq.derham_map(mesh, dcoords, k, lambda p: poly_form(torch, p, k, ncomp), degree).cpu().numpy()
            assert rel(got, want) < TOL, (k, degree)


def test_derham_map_commutes_with_the_coboundary(oracle, ctx):
    """Stokes on the device: R d w = d R w for w = (y z, x^2, x y)."""
    import torch

    cx, coords, mesh, dcoords = setup(oracle, ctx, 3, 4)
    f1 = lambda p: torch.stack([p[:, 1] * p[:, 2], p[:, 0] ** 2, p[:, 0] * p[:, 1]], 1)
    df1 = lambda p: torch.stack([2 * p[:, 0] - p[:, 2], 0 * p[:, 0], p[:, 0]], 1)
    r1 = fq.derham_map(mesh, dcoords, 1, f1, 3).cpu().numpy()
    r2 = fq.derham_map(mesh, dcoords, 2, df1, 3).cpu().numpy()
    d1 = fq.WhitneyComplex(mesh).dif(1).to_scipy()
    assert np.abs(d1 @ r1 - r2).max() < 1e-13


def test_configuration_1_load(oracle, ctx):
    """f = (sin(pi x) cos(pi y), cos(pi x) sin(pi y)) on the jittered 2D unit
    square: the Galerkin load M_1 R f of its Whitney interpolant."""
    import torch

    cx, coords, mesh, dcoords = setup(oracle, ctx, 2, 16)
    pi = math.pi
    fn = lambda p: np.stack([np.sin(pi * p[:, 0]) * np.cos(pi * p[:, 1]), np.cos(pi * p[:, 0]) * np.sin(pi * p[:, 1])], 1)
    ft = lambda p: torch.stack([torch.sin(pi * p[:, 0]) * torch.cos(pi * p[:, 1]),
                                torch.cos(pi * p[:, 0]) * torch.sin(pi * p[:, 1])], 1)
    rf_o = oracle.derham_map(cx, coords, 1, fn, 3)
    rf = fq.derham_map(mesh, dcoords, 1, ft, 3)
    assert rel(rf.cpu().numpy(), rf_o) < TOL
    m1 = fq.WhitneyComplex(mesh).mass(1)
    b = torch.empty_like(rf)
    torch.cuda.synchronize()
    ctx.check(ctx.L.fq_spmv(ctx.h, m1.h, fq._P(rf.data_ptr()), fq._P(b.data_ptr())))
    ctx.synchronize()
    want = oracle.WhitneyComplex(cx, cx.edge_lengths_sq(coords)).mass(1) @ rf_o
    assert rel(b.cpu().numpy(), want) < 1e-12
