"""The device HX-multigrid preconditioner against its CPU restatement, and the
solves it preconditions against direct solves.

References: formoniq/src/hx.rs (hx_preconditioner and its tests
hx_cg_matches_the_direct_solve / hx_multigrid_matches_the_direct_solve),
formoniq/src/multigrid.rs, iterative/src/aux_space.rs,
problems/elliptic.rs:29-47 (the mixed system's block preconditioner).
"""
import math

import numpy as np
import pytest
import scipy.sparse.linalg as spla

import formoniq_gb300 as fq
import hx_oracle as hxo

pytestmark = pytest.mark.gpu

APPLY_TOL = 1e-11   # B r on the device vs the restatement (different summation orders)
SOLVE_TOL = 1e-8


def kuhn_pair(oracle, ctx, dim, nb, relative=False, seed=7, jitter=0.1):
    cx, coords = oracle.cartesian_unit(dim, nb)
    coords = oracle.jitter_coords(coords, nb, seed, jitter)
    lengths = cx.edge_lengths_sq(coords)
    mesh = fq.Mesh.kuhn_cube(ctx, dim, nb)
    mesh.set_lengths_sq(lengths)
    return cx, mesh, lengths, oracle.WhitneyComplex(cx, lengths, relative=relative)


@pytest.mark.parametrize("dim,nb", [(1, 40), (2, 8), (2, 20), (3, 4), (3, 9), (4, 4)])
@pytest.mark.parametrize("relative", [False, True])
def test_hx_apply_matches_the_restatement(oracle, ctx, dim, nb, relative):
    cx, mesh, lengths, wc = kuhn_pair(oracle, ctx, dim, nb, relative)
    hx = hxo.HxPreconditioner(wc, cx, lengths, nb, relative)
    bc = fq.FQ_RELATIVE if relative else fq.FQ_ABSOLUTE
    rng = np.random.default_rng(dim * 100 + nb)
    for j in range(min(dim, 3) + 1):
        n = wc.ndofs(j)
        if n == 0:
            continue
        r = rng.standard_normal(n)
        got = fq.hx_apply(mesh, j, bc, r)
        want = hx.apply(j, r)
        err = np.linalg.norm(got - want) / np.linalg.norm(want)
        assert err < APPLY_TOL, (j, err)
    mesh.close()


@pytest.mark.parametrize("dim,nb", [(2, 16), (3, 6)])
@pytest.mark.parametrize("relative", [False, True])
def test_hx_cg_matches_the_direct_solve(oracle, ctx, dim, nb, relative):
    cx, mesh, lengths, wc = kuhn_pair(oracle, ctx, dim, nb, relative)
    bc = fq.FQ_RELATIVE if relative else fq.FQ_ABSOLUTE
    for j in range(1, dim + 1):
        A = wc.hdif_gram(j).tocsc()
        rhs = np.cos(np.arange(A.shape[0]) ** 2 + 1.0)
        x, rep = fq.hx_cg(mesh, j, bc, rhs, fq.SolveOpts.default(rtol=1e-10))
        assert rep.converged and rep.iters < 100, (j, rep)
        direct = spla.spsolve(A, rhs)
        assert np.linalg.norm(x - direct) < 1e-7 * max(1.0, np.linalg.norm(direct)), j
    mesh.close()


def test_hx_cg_iterations_stay_flat_under_refinement(oracle, ctx):
    its = []
    for nb in (8, 16, 32):
        cx, mesh, lengths, wc = kuhn_pair(oracle, ctx, 3, nb)
        n = mesh.nsimplices(1)
        rhs = np.log(np.arange(n) + 2.0)
        _, rep = fq.hx_cg(mesh, 1, fq.FQ_ABSOLUTE, rhs, fq.SolveOpts.default(rtol=1e-10))
        assert rep.converged
        its.append(rep.iters)
        mesh.close()
    assert its[-1] <= its[0] + 10, its


@pytest.mark.parametrize("dim,nb,grade", [(2, 12, 1), (3, 6, 1), (3, 6, 2), (4, 3, 2)])
@pytest.mark.parametrize("relative", [False, True])
def test_mixed_solve_with_hx_blocks_matches_direct(oracle, ctx, dim, nb, grade, relative):
    cx, mesh, lengths, owc = kuhn_pair(oracle, ctx, dim, nb, relative, seed=11)
    src = np.random.default_rng(grade).standard_normal(cx.nsimplices(grade))
    harm = oracle.harmonics(owc, grade)
    a, rhs, ns, nu = oracle.assemble_mixed_kkt(owc, src, grade, harm)
    x = oracle.direct_solve(a, rhs)
    sig_o = owc.inclusion(grade - 1) @ x[:ns] if grade > 0 else np.zeros(0)
    u_o = owc.inclusion(grade) @ x[ns:ns + nu]
    gwc = fq.WhitneyComplex(mesh, relative=relative)
    res = {}
    for pc in (fq.FQ_PC_HX, fq.FQ_PC_JACOBI):
        sigma, u, p, rep = fq.solve_source(gwc, src, grade, fq.SolveOpts.default(rtol=1e-12, preconditioner=pc))
        assert rep.converged, (pc, rep)
        scale = max(np.linalg.norm(x), 1.0)
        err = math.sqrt(np.linalg.norm(u - u_o) ** 2 + (np.linalg.norm(sigma - sig_o) ** 2 if grade else 0.0))
        assert err / scale < SOLVE_TOL, (pc, err / scale, rep)
        res[pc] = rep.iters
    assert res[fq.FQ_PC_HX] < res[fq.FQ_PC_JACOBI], res
    mesh.close()


def test_mixed_fp32_refinement_with_hx(oracle, ctx):
    cx, mesh, lengths, owc = kuhn_pair(oracle, ctx, 3, 8, seed=12)
    src = np.random.default_rng(2).standard_normal(cx.nsimplices(1))
    a, rhs, ns, nu = oracle.assemble_mixed_kkt(owc, src, 1, np.zeros((cx.nsimplices(1), 0)))
    x = oracle.direct_solve(a, rhs)
    prob = fq.MixedProblem(mesh, 1, fq.FQ_ABSOLUTE, fq.FQ_FP32)
    opts = fq.SolveOpts.default(rtol=1e-6, precision=fq.FQ_FP32, refine_rtol=1e-12, preconditioner=fq.FQ_PC_HX)
    sigma, u, p, rep = prob.solve(src, opts)
    assert rep.true_residual <= 1e-12, rep
    err = math.sqrt(np.linalg.norm(u - x[ns:]) ** 2 + np.linalg.norm(sigma - x[:ns]) ** 2) / np.linalg.norm(x)
    assert err < SOLVE_TOL, err
    prob.close()
    mesh.close()


def test_hx_refuses_non_kuhn_and_lorentzian_meshes(oracle, ctx):
    cx, coords = oracle.cartesian_unit(2, 4)
    mesh = fq.Mesh.from_cells(ctx, oracle.kuhn_cells(2, 4))
    mesh.set_lengths_sq(cx.edge_lengths_sq(coords))
    with pytest.raises(fq.FqError):
        fq.hx_cg(mesh, 1, fq.FQ_ABSOLUTE, np.ones(mesh.nsimplices(1)))
    mesh.close()
    cx, coords, signs = oracle.minkowski(2, 4)
    mesh = fq.Mesh.kuhn_cube(ctx, 2, 4)
    mesh.set_lengths_sq(cx.edge_lengths_sq(coords, signs))
    with pytest.raises(fq.FqError):
        fq.hx_apply(mesh, 1, fq.FQ_ABSOLUTE, np.ones(mesh.nsimplices(1)))
    mesh.close()


def test_refresh_after_new_lengths_equals_a_fresh_build(oracle, ctx):
    """Reassembly with new lengths refreshes the preconditioner's numbers on the
    kept lattice structure; the solve is then the one a fresh problem gives."""
    dim, nb, grade = 3, 6, 1
    cx, coords = oracle.cartesian_unit(dim, nb)
    l1 = cx.edge_lengths_sq(oracle.jitter_coords(coords, nb, 1, 0.1))
    l2 = cx.edge_lengths_sq(oracle.jitter_coords(coords, nb, 2, 0.15))
    src = np.random.default_rng(5).standard_normal(cx.nsimplices(grade))
    opts = fq.SolveOpts.default(rtol=1e-12, preconditioner=fq.FQ_PC_HX)
    mesh = fq.Mesh.kuhn_cube(ctx, dim, nb)
    mesh.set_lengths_sq(l1)
    prob = fq.MixedProblem(mesh, grade, fq.FQ_ABSOLUTE, fq.FQ_FP64)
    prob.solve(src, opts)
    mesh.set_lengths_sq(l2)
    prob.reassemble()
    s1, u1, _, r1 = prob.solve(src, opts)
    prob.close()
    mesh.close()
    fresh = fq.Mesh.kuhn_cube(ctx, dim, nb)
    fresh.set_lengths_sq(l2)
    prob2 = fq.MixedProblem(fresh, grade, fq.FQ_ABSOLUTE, fq.FQ_FP64)
    s2, u2, _, r2 = prob2.solve(src, opts)
    prob2.close()
    fresh.close()
    assert r1.iters == r2.iters, (r1, r2)
    np.testing.assert_array_equal(u1, u2)
    np.testing.assert_array_equal(s1, s2)
