"""The sparse direct solver (fq_sparse_lu_*) and the direct route of the
Hodge-Dirac source problem, against SciPy SuperLU (the faer LU stand-in) on the
oracle's systems.

Bars: solutions within 1e-8 relative of the direct solve (the reference's
block-MINRES-vs-LU assertion is 1e-7, problems/elliptic.rs:280-284). GMRES
stops on the true FP64 relative residual, or at the FP64 backward-error floor
of a nearly singular system, where an LU solve stops too."""
import numpy as np
import pytest
import scipy.sparse.linalg as spla

import formoniq_gb300 as fq

pytestmark = pytest.mark.gpu

SOLVE_TOL = 1e-8


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def lattice_mesh(oracle, ctx, dim, nb, minkowski, seed=8, jitter=0.05):
    """A Kuhn box with signed squared lengths s (1 + U(-jitter, jitter))
    (Minkowski: time axis 0 scaled 0.7), on both sides."""
    if minkowski:
        cx, coords, signs = oracle.minkowski(dim, nb)
        lengths = cx.edge_lengths_sq(coords, signs)
    else:
        cx, coords = oracle.cartesian_unit(dim, nb)
        lengths = cx.edge_lengths_sq(coords)
    lengths = lengths * (1.0 + jitter * oracle.uniform_pm1(seed, np.arange(len(lengths), dtype=np.uint64)))
    mesh = fq.Mesh.kuhn_cube(ctx, dim, nb)
    mesh.set_lengths_sq(lengths)
    return cx, lengths, mesh


@pytest.mark.parametrize("dim,nb,mink", [(3, 3, True), (3, 4, True), (3, 6, True), (3, 5, False), (2, 12, True),
                                         (2, 9, False), (4, 2, True), (4, 3, False)])
def test_dirac_direct_matches_superlu(oracle, ctx, dim, nb, mink):
    cx, lengths, mesh = lattice_mesh(oracle, ctx, dim, nb, mink)
    ntot = sum(cx.nsimplices(k) for k in range(dim + 1))
    rng = np.random.default_rng(nb)
    load = rng.standard_normal(ntot)
    lift = np.where(rng.random(ntot) < 0.3, rng.standard_normal(ntot), 0.0)
    want = oracle.dirac_solve_source(cx, lengths, 1.5, load, lift)
    x, rep = fq.solve_dirac_source(mesh, 1.5, load, lift, fq.SolveOpts.default(rtol=1e-12, max_iters=300))
    assert rep.converged, rep
    assert rel(x, want) < SOLVE_TOL
    mesh.close()


@pytest.mark.parametrize("nb", [8, 10])
def test_dirac_direct_at_stream_sizes(oracle, ctx, nb):
    """Minkowski 1+2 boxes of the served stream's sizes (N = 8: 3,072 cells;
    N = 10: 6,000 cells), where MINRES with the comparison preconditioners
    needs 18,000+ iterations or does not converge."""
    cx, lengths, mesh = lattice_mesh(oracle, ctx, 3, nb, True, seed=nb)
    ntot = sum(cx.nsimplices(k) for k in range(4))
    load = np.random.default_rng(nb + 1).standard_normal(ntot)
    want = oracle.dirac_solve_source(cx, lengths, 1.5, load, np.zeros(ntot))
    x, rep = fq.solve_dirac_source(mesh, 1.5, load, None, fq.SolveOpts.default(rtol=1e-10, max_iters=300))
    assert rep.converged, rep
    assert rel(x, want) < SOLVE_TOL
    mesh.close()


@pytest.mark.parametrize("dim,nb,mink", [(3, 4, True), (3, 4, False), (2, 8, True), (3, 8, True), (4, 3, True),
                                         (4, 3, False)])
def test_massless_dirac_bordered(oracle, ctx, dim, nb, mink):
    """m = 0: the relative system is singular with the top-grade harmonic as its
    kernel; both sides border it (solve_bordered, problems/dirac.rs:578-598) and
    return the solution orthogonal to it. The device factors the bordered
    system with a small mass shift (the unshifted one has structurally zero
    pivots); GMRES on the exact system then needs few iterations."""
    cx, lengths, mesh = lattice_mesh(oracle, ctx, dim, nb, mink)
    ntot = sum(cx.nsimplices(k) for k in range(dim + 1))
    load = np.random.default_rng(3).standard_normal(ntot)
    want = oracle.dirac_solve_source(cx, lengths, 0.0, load, np.zeros(ntot))
    x, rep = fq.solve_dirac_source(mesh, 0.0, load, None, fq.SolveOpts.default(rtol=1e-12, max_iters=300))
    assert rep.converged, rep
    assert rep.iters <= 40, rep
    assert rel(x, want) < SOLVE_TOL
    mesh.close()


@pytest.mark.parametrize("mass", [1e-5, -1e-5])
def test_nearly_massless_dirac(oracle, ctx, mass):
    """0 < |m| below the shift: the system is regular (no border) but nearly
    singular; the factored matrix carries the shift, GMRES the true mass."""
    dim, nb = 3, 4
    cx, lengths, mesh = lattice_mesh(oracle, ctx, dim, nb, True)
    ntot = sum(cx.nsimplices(k) for k in range(dim + 1))
    load = np.random.default_rng(4).standard_normal(ntot)
    want = oracle.dirac_solve_source(cx, lengths, mass, load, np.zeros(ntot))
    x, rep = fq.solve_dirac_source(mesh, mass, load, None, fq.SolveOpts.default(rtol=1e-12, max_iters=300))
    assert rep.converged, rep
    assert rep.iters <= 40, rep
    assert rel(x, want) < SOLVE_TOL
    mesh.close()


def test_massless_dirac_needs_the_direct_route(oracle, ctx):
    cx, lengths, mesh = lattice_mesh(oracle, ctx, 3, 3, True)
    ntot = sum(cx.nsimplices(k) for k in range(4))
    with pytest.raises(fq.FqError) as e:
        fq.solve_dirac_source(mesh, 0.0, np.ones(ntot), None, fq.SolveOpts.default(preconditioner=fq.FQ_PC_JACOBI))
    assert e.value.name == "FQ_UNSUPPORTED"
    mesh.close()


@pytest.mark.parametrize("which", ["dirac", "kkt"])
def test_sparse_lu_api_against_superlu(oracle, ctx, which):
    """fq_sparse_lu_create / factor / solve on an assembled system: the
    relative Dirac system, and the Lorentzian mixed k=1 KKT system (no SPD
    preconditioner: the reference's LU route of solve_source)."""
    dim, nb = 3, 5
    cx, lengths, mesh = lattice_mesh(oracle, ctx, dim, nb, True)
    if which == "dirac":
        a = fq.dirac_system(mesh, 1.5)
    else:
        prob = fq.MixedProblem(mesh, 1, fq.FQ_ABSOLUTE, fq.FQ_FP64)
        a = prob.system()
    lu = fq.SparseLu(mesh, a).factor()
    info = lu.info()
    assert info["fronts"] > 1 and info["levels"] > 1 and info["factor_bytes"] > 0
    A = a.to_scipy()
    b = np.random.default_rng(11).standard_normal(A.shape[0])
    want = spla.spsolve(A.tocsc(), b)
    for _ in range(2):  # a second solve on the same factors
        x, rep = lu.solve(b, fq.SolveOpts.default(rtol=1e-12, max_iters=300))
        assert rep.converged, rep
        assert rel(x, want) < SOLVE_TOL
    # re-factor after new values on the same pattern
    lengths2 = lengths * (1.0 + 0.01 * oracle.uniform_pm1(99, np.arange(len(lengths), dtype=np.uint64)))
    mesh.set_lengths_sq(lengths2)
    if which == "dirac":
        a.reassemble(mesh)
    else:
        prob.reassemble()
    lu.factor()
    A2 = a.to_scipy()
    x, rep = lu.solve(b, fq.SolveOpts.default(rtol=1e-12, max_iters=300))
    assert rep.converged and rel(x, spla.spsolve(A2.tocsc(), b)) < SOLVE_TOL
    # max_refinements = 0: GMRES on the given factors only, no refactorization: FP32,
    # float-float (FQ_FP64) and IEEE FP64 factors each precondition to the same solution
    want2 = spla.spsolve(A2.tocsc(), b)
    iters = {}
    for prec in (fq.FQ_FP32, fq.FQ_FP64, fq.FQ_FP64_IEEE):
        lu.factor(prec)
        x, rep = lu.solve(b, fq.SolveOpts.default(rtol=1e-12, max_iters=300, max_refinements=0))
        assert rep.converged and rep.refinements == 0, (prec, rep)
        assert rel(x, want2) < SOLVE_TOL, prec
        iters[prec] = rep.iters
    # the 48-bit factors are as good a preconditioner as the 53-bit ones
    assert iters[fq.FQ_FP64] <= iters[fq.FQ_FP64_IEEE] + 1, iters
    lu.close()


def test_sparse_lu_rejects_non_lattice_meshes(oracle, ctx):
    mesh = fq.Mesh.from_cells(ctx, oracle.kuhn_cells(3, 3))
    cx2, coords = oracle.cartesian_unit(3, 3)
    mesh.set_lengths_sq(cx2.edge_lengths_sq(coords))
    a = fq.dirac_system(mesh, 1.5)
    with pytest.raises(fq.FqError) as e:
        fq.SparseLu(mesh, a)
    assert e.value.name == "FQ_UNSUPPORTED"


@pytest.mark.parametrize("dim,nb,k,relative", [(3, 4, 1, False), (2, 8, 1, True), (3, 3, 2, False), (2, 6, 0, False)])
def test_lorentzian_mixed_solve_by_sparse_lu(oracle, ctx, dim, nb, k, relative):
    """solve_source on a Minkowski mesh: the hdif_gram blocks are indefinite,
    so no block preconditioner exists and LU carries the solve
    (elliptic.rs:153-160); the device counts the cells whose metric is not
    positive definite and takes the sparse direct route."""
    cx, lengths, mesh = lattice_mesh(oracle, ctx, dim, nb, True)
    owc = oracle.WhitneyComplex(cx, lengths, relative=relative)
    src = np.random.default_rng(21).standard_normal(cx.nsimplices(k))
    harm = oracle.harmonics(owc, k)
    a, rhs, ns, nu = oracle.assemble_mixed_kkt(owc, src, k, harm)
    x_o = oracle.direct_solve(a, rhs)
    want = np.concatenate(([owc.inclusion(k - 1) @ x_o[:ns]] if k > 0 else []) + [owc.inclusion(k) @ x_o[ns:ns + nu]])
    gwc = fq.WhitneyComplex(mesh, relative=relative)
    sigma, u, _, rep = fq.solve_source(gwc, src, k, fq.SolveOpts.default(rtol=1e-12, max_iters=300))
    assert rep.converged, rep
    assert rep.iters <= 60, rep
    got = np.concatenate(([sigma] if k > 0 else []) + [u])
    assert rel(got, want) < SOLVE_TOL
    mesh.close()
