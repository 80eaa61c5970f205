"""Parity at the benchmarked workloads' own sizes, through the C ABI.

The other parity tests use small meshes that the oracle finishes in seconds.
These run the timed workloads themselves against the oracle on the same seeded
inputs:

- the 3D 32^3 assembly step (196,608 tets): M_1, M_2, dif_both(2), dif_both(3)
  in both FP64 modes, CSR pattern bit-exact, values within 1e-12 relative
  Frobenius;
- the 3D 32^3 mixed k=1 solve (274,625 DOFs) in FP64 and FP32-with-FP64-
  refinement, within 1e-8 of the oracle's MINRES at rtol 1e-12 (Paige-Saunders,
  iterative/src/krylov.rs:113-211; the solution does not depend on the
  preconditioner, so the oracle uses its restatement of the HX blocks);
- the 2D 64^2 source problem end to end (elliptic.rs:132-182): de Rham map of
  f = (sin(pi x) cos(pi y), cos(pi x) sin(pi y)), the Galerkin load M_1 R f and
  the mixed k=1 solve, within 1e-8 of SciPy SuperLU (the faer LU stand-in) on
  the oracle's KKT system, on the full and the relative complex;
- the 4D 12^4 mixed k=2 system (1,483,536 DOFs, 94 M nonzeros): the KKT matrix
  against the oracle's assemble_mixed_kkt, and the FP64 and FP32-refined
  solutions within 1e-8 of the oracle's MINRES at rtol 1e-12.
"""
import math

import numpy as np
import pytest

import formoniq_gb300 as fq

pytestmark = pytest.mark.gpu

SEED = 20261203
FP64_TOL = 1e-12
SOLVE_TOL = 1e-8


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def config_mesh(oracle, ctx, dim, nb, seed=SEED):
    """The seeded +-0.1h jittered Kuhn mesh of a workload, on both sides."""
    cx, coords = oracle.cartesian_unit(dim, nb)
    coords = oracle.jitter_coords(coords, nb, seed, 0.1)
    lengths = cx.edge_lengths_sq(coords)
    mesh = fq.Mesh.kuhn_cube(ctx, dim, nb)
    mesh.set_lengths_sq(lengths)
    return cx, coords, lengths, mesh


def assert_csr_parity(got, want, tol=FP64_TOL):
    assert got.shape == want.shape
    np.testing.assert_array_equal(got.indptr.astype(np.int64), want.indptr.astype(np.int64))
    np.testing.assert_array_equal(got.indices.astype(np.int64), want.indices.astype(np.int64))
    err = rel(got.data, want.data)
    assert err <= tol, err
    return err


def oracle_mixed_minres(oracle, cx, lengths, nb, k, source, rtol=1e-12):
    """The oracle's solve_source system at rtol 1e-12: assemble_mixed_kkt and
    MINRES with block preconditioner (HX restatement for both blocks)."""
    import hx_oracle

    wc = oracle.WhitneyComplex(cx, lengths)
    harm = oracle.harmonics(wc, k)
    a, rhs, ns, nu = oracle.assemble_mixed_kkt(wc, source, k, harm)
    hx = hx_oracle.HxPreconditioner(wc, cx, lengths, nb, False)

    def pc(r):
        parts = [hx.apply(k - 1, r[:ns])] if k > 0 else []
        return np.concatenate(parts + [hx.apply(k, r[ns:ns + nu]), r[ns + nu:]])

    x, rep = oracle.minres(a, pc, rhs, rtol=rtol)
    assert rep.converged, rep
    return a, x, ns, nu


# ---------------------------------------------------------------------------
# 3D 32^3: the timed assembly step and the timed solve
# ---------------------------------------------------------------------------

@pytest.fixture(scope="module")
def cube32(oracle, ctx):
    cx, coords, lengths, mesh = config_mesh(oracle, ctx, 3, 32)
    yield cx, lengths, mesh
    mesh.close()


def test_device_lengths_of_the_benchmarked_mesh(oracle, ctx, cube32):
    """The bench generates the jittered lengths on the device; they are the
    oracle's to rounding."""
    _, lengths, _ = cube32
    m = fq.Mesh.kuhn_cube(ctx, 3, 32)
    m.kuhn_lengths(jitter=0.1, seed=SEED)
    np.testing.assert_allclose(m.lengths_sq(), lengths, rtol=1e-14)
    m.close()


@pytest.mark.parametrize("precision", [fq.FQ_FP64, fq.FQ_FP64_IEEE])
def test_step_matrices_3d32(oracle, ctx, cube32, precision):
    cx, lengths, mesh = cube32
    owc = oracle.WhitneyComplex(cx, lengths)
    gwc = fq.WhitneyComplex(mesh, precision=precision)
    for name, k in (("mass", 1), ("mass", 2), ("dif_both", 2), ("dif_both", 3)):
        g = getattr(gwc, name)(k)
        g.reassemble(mesh)  # the timed path: re-assembly on the built plan
        assert_csr_parity(g.to_scipy(), getattr(owc, name)(k))
        g.close()


def test_mixed_solve_3d32(oracle, ctx, cube32):
    cx, lengths, mesh = cube32
    src = np.random.default_rng(SEED).standard_normal(cx.nsimplices(1))
    _, want, ns, nu = oracle_mixed_minres(oracle, cx, lengths, 32, 1, src)
    p64 = fq.MixedProblem(mesh, 1, fq.FQ_ABSOLUTE, fq.FQ_FP64)
    sig, u, _, rep = p64.solve(src, fq.SolveOpts.default(rtol=1e-10))
    assert rep.converged
    assert rel(np.concatenate([sig, u]), want) < SOLVE_TOL
    p64.close()
    p32 = fq.MixedProblem(mesh, 1, fq.FQ_ABSOLUTE, fq.FQ_FP32)
    opts = fq.SolveOpts.default(rtol=1e-5, precision=fq.FQ_FP32, refine_rtol=1e-10, max_refinements=8)
    sig, u, _, rep = p32.solve(src, opts)
    assert rep.converged
    assert rel(np.concatenate([sig, u]), want) < SOLVE_TOL
    p32.close()


# ---------------------------------------------------------------------------
# 2D 64^2: the source problem end to end
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("relative", [False, True])
def test_source_problem_2d64_end_to_end(oracle, ctx, relative):
    import torch

    dim, nb, k = 2, 64, 1
    cx, coords, lengths, mesh = config_mesh(oracle, ctx, dim, nb)
    pi = math.pi
    fn = lambda p: np.stack([np.sin(pi * p[:, 0]) * np.cos(pi * p[:, 1]),
                             np.cos(pi * p[:, 0]) * np.sin(pi * p[:, 1])], 1)
    ft = lambda p: torch.stack([torch.sin(pi * p[:, 0]) * torch.cos(pi * p[:, 1]),
                                torch.cos(pi * p[:, 0]) * torch.sin(pi * p[:, 1])], 1)
    # the device side: de Rham map, load M_1 R f, mixed solve
    rf = fq.derham_map(mesh, torch.tensor(coords, device="cuda"), k, ft, 3)
    m1 = fq.WhitneyComplex(mesh).mass(k)
    load = torch.empty_like(rf)
    torch.cuda.synchronize()
    ctx.check(ctx.L.fq_spmv(ctx.h, m1.h, fq._P(rf.data_ptr()), fq._P(load.data_ptr())))
    ctx.synchronize()
    gwc = fq.WhitneyComplex(mesh, relative=relative)
    sig, u, _, rep = fq.solve_source(gwc, load.cpu().numpy(), k, fq.SolveOpts.default(rtol=1e-10))
    assert rep.converged
    # the oracle: the same load from its own de Rham map and mass, SuperLU on its KKT
    owc = oracle.WhitneyComplex(cx, lengths, relative=relative)
    oload = oracle.WhitneyComplex(cx, lengths).mass(k) @ oracle.derham_map(cx, coords, k, fn, 3)
    assert rel(load.cpu().numpy(), oload) < FP64_TOL
    harm = oracle.harmonics(owc, k)
    a, rhs, ns, nu = oracle.assemble_mixed_kkt(owc, oload, k, harm)
    x = oracle.direct_solve(a, rhs)
    want = np.concatenate([owc.inclusion(k - 1) @ x[:ns], owc.inclusion(k) @ x[ns:ns + nu]])
    assert rel(np.concatenate([sig, u]), want) < SOLVE_TOL
    m1.close()
    mesh.close()


# ---------------------------------------------------------------------------
# 4D 12^4: the precision workload's system and solutions
# ---------------------------------------------------------------------------

def test_mixed_k2_4d12(oracle, ctx):
    import torch

    dim, nb, k = 4, 12, 2
    cx, coords, lengths, mesh = config_mesh(oracle, ctx, dim, nb)
    src = np.random.default_rng(SEED + 4).standard_normal(cx.nsimplices(k))
    a, want, ns, nu = oracle_mixed_minres(oracle, cx, lengths, nb, k, src)
    p64 = fq.MixedProblem(mesh, k, fq.FQ_ABSOLUTE, fq.FQ_FP64)
    assert_csr_parity(p64.system().to_scipy(), a)
    sig, u, _, rep = p64.solve(src, fq.SolveOpts.default(rtol=1e-10))
    assert rep.converged
    assert rel(np.concatenate([sig, u]), want) < SOLVE_TOL
    p64.close()
    p32 = fq.MixedProblem(mesh, k, fq.FQ_ABSOLUTE, fq.FQ_FP32)
    opts = fq.SolveOpts.default(rtol=1e-5, precision=fq.FQ_FP32, refine_rtol=1e-10, max_refinements=8)
    sig, u, _, rep = p32.solve(src, opts)
    assert rep.converged
    assert rel(np.concatenate([sig, u]), want) < SOLVE_TOL
    p32.close()
    mesh.close()
    torch.cuda.synchronize()
