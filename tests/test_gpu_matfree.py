"""The matrix-free Whitney operators (fq_elemop_*) against the assembled ones.

Mirrors the reference's own laws for ElementOperator
(formoniq/src/matfree.rs:194-322): the matrix-free apply is the assembled
matvec on every pairing and grade (rectangular ones included), the gathered
diagonal is the assembled diagonal, CG driven matrix-free takes the assembled
run's iterations and lands on its solution, and the gathered Jacobi
preconditions. The assembled side is the oracle's CSR; the bar is 1e-12
relative (the reference asserts 1e-9).
"""
import numpy as np
import pytest

import formoniq_gb300 as fq

pytestmark = pytest.mark.gpu

MASS, DIF_TRIAL, DIF_TEST, DIF_BOTH = 0, 1, 2, 3
NAMES = {MASS: "mass", DIF_TRIAL: "dif_trial", DIF_TEST: "dif_test", DIF_BOTH: "dif_both"}


def dev(x):
    import torch

    return torch.tensor(np.asarray(x, np.float64), device="cuda")


def probe(n):
    return ((7 * np.arange(n)) % 13).astype(np.float64) - 6.0


def mesh_pair(oracle, ctx, dim, nb, seed=4):
    cx, coords = oracle.cartesian_unit(dim, nb)
    lengths = cx.edge_lengths_sq(oracle.jitter_coords(coords, nb, seed, 0.1))
    mesh = fq.Mesh.from_cells(ctx, oracle.kuhn_cells(dim, nb))
    mesh.set_lengths_sq(lengths)
    return cx, mesh, lengths


def pairings(dim):
    for grade in range(dim + 1):
        yield MASS, grade
        if grade >= 1:
            yield DIF_TRIAL, grade
            yield DIF_TEST, grade
        if grade < dim:
            yield DIF_BOTH, grade + 1


@pytest.mark.parametrize("dim,nb", [(1, 6), (2, 4), (3, 3), (4, 2)])
@pytest.mark.parametrize("relative", [False, True])
def test_the_matrix_free_apply_is_the_assembled_matvec(oracle, ctx, dim, nb, relative):
    import torch

    cx, mesh, lengths = mesh_pair(oracle, ctx, dim, nb)
    owc = oracle.WhitneyComplex(cx, lengths, relative=relative)
    bc = fq.FQ_RELATIVE if relative else fq.FQ_ABSOLUTE
    for form, grade in pairings(dim):
        a = getattr(owc, NAMES[form])(grade)
        op = fq.ElementOperator(mesh, form, grade, bc)
        assert op.shape == a.shape, (form, grade)
        if a.shape[0] == 0 or a.shape[1] == 0:
            continue
        x = probe(a.shape[1])
        want = a @ x
        xd = dev(x)
        yd = torch.empty(a.shape[0], dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        op.apply(xd.data_ptr(), yd.data_ptr())
        got = yd.cpu().numpy()
        assert np.linalg.norm(got - want) <= 1e-12 * max(np.linalg.norm(want), 1e-300), (form, grade)
        op.close()


def test_the_mixed_forms_pair_two_grades(oracle, ctx):
    _, mesh, _ = mesh_pair(oracle, ctx, 2, 2)
    dif = fq.ElementOperator(mesh, DIF_TRIAL, 1)
    mixed = fq.ElementOperator(mesh, DIF_TEST, 1)
    assert dif.shape[0] != dif.shape[1] and mixed.shape[0] != mixed.shape[1]
    assert dif.shape == mixed.shape[::-1]


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_the_gathered_diagonal_is_the_assembled_one(oracle, ctx, dim):
    import torch

    cx, mesh, lengths = mesh_pair(oracle, ctx, dim, 3)
    owc = oracle.WhitneyComplex(cx, lengths)
    for grade in range(dim + 1):
        for form, g in ((MASS, grade), (DIF_BOTH, grade + 1)):
            if g > dim:
                continue
            a = getattr(owc, NAMES[form])(g)
            op = fq.ElementOperator(mesh, form, g)
            d = torch.empty(a.shape[0], dtype=torch.float64, device="cuda")
            torch.cuda.synchronize()
            op.diagonal(d.data_ptr())
            want = a.diagonal()
            assert np.linalg.norm(d.cpu().numpy() - want) <= 1e-12 * np.linalg.norm(want)


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_conjugate_gradients_does_not_notice_the_difference(oracle, ctx, dim):
    import torch

    cx, mesh, lengths = mesh_pair(oracle, ctx, dim, 3)
    gwc = fq.WhitneyComplex(mesh)
    for grade in range(dim + 1):
        a = gwc.mass(grade)
        op = fq.ElementOperator(mesh, MASS, grade)
        n = op.shape[0]
        b = dev(probe(n))
        xa = torch.zeros(n, dtype=torch.float64, device="cuda")
        xf = torch.zeros(n, dtype=torch.float64, device="cuda")
        opts = fq.SolveOpts.default(rtol=1e-10)
        torch.cuda.synchronize()
        ra = fq.cg(a, b.data_ptr(), xa.data_ptr(), 0, opts)
        rf = op.cg(b.data_ptr(), xf.data_ptr(), 0, opts)
        assert ra.converged and rf.converged
        # the same recurrence on applies that agree to roundoff
        assert abs(ra.iters - rf.iters) <= 1, (dim, grade, ra, rf)
        xa_h, xf_h = xa.cpu().numpy(), xf.cpu().numpy()
        assert np.linalg.norm(xa_h - xf_h) <= 1e-9 * np.linalg.norm(xa_h)


def test_the_matrix_free_jacobi_preconditions(oracle, ctx):
    import torch

    # a graded mesh (x -> x^1.8 per axis), so the diagonal varies across it
    nb = 6
    cx, coords = oracle.cartesian_unit(3, nb)
    mesh = fq.Mesh.from_cells(ctx, oracle.kuhn_cells(3, nb))
    mesh.set_lengths_sq(cx.edge_lengths_sq(np.ascontiguousarray(coords ** 1.8)))
    op = fq.ElementOperator(mesh, DIF_BOTH, 1, fq.FQ_RELATIVE)
    n = op.shape[0]
    b = dev(probe(n))
    d = torch.empty(n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    op.diagonal(d.data_ptr())
    inv = (1.0 / d).contiguous()
    x0 = torch.zeros(n, dtype=torch.float64, device="cuda")
    x1 = torch.zeros(n, dtype=torch.float64, device="cuda")
    opts = fq.SolveOpts.default(rtol=1e-10)
    plain = op.cg(b.data_ptr(), x0.data_ptr(), 0, opts)
    jac = op.cg(b.data_ptr(), x1.data_ptr(), inv.data_ptr(), opts)
    assert plain.converged and jac.converged
    assert jac.iters < plain.iters, (jac, plain)


def test_new_lengths_take_effect_at_the_next_apply(oracle, ctx):
    import torch

    cx, mesh, lengths = mesh_pair(oracle, ctx, 3, 2)
    op = fq.ElementOperator(mesh, MASS, 2)
    l2 = lengths * 1.7
    mesh.set_lengths_sq(l2)
    a = oracle.WhitneyComplex(cx, l2).mass(2)
    x = probe(a.shape[1])
    xd = dev(x)
    y = torch.empty(a.shape[0], dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    op.apply(xd.data_ptr(), y.data_ptr())
    want = a @ x
    assert np.linalg.norm(y.cpu().numpy() - want) <= 1e-12 * np.linalg.norm(want)
