"""Parity of the CUDA path (through the C ABI) with the oracle.

Bars (stated per test): CSR row_ptr/col_idx and coboundary signs bit-exact;
FP64 element and global matrices within 1e-12 relative Frobenius; FP32 element
matrices within 1e-5; solutions within 1e-8 relative of the direct solve.
"""
import math

import numpy as np
import pytest
import scipy.sparse as sp

import formoniq_gb300 as fq

pytestmark = pytest.mark.gpu

MASS, DIF_TRIAL, DIF_TEST, DIF_BOTH = 0, 1, 2, 3
FP64_TOL = 1e-12
FP32_TOL = 1e-5
SOLVE_TOL = 1e-8


def rel_frob(a, b):
    a = a.toarray() if sp.issparse(a) else np.asarray(a, np.float64)
    b = b.toarray() if sp.issparse(b) else np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def make_pair(oracle, ctx, dim, nb, jitter=0.1, seed=11, minkowski=False):
    """The same mesh and lengths on both sides."""
    if minkowski:
        cx, coords, signs = oracle.minkowski(dim, nb)
        side = np.ones(dim)
        side[0] = 0.7
    else:
        (cx, coords), signs, side = oracle.cartesian_unit(dim, nb), None, np.ones(dim)
    if jitter:
        coords = oracle.jitter_coords(coords, nb, seed, jitter, side=side)
    lengths = cx.edge_lengths_sq(coords, signs)
    mesh = fq.Mesh.from_cells(ctx, oracle.kuhn_cells(dim, nb))
    mesh.set_lengths_sq(lengths)
    return cx, mesh, lengths, coords


def csr_equal_pattern(a: sp.csr_matrix, b: sp.csr_matrix):
    assert a.shape == b.shape
    np.testing.assert_array_equal(a.indptr.astype(np.int64), b.indptr.astype(np.int64))
    np.testing.assert_array_equal(a.indices.astype(np.int64), b.indices.astype(np.int64))


# ---------------------------------------------------------------------------
# topology and geometry inputs
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("dim,nb", [(1, 3), (2, 3), (3, 2), (4, 2)])
def test_topology_matches_oracle(oracle, ctx, dim, nb):
    cx = oracle.Complex.from_cells(oracle.kuhn_cells(dim, nb))
    mesh = fq.Mesh.kuhn_cube(ctx, dim, nb)
    for k in range(dim + 1):
        np.testing.assert_array_equal(mesh.simplices(k), cx.simplices(k))
        np.testing.assert_array_equal(mesh.interior(k), cx.interior(k))
    assert np.array_equal(np.abs(mesh.orientation()), np.ones(cx.ncells(), np.int8))
    z = oracle.orientation_signs(cx)
    o = mesh.orientation().astype(float)
    assert np.array_equal(o, z) or np.array_equal(o, -z)


@pytest.mark.parametrize("dim,nb", [(2, 5), (3, 3)])
def test_kuhn_lengths_match_oracle(oracle, ctx, dim, nb):
    cx, coords = oracle.cartesian_unit(dim, nb)
    expect = cx.edge_lengths_sq(oracle.jitter_coords(coords, nb, 5, 0.1))
    mesh = fq.Mesh.kuhn_cube(ctx, dim, nb)
    mesh.kuhn_lengths(jitter=0.1, seed=5)
    np.testing.assert_allclose(mesh.lengths_sq(), expect, rtol=1e-14)


# ---------------------------------------------------------------------------
# kernel (a): per-cell metric, inverse, determinant, volume
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("dim,nb,mink", [(2, 6, False), (3, 4, False), (4, 2, False), (3, 3, True)])
def test_cell_metrics(oracle, ctx, dim, nb, mink):
    import torch

    cx, mesh, lengths, _ = make_pair(oracle, ctx, dim, nb, minkowski=mink, jitter=0.1 if not mink else 0.0)
    g, gi, det, vol, bad = cx.cell_metrics(lengths)
    nc = cx.ncells()
    d_gi = torch.empty((dim * dim, nc), dtype=torch.float64, device="cuda")
    d_det = torch.empty(nc, dtype=torch.float64, device="cuda")
    d_vol = torch.empty(nc, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    ctx.check(ctx.L.fq_cell_metrics(ctx.h, mesh.h, fq._P(d_gi.data_ptr()), fq._P(d_det.data_ptr()),
                                    fq._P(d_vol.data_ptr())))
    gi_gpu = d_gi.cpu().numpy().T.reshape(nc, dim, dim)
    assert rel_frob(gi_gpu.reshape(nc, -1), gi.reshape(nc, -1)) < FP64_TOL
    assert rel_frob(d_det.cpu().numpy(), det) < FP64_TOL
    assert rel_frob(d_vol.cpu().numpy(), vol) < FP64_TOL


# ---------------------------------------------------------------------------
# kernel (b): element matrices
# ---------------------------------------------------------------------------

FORMS = [(MASS, "mass"), (DIF_TRIAL, "dif_trial"), (DIF_TEST, "dif_test"), (DIF_BOTH, "dif_both")]


@pytest.mark.parametrize("dim", [1, 2, 3, 4])
@pytest.mark.parametrize("prec", [fq.FQ_FP64, fq.FQ_FP32])
def test_element_matrices(oracle, ctx, dim, prec):
    import torch

    nb = 2
    cx, mesh, lengths, _ = make_pair(oracle, ctx, dim, nb, jitter=0.15, seed=3)
    nc = cx.ncells()
    edges = cx.cell_faces(1)
    sample = list(range(0, nc, max(1, nc // 7)))
    for form, _name in FORMS:
        for grade in range(0, dim + 1):
            tg = grade - 1 if form in (DIF_TEST, DIF_BOTH) else grade
            sg = grade - 1 if form in (DIF_TRIAL, DIF_BOTH) else grade
            if tg < 0 or sg < 0:
                continue
            lr, lc = math.comb(dim + 1, tg + 1), math.comb(dim + 1, sg + 1)
            dt = torch.float32 if prec == fq.FQ_FP32 else torch.float64
            out = torch.zeros((lr * lc, nc), dtype=dt, device="cuda")
            r, c = fq.ctypes.c_int(), fq.ctypes.c_int()
            torch.cuda.synchronize()
            ctx.check(ctx.L.fq_element_matrices(ctx.h, mesh.h, form, grade, prec, fq._P(out.data_ptr()),
                                                fq.ctypes.byref(r), fq.ctypes.byref(c)))
            assert (r.value, c.value) == (lr, lc)
            host = out.cpu().numpy().astype(np.float64)
            for cell in sample:
                expect = oracle.element_matrix(dim, form, grade, lengths[edges[cell]])
                got = host[:, cell].reshape(lr, lc)
                tol = FP32_TOL if prec == fq.FQ_FP32 else FP64_TOL
                assert rel_frob(got, expect) < tol, (form, grade, cell)


# ---------------------------------------------------------------------------
# kernel (c): assembled global matrices
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("dim,nb", [(1, 5), (2, 4), (3, 3), (4, 2)])
@pytest.mark.parametrize("relative", [False, True])
@pytest.mark.parametrize("prec", [fq.FQ_FP64, fq.FQ_FP64_IEEE])
def test_assembly_parity_jittered(oracle, ctx, dim, nb, relative, prec):
    """FQ_FP64 computes element entries and scatter sums in float-float on the
    FP32 pipe; FQ_FP64_IEEE in IEEE double. Both must meet the 1e-12 bar."""
    cx, mesh, lengths, _ = make_pair(oracle, ctx, dim, nb, jitter=0.1, seed=dim * 10 + nb)
    owc = oracle.WhitneyComplex(cx, lengths, relative=relative)
    gwc = fq.WhitneyComplex(mesh, relative=relative, precision=prec)
    for grade in range(-1, dim + 2):
        for name in ("mass", "dif_trial", "dif_test", "dif_both"):
            a = getattr(owc, name)(grade)
            b = getattr(gwc, name)(grade).to_scipy()
            csr_equal_pattern(b, a)
            if a.nnz:
                assert rel_frob(b, a) < FP64_TOL, (name, grade)
        a = owc.hdif_gram(grade) if 0 <= grade <= dim else None
        if a is not None:
            b = gwc.hdif_gram(grade).to_scipy()
            csr_equal_pattern(b, a)
            assert rel_frob(b, a) < FP64_TOL
        d = owc.dif(grade)
        e = gwc.dif(grade).to_scipy()
        csr_equal_pattern(e, d)
        np.testing.assert_array_equal(e.data, d.data)


@pytest.mark.parametrize("dim,nb", [(2, 4), (3, 3)])
def test_assembly_fp32(oracle, ctx, dim, nb):
    cx, mesh, lengths, _ = make_pair(oracle, ctx, dim, nb, jitter=0.1, seed=2)
    owc = oracle.WhitneyComplex(cx, lengths)
    gwc = fq.WhitneyComplex(mesh, precision=fq.FQ_FP32)
    for grade in range(0, dim + 1):
        for name in ("mass", "dif_test", "dif_both"):
            a = getattr(owc, name)(grade)
            b = getattr(gwc, name)(grade).to_scipy()
            csr_equal_pattern(b, a)
            if a.nnz:
                assert rel_frob(b, a) < FP32_TOL


def pattern_difference_is_roundoff(gpu: sp.csr_matrix, ref: sp.csr_matrix, rel=1e-14):
    """Slots present on one side only must hold values at roundoff level: the
    `val != 0.0` rule (galerkin.rs:173) keeps a mathematically zero entry exactly
    when its rounding happens to leave a nonzero, which depends on the order of
    operations, not on the mathematics."""
    g = gpu.tocoo()
    r = ref.tocoo()
    gs = {(i, j): v for i, j, v in zip(g.row, g.col, g.data)}
    rs = {(i, j): v for i, j, v in zip(r.row, r.col, r.data)}
    scale = max(np.abs(r.data).max() if r.nnz else 0.0, np.abs(g.data).max() if g.nnz else 0.0, 1e-300)
    only = [abs(gs[k]) for k in gs.keys() - rs.keys()] + [abs(rs[k]) for k in rs.keys() - gs.keys()]
    assert all(v <= rel * scale for v in only), max(only) / scale
    return len(only)


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_assembly_unjittered_pattern_follows_the_nonzero_rule(oracle, ctx, dim):
    """The reference's own unjittered N = 2 unit meshes, where mathematically
    zero element entries occur: both sides drop exact zeros, and every slot that
    one side keeps and the other drops holds a roundoff-level value."""
    cx, mesh, lengths, _ = make_pair(oracle, ctx, dim, 2, jitter=0.0)
    owc = oracle.WhitneyComplex(cx, lengths)
    gwc = fq.WhitneyComplex(mesh)
    for grade in range(0, dim + 2):
        for name in ("mass", "dif_trial", "dif_test", "dif_both"):
            a = getattr(owc, name)(grade)
            b = getattr(gwc, name)(grade).to_scipy()
            assert a.shape == b.shape
            pattern_difference_is_roundoff(b, a)
            if a.nnz:
                assert rel_frob(b, a) < FP64_TOL


def test_reassembly_is_deterministic(oracle, ctx):
    cx, mesh, lengths, _ = make_pair(oracle, ctx, 3, 3)
    gwc = fq.WhitneyComplex(mesh)
    m = gwc.mass(1)
    v1 = m.to_scipy().data.copy()
    m.reassemble(mesh)
    v2 = m.to_scipy().data.copy()
    np.testing.assert_array_equal(v1, v2)
    # new lengths, same pattern, new values match the oracle
    lengths2 = lengths * 1.5
    mesh.set_lengths_sq(lengths2)
    m.reassemble(mesh)
    assert rel_frob(m.to_scipy(), oracle.WhitneyComplex(cx, lengths2).mass(1)) < FP64_TOL


def test_reassemble_many_equals_one_by_one(oracle, ctx):
    """fq_reassemble_many over forms of two meshes, one of them unjittered (its
    exact-zero slots are compacted away): the same patterns and values, bit for
    bit, as fq_reassemble on each matrix."""
    _, mesh_a, _, _ = make_pair(oracle, ctx, 3, 3)
    cx_b, mesh_b, lengths_b, _ = make_pair(oracle, ctx, 2, 2, jitter=0.0)
    forms = [(mesh_a, "mass", 1), (mesh_a, "mass", 2), (mesh_a, "dif_both", 2), (mesh_a, "dif_both", 3),
             (mesh_b, "mass", 1), (mesh_b, "dif_test", 1), (mesh_b, "dif_both", 2)]
    wcs = {id(mesh_a): fq.WhitneyComplex(mesh_a), id(mesh_b): fq.WhitneyComplex(mesh_b)}
    many = [getattr(wcs[id(m)], name)(k) for m, name, k in forms]
    single = [getattr(wcs[id(m)], name)(k) for m, name, k in forms]
    for (m, _, _), mat in zip(forms, single):
        mat.reassemble(m)
    fq.Matrix.reassemble_many(many)
    for a, b in zip(many, single):
        sa, sb = a.to_scipy(), b.to_scipy()
        np.testing.assert_array_equal(sa.indptr, sb.indptr)
        np.testing.assert_array_equal(sa.indices, sb.indices)
        np.testing.assert_array_equal(sa.data, sb.data)
    # the unjittered mesh's pattern is the oracle's (exact zeros dropped)
    ref = oracle.WhitneyComplex(cx_b, lengths_b).dif_both(2)
    pattern_difference_is_roundoff(many[-1].to_scipy(), ref)


def test_fq_assemble_host_e2e(oracle, ctx):
    import ctypes

    cx, mesh, lengths, _ = make_pair(oracle, ctx, 3, 3)
    m = fq.WhitneyComplex(mesh).dif_both(2)
    nnz = m.nnz
    out = np.zeros(nnz)
    l2 = np.ascontiguousarray(lengths * 0.75)
    ctx.check(ctx.L.fq_assemble_host(ctx.h, mesh.h, m.h, l2.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                     out.ctypes.data_as(ctypes.c_void_p)))
    ref = oracle.WhitneyComplex(cx, l2).dif_both(2)
    assert rel_frob(out, ref.data) < FP64_TOL


def test_fq_assemble_host_many_e2e(oracle, ctx):
    """Host lengths in, every matrix's host values out, downloads overlapped with
    the next matrix's kernels; an unjittered mesh's exact-zero slots still come
    out compacted."""
    import ctypes

    import torch

    for dim, nb, jit in ((3, 3, 0.1), (2, 2, 0.0)):
        cx, mesh, lengths, _ = make_pair(oracle, ctx, dim, nb, jitter=jit)
        gwc = fq.WhitneyComplex(mesh)
        forms = [("mass", 1), ("dif_both", 2), ("dif_test", 1), ("mass", 0)]
        mats = [getattr(gwc, n)(k) for n, k in forms]
        l2 = np.ascontiguousarray(lengths * 0.75)
        owc = oracle.WhitneyComplex(cx, l2)
        for pinned in (True, False):
            outs = [torch.zeros(m.nnz, dtype=torch.float64) for m in mats]
            if pinned:
                outs = [o.pin_memory() for o in outs]
            arr = (ctypes.c_void_p * len(mats))(*[m.h for m in mats])
            oarr = (ctypes.c_void_p * len(mats))(*[o.data_ptr() for o in outs])
            ctx.check(ctx.L.fq_assemble_host_many(ctx.h, mesh.h, l2.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                                  arr, oarr, len(mats)))
            for (n, k), m, o in zip(forms, mats, outs):
                ref = getattr(owc, n)(k)
                got = m.to_scipy()
                np.testing.assert_array_equal(o.numpy()[:m.nnz], got.data)
                pattern_difference_is_roundoff(got, ref)
                if jit > 0:
                    np.testing.assert_array_equal(got.indptr, ref.indptr)
                    assert rel_frob(got, ref) < FP64_TOL


# ---------------------------------------------------------------------------
# kernel (d): Krylov solves
# ---------------------------------------------------------------------------

def _dev(x):
    import torch

    return torch.tensor(np.asarray(x, np.float64), device="cuda")


@pytest.mark.parametrize("solver", ["cg", "minres"])
def test_krylov_on_hdif_gram(oracle, ctx, solver):
    import torch

    cx, mesh, lengths, _ = make_pair(oracle, ctx, 3, 4, seed=9)
    gwc = fq.WhitneyComplex(mesh)
    a = gwc.hdif_gram(1)
    ah = a.to_scipy()
    b = np.random.default_rng(0).standard_normal(ah.shape[0])
    db, dx = _dev(b), torch.zeros(ah.shape[0], dtype=torch.float64, device="cuda")
    dinv = _dev(1.0 / ah.diagonal())
    torch.cuda.synchronize()
    opts = fq.SolveOpts.default(rtol=1e-12)
    rep = getattr(fq, solver)(a, db.data_ptr(), dx.data_ptr(), dinv.data_ptr(), opts)
    assert rep.converged
    x = dx.cpu().numpy()
    xs = sp.linalg.spsolve(sp.csc_matrix(ah), b)
    assert np.linalg.norm(x - xs) / np.linalg.norm(xs) < SOLVE_TOL
    # the oracle's restated recurrence converges in a similar number of steps
    _, orep = getattr(oracle, solver)(ah, oracle.jacobi(ah.diagonal()), b, rtol=1e-12)
    assert abs(orep.iters - rep.iters) <= max(3, 0.05 * orep.iters)


@pytest.mark.parametrize("dim", [1, 2, 3])
@pytest.mark.parametrize("relative", [False, True])
def test_kkt_system_parity(oracle, ctx, dim, relative):
    cx, mesh, lengths, _ = make_pair(oracle, ctx, dim, 3, jitter=0.1, seed=4)
    owc = oracle.WhitneyComplex(cx, lengths, relative=relative)
    for grade in range(dim + 1):
        harm = oracle.harmonics(owc, grade)
        a, _, ns, nu = oracle.assemble_mixed_kkt(owc, np.zeros(cx.nsimplices(grade)), grade, harm)
        prob = fq.MixedProblem(mesh, grade, fq.FQ_RELATIVE if relative else fq.FQ_ABSOLUTE)
        gns, gnu, gnh, _ = prob.info()
        assert (gns, gnu, gnh) == (ns, nu, harm.shape[1])
        b = prob.system().to_scipy()
        csr_equal_pattern(b, a)
        if harm.shape[1]:
            # the border is unique up to the sign of h
            bb, aa = b.toarray(), a.toarray()
            n0 = ns + nu
            if np.sign(bb[n0, ns:n0] @ aa[n0, ns:n0]) < 0:
                bb[n0, :] *= -1
                bb[:, n0] *= -1
            assert rel_frob(bb, aa) < 1e-10
        else:
            assert rel_frob(b, a) < FP64_TOL
        prob.close()


@pytest.mark.parametrize("dim,nb", [(1, 2), (2, 2), (3, 2), (2, 6), (3, 3)])
@pytest.mark.parametrize("relative", [False, True])
def test_solve_source_matches_direct(oracle, ctx, dim, nb, relative):
    jitter = 0.0 if nb == 2 else 0.1
    cx, mesh, lengths, _ = make_pair(oracle, ctx, dim, nb, jitter=jitter, seed=8)
    owc = oracle.WhitneyComplex(cx, lengths, relative=relative)
    gwc = fq.WhitneyComplex(mesh, relative=relative)
    for grade in range(dim + 1):
        src = (np.arange(cx.nsimplices(grade)) % 7) - 3.0
        harm = oracle.harmonics(owc, grade)
        a, rhs, ns, nu = oracle.assemble_mixed_kkt(owc, src, grade, harm)
        x = oracle.direct_solve(a, rhs)
        sig_o = owc.inclusion(grade - 1) @ x[:ns] if grade > 0 else np.zeros(0)
        u_o = owc.inclusion(grade) @ x[ns:ns + nu]
        sigma, u, p, rep = fq.solve_source(gwc, src, grade, fq.SolveOpts.default(rtol=1e-12))
        assert rep.converged, (grade, rep)
        scale = max(np.linalg.norm(x), 1.0)
        err = math.sqrt(np.linalg.norm(u - u_o) ** 2 + (np.linalg.norm(sigma - sig_o) ** 2 if grade else 0.0))
        assert err / scale < SOLVE_TOL, (grade, err / scale, rep)


def test_minres_iteration_count_matches_the_oracle_recurrence(oracle, ctx):
    """Same recurrence, same Jacobi preconditioner: the GPU and the restated
    krylov.rs MINRES take the same number of steps up to roundoff."""
    cx, mesh, lengths, _ = make_pair(oracle, ctx, 2, 8, seed=3)
    owc = oracle.WhitneyComplex(cx, lengths)
    src = np.random.default_rng(1).standard_normal(cx.nsimplices(1))
    a, rhs, ns, nu = oracle.assemble_mixed_kkt(owc, src, 1, np.zeros((nu_ := cx.nsimplices(1), 0)))
    dinv = 1.0 / oracle.mixed_block_preconditioner_diag(owc, 1, 0)
    _, orep = oracle.minres(a, lambda r: r * dinv, rhs, rtol=1e-10)
    _, _, _, grep = fq.solve_source(fq.WhitneyComplex(mesh), src, 1, fq.SolveOpts.default(rtol=1e-10))
    assert abs(orep.iters - grep.iters) <= max(2, 0.02 * orep.iters), (orep, grep)


def test_mixed_precision_refinement_reaches_1e8(oracle, ctx):
    cx, mesh, lengths, _ = make_pair(oracle, ctx, 3, 4, seed=12)
    owc = oracle.WhitneyComplex(cx, lengths)
    src = np.random.default_rng(2).standard_normal(cx.nsimplices(1))
    a, rhs, ns, nu = oracle.assemble_mixed_kkt(owc, src, 1, np.zeros((cx.nsimplices(1), 0)))
    x = oracle.direct_solve(a, rhs)
    prob = fq.MixedProblem(mesh, 1, fq.FQ_ABSOLUTE, fq.FQ_FP32)
    opts = fq.SolveOpts.default(rtol=1e-6, precision=fq.FQ_FP32, refine_rtol=1e-12)
    sigma, u, p, rep = prob.solve(src, opts)
    assert rep.refinements >= 1 and rep.true_residual <= 1e-12
    err = math.sqrt(np.linalg.norm(u - x[ns:]) ** 2 + np.linalg.norm(sigma - x[:ns]) ** 2) / np.linalg.norm(x)
    assert err < SOLVE_TOL, err


# ---------------------------------------------------------------------------
# Hodge-Dirac
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("dim", [1, 2, 3, 4])
@pytest.mark.parametrize("mink", [False, True])
def test_dirac_system_parity(oracle, ctx, dim, mink):
    cx, mesh, lengths, _ = make_pair(oracle, ctx, dim, 2 if dim == 4 else 3, jitter=0.0, minkowski=mink)
    lengths = lengths * (1.0 + 0.05 * oracle.uniform_pm1(3, np.arange(len(lengths), dtype=np.uint64)))
    mesh.set_lengths_sq(lengths)
    s_rel, _, _, _ = oracle.dirac_source_system(cx, lengths, 1.5, np.zeros(sum(cx.nsimplices(k) for k in
                                                                               range(dim + 1))),
                                                np.zeros(sum(cx.nsimplices(k) for k in range(dim + 1))))
    g = fq.dirac_system(mesh, 1.5).to_scipy()
    csr_equal_pattern(g, s_rel.tocsr())
    assert rel_frob(g, s_rel) < FP64_TOL


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_dirac_source_reproduces_constant_field(oracle, ctx, dim):
    from test_oracle_golden import derham_constant

    for mink in (False, True):
        cx, mesh, lengths, coords = make_pair(oracle, ctx, dim, 2, jitter=0.0, minkowski=mink)
        exact = np.concatenate([derham_constant(cx, coords, k) for k in range(dim + 1)])
        _, mb, _ = oracle.dirac_selfadjoint(oracle.WhitneyComplex(cx, lengths))
        load = mb @ exact
        x, rep = fq.solve_dirac_source(mesh, 1.0, load, exact, fq.SolveOpts.default(rtol=1e-13))
        assert rep.converged
        np.testing.assert_allclose(x, exact, atol=1e-9)


def test_dirac_minkowski_matches_direct(oracle, ctx):
    cx, mesh, lengths, _ = make_pair(oracle, ctx, 3, 3, jitter=0.0, minkowski=True)
    lengths = lengths * (1.0 + 0.05 * oracle.uniform_pm1(21, np.arange(len(lengths), dtype=np.uint64)))
    mesh.set_lengths_sq(lengths)
    ntot = sum(cx.nsimplices(k) for k in range(4))
    load = np.random.default_rng(5).standard_normal(ntot)
    lift = np.zeros(ntot)
    x_o = oracle.dirac_solve_source(cx, lengths, 1.5, load, lift)
    x, rep = fq.solve_dirac_source(mesh, 1.5, load, lift, fq.SolveOpts.default(rtol=1e-13, max_iters=50000))
    assert rep.converged, rep
    assert np.linalg.norm(x - x_o) / np.linalg.norm(x_o) < SOLVE_TOL


@pytest.mark.parametrize("nb,mink,pc", [(4, True, fq.FQ_PC_COMPARISON), (5, True, fq.FQ_PC_COMPARISON),
                                        (4, False, fq.FQ_PC_COMPARISON),
                                        (4, True, fq.FQ_PC_HX), (4, False, fq.FQ_PC_HX)])
def test_dirac_comparison_preconditioners(oracle, ctx, nb, mink, pc):
    """Kuhn cube meshes: MINRES preconditioned from the Euclidean comparison
    lattice (its mass diagonal, or HX blocks of its hdif_gram) converges where
    |diag(S)| Jacobi does not (Minkowski N = 5: not converged after 20,000
    iterations in the oracle's MINRES) and matches the direct solve."""
    dim = 3
    if mink:
        cx, coords, signs = oracle.minkowski(dim, nb)
        lengths = cx.edge_lengths_sq(coords, signs)
    else:
        cx, coords = oracle.cartesian_unit(dim, nb)
        lengths = cx.edge_lengths_sq(coords)
    lengths = lengths * (1.0 + 0.05 * oracle.uniform_pm1(8, np.arange(len(lengths), dtype=np.uint64)))
    mesh = fq.Mesh.kuhn_cube(ctx, dim, nb)
    mesh.set_lengths_sq(lengths)
    ntot = sum(cx.nsimplices(k) for k in range(dim + 1))
    load = np.random.default_rng(6).standard_normal(ntot)
    x_o = oracle.dirac_solve_source(cx, lengths, 1.5, load, np.zeros(ntot))
    x, rep = fq.solve_dirac_source(mesh, 1.5, load, None,
                                   fq.SolveOpts.default(rtol=1e-12, max_iters=20000, preconditioner=pc))
    assert rep.converged, rep
    assert np.linalg.norm(x - x_o) / np.linalg.norm(x_o) < SOLVE_TOL
    if mink:
        _, jrep = fq.solve_dirac_source(mesh, 1.5, load, None,
                                        fq.SolveOpts.default(rtol=1e-12, max_iters=20000,
                                                             preconditioner=fq.FQ_PC_JACOBI))
        assert not jrep.converged or jrep.iters > 2 * rep.iters, (rep, jrep)


# ---------------------------------------------------------------------------
# failure paths: host-side, no GPU fault
# ---------------------------------------------------------------------------

def test_degenerate_cell_is_reported(oracle, ctx):
    cx, mesh, lengths, _ = make_pair(oracle, ctx, 2, 2, jitter=0.0)
    bad = lengths.copy()
    bad[:] = 0.0
    mesh.set_lengths_sq(bad)
    with pytest.raises(fq.FqError) as e:
        fq.WhitneyComplex(mesh).mass(1)
    assert e.value.name == "FQ_DEGENERATE_CELL"


def test_invalid_cells_are_rejected(ctx):
    with pytest.raises(fq.FqError) as e:
        fq.Mesh.from_cells(ctx, np.array([[0, 0, 1]], np.int32))
    assert e.value.name == "FQ_INVALID_ARG"
    with pytest.raises(fq.FqError):
        fq.Mesh.from_cells(ctx, np.array([[0, 2, 3]], np.int32))  # vertex 1 unused


def test_budget_is_enforced():
    small = fq.Context(0, budget_bytes=1 << 16)
    with pytest.raises(fq.FqError) as e:
        m = fq.Mesh.kuhn_cube(small, 3, 16)
        m.kuhn_lengths()
        fq.WhitneyComplex(m).mass(1)
    assert e.value.name == "FQ_OOM_BUDGET"
    small.close()


def test_scatter_bytes_accounting(oracle, ctx):
    """fq_matrix_scatter_bytes counts every packed element entry once, one
    16-byte record per upper slot, the plan indices of slots with more than two
    contributions, and every assembled value once."""
    cx, coords = oracle.cartesian_unit(3, 4)
    coords = oracle.jitter_coords(coords, 4, seed=3, amplitude=0.1)
    mesh = fq.Mesh.from_cells(ctx, oracle.kuhn_cells(3, 4))
    mesh.set_lengths_sq(cx.edge_lengths_sq(coords))
    m1 = fq.WhitneyComplex(mesh).mass(1)
    nr, nc, nnz, _ = m1.info()
    nent = 6 * 7 // 2
    nup = (nnz + nr) // 2
    base = cx.ncells() * nent * 8 + nup * 16 + nnz * 8
    b = m1.scatter_bytes()
    assert base <= b <= base + cx.ncells() * nent * 8, (b, base)
    m1.close()
    mesh.close()


@pytest.mark.parametrize("kuhn", [True, False])
@pytest.mark.parametrize("which", ["dirac", "mixed"])
def test_lu_finishes_an_unconverged_minres(oracle, ctx, which, kuhn):
    """The reference's LU fallback (elliptic.rs:147-160): a MINRES stopped
    after a few iterations is finished by a direct solve, the sparse LU
    (GMRES on its factors) on a Kuhn cube mesh, the dense LU on a small mesh
    given by its cells."""
    def make_mesh(dim, nb, lengths):
        m = fq.Mesh.kuhn_cube(ctx, dim, nb) if kuhn else fq.Mesh.from_cells(ctx, oracle.kuhn_cells(dim, nb))
        m.set_lengths_sq(lengths)
        return m

    if which == "dirac":
        cx, coords, signs = oracle.minkowski(3, 3)
        lengths = cx.edge_lengths_sq(coords, signs)
        mesh = make_mesh(3, 3, lengths)
        ntot = sum(cx.nsimplices(k) for k in range(4))
        load = np.random.default_rng(8).standard_normal(ntot)
        x_o = oracle.dirac_solve_source(cx, lengths, 1.5, load, np.zeros(ntot))
        x, rep = fq.solve_dirac_source(mesh, 1.5, load, None, fq.SolveOpts.default(rtol=1e-12, max_iters=5,
                                                                                   preconditioner=fq.FQ_PC_JACOBI))
        assert rep.converged and rep.iters <= (5 + 60 if kuhn else 6), rep
        assert np.linalg.norm(x - x_o) / np.linalg.norm(x_o) < 1e-9
        assert rep.true_residual < 1e-11
    else:
        cx, coords = oracle.cartesian_unit(2, 6)
        coords = oracle.jitter_coords(coords, 6, seed=2, amplitude=0.1)
        lengths = cx.edge_lengths_sq(coords)
        mesh = make_mesh(2, 6, lengths)
        owc = oracle.WhitneyComplex(cx, lengths)
        src = np.random.default_rng(3).standard_normal(cx.nsimplices(1))
        a, rhs, ns, nu = oracle.assemble_mixed_kkt(owc, src, 1, oracle.harmonics(owc, 1))
        x_o = oracle.direct_solve(a, rhs)
        sigma, u, p, rep = fq.solve_source(fq.WhitneyComplex(mesh), src, 1,
                                           fq.SolveOpts.default(rtol=1e-12, max_iters=3))
        assert rep.converged and rep.iters <= (3 + 60 if kuhn else 4), rep
        x = np.concatenate([sigma, u])
        assert np.linalg.norm(x - x_o[:ns + nu]) / np.linalg.norm(x_o) < 1e-9
    mesh.close()


@pytest.mark.parametrize("precision", [fq.FQ_FP64, fq.FQ_FP64_IEEE, fq.FQ_FP32])
@pytest.mark.parametrize("dim,nb", [(1, 9), (2, 6), (3, 4)])
def test_multi_matrix_assembly_shares_one_element_pass(oracle, ctx, precision, dim, nb):
    """fq_reassemble_many of up to four mass / dif_both matrices of one mesh
    runs one element pass for all of them (the cell's metric once). Its
    matrices equal the per-matrix assembly (bit for bit in float-float, whose
    operations are never contracted; to rounding otherwise) and the oracle."""
    cx, mesh, lengths, _ = make_pair(oracle, ctx, dim, nb)
    forms = [("mass", 1), ("mass", min(2, dim)), ("dif_both", 1), ("dif_both", dim)][:4]
    gwc = fq.WhitneyComplex(mesh, precision=precision)
    owc = oracle.WhitneyComplex(cx, lengths)
    many = [getattr(gwc, name)(k) for name, k in forms]
    fq.Matrix.reassemble_many(many)
    tol = FP32_TOL if precision == fq.FQ_FP32 else FP64_TOL
    for (name, k), m in zip(forms, many):
        single = getattr(fq.WhitneyComplex(mesh, precision=precision), name)(k)
        single.reassemble(mesh)
        a, b = m.to_scipy(), single.to_scipy()
        csr_equal_pattern(a, b)
        if precision == fq.FQ_FP64:
            np.testing.assert_array_equal(a.data, b.data)
        else:
            assert rel_frob(a, b) < (1e-6 if precision == fq.FQ_FP32 else 1e-15)
        assert rel_frob(a, getattr(owc, name)(k)) < tol
        single.close()
        m.close()
    mesh.close()
