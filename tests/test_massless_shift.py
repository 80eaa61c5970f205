"""The massless Dirac solve's method, checked on the CPU with the oracle.

At m = 0 the relative Hodge-Dirac system couples even grades to odd ones only,
so its same-grade blocks vanish; the device factors the bordered system with a
small mass shift tau ([[S + tau M, h], [h^T, 0]], tau = 1e-3 / diameter) and
runs GMRES on the exact bordered system ([[S, h], [h^T, 0]], solve_bordered,
problems/dirac.rs:578-598). This restates that scheme with SciPy (SuperLU for
the shifted factors) on the oracle's systems: GMRES needs few iterations and
returns the oracle's bordered solution. It checks the method, not the device
kernels (tests/test_gpu_sparse_lu.py does that)."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def bordered(s, h):
    n = s.shape[0]
    nz = np.nonzero(h)[0]
    col = sp.csr_matrix((h[nz], (nz, np.zeros(len(nz), int))), shape=(n, 1))
    return sp.bmat([[s, col], [col.T, None]]).tocsc()


@pytest.mark.parametrize("dim,nb,minkowski", [(2, 6, True), (3, 3, True), (3, 3, False)])
def test_shifted_factors_precondition_the_massless_bordered_system(oracle, dim, nb, minkowski):
    if minkowski:
        cx, coords, signs = oracle.minkowski(dim, nb)
        lengths = cx.edge_lengths_sq(coords, signs)
    else:
        cx, coords = oracle.cartesian_unit(dim, nb)
        lengths = cx.edge_lengths_sq(coords)
    lengths = lengths * (1.0 + 0.05 * oracle.uniform_pm1(8, np.arange(len(lengths), dtype=np.uint64)))
    ntot = sum(cx.nsimplices(k) for k in range(dim + 1))
    load = np.random.default_rng(3).standard_normal(ntot)
    s0, rhs, _, _ = oracle.dirac_source_system(cx, lengths, 0.0, load, np.zeros(ntot))
    diam = nb * np.sqrt(np.mean(np.abs(lengths)))
    tau = 1e-3 / diam
    st, _, _, _ = oracle.dirac_source_system(cx, lengths, tau, load, np.zeros(ntot))
    h = oracle.top_harmonic(cx, lengths)
    b = np.concatenate([rhs, [0.0]])
    lu = spla.splu(bordered(st, h))
    its = [0]

    def count(_):
        its[0] += 1

    x, info = spla.gmres(bordered(s0, h), b, M=spla.LinearOperator((len(b),) * 2, matvec=lu.solve), rtol=1e-12,
                         restart=30, maxiter=5, callback=count, callback_type="pr_norm")
    assert info == 0 and its[0] <= 12, (info, its[0])
    want = oracle.dirac_solve_source(cx, lengths, 0.0, load, np.zeros(ntot))
    got = np.zeros(ntot)
    keep = np.concatenate([cx.interior(k) + sum(cx.nsimplices(j) for j in range(k)) for k in range(dim + 1)])
    got[keep] = x[:-1]
    assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-8
