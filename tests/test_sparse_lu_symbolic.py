"""The sparse direct solver's symbolic analysis on the host (no GPU), through
fq_sparse_lu_analyse_host: the nested-dissection ordering of the Kuhn lattice
eliminates every unknown exactly once, the fronts and maps it builds keep every
index the kernels form inside its buffer (the analysis checks this itself and
fails otherwise), and unknowns whose vertices do not lie on one branch of the
dissection are rejected. The systems are the oracle's: the relative Dirac
system (with and without the harmonic border row) and the mixed KKT system."""
import ctypes

import numpy as np
import pytest

import formoniq_gb300 as fq


@pytest.fixture(scope="module")
def native():
    from formoniq_gb300 import _build

    _build.build()
    return fq.load()


def dof_vertices(cx, grades, relative):
    rows = []
    for k in grades:
        simp = cx.simplices(k)
        keep = cx.interior(k) if relative else np.arange(len(simp))
        for s in keep:
            rows.append(list(simp[s]) + [-1] * (4 - k))
    return np.array(rows, np.int32).reshape(-1, 5)


def analyse(native, dim, nb, a, dofv):
    a = a.tocsr()
    a.sort_indices()
    rp = np.ascontiguousarray(a.indptr, np.int32)
    ci = np.ascontiguousarray(a.indices, np.int32)
    dv = np.ascontiguousarray(dofv, np.int32)
    stats = np.zeros(6)
    s = native.fq_sparse_lu_analyse_host(dim, nb, a.shape[0], rp.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                         ci.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                         dv.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                         stats.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return s, stats


def dirac(oracle, dim, nb, mass=1.5):
    cx, coords, signs = oracle.minkowski(dim, nb)
    lengths = cx.edge_lengths_sq(coords, signs)
    ntot = sum(cx.nsimplices(k) for k in range(dim + 1))
    s_rel, _, _, _ = oracle.dirac_source_system(cx, lengths, mass, np.zeros(ntot), np.zeros(ntot))
    return cx, lengths, s_rel


@pytest.mark.parametrize("dim,nb", [(1, 9), (2, 7), (3, 5), (4, 3)])
def test_dirac_ordering_eliminates_every_unknown_once(native, oracle, dim, nb):
    cx, _, s_rel = dirac(oracle, dim, nb)
    st, stats = analyse(native, dim, nb, s_rel, dof_vertices(cx, range(dim + 1), True))
    assert st == 0
    fronts, levels, flops, nbytes, maxm, sumf = stats
    assert sumf == s_rel.shape[0]
    assert fronts >= 1 and levels >= 1 and flops > 0 and nbytes > 0 and maxm <= s_rel.shape[0]
    if dim >= 2:
        # the dissection pays: the factorization costs far less than a dense LU
        assert flops < 2.0 / 3.0 * s_rel.shape[0] ** 3 / 4


def test_bordered_system_puts_the_border_at_the_root(native, oracle):
    import scipy.sparse as sp

    dim, nb = 3, 4
    cx, lengths, s_rel = dirac(oracle, dim, nb, mass=0.0)
    h = oracle.top_harmonic(cx, lengths)
    n = s_rel.shape[0]
    nz = np.nonzero(h)[0]
    border = sp.csr_matrix((h[nz], (nz, np.full(len(nz), 0))), shape=(n, 1))
    b = sp.bmat([[s_rel, border], [border.T, None]]).tocsr()
    dv = np.vstack([dof_vertices(cx, range(dim + 1), True), -np.ones((1, 5), np.int32)])
    st, stats = analyse(native, dim, nb, b, dv)
    assert st == 0 and stats[5] == n + 1


def test_kkt_system(native, oracle):
    dim, nb, k = 3, 4, 1
    cx, coords = oracle.cartesian_unit(dim, nb)
    wc = oracle.WhitneyComplex(cx, cx.edge_lengths_sq(coords))
    a, _, ns, nu = oracle.assemble_mixed_kkt(wc, np.zeros(cx.nsimplices(k)), k, np.zeros((cx.nsimplices(k), 0)))
    st, stats = analyse(native, dim, nb, a, dof_vertices(cx, [k - 1, k], False))
    assert st == 0 and stats[5] == ns + nu


def test_unknowns_across_branches_are_rejected(native, oracle):
    """A vertex list joining opposite corners of the lattice cannot come from a
    Kuhn simplex: the analysis refuses it instead of building a wrong tree."""
    dim, nb = 3, 4
    cx, _, s_rel = dirac(oracle, dim, nb)
    dv = dof_vertices(cx, range(dim + 1), True)
    dv[0, :2] = [0, (nb + 1) ** dim - 1]
    st, _ = analyse(native, dim, nb, s_rel, dv)
    assert st == 9  # FQ_UNSUPPORTED
