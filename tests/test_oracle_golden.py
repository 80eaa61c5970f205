"""Pin the oracle (the CPU restatement) against the reference's own known-answer
tests and laws. CPU only: these run without a GPU.

Each test names the reference test it ports.
"""
import itertools
import math

import numpy as np
import pytest
import scipy.sparse as sp

from golden import reference_known_answers as KA

MASS, DIF_TRIAL, DIF_TEST, DIF_BOTH = 0, 1, 2, 3


def rel_frob(a, b):
    a = a.toarray() if sp.issparse(a) else np.asarray(a)
    b = b.toarray() if sp.issparse(b) else np.asarray(b)
    den = max(np.linalg.norm(b), 1e-300)
    return np.linalg.norm(a - b) / den


# ---- element matrices on the reference cell (operators.rs, tests/unit_elmat.rs) ----

def test_hodge_mass_dim2_grade1(oracle):
    m = oracle.element_matrix(2, MASS, 1, oracle.unit_lengths(2))
    np.testing.assert_allclose(m, KA.HODGE_MASS_DIM2_GRADE1, atol=1e-15)


def test_dif_trial_and_dif_test_n2_k1(oracle):
    np.testing.assert_allclose(oracle.element_matrix(2, DIF_TRIAL, 1, oracle.unit_lengths(2)), KA.DIF_TRIAL_N2_K1,
                               atol=1e-15)
    np.testing.assert_allclose(oracle.element_matrix(2, DIF_TEST, 1, oracle.unit_lengths(2)), KA.DIF_TEST_N2_K1,
                               atol=1e-15)


@pytest.mark.parametrize("dim", [0, 1, 2, 3])
def test_unit_mass_and_mass0_is_scalar_mass(oracle, dim):
    m = oracle.element_matrix(dim, MASS, 0, oracle.unit_lengths(dim))
    np.testing.assert_allclose(m, KA.UNIT_MASS[dim], atol=1e-15)
    # hodge_mass0_is_scalar_mass (operators.rs:920-929): vol * Q
    nv = dim + 1
    q = (np.ones((nv, nv)) + np.eye(nv)) / (nv * (nv + 1))
    np.testing.assert_allclose(m, q / math.factorial(dim), atol=1e-15)


@pytest.mark.parametrize("dim", list(range(1, 11)))
def test_unit_laplacian(oracle, dim):
    m = oracle.element_matrix(dim, DIF_BOTH, 1, oracle.unit_lengths(dim))
    np.testing.assert_allclose(m, KA.unit_laplacian(dim), rtol=1e-13, atol=1e-15)


def _compound(b, k):
    n = b.shape[0]
    subs = [c for c in itertools.combinations(range(n), k)]
    subs.sort(key=lambda c: sum(1 << v for v in c))  # colex
    out = np.zeros((len(subs), len(subs)))
    for i, r in enumerate(subs):
        for j, c in enumerate(subs):
            out[i, j] = np.linalg.det(b[np.ix_(r, c)]) if k else 1.0
    return out


def _random_cell_lengths(n, rng):
    x = np.vstack([np.zeros(n), np.eye(n) + 0.2 * rng.standard_normal((n, n))])
    edges = [(a, b) for b in range(n + 1) for a in range(b)]
    return np.array([np.sum((x[b] - x[a]) ** 2) for a, b in edges]), x


@pytest.mark.parametrize("dim", [1, 2, 3, 4])
def test_dif_both_is_gramian_of_difwhitneys(oracle, dim):
    """operators.rs:977-997: dif_both(k+1) = vol (k+1)!^2 <dlambda_I, dlambda_J>."""
    rng = np.random.default_rng(dim)
    lengths, x = _random_cell_lengths(dim, rng)
    e = (x[1:] - x[0])
    g = e @ e.T
    gi = np.linalg.inv(g)
    L = np.vstack([-np.ones(dim), np.eye(dim)])
    B = L @ gi @ L.T
    vol = math.sqrt(abs(np.linalg.det(g))) / math.factorial(dim)
    for grade in range(dim):
        k = grade + 1
        d = oracle.element_matrix(dim, DIF_BOTH, k, lengths)
        expect = vol * math.factorial(k) ** 2 * _compound(B, k)
        assert rel_frob(d, expect) < 1e-12


# ---- meshes (regge/src/mesher/cartesian.rs, simplicial/src/mesher/grid.rs) ----

def test_unit_cube_mesh(oracle):
    cx, coords = oracle.cartesian_unit(3, 1)
    np.testing.assert_array_equal(cx.simplices(3), KA.UNIT_CUBE_CELLS)
    np.testing.assert_array_equal(coords, KA.UNIT_CUBE_COORDS)


def test_unit_square_mesh(oracle):
    cx, coords = oracle.cartesian_unit(2, 2)
    np.testing.assert_array_equal(cx.simplices(2), KA.UNIT_SQUARE_CELLS)
    np.testing.assert_array_equal(coords, KA.UNIT_SQUARE_COORDS)


@pytest.mark.parametrize("dim", [1, 2, 3, 4])
@pytest.mark.parametrize("n", [1, 2, 3])
def test_the_counts_hold_at_every_size(oracle, dim, n):
    """grid.rs:143-154."""
    cx = oracle.Complex.from_cells(oracle.kuhn_cells(dim, n))
    assert cx.ncells() == math.factorial(dim) * n ** dim
    assert cx.nsimplices(0) == (n + 1) ** dim


def test_skeletons_are_colex_sorted(oracle):
    cx = oracle.Complex.from_cells(oracle.kuhn_cells(3, 2))
    for k in range(4):
        s = cx.simplices(k)
        keys = [tuple(reversed(r)) for r in s.tolist()]
        assert keys == sorted(keys) and len(set(keys)) == len(keys)


# ---- topology (simplicial/src/topology/{complex,orientation}.rs) ----

@pytest.mark.parametrize("dim", [1, 2, 3])
def test_coboundary_squares_to_zero(oracle, dim):
    """complex.rs:394-408: dif(k+1) dif(k) = 0 exactly on cube(dim, 2), on the
    full and on the relative complex."""
    cx, coords = oracle.cartesian_unit(dim, 2)
    lengths = cx.edge_lengths_sq(coords)
    for relative in (False, True):
        wc = oracle.WhitneyComplex(cx, lengths, relative=relative)
        for k in range(dim - 1):
            dd = (wc.dif(k + 1) @ wc.dif(k)).tocsr()
            assert np.all(dd.data == 0.0), (relative, k)


def coherent(cx, sgn):
    """Adjacent cells induce opposite orientations on their shared facet: the
    facet that drops vertex position p of a cell with sign s gets s (-1)^p."""
    facets = {}
    for c, cell in enumerate(cx.simplices(cx.dim)):
        for p in range(cx.dim + 1):
            f = tuple(np.delete(cell, p).tolist())
            induced = sgn[c] * (-1.0) ** p
            if f in facets:
                if facets.pop(f) != -induced:
                    return False
            else:
                facets[f] = induced
    return True


@pytest.mark.parametrize("dim", [1, 2, 3, 4])
def test_kuhn_boxes_are_coherently_oriented(oracle, dim):
    """orientation.rs:240-275: the orientation the top harmonic is built on
    (z = M_n h) is coherent on the Kuhn boxes N = 2, every sign +-1."""
    cx = oracle.Complex.from_cells(oracle.kuhn_cells(dim, 2))
    sgn = oracle.orientation_signs(cx)
    assert np.all(np.abs(sgn) == 1.0)
    assert coherent(cx, sgn)


def test_sphere_is_orientable_and_not_trivially_signed(oracle):
    """orientation.rs:327-343: the boundary of a tetrahedron is coherently
    oriented, and not by all-positive signs (its colex frames disagree)."""
    cx = oracle.Complex.from_cells(np.array([[0, 1, 2], [0, 1, 3], [0, 2, 3], [1, 2, 3]], np.int32))
    sgn = oracle.orientation_signs(cx)
    assert np.all(np.abs(sgn) == 1.0) and coherent(cx, sgn)
    assert (sgn < 0).any()
    assert not coherent(cx, np.ones(4))


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_boundary_facets_are_the_facets_of_one_cell(oracle, dim):
    """complex.rs:410-424: the (n-1)-simplices the relative complex drops are
    exactly the facets that belong to a single cell."""
    cx = oracle.Complex.from_cells(oracle.kuhn_cells(dim, 2))
    count = {}
    for cell in cx.simplices(dim):
        for p in range(dim + 1):
            f = tuple(np.delete(cell, p).tolist())
            count[f] = count.get(f, 0) + 1
    facets = cx.simplices(dim - 1)
    single = {i for i, f in enumerate(facets) if count[tuple(f.tolist())] == 1}
    assert set(range(len(facets))) - set(cx.interior(dim - 1).tolist()) == single


# ---- geometry (regge/src/lengths/simplex.rs:350-436) ----

@pytest.mark.parametrize("dim", [1, 2, 3, 4])
def test_metric_tensor_roundtrip(oracle, dim):
    for q in range(dim + 1):
        j = np.eye(dim)
        for i in range(dim):
            for jj in range(i):
                j[i, jj] = ((2 * i + 3 * jj) % 4) / 8
        eta = np.diag([1.0] * (dim - q) + [-1.0] * q)
        g = j.T @ eta @ j
        edges = [(a, b) for b in range(dim + 1) for a in range(b)]
        lengths = np.array([g[b - 1, b - 1] if a == 0 else g[a - 1, a - 1] + g[b - 1, b - 1] - 2 * g[a - 1, b - 1]
                            for a, b in edges])
        cx = oracle.Complex.from_cells(np.arange(dim + 1, dtype=np.int32)[None, :])
        G, Gi, det, vol, bad = cx.cell_metrics(lengths)
        assert bad == 0
        np.testing.assert_allclose(G[0], g, atol=1e-12)
        np.testing.assert_allclose(Gi[0] @ g, np.eye(dim), atol=1e-10)
        assert np.sign(det[0]) == (-1) ** q


@pytest.mark.parametrize("dim", [2, 3, 4])
def test_minkowski_regge_volume(oracle, dim):
    """simplex.rs:414-431: the Minkowski reference cell has the unit volume."""
    eta = np.diag([-1.0] + [1.0] * (dim - 1))
    edges = [(a, b) for b in range(dim + 1) for a in range(b)]
    lengths = np.array([eta[b - 1, b - 1] if a == 0 else eta[a - 1, a - 1] + eta[b - 1, b - 1] - 2 * eta[a - 1, b - 1]
                        for a, b in edges])
    cx = oracle.Complex.from_cells(np.arange(dim + 1, dtype=np.int32)[None, :])
    _, _, _, vol, _ = cx.cell_metrics(lengths)
    assert abs(vol[0] - 1 / math.factorial(dim)) < 1e-12


@pytest.mark.parametrize("dim", [2, 3, 4])
def test_degeneracy_is_scale_invariant(oracle, dim):
    """simplex.rs:378-390: the unit simplex scaled by s^2 (s = 1e-4, 1, 1e4) is
    not degenerate; with edge (1, 2) collapsed to 0 it is, at every scale (the
    oracle flags the cell whose metric has no inverse, where Metric::dual
    would panic)."""
    edges = [(a, b) for b in range(dim + 1) for a in range(b)]
    unit = np.array([1.0 if a == 0 else 2.0 for a, b in edges])
    cx = oracle.Complex.from_cells(np.arange(dim + 1, dtype=np.int32)[None, :])
    for s in (1e-4, 1.0, 1e4):
        lengths = unit * s * s
        assert cx.cell_metrics(lengths)[4] == 0
        lengths[edges.index((1, 2))] = 0.0
        assert cx.cell_metrics(lengths)[4] == 1


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_edge_length_is_endpoint_distance(oracle, dim):
    """coord/mesh.rs:327-342: an edge's squared length is the squared distance
    of its endpoints, exactly (unit boxes N = 2)."""
    cx, coords = oracle.cartesian_unit(dim, 2)
    e = cx.simplices(1)
    d = coords[e[:, 1]] - coords[e[:, 0]]
    want = np.zeros(len(e))
    for a in range(coords.shape[1]):
        want = want + d[:, a] * d[:, a]
    np.testing.assert_array_equal(cx.edge_lengths_sq(coords), want)


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_minkowski_ambient_induces_lorentzian_cell_metrics(oracle, dim):
    """coord/mesh.rs:344-363: the unit box N = 2 in Minkowski ambient space
    (its diagonal edges null) has every cell metric of signature (n-1, 1)."""
    cx, coords = oracle.cartesian_unit(dim, 2)
    signs = np.ones(dim)
    signs[0] = -1.0
    g, _, det, _, bad = cx.cell_metrics(cx.edge_lengths_sq(coords, signs))
    assert bad == 0 and np.all(det < 0)
    for gc in g:
        ev = np.linalg.eigvalsh(gc)
        assert (ev < 0).sum() == 1 and (ev > 0).sum() == dim - 1


def test_lorentzian_ambient_realizes_lorentzian_regge_data(oracle):
    """coord/mesh.rs:365-398: the 2D box N = 1 with time scaled 0.7 has both
    timelike and spacelike edges, and each cell metric rebuilt from the signed
    lengths is the embedding's E^T eta E (1e-12), signature (1, 1)."""
    cx, coords, signs = oracle.minkowski(2, 1)
    lengths = cx.edge_lengths_sq(coords, signs)
    assert (lengths < 0).any() and (lengths > 0).any()
    g = cx.cell_metrics(lengths)[0]
    eta = np.diag(signs)
    for c, cell in enumerate(cx.simplices(2)):
        e = (coords[cell[1:]] - coords[cell[0]]).T
        np.testing.assert_allclose(g[c], e.T @ eta @ e, rtol=0, atol=1e-12)
        ev = np.linalg.eigvalsh(g[c])
        assert (ev < 0).sum() == 1 and (ev > 0).sum() == 1


def lengths_from_cell_gramians(cx, gramian_of_cell):
    """Per-cell Gram matrices G (edge vectors from the cell's first vertex) read
    back as edge lengths, l_ij = G_ii + G_jj - 2 G_ij with G_0. = 0: the
    reference's metric -> lengths conversion (CellGramians::to_edge_lengths_sq).
    Every cell sharing an edge must read back the same length."""
    index = {tuple(e): i for i, e in enumerate(cx.simplices(1))}
    out = np.full(len(index), np.nan)
    for c in cx.simplices(cx.dim):
        g = np.zeros((len(c), len(c)))
        g[1:, 1:] = gramian_of_cell(c)
        for i in range(len(c)):
            for j in range(i + 1, len(c)):
                ln = g[i, i] + g[j, j] - 2 * g[i, j]
                e = index[(c[i], c[j])]
                if np.isnan(out[e]):
                    out[e] = ln
                else:
                    assert abs(out[e] - ln) <= 1e-12 * max(1.0, abs(ln))
    assert not np.isnan(out).any()
    return out


def masses_agree(oracle, cx, a_lengths, b_lengths):
    wa, wb = oracle.WhitneyComplex(cx, a_lengths), oracle.WhitneyComplex(cx, b_lengths)
    for k in range(cx.dim + 1):
        a, b = wa.mass(k).toarray(), wb.mass(k).toarray()
        assert np.abs(a - b).max() <= 1e-12 * max(1.0, np.abs(a).max()), k


def test_cell_gramians_round_trip_assembles_identically(oracle):
    """galerkin.rs:380-392: lengths -> per-cell metrics -> lengths on the unit
    3D box N = 2 gives the same masses (1e-12)."""
    cx, coords = oracle.cartesian_unit(3, 2)
    lengths = cx.edge_lengths_sq(coords)
    index = {tuple(e): i for i, e in enumerate(cx.simplices(1))}

    def from_lengths(c):  # G_ij = (l_0i + l_0j - l_ij) / 2
        l0 = [lengths[index[(c[0], v)]] for v in c[1:]]
        n = len(c) - 1
        lij = lambda i, j: lengths[index[(c[min(i, j) + 1], c[max(i, j) + 1])]]
        return np.array([[l0[i] if i == j else (l0[i] + l0[j] - lij(i, j)) / 2 for j in range(n)] for i in range(n)])

    masses_agree(oracle, cx, lengths, lengths_from_cell_gramians(cx, from_lengths))


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_lorentzian_sources_reduce_to_the_same_regge_data(oracle, dim):
    """galerkin.rs:394-421: on the Minkowski box (time axis scaled 0.7) the
    lengths of the embedding and the lengths read back from the per-cell
    Gramians E^T eta E it induces assemble the same masses (1e-12)."""
    cx, coords, signs = oracle.minkowski(dim, 2)
    eta = np.diag(signs)

    def from_coords(c):
        e = (coords[c[1:]] - coords[c[0]]).T
        return e.T @ eta @ e

    masses_agree(oracle, cx, cx.edge_lengths_sq(coords, signs), lengths_from_cell_gramians(cx, from_coords))


# ---- global operators (tests/fem3d.rs, tests/fdm.rs, whitney_complex.rs tests) ----

def _fem3d(n):
    """The reference's hand-written 3D P1 stiffness (tests/fem3d.rs:18-104)."""
    nvd = n + 1
    nv = nvd ** 3
    h = 1.0 / n
    coords = np.zeros((nv, 3))
    for z in range(nvd):
        for y in range(nvd):
            for x in range(nvd):
                coords[x + nvd * (y + nvd * z)] = (h * x, h * y, h * z)
    tet_vol = h ** 3 / 6
    gal = np.zeros((nv, nv))
    for zb in range(n):
        for yb in range(n):
            for xb in range(n):
                box = [0] * 8
                for k in range(2):
                    for j in range(2):
                        for i in range(2):
                            box[i + 2 * (j + 2 * k)] = (xb + i) + nvd * ((yb + j) + nvd * (zb + k))
                for tet in KA.FEM3D_TETS:
                    gv = [box[i] for i in tet]
                    pts = coords[gv]
                    ns = []
                    for i in range(4):
                        face = np.delete(pts, i, axis=0)
                        sign = 1.0 if i % 2 == 0 else -1.0
                        ns.append(sign * np.cross(face[1] - face[0], face[2] - face[0]))
                    el = np.array([[ns[i] @ ns[j] for j in range(4)] for i in range(4)]) / (36 * tet_vol)
                    for a in range(4):
                        for b in range(4):
                            gal[gv[a], gv[b]] += el[a, b]
    return gal


@pytest.mark.parametrize("n", [1, 2, 3, 4])
def test_feec_vs_fem3d(oracle, n):
    cx, coords = oracle.cartesian_unit(3, n)
    wc = oracle.WhitneyComplex(cx, cx.edge_lengths_sq(coords))
    np.testing.assert_allclose(wc.dif_both(1).toarray(), _fem3d(n), atol=1e-12, rtol=1e-12)


def _kron_sum(mats):
    out = 0
    sizes = [m.shape[0] for m in mats]
    for d, m in enumerate(mats):
        before = np.eye(int(np.prod(sizes[:d]))) if d else np.eye(1)
        after = np.eye(int(np.prod(sizes[d + 1:]))) if d + 1 < len(sizes) else np.eye(1)
        out = out + np.kron(np.kron(before, m), after)
    return out


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_fdm_vs_handchecked_interior(dim):
    lap1 = np.array([[2, -1], [-1, 2]])
    np.testing.assert_array_equal(_kron_sum([lap1] * dim), KA.LAPLACE_MATRICES_INTERIOR[dim])


@pytest.mark.parametrize("dim", [1, 2, 3, 4])
@pytest.mark.parametrize("nb", [1, 2, 3])
def test_feec_vs_fdm_interior(oracle, dim, nb):
    """tests/fdm.rs:166-206."""
    if dim == 4 and nb == 3:
        pytest.skip("covered at smaller sizes")
    n = nb + 2
    cx = oracle.Complex.from_cells(oracle.kuhn_cells(dim, n))
    coords = oracle.grid_coords(dim, n, side=np.full(dim, float(n)))
    wc = oracle.WhitneyComplex(cx, cx.edge_lengths_sq(coords))
    gal = wc.dif_both(1).toarray()
    galvec = wc.mass(0) @ np.ones(cx.nsimplices(0))
    gal = gal / galvec[:, None]
    cart = np.array([[(v // (n + 1) ** a) % (n + 1) for a in range(dim)] for v in range(cx.nsimplices(0))])
    interior = np.all((cart != 0) & (cart != n), axis=1)
    sub = gal[np.ix_(interior, interior)]
    assert np.all(np.abs(sub - np.round(sub)) <= 1e-11)
    lap1 = np.diag(2 * np.ones(nb + 1)) - np.diag(np.ones(nb), 1) - np.diag(np.ones(nb), -1)
    np.testing.assert_array_equal(np.round(sub).astype(int), _kron_sum([lap1] * dim).astype(int))


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_dif_both_and_dif_test_local_and_global_routes_agree(oracle, dim):
    """whitney_complex.rs:733-815."""
    cx, coords = oracle.cartesian_unit(dim, 2)
    wc = oracle.WhitneyComplex(cx, cx.edge_lengths_sq(coords))
    for grade in range(dim + 1):
        local = wc.dif_both(grade + 1)
        d = wc.dif(grade)
        glob = d.T @ wc.mass(grade + 1) @ d
        scale = max(np.abs(local.toarray()).max() if local.nnz else 0.0, 1.0)
        assert local.shape == glob.shape
        assert np.abs((local - glob).toarray()).max() <= 1e-12 * scale
        lt = wc.dif_test(grade)
        gt = wc.dif(grade - 1).T @ wc.mass(grade)
        assert lt.shape == gt.shape
        if lt.shape[0] and lt.shape[1]:
            assert np.abs((lt - gt).toarray()).max() <= 1e-12 * max(np.abs(lt.toarray()).max(), 1.0)


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_hdif_norm_and_gram_agree(oracle, dim):
    """whitney_complex.rs:866-891: the quadratic form of hdif_gram(k) is the
    squared L2 norm plus the squared dif seminorm (by the global product
    D_k u against M_{k+1}), on the unit boxes N = 2, every grade (1e-10)."""
    cx, coords = oracle.cartesian_unit(dim, 2)
    wc = oracle.WhitneyComplex(cx, cx.edge_lengths_sq(coords))
    for k in range(dim + 1):
        u = (np.arange(cx.nsimplices(k)) % 5) - 2.0
        l2 = u @ (wc.mass(k) @ u)
        semi = 0.0
        if k < dim:
            du = wc.dif(k) @ u
            semi = du @ (wc.mass(k + 1) @ du)
        gram = u @ (wc.hdif_gram(k) @ u)
        assert semi >= -1e-12
        assert abs(math.sqrt(gram) - math.sqrt(l2 + semi)) < 1e-10, (k, gram, l2 + semi)


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_the_relative_stiffness_is_the_restriction_of_the_full_one(oracle, dim):
    """whitney_complex.rs:825-861."""
    cx, coords = oracle.cartesian_unit(dim, 2)
    rel = oracle.WhitneyComplex(cx, cx.edge_lengths_sq(coords), relative=True)
    for grade in range(dim + 1):
        if grade < dim:
            assert rel.ndofs(grade) < cx.nsimplices(grade)
        r = rel.dif_both(grade + 1)
        d = rel.dif(grade)
        by_def = d.T @ rel.mass(grade + 1) @ d
        assert np.abs((r - by_def).toarray()).max() <= 1e-12 * max(np.abs(r.toarray()).max() if r.nnz else 0, 1.0)


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_operators_are_total_at_the_trivial_ends(oracle, dim):
    """whitney_complex.rs:989-1027."""
    cx, coords = oracle.cartesian_unit(dim, 2)
    wc = oracle.WhitneyComplex(cx, cx.edge_lengths_sq(coords))
    for ghost in (-1, dim + 1):
        assert wc.ndofs(ghost) == 0
        assert wc.mass(ghost).shape == (0, 0)
        assert wc.dif_both(ghost + 1).shape == (0, 0)
    assert wc.dif(-1).shape == (wc.ndofs(0), 0)
    assert wc.dif(dim).shape == (0, wc.ndofs(dim))
    top = wc.dif_both(dim + 1)
    assert top.shape == (wc.ndofs(dim), wc.ndofs(dim)) and top.nnz == 0


# ---- Krylov (iterative/src/krylov.rs:224-320) ----

def _sym_from_spectrum(eigs, seed=0):
    n = len(eigs)
    if n == 0:
        return np.zeros((0, 0))
    q, _ = np.linalg.qr(np.random.default_rng(seed).standard_normal((n, n)))
    return q @ np.diag(eigs) @ q.T


@pytest.mark.parametrize("n", list(range(0, 9)))
def test_cg_terminates_in_at_most_n_steps(oracle, n):
    a = _sym_from_spectrum([1.0 + k for k in range(n)])
    x_true = np.log(np.arange(1, n + 1, dtype=float))
    b = a @ x_true
    x, rep = oracle.cg(sp.csr_matrix(a), lambda r: r, b, rtol=1e-10, max_iters=max(n, 1))
    assert rep.converged and rep.iters <= n
    if n:
        assert np.linalg.norm(x - x_true) < 1e-7


@pytest.mark.parametrize("n", list(range(0, 9)))
def test_minres_solves_symmetric_indefinite_systems(oracle, n):
    eigs = [(k // 2 + 1) * (1 if k % 2 == 0 else -1) for k in range(n)]
    a = _sym_from_spectrum(eigs)
    b = np.sqrt(np.arange(1, n + 1, dtype=float))
    x, rep = oracle.minres(sp.csr_matrix(a), lambda r: r, b, rtol=1e-11)
    assert rep.converged
    if n:
        assert np.linalg.norm(x - np.linalg.solve(a, b)) < 1e-7


def test_minres_agrees_with_cg_on_spd(oracle):
    n = 25
    a = sp.diags([np.ones(n - 1), 4 * np.ones(n), np.ones(n - 1)], [-1, 0, 1]).tocsr()
    x_true = np.sin(np.arange(n, dtype=float))
    b = a @ x_true
    jac = oracle.jacobi(a.diagonal())
    xm, rm = oracle.minres(a, jac, b, rtol=1e-12)
    xc, _ = oracle.cg(a, jac, b, rtol=1e-12)
    assert rm.converged
    assert np.linalg.norm(xm - x_true) < 1e-8
    assert np.linalg.norm(xm - xc) < 1e-7


def test_preconditioning_preserves_the_solution(oracle):
    """krylov.rs:247-262: Jacobi-preconditioned CG and plain CG reach the same
    solution of tridiag(20; 1, 4, 1) (1e-9)."""
    n = 20
    a = sp.diags([np.ones(n - 1), 4.0 * np.ones(n), np.ones(n - 1)], [-1, 0, 1]).tocsr()
    x_true = np.cos(np.arange(n) ** 2.0)
    b = a @ x_true
    x_plain, r1 = oracle.cg(a, lambda r: r, b, rtol=1e-12)
    x_jacobi, r2 = oracle.cg(a, lambda r: r / a.diagonal(), b, rtol=1e-12)
    assert r1.converged and r2.converged
    assert np.linalg.norm(x_plain - x_true) < 1e-9
    assert np.linalg.norm(x_jacobi - x_true) < 1e-9
    assert np.linalg.norm(x_plain - x_jacobi) < 1e-9


def test_block_diagonal_of_exact_blocks_is_exact(oracle):
    """precond.rs:217-240: on a block-diagonal operator (blocks of 3, 4 and 2
    distinct diagonal entries) the block-Jacobi preconditioner is the exact
    inverse, so preconditioned CG converges in one step (the oracle's MINRES
    too); precond.rs:242-255: the block preconditioner is self-adjoint."""
    sizes = [3, 4, 2]
    offs = np.cumsum([0] + sizes)
    d = 1.0 + (np.arange(offs[-1]) % 6)
    a = sp.diags(d).tocsr()
    blocks = [1.0 / d[offs[i]:offs[i + 1]] for i in range(len(sizes))]

    def precond(r):
        return np.concatenate([blocks[i] * r[offs[i]:offs[i + 1]] for i in range(len(sizes))])

    b = np.cos(np.arange(offs[-1]) - 4.0)
    for solve in (oracle.cg, oracle.minres):
        x, rep = solve(a, precond, b, rtol=1e-12)
        assert rep.converged and rep.iters <= 1, (solve.__name__, rep)
        assert np.linalg.norm(x - b / d) < 1e-9
    r = np.log(np.arange(1.0, offs[-1] + 1))
    s = np.cos(2.0 * np.arange(offs[-1]))
    assert abs(precond(r) @ s - r @ precond(s)) < 1e-12


# ---- the mixed problem (problems/elliptic.rs:259-367) ----

@pytest.mark.parametrize("dim", [1, 2, 3])
def test_block_minres_matches_direct_on_the_mixed_system(oracle, dim):
    cx, coords = oracle.cartesian_unit(dim, 2)
    rel = oracle.WhitneyComplex(cx, cx.edge_lengths_sq(coords), relative=True)
    for grade in range(dim + 1):
        harm = oracle.harmonics(rel, grade)
        src = (np.arange(cx.nsimplices(grade)) % 7) - 3.0
        a, b, ns, nu = oracle.assemble_mixed_kkt(rel, src, grade, harm)
        assert abs(a - a.T).max() <= 1e-14 * max(abs(a).max(), 1.0)  # symmetrised saddle point
        blocks = []
        if grade > 0:
            blocks.append(rel.hdif_gram(grade - 1))
        blocks.append(rel.hdif_gram(grade))
        if harm.shape[1]:
            blocks.append(sp.identity(harm.shape[1], format="csr"))
        x, rep = oracle.minres(a, oracle.BlockDiagonal(blocks), b, rtol=1e-11)
        assert rep.converged
        x_lu = oracle.direct_solve(a, b)
        err = np.linalg.norm(x - x_lu) / max(np.linalg.norm(x_lu), 1.0)
        assert err < KA.BLOCK_MINRES_VS_LU_TOL


def test_block_minres_iteration_count_is_mesh_independent(oracle):
    def iters(nb):
        cx, coords = oracle.cartesian_unit(2, nb)
        rel = oracle.WhitneyComplex(cx, cx.edge_lengths_sq(coords), relative=True)
        src = ((np.arange(cx.nsimplices(1)) % 5) - 2.0) * 0.3
        _, _, _, rep = oracle.solve_source(rel, src, 1, rtol=1e-10)
        assert rep.converged
        return rep.iters

    assert iters(8) <= iters(4) + KA.MINRES_ITER_SLACK


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_harmonics_are_harmonic(oracle, dim):
    """harmonic.rs tests: dh = 0, D^T M h = 0, M-orthonormal (closed forms)."""
    cx, coords = oracle.cartesian_unit(dim, 2)
    for relative in (False, True):
        wc = oracle.WhitneyComplex(cx, cx.edge_lengths_sq(coords), relative=relative)
        for grade in range(dim + 1):
            h = oracle.harmonics(wc, grade)
            m = wc.mass(grade)
            for col in h.T:
                assert np.linalg.norm(wc.dif(grade) @ col) <= 1e-8 * max(np.linalg.norm(col), 1)
                assert np.linalg.norm(wc.dif(grade - 1).T @ (m @ col)) <= 1e-8 * max(np.linalg.norm(col), 1)
                assert abs(col @ (m @ col) - 1.0) < 1e-8


# ---- Hodge-Dirac (problems/dirac.rs:632-947) ----

@pytest.mark.parametrize("dim", [1, 2, 3])
def test_selfadjoint_operator_is_symmetric(oracle, dim):
    for mink in (False, True):
        if mink:
            cx, coords, signs = oracle.minkowski(dim, 2)
        else:
            (cx, coords), signs = oracle.cartesian_unit(dim, 2), None
        full = oracle.WhitneyComplex(cx, cx.edge_lengths_sq(coords, signs))
        _, _, a = oracle.dirac_selfadjoint(full)
        assert abs(a - a.T).max() == 0.0


def dirac_squared_error(oracle, full, delta_sign, seed):
    """D = M^-1 A of HodgeDirac::assemble_signed(delta_sign) (A built from the
    global products M_k D_{k-1}) applied twice to a seeded field, against
    delta_sign times the Hodge Laplacian of the element-assembled blocks,
    M_k^-1 (dif_both(k+1) u + dif_test(k)^T M_{k-1}^-1 dif_test(k) u) (the
    grade-shifting-by-two terms cancel by d d = 0). Returns the worst grade's
    ||D^2 u - sign Lap u|| / max(||Lap u||, 1)."""
    import scipy.sparse.linalg as spla

    n = full.dim
    off, _, a = oracle.dirac_signed(full, delta_sign)
    lus = [spla.splu(full.mass(k).tocsc()) for k in range(n + 1)]

    def apply(u):
        mv = a @ u
        return np.concatenate([lus[k].solve(mv[off[k]:off[k + 1]]) for k in range(n + 1)])

    u = np.random.default_rng(seed).standard_normal(int(off[-1]))
    d2u = apply(apply(u))
    worst = 0.0
    for k in range(n + 1):
        uk = u[off[k]:off[k + 1]]
        up = full.dif_both(k + 1) @ uk
        if k > 0:
            bt = full.dif_test(k)
            up = up + bt.T @ lus[k - 1].solve(bt @ uk)
        lap = lus[k].solve(up)
        err = np.linalg.norm(d2u[off[k]:off[k + 1]] - delta_sign * lap) / max(np.linalg.norm(lap), 1.0)
        worst = max(worst, err)
    return worst


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_selfadjoint_dirac_squares_to_hodge_laplacian_on_minkowski(oracle, dim):
    """dirac.rs:824-871: the self-adjoint D squares to the Hodge Laplacian
    (1e-9) on the Minkowski boxes N = 2, whose masses are indefinite."""
    cx, coords, signs = oracle.minkowski(dim, 2)
    full = oracle.WhitneyComplex(cx, cx.edge_lengths_sq(coords, signs))
    assert dirac_squared_error(oracle, full, 1.0, dim) <= 1e-9


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_dirac_squared_is_negative_hodge_laplacian(oracle, dim):
    """dirac.rs:683-731: the skew D = dif - delta of the evolution squares to
    minus the Hodge Laplacian (1e-9) on the unit boxes N = 2."""
    cx, coords = oracle.cartesian_unit(dim, 2)
    full = oracle.WhitneyComplex(cx, cx.edge_lengths_sq(coords))
    assert dirac_squared_error(oracle, full, -1.0, dim) <= 1e-9


@pytest.mark.parametrize("dim", [1, 2, 3, 4])
def test_top_harmonic_is_annihilated(oracle, dim):
    """dirac.rs:630-653: the top-grade harmonic h = M_n^-1 z of the relative
    complex is annihilated by the massless self-adjoint Dirac operator,
    |S h| / |h| < 1e-9, on the unit and the Minkowski boxes N = 2 (the kernel
    the device's massless solve borders with)."""
    for mink in (False, True):
        if mink:
            cx, coords, signs = oracle.minkowski(dim, 2)
        else:
            (cx, coords), signs = oracle.cartesian_unit(dim, 2), None
        lengths = cx.edge_lengths_sq(coords, signs)
        ntot = sum(cx.nsimplices(k) for k in range(dim + 1))
        s_rel = oracle.dirac_source_system(cx, lengths, 0.0, np.zeros(ntot), np.zeros(ntot))[0]
        h = oracle.top_harmonic(cx, lengths)
        assert np.linalg.norm(s_rel @ h) / np.linalg.norm(h) < 1e-9, (dim, mink)


def derham_constant(cx, coords, k):
    """de Rham coefficients of the constant k-form with every component 1:
    sum_I det((x_j - x_0)_I) / k! over the simplex (derham/src/project.rs)."""
    s = cx.simplices(k)
    dim = coords.shape[1]
    if k == 0:
        return np.ones(len(s))
    out = np.zeros(len(s))
    subs = list(itertools.combinations(range(dim), k))
    for i, simp in enumerate(s):
        e = (coords[simp[1:]] - coords[simp[0]]).T  # dim x k
        out[i] = sum(np.linalg.det(e[list(I), :]) for I in subs) / math.factorial(k)
    return out


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_dirac_source_reproduces_constant_field(oracle, dim):
    for mink in (False, True):
        if mink:
            cx, coords, signs = oracle.minkowski(dim, 2)
        else:
            (cx, coords), signs = oracle.cartesian_unit(dim, 2), None
        lengths = cx.edge_lengths_sq(coords, signs)
        exact = np.concatenate([derham_constant(cx, coords, k) for k in range(dim + 1)])
        full = oracle.WhitneyComplex(cx, lengths)
        _, mb, _ = oracle.dirac_selfadjoint(full)
        load = mb @ exact
        sol = oracle.dirac_solve_source(cx, lengths, 1.0, load, exact)
        np.testing.assert_allclose(sol, exact, atol=1e-9)
