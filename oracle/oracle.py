"""TEST INFRASTRUCTURE, NOT PRODUCT CODE: the CPU oracle of formoniq's Galerkin path.

Only tests/, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline and
reference arms may import this module, and only as the oracle. It wraps the C++
restatement in ``oracle/fq_oracle.cpp`` (built into ``oracle/_build``) and adds
the parts the reference writes on top of assembled sparse matrices:

* ``assemble_mixed_kkt``  -- formoniq/src/problems/elliptic.rs:54-114
* ``minres`` / ``cg``     -- iterative/src/krylov.rs:113-211 / :48-95
* ``direct_solve``        -- the faer sparse LU (formoniq/src/linalg/faer.rs:41-57),
  stood in for by SciPy SuperLU (faer is a Rust crate and cannot run here)
* ``dirac_selfadjoint``   -- formoniq/src/problems/dirac.rs:213-260, 473-531

Parity status: pinned against the reference's own known-answer tests (see
tests/test_oracle_golden.py); faer-specific and nalgebra-sparse-specific
rounding is unpinned beyond the tolerances those tests assert.
"""
from __future__ import annotations

import ctypes
import itertools
import math
import os
from dataclasses import dataclass

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libfq_oracle.so")

MASS, DIF_TRIAL, DIF_TEST, DIF_BOTH = 0, 1, 2, 3

_lib = None


def build(force: bool = False) -> str:
    """Compile the C++ restatement (g++, OpenMP). Returns the library path."""
    src = os.path.join(_HERE, "fq_oracle.cpp")
    os.makedirs(os.path.dirname(_LIB_PATH), exist_ok=True)
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        import subprocess

        subprocess.check_call(
            ["g++", "-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off",
             "-o", _LIB_PATH, src]
        )
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.c_void_p
        i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
        i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
        f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
        u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
        L.or_kuhn_ncells.restype = ctypes.c_int64
        L.or_kuhn_ncells.argtypes = [ctypes.c_int, ctypes.c_int]
        L.or_kuhn_cells.argtypes = [ctypes.c_int, ctypes.c_int, i32p]
        L.or_grid_coords.argtypes = [ctypes.c_int, ctypes.c_int, f64p, f64p, f64p]
        L.or_complex_build.restype = P
        L.or_complex_build.argtypes = [ctypes.c_int, ctypes.c_int64, i32p]
        L.or_complex_free.argtypes = [P]
        L.or_complex_nsimplices.restype = ctypes.c_int64
        L.or_complex_nsimplices.argtypes = [P, ctypes.c_int]
        L.or_complex_simplices.argtypes = [P, ctypes.c_int, i32p]
        L.or_complex_cell_faces.argtypes = [P, ctypes.c_int, i32p]
        L.or_complex_boundary_flags.argtypes = [P, ctypes.c_int, u8p]
        L.or_edge_lengths_sq.argtypes = [P, f64p, ctypes.c_int, f64p, f64p]
        L.or_cell_metrics.restype = ctypes.c_int64
        L.or_cell_metrics.argtypes = [P, f64p, P, P, P, P]
        L.or_element_matrix.restype = ctypes.c_int
        L.or_element_matrix.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, f64p, f64p,
                                        ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
        L.or_assemble.restype = P
        L.or_assemble.argtypes = [P, f64p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.or_coboundary.restype = P
        L.or_coboundary.argtypes = [P, ctypes.c_int, ctypes.c_int]
        L.or_csr_shape.argtypes = [P, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                                   ctypes.POINTER(ctypes.c_int64)]
        L.or_csr_copy.argtypes = [P, i64p, i64p, f64p]
        L.or_csr_free.argtypes = [P]
        L.or_num_threads.restype = ctypes.c_int
        L.or_set_num_threads.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def num_threads() -> int:
    return lib().or_num_threads()


def set_num_threads(t: int) -> None:
    lib().or_set_num_threads(int(t))


# ---------------------------------------------------------------------------
# Meshes: CartesianGrid / CartesianTopology (regge/src/mesher/cartesian.rs,
# simplicial/src/mesher/grid.rs)
# ---------------------------------------------------------------------------

def kuhn_cells(dim: int, nbox: int) -> np.ndarray:
    """Kuhn cells of the cube, unsorted (grid.rs:77-98)."""
    L = lib()
    n = L.or_kuhn_ncells(dim, nbox)
    out = np.empty((n, dim + 1), np.int32)
    if n:
        L.or_kuhn_cells(dim, nbox, out)
    return out


def grid_coords(dim: int, nbox: int, side=None, minv=None) -> np.ndarray:
    """Vertex coordinates c/N * side + min (cartesian.rs:158-169), [vertex, axis]."""
    side = np.ones(dim) if side is None else np.asarray(side, np.float64)
    minv = np.zeros(dim) if minv is None else np.asarray(minv, np.float64)
    nv = (nbox + 1) ** dim
    out = np.empty((nv, dim), np.float64)
    lib().or_grid_coords(dim, nbox, np.ascontiguousarray(side), np.ascontiguousarray(minv), out)
    return out


def jitter_coords(coords: np.ndarray, nbox: int, seed: int, amplitude: float = 0.1,
                  side=None) -> np.ndarray:
    """Seeded uniform +-amplitude*h jitter of every coordinate of every vertex.

    Boundary vertices move too: a vertex left on an axis-aligned face keeps
    right angles in the corner cells, where mathematically zero element entries
    then round to 0.0 or not depending on operation order, which makes the
    reference's value-dependent `val != 0.0` pattern ill-posed for comparison.
    Same counter-based hash as the library's mesh generator (splitmix64 of
    seed and vertex*dim + axis), so both sides see identical inputs.
    """
    nv, dim = coords.shape
    side = np.ones(dim) if side is None else np.asarray(side, np.float64)
    out = coords.copy()
    v = np.arange(nv, dtype=np.uint64)
    for a in range(dim):
        u = uniform_pm1(seed, v * np.uint64(dim) + np.uint64(a))
        h = side[a] / nbox
        out[:, a] = coords[:, a] + amplitude * h * u
    return out


def splitmix64(x: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = (x + np.uint64(0x9E3779B97F4A7C15)).astype(np.uint64)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def uniform_pm1(seed: int, counter: np.ndarray) -> np.ndarray:
    """Uniform on [-1, 1) from (seed, counter): 53 high bits of splitmix64."""
    with np.errstate(over="ignore"):
        key = splitmix64(np.uint64(seed) ^ splitmix64(counter.astype(np.uint64)))
    return (key >> np.uint64(11)).astype(np.float64) * (2.0 / 2.0 ** 53) - 1.0


@dataclass
class Complex:
    """Complex::from_cells (simplicial/src/topology/complex.rs:298-336)."""

    handle: int
    dim: int

    @staticmethod
    def from_cells(cells: np.ndarray) -> "Complex":
        cells = np.ascontiguousarray(cells, np.int32)
        dim = cells.shape[1] - 1
        h = lib().or_complex_build(dim, cells.shape[0], cells)
        return Complex(h, dim)

    def __del__(self):
        if getattr(self, "handle", None) and _lib is not None:
            _lib.or_complex_free(self.handle)
            self.handle = None

    def nsimplices(self, k: int) -> int:
        if k < 0 or k > self.dim:
            return 0
        return lib().or_complex_nsimplices(self.handle, k)

    def simplices(self, k: int) -> np.ndarray:
        out = np.empty((self.nsimplices(k), k + 1), np.int32)
        if out.size:
            lib().or_complex_simplices(self.handle, k, out)
        return out

    def ncells(self) -> int:
        return self.nsimplices(self.dim)

    def cell_faces(self, k: int) -> np.ndarray:
        nloc = math.comb(self.dim + 1, k + 1)
        out = np.empty((self.ncells(), nloc), np.int32)
        if out.size:
            lib().or_complex_cell_faces(self.handle, k, out)
        return out

    def boundary_flags(self, k: int) -> np.ndarray:
        out = np.zeros(self.nsimplices(k), np.uint8)
        if out.size:
            lib().or_complex_boundary_flags(self.handle, k, out)
        return out.astype(bool)

    def interior(self, k: int) -> np.ndarray:
        """Kept kidx of the relative complex, increasing (whitney_complex.rs:523-566)."""
        return np.nonzero(~self.boundary_flags(k))[0]

    def edge_lengths_sq(self, coords: np.ndarray, ambient_signs=None) -> np.ndarray:
        coords = np.ascontiguousarray(coords, np.float64)
        adim = coords.shape[1]
        signs = np.ones(adim) if ambient_signs is None else np.asarray(ambient_signs, np.float64)
        out = np.empty(self.nsimplices(1), np.float64)
        if out.size:
            lib().or_edge_lengths_sq(self.handle, coords, adim, np.ascontiguousarray(signs), out)
        return out

    def cell_metrics(self, lengths: np.ndarray):
        n, nc = self.dim, self.ncells()
        g = np.empty((nc, n, n))
        gi = np.empty((nc, n, n))
        det = np.empty(nc)
        vol = np.empty(nc)
        bad = lib().or_cell_metrics(self.handle, np.ascontiguousarray(lengths, np.float64),
                                    g.ctypes.data, gi.ctypes.data, det.ctypes.data, vol.ctypes.data)
        return g, gi, det, vol, bad


def cartesian_unit(dim: int, nbox: int):
    """CartesianGrid::new_unit(dim, nbox).triangulate() (cartesian.rs:210-213)."""
    cx = Complex.from_cells(kuhn_cells(dim, nbox))
    return cx, grid_coords(dim, nbox)


def minkowski(dim: int, nbox: int, time_scale: float = 0.7):
    """CartesianGrid::minkowski (cartesian.rs:192-208): [0,0.7] x [0,1]^(d-1)."""
    side = np.ones(dim)
    if dim > 0:
        side[0] = time_scale
    cx = Complex.from_cells(kuhn_cells(dim, nbox))
    signs = np.ones(dim)
    if dim > 0:
        signs[0] = -1.0
    return cx, grid_coords(dim, nbox, side=side), signs


def _csr_from_handle(h) -> sp.csr_matrix:
    L = lib()
    nr, nc, nnz = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    L.or_csr_shape(h, ctypes.byref(nr), ctypes.byref(nc), ctypes.byref(nnz))
    rp = np.empty(nr.value + 1, np.int64)
    ci = np.empty(max(nnz.value, 1), np.int64)
    vv = np.empty(max(nnz.value, 1), np.float64)
    L.or_csr_copy(h, rp, ci, vv)
    L.or_csr_free(h)
    m = sp.csr_matrix((vv[: nnz.value], ci[: nnz.value], rp), shape=(nr.value, nc.value))
    m.has_sorted_indices = True
    return m


def element_matrix(n: int, form: int, grade: int, local_lengths) -> np.ndarray:
    """BilinearForm::element of a WhitneyPairing on one cell (operators.rs:201-211)."""
    ll = np.ascontiguousarray(local_lengths, np.float64)
    if ll.size == 0:
        ll = np.zeros(1)
    rows, cols = ctypes.c_int(), ctypes.c_int()
    tg = grade - 1 if form in (DIF_TEST, DIF_BOTH) else grade
    sg = grade - 1 if form in (DIF_TRIAL, DIF_BOTH) else grade
    cap = max(math.comb(n + 1, tg + 1) if 0 <= tg <= n else 0, 1) * max(
        math.comb(n + 1, sg + 1) if 0 <= sg <= n else 0, 1)
    out = np.zeros(cap)
    lib().or_element_matrix(n, form, grade, ll, out, ctypes.byref(rows), ctypes.byref(cols))
    return out[: rows.value * cols.value].reshape(rows.value, cols.value)


def unit_lengths(n: int) -> np.ndarray:
    """SimplexLengthsSq::unit: the reference cell, s_{0,i}=1, s_{i,j}=2."""
    edges = [(a, b) for b in range(n + 1) for a in range(b)]
    return np.array([1.0 if a == 0 else 2.0 for (a, b) in edges], np.float64)


class WhitneyComplex:
    """HilbertComplex over the oracle (formoniq/src/whitney_complex.rs)."""

    def __init__(self, cx: Complex, lengths: np.ndarray, relative: bool = False):
        self.cx = cx
        self.lengths = np.ascontiguousarray(lengths, np.float64)
        self.relative = relative

    @property
    def dim(self):
        return self.cx.dim

    def ndofs(self, k: int) -> int:
        if k < 0 or k > self.dim:
            return 0
        return len(self.cx.interior(k)) if self.relative else self.cx.nsimplices(k)

    def _pairing(self, form: int, k: int) -> sp.csr_matrix:
        tg = k - 1 if form in (DIF_TEST, DIF_BOTH) else k
        sg = k - 1 if form in (DIF_TRIAL, DIF_BOTH) else k
        r, c = self.ndofs(tg), self.ndofs(sg)
        if r == 0 or c == 0:
            return sp.csr_matrix((r, c))
        return _csr_from_handle(lib().or_assemble(self.cx.handle, self.lengths, form, k, int(self.relative)))

    def mass(self, k):
        return self._pairing(MASS, k)

    def dif_trial(self, k):
        return self._pairing(DIF_TRIAL, k)

    def dif_test(self, k):
        return self._pairing(DIF_TEST, k)

    def dif_both(self, k):
        return self._pairing(DIF_BOTH, k)

    def hdif_gram(self, k):
        """M_k + dif_both(k+1) (whitney_complex.rs:180-183), union pattern."""
        return csr_add(self.mass(k), self.dif_both(k + 1))

    def dif(self, k):
        """Coboundary (whitney_complex.rs:417-423; relative :640-643)."""
        if k < 0 or k > self.dim:
            return sp.csr_matrix((self.ndofs(k + 1), self.ndofs(k)))
        return _csr_from_handle(lib().or_coboundary(self.cx.handle, k, int(self.relative)))

    def inclusion(self, k):
        n = self.cx.nsimplices(k) if 0 <= k <= self.dim else 0
        if not self.relative:
            return sp.identity(n, format="csr")
        keep = self.cx.interior(k) if 0 <= k <= self.dim else np.zeros(0, np.int64)
        return sp.csr_matrix((np.ones(len(keep)), (keep, np.arange(len(keep)))), shape=(n, len(keep)))


def csr_add(a: sp.csr_matrix, b: sp.csr_matrix) -> sp.csr_matrix:
    """nalgebra-sparse CSR + CSR: union pattern, no zero dropping."""
    ca, cb = a.tocoo(), b.tocoo()
    rows = np.concatenate([ca.row, cb.row])
    cols = np.concatenate([ca.col, cb.col])
    vals = np.concatenate([ca.data, cb.data])
    return coo_to_csr(rows, cols, vals, a.shape)


def coo_to_csr(rows, cols, vals, shape) -> sp.csr_matrix:
    """Sorted columns, duplicates summed in input order, explicit zeros kept."""
    rows = np.asarray(rows, np.int64)
    cols = np.asarray(cols, np.int64)
    vals = np.asarray(vals, np.float64)
    order = np.lexsort((np.arange(len(rows)), cols, rows))
    r, c, v = rows[order], cols[order], vals[order]
    if len(r):
        new = np.ones(len(r), bool)
        new[1:] = (r[1:] != r[:-1]) | (c[1:] != c[:-1])
        seg = np.cumsum(new) - 1
        nslot = seg[-1] + 1
        sv = np.zeros(nslot)
        np.add.at(sv, seg, v)  # unbuffered: duplicates summed in input order
        rr, cc = r[new], c[new]
    else:
        sv = np.zeros(0)
        rr = cc = np.zeros(0, np.int64)
    rp = np.zeros(shape[0] + 1, np.int64)
    np.add.at(rp, rr + 1, 1)
    rp = np.cumsum(rp)
    m = sp.csr_matrix((sv, cc, rp), shape=shape)
    m.has_sorted_indices = True
    return m


# ---------------------------------------------------------------------------
# Mixed Hodge-Laplace (formoniq/src/hodge.rs:36-99, problems/elliptic.rs:29-182)
# ---------------------------------------------------------------------------

def harmonics(wc: WhitneyComplex, k: int) -> np.ndarray:
    """M_k-orthonormal harmonic basis for the cases a Kuhn cube has
    (elliptic.rs:197-220, harmonic.rs): b_0 = 1 on the full complex (constants),
    b_n = 1 on the relative complex (h proportional to M_n^{-1} z, z the coherent
    orientation, dirac.rs:553-568); every other Betti number of a cube is 0."""
    n = wc.dim
    if not wc.relative and k == 0:
        m0 = wc.mass(0)
        one = np.ones(wc.ndofs(0))
        return (one / math.sqrt(one @ (m0 @ one)))[:, None]
    if wc.relative and k == n and n >= 1:
        z = orientation_signs(wc.cx)
        mn = wc.mass(n).tocsc()
        h = spla.spsolve(mn, z)
        return (h / math.sqrt(h @ (mn @ h)))[:, None]
    if wc.relative and k == n and n == 0:
        return np.ones((wc.ndofs(0), 1)) / math.sqrt(wc.mass(0)[0, 0])
    return np.zeros((wc.ndofs(k), 0))


def orientation_signs(cx: Complex) -> np.ndarray:
    """A coherent orientation of the cells (topology/orientation.rs): adjacent
    cells induce opposite signs on their shared facet. Fixed so cell 0 is +1."""
    n = cx.dim
    cells = cx.simplices(n)
    ncell = len(cells)
    fac = cx.cell_faces(n - 1)  # local facet l = cell minus vertex (n - l) in colex order
    # local facet index l (colex) omits vertex position n-l; boundary sign (-1)^p
    nloc = n + 1
    sign_of_local = np.array([(-1.0) ** (n - l) for l in range(nloc)])
    owner = {}
    adj = [[] for _ in range(ncell)]
    for c in range(ncell):
        for l in range(nloc):
            f = int(fac[c, l])
            if f in owner:
                oc, ol = owner[f]
                adj[c].append((oc, l, ol))
                adj[oc].append((c, ol, l))
            else:
                owner[f] = (c, l)
    sgn = np.zeros(ncell)
    sgn[0] = 1.0
    stack = [0]
    while stack:
        c = stack.pop()
        for (o, lc, lo) in adj[c]:
            want = -sgn[c] * sign_of_local[lc] * sign_of_local[lo]
            if sgn[o] == 0:
                sgn[o] = want
                stack.append(o)
    return sgn


def assemble_mixed_kkt(wc: WhitneyComplex, source: np.ndarray, k: int, harm: np.ndarray):
    """assemble_mixed_kkt (elliptic.rs:54-114): [[-M_{k-1}, B, 0], [B^T, K, M_k H],
    [0, (M_k H)^T, 0]] with B = dif_test(k), K = dif_both(k+1); rhs [0; E^T f; 0]."""
    ms = wc.mass(k - 1)
    mu = wc.mass(k)
    b = wc.dif_test(k)
    kk = wc.dif_both(k + 1)
    ns, nu = wc.ndofs(k - 1), wc.ndofs(k)
    nh = harm.shape[1]
    mh = mu @ harm if nh else np.zeros((nu, 0))
    rows, cols, vals = [], [], []

    def put(m, ro, co, scale=1.0):
        c = sp.coo_matrix(m)
        rows.append(c.row + ro)
        cols.append(c.col + co)
        vals.append(scale * c.data)

    put(ms, 0, 0)
    put(b, 0, ns, -1.0)
    put(b.T.tocsr(), ns, 0)
    put(kk, ns, ns)
    if nh:
        r, c = np.meshgrid(np.arange(nu), np.arange(nh), indexing="ij")
        rows.append(r.ravel() + ns)
        cols.append(c.ravel() + ns + nu)
        vals.append(mh.ravel())
        rows.append(c.ravel() + ns + nu)
        cols.append(r.ravel() + ns)
        vals.append(mh.ravel())
    ntot = ns + nu + nh
    a = coo_to_csr(np.concatenate(rows) if rows else [], np.concatenate(cols) if cols else [],
                   np.concatenate(vals) if vals else [], (ntot, ntot))
    # sign flip of the sigma rows (elliptic.rs:102-113): an exact negation of the
    # stored values of rows < ns, pattern and column order unchanged
    sign = np.ones(ntot)
    sign[:ns] = -1.0
    a = a.copy()
    a.data = a.data * np.repeat(sign, np.diff(a.indptr))
    src = wc.inclusion(k).T @ source
    rhs = np.concatenate([np.zeros(ns), src, np.zeros(nh)])
    return a, sign * rhs, ns, nu


def direct_solve(a: sp.csr_matrix, b: np.ndarray) -> np.ndarray:
    """The faer sparse LU stand-in: SciPy SuperLU on the identical CSR."""
    if a.shape[0] == 0:
        return np.zeros(0)
    return spla.splu(sp.csc_matrix(a)).solve(b)


class BlockDiagonal:
    """iterative/src/precond.rs:138-167 with exact (SuperLU) blocks."""

    def __init__(self, blocks):
        self.blocks = blocks
        self.sizes = [blk.shape[0] for blk in blocks]
        self.solvers = [spla.splu(sp.csc_matrix(blk)) if blk.shape[0] else None for blk in blocks]

    def __call__(self, r):
        out = np.empty_like(r)
        o = 0
        for s, d in zip(self.solvers, self.sizes):
            out[o:o + d] = s.solve(r[o:o + d]) if d else r[o:o + d]
            o += d
        return out


def jacobi(diag: np.ndarray):
    inv = 1.0 / diag
    return lambda r: r * inv


def mixed_block_preconditioner_diag(wc: WhitneyComplex, k: int, nh: int) -> np.ndarray:
    """Diagonal of the blocks of mixed_block_preconditioner (elliptic.rs:29-47)."""
    parts = []
    if k > 0:
        parts.append(wc.hdif_gram(k - 1).diagonal())
    parts.append(wc.hdif_gram(k).diagonal())
    parts.append(np.ones(nh))
    return np.concatenate(parts)


@dataclass
class Report:
    iters: int
    residual: float
    converged: bool


def minres(a, precond, b, rtol=1e-10, max_iters=10_000):
    """Preconditioned Paige-Saunders MINRES, krylov.rs:113-211, verbatim recurrences."""
    eps = np.finfo(np.float64).eps
    apply = (lambda v: a @ v) if not callable(a) else a
    r1 = b.copy()
    y = precond(r1)
    beta1_sq = float(r1 @ y)
    if beta1_sq <= 0.0:
        return np.zeros_like(b), Report(0, 0.0, True)
    x = np.zeros_like(b)
    beta1 = math.sqrt(beta1_sq)
    oldb, beta, dbar, epsln, phibar = 0.0, beta1, 0.0, 0.0, beta1
    cs, sn = -1.0, 0.0
    w = np.zeros_like(b)
    w2 = np.zeros_like(b)
    r2 = r1.copy()
    residual, converged, iters = 1.0, False, 0
    while iters < max_iters:
        iters += 1
        v = y * (1.0 / beta)
        y_next = apply(v)
        if iters >= 2:
            y_next = y_next + (-beta / oldb) * r1
        alfa = float(v @ y_next)
        y_next = y_next + (-alfa / beta) * r2
        r1 = r2
        r2 = y_next
        y = precond(r2)
        oldb = beta
        beta = math.sqrt(max(float(r2 @ y), 0.0))
        oldeps = epsln
        delta = cs * dbar + sn * alfa
        gbar = sn * dbar - cs * alfa
        epsln = sn * beta
        dbar = -cs * beta
        gamma = max(math.sqrt(gbar * gbar + beta * beta), eps)
        cs = gbar / gamma
        sn = beta / gamma
        phi = cs * phibar
        phibar *= sn
        wnew = v + (-oldeps) * w2
        wnew = wnew + (-delta) * w
        wnew = wnew * (1.0 / gamma)
        w2 = w
        w = wnew
        x = x + phi * w
        residual = phibar / beta1
        if residual <= rtol:
            converged = True
            break
    return x, Report(iters, residual, converged)


def cg(a, precond, b, rtol=1e-10, max_iters=10_000):
    """Preconditioned CG, krylov.rs:48-95."""
    apply = (lambda v: a @ v) if not callable(a) else a
    b_norm = float(np.linalg.norm(b))
    if b_norm == 0.0:
        return np.zeros_like(b), Report(0, 0.0, True)
    x = np.zeros_like(b)
    r = b.copy()
    z = precond(r)
    p = z.copy()
    rz = float(r @ z)
    iters = 0
    while True:
        residual = float(np.linalg.norm(r)) / b_norm
        converged = residual <= rtol
        if converged or iters >= max_iters:
            break
        ap = apply(p)
        alpha = rz / float(p @ ap)
        x = x + alpha * p
        r = r + (-alpha) * ap
        z = precond(r)
        rz_next = float(r @ z)
        beta = rz_next / rz
        p = p * beta + z
        rz = rz_next
        iters += 1
    return x, Report(iters, residual, converged)


def solve_source(wc: WhitneyComplex, source: np.ndarray, k: int, rtol=1e-10):
    """solve_source (elliptic.rs:132-182) with the exact block preconditioner
    (SuperLU blocks standing in for faer Cholesky) and the LU fallback."""
    harm = harmonics(wc, k)
    a, rhs, ns, nu = assemble_mixed_kkt(wc, source, k, harm)
    blocks = []
    if k > 0:
        blocks.append(wc.hdif_gram(k - 1))
    blocks.append(wc.hdif_gram(k))
    if harm.shape[1]:
        blocks.append(sp.identity(harm.shape[1], format="csr"))
    sol, rep = minres(a, BlockDiagonal(blocks), rhs, rtol)
    if not rep.converged:
        sol = direct_solve(a, rhs)
    sigma = sol[:ns]
    u = sol[ns:ns + nu]
    p = sol[ns + nu:]
    if k > 0:
        sigma = wc.inclusion(k - 1) @ sigma
    u = wc.inclusion(k) @ u
    return sigma, u, p, rep


# ---------------------------------------------------------------------------
# Hodge-Dirac (formoniq/src/problems/dirac.rs:181-260, 473-531)
# ---------------------------------------------------------------------------

def dirac_selfadjoint(full: WhitneyComplex):
    """HodgeDirac::assemble_signed(+1): block-diagonal mass M and the
    block-tridiagonal A with U_k = M_k D_{k-1} (global product) below and U_k^T
    above. Returns (offsets, M, A)."""
    return dirac_signed(full, 1.0)


def dirac_signed(full: WhitneyComplex, delta_sign: float):
    """HodgeDirac::assemble_signed (dirac.rs:213-260): the super-diagonal block is
    delta_sign U_k^T (-1: the skew evolution generator dif - delta)."""
    n = full.dim
    masses = [full.mass(k) for k in range(n + 1)]
    difs = [full.dif(k) for k in range(n)]
    offsets = np.concatenate([[0], np.cumsum([m.shape[0] for m in masses])]).astype(np.int64)
    tot = int(offsets[-1])
    mr, mc, mv = [], [], []
    for k, m in enumerate(masses):
        c = m.tocoo()
        mr.append(c.row + offsets[k])
        mc.append(c.col + offsets[k])
        mv.append(c.data)
    mb = coo_to_csr(np.concatenate(mr), np.concatenate(mc), np.concatenate(mv), (tot, tot))
    ar, ac, av = [], [], []
    for k in range(1, n + 1):
        u = spgemm(masses[k], difs[k - 1]).tocoo()
        row, col = offsets[k], offsets[k - 1]
        # interleave (r,c) and (c,r) pushes as the reference does
        ar.append(np.stack([row + u.row, col + u.col], 1).ravel())
        ac.append(np.stack([col + u.col, row + u.row], 1).ravel())
        av.append(np.stack([u.data, delta_sign * u.data], 1).ravel())
    a = coo_to_csr(np.concatenate(ar) if ar else [], np.concatenate(ac) if ac else [],
                   np.concatenate(av) if av else [], (tot, tot))
    return offsets, mb, a


def spgemm(a: sp.csr_matrix, b: sp.csr_matrix) -> sp.csr_matrix:
    """Sparse product with the symbolic pattern kept (no zero dropping)."""
    a = sp.csr_matrix(a)
    b = sp.csr_matrix(b)
    rows, cols, vals = [], [], []
    for i in range(a.shape[0]):
        acc = {}
        for t in range(a.indptr[i], a.indptr[i + 1]):
            kk, av = a.indices[t], a.data[t]
            for s in range(b.indptr[kk], b.indptr[kk + 1]):
                j = b.indices[s]
                acc[j] = acc.get(j, 0.0) + av * b.data[s]
        for j in sorted(acc):
            rows.append(i)
            cols.append(j)
            vals.append(acc[j])
    return coo_to_csr(rows, cols, vals, (a.shape[0], b.shape[1]))


def dirac_source_system(cx: Complex, lengths: np.ndarray, mass_term: float, load: np.ndarray,
                        lift: np.ndarray):
    """solve_dirac_source (dirac.rs:473-531) up to the solve: S = A + mM on the full
    space, restricted to the relative DOFs; rhs = E^T (load - S lift)."""
    full = WhitneyComplex(cx, lengths, relative=False)
    offsets, mb, a = dirac_selfadjoint(full)
    s = csr_add(a, mass_term * mb) if mass_term != 0.0 else a
    keep = np.concatenate([cx.interior(k) + offsets[k] for k in range(cx.dim + 1)])
    e = sp.csr_matrix((np.ones(len(keep)), (keep, np.arange(len(keep)))), shape=(int(offsets[-1]), len(keep)))
    rhs = e.T @ (load - s @ lift)
    # E^T S E: keep interior rows and columns, renumbered (explicit entries kept)
    newidx = -np.ones(int(offsets[-1]), np.int64)
    newidx[keep] = np.arange(len(keep))
    c = s.tocoo()
    sel = (newidx[c.row] >= 0) & (newidx[c.col] >= 0)
    s_rel = coo_to_csr(newidx[c.row[sel]], newidx[c.col[sel]], c.data[sel], (len(keep), len(keep)))
    return s_rel, rhs, keep, offsets


def top_harmonic(cx: Complex, lengths: np.ndarray) -> np.ndarray:
    """top_harmonic (dirac.rs:552-570): zero below the top grade, M_n^-1 z on
    the cells (relative top-grade mass, z the coherent orientation), in the flat
    relative layout."""
    rel = WhitneyComplex(cx, lengths, relative=True)
    n = cx.dim
    z = orientation_signs(cx).astype(np.float64)
    h_n = direct_solve(rel.mass(n), z)
    sizes = [len(cx.interior(k)) for k in range(n + 1)]
    h = np.zeros(sum(sizes))
    h[sum(sizes[:n]):] = h_n
    return h


def solve_bordered(s: sp.csr_matrix, rhs: np.ndarray, h: np.ndarray) -> np.ndarray:
    """solve_bordered (dirac.rs:578-598): [[S, h], [h^T, 0]] [u; c] = [f; 0] by LU."""
    n = len(rhs)
    c = s.tocoo()
    nzh = np.nonzero(h != 0.0)[0]
    rows = np.concatenate([c.row, nzh, np.full(len(nzh), n)])
    cols = np.concatenate([c.col, np.full(len(nzh), n), nzh])
    vals = np.concatenate([c.data, h[nzh], h[nzh]])
    b = coo_to_csr(rows, cols, vals, (n + 1, n + 1))
    return direct_solve(b, np.concatenate([rhs, [0.0]]))[:n]


def dirac_solve_source(cx, lengths, mass_term, load, lift):
    """solve_dirac_source (dirac.rs:473-531): LU of the relative system, bordered
    with the top harmonic at m = 0 when it spans the kernel."""
    s_rel, rhs, keep, offsets = dirac_source_system(cx, lengths, mass_term, load, lift)
    interior = None
    if mass_term == 0.0:
        h = top_harmonic(cx, lengths)
        if np.linalg.norm(s_rel @ h) <= 1e-8 * np.linalg.norm(h):
            interior = solve_bordered(s_rel, rhs, h)
    if interior is None:
        interior = direct_solve(s_rel, rhs)
    out = lift.copy()
    out[keep] += interior
    return out


# ---------------------------------------------------------------------------
# The de Rham map (derham/src/project.rs:53-96) with the Grundmann-Moeller rule
# (simplicial/src/atlas/quadrature.rs:38-82)
# ---------------------------------------------------------------------------

def gm_rule(k: int, degree: int):
    """SimplexQuadRule::degree(k, degree): the Grundmann-Moeller rule of index
    s = degree // 2 on the k-simplex, barycentric points [nq, k+1] and weights
    normalised to sum 1."""
    s = degree // 2
    d = 2 * s + 1
    pts, w = [], []

    def compositions(parts, total):
        if parts == 1:
            yield (total,)
            return
        for b in range(total, -1, -1):
            for rest in compositions(parts - 1, total - b):
                yield (b,) + rest

    for i in range(s + 1):
        den = d + k - 2 * i
        wi = (-1) ** i * 2.0 ** (-2 * s) * float(den) ** d / (math.factorial(i) * math.factorial(d + k - i))
        for beta in compositions(k + 1, s - i):
            pts.append([(2 * b + 1) / den for b in beta])
            w.append(wi)
    w = np.array(w)
    return np.array(pts, np.float64).reshape(len(w), k + 1), w / w.sum()


def colex_subsets(n: int, k: int):
    """k-subsets of range(n) in colex order (compare from the largest element)."""
    return sorted(itertools.combinations(range(n), k), key=lambda c: c[::-1])


def derham_map(cx: Complex, coords: np.ndarray, k: int, field, degree: int = 3) -> np.ndarray:
    """derham_map (project.rs:53-69) + integrate_face (:77-96) for an ambient
    form: (R w)_s = (1/k!) sum_q w_q <w(x_q), v_1 ^ ... ^ v_k>, v_i = x_{s_i} - x_{s_0}.
    `field` maps nodes [m, adim] to components [m, C(adim, k)] on dx^I, I colex."""
    simp = cx.simplices(k)
    adim = coords.shape[1]
    bary, w = gm_rule(k, degree)
    x = coords[simp]  # [ns, k+1, adim]
    nodes = np.einsum("qi,sia->sqa", bary, x)
    vals = np.asarray(field(nodes.reshape(-1, adim)), np.float64).reshape(len(simp), len(w), -1)
    subs = colex_subsets(adim, k)
    if k == 0:
        blade = np.ones((len(simp), 1))
    else:
        v = x[:, 1:, :] - x[:, :1, :]  # [ns, k, adim]
        blade = np.stack([np.linalg.det(v[:, :, list(I)]) for I in subs], axis=1)
    return np.einsum("q,sqc,sc->s", w, vals, blade) / math.factorial(k)


# ---------------------------------------------------------------------------
# The source load: SourceForm::element (formoniq/src/operators.rs:598-635)
# summed by assemble_vector (formoniq/src/galerkin.rs:279-312)
# ---------------------------------------------------------------------------

def _subset_dets(mats: np.ndarray, rows, cols) -> np.ndarray:
    """det of mats[..., R, C] for every R in rows, C in cols: [..., len(rows), len(cols)]."""
    out = np.empty(mats.shape[:-2] + (len(rows), len(cols)))
    for i, r in enumerate(rows):
        for j, c in enumerate(cols):
            out[..., i, j] = np.linalg.det(mats[..., list(r), :][..., :, list(c)]) if len(r) else 1.0
    return out


def whitney_at(n: int, k: int, bary: np.ndarray) -> np.ndarray:
    """WhitneyLsf::at_bary (derham/src/interpolate/form.rs:108-112) for every
    local k-face s (colex (k+1)-subsets of {0..n}) at barycentric nodes [nq, n+1]:
    W_s = k! sum_p (-1)^p lambda_{s_p} dlambda_{s without s_p}, with dlambda from
    unit_difbarys (simplicial/src/atlas.rs:174-182), as components on dxi^J
    (J colex k-subsets of {0..n-1}): [nq, C(n+1,k+1), C(n,k)]."""
    L = np.zeros((n + 1, n))
    L[0, :] = -1.0
    L[1:, :] = np.eye(n)
    taus = colex_subsets(n + 1, k)
    D = _subset_dets(L, taus, colex_subsets(n, k))  # Lambda^k L
    rank = {t: i for i, t in enumerate(taus)}
    faces = colex_subsets(n + 1, k + 1)
    W = np.zeros((len(bary), len(faces), D.shape[1]))
    for si, s in enumerate(faces):
        for p, v in enumerate(s):
            W[:, si, :] += (-1) ** p * np.outer(bary[:, v], D[rank[s[:p] + s[p + 1:]]])
    return math.factorial(k) * W


def pullback_values(cx: Complex, coords: np.ndarray, k: int, values: np.ndarray) -> np.ndarray:
    """Pullback::identity (derham/src/section.rs:95-140) of a flat ambient form:
    components on dx^A [ncells, nq, C(adim,k)] -> the cells' reference frames
    [ncells, nq, C(n,k)], f_J = sum_A w_A det(E[A, J]), E = [x_{v_j} - x_{v_0}]."""
    n = cx.dim
    cells = cx.simplices(n)
    adim = coords.shape[1]
    E = np.transpose(coords[cells[:, 1:]] - coords[cells[:, :1]], (0, 2, 1))  # [nc, adim, n]
    P = _subset_dets(E, colex_subsets(adim, k), colex_subsets(n, k))  # [nc, C(adim,k), C(n,k)]
    return np.einsum("cqa,caj->cqj", values, P)


def whitney_interpolant_values(cx: Complex, k: int, cochain: np.ndarray, bary: np.ndarray) -> np.ndarray:
    """WhitneyInterpolant of a cochain (derham/src/interpolate/interpolant.rs) at
    the barycentric nodes of every cell, in the cells' reference frames:
    [ncells, nq, C(n,k)]."""
    W = whitney_at(cx.dim, k, bary)
    return np.einsum("cs,qsj->cqj", cochain[cx.cell_faces(k)], W)


def source_form(cx: Complex, lengths: np.ndarray, k: int, values: np.ndarray, degree: int = 1,
                coords: np.ndarray | None = None, relative: bool = False) -> np.ndarray:
    """SourceForm::new(source, qr).assemble(topology, lengths): per cell
    vol sum_q w_q <f_q, W_s(x_q)>_{Lambda^k G^{-1}} (CellQuadrature::integrate,
    operators.rs:246-261; inner, metric/src/tensor.rs:140-155, with the induced
    form multiform_metric, :127-131), summed per face in cell order
    (galerkin.rs:292-311). values: [ncells, nq, C(n,k)] in the cells' reference
    frames, or a flat ambient form's [ncells, nq, C(adim,k)] when coords is given."""
    n = cx.dim
    bary, w = gm_rule(n, degree)
    values = np.asarray(values, np.float64).reshape(cx.ncells(), len(w), -1)
    if coords is not None:
        values = pullback_values(cx, coords, k, values)
    W = whitney_at(n, k, bary)
    _, gi, _, vol, _ = cx.cell_metrics(lengths)
    Js = colex_subsets(n, k)
    lg = _subset_dets(gi, Js, Js)  # Lambda^k G^{-1} per cell
    elvec = vol[:, None] * np.einsum("q,cqi,cij,qsj->cs", w, values, lg, W)
    out = np.zeros(cx.nsimplices(k))
    np.add.at(out, cx.cell_faces(k).ravel(), elvec.ravel())
    return out[cx.interior(k)] if relative else out


# ---------------------------------------------------------------------------
# Maxwell evolution: time::Leapfrog (formoniq/src/time.rs:292-420) as used by
# solve_dirac_leapfrog (problems/dirac.rs:404-434)
# ---------------------------------------------------------------------------

def grade_parity_coloring(offsets: np.ndarray) -> np.ndarray:
    """HodgeDirac::grade_parity_coloring (dirac.rs:337-349): True on odd grades."""
    color = np.zeros(int(offsets[-1]), bool)
    for k in range(1, len(offsets) - 1, 2):
        color[offsets[k]:offsets[k + 1]] = True
    return color


class Leapfrog:
    """Leapfrog::new / step / conserved_energy with exact block solves."""

    def __init__(self, mass: sp.csr_matrix, op: sp.csr_matrix, color: np.ndarray, dt: float):
        self.idx0 = np.flatnonzero(~color)
        self.idx1 = np.flatnonzero(color)
        m = sp.csr_matrix(mass)
        a = sp.csr_matrix(op)
        self.mass0 = m[self.idx0][:, self.idx0].tocsc()
        self.mass1 = m[self.idx1][:, self.idx1].tocsc()
        self.a01 = a[self.idx0][:, self.idx1].tocsr()
        self.a10 = a[self.idx1][:, self.idx0].tocsr()
        self.lu0 = spla.splu(self.mass0) if self.mass0.shape[0] else None
        self.lu1 = spla.splu(self.mass1) if self.mass1.shape[0] else None
        self.dt = dt
        self.n = m.shape[0]

    def _solve(self, lu, r):
        return lu.solve(r) if lu is not None else r

    def step(self, y0: np.ndarray) -> np.ndarray:
        q = y0[self.idx0].copy()
        p = y0[self.idx1].copy()
        p += 0.5 * self.dt * self._solve(self.lu1, self.a10 @ q)
        q += self.dt * self._solve(self.lu0, self.a01 @ p)
        p += 0.5 * self.dt * self._solve(self.lu1, self.a10 @ q)
        y1 = np.zeros(self.n)
        y1[self.idx0] = q
        y1[self.idx1] = p
        return y1

    def conserved_energy(self, y: np.ndarray) -> float:
        q, p = y[self.idx0], y[self.idx1]
        a10q = self.a10 @ q
        defect = a10q @ self._solve(self.lu1, a10q)
        return 0.5 * q @ (self.mass0 @ q) + 0.5 * p @ (self.mass1 @ p) - self.dt ** 2 / 8.0 * defect


def leapfrog_for(wc: WhitneyComplex, dt: float):
    """solve_dirac_leapfrog's set-up on a (full or relative) complex: returns
    (offsets, mass block, Leapfrog)."""
    offsets, mb, a = dirac_signed(wc, -1.0)
    return offsets, mb, Leapfrog(mb, a, grade_parity_coloring(offsets), dt)
