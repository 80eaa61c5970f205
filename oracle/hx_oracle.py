"""CPU restatement of the HX-multigrid preconditioner (test infrastructure only).

This is the test oracle of the device preconditioner behind fq_hx_apply / fq_hx_cg and
of the mixed solve's HX blocks; nothing in the product imports it.

What it restates, and from where:
  - the additive auxiliary-space preconditioner B = S + sum_c Pi_c B_c Pi_c^T
    (iterative/src/aux_space.rs:AuxiliarySpace::apply) with the FEEC wiring of
    formoniq/src/hx.rs:hx_preconditioner: smoother S_j = Jacobi::smoother(A_j)
    (weight 2/3, iterative/src/precond.rs:89-94), gradient correction through
    D_{j-1} with the grade-(j-1) preconditioner (MultigridBlocks::gradient), and
    the vector-nodal correction through Pi_j with C(n, j) nodal V-cycles
    (vector_nodal_prolongation, ReplicatedBlock);
  - the V-cycle of iterative/src/multigrid.rs:VCycle::cycle (pre-smoothing from
    zero, restriction by P^T, recursive correction, post-smoothing; exact solve on
    the coarsest level) with Galerkin coarse operators P^T A P
    (formoniq/src/multigrid.rs, "coarse operators are formed by the Galerkin
    triple product").
Two ingredients are this project's, not the reference's, because a mesh on the
device carries lengths and no coordinates or refinement tower: the levels come
from coarsening a Kuhn lattice (N -> ceil(N/2), piecewise-linear interpolation at
the fine lattice points), and Pi_j reads its frame off the lattice scaled by the
root mean squared axis-edge length. They are restated here exactly as the device
builds them, so this module pins the device preconditioner; it does not pin the
reference's own tower or embedding (parity unpinned for those two choices).
"""
from __future__ import annotations

import itertools
import math

import numpy as np
import scipy.sparse as sp

OMEGA = 2.0 / 3.0
COARSE_MAX = 256


def level_nodes(n: int, nbox: int, relative: bool) -> int:
    return max(nbox - 1, 0) ** n if relative else (nbox + 1) ** n


def node_index(c, n: int, nbox: int, relative: bool) -> int:
    idx, stride = 0, 1
    for a in range(n):
        if relative:
            if c[a] <= 0 or c[a] >= nbox:
                return -1
            idx += (c[a] - 1) * stride
            stride *= nbox - 1
        else:
            idx += c[a] * stride
            stride *= nbox + 1
    return idx


def lattice_coords(v: int, n: int, nbox: int):
    c = []
    for _ in range(n):
        c.append(v % (nbox + 1))
        v //= nbox + 1
    return c


def lattice_prolongation(n: int, nf: int, nc: int, relative: bool) -> sp.csr_matrix:
    """Interpolation of the nc-lattice's piecewise-linear functions at the nf lattice points."""
    rows, cols, vals = [], [], []
    for v in range((nf + 1) ** n):
        c = lattice_coords(v, n, nf)
        row = node_index(c, n, nf, relative)
        if row < 0:
            continue
        b, rho = [], []
        for a in range(n):
            y = c[a] * nc
            bb, rr = divmod(y, nf)
            if bb >= nc:
                bb, rr = nc - 1, nf
            b.append(bb)
            rho.append(rr)
        order = sorted(range(n), key=lambda a: -rho[a])  # stable: ties keep axis order
        w = list(b)
        for i in range(n + 1):
            if i > 0:
                w[order[i - 1]] += 1
            hi = nf if i == 0 else rho[order[i - 1]]
            lo = 0 if i == n else rho[order[i]]
            lam = (hi - lo) / nf
            if lam == 0.0:
                continue
            col = node_index(w, n, nc, relative)
            if col < 0:
                continue
            rows.append(row)
            cols.append(col)
            vals.append(lam)
    return sp.csr_matrix((vals, (rows, cols)), shape=(level_nodes(n, nf, relative), level_nodes(n, nc, relative)))


class NodalMultigrid:
    """The nodal V-cycle over the coarsened Kuhn lattices."""

    def __init__(self, a0: sp.csr_matrix, n: int, nbox: int, relative: bool, sweeps: int = 2):
        boxes = [nbox]
        while level_nodes(n, boxes[-1], relative) > COARSE_MAX and boxes[-1] > 2:
            boxes.append((boxes[-1] + 1) // 2)
        self.sweeps = sweeps
        self.A = [sp.csr_matrix(a0)]
        self.P = []
        for lvl in range(len(boxes) - 1):
            P = lattice_prolongation(n, boxes[lvl], boxes[lvl + 1], relative)
            self.P.append(P)
            self.A.append(sp.csr_matrix(P.T @ self.A[-1] @ P))
        self.dinv = [OMEGA / a.diagonal() for a in self.A]
        ac = self.A[-1].toarray()
        self.coarse_inv = np.linalg.inv(ac) if ac.size else ac

    def cycle(self, lvl: int, r: np.ndarray) -> np.ndarray:
        if lvl == len(self.A) - 1:
            return self.coarse_inv @ r
        A, d = self.A[lvl], self.dinv[lvl][:, None]
        x = np.zeros_like(r)
        for _ in range(self.sweeps):
            x = x + d * (r - A @ x)
        res = r - A @ x
        x = x + self.P[lvl] @ self.cycle(lvl + 1, self.P[lvl].T @ res)
        for _ in range(self.sweeps):
            x = x + d * (r - A @ x)
        return x

    def apply(self, r: np.ndarray) -> np.ndarray:
        return self.cycle(0, r)


def lattice_spacing(cx, lengths: np.ndarray, n: int, nbox: int) -> np.ndarray:
    """Per axis, the root mean squared length of the single-axis edges
    (v, v + (N+1)^a), averaged in increasing v."""
    edges = np.asarray(cx.simplices(1), np.int64)
    nv = (nbox + 1) ** n
    keys = edges[:, 0] * nv + edges[:, 1]
    order = np.argsort(keys, kind="stable")
    v = np.arange(nv, dtype=np.int64)
    h = np.zeros(n)
    for a in range(n):
        stride = (nbox + 1) ** a
        vv = v[(v // stride) % (nbox + 1) < nbox]
        want = vv * nv + vv + stride
        idx = order[np.searchsorted(keys, want, sorter=order)]
        h[a] = math.sqrt(float(np.mean(lengths[idx])))
    return h


def colex_subsets(n: int, j: int):
    subs = [list(s) for s in itertools.combinations(range(n), j)]
    return sorted(subs, key=lambda s: tuple(reversed(s)))


def vector_nodal(cx, j: int, n: int, nbox: int, relative: bool, h: np.ndarray) -> sp.csr_matrix:
    """Pi_j: rows the grade-j unknowns, columns (node, I) node-major. Entry
    (s, (node(v), I)) = det(E_s[I, :]) / (j+1)! for every vertex v of s, with E_s
    the lattice edge vectors (scaled per axis by h) from the first vertex of s."""
    ncomp = 1 if j == 0 else math.comb(n, j)
    n0 = level_nodes(n, nbox, relative)
    simp = np.asarray(cx.simplices(j), np.int64)
    keep = np.arange(len(simp)) if not relative else np.asarray(cx.interior(j), np.int64)
    verts = simp[keep]                                       # [m, j+1]
    m = len(keep)
    lat = np.stack([(verts // (nbox + 1) ** a) % (nbox + 1) for a in range(n)], -1)  # [m, j+1, n]
    factor = 1.0 / math.factorial(j + 1)
    if j == 0:
        comp = np.ones((m, 1))
    else:
        E = np.transpose((lat[:, 1:, :] - lat[:, :1, :]) * h, (0, 2, 1))  # [m, n, j]
        comp = np.stack([np.linalg.det(E[:, sub, :]) for sub in colex_subsets(n, j)], 1)  # [m, ncomp]
    if relative:
        inside = np.all((lat > 0) & (lat < nbox), -1)            # [m, j+1]
        node = np.zeros(lat.shape[:2], np.int64)
        stride = 1
        for a in range(n):
            node += (lat[:, :, a] - 1) * stride
            stride *= nbox - 1
        node[~inside] = -1
    else:
        node = verts
    rows = np.repeat(np.arange(m), (j + 1) * ncomp).reshape(m, j + 1, ncomp)
    cols = node[:, :, None] * ncomp + np.arange(ncomp)[None, None, :]
    vals = np.broadcast_to((factor * comp)[:, None, :], (m, j + 1, ncomp))
    ok = (node[:, :, None] >= 0) & (vals != 0.0)
    return sp.csr_matrix((vals[ok], (rows[ok], cols[ok])), shape=(m, n0 * ncomp))


class HxPreconditioner:
    """B_j = S_j + D_{j-1} B_{j-1} D_{j-1}^T + Pi_j V^{C(n,j)} Pi_j^T, B_0 = S_0 + V."""

    def __init__(self, wc, cx, lengths: np.ndarray, nbox: int, relative: bool):
        self.wc, self.n, self.nbox, self.relative = wc, cx.dim, nbox, relative
        self.mg = NodalMultigrid(wc.hdif_gram(0), cx.dim, nbox, relative)
        self.h = lattice_spacing(cx, lengths, cx.dim, nbox)
        self.cx = cx
        self._pi = {}
        self._s = {}
        self._d = {}

    def smoother(self, j: int) -> np.ndarray:
        if j not in self._s:
            self._s[j] = OMEGA / self.wc.hdif_gram(j).diagonal()
        return self._s[j]

    def pi(self, j: int) -> sp.csr_matrix:
        if j not in self._pi:
            self._pi[j] = vector_nodal(self.cx, j, self.n, self.nbox, self.relative, self.h)
        return self._pi[j]

    def nodal(self, j: int, r: np.ndarray) -> np.ndarray:
        """Pi_j V^{C(n,j)} Pi_j^T r (the copies share one V-cycle)."""
        ncomp = 1 if j == 0 else math.comb(self.n, j)
        pi = self.pi(j)
        z = (pi.T @ r).reshape(-1, ncomp)
        return pi @ self.mg.apply(z).reshape(-1)

    def apply(self, j: int, r: np.ndarray) -> np.ndarray:
        y = self.smoother(j) * r + self.nodal(j, r)
        if j >= 1:
            if j - 1 not in self._d:
                self._d[j - 1] = self.wc.dif(j - 1)
            D = self._d[j - 1]
            y = y + D @ self.apply(j - 1, D.T @ r)
        return y
