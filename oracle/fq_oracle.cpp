// fq_oracle.cpp -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.
//
// A plain C++17 (OpenMP) restatement of formoniq's Galerkin assembly path, used
// only as the test oracle: by the tests under tests/, by __graft_entry__.smoke() and
// by bench.py's CPU-baseline / reference arm. Nothing in formoniq_gb300/ links,
// loads or calls this file.
//
// Every function names the reference function it restates (paths are relative
// to the luiswirth/formoniq workspace root). The reference is Rust and cannot be
// built in this environment (no cargo/rustc, no crate registry), so this is a
// restatement, pinned against the reference's own known-answer tests (closed
// form element matrices, Kuhn mesh cell lists, P1 FEM stiffness, FDM stencils)
// in tests/test_oracle_golden.py. Third-party arithmetic it cannot reproduce bit
// for bit: nalgebra's dense LU/cofactor inverse and gemm summation order, and
// nalgebra-sparse's COO->CSR duplicate summation order (restated here as
// "sorted columns, duplicates summed in triplet (cell) order").
//
// Build (done by __graft_entry__.build()): g++ -O2 -std=c++17 -fopenmp -fPIC
// -shared -ffp-contract=off -o oracle/_build/libfq_oracle.so oracle/fq_oracle.cpp

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

using i64 = int64_t;
using Mat = std::vector<double>;  // row-major dense, dims carried alongside

i64 binom(int n, int k) {
  if (k < 0 || n < 0 || k > n) return 0;
  i64 r = 1;
  for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
  return r;
}

double factorial_f64(int n) {
  double r = 1.0;
  for (int i = 2; i <= n; ++i) r *= double(i);
  return r;
}

// k-subsets of {0..m-1} in colex order.
// multiindex/src/combination.rs (colex rank), multiindex::combinations.
// Increasing bitmask order is colex order: the largest element decides first.
std::vector<std::vector<int>> combinations(int m, int k) {
  std::vector<std::vector<int>> out;
  if (k < 0 || k > m) return out;
  for (uint32_t mask = 0; mask < (1u << m); ++mask) {
    if (__builtin_popcount(mask) != k) continue;
    std::vector<int> c;
    for (int b = 0; b < m; ++b)
      if (mask & (1u << b)) c.push_back(b);
    out.push_back(c);
  }
  return out;
}

// Colex rank sum_i C(c_i, i+1).
i64 colex_rank(const std::vector<int>& c) {
  i64 r = 0;
  for (size_t i = 0; i < c.size(); ++i) r += binom(c[i], int(i) + 1);
  return r;
}

// Permutation::all (multiindex/src/permutation.rs:160-169): lexicographic words,
// each emitted reversed. Returns (perm, sign).
struct Perm {
  std::vector<int> p;
  int sign;
};
std::vector<Perm> all_permutations(int n) {
  std::vector<Perm> out;
  std::vector<int> w(n);
  std::iota(w.begin(), w.end(), 0);
  do {
    Perm q;
    q.p.assign(w.rbegin(), w.rend());
    int inv = 0;
    for (int i = 0; i < n; ++i)
      for (int j = i + 1; j < n; ++j)
        if (q.p[i] > q.p[j]) ++inv;
    q.sign = (inv % 2) ? -1 : 1;
    out.push_back(q);
  } while (std::next_permutation(w.begin(), w.end()));
  return out;
}

// Leibniz determinant, multialgebra/src/lib.rs:447-456.
double leibniz_det(const Mat& a, int n) {
  auto perms = all_permutations(n);
  double acc = 0.0;
  for (const auto& s : perms) {
    double prod = 1.0;
    for (int i = 0; i < n; ++i) prod = prod * a[i * n + s.p[i]];
    acc = acc + double(s.sign) * prod;
  }
  return acc;
}

// Dense product C = A (r x m) * B (m x c), inner index ascending.
Mat matmul(const Mat& a, const Mat& b, int r, int m, int c) {
  Mat out(size_t(r) * c, 0.0);
  for (int i = 0; i < r; ++i)
    for (int j = 0; j < c; ++j) {
      double s = 0.0;
      for (int t = 0; t < m; ++t) s += a[i * m + t] * b[t * c + j];
      out[i * c + j] = s;
    }
  return out;
}

Mat transpose(const Mat& a, int r, int c) {
  Mat t(size_t(r) * c);
  for (int i = 0; i < r; ++i)
    for (int j = 0; j < c; ++j) t[j * r + i] = a[i * c + j];
  return t;
}

// Determinant of a small symmetric metric: closed forms for n <= 3, LU with
// partial pivoting above (nalgebra Matrix::determinant; metric/src/lib.rs:179-190).
double metric_det(const Mat& g, int n) {
  if (n == 0) return 1.0;
  if (n == 1) return g[0];
  if (n == 2) return g[0] * g[3] - g[2] * g[1];
  if (n == 3) {
    const double m11 = g[0], m12 = g[1], m13 = g[2], m21 = g[3], m22 = g[4], m23 = g[5],
                 m31 = g[6], m32 = g[7], m33 = g[8];
    const double minor_1 = m22 * m33 - m32 * m23;
    const double minor_2 = m21 * m33 - m31 * m23;
    const double minor_3 = m21 * m32 - m31 * m22;
    return m11 * minor_1 - m12 * minor_2 + m13 * minor_3;
  }
  Mat a = g;
  double det = 1.0;
  for (int c = 0; c < n; ++c) {
    int piv = c;
    for (int r = c + 1; r < n; ++r)
      if (std::fabs(a[r * n + c]) > std::fabs(a[piv * n + c])) piv = r;
    if (a[piv * n + c] == 0.0) return 0.0;
    if (piv != c) {
      for (int j = 0; j < n; ++j) std::swap(a[c * n + j], a[piv * n + j]);
      det = -det;
    }
    det *= a[c * n + c];
    for (int r = c + 1; r < n; ++r) {
      const double f = a[r * n + c] / a[c * n + c];
      for (int j = c; j < n; ++j) a[r * n + j] -= f * a[c * n + j];
    }
  }
  return det;
}

// Inverse of the metric: Metric::dual (metric/src/lib.rs:250-257), nalgebra
// try_inverse (closed cofactor forms up to 4x4). Restated as adjugate / det.
bool metric_inverse(const Mat& g, int n, Mat& inv) {
  inv.assign(size_t(n) * n, 0.0);
  if (n == 0) return true;
  if (n == 1) {
    if (g[0] == 0.0) return false;
    inv[0] = 1.0 / g[0];
    return true;
  }
  // adjugate by cofactors
  const double det = metric_det(g, n);
  if (det == 0.0) return false;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      // cofactor C_ji (adjugate = cofactor transpose)
      Mat minor;
      for (int r = 0; r < n; ++r) {
        if (r == j) continue;
        for (int c = 0; c < n; ++c) {
          if (c == i) continue;
          minor.push_back(g[r * n + c]);
        }
      }
      const double m = metric_det(minor, n - 1);
      inv[i * n + j] = (((i + j) % 2) ? -m : m) / det;
    }
  return true;
}

// Per-(dim) reference-cell constants.
struct RefCell {
  int n;
  // unit_difbarys (simplicial/src/atlas.rs:174-182): (n+1) x n
  Mat difbarys;
  // unit_bary_gramian (simplicial/src/atlas.rs:198-204): (n+1) x (n+1)
  Mat bary_gramian;
  explicit RefCell(int n_) : n(n_) {
    difbarys.assign(size_t(n + 1) * n, 0.0);
    for (int j = 0; j < n; ++j) difbarys[0 * n + j] = -1.0;
    for (int i = 0; i < n; ++i) difbarys[(i + 1) * n + i] = 1.0;
    const int nv = n + 1;
    const double scale = 1.0 / double(nv * (nv + 1));
    bary_gramian.assign(size_t(nv) * nv, scale);
    for (int i = 0; i < nv; ++i) bary_gramian[i * nv + i] = 2.0 * scale;
  }
};

// exterior_power (multialgebra/src/lib.rs:493-512): k-th compound on colex subsets.
Mat exterior_power(const Mat& map, int nrows, int ncols, int k, int& orows, int& ocols) {
  auto rs = combinations(nrows, k), cs = combinations(ncols, k);
  orows = int(rs.size());
  ocols = int(cs.size());
  Mat power(size_t(orows) * ocols, 0.0);
  if (k < 0) return power;
  Mat minor(size_t(k) * k);
  for (int i = 0; i < orows; ++i)
    for (int j = 0; j < ocols; ++j) {
      for (int ii = 0; ii < k; ++ii)
        for (int jj = 0; jj < k; ++jj) minor[ii * k + jj] = map[rs[i][ii] * ncols + cs[j][jj]];
      power[i * ocols + j] = leibniz_det(minor, k);
    }
  return power;
}

// Factor::induced_form alternating (multialgebra/src/lib.rs:285-306): the k x k
// minors of a square form on colex k-subsets, by Leibniz.
Mat induced_alternating(const Mat& single, int dim, int k, int& size) {
  auto basis = combinations(dim, k);
  size = int(basis.size());
  Mat out(size_t(size) * size, 0.0);
  Mat minor(size_t(k) * k);
  for (int i = 0; i < size; ++i)
    for (int j = 0; j < size; ++j) {
      for (int a = 0; a < k; ++a)
        for (int b = 0; b < k; ++b) minor[a * k + b] = single[basis[i][a] * dim + basis[j][b]];
      out[i * size + j] = leibniz_det(minor, k);
    }
  return out;
}

// unit_boundary_operator (simplicial/src/topology/simplex.rs:223-237):
// C(n+1,k) x C(n+1,k+1), entry (-1)^p at (rank(sigma \ sigma_p), sigma).
Mat unit_boundary_operator(int n, int k, int& rows, int& cols) {
  auto cofaces = (k >= 0 && k <= n) ? combinations(n + 1, k + 1) : std::vector<std::vector<int>>{};
  const bool below_in_range = (k - 1 >= 0 && k - 1 <= n);
  rows = below_in_range ? int(binom(n + 1, k)) : 0;
  cols = int(cofaces.size());
  Mat m(size_t(rows) * cols, 0.0);
  if (!below_in_range) return m;
  for (int c = 0; c < cols; ++c) {
    const auto& sigma = cofaces[c];
    for (int p = 0; p < int(sigma.size()); ++p) {
      std::vector<int> face;
      for (int q = 0; q < int(sigma.size()); ++q)
        if (q != p) face.push_back(sigma[q]);
      m[colex_rank(face) * cols + c] = (p % 2) ? -1.0 : 1.0;
    }
  }
  return m;
}

enum Form { MASS = 0, DIF_TRIAL = 1, DIF_TEST = 2, DIF_BOTH = 3 };

// A WhitneyPairing (formoniq/src/operators.rs:134-212) with its precomputed
// cell-independent data: HodgeMass (operators.rs:58-95) = exterior power of the
// difbarys, the Whitney expansion (derham/src/interpolate/form.rs:142-234) and the
// barycentric Gramian.
struct Pairing {
  int n, k, form;
  int test_grade, trial_grade;
  int nblade, ndof;        // C(n+1,k) blades, C(n+1,k+1) dofs of the mass
  int dpow_rows, dpow_cols;  // exterior_power(unit_difbarys(n), k)
  Mat dpow;
  Mat bary;
  std::vector<std::vector<int>> dofs;
  int brows = 0, bcols = 0;  // boundary operator at grade k
  Mat bnd;
  Pairing(int n_, int k_, int form_) : n(n_), k(k_), form(form_) {
    RefCell rc(n);
    dpow = exterior_power(rc.difbarys, n + 1, n, k, dpow_rows, dpow_cols);
    bary = rc.bary_gramian;
    dofs = (k >= 0 && k <= n) ? combinations(n + 1, k + 1) : std::vector<std::vector<int>>{};
    ndof = int(dofs.size());
    nblade = dpow_rows;
    bnd = unit_boundary_operator(n, k, brows, bcols);
    test_grade = (form == DIF_TEST || form == DIF_BOTH) ? k - 1 : k;
    trial_grade = (form == DIF_TRIAL || form == DIF_BOTH) ? k - 1 : k;
  }

  // HodgeMass::element (operators.rs:84-94).
  Mat hodge_mass(const Mat& ginv, double vol) const {
    int lsize = 0;
    Mat lam = induced_alternating(ginv, n, k, lsize);  // multiform_metric (metric/src/tensor.rs:127-131)
    // blade Gramian D * Lambda * D^T (operators.rs:90-91)
    Mat dl = matmul(dpow, lam, dpow_rows, dpow_cols, dpow_cols);
    Mat dt = transpose(dpow, dpow_rows, dpow_cols);
    Mat blade = matmul(dl, dt, dpow_rows, dpow_cols, dpow_rows);
    // WhitneyExpansion::pullback (form.rs:222-234), k! in each column (form.rs:195-200)
    const double scale = factorial_f64(k);
    Mat out(size_t(ndof) * ndof, 0.0);
    for (int i = 0; i < ndof; ++i)
      for (int j = 0; j < ndof; ++j) {
        double s = 0.0;
        const auto& si = dofs[i];
        const auto& sj = dofs[j];
        for (int p = 0; p < int(si.size()); ++p) {
          std::vector<int> ab;
          for (int q = 0; q < int(si.size()); ++q)
            if (q != p) ab.push_back(si[q]);
          const double av = ((p % 2) ? -1.0 : 1.0) * scale;
          const i64 ar = colex_rank(ab);
          for (int q = 0; q < int(sj.size()); ++q) {
            std::vector<int> bb;
            for (int r = 0; r < int(sj.size()); ++r)
              if (r != q) bb.push_back(sj[r]);
            const double bv = ((q % 2) ? -1.0 : 1.0) * scale;
            const i64 br = colex_rank(bb);
            s += av * bv * blade[ar * nblade + br] * bary[si[p] * (n + 1) + sj[q]];
          }
        }
        out[i * ndof + j] = s;
      }
    for (auto& v : out) v = vol * v;
    return out;
  }

  // WhitneyPairing::element (operators.rs:201-211): row * (mass * col).
  Mat element(const Mat& ginv, double vol, int& rows, int& cols) const {
    Mat mass = hodge_mass(ginv, vol);
    int mr = ndof, mc = ndof;
    if (form == DIF_TRIAL || form == DIF_BOTH) {
      Mat col = transpose(bnd, brows, bcols);  // bcols x brows = ndof x C(n+1,k)
      mass = matmul(mass, col, mr, mc, brows);
      mc = brows;
    }
    if (form == DIF_TEST || form == DIF_BOTH) {
      mass = matmul(bnd, mass, brows, bcols, mc);
      mr = brows;
    }
    rows = mr;
    cols = mc;
    return mass;
  }
};

// ---------------------------------------------------------------------------
// Simplicial complex (simplicial/src/topology/{complex.rs:298-336, skeleton.rs:50-83})
// ---------------------------------------------------------------------------
struct Complex {
  int dim = 0;
  i64 nverts = 0;
  std::vector<std::vector<int32_t>> skel;        // skel[k]: N_k x (k+1), colex sorted
  std::vector<std::vector<int32_t>> cell_faces;  // [k]: ncells x C(n+1,k+1) kidx
  std::vector<std::vector<uint8_t>> on_boundary; // [k]: N_k flags
  i64 ncells() const { return i64(skel[dim].size()) / (dim + 1); }
  i64 nsimp(int k) const {
    if (k < 0 || k > dim) return 0;
    return i64(skel[k].size()) / (k + 1);
  }
};

// impl Ord for Simplex (topology/simplex.rs:126-130): compare from the largest
// vertex downward.
struct ColexLess {
  const int32_t* base;
  int w;
  bool operator()(i64 a, i64 b) const {
    const int32_t* x = base + a * w;
    const int32_t* y = base + b * w;
    for (int i = w - 1; i >= 0; --i) {
      if (x[i] != y[i]) return x[i] < y[i];
    }
    return false;
  }
};

Complex* build_complex(int dim, i64 ncells_in, const int32_t* cells_in) {
  auto* cx = new Complex();
  cx->dim = dim;
  const int nv = dim + 1;
  // Skeleton::new on the cells: sort colex, dedup.
  std::vector<i64> order(static_cast<size_t>(ncells_in));
  std::iota(order.begin(), order.end(), 0);
  std::vector<int32_t> cells_sorted_in(cells_in, cells_in + ncells_in * nv);
  for (i64 c = 0; c < ncells_in; ++c) std::sort(&cells_sorted_in[c * nv], &cells_sorted_in[c * nv] + nv);
  std::sort(order.begin(), order.end(), ColexLess{cells_sorted_in.data(), nv});
  std::vector<int32_t> cells;
  cells.reserve(size_t(ncells_in) * nv);
  for (i64 i = 0; i < ncells_in; ++i) {
    const int32_t* c = &cells_sorted_in[order[i] * nv];
    if (!cells.empty() && std::equal(c, c + nv, cells.end() - nv)) continue;
    cells.insert(cells.end(), c, c + nv);
  }
  const i64 ncells = i64(cells.size()) / nv;
  int32_t maxv = -1;
  for (auto v : cells) maxv = std::max(maxv, v);
  cx->nverts = maxv + 1;
  cx->skel.assign(dim + 1, {});
  cx->cell_faces.assign(dim + 1, {});
  for (int k = 0; k <= dim; ++k) {
    auto locals = combinations(nv, k + 1);
    const int nloc = int(locals.size());
    const int w = k + 1;
    std::vector<int32_t> faces(size_t(ncells) * nloc * w);
    for (i64 c = 0; c < ncells; ++c)
      for (int l = 0; l < nloc; ++l)
        for (int i = 0; i < w; ++i) faces[(c * nloc + l) * w + i] = cells[c * nv + locals[l][i]];
    const i64 nf = ncells * nloc;
    std::vector<i64> idx(static_cast<size_t>(nf));
    std::iota(idx.begin(), idx.end(), 0);
    std::sort(idx.begin(), idx.end(), ColexLess{faces.data(), w});
    std::vector<int32_t>& sk = cx->skel[k];
    std::vector<int32_t>& cf = cx->cell_faces[k];
    cf.assign(size_t(nf), -1);
    i64 kidx = -1;
    for (i64 t = 0; t < nf; ++t) {
      const int32_t* f = &faces[idx[t] * w];
      if (kidx < 0 || !std::equal(f, f + w, sk.end() - w)) {
        sk.insert(sk.end(), f, f + w);
        ++kidx;
      }
      cf[idx[t]] = int32_t(kidx);
    }
  }
  // Boundary: facets in exactly one cell; boundary simplices are their faces
  // (complex.rs:140-151 boundary_simplices).
  cx->on_boundary.assign(dim + 1, {});
  for (int k = 0; k <= dim; ++k) cx->on_boundary[k].assign(size_t(cx->nsimp(k)), 0);
  if (dim >= 1) {
    const int nfac = int(binom(nv, dim));
    std::vector<int32_t> count(size_t(cx->nsimp(dim - 1)), 0);
    for (i64 c = 0; c < ncells; ++c)
      for (int l = 0; l < nfac; ++l) count[cx->cell_faces[dim - 1][c * nfac + l]]++;
    for (i64 f = 0; f < cx->nsimp(dim - 1); ++f) {
      if (count[f] != 1) continue;
      const int32_t* fv = &cx->skel[dim - 1][f * dim];
      // mark every sub-face of the facet: find its kidx by binary search
      for (int k = 0; k <= dim - 1; ++k) {
        auto subs = combinations(dim, k + 1);
        const int w = k + 1;
        for (const auto& s : subs) {
          std::vector<int32_t> tup(w);
          for (int i = 0; i < w; ++i) tup[i] = fv[s[i]];
          // binary search in skel[k] (colex sorted)
          i64 lo = 0, hi = cx->nsimp(k) - 1;
          const int32_t* sk = cx->skel[k].data();
          while (lo <= hi) {
            i64 mid = (lo + hi) / 2;
            int cmp = 0;
            for (int i = w - 1; i >= 0; --i) {
              if (sk[mid * w + i] != tup[i]) {
                cmp = sk[mid * w + i] < tup[i] ? -1 : 1;
                break;
              }
            }
            if (cmp == 0) {
              cx->on_boundary[k][mid] = 1;
              break;
            }
            if (cmp < 0)
              lo = mid + 1;
            else
              hi = mid - 1;
          }
        }
      }
    }
  }
  return cx;
}

// Triplets -> CSR with nalgebra-sparse semantics as restated: columns sorted per
// row, duplicates summed in triplet order, explicit zeros kept
// (formoniq/src/galerkin.rs:184-187).
struct Csr {
  i64 nrows = 0, ncols = 0;
  std::vector<int64_t> row_ptr;
  std::vector<int64_t> col_idx;
  std::vector<double> values;
};

Csr* coo_to_csr(i64 nrows, i64 ncols, const std::vector<i64>& rows, const std::vector<i64>& cols,
                const std::vector<double>& vals) {
  auto* m = new Csr();
  m->nrows = nrows;
  m->ncols = ncols;
  const i64 nt = i64(rows.size());
  std::vector<i64> cnt(size_t(nrows) + 1, 0);
  for (i64 t = 0; t < nt; ++t) cnt[rows[t] + 1]++;
  for (i64 r = 0; r < nrows; ++r) cnt[r + 1] += cnt[r];
  std::vector<i64> pos(cnt.begin(), cnt.end() - 1);
  std::vector<i64> order(static_cast<size_t>(nt));
  for (i64 t = 0; t < nt; ++t) order[pos[rows[t]]++] = t;  // stable by row
  m->row_ptr.assign(size_t(nrows) + 1, 0);
  std::vector<std::vector<std::pair<i64, double>>> rowsum(static_cast<size_t>(nrows));
#pragma omp parallel for schedule(dynamic, 256)
  for (i64 r = 0; r < nrows; ++r) {
    std::vector<i64> seg(order.begin() + cnt[r], order.begin() + cnt[r + 1]);
    std::stable_sort(seg.begin(), seg.end(), [&](i64 a, i64 b) { return cols[a] < cols[b]; });
    auto& out = rowsum[r];
    for (i64 t : seg) {
      if (!out.empty() && out.back().first == cols[t])
        out.back().second += vals[t];
      else
        out.emplace_back(cols[t], vals[t]);
    }
  }
  for (i64 r = 0; r < nrows; ++r) m->row_ptr[r + 1] = m->row_ptr[r] + i64(rowsum[r].size());
  m->col_idx.resize(size_t(m->row_ptr[nrows]));
  m->values.resize(size_t(m->row_ptr[nrows]));
  for (i64 r = 0; r < nrows; ++r) {
    i64 o = m->row_ptr[r];
    for (auto& e : rowsum[r]) {
      m->col_idx[o] = e.first;
      m->values[o] = e.second;
      ++o;
    }
  }
  return m;
}

// SimplexLengthsSq::metric (regge/src/lengths/simplex.rs:308-326) with the edge
// lengths of the cell gathered in local colex edge order (lengths/mesh.rs:153-162).
void cell_metric(const Complex& cx, const double* lengths, i64 cell, Mat& g) {
  const int n = cx.dim;
  const int ne = int(binom(n + 1, 2));
  g.assign(size_t(n) * n, 0.0);
  if (n == 0) return;
  const int32_t* ce = &cx.cell_faces[1][cell * ne];
  auto s = [&](int a, int b) {  // edge_index(a,b) = C(b,2)+a for a<b
    const int lo = std::min(a, b), hi = std::max(a, b);
    return lengths[ce[binom(hi, 2) + lo]];
  };
  for (int i = 0; i < n; ++i) g[i * n + i] = s(0, i + 1);
  for (int i = 0; i < n; ++i)
    for (int j = i + 1; j < n; ++j) {
      const double s0i = s(0, i + 1), s0j = s(0, j + 1), sij = s(i + 1, j + 1);
      const double val = 0.5 * (s0i + s0j - sij);
      g[i * n + j] = val;
      g[j * n + i] = val;
    }
}

// cell_volume (regge/src/lib.rs:26-28) = unit_simplex_volume * sqrt(|det g|).
double cell_volume(const Mat& g, int n) { return (1.0 / factorial_f64(n)) * std::sqrt(std::fabs(metric_det(g, n))); }

struct Assembled {
  Csr* csr;
};

// Interior renumbering of grade k for the relative complex
// (whitney_complex.rs:523-566): -1 on the boundary.
std::vector<i64> interior_map(const Complex& cx, int k, i64& count) {
  std::vector<i64> m(size_t(cx.nsimp(k)), -1);
  count = 0;
  for (i64 i = 0; i < cx.nsimp(k); ++i)
    if (!cx.on_boundary[k][i]) m[i] = count++;
  return m;
}

}  // namespace

// ===========================================================================
// extern "C" surface used by tests (ctypes). All host memory.
// ===========================================================================
extern "C" {

typedef struct OrComplex OrComplex;
typedef struct OrCsr OrCsr;

int or_num_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void or_set_num_threads(int t) {
#ifdef _OPENMP
  if (t > 0) omp_set_num_threads(t);
#else
  (void)t;
#endif
}

// CartesianTopology::cell_skeleton (simplicial/src/mesher/grid.rs:77-98) for the
// cube with `nbox` boxes per axis: per box (radix order, axis 0 fastest,
// multiindex/src/cartesian.rs:78-135) and per axis permutation, the chain of
// corners. Unsorted; build_complex sorts. Returns ncells = nbox^dim * dim!.
int64_t or_kuhn_ncells(int dim, int nbox) {
  int64_t nb = 1;
  for (int a = 0; a < dim; ++a) nb *= nbox;
  int64_t f = 1;
  for (int a = 2; a <= dim; ++a) f *= a;
  return nb * f;
}
void or_kuhn_cells(int dim, int nbox, int32_t* out) {
  const int nv = dim + 1;
  std::vector<int64_t> stride(dim);
  int64_t s = 1;
  for (int a = 0; a < dim; ++a) {
    stride[a] = s;
    s *= (nbox + 1);
  }
  int64_t nboxes = 1;
  for (int a = 0; a < dim; ++a) nboxes *= nbox;
  std::vector<int> perm(dim);
  std::iota(perm.begin(), perm.end(), 0);
  std::vector<std::vector<int>> perms;
  do perms.push_back(perm);
  while (std::next_permutation(perm.begin(), perm.end()));
  int64_t c = 0;
  for (int64_t b = 0; b < nboxes; ++b) {
    int64_t rem = b, origin = 0;
    for (int a = 0; a < dim; ++a) {
      origin += (rem % nbox) * stride[a];
      rem /= nbox;
    }
    for (const auto& p : perms) {
      int64_t v = origin;
      out[c * nv + 0] = int32_t(v);
      for (int i = 0; i < dim; ++i) {
        v += stride[p[i]];
        out[c * nv + i + 1] = int32_t(v);
      }
      ++c;
    }
  }
}

// CartesianGrid::vertex_pos (regge/src/mesher/cartesian.rs:158-169): coords of the
// (nbox+1)^dim grid vertices, x_a = c_a/nbox * side_a + min_a. Row-major
// [vertex][axis].
void or_grid_coords(int dim, int nbox, const double* side, const double* minv, double* out) {
  int64_t nverts = 1;
  for (int a = 0; a < dim; ++a) nverts *= (nbox + 1);
  for (int64_t v = 0; v < nverts; ++v) {
    int64_t rem = v;
    for (int a = 0; a < dim; ++a) {
      const int64_t c = rem % (nbox + 1);
      rem /= (nbox + 1);
      out[v * dim + a] = (double(c) / double(nbox)) * side[a] + minv[a];
    }
  }
}

OrComplex* or_complex_build(int dim, int64_t ncells, const int32_t* cells) {
  return reinterpret_cast<OrComplex*>(build_complex(dim, ncells, cells));
}
void or_complex_free(OrComplex* c) { delete reinterpret_cast<Complex*>(c); }
int64_t or_complex_nsimplices(OrComplex* c, int k) { return reinterpret_cast<Complex*>(c)->nsimp(k); }
void or_complex_simplices(OrComplex* c, int k, int32_t* out) {
  auto* cx = reinterpret_cast<Complex*>(c);
  std::memcpy(out, cx->skel[k].data(), cx->skel[k].size() * sizeof(int32_t));
}
void or_complex_cell_faces(OrComplex* c, int k, int32_t* out) {
  auto* cx = reinterpret_cast<Complex*>(c);
  std::memcpy(out, cx->cell_faces[k].data(), cx->cell_faces[k].size() * sizeof(int32_t));
}
void or_complex_boundary_flags(OrComplex* c, int k, uint8_t* out) {
  auto* cx = reinterpret_cast<Complex*>(c);
  std::memcpy(out, cx->on_boundary[k].data(), cx->on_boundary[k].size());
}

// MeshCoords::to_edge_lengths_sq (regge/src/coord/mesh.rs:208-216): s_e =
// (x_j-x_i)^T eta (x_j-x_i), eta = diag(ambient_signs). Coords row-major.
void or_edge_lengths_sq(OrComplex* c, const double* coords, int ambient_dim, const double* ambient_signs,
                        double* out) {
  auto* cx = reinterpret_cast<Complex*>(c);
  const int64_t ne = cx->nsimp(1);
  for (int64_t e = 0; e < ne; ++e) {
    const int32_t vi = cx->skel[1][e * 2], vj = cx->skel[1][e * 2 + 1];
    double acc = 0.0;
    for (int a = 0; a < ambient_dim; ++a) {
      const double d = coords[int64_t(vj) * ambient_dim + a] - coords[int64_t(vi) * ambient_dim + a];
      acc += d * (ambient_signs[a] * d);
    }
    out[e] = acc;
  }
}

// Per-cell Regge metric, inverse and volume for every cell (kernel (a) oracle).
// g_out / ginv_out: ncells x n x n; vol_out: ncells. Returns the number of cells
// whose metric was singular.
int64_t or_cell_metrics(OrComplex* c, const double* lengths, double* g_out, double* ginv_out, double* det_out,
                        double* vol_out) {
  auto* cx = reinterpret_cast<Complex*>(c);
  const int n = cx->dim;
  int64_t bad = 0;
  const int64_t nc = cx->ncells();
#pragma omp parallel for reduction(+ : bad)
  for (int64_t cell = 0; cell < nc; ++cell) {
    Mat g, ginv;
    cell_metric(*cx, lengths, cell, g);
    if (!metric_inverse(g, n, ginv)) ++bad;
    const double det = metric_det(g, n);
    if (g_out) std::memcpy(g_out + cell * n * n, g.data(), sizeof(double) * n * n);
    if (ginv_out) std::memcpy(ginv_out + cell * n * n, ginv.data(), sizeof(double) * n * n);
    if (det_out) det_out[cell] = det;
    if (vol_out) vol_out[cell] = cell_volume(g, n);
  }
  return bad;
}

// BilinearForm::element for a WhitneyPairing on one cell given its local edge
// lengths (C(n+1,2), local colex order): the element matrix (row-major).
// Returns rows*cols; fills rows/cols.
int or_element_matrix(int n, int form, int grade, const double* local_lengths, double* out, int* rows,
                      int* cols) {
  Mat g(size_t(n) * n, 0.0);
  auto s = [&](int a, int b) {
    const int lo = std::min(a, b), hi = std::max(a, b);
    return local_lengths[binom(hi, 2) + lo];
  };
  for (int i = 0; i < n; ++i) g[i * n + i] = s(0, i + 1);
  for (int i = 0; i < n; ++i)
    for (int j = i + 1; j < n; ++j) {
      const double val = 0.5 * (s(0, i + 1) + s(0, j + 1) - s(i + 1, j + 1));
      g[i * n + j] = val;
      g[j * n + i] = val;
    }
  Mat ginv;
  metric_inverse(g, n, ginv);
  const double vol = cell_volume(g, n);
  Pairing p(n, grade, form);
  int r = 0, cc = 0;
  Mat e = p.element(ginv, vol, r, cc);
  *rows = r;
  *cols = cc;
  if (out) std::memcpy(out, e.data(), sizeof(double) * e.size());
  return r * cc;
}

// assemble_matrix (formoniq/src/galerkin.rs:138-188) for a WhitneyPairing, through
// HilbertComplex::pairing (whitney_complex.rs:113-122) on the full complex, or the
// relative one (E^T A E, whitney_complex.rs:620-624) when `relative` != 0.
OrCsr* or_assemble(OrComplex* c, const double* lengths, int form, int grade, int relative) {
  auto* cx = reinterpret_cast<Complex*>(c);
  const int n = cx->dim;
  Pairing p(n, grade, form);
  const int tg = p.test_grade, sg = p.trial_grade;
  i64 nrows_full = cx->nsimp(tg), ncols_full = cx->nsimp(sg);
  std::vector<i64> rmap, cmap;
  i64 nrows = nrows_full, ncols = ncols_full;
  if (relative) {
    if (tg >= 0 && tg <= n) rmap = interior_map(*cx, tg, nrows);
    if (sg >= 0 && sg <= n) cmap = interior_map(*cx, sg, ncols);
  }
  std::vector<i64> rows, cols;
  std::vector<double> vals;
  if (nrows > 0 && ncols > 0) {
    const i64 nc = cx->ncells();
    const int nthreads = or_num_threads();
    std::vector<std::vector<i64>> trow(nthreads), tcol(nthreads);
    std::vector<std::vector<double>> tval(nthreads);
    const int ntest = int(binom(n + 1, tg + 1)), ntrial = int(binom(n + 1, sg + 1));
#pragma omp parallel num_threads(nthreads)
    {
      int tid = 0, nt = 1;
#ifdef _OPENMP
      tid = omp_get_thread_num();
      nt = omp_get_num_threads();
#endif
      // contiguous cell ranges per thread, concatenated in thread order = cell order
      const i64 lo = nc * tid / nt, hi = nc * (tid + 1) / nt;
      auto& R = trow[tid];
      auto& C = tcol[tid];
      auto& V = tval[tid];
      Mat g, ginv;
      for (i64 cell = lo; cell < hi; ++cell) {
        cell_metric(*cx, lengths, cell, g);
        metric_inverse(g, n, ginv);
        const double vol = cell_volume(g, n);
        int er = 0, ec = 0;
        Mat e = p.element(ginv, vol, er, ec);
        for (int i = 0; i < er; ++i) {
          const i64 gi = cx->cell_faces[tg][cell * ntest + i];
          for (int j = 0; j < ec; ++j) {
            const double val = e[i * ec + j];
            if (val != 0.0) {
              const i64 gj = cx->cell_faces[sg][cell * ntrial + j];
              R.push_back(gi);
              C.push_back(gj);
              V.push_back(val);
            }
          }
        }
      }
    }
    for (int t = 0; t < nthreads; ++t) {
      rows.insert(rows.end(), trow[t].begin(), trow[t].end());
      cols.insert(cols.end(), tcol[t].begin(), tcol[t].end());
      vals.insert(vals.end(), tval[t].begin(), tval[t].end());
    }
  }
  if (relative && nrows > 0 && ncols > 0) {
    // E_test^T A E_trial: keep interior rows and columns, renumbered.
    std::vector<i64> r2, c2;
    std::vector<double> v2;
    for (size_t t = 0; t < rows.size(); ++t) {
      const i64 rr = rmap[rows[t]], cc2 = cmap[cols[t]];
      if (rr < 0 || cc2 < 0) continue;
      r2.push_back(rr);
      c2.push_back(cc2);
      v2.push_back(vals[t]);
    }
    rows.swap(r2);
    cols.swap(c2);
    vals.swap(v2);
  }
  return reinterpret_cast<OrCsr*>(coo_to_csr(nrows, ncols, rows, cols, vals));
}

// Coboundary D_k = (boundary_operator(k+1))^T as CSR (complex.rs:168-217,
// whitney_complex.rs:417-423): N_{k+1} x N_k, entry (-1)^p at (coface, coface\p).
OrCsr* or_coboundary(OrComplex* c, int k, int relative) {
  auto* cx = reinterpret_cast<Complex*>(c);
  const int n = cx->dim;
  i64 nr = cx->nsimp(k + 1), ncol = cx->nsimp(k);
  std::vector<i64> rows, cols;
  std::vector<double> vals;
  std::vector<i64> rmap, cmap;
  if (relative) {
    if (k + 1 >= 0 && k + 1 <= n) rmap = interior_map(*cx, k + 1, nr);
    if (k >= 0 && k <= n) cmap = interior_map(*cx, k, ncol);
  }
  if (k >= 0 && k < n) {
    const int w = k + 2;
    const i64 ncof = cx->nsimp(k + 1);
    for (i64 cof = 0; cof < ncof; ++cof) {
      const int32_t* cv = &cx->skel[k + 1][cof * w];
      for (int p = 0; p < w; ++p) {
        // locate the face cv \ cv[p] in skel[k] by binary search
        std::vector<int32_t> tup;
        for (int q = 0; q < w; ++q)
          if (q != p) tup.push_back(cv[q]);
        const int fw = w - 1;
        i64 lo = 0, hi = cx->nsimp(k) - 1, found = -1;
        const int32_t* sk = cx->skel[k].data();
        while (lo <= hi) {
          i64 mid = (lo + hi) / 2;
          int cmp = 0;
          for (int i = fw - 1; i >= 0; --i)
            if (sk[mid * fw + i] != tup[i]) {
              cmp = sk[mid * fw + i] < tup[i] ? -1 : 1;
              break;
            }
          if (cmp == 0) {
            found = mid;
            break;
          }
          if (cmp < 0)
            lo = mid + 1;
          else
            hi = mid - 1;
        }
        i64 r = cof, cc2 = found;
        if (relative) {
          r = rmap[cof];
          cc2 = cmap[found];
          if (r < 0 || cc2 < 0) continue;
        }
        rows.push_back(r);
        cols.push_back(cc2);
        vals.push_back((p % 2) ? -1.0 : 1.0);
      }
    }
  }
  return reinterpret_cast<OrCsr*>(coo_to_csr(nr, ncol, rows, cols, vals));
}

void or_csr_shape(OrCsr* m, int64_t* nrows, int64_t* ncols, int64_t* nnz) {
  auto* a = reinterpret_cast<Csr*>(m);
  *nrows = a->nrows;
  *ncols = a->ncols;
  *nnz = a->row_ptr.empty() ? 0 : a->row_ptr.back();
}
void or_csr_copy(OrCsr* m, int64_t* row_ptr, int64_t* col_idx, double* values) {
  auto* a = reinterpret_cast<Csr*>(m);
  std::memcpy(row_ptr, a->row_ptr.data(), a->row_ptr.size() * sizeof(int64_t));
  std::memcpy(col_idx, a->col_idx.data(), a->col_idx.size() * sizeof(int64_t));
  std::memcpy(values, a->values.data(), a->values.size() * sizeof(double));
}
void or_csr_free(OrCsr* m) { delete reinterpret_cast<Csr*>(m); }

// CSR matrix-vector product y = A x (iterative/src/operator.rs:5-13), OpenMP rows.
void or_csr_matvec(OrCsr* m, const double* x, double* y) {
  auto* a = reinterpret_cast<Csr*>(m);
#pragma omp parallel for schedule(static)
  for (i64 r = 0; r < a->nrows; ++r) {
    double s = 0.0;
    for (i64 t = a->row_ptr[r]; t < a->row_ptr[r + 1]; ++t) s += a->values[t] * x[a->col_idx[t]];
    y[r] = s;
  }
}

}  // extern "C"
