// Set-up of the HX-multigrid preconditioner on a Kuhn cube (host side).
//
// Nodal hierarchy. The reference builds its levels by refining a coarse base
// mesh (formoniq/src/multigrid.rs:RefinementTower). A Kuhn cube of N boxes per
// axis is coarsened instead: level l+1 is the Kuhn lattice of ceil(N_l / 2)
// boxes over the same cube, and P_l interpolates its piecewise-linear nodal
// functions at the lattice points of level l. A lattice point with local
// coordinates t in a coarse box lies in the Kuhn simplex that follows the axes in
// decreasing t, where its barycentric weights are 1 - t_(1), t_(1) - t_(2), ...,
// t_(n). For even N this is the nested two-point average; for odd N the levels
// are not nested and P is the interpolation between them. The coarse operators
// are the Galerkin products P^T A P, as in the reference; the coarsest level
// (at most 256 unknowns) is inverted densely.
//
// Vector-nodal interpolation (formoniq/src/hx.rs:vector_nodal_prolongation):
// Pi_j[sigma, (a, I)] = <e_I, tau_sigma> / (j+1)! for each vertex a of the
// j-simplex sigma, tau_sigma the wedge of its edge vectors from its first vertex
// in an ambient frame. The reference reads the frame off the mesh coordinates; a
// mesh here carries lengths only, so the frame is the Kuhn lattice, scaled per
// axis by the root mean squared length of that axis' lattice edges.
#include <algorithm>
#include <cmath>
#include <memory>
#include <vector>

#include "fq_hx.h"

namespace fq {

fq_status make_matrix(fq_ctx* ctx, fq_mesh* mesh, int kind, int grade, int bc, int precision, double param,
                      fq_matrix** out);
fq_status assemble_into(fq_ctx* ctx, fq_matrix* m);
fq_status device_scaled_recip(fq_ctx* ctx, const double* d, int64_t n, double omega, DevBuf& out);

namespace {

constexpr double kOmega = 2.0 / 3.0;  // Jacobi::smoother (iterative/src/precond.rs:92-94)
constexpr int64_t kCoarseMax = 256;

int64_t ipow(int64_t b, int e) {
  int64_t r = 1;
  for (int i = 0; i < e; ++i) r *= b;
  return r;
}

int binom(int n, int k) {
  if (k < 0 || k > n) return 0;
  int r = 1;
  for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
  return r;
}

// Unknowns of a lattice level: every node, or the interior ones.
int64_t level_nodes(int n, int nbox, int bc) {
  return bc == FQ_RELATIVE ? ipow(std::max(nbox - 1, 0), n) : ipow(nbox + 1, n);
}

// Unknown index of lattice point c on an nbox lattice, -1 if not an unknown.
// Interior points are numbered in the order of their vertex index, which is
// the order of the relative complex.
int64_t node_index(const int* c, int n, int nbox, int bc) {
  int64_t idx = 0, stride = 1;
  for (int a = 0; a < n; ++a) {
    if (bc == FQ_RELATIVE) {
      if (c[a] <= 0 || c[a] >= nbox) return -1;
      idx += int64_t(c[a] - 1) * stride;
      stride *= (nbox - 1);
    } else {
      idx += int64_t(c[a]) * stride;
      stride *= (nbox + 1);
    }
  }
  return idx;
}

void lattice_coords(int64_t v, int n, int nbox, int* c) {
  for (int a = 0; a < n; ++a) {
    c[a] = int(v % (nbox + 1));
    v /= (nbox + 1);
  }
}

// P: unknowns of the nf lattice <- unknowns of the nc lattice.
HCsr lattice_prolongation(int n, int nf, int nc, int bc) {
  HCsr P;
  P.nrows = level_nodes(n, nf, bc);
  P.ncols = level_nodes(n, nc, bc);
  P.rp.assign(1, 0);
  const int64_t nv = ipow(nf + 1, n);
  int c[4], b[4], w[4];
  int64_t rho[4];
  for (int64_t v = 0; v < nv; ++v) {
    lattice_coords(v, n, nf, c);
    if (node_index(c, n, nf, bc) < 0) continue;
    int order[4];
    for (int a = 0; a < n; ++a) {
      const int64_t y = int64_t(c[a]) * nc;  // coarse coordinate times nf
      int64_t bb = y / nf;
      int64_t rr = y - bb * nf;
      if (bb >= nc) {
        bb = nc - 1;
        rr = nf;
      }
      b[a] = int(bb);
      rho[a] = rr;
      order[a] = a;
    }
    // axes by decreasing t (stable: ties keep the axis order)
    std::stable_sort(order, order + n, [&](int x, int y) { return rho[x] > rho[y]; });
    std::vector<std::pair<int32_t, double>> ent;
    for (int a = 0; a < n; ++a) w[a] = b[a];
    for (int i = 0; i <= n; ++i) {
      if (i > 0) w[order[i - 1]] += 1;
      const int64_t hi = i == 0 ? nf : rho[order[i - 1]];
      const int64_t lo = i == n ? 0 : rho[order[i]];
      const double lam = double(hi - lo) / double(nf);
      if (lam == 0.0) continue;
      const int64_t col = node_index(w, n, nc, bc);
      if (col < 0) continue;
      ent.emplace_back(int32_t(col), lam);
    }
    std::sort(ent.begin(), ent.end());
    for (auto& e : ent) {
      P.ci.push_back(e.first);
      P.v.push_back(e.second);
    }
    P.rp.push_back(int32_t(P.ci.size()));
  }
  return P;
}

// Dense Cholesky inverse of an SPD matrix (row-major, in place). False if not SPD.
bool spd_inverse(std::vector<double>& a, int64_t n) {
  std::vector<double> L(size_t(n * n), 0.0);
  for (int64_t j = 0; j < n; ++j) {
    double d = a[j * n + j];
    for (int64_t k = 0; k < j; ++k) d -= L[j * n + k] * L[j * n + k];
    if (!(d > 0.0)) return false;
    const double ljj = std::sqrt(d);
    L[j * n + j] = ljj;
    for (int64_t i = j + 1; i < n; ++i) {
      double s = a[i * n + j];
      for (int64_t k = 0; k < j; ++k) s -= L[i * n + k] * L[j * n + k];
      L[i * n + j] = s / ljj;
    }
  }
  // inverse of L (lower triangular), then A^{-1} = L^{-T} L^{-1}
  std::vector<double> Li(size_t(n * n), 0.0);
  for (int64_t j = 0; j < n; ++j) {
    Li[j * n + j] = 1.0 / L[j * n + j];
    for (int64_t i = j + 1; i < n; ++i) {
      double s = 0.0;
      for (int64_t k = j; k < i; ++k) s -= L[i * n + k] * Li[k * n + j];
      Li[i * n + j] = s / L[i * n + i];
    }
  }
  for (int64_t i = 0; i < n; ++i)
    for (int64_t j = 0; j <= i; ++j) {
      double s = 0.0;
      for (int64_t k = i; k < n; ++k) s += Li[k * n + i] * Li[k * n + j];
      a[i * n + j] = a[j * n + i] = s;
    }
  return true;
}

int64_t find_edge(const fq_mesh* m, int32_t u, int32_t v) {
  // skel[1] is colex: sorted by (v1, v0)
  const auto& e = m->skel[1];
  int64_t lo = 0, hi = m->nsimp[1] - 1;
  while (lo <= hi) {
    const int64_t mid = (lo + hi) / 2;
    const int32_t a0 = e[mid * 2], a1 = e[mid * 2 + 1];
    if (a1 == v && a0 == u) return mid;
    if (a1 < v || (a1 == v && a0 < u))
      lo = mid + 1;
    else
      hi = mid - 1;
  }
  return -1;
}

// Identity from unknown i to slot `slot` of node i (and its transpose, the
// identity on unknowns): the grade-0 vector-nodal map.
void slot_identity(int64_t n0, int mslots, int slot, HCsr& Pi, HCsr& Pit) {
  Pi = HCsr();
  Pi.nrows = n0;
  Pi.ncols = n0 * mslots;
  Pit = HCsr();
  Pit.nrows = n0;
  Pit.ncols = n0;
  for (int64_t i = 0; i < n0; ++i) {
    Pi.ci.push_back(int32_t(i * mslots + slot));
    Pi.v.push_back(1.0);
    Pi.mask.push_back(0);
    Pi.rp.push_back(int32_t(i + 1));
    Pit.ci.push_back(int32_t(i));
    Pit.v.push_back(1.0);
    Pit.mask.push_back(0);
    Pit.rp.push_back(int32_t(i + 1));
  }
}

fq_status upload(fq_ctx* ctx, const HCsr& h, DCsr& d) { return d.upload(ctx, h.nrows, h.ncols, h.rp, h.ci, h.v); }

}  // namespace

HCsr transpose(const HCsr& a) {
  HCsr t;
  t.nrows = a.ncols;
  t.ncols = a.nrows;
  t.rp.assign(size_t(t.nrows) + 1, 0);
  for (int32_t c : a.ci) t.rp[c + 1]++;
  for (int64_t i = 0; i < t.nrows; ++i) t.rp[i + 1] += t.rp[i];
  t.ci.resize(a.ci.size());
  t.v.resize(a.v.size());
  std::vector<int32_t> pos(t.rp.begin(), t.rp.end() - 1);
  for (int64_t r = 0; r < a.nrows; ++r)
    for (int32_t q = a.rp[r]; q < a.rp[r + 1]; ++q) {
      const int32_t p = pos[a.ci[q]]++;
      t.ci[p] = int32_t(r);
      t.v[p] = a.v[q];
    }
  return t;
}

bool hx_supported(const fq_mesh* m) { return m && m->kuhn_nbox > 0 && m->dim >= 1 && m->dim <= 4 && m->has_lengths; }

bool hx_matches(const HxPrecond& pc, const fq_mesh* m, int bc, const std::vector<int>& grades, int64_t ident) {
  return pc.mesh == m && pc.bc == bc && pc.grades == grades && pc.ident_len == ident;
}

fq_status hx_build(fq_ctx* ctx, fq_mesh* m, int bc, const std::vector<int>& grades, int64_t ident,
                   const double* diag_blocks, HxPrecond& out) {
  if (!hx_supported(m)) return set_error(ctx, FQ_UNSUPPORTED, "HX multigrid needs a Kuhn cube mesh with lengths");
  const int n = m->dim, nb = m->kuhn_nbox;
  cudaStream_t st = ctx->stream;
  out = HxPrecond();
  out.mesh = m;
  out.bc = bc;
  out.grades = grades;

  // lattice edges per axis, for the frame scaling
  {
    std::vector<int32_t> edges;
    out.axis_off.assign(1, 0);
    const int64_t nv = ipow(nb + 1, n);
    int c[4];
    for (int a = 0; a < n; ++a) {
      const int64_t stride = ipow(nb + 1, a);
      for (int64_t v = 0; v < nv; ++v) {
        lattice_coords(v, n, nb, c);
        if (c[a] >= nb) continue;
        const int64_t e = find_edge(m, int32_t(v), int32_t(v + stride));
        if (e < 0) return set_error(ctx, FQ_UNSUPPORTED, "mesh is not a Kuhn lattice");
        edges.push_back(int32_t(e));
      }
      out.axis_off.push_back(int64_t(edges.size()));
    }
    FQ_TRY(out.axis_edges.alloc(ctx, std::max<size_t>(edges.size(), 1) * 4));
    if (!edges.empty())
      FQ_CUDA(ctx, cudaMemcpyAsync(out.axis_edges.p, edges.data(), edges.size() * 4, cudaMemcpyHostToDevice, st));
    FQ_TRY(out.hprod.alloc(ctx, 16 * 8));
    FQ_TRY(out.flag.alloc(ctx, 8));
    FQ_CUDA(ctx, cudaStreamSynchronize(st));
  }

  // slot layout
  int mslots = 0;
  out.blocks.resize(grades.size());
  int64_t off = 0;
  for (size_t b = 0; b < grades.size(); ++b) {
    HxBlock& B = out.blocks[b];
    B.grade = grades[b];
    B.off = off;
    B.size = bc == FQ_RELATIVE ? m->ninterior[B.grade] : m->nsimp[B.grade];
    off += B.size;
    if (B.grade >= 1) {
      B.grad_slot = mslots;
      B.grad_count = B.grade - 1 == 0 ? 1 : binom(n, B.grade - 1);
      mslots += B.grad_count;
    }
    B.vec_slot = mslots;
    B.vec_count = B.grade == 0 ? 1 : binom(n, B.grade);
    mslots += B.vec_count;
  }
  out.ident_off = off;
  out.ident_len = ident;
  out.n = off + ident;
  out.m = mslots;

  // nodal hierarchy: lattices, prolongations, work blocks
  NodalHierarchy& mg = out.mg;
  mg.dim = n;
  mg.bc = bc;
  mg.mmax = mslots;
  std::vector<int> boxes{nb};
  while (level_nodes(n, boxes.back(), bc) > kCoarseMax && boxes.back() > 2) boxes.push_back((boxes.back() + 1) / 2);
  mg.lv.resize(boxes.size());
  for (size_t l = 0; l < boxes.size(); ++l) {
    NodalLevel& L = mg.lv[l];
    L.nbox = boxes[l];
    L.n = level_nodes(n, boxes[l], bc);
    const size_t wb = size_t(std::max<int64_t>(L.n * mslots, 1)) * 8;
    FQ_TRY(L.x[0].alloc(ctx, wb));
    FQ_TRY(L.x[1].alloc(ctx, wb));
    FQ_TRY(L.r.alloc(ctx, wb));
    FQ_TRY(L.t.alloc(ctx, wb));
    if (l + 1 < boxes.size()) {
      HCsr P = lattice_prolongation(n, boxes[l], boxes[l + 1], bc);
      FQ_TRY(upload(ctx, P, L.P));
      FQ_TRY(upload(ctx, transpose(P), L.R));
    }
  }
  {
    fq_matrix* a0 = nullptr;
    FQ_TRY(make_matrix(ctx, m, EK_HDIF, 0, bc, FQ_FP64, 0.0, &a0));
    out.a0.reset(a0);
    if (a0->nrows != mg.lv[0].n) return set_error(ctx, FQ_UNSUPPORTED, "nodal operator size does not match the lattice");
  }

  // blocks: transfer maps (lattice values; scaled by the spacing in hx_refresh)
  const int64_t n0 = mg.lv[0].n;
  for (HxBlock& B : out.blocks) {
    if (B.grade == 0) {
      HCsr Pi, Pit;
      slot_identity(n0, mslots, B.vec_slot, Pi, Pit);
      FQ_TRY(upload_scalable(ctx, Pi, B.Pi));
      FQ_TRY(upload_scalable(ctx, Pit, B.Pit));
    } else {
      FQ_TRY(vector_nodal_device(ctx, m, B.grade, bc, mslots, B.vec_slot, B.Pi, B.Pit));
    }
    if (B.grade >= 1) {
      const int g = B.grade - 1;
      FQ_TRY(coboundary_device(ctx, m, g, bc, B.D));
      FQ_TRY(device_transpose(ctx, B.D, nullptr, B.D.ncols, 0, 0, 1, B.Dt, nullptr));
      const int64_t nl = B.D.ncols;
      FQ_TRY(B.t.alloc(ctx, std::max<int64_t>(nl, 1) * 8));
      FQ_TRY(B.t2.alloc(ctx, std::max<int64_t>(nl, 1) * 8));
      if (g == 0) {
        HCsr PiL, PiLt;
        slot_identity(n0, mslots, B.grad_slot, PiL, PiLt);
        FQ_TRY(upload_scalable(ctx, PiL, B.PiL));
        FQ_TRY(upload_scalable(ctx, PiLt, B.PiLt));
      } else {
        FQ_TRY(vector_nodal_device(ctx, m, g, bc, mslots, B.grad_slot, B.PiL, B.PiLt));
      }
      // a gradient smoother of a grade that is neither a block nor the nodal one
      bool have = g == 0;
      for (int o : grades) have = have || o == g;
      for (int o : out.aux_grade) have = have || o == g;
      if (!have) {
        fq_matrix* ag = nullptr;
        FQ_TRY(make_matrix(ctx, m, EK_HDIF, g, bc, FQ_FP64, 0.0, &ag));
        out.aux.emplace_back(ag);
        out.aux_grade.push_back(g);
      }
    }
  }
  return hx_refresh(ctx, m, diag_blocks, out);
}

fq_status hx_refresh(fq_ctx* ctx, fq_mesh* m, const double* diag_blocks, HxPrecond& pc) {
  cudaStream_t st = ctx->stream;
  const int n = m->dim;
  NodalHierarchy& mg = pc.mg;
  // frame spacing from the current lengths
  launch_lattice_spacing(m->lengths.as<double>(), pc.axis_edges.as<int32_t>(), pc.axis_off.data(), n,
                         pc.hprod.as<double>(), pc.flag.as<int>(), st);
  int bad = 0;
  FQ_CUDA(ctx, cudaMemcpyAsync(&bad, pc.flag.p, 4, cudaMemcpyDeviceToHost, st));
  FQ_CUDA(ctx, cudaStreamSynchronize(st));
  if (bad) return set_error(ctx, FQ_UNSUPPORTED, "HX multigrid needs positive squared lengths (a Riemannian metric)");
  auto scale = [&](DCsr& d) {
    if (d.scalable)
      launch_scale_by_mask(d.own_base.as<double>(), d.own_mask.as<uint8_t>(), pc.hprod.as<double>(),
                           d.own_v64.as<double>(), d.nnz, st);
  };
  for (HxBlock& B : pc.blocks) {
    scale(B.Pi);
    scale(B.Pit);
    if (B.grade >= 1) {
      scale(B.PiL);
      scale(B.PiLt);
    }
  }
  // operators: the nodal operator and the Galerkin products
  FQ_TRY(assemble_into(ctx, pc.a0.get()));
  for (auto& a : pc.aux) FQ_TRY(assemble_into(ctx, a.get()));
  mg.lv[0].A.view(pc.a0.get());
  for (size_t l = 0; l < mg.lv.size(); ++l) {
    NodalLevel& L = mg.lv[l];
    FQ_TRY(device_diag_recip(ctx, L.A, kOmega, L.dinv64));
    if (l + 1 < mg.lv.size()) FQ_TRY(galerkin_product(ctx, L.A, L.P, mg.lv[l + 1].A));
  }
  {
    NodalLevel& C = mg.lv.back();
    mg.nc = C.n;
    HCsr hc;
    FQ_TRY(device_to_host(ctx, C.A, hc));
    std::vector<double> dense(size_t(std::max<int64_t>(C.n * C.n, 1)), 0.0);
    for (int64_t r = 0; r < C.n; ++r)
      for (int32_t q = hc.rp[r]; q < hc.rp[r + 1]; ++q) dense[r * C.n + hc.ci[q]] += hc.v[q];
    if (C.n > 0 && !spd_inverse(dense, C.n))
      return set_error(ctx, FQ_UNSUPPORTED, "coarsest nodal operator is not positive definite");
    FQ_TRY(mg.coarse_inv64.alloc(ctx, dense.size() * 8));
    FQ_CUDA(ctx, cudaMemcpyAsync(mg.coarse_inv64.p, dense.data(), dense.size() * 8, cudaMemcpyHostToDevice, st));
  }
  // smoothers
  for (HxBlock& B : pc.blocks) {
    FQ_TRY(device_scaled_recip(ctx, diag_blocks + B.off, B.size, kOmega, B.s64));
    if (B.grade < 1) continue;
    const int g = B.grade - 1;
    const HxBlock* same = nullptr;
    for (const HxBlock& o : pc.blocks)
      if (o.grade == g) same = &o;
    if (same) {
      FQ_TRY(device_scaled_recip(ctx, diag_blocks + same->off, same->size, kOmega, B.sl64));
    } else if (g == 0) {
      FQ_TRY(device_diag_recip(ctx, mg.lv[0].A, kOmega, B.sl64));
    } else {
      for (size_t i = 0; i < pc.aux.size(); ++i)
        if (pc.aux_grade[i] == g) {
          DCsr view;
          view.view(pc.aux[i].get());
          FQ_TRY(device_diag_recip(ctx, view, kOmega, B.sl64));
        }
    }
  }
  FQ_CUDA(ctx, cudaStreamSynchronize(st));
  if (pc.has_f32) {
    pc.has_f32 = false;
    FQ_TRY(pc.make_f32(ctx));
  }
  return FQ_OK;
}

}  // namespace fq
