// C ABI of the sparse direct solver (fq_sparse_lu.h): the factorization of an
// assembled system of a Kuhn mesh, and its FP64 GMRES solve.
#include <algorithm>
#include <cstring>
#include <memory>
#include <vector>

#include "fq_sparse_lu.h"

struct fq_sparse_lu {
  fq_ctx* ctx = nullptr;
  const fq_mesh* mesh = nullptr;
  const fq_matrix* pattern = nullptr;
  fq::SparseLu lu;
};

namespace fq {

fq_status sparse_lu_build(fq_ctx* ctx, const fq_mesh* m, int64_t n, const int32_t* rp, const int32_t* ci,
                          const std::vector<int32_t>& dofv, SparseLu& lu) {
  if (m->kuhn_nbox <= 0) return set_error(ctx, FQ_UNSUPPORTED, "sparse LU: needs a Kuhn cube mesh (fq_mesh_kuhn_cube)");
  if (int64_t(dofv.size()) != 5 * n) return set_error(ctx, FQ_INVALID_ARG, "sparse LU: one vertex list per unknown");
  std::vector<int32_t> hrp(static_cast<size_t>(n) + 1);
  FQ_CUDA(ctx, cudaMemcpyAsync(hrp.data(), rp, (n + 1) * 4, cudaMemcpyDeviceToHost, ctx->stream));
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  const int64_t nnz = hrp[n];
  std::vector<int32_t> hci(static_cast<size_t>(std::max<int64_t>(nnz, 1)));
  if (nnz > 0) FQ_CUDA(ctx, cudaMemcpyAsync(hci.data(), ci, nnz * 4, cudaMemcpyDeviceToHost, ctx->stream));
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return sparse_lu_analyse(ctx, lu, m->dim, m->kuhn_nbox, n, hrp.data(), hci.data(), dofv.data());
}

}  // namespace fq

using namespace fq;

extern "C" {

fq_status fq_sparse_lu_create(fq_ctx* ctx, fq_mesh* mesh, const fq_matrix* a, fq_sparse_lu** out) {
  if (!ctx || !mesh || !a || !out) return FQ_INVALID_ARG;
  *out = nullptr;
  if (a->mesh != mesh || (!a->plan && a->kind != EK_KKT))
    return set_error(ctx, FQ_INVALID_ARG, "sparse LU: an assembled system of this mesh (fq_assemble, fq_dirac_system, "
                                          "fq_mixed_system)");
  if (a->nrows != a->ncols) return set_error(ctx, FQ_INVALID_ARG, "sparse LU: the matrix must be square");
  if (a->precision != FQ_FP64 && a->precision != FQ_FP64_IEEE)
    return set_error(ctx, FQ_INVALID_ARG, "sparse LU: the matrix must hold FP64 values");
  FQ_GUARD_BEGIN
  auto s = std::make_unique<fq_sparse_lu>();
  s->ctx = ctx;
  s->mesh = mesh;
  s->pattern = a;
  std::vector<int32_t> dofv;
  FQ_TRY(layout_dof_vertices(ctx, mesh, a->kind, a->grade, a->bc, a->nrows, dofv));
  FQ_TRY(sparse_lu_build(ctx, mesh, a->nrows, a->rp, a->ci, dofv, s->lu));
  *out = s.release();
  return FQ_OK;
  FQ_GUARD_END(ctx)
}

fq_status fq_sparse_lu_factor(fq_sparse_lu* s, const fq_matrix* a, int precision) {
  if (!s || !a) return FQ_INVALID_ARG;
  if (precision != FQ_FP32 && precision != FQ_FP64 && precision != FQ_FP64_IEEE)
    return set_error(s->ctx, FQ_INVALID_ARG, "sparse LU: factors in FQ_FP32, FQ_FP64 or FQ_FP64_IEEE");
  if (a->nrows != s->lu.n || a->nnz != s->lu.nnz)
    return set_error(s->ctx, FQ_INVALID_ARG, "sparse LU: the matrix's pattern is not the analysed one");
  FQ_GUARD_BEGIN
  return sparse_lu_factor(s->ctx, s->lu, a->rp, a->ci, a->values.as<double>(), precision);
  FQ_GUARD_END(s->ctx)
}

fq_status fq_sparse_lu_solve(fq_sparse_lu* s, const fq_matrix* a, const double* b, double* x,
                             const fq_solve_opts* opts, fq_report* rep) {
  if (!s || !a || !b || !x) return FQ_INVALID_ARG;
  if (!s->lu.factored) return set_error(s->ctx, FQ_INVALID_ARG, "sparse LU: factor first");
  if (a->nrows != s->lu.n || a->nnz != s->lu.nnz)
    return set_error(s->ctx, FQ_INVALID_ARG, "sparse LU: the matrix's pattern is not the analysed one");
  fq_solve_opts d;
  fq_default_solve_opts(&d);
  if (!opts) opts = &d;
  FQ_GUARD_BEGIN
  if (opts->max_refinements == 0) {
    fq_report r{};
    const fq_status st = sparse_lu_gmres(s->ctx, s->lu, a->rp, a->ci, a->values.as<double>(), b, x, opts->rtol,
                                         opts->max_iters, &r);
    r.refinements = 0;
    if (rep) *rep = r;
    return st;
  }
  return sparse_lu_solve(s->ctx, s->lu, a->rp, a->ci, a->values.as<double>(), b, x, opts->rtol, opts->max_iters, rep);
  FQ_GUARD_END(s->ctx)
}

fq_status fq_sparse_lu_info(const fq_sparse_lu* s, int64_t* fronts, int64_t* levels, double* flops,
                            int64_t* factor_bytes, int64_t* perturbed_pivots) {
  if (!s) return FQ_INVALID_ARG;
  if (fronts) *fronts = s->lu.nfronts;
  if (levels) *levels = s->lu.nlevels;
  if (flops) *flops = s->lu.flops;
  if (factor_bytes) *factor_bytes = (s->lu.pool_elems + s->lu.tile_elems) * (s->lu.precision == FQ_FP32 ? 4 : 8);
  if (perturbed_pivots) *perturbed_pivots = s->lu.perturbed;
  return FQ_OK;
}

void fq_sparse_lu_destroy(fq_sparse_lu* s) { delete s; }

fq_status fq_sparse_lu_analyse_host(int dim, int nbox, int64_t n, const int32_t* rp, const int32_t* ci,
                                    const int32_t* dof_vertices, double* stats) {
  if (!rp || !ci || !dof_vertices || !stats) return FQ_INVALID_ARG;
  FQ_GUARD_BEGIN
  SparseLu lu;
  SparseLuMaps mp;
  FQ_TRY(sparse_lu_analyse_host(nullptr, lu, dim, nbox, n, rp, ci, dof_vertices, mp));
  int64_t maxm = 0, sumf = 0;
  for (int x = 0; x < lu.nfronts; ++x) {
    maxm = std::max<int64_t>(maxm, lu.front_m[x]);
    sumf += lu.front_f[x];
  }
  stats[0] = lu.nfronts;
  stats[1] = lu.nlevels;
  stats[2] = lu.flops;
  stats[3] = double(lu.pool_elems + lu.tile_elems) * 4.0;
  stats[4] = double(maxm);
  stats[5] = double(sumf);
  return FQ_OK;
  FQ_GUARD_END(nullptr)
}

}  // extern "C"
