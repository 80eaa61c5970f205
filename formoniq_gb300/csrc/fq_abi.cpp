// The extern "C" boundary (include/formoniq_gpu.h) and the host drivers behind
// it. Every entry point catches every C++ exception and converts CUDA errors to
// fq_status; nothing unwinds across the ABI.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <exception>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "fq_hx.h"
#include "fq_sparse_lu.h"
#include "fq_internal.h"

namespace fq {

fq_status build_topology(fq_ctx* ctx, fq_mesh* m, int dim, int64_t ncells, const int32_t* cells);
std::vector<int32_t> kuhn_cells(int dim, int nbox);
double uniform_pm1(uint64_t seed, uint64_t counter);
void compute_orientation(fq_mesh* m, const std::vector<int32_t>& facet_of_cell);

template <typename VT>
fq_status minres_run(fq_ctx*, const int32_t*, const int32_t*, const VT*, int64_t, int64_t, const VT*,
                     const HxPrecond*, const VT*, VT*, double, int64_t, fq_report*);
template <typename VT>
fq_status cg_run(fq_ctx*, const int32_t*, const int32_t*, const VT*, int64_t, int64_t, const VT*, const HxPrecond*,
                 const VT*, VT*, double, int64_t, fq_report*);
fq_status residual64(fq_ctx*, const int32_t*, const int32_t*, const double*, int64_t, const double*, const double*,
                     double*, double*, double*);
void launch_to_float(const double* a, float* o, int64_t n, cudaStream_t st);
void launch_to_float_scaled(const double* a, float* o, double s, int64_t n, cudaStream_t st);
void launch_axpy_from_float(double* x, const float* d, double s, int64_t n, cudaStream_t st);
void vec_diag(const fq_matrix* a, double* d, cudaStream_t st);
void vec_recip(const double* d, double* inv, float* inv32, int64_t n, int absval, cudaStream_t st);
void vec_gather(const double* in, const int32_t* map, double* out, int64_t n, cudaStream_t st);
void vec_scatter_map(const double* in, const int32_t* map, double* out, int64_t n, cudaStream_t st);
void vec_sub(double* a, const double* b, int64_t n, cudaStream_t st);
void vec_add(double* a, const double* b, int64_t n, cudaStream_t st);
void vec_fill(double* a, double v, int64_t n, cudaStream_t st);
void vec_scale(double* a, double s, int64_t n, cudaStream_t st);
fq_status border_csr(fq_ctx* ctx, const fq_matrix* a, const double* mh, int64_t ns, int64_t nu, DevBuf& nrp,
                     DevBuf& nci, DevBuf& nval);
fq_status count_indefinite_cells(fq_ctx* ctx, const fq_mesh* m, int64_t* out);

// ---- DevBuf -----------------------------------------------------------------
DevBuf& DevBuf::operator=(DevBuf&& o) noexcept {
  if (this != &o) {
    release();
    ctx = o.ctx;
    p = o.p;
    bytes = o.bytes;
    o.ctx = nullptr;
    o.p = nullptr;
    o.bytes = 0;
  }
  return *this;
}

fq_status DevBuf::alloc(fq_ctx* c, size_t nbytes) {
  release();
  if (nbytes == 0) nbytes = 16;
  if (c->budget && c->in_use + nbytes > c->budget)
    return set_error(c, FQ_OOM_BUDGET, "HBM budget exceeded: " + std::to_string(c->in_use + nbytes) + " > " +
                                           std::to_string(c->budget) + " bytes");
  // Stream-ordered allocation from the device's memory pool: neither this nor
  // the matching free synchronizes the device, so contexts on other streams (the
  // lanes of a server) keep running while one allocates.
  void* q = nullptr;
  cudaError_t e = cudaMallocAsync(&q, nbytes, c->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(c, e == cudaErrorMemoryAllocation ? FQ_OOM_BUDGET : FQ_CUDA_ERROR,
                     std::string("cudaMallocAsync: ") + cudaGetErrorString(e));
  }
  ctx = c;
  p = q;
  bytes = nbytes;
  c->in_use += nbytes;
  return FQ_OK;
}

void DevBuf::release() {
  if (p) {
    if (ctx) {
      cudaFreeAsync(p, ctx->stream);  // after the work already queued on the owner's stream
      ctx->in_use -= bytes;
    } else {
      cudaFree(p);
    }
  }
  p = nullptr;
  bytes = 0;
  ctx = nullptr;
}

fq_status dev_alloc(fq_ctx* ctx, DevBuf& b, size_t bytes) { return b.alloc(ctx, bytes); }

fq_status set_error(fq_ctx* ctx, fq_status s, const std::string& msg) {
  if (ctx) ctx->last_error = msg;
  return s;
}

fq_status cuda_check(fq_ctx* ctx, cudaError_t e, const char* what) {
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  return set_error(ctx, FQ_CUDA_ERROR, m);
}

fq_status make_matrix(fq_ctx* ctx, fq_mesh* mesh, int kind, int grade, int bc, int precision, double param,
                      fq_matrix** out) {
  Plan* plan = nullptr;
  FQ_TRY(get_plan(ctx, mesh, kind, grade, bc, bc, &plan));
  auto* m = new fq_matrix();
  m->ctx = ctx;
  m->mesh = mesh;
  m->plan = plan;
  m->kind = kind;
  m->grade = grade;
  m->bc = bc;
  m->precision = precision;
  m->param = param;
  m->nrows = plan->nrows;
  m->ncols = plan->ncols;
  fq_status s = assemble_into(ctx, m);
  if (s != FQ_OK) {
    delete m;
    return s;
  }
  *out = m;
  return FQ_OK;
}

// Relative -> ambient index list of grade k (device), built on demand.
static fq_status interior_list(fq_ctx* ctx, fq_mesh* m, int k, DevBuf& out) {
  std::vector<int32_t> lst;
  for (int64_t i = 0; i < m->nsimp[k]; ++i)
    if (!m->boundary[k][i]) lst.push_back(int32_t(i));
  FQ_TRY(out.alloc(ctx, std::max<size_t>(lst.size(), 1) * 4));
  if (!lst.empty())
    FQ_CUDA(ctx, cudaMemcpyAsync(out.p, lst.data(), lst.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return FQ_OK;
}

static int64_t ndofs(const fq_mesh* m, int k, int bc) {
  if (k < 0 || k > m->dim) return 0;
  return bc == FQ_RELATIVE ? m->ninterior[k] : m->nsimp[k];
}

static bool valid_form_shape(const fq_mesh* m, int form, int grade, int bc, int64_t* rows, int64_t* cols) {
  const int tg = (form == FQ_DIF_TEST || form == FQ_DIF_BOTH) ? grade - 1 : grade;
  const int sg = (form == FQ_DIF_TRIAL || form == FQ_DIF_BOTH) ? grade - 1 : grade;
  *rows = ndofs(m, tg, bc);
  *cols = ndofs(m, sg, bc);
  return *rows > 0 && *cols > 0;
}

static fq_status empty_matrix(fq_ctx* ctx, fq_mesh* mesh, int64_t rows, int64_t cols, int precision,
                              fq_matrix** out) {
  auto* m = new fq_matrix();
  m->ctx = ctx;
  m->mesh = mesh;
  m->nrows = rows;
  m->ncols = cols;
  m->nnz = 0;
  m->precision = precision;
  fq_status s = m->row_ptr.alloc(ctx, (rows + 1) * 4);
  if (s == FQ_OK) s = m->col_idx.alloc(ctx, 4);
  if (s == FQ_OK) s = m->values.alloc(ctx, 8);
  if (s != FQ_OK) {
    delete m;
    return s;
  }
  cudaMemsetAsync(m->row_ptr.p, 0, (rows + 1) * 4, ctx->stream);
  cudaStreamSynchronize(ctx->stream);
  m->rp = m->row_ptr.as<int32_t>();
  m->ci = m->col_idx.as<int32_t>();
  *out = m;
  return FQ_OK;
}

// Coboundary D_k (Complex::coboundary_operator, topology/complex.rs:215-217):
// rows the (k+1)-simplices, entry (-1)^p at the face omitting vertex position p;
// the relative complex keeps interior simplices on both sides.

}  // namespace fq

using namespace fq;

// ============================================================================
// The mixed Hodge-Laplace problem
// ============================================================================
struct fq_mixed {
  fq_ctx* ctx = nullptr;
  fq_mesh* mesh = nullptr;
  int grade = 0, bc = 0, precision = 0;
  int64_t ns = 0, nu = 0, nh = 0, n = 0;
  fq_matrix* kkt = nullptr;    // FP64, unbordered
  fq_matrix* kkt32 = nullptr;  // FP32 element values (FQ_FP32)
  DevBuf diag, dinv;           // FP64 preconditioner diagonal / reciprocal (size n)
  DevBuf dinv32;
  DevBuf mh;                   // border M_k h (size nu) when nh = 1
  DevBuf brp, bci, bval, brp32, bci32, bval32;  // bordered systems
  DevBuf list_sigma, list_u;   // relative -> ambient maps
  // system actually solved
  const int32_t* rp = nullptr;
  const int32_t* ci = nullptr;
  const double* val = nullptr;
  int64_t nnz = 0;
  const int32_t* rp32 = nullptr;
  const int32_t* ci32 = nullptr;
  const float* val32 = nullptr;
  int64_t nnz32 = 0;
  fq_matrix sysview;  // non-owning view handed out by fq_mixed_system
  // HX-multigrid block preconditioner, built at the first solve that asks for it
  // and rebuilt after a reassembly; hx_failed remembers an FQ_PC_AUTO fallback
  std::unique_ptr<HxPrecond> hx;
  bool hx_stale = true, hx_failed = false;
  // the sparse direct route (Kuhn meshes): the LU carries the Lorentzian solve
  // and finishes an unconverged MINRES (elliptic.rs:147-160); the analysis
  // is kept while the pattern stays, the factors while the values stay
  std::unique_ptr<SparseLu> lu;
  int indefinite = -1;  // cells with an indefinite metric > 0: 1; none: 0; not yet counted: -1
  ~fq_mixed() {
    delete kkt;
    delete kkt32;
  }
};

namespace fq {

// Harmonic border of the contractible case: b_0 = 1 on the full complex
// (constants), b_n = 1 on the relative complex (M_n^{-1} z, z the coherent
// orientation); every other Betti number of a contractible mesh is zero.
static fq_status mixed_harmonic(fq_mixed* P) {
  fq_ctx* ctx = P->ctx;
  fq_mesh* m = P->mesh;
  const int n = m->dim, k = P->grade;
  P->nh = 0;
  if (P->bc == FQ_ABSOLUTE && k == 0) P->nh = 1;
  if (P->bc == FQ_RELATIVE && k == n) P->nh = 1;
  if (!P->nh) return FQ_OK;
  FQ_TRY(P->mh.alloc(ctx, std::max<int64_t>(P->nu, 1) * 8));
  fq_matrix* mass = nullptr;
  FQ_TRY(make_matrix(ctx, m, EK_MASS, k, P->bc, FQ_FP64, 0.0, &mass));
  std::unique_ptr<fq_matrix> guard(mass);
  const int64_t nu = P->nu;
  DevBuf tmp, g;
  FQ_TRY(tmp.alloc(ctx, nu * 8));
  FQ_TRY(g.alloc(ctx, nu * 8));
  std::vector<double> host(nu);
  if (k == 0 && P->bc == FQ_ABSOLUTE) {
    vec_fill(tmp.as<double>(), 1.0, nu, ctx->stream);
    launch_spmv(mass, tmp.p, P->mh.p, ctx->stream);  // M 1
    FQ_CUDA(ctx, cudaMemcpyAsync(host.data(), P->mh.p, nu * 8, cudaMemcpyDeviceToHost, ctx->stream));
    FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    double s = 0.0;
    for (double v : host) s += v;  // 1^T M 1
    vec_scale(P->mh.as<double>(), 1.0 / std::sqrt(s), nu, ctx->stream);
  } else {
    if (m->orientation.empty()) {
      if (n == 0) {
        m->orientation.assign(size_t(m->ncells), 1);
      } else {
        compute_orientation(m, m->cell_faces_host[n - 1]);
      }
    }
    std::vector<double> z(nu);
    for (int64_t i = 0; i < nu; ++i) z[i] = m->orientation[i];
    FQ_CUDA(ctx, cudaMemcpyAsync(tmp.p, z.data(), nu * 8, cudaMemcpyHostToDevice, ctx->stream));
    DevBuf d, dinv;
    FQ_TRY(d.alloc(ctx, nu * 8));
    FQ_TRY(dinv.alloc(ctx, nu * 8));
    vec_diag(mass, d.as<double>(), ctx->stream);
    vec_recip(d.as<double>(), dinv.as<double>(), nullptr, nu, 0, ctx->stream);
    fq_report rep{};
    FQ_TRY(cg_run<double>(ctx, mass->rp, mass->ci, mass->values.as<double>(), nu, mass->nnz, dinv.as<double>(),
                          nullptr, tmp.as<double>(), g.as<double>(), 1e-14, 10000, &rep));
    std::vector<double> gh(nu);
    FQ_CUDA(ctx, cudaMemcpyAsync(gh.data(), g.p, nu * 8, cudaMemcpyDeviceToHost, ctx->stream));
    FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    double s = 0.0;
    for (int64_t i = 0; i < nu; ++i) s += gh[i] * z[i];  // z^T M^{-1} z
    // M h = z / sqrt(z^T M^{-1} z)
    FQ_CUDA(ctx, cudaMemcpyAsync(P->mh.p, tmp.p, nu * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    vec_scale(P->mh.as<double>(), 1.0 / std::sqrt(s), nu, ctx->stream);
  }
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return FQ_OK;
}

static fq_status mixed_assemble(fq_mixed* P) {
  fq_ctx* ctx = P->ctx;
  fq_mesh* m = P->mesh;
  P->hx_stale = true;
  P->indefinite = -1;
  if (P->lu) P->lu->factored = false;
  if (P->kkt) {
    FQ_TRY(assemble_into(ctx, P->kkt));
  } else {
    FQ_TRY(make_matrix(ctx, m, EK_KKT, P->grade, P->bc, FQ_FP64, 0.0, &P->kkt));
  }
  // preconditioner diagonal from the same element pass (mesh->elem still holds it)
  const int64_t n0 = P->ns + P->nu;
  FQ_TRY(P->diag.alloc(ctx, std::max<int64_t>(P->n, 1) * 8));
  FQ_TRY(P->dinv.alloc(ctx, std::max<int64_t>(P->n, 1) * 8));
  launch_scatter_diag(*P->kkt->plan, m->elem.p, P->diag.as<double>(), P->kkt->precision, ctx->stream);
  ctx->launches++;
  if (P->nh) vec_fill(P->diag.as<double>() + n0, 1.0, P->nh, ctx->stream);
  FQ_TRY(mixed_harmonic(P));
  if (P->precision == FQ_FP32) {
    FQ_TRY(P->dinv32.alloc(ctx, std::max<int64_t>(P->n, 1) * 4));
    vec_recip(P->diag.as<double>(), P->dinv.as<double>(), P->dinv32.as<float>(), P->n, 0, ctx->stream);
    if (P->kkt32) {
      FQ_TRY(assemble_into(ctx, P->kkt32));
    } else {
      FQ_TRY(make_matrix(ctx, m, EK_KKT, P->grade, P->bc, FQ_FP32, 0.0, &P->kkt32));
    }
  } else {
    vec_recip(P->diag.as<double>(), P->dinv.as<double>(), nullptr, P->n, 0, ctx->stream);
  }
  if (P->nh) {
    FQ_TRY(border_csr(ctx, P->kkt, P->mh.as<double>(), P->ns, P->nu, P->brp, P->bci, P->bval));
    P->rp = P->brp.as<int32_t>();
    P->ci = P->bci.as<int32_t>();
    P->val = P->bval.as<double>();
    P->nnz = P->kkt->nnz + 2 * P->nu;
    if (P->kkt32) {
      FQ_TRY(border_csr(ctx, P->kkt32, P->mh.as<double>(), P->ns, P->nu, P->brp32, P->bci32, P->bval32));
      P->rp32 = P->brp32.as<int32_t>();
      P->ci32 = P->bci32.as<int32_t>();
      P->val32 = P->bval32.as<float>();
      P->nnz32 = P->kkt32->nnz + 2 * P->nu;
    }
  } else {
    P->rp = P->kkt->rp;
    P->ci = P->kkt->ci;
    P->val = P->kkt->values.as<double>();
    P->nnz = P->kkt->nnz;
    if (P->kkt32) {
      P->rp32 = P->kkt32->rp;
      P->ci32 = P->kkt32->ci;
      P->val32 = P->kkt32->values.as<float>();
      P->nnz32 = P->kkt32->nnz;
    }
  }
  P->sysview.ctx = ctx;
  P->sysview.mesh = m;
  P->sysview.kind = EK_KKT;  // the layout of its unknowns (a border row last)
  P->sysview.grade = P->grade;
  P->sysview.bc = P->bc;
  P->sysview.nrows = P->sysview.ncols = P->n;
  P->sysview.nnz = P->nnz;
  P->sysview.precision = FQ_FP64;
  P->sysview.rp = P->rp;
  P->sysview.ci = P->ci;
  P->sysview.values.p = const_cast<double*>(P->val);  // non-owning
  P->sysview.values.ctx = nullptr;
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return FQ_OK;
}

// Solve the assembled (bordered) system for rhs (device, size n) into x (device).
// The block preconditioner the options ask for: HX-multigrid blocks for the
// grades k-1 and k (the blocks hdif_gram(k-1), hdif_gram(k) of
// mixed_block_preconditioner, problems/elliptic.rs:29-47), or null for the
// Jacobi diagonal.
static fq_status mixed_precond(fq_mixed* P, const fq_solve_opts* o, const HxPrecond** out) {
  *out = nullptr;
  const int want = o->preconditioner;
  if (want == FQ_PC_JACOBI) return FQ_OK;
  if (want != FQ_PC_AUTO && want != FQ_PC_HX) return set_error(P->ctx, FQ_INVALID_ARG, "unknown preconditioner");
  if (!P->hx_stale) {
    if (P->hx && !P->hx_failed) {
      *out = P->hx.get();
      return FQ_OK;
    }
    if (P->hx_failed && want == FQ_PC_AUTO) return FQ_OK;  // Jacobi, as decided for these lengths
  }
  std::vector<int> grades;
  if (P->grade >= 1) grades.push_back(P->grade - 1);
  grades.push_back(P->grade);
  fq_status s = FQ_OK;
  if (!hx_supported(P->mesh)) {
    s = set_error(P->ctx, FQ_UNSUPPORTED, "HX multigrid needs a Kuhn cube mesh");
  } else if (P->hx && hx_matches(*P->hx, P->mesh, P->bc, grades, P->nh)) {
    // new lengths on the same mesh: keep the lattice structure, refresh the numbers
    s = hx_refresh(P->ctx, P->mesh, P->diag.as<double>(), *P->hx);
  } else {
    auto hx = std::make_unique<HxPrecond>();
    s = hx_build(P->ctx, P->mesh, P->bc, grades, P->nh, P->diag.as<double>(), *hx);
    if (s == FQ_OK) P->hx = std::move(hx);
  }
  if (s == FQ_OK && P->precision == FQ_FP32) s = P->hx->make_f32(P->ctx);
  P->hx_stale = false;
  P->hx_failed = s != FQ_OK;
  if (s != FQ_OK) return want == FQ_PC_HX ? s : FQ_OK;  // FQ_PC_AUTO: Jacobi
  *out = P->hx.get();
  return FQ_OK;
}

// GMRES iterations the sparse LU may take when it finishes an unconverged
// Krylov solve (whatever that solve's own cap was)
static constexpr int64_t kLuFallbackIters = 300;

// The whole KKT system by the sparse direct solver: GMRES in FP64 on the
// system, preconditioned by its LU (FP32 factors first, FP64 when those do not
// converge; report.refinements = 1 then). The factors stay for the next solve
// on the same values.
static fq_status mixed_direct(fq_mixed* P, const double* rhs, double* x, double rtol, int64_t max_iters,
                              fq_report* rep, bool float_float_first = false) {
  fq_ctx* ctx = P->ctx;
  if (!P->lu || P->lu->n != P->n || P->lu->nnz != P->nnz) {
    std::vector<int32_t> dofv;
    FQ_TRY(layout_dof_vertices(ctx, P->mesh, EK_KKT, P->grade, P->bc, P->n, dofv));
    auto lu = std::make_unique<SparseLu>();
    FQ_TRY(sparse_lu_build(ctx, P->mesh, P->n, P->rp, P->ci, dofv, *lu));
    P->lu = std::move(lu);
  }
  // Lorentzian systems: float-float factors at once (FP32 factors of the
  // Minkowski KKT systems stop converging from about 1.5e4 unknowns)
  if (float_float_first && !P->lu->factored) FQ_TRY(sparse_lu_factor(ctx, *P->lu, P->rp, P->ci, P->val, FQ_FP64));
  fq_report r{};
  const fq_status s = sparse_lu_solve(ctx, *P->lu, P->rp, P->ci, P->val, rhs, x, rtol, max_iters, &r);
  if (s != FQ_OK && s != FQ_NOT_CONVERGED) return s;
  *rep = r;
  return FQ_OK;
}

// The signature guard: whether a cell metric of the mesh is not positive
// definite (then a block of the preconditioner is indefinite and the sparse
// LU carries the solve, as FaerLu does in elliptic.rs:153-160).
static fq_status mixed_indefinite(fq_mixed* P, bool* out) {
  if (P->indefinite < 0) {
    int64_t c = 0;
    FQ_TRY(count_indefinite_cells(P->ctx, P->mesh, &c));
    P->indefinite = c > 0 ? 1 : 0;
  }
  *out = P->indefinite == 1;
  return FQ_OK;
}

static fq_status mixed_krylov(fq_mixed* P, const double* rhs, double* x, const fq_solve_opts* o, fq_report* rep) {
  fq_ctx* ctx = P->ctx;
  const int64_t n = P->n;
  rep->refinements = 0;
  const bool kuhn = P->mesh->kuhn_nbox > 0;
  if (o->preconditioner == FQ_PC_DIRECT && !kuhn)
    return set_error(ctx, FQ_UNSUPPORTED, "the sparse direct solve needs a Kuhn cube mesh (fq_mesh_kuhn_cube)");
  bool indefinite = false;
  if (kuhn && o->preconditioner == FQ_PC_AUTO) FQ_TRY(mixed_indefinite(P, &indefinite));
  if (kuhn && (o->preconditioner == FQ_PC_DIRECT || indefinite))
    return mixed_direct(P, rhs, x, o->rtol, o->max_iters, rep, indefinite);
  const HxPrecond* pc = nullptr;
  FQ_TRY(mixed_precond(P, o, &pc));
  if (P->precision != FQ_FP32 || !P->kkt32) {
    FQ_TRY(minres_run<double>(ctx, P->rp, P->ci, P->val, n, P->nnz, P->dinv.as<double>(), pc, rhs, x, o->rtol,
                              o->max_iters, rep));
    // LU catches the rare non-convergence of the iterative path (elliptic.rs:147-159): the
    // sparse direct solver on Kuhn meshes (its GMRES is not held to the MINRES cap: FaerLu
    // has none), a dense factorization for small other systems
    if (!rep->converged && kuhn) {
      const int64_t its = rep->iters;
      FQ_TRY(mixed_direct(P, rhs, x, o->rtol, std::max<int64_t>(o->max_iters, kLuFallbackIters), rep));
      rep->iters += its;
    } else if (!rep->converged && ctx->dense_fallback && n <= kDenseMax && dense_fallback_available()) {
      FQ_TRY(dense_lu_solve(ctx, P->rp, P->ci, P->val, n, rhs, x));
      rep->converged = 1;
    }
  } else {
    // FP64 residual and update around an FP32 MINRES (iterative refinement).
    DevBuf r, r32, d32;
    FQ_TRY(r.alloc(ctx, std::max<int64_t>(n, 1) * 8));
    FQ_TRY(r32.alloc(ctx, std::max<int64_t>(n, 1) * 4));
    FQ_TRY(d32.alloc(ctx, std::max<int64_t>(n, 1) * 4));
    FQ_CUDA(ctx, cudaMemsetAsync(x, 0, std::max<int64_t>(n, 1) * 8, ctx->stream));
    int64_t total = 0;
    fq_report inner{};
    for (int64_t ref = 0; ref <= o->max_refinements; ++ref) {
      double rn = 0, bn = 0;
      FQ_TRY(residual64(ctx, P->rp, P->ci, P->val, n, x, rhs, r.as<double>(), &rn, &bn));
      if (bn == 0.0 || rn <= o->refine_rtol * bn || ref == o->max_refinements) break;
      launch_to_float_scaled(r.as<double>(), r32.as<float>(), 1.0 / rn, n, ctx->stream);
      FQ_TRY(minres_run<float>(ctx, P->rp32, P->ci32, P->val32, n, P->nnz32, P->dinv32.as<float>(), pc,
                               r32.as<float>(), d32.as<float>(), o->rtol, o->max_iters, &inner));
      launch_axpy_from_float(x, d32.as<float>(), rn, n, ctx->stream);
      total += inner.iters;
      rep->refinements++;
    }
    rep->iters = total;
    rep->residual = inner.residual;
    rep->converged = inner.converged;
  }
  // true FP64 residual
  DevBuf r;
  FQ_TRY(r.alloc(ctx, std::max<int64_t>(n, 1) * 8));
  double rn = 0, bn = 0;
  FQ_TRY(residual64(ctx, P->rp, P->ci, P->val, n, x, rhs, r.as<double>(), &rn, &bn));
  rep->true_residual = bn > 0 ? rn / bn : 0.0;
  if (P->precision == FQ_FP32) {
    rep->converged = rep->true_residual <= o->refine_rtol;
    // the refinement did not reach its tolerance: the sparse LU finishes it
    if (!rep->converged && kuhn) {
      const int64_t its = rep->iters;
      FQ_TRY(mixed_direct(P, rhs, x, o->refine_rtol, std::max<int64_t>(o->max_iters, kLuFallbackIters), rep));
      rep->iters += its;
    }
  }
  return FQ_OK;
}

}  // namespace fq

// ============================================================================
// extern "C"
// ============================================================================

extern "C" {

const char* fq_status_name(fq_status s) {
  switch (s) {
    case FQ_OK:
      return "FQ_OK";
    case FQ_INVALID_ARG:
      return "FQ_INVALID_ARG";
    case FQ_DEGENERATE_CELL:
      return "FQ_DEGENERATE_CELL";
    case FQ_NOT_CONVERGED:
      return "FQ_NOT_CONVERGED";
    case FQ_BREAKDOWN:
      return "FQ_BREAKDOWN";
    case FQ_OOM_BUDGET:
      return "FQ_OOM_BUDGET";
    case FQ_TIMEOUT:
      return "FQ_TIMEOUT";
    case FQ_CUDA_ERROR:
      return "FQ_CUDA_ERROR";
    case FQ_NO_DEVICE:
      return "FQ_NO_DEVICE";
    case FQ_UNSUPPORTED:
      return "FQ_UNSUPPORTED";
  }
  return "FQ_UNKNOWN";
}

void fq_default_solve_opts(fq_solve_opts* o) {
  if (!o) return;
  o->rtol = 1e-10;
  o->max_iters = 10000;
  o->precision = FQ_FP64;
  o->refine_rtol = 1e-12;
  o->max_refinements = 6;
  o->preconditioner = FQ_PC_AUTO;
}

fq_status fq_ctx_create(int device, void* stream, uint64_t budget, fq_ctx** out) {
  if (!out) return FQ_INVALID_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return FQ_NO_DEVICE;
  }
  if (device < 0 || device >= ndev) return FQ_INVALID_ARG;
  auto* ctx = new (std::nothrow) fq_ctx();
  if (!ctx) return FQ_OOM_BUDGET;
  ctx->device = device;
  ctx->budget = budget;
  if (cudaSetDevice(device) != cudaSuccess) {
    delete ctx;
    return FQ_CUDA_ERROR;
  }
  if (stream) {
    ctx->stream = static_cast<cudaStream_t>(stream);
  } else {
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
      delete ctx;
      return FQ_CUDA_ERROR;
    }
    ctx->owns_stream = true;
  }
  {
    // keep freed pool memory with the process instead of returning it at every
    // synchronization, so steady-state solves do not go back to the driver
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
      uint64_t keep = UINT64_MAX;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
  }
  if (ctx->status.alloc(ctx, 8 * sizeof(int)) != FQ_OK ||
      cudaMallocHost(reinterpret_cast<void**>(&ctx->host_status), 8 * sizeof(int)) != cudaSuccess ||
      cudaMallocHost(&ctx->host_solver, 1024) != cudaSuccess) {
    fq_ctx_destroy(ctx);
    return FQ_CUDA_ERROR;
  }
  cudaMemsetAsync(ctx->status.p, 0, 8 * sizeof(int), ctx->stream);
  *out = ctx;
  return FQ_OK;
}

void fq_ctx_destroy(fq_ctx* ctx) {
  if (!ctx) return;
  cudaStreamSynchronize(ctx->stream);
  for (auto& e : ctx->ev)
    if (e) cudaEventDestroy(e);
  for (auto e : ctx->prof_events) cudaEventDestroy(e);
  for (auto e : ctx->copy_events) cudaEventDestroy(e);
  if (ctx->copy_stream) {
    cudaStreamSynchronize(ctx->copy_stream);
    cudaStreamDestroy(ctx->copy_stream);
  }
  ctx->status.release();
  ctx->scratch.release();
  cudaStreamSynchronize(ctx->stream);
  if (ctx->host_status) cudaFreeHost(ctx->host_status);
  if (ctx->host_solver) cudaFreeHost(ctx->host_solver);
  if (ctx->owns_stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

const char* fq_ctx_last_error(const fq_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

fq_status fq_ctx_synchronize(fq_ctx* ctx) {
  if (!ctx) return FQ_INVALID_ARG;
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return FQ_OK;
}

uint64_t fq_ctx_bytes_in_use(const fq_ctx* ctx) { return ctx ? ctx->in_use : 0; }

fq_status fq_ctx_set_profiling(fq_ctx* ctx, int enable) {
  if (!ctx) return FQ_INVALID_ARG;
  if (enable && !ctx->ev[0]) {
    for (auto& e : ctx->ev) FQ_CUDA(ctx, cudaEventCreate(&e));
  }
  ctx->profiling = enable != 0;
  return FQ_OK;
}

fq_status fq_ctx_profile(fq_ctx* ctx, double* ms, int64_t* launches, int nslots, int reset) {
  if (!ctx) return FQ_INVALID_ARG;
  for (int i = 0; i < nslots && i < 4; ++i) {
    if (ms) ms[i] = ctx->prof_ms[i];
    if (launches) launches[i] = ctx->prof_n[i];
  }
  if (reset)
    for (int i = 0; i < 4; ++i) {
      ctx->prof_ms[i] = 0.0;
      ctx->prof_n[i] = 0;
    }
  return FQ_OK;
}
uint64_t fq_ctx_kernel_launches(const fq_ctx* ctx) { return ctx ? ctx->launches : 0; }

fq_status fq_ctx_set_scatter_shape(fq_ctx* ctx, int slots_per_thread, int blocks_per_sm) {
  if (!ctx) return FQ_INVALID_ARG;
  if (!(slots_per_thread == -1 || slots_per_thread == 0 || slots_per_thread == 1 || slots_per_thread == 2 ||
        slots_per_thread == 4 || slots_per_thread == 8) ||
      blocks_per_sm < 0 || blocks_per_sm > 8)
    return set_error(ctx, FQ_INVALID_ARG, "scatter shape: slots per thread in {-1,0,1,2,4,8}, blocks per SM in 0..8");
  ctx->scatter_shape.slots_per_thread = slots_per_thread;
  ctx->scatter_shape.blocks_per_sm = blocks_per_sm;
  return FQ_OK;
}

// ---- meshes -----------------------------------------------------------------
fq_status fq_mesh_from_cells(fq_ctx* ctx, int dim, int64_t ncells, const int32_t* cells, fq_mesh** out) {
  if (!ctx || !out) return FQ_INVALID_ARG;
  *out = nullptr;
  if (dim < 0 || dim > 4) return set_error(ctx, FQ_UNSUPPORTED, "dimension outside 0..4");
  if (ncells <= 0 || !cells) return set_error(ctx, FQ_INVALID_ARG, "a mesh needs at least one cell");
  FQ_GUARD_BEGIN
  auto* m = new fq_mesh();
  m->ctx = ctx;
  fq_status s = build_topology(ctx, m, dim, ncells, cells);
  if (s != FQ_OK) {
    delete m;
    return s;
  }
  *out = m;
  return FQ_OK;
  FQ_GUARD_END(ctx)
}

fq_status fq_mesh_kuhn_cube(fq_ctx* ctx, int dim, int nbox, fq_mesh** out) {
  if (!ctx || !out) return FQ_INVALID_ARG;
  if (dim < 1 || dim > 4 || nbox < 1) return set_error(ctx, FQ_INVALID_ARG, "kuhn cube needs dim 1..4, n >= 1");
  FQ_GUARD_BEGIN
  auto cells = kuhn_cells(dim, nbox);
  fq_status s = fq_mesh_from_cells(ctx, dim, int64_t(cells.size()) / (dim + 1), cells.data(), out);
  if (s == FQ_OK) (*out)->kuhn_nbox = nbox;
  return s;
  FQ_GUARD_END(ctx)
}

void fq_mesh_destroy(fq_mesh* m) {
  if (!m) return;
  cudaStreamSynchronize(m->ctx->stream);
  delete m;
}

int fq_mesh_dim(const fq_mesh* m) { return m ? m->dim : -1; }

int64_t fq_mesh_nsimplices(const fq_mesh* m, int k) {
  if (!m || k < 0 || k > m->dim) return 0;
  return m->nsimp[k];
}

int64_t fq_mesh_ndofs(const fq_mesh* m, int k, fq_bc bc) { return m ? ndofs(m, k, bc) : 0; }

fq_status fq_mesh_simplices(const fq_mesh* m, int k, int32_t* out) {
  if (!m || !out || k < 0 || k > m->dim) return FQ_INVALID_ARG;
  std::memcpy(out, m->skel[k].data(), m->skel[k].size() * sizeof(int32_t));
  return FQ_OK;
}

fq_status fq_mesh_interior(const fq_mesh* m, int k, int64_t* out) {
  if (!m || !out || k < 0 || k > m->dim) return FQ_INVALID_ARG;
  int64_t c = 0;
  for (int64_t i = 0; i < m->nsimp[k]; ++i)
    if (!m->boundary[k][i]) out[c++] = i;
  return FQ_OK;
}

fq_status fq_mesh_orientation(const fq_mesh* mc, int8_t* out) {
  auto* m = const_cast<fq_mesh*>(mc);
  if (!m || !out) return FQ_INVALID_ARG;
  FQ_GUARD_BEGIN
  if (m->orientation.empty()) {
    if (m->dim == 0)
      m->orientation.assign(size_t(m->ncells), 1);
    else
      compute_orientation(m, m->cell_faces_host[m->dim - 1]);
  }
  std::memcpy(out, m->orientation.data(), m->orientation.size());
  return FQ_OK;
  FQ_GUARD_END(m->ctx)
}

fq_status fq_mesh_set_lengths_sq(fq_mesh* m, const double* l, int on_device) {
  if (!m || (!l && m->nsimp[1] > 0)) return FQ_INVALID_ARG;
  fq_ctx* ctx = m->ctx;
  const int64_t ne = m->dim >= 1 ? m->nsimp[1] : 0;
  if (m->lengths.bytes < size_t(std::max<int64_t>(ne, 1)) * 8) FQ_TRY(m->lengths.alloc(ctx, std::max<int64_t>(ne, 1) * 8));
  if (ne > 0)
    FQ_CUDA(ctx, cudaMemcpyAsync(m->lengths.p, l, ne * 8, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                 ctx->stream));
  m->has_lengths = true;
  return FQ_OK;
}

fq_status fq_mesh_get_lengths_sq(const fq_mesh* m, double* out) {
  if (!m || !out || !m->has_lengths) return FQ_INVALID_ARG;
  const int64_t ne = m->dim >= 1 ? m->nsimp[1] : 0;
  if (ne > 0) FQ_CUDA(m->ctx, cudaMemcpyAsync(out, m->lengths.p, ne * 8, cudaMemcpyDeviceToHost, m->ctx->stream));
  FQ_CUDA(m->ctx, cudaStreamSynchronize(m->ctx->stream));
  return FQ_OK;
}

fq_status fq_mesh_lengths_from_coords(fq_mesh* m, const double* coords, int adim, const double* signs) {
  if (!m || !coords || adim <= 0) return FQ_INVALID_ARG;
  FQ_GUARD_BEGIN
  const int64_t ne = m->dim >= 1 ? m->nsimp[1] : 0;
  std::vector<double> l(size_t(std::max<int64_t>(ne, 1)));
  for (int64_t e = 0; e < ne; ++e) {
    const int32_t vi = m->skel[1][e * 2], vj = m->skel[1][e * 2 + 1];
    double acc = 0.0;
    for (int a = 0; a < adim; ++a) {
      const double d = coords[int64_t(vj) * adim + a] - coords[int64_t(vi) * adim + a];
      acc += d * ((signs ? signs[a] : 1.0) * d);
    }
    l[e] = acc;
  }
  return fq_mesh_set_lengths_sq(m, l.data(), 0);
  FQ_GUARD_END(m->ctx)
}

fq_status fq_mesh_kuhn_lengths(fq_mesh* m, const double* side, const double* signs, double jitter, uint64_t seed) {
  if (!m || m->kuhn_nbox <= 0) return m ? set_error(m->ctx, FQ_INVALID_ARG, "not a kuhn cube mesh") : FQ_INVALID_ARG;
  FQ_GUARD_BEGIN
  const int d = m->dim, nb = m->kuhn_nbox;
  int64_t nv = 1;
  for (int a = 0; a < d; ++a) nv *= (nb + 1);
  std::vector<double> x(size_t(nv * d));
  for (int64_t v = 0; v < nv; ++v) {
    int64_t rem = v;
    for (int a = 0; a < d; ++a) {
      const int64_t c = rem % (nb + 1);
      rem /= (nb + 1);
      const double sa = side ? side[a] : 1.0;
      double pos = (double(c) / double(nb)) * sa;
      if (jitter != 0.0) {
        const double u = uniform_pm1(seed, uint64_t(v) * uint64_t(d) + uint64_t(a));
        pos = pos + jitter * (sa / nb) * u;
      }
      x[v * d + a] = pos;
    }
  }
  return fq_mesh_lengths_from_coords(m, x.data(), d, signs);
  FQ_GUARD_END(m->ctx)
}

// ---- kernels (a), (b) -----------------------------------------------------------
fq_status fq_cell_metrics(fq_ctx* ctx, fq_mesh* m, double* ginv, double* det, double* vol) {
  if (!ctx || !m) return FQ_INVALID_ARG;
  if (!m->has_lengths) return set_error(ctx, FQ_INVALID_ARG, "mesh has no edge lengths");
  FQ_GUARD_BEGIN
  ElemArgs a;
  a.ncells = m->ncells;
  a.lengths = m->lengths.as<double>();
  a.cell_edges = m->dim >= 1 ? m->cell_faces[1].as<int32_t>() : nullptr;
  a.out = nullptr;
  a.ginv_out = ginv;
  a.det_out = det;
  a.vol_out = vol;
  a.param = 0.0;
  a.status = ctx->status.as<int>();
  a.nent = 0;
  FQ_CUDA(ctx, cudaMemsetAsync(ctx->status.p, 0, 8 * sizeof(int), ctx->stream));
  if (launch_element(m->dim, 0, EK_METRIC, 0, a, ctx->stream) != 0) return set_error(ctx, FQ_UNSUPPORTED, "dim");
  ctx->launches++;
  FQ_CUDA(ctx, cudaGetLastError());
  FQ_CUDA(ctx, cudaMemcpyAsync(ctx->host_status, ctx->status.p, 8 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (ctx->host_status[0] & 1) return set_error(ctx, FQ_DEGENERATE_CELL, "a cell metric is singular or not finite");
  return FQ_OK;
  FQ_GUARD_END(ctx)
}

fq_status fq_element_matrices(fq_ctx* ctx, fq_mesh* m, fq_form form, int grade, fq_precision prec, void* out,
                              int* rows, int* cols) {
  if (!ctx || !m || !out) return FQ_INVALID_ARG;
  if (!m->has_lengths) return set_error(ctx, FQ_INVALID_ARG, "mesh has no edge lengths");
  FQ_GUARD_BEGIN
  const int n = m->dim;
  const int tg = (form == FQ_DIF_TEST || form == FQ_DIF_BOTH) ? grade - 1 : grade;
  const int sg = (form == FQ_DIF_TRIAL || form == FQ_DIF_BOTH) ? grade - 1 : grade;
  const int lr = (tg >= 0 && tg <= n) ? cbinom(n + 1, tg + 1) : 0;
  const int lc = (sg >= 0 && sg <= n) ? cbinom(n + 1, sg + 1) : 0;
  if (rows) *rows = lr;
  if (cols) *cols = lc;
  if (lr == 0 || lc == 0 || grade > n) return FQ_OK;
  const int kind = int(form);
  Layout lay = make_layout(n, kind, grade);
  const int mode = int(prec);
  FQ_CUDA(ctx, cudaMemsetAsync(ctx->status.p, 0, 8 * sizeof(int), ctx->stream));
  FQ_TRY(element_pass(ctx, m, kind, grade, mode, 0.0, m->elem, lay.nent));
  // expand packed/full entries into row-major [lr*lc][ncells]
  const size_t w = mode == FQ_FP32 ? 4 : 8;
  for (int i = 0; i < lr; ++i)
    for (int j = 0; j < lc; ++j) {
      const int e = lay.entry[size_t(i) * lc + j];
      char* dst = static_cast<char*>(out) + (size_t(i) * lc + j) * m->ncells * w;
      const char* src = m->elem.as<char>() + size_t(e) * m->ncells * w;
      if (e < 0)
        FQ_CUDA(ctx, cudaMemsetAsync(dst, 0, m->ncells * w, ctx->stream));
      else if (mode == FQ_FP64)
        launch_df64_to_double(src, reinterpret_cast<double*>(dst), m->ncells, ctx->stream);
      else
        FQ_CUDA(ctx, cudaMemcpyAsync(dst, src, m->ncells * w, cudaMemcpyDeviceToDevice, ctx->stream));
    }
  FQ_CUDA(ctx, cudaMemcpyAsync(ctx->host_status, ctx->status.p, 8 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (ctx->host_status[0] & 2) return set_error(ctx, FQ_INVALID_ARG, "element program wrote outside its layout");
  if (ctx->host_status[0] & 1) return set_error(ctx, FQ_DEGENERATE_CELL, "a cell metric is singular or not finite");
  return FQ_OK;
  FQ_GUARD_END(ctx)
}

// ---- assembly ---------------------------------------------------------------------
fq_status fq_assemble(fq_ctx* ctx, fq_mesh* m, fq_form form, int grade, fq_bc bc, fq_precision prec,
                      fq_matrix** out) {
  if (!ctx || !m || !out) return FQ_INVALID_ARG;
  *out = nullptr;
  if (int(form) < 0 || int(form) > 3) return set_error(ctx, FQ_INVALID_ARG, "unknown form");
  if (int(prec) < 0 || int(prec) > 2) return set_error(ctx, FQ_INVALID_ARG, "unknown precision");
  FQ_GUARD_BEGIN
  int64_t rows = 0, cols = 0;
  if (!valid_form_shape(m, form, grade, bc, &rows, &cols) || grade > m->dim)
    return empty_matrix(ctx, m, rows, cols, prec, out);
  return make_matrix(ctx, m, int(form), grade, int(bc), int(prec), 0.0, out);
  FQ_GUARD_END(ctx)
}

fq_status fq_reassemble(fq_ctx* ctx, fq_mesh* m, fq_matrix* mat) {
  if (!ctx || !m || !mat || mat->mesh != m) return FQ_INVALID_ARG;
  if (!mat->plan) return FQ_OK;
  FQ_GUARD_BEGIN
  return assemble_into(ctx, mat);
  FQ_GUARD_END(ctx)
}

fq_status fq_reassemble_many(fq_ctx* ctx, fq_matrix* const* mats, int count) {
  if (!ctx || (count > 0 && !mats) || count < 0) return FQ_INVALID_ARG;
  for (int i = 0; i < count; ++i)
    if (!mats[i] || mats[i]->ctx != ctx) return set_error(ctx, FQ_INVALID_ARG, "matrix of another context");
  FQ_GUARD_BEGIN
  return assemble_many(ctx, mats, count);
  FQ_GUARD_END(ctx)
}

fq_status fq_hdif_gram(fq_ctx* ctx, fq_mesh* m, int grade, fq_bc bc, fq_matrix** out) {
  if (!ctx || !m || !out) return FQ_INVALID_ARG;
  FQ_GUARD_BEGIN
  const int64_t nk = ndofs(m, grade, bc);
  if (nk == 0) return empty_matrix(ctx, m, nk, nk, FQ_FP64, out);
  return make_matrix(ctx, m, EK_HDIF, grade, int(bc), FQ_FP64, 0.0, out);
  FQ_GUARD_END(ctx)
}

fq_status fq_coboundary(fq_ctx* ctx, fq_mesh* m, int k, fq_bc bc, fq_matrix** out) {
  if (!ctx || !m || !out) return FQ_INVALID_ARG;
  FQ_GUARD_BEGIN
  const int64_t nr = ndofs(m, k + 1, bc), nc = ndofs(m, k, bc);
  if (k < 0 || k >= m->dim || nr == 0 || nc == 0) return empty_matrix(ctx, m, nr, nc, FQ_FP64, out);
  DCsr d;
  FQ_TRY(coboundary_device(ctx, m, k, int(bc), d));
  auto* mat = new fq_matrix();
  mat->ctx = ctx;
  mat->mesh = m;
  mat->nrows = nr;
  mat->ncols = nc;
  mat->nnz = d.nnz;
  mat->precision = FQ_FP64;
  mat->row_ptr = std::move(d.own_rp);
  mat->col_idx = std::move(d.own_ci);
  mat->values = std::move(d.own_v64);
  mat->rp = mat->row_ptr.as<int32_t>();
  mat->ci = mat->col_idx.as<int32_t>();
  *out = mat;
  return FQ_OK;
  FQ_GUARD_END(ctx)
}

fq_status fq_assemble_host(fq_ctx* ctx, fq_mesh* m, fq_matrix* mat, const double* lengths, void* values_out) {
  if (!ctx || !m || !mat || !lengths || !values_out) return FQ_INVALID_ARG;
  FQ_GUARD_BEGIN
  FQ_TRY(fq_mesh_set_lengths_sq(m, lengths, 0));
  if (mat->plan) FQ_TRY(assemble_into(ctx, mat));
  const size_t w = mat->precision == FQ_FP32 ? 4 : 8;
  if (mat->nnz > 0)
    FQ_CUDA(ctx, cudaMemcpyAsync(values_out, mat->values.p, mat->nnz * w, cudaMemcpyDeviceToHost, ctx->stream));
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return FQ_OK;
  FQ_GUARD_END(ctx)
}

fq_status fq_assemble_host_many(fq_ctx* ctx, fq_mesh* m, const double* lengths, fq_matrix* const* mats,
                                void* const* values_out, int count) {
  if (!ctx || !m || !lengths || count < 0 || (count > 0 && (!mats || !values_out))) return FQ_INVALID_ARG;
  for (int i = 0; i < count; ++i) {
    if (!mats[i] || mats[i]->mesh != m) return set_error(ctx, FQ_INVALID_ARG, "every matrix must be of this mesh");
    if (!values_out[i] && mats[i]->nnz > 0) return FQ_INVALID_ARG;
  }
  FQ_GUARD_BEGIN
  return assemble_host_many(ctx, m, lengths, mats, values_out, count);
  FQ_GUARD_END(ctx)
}

fq_status fq_matrix_info(const fq_matrix* a, int64_t* nrows, int64_t* ncols, int64_t* nnz, int* precision) {
  if (!a) return FQ_INVALID_ARG;
  if (nrows) *nrows = a->nrows;
  if (ncols) *ncols = a->ncols;
  if (nnz) *nnz = a->nnz;
  if (precision) *precision = a->precision;
  return FQ_OK;
}

fq_status fq_matrix_scatter_bytes(const fq_matrix* a, int64_t* bytes) {
  if (!a || !bytes) return FQ_INVALID_ARG;
  *bytes = 0;
  const Plan* p = a->plan;
  if (!p) return FQ_OK;
  const int64_t we = a->precision == FQ_FP32 ? 4 : 8;  // element values (float pairs in FQ_FP64)
  const int64_t wv = a->precision == FQ_FP32 ? 4 : 8;  // assembled values
  if (p->nup > 0)
    *bytes = a->mesh->ncells * int64_t(p->nent) * we + p->nup * 16 + p->ntail_slots * 4 + p->ntail * 4 +
             p->nslots * wv;
  else
    *bytes = p->ntrip * (we + 4) + (p->nslots + 1) * 4 + p->nslots * wv;
  return FQ_OK;
}

fq_status fq_matrix_device_arrays(const fq_matrix* a, const int32_t** rp, const int32_t** ci, const void** val) {
  if (!a) return FQ_INVALID_ARG;
  if (rp) *rp = a->rp;
  if (ci) *ci = a->ci;
  if (val) *val = a->values.p;
  return FQ_OK;
}

fq_status fq_matrix_copy_to_host(fq_ctx* ctx, const fq_matrix* a, int32_t* rp, int32_t* ci, void* val) {
  if (!ctx || !a) return FQ_INVALID_ARG;
  const size_t w = a->precision == FQ_FP32 ? 4 : 8;
  if (rp) FQ_CUDA(ctx, cudaMemcpyAsync(rp, a->rp, (a->nrows + 1) * 4, cudaMemcpyDeviceToHost, ctx->stream));
  if (a->nnz > 0) {
    if (ci) FQ_CUDA(ctx, cudaMemcpyAsync(ci, a->ci, a->nnz * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (val) FQ_CUDA(ctx, cudaMemcpyAsync(val, a->values.p, a->nnz * w, cudaMemcpyDeviceToHost, ctx->stream));
  }
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return FQ_OK;
}

void fq_matrix_destroy(fq_matrix* a) {
  if (!a) return;
  if (a->ctx) cudaStreamSynchronize(a->ctx->stream);
  delete a;
}

// ---- solvers --------------------------------------------------------------------------
fq_status fq_spmv(fq_ctx* ctx, const fq_matrix* a, const void* x, void* y) {
  if (!ctx || !a || (a->nrows && (!x || !y))) return FQ_INVALID_ARG;
  launch_spmv(a, x, y, ctx->stream);
  ctx->launches++;
  FQ_CUDA(ctx, cudaGetLastError());
  return FQ_OK;
}

static fq_status check_square(fq_ctx* ctx, const fq_matrix* a) {
  if (a->nrows != a->ncols) return set_error(ctx, FQ_INVALID_ARG, "operator must be square");
  if (a->precision == FQ_FP32) return set_error(ctx, FQ_INVALID_ARG, "solver takes an FP64 operator");
  return FQ_OK;
}

fq_status fq_minres(fq_ctx* ctx, const fq_matrix* a, const double* dinv, const double* b, double* x,
                    const fq_solve_opts* o, fq_report* rep) {
  if (!ctx || !a || !b || !x) return FQ_INVALID_ARG;
  FQ_TRY(check_square(ctx, a));
  FQ_GUARD_BEGIN
  fq_solve_opts d;
  fq_default_solve_opts(&d);
  if (!o) o = &d;
  fq_report r{};
  FQ_TRY(minres_run<double>(ctx, a->rp, a->ci, a->values.as<double>(), a->nrows, a->nnz, dinv, nullptr, b, x, o->rtol,
                            o->max_iters, &r));
  if (rep) *rep = r;
  return r.converged ? FQ_OK : FQ_NOT_CONVERGED;
  FQ_GUARD_END(ctx)
}

fq_status fq_cg(fq_ctx* ctx, const fq_matrix* a, const double* dinv, const double* b, double* x,
                const fq_solve_opts* o, fq_report* rep) {
  if (!ctx || !a || !b || !x) return FQ_INVALID_ARG;
  FQ_TRY(check_square(ctx, a));
  FQ_GUARD_BEGIN
  fq_solve_opts d;
  fq_default_solve_opts(&d);
  if (!o) o = &d;
  fq_report r{};
  FQ_TRY(cg_run<double>(ctx, a->rp, a->ci, a->values.as<double>(), a->nrows, a->nnz, dinv, nullptr, b, x, o->rtol,
                        o->max_iters, &r));
  if (rep) *rep = r;
  return r.converged ? FQ_OK : FQ_NOT_CONVERGED;
  FQ_GUARD_END(ctx)
}

// ---- HX multigrid on one grade ------------------------------------------------
// A = hdif_gram(grade) and its grade-`grade` HX preconditioner.
static fq_status hx_single(fq_ctx* ctx, fq_mesh* m, int grade, int bc, std::unique_ptr<fq_matrix>& A,
                           HxPrecond& pc, DevBuf& diag) {
  if (grade < 0 || grade > m->dim) return set_error(ctx, FQ_INVALID_ARG, "grade out of range");
  if (!hx_supported(m)) return set_error(ctx, FQ_UNSUPPORTED, "HX multigrid needs a Kuhn cube mesh with lengths");
  if (ndofs(m, grade, bc) == 0) return set_error(ctx, FQ_INVALID_ARG, "no degrees of freedom at this grade");
  fq_matrix* a = nullptr;
  FQ_TRY(make_matrix(ctx, m, EK_HDIF, grade, bc, FQ_FP64, 0.0, &a));
  A.reset(a);
  FQ_TRY(diag.alloc(ctx, std::max<int64_t>(a->nrows, 1) * 8));
  vec_diag(a, diag.as<double>(), ctx->stream);
  ctx->launches++;
  return hx_build(ctx, m, bc, std::vector<int>{grade}, 0, diag.as<double>(), pc);
}

fq_status fq_hx_cg(fq_ctx* ctx, fq_mesh* m, int grade, fq_bc bc, const double* rhs_h, double* x_h,
                   const fq_solve_opts* o, fq_report* rep) {
  if (!ctx || !m || !rhs_h || !x_h) return FQ_INVALID_ARG;
  FQ_GUARD_BEGIN
  fq_solve_opts d;
  fq_default_solve_opts(&d);
  if (!o) o = &d;
  std::unique_ptr<fq_matrix> A;
  HxPrecond pc;
  DevBuf diag, b, x;
  FQ_TRY(hx_single(ctx, m, grade, int(bc), A, pc, diag));
  const int64_t n = A->nrows;
  FQ_TRY(b.alloc(ctx, n * 8));
  FQ_TRY(x.alloc(ctx, n * 8));
  FQ_CUDA(ctx, cudaMemcpyAsync(b.p, rhs_h, n * 8, cudaMemcpyHostToDevice, ctx->stream));
  fq_report r{};
  FQ_TRY(cg_run<double>(ctx, A->rp, A->ci, A->values.as<double>(), n, A->nnz, nullptr, &pc, b.as<double>(),
                        x.as<double>(), o->rtol, o->max_iters, &r));
  {
    DevBuf rr;
    FQ_TRY(rr.alloc(ctx, n * 8));
    double rn = 0, bn = 0;
    FQ_TRY(residual64(ctx, A->rp, A->ci, A->values.as<double>(), n, x.as<double>(), b.as<double>(), rr.as<double>(),
                      &rn, &bn));
    r.true_residual = bn > 0 ? rn / bn : 0.0;
  }
  FQ_CUDA(ctx, cudaMemcpyAsync(x_h, x.p, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (rep) *rep = r;
  return r.converged ? FQ_OK : FQ_NOT_CONVERGED;
  FQ_GUARD_END(ctx)
}

fq_status fq_hx_apply(fq_ctx* ctx, fq_mesh* m, int grade, fq_bc bc, const double* r_h, double* y_h) {
  if (!ctx || !m || !r_h || !y_h) return FQ_INVALID_ARG;
  FQ_GUARD_BEGIN
  std::unique_ptr<fq_matrix> A;
  HxPrecond pc;
  DevBuf diag, r, y;
  FQ_TRY(hx_single(ctx, m, grade, int(bc), A, pc, diag));
  const int64_t n = A->nrows;
  FQ_TRY(r.alloc(ctx, n * 8));
  FQ_TRY(y.alloc(ctx, n * 8));
  FQ_CUDA(ctx, cudaMemcpyAsync(r.p, r_h, n * 8, cudaMemcpyHostToDevice, ctx->stream));
  hx_apply<double>(pc, r.as<double>(), y.as<double>(), nullptr, ctx->stream);
  FQ_CUDA(ctx, cudaGetLastError());
  FQ_CUDA(ctx, cudaMemcpyAsync(y_h, y.p, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return FQ_OK;
  FQ_GUARD_END(ctx)
}

// ---- mixed problem ----------------------------------------------------------------
fq_status fq_mixed_create(fq_ctx* ctx, fq_mesh* m, int grade, fq_bc bc, int precision, fq_mixed** out) {
  if (!ctx || !m || !out) return FQ_INVALID_ARG;
  *out = nullptr;
  if (grade < 0 || grade > m->dim) return set_error(ctx, FQ_INVALID_ARG, "grade outside 0..dim");
  FQ_GUARD_BEGIN
  // The closed-form harmonic border needs the cohomology of a ball.
  int64_t chi = 0;
  for (int k = 0; k <= m->dim; ++k) chi += (k % 2 ? -1 : 1) * m->nsimp[k];
  if (chi != 1)
    return set_error(ctx, FQ_UNSUPPORTED, "mixed solve supports meshes with the cohomology of a ball (Euler characteristic 1)");
  auto* P = new fq_mixed();
  P->ctx = ctx;
  P->mesh = m;
  P->grade = grade;
  P->bc = bc;
  P->precision = precision;
  P->ns = ndofs(m, grade - 1, bc);
  P->nu = ndofs(m, grade, bc);
  P->nh = ((bc == FQ_ABSOLUTE && grade == 0) || (bc == FQ_RELATIVE && grade == m->dim)) ? 1 : 0;
  P->n = P->ns + P->nu + P->nh;
  fq_status s = FQ_OK;
  if (grade >= 1) s = interior_list(ctx, m, grade - 1, P->list_sigma);
  if (s == FQ_OK) s = interior_list(ctx, m, grade, P->list_u);
  if (s == FQ_OK) s = mixed_assemble(P);
  if (s != FQ_OK) {
    delete P;
    return s;
  }
  *out = P;
  return FQ_OK;
  FQ_GUARD_END(ctx)
}

fq_status fq_mixed_reassemble(fq_mixed* P) {
  if (!P) return FQ_INVALID_ARG;
  FQ_GUARD_BEGIN
  return mixed_assemble(P);
  FQ_GUARD_END(P->ctx)
}

fq_status fq_mixed_info(const fq_mixed* P, int64_t* ns, int64_t* nu, int64_t* nh, int64_t* nnz) {
  if (!P) return FQ_INVALID_ARG;
  if (ns) *ns = P->ns;
  if (nu) *nu = P->nu;
  if (nh) *nh = P->nh;
  if (nnz) *nnz = P->nnz;
  return FQ_OK;
}

const fq_matrix* fq_mixed_system(const fq_mixed* P) { return P ? &P->sysview : nullptr; }

void fq_mixed_destroy(fq_mixed* P) {
  if (!P) return;
  cudaStreamSynchronize(P->ctx->stream);
  P->sysview.values.p = nullptr;
  delete P;
}

fq_status fq_mixed_solve_device(fq_mixed* P, const double* src, double* sigma, double* u, double* p,
                                const fq_solve_opts* o, fq_report* rep) {
  if (!P || !src) return FQ_INVALID_ARG;
  FQ_GUARD_BEGIN
  fq_ctx* ctx = P->ctx;
  fq_mesh* m = P->mesh;
  fq_solve_opts d;
  fq_default_solve_opts(&d);
  if (!o) o = &d;
  const int64_t n = P->n;
  DevBuf rhs, x;
  FQ_TRY(rhs.alloc(ctx, std::max<int64_t>(n, 1) * 8));
  FQ_TRY(x.alloc(ctx, std::max<int64_t>(n, 1) * 8));
  FQ_CUDA(ctx, cudaMemsetAsync(rhs.p, 0, std::max<int64_t>(n, 1) * 8, ctx->stream));
  // rhs = [0; E^T f; 0]
  vec_gather(src, P->bc == FQ_RELATIVE ? P->list_u.as<int32_t>() : nullptr, rhs.as<double>() + P->ns, P->nu,
             ctx->stream);
  fq_report r{};
  FQ_TRY(mixed_krylov(P, rhs.as<double>(), x.as<double>(), o, &r));
  // split and extend by E
  if (sigma && P->grade >= 1) {
    const int64_t amb = m->nsimp[P->grade - 1];
    FQ_CUDA(ctx, cudaMemsetAsync(sigma, 0, std::max<int64_t>(amb, 1) * 8, ctx->stream));
    vec_scatter_map(x.as<double>(), P->bc == FQ_RELATIVE ? P->list_sigma.as<int32_t>() : nullptr, sigma, P->ns,
                    ctx->stream);
  }
  if (u) {
    const int64_t amb = m->nsimp[P->grade];
    FQ_CUDA(ctx, cudaMemsetAsync(u, 0, std::max<int64_t>(amb, 1) * 8, ctx->stream));
    vec_scatter_map(x.as<double>() + P->ns, P->bc == FQ_RELATIVE ? P->list_u.as<int32_t>() : nullptr, u, P->nu,
                    ctx->stream);
  }
  if (p && P->nh)
    FQ_CUDA(ctx, cudaMemcpyAsync(p, x.as<double>() + P->ns + P->nu, P->nh * 8, cudaMemcpyDeviceToDevice, ctx->stream));
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (rep) *rep = r;
  return r.converged ? FQ_OK : FQ_NOT_CONVERGED;
  FQ_GUARD_END(P->ctx)
}

fq_status fq_mixed_solve(fq_mixed* P, const double* src_h, double* sigma_h, double* u_h, double* p_h,
                         const fq_solve_opts* o, fq_report* rep) {
  if (!P || !src_h) return FQ_INVALID_ARG;
  FQ_GUARD_BEGIN
  fq_ctx* ctx = P->ctx;
  fq_mesh* m = P->mesh;
  const int64_t nk = m->nsimp[P->grade];
  const int64_t nkm = P->grade >= 1 ? m->nsimp[P->grade - 1] : 0;
  DevBuf src, sg, uu, pp;
  FQ_TRY(src.alloc(ctx, std::max<int64_t>(nk, 1) * 8));
  FQ_TRY(sg.alloc(ctx, std::max<int64_t>(nkm, 1) * 8));
  FQ_TRY(uu.alloc(ctx, std::max<int64_t>(nk, 1) * 8));
  FQ_TRY(pp.alloc(ctx, 16));
  FQ_CUDA(ctx, cudaMemcpyAsync(src.p, src_h, nk * 8, cudaMemcpyHostToDevice, ctx->stream));
  fq_status s = fq_mixed_solve_device(P, src.as<double>(), sg.as<double>(), uu.as<double>(), pp.as<double>(), o, rep);
  if (s != FQ_OK && s != FQ_NOT_CONVERGED) return s;
  if (sigma_h && nkm > 0) FQ_CUDA(ctx, cudaMemcpyAsync(sigma_h, sg.p, nkm * 8, cudaMemcpyDeviceToHost, ctx->stream));
  if (u_h) FQ_CUDA(ctx, cudaMemcpyAsync(u_h, uu.p, nk * 8, cudaMemcpyDeviceToHost, ctx->stream));
  if (p_h && P->nh) FQ_CUDA(ctx, cudaMemcpyAsync(p_h, pp.p, P->nh * 8, cudaMemcpyDeviceToHost, ctx->stream));
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return s;
  FQ_GUARD_END(P->ctx)
}

fq_status fq_solve_source(fq_ctx* ctx, fq_mesh* m, int grade, fq_bc bc, const double* src, double* sigma, double* u,
                          double* p, const fq_solve_opts* o, fq_report* rep) {
  if (!ctx || !m || !src) return FQ_INVALID_ARG;
  fq_mixed* P = nullptr;
  fq_solve_opts d;
  fq_default_solve_opts(&d);
  if (!o) o = &d;
  FQ_TRY(fq_mixed_create(ctx, m, grade, bc, o->precision, &P));
  fq_status s = fq_mixed_solve(P, src, sigma, u, p, o, rep);
  fq_mixed_destroy(P);
  return s;
}

// ---- Dirac ----------------------------------------------------------------------------
fq_status fq_dirac_system(fq_ctx* ctx, fq_mesh* m, double mass_term, fq_matrix** out) {
  if (!ctx || !m || !out) return FQ_INVALID_ARG;
  FQ_GUARD_BEGIN
  return make_matrix(ctx, m, EK_DIRAC, 0, FQ_RELATIVE, FQ_FP64, mass_term, out);
  FQ_GUARD_END(ctx)
}

// A mesh with m's topology (host tables and device face tables copied) and no
// lengths, plans or element buffer.
static fq_status clone_topology(fq_ctx* ctx, const fq_mesh* m, std::unique_ptr<fq_mesh>& out) {
  auto c = std::make_unique<fq_mesh>();
  c->ctx = ctx;
  c->dim = m->dim;
  c->ncells = m->ncells;
  c->kuhn_nbox = m->kuhn_nbox;
  for (int k = 0; k < 6; ++k) c->nsimp[k] = m->nsimp[k];
  for (int k = 0; k < 5; ++k) {
    c->skel[k] = m->skel[k];
    c->boundary[k] = m->boundary[k];
    c->interior_map[k] = m->interior_map[k];
    c->ninterior[k] = m->ninterior[k];
    c->cell_faces_host[k] = m->cell_faces_host[k];
    if (m->cell_faces[k].p) {
      FQ_TRY(c->cell_faces[k].alloc(ctx, m->cell_faces[k].bytes));
      FQ_CUDA(ctx, cudaMemcpyAsync(c->cell_faces[k].p, m->cell_faces[k].p, m->cell_faces[k].bytes,
                                   cudaMemcpyDeviceToDevice, ctx->stream));
    }
    if (m->interior_dev[k].p) {
      FQ_TRY(c->interior_dev[k].alloc(ctx, m->interior_dev[k].bytes));
      FQ_CUDA(ctx, cudaMemcpyAsync(c->interior_dev[k].p, m->interior_dev[k].p, m->interior_dev[k].bytes,
                                   cudaMemcpyDeviceToDevice, ctx->stream));
    }
  }
  c->orientation = m->orientation;
  out = std::move(c);
  return FQ_OK;
}

// Euclidean comparison lengths of a Kuhn lattice mesh with signed squared
// lengths: every lattice axis gets the mean |s| of its single-axis edges, h_a^2,
// and an edge spanning the axis set I gets sum_{a in I} h_a^2 -- the lattice
// with the metric's signs made positive (time and space scales kept), the
// Riemannian geometry the reference measures Lorentzian fields against
// (examples/minkowski_dirac.rs). Kuhn edges join lattice points whose
// coordinates differ by 0 or 1 on each axis.
static fq_status comparison_lengths(fq_ctx* ctx, const fq_mesh* m, std::vector<double>& out) {
  const int n = m->dim, nb = m->kuhn_nbox;
  const int64_t ne = m->nsimp[1];
  std::vector<double> l(size_t(std::max<int64_t>(ne, 1)));
  if (ne > 0) FQ_CUDA(ctx, cudaMemcpyAsync(l.data(), m->lengths.p, ne * 8, cudaMemcpyDeviceToHost, ctx->stream));
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  std::vector<int> axes(size_t(std::max<int64_t>(ne, 1)), 0);
  double sum[4] = {0, 0, 0, 0}, cnt[4] = {0, 0, 0, 0};
  for (int64_t e = 0; e < ne; ++e) {
    int64_t a = m->skel[1][2 * e], b = m->skel[1][2 * e + 1];
    int mask = 0;
    for (int ax = 0; ax < n; ++ax) {
      if (a % (nb + 1) != b % (nb + 1)) mask |= 1 << ax;
      a /= nb + 1;
      b /= nb + 1;
    }
    axes[e] = mask;
    if (mask && !(mask & (mask - 1))) {
      const int ax = __builtin_ctz(unsigned(mask));
      sum[ax] += std::fabs(l[e]);
      cnt[ax] += 1;
    }
  }
  double h2[4];
  for (int ax = 0; ax < n; ++ax) {
    if (cnt[ax] == 0 || !(sum[ax] > 0)) return set_error(ctx, FQ_UNSUPPORTED, "lattice axis without lengths");
    h2[ax] = sum[ax] / cnt[ax];
  }
  out.assign(size_t(ne), 0.0);
  for (int64_t e = 0; e < ne; ++e)
    for (int ax = 0; ax < n; ++ax)
      if (axes[e] & (1 << ax)) out[e] += h2[ax];
  return FQ_OK;
}

// SPD preconditioners of the relative Dirac system on a Kuhn mesh, both from
// the Euclidean comparison geometry (the operator's Lorentzian mass is
// indefinite, so |diag(S)| = m |diag(M)| weighs time-like faces badly):
//   FQ_PC_COMPARISON: the inverse diagonal of the comparison masses M_j, j = 0..n
//     (the L^2 Riesz map's diagonal; as cheap per iteration as Jacobi);
//   FQ_PC_HX:   diag(hdif_gram(j)) of the comparison geometry, each block an HX
//     multigrid (the H Lambda Riesz map; fewer iterations on small meshes, a
//     V-cycle per iteration).
// MINRES needs no more than a fixed SPD operator.
struct DiracPrecond {
  std::unique_ptr<fq_mesh> cmp;
  std::vector<std::unique_ptr<fq_matrix>> mats;
  DevBuf diag, dinv;
  HxPrecond hx;
  bool use_hx = false;
};

static fq_status dirac_comparison(fq_ctx* ctx, fq_mesh* m, bool hx, DiracPrecond& dp) {
  std::vector<double> le;
  FQ_TRY(comparison_lengths(ctx, m, le));
  FQ_TRY(clone_topology(ctx, m, dp.cmp));
  FQ_TRY(fq_mesh_set_lengths_sq(dp.cmp.get(), le.data(), 0));
  const int n = m->dim;
  int64_t nrel = 0;
  for (int k = 0; k <= n; ++k) nrel += m->ninterior[k];
  FQ_TRY(dp.diag.alloc(ctx, std::max<int64_t>(nrel, 1) * 8));
  std::vector<int> grades;
  int64_t off = 0;
  for (int j = 0; j <= n; ++j) {
    grades.push_back(j);
    if (m->ninterior[j] == 0) continue;
    fq_matrix* a = nullptr;
    FQ_TRY(make_matrix(ctx, dp.cmp.get(), hx ? EK_HDIF : EK_MASS, j, FQ_RELATIVE, FQ_FP64, 0.0, &a));
    dp.mats.emplace_back(a);
    vec_diag(a, dp.diag.as<double>() + off, ctx->stream);
    ctx->launches++;
    off += m->ninterior[j];
  }
  dp.use_hx = hx;
  if (hx) return hx_build(ctx, dp.cmp.get(), FQ_RELATIVE, grades, 0, dp.diag.as<double>(), dp.hx);
  FQ_TRY(dp.dinv.alloc(ctx, std::max<int64_t>(nrel, 1) * 8));
  vec_recip(dp.diag.as<double>(), dp.dinv.as<double>(), nullptr, nrel, 1, ctx->stream);
  ctx->launches++;
  return FQ_OK;
}

// The relative harmonic field of the massless Dirac operator in the flat
// relative layout (top_harmonic, problems/dirac.rs:552-570): zero below the top
// grade, h_n = M_n^-1 z on the cells, z the coherent orientation. The relative
// top-grade mass is diagonal (one Whitney n-form per cell).
static fq_status top_harmonic(fq_ctx* ctx, fq_mesh* m, int64_t nrel, DevBuf& h, int64_t* top_off) {
  const int n = m->dim;
  if (m->orientation.empty()) {
    std::vector<int8_t> tmp(static_cast<size_t>(m->ncells));
    FQ_TRY(fq_mesh_orientation(m, tmp.data()));
  }
  fq_matrix* mn = nullptr;
  FQ_TRY(make_matrix(ctx, m, EK_MASS, n, FQ_RELATIVE, FQ_FP64, 0.0, &mn));
  std::unique_ptr<fq_matrix> g(mn);
  const int64_t nt = m->ninterior[n];
  DevBuf d;
  FQ_TRY(d.alloc(ctx, std::max<int64_t>(nt, 1) * 8));
  vec_diag(mn, d.as<double>(), ctx->stream);
  ctx->launches++;
  std::vector<double> dh(static_cast<size_t>(std::max<int64_t>(nt, 1))),
      hh(static_cast<size_t>(std::max<int64_t>(nrel, 1)), 0.0);
  FQ_CUDA(ctx, cudaMemcpyAsync(dh.data(), d.p, nt * 8, cudaMemcpyDeviceToHost, ctx->stream));
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  int64_t off = 0;
  for (int k = 0; k < n; ++k) off += m->ninterior[k];
  for (int64_t c = 0; c < nt; ++c) hh[off + c] = double(m->orientation[c]) / dh[c];
  FQ_TRY(h.alloc(ctx, std::max<int64_t>(nrel, 1) * 8));
  FQ_CUDA(ctx, cudaMemcpyAsync(h.p, hh.data(), nrel * 8, cudaMemcpyHostToDevice, ctx->stream));
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  *top_off = off;
  return FQ_OK;
}

// The mass term whose system is factored in place of a massless (or nearly
// massless) one: 1e-3 over the mesh's diameter, estimated as nbox times the
// root mean square edge length. The Hodge-Dirac operator pairs even and odd
// grades only, so at m = 0 the fully summed block of every leaf front is
// structurally singular (its even and odd counts differ); with the mass shift
// every pivot is defined, and the eigenvalues (l + m) / (l + tau) of the
// preconditioned system stay near 1 for the operator's nonzero spectrum
// |l| >~ 1 / diameter, so GMRES on the exact system needs a handful of
// iterations. The pivots of size tau grow the factors by about 1 / tau: they
// are kept in FP64.
static constexpr double kMasslessShift = 1e-3;
static fq_status massless_shift(fq_ctx* ctx, const fq_mesh* m, double* tau) {
  const int64_t ne = m->nsimp[1];
  std::vector<double> l(static_cast<size_t>(std::max<int64_t>(ne, 1)));
  FQ_CUDA(ctx, cudaMemcpyAsync(l.data(), m->lengths.p, ne * 8, cudaMemcpyDeviceToHost, ctx->stream));
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  double acc = 0;
  for (int64_t e = 0; e < ne; ++e) acc += std::fabs(l[e]);
  const double rms = ne > 0 ? std::sqrt(acc / double(ne)) : 0.0;
  const double diam = double(std::max(m->kuhn_nbox, 1)) * rms;
  if (!(diam > 0) || !std::isfinite(diam))
    return set_error(ctx, FQ_INVALID_ARG, "the massless Dirac solve needs finite nonzero edge lengths");
  *tau = kMasslessShift / diam;
  return FQ_OK;
}

// The direct route of the Dirac source problem: the relative system (bordered
// with the top harmonic at m = 0 when it spans the kernel, as solve_bordered,
// problems/dirac.rs:525-531, 578-598) factored by the sparse direct solver,
// GMRES in FP64 to opts->rtol, on float-float factors. When |m| is below the
// massless shift tau, the factored matrix is the one with mass term tau (same
// sign as m); GMRES still runs on the system with mass term m.
static fq_status dirac_direct(fq_ctx* ctx, fq_mesh* m, fq_matrix* sii, double mass_term, int64_t nrel,
                              const double* rhs, double* x, double rtol, int64_t max_iters, fq_report* r) {
  std::vector<int32_t> dofv;
  FQ_TRY(layout_dof_vertices(ctx, m, EK_DIRAC, 0, FQ_RELATIVE, nrel, dofv));
  const int32_t* rp = sii->rp;
  const int32_t* ci = sii->ci;
  const double* val = sii->values.as<double>();
  int64_t nsys = nrel;
  DevBuf brp, bci, bval, bb, bx, h, trp, tci, tval;
  bool bordered = false;
  // the shifted system to factor, when the mass term is below the shift
  double tau = 0;
  FQ_TRY(massless_shift(ctx, m, &tau));
  std::unique_ptr<fq_matrix> shifted;
  if (std::fabs(mass_term) < tau && nrel > 0) {
    fq_matrix* t = nullptr;
    FQ_TRY(make_matrix(ctx, m, EK_DIRAC, 0, FQ_RELATIVE, FQ_FP64, mass_term < 0 ? -tau : tau, &t));
    shifted.reset(t);
  }
  // the matrix factored: the system's own, or the shifted one, whose pattern
  // holds the mass blocks that assembly drops as all-zero slots at m = 0
  const int32_t* frp = shifted ? shifted->rp : rp;
  const int32_t* fci = shifted ? shifted->ci : ci;
  const double* fval = shifted ? shifted->values.as<double>() : nullptr;
  int64_t off = 0;
  if (mass_term == 0.0 && nrel > 0) {
    DevBuf sh;
    FQ_TRY(top_harmonic(ctx, m, nrel, h, &off));
    FQ_TRY(sh.alloc(ctx, std::max<int64_t>(nrel, 1) * 8));
    launch_spmv(sii, h.p, sh.p, ctx->stream);
    ctx->launches++;
    std::vector<double> hv(static_cast<size_t>(nrel)), sv(static_cast<size_t>(nrel));
    FQ_CUDA(ctx, cudaMemcpyAsync(hv.data(), h.p, nrel * 8, cudaMemcpyDeviceToHost, ctx->stream));
    FQ_CUDA(ctx, cudaMemcpyAsync(sv.data(), sh.p, nrel * 8, cudaMemcpyDeviceToHost, ctx->stream));
    FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    double hn = 0, sn = 0;
    for (int64_t i = 0; i < nrel; ++i) {
      hn += hv[i] * hv[i];
      sn += sv[i] * sv[i];
    }
    if (std::sqrt(sn) <= 1e-8 * std::sqrt(hn)) {
      // the top harmonic spans the kernel: border the system with it
      FQ_TRY(border_csr(ctx, sii, h.as<double>() + off, off, m->ninterior[m->dim], brp, bci, bval));
      rp = brp.as<int32_t>();
      ci = bci.as<int32_t>();
      val = bval.as<double>();
      if (shifted) {
        // the same border on the shifted matrix
        FQ_TRY(border_csr(ctx, shifted.get(), h.as<double>() + off, off, m->ninterior[m->dim], trp, tci, tval));
        frp = trp.as<int32_t>();
        fci = tci.as<int32_t>();
        fval = tval.as<double>();
      } else {
        frp = rp;
        fci = ci;
      }
      nsys = nrel + 1;
      dofv.resize(size_t(nsys) * 5, -1);
      FQ_TRY(bb.alloc(ctx, nsys * 8));
      FQ_TRY(bx.alloc(ctx, nsys * 8));
      FQ_CUDA(ctx, cudaMemsetAsync(bb.p, 0, nsys * 8, ctx->stream));
      FQ_CUDA(ctx, cudaMemcpyAsync(bb.p, rhs, nrel * 8, cudaMemcpyDeviceToDevice, ctx->stream));
      bordered = true;
    }
  }
  // the analysis depends on the pattern only: kept on the mesh for the next
  // solve (new lengths or load), redone when the pattern changed
  std::shared_ptr<SparseLu>& cached = m->dirac_lu[bordered ? 1 : 0];
  int32_t nnz32 = 0;
  FQ_CUDA(ctx, cudaMemcpyAsync(&nnz32, frp + nsys, 4, cudaMemcpyDeviceToHost, ctx->stream));
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  const int64_t nnz = nnz32;
  if (!cached || cached->n != nsys || cached->nnz != nnz) {
    cached.reset();
    auto lu = std::make_shared<SparseLu>();
    FQ_TRY(sparse_lu_build(ctx, m, nsys, frp, fci, dofv, *lu));
    cached = lu;
  }
  SparseLu& lu = *cached;
  // float-float factors at once (of the shifted matrix when there is one): FP32
  // factors of the Lorentzian systems stop converging from about 2e5 unknowns,
  // and the float-float factorization costs 1.2-1.8x the FP32 one; the solve
  // then runs GMRES on the system
  FQ_TRY(sparse_lu_factor(ctx, lu, frp, fci, fval ? fval : val, FQ_FP64));
  const fq_status gs = sparse_lu_solve(ctx, lu, rp, ci, val, bordered ? bb.as<double>() : rhs,
                                       bordered ? bx.as<double>() : x, rtol, max_iters, r);
  if (gs != FQ_OK && gs != FQ_NOT_CONVERGED) return gs;
  if (bordered) FQ_CUDA(ctx, cudaMemcpyAsync(x, bx.p, nrel * 8, cudaMemcpyDeviceToDevice, ctx->stream));
  return FQ_OK;
}

fq_status fq_solve_dirac_source(fq_ctx* ctx, fq_mesh* m, double mass_term, const double* load_h,
                                const double* lift_h, double* x_h, const fq_solve_opts* o, fq_report* rep) {
  if (!ctx || !m || !load_h || !x_h) return FQ_INVALID_ARG;
  FQ_GUARD_BEGIN
  fq_solve_opts d;
  fq_default_solve_opts(&d);
  if (!o) o = &d;
  const int n = m->dim;
  const int pcsel = o->preconditioner;
  const bool kuhn = m->kuhn_nbox > 0;
  if (pcsel == FQ_PC_DIRECT && !kuhn)
    return set_error(ctx, FQ_UNSUPPORTED, "the direct Dirac solve needs a Kuhn cube mesh (fq_mesh_kuhn_cube)");
  if ((pcsel == FQ_PC_HX || pcsel == FQ_PC_COMPARISON) && !kuhn)
    return set_error(ctx, FQ_UNSUPPORTED, "the comparison-lattice Dirac preconditioners need a Kuhn cube mesh");
  const bool direct = pcsel == FQ_PC_DIRECT || (pcsel == FQ_PC_AUTO && kuhn);
  if (mass_term == 0.0 && !direct)
    return set_error(ctx, FQ_UNSUPPORTED, "the massless Dirac system is singular: it needs the bordered direct solve "
                                          "(FQ_PC_AUTO or FQ_PC_DIRECT on a Kuhn cube mesh)");
  int64_t nfull = 0, nrel = 0;
  for (int k = 0; k <= n; ++k) {
    nfull += m->nsimp[k];
    nrel += m->ninterior[k];
  }
  // S_II (solve) and S_IB (rhs lift term) from the same element program
  fq_matrix* sii = nullptr;
  FQ_TRY(make_matrix(ctx, m, EK_DIRAC, 0, FQ_RELATIVE, FQ_FP64, mass_term, &sii));
  std::unique_ptr<fq_matrix> g1(sii);
  Plan* pib = nullptr;
  FQ_TRY(get_plan(ctx, m, EK_DIRAC, 0, FQ_RELATIVE, FQ_ABSOLUTE, &pib));
  auto sib = std::make_unique<fq_matrix>();
  sib->ctx = ctx;
  sib->mesh = m;
  sib->plan = pib;
  sib->kind = EK_DIRAC;
  sib->bc = FQ_RELATIVE;
  sib->precision = FQ_FP64;
  sib->param = mass_term;
  sib->nrows = pib->nrows;
  sib->ncols = pib->ncols;
  FQ_TRY(assemble_into(ctx, sib.get()));
  // relative -> ambient flattened map
  std::vector<int32_t> map;
  {
    int64_t off = 0;
    for (int k = 0; k <= n; ++k) {
      for (int64_t i = 0; i < m->nsimp[k]; ++i)
        if (!m->boundary[k][i]) map.push_back(int32_t(off + i));
      off += m->nsimp[k];
    }
  }
  DevBuf dmap, load, lift, rhs, tmp, x, diag, dinv;
  FQ_TRY(dmap.alloc(ctx, std::max<size_t>(map.size(), 1) * 4));
  FQ_TRY(load.alloc(ctx, std::max<int64_t>(nfull, 1) * 8));
  FQ_TRY(lift.alloc(ctx, std::max<int64_t>(nfull, 1) * 8));
  FQ_TRY(rhs.alloc(ctx, std::max<int64_t>(nrel, 1) * 8));
  FQ_TRY(tmp.alloc(ctx, std::max<int64_t>(nrel, 1) * 8));
  FQ_TRY(x.alloc(ctx, std::max<int64_t>(nrel, 1) * 8));
  FQ_TRY(diag.alloc(ctx, std::max<int64_t>(nrel, 1) * 8));
  FQ_TRY(dinv.alloc(ctx, std::max<int64_t>(nrel, 1) * 8));
  cudaStream_t st = ctx->stream;
  if (!map.empty()) FQ_CUDA(ctx, cudaMemcpyAsync(dmap.p, map.data(), map.size() * 4, cudaMemcpyHostToDevice, st));
  FQ_CUDA(ctx, cudaMemcpyAsync(load.p, load_h, nfull * 8, cudaMemcpyHostToDevice, st));
  if (lift_h)
    FQ_CUDA(ctx, cudaMemcpyAsync(lift.p, lift_h, nfull * 8, cudaMemcpyHostToDevice, st));
  else
    FQ_CUDA(ctx, cudaMemsetAsync(lift.p, 0, nfull * 8, st));
  // rhs = E^T load - S_IB lift
  vec_gather(load.as<double>(), dmap.as<int32_t>(), rhs.as<double>(), nrel, st);
  launch_spmv(sib.get(), lift.p, tmp.p, st);
  vec_sub(rhs.as<double>(), tmp.as<double>(), nrel, st);
  ctx->launches += 3;
  fq_report r{};
  if (direct) {
    FQ_TRY(dirac_direct(ctx, m, sii, mass_term, nrel, rhs.as<double>(), x.as<double>(), o->rtol, o->max_iters, &r));
  } else {
    vec_diag(sii, diag.as<double>(), st);
    vec_recip(diag.as<double>(), dinv.as<double>(), nullptr, nrel, 1, st);
    ctx->launches += 2;
    // preconditioner: from the comparison lattice on Kuhn meshes (its mass
    // diagonal, or HX blocks of its hdif_gram), else |diag(S)|
    std::unique_ptr<DiracPrecond> dp;
    if ((pcsel == FQ_PC_COMPARISON || pcsel == FQ_PC_HX) && nrel > 0) {
      dp = std::make_unique<DiracPrecond>();
      FQ_TRY(dirac_comparison(ctx, m, pcsel == FQ_PC_HX, *dp));
    }
    const double* pc_diag = !dp ? dinv.as<double>() : (dp->use_hx ? nullptr : dp->dinv.as<double>());
    FQ_TRY(minres_run<double>(ctx, sii->rp, sii->ci, sii->values.as<double>(), nrel, sii->nnz, pc_diag,
                              dp && dp->use_hx ? &dp->hx : nullptr, rhs.as<double>(), x.as<double>(), o->rtol,
                              o->max_iters, &r));
    // the reference solves this system by LU: one that MINRES left unconverged is finished
    // that way, by the sparse direct route on Kuhn meshes, densely when small otherwise
    if (!r.converged && kuhn) {
      const int64_t its = r.iters;
      FQ_TRY(dirac_direct(ctx, m, sii, mass_term, nrel, rhs.as<double>(), x.as<double>(), o->rtol,
                          std::max<int64_t>(o->max_iters, kLuFallbackIters), &r));
      r.iters += its;
    } else if (!r.converged && ctx->dense_fallback && nrel <= kDenseMax && dense_fallback_available()) {
      FQ_TRY(dense_lu_solve(ctx, sii->rp, sii->ci, sii->values.as<double>(), nrel, rhs.as<double>(), x.as<double>()));
      r.converged = 1;
    }
    DevBuf rr;
    FQ_TRY(rr.alloc(ctx, std::max<int64_t>(nrel, 1) * 8));
    double rn = 0, bn = 0;
    FQ_TRY(residual64(ctx, sii->rp, sii->ci, sii->values.as<double>(), nrel, x.as<double>(), rhs.as<double>(),
                      rr.as<double>(), &rn, &bn));
    r.true_residual = bn > 0 ? rn / bn : 0.0;
  }
  // x = lift + E x_int
  DevBuf ext;
  FQ_TRY(ext.alloc(ctx, std::max<int64_t>(nfull, 1) * 8));
  FQ_CUDA(ctx, cudaMemsetAsync(ext.p, 0, nfull * 8, st));
  vec_scatter_map(x.as<double>(), dmap.as<int32_t>(), ext.as<double>(), nrel, st);
  vec_add(ext.as<double>(), lift.as<double>(), nfull, st);
  ctx->launches += 2;
  FQ_CUDA(ctx, cudaMemcpyAsync(x_h, ext.p, nfull * 8, cudaMemcpyDeviceToHost, st));
  FQ_CUDA(ctx, cudaStreamSynchronize(st));
  if (rep) *rep = r;
  return r.converged ? FQ_OK : FQ_NOT_CONVERGED;
  FQ_GUARD_END(ctx)
}

}  // extern "C"
