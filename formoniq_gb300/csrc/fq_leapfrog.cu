// Explicit leapfrog of the Hodge-Dirac Maxwell flow M du/dt = A u, A = dif - delta
// (formoniq/src/problems/dirac.rs:404-434, Leapfrog in formoniq/src/time.rs:271-420).
//
// The grades are 2-coloured by parity; A couples only neighbouring grades, so in
// the (even, odd) split it is block-antidiagonal and one step is
//   p += dt/2 M_1^{-1} A_10 q,   q += dt M_0^{-1} A_01 p,   p += dt/2 M_1^{-1} A_10 q
// with q the even grades, p the odd ones. Per grade k the coupling rows are
//   (A u)_k = U_k u_{k-1} - U_{k+1}^T u_{k+1},   U_k = M_k D_{k-1},
// and U_k is the Whitney pairing dif_trial(k) (U_k^T = dif_test(k)), so every
// block comes from the assembly kernels, relative complex included (the relative
// coboundary of an interior face has no boundary components). M_k^{-1} is a
// Jacobi-preconditioned CG to `mass_rtol` where the reference factors M_k once
// (Cholesky); masses are uniformly well conditioned, so the count stays small.
// All grades of one parity are solved together: one CG on the block-diagonal
// mass of that parity (built once from the per-grade CSRs), so a step runs
// three CG loops instead of one per grade and half kick.
#include <algorithm>
#include <memory>
#include <vector>

#include "fq_hx.h"
#include "fq_internal.h"

struct fq_leapfrog {
  fq_ctx* ctx = nullptr;
  fq_mesh* mesh = nullptr;
  int bc = 0, n = 0;
  double dt = 0.0, mass_rtol = 1e-13;
  int64_t max_inner = 1000;
  std::vector<int64_t> off;                      // [n+2] offsets of the grades in the flat field
  std::vector<std::unique_ptr<fq_matrix>> mass;  // M_k
  std::vector<std::unique_ptr<fq_matrix>> up;    // U_k = dif_trial(k), index k (0 unused)
  std::vector<std::unique_ptr<fq_matrix>> down;  // U_k^T = dif_test(k)
  std::vector<fq::DevBuf> dinv;                  // 1 / diag(M_k)
  // block-diagonal mass of each parity: CSR over the grades k = parity, parity + 2, ...
  fq::DevBuf prp[2], pci[2], pval[2], pdinv[2];
  int64_t prows[2] = {0, 0}, pnnz[2] = {0, 0};
  std::vector<int64_t> poff;                     // [n+1] row offset of grade k inside its parity block
  fq::DevBuf r, t, z, acc;                       // work vectors, max parity-block size; acc: 2 doubles
  int64_t inner_iters = 0;
};

namespace fq {

template <typename VT>
fq_status cg_run(fq_ctx*, const int32_t*, const int32_t*, const VT*, int64_t, int64_t, const VT*, const HxPrecond*,
                 const VT*, VT*, double, int64_t, fq_report*);
void vec_diag(const fq_matrix* a, double* d, cudaStream_t st);
void vec_recip(const double* d, double* inv, float* inv32, int64_t n, int absval, cudaStream_t st);

namespace {

__global__ void lf_axpy(double* __restrict__ y, const double* __restrict__ x, double a, int64_t n) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    y[i] += a * x[i];
}

__global__ void lf_dot(const double* __restrict__ a, const double* __restrict__ b, int64_t n, double* out) {
  double s = 0.0;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    s += a[i] * b[i];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, s);
}

int lf_grid(int64_t n) { return int(std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 8))); }

// One grade's CSR placed on the diagonal of its parity block: row pointers and
// column indices shifted by the block's row and entry offsets.
__global__ void lf_block_csr(const int32_t* __restrict__ rp, const int32_t* __restrict__ ci, int64_t nrows,
                             int64_t nnz, int64_t row_off, int64_t nnz_off, int32_t* __restrict__ rp_out,
                             int32_t* __restrict__ ci_out) {
  const int64_t total = std::max(nrows + 1, nnz);
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < total; i += int64_t(gridDim.x) * blockDim.x) {
    if (i <= nrows) rp_out[row_off + i] = int32_t(rp[i] + nnz_off);
    if (i < nnz) ci_out[nnz_off + i] = int32_t(ci[i] + row_off);
  }
}

}  // namespace

static int64_t grade_size(const fq_leapfrog* L, int k) { return L->off[size_t(k) + 1] - L->off[size_t(k)]; }

// r = (A y)_k = U_k y_{k-1} - U_{k+1}^T y_{k+1}
static fq_status coupling_row(fq_leapfrog* L, const double* y, int k, double* r) {
  fq_ctx* ctx = L->ctx;
  cudaStream_t st = ctx->stream;
  const int64_t nk = grade_size(L, k);
  FQ_CUDA(ctx, cudaMemsetAsync(r, 0, size_t(std::max<int64_t>(nk, 1)) * 8, st));
  if (nk == 0) return FQ_OK;
  if (k >= 1 && grade_size(L, k - 1) > 0 && L->up[size_t(k)]->nnz > 0) {
    launch_spmv(L->up[size_t(k)].get(), y + L->off[size_t(k) - 1], r, st);
    ctx->launches++;
  }
  if (k < L->n && grade_size(L, k + 1) > 0 && L->down[size_t(k) + 1]->nnz > 0) {
    launch_spmv(L->down[size_t(k) + 1].get(), y + L->off[size_t(k) + 1], L->t.as<double>(), st);
    lf_axpy<<<lf_grid(nk), 256, 0, st>>>(r, L->t.as<double>(), -1.0, nk);
    ctx->launches += 2;
  }
  return FQ_OK;
}

// z = M_k^{-1} r
static fq_status mass_solve(fq_leapfrog* L, int k, const double* r, double* z) {
  const fq_matrix* m = L->mass[size_t(k)].get();
  fq_report rep{};
  FQ_TRY(cg_run<double>(L->ctx, m->rp, m->ci, m->values.as<double>(), m->nrows, m->nnz,
                        L->dinv[size_t(k)].as<double>(), nullptr, r, z, L->mass_rtol, L->max_inner, &rep));
  L->inner_iters += rep.iters;
  if (!rep.converged) return set_error(L->ctx, FQ_NOT_CONVERGED, "mass solve of the leapfrog did not converge");
  return FQ_OK;
}

// y_k += c M_k^{-1} (A y)_k for every grade k of the given parity, the mass
// solves of all those grades in one CG on the parity's block-diagonal mass
static fq_status kick(fq_leapfrog* L, double* y, int parity, double c) {
  const int64_t np = L->prows[parity];
  if (np == 0) return FQ_OK;
  for (int k = parity; k <= L->n; k += 2)
    if (grade_size(L, k) > 0) FQ_TRY(coupling_row(L, y, k, L->r.as<double>() + L->poff[size_t(k)]));
  fq_report rep{};
  FQ_TRY(cg_run<double>(L->ctx, L->prp[parity].as<int32_t>(), L->pci[parity].as<int32_t>(),
                        L->pval[parity].as<double>(), np, L->pnnz[parity], L->pdinv[parity].as<double>(), nullptr,
                        L->r.as<double>(), L->z.as<double>(), L->mass_rtol, L->max_inner, &rep));
  L->inner_iters += rep.iters;
  if (!rep.converged) return set_error(L->ctx, FQ_NOT_CONVERGED, "mass solve of the leapfrog did not converge");
  for (int k = parity; k <= L->n; k += 2) {
    const int64_t nk = grade_size(L, k);
    if (nk == 0) continue;
    lf_axpy<<<lf_grid(nk), 256, 0, L->ctx->stream>>>(y + L->off[size_t(k)], L->z.as<double>() + L->poff[size_t(k)],
                                                      c, nk);
    L->ctx->launches++;
  }
  return FQ_OK;
}

static fq_status dot_dev(fq_leapfrog* L, const double* a, const double* b, int64_t n, double* out) {
  fq_ctx* ctx = L->ctx;
  cudaStream_t st = ctx->stream;
  FQ_CUDA(ctx, cudaMemsetAsync(L->acc.p, 0, 8, st));
  if (n > 0) {
    lf_dot<<<lf_grid(n), 256, 0, st>>>(a, b, n, L->acc.as<double>());
    ctx->launches++;
  }
  FQ_CUDA(ctx, cudaMemcpyAsync(out, L->acc.p, 8, cudaMemcpyDeviceToHost, st));
  FQ_CUDA(ctx, cudaStreamSynchronize(st));
  return FQ_OK;
}

}  // namespace fq

using namespace fq;

extern "C" {

fq_status fq_leapfrog_create(fq_ctx* ctx, fq_mesh* m, fq_bc bc, double dt, double mass_rtol, fq_leapfrog** out) {
  if (!ctx || !m || !out) return FQ_INVALID_ARG;
  *out = nullptr;
  if (!m->has_lengths) return set_error(ctx, FQ_INVALID_ARG, "mesh has no edge lengths");
  if (!(dt > 0.0)) return set_error(ctx, FQ_INVALID_ARG, "time step must be positive");
  FQ_GUARD_BEGIN
  auto L = std::make_unique<fq_leapfrog>();
  L->ctx = ctx;
  L->mesh = m;
  L->bc = int(bc);
  L->n = m->dim;
  L->dt = dt;
  if (mass_rtol > 0.0) L->mass_rtol = mass_rtol;
  const int n = m->dim;
  L->off.assign(size_t(n) + 2, 0);
  int64_t maxk = 1;
  for (int k = 0; k <= n; ++k) {
    const int64_t nk = bc == FQ_RELATIVE ? m->ninterior[k] : m->nsimp[k];
    L->off[size_t(k) + 1] = L->off[size_t(k)] + nk;
    maxk = std::max(maxk, nk);
  }
  L->mass.resize(size_t(n) + 1);
  L->up.resize(size_t(n) + 1);
  L->down.resize(size_t(n) + 1);
  L->dinv.resize(size_t(n) + 1);
  for (int k = 0; k <= n; ++k) {
    fq_matrix* a = nullptr;
    FQ_TRY(make_matrix(ctx, m, EK_MASS, k, int(bc), FQ_FP64, 0.0, &a));
    L->mass[size_t(k)].reset(a);
    const int64_t nk = grade_size(L.get(), k);
    FQ_TRY(L->dinv[size_t(k)].alloc(ctx, std::max<int64_t>(nk, 1) * 8));
    if (nk > 0) {
      vec_diag(a, L->dinv[size_t(k)].as<double>(), ctx->stream);
      vec_recip(L->dinv[size_t(k)].as<double>(), L->dinv[size_t(k)].as<double>(), nullptr, nk, 0, ctx->stream);
      ctx->launches += 2;
    }
    if (k >= 1) {
      FQ_TRY(make_matrix(ctx, m, EK_DIF_TRIAL, k, int(bc), FQ_FP64, 0.0, &a));
      L->up[size_t(k)].reset(a);
      FQ_TRY(make_matrix(ctx, m, EK_DIF_TEST, k, int(bc), FQ_FP64, 0.0, &a));
      L->down[size_t(k)].reset(a);
    }
  }
  // the parity blocks
  L->poff.assign(size_t(n) + 1, 0);
  for (int par = 0; par < 2; ++par) {
    int64_t rows = 0, nnz = 0;
    for (int k = par; k <= n; k += 2) {
      L->poff[size_t(k)] = rows;
      rows += grade_size(L.get(), k);
      nnz += L->mass[size_t(k)]->nnz;
    }
    L->prows[par] = rows;
    L->pnnz[par] = nnz;
    if (nnz >= (int64_t(1) << 31)) return set_error(ctx, FQ_UNSUPPORTED, "parity block too large for 32-bit indices");
    FQ_TRY(L->prp[par].alloc(ctx, (rows + 1) * 4));
    FQ_TRY(L->pci[par].alloc(ctx, std::max<int64_t>(nnz, 1) * 4));
    FQ_TRY(L->pval[par].alloc(ctx, std::max<int64_t>(nnz, 1) * 8));
    FQ_TRY(L->pdinv[par].alloc(ctx, std::max<int64_t>(rows, 1) * 8));
    if (rows == 0) FQ_CUDA(ctx, cudaMemsetAsync(L->prp[par].p, 0, 4, ctx->stream));
    int64_t z0 = 0;
    for (int k = par; k <= n; k += 2) {
      const fq_matrix* a = L->mass[size_t(k)].get();
      const int64_t nk = grade_size(L.get(), k);
      if (nk == 0) continue;
      lf_block_csr<<<lf_grid(std::max(nk + 1, a->nnz)), 256, 0, ctx->stream>>>(
          a->rp, a->ci, nk, a->nnz, L->poff[size_t(k)], z0, L->prp[par].as<int32_t>(), L->pci[par].as<int32_t>());
      ctx->launches++;
      if (a->nnz > 0)
        FQ_CUDA(ctx, cudaMemcpyAsync(L->pval[par].as<double>() + z0, a->values.p, size_t(a->nnz) * 8,
                                     cudaMemcpyDeviceToDevice, ctx->stream));
      FQ_CUDA(ctx, cudaMemcpyAsync(L->pdinv[par].as<double>() + L->poff[size_t(k)], L->dinv[size_t(k)].p,
                                   size_t(nk) * 8, cudaMemcpyDeviceToDevice, ctx->stream));
      z0 += a->nnz;
    }
    maxk = std::max(maxk, rows);
  }
  FQ_CUDA(ctx, cudaGetLastError());
  FQ_TRY(L->r.alloc(ctx, maxk * 8));
  FQ_TRY(L->t.alloc(ctx, maxk * 8));
  FQ_TRY(L->z.alloc(ctx, maxk * 8));
  FQ_TRY(L->acc.alloc(ctx, 16));
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  *out = L.release();
  return FQ_OK;
  FQ_GUARD_END(ctx)
}

fq_status fq_leapfrog_info(const fq_leapfrog* L, int64_t* ndofs, int64_t* offsets, int64_t* inner_iters) {
  if (!L) return FQ_INVALID_ARG;
  if (ndofs) *ndofs = L->off.back();
  if (offsets)
    for (size_t i = 0; i < L->off.size(); ++i) offsets[i] = L->off[i];
  if (inner_iters) *inner_iters = L->inner_iters;
  return FQ_OK;
}

fq_status fq_leapfrog_step(fq_leapfrog* L, double* y, int64_t nsteps) {
  if (!L || !y || nsteps < 0) return FQ_INVALID_ARG;
  fq_ctx* ctx = L->ctx;
  FQ_GUARD_BEGIN
  for (int64_t s = 0; s < nsteps; ++s) {
    FQ_TRY(kick(L, y, 1, 0.5 * L->dt));
    FQ_TRY(kick(L, y, 0, L->dt));
    FQ_TRY(kick(L, y, 1, 0.5 * L->dt));
  }
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  FQ_CUDA(ctx, cudaGetLastError());
  return FQ_OK;
  FQ_GUARD_END(ctx)
}

fq_status fq_leapfrog_energy(fq_leapfrog* L, const double* y, double* energy, double* conserved) {
  if (!L || !y) return FQ_INVALID_ARG;
  fq_ctx* ctx = L->ctx;
  FQ_GUARD_BEGIN
  cudaStream_t st = ctx->stream;
  double e = 0.0, defect = 0.0;
  for (int k = 0; k <= L->n; ++k) {
    const int64_t nk = grade_size(L, k);
    if (nk == 0) continue;
    const double* yk = y + L->off[size_t(k)];
    launch_spmv(L->mass[size_t(k)].get(), yk, L->r.as<double>(), st);
    ctx->launches++;
    double d = 0.0;
    FQ_TRY(dot_dev(L, yk, L->r.as<double>(), nk, &d));
    e += 0.5 * d;
    if (k % 2 == 1) {
      // the leapfrog defect (A_10 q)^T M_1^{-1} (A_10 q): only the even grades of y enter
      FQ_TRY(coupling_row(L, y, k, L->r.as<double>()));
      FQ_TRY(mass_solve(L, k, L->r.as<double>(), L->z.as<double>()));
      FQ_TRY(dot_dev(L, L->r.as<double>(), L->z.as<double>(), nk, &d));
      defect += d;
    }
  }
  if (energy) *energy = e;
  if (conserved) *conserved = e - L->dt * L->dt / 8.0 * defect;
  return FQ_OK;
  FQ_GUARD_END(ctx)
}

void fq_leapfrog_destroy(fq_leapfrog* L) {
  if (!L) return;
  cudaStreamSynchronize(L->ctx->stream);
  delete L;
}

}  // extern "C"
