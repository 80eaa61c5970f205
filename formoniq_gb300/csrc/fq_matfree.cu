// Matrix-free Whitney operators, host side: the incidence of the test faces
// (each degree of freedom's (cell, local row) slots, in cell order), the
// two-stage apply, the gathered diagonal and CG driven by the apply.
//
// Reference: ElementOperator::{new, apply}, diagonal, jacobi
// (formoniq/src/matfree.rs:54-172); the incidence is FaceIncidence's
// face_cells reading (simplicial/src/topology/incidence.rs).
#include <cub/cub.cuh>

#include <algorithm>
#include <memory>

#include "fq_matfree.cuh"
#include "fq_internal.h"

struct fq_elemop {
  fq_ctx* ctx = nullptr;
  fq_mesh* mesh = nullptr;
  int kind = 0, grade = 0, bc = 0;
  int row_grade = 0, col_grade = 0, lr = 0, lc = 0;
  int64_t nrows = 0, ncols = 0;
  fq::DevBuf row_ptr;  // int32 [nrows+1]
  fq::DevBuf row_src;  // int32: local row * ncells + cell, grouped by degree of freedom, cell order within
  fq::DevBuf contrib;  // df64 [lr][ncells]
};

namespace fq {

int launch_elemop_cells_dim(int n, int K, int kind, const ElemopArgs& a, cudaStream_t st);

int64_t ndofs_of(const fq_mesh* m, int grade, int bc) {
  if (grade < 0 || grade > m->dim) return 0;
  return bc == FQ_RELATIVE ? m->ninterior[grade] : m->nsimp[grade];
}

namespace {

__global__ void elemop_keys_kernel(const int32_t* __restrict__ row_faces, const int32_t* __restrict__ row_map,
                                   int64_t ncells, int lr, uint64_t sentinel, uint64_t* keys, int32_t* vals) {
  // listed cell by cell, so the stable sort leaves every degree of freedom's
  // slots in cell order (the reference's summation order, matfree.rs:118-127)
  const int64_t total = ncells * lr;
  for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < total; t += int64_t(gridDim.x) * blockDim.x) {
    const int64_t cell = t / lr, i = t - cell * lr;
    const int64_t src = i * ncells + cell;  // slot: local row * ncells + cell
    int32_t r = row_faces[src];
    if (row_map) r = row_map[r];
    keys[t] = r >= 0 ? uint64_t(r) : sentinel;
    vals[t] = int32_t(src);
  }
}

// Second stage: every degree of freedom sums the slots of its cells, in order.
__global__ void __launch_bounds__(256) elemop_rows_kernel(const int32_t* __restrict__ rp,
                                                          const int32_t* __restrict__ src,
                                                          const df64* __restrict__ contrib, double* __restrict__ y,
                                                          int64_t nrows, const int* done) {
  if (done && *done) return;
  for (int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; r < nrows; r += int64_t(gridDim.x) * blockDim.x) {
    const int b = __ldg(rp + r), e = __ldg(rp + r + 1);
    df64 acc(0);
    for (int t = b; t < e; ++t) acc += contrib[__ldg(src + t)];
    y[r] = acc.to_double();
  }
}

int grid_of(int64_t n, int threads) {
  return int(std::max<int64_t>(1, std::min<int64_t>((n + threads - 1) / threads, 152 * 16)));
}

}  // namespace

void launch_gather_rows(const int32_t* rp, const int32_t* src, const df64* contrib, double* y, int64_t nrows,
                        const int* done, cudaStream_t st) {
  if (nrows <= 0) return;
  elemop_rows_kernel<<<grid_of(nrows, 256), 256, 0, st>>>(rp, src, contrib, y, nrows, done);
}

fq_status build_face_incidence(fq_ctx* ctx, fq_mesh* m, int grade, int bc, DevBuf& row_ptr, DevBuf& row_src) {
  cudaStream_t st = ctx->stream;
  const int64_t nc = m->ncells;
  const int lr = cbinom(m->dim + 1, grade + 1);
  const int64_t total = nc * lr;
  const int64_t nrows = ndofs_of(m, grade, bc);
  if (total >= (int64_t(1) << 31)) return set_error(ctx, FQ_UNSUPPORTED, "mesh too large for 32-bit slot indices");
  DevBuf keys, keys2, vals;
  FQ_TRY(keys.alloc(ctx, std::max<int64_t>(total, 1) * 8));
  FQ_TRY(keys2.alloc(ctx, std::max<int64_t>(total, 1) * 8));
  FQ_TRY(vals.alloc(ctx, std::max<int64_t>(total, 1) * 4));
  FQ_TRY(row_src.alloc(ctx, std::max<int64_t>(total, 1) * 4));
  FQ_TRY(row_ptr.alloc(ctx, (nrows + 1) * 4));
  const uint64_t sentinel = uint64_t(std::max<int64_t>(nrows, 1));
  int end_bit = 1;
  while (end_bit < 64 && (sentinel >> end_bit)) ++end_bit;
  elemop_keys_kernel<<<grid_of(total, 256), 256, 0, st>>>(
      m->cell_faces[grade].as<int32_t>(), bc == FQ_RELATIVE ? m->interior_dev[grade].as<int32_t>() : nullptr, nc, lr,
      sentinel, keys.as<uint64_t>(), vals.as<int32_t>());
  ctx->launches++;
  size_t tmp_bytes = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys.as<uint64_t>(), keys2.as<uint64_t>(), vals.as<int32_t>(),
                                  row_src.as<int32_t>(), int(total), 0, end_bit, st);
  DevBuf tmp;
  FQ_TRY(tmp.alloc(ctx, std::max<size_t>(tmp_bytes, 16)));
  FQ_CUDA(ctx, cub::DeviceRadixSort::SortPairs(tmp.p, tmp_bytes, keys.as<uint64_t>(), keys2.as<uint64_t>(),
                                               vals.as<int32_t>(), row_src.as<int32_t>(), int(total), 0, end_bit, st));
  launch_lower_bound_rows(keys2.as<uint64_t>(), total, nrows, 1, row_ptr.as<int32_t>(), st);
  ctx->launches++;
  FQ_CUDA(ctx, cudaStreamSynchronize(st));
  FQ_CUDA(ctx, cudaGetLastError());
  return FQ_OK;
}

// Both stages on the context's stream; x null = the diagonal.
static void elemop_launch(const fq_elemop* op, const double* x, double* y, const int* done, cudaStream_t st) {
  fq_mesh* m = op->mesh;
  ElemopArgs a;
  a.ncells = m->ncells;
  a.lengths = m->lengths.as<double>();
  a.cell_edges = m->dim >= 1 ? m->cell_faces[1].as<int32_t>() : nullptr;
  a.col_faces = m->cell_faces[op->col_grade].as<int32_t>();
  a.col_map = op->bc == FQ_RELATIVE ? m->interior_dev[op->col_grade].as<int32_t>() : nullptr;
  a.x = x;
  a.contrib = op->contrib.as<df64>();
  a.done = done;
  a.status = op->ctx->status.as<int>();
  a.grid = 152 * 12;
  launch_elemop_cells_dim(m->dim, op->grade, op->kind, a, st);
  launch_gather_rows(op->row_ptr.as<int32_t>(), op->row_src.as<int32_t>(), op->contrib.as<df64>(), y, op->nrows,
                     done, st);
  op->ctx->launches += 2;
}

static void elemop_hook_apply(const void* self, const double* x, double* y, const int* done, cudaStream_t st) {
  elemop_launch(static_cast<const fq_elemop*>(self), x, y, done, st);
}

static fq_status elemop_status(fq_ctx* ctx) {
  FQ_CUDA(ctx, cudaGetLastError());
  FQ_CUDA(ctx, cudaMemcpyAsync(ctx->host_status, ctx->status.p, 8 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (ctx->host_status[0] & 1) return set_error(ctx, FQ_DEGENERATE_CELL, "a cell metric is singular or not finite");
  return FQ_OK;
}

}  // namespace fq

using namespace fq;

extern "C" {

fq_status fq_elemop_create(fq_ctx* ctx, fq_mesh* m, fq_form form, int grade, fq_bc bc, fq_elemop** out) {
  if (!ctx || !m || !out) return FQ_INVALID_ARG;
  *out = nullptr;
  if (int(form) < 0 || int(form) > 3) return set_error(ctx, FQ_INVALID_ARG, "unknown form");
  if (!m->has_lengths) return set_error(ctx, FQ_INVALID_ARG, "mesh has no edge lengths");
  const int n = m->dim;
  const int kind = int(form);
  const int rg = (kind == EK_DIF_TEST || kind == EK_DIF_BOTH) ? grade - 1 : grade;
  const int cg = (kind == EK_DIF_TRIAL || kind == EK_DIF_BOTH) ? grade - 1 : grade;
  if (n < 1 || grade < 0 || grade > n || rg < 0 || cg < 0)
    return set_error(ctx, FQ_INVALID_ARG, "no element operator for this form, grade and dimension");
  try {
    auto op = std::make_unique<fq_elemop>();
    op->ctx = ctx;
    op->mesh = m;
    op->kind = kind;
    op->grade = grade;
    op->bc = int(bc);
    op->row_grade = rg;
    op->col_grade = cg;
    op->lr = cbinom(n + 1, rg + 1);
    op->lc = cbinom(n + 1, cg + 1);
    op->nrows = ndofs_of(m, rg, int(bc));
    op->ncols = ndofs_of(m, cg, int(bc));
    FQ_TRY(op->contrib.alloc(ctx, std::max<int64_t>(m->ncells * op->lr, 1) * 8));
    FQ_TRY(build_face_incidence(ctx, m, rg, int(bc), op->row_ptr, op->row_src));
    *out = op.release();
    return FQ_OK;
  } catch (const std::exception& e) {
    return set_error(ctx, FQ_CUDA_ERROR, e.what());
  }
}

fq_status fq_elemop_info(const fq_elemop* op, int64_t* nrows, int64_t* ncols) {
  if (!op) return FQ_INVALID_ARG;
  if (nrows) *nrows = op->nrows;
  if (ncols) *ncols = op->ncols;
  return FQ_OK;
}

fq_status fq_elemop_apply(fq_elemop* op, const double* x, double* y) {
  if (!op || (!x && op->ncols > 0) || (!y && op->nrows > 0)) return FQ_INVALID_ARG;
  fq_ctx* ctx = op->ctx;
  if (!op->mesh->has_lengths) return set_error(ctx, FQ_INVALID_ARG, "mesh has no edge lengths");
  FQ_CUDA(ctx, cudaMemsetAsync(ctx->status.p, 0, 8 * sizeof(int), ctx->stream));
  elemop_launch(op, x, y, nullptr, ctx->stream);
  return elemop_status(ctx);
}

fq_status fq_elemop_diagonal(fq_elemop* op, double* diag) {
  if (!op || (!diag && op->nrows > 0)) return FQ_INVALID_ARG;
  fq_ctx* ctx = op->ctx;
  if (op->row_grade != op->col_grade || (op->kind != EK_MASS && op->kind != EK_DIF_BOTH))
    return set_error(ctx, FQ_INVALID_ARG, "a diagonal needs a square operator");
  FQ_CUDA(ctx, cudaMemsetAsync(ctx->status.p, 0, 8 * sizeof(int), ctx->stream));
  elemop_launch(op, nullptr, diag, nullptr, ctx->stream);
  return elemop_status(ctx);
}

fq_status fq_elemop_cg(fq_elemop* op, const double* b, double* x, const double* inv_diag, const fq_solve_opts* o,
                       fq_report* rep) {
  if (!op || !b || !x) return FQ_INVALID_ARG;
  fq_ctx* ctx = op->ctx;
  if (op->nrows != op->ncols || op->row_grade != op->col_grade)
    return set_error(ctx, FQ_INVALID_ARG, "CG needs a square operator");
  fq_solve_opts d;
  fq_default_solve_opts(&d);
  if (!o) o = &d;
  OpHook hook;
  hook.apply = elemop_hook_apply;
  hook.self = op;
  fq_report r{};
  FQ_CUDA(ctx, cudaMemsetAsync(ctx->status.p, 0, 8 * sizeof(int), ctx->stream));
  fq_status s = cg_run_op(ctx, hook, op->nrows, inv_diag, b, x, o->rtol, o->max_iters, &r);
  if (s != FQ_OK) return s;
  FQ_TRY(elemop_status(ctx));
  if (rep) *rep = r;
  return r.converged ? FQ_OK : FQ_NOT_CONVERGED;
}

void fq_elemop_destroy(fq_elemop* op) {
  if (!op) return;
  cudaStreamSynchronize(op->ctx->stream);
  delete op;
}

}  // extern "C"

namespace fq {
extern template int launch_elemop_cells<1>(int, int, const ElemopArgs&, cudaStream_t);
extern template int launch_elemop_cells<2>(int, int, const ElemopArgs&, cudaStream_t);
extern template int launch_elemop_cells<3>(int, int, const ElemopArgs&, cudaStream_t);
extern template int launch_elemop_cells_sel<4, 1u << EK_MASS>(int, int, const ElemopArgs&, cudaStream_t);
extern template int launch_elemop_cells_sel<4, 1u << EK_DIF_TRIAL>(int, int, const ElemopArgs&, cudaStream_t);
extern template int launch_elemop_cells_sel<4, 1u << EK_DIF_TEST>(int, int, const ElemopArgs&, cudaStream_t);
extern template int launch_elemop_cells_sel<4, 1u << EK_DIF_BOTH>(int, int, const ElemopArgs&, cudaStream_t);

int launch_elemop_cells_dim(int n, int K, int kind, const ElemopArgs& a, cudaStream_t st) {
  switch (n) {
    case 1:
      return launch_elemop_cells<1>(K, kind, a, st);
    case 2:
      return launch_elemop_cells<2>(K, kind, a, st);
    case 3:
      return launch_elemop_cells<3>(K, kind, a, st);
    case 4:
      switch (kind) {
        case EK_MASS:
          return launch_elemop_cells_sel<4, 1u << EK_MASS>(K, kind, a, st);
        case EK_DIF_TRIAL:
          return launch_elemop_cells_sel<4, 1u << EK_DIF_TRIAL>(K, kind, a, st);
        case EK_DIF_TEST:
          return launch_elemop_cells_sel<4, 1u << EK_DIF_TEST>(K, kind, a, st);
        case EK_DIF_BOTH:
          return launch_elemop_cells_sel<4, 1u << EK_DIF_BOTH>(K, kind, a, st);
        default:
          return -1;
      }
    default:
      return -1;
  }
}
}  // namespace fq
