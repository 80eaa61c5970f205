// The source load (SourceForm, formoniq/src/operators.rs:598-635, assembled by
// assemble_vector, formoniq/src/galerkin.rs:279-312), host side: the
// quadrature tables, the nodes a caller evaluates its field at, the cell
// kernels and the incidence gather.
//
// A field is caller code, so, as for the de Rham map, it does not cross the C
// ABI: fq_source_nodes emits the quadrature nodes (barycentric, or in ambient
// coordinates for a flat form), the caller evaluates its form there on the
// device, and fq_source_assemble integrates the values against the Whitney
// forms of every cell and sums the element vectors per face in cell order
// (the reference's `galvec[irow] += val` over the cell-ordered entries).
#include <algorithm>
#include <vector>

#include "fq_matfree.cuh"
#include "fq_source.cuh"

namespace fq {

void gm_rule(int k, int degree, std::vector<double>& pts, std::vector<double>& w);

extern template int launch_source_cells<1>(int, int, const SourceArgs&, cudaStream_t);
extern template int launch_source_cells<2>(int, int, const SourceArgs&, cudaStream_t);
extern template int launch_source_cells<3>(int, int, const SourceArgs&, cudaStream_t);
extern template int launch_source_cells<4>(int, int, const SourceArgs&, cudaStream_t);

namespace {

constexpr int kMaxDegree = 21;

__global__ void source_nodes_kernel(const int32_t* __restrict__ cell_verts, const int32_t* __restrict__ vertex_ids,
                                    const double* __restrict__ coords, const double* __restrict__ bary,
                                    int64_t ncells, int n, int nq, int adim, double* __restrict__ nodes) {
  // nodes[(cell * nq + q) * adim + d] = sum_v lambda_q[v] x_{cell_v}[d]
  const int64_t total = ncells * nq * adim;
  for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < total; t += int64_t(gridDim.x) * blockDim.x) {
    const int64_t cq = t / adim;
    const int d = int(t - cq * adim);
    const int64_t cell = cq / nq;
    const int q = int(cq - cell * nq);
    double x = 0.0;
    for (int v = 0; v <= n; ++v) {
      const int32_t vid = __ldg(vertex_ids + __ldg(cell_verts + int64_t(v) * ncells + cell));
      x = fma(__ldg(bary + q * (n + 1) + v), __ldg(coords + int64_t(vid) * adim + d), x);
    }
    nodes[t] = x;
  }
}

int grid_for(int64_t n) { return int(std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 16))); }

fq_status check_rule(fq_ctx* ctx, const fq_mesh* m, int degree) {
  if (m->dim < 1 || m->dim > 4) return set_error(ctx, FQ_UNSUPPORTED, "source loads need a cell dimension in 1..4");
  if (degree < 0 || degree > kMaxDegree) return set_error(ctx, FQ_INVALID_ARG, "quadrature degree outside 0..21");
  return FQ_OK;
}

int launch_source_dim(int n, int K, int adim, const SourceArgs& a, cudaStream_t st) {
  switch (n) {
    case 1:
      return launch_source_cells<1>(K, adim, a, st);
    case 2:
      return launch_source_cells<2>(K, adim, a, st);
    case 3:
      return launch_source_cells<3>(K, adim, a, st);
    case 4:
      return launch_source_cells<4>(K, adim, a, st);
    default:
      return -1;
  }
}

}  // namespace
}  // namespace fq

using namespace fq;

extern "C" {

int fq_source_npoints(int dim, int degree) {
  if (dim < 1 || dim > 4 || degree < 0 || degree > kMaxDegree) return 0;
  std::vector<double> p, w;
  gm_rule(dim, degree, p, w);
  return int(w.size());
}

fq_status fq_source_nodes(fq_ctx* ctx, fq_mesh* m, const double* coords, int adim, int degree, double* nodes) {
  if (!ctx || !m || !nodes) return FQ_INVALID_ARG;
  FQ_GUARD_BEGIN
  FQ_TRY(check_rule(ctx, m, degree));
  const int n = m->dim;
  std::vector<double> pts, w;
  gm_rule(n, degree, pts, w);
  const int nq = int(w.size());
  if (!coords) {
    FQ_CUDA(ctx, cudaMemcpyAsync(nodes, pts.data(), pts.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return FQ_OK;
  }
  if (adim < n || adim > 4) return set_error(ctx, FQ_UNSUPPORTED, "ambient dimension must be in [cell dimension, 4]");
  DevBuf bary;
  FQ_TRY(bary.alloc(ctx, pts.size() * sizeof(double)));
  FQ_CUDA(ctx, cudaMemcpyAsync(bary.p, pts.data(), pts.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  const int32_t* vids = nullptr;
  FQ_TRY(device_skeleton(ctx, m, 0, &vids));
  const int64_t total = m->ncells * nq * adim;
  if (total > 0) {
    source_nodes_kernel<<<grid_for(total), 256, 0, ctx->stream>>>(m->cell_faces[0].as<int32_t>(), vids, coords,
                                                                  bary.as<double>(), m->ncells, n, nq, adim, nodes);
    ctx->launches++;
  }
  FQ_CUDA(ctx, cudaGetLastError());
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return FQ_OK;
  FQ_GUARD_END(ctx)
}

fq_status fq_source_assemble(fq_ctx* ctx, fq_mesh* m, int grade, fq_bc bc, int degree, const double* coords, int adim,
                             const double* values, double* out) {
  if (!ctx || !m || !out) return FQ_INVALID_ARG;
  FQ_GUARD_BEGIN
  FQ_TRY(check_rule(ctx, m, degree));
  const int n = m->dim;
  if (grade < 0 || grade > n) return set_error(ctx, FQ_INVALID_ARG, "grade out of range");
  if (int(bc) != FQ_ABSOLUTE && int(bc) != FQ_RELATIVE) return set_error(ctx, FQ_INVALID_ARG, "unknown bc");
  if (!m->has_lengths) return set_error(ctx, FQ_INVALID_ARG, "mesh has no edge lengths");
  if (coords && (adim < n || adim > 4))
    return set_error(ctx, FQ_UNSUPPORTED, "ambient dimension must be in [cell dimension, 4]");
  if (!values && m->ncells > 0) return FQ_INVALID_ARG;
  const int b = int(bc);
  const int64_t nrows = ndofs_of(m, grade, b);
  cudaStream_t st = ctx->stream;
  if (!m->inc_ptr[b][grade].p) FQ_TRY(build_face_incidence(ctx, m, grade, b, m->inc_ptr[b][grade], m->inc_src[b][grade]));

  std::vector<double> pts, w;
  gm_rule(n, degree, pts, w);
  const int nq = int(w.size());
  std::vector<double> wlam(pts.size());
  for (int q = 0; q < nq; ++q)
    for (int v = 0; v <= n; ++v) wlam[q * (n + 1) + v] = w[q] * pts[q * (n + 1) + v];
  if (m->source_degree != degree) {
    m->source_degree = -1;
    FQ_TRY(m->source_rule.alloc(ctx, wlam.size() * sizeof(double)));
    FQ_CUDA(ctx, cudaMemcpyAsync(m->source_rule.p, wlam.data(), wlam.size() * sizeof(double), cudaMemcpyHostToDevice,
                                 st));
    m->source_degree = degree;
  }
  const int lf = cbinom(n + 1, grade + 1);
  const size_t slot_bytes = size_t(std::max<int64_t>(m->ncells * lf, 1)) * sizeof(df64);
  if (m->source_slots.bytes < slot_bytes) FQ_TRY(m->source_slots.alloc(ctx, slot_bytes));
  DevBuf& rule = m->source_rule;
  DevBuf& contrib = m->source_slots;

  SourceArgs a;
  a.ncells = m->ncells;
  a.lengths = m->lengths.as<double>();
  a.cell_edges = m->cell_faces[1].as<int32_t>();
  a.cell_verts = m->cell_faces[0].as<int32_t>();
  if (coords) FQ_TRY(device_skeleton(ctx, m, 0, &a.vertex_ids));
  a.coords = coords;
  a.values = values;
  a.wlam = rule.as<double>();
  a.nq = nq;
  const int cin = coords ? cbinom(adim, grade) : cbinom(n, grade);
  a.chunk = std::max(1, std::min(nq, kSourceStageDoubles / cin));
  a.stride = (a.chunk * cin) | 1;
  a.contrib = contrib.as<df64>();
  a.status = ctx->status.as<int>();
  a.grid = 152 * 8;
  FQ_CUDA(ctx, cudaMemsetAsync(ctx->status.p, 0, 8 * sizeof(int), st));
  if (launch_source_dim(n, grade, coords ? adim : 0, a, st) != 0)
    return set_error(ctx, FQ_UNSUPPORTED, "no source kernel for this grade and ambient dimension");
  FQ_CUDA(ctx, cudaGetLastError());
  launch_gather_rows(m->inc_ptr[b][grade].as<int32_t>(), m->inc_src[b][grade].as<int32_t>(), contrib.as<df64>(), out,
                     nrows, nullptr, st);
  ctx->launches += 2;
  FQ_CUDA(ctx, cudaGetLastError());
  FQ_CUDA(ctx, cudaMemcpyAsync(ctx->host_status, ctx->status.p, 8 * sizeof(int), cudaMemcpyDeviceToHost, st));
  FQ_CUDA(ctx, cudaStreamSynchronize(st));
  if (ctx->host_status[0] & 1) return set_error(ctx, FQ_DEGENERATE_CELL, "a cell metric is singular or not finite");
  return FQ_OK;
  FQ_GUARD_END(ctx)
}

}  // extern "C"
