// Small device kernels used by the problem drivers: diagonal extraction,
// restriction / extension by the relative-complex inclusion E
// (whitney_complex.rs:704-713), reciprocal preconditioner diagonals, and the
// harmonic border of the mixed system (elliptic.rs:62-84).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "fq_internal.h"

namespace fq {

static int g1(int64_t n) { return int(std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 8))); }
#define GRID_STRIDE(i, n) for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < (n); i += int64_t(gridDim.x) * blockDim.x)

template <typename VT>
__global__ void diag_kernel(const int32_t* rp, const int32_t* ci, const VT* val, int64_t n, double* d) {
  GRID_STRIDE(r, n) {
    double v = 0.0;
    for (int t = rp[r]; t < rp[r + 1]; ++t)
      if (ci[t] == r) v = double(val[t]);
    d[r] = v;
  }
}

// inv[i] = 1/|d[i]| (or 1/d[i]); 0 -> 1 (identity on an empty diagonal).
__global__ void recip_kernel(const double* d, double* inv, float* inv32, int64_t n, int absval) {
  GRID_STRIDE(i, n) {
    double v = absval ? fabs(d[i]) : d[i];
    const double r = v != 0.0 ? 1.0 / v : 1.0;
    if (inv) inv[i] = r;
    if (inv32) inv32[i] = float(r);
  }
}

// out[i] = in[map[i]] (restriction E^T), map: relative index -> ambient index.
__global__ void gather_kernel(const double* in, const int32_t* map, double* out, int64_t n) {
  GRID_STRIDE(i, n) out[i] = map ? in[map[i]] : in[i];
}
// out[map[i]] = in[i] (extension E, out pre-zeroed).
__global__ void scatter_map_kernel(const double* in, const int32_t* map, double* out, int64_t n) {
  GRID_STRIDE(i, n) {
    if (map)
      out[map[i]] = in[i];
    else
      out[i] = in[i];
  }
}
__global__ void sub_kernel(double* a, const double* b, int64_t n) {
  GRID_STRIDE(i, n) a[i] -= b[i];
}
__global__ void add_kernel(double* a, const double* b, int64_t n) {
  GRID_STRIDE(i, n) a[i] += b[i];
}
__global__ void fill_kernel(double* a, double v, int64_t n) {
  GRID_STRIDE(i, n) a[i] = v;
}
__global__ void scale_kernel(double* a, double s, int64_t n) {
  GRID_STRIDE(i, n) a[i] *= s;
}

// Bordered CSR: rows [ns, ns+nu) gain column nb = ns+nu+... (one harmonic,
// appended last, keeps columns sorted); a new last row holds the border.
template <typename VT>
__global__ void border_rows_kernel(const int32_t* rp, int64_t n, int64_t ns, int64_t nu, int32_t* nrp) {
  GRID_STRIDE(r, n + 2) {
    if (r <= n) {
      const int64_t extra = std::min<int64_t>(std::max<int64_t>(r - ns, 0), nu);
      nrp[r] = int32_t(rp[r] + extra);
    } else {
      nrp[r] = int32_t(rp[n] + nu + nu);
    }
  }
}
template <typename VT>
__global__ void border_fill_kernel(const int32_t* rp, const int32_t* ci, const VT* val, const int32_t* nrp,
                                   const double* mh, int64_t n, int64_t ns, int64_t nu, int32_t* nci, VT* nval) {
  GRID_STRIDE(r, n + 1) {
    if (r < n) {
      int32_t o = nrp[r];
      for (int t = rp[r]; t < rp[r + 1]; ++t, ++o) {
        nci[o] = ci[t];
        nval[o] = val[t];
      }
      if (r >= ns && r < ns + nu) {
        nci[o] = int32_t(n);
        nval[o] = VT(mh[r - ns]);
      }
    } else {
      int32_t o = nrp[n];
      for (int64_t i = 0; i < nu; ++i, ++o) {
        nci[o] = int32_t(ns + i);
        nval[o] = VT(mh[i]);
      }
    }
  }
}

void vec_diag(const fq_matrix* a, double* d, cudaStream_t st) {
  if (a->nrows == 0) return;
  if (a->precision == FQ_FP32)
    diag_kernel<float><<<g1(a->nrows), 256, 0, st>>>(a->rp, a->ci, a->values.as<float>(), a->nrows, d);
  else
    diag_kernel<double><<<g1(a->nrows), 256, 0, st>>>(a->rp, a->ci, a->values.as<double>(), a->nrows, d);
}
void vec_recip(const double* d, double* inv, float* inv32, int64_t n, int absval, cudaStream_t st) {
  if (n > 0) recip_kernel<<<g1(n), 256, 0, st>>>(d, inv, inv32, n, absval);
}
void vec_gather(const double* in, const int32_t* map, double* out, int64_t n, cudaStream_t st) {
  if (n > 0) gather_kernel<<<g1(n), 256, 0, st>>>(in, map, out, n);
}
void vec_scatter_map(const double* in, const int32_t* map, double* out, int64_t n, cudaStream_t st) {
  if (n > 0) scatter_map_kernel<<<g1(n), 256, 0, st>>>(in, map, out, n);
}
void vec_sub(double* a, const double* b, int64_t n, cudaStream_t st) {
  if (n > 0) sub_kernel<<<g1(n), 256, 0, st>>>(a, b, n);
}
void vec_add(double* a, const double* b, int64_t n, cudaStream_t st) {
  if (n > 0) add_kernel<<<g1(n), 256, 0, st>>>(a, b, n);
}
void vec_fill(double* a, double v, int64_t n, cudaStream_t st) {
  if (n > 0) fill_kernel<<<g1(n), 256, 0, st>>>(a, v, n);
}
void vec_scale(double* a, double s, int64_t n, cudaStream_t st) {
  if (n > 0) scale_kernel<<<g1(n), 256, 0, st>>>(a, s, n);
}

// Build the bordered copy of a square CSR (n x n -> n+1 x n+1).
fq_status border_csr(fq_ctx* ctx, const fq_matrix* a, const double* mh, int64_t ns, int64_t nu, DevBuf& nrp,
                     DevBuf& nci, DevBuf& nval) {
  const int64_t n = a->nrows;
  const int64_t nnz = a->nnz + 2 * nu;
  const size_t w = a->precision == FQ_FP32 ? 4 : 8;
  FQ_TRY(nrp.alloc(ctx, (n + 2) * 4));
  FQ_TRY(nci.alloc(ctx, std::max<int64_t>(nnz, 1) * 4));
  FQ_TRY(nval.alloc(ctx, std::max<int64_t>(nnz, 1) * w));
  cudaStream_t st = ctx->stream;
  if (w == 4) {
    border_rows_kernel<float><<<g1(n + 2), 256, 0, st>>>(a->rp, n, ns, nu, nrp.as<int32_t>());
    border_fill_kernel<float><<<g1(n + 1), 256, 0, st>>>(a->rp, a->ci, a->values.as<float>(), nrp.as<int32_t>(), mh,
                                                          n, ns, nu, nci.as<int32_t>(), nval.as<float>());
  } else {
    border_rows_kernel<double><<<g1(n + 2), 256, 0, st>>>(a->rp, n, ns, nu, nrp.as<int32_t>());
    border_fill_kernel<double><<<g1(n + 1), 256, 0, st>>>(a->rp, a->ci, a->values.as<double>(), nrp.as<int32_t>(),
                                                           mh, n, ns, nu, nci.as<int32_t>(), nval.as<double>());
  }
  ctx->launches += 2;
  FQ_CUDA(ctx, cudaGetLastError());
  return FQ_OK;
}

// The signature guard of the mixed solve: the number of cells whose Regge
// metric G_ij = (s_0i + s_0j - s_ij) / 2 (squared edge lengths s of the cell's
// local edges) is not positive definite, by an FP64 Cholesky per cell. The
// reference reads the same fact off the failing Cholesky of an indefinite
// hdif_gram block (mixed_block_preconditioner, problems/elliptic.rs:25-47).
__global__ void indefinite_cells_kernel(const double* lengths, const int32_t* cell_edges, int64_t nc, int n,
                                        unsigned long long* count) {
  unsigned long long local = 0;
  const int ne = n * (n + 1) / 2;
  GRID_STRIDE(c, nc) {
    double s[10];
    for (int e = 0; e < ne; ++e) s[e] = lengths[cell_edges[int64_t(e) * nc + c]];
    auto ei = [](int a, int b) { return (b * (b - 1)) / 2 + a; };
    double l[4][4] = {};
    bool pd = true;
    for (int j = 0; j < n && pd; ++j) {
      for (int i = j; i < n; ++i) {
        double g = i == j ? s[ei(0, j + 1)] : 0.5 * (s[ei(0, i + 1)] + s[ei(0, j + 1)] - s[ei(j + 1, i + 1)]);
        for (int k = 0; k < j; ++k) g -= l[i][k] * l[j][k];
        if (i == j) {
          if (!(g > 0.0)) {
            pd = false;
            break;
          }
          l[j][j] = sqrt(g);
        } else {
          l[i][j] = g / l[j][j];
        }
      }
    }
    if (!pd) ++local;
  }
  if (local) atomicAdd(count, local);
}

fq_status count_indefinite_cells(fq_ctx* ctx, const fq_mesh* m, int64_t* out) {
  *out = 0;
  if (m->dim < 1 || m->ncells == 0) return FQ_OK;
  if (!m->has_lengths) return set_error(ctx, FQ_INVALID_ARG, "mesh has no edge lengths");
  DevBuf cnt;
  FQ_TRY(cnt.alloc(ctx, 8));
  FQ_CUDA(ctx, cudaMemsetAsync(cnt.p, 0, 8, ctx->stream));
  indefinite_cells_kernel<<<g1(m->ncells), 256, 0, ctx->stream>>>(
      m->lengths.as<double>(), m->cell_faces[1].as<int32_t>(), m->ncells, m->dim,
      static_cast<unsigned long long*>(cnt.p));
  ctx->launches++;
  FQ_CUDA(ctx, cudaGetLastError());
  unsigned long long h = 0;
  FQ_CUDA(ctx, cudaMemcpyAsync(&h, cnt.p, 8, cudaMemcpyDeviceToHost, ctx->stream));
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  *out = int64_t(h);
  return FQ_OK;
}

}  // namespace fq
