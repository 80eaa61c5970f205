// Device side of the HX-multigrid preconditioner: the Galerkin coarse-operator
// product, the nodal V-cycle over interleaved multi-right-hand-side blocks, and
// the HX gather / scatter of the block preconditioner.
//
// V-cycle (iterative/src/multigrid.rs:VCycle::cycle): from x = 0, `sweeps`
// damped-Jacobi steps x += S (r - A x), the residual restricted by R = P^T, the
// coarse correction prolongated by P, `sweeps` more Jacobi steps; the coarsest
// level is solved exactly (here by its dense inverse). Nodal blocks are stored
// interleaved, X[node * m + slot], so one sparse row serves all m right-hand
// sides with a single read of its indices and values.
#include <cuda_runtime.h>

#include <cub/cub.cuh>

#include <algorithm>
#include <type_traits>
#include <vector>

#include "fq_hx.h"

namespace fq {

namespace {

constexpr int MT = 256;

inline int grid_for_n(int64_t n) { return int(std::max<int64_t>(1, std::min<int64_t>((n + MT - 1) / MT, 152 * 32))); }

// sum_{q in [b, e)} val[q] x[ci[q] * m + c], accumulated in q order (the plain
// loop's rounding), with the index and value loads of four entries issued
// before their gathers: the coarse levels have too few rows to hide a load chain
// per entry, and the sum's order does not change.
template <typename VT>
__device__ __forceinline__ VT row_sum4(const int32_t* __restrict__ ci, const VT* __restrict__ val,
                                       const VT* __restrict__ x, int b, int e, int m, int c, VT a) {
  int q = b;
  for (; q + 4 <= e; q += 4) {
    const int32_t c0 = __ldg(ci + q), c1 = __ldg(ci + q + 1), c2 = __ldg(ci + q + 2), c3 = __ldg(ci + q + 3);
    const VT v0 = __ldg(val + q), v1 = __ldg(val + q + 1), v2 = __ldg(val + q + 2), v3 = __ldg(val + q + 3);
    const VT x0 = __ldg(x + int64_t(c0) * m + c), x1 = __ldg(x + int64_t(c1) * m + c);
    const VT x2 = __ldg(x + int64_t(c2) * m + c), x3 = __ldg(x + int64_t(c3) * m + c);
    a += v0 * x0;
    a += v1 * x1;
    a += v2 * x2;
    a += v3 * x3;
  }
  for (; q < e; ++q) a += __ldg(val + q) * __ldg(x + int64_t(__ldg(ci + q)) * m + c);
  return a;
}

// y[out(row)] = (acc ? y[out(row)] : 0) + (s ? s[row] r[row] : 0) + sum_j A[row, j] x[j],
// out(row) = (row / nI) m + c0 + row % nI.
template <typename VT>
__global__ void __launch_bounds__(MT) gen_spmv_kernel(const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                                      const VT* __restrict__ val, const VT* __restrict__ x,
                                                      VT* __restrict__ y, int64_t nrows, const VT* __restrict__ s,
                                                      const VT* __restrict__ r, int acc, int nI, int m, int c0,
                                                      const int* __restrict__ done) {
  if (done && *done) return;
  for (int64_t row = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; row < nrows;
       row += int64_t(gridDim.x) * blockDim.x) {
    const int b = rp[row], e = rp[row + 1];
    VT a = row_sum4<VT>(ci, val, x, b, e, 1, 0, VT(0));
    if (s) a += s[row] * r[row];
    const int64_t o = nI == 1 && m == 1 ? row : (row / nI) * m + c0 + row % nI;
    y[o] = acc ? y[o] + a : a;
  }
}

// The same with W lanes per row (rows with many entries).
template <int W, typename VT>
__global__ void __launch_bounds__(MT) gen_spmv_w_kernel(const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                                        const VT* __restrict__ val, const VT* __restrict__ x,
                                                        VT* __restrict__ y, int64_t nrows, const VT* __restrict__ s,
                                                        const VT* __restrict__ r, int acc, int nI, int m, int c0,
                                                        const int* __restrict__ done) {
  if (done && *done) return;
  const int lane = threadIdx.x % W;
  const int64_t rows_per_grid = int64_t(gridDim.x) * (blockDim.x / W);
  for (int64_t base = int64_t(blockIdx.x) * (blockDim.x / W); base < nrows; base += rows_per_grid) {
    const int64_t row = base + threadIdx.x / W;
    VT a = VT(0);
    if (row < nrows) {
      const int b = rp[row], e = rp[row + 1];
      for (int t = b + lane; t < e; t += W) a += val[t] * x[ci[t]];
    }
#pragma unroll
    for (int o = W / 2; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o, W);
    if (row < nrows && lane == 0) {
      if (s) a += s[row] * r[row];
      const int64_t o = nI == 1 && m == 1 ? row : (row / nI) * m + c0 + row % nI;
      y[o] = acc ? y[o] + a : a;
    }
  }
}

template <typename VT>
__global__ void __launch_bounds__(MT) mg_jacobi_first(const VT* __restrict__ dinv, const VT* __restrict__ r,
                                                      VT* __restrict__ x, int64_t n, int m, const int* done) {
  if (done && *done) return;
  const int64_t total = n * m;
  for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < total; t += int64_t(gridDim.x) * blockDim.x)
    x[t] = dinv[t / m] * r[t];
}

// xo = xi + dinv (r - A xi)   (mode 0)   or   xo = r - A xi   (mode 1: residual)
template <typename VT>
__global__ void __launch_bounds__(MT) mg_sweep(const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                               const VT* __restrict__ val, const VT* __restrict__ dinv,
                                               const VT* __restrict__ r, const VT* __restrict__ xi,
                                               VT* __restrict__ xo, int64_t n, int m, int mode, const int* done) {
  if (done && *done) return;
  const int64_t total = n * m;
  for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < total; t += int64_t(gridDim.x) * blockDim.x) {
    const int64_t i = t / m;
    const int c = int(t - i * m);
    const int b = rp[i], e = rp[i + 1];
    const VT ax = row_sum4<VT>(ci, val, xi, b, e, m, c, VT(0));
    const VT res = r[t] - ax;
    xo[t] = mode == 0 ? xi[t] + dinv[i] * res : res;
  }
}

// y = (acc ? y : 0) + A x over interleaved blocks
template <typename VT>
__global__ void __launch_bounds__(MT) mg_spmm(const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                              const VT* __restrict__ val, const VT* __restrict__ x,
                                              VT* __restrict__ y, int64_t n, int m, int acc, const int* done) {
  if (done && *done) return;
  const int64_t total = n * m;
  for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < total; t += int64_t(gridDim.x) * blockDim.x) {
    const int64_t i = t / m;
    const int c = int(t - i * m);
    const int b = rp[i], e = rp[i + 1];
    const VT a = row_sum4<VT>(ci, val, x, b, e, m, c, VT(0));
    y[t] = acc ? y[t] + a : a;
  }
}

// x[a][c] = sum_b Ainv[a][b] r[b][c]  (coarsest level, dense inverse): one block
// per coarse row, one warp per slot, lanes over b (coalesced reads of the row).
template <typename VT>
__global__ void __launch_bounds__(MT) mg_dense(const VT* __restrict__ ainv, const VT* __restrict__ r,
                                               VT* __restrict__ x, int64_t nc, int m, const int* done) {
  if (done && *done) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  for (int64_t a = blockIdx.x; a < nc; a += gridDim.x) {
    const VT* row = ainv + a * nc;
    for (int c = warp; c < m; c += nwarps) {
      VT acc = VT(0);
      for (int64_t b = lane; b < nc; b += 32) acc += row[b] * r[b * m + c];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if (lane == 0) x[a * m + c] = acc;
    }
  }
}

template <typename VT>
__global__ void copy_kernel(const VT* __restrict__ a, VT* __restrict__ b, int64_t n, const int* done) {
  if (done && *done) return;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    b[i] = a[i];
}

__global__ void f64_to_f32_kernel(const double* a, float* o, int64_t n) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    o[i] = float(a[i]);
}

// ---- Galerkin product P^T A P ----
// Products of each A entry with the rows of P at its row and column.
__global__ void gp_count(const int32_t* __restrict__ arp, const int32_t* __restrict__ aci,
                         const int32_t* __restrict__ prp, int64_t n, int32_t* __restrict__ rowof,
                         int64_t* __restrict__ cnt) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const int pi = prp[i + 1] - prp[i];
    for (int q = arp[i]; q < arp[i + 1]; ++q) {
      const int j = aci[q];
      rowof[q] = int32_t(i);
      cnt[q] = int64_t(pi) * (prp[j + 1] - prp[j]);
    }
  }
}

__global__ void gp_expand(const int32_t* __restrict__ rowof, const int32_t* __restrict__ aci,
                          const double* __restrict__ aval, int64_t annz, const int32_t* __restrict__ prp,
                          const int32_t* __restrict__ pci, const double* __restrict__ pval,
                          const int64_t* __restrict__ off, int64_t nc, uint64_t* __restrict__ keys,
                          double* __restrict__ vals) {
  for (int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; q < annz; q += int64_t(gridDim.x) * blockDim.x) {
    const int i = rowof[q], j = aci[q];
    const double a = aval[q];
    int64_t o = off[q];
    for (int u = prp[i]; u < prp[i + 1]; ++u)
      for (int w = prp[j]; w < prp[j + 1]; ++w) {
        keys[o] = uint64_t(pci[u]) * uint64_t(nc) + uint64_t(pci[w]);
        vals[o] = pval[u] * a * pval[w];
        ++o;
      }
  }
}

// In-order sum of each run of equal keys (deterministic).
__global__ void gp_segsum(const double* __restrict__ vals, const int64_t* __restrict__ start,
                          const int32_t* __restrict__ len, const uint64_t* __restrict__ ukeys, int64_t nruns,
                          int64_t nc, double* __restrict__ out, int32_t* __restrict__ col) {
  for (int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; s < nruns; s += int64_t(gridDim.x) * blockDim.x) {
    double a = 0.0;
    const int64_t b = start[s];
    for (int q = 0; q < len[s]; ++q) a += vals[b + q];
    out[s] = a;
    col[s] = int32_t(ukeys[s] % uint64_t(nc));
  }
}

__global__ void gp_rowptr(const uint64_t* __restrict__ ukeys, int64_t nruns, int64_t nrows, int64_t nc,
                          int32_t* __restrict__ rp) {
  for (int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; r <= nrows; r += int64_t(gridDim.x) * blockDim.x) {
    const uint64_t key = uint64_t(r) * uint64_t(nc);
    int64_t lo = 0, hi = nruns;
    while (lo < hi) {
      const int64_t mid = (lo + hi) / 2;
      if (ukeys[mid] < key)
        lo = mid + 1;
      else
        hi = mid;
    }
    rp[r] = int32_t(lo);
  }
}

__global__ void diag_recip_kernel(const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                  const double* __restrict__ val, int64_t n, double omega, double* __restrict__ out) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    double d = 0.0;
    for (int q = rp[i]; q < rp[i + 1]; ++q)
      if (ci[q] == i) d = val[q];
    out[i] = d != 0.0 ? omega / d : 0.0;
  }
}

template <typename VT>
void gen_spmv(const DCsr& A, const VT* x, VT* y, const VT* s, const VT* r, int acc, int nI, int m, int c0,
              const int* done, cudaStream_t st) {
  if (A.nrows == 0) return;
  const double avg = double(A.nnz) / double(A.nrows);
  auto blocks = [&](int W) { return grid_for_n(A.nrows * W); };
  // FP64 rows stay on one thread longer: a lane split adds FP64 shuffle sums,
  // and the FP64 pipe, not memory, bounds these products on GB300
  const double one_thread = std::is_same<VT, double>::value ? 32 : 8;
  if (avg <= one_thread) {
    gen_spmv_kernel<VT><<<grid_for_n(A.nrows), MT, 0, st>>>(A.rp, A.ci, A.val<VT>(), x, y, A.nrows, s, r, acc, nI, m,
                                                            c0, done);
  } else if (avg <= 24) {
    gen_spmv_w_kernel<4, VT><<<blocks(4), MT, 0, st>>>(A.rp, A.ci, A.val<VT>(), x, y, A.nrows, s, r, acc, nI, m, c0,
                                                       done);
  } else if (avg <= 64) {
    gen_spmv_w_kernel<8, VT><<<blocks(8), MT, 0, st>>>(A.rp, A.ci, A.val<VT>(), x, y, A.nrows, s, r, acc, nI, m, c0,
                                                       done);
  } else {
    gen_spmv_w_kernel<16, VT><<<blocks(16), MT, 0, st>>>(A.rp, A.ci, A.val<VT>(), x, y, A.nrows, s, r, acc, nI, m,
                                                         c0, done);
  }
}

template <typename VT>
const VT* buf(const DevBuf& b) {
  return b.as<VT>();
}

template <typename VT>
const VT* pick(const DevBuf& b64, const DevBuf& b32) {
  if constexpr (std::is_same<VT, double>::value)
    return b64.as<double>();
  else
    return b32.as<float>();
}

template <typename VT>
VT* vcycle(const NodalHierarchy& mg, size_t l, int m, const int* done, cudaStream_t st) {
  const NodalLevel& L = mg.lv[l];
  VT* x0 = L.x[0].as<VT>();
  VT* x1 = L.x[1].as<VT>();
  const VT* r = L.r.as<VT>();
  const int64_t tot = L.n * m;
  if (L.n == 0) return x0;
  if (l + 1 == mg.lv.size()) {
    mg_dense<VT><<<int(std::min<int64_t>(L.n, 152 * 8)), MT, 0, st>>>(pick<VT>(mg.coarse_inv64, mg.coarse_inv32), r,
                                                                      x0, L.n, m, done);
    return x0;
  }
  const VT* dinv = pick<VT>(L.dinv64, L.dinv32);
  const VT* av = L.A.val<VT>();
  VT* xs[2] = {x0, x1};
  int cur = 0;
  mg_jacobi_first<VT><<<grid_for_n(tot), MT, 0, st>>>(dinv, r, xs[0], L.n, m, done);
  for (int s = 1; s < mg.sweeps; ++s) {
    mg_sweep<VT><<<grid_for_n(tot), MT, 0, st>>>(L.A.rp, L.A.ci, av, dinv, r, xs[cur], xs[1 - cur], L.n, m, 0, done);
    cur ^= 1;
  }
  VT* t = L.t.as<VT>();
  mg_sweep<VT><<<grid_for_n(tot), MT, 0, st>>>(L.A.rp, L.A.ci, av, dinv, r, xs[cur], t, L.n, m, 1, done);
  const NodalLevel& C = mg.lv[l + 1];
  if (C.n > 0) {
    mg_spmm<VT><<<grid_for_n(C.n * m), MT, 0, st>>>(L.R.rp, L.R.ci, L.R.val<VT>(), t, C.r.as<VT>(), C.n, m, 0, done);
    VT* xc = vcycle<VT>(mg, l + 1, m, done, st);
    mg_spmm<VT><<<grid_for_n(tot), MT, 0, st>>>(L.P.rp, L.P.ci, L.P.val<VT>(), xc, xs[cur], L.n, m, 1, done);
  }
  for (int s = 0; s < mg.sweeps; ++s) {
    mg_sweep<VT><<<grid_for_n(tot), MT, 0, st>>>(L.A.rp, L.A.ci, av, dinv, r, xs[cur], xs[1 - cur], L.n, m, 0, done);
    cur ^= 1;
  }
  return xs[cur];
}

}  // namespace

// ---------------------------------------------------------------------------
// DCsr
// ---------------------------------------------------------------------------
fq_status DCsr::upload(fq_ctx* ctx, int64_t nr, int64_t nc, const std::vector<int32_t>& hrp,
                       const std::vector<int32_t>& hci, const std::vector<double>& hv) {
  nrows = nr;
  ncols = nc;
  nnz = int64_t(hci.size());
  FQ_TRY(own_rp.alloc(ctx, (nr + 1) * 4));
  FQ_TRY(own_ci.alloc(ctx, std::max<int64_t>(nnz, 1) * 4));
  FQ_TRY(own_v64.alloc(ctx, std::max<int64_t>(nnz, 1) * 8));
  FQ_CUDA(ctx, cudaMemcpyAsync(own_rp.p, hrp.data(), (nr + 1) * 4, cudaMemcpyHostToDevice, ctx->stream));
  if (nnz) {
    FQ_CUDA(ctx, cudaMemcpyAsync(own_ci.p, hci.data(), nnz * 4, cudaMemcpyHostToDevice, ctx->stream));
    FQ_CUDA(ctx, cudaMemcpyAsync(own_v64.p, hv.data(), nnz * 8, cudaMemcpyHostToDevice, ctx->stream));
  }
  // the host vectors may be freed by the caller right after this returns
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  rp = own_rp.as<int32_t>();
  ci = own_ci.as<int32_t>();
  v64 = own_v64.as<double>();
  v32 = nullptr;
  own_v32.release();
  return FQ_OK;
}

void DCsr::view(const fq_matrix* m) {
  nrows = m->nrows;
  ncols = m->ncols;
  nnz = m->nnz;
  rp = m->rp;
  ci = m->ci;
  v64 = m->values.as<double>();
  v32 = nullptr;
}

fq_status DCsr::make_f32(fq_ctx* ctx) {
  FQ_TRY(own_v32.alloc(ctx, std::max<int64_t>(nnz, 1) * 4));
  launch_f64_to_f32(v64, own_v32.as<float>(), nnz, ctx->stream);
  v32 = own_v32.as<float>();
  return FQ_OK;
}

template <>
const double* DCsr::val<double>() const {
  return v64;
}
template <>
const float* DCsr::val<float>() const {
  return v32;
}

void launch_f64_to_f32(const double* a, float* o, int64_t n, cudaStream_t st) {
  if (n > 0) f64_to_f32_kernel<<<grid_for_n(n), MT, 0, st>>>(a, o, n);
}

__global__ void scaled_recip_kernel(const double* __restrict__ d, int64_t n, double omega, double* __restrict__ out) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    out[i] = d[i] != 0.0 ? omega / d[i] : 0.0;
}

struct AxisOffsets {
  int64_t o[5];
};

// One block: deterministic per-axis means, then the 2^n products.
__global__ void lattice_spacing_kernel(const double* __restrict__ len, const int32_t* __restrict__ edges, AxisOffsets off,
                                       int n, double* __restrict__ hprod, int* __restrict__ flag) {
  __shared__ double sh[32];
  __shared__ double h[4];
  __shared__ int bad;
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  for (int a = 0; a < n; ++a) {
    double acc = 0.0;
    for (int64_t i = off.o[a] + threadIdx.x; i < off.o[a + 1]; i += blockDim.x) {
      const double v = len[edges[i]];
      if (!(v > 0.0)) bad = 1;
      acc += v;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int w = 0; w < int(blockDim.x >> 5); ++w) t += sh[w];
      const int64_t cnt = off.o[a + 1] - off.o[a];
      h[a] = cnt > 0 ? sqrt(fmax(t / double(cnt), 0.0)) : 1.0;
    }
    __syncthreads();
  }
  if (threadIdx.x < 16) {
    double p = 1.0;
    for (int a = 0; a < n; ++a)
      if (threadIdx.x & (1u << a)) p *= h[a];
    hprod[threadIdx.x] = p;
  }
  if (threadIdx.x == 0) *flag = bad;
}

__global__ void scale_by_mask_kernel(const double* __restrict__ base, const uint8_t* __restrict__ mask,
                                     const double* __restrict__ hprod, double* __restrict__ out, int64_t nnz) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < nnz; i += int64_t(gridDim.x) * blockDim.x)
    out[i] = base[i] * hprod[mask[i]];
}

void launch_lattice_spacing(const double* lengths, const int32_t* axis_edges, const int64_t* off_host, int n,
                            double* hprod, int* flag, cudaStream_t st) {
  AxisOffsets o{};
  for (int a = 0; a <= n; ++a) o.o[a] = off_host[a];
  lattice_spacing_kernel<<<1, 1024, 0, st>>>(lengths, axis_edges, o, n, hprod, flag);
}

void launch_scale_by_mask(const double* base, const uint8_t* mask, const double* hprod, double* out, int64_t nnz,
                          cudaStream_t st) {
  if (nnz > 0) scale_by_mask_kernel<<<grid_for_n(nnz), MT, 0, st>>>(base, mask, hprod, out, nnz);
}

fq_status upload_scalable(fq_ctx* ctx, const HCsr& h, DCsr& d) {
  FQ_TRY(d.upload(ctx, h.nrows, h.ncols, h.rp, h.ci, h.v));
  FQ_TRY(d.own_base.alloc(ctx, std::max<int64_t>(d.nnz, 1) * 8));
  FQ_TRY(d.own_mask.alloc(ctx, std::max<int64_t>(d.nnz, 1)));
  if (d.nnz) {
    FQ_CUDA(ctx, cudaMemcpyAsync(d.own_base.p, d.own_v64.p, d.nnz * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    FQ_CUDA(ctx, cudaMemcpyAsync(d.own_mask.p, h.mask.data(), d.nnz, cudaMemcpyHostToDevice, ctx->stream));
  }
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  d.scalable = true;
  return FQ_OK;
}

fq_status device_scaled_recip(fq_ctx* ctx, const double* d, int64_t n, double omega, DevBuf& out) {
  FQ_TRY(out.alloc(ctx, std::max<int64_t>(n, 1) * 8));
  if (n > 0) scaled_recip_kernel<<<grid_for_n(n), MT, 0, ctx->stream>>>(d, n, omega, out.as<double>());
  ctx->launches++;
  return FQ_OK;
}

fq_status device_diag_recip(fq_ctx* ctx, const DCsr& A, double omega, DevBuf& out) {
  FQ_TRY(out.alloc(ctx, std::max<int64_t>(A.nrows, 1) * 8));
  if (A.nrows > 0)
    diag_recip_kernel<<<grid_for_n(A.nrows), MT, 0, ctx->stream>>>(A.rp, A.ci, A.v64, A.nrows, omega,
                                                                    out.as<double>());
  ctx->launches++;
  return FQ_OK;
}

fq_status device_to_host(fq_ctx* ctx, const DCsr& A, HCsr& out) {
  out.nrows = A.nrows;
  out.ncols = A.ncols;
  out.rp.resize(A.nrows + 1);
  out.ci.resize(A.nnz);
  out.v.resize(A.nnz);
  FQ_CUDA(ctx, cudaMemcpyAsync(out.rp.data(), A.rp, (A.nrows + 1) * 4, cudaMemcpyDeviceToHost, ctx->stream));
  if (A.nnz) {
    FQ_CUDA(ctx, cudaMemcpyAsync(out.ci.data(), A.ci, A.nnz * 4, cudaMemcpyDeviceToHost, ctx->stream));
    FQ_CUDA(ctx, cudaMemcpyAsync(out.v.data(), A.v64, A.nnz * 8, cudaMemcpyDeviceToHost, ctx->stream));
  }
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return FQ_OK;
}

// ---------------------------------------------------------------------------
// Galerkin coarse operator P^T A P (formoniq/src/multigrid.rs: the coarse
// operators are the triple product, not a reassembly). Every product of an A
// entry with one P entry on each side is expanded, stably sorted by its coarse
// (row, col) key and summed run by run in expansion order, so the result does
// not depend on scheduling.
// ---------------------------------------------------------------------------
fq_status galerkin_product(fq_ctx* ctx, const DCsr& A, const DCsr& P, DCsr& out) {
  cudaStream_t st = ctx->stream;
  const int64_t n = A.nrows, nc = P.ncols, annz = A.nnz;
  out.nrows = out.ncols = nc;
  FQ_TRY(out.own_rp.alloc(ctx, (nc + 1) * 4));
  if (annz == 0 || nc == 0) {
    FQ_CUDA(ctx, cudaMemsetAsync(out.own_rp.p, 0, (nc + 1) * 4, st));
    FQ_TRY(out.own_ci.alloc(ctx, 4));
    FQ_TRY(out.own_v64.alloc(ctx, 8));
    out.nnz = 0;
    out.rp = out.own_rp.as<int32_t>();
    out.ci = out.own_ci.as<int32_t>();
    out.v64 = out.own_v64.as<double>();
    return FQ_OK;
  }
  DevBuf rowof, cnt, off;
  FQ_TRY(rowof.alloc(ctx, annz * 4));
  FQ_TRY(cnt.alloc(ctx, (annz + 1) * 8));
  FQ_TRY(off.alloc(ctx, (annz + 1) * 8));
  FQ_CUDA(ctx, cudaMemsetAsync(cnt.as<int64_t>() + annz, 0, 8, st));
  gp_count<<<grid_for_n(n), MT, 0, st>>>(A.rp, A.ci, P.rp, n, rowof.as<int32_t>(), cnt.as<int64_t>());
  size_t tb = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, tb, cnt.as<int64_t>(), off.as<int64_t>(), int(annz + 1), st);
  {
    DevBuf tmp;
    FQ_TRY(tmp.alloc(ctx, std::max<size_t>(tb, 16)));
    FQ_CUDA(ctx, cub::DeviceScan::ExclusiveSum(tmp.p, tb, cnt.as<int64_t>(), off.as<int64_t>(), int(annz + 1), st));
  }
  int64_t total = 0;
  FQ_CUDA(ctx, cudaMemcpyAsync(&total, off.as<int64_t>() + annz, 8, cudaMemcpyDeviceToHost, st));
  FQ_CUDA(ctx, cudaStreamSynchronize(st));
  if (total >= (int64_t(1) << 31)) return set_error(ctx, FQ_UNSUPPORTED, "Galerkin product too large");
  if (total == 0) {
    FQ_CUDA(ctx, cudaMemsetAsync(out.own_rp.p, 0, (nc + 1) * 4, st));
    FQ_TRY(out.own_ci.alloc(ctx, 4));
    FQ_TRY(out.own_v64.alloc(ctx, 8));
    FQ_CUDA(ctx, cudaStreamSynchronize(st));
    out.nnz = 0;
    out.rp = out.own_rp.as<int32_t>();
    out.ci = out.own_ci.as<int32_t>();
    out.v64 = out.own_v64.as<double>();
    return FQ_OK;
  }
  DevBuf k1, k2, v1, v2;
  FQ_TRY(k1.alloc(ctx, std::max<int64_t>(total, 1) * 8));
  FQ_TRY(k2.alloc(ctx, std::max<int64_t>(total, 1) * 8));
  FQ_TRY(v1.alloc(ctx, std::max<int64_t>(total, 1) * 8));
  FQ_TRY(v2.alloc(ctx, std::max<int64_t>(total, 1) * 8));
  gp_expand<<<grid_for_n(annz), MT, 0, st>>>(rowof.as<int32_t>(), A.ci, A.v64, annz, P.rp, P.ci, P.v64,
                                            off.as<int64_t>(), nc, k1.as<uint64_t>(), v1.as<double>());
  int end_bit = 1;
  while (end_bit < 64 && (uint64_t(1) << end_bit) <= uint64_t(nc) * uint64_t(nc)) ++end_bit;
  tb = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, tb, k1.as<uint64_t>(), k2.as<uint64_t>(), v1.as<double>(), v2.as<double>(),
                                  int(total), 0, end_bit, st);
  {
    DevBuf tmp;
    FQ_TRY(tmp.alloc(ctx, std::max<size_t>(tb, 16)));
    FQ_CUDA(ctx, cub::DeviceRadixSort::SortPairs(tmp.p, tb, k1.as<uint64_t>(), k2.as<uint64_t>(), v1.as<double>(),
                                                 v2.as<double>(), int(total), 0, end_bit, st));
  }
  DevBuf ukeys, lens, nr, starts;
  FQ_TRY(ukeys.alloc(ctx, total * 8));
  FQ_TRY(lens.alloc(ctx, (total + 1) * 4));
  FQ_TRY(nr.alloc(ctx, 8));
  tb = 0;
  cub::DeviceRunLengthEncode::Encode(nullptr, tb, k2.as<uint64_t>(), ukeys.as<uint64_t>(), lens.as<int32_t>(),
                                     nr.as<int32_t>(), int(total), st);
  {
    DevBuf tmp;
    FQ_TRY(tmp.alloc(ctx, std::max<size_t>(tb, 16)));
    FQ_CUDA(ctx, cub::DeviceRunLengthEncode::Encode(tmp.p, tb, k2.as<uint64_t>(), ukeys.as<uint64_t>(),
                                                    lens.as<int32_t>(), nr.as<int32_t>(), int(total), st));
  }
  int32_t nruns = 0;
  FQ_CUDA(ctx, cudaMemcpyAsync(&nruns, nr.p, 4, cudaMemcpyDeviceToHost, st));
  FQ_CUDA(ctx, cudaStreamSynchronize(st));
  FQ_TRY(starts.alloc(ctx, (int64_t(nruns) + 1) * 8));
  {
    // run starts: exclusive scan of the run lengths (as 64-bit)
    std::vector<int32_t> hl(nruns);
    FQ_CUDA(ctx, cudaMemcpyAsync(hl.data(), lens.p, int64_t(nruns) * 4, cudaMemcpyDeviceToHost, st));
    FQ_CUDA(ctx, cudaStreamSynchronize(st));
    std::vector<int64_t> hs(size_t(nruns) + 1, 0);
    for (int32_t i = 0; i < nruns; ++i) hs[i + 1] = hs[i] + hl[i];
    FQ_CUDA(ctx, cudaMemcpyAsync(starts.p, hs.data(), (int64_t(nruns) + 1) * 8, cudaMemcpyHostToDevice, st));
    FQ_CUDA(ctx, cudaStreamSynchronize(st));
  }
  out.nnz = nruns;
  FQ_TRY(out.own_ci.alloc(ctx, std::max<int64_t>(nruns, 1) * 4));
  FQ_TRY(out.own_v64.alloc(ctx, std::max<int64_t>(nruns, 1) * 8));
  gp_segsum<<<grid_for_n(nruns), MT, 0, st>>>(v2.as<double>(), starts.as<int64_t>(), lens.as<int32_t>(),
                                             ukeys.as<uint64_t>(), nruns, nc, out.own_v64.as<double>(),
                                             out.own_ci.as<int32_t>());
  gp_rowptr<<<grid_for_n(nc + 1), MT, 0, st>>>(ukeys.as<uint64_t>(), nruns, nc, nc, out.own_rp.as<int32_t>());
  ctx->launches += 4;
  FQ_CUDA(ctx, cudaGetLastError());
  FQ_CUDA(ctx, cudaStreamSynchronize(st));
  out.rp = out.own_rp.as<int32_t>();
  out.ci = out.own_ci.as<int32_t>();
  out.v64 = out.own_v64.as<double>();
  out.v32 = nullptr;
  return FQ_OK;
}

// ---------------------------------------------------------------------------
// The HX block preconditioner (formoniq/src/hx.rs:hx_preconditioner with the
// blocks of MultigridBlocks), unrolled as in fq_hx.h.
// ---------------------------------------------------------------------------
template <typename VT>
void hx_apply(const HxPrecond& pc, const VT* r, VT* y, const int* done, cudaStream_t st) {
  const int m = pc.m;
  const NodalHierarchy& mg = pc.mg;
  VT* X = mg.lv[0].r.as<VT>();
  // gather the nodal right-hand sides
  for (const HxBlock& b : pc.blocks) {
    if (b.size == 0) continue;
    const VT* rb = r + b.off;
    if (b.grade >= 1) {
      gen_spmv<VT>(b.Dt, rb, b.t.as<VT>(), nullptr, nullptr, 0, 1, 1, 0, done, st);
      gen_spmv<VT>(b.PiLt, b.t.as<VT>(), X, nullptr, nullptr, 0, b.grad_count, m, b.grad_slot, done, st);
    }
    gen_spmv<VT>(b.Pit, rb, X, nullptr, nullptr, 0, b.vec_count, m, b.vec_slot, done, st);
  }
  const VT* V = vcycle<VT>(mg, 0, m, done, st);
  // scatter: y = S r + Pi V(..) [+ D (S_{j-1} t + Pi_{j-1} V(..))]
  for (const HxBlock& b : pc.blocks) {
    if (b.size == 0) continue;
    const VT* rb = r + b.off;
    VT* yb = y + b.off;
    gen_spmv<VT>(b.Pi, V, yb, pick<VT>(b.s64, b.s32), rb, 0, 1, 1, 0, done, st);
    if (b.grade >= 1) {
      gen_spmv<VT>(b.PiL, V, b.t2.as<VT>(), pick<VT>(b.sl64, b.sl32), b.t.as<VT>(), 0, 1, 1, 0, done, st);
      gen_spmv<VT>(b.D, b.t2.as<VT>(), yb, nullptr, nullptr, 1, 1, 1, 0, done, st);
    }
  }
  if (pc.ident_len > 0)
    copy_kernel<VT><<<grid_for_n(pc.ident_len), MT, 0, st>>>(r + pc.ident_off, y + pc.ident_off, pc.ident_len, done);
}

template void hx_apply<double>(const HxPrecond&, const double*, double*, const int*, cudaStream_t);
template void hx_apply<float>(const HxPrecond&, const float*, float*, const int*, cudaStream_t);

fq_status HxPrecond::make_f32(fq_ctx* ctx) {
  if (has_f32) return FQ_OK;
  auto conv = [&](const DevBuf& a, DevBuf& b, int64_t n) -> fq_status {
    FQ_TRY(b.alloc(ctx, std::max<int64_t>(n, 1) * 4));
    launch_f64_to_f32(a.as<double>(), b.as<float>(), n, ctx->stream);
    return FQ_OK;
  };
  for (auto& L : mg.lv) {
    FQ_TRY(L.A.make_f32(ctx));
    FQ_TRY(conv(L.dinv64, L.dinv32, L.n));
    if (L.P.nrows) FQ_TRY(L.P.make_f32(ctx));
    if (L.R.nrows) FQ_TRY(L.R.make_f32(ctx));
  }
  FQ_TRY(conv(mg.coarse_inv64, mg.coarse_inv32, mg.nc * mg.nc));
  for (auto& b : blocks) {
    FQ_TRY(conv(b.s64, b.s32, b.size));
    FQ_TRY(b.Pi.make_f32(ctx));
    FQ_TRY(b.Pit.make_f32(ctx));
    if (b.grade >= 1) {
      FQ_TRY(b.D.make_f32(ctx));
      FQ_TRY(b.Dt.make_f32(ctx));
      FQ_TRY(b.PiL.make_f32(ctx));
      FQ_TRY(b.PiLt.make_f32(ctx));
      FQ_TRY(conv(b.sl64, b.sl32, b.Dt.nrows));
    }
  }
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  has_f32 = true;
  return FQ_OK;
}

}  // namespace fq
