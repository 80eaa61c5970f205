// Kernel (d): the operator apply and the Krylov solvers, device resident.
//
// krylov::minres (iterative/src/krylov.rs:113-211) and krylov::cg (:48-95) are
// restated with their recurrences unchanged; only the data movement is new.
// Each iteration is three kernels:
//   A: the SpMV, fused with the Lanczos/CG vector update that consumes it,
//      and a per-block partial of the first inner product;
//   B: the remaining vector updates, the diagonal preconditioner, and the
//      partials of the second inner product;
//   C: the scalar recurrence (Givens rotation / step lengths), recomputed
//      identically by every block from the partials, and the solution update.
// Inner products are reduced in two fixed-order levels (block partials, then a
// per-block re-reduction of all partials), so results are deterministic and no
// scalar ever travels to the host inside the loop. The scalar state lives in
// two device slots written alternately, so a block never reads a slot that
// another block of the same kernel writes. The host only polls for convergence
// every few iterations.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <type_traits>
#include <vector>

#include "fq_df64.cuh"
#include "fq_hx.h"
#include "fq_internal.h"

namespace fq {

constexpr int KT = 256;          // threads per block of the vector kernels
constexpr int KBLOCKS = 152 * 4; // grid of the vector kernels: 4 blocks per SM
constexpr int PBLOCKS = 152 * 8; // grid cap of the fused SpMV kernels: 8 resident blocks per SM

struct SolverState {
  double beta1, beta, oldb, dbar, epsln, phibar, cs, sn;  // MINRES
  double alfa;
  double rbeta, c1;  // MINRES: 1 / beta and -beta / oldb for the next A kernel
  double rz, bnorm;                                       // CG
  double residual;
  long long iters;
  int done, converged, breakdown, pad;
};

__device__ __forceinline__ double block_sum(double v, double* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  double r = 0.0;
  if (w == 0) {
    r = (l < int(blockDim.x >> 5)) ? sh[l] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
    if (l == 0) sh[0] = r;
  }
  __syncthreads();
  r = sh[0];
  __syncthreads();
  return r;
}

// Every block reduces the same partial array in the same order.
__device__ __forceinline__ double reduce_partials(const double* part, int np, double* sh) {
  double v = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) v += part[i];
  return block_sum(v, sh);
}

// Per-iteration scalars of the Krylov loops and the arrival counters of their
// two grid reductions (device memory next to the two solver states).
struct IterScalars {
  double alfa, c2;        // MINRES, after A
  double ce, cd, cg, cp;  // MINRES, after the (preconditioned) product r2.y
  double alpha, beta;     // CG
  unsigned count[2];
  unsigned pad[2];
};

// A grid reduction without a second kernel and without every block repeating
// it: each block leaves its partial (thread 0, before the call), and the block
// that arrives last - told by a device-scope counter after a fence - reduces all
// partials and resets the counter for the next iteration. It sums in index
// order with reduce_partials' per-thread stride, so the total is bit-identical
// to the one every block used to recompute. The scalar recurrence (FP64
// divisions and square roots) then runs once, on that block's thread 0:
// repeated by every thread of a full grid it cost more on GB300's narrow FP64
// pipe than the vector work.
__device__ __forceinline__ bool arrive_last(unsigned* counter) {
  __shared__ unsigned ticket;
  if (threadIdx.x == 0) {
    __threadfence();
    ticket = atomicAdd(counter, 1u);
  }
  __syncthreads();
  return ticket == gridDim.x - 1;
}

__device__ __forceinline__ double reduce_arrived(const double* part, int np, double* sh) {
  double v = 0.0;
  for (int i = threadIdx.x; i < np; i += blockDim.x) v += __ldcg(part + i);
  return block_sum(v, sh);
}

// Sub-warp CSR row product: W lanes per row, fixed lane order.
template <int W, typename VT>
__device__ __forceinline__ VT row_dot(const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                      const VT* __restrict__ val, const VT* __restrict__ x, int64_t row, bool valid,
                                      int lane) {
  // two independent accumulators keep two gathers in flight per lane
  VT acc0 = VT(0), acc1 = VT(0);
  if (valid) {
    const int b = __ldg(rp + row), e = __ldg(rp + row + 1);
    int t = b + lane;
    for (; t + W < e; t += 2 * W) {
      const int c0 = __ldg(ci + t), c1 = __ldg(ci + t + W);
      const VT v0 = __ldg(val + t), v1 = __ldg(val + t + W);
      acc0 += v0 * __ldg(x + c0);
      acc1 += v1 * __ldg(x + c1);
    }
    if (t < e) acc0 += __ldg(val + t) * __ldg(x + __ldg(ci + t));
  }
  VT acc = acc0 + acc1;
#pragma unroll
  for (int o = W / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, W);
  return acc;
}

// The same product for an FP64 operator evaluated on the FP32 pipe: values and
// the gathered vector as float-float pairs (each split once from its double,
// exactly to 48 bits), products and sums in float-float, one FP64 add per row
// to round the result. GB300's FP64 pipe issues a small fraction of the FP32
// rate, and an FP64 CSR product with ~30 entries per row is bound by it, not by
// memory; the pairs occupy the same 8 bytes as the doubles.
__device__ __forceinline__ df64 ldg_df(const df64* p) {
  const float2 f = __ldg(reinterpret_cast<const float2*>(p));
  return df64(f.x, f.y);
}

template <int W>
__device__ __forceinline__ df64 row_dot_split(const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                              const df64* __restrict__ val, const df64* __restrict__ x, int64_t row,
                                              bool valid, int lane) {
  df64 acc0, acc1;
  if (valid) {
    const int b = __ldg(rp + row), e = __ldg(rp + row + 1);
    int t = b + lane;
    for (; t + W < e; t += 2 * W) {
      const int c0 = __ldg(ci + t), c1 = __ldg(ci + t + W);
      const df64 v0 = ldg_df(val + t), v1 = ldg_df(val + t + W);
      acc0 += v0 * ldg_df(x + c0);
      acc1 += v1 * ldg_df(x + c1);
    }
    if (t < e) acc0 += ldg_df(val + t) * ldg_df(x + __ldg(ci + t));
  }
  df64 acc = acc0 + acc1;
#pragma unroll
  for (int o = W / 2; o > 0; o >>= 1) {
    const df64 other(__shfl_xor_sync(0xffffffffu, acc.hi, o, W), __shfl_xor_sync(0xffffffffu, acc.lo, o, W));
    acc = acc + other;
  }
  return acc;
}

__global__ void split_kernel(const double* __restrict__ a, df64* __restrict__ out, int64_t n) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    out[i] = df64(a[i]);
}

// ---------------------------------------------------------------------------
// plain SpMV (LinearOperator::apply)
// ---------------------------------------------------------------------------
template <int W, typename VT>
__global__ void __launch_bounds__(KT) spmv_kernel(const int32_t* rp, const int32_t* ci, const VT* val, const VT* x,
                                                  VT* y, int64_t nrows) {
  const int lane = threadIdx.x % W;
  const int64_t rows_per_grid = int64_t(gridDim.x) * (blockDim.x / W);
  for (int64_t base = int64_t(blockIdx.x) * (blockDim.x / W); base < nrows; base += rows_per_grid) {
    const int64_t row = base + threadIdx.x / W;
    const bool valid = row < nrows;
    const VT acc = row_dot<W, VT>(rp, ci, val, x, row, valid, lane);
    if (valid && lane == 0) y[row] = acc;
  }
}

// Lanes per row of the sub-warp CSR kernels. In FP64 each lane's products, the
// join of its two accumulators and every shuffle level are FP64 instructions,
// and GB300 issues FP64 at a small fraction of the FP32 rate (the fused MINRES
// SpMV measured FP64-pipe bound at W = 16), so FP64 rows get fewer lanes: more
// rows per warp and fewer reduction adds per row. FP32 keeps the memory-tuned
// choice.
template <typename VT>
static int pick_w(int64_t nnz, int64_t nrows) {
  const double avg = nrows > 0 ? double(nnz) / double(nrows) : 0.0;
  if (std::is_same<VT, double>::value) {
    if (avg <= 48) return 4;
    if (avg <= 160) return 8;
    return 16;
  }
  if (avg <= 6) return 4;
  if (avg <= 14) return 8;
  if (avg <= 80) return 16;
  return 32;
}

// Lanes per row of the split (float-float) FP64 product. Its sums run on the
// FP32 pipe, but the per-row epilogue (scaling, the dot partial) stays FP64 and
// costs a warp instruction per row group, so rows keep few lanes: W = 4 puts 8
// rows in each of those instructions.
static int pick_w_split(int64_t nnz, int64_t nrows) {
  const double avg = nrows > 0 ? double(nnz) / double(nrows) : 0.0;
  if (avg <= 48) return 4;
  if (avg <= 160) return 8;
  return 16;
}

static int spmv_blocks(int64_t nrows, int W) {
  const int64_t rows_per_block = KT / W;
  return int(std::max<int64_t>(1, std::min<int64_t>((nrows + rows_per_block - 1) / rows_per_block, 152 * 16)));
}

template <typename VT>
static void spmv_dispatch(const int32_t* rp, const int32_t* ci, const VT* val, const VT* x, VT* y, int64_t nrows,
                          int64_t nnz, cudaStream_t st) {
  const int W = pick_w<VT>(nnz, nrows);
  const int g = spmv_blocks(nrows, W);
  switch (W) {
    case 4:
      spmv_kernel<4, VT><<<g, KT, 0, st>>>(rp, ci, val, x, y, nrows);
      break;
    case 8:
      spmv_kernel<8, VT><<<g, KT, 0, st>>>(rp, ci, val, x, y, nrows);
      break;
    case 16:
      spmv_kernel<16, VT><<<g, KT, 0, st>>>(rp, ci, val, x, y, nrows);
      break;
    default:
      spmv_kernel<32, VT><<<g, KT, 0, st>>>(rp, ci, val, x, y, nrows);
      break;
  }
}

void launch_spmv(const fq_matrix* a, const void* x, void* y, cudaStream_t st) {
  if (a->nrows == 0) return;
  if (a->precision == FQ_FP32)
    spmv_dispatch<float>(a->rp, a->ci, a->values.as<float>(), static_cast<const float*>(x), static_cast<float*>(y),
                         a->nrows, a->nnz, st);
  else
    spmv_dispatch<double>(a->rp, a->ci, a->values.as<double>(), static_cast<const double*>(x),
                          static_cast<double*>(y), a->nrows, a->nnz, st);
}

// ---------------------------------------------------------------------------
// MINRES
// ---------------------------------------------------------------------------
template <typename VT>
struct MinresVecs {
  VT *x, *r1, *r2, *y, *v, *z, *w, *w2;
  const VT* dinv;  // may be null: identity preconditioner
  int external;    // 1: y = P r2 is applied by separate kernels (dinv unused)
  const VT* b;
  double *partA, *partB;
  df64* y2;  // FP64: y as float-float pairs for the split product (null otherwise)
};

template <typename VT>
__global__ void __launch_bounds__(KT) minres_init(MinresVecs<VT> m, int64_t n) {
  __shared__ double sh[32];
  double acc = 0.0;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const VT bi = m.b[i];
    const VT yi = m.dinv ? bi * m.dinv[i] : bi;
    m.r1[i] = bi;
    m.r2[i] = bi;
    m.y[i] = yi;
    if constexpr (std::is_same<VT, double>::value)
      if (m.y2) m.y2[i] = df64(yi);
    m.x[i] = VT(0);
    m.w[i] = VT(0);
    m.w2[i] = VT(0);
    acc += double(bi) * double(yi);
  }
  acc = block_sum(acc, sh);
  if (threadIdx.x == 0) m.partB[blockIdx.x] = acc;
}

__global__ void minres_init_state(SolverState* s0, SolverState* s1, const double* partB, int np, double rtol,
                                  long long max_iters) {
  __shared__ double sh[32];
  const double beta1_sq = reduce_partials(partB, np, sh);
  if (threadIdx.x == 0) {
    SolverState s{};
    s.iters = 0;
    if (!(beta1_sq > 0.0)) {
      // b = 0 (trivial solve) or a non-positive preconditioner product.
      s.done = 1;
      s.converged = beta1_sq == 0.0 ? 1 : 0;
      s.breakdown = beta1_sq == 0.0 ? 0 : 1;
      s.residual = 0.0;
    } else {
      const double beta1 = sqrt(beta1_sq);
      s.beta1 = beta1;
      s.beta = beta1;
      s.oldb = 0.0;
      s.dbar = 0.0;
      s.epsln = 0.0;
      s.phibar = beta1;
      s.cs = -1.0;
      s.sn = 0.0;
      s.rbeta = 1.0 / beta1;
      s.c1 = 0.0;
      s.residual = 1.0;
      s.done = max_iters <= 0 ? 1 : 0;
    }
    (void)rtol;
    *s0 = s;
    *s1 = s;
  }
}

// The MINRES rotation (krylov.rs:113-211) on one thread: the next state into
// *out and the w/x update coefficients into X.
__device__ void minres_rotate(const SolverState& in, double alfa, double beta_sq, double rtol, long long max_iters,
                              IterScalars* X, SolverState* out) {
  SolverState s = in;
  const double eps = DBL_EPSILON;
  const double oldb = s.beta;
  const double beta = sqrt(fmax(beta_sq, 0.0));
  const double oldeps = s.epsln;
  const double delta = s.cs * s.dbar + s.sn * alfa;
  const double gbar = s.sn * s.dbar - s.cs * alfa;
  const double epsln = s.sn * beta;
  const double dbar = -s.cs * beta;
  const double gamma = fmax(sqrt(gbar * gbar + beta * beta), eps);
  const double cs = gbar / gamma;
  const double sn = beta / gamma;
  const double phi = cs * s.phibar;
  const double phibar = s.phibar * sn;
  X->ce = -oldeps;
  X->cd = -delta;
  X->cg = 1.0 / gamma;
  X->cp = phi;
  s.oldb = oldb;
  s.beta = beta;
  s.epsln = epsln;
  s.dbar = dbar;
  s.cs = cs;
  s.sn = sn;
  s.phibar = phibar;
  s.alfa = alfa;
  s.rbeta = 1.0 / beta;
  s.c1 = -beta / oldb;
  s.iters += 1;
  s.residual = phibar / s.beta1;
  if (!isfinite(s.residual)) {
    s.breakdown = 1;
    s.done = 1;
  }
  if (s.residual <= rtol) {
    s.converged = 1;
    s.done = 1;
  }
  if (s.iters >= max_iters) s.done = 1;
  *out = s;
}

// The last block of A: alfa = v.z and the coefficient of B.
__device__ __forceinline__ void minres_after_a(double acc, double* partA, const SolverState* S, IterScalars* X,
                                               double* sh) {
  if (threadIdx.x == 0) partA[blockIdx.x] = acc;
  if (arrive_last(&X->count[0])) {
    const double alfa = reduce_arrived(partA, gridDim.x, sh);
    if (threadIdx.x == 0) {
      X->alfa = alfa;
      X->c2 = -alfa / S->beta;
      X->count[0] = 0u;
    }
  }
}

// The last block of the kernel that forms r2.y: the rotation.
__device__ __forceinline__ void minres_after_b(double acc, double* partB, const SolverState* S, IterScalars* X,
                                               SolverState* Sout, double rtol, long long max_iters, double* sh) {
  if (threadIdx.x == 0) partB[blockIdx.x] = acc;
  if (arrive_last(&X->count[1])) {
    const double beta_sq = reduce_arrived(partB, gridDim.x, sh);
    if (threadIdx.x == 0) {
      minres_rotate(*S, X->alfa, beta_sq, rtol, max_iters, X, Sout);
      X->count[1] = 0u;
    }
  }
}

// A: v = y / beta, z = A v - (beta/oldb) r1, alfa = v.z
template <int W, typename VT>
__global__ void __launch_bounds__(KT) minres_a(const int32_t* rp, const int32_t* ci, const VT* val, MinresVecs<VT> m,
                                               const SolverState* __restrict__ S, IterScalars* X, int64_t n) {
  __shared__ double sh[32];
  if (S->done) return;
  const VT rbt = VT(S->rbeta), c1t = VT(S->c1);
  const int lane = threadIdx.x % W;
  double acc = 0.0;
  const int64_t rows_per_grid = int64_t(gridDim.x) * (blockDim.x / W);
  for (int64_t base = int64_t(blockIdx.x) * (blockDim.x / W); base < n; base += rows_per_grid) {
    const int64_t row = base + threadIdx.x / W;
    const bool valid = row < n;
    const VT av = row_dot<W, VT>(rp, ci, val, m.y, row, valid, lane);
    if (valid && lane == 0) {
      const VT vi = m.y[row] * rbt;
      const VT zi = av * rbt + c1t * m.r1[row];
      m.v[row] = vi;
      m.z[row] = zi;
      acc += double(vi) * double(zi);
    }
  }
  acc = block_sum(acc, sh);
  minres_after_a(acc, m.partA, S, X, sh);
}

// A for an FP64 operator on the FP32 pipe (values and y as float-float pairs).
template <int W>
__global__ void __launch_bounds__(KT) minres_a_split(const int32_t* rp, const int32_t* ci, const df64* val,
                                                     MinresVecs<double> m, const SolverState* __restrict__ S,
                                                     IterScalars* X, int64_t n) {
  __shared__ double sh[32];
  if (S->done) return;
  const double rbt = S->rbeta, c1t = S->c1;
  const int lane = threadIdx.x % W;
  double acc = 0.0;
  const int64_t rows_per_grid = int64_t(gridDim.x) * (blockDim.x / W);
  for (int64_t base = int64_t(blockIdx.x) * (blockDim.x / W); base < n; base += rows_per_grid) {
    const int64_t row = base + threadIdx.x / W;
    const bool valid = row < n;
    const df64 av = row_dot_split<W>(rp, ci, val, m.y2, row, valid, lane);
    if (valid && lane == 0) {
      const double vi = m.y[row] * rbt;
      const double zi = av.to_double() * rbt + c1t * m.r1[row];
      m.v[row] = vi;
      m.z[row] = zi;
      acc += vi * zi;
    }
  }
  acc = block_sum(acc, sh);
  minres_after_a(acc, m.partA, S, X, sh);
}

// B: z -= (alfa/beta) r2; r1 = r2; r2 = z; y = P r2 (diagonal P); r2.y and the rotation
template <typename VT>
__global__ void __launch_bounds__(KT) minres_b(MinresVecs<VT> m, const SolverState* __restrict__ S, IterScalars* X,
                                               SolverState* __restrict__ Sout, double rtol, long long max_iters,
                                               int64_t n) {
  __shared__ double sh[32];
  if (S->done) return;
  const VT c2 = VT(X->c2);
  double acc = 0.0;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const VT r2 = m.r2[i];
    const VT zi = m.z[i] + c2 * r2;
    m.r1[i] = r2;
    m.r2[i] = zi;
    if (!m.external) {
      const VT yi = m.dinv ? zi * m.dinv[i] : zi;
      m.y[i] = yi;
      if constexpr (std::is_same<VT, double>::value)
        if (m.y2) m.y2[i] = df64(yi);
      acc += double(zi) * double(yi);
    }
  }
  if (m.external) return;  // y = P r2 and r2.y come from the preconditioner and minres_dot
  acc = block_sum(acc, sh);
  minres_after_b(acc, m.partB, S, X, Sout, rtol, max_iters, sh);
}

// r2.y after an external preconditioner wrote y = P r2 (and y's float pairs),
// then the rotation.
template <typename VT>
__global__ void __launch_bounds__(KT) minres_dot(MinresVecs<VT> m, const SolverState* __restrict__ S,
                                                 IterScalars* X, SolverState* __restrict__ Sout, double rtol,
                                                 long long max_iters, int64_t n) {
  __shared__ double sh[32];
  if (S->done) return;
  double acc = 0.0;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const VT yi = m.y[i];
    acc += double(m.r2[i]) * double(yi);
    if constexpr (std::is_same<VT, double>::value)
      if (m.y2) m.y2[i] = df64(yi);
  }
  acc = block_sum(acc, sh);
  minres_after_b(acc, m.partB, S, X, Sout, rtol, max_iters, sh);
}

// Partials of a.b (after an external preconditioner wrote b = P a).
template <typename VT>
__global__ void __launch_bounds__(KT) dot_partials(const VT* __restrict__ a, const VT* __restrict__ b,
                                                   double* __restrict__ part, int64_t n, const int* __restrict__ done,
                                                   df64* __restrict__ b2 = nullptr) {
  __shared__ double sh[32];
  if (done && *done) return;
  double acc = 0.0;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    acc += double(a[i]) * double(b[i]);
    if constexpr (std::is_same<VT, double>::value)
      if (b2) b2[i] = df64(b[i]);  // the split copy of b the next product gathers
  }
  acc = block_sum(acc, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

// C: the w/x update with the rotation's coefficients; a finished loop carries
// its state to the other slot
template <typename VT>
__global__ void __launch_bounds__(KT) minres_c(MinresVecs<VT> m, const SolverState* __restrict__ Sin,
                                               SolverState* __restrict__ Sout, const IterScalars* __restrict__ X,
                                               int64_t n) {
  if (Sin->done) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *Sout = *Sin;
    return;
  }
  const VT ce = VT(X->ce), cd = VT(X->cd), cg = VT(X->cg), cp = VT(X->cp);
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const VT w = m.w[i];
    VT wn = m.v[i] + ce * m.w2[i];
    wn = wn + cd * w;
    wn = wn * cg;
    m.w2[i] = w;
    m.w[i] = wn;
    m.x[i] = m.x[i] + cp * wn;
  }
}

// ---------------------------------------------------------------------------
// CG
// ---------------------------------------------------------------------------
template <typename VT>
struct CgVecs {
  VT *x, *r, *z, *p, *ap;
  const VT* dinv;
  int external;  // 1: z = P r is applied by separate kernels (dinv unused)
  const VT* b;
  double *partA, *partB, *partC;
  df64* p2;  // FP64: p as float-float pairs for the split product (null otherwise)
};

template <typename VT>
__global__ void __launch_bounds__(KT) cg_init(CgVecs<VT> c, int64_t n) {
  __shared__ double sh[32];
  double rz = 0.0, bb = 0.0;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const VT bi = c.b[i];
    const VT zi = c.dinv ? bi * c.dinv[i] : bi;
    c.x[i] = VT(0);
    c.r[i] = bi;
    c.z[i] = zi;
    c.p[i] = zi;
    if constexpr (std::is_same<VT, double>::value)
      if (c.p2) c.p2[i] = df64(zi);
    rz += double(bi) * double(zi);
    bb += double(bi) * double(bi);
  }
  rz = block_sum(rz, sh);
  bb = block_sum(bb, sh);
  if (threadIdx.x == 0) {
    c.partB[blockIdx.x] = rz;
    c.partC[blockIdx.x] = bb;
  }
}

__global__ void cg_init_state(SolverState* s0, SolverState* s1, const double* partB, const double* partC, int np,
                              double rtol, long long max_iters) {
  __shared__ double sh[32];
  const double rz = reduce_partials(partB, np, sh);
  const double bb = reduce_partials(partC, np, sh);
  if (threadIdx.x == 0) {
    SolverState s{};
    s.bnorm = sqrt(bb);
    s.rz = rz;
    s.iters = 0;
    if (s.bnorm == 0.0) {
      s.done = 1;
      s.converged = 1;
      s.residual = 0.0;
    } else {
      s.residual = 1.0;
      s.converged = s.residual <= rtol;
      s.done = s.converged || max_iters <= 0;
    }
    *s0 = s;
    *s1 = s;
  }
}

// CG's scalar step on one thread: beta and the next state.
__device__ void cg_advance(const SolverState& in, double rz_next, double rr, double rtol, long long max_iters,
                           IterScalars* X, SolverState* out) {
  SolverState s = in;
  X->beta = rz_next / in.rz;
  s.rz = rz_next;
  s.iters += 1;
  s.residual = sqrt(rr) / s.bnorm;
  if (!isfinite(s.residual)) {
    s.breakdown = 1;
    s.done = 1;
  }
  if (s.residual <= rtol) {
    s.converged = 1;
    s.done = 1;
  }
  if (s.iters >= max_iters) s.done = 1;
  *out = s;
}

// The last block of A: alpha = rz / p.ap.
__device__ __forceinline__ void cg_after_a(double acc, double* partA, const SolverState* S, IterScalars* X,
                                           double* sh) {
  if (threadIdx.x == 0) partA[blockIdx.x] = acc;
  if (arrive_last(&X->count[0])) {
    const double pap = reduce_arrived(partA, gridDim.x, sh);
    if (threadIdx.x == 0) {
      X->alpha = S->rz / pap;
      X->count[0] = 0u;
    }
  }
}

// The last block of the kernel that forms r.z (r.r from cg_b, npc partials):
// beta and the next state.
__device__ __forceinline__ void cg_after_b(const double* partB, const double* partC, int npc, const SolverState* S,
                                           IterScalars* X, SolverState* Sout, double rtol, long long max_iters,
                                           double* sh) {
  if (arrive_last(&X->count[1])) {
    const double rz_next = reduce_arrived(partB, gridDim.x, sh);
    const double rr = reduce_arrived(partC, npc, sh);
    if (threadIdx.x == 0) {
      cg_advance(*S, rz_next, rr, rtol, max_iters, X, Sout);
      X->count[1] = 0u;
    }
  }
}

// A: ap = A p, alpha
template <int W, typename VT>
__global__ void __launch_bounds__(KT) cg_a(const int32_t* rp, const int32_t* ci, const VT* val, CgVecs<VT> c,
                                           const SolverState* __restrict__ S, IterScalars* X, int64_t n) {
  __shared__ double sh[32];
  if (S->done) return;
  const int lane = threadIdx.x % W;
  double acc = 0.0;
  const int64_t rows_per_grid = int64_t(gridDim.x) * (blockDim.x / W);
  for (int64_t base = int64_t(blockIdx.x) * (blockDim.x / W); base < n; base += rows_per_grid) {
    const int64_t row = base + threadIdx.x / W;
    const bool valid = row < n;
    const VT av = row_dot<W, VT>(rp, ci, val, c.p, row, valid, lane);
    if (valid && lane == 0) {
      c.ap[row] = av;
      acc += double(c.p[row]) * double(av);
    }
  }
  acc = block_sum(acc, sh);
  cg_after_a(acc, c.partA, S, X, sh);
}

// A for an FP64 operator on the FP32 pipe (values and p as float-float pairs).
template <int W>
__global__ void __launch_bounds__(KT) cg_a_split(const int32_t* rp, const int32_t* ci, const df64* val,
                                                 CgVecs<double> c, const SolverState* __restrict__ S, IterScalars* X,
                                                 int64_t n) {
  __shared__ double sh[32];
  if (S->done) return;
  const int lane = threadIdx.x % W;
  double acc = 0.0;
  const int64_t rows_per_grid = int64_t(gridDim.x) * (blockDim.x / W);
  for (int64_t base = int64_t(blockIdx.x) * (blockDim.x / W); base < n; base += rows_per_grid) {
    const int64_t row = base + threadIdx.x / W;
    const bool valid = row < n;
    const df64 av = row_dot_split<W>(rp, ci, val, c.p2, row, valid, lane);
    if (valid && lane == 0) {
      const double a = av.to_double();
      c.ap[row] = a;
      acc += c.p[row] * a;
    }
  }
  acc = block_sum(acc, sh);
  cg_after_a(acc, c.partA, S, X, sh);
}

// p.ap after an operator hook wrote ap = A p (matrix-free), then alpha.
__global__ void __launch_bounds__(KT) cg_pap(CgVecs<double> c, const SolverState* __restrict__ S, IterScalars* X,
                                             int64_t n) {
  __shared__ double sh[32];
  if (S->done) return;
  double acc = 0.0;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    acc += c.p[i] * c.ap[i];
  acc = block_sum(acc, sh);
  cg_after_a(acc, c.partA, S, X, sh);
}

// B: x += alpha p; r -= alpha ap; z = P r (diagonal P); r.z, r.r and the scalar step
template <typename VT>
__global__ void __launch_bounds__(KT) cg_b(CgVecs<VT> c, const SolverState* __restrict__ S, IterScalars* X,
                                           SolverState* __restrict__ Sout, double rtol, long long max_iters,
                                           int64_t n) {
  __shared__ double sh[32];
  if (S->done) return;
  const double alpha = X->alpha;
  const VT at = VT(alpha), mat = VT(-alpha);
  double rz = 0.0, rr = 0.0;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    c.x[i] = c.x[i] + at * c.p[i];
    const VT ri = c.r[i] + mat * c.ap[i];
    c.r[i] = ri;
    if (!c.external) {
      const VT zi = c.dinv ? ri * c.dinv[i] : ri;
      c.z[i] = zi;
      rz += double(ri) * double(zi);
    }
    rr += double(ri) * double(ri);
  }
  rz = block_sum(rz, sh);
  rr = block_sum(rr, sh);
  if (threadIdx.x == 0) {
    if (!c.external) c.partB[blockIdx.x] = rz;
    c.partC[blockIdx.x] = rr;
  }
  if (c.external) return;  // z = P r and r.z come from the preconditioner and cg_dot
  cg_after_b(c.partB, c.partC, gridDim.x, S, X, Sout, rtol, max_iters, sh);
}

// r.z after an external preconditioner wrote z = P r, then the scalar step
// (r.r from cg_b's npc partials).
template <typename VT>
__global__ void __launch_bounds__(KT) cg_dot(CgVecs<VT> c, const SolverState* __restrict__ S, IterScalars* X,
                                             SolverState* __restrict__ Sout, int npc, double rtol,
                                             long long max_iters, int64_t n) {
  __shared__ double sh[32];
  if (S->done) return;
  double acc = 0.0;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    acc += double(c.r[i]) * double(c.z[i]);
  acc = block_sum(acc, sh);
  if (threadIdx.x == 0) c.partB[blockIdx.x] = acc;
  cg_after_b(c.partB, c.partC, npc, S, X, Sout, rtol, max_iters, sh);
}

// External preconditioner, first step: p = z (= P b), partials of b.z.
template <typename VT>
__global__ void __launch_bounds__(KT) cg_init_p(CgVecs<VT> c, int64_t n) {
  __shared__ double sh[32];
  double rz = 0.0;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const VT zi = c.z[i];
    c.p[i] = zi;
    if constexpr (std::is_same<VT, double>::value)
      if (c.p2) c.p2[i] = df64(zi);
    rz += double(c.b[i]) * double(zi);
  }
  rz = block_sum(rz, sh);
  if (threadIdx.x == 0) c.partB[blockIdx.x] = rz;
}

// C: p = beta p + z; a finished loop carries its state to the other slot
template <typename VT>
__global__ void __launch_bounds__(KT) cg_c(CgVecs<VT> c, const SolverState* __restrict__ Sin,
                                           SolverState* __restrict__ Sout, const IterScalars* __restrict__ X,
                                           int64_t n) {
  if (Sin->done) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *Sout = *Sin;
    return;
  }
  const VT bt = VT(X->beta);
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const VT pi = c.p[i] * bt + c.z[i];
    c.p[i] = pi;
    if constexpr (std::is_same<VT, double>::value)
      if (c.p2) c.p2[i] = df64(pi);
  }
}

// ---------------------------------------------------------------------------
// Host drivers
// ---------------------------------------------------------------------------

// Runs `one_iteration(parity)` (the three kernels of one iteration, reading
// state slot `parity` and writing slot 1 - parity) as a CUDA graph of two
// iterations, relaunched until the device state says done. Convergence is
// polled through pinned memory one batch behind the launches, so the device
// always has the next batch queued; iterations after convergence are no-ops.
template <typename F>
static fq_status run_graph_loop(fq_ctx* ctx, SolverState* S, int64_t max_iters, F&& one_iteration,
                                SolverState* final_state, int64_t max_batch = 64) {
  cudaStream_t st = ctx->stream;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  // A stream that cannot be captured (the legacy default stream) falls back to
  // direct launches of the same kernels.
  if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
    one_iteration(0);
    one_iteration(1);
    // a launch refused during capture leaves its kernel out of the graph: an
    // error, not an iteration to run without it
    const cudaError_t le = cudaGetLastError();
    cudaError_t ce = cudaStreamEndCapture(st, &graph);
    if (le != cudaSuccess) {
      if (ce == cudaSuccess) cudaGraphDestroy(graph);
      return cuda_check(ctx, le, "iteration launch (capture)");
    }
    if (ce == cudaSuccess) {
      ce = cudaGraphInstantiate(&exec, graph, 0);
      cudaGraphDestroy(graph);
      if (ce != cudaSuccess) exec = nullptr;
    }
    // a capture that failed leaves the iteration to direct launches
    if (ce != cudaSuccess) cudaGetLastError();
  } else {
    cudaGetLastError();
  }
  static_assert(2 * sizeof(SolverState) <= 1024, "pinned polling slots");
  SolverState* pinned = static_cast<SolverState*>(ctx->host_solver);
  cudaEvent_t ev[2];
  cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming);
  cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming);
  fq_status status = FQ_OK;
  int64_t launched = 0;  // iterations enqueued
  int64_t batch = 4;     // graph launches (x2 iterations) per batch
  int slot = 0;
  bool have_prev = false;
  for (;;) {
    const int64_t nlaunch = std::min<int64_t>(batch, (max_iters - launched + 1) / 2 + 1);
    for (int64_t i = 0; i < nlaunch; ++i) {
      cudaError_t e = cudaSuccess;
      if (exec) {
        e = cudaGraphLaunch(exec, st);
      } else {
        one_iteration(0);
        one_iteration(1);
        e = cudaGetLastError();
      }
      if (e != cudaSuccess) {
        status = cuda_check(ctx, e, "iteration launch");
        break;
      }
    }
    if (status != FQ_OK) break;
    ctx->launches += uint64_t(6 * nlaunch);
    launched += 2 * nlaunch;
    cudaMemcpyAsync(pinned + slot, S, sizeof(SolverState), cudaMemcpyDeviceToHost, st);
    cudaEventRecord(ev[slot], st);
    if (have_prev) {
      cudaEventSynchronize(ev[1 - slot]);
      if (pinned[1 - slot].done) break;
    }
    have_prev = true;
    slot = 1 - slot;
    if (launched > max_iters + 2) {
      cudaEventSynchronize(ev[1 - slot]);
      break;
    }
    batch = std::min<int64_t>(batch * 2, max_batch);
  }
  cudaError_t e = cudaMemcpyAsync(pinned, S, sizeof(SolverState), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) *final_state = pinned[0];
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  if (exec) cudaGraphExecDestroy(exec);
  if (status != FQ_OK) return status;
  if (e != cudaSuccess) return cuda_check(ctx, e, "cudaMemcpy state");
  return FQ_OK;
}

template <typename VT>
fq_status minres_run(fq_ctx* ctx, const int32_t* rp, const int32_t* ci, const VT* val, int64_t n, int64_t nnz,
                     const VT* dinv, const HxPrecond* pc, const VT* b, VT* x, double rtol, int64_t max_iters,
                     fq_report* rep) {
  cudaStream_t st = ctx->stream;
  DevBuf vecs, parts, state;
  const size_t vb = size_t(std::max<int64_t>(n, 1)) * sizeof(VT);
  FQ_TRY(vecs.alloc(ctx, vb * 7));
  FQ_TRY(parts.alloc(ctx, 2 * PBLOCKS * sizeof(double)));
  FQ_TRY(state.alloc(ctx, 2 * sizeof(SolverState) + sizeof(IterScalars)));
  MinresVecs<VT> m;
  char* base = vecs.as<char>();
  m.x = x;
  m.r1 = reinterpret_cast<VT*>(base + 0 * vb);
  m.r2 = reinterpret_cast<VT*>(base + 1 * vb);
  m.y = reinterpret_cast<VT*>(base + 2 * vb);
  m.v = reinterpret_cast<VT*>(base + 3 * vb);
  m.z = reinterpret_cast<VT*>(base + 4 * vb);
  m.w = reinterpret_cast<VT*>(base + 5 * vb);
  m.w2 = reinterpret_cast<VT*>(base + 6 * vb);
  m.dinv = pc ? nullptr : dinv;
  m.external = pc ? 1 : 0;
  m.b = b;
  m.partA = parts.as<double>();
  m.partB = parts.as<double>() + PBLOCKS;
  m.y2 = nullptr;
  SolverState* S = state.as<SolverState>();
  IterScalars* X = reinterpret_cast<IterScalars*>(S + 2);  // per-iteration scalars, reduction counters at 0
  FQ_CUDA(ctx, cudaMemsetAsync(X, 0, sizeof(IterScalars), st));
  // FP64: the product runs on float-float pairs of the values and of y
  constexpr bool split = std::is_same<VT, double>::value;
  DevBuf val2, y2;
  if constexpr (split) {
    FQ_TRY(val2.alloc(ctx, size_t(std::max<int64_t>(nnz, 1)) * sizeof(df64)));
    FQ_TRY(y2.alloc(ctx, size_t(std::max<int64_t>(n, 1)) * sizeof(df64)));
    m.y2 = y2.as<df64>();
    if (nnz > 0) {
      split_kernel<<<int(std::min<int64_t>((nnz + KT - 1) / KT, KBLOCKS)), KT, 0, st>>>(
          val, val2.as<df64>(), nnz);
      ctx->launches++;
    }
  }
  const int W = split ? pick_w_split(nnz, n) : pick_w<VT>(nnz, n);
  const int ga = std::min(spmv_blocks(n, W), PBLOCKS);
  const int gv = int(std::max<int64_t>(1, std::min<int64_t>((n + KT - 1) / KT, KBLOCKS)));
  minres_init<VT><<<gv, KT, 0, st>>>(m, n);
  if (pc) {
    hx_apply<VT>(*pc, b, m.y, nullptr, st);
    dot_partials<VT><<<gv, KT, 0, st>>>(b, m.y, m.partB, n, nullptr, m.y2);
  }
  minres_init_state<<<1, KT, 0, st>>>(S, S + 1, m.partB, gv, rtol, (long long)max_iters);
  ctx->launches += 2;
  SolverState hs{};
  // (a runtime branch around the constexpr one: a kernel launch that follows an
  // `if constexpr ... else` in this lambda was dropped from the device code)
  auto iteration = [&](int cur) {
    if (split) {
      if constexpr (split) {
        const df64* v2 = val2.as<df64>();
        switch (W) {
          case 4:
            minres_a_split<4><<<ga, KT, 0, st>>>(rp, ci, v2, m, S + cur, X, n);
            break;
          case 8:
            minres_a_split<8><<<ga, KT, 0, st>>>(rp, ci, v2, m, S + cur, X, n);
            break;
          case 16:
            minres_a_split<16><<<ga, KT, 0, st>>>(rp, ci, v2, m, S + cur, X, n);
            break;
          default:
            minres_a_split<32><<<ga, KT, 0, st>>>(rp, ci, v2, m, S + cur, X, n);
            break;
        }
      }
    } else {
      switch (W) {
        case 4:
          minres_a<4, VT><<<ga, KT, 0, st>>>(rp, ci, val, m, S + cur, X, n);
          break;
        case 8:
          minres_a<8, VT><<<ga, KT, 0, st>>>(rp, ci, val, m, S + cur, X, n);
          break;
        case 16:
          minres_a<16, VT><<<ga, KT, 0, st>>>(rp, ci, val, m, S + cur, X, n);
          break;
        default:
          minres_a<32, VT><<<ga, KT, 0, st>>>(rp, ci, val, m, S + cur, X, n);
          break;
      }
    }
    minres_b<VT><<<gv, KT, 0, st>>>(m, S + cur, X, S + (1 - cur), rtol, (long long)max_iters, n);
    if (pc) {
      const int* done = &(S + cur)->done;
      hx_apply<VT>(*pc, m.r2, m.y, done, st);
      minres_dot<VT><<<gv, KT, 0, st>>>(m, S + cur, X, S + (1 - cur), rtol, (long long)max_iters, n);
    }
    minres_c<VT><<<gv, KT, 0, st>>>(m, S + cur, S + (1 - cur), X, n);
  };
  // a preconditioned iteration costs more: poll more often so fewer finished
  // iterations are queued past convergence
  FQ_TRY(run_graph_loop(ctx, S, max_iters, iteration, &hs, pc ? 4 : 64));
  rep->iters = hs.iters;
  rep->residual = hs.residual;
  rep->converged = hs.converged;
  if (hs.breakdown) return set_error(ctx, FQ_BREAKDOWN, "MINRES breakdown (non-positive preconditioner product or NaN)");
  return FQ_OK;
}

// CG on A given either as CSR (rp, ci, val) or, with `hook`, as an operator
// applied by its own kernels (matrix-free); the recurrences are the same.
template <typename VT>
static fq_status cg_impl(fq_ctx* ctx, const int32_t* rp, const int32_t* ci, const VT* val, const OpHook* hook,
                         int64_t n, int64_t nnz, const VT* dinv, const HxPrecond* pc, const VT* b, VT* x, double rtol,
                         int64_t max_iters, fq_report* rep) {
  cudaStream_t st = ctx->stream;
  DevBuf vecs, parts, state;
  const size_t vb = size_t(std::max<int64_t>(n, 1)) * sizeof(VT);
  FQ_TRY(vecs.alloc(ctx, vb * 4));
  FQ_TRY(parts.alloc(ctx, 3 * PBLOCKS * sizeof(double)));
  FQ_TRY(state.alloc(ctx, 2 * sizeof(SolverState) + sizeof(IterScalars)));
  CgVecs<VT> c;
  char* base = vecs.as<char>();
  c.x = x;
  c.r = reinterpret_cast<VT*>(base + 0 * vb);
  c.z = reinterpret_cast<VT*>(base + 1 * vb);
  c.p = reinterpret_cast<VT*>(base + 2 * vb);
  c.ap = reinterpret_cast<VT*>(base + 3 * vb);
  c.dinv = pc ? nullptr : dinv;
  c.external = pc ? 1 : 0;
  c.b = b;
  c.partA = parts.as<double>();
  c.partB = parts.as<double>() + PBLOCKS;
  c.partC = parts.as<double>() + 2 * PBLOCKS;
  c.p2 = nullptr;
  SolverState* S = state.as<SolverState>();
  IterScalars* X = reinterpret_cast<IterScalars*>(S + 2);  // per-iteration scalars, reduction counters at 0
  FQ_CUDA(ctx, cudaMemsetAsync(X, 0, sizeof(IterScalars), st));
  // FP64 CSR operators: the product runs on float-float pairs of the values and of p
  constexpr bool split_type = std::is_same<VT, double>::value;
  const bool split = split_type && !hook;
  DevBuf val2, p2;
  if constexpr (split_type) {
    if (split) {
      FQ_TRY(val2.alloc(ctx, size_t(std::max<int64_t>(nnz, 1)) * sizeof(df64)));
      FQ_TRY(p2.alloc(ctx, size_t(std::max<int64_t>(n, 1)) * sizeof(df64)));
      c.p2 = p2.as<df64>();
      if (nnz > 0) {
        split_kernel<<<int(std::min<int64_t>((nnz + KT - 1) / KT, KBLOCKS)), KT, 0, st>>>(val, val2.as<df64>(), nnz);
        ctx->launches++;
      }
    }
  }
  const int W = split ? pick_w_split(nnz, n) : pick_w<VT>(nnz, n);
  const int ga = std::min(spmv_blocks(n, W), PBLOCKS);
  const int gv = int(std::max<int64_t>(1, std::min<int64_t>((n + KT - 1) / KT, KBLOCKS)));
  cg_init<VT><<<gv, KT, 0, st>>>(c, n);
  if (pc) {
    hx_apply<VT>(*pc, b, c.z, nullptr, st);
    cg_init_p<VT><<<gv, KT, 0, st>>>(c, n);
  }
  cg_init_state<<<1, KT, 0, st>>>(S, S + 1, c.partB, c.partC, gv, rtol, (long long)max_iters);
  ctx->launches += 2;
  SolverState hs{};
  auto iteration = [&](int cur) {
    if (hook) {
      if constexpr (std::is_same<VT, double>::value) {
        const int* done = &(S + cur)->done;
        hook->apply(hook->self, c.p, c.ap, done, st);
        cg_pap<<<ga, KT, 0, st>>>(c, S + cur, X, n);
      }
    } else if (split) {
      if constexpr (split_type) {
        const df64* v2 = val2.as<df64>();
        switch (W) {
          case 4:
            cg_a_split<4><<<ga, KT, 0, st>>>(rp, ci, v2, c, S + cur, X, n);
            break;
          case 8:
            cg_a_split<8><<<ga, KT, 0, st>>>(rp, ci, v2, c, S + cur, X, n);
            break;
          case 16:
            cg_a_split<16><<<ga, KT, 0, st>>>(rp, ci, v2, c, S + cur, X, n);
            break;
          default:
            cg_a_split<32><<<ga, KT, 0, st>>>(rp, ci, v2, c, S + cur, X, n);
            break;
        }
      }
    } else switch (W) {
      case 4:
        cg_a<4, VT><<<ga, KT, 0, st>>>(rp, ci, val, c, S + cur, X, n);
        break;
      case 8:
        cg_a<8, VT><<<ga, KT, 0, st>>>(rp, ci, val, c, S + cur, X, n);
        break;
      case 16:
        cg_a<16, VT><<<ga, KT, 0, st>>>(rp, ci, val, c, S + cur, X, n);
        break;
      default:
        cg_a<32, VT><<<ga, KT, 0, st>>>(rp, ci, val, c, S + cur, X, n);
        break;
    }
    cg_b<VT><<<gv, KT, 0, st>>>(c, S + cur, X, S + (1 - cur), rtol, (long long)max_iters, n);
    if (pc) {
      const int* done = &(S + cur)->done;
      hx_apply<VT>(*pc, c.r, c.z, done, st);
      cg_dot<VT><<<gv, KT, 0, st>>>(c, S + cur, X, S + (1 - cur), gv, rtol, (long long)max_iters, n);
    }
    cg_c<VT><<<gv, KT, 0, st>>>(c, S + cur, S + (1 - cur), X, n);
  };
  FQ_TRY(run_graph_loop(ctx, S, max_iters, iteration, &hs, pc ? 4 : 64));
  rep->iters = hs.iters;
  rep->residual = hs.residual;
  rep->converged = hs.converged;
  if (hs.breakdown) return set_error(ctx, FQ_BREAKDOWN, "CG breakdown (NaN)");
  return FQ_OK;
}

template <typename VT>
fq_status cg_run(fq_ctx* ctx, const int32_t* rp, const int32_t* ci, const VT* val, int64_t n, int64_t nnz,
                 const VT* dinv, const HxPrecond* pc, const VT* b, VT* x, double rtol, int64_t max_iters,
                 fq_report* rep) {
  return cg_impl<VT>(ctx, rp, ci, val, nullptr, n, nnz, dinv, pc, b, x, rtol, max_iters, rep);
}

fq_status cg_run_op(fq_ctx* ctx, const OpHook& hook, int64_t n, const double* dinv, const double* b, double* x,
                    double rtol, int64_t max_iters, fq_report* rep) {
  return cg_impl<double>(ctx, nullptr, nullptr, nullptr, &hook, n, n, dinv, nullptr, b, x, rtol, max_iters, rep);
}

template fq_status minres_run<double>(fq_ctx*, const int32_t*, const int32_t*, const double*, int64_t, int64_t,
                                      const double*, const HxPrecond*, const double*, double*, double, int64_t,
                                      fq_report*);
template fq_status minres_run<float>(fq_ctx*, const int32_t*, const int32_t*, const float*, int64_t, int64_t,
                                     const float*, const HxPrecond*, const float*, float*, double, int64_t,
                                     fq_report*);
template fq_status cg_run<double>(fq_ctx*, const int32_t*, const int32_t*, const double*, int64_t, int64_t,
                                  const double*, const HxPrecond*, const double*, double*, double, int64_t,
                                  fq_report*);
template fq_status cg_run<float>(fq_ctx*, const int32_t*, const int32_t*, const float*, int64_t, int64_t,
                                 const float*, const HxPrecond*, const float*, float*, double, int64_t, fq_report*);

// ---------------------------------------------------------------------------
// Small vector kernels used by the problem drivers
// ---------------------------------------------------------------------------
// r = b - A x (FP64), partial ||r||^2 and ||b||^2
__global__ void __launch_bounds__(KT) residual64_kernel(const int32_t* rp, const int32_t* ci, const double* val,
                                                        const double* x, const double* b, double* r, double* part,
                                                        int64_t n) {
  __shared__ double sh[32];
  constexpr int W = 8;
  const int lane = threadIdx.x % W;
  double rr = 0.0, bb = 0.0;
  const int64_t rows_per_grid = int64_t(gridDim.x) * (blockDim.x / W);
  for (int64_t base = int64_t(blockIdx.x) * (blockDim.x / W); base < n; base += rows_per_grid) {
    const int64_t row = base + threadIdx.x / W;
    const bool valid = row < n;
    const double ax = row_dot<W, double>(rp, ci, val, x, row, valid, lane);
    if (valid && lane == 0) {
      const double ri = b[row] - ax;
      r[row] = ri;
      rr += ri * ri;
      bb += b[row] * b[row];
    }
  }
  rr = block_sum(rr, sh);
  bb = block_sum(bb, sh);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = rr;
    part[KBLOCKS + blockIdx.x] = bb;
  }
}

__global__ void to_float_scaled(const double* a, float* o, double s, int64_t n) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    o[i] = float(a[i] * s);
}
__global__ void axpy_from_float(double* x, const float* d, double s, int64_t n) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    x[i] += s * double(d[i]);
}
__global__ void to_float_kernel(const double* a, float* o, int64_t n) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    o[i] = float(a[i]);
}

static int vgrid(int64_t n) { return int(std::max<int64_t>(1, std::min<int64_t>((n + KT - 1) / KT, KBLOCKS))); }

// ||b - A x|| and ||b|| in FP64 (r receives the residual).
fq_status residual64(fq_ctx* ctx, const int32_t* rp, const int32_t* ci, const double* val, int64_t n,
                     const double* x, const double* b, double* r, double* rnorm, double* bnorm) {
  DevBuf part;
  FQ_TRY(part.alloc(ctx, 2 * KBLOCKS * sizeof(double)));
  FQ_CUDA(ctx, cudaMemsetAsync(part.p, 0, 2 * KBLOCKS * sizeof(double), ctx->stream));
  const int g = std::min(spmv_blocks(n, 8), KBLOCKS);
  residual64_kernel<<<g, KT, 0, ctx->stream>>>(rp, ci, val, x, b, r, part.as<double>(), n);
  ctx->launches++;
  std::vector<double> h(2 * KBLOCKS);
  FQ_CUDA(ctx, cudaMemcpyAsync(h.data(), part.p, 2 * KBLOCKS * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  double rr = 0, bb = 0;
  for (int i = 0; i < KBLOCKS; ++i) {
    rr += h[i];
    bb += h[KBLOCKS + i];
  }
  *rnorm = std::sqrt(rr);
  *bnorm = std::sqrt(bb);
  return FQ_OK;
}

void launch_to_float(const double* a, float* o, int64_t n, cudaStream_t st) {
  if (n > 0) to_float_kernel<<<vgrid(n), KT, 0, st>>>(a, o, n);
}
void launch_to_float_scaled(const double* a, float* o, double s, int64_t n, cudaStream_t st) {
  if (n > 0) to_float_scaled<<<vgrid(n), KT, 0, st>>>(a, o, s, n);
}
void launch_axpy_from_float(double* x, const float* d, double s, int64_t n, cudaStream_t st) {
  if (n > 0) axpy_from_float<<<vgrid(n), KT, 0, st>>>(x, d, s, n);
}

}  // namespace fq
