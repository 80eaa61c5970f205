// Numeric phase of the sparse direct solver (fq_sparse_lu.h): batched front
// assembly, partial LU in tiles with tournament pivoting, triangular solves,
// and the FP64 GMRES that the factors precondition. The factorization runs in
// FP32 (tiles of 128 columns) or FP64 (tiles of 64 columns).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "fq_df64.cuh"
#include "fq_sparse_lu.h"

namespace fq {

namespace {

// Arithmetic of the three factor types: FP32, IEEE FP64, and float-float
// (df64: a value as the unevaluated sum of two floats, 48-bit significand, all
// arithmetic on the FP32 pipe, which on this GPU runs many times faster than
// the FP64 one). mag() is a magnitude for pivot comparisons (the leading part
// of a float-float).
template <typename T>
struct Num;
template <>
struct Num<float> {
  static constexpr int kPrecision = FQ_FP32;
  static __device__ __forceinline__ float mag(float a) { return fabsf(a); }
  static __device__ __forceinline__ bool finite(float a) { return isfinite(a); }
  static __device__ __forceinline__ bool nonzero(float a) { return a != 0.f; }
  static __device__ __forceinline__ bool negative(float a) { return a < 0.f; }
  static __device__ __forceinline__ float fma(float a, float b, float c) { return fmaf(a, b, c); }
  static __device__ __forceinline__ float fma_acc(float a, float b, float c) { return fmaf(a, b, c); }
  static __device__ __forceinline__ float finish(float c) { return c; }
  static __device__ __forceinline__ float recip(float a) { return 1.f / a; }
  static __device__ __forceinline__ float div(float a, float b) { return a / b; }
  static __device__ __forceinline__ float mul(float a, float b) { return a * b; }
  static __device__ __forceinline__ float ldcg(const float* p) { return __ldcg(p); }
  static __host__ __device__ __forceinline__ float from_double(double d) { return float(d); }
  static __device__ __forceinline__ double to_double(float a) { return double(a); }
};
template <>
struct Num<double> {
  static constexpr int kPrecision = FQ_FP64_IEEE;
  static __device__ __forceinline__ double mag(double a) { return fabs(a); }
  static __device__ __forceinline__ bool finite(double a) { return isfinite(a); }
  static __device__ __forceinline__ bool nonzero(double a) { return a != 0.0; }
  static __device__ __forceinline__ bool negative(double a) { return a < 0.0; }
  static __device__ __forceinline__ double fma(double a, double b, double c) { return ::fma(a, b, c); }
  static __device__ __forceinline__ double fma_acc(double a, double b, double c) { return ::fma(a, b, c); }
  static __device__ __forceinline__ double finish(double c) { return c; }
  static __device__ __forceinline__ double recip(double a) { return 1.0 / a; }
  static __device__ __forceinline__ double div(double a, double b) { return a / b; }
  static __device__ __forceinline__ double mul(double a, double b) { return a * b; }
  static __device__ __forceinline__ double ldcg(const double* p) { return __ldcg(p); }
  static __host__ __device__ __forceinline__ double from_double(double d) { return d; }
  static __device__ __forceinline__ double to_double(double a) { return a; }
};
template <>
struct Num<df64> {
  static constexpr int kPrecision = FQ_FP64;
  static __device__ __forceinline__ float mag(df64 a) { return fabsf(a.hi); }
  static __device__ __forceinline__ bool finite(df64 a) { return isfinite(a.hi) && isfinite(a.lo); }
  static __device__ __forceinline__ bool nonzero(df64 a) { return a.hi != 0.f || a.lo != 0.f; }
  static __device__ __forceinline__ bool negative(df64 a) { return a.hi < 0.f; }
  // c + a b: the product's leading part and its error (exact by FMA, plus the
  // cross terms), TwoSum of the leading parts, the trailing parts in FP32,
  // one renormalisation (15 FP32 operations; error about 2^-46 of the terms)
  static __device__ __forceinline__ df64 fma(df64 a, df64 b, df64 c) {
    const float p = f_mul(a.hi, b.hi);
    float e = f_fma(a.hi, b.hi, -p);
    e = f_fma(a.hi, b.lo, e);
    e = f_fma(a.lo, b.hi, e);
    const df64 s = two_sum(c.hi, p);
    const float t = f_add(c.lo, f_add(e, s.lo));
    return fast_two_sum(s.hi, t);
  }
  // The same inside a product's K loop, without the renormalisation (12 FP32
  // operations): the leading part stays the exact TwoSum of the leading parts,
  // the trailing part collects the rest in FP32 and grows by at most an ulp of
  // the leading part per step; finish() renormalises once, after at most TILE
  // steps (about 2^-42 relative, against 2^-46 renormalising every step).
  static __device__ __forceinline__ df64 fma_acc(df64 a, df64 b, df64 c) {
    const float p = f_mul(a.hi, b.hi);
    float e = f_fma(a.hi, b.hi, -p);
    e = f_fma(a.hi, b.lo, e);
    e = f_fma(a.lo, b.hi, e);
    const df64 s = two_sum(c.hi, p);
    return df64(s.hi, f_add(c.lo, f_add(e, s.lo)));
  }
  static __device__ __forceinline__ df64 finish(df64 c) { return fast_two_sum(c.hi, c.lo); }
  // 1 / a: the FP32 reciprocal refined by one Newton step in float-float
  // (the division of Bailey's double-double arithmetic)
  static __device__ __forceinline__ df64 recip(df64 a) {
    const df64 q(__frcp_rn(a.hi), 0.f);
    const df64 e = df64(1.f, 0.f) - a * q;
    return q + q * e;
  }
  static __device__ __forceinline__ df64 div(df64 a, df64 b) { return a * recip(b); }
  static __device__ __forceinline__ df64 mul(df64 a, df64 b) { return a * b; }
  static __device__ __forceinline__ df64 ldcg(const df64* p) {
    const float2 v = __ldcg(reinterpret_cast<const float2*>(p));
    return df64(v.x, v.y);
  }
  static __host__ __device__ __forceinline__ df64 from_double(double d) { return df64(d); }
  static __device__ __forceinline__ double to_double(df64 a) { return a.to_double(); }
};

template <typename T>
struct SlCfg;
template <>
struct SlCfg<float> {
  static constexpr int TILE = 128;    // columns per tile step
  static constexpr int ROWS = 256;    // rows of a tournament leaf or merge
  static constexpr int BM = 128;      // product tile (BM x BM outputs per CTA)
  static constexpr int TM = 8;        // outputs per thread and dimension
  static constexpr int MINB = 2;      // resident product CTAs per SM the registers allow
};
template <>
struct SlCfg<double> {
  static constexpr int TILE = 64;
  static constexpr int ROWS = 128;
  static constexpr int BM = 64;
  static constexpr int TM = 4;
  static constexpr int MINB = 4;
};
template <>
struct SlCfg<df64> {
  static constexpr int TILE = 64;
  static constexpr int ROWS = 256;  // leaves twice the IEEE type's: one merge round fewer per tile step
  static constexpr int BM = 64;
  static constexpr int TM = 4;
  static constexpr int MINB = 4;
};
static_assert(SlCfg<float>::TILE <= kTile && SlCfg<double>::TILE <= kTile, "tile store sized for kTile");

constexpr int kBK = 32;  // K chunk of the products
constexpr int kThreads = 256;
constexpr int kMaxComposeRows = 46000;  // fully summed rows whose interchanges one CTA composes in shared memory

// A shared-memory array of n values of T, declared as raw storage (float-float
// has a constructor, which shared memory cannot run)
#define SL_SHARED_ARRAY(T, name, n)                                     \
  __shared__ __align__(16) unsigned char name##_raw[sizeof(T) * (n)]; \
  T* name = reinterpret_cast<T*>(name##_raw)

// ---------------------------------------------------------------------------
// assembly
// ---------------------------------------------------------------------------
template <typename T>
__global__ void sl_assemble_kernel(const int32_t* __restrict__ slot, const int32_t* __restrict__ row,
                                   const int64_t* __restrict__ off, int64_t b, int64_t e,
                                   const int32_t* __restrict__ ci, const double* __restrict__ val,
                                   const double* __restrict__ d, T* __restrict__ pool) {
  for (int64_t q = b + int64_t(blockIdx.x) * blockDim.x + threadIdx.x; q < e; q += int64_t(gridDim.x) * blockDim.x) {
    const int32_t s = slot[q];
    pool[off[q]] = Num<T>::from_double(d[row[q]] * val[s] * d[ci[s]]);
  }
}

// d_i = 1 / sqrt(max_j |a_ij|) (1 for an empty or zero row)
__global__ void sl_row_scale_kernel(const int32_t* __restrict__ rp, const double* __restrict__ val, int64_t n,
                                    double* __restrict__ d) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    double mx = 0.0;
    for (int32_t t = rp[i]; t < rp[i + 1]; ++t) mx = fmax(mx, fabs(val[t]));
    d[i] = mx > 0.0 && isfinite(mx) ? 1.0 / sqrt(mx) : 1.0;
  }
}

// The Schur complement of child `which` (0 or 1) of every front of the list
// added into the front at its parent-local rows and columns.
template <typename T>
__global__ void sl_extend_add_kernel(const FrontDesc* __restrict__ fd, const int32_t* __restrict__ list, int which,
                                     const int32_t* __restrict__ ea, T* __restrict__ pool) {
  const FrontDesc X = fd[list[blockIdx.y]];
  const int c = which == 0 ? X.child0 : X.child1;
  if (c < 0) return;
  const FrontDesc C = fd[c];
  const int64_t u = C.m - C.f;
  const int64_t total = u * u;
  const int32_t* map = ea + C.ea_off;
  for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < total; t += int64_t(gridDim.x) * blockDim.x) {
    const int64_t bcol = t / u, arow = t - bcol * u;
    const T v = pool[C.off + (C.f + bcol) * C.m + (C.f + arow)];
    pool[X.off + int64_t(map[bcol]) * X.m + map[arow]] += v;
  }
}

// ---------------------------------------------------------------------------
// pivot selection over the whole fully summed panel (tournament pivoting):
// the panel of a step is the front's fully summed rows k..f-1 in the step's
// columns k..k+b-1. Leaves of ROWS rows each pick b candidate rows by Gaussian
// elimination with partial pivoting (GEPP); pairs of candidate sets are merged
// by GEPP on their original rows, up a binary tree, until b winners remain, in
// GEPP's pivot order. Moving them to the top rows and factoring the tile
// without further interchanges reproduces the final GEPP (communication-
// avoiding LU, Grigori, Demmel and Xiang, SIAM J. Matrix Anal. Appl. 32,
// 2011): a pivoting as wide as partial pivoting restricted to the front's
// fully summed rows.
// ---------------------------------------------------------------------------
// GEPP on the rows x b block held column-major in blk (column stride ld);
// idx[i] names row i. On return idx[0..min(rows, b)) are the pivot rows in
// pivot order.
template <typename T>
__device__ void gepp_select(T* blk, int ld, int* idx, int rows, int b) {
  __shared__ int s_p;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int steps = min(rows, b);
  for (int j = 0; j < steps; ++j) {
    if (tid < 32) {
      using M = decltype(Num<T>::mag(T()));
      M best = M(-1);
      int bi = j;
      for (int i = j + tid; i < rows; i += 32) {
        const M a = Num<T>::mag(blk[j * ld + i]);
        if (a > best || (a == best && i < bi)) {
          best = a;
          bi = i;
        }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const M ob = __shfl_down_sync(0xffffffffu, best, o);
        const int oi = __shfl_down_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) {
          best = ob;
          bi = oi;
        }
      }
      if (tid == 0) s_p = bi;
    }
    __syncthreads();
    const int p = s_p;
    if (p != j) {
      for (int l = tid; l < b; l += nt) {
        const T t = blk[l * ld + j];
        blk[l * ld + j] = blk[l * ld + p];
        blk[l * ld + p] = t;
      }
      if (tid == 0) {
        const int t = idx[j];
        idx[j] = idx[p];
        idx[p] = t;
      }
    }
    __syncthreads();
    const T d = blk[j * ld + j];
    if (Num<T>::nonzero(d) && Num<T>::finite(d)) {
      const T rinv = Num<T>::recip(d);
      for (int i = j + 1 + tid; i < rows; i += nt) blk[j * ld + i] = Num<T>::mul(blk[j * ld + i], rinv);
      __syncthreads();
      const int w = rows - j - 1, c = b - j - 1;
      for (int t = tid; t < w * c; t += nt) {
        const int l = j + 1 + t / w, i = j + 1 + t % w;
        blk[l * ld + i] = Num<T>::fma(-blk[j * ld + i], blk[l * ld + j], blk[l * ld + i]);
      }
    }
    __syncthreads();
  }
}

// Leaves: block q of every front's panel; candidate set q = its b GEPP winners.
template <typename T>
__global__ void __launch_bounds__(kThreads) sl_tourn_leaf_kernel(const FrontDesc* __restrict__ fd,
                                                                 const int32_t* __restrict__ list, int k,
                                                                 const T* __restrict__ pool, int maxsets,
                                                                 int32_t* __restrict__ cand,
                                                                 int32_t* __restrict__ ccount) {
  using C = SlCfg<T>;
  extern __shared__ __align__(16) unsigned char smraw[];
  T* blk = reinterpret_cast<T*>(smraw);
  __shared__ int idx[C::ROWS];
  const FrontDesc F = fd[list[blockIdx.y]];
  if (F.f <= k) return;
  const int b = min(C::TILE, F.f - k);
  const int q = blockIdx.x;
  const int r0 = k + q * C::ROWS;
  if (r0 >= F.f) return;
  const int rows = min(C::ROWS, F.f - r0);
  const int64_t m = F.m;
  const T* A = pool + F.off;
  for (int t = threadIdx.x; t < rows * b; t += blockDim.x) {
    const int col = t / rows, row = t - col * rows;
    blk[col * (C::ROWS + 1) + row] = A[(k + col) * m + (r0 + row)];
  }
  for (int i = threadIdx.x; i < rows; i += blockDim.x) idx[i] = r0 + i;
  __syncthreads();
  gepp_select<T>(blk, C::ROWS + 1, idx, rows, b);
  const int64_t set = int64_t(blockIdx.y) * maxsets + q;
  const int nw = min(rows, b);
  for (int i = threadIdx.x; i < nw; i += blockDim.x) cand[set * kTile + i] = idx[i];
  if (threadIdx.x == 0) ccount[set] = nw;
}

// One tournament round: set q of the output = GEPP winners of sets 2q and
// 2q+1 of the input, or set 2q copied when 2q+1 is empty. Sets beyond a
// front's own count are empty (count 0).
template <typename T>
__global__ void __launch_bounds__(kThreads) sl_tourn_merge_kernel(const FrontDesc* __restrict__ fd,
                                                                  const int32_t* __restrict__ list, int k,
                                                                  const T* __restrict__ pool, int maxsets,
                                                                  int nsets_in, const int32_t* __restrict__ cin,
                                                                  const int32_t* __restrict__ nin,
                                                                  int32_t* __restrict__ cout,
                                                                  int32_t* __restrict__ nout) {
  using C = SlCfg<T>;
  extern __shared__ __align__(16) unsigned char smraw[];
  T* blk = reinterpret_cast<T*>(smraw);
  __shared__ int idx[C::ROWS];
  const FrontDesc F = fd[list[blockIdx.y]];
  const int q = blockIdx.x;
  const int64_t base = int64_t(blockIdx.y) * maxsets;
  if (F.f <= k) {
    if (threadIdx.x == 0) nout[base + q] = 0;
    return;
  }
  const int b = min(C::TILE, F.f - k);
  const int64_t a0 = base + 2 * q, a1 = base + 2 * q + 1;
  const int na = 2 * q < nsets_in ? nin[a0] : 0;
  const int nb = 2 * q + 1 < nsets_in ? nin[a1] : 0;
  if (nb == 0) {
    for (int i = threadIdx.x; i < na; i += blockDim.x) cout[(base + q) * kTile + i] = cin[a0 * kTile + i];
    if (threadIdx.x == 0) nout[base + q] = na;
    return;
  }
  const int rows = na + nb;
  for (int i = threadIdx.x; i < rows; i += blockDim.x) idx[i] = i < na ? cin[a0 * kTile + i] : cin[a1 * kTile + i - na];
  __syncthreads();
  const int64_t m = F.m;
  const T* A = pool + F.off;
  for (int t = threadIdx.x; t < rows * b; t += blockDim.x) {
    const int col = t / rows, row = t - col * rows;
    blk[col * (C::ROWS + 1) + row] = A[(k + col) * m + idx[row]];
  }
  __syncthreads();
  gepp_select<T>(blk, C::ROWS + 1, idx, rows, b);
  const int nw = min(rows, b);
  for (int i = threadIdx.x; i < nw; i += blockDim.x) cout[(base + q) * kTile + i] = idx[i];
  if (threadIdx.x == 0) nout[base + q] = nw;
}

// The winners (set 0) as a sequence of row interchanges: for j = 0..b-1, row
// k+j is swapped with row piv[start + k + j] (front-local), applied in order,
// which leaves winner j at row k+j. Positions k+j not yet filled hold rows of
// the top block k..k+b-1 (an interchange only ever moves a top row down), so
// tracking where those rows are suffices.
__global__ void sl_swap_sequence_kernel(const FrontDesc* __restrict__ fd, const int32_t* __restrict__ list, int k,
                                        int tile, int maxsets, const int32_t* __restrict__ cand,
                                        int32_t* __restrict__ piv) {
  __shared__ int at_top[kTile];  // original top row now at position k+i (i not yet filled)
  __shared__ int where[kTile];   // position of original top row k+i
  const FrontDesc F = fd[list[blockIdx.x]];
  if (F.f <= k || threadIdx.x != 0) return;
  const int b = min(tile, F.f - k);
  const int32_t* w = cand + int64_t(blockIdx.x) * maxsets * kTile;
  for (int i = 0; i < b; ++i) {
    at_top[i] = k + i;
    where[i] = k + i;
  }
  for (int j = 0; j < b; ++j) {
    const int r = w[j];
    const bool top = r >= k && r < k + b;
    const int t = top ? where[r - k] : r;
    piv[F.start + k + j] = t;
    if (t != k + j) {
      const int x = at_top[j];  // the top row at k+j moves to t
      where[x - k] = t;
      if (t < k + b) at_top[t - k] = x;
    }
    if (top) where[r - k] = k + j;
    at_top[j] = r;
  }
}

// The step's interchanges on every column of the front (fully summed rows only).
template <typename T>
__global__ void sl_apply_swaps_kernel(const FrontDesc* __restrict__ fd, const int32_t* __restrict__ list, int k,
                                      int tile, const int32_t* __restrict__ piv, T* __restrict__ pool) {
  const FrontDesc F = fd[list[blockIdx.y]];
  if (F.f <= k) return;
  const int b = min(tile, F.f - k);
  const int64_t m = F.m;
  T* A = pool + F.off;
  for (int64_t c = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; c < m; c += int64_t(gridDim.x) * blockDim.x) {
    T* col = A + c * m;
    for (int j = 0; j < b; ++j) {
      const int t = piv[F.start + k + j];
      if (t != k + j) {
        const T v = col[k + j];
        col[k + j] = col[t];
        col[t] = v;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// the tile of the partial factorization (its rows already in pivot order): LU
// without interchanges, a pivot below the floor perturbed, and the tile's
// triangular inverses
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(kThreads) sl_tile_kernel(const FrontDesc* __restrict__ fd,
                                                           const int32_t* __restrict__ list, int k,
                                                           T* __restrict__ pool, T* __restrict__ tiles,
                                                           int* __restrict__ status, T thresh) {
  using C = SlCfg<T>;
  constexpr int TL = C::TILE, LD = C::TILE + 1;
  extern __shared__ __align__(16) unsigned char smraw[];
  T* Tt = reinterpret_cast<T*>(smraw);  // [TL][LD], column-major Tt[col * LD + row]
  T* Xs = Tt + TL * LD;                 // inverse under construction
  SL_SHARED_ARRAY(T, s_val, 1);
  const FrontDesc F = fd[list[blockIdx.x]];
  if (F.f <= k) return;
  const int b = min(TL, F.f - k);
  const int64_t m = F.m;
  T* A = pool + F.off;
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int t = tid; t < b * b; t += nt) {
    const int col = t / b, row = t - col * b;
    Tt[col * LD + row] = A[(k + col) * m + (k + row)];
  }
  __syncthreads();
  int npert = 0, nbad = 0;
  for (int j = 0; j < b; ++j) {
    if (tid == 0) {
      T d = Tt[j * LD + j];
      if (!Num<T>::finite(d)) {
        if (nbad == 0 && atomicCAS(status + 2, 0, list[blockIdx.x] + 1) == 0) status[3] = k + j;
        ++nbad;
        d = thresh;
      } else if (Num<T>::mag(d) < Num<T>::mag(thresh)) {
        ++npert;
        d = Num<T>::negative(d) ? -thresh : thresh;
      }
      Tt[j * LD + j] = d;
      s_val[0] = Num<T>::recip(d);
    }
    __syncthreads();
    const T rinv = s_val[0];
    for (int i = j + 1 + tid; i < b; i += nt) Tt[j * LD + i] = Num<T>::mul(Tt[j * LD + i], rinv);
    __syncthreads();
    const int w = b - j - 1;
    for (int t = tid; t < w * w; t += nt) {
      const int l = j + 1 + t / w, i = j + 1 + t % w;
      Tt[l * LD + i] = Num<T>::fma(-Tt[j * LD + i], Tt[l * LD + j], Tt[l * LD + i]);
    }
    __syncthreads();
  }
  if (tid == 0 && (npert || nbad)) {
    atomicAdd(status, npert);
    atomicAdd(status + 1, nbad);
  }
  for (int t = tid; t < b * b; t += nt) {
    const int col = t / b, row = t - col * b;
    A[(k + col) * m + (k + row)] = Tt[col * LD + row];
  }
  // inverses: unit lower L^-1, then U^-1; one thread per column
  T* out = tiles + F.tile_off + int64_t(k / TL) * 2 * TL * TL;
  if (tid < b) {
    const int j = tid;
    for (int i = 0; i < b; ++i) Xs[j * LD + i] = T(0);
    Xs[j * LD + j] = T(1);
    for (int i = j + 1; i < b; ++i) {
      T s = T(0);
      for (int l = j; l < i; ++l) s = Num<T>::fma(Tt[l * LD + i], Xs[j * LD + l], s);
      Xs[j * LD + i] = -s;
    }
  }
  __syncthreads();
  for (int t = tid; t < TL * TL; t += nt) {
    const int col = t / TL, row = t - col * TL;
    out[t] = (col < b && row < b) ? Xs[col * LD + row] : T(0);
  }
  __syncthreads();
  if (tid < b) {
    const int j = tid;
    for (int i = 0; i < b; ++i) Xs[j * LD + i] = T(0);
    Xs[j * LD + j] = Num<T>::recip(Tt[j * LD + j]);
    for (int i = j - 1; i >= 0; --i) {
      T s = T(0);
      for (int l = i + 1; l <= j; ++l) s = Num<T>::fma(Tt[l * LD + i], Xs[j * LD + l], s);
      Xs[j * LD + i] = Num<T>::div(-s, Tt[i * LD + i]);
    }
  }
  __syncthreads();
  for (int t = tid; t < TL * TL; t += nt) {
    const int col = t / TL, row = t - col * TL;
    out[TL * TL + t] = (col < b && row < b) ? Xs[col * LD + row] : T(0);
  }
}

// ---------------------------------------------------------------------------
// the three products of a tile step, one kernel: a BM x BM output tile per CTA,
// K <= TILE in chunks of kBK, TM x TM outputs per thread.
//   mode 0 (L panel):  A[k+b+r, k+c]   = sum_q A[k+b+r, k+q] invU[q, c]        (rows below the tile)
//   mode 1 (U panel):  A[k+r, k+b+c]   = sum_q invL[r, q] A[k+q, k+b+c]        (columns right of it)
//   mode 2 (trailing): A[k+b+r, k+b+c] -= sum_q A[k+b+r, k+q] A[k+q, k+b+c]
// In modes 0 and 1 the output overwrites an operand; each CTA owns whole rows
// (mode 0) or whole columns (mode 1) of it and writes after its last read.
// ---------------------------------------------------------------------------
template <typename T>
struct Vec16;  // TM/2 consecutive values in one 16-byte load
template <>
struct Vec16<float> {
  static __device__ __forceinline__ void load(const float* p, float* o) {
    const float4 v = *reinterpret_cast<const float4*>(p);
    o[0] = v.x;
    o[1] = v.y;
    o[2] = v.z;
    o[3] = v.w;
  }
};
template <>
struct Vec16<double> {
  static __device__ __forceinline__ void load(const double* p, double* o) {
    const double2 v = *reinterpret_cast<const double2*>(p);
    o[0] = v.x;
    o[1] = v.y;
  }
};
template <>
struct Vec16<df64> {
  static __device__ __forceinline__ void load(const df64* p, df64* o) {
    const float4 v = *reinterpret_cast<const float4*>(p);
    o[0] = df64(v.x, v.y);
    o[1] = df64(v.z, v.w);
  }
};

// The operands of a tile step's product for one BM x BM output tile (mode as
// above); false when the CTA has no tile.
template <typename T>
struct GemmTile {
  const T* Xp;
  int64_t ldx;
  const T* Yp;
  int64_t ldy;
  T* Cp;
  int64_t m, rlim, clim;
  int b;
};

template <typename T>
__device__ __forceinline__ bool gemm_tile(const FrontDesc& F, int k, int mode, T* pool, const T* tiles,
                                          GemmTile<T>& g) {
  using C = SlCfg<T>;
  constexpr int BM = C::BM, TL = C::TILE;
  if (F.f <= k) return false;
  const int b = min(TL, F.f - k);
  const int64_t m = F.m;
  const int64_t rest = m - k - b;
  int64_t rows, cols;
  if (mode == 0) {
    rows = rest;
    cols = b;
  } else if (mode == 1) {
    rows = b;
    cols = rest;
  } else {
    rows = rest;
    cols = rest;
  }
  if (rows <= 0 || cols <= 0) return false;
  const int64_t tr = (rows + BM - 1) / BM, tc = (cols + BM - 1) / BM;
  const int64_t tile = blockIdx.x;
  if (tile >= tr * tc) return false;
  const int64_t r0 = (tile % tr) * BM, c0 = (tile / tr) * BM;
  T* P = pool + F.off;
  const T* inv = tiles + F.tile_off + int64_t(k / TL) * 2 * TL * TL;
  if (mode == 0) {
    g.Xp = P + int64_t(k) * m + (k + b + r0);
    g.ldx = m;
    g.Yp = inv + TL * TL + c0 * TL;  // invU, ld TL
    g.ldy = TL;
    g.Cp = P + int64_t(k + c0) * m + (k + b + r0);
  } else if (mode == 1) {
    g.Xp = inv + r0;  // invL, ld TL
    g.ldx = TL;
    g.Yp = P + (k + b + c0) * m + k;
    g.ldy = m;
    g.Cp = P + (k + b + c0) * m + (k + r0);
  } else {
    g.Xp = P + int64_t(k) * m + (k + b + r0);
    g.ldx = m;
    g.Yp = P + (k + b + c0) * m + k;
    g.ldy = m;
    g.Cp = P + (k + b + c0) * m + (k + b + r0);
  }
  g.m = m;
  g.rlim = rows - r0;
  g.clim = cols - c0;
  g.b = b;
  return true;
}

// TM x TM outputs of a thread written back (mode 2: subtracted)
template <typename T, int BM, int TM>
__device__ __forceinline__ void gemm_store(const GemmTile<T>& g, int mode, int tx, int ty, const T (&acc)[TM][TM]) {
  constexpr int H = TM / 2;
#pragma unroll
  for (int j = 0; j < TM; ++j) {
    const int c = (j < H ? tx * H + j : BM / 2 + tx * H + (j - H));
    if (c >= g.clim) continue;
#pragma unroll
    for (int i = 0; i < TM; ++i) {
      const int r = (i < H ? ty * H + i : BM / 2 + ty * H + (i - H));
      if (r >= g.rlim) continue;
      T* dst = g.Cp + int64_t(c) * g.m + r;
      if (mode == 2)
        *dst -= acc[i][j];
      else
        *dst = acc[i][j];
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(kThreads, SlCfg<T>::MINB) sl_gemm_kernel(const FrontDesc* __restrict__ fd,
                                                           const int32_t* __restrict__ list, int k, int mode,
                                                           T* __restrict__ pool, const T* __restrict__ tiles) {
  using C = SlCfg<T>;
  constexpr int BM = C::BM, TM = C::TM, H = TM / 2;
  constexpr int BP = BM + 16 / int(sizeof(T));  // padded row of the B chunk, 16-byte aligned
  SL_SHARED_ARRAY(T, As, kBK * BM);  // [q][row]
  SL_SHARED_ARRAY(T, Bs, kBK * BP);  // [q][col], padded rows
  GemmTile<T> g;
  if (!gemm_tile<T>(fd[list[blockIdx.y]], k, mode, pool, tiles, g)) return;
  const int b = g.b;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  T acc[TM][TM];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TM; ++j) acc[i][j] = T(0);
  for (int q0 = 0; q0 < b; q0 += kBK) {
    for (int t = tid; t < BM * kBK; t += kThreads) {
      const int q = t / BM, r = t - q * BM;
      As[q * BM + r] = (r < g.rlim && q0 + q < b) ? g.Xp[int64_t(q0 + q) * g.ldx + r] : T(0);
    }
    for (int t = tid; t < BM * kBK; t += kThreads) {
      const int c = t / kBK, q = t - c * kBK;
      Bs[q * BP + c] = (c < g.clim && q0 + q < b) ? g.Yp[int64_t(c) * g.ldy + q0 + q] : T(0);
    }
    __syncthreads();
#pragma unroll 8
    for (int q = 0; q < kBK; ++q) {
      T av[TM], bv[TM];
      Vec16<T>::load(As + q * BM + ty * H, av);
      Vec16<T>::load(As + q * BM + BM / 2 + ty * H, av + H);
      Vec16<T>::load(Bs + q * BP + tx * H, bv);
      Vec16<T>::load(Bs + q * BP + BM / 2 + tx * H, bv + H);
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TM; ++j) acc[i][j] = Num<T>::fma_acc(av[i], bv[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TM; ++j) acc[i][j] = Num<T>::finish(acc[i][j]);
  gemm_store<T, BM, TM>(g, mode, tx, ty, acc);
}

// ---------------------------------------------------------------------------
// solve: one CTA per row block (the rows of one tile) of every front of a
// level. Tile solutions are published through per-tile flags: the producer
// writes its rows, fences, and stores the phase's target value; a consumer
// acquires the flag before it reads them (L2, not L1). CTAs take their row
// blocks by ticket, in list order, and a block waits only for blocks earlier
// in the list, which already hold a CTA: every wait ends. A wait is bounded
// all the same; one that runs out sets the solve status and goes on.
// ---------------------------------------------------------------------------
constexpr int kSolveThreads = 128;  // four warps; a lane holds TILE / 32 rows of the block
constexpr int kWaitPolls = 1 << 20;  // about a second of polling

__device__ __forceinline__ int load_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void store_release(int* p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// thread 0 waits for the flag, then the block goes on
// (once any wait has run out, the others give up at once: the solve is void)
__device__ void wait_tile(const int* flag, int target, int* status) {
  if (threadIdx.x == 0) {
    bool ok = false;
    for (int it = 0; it < kWaitPolls && !ok; ++it) {
      ok = load_acquire(flag) == target;
      if (!ok) {
        if (load_acquire(status) != 0) break;
        __nanosleep(64);
      }
    }
    if (!ok) atomicOr(status, 1);
  }
  __syncthreads();
}

// The composed row interchanges of every front: the swaps p <-> piv[p], in
// order of p, applied to the identity; fperm[start + i] names the front-local
// row whose value ends at position i.
__global__ void sl_compose_pivots_kernel(const FrontDesc* __restrict__ fd, const int32_t* __restrict__ piv,
                                         int32_t* __restrict__ fperm) {
  extern __shared__ int a[];
  __shared__ int pv[1024];
  const FrontDesc F = fd[blockIdx.x];
  const int f = F.f, tid = threadIdx.x, nt = blockDim.x;
  for (int i = tid; i < f; i += nt) a[i] = i;
  __syncthreads();
  for (int p0 = 0; p0 < f; p0 += 1024) {
    const int np = min(1024, f - p0);
    for (int t = tid; t < np; t += nt) pv[t] = piv[F.start + p0 + t];
    __syncthreads();
    if (tid == 0)
      for (int q = 0; q < np; ++q) {
        const int p = p0 + q, t = pv[q];
        if (t != p && t >= 0 && t < f) {
          const int v = a[p];
          a[p] = a[t];
          a[t] = v;
        }
      }
    __syncthreads();
  }
  for (int i = tid; i < f; i += nt) fperm[F.start + i] = a[i];
}

// Forward: row block w.y of front w.x. A block of the fully summed rows
// (w.y < its tile count) takes rows of tile w.y and publishes that tile's y;
// a later block takes update rows and writes the front's update vector.
template <typename T>
__global__ void __launch_bounds__(kSolveThreads) sl_forward_rows_kernel(
    const int2* __restrict__ items, int nitems, int* __restrict__ ticket, const FrontDesc* __restrict__ fd,
    const T* __restrict__ pool, const T* __restrict__ tiles, const int32_t* __restrict__ fperm,
    const int32_t* __restrict__ rinv, const T* __restrict__ work, T* ybuf, T* uvec, int* flags, int target,
    int* status) {
  using C = SlCfg<T>;
  constexpr int TL = C::TILE;
  constexpr int R = TL / 32;
  constexpr int NW = kSolveThreads / 32;
  __shared__ int s_item;
  SL_SHARED_ARRAY(T, sy, TL);
  SL_SHARED_ARRAY(T, part, NW * TL);  // [warp][row]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) s_item = atomicAdd(ticket, 1);
  __syncthreads();
  const int it = s_item;
  if (it >= nitems) return;
  const int2 w = items[it];
  const FrontDesc F = fd[w.x];
  const int m = F.m, f = F.f, nF = (f + TL - 1) / TL;
  const bool diag = w.y < nF;
  const int r0 = diag ? w.y * TL : f + (w.y - nF) * TL;
  const int nr = diag ? min(TL, f - r0) : min(TL, m - r0);
  const int jmax = diag ? w.y : nF;
  const int64_t ftile = F.tile_off / (2 * TL * TL);
  const T* P = pool + F.off;
  T acc[R];
#pragma unroll
  for (int q = 0; q < R; ++q) acc[q] = T(0);
  for (int j = 0; j < jmax; ++j) {
    wait_tile(flags + ftile + j, target, status);
    const int k = j * TL, b = min(TL, f - k);
    if (tid < b) sy[tid] = Num<T>::ldcg(ybuf + F.start + k + tid);
    __syncthreads();
#pragma unroll 4
    for (int l = warp; l < b; l += NW) {
      const T yl = sy[l];
      const T* col = P + int64_t(k + l) * m + r0;
#pragma unroll
      for (int q = 0; q < R; ++q) {
        const int i = lane + 32 * q;
        if (i < nr) acc[q] = Num<T>::fma(col[i], yl, acc[q]);
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < R; ++q) part[warp * TL + lane + 32 * q] = acc[q];
  __syncthreads();
  // the assembled, interchanged right-hand side of the block's rows, less the panel sums
  if (tid < nr) {
    const int row = r0 + tid;
    const int src = row < f ? fperm[F.start + row] : row;
    T v = src < f ? work[F.start + src] : T(0);
    if (F.child0 >= 0) {
      const int32_t q = rinv[2 * (F.roff + src)];
      if (q >= 0) v += uvec[fd[F.child0].uvec_off + q];
    }
    if (F.child1 >= 0) {
      const int32_t q = rinv[2 * (F.roff + src) + 1];
      if (q >= 0) v += uvec[fd[F.child1].uvec_off + q];
    }
    T sum = T(0);
#pragma unroll
    for (int ww = 0; ww < NW; ++ww) sum += part[ww * TL + tid];
    v -= sum;
    if (diag)
      sy[tid] = v;
    else
      uvec[F.uvec_off + (row - f)] = v;
  }
  if (!diag) return;
  __syncthreads();
  // y = L_tt^-1 v, L_tt^-1 from the tile store (column-major, stride TL)
  const T* iL = tiles + F.tile_off + int64_t(w.y) * 2 * TL * TL;
  if (tid < nr) {
    T y = T(0);
    for (int l = 0; l <= tid; ++l) y = Num<T>::fma(iL[l * TL + tid], sy[l], y);
    ybuf[F.start + r0 + tid] = y;
    __threadfence();
  }
  __syncthreads();
  if (tid == 0) store_release(flags + ftile + w.y, target);
}

// Backward: tile w.y of front w.x (the list takes a front's tiles last to
// first). x_t = U_tt^-1 (y_t - U_t,later x_later - U_t,update x_update); the
// update unknowns' x come from the ancestors, solved in earlier launches.
template <typename T>
__global__ void __launch_bounds__(kSolveThreads) sl_backward_rows_kernel(
    const int2* __restrict__ items, int nitems, int* __restrict__ ticket, const FrontDesc* __restrict__ fd,
    const T* __restrict__ pool, const T* __restrict__ tiles, const int32_t* __restrict__ urows,
    const T* __restrict__ ybuf, T* work, int* flags, int target, int* status) {
  using C = SlCfg<T>;
  constexpr int TL = C::TILE;
  constexpr int R = TL / 32;
  constexpr int NW = kSolveThreads / 32;
  __shared__ int s_item;
  SL_SHARED_ARRAY(T, sx, TL);
  SL_SHARED_ARRAY(T, part, NW * TL);  // [warp][row]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) s_item = atomicAdd(ticket, 1);
  __syncthreads();
  const int it = s_item;
  if (it >= nitems) return;
  const int2 w = items[it];
  const FrontDesc F = fd[w.x];
  const int m = F.m, f = F.f, nF = (f + TL - 1) / TL;
  const int t = w.y, r0 = t * TL, nr = min(TL, f - r0);
  const int64_t ftile = F.tile_off / (2 * TL * TL);
  const T* P = pool + F.off;
  T acc[R];
#pragma unroll
  for (int q = 0; q < R; ++q) acc[q] = T(0);
  // the update columns, known before the level starts
  for (int c0 = f; c0 < m; c0 += TL) {
    const int b = min(TL, m - c0);
    if (tid < b) sx[tid] = work[urows[F.ea_off + (c0 - f) + tid]];
    __syncthreads();
#pragma unroll 4
    for (int l = warp; l < b; l += NW) {
      const T xl = sx[l];
      const T* col = P + int64_t(c0 + l) * m + r0;
#pragma unroll
      for (int q = 0; q < R; ++q) {
        const int i = lane + 32 * q;
        if (i < nr) acc[q] = Num<T>::fma(col[i], xl, acc[q]);
      }
    }
    __syncthreads();
  }
  // the later tiles of the front, as they are published
  for (int j = nF - 1; j > t; --j) {
    wait_tile(flags + ftile + j, target, status);
    const int k = j * TL, b = min(TL, f - k);
    if (tid < b) sx[tid] = Num<T>::ldcg(work + F.start + k + tid);
    __syncthreads();
#pragma unroll 4
    for (int l = warp; l < b; l += NW) {
      const T xl = sx[l];
      const T* col = P + int64_t(k + l) * m + r0;
#pragma unroll
      for (int q = 0; q < R; ++q) {
        const int i = lane + 32 * q;
        if (i < nr) acc[q] = Num<T>::fma(col[i], xl, acc[q]);
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < R; ++q) part[warp * TL + lane + 32 * q] = acc[q];
  __syncthreads();
  if (tid < nr) {
    T z = ybuf[F.start + r0 + tid];
#pragma unroll
    for (int ww = 0; ww < NW; ++ww) z -= part[ww * TL + tid];
    sx[tid] = z;
  }
  __syncthreads();
  const T* iU = tiles + F.tile_off + int64_t(t) * 2 * TL * TL + TL * TL;
  if (tid < nr) {
    T x = T(0);
    for (int l = tid; l < nr; ++l) x = Num<T>::fma(iU[l * TL + tid], sx[l], x);
    work[F.start + r0 + tid] = x;
    __threadfence();
  }
  __syncthreads();
  if (tid == 0) store_release(flags + ftile + t, target);
}

// (D A D)^-1 = D^-1 A^-1 D^-1, so A^-1 r = D (D A D)^-1 D r
template <typename T>
__global__ void sl_permute_in_kernel(const double* __restrict__ r, const int32_t* __restrict__ perm,
                                     const double* __restrict__ d, int64_t n, T* __restrict__ w) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    w[perm[i]] = Num<T>::from_double(d[i] * r[i]);
}

template <typename T>
__global__ void sl_permute_out_kernel(const T* __restrict__ w, const int32_t* __restrict__ perm,
                                      const double* __restrict__ d, int64_t n, double* __restrict__ z) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    z[i] = d[i] * Num<T>::to_double(w[perm[i]]);
}

// ---------------------------------------------------------------------------
// FP64 vector kernels of the GMRES
// ---------------------------------------------------------------------------
__global__ void sl_spmv_kernel(const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                               const double* __restrict__ val, const double* __restrict__ x, int64_t n,
                               double* __restrict__ y) {
  // four lanes per row
  const int64_t g = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t row = g >> 2;
  const int lane = int(g & 3);
  double s = 0.0;
  if (row < n)
    for (int32_t t = rp[row] + lane; t < rp[row + 1]; t += 4) s += val[t] * x[ci[t]];
  s += __shfl_down_sync(0xffffffffu, s, 2, 4);
  s += __shfl_down_sync(0xffffffffu, s, 1, 4);
  if (row < n && lane == 0) y[row] = s;
}

// partial[j * nblocks + block] = sum over the block's range of V[j] . w, j < nv
__global__ void sl_multidot_kernel(const double* __restrict__ V, int64_t ldv, int nv, const double* __restrict__ w,
                                   int64_t n, double* __restrict__ partial) {
  __shared__ double red[8][33];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int j0 = 0; j0 < nv; j0 += 32) {
    const int jn = min(32, nv - j0);
    double s[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) s[j] = 0.0;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + tid; i < n; i += int64_t(gridDim.x) * blockDim.x) {
      const double wi = w[i];
#pragma unroll
      for (int j = 0; j < 32; ++j)
        if (j < jn) s[j] += V[int64_t(j0 + j) * ldv + i] * wi;
    }
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      double v = s[j];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if (lane == 0) red[warp][j] = v;
    }
    __syncthreads();
    if (tid < jn) {
      double v = 0.0;
      for (int w2 = 0; w2 < int(blockDim.x >> 5); ++w2) v += red[w2][tid];
      partial[int64_t(j0 + tid) * gridDim.x + blockIdx.x] = v;
    }
    __syncthreads();
  }
}

__global__ void sl_sum_partials_kernel(const double* __restrict__ partial, int nblocks, int nv,
                                       double* __restrict__ out) {
  const int j = blockIdx.x;
  if (j >= nv) return;
  __shared__ double red[256];
  double s = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) s += partial[int64_t(j) * nblocks + b];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (int(threadIdx.x) < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[j] = red[0];
}

// w += sign * sum_j h[j] V[j]
__global__ void sl_multiaxpy_kernel(const double* __restrict__ V, int64_t ldv, int nv, const double* __restrict__ h,
                                    double sign, int64_t n, double* __restrict__ w) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    double s = 0.0;
    for (int j = 0; j < nv; ++j) s += h[j] * V[int64_t(j) * ldv + i];
    w[i] += sign * s;
  }
}

__global__ void sl_residual_kernel(const double* __restrict__ b, const double* __restrict__ ax, int64_t n,
                                   double* __restrict__ r) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    r[i] = b[i] - ax[i];
}

__global__ void sl_scale_into_kernel(const double* __restrict__ a, double s, int64_t n, double* __restrict__ out) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    out[i] = a[i] * s;
}

int grid_of(int64_t n, int threads) {
  return int(std::max<int64_t>(1, std::min<int64_t>((n + threads - 1) / threads, 152 * 16)));
}

// shared memory sizes of the kernels that take more than 48 KiB (a host-side
// setting of each kernel, set before its launches)
template <typename T>
fq_status set_attributes(fq_ctx* ctx) {
  using C = SlCfg<T>;
  const int tile_smem = 2 * C::TILE * (C::TILE + 1) * int(sizeof(T));
  const int blk_smem = C::TILE * (C::ROWS + 1) * int(sizeof(T));
  FQ_CUDA(ctx, cudaFuncSetAttribute(sl_tile_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, tile_smem));
  FQ_CUDA(ctx, cudaFuncSetAttribute(sl_tourn_leaf_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, blk_smem));
  FQ_CUDA(ctx, cudaFuncSetAttribute(sl_tourn_merge_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, blk_smem));
  FQ_CUDA(ctx, cudaFuncSetAttribute(sl_compose_pivots_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    kMaxComposeRows * 4));
  return FQ_OK;
}

template <typename T>
fq_status factor_impl(fq_ctx* ctx, SparseLu& lu, const int32_t* rp, const int32_t* ci, const double* val) {
  using C = SlCfg<T>;
  cudaStream_t st = ctx->stream;
  int64_t maxf_all = 0;
  for (int x = 0; x < lu.nfronts; ++x) maxf_all = std::max<int64_t>(maxf_all, lu.front_f[x]);
  if (maxf_all > kMaxComposeRows)
    return set_error(ctx, FQ_UNSUPPORTED, "sparse LU: a front with more fully summed rows than the solve holds");
  const int prec = Num<T>::kPrecision;
  if (lu.precision != prec) {
    lu.pool.release();
    lu.tiles.release();
    lu.uvec.release();
    lu.work.release();
    lu.precision = prec;
  }
  if (!lu.pool.p) {
    FQ_TRY(lu.pool.alloc(ctx, size_t(lu.pool_elems) * sizeof(T)));
    FQ_TRY(lu.tiles.alloc(ctx, size_t(lu.tile_elems) * sizeof(T)));
    FQ_TRY(lu.uvec.alloc(ctx, size_t(lu.uvec_elems) * sizeof(T)));
    FQ_TRY(lu.work.alloc(ctx, size_t(std::max<int64_t>(lu.n, 1)) * sizeof(T)));
  }
  const int64_t half_sets = std::max<int64_t>(lu.tourn_sets, 1) * 2;  // IEEE FP64 leaves are half as tall
  if (!lu.piv.p) {
    FQ_TRY(lu.piv.alloc(ctx, size_t(std::max<int64_t>(lu.n, 1)) * 4));
    FQ_TRY(lu.fperm.alloc(ctx, size_t(std::max<int64_t>(lu.n, 1)) * 4));
    FQ_TRY(lu.ybuf.alloc(ctx, size_t(std::max<int64_t>(lu.n, 1)) * 8));
    // one flag per tile of the narrowest tiles (FP64), zero: no phase published
    const size_t nflags = size_t(lu.tile_elems / (2 * SlCfg<double>::TILE * SlCfg<double>::TILE) + 1);
    FQ_TRY(lu.flags.alloc(ctx, nflags * 4));
    FQ_CUDA(ctx, cudaMemsetAsync(lu.flags.p, 0, nflags * 4, st));
    FQ_TRY(lu.tickets.alloc(ctx, size_t(2 * std::max(lu.nlevels, 1)) * 4));
    FQ_TRY(lu.solve_status.alloc(ctx, 4));
    FQ_CUDA(ctx, cudaMemsetAsync(lu.solve_status.p, 0, 4, st));
    FQ_TRY(lu.status.alloc(ctx, 4 * sizeof(int)));
    FQ_TRY(lu.scale.alloc(ctx, size_t(std::max<int64_t>(lu.n, 1)) * 8));
    FQ_TRY(lu.tourn_cand.alloc(ctx, size_t(half_sets) * 2 * kTile * 4));
    FQ_TRY(lu.tourn_count.alloc(ctx, size_t(half_sets) * 2 * 4));
  }
  FQ_TRY(set_attributes<T>(ctx));
  // the symmetric scaling D A D, d_i = 1 / sqrt(max_j |a_ij|): on a symmetric
  // matrix every entry is then at most 1 in magnitude
  sl_row_scale_kernel<<<grid_of(lu.n, 256), 256, 0, st>>>(rp, val, lu.n, lu.scale.as<double>());
  ctx->launches++;
  // the pivot floor, relative to the scaled matrix's largest entry (1): about
  // ten units in the last place of FP32; far below any pivot the near-resonant
  // systems need in float-float (48-bit) and FP64
  const T thresh = Num<T>::from_double(prec == FQ_FP32 ? 1e-6 : prec == FQ_FP64 ? 1e-12 : 1e-13);
  FQ_CUDA(ctx, cudaMemsetAsync(lu.status.p, 0, 4 * sizeof(int), st));
  FQ_CUDA(ctx, cudaMemsetAsync(lu.piv.p, 0, size_t(std::max<int64_t>(lu.n, 1)) * 4, st));
  const int tile_smem = 2 * C::TILE * (C::TILE + 1) * int(sizeof(T));
  const int blk_smem = C::TILE * (C::ROWS + 1) * int(sizeof(T));
  const FrontDesc* fd = lu.fronts.as<FrontDesc>();
  const int32_t* lists = lu.level_list.as<int32_t>();
  T* pool = lu.pool.as<T>();
  T* tiles = lu.tiles.as<T>();
  for (int l = 0; l < lu.nlevels; ++l) {
    const int32_t q0 = lu.level_ptr[l], q1 = lu.level_ptr[l + 1];
    const int nl = q1 - q0;
    if (nl <= 0) continue;
    if (nl > 65535) return set_error(ctx, FQ_UNSUPPORTED, "sparse LU: more than 65,535 fronts in one level");
    const int32_t* list = lists + q0;
    // zero the level's fronts (contiguous in the pool)
    const int first = lu.level_fronts[q0], last = lu.level_fronts[q1 - 1];
    const int64_t zb = lu.front_off[first];
    const int64_t ze = lu.front_off[last] + int64_t(lu.front_m[last]) * lu.front_m[last];
    if (ze > zb) FQ_CUDA(ctx, cudaMemsetAsync(pool + zb, 0, size_t(ze - zb) * sizeof(T), st));
    const int64_t ab = lu.asm_ptr_h[l], ae = lu.asm_ptr_h[l + 1];
    if (ae > ab) {
      sl_assemble_kernel<T><<<grid_of(ae - ab, 256), 256, 0, st>>>(lu.asm_slot.as<int32_t>(), lu.asm_row.as<int32_t>(),
                                                                  lu.asm_off.as<int64_t>(), ab, ae, ci, val,
                                                                  lu.scale.as<double>(), pool);
      ctx->launches++;
    }
    if (l > 0) {
      // the children's update sizes bound the grid
      int64_t maxu2 = 0;
      for (int32_t q = q0; q < q1; ++q) {
        const int x = lu.level_fronts[q];
        for (int c : {lu.child0[x], lu.child1[x]})
          if (c >= 0) {
            const int64_t u = lu.front_m[c] - lu.front_f[c];
            maxu2 = std::max(maxu2, u * u);
          }
      }
      const int64_t want = (maxu2 + 255) / 256;
      const unsigned gx = unsigned(std::max<int64_t>(1, std::min<int64_t>(want, std::max<int64_t>(1, 152 * 16 / nl))));
      for (int which = 0; which < 2; ++which) {
        sl_extend_add_kernel<T><<<dim3(gx, unsigned(nl)), 256, 0, st>>>(fd, list, which, lu.ea_map.as<int32_t>(), pool);
        ctx->launches++;
      }
    }
    // partial factorization, tile by tile
    int maxf = 0;
    int64_t maxm = 0;
    for (int32_t q = q0; q < q1; ++q) {
      maxf = std::max(maxf, lu.front_f[lu.level_fronts[q]]);
      maxm = std::max<int64_t>(maxm, lu.front_m[lu.level_fronts[q]]);
    }
    for (int k = 0; k < maxf; k += C::TILE) {
      // pivot rows over the whole fully summed panel (tournament), moved to the top
      const int sets = (maxf - k + C::ROWS - 1) / C::ROWS;
      if (int64_t(nl) * sets > half_sets) return set_error(ctx, FQ_CUDA_ERROR, "sparse LU: tournament buffer too small");
      int32_t* cand[2] = {lu.tourn_cand.as<int32_t>(), lu.tourn_cand.as<int32_t>() + half_sets * kTile};
      int32_t* cnt[2] = {lu.tourn_count.as<int32_t>(), lu.tourn_count.as<int32_t>() + half_sets};
      FQ_CUDA(ctx, cudaMemsetAsync(cnt[0], 0, size_t(nl) * sets * 4, st));
      sl_tourn_leaf_kernel<T><<<dim3(unsigned(sets), unsigned(nl)), kThreads, blk_smem, st>>>(fd, list, k, pool, sets,
                                                                                             cand[0], cnt[0]);
      ctx->launches++;
      int cur = 0;
      for (int nsets = sets; nsets > 1; nsets = (nsets + 1) / 2) {
        sl_tourn_merge_kernel<T><<<dim3(unsigned((nsets + 1) / 2), unsigned(nl)), kThreads, blk_smem, st>>>(
            fd, list, k, pool, sets, nsets, cand[cur], cnt[cur], cand[cur ^ 1], cnt[cur ^ 1]);
        ctx->launches++;
        cur ^= 1;
      }
      sl_swap_sequence_kernel<<<unsigned(nl), 32, 0, st>>>(fd, list, k, C::TILE, sets, cand[cur],
                                                            lu.piv.as<int32_t>());
      const unsigned gcols = unsigned(std::max<int64_t>(1, std::min<int64_t>((maxm + 255) / 256, 64)));
      sl_apply_swaps_kernel<T><<<dim3(gcols, unsigned(nl)), 256, 0, st>>>(fd, list, k, C::TILE, lu.piv.as<int32_t>(),
                                                                         pool);
      sl_tile_kernel<T><<<unsigned(nl), kThreads, tile_smem, st>>>(fd, list, k, pool, tiles, lu.status.as<int>(),
                                                                   thresh);
      ctx->launches += 3;
      const int64_t rest = std::max<int64_t>(0, maxm - k);
      const int64_t tl = (rest + C::BM - 1) / C::BM;
      if (tl > 0) {
        const unsigned grids[3] = {unsigned(tl), unsigned(tl), unsigned(tl * tl)};
        for (int mode = 0; mode < 3; ++mode)
          sl_gemm_kernel<T><<<dim3(grids[mode], unsigned(nl)), kThreads, 0, st>>>(fd, list, k, mode, pool, tiles);
        ctx->launches += 3;
      }
    }
  }
  // the composed interchanges of every front, for the solve
  sl_compose_pivots_kernel<<<unsigned(lu.nfronts), 256, size_t(maxf_all) * 4, st>>>(fd, lu.piv.as<int32_t>(),
                                                                                   lu.fperm.as<int32_t>());
  ctx->launches++;
  FQ_CUDA(ctx, cudaGetLastError());
  int hs[4] = {0, 0, 0, 0};
  FQ_CUDA(ctx, cudaMemcpyAsync(hs, lu.status.p, sizeof hs, cudaMemcpyDeviceToHost, st));
  FQ_CUDA(ctx, cudaStreamSynchronize(st));
  lu.perturbed = hs[0];
  lu.nonfinite = hs[1];
  lu.factored = hs[1] == 0;
  if (hs[1] > 0) {
    const int x = hs[2] - 1;
    int lev = -1;
    for (int l = 0; l < lu.nlevels && x >= 0; ++l)
      for (int32_t q = lu.level_ptr[l]; q < lu.level_ptr[l + 1]; ++q)
        if (lu.level_fronts[q] == x) lev = l;
    return set_error(ctx, FQ_BREAKDOWN,
                     std::string("sparse LU: non-finite pivot (") +
                         (prec == FQ_FP32 ? "FP32" : prec == FQ_FP64 ? "float-float" : "FP64") + ", front " +
                         std::to_string(x) + " of level " + std::to_string(lev) + "/" + std::to_string(lu.nlevels) +
                         ", m " + std::to_string(x >= 0 ? lu.front_m[x] : -1) + ", f " +
                         std::to_string(x >= 0 ? lu.front_f[x] : -1) + ", column " + std::to_string(hs[3]) + ")");
  }
  return FQ_OK;
}

// The solve's row blocks, level by level, for tiles of width tl: forward, every
// front's fully summed tiles in order, then its update rows; backward, its
// tiles last to first.
fq_status make_items(fq_ctx* ctx, SparseLu& lu, int tl) {
  std::vector<int2> fw, bw;
  lu.fwd_ptr.assign(size_t(lu.nlevels) + 1, 0);
  lu.bwd_ptr.assign(size_t(lu.nlevels) + 1, 0);
  for (int l = 0; l < lu.nlevels; ++l) {
    for (int32_t q = lu.level_ptr[l]; q < lu.level_ptr[l + 1]; ++q) {
      const int x = lu.level_fronts[q];
      const int f = lu.front_f[x], u = lu.front_m[x] - f;
      const int nF = (f + tl - 1) / tl, nU = (u + tl - 1) / tl;
      for (int b = 0; b < nF + nU; ++b) fw.push_back(make_int2(x, b));
      for (int b = nF - 1; b >= 0; --b) bw.push_back(make_int2(x, b));
    }
    lu.fwd_ptr[l + 1] = int64_t(fw.size());
    lu.bwd_ptr[l + 1] = int64_t(bw.size());
  }
  for (int l = 0; l < lu.nlevels; ++l)
    if (lu.fwd_ptr[l + 1] - lu.fwd_ptr[l] > 0x7fffffff)
      return set_error(ctx, FQ_UNSUPPORTED, "sparse LU: a level with more row blocks than one launch takes");
  FQ_TRY(lu.fwd_items.alloc(ctx, std::max<size_t>(fw.size(), 1) * sizeof(int2)));
  FQ_TRY(lu.bwd_items.alloc(ctx, std::max<size_t>(bw.size(), 1) * sizeof(int2)));
  if (!fw.empty())
    FQ_CUDA(ctx, cudaMemcpyAsync(lu.fwd_items.p, fw.data(), fw.size() * sizeof(int2), cudaMemcpyHostToDevice,
                                 ctx->stream));
  if (!bw.empty())
    FQ_CUDA(ctx, cudaMemcpyAsync(lu.bwd_items.p, bw.data(), bw.size() * sizeof(int2), cudaMemcpyHostToDevice,
                                 ctx->stream));
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));  // the host lists go out of scope
  return FQ_OK;
}

template <typename T>
fq_status apply_impl(fq_ctx* ctx, SparseLu& lu, const double* r, double* z) {
  using C = SlCfg<T>;
  cudaStream_t st = ctx->stream;
  if (lu.items_precision != lu.precision) {
    FQ_TRY(make_items(ctx, lu, C::TILE));
    lu.items_precision = lu.precision;
  }
  const FrontDesc* fd = lu.fronts.as<FrontDesc>();
  T* work = lu.work.as<T>();
  T* ybuf = lu.ybuf.as<T>();
  int* tickets = lu.tickets.as<int>();
  int* flags = lu.flags.as<int>();
  int* status = lu.solve_status.as<int>();
  ++lu.epoch;
  const int fwd_target = int(2u * lu.epoch + 1u), bwd_target = int(2u * lu.epoch + 2u);
  FQ_CUDA(ctx, cudaMemsetAsync(tickets, 0, size_t(2 * std::max(lu.nlevels, 1)) * 4, st));
  sl_permute_in_kernel<T><<<grid_of(lu.n, 256), 256, 0, st>>>(r, lu.perm.as<int32_t>(), lu.scale.as<double>(), lu.n,
                                                              work);
  ctx->launches++;
  const int2* fwi = lu.fwd_items.as<int2>();
  const int2* bwi = lu.bwd_items.as<int2>();
  for (int l = 0; l < lu.nlevels; ++l) {
    const int64_t b = lu.fwd_ptr[l], e = lu.fwd_ptr[l + 1];
    if (e <= b) continue;
    sl_forward_rows_kernel<T><<<unsigned(e - b), kSolveThreads, 0, st>>>(
        fwi + b, int(e - b), tickets + l, fd, lu.pool.as<T>(), lu.tiles.as<T>(), lu.fperm.as<int32_t>(),
        lu.rinv.as<int32_t>(), work, ybuf, lu.uvec.as<T>(), flags, fwd_target, status);
    ctx->launches++;
  }
  for (int l = lu.nlevels - 1; l >= 0; --l) {
    const int64_t b = lu.bwd_ptr[l], e = lu.bwd_ptr[l + 1];
    if (e <= b) continue;
    sl_backward_rows_kernel<T><<<unsigned(e - b), kSolveThreads, 0, st>>>(
        bwi + b, int(e - b), tickets + lu.nlevels + l, fd, lu.pool.as<T>(), lu.tiles.as<T>(),
        lu.urows.as<int32_t>(), ybuf, work, flags, bwd_target, status);
    ctx->launches++;
  }
  sl_permute_out_kernel<T><<<grid_of(lu.n, 256), 256, 0, st>>>(work, lu.perm.as<int32_t>(), lu.scale.as<double>(),
                                                               lu.n, z);
  ctx->launches++;
  FQ_CUDA(ctx, cudaGetLastError());
  return FQ_OK;
}

struct GmresSpace {
  DevBuf V, Z, w, partial, h;
  int nblocks = 0;
};

fq_status multidot(fq_ctx* ctx, GmresSpace& g, int64_t n, int nv, const double* w, std::vector<double>& out) {
  cudaStream_t st = ctx->stream;
  sl_multidot_kernel<<<g.nblocks, 256, 0, st>>>(g.V.as<double>(), n, nv, w, n, g.partial.as<double>());
  sl_sum_partials_kernel<<<nv, 256, 0, st>>>(g.partial.as<double>(), g.nblocks, nv, g.h.as<double>());
  ctx->launches += 2;
  out.assign(nv, 0.0);
  FQ_CUDA(ctx, cudaMemcpyAsync(out.data(), g.h.p, nv * 8, cudaMemcpyDeviceToHost, st));
  FQ_CUDA(ctx, cudaStreamSynchronize(st));
  return FQ_OK;
}

fq_status self_dot(fq_ctx* ctx, GmresSpace& g, int64_t n, const double* w, double* out) {
  cudaStream_t st = ctx->stream;
  // the vector against itself through the same two-stage reduction
  sl_multidot_kernel<<<g.nblocks, 256, 0, st>>>(w, n, 1, w, n, g.partial.as<double>());
  sl_sum_partials_kernel<<<1, 256, 0, st>>>(g.partial.as<double>(), g.nblocks, 1, g.h.as<double>());
  ctx->launches += 2;
  FQ_CUDA(ctx, cudaMemcpyAsync(out, g.h.p, 8, cudaMemcpyDeviceToHost, st));
  FQ_CUDA(ctx, cudaStreamSynchronize(st));
  return FQ_OK;
}

fq_status axpy_h(fq_ctx* ctx, GmresSpace& g, const double* V, int64_t n, int nv, const std::vector<double>& h,
                 double sign, double* w) {
  cudaStream_t st = ctx->stream;
  FQ_CUDA(ctx, cudaMemcpyAsync(g.h.p, h.data(), nv * 8, cudaMemcpyHostToDevice, st));
  sl_multiaxpy_kernel<<<grid_of(n, 256), 256, 0, st>>>(V, n, nv, g.h.as<double>(), sign, n, w);
  ctx->launches++;
  FQ_CUDA(ctx, cudaStreamSynchronize(st));  // h is a host vector reused by the caller
  return FQ_OK;
}

}  // namespace

fq_status sparse_lu_factor(fq_ctx* ctx, SparseLu& lu, const int32_t* rp, const int32_t* ci, const double* val,
                           int precision) {
  lu.factored = false;
  if (precision == FQ_FP32) return factor_impl<float>(ctx, lu, rp, ci, val);
  if (precision == FQ_FP64_IEEE) return factor_impl<double>(ctx, lu, rp, ci, val);
  return factor_impl<df64>(ctx, lu, rp, ci, val);
}

fq_status sparse_lu_apply(fq_ctx* ctx, SparseLu& lu, const double* r, double* z) {
  if (!lu.factored) return set_error(ctx, FQ_INVALID_ARG, "sparse LU: not factored");
  if (lu.precision == FQ_FP32) return apply_impl<float>(ctx, lu, r, z);
  if (lu.precision == FQ_FP64_IEEE) return apply_impl<double>(ctx, lu, r, z);
  return apply_impl<df64>(ctx, lu, r, z);
}

// A solve ends when the relative residual meets rtol, or when the normwise
// backward error ||b - A x|| / (||A||_F ||x|| + ||b||) has reached the rounding
// level of FP64 (kBackwardFloor): what an LU solve of the same system
// delivers. On a nearly singular system (the near-resonant Lorentzian boxes)
// a residual of rtol may lie below that floor; GMRES then stops there instead
// of iterating on rounding errors.
constexpr double kBackwardFloor = 1e-14;

fq_status sparse_lu_gmres(fq_ctx* ctx, SparseLu& lu, const int32_t* rp, const int32_t* ci, const double* val,
                          const double* b, double* x, double rtol, int64_t max_iters, fq_report* rep) {
  const int64_t n = lu.n;
  const int restart = 30;
  cudaStream_t st = ctx->stream;
  GmresSpace g;
  g.nblocks = std::min<int>(int((n + 255) / 256), 152 * 4);
  FQ_TRY(g.V.alloc(ctx, size_t(restart + 1) * n * 8));
  FQ_TRY(g.Z.alloc(ctx, size_t(restart) * n * 8));
  FQ_TRY(g.w.alloc(ctx, size_t(n) * 8));
  FQ_TRY(g.partial.alloc(ctx, size_t(g.nblocks) * (restart + 2) * 8));
  FQ_TRY(g.h.alloc(ctx, size_t(restart + 2) * 8));
  double* V = g.V.as<double>();
  double* Z = g.Z.as<double>();
  double* w = g.w.as<double>();
  const unsigned spmv_blocks = unsigned((n * 4 + 255) / 256);
  FQ_CUDA(ctx, cudaMemsetAsync(x, 0, size_t(n) * 8, st));
  double bnorm2 = 0.0, anorm2 = 0.0;
  // the iterated matrix's own slot count: it may differ from the factored
  // pattern's (a shifted matrix whose pattern holds more slots)
  int32_t nnz_a = 0;
  FQ_CUDA(ctx, cudaMemcpyAsync(&nnz_a, rp + n, 4, cudaMemcpyDeviceToHost, st));
  FQ_CUDA(ctx, cudaStreamSynchronize(st));
  FQ_TRY(self_dot(ctx, g, n, b, &bnorm2));
  FQ_TRY(self_dot(ctx, g, nnz_a, val, &anorm2));
  const double bnorm = std::sqrt(bnorm2), anorm = std::sqrt(anorm2);
  fq_report r{};
  if (!(bnorm > 0.0)) {
    r.converged = 1;
    if (rep) *rep = r;
    return FQ_OK;
  }
  int64_t it = 0;
  double relres = 1.0;
  bool done = false;
  const int stale_limit = lu.precision == FQ_FP32 ? 3 : 5;
  std::vector<double> h, h2;
  while (!done && it < max_iters) {
    // r = b - A x into V[0]; the true residual and the backward error of x
    sl_spmv_kernel<<<spmv_blocks, 256, 0, st>>>(rp, ci, val, x, n, w);
    sl_residual_kernel<<<grid_of(n, 256), 256, 0, st>>>(b, w, n, V);
    ctx->launches += 2;
    double beta2 = 0.0, x2 = 0.0;
    FQ_TRY(self_dot(ctx, g, n, V, &beta2));
    FQ_TRY(self_dot(ctx, g, n, x, &x2));
    const double beta = std::sqrt(beta2);
    relres = beta / bnorm;
    if (relres <= rtol || (it > 0 && beta <= kBackwardFloor * (anorm * std::sqrt(x2) + bnorm))) {
      done = true;
      break;
    }
    sl_scale_into_kernel<<<grid_of(n, 256), 256, 0, st>>>(V, 1.0 / beta, n, V);
    ctx->launches++;
    std::vector<std::vector<double>> H(restart + 1, std::vector<double>(restart, 0.0));
    std::vector<double> cs(restart, 0.0), sn(restart, 0.0), gv(restart + 1, 0.0);
    gv[0] = beta;
    int j = 0;
    double best = relres;
    int stale = 0;
    for (; j < restart && it < max_iters; ++j, ++it) {
      FQ_TRY(sparse_lu_apply(ctx, lu, V + int64_t(j) * n, Z + int64_t(j) * n));
      sl_spmv_kernel<<<spmv_blocks, 256, 0, st>>>(rp, ci, val, Z + int64_t(j) * n, n, w);
      ctx->launches++;
      // classical Gram-Schmidt, twice
      FQ_TRY(multidot(ctx, g, n, j + 1, w, h));
      FQ_TRY(axpy_h(ctx, g, V, n, j + 1, h, -1.0, w));
      FQ_TRY(multidot(ctx, g, n, j + 1, w, h2));
      FQ_TRY(axpy_h(ctx, g, V, n, j + 1, h2, -1.0, w));
      for (int i = 0; i <= j; ++i) H[i][j] = h[i] + h2[i];
      double hn2 = 0.0;
      FQ_TRY(self_dot(ctx, g, n, w, &hn2));
      const double hn = std::sqrt(hn2);
      H[j + 1][j] = hn;
      if (hn > 0.0) {
        sl_scale_into_kernel<<<grid_of(n, 256), 256, 0, st>>>(w, 1.0 / hn, n, V + int64_t(j + 1) * n);
        ctx->launches++;
      }
      for (int i = 0; i < j; ++i) {
        const double a = H[i][j], c = H[i + 1][j];
        H[i][j] = cs[i] * a + sn[i] * c;
        H[i + 1][j] = -sn[i] * a + cs[i] * c;
      }
      const double a = H[j][j], c = H[j + 1][j];
      const double d = std::hypot(a, c);
      cs[j] = d > 0 ? a / d : 1.0;
      sn[j] = d > 0 ? c / d : 0.0;
      H[j][j] = d;
      H[j + 1][j] = 0.0;
      gv[j + 1] = -sn[j] * gv[j];
      gv[j] = cs[j] * gv[j];
      relres = std::fabs(gv[j + 1]) / bnorm;
      // stagnation: five iterations without halving the residual estimate (three
      // on FP32 factors, which then give way to FP64 ones) end the cycle early
      // (the true residual then decides)
      if (relres < 0.5 * best) {
        best = relres;
        stale = 0;
      } else if (++stale >= stale_limit) {
        ++j;
        ++it;
        break;
      }
      if (relres <= rtol || hn == 0.0) {
        ++j;
        ++it;
        break;
      }
    }
    // x += Z y, y = H^-1 g (upper triangular j x j)
    std::vector<double> y(j, 0.0);
    for (int i = j - 1; i >= 0; --i) {
      double s = gv[i];
      for (int l = i + 1; l < j; ++l) s -= H[i][l] * y[l];
      y[i] = H[i][i] != 0.0 ? s / H[i][i] : 0.0;
    }
    if (j > 0) FQ_TRY(axpy_h(ctx, g, Z, n, j, y, 1.0, x));
    if (stale >= stale_limit && it < max_iters) {
      // a stagnating cycle: accept x if it is at the rounding level, else the
      // restart continues (and a stagnating FP32 preconditioner gives way to
      // float-float factors in sparse_lu_solve)
      sl_spmv_kernel<<<spmv_blocks, 256, 0, st>>>(rp, ci, val, x, n, w);
      sl_residual_kernel<<<grid_of(n, 256), 256, 0, st>>>(b, w, n, w);
      ctx->launches += 2;
      double t2 = 0.0, xx = 0.0;
      FQ_TRY(self_dot(ctx, g, n, w, &t2));
      FQ_TRY(self_dot(ctx, g, n, x, &xx));
      relres = std::sqrt(t2) / bnorm;
      if (relres <= rtol || std::sqrt(t2) <= kBackwardFloor * (anorm * std::sqrt(xx) + bnorm)) {
        done = true;
        break;
      }
      if (lu.precision == FQ_FP32) break;  // the float-float factors take over
    }
  }
  if (!done) {
    // out of iterations: the last iterate's true residual and backward error
    sl_spmv_kernel<<<spmv_blocks, 256, 0, st>>>(rp, ci, val, x, n, w);
    sl_residual_kernel<<<grid_of(n, 256), 256, 0, st>>>(b, w, n, w);
    ctx->launches += 2;
    double t2 = 0.0, xx = 0.0;
    FQ_TRY(self_dot(ctx, g, n, w, &t2));
    FQ_TRY(self_dot(ctx, g, n, x, &xx));
    relres = std::sqrt(t2) / bnorm;
    done = relres <= rtol || std::sqrt(t2) <= kBackwardFloor * (anorm * std::sqrt(xx) + bnorm);
  }
  r.iters = it;
  r.residual = relres;
  r.true_residual = relres;
  r.converged = done ? 1 : 0;
  if (rep) *rep = r;
  // a wait of the triangular solves that ran out (none should) voids the result
  int waits = 0;
  FQ_CUDA(ctx, cudaMemcpyAsync(&waits, lu.solve_status.p, 4, cudaMemcpyDeviceToHost, st));
  FQ_CUDA(ctx, cudaStreamSynchronize(st));
  if (waits) {
    FQ_CUDA(ctx, cudaMemsetAsync(lu.solve_status.p, 0, 4, st));
    return set_error(ctx, FQ_CUDA_ERROR, "sparse LU solve: a wait for a tile's solution ran out");
  }
  return r.converged ? FQ_OK : FQ_NOT_CONVERGED;
}

fq_status sparse_lu_solve(fq_ctx* ctx, SparseLu& lu, const int32_t* rp, const int32_t* ci, const double* val,
                          const double* b, double* x, double rtol, int64_t max_iters, fq_report* rep) {
  fq_report r{};
  if (lu.factored && lu.precision != FQ_FP32) {
    const fq_status s64 = sparse_lu_gmres(ctx, lu, rp, ci, val, b, x, rtol, max_iters, &r);
    r.refinements = 1;
    if (rep) *rep = r;
    return s64;
  }
  fq_status s = FQ_NOT_CONVERGED;
  if (!lu.factored && lu.prefer_fp64) {
    // FP32 factors of this pattern did not converge before: FP64 ones at once
    FQ_TRY(sparse_lu_factor(ctx, lu, rp, ci, val, FQ_FP64));
    const fq_status s64 = sparse_lu_gmres(ctx, lu, rp, ci, val, b, x, rtol, max_iters, &r);
    r.refinements = 1;
    if (rep) *rep = r;
    return s64;
  }
  fq_status fs = lu.factored ? FQ_OK : sparse_lu_factor(ctx, lu, rp, ci, val, FQ_FP32);
  if (fs == FQ_OK) {
    s = sparse_lu_gmres(ctx, lu, rp, ci, val, b, x, rtol, std::min<int64_t>(max_iters, kFp32Iterations), &r);
    if (s != FQ_OK && s != FQ_NOT_CONVERGED) return s;
  } else if (fs != FQ_BREAKDOWN && fs != FQ_UNSUPPORTED) {
    return fs;
  }
  if (s == FQ_OK) {
    r.refinements = 0;
    if (rep) *rep = r;
    return FQ_OK;
  }
  // the FP32 factors were not enough: float-float factors, GMRES from zero (and those
  // at once for the next values of this pattern)
  lu.prefer_fp64 = true;
  fs = sparse_lu_factor(ctx, lu, rp, ci, val, FQ_FP64);
  if (fs == FQ_UNSUPPORTED || fs == FQ_BREAKDOWN) {
    if (rep) *rep = r;
    return FQ_NOT_CONVERGED;
  }
  FQ_TRY(fs);
  fq_report r2{};
  s = sparse_lu_gmres(ctx, lu, rp, ci, val, b, x, rtol, std::max<int64_t>(1, max_iters - r.iters), &r2);
  r2.iters += r.iters;
  r2.refinements = 1;
  if (rep) *rep = r2;
  return s;
}

}  // namespace fq
