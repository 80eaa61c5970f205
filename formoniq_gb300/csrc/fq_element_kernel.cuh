// The fused per-cell kernel: kernel (a) (Regge metric, FP64) feeding kernel (b)
// (Whitney element matrices) for one of the element programs below. One thread
// per cell; cell data arrive entry-major ([local][cell]) so every load and store
// of a warp is one coalesced 128 B (FP32) / 256 B (FP64) transaction.
#pragma once

#include <cmath>
#include <type_traits>

#include "fq_df64.cuh"
#include "fq_element.cuh"
#include "fq_kinds.h"

namespace fq {

// One cell's element program: the entries of element KIND at grade K from the
// cell's inverse metric and volume, handed to put(entry, value) in the entry
// numbering of the program (packed upper triangle, or row-major for the
// rectangular dif_test/dif_trial). Shared by the device kernel and host checks.
// Kernel (a) for the element programs: from a cell's squared lengths to the
// barycentric Gramian B in T, with the metric determinant (as a double). In
// float-float for n <= 3 the metric, its inverse and determinant of a
// Riemannian cell (every squared length positive) are float-float too (the
// FP64 pipe runs at 1/62 of the FP32 rate on GB300 and would bound the
// kernel); the cofactor cancellation then costs about 20x the IEEE-double
// rounding, 2e-13 relative at 3D on 0.15h-jittered cells, which leaves the
// 1e-12 element tolerance a margin. At 4D the same loss reaches 9e-13, and a
// Lorentzian cell may be near null, so for those, as in the other modes, they
// stay IEEE double. FP32 programs take the float-float inverse of every
// Riemannian cell, 4D included (far inside their 1e-5 tolerance), rounded to
// FP32.
template <int N, typename T>
FQ_HD T cell_bary(const double* s, Bary<N, T>& B, bool& bad) {
  constexpr int NE = cbinom(N + 1, 2);
  // every squared length positive, tested on the bits (positive doubles are the
  // positive 64-bit integers): a double compare would issue on the FP64 pipe
  bool riemannian = true;
#pragma unroll
  for (int e = 0; e < NE; ++e) riemannian = riemannian && int64_t(bits_of(s[e])) > 0;
  if (std::is_same<T, df64>::value && N <= 3 && riemannian) {
    if constexpr (std::is_same<T, df64>::value && N <= 3) {
      df64 sd[NE > 0 ? NE : 1];
#pragma unroll
      for (int e = 0; e < NE; ++e) sd[e] = df64(s[e]);
      df64 g[N > 0 ? N : 1][N > 0 ? N : 1];
      df64 gi[N > 0 ? N : 1][N > 0 ? N : 1];
      regge_metric_t<N, df64>(sd, g);
      const df64 det = sym_inverse_t<N, df64>(g, gi);
      bary_gramian_t<N, df64>(gi, B);
      B.rdet = recip(det);
      bad = !(det.hi != 0.f) || !isfinite(det.hi);
      // vol = sqrt|det| / n!  (regge/src/lib.rs:26-28)
      return dd_sqrt(dd_abs(det)) * df64(1.0 / double(cfact(N)));
    }
  }
  // FP32 programs on the same cells: the float-float metric and inverse (on the
  // FP32 pipe, where IEEE double would bind the FP64 pipe), rounded to FP32
  if (std::is_same<T, float>::value && riemannian) {
    if constexpr (std::is_same<T, float>::value) {
      df64 sd[NE > 0 ? NE : 1];
#pragma unroll
      for (int e = 0; e < NE; ++e) sd[e] = df64(s[e]);
      df64 g[N > 0 ? N : 1][N > 0 ? N : 1];
      df64 gi[N > 0 ? N : 1][N > 0 ? N : 1];
      regge_metric_t<N, df64>(sd, g);
      const df64 det = sym_inverse_t<N, df64>(g, gi);
      float gf[N > 0 ? N : 1][N > 0 ? N : 1];
#pragma unroll
      for (int i = 0; i < N; ++i)
#pragma unroll
        for (int j = 0; j < N; ++j) gf[i][j] = f_add(gi[i][j].hi, gi[i][j].lo);
      bary_gramian_t<N, float>(gf, B);
      const df64 rd = recip(det);
      B.rdet = f_add(rd.hi, rd.lo);
      bad = !(det.hi != 0.f) || !isfinite(det.hi);
      const df64 v = dd_sqrt(dd_abs(det)) * df64(1.0 / double(cfact(N)));
      return f_add(v.hi, v.lo);
    }
  }
  double g[N > 0 ? N : 1][N > 0 ? N : 1];
  double gi[N > 0 ? N : 1][N > 0 ? N : 1];
  regge_metric<N>(s, g);
  const double det = sym_inverse<N>(g, gi);
  bary_gramian<N, T>(gi, B);
  B.rdet = T(1.0 / det);
  bad = !(det != 0.0) || !isfinite(det);
  return T(sqrt(fabs(det)) * (1.0 / double(cfact(N))));
}

template <int N, int K, int KIND, typename T, typename Put>
FQ_HD void element_entries(const Bary<N, T>& B, T vol, double param, Put&& put) {
  static_assert(KIND != EK_METRIC, "the metric program has no element entries");
  // mass scale vol (k!)^2 / ((n+1)(n+2)); dif_test scale vol (k!)^2 / (n+1);
  // stiffness scale vol (k!)^2.
  // (the constant factors are compile-time constants converted to T)
  auto mscale = [&](int k) { return vol * T(double(cfact(k)) * double(cfact(k)) / double((N + 1) * (N + 2))); };
  auto tscale = [&](int k) { return vol * T(double(cfact(k)) * double(cfact(k)) / double(N + 1)); };
  auto bscale = [&](int k) { return vol * T(double(cfact(k)) * double(cfact(k))); };

  if constexpr (KIND == EK_MASS) {
    constexpr int L = cbinom(N + 1, K + 1);
    Blades<N, K, T> H;
    compute_blades<N, K, T>(B, H);
    const T sc = mscale(K);
    static_for<L>([&](auto I) {
      static_for<L>([&](auto J) {
        constexpr int i = decltype(I)::value, j = decltype(J)::value;
        if constexpr (i <= j) put(packed_index(i, j, L), sc * mass_sum<N, K, i, j, T>(H));
      });
    });
  } else if constexpr (KIND == EK_DIF_BOTH) {
    constexpr int L = cbinom(N + 1, K);
    const T sc = bscale(K);
    static_for<L>([&](auto I) {
      static_for<L>([&](auto J) {
        constexpr int i = decltype(I)::value, j = decltype(J)::value;
        if constexpr (i <= j) put(packed_index(i, j, L), sc * blade_entry<N, K, i, j, T>(B));
      });
    });
  } else if constexpr (KIND == EK_HDIF) {
    constexpr int L = cbinom(N + 1, K + 1);
    Blades<N, K, T> H;
    compute_blades<N, K, T>(B, H);
    const T sm = mscale(K), sb = bscale(K + 1);
    static_for<L>([&](auto I) {
      static_for<L>([&](auto J) {
        constexpr int i = decltype(I)::value, j = decltype(J)::value;
        if constexpr (i <= j) {
          T v = sm * mass_sum<N, K, i, j, T>(H);
          if constexpr (K + 1 <= N) v += sb * blade_entry<N, K + 1, i, j, T>(B);
          put(packed_index(i, j, L), v);
        }
      });
    });
  } else if constexpr (KIND == EK_DIF_TEST || KIND == EK_DIF_TRIAL) {
    constexpr int LR = cbinom(N + 1, K);      // (k-1)-faces
    constexpr int LC = cbinom(N + 1, K + 1);  // k-faces
    Blades<N, K, T> H;
    compute_blades<N, K, T>(B, H);
    const T sc = tscale(K);
    static_for<LR>([&](auto R) {
      static_for<LC>([&](auto C) {
        constexpr int r = decltype(R)::value, c = decltype(C)::value;
        const T v = sc * dif_test_sum<N, K, r, c, T>(H);
        if constexpr (KIND == EK_DIF_TEST)
          put(r * LC + c, v);
        else
          put(c * LR + r, v);
      });
    });
  } else if constexpr (KIND == EK_KKT) {
    // Local composite: sigma = (k-1)-faces, then u = k-faces.
    constexpr int LS = kkt_sigma_local(N, K);
    constexpr int LU = cbinom(N + 1, K + 1);
    constexpr int L = LS + LU;
    constexpr int P = (L * (L + 1)) / 2;
    Blades<N, (K > 0 ? K - 1 : 0), T> Hs;
    if constexpr (K > 0) compute_blades<N, K - 1, T>(B, Hs);
    Blades<N, K, T> Hu;
    compute_blades<N, K, T>(B, Hu);
    const T sms = mscale(K > 0 ? K - 1 : 0), st = tscale(K), sbs = bscale(K);
    const T smu = mscale(K), sbu = bscale(K + 1);
    if constexpr (K > 0) {
      static_for<LS>([&](auto I) {
        constexpr int i = decltype(I)::value;
        static_for<LS>([&](auto J) {
          constexpr int j = decltype(J)::value;
          if constexpr (i <= j) {
            const T m = sms * mass_sum<N, K - 1, i, j, T>(Hs);
            put(packed_index(i, j, L), -m);
            if constexpr (i == j) put(P + i, m + sbs * Hu.template at<i, i>());
          }
        });
        static_for<LU>([&](auto J) {
          constexpr int j = decltype(J)::value;
          put(packed_index(i, LS + j, L), st * dif_test_sum<N, K, i, j, T>(Hu));
        });
      });
    }
    static_for<LU>([&](auto I) {
      constexpr int i = decltype(I)::value;
      static_for<LU>([&](auto J) {
        constexpr int j = decltype(J)::value;
        if constexpr (i <= j) {
          T st2 = T(0);
          if constexpr (K + 1 <= N) st2 = sbu * blade_entry<N, K + 1, i, j, T>(B);
          if constexpr (K + 1 <= N) put(packed_index(LS + i, LS + j, L), st2);
          if constexpr (i == j) put(P + LS + i, smu * mass_sum<N, K, i, i, T>(Hu) + st2);
        }
      });
    });
  } else if constexpr (KIND == EK_DIRAC) {
    // Local composite over every grade j = 0..n, block offsets o_j.
    constexpr int L = (1 << (N + 1)) - 1;
    const T mt = T(param);
    Blades<N, 0, T> H0;
    compute_blades<N, 0, T>(B, H0);
    Blades<N, (N >= 1 ? 1 : 0), T> H1;
    Blades<N, (N >= 2 ? 2 : 0), T> H2;
    Blades<N, (N >= 3 ? 3 : 0), T> H3;
    Blades<N, (N >= 4 ? 4 : 0), T> H4;
    if constexpr (N >= 1) compute_blades<N, 1, T>(B, H1);
    if constexpr (N >= 2) compute_blades<N, 2, T>(B, H2);
    if constexpr (N >= 3) compute_blades<N, 3, T>(B, H3);
    if constexpr (N >= 4) compute_blades<N, 4, T>(B, H4);
    auto grade_block = [&](auto JG, const auto& HJ) {
      constexpr int j = decltype(JG)::value;
      constexpr int off = grade_offset(N, j);
      constexpr int LJ = cbinom(N + 1, j + 1);
      const T sm = mt * mscale(j);
      static_for<LJ>([&](auto I) {
        static_for<LJ>([&](auto J2) {
          constexpr int a2 = decltype(I)::value, b2 = decltype(J2)::value;
          if constexpr (a2 <= b2) put(packed_index(off + a2, off + b2, L), sm * mass_sum<N, j, a2, b2, T>(HJ));
        });
      });
      if constexpr (j >= 1) {
        constexpr int offm = off - cbinom(N + 1, j);
        constexpr int LM = cbinom(N + 1, j);
        const T st = tscale(j);
        static_for<LM>([&](auto R) {
          static_for<LJ>([&](auto C) {
            constexpr int r = decltype(R)::value, c = decltype(C)::value;
            put(packed_index(offm + r, off + c, L), st * dif_test_sum<N, j, r, c, T>(HJ));
          });
        });
      }
    };
    grade_block(std::integral_constant<int, 0>{}, H0);
    if constexpr (N >= 1) grade_block(std::integral_constant<int, 1>{}, H1);
    if constexpr (N >= 2) grade_block(std::integral_constant<int, 2>{}, H2);
    if constexpr (N >= 3) grade_block(std::integral_constant<int, 3>{}, H3);
    if constexpr (N >= 4) grade_block(std::integral_constant<int, 4>{}, H4);
  }
}

// One cell of an element program: squared lengths in, the packed entries out
// ([nent][nc] layout of its mesh's buffer).
template <int N, int K, int KIND, typename T>
__device__ __forceinline__ void element_cell(const double* lengths, const int32_t* cell_edges, int64_t nc,
                                             int64_t cell, void* outp, int nent, double param, int* status) {
  constexpr int NE = cbinom(N + 1, 2);
  double s[NE > 0 ? NE : 1];
#pragma unroll
  for (int e = 0; e < NE; ++e) s[e] = __ldg(lengths + __ldg(cell_edges + int64_t(e) * nc + cell));
  Bary<N, T> B;
  bool bad = false;
  const T vol = cell_bary<N, T>(s, B, bad);
  if (bad) atomicOr(status, 1);
  T* out = static_cast<T*>(outp);
  element_entries<N, K, KIND, T>(B, vol, param, [&](int e, T v) {
    if (e < nent)
      out[int64_t(e) * nc + cell] = v;
    else
      atomicOr(status, 2);
  });
}

template <int N, int K, int KIND, typename T>
__global__ void __launch_bounds__(128) element_kernel(ElemArgs a) {
  const int64_t total = a.batch ? a.total : a.ncells;
  for (int64_t g = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; g < total; g += int64_t(gridDim.x) * blockDim.x) {
    // the cell's mesh: the launch's own, or the batch entry holding index g
    int64_t cell = g, nc = a.ncells;
    const double* lengths = a.lengths;
    const int32_t* cell_edges = a.cell_edges;
    void* outp = a.out;
    if (a.batch) {
      int lo = 0, hi = a.nbatch - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (a.batch[mid].begin <= g)
          lo = mid;
        else
          hi = mid - 1;
      }
      const ElemBatchEntry& b = a.batch[lo];
      cell = g - b.begin;
      nc = b.ncells;
      lengths = b.lengths;
      cell_edges = b.cell_edges;
      outp = b.out;
    }
    if constexpr (KIND == EK_METRIC) {
      constexpr int NE = cbinom(N + 1, 2);
      double s[NE > 0 ? NE : 1];
#pragma unroll
      for (int e = 0; e < NE; ++e) s[e] = __ldg(lengths + __ldg(cell_edges + int64_t(e) * nc + cell));
      double gm[N > 0 ? N : 1][N > 0 ? N : 1];
      double ginv[N > 0 ? N : 1][N > 0 ? N : 1];
      regge_metric<N>(s, gm);
      const double det = sym_inverse<N>(gm, ginv);
      const double vol = sqrt(fabs(det)) * (1.0 / double(cfact(N)));
      if (!(det != 0.0) || !isfinite(det)) atomicOr(a.status, 1);
      if (a.ginv_out) {
#pragma unroll
        for (int i = 0; i < N; ++i)
#pragma unroll
          for (int j = 0; j < N; ++j) a.ginv_out[int64_t(i * N + j) * nc + cell] = ginv[i][j];
      }
      if (a.det_out) a.det_out[cell] = det;
      if (a.vol_out) a.vol_out[cell] = vol;
    } else {
      element_cell<N, K, KIND, T>(lengths, cell_edges, nc, cell, outp, a.nent, a.param, a.status);
    }
  }
}

// The multi-program pass (ElemMultiArgs): one thread per cell, the cell's
// barycentric Gramian once, then each program's entries into its buffer.
// The Gramian and volume wait in shared memory between programs, so that they
// do not hold registers through every program.
template <int N, typename T>
__global__ void __launch_bounds__(128) element_multi_kernel(ElemMultiArgs a) {
  __shared__ __align__(16) unsigned char stage_raw[sizeof(Bary<N, T>) * 128];
  __shared__ __align__(16) unsigned char vol_raw[sizeof(T) * 128];
  Bary<N, T>& Bsh = reinterpret_cast<Bary<N, T>*>(stage_raw)[threadIdx.x];
  T& vsh = reinterpret_cast<T*>(vol_raw)[threadIdx.x];
  const int64_t nc = a.ncells;
  for (int64_t cell = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; cell < nc;
       cell += int64_t(gridDim.x) * blockDim.x) {
    {
      constexpr int NE = cbinom(N + 1, 2);
      double s[NE > 0 ? NE : 1];
#pragma unroll
      for (int e = 0; e < NE; ++e) s[e] = __ldg(a.lengths + __ldg(a.cell_edges + int64_t(e) * nc + cell));
      Bary<N, T> B;
      bool bad = false;
      vsh = cell_bary<N, T>(s, B, bad);
      Bsh = B;
      if (bad) atomicOr(a.status, 1);
    }
    for (int p = 0; p < a.nprog; ++p) {
      // reloaded per program: the programs' stores go through generic pointers,
      // which the compiler cannot tell from this shared-memory copy
      const Bary<N, T> B = Bsh;
      const T vol = vsh;
      T* out = static_cast<T*>(a.out[p]);
      const int nent = a.nent[p];
      auto put = [&](int e, T v) {
        if (e < nent)
          out[int64_t(e) * nc + cell] = v;
        else
          atomicOr(a.status, 2);
      };
      const int key = a.kind[p] * 8 + a.grade[p];
      static_for<N + 1>([&](auto KK) {
        constexpr int K = decltype(KK)::value;
        if (key == EK_MASS * 8 + K) element_entries<N, K, EK_MASS, T>(B, vol, 0.0, put);
        if constexpr (K >= 1)
          if (key == EK_DIF_BOTH * 8 + K) element_entries<N, K, EK_DIF_BOTH, T>(B, vol, 0.0, put);
      });
    }
  }
}

// Launch helper for one dimension and arithmetic type, every program and grade.
template <int N, typename T>
int launch_typed(int K, int kind, const ElemArgs& a, cudaStream_t st);
template <int N, typename T>
int launch_multi_typed(const ElemMultiArgs& a, cudaStream_t st);

}  // namespace fq
