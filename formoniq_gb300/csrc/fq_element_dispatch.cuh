// Compile-time dispatch of the element programs for one dimension N.
#pragma once

#include <cuda_runtime.h>

#include "fq_element_kernel.cuh"

namespace fq {

// One arithmetic type per translation unit: launch_typed<N, T> is defined by
// instantiating this header in fq_element_n{N}_{df,f,d}.cu.
template <int N, int K, int KIND, typename T>
int launch_one_t(const ElemArgs& a, cudaStream_t st) {
  constexpr int threads = 128;
  const unsigned blocks = unsigned((a.ncells + threads - 1) / threads);
  if (blocks == 0) return 0;
  element_kernel<N, K, KIND, T><<<blocks, threads, 0, st>>>(a);
  return 0;
}

template <int N, typename T>
int launch_typed(int K, int kind, const ElemArgs& a, cudaStream_t st);

// mode: 0 float-float (df64), 1 float, 2 IEEE double; the metric kernel is double.
template <int N, int K, int KIND>
int launch_one(int mode, const ElemArgs& a, cudaStream_t st) {
  (void)mode;
  return launch_one_t<N, K, KIND, FQ_ELEM_T>(a, st);
}
#ifdef FQ_SPLIT_KKT
// The mixed-system program of this (dimension, type) lives in its own
// translation unit (compile time).
int launch_kkt_split(int K, const ElemArgs& a, cudaStream_t st);
int launch_hdif_split(int K, const ElemArgs& a, cudaStream_t st);
#endif

template <int N, int K>
int launch_k(int kind, int mode, const ElemArgs& a, cudaStream_t st) {
  switch (kind) {
    case EK_MASS:
      return launch_one<N, K, EK_MASS>(mode, a, st);
    case EK_HDIF:
#ifdef FQ_SPLIT_KKT
      return launch_hdif_split(K, a, st);
#else
      return launch_one<N, K, EK_HDIF>(mode, a, st);
#endif
    case EK_KKT:
#ifdef FQ_SPLIT_KKT
      return launch_kkt_split(K, a, st);
#else
      return launch_one<N, K, EK_KKT>(mode, a, st);
#endif
    case EK_DIF_BOTH:
      if constexpr (K >= 1) return launch_one<N, K, EK_DIF_BOTH>(mode, a, st);
      break;
    case EK_DIF_TEST:
      if constexpr (K >= 1) return launch_one<N, K, EK_DIF_TEST>(mode, a, st);
      break;
    case EK_DIF_TRIAL:
      if constexpr (K >= 1) return launch_one<N, K, EK_DIF_TRIAL>(mode, a, st);
      break;
    case EK_DIRAC:
      if constexpr (K == 0 && !(N == 4 && std::is_same<FQ_ELEM_T, df64>::value))
        return launch_one<N, 0, EK_DIRAC>(mode, a, st);
      break;
    case EK_METRIC:
      if constexpr (K == 0 && std::is_same<FQ_ELEM_T, double>::value) return launch_one<N, 0, EK_METRIC>(0, a, st);
      break;
    default:
      break;
  }
  return -1;
}

template <int N, typename T>
int launch_typed(int K, int kind, const ElemArgs& a, cudaStream_t st) {
  if (kind == EK_DIRAC || kind == EK_METRIC) K = 0;
  if constexpr (N >= 0) if (K == 0) return launch_k<N, 0>(kind, 0, a, st);
  if constexpr (N >= 1) if (K == 1) return launch_k<N, 1>(kind, 0, a, st);
  if constexpr (N >= 2) if (K == 2) return launch_k<N, 2>(kind, 0, a, st);
  if constexpr (N >= 3) if (K == 3) return launch_k<N, 3>(kind, 0, a, st);
  if constexpr (N >= 4) if (K == 4) return launch_k<N, 4>(kind, 0, a, st);
  return -1;
}

}  // namespace fq
