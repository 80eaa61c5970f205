// Compile-time dispatch of the element programs for one dimension N.
#pragma once

#include <cuda_runtime.h>

#include "fq_element_kernel.cuh"

namespace fq {

template <int N, int K, int KIND>
int launch_one(int fp32, const ElemArgs& a, cudaStream_t st) {
  constexpr int threads = 128;
  const unsigned blocks = unsigned((a.ncells + threads - 1) / threads);
  if (blocks == 0) return 0;
  if (fp32 && KIND != EK_METRIC)
    element_kernel<N, K, KIND, float><<<blocks, threads, 0, st>>>(a);
  else
    element_kernel<N, K, KIND, double><<<blocks, threads, 0, st>>>(a);
  return 0;
}

template <int N, int K>
int launch_k(int kind, int fp32, const ElemArgs& a, cudaStream_t st) {
  switch (kind) {
    case EK_MASS:
      return launch_one<N, K, EK_MASS>(fp32, a, st);
    case EK_HDIF:
      return launch_one<N, K, EK_HDIF>(fp32, a, st);
    case EK_KKT:
      return launch_one<N, K, EK_KKT>(fp32, a, st);
    case EK_DIF_BOTH:
      if constexpr (K >= 1) return launch_one<N, K, EK_DIF_BOTH>(fp32, a, st);
      break;
    case EK_DIF_TEST:
      if constexpr (K >= 1) return launch_one<N, K, EK_DIF_TEST>(fp32, a, st);
      break;
    case EK_DIF_TRIAL:
      if constexpr (K >= 1) return launch_one<N, K, EK_DIF_TRIAL>(fp32, a, st);
      break;
    case EK_DIRAC:
      if constexpr (K == 0) return launch_one<N, 0, EK_DIRAC>(fp32, a, st);
      break;
    case EK_METRIC:
      if constexpr (K == 0) return launch_one<N, 0, EK_METRIC>(0, a, st);
      break;
    default:
      break;
  }
  return -1;
}

template <int N>
int launch_element_dim(int K, int kind, int fp32, const ElemArgs& a, cudaStream_t st) {
  if (kind == EK_DIRAC || kind == EK_METRIC) K = 0;
  if constexpr (N >= 0) if (K == 0) return launch_k<N, 0>(kind, fp32, a, st);
  if constexpr (N >= 1) if (K == 1) return launch_k<N, 1>(kind, fp32, a, st);
  if constexpr (N >= 2) if (K == 2) return launch_k<N, 2>(kind, fp32, a, st);
  if constexpr (N >= 3) if (K == 3) return launch_k<N, 3>(kind, fp32, a, st);
  if constexpr (N >= 4) if (K == 4) return launch_k<N, 4>(kind, fp32, a, st);
  return -1;
}

}  // namespace fq
