// Compile-time dispatch of the element programs for one dimension N and one
// arithmetic type T. Every template here takes T explicitly, so the instances
// made in different translation units (one per (N, T)) have distinct names.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <type_traits>

#include "fq_element_kernel.cuh"

namespace fq {

constexpr int kElemMultiThreads = 128;

template <int N, int K, int KIND, typename T>
int launch_one_t(const ElemArgs& a, cudaStream_t st) {
  constexpr int threads = 128;
  const int64_t total = a.batch ? a.total : a.ncells;
  if (total <= 0) return 0;
  const int64_t need = (total + threads - 1) / threads;
  const unsigned blocks = unsigned(a.grid > 0 ? std::min<int64_t>(a.grid, need) : need);
  element_kernel<N, K, KIND, T><<<blocks, threads, 0, st>>>(a);
  return 0;
}

// Programs of a (dimension, type) that live in their own translation unit to
// bound compile time: the float-float 4D mixed-system and H(d) Gram programs.
int launch_kkt_n4_df(int K, const ElemArgs& a, cudaStream_t st);
int launch_hdif_n4_df(int K, const ElemArgs& a, cudaStream_t st);

template <int N, typename T>
constexpr bool split_n4_df() {
  return N == 4 && std::is_same<T, df64>::value;
}

template <int N, int K, typename T>
int launch_k_t(int kind, const ElemArgs& a, cudaStream_t st) {
  switch (kind) {
    case EK_MASS:
      return launch_one_t<N, K, EK_MASS, T>(a, st);
    case EK_HDIF:
      if constexpr (split_n4_df<N, T>())
        return launch_hdif_n4_df(K, a, st);
      else
        return launch_one_t<N, K, EK_HDIF, T>(a, st);
    case EK_KKT:
      if constexpr (split_n4_df<N, T>())
        return launch_kkt_n4_df(K, a, st);
      else
        return launch_one_t<N, K, EK_KKT, T>(a, st);
    case EK_DIF_BOTH:
      if constexpr (K >= 1) return launch_one_t<N, K, EK_DIF_BOTH, T>(a, st);
      break;
    case EK_DIF_TEST:
      if constexpr (K >= 1) return launch_one_t<N, K, EK_DIF_TEST, T>(a, st);
      break;
    case EK_DIF_TRIAL:
      if constexpr (K >= 1) return launch_one_t<N, K, EK_DIF_TRIAL, T>(a, st);
      break;
    case EK_DIRAC:
      // the 4D Dirac program is dispatched to IEEE double by the caller
      if constexpr (K == 0 && !split_n4_df<N, T>()) return launch_one_t<N, 0, EK_DIRAC, T>(a, st);
      break;
    case EK_METRIC:
      if constexpr (K == 0 && std::is_same<T, double>::value) return launch_one_t<N, 0, EK_METRIC, T>(a, st);
      break;
    default:
      break;
  }
  return -1;
}

template <int N, typename T>
int launch_multi_typed(const ElemMultiArgs& a, cudaStream_t st) {
  if (a.ncells <= 0) return 0;
  const unsigned blocks = unsigned((a.ncells + kElemMultiThreads - 1) / kElemMultiThreads);
  element_multi_kernel<N, T><<<blocks, kElemMultiThreads, 0, st>>>(a);
  return 0;
}

template <int N, typename T>
int launch_typed(int K, int kind, const ElemArgs& a, cudaStream_t st) {
  if (kind == EK_DIRAC || kind == EK_METRIC) K = 0;
  if constexpr (N >= 0)
    if (K == 0) return launch_k_t<N, 0, T>(kind, a, st);
  if constexpr (N >= 1)
    if (K == 1) return launch_k_t<N, 1, T>(kind, a, st);
  if constexpr (N >= 2)
    if (K == 2) return launch_k_t<N, 2, T>(kind, a, st);
  if constexpr (N >= 3)
    if (K == 3) return launch_k_t<N, 3, T>(kind, a, st);
  if constexpr (N >= 4)
    if (K == 4) return launch_k_t<N, 4, T>(kind, a, st);
  return -1;
}

}  // namespace fq
