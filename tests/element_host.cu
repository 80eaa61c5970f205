// Host build of the per-cell element programs (the code the element kernels run,
// compiled by the host compiler), exported for the CPU tests: one cell's signed
// squared edge lengths in, the program's entries out. Lets the element algebra,
// including the float-float arithmetic, be checked against the oracle without a
// GPU.
//
// Compiled once per (dimension, arithmetic type) with -DEH_DIM=n and
// -DEH_TYPE=t (t in the fq_precision numbering: 0 float-float, 1 float,
// 2 double); each object exports eh_element_t<t>_n<n>.
#include <cstdint>
#include <type_traits>

#include "fq_element_kernel.cuh"

using namespace fq;

namespace {

template <typename T>
FQ_HD double as_double(T v) {
  if constexpr (std::is_same<T, df64>::value)
    return v.to_double();
  else
    return double(v);
}

// The entry sink handed to the program: records entries into a host array.
// Host+device only so that it may be called from the program's shared code.
template <typename T>
struct HostSink {
  double* out;
  int cap;
  int nent;
  bool overflow;
  FQ_HD void operator()(int e, T v) {
    if (e >= cap) {
      overflow = true;
      return;
    }
    out[e] = as_double(v);
    if (e + 1 > nent) nent = e + 1;
  }
};

template <int N, int K, int KIND, typename T>
int run_program(const double* s, double param, double* out, int cap, double* det_out) {
  Bary<N, T> B;
  bool bad = false;
  const T vol = cell_bary<N, T>(s, B, bad);
  if (det_out) *det_out = bad ? 0.0 : 1.0;
  HostSink<T> sink{out, cap, 0, false};
  element_entries<N, K, KIND, T>(B, vol, param, sink);
  return sink.overflow ? -2 : sink.nent;
}

template <int N, int K, typename T>
int run_kind(int kind, const double* s, double param, double* out, int cap, double* det) {
  switch (kind) {
    case EK_MASS:
      return run_program<N, K, EK_MASS, T>(s, param, out, cap, det);
    case EK_HDIF:
      return run_program<N, K, EK_HDIF, T>(s, param, out, cap, det);
    case EK_KKT:
      return run_program<N, K, EK_KKT, T>(s, param, out, cap, det);
    case EK_DIF_BOTH:
      if constexpr (K >= 1) return run_program<N, K, EK_DIF_BOTH, T>(s, param, out, cap, det);
      break;
    case EK_DIF_TEST:
      if constexpr (K >= 1) return run_program<N, K, EK_DIF_TEST, T>(s, param, out, cap, det);
      break;
    case EK_DIF_TRIAL:
      if constexpr (K >= 1) return run_program<N, K, EK_DIF_TRIAL, T>(s, param, out, cap, det);
      break;
    case EK_DIRAC:
      if constexpr (K == 0) return run_program<N, 0, EK_DIRAC, T>(s, param, out, cap, det);
      break;
    default:
      break;
  }
  return -1;
}

template <int N, typename T>
int run_n(int k, int kind, const double* s, double param, double* out, int cap, double* det) {
  if (kind == EK_DIRAC) k = 0;
  if constexpr (N >= 0)
    if (k == 0) return run_kind<N, 0, T>(kind, s, param, out, cap, det);
  if constexpr (N >= 1)
    if (k == 1) return run_kind<N, 1, T>(kind, s, param, out, cap, det);
  if constexpr (N >= 2)
    if (k == 2) return run_kind<N, 2, T>(kind, s, param, out, cap, det);
  if constexpr (N >= 3)
    if (k == 3) return run_kind<N, 3, T>(kind, s, param, out, cap, det);
  if constexpr (N >= 4)
    if (k == 4) return run_kind<N, 4, T>(kind, s, param, out, cap, det);
  return -1;
}

}  // namespace

#if EH_TYPE == 0
using EhT = df64;
#elif EH_TYPE == 1
using EhT = float;
#else
using EhT = double;
#endif

#define EH_CAT2(a, b, c, d) a##b##c##d
#define EH_CAT(a, b, c, d) EH_CAT2(a, b, c, d)
#define EH_NAME EH_CAT(eh_element_t, EH_TYPE, _n, EH_DIM)

// Returns the number of entries written, -1 for an unknown program, -2 when
// cap is too small.
extern "C" int EH_NAME(int k, int kind, const double* lengths_sq, double param, double* out, int cap, double* det) {
  return run_n<EH_DIM, EhT>(k, kind, lengths_sq, param, out, cap, det);
}

#if EH_DIM == 1 && EH_TYPE == 0
// The float-float conversions and square root, for the CPU tests.
extern "C" void eh_df64_split(const double* d, float* hi, float* lo, int n) {
  for (int i = 0; i < n; ++i) {
    const df64 v(d[i]);
    hi[i] = v.hi;
    lo[i] = v.lo;
  }
}
extern "C" void eh_df64_to_double(const float* hi, const float* lo, double* out, int n) {
  for (int i = 0; i < n; ++i) out[i] = df64(hi[i], lo[i]).to_double();
}
extern "C" void eh_df64_sqrt(const float* hi, const float* lo, float* ohi, float* olo, int n) {
  for (int i = 0; i < n; ++i) {
    const df64 r = dd_sqrt(df64(hi[i], lo[i]));
    ohi[i] = r.hi;
    olo[i] = r.lo;
  }
}
#endif
