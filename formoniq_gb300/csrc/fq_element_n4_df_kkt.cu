// The float-float mixed-system element program for cell dimension 4 (its own
// translation unit to bound compile time).
#include "fq_element_dispatch.cuh"

namespace fq {
int launch_kkt_n4_df(int K, const ElemArgs& a, cudaStream_t st) {
  switch (K) {
    case 0:
      return launch_one_t<4, 0, EK_KKT, df64>(a, st);
    case 1:
      return launch_one_t<4, 1, EK_KKT, df64>(a, st);
    case 2:
      return launch_one_t<4, 2, EK_KKT, df64>(a, st);
    case 3:
      return launch_one_t<4, 3, EK_KKT, df64>(a, st);
    case 4:
      return launch_one_t<4, 4, EK_KKT, df64>(a, st);
    default:
      return -1;
  }
}
}  // namespace fq
