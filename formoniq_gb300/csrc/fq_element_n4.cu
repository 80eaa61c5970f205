// Element programs instantiated for cell dimension 4.
#include "fq_element_dispatch.cuh"

namespace fq {
template int launch_element_dim<4>(int K, int kind, int fp32, const ElemArgs& a, cudaStream_t st);
}  // namespace fq
