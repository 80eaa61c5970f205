// Element programs instantiated for cell dimension 0.
#include "fq_element_dispatch.cuh"

namespace fq {
template int launch_element_dim<0>(int K, int kind, int fp32, const ElemArgs& a, cudaStream_t st);
}  // namespace fq
