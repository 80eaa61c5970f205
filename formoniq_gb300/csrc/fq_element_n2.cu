// Element programs instantiated for cell dimension 2.
#include "fq_element_dispatch.cuh"

namespace fq {
template int launch_element_dim<2>(int K, int kind, int fp32, const ElemArgs& a, cudaStream_t st);
}  // namespace fq
