// Element programs instantiated for cell dimension 3.
#include "fq_element_dispatch.cuh"

namespace fq {
template int launch_element_dim<3>(int K, int kind, int fp32, const ElemArgs& a, cudaStream_t st);
}  // namespace fq
