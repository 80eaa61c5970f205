// Element programs for cell dimension 2 in float arithmetic.
#include "fq_element_dispatch.cuh"

namespace fq {
template int launch_typed<2, float>(int K, int kind, const ElemArgs& a, cudaStream_t st);
template int launch_multi_typed<2, float>(const ElemMultiArgs& a, cudaStream_t st);
}  // namespace fq
