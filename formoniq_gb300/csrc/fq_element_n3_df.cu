// Element programs for cell dimension 3 in df64 arithmetic.
#include "fq_element_dispatch.cuh"

namespace fq {
template int launch_typed<3, df64>(int K, int kind, const ElemArgs& a, cudaStream_t st);
template int launch_multi_typed<3, df64>(const ElemMultiArgs& a, cudaStream_t st);
}  // namespace fq
