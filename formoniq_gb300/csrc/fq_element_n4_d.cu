// Element programs for cell dimension 4 in double arithmetic.
#include "fq_element_dispatch.cuh"

namespace fq {
template int launch_typed<4, double>(int K, int kind, const ElemArgs& a, cudaStream_t st);
}  // namespace fq
