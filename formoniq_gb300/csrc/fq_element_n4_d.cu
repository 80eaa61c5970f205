// Element programs for cell dimension 4 in double arithmetic.
#define FQ_ELEM_T double
#include "fq_element_dispatch.cuh"

namespace fq {
template int launch_typed<4, double>(int K, int kind, const ElemArgs& a, cudaStream_t st);
}  // namespace fq
