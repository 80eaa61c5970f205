// Element programs for cell dimension 2 in double arithmetic.
#define FQ_ELEM_T double
#include "fq_element_dispatch.cuh"

namespace fq {
template int launch_typed<2, double>(int K, int kind, const ElemArgs& a, cudaStream_t st);
}  // namespace fq
