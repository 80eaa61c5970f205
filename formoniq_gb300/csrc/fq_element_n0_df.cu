// Element programs for cell dimension 0 in df64 arithmetic.
#define FQ_ELEM_T df64
#include "fq_element_dispatch.cuh"

namespace fq {
template int launch_typed<0, df64>(int K, int kind, const ElemArgs& a, cudaStream_t st);
}  // namespace fq
