// Element programs for cell dimension 4 in float-float arithmetic (the
// mixed-system and H(d) Gram programs are in fq_element_n4_df_{kkt,hdif}.cu).
#define FQ_ELEM_T df64
#define FQ_SPLIT_KKT
#include "fq_element_dispatch.cuh"

namespace fq {
template int launch_typed<4, df64>(int K, int kind, const ElemArgs& a, cudaStream_t st);
}  // namespace fq
