// Matrix-free cell kernels for cell dimension 4: mass (one kind per
// translation unit keeps each compile short).
#include "fq_matfree.cuh"

namespace fq {
template int launch_elemop_cells_sel<4, 1u << EK_MASS>(int K, int kind, const ElemopArgs& a, cudaStream_t st);
}  // namespace fq
