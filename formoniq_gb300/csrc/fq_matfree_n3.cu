// Matrix-free cell kernels for cell dimension 3.
#include "fq_matfree.cuh"

namespace fq {
template int launch_elemop_cells<3>(int K, int kind, const ElemopArgs& a, cudaStream_t st);
}  // namespace fq
