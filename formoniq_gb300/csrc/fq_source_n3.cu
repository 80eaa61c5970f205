// Source-load cell kernels for cell dimension 3.
#include "fq_source.cuh"

namespace fq {
template int launch_source_cells<3>(int K, int adim, const SourceArgs& a, cudaStream_t st);
}  // namespace fq
