// Source-load cell kernels for cell dimension 1.
#include "fq_source.cuh"

namespace fq {
template int launch_source_cells<1>(int K, int adim, const SourceArgs& a, cudaStream_t st);
}  // namespace fq
