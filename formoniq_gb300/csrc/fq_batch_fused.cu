// The batch's element pass as one launch over every class: the H(d) Gram
// programs hdif_gram(k) = M_k + dif_both(k+1) (whitney_complex.rs:180-183) of
// dimensions 2-4 and every grade, in float-float. A thread finds its mesh by
// binary search over the entries' first cells and runs that mesh's program,
// chosen by a switch on (dimension, grade). Registers are allocated per kernel,
// so every class runs at the occupancy of the heaviest program; the per-class
// launches of fq_batch.cu do not pay that, and the batch measures both.
#include <cuda_runtime.h>

#include "fq_element_kernel.cuh"
#include "fq_internal.h"

namespace fq {

__global__ void __launch_bounds__(128) batch_fused_hdif_kernel(const ElemFusedEntry* __restrict__ ent, int n,
                                                               int64_t total, int* status) {
  for (int64_t g = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; g < total; g += int64_t(gridDim.x) * blockDim.x) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (ent[mid].begin <= g)
        lo = mid;
      else
        hi = mid - 1;
    }
    const ElemFusedEntry& e = ent[lo];
    const int64_t cell = g - e.begin;
    switch (e.dim * 8 + e.grade) {
#define FQ_FUSED_CASE(N, K)                                                                                   \
  case N * 8 + K:                                                                                             \
    element_cell<N, K, EK_HDIF, df64>(e.lengths, e.cell_edges, e.ncells, cell, e.out, e.nent, 0.0, status); \
    break;
      FQ_FUSED_CASE(2, 0)
      FQ_FUSED_CASE(2, 1)
      FQ_FUSED_CASE(2, 2)
      FQ_FUSED_CASE(3, 0)
      FQ_FUSED_CASE(3, 1)
      FQ_FUSED_CASE(3, 2)
      FQ_FUSED_CASE(3, 3)
      FQ_FUSED_CASE(4, 0)
      FQ_FUSED_CASE(4, 1)
      FQ_FUSED_CASE(4, 2)
      FQ_FUSED_CASE(4, 3)
      FQ_FUSED_CASE(4, 4)
#undef FQ_FUSED_CASE
      default:
        atomicOr(status, 2);  // no program: reported like an entry outside its layout
    }
  }
}

bool batch_fused_supported(int kind, int dim, int grade) {
  return kind == EK_HDIF && dim >= 2 && dim <= 4 && grade >= 0 && grade <= dim;
}

void launch_batch_fused_hdif(const ElemFusedEntry* ent, int n, int64_t total, int grid, int* status,
                             cudaStream_t st) {
  if (total <= 0) return;
  const int64_t need = (total + 127) / 128;
  const unsigned blocks = unsigned(grid > 0 ? std::min<int64_t>(grid, need) : need);
  batch_fused_hdif_kernel<<<blocks, 128, 0, st>>>(ent, n, total, status);
}

int batch_fused_registers() {
  cudaFuncAttributes fa{};
  if (cudaFuncGetAttributes(&fa, batch_fused_hdif_kernel) != cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
  return fa.numRegs;
}

}  // namespace fq
