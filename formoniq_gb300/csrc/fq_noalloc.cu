// Re-assembly that allocates nothing.
//
// Some callers of this library cannot let it call cudaMalloc: a host program
// that owns all device memory through its own arena (an embedding runtime with
// its own allocator, or a serving process that reserves its pool up front and
// forbids any other allocation), and latency-critical loops, where a
// cudaMalloc/cudaFree pair can synchronise the whole device. For them the
// per-cell element buffer that an assembly needs between the element kernel
// and the scatter lives here, in one statically sized device array, and
// fq_reassemble_noalloc writes the matrix values into the caller's buffer.
//
// The array is a file-scope __device__ variable of kNoAllocScratchBytes, so
// every GPU that loads this library holds it until the process exits. All calls
// on a device share it and it keeps the last call's contents; calls whose work
// overlaps on the GPU (two streams, or two host threads) race on it.
#include <cuda_runtime.h>

#include <string>

#include "fq_element_kernel.cuh"
#include "fq_internal.h"

namespace fq {

// 32 MiB: the element buffer of up to 4 Mi FP64 (8 Mi FP32) entries, e.g. M_1
// of a 199,728-cell 3D mesh at 21 entries per cell.
constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Set-up, with the context's device current: the host-side name of a
// __device__ array is only a stand-in, so its device address is looked up. It
// is looked up on every call (a cheap table lookup next to the status read the
// call ends with), so an address never outlives the module instance it came
// from, e.g. across a device reset.
static fq_status noalloc_scratch(fq_ctx* ctx, void** out) {
  int prev = 0;
  FQ_CUDA(ctx, cudaGetDevice(&prev));
  if (prev != ctx->device) FQ_CUDA(ctx, cudaSetDevice(ctx->device));
  void* ptr = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
  if (prev != ctx->device) cudaSetDevice(prev);
  if (e != cudaSuccess) return cuda_check(ctx, e, "cudaGetSymbolAddress(g_noalloc_scratch)");
  *out = ptr;
  return FQ_OK;
}

}  // namespace fq

using namespace fq;

extern "C" fq_status fq_reassemble_noalloc(fq_ctx* ctx, fq_mesh* mesh, const fq_matrix* pattern, void* values_out) {
  if (!ctx || !mesh || !pattern || !values_out) return FQ_INVALID_ARG;
  if (pattern->mesh != mesh || !pattern->plan)
    return set_error(ctx, FQ_INVALID_ARG, "pattern must be an assembled matrix of this mesh");
  if (pattern->compacted)
    return set_error(ctx, FQ_UNSUPPORTED, "pattern was compacted (exact-zero slots); use fq_reassemble");
  if (!mesh->has_lengths) return set_error(ctx, FQ_INVALID_ARG, "mesh has no edge lengths");
  const Plan& p = *pattern->plan;
  const int mode = pattern->precision;
  const size_t w = mode == FQ_FP32 ? 4 : 8;
  const size_t need = size_t(p.nent) * size_t(mesh->ncells) * w;
  if (need > kNoAllocScratchBytes)
    return set_error(ctx, FQ_INVALID_ARG,
                     "fq_reassemble_noalloc: needs " + std::to_string(need) + " bytes of scratch, the static maximum is " +
                         std::to_string(kNoAllocScratchBytes) + " bytes (element entries x cells x value width)");
  void* scratch = nullptr;
  FQ_TRY(noalloc_scratch(ctx, &scratch));
  unsigned char* base = static_cast<unsigned char*>(scratch);
  cudaStream_t st = ctx->stream;
  // the status words (degenerate-cell flag, zero-slot counter) start at zero
  FQ_CUDA(ctx, cudaMemsetAsync(ctx->status.p, 0, 8 * sizeof(int), st));
  if (p.nslots > 0) {
    ElemArgs a;
    a.ncells = mesh->ncells;
    a.lengths = mesh->lengths.as<double>();
    a.cell_edges = mesh->dim >= 1 ? mesh->cell_faces[1].as<int32_t>() : nullptr;
    a.out = base;
    a.ginv_out = a.det_out = a.vol_out = nullptr;
    a.param = pattern->param;
    a.status = ctx->status.as<int>();
    a.nent = p.nent;
    if (launch_element(mesh->dim, pattern->grade, pattern->kind, mode, a, st) != 0)
      return set_error(ctx, FQ_UNSUPPORTED, "no element program for this dimension/grade");
    ctx->launches++;
    FQ_CUDA(ctx, cudaGetLastError());
    launch_scatter(p, base, values_out, nullptr, ctx->status.as<int>(), element_buffer_mode(mesh->dim, pattern->kind, mode), st,
                   ctx->scatter_shape);
    ctx->launches++;
    FQ_CUDA(ctx, cudaGetLastError());
  }
  FQ_CUDA(ctx, cudaMemcpyAsync(ctx->host_status, ctx->status.p, 8 * sizeof(int), cudaMemcpyDeviceToHost, st));
  FQ_CUDA(ctx, cudaStreamSynchronize(st));
  if (ctx->host_status[0] & 4) return set_error(ctx, FQ_CUDA_ERROR, "symmetric plan without a mirror slot");
  if (ctx->host_status[0] & 2) return set_error(ctx, FQ_INVALID_ARG, "element program wrote outside its layout");
  if (ctx->host_status[0] & 1) return set_error(ctx, FQ_DEGENERATE_CELL, "a cell metric is singular or not finite");
  if (ctx->host_status[1] > 0)
    return set_error(ctx, FQ_UNSUPPORTED,
                     "some slots summed exact zeros only: the pattern would change; use fq_reassemble");
  return FQ_OK;
}
