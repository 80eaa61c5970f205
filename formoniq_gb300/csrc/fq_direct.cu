// The direct fallback of the solves: the reference factors the system with a
// sparse LU when its MINRES does not converge (problems/elliptic.rs:142-160,
// "LU also catches the rare non-convergence of the iterative path") and always
// for the Dirac source problem (problems/dirac.rs:473-531). Here a system of at
// most kDenseMax unknowns that MINRES left unconverged is solved by a dense LU
// with partial pivoting on the device (cuSOLVER getrf/getrs). cuSOLVER is loaded
// at run time; without it the fallback reports FQ_UNSUPPORTED and the caller
// keeps the iterative result.
#include <dlfcn.h>

#include <cusolverDn.h>

#include <algorithm>
#include <mutex>

#include "fq_internal.h"

namespace fq {

namespace {

struct Cusolver {
  bool ok = false;
  decltype(&cusolverDnCreate) create = nullptr;
  decltype(&cusolverDnDestroy) destroy = nullptr;
  decltype(&cusolverDnSetStream) set_stream = nullptr;
  decltype(&cusolverDnDgetrf_bufferSize) getrf_buffer = nullptr;
  decltype(&cusolverDnDgetrf) getrf = nullptr;
  decltype(&cusolverDnDgetrs) getrs = nullptr;
};

const Cusolver& cusolver() {
  static Cusolver c;
  static std::once_flag once;
  std::call_once(once, [] {
    void* h = nullptr;
    for (const char* name : {"libcusolver.so", "libcusolver.so.12", "libcusolver.so.11"}) {
      h = dlopen(name, RTLD_NOW | RTLD_LOCAL);
      if (h) break;
    }
    if (!h) return;
    c.create = reinterpret_cast<decltype(c.create)>(dlsym(h, "cusolverDnCreate"));
    c.destroy = reinterpret_cast<decltype(c.destroy)>(dlsym(h, "cusolverDnDestroy"));
    c.set_stream = reinterpret_cast<decltype(c.set_stream)>(dlsym(h, "cusolverDnSetStream"));
    c.getrf_buffer = reinterpret_cast<decltype(c.getrf_buffer)>(dlsym(h, "cusolverDnDgetrf_bufferSize"));
    c.getrf = reinterpret_cast<decltype(c.getrf)>(dlsym(h, "cusolverDnDgetrf"));
    c.getrs = reinterpret_cast<decltype(c.getrs)>(dlsym(h, "cusolverDnDgetrs"));
    c.ok = c.create && c.destroy && c.set_stream && c.getrf_buffer && c.getrf && c.getrs;
  });
  return c;
}

// Column-major dense copy of a CSR matrix (zero-filled before).
__global__ void csr_to_dense_kernel(const int32_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                    const double* __restrict__ val, int64_t n, double* __restrict__ a) {
  for (int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; r < n; r += int64_t(gridDim.x) * blockDim.x)
    for (int32_t q = rp[r]; q < rp[r + 1]; ++q) a[int64_t(ci[q]) * n + r] += val[q];
}

}  // namespace

bool dense_fallback_available() { return cusolver().ok; }

fq_status dense_lu_solve(fq_ctx* ctx, const int32_t* rp, const int32_t* ci, const double* val, int64_t n,
                         const double* b, double* x) {
  if (n <= 0) return FQ_OK;
  if (n > kDenseMax) return set_error(ctx, FQ_UNSUPPORTED, "system too large for the dense direct fallback");
  const Cusolver& cs = cusolver();
  if (!cs.ok) return set_error(ctx, FQ_UNSUPPORTED, "the dense direct fallback needs cuSOLVER at run time");
  cudaStream_t st = ctx->stream;
  DevBuf a, ipiv, info;
  FQ_TRY(a.alloc(ctx, size_t(n) * size_t(n) * 8));
  FQ_TRY(ipiv.alloc(ctx, size_t(n) * 4));
  FQ_TRY(info.alloc(ctx, 8));  // getrf's status, getrs's status
  FQ_CUDA(ctx, cudaMemsetAsync(a.p, 0, size_t(n) * size_t(n) * 8, st));
  csr_to_dense_kernel<<<int(std::min<int64_t>((n + 255) / 256, 152 * 8)), 256, 0, st>>>(rp, ci, val, n,
                                                                                        a.as<double>());
  ctx->launches++;
  FQ_CUDA(ctx, cudaGetLastError());
  FQ_CUDA(ctx, cudaMemcpyAsync(x, b, size_t(n) * 8, cudaMemcpyDeviceToDevice, st));
  cusolverDnHandle_t h = nullptr;
  if (cs.create(&h) != CUSOLVER_STATUS_SUCCESS) return set_error(ctx, FQ_CUDA_ERROR, "cusolverDnCreate failed");
  fq_status s = FQ_OK;
  int lwork = 0;
  DevBuf work;
  int host_info[2] = {0, 0};
  if (cs.set_stream(h, st) != CUSOLVER_STATUS_SUCCESS ||
      cs.getrf_buffer(h, int(n), int(n), a.as<double>(), int(n), &lwork) != CUSOLVER_STATUS_SUCCESS) {
    s = set_error(ctx, FQ_CUDA_ERROR, "cuSOLVER set-up failed");
  } else if ((s = work.alloc(ctx, std::max<size_t>(size_t(lwork) * 8, 16))) == FQ_OK) {
    if (cs.getrf(h, int(n), int(n), a.as<double>(), int(n), work.as<double>(), ipiv.as<int>(), info.as<int>()) !=
            CUSOLVER_STATUS_SUCCESS ||
        cs.getrs(h, CUBLAS_OP_N, int(n), 1, a.as<double>(), int(n), ipiv.as<int>(), x, int(n),
                 info.as<int>() + 1) != CUSOLVER_STATUS_SUCCESS) {
      s = set_error(ctx, FQ_CUDA_ERROR, "cuSOLVER getrf/getrs failed");
    } else {
      cudaMemcpyAsync(host_info, info.p, 8, cudaMemcpyDeviceToHost, st);
      if (cudaStreamSynchronize(st) != cudaSuccess)
        s = set_error(ctx, FQ_CUDA_ERROR, "dense LU failed");
      else if (host_info[0] != 0 || host_info[1] != 0)
        s = set_error(ctx, FQ_BREAKDOWN, "dense LU: singular system");
    }
  }
  cudaStreamSynchronize(st);
  cs.destroy(h);
  // cuSOLVER's return codes and getrf's info are checked above; a runtime error
  // the library left in this thread's last-error slot would otherwise surface in
  // the next unrelated call of the same host thread (a server lane's next request)
  cudaGetLastError();
  return s;
}

}  // namespace fq
