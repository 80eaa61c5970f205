// Host-side internals of the library: context, device buffers, meshes, scatter
// plans and assembled matrices.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <exception>
#include <map>
#include <new>
#include <memory>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/formoniq_gpu.h"
#include "fq_kinds.h"

struct fq_ctx;

namespace fq {
struct SparseLu;

// Launch shape of the symmetric scatter: slots_per_thread -1 = by precision
// (measured on the 3D 32^3 step: one thread per upper slot for float-float
// values, one slot per thread on a persistent grid for FP32 and IEEE FP64),
// 0 = one thread per upper slot (scatter_sym_kernel), 1/2/4/8 = that many slots
// per thread on a persistent grid of blocks_per_sm 256-thread blocks per SM
// (0 = as many as are resident at once).
struct ScatterShape {
  int slots_per_thread = -1;
  int blocks_per_sm = 0;
};

// Owned device allocation, charged against the context's HBM budget.
struct DevBuf {
  fq_ctx* ctx = nullptr;
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept { *this = std::move(o); }
  DevBuf& operator=(DevBuf&& o) noexcept;
  ~DevBuf() { release(); }
  fq_status alloc(fq_ctx* c, size_t nbytes);
  void release();
  template <typename T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

// The scatter plan of one element program on one mesh: the CSR pattern and the
// contributions of every slot, sorted by (row, col) and, within a slot, by cell
// (the reference's summation order: per-thread triplets concatenated in cell
// order, galerkin.rs:150-188).
struct Plan {
  int kind = 0, grade = 0, row_bc = 0, col_bc = 0;
  int64_t nrows = 0, ncols = 0;
  int64_t nslots = 0;   // topological nnz
  int64_t ntrip = 0;    // contributions
  int nent = 0;         // element entries per cell of the program
  DevBuf row_ptr;       // int32 [nrows+1]
  DevBuf col_idx;       // int32 [nslots]
  DevBuf slot_ptr;      // int32 [nslots+1]
  DevBuf perm;          // int32 [ntrip]: element buffer index entry*ncells + cell
  // Symmetric programs on one space (row space = column space): the slots with
  // row <= col, each with its own index and its mirror's ((col,row); itself on
  // the diagonal), and their contributions. Slot (i,j) and (j,i) sum the same
  // packed element entries in the same cell order, so one sum serves both.
  int64_t nup = 0, ntrip_up = 0;
  DevBuf up_pair;       // int2 [nup]: (slot, mirror slot)
  DevBuf up_ptr;        // int32 [nup+1]
  DevBuf up_perm;       // int32 [ntrip_up]
  DevBuf up_rec;        // int4 [nup]: slot, mirror, first contribution, then the second one,
                        // -1 (only one) or -(2 + its position in up_perm) (more than two)
  int64_t ntail_slots = 0, ntail = 0;  // upper slots with more than two contributions; their contributions
                                       // past the first (read from up_perm)
  // Diagonal plan (EK_KKT preconditioner): slots = rows.
  int64_t ndiag_trip = 0;
  DevBuf diag_ptr;      // int32 [nrows+1]
  DevBuf diag_perm;     // int32 [ndiag_trip]
};

// Local degree-of-freedom layout of an element program (host mirror of the
// entry numbering in fq_element_kernel.cuh).
struct Layout {
  int nrow_local = 0, ncol_local = 0;
  std::vector<int> row_grade, row_face, row_block;  // per local row
  std::vector<int> col_grade, col_face, col_block;
  std::vector<int> entry;  // [nrow_local * ncol_local], -1 = structurally zero
  int nent = 0;            // entries written per cell
  std::vector<int> diag_entry;  // EK_KKT: preconditioner diagonal entry per local dof
  int nblocks = 0;
  std::vector<int> block_grade;  // grade of each block
};
Layout make_layout(int n, int kind, int grade);

}  // namespace fq

struct fq_mesh {
  fq_ctx* ctx = nullptr;
  int dim = 0;
  int64_t ncells = 0;
  int64_t nsimp[6] = {0, 0, 0, 0, 0, 0};
  int kuhn_nbox = 0;  // > 0 when made by fq_mesh_kuhn_cube
  // host topology
  std::vector<int32_t> skel[5];        // colex skeletons [N_k][k+1]
  std::vector<uint8_t> boundary[5];    // per simplex: on the boundary subcomplex
  std::vector<int32_t> interior_map[5];  // kidx -> relative index or -1
  int64_t ninterior[5] = {0, 0, 0, 0, 0};
  std::vector<int8_t> orientation;     // lazily computed
  std::vector<int32_t> cell_faces_host[5];  // cell-major [ncells][C(n+1,k+1)]
  // device topology: cell -> face kidx, entry-major [C(n+1,k+1)][ncells]
  fq::DevBuf cell_faces[5];
  fq::DevBuf interior_dev[5];  // int32 relative map
  fq::DevBuf skel_dev[5];      // int32 [N_k][k+1], uploaded on first use
  // geometry
  fq::DevBuf lengths;  // double [N_1]
  bool has_lengths = false;
  // cached scatter plans
  std::map<std::tuple<int, int, int, int>, std::unique_ptr<fq::Plan>> plans;
  // element buffer reused across assemblies
  fq::DevBuf elem;
  // face incidences [bc][grade] of the vector assemblies, built on first use
  fq::DevBuf inc_ptr[2][5], inc_src[2][5];
  // source loads: the last quadrature table (degree, w_q lambda_q) and the
  // per-cell slot buffer, kept across calls
  int source_degree = -1;
  fq::DevBuf source_rule, source_slots;
  // the sparse direct solver's analysis of the relative Dirac system (plain,
  // and bordered for the massless case), kept for the next solve on this mesh
  std::shared_ptr<fq::SparseLu> dirac_lu[2];
};

struct fq_matrix {
  fq_ctx* ctx = nullptr;
  fq_mesh* mesh = nullptr;
  fq::Plan* plan = nullptr;  // owned by the mesh; null for coboundaries
  int kind = 0, grade = 0, bc = 0, precision = 0;
  double param = 0.0;
  int64_t nrows = 0, ncols = 0, nnz = 0;
  bool compacted = false;  // some topological slot summed exact zeros only
  const int32_t* rp = nullptr;  // row_ptr in use (plan's or own)
  const int32_t* ci = nullptr;  // col_idx in use
  fq::DevBuf row_ptr, col_idx, values;
  // topological-pattern values and flags before compaction
  fq::DevBuf full_values, zero_flags;
  // own element buffer, for the multi-program pass of a multi-matrix assembly
  fq::DevBuf elem;
};

struct fq_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool owns_stream = false;
  uint64_t budget = 0;
  uint64_t in_use = 0;
  uint64_t launches = 0;
  std::string last_error;
  fq::DevBuf status;       // int [8] device status words
  int* host_status = nullptr;  // pinned mirror
  void* host_solver = nullptr; // pinned slots for polling Krylov state (1 KiB)
  fq::DevBuf scratch;      // reusable temporary storage
  // instrumentation: CUDA events on `stream` around element passes (slot 0) and
  // scatters (slot 1) of every assembly while `profiling` is set
  // the dense direct fallback of unconverged MINRES solves (fq_direct.cu); server
  // lanes leave it off (see fq_server.cpp)
  bool dense_fallback = true;
  fq::ScatterShape scatter_shape;  // launch shape of the symmetric scatter (fq_ctx_set_scatter_shape)
  bool profiling = false;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  std::vector<cudaEvent_t> prof_events;  // four per matrix of a multi-matrix assembly
  cudaStream_t copy_stream = nullptr;     // downloads overlapped with kernels (host-buffer assembly)
  std::vector<cudaEvent_t> copy_events;
  double prof_ms[4] = {0, 0, 0, 0};
  int64_t prof_n[4] = {0, 0, 0, 0};
};

namespace fq {

fq_status set_error(fq_ctx* ctx, fq_status s, const std::string& msg);

// The direct fallback (fq_direct.cu): A x = b by a dense LU with partial
// pivoting on the device, for systems of at most kDenseMax unknowns (A as CSR,
// b and x device vectors). FQ_UNSUPPORTED without cuSOLVER or above the size.
constexpr int64_t kDenseMax = 8192;
bool dense_fallback_available();
fq_status dense_lu_solve(fq_ctx* ctx, const int32_t* rp, const int32_t* ci, const double* val, int64_t n,
                         const double* b, double* x);

// The simplices of grade k on the device, [N_k][k+1] vertex ids (uploaded once
// per mesh, kept by the mesh).
fq_status device_skeleton(fq_ctx* ctx, fq_mesh* m, int k, const int32_t** out);
fq_status cuda_check(fq_ctx* ctx, cudaError_t e, const char* what);
#define FQ_CUDA(ctx, call)                                        \
  do {                                                            \
    cudaError_t _e = (call);                                      \
    if (_e != cudaSuccess) return ::fq::cuda_check(ctx, _e, #call); \
  } while (0)
#define FQ_TRY(expr)                  \
  do {                                \
    fq_status _s = (expr);            \
    if (_s != FQ_OK) return _s;       \
  } while (0)

// Exceptions never cross the C ABI: every extern "C" body sits in a guard.
#define FQ_GUARD_BEGIN try {
#define FQ_GUARD_END(ctx)                                                  \
  }                                                                        \
  catch (const std::bad_alloc&) {                                          \
    return fq::set_error(ctx, FQ_OOM_BUDGET, "host allocation failed");    \
  }                                                                        \
  catch (const std::exception& e) {                                        \
    return fq::set_error(ctx, FQ_INVALID_ARG, e.what());                   \
  }                                                                        \
  catch (...) {                                                            \
    return fq::set_error(ctx, FQ_INVALID_ARG, "unknown error");            \
  }

// ---- device entry points (implemented in .cu files) ----
struct ElemArgs;
// mode = fq_precision: 0 float-float compute with FP64 values, 1 FP32, 2 IEEE FP64.
int launch_element(int n, int grade, int kind, int mode, const ElemArgs& a, cudaStream_t st);

// Build the scatter plan on the device (sort with CUB).
fq_status build_plan(fq_ctx* ctx, fq_mesh* mesh, Plan& plan, const Layout& lay);

// values[s] = sum of elem[perm[t]] over the slot's contributions; zero_flags[s]
// = 1 when every contribution was exactly 0.0; status[1] += count of such
// slots; status[0] |= 4 if a symmetric plan misses a mirror slot.
// The element buffer's type (as a precision mode) of a program in a mode: the
// 4D Dirac program writes doubles in FQ_FP64 too.
int element_buffer_mode(int n, int kind, int mode);
void launch_scatter(const Plan& plan, const void* elem, void* values, uint8_t* zero_flags, int* status, int mode,
                    cudaStream_t st, ScatterShape shape = ScatterShape());
void launch_scatter_diag(const Plan& plan, const void* elem, double* out, int mode, cudaStream_t st);
void launch_df64_to_double(const void* in, double* out, int64_t n, cudaStream_t st);

// Compaction: drop slots whose flag is set.
fq_status compact_csr(fq_ctx* ctx, fq_matrix* m, int64_t nzero);

fq_status element_pass(fq_ctx* ctx, fq_mesh* mesh, int kind, int grade, int mode, double param, DevBuf& buf,
                       int nent);
fq_status get_plan(fq_ctx* ctx, fq_mesh* mesh, int kind, int grade, int row_bc, int col_bc, Plan** out);
fq_status assemble_into(fq_ctx* ctx, fq_matrix* m);
fq_status assemble_many(fq_ctx* ctx, fq_matrix* const* mats, int count);
fq_status assemble_host_many(fq_ctx* ctx, fq_mesh* mesh, const double* lengths, fq_matrix* const* mats,
                             void* const* out, int count);
fq_status make_matrix(fq_ctx* ctx, fq_mesh* mesh, int kind, int grade, int bc, int precision, double param,
                      fq_matrix** out);

// An operator applied by its own kernels (matrix-free): y = A x on `st`, every
// kernel returning at once when *done != 0 (a converged Krylov loop).
struct OpHook {
  void (*apply)(const void* self, const double* x, double* y, const int* done, cudaStream_t st) = nullptr;
  const void* self = nullptr;
};
// CG (iterative/src/krylov.rs:48-95) on an operator hook, diagonal
// preconditioner dinv (null = identity).
fq_status cg_run_op(fq_ctx* ctx, const OpHook& hook, int64_t n, const double* dinv, const double* b, double* x,
                    double rtol, int64_t max_iters, fq_report* rep);
void launch_lower_bound_rows(const uint64_t* keys, int64_t nkeys, int64_t nrows, uint64_t stride, int32_t* out,
                             cudaStream_t st);

// SpMV and vector kernels
void launch_spmv(const fq_matrix* a, const void* x, void* y, cudaStream_t st);
fq_status dev_alloc(fq_ctx* ctx, DevBuf& b, size_t bytes);

}  // namespace fq
