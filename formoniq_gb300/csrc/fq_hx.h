// Hiptmair-Xu auxiliary-space preconditioning over a nodal multigrid hierarchy
// (host-side structures; kernels in fq_mg.cu, set-up in fq_hx.cpp).
//
// Reference: formoniq/src/hx.rs (hx_preconditioner, vector_nodal_prolongation,
// MultigridBlocks), formoniq/src/multigrid.rs (RefinementTower::grade_vcycle,
// Galerkin coarse operators), iterative/src/multigrid.rs (VCycle::cycle),
// iterative/src/aux_space.rs (AuxiliarySpace::apply) and iterative/src/precond.rs
// (Jacobi::smoother, weight 2/3).
//
// The grade-j preconditioner is the reference's recursion
//   B_0 = S_0 + V,   B_j = S_j + D_{j-1} B_{j-1} D_{j-1}^T + Pi_j V^{C(n,j)} Pi_j^T,
// S_j the weighted Jacobi smoother of A_j = hdif_gram(j), V the nodal V-cycle
// of A_0 and Pi_j the vector-nodal interpolation. Because D_{j-1} D_{j-2} = 0,
// unrolling the recursion leaves
//   B_j r = S_j r + D_{j-1} (S_{j-1} t + Pi_{j-1} V Pi_{j-1}^T t) + Pi_j V Pi_j^T r,
//   t = D_{j-1}^T r,
// so every nodal solve a block needs is known before any V-cycle runs: all
// blocks of the mixed system gather their nodal right-hand sides into one
// interleaved block X[node][slot] and a single multi-right-hand-side V-cycle
// serves them all.
#pragma once

#include <cstdint>
#include <memory>
#include <vector>

#include "fq_internal.h"

namespace fq {

// Device CSR. Values in FP64 and, on demand, FP32. Either owns its arrays or
// views another object's.
struct DCsr {
  int64_t nrows = 0, ncols = 0, nnz = 0;
  const int32_t* rp = nullptr;
  const int32_t* ci = nullptr;
  const double* v64 = nullptr;
  const float* v32 = nullptr;
  DevBuf own_rp, own_ci, own_v64, own_v32;
  // Vector-nodal maps keep their lattice values (unit spacing) and, per entry,
  // the axis set I of its component: value = base * prod_{a in I} h_a.
  DevBuf own_base, own_mask;
  bool scalable = false;

  fq_status upload(fq_ctx* ctx, int64_t nr, int64_t nc, const std::vector<int32_t>& hrp,
                   const std::vector<int32_t>& hci, const std::vector<double>& hv);
  void view(const fq_matrix* m);
  fq_status make_f32(fq_ctx* ctx);
  template <typename VT>
  const VT* val() const;
};

// Host CSR.
struct HCsr {
  int64_t nrows = 0, ncols = 0;
  std::vector<int32_t> rp{0}, ci;
  std::vector<double> v;
  std::vector<uint8_t> mask;  // optional: axis set of each entry's component
};
HCsr transpose(const HCsr& a);

// One level of the nodal hierarchy (finest first).
struct NodalLevel {
  int nbox = 0;        // lattice boxes per axis
  int64_t n = 0;       // unknowns (nodes, interior nodes for the relative complex)
  DCsr A;              // operator: the mesh's hdif_gram(0), then P^T A P
  DevBuf dinv64;       // 2/3 / diag(A)
  DevBuf dinv32;
  DCsr P, R;           // this level <- the next coarser level, R = P^T
  DevBuf x[2], r, t;   // work blocks [n][mmax] (x ping-pong)
};

struct NodalHierarchy {
  int dim = 0, bc = 0, sweeps = 2, mmax = 0;
  std::vector<NodalLevel> lv;   // lv.back() is solved densely
  DevBuf coarse_inv64, coarse_inv32;  // [nc][nc]
  int64_t nc = 0;
};

// One diagonal block of a block preconditioner: grade j, at offset `off` of the
// block vector, with its HX ingredients.
struct HxBlock {
  int grade = 0;
  int64_t off = 0, size = 0;
  DevBuf s64, s32;           // S_j: 2/3 / diag(A_j)
  // gradient path (grade >= 1)
  DCsr D, Dt;                // D_{j-1} (size x n_{j-1}) and transpose
  DevBuf sl64, sl32;         // S_{j-1}
  DevBuf t, t2;              // n_{j-1} work vectors (VT-sized, max FP64)
  int grad_slot = 0, grad_count = 0;
  DCsr PiL, PiLt;            // Pi_{j-1} (cols = X offsets) and transpose (j-1 >= 1), or the
                             // slot identity (j-1 == 0)
  // vector-nodal path
  int vec_slot = 0, vec_count = 0;
  DCsr Pi, Pit;              // Pi_j (cols = X offsets) and transpose
};

struct HxPrecond {
  NodalHierarchy mg;
  std::vector<HxBlock> blocks;
  int64_t n = 0;             // length of the block vector
  int64_t ident_off = 0, ident_len = 0;  // identity tail (harmonic border)
  int m = 0;                 // nodal slots
  bool has_f32 = false;
  // structure key: what the lattice-only parts were built for
  const fq_mesh* mesh = nullptr;
  int bc = 0;
  std::vector<int> grades;
  // length-dependent inputs, reassembled by hx_refresh
  std::unique_ptr<fq_matrix> a0;                 // hdif_gram(0)
  std::vector<std::unique_ptr<fq_matrix>> aux;   // hdif_gram(g) of gradient smoothers
  std::vector<int> aux_grade;
  DevBuf axis_edges;                             // lattice edge kidx per axis, concatenated
  std::vector<int64_t> axis_off;                 // [n+1]
  DevBuf hprod, flag;                            // [16] products of spacings; [1] non-positive length seen
  fq_status make_f32(fq_ctx* ctx);
};

// ---- set-up (fq_hx.cpp) ----
// Whether the HX-multigrid preconditioner applies to this mesh: a Kuhn cube
// whose nodal operator is positive definite (Riemannian lengths).
bool hx_supported(const fq_mesh* m);
// Build the preconditioner of the block-diagonal operator diag(hdif_gram(j) for
// j in grades), blocks laid out in that order, plus `ident` trailing identity
// rows. diag_blocks holds the FP64 diagonal of each block's A_j (device, the
// block vector layout). Recomputes everything that depends on the lengths.
fq_status hx_build(fq_ctx* ctx, fq_mesh* m, int bc, const std::vector<int>& grades, int64_t ident,
                   const double* diag_blocks, HxPrecond& out);
// Whether `pc` was built for this mesh, boundary condition and block grades.
bool hx_matches(const HxPrecond& pc, const fq_mesh* m, int bc, const std::vector<int>& grades, int64_t ident);
// Recompute everything that depends on the lengths (operators, Galerkin
// products, coarse inverse, smoothers, frame scaling), keeping the structure.
fq_status hx_refresh(fq_ctx* ctx, fq_mesh* m, const double* diag_blocks, HxPrecond& pc);

// ---- device builders of the set-up maps (fq_hx_setup.cu) ----
// The device skeleton of grade k ([N_k][k+1]), uploaded on first use.
fq_status device_skeleton(fq_ctx* ctx, fq_mesh* m, int k, const int32_t** out);
// The coboundary D_k (rows (k+1)-simplices, columns k-simplices; relative: interior ones).
fq_status coboundary_device(fq_ctx* ctx, fq_mesh* m, int k, int bc, DCsr& D);
// The vector-nodal map Pi_j (columns node * mslots + slot + I) and its transpose
// with rows (node, I), both scalable (lattice values in own_base, axis sets in own_mask).
fq_status vector_nodal_device(fq_ctx* ctx, fq_mesh* m, int j, int bc, int mslots, int slot, DCsr& Pi, DCsr& Pit);
// A^T (mslots == 0), stable; with mask, the per-entry masks follow the entries.
fq_status device_transpose(fq_ctx* ctx, const DCsr& a, const uint8_t* mask, int64_t nt_rows, int mslots, int slot,
                           int ncomp, DCsr& out, DevBuf* out_mask);

// ---- device parts (fq_mg.cu) ----
fq_status galerkin_product(fq_ctx* ctx, const DCsr& A, const DCsr& P, DCsr& out);
fq_status device_diag_recip(fq_ctx* ctx, const DCsr& A, double omega, DevBuf& out);
fq_status device_to_host(fq_ctx* ctx, const DCsr& A, HCsr& out);
void launch_f64_to_f32(const double* a, float* o, int64_t n, cudaStream_t st);
// h_a = sqrt(mean of the axis-a lattice edge lengths), hprod[I] = prod_{a in I} h_a;
// flag = 1 when a length is not positive.
void launch_lattice_spacing(const double* lengths, const int32_t* axis_edges, const int64_t* off_host, int n,
                            double* hprod, int* flag, cudaStream_t st);
fq_status upload_scalable(fq_ctx* ctx, const HCsr& h, DCsr& d);
void launch_scale_by_mask(const double* base, const uint8_t* mask, const double* hprod, double* out, int64_t nnz,
                          cudaStream_t st);

// y = B r on `st`; every kernel returns at once when *done != 0 (a Krylov loop
// that has converged), so the preconditioner can sit inside a captured graph.
template <typename VT>
void hx_apply(const HxPrecond& pc, const VT* r, VT* y, const int* done, cudaStream_t st);

}  // namespace fq
