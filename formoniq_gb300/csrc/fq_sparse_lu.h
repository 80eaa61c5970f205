// A sparse direct solver for the indefinite systems of the path (the relative
// Hodge-Dirac system, the mixed Hodge-Laplace KKT system, their bordered
// singular variants), standing in for the reference's FaerLu
// (formoniq/src/linalg/faer.rs:51-74) where the reference factors instead of
// iterating: solve_dirac_source (problems/dirac.rs:525-531, 578-598) and the LU
// fallback of solve_source (problems/elliptic.rs:147-160).
//
// Method: multifrontal LU on a nested-dissection ordering, GPU-native.
//   - Ordering: geometric nested dissection of the Kuhn vertex lattice. A box
//     of lattice points is split across its longest axis by the plane of points
//     at its middle coordinate; Kuhn edges join points whose coordinates differ
//     by at most 1 per axis, so no edge crosses the plane and the plane's points
//     separate the two halves. Every degree of freedom is a simplex; its
//     vertices lie on one root-to-leaf chain of the tree, and it is eliminated
//     at the deepest node of that chain. Extra (border) unknowns go to the root.
//   - Symbolic analysis (host, once per pattern): the fully summed unknowns F
//     and update unknowns U of every front, the map of every matrix slot into
//     the front where it is assembled, the extend-add maps, and a level
//     schedule (a front's level is one more than its highest child's).
//   - Scaling: D A D is factored, d_i = 1 / sqrt(max_j |a_ij|), so that the
//     grades' very different entry scales meet one pivot floor.
//   - Numeric factorization (device, once per set of values), level by level,
//     all fronts of a level batched in each launch: zero the fronts, assemble
//     the matrix slots, extend-add the children's Schur complements, then a
//     partial LU of the fully summed block in tiles: the pivot rows of a tile
//     chosen over all the front's fully summed rows by tournament pivoting and
//     moved to the top, the tile's LU (a pivot below 1e-6 of the scaled
//     matrix's largest entry is perturbed to +-1e-6) and triangular inverses,
//     the L and U panels by products with those inverses, and the trailing
//     Schur update, each a batched product (FP32: tiles of 128 columns on the
//     FP32 pipe; FP64: tiles of 64 columns).
//   - Solve: forward and backward substitution level by level, one launch per
//     level and direction, one CTA per row block (a tile's rows) of every
//     front of the level: a block streams its rows of the L (U) panel against
//     the tile solutions before it (after it), waiting for each on a flag its
//     producer publishes, then applies the tile's triangular inverse. CTAs take
//     row blocks by ticket, so a block only waits for blocks already running.
//     Update vectors go to the parent like the Schur complements.
//   - Accuracy: the factors precondition a restarted GMRES in FP64 on the FP64
//     matrix (GMRES-based iterative refinement), which stops on the true FP64
//     relative residual; FP32 factors first, float-float ones (FQ_FP64) when
//     those do not converge (the near-resonant Lorentzian systems). Float-float
//     arithmetic runs on the FP32 pipe, which this GPU has many times the
//     throughput of its FP64 pipe; IEEE FP64 factors remain on request.
#pragma once

#include <cstdint>
#include <vector>

#include "fq_internal.h"

namespace fq {

constexpr int kTile = 128;  // widest tile (FP32); the tile store and candidate sets are sized for it

// One front, as the kernels see it.
struct FrontDesc {
  int64_t off;       // pool offset
  int64_t tile_off;  // offset of its first tile's inverses in the tile store
  int64_t start;     // elimination position of its first fully summed unknown
  int64_t ea_off;    // offset of its update unknowns in ea_map / urows
  int64_t uvec_off;  // offset of its forward update vector
  int64_t roff;      // offset of its rows in the per-row maps (rinv)
  int32_t m, f;      // front size, fully summed count
  int32_t parent;    // parent front or -1
  int32_t child0, child1;  // children or -1
  int32_t pad;
};

struct SparseLu {
  int64_t n = 0;    // unknowns
  int64_t nnz = 0;  // matrix slots
  int nfronts = 0, nlevels = 0;
  // host symbolic data
  std::vector<int64_t> front_off;    // element offset of each front in the pool (m x m, column-major)
  std::vector<int32_t> front_m, front_f;  // front size, fully summed count
  std::vector<int64_t> front_start;  // elimination position of the first fully summed unknown
  std::vector<int32_t> level_ptr;    // fronts of level l: level_fronts[level_ptr[l] .. level_ptr[l+1])
  std::vector<int32_t> level_fronts;
  std::vector<int32_t> parent;           // parent front or -1
  std::vector<int32_t> child0, child1;   // children or -1
  int64_t pool_elems = 0;
  int64_t tile_elems = 0;  // entries of the tiles' triangular inverses (two kTile^2 blocks per 128 columns)
  int64_t uvec_elems = 0;  // entries of the forward update vectors (u per front)
  int64_t row_elems = 0;   // rows of all fronts (m per front)
  double flops = 0.0;      // of the numeric factorization
  int64_t tourn_sets = 0;  // candidate sets of the widest level: fronts x ceil(max f / 256)
  // device data
  DevBuf perm;        // int32 [n]: elimination position of each unknown
  DevBuf fronts;      // FrontDesc [nfronts]
  DevBuf level_list;  // int32 [nfronts]: fronts in level order
  DevBuf asm_slot;    // int32 [nnz]: the matrix slots, grouped by the level of their front
  DevBuf asm_off;     // int64 [nnz]: pool offset of each slot (same order)
  DevBuf asm_row;     // int32 [nnz]: row of each slot (same order)
  std::vector<int64_t> asm_ptr_h;  // [nlevels + 1]
  DevBuf ea_map;      // int32: per front, the parent-local index of each of its update unknowns
  DevBuf urows;       // int32: per front, the elimination positions of its update unknowns
  DevBuf rinv;        // int32 [2 x row_elems]: per front row, its index among child 0's and
                      // child 1's update unknowns (-1: none), the extend-add maps inverted
  int precision = -1; // the type of the factors below: FQ_FP32, FQ_FP64 (float-float) or FQ_FP64_IEEE
  DevBuf pool;        // the fronts
  DevBuf tiles;       // per tile, inverse of unit L then inverse of U (tile x tile each)
  DevBuf piv;         // int32 [n]: per fully summed position p, the front-local row
                      // interchanged with row p (applied in order of p)
  DevBuf uvec;        // forward update vectors
  DevBuf work;        // [n]: permuted right-hand side / solution
  DevBuf scale;       // double [n]: symmetric scaling d_i = 1 / sqrt(max_j |a_ij|); D A D is factored
  DevBuf status;      // int [4]: perturbed pivots, non-finite pivots
  DevBuf tourn_cand;  // int32: tournament candidates (ping-pong)
  DevBuf tourn_count; // int32: their counts
  // the solve: row blocks of the fronts, one CTA each, level by level
  DevBuf fperm;       // int32 [n]: per fully summed position, the front-local row whose value
                      // the composed interchanges move there
  DevBuf ybuf;        // [n]: forward solution of the fully summed rows
  DevBuf flags;       // int32: per tile, the solve phase whose solution is published
  DevBuf tickets;     // int32 [2 x nlevels]: row-block tickets of the level launches
  DevBuf solve_status;  // int32: waits that ran out
  int items_precision = -1;  // the tile width the item lists below were made for
  DevBuf fwd_items, bwd_items;  // int2 (front, row block), by level
  std::vector<int64_t> fwd_ptr, bwd_ptr;  // [nlevels + 1]
  uint32_t epoch = 0;   // solves so far (flags carry 2 epoch + 1 forward, 2 epoch + 2 backward)
  int perturbed = 0, nonfinite = 0;
  bool factored = false;
  bool prefer_fp64 = false;  // an FP32 factorization of this pattern did not converge: later solves factor in FP64
};

// The host maps of a symbolic analysis (uploaded by sparse_lu_analyse).
struct SparseLuMaps {
  std::vector<int32_t> pos, aslot, arow, ea, ur, rinv;
  std::vector<int64_t> aoff;
  std::vector<FrontDesc> fd;
};

// The symbolic analysis without the upload; it also checks that every index
// the kernels form stays inside its buffer (FQ_CUDA_ERROR otherwise).
fq_status sparse_lu_analyse_host(fq_ctx* ctx, SparseLu& lu, int dim, int nbox, int64_t n, const int32_t* rp,
                                 const int32_t* ci, const int32_t* dof_vertices, SparseLuMaps& maps);
// Symbolic analysis on the host: the system's pattern (host CSR, square,
// structurally symmetric), and for every unknown up to five vertex ids (-1
// padded; an unknown with no vertex goes to the root), on a Kuhn lattice of
// nbox boxes per axis in dimension dim; then the maps go to the device.
fq_status sparse_lu_analyse(fq_ctx* ctx, SparseLu& lu, int dim, int nbox, int64_t n, const int32_t* rp,
                            const int32_t* ci, const int32_t* dof_vertices);
// The same for a device CSR system of n unknowns on a Kuhn mesh (pattern
// downloaded once), unknowns described by dofv (five vertex ids each).
fq_status sparse_lu_build(fq_ctx* ctx, const fq_mesh* m, int64_t n, const int32_t* rp, const int32_t* ci,
                          const std::vector<int32_t>& dofv, SparseLu& lu);
// Numeric factorization from the device CSR values (FP64) of the analysed
// pattern, in FQ_FP32, FQ_FP64 (float-float: pairs of floats, 48-bit
// significand, on the FP32 pipe) or FQ_FP64_IEEE (IEEE double).
fq_status sparse_lu_factor(fq_ctx* ctx, SparseLu& lu, const int32_t* rp, const int32_t* ci, const double* val,
                           int precision);
// z = (LU)^-1 r on the device (FP64 in and out, the factors' type inside).
fq_status sparse_lu_apply(fq_ctx* ctx, SparseLu& lu, const double* r, double* z);
// GMRES(restart) in FP64 on A (device CSR), right-preconditioned by the
// factorization, from x = 0 to ||b - A x|| <= rtol ||b||.
fq_status sparse_lu_gmres(fq_ctx* ctx, SparseLu& lu, const int32_t* rp, const int32_t* ci, const double* val,
                          const double* b, double* x, double rtol, int64_t max_iters, fq_report* rep);
// The solve with precision adaptation: GMRES on FP32 factors (factored here if
// the current ones are not FP32) for at most kFp32Iterations iterations; if it
// has not converged, the system is factored in FP64 and GMRES starts again from
// zero (report.refinements = 1 then; iterations of both counted). After such a
// fallback the analysis remembers it, and the next unfactored solve of the
// pattern factors in FP64 at once.
constexpr int64_t kFp32Iterations = 60;
fq_status sparse_lu_solve(fq_ctx* ctx, SparseLu& lu, const int32_t* rp, const int32_t* ci, const double* val,
                          const double* b, double* x, double rtol, int64_t max_iters, fq_report* rep);

// Vertex lists of the unknowns of an element program's system on a mesh (the
// layout's grade blocks under boundary condition bc, each simplex by its
// vertices); rows past the blocks (a harmonic border) get none.
fq_status layout_dof_vertices(fq_ctx* ctx, const fq_mesh* m, int kind, int grade, int bc, int64_t nrows,
                              std::vector<int32_t>& out);

}  // namespace fq
