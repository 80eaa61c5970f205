// Element programs shared by the device kernels and the host plan builder.
#pragma once

#include <cstdint>

#include "fq_combinatorics.cuh"

namespace fq {

enum ElemKind {
  EK_MASS = 0,      // WhitneyPairing::mass(k)                  operators.rs:169-171
  EK_DIF_TRIAL = 1, // WhitneyPairing::dif_trial(k)             operators.rs:175-177
  EK_DIF_TEST = 2,  // WhitneyPairing::dif_test(k)              operators.rs:182-184
  EK_DIF_BOTH = 3,  // WhitneyPairing::dif_both(k)              operators.rs:189-191
  EK_HDIF = 4,      // HilbertComplex::hdif_gram(k) = M_k + dif_both(k+1)  whitney_complex.rs:180-183
  EK_KKT = 5,       // assemble_mixed_kkt blocks + preconditioner diagonal  elliptic.rs:29-114
  EK_DIRAC = 6,     // HodgeDirac::assemble_selfadjoint + m M   dirac.rs:205-260, 473-500
  EK_METRIC = 7     // kernel (a) alone
};

// Sum of C(n+1, i+1) for i < j: the local offset of the grade-j block of the
// Dirac composite.
FQ_HD constexpr int grade_offset(int n, int j) {
  int o = 0;
  for (int i = 0; i < j; ++i) o += cbinom(n + 1, i + 1);
  return o;
}

// Local sigma-block size of the mixed system at grade k: the (k-1)-faces of a
// cell, none at grade 0 (Lambda^{-1} = 0).
FQ_HD constexpr int kkt_sigma_local(int n, int k) { return k > 0 ? cbinom(n + 1, k) : 0; }

// One mesh of a batched element launch: its cells are the global cell indices
// [begin, begin + ncells) of the launch.
struct ElemBatchEntry {
  int64_t begin, ncells;
  const double* lengths;
  const int32_t* cell_edges;
  void* out;
};

// One mesh of the fused batch element launch (every class in one launch): as
// ElemBatchEntry, plus the mesh's program (dimension, grade) and its entries
// per cell.
struct ElemFusedEntry {
  int64_t begin, ncells;
  const double* lengths;
  const int32_t* cell_edges;
  void* out;
  int nent, dim, grade, pad;
};

// Several element programs of one mesh in one pass: each cell's metric,
// inverse and barycentric Gramian computed once for all of them. Programs:
// EK_MASS or EK_DIF_BOTH at their grades, each into its own buffer.
constexpr int kMultiPrograms = 4;
struct ElemMultiArgs {
  int64_t ncells;
  const double* lengths;
  const int32_t* cell_edges;
  int* status;
  int nprog;
  int kind[kMultiPrograms], grade[kMultiPrograms], nent[kMultiPrograms];
  void* out[kMultiPrograms];
};

// Arguments of the per-cell kernel (device pointers).
struct ElemArgs {
  int64_t ncells;
  const double* lengths;     // [N1]
  const int32_t* cell_edges; // [C(n+1,2)][ncells]
  void* out;                 // [nent][ncells], T
  double* ginv_out;          // optional [n*n][ncells]
  double* det_out;           // optional [ncells]
  double* vol_out;           // optional [ncells]
  double param;              // mass term of the Dirac program
  int* status;               // bit 0: a singular or non-finite cell metric;
                             // bit 1: an element entry index outside [0, nent)
  int nent;                  // entries per cell the output buffer holds
  // Batched launch (null for one mesh): `nbatch` meshes sorted by begin,
  // `total` cells in all; the single-mesh fields above are then unused.
  const ElemBatchEntry* batch = nullptr;
  int nbatch = 0;
  int64_t total = 0;
  int grid = 0;              // CTAs of the launch (0: one thread per cell)
};

}  // namespace fq
