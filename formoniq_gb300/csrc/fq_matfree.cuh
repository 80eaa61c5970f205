// Matrix-free Whitney operators (ElementOperator, formoniq/src/matfree.rs:54-172).
//
// y = sum_K P_K^T A_K P_K x without storing A_K or a sparsity pattern. The
// reference keeps one metric per cell and rebuilds each A_K per apply; here
// the cell kernel rebuilds A_K from the cell's squared lengths (the metric,
// its inverse and the element entries of the element programs, in
// float-float), gathers x at the cell's trial faces, and writes A_K P_K x to
// the cell's own slots [local row][cell] -- disjoint by construction. A second
// kernel then gathers, per degree of freedom, the slots of the cells incident
// to it, in cell order: the reference's two-stage gather, race-free without
// atomics (matfree.rs:20-33, 98-131).
#pragma once

#include "fq_element_kernel.cuh"
#include "fq_internal.h"

namespace fq {

// The incidence of the grade-`grade` faces: for every degree of freedom (the
// relative numbering under FQ_RELATIVE; boundary faces dropped), the slots
// local face * ncells + cell of the cells containing it, in cell order. Built
// by one stable radix sort of the cell -> face table; row_ptr has ndofs + 1
// entries.
fq_status build_face_incidence(fq_ctx* ctx, fq_mesh* m, int grade, int bc, DevBuf& row_ptr, DevBuf& row_src);

// y[r] = sum over the incidence row r of contrib[slot], in cell order, summed in
// float-float and rounded once (the second stage of the two-stage gather).
void launch_gather_rows(const int32_t* rp, const int32_t* src, const df64* contrib, double* y, int64_t nrows,
                        const int* done, cudaStream_t st);

int64_t ndofs_of(const fq_mesh* m, int grade, int bc);

struct ElemopArgs {
  int64_t ncells = 0;
  const double* lengths = nullptr;     // [N1]
  const int32_t* cell_edges = nullptr; // [C(n+1,2)][ncells]
  const int32_t* col_faces = nullptr;  // [LC][ncells] kidx of the trial faces
  const int32_t* col_map = nullptr;    // relative complex: kidx -> column, -1 on the boundary; null: identity
  const double* x = nullptr;           // [ncols]; null: the diagonal entries instead of A_K P_K x
  df64* contrib = nullptr;             // [LR][ncells]
  const int* done = nullptr;           // a converged Krylov loop: return at once
  int* status = nullptr;               // bit 0: a singular or non-finite cell metric
  int grid = 0;
};

// Local shape of a pairing: test (row) and trial (column) grades and counts.
template <int N, int K, int KIND>
struct PairingShape {
  static constexpr int row_grade = (KIND == EK_DIF_TEST || KIND == EK_DIF_BOTH) ? K - 1 : K;
  static constexpr int col_grade = (KIND == EK_DIF_TRIAL || KIND == EK_DIF_BOTH) ? K - 1 : K;
  static constexpr int LR = cbinom(N + 1, row_grade + 1);
  static constexpr int LC = cbinom(N + 1, col_grade + 1);
  static constexpr bool sym = KIND == EK_MASS || KIND == EK_DIF_BOTH;
  static constexpr int nent = sym ? (LR * (LR + 1)) / 2 : LR * LC;
  // entry numbering of element_entries: packed upper triangle, or row-major
  static constexpr int entry(int i, int j) { return sym ? packed_index(i < j ? i : j, i < j ? j : i, LR) : i * LC + j; }
};

template <int N, int K, int KIND>
__global__ void __launch_bounds__(128) elemop_cell_kernel(ElemopArgs a) {
  using S = PairingShape<N, K, KIND>;
  constexpr int NE = cbinom(N + 1, 2);
  const int64_t nc = a.ncells;
  if (a.done && *a.done) return;
  for (int64_t cell = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; cell < nc;
       cell += int64_t(gridDim.x) * blockDim.x) {
    double s[NE > 0 ? NE : 1];
#pragma unroll
    for (int e = 0; e < NE; ++e) s[e] = __ldg(a.lengths + __ldg(a.cell_edges + int64_t(e) * nc + cell));
    Bary<N, df64> B;
    bool bad = false;
    const df64 vol = cell_bary<N, df64>(s, B, bad);
    if (bad) atomicOr(a.status, 1);
    df64 A[S::nent];
    element_entries<N, K, KIND, df64>(B, vol, 0.0, [&](int e, df64 v) { A[e] = v; });
    if (a.x) {
      df64 xl[S::LC];
      static_for<S::LC>([&](auto J) {
        constexpr int j = decltype(J)::value;
        int idx = __ldg(a.col_faces + int64_t(j) * nc + cell);
        if (a.col_map) idx = __ldg(a.col_map + idx);
        xl[j] = idx >= 0 ? df64(__ldg(a.x + idx)) : df64(0);
      });
      static_for<S::LR>([&](auto I) {
        constexpr int i = decltype(I)::value;
        df64 acc(0);
        static_for<S::LC>([&](auto J) {
          constexpr int j = decltype(J)::value;
          acc += A[S::entry(i, j)] * xl[j];
        });
        a.contrib[int64_t(i) * nc + cell] = acc;
      });
    } else if constexpr (S::sym) {
      static_for<S::LR>([&](auto I) {
        constexpr int i = decltype(I)::value;
        a.contrib[int64_t(i) * nc + cell] = A[S::entry(i, i)];
      });
    }
  }
}

template <int N, int K, int KIND>
int launch_elemop_one(const ElemopArgs& a, cudaStream_t st) {
  constexpr int threads = 128;
  if (a.ncells <= 0) return 0;
  const int64_t need = (a.ncells + threads - 1) / threads;
  const unsigned blocks = unsigned(a.grid > 0 ? (need < a.grid ? need : a.grid) : need);
  elemop_cell_kernel<N, K, KIND><<<blocks, threads, 0, st>>>(a);
  return 0;
}

// The pairings whose kinds are in KINDS (bit EK_x), at every grade of
// dimension N; -1 when (K, kind) is not among them. The kinds of one dimension
// may be split over several translation units to keep each compile short.
template <int N, unsigned KINDS>
int launch_elemop_cells_sel(int K, int kind, const ElemopArgs& a, cudaStream_t st) {
  int r = -1;
  static_for<N + 1>([&](auto KC) {
    constexpr int k = decltype(KC)::value;
    if (k != K) return;
    if constexpr (bool(KINDS & (1u << EK_MASS)))
      if (kind == EK_MASS) r = launch_elemop_one<N, k, EK_MASS>(a, st);
    if constexpr (k >= 1) {
      if constexpr (bool(KINDS & (1u << EK_DIF_TRIAL)))
        if (kind == EK_DIF_TRIAL) r = launch_elemop_one<N, k, EK_DIF_TRIAL>(a, st);
      if constexpr (bool(KINDS & (1u << EK_DIF_TEST)))
        if (kind == EK_DIF_TEST) r = launch_elemop_one<N, k, EK_DIF_TEST>(a, st);
      if constexpr (bool(KINDS & (1u << EK_DIF_BOTH)))
        if (kind == EK_DIF_BOTH) r = launch_elemop_one<N, k, EK_DIF_BOTH>(a, st);
    }
  });
  // dif_both(N+1) has no entries; callers never launch it
  return r;
}

// The four pairings at every grade of dimension N (one translation unit per N).
template <int N>
int launch_elemop_cells(int K, int kind, const ElemopArgs& a, cudaStream_t st) {
  return launch_elemop_cells_sel<N, 0xFu>(K, kind, a, st);
}

}  // namespace fq
