// Compile-time combinatorics of the reference cell: colex-ordered vertex subsets
// of the n-simplex, their ranks and their signed deletions.
//
// Reference semantics: multiindex Combination (colex rank sum_i C(c_i, i+1)),
// Combination::deletions (multiindex/src/monotone.rs:617-637: position p gives
// sign (-1)^p, the deleted vertex and the remaining subset), and
// unit_subsimps (simplicial/src/topology/simplex.rs:184-197).
//
// Everything here is constexpr so that, inside fully unrolled device loops,
// subset vertices, ranks and deletion signs fold to immediates: no table loads
// and no multiplications by +-1 reach the FP pipes.
#pragma once

// FQ_HD marks code that both the device kernels and host-side checks compile;
// FQ_HDI is the same for small helpers that must inline.
#if defined(__CUDACC__)
#define FQ_HD __host__ __device__
#define FQ_HDI __host__ __device__ __forceinline__
#else
#define FQ_HD
#define FQ_HDI inline
#endif

namespace fq {

FQ_HD constexpr int cbinom(int n, int k) {
  if (k < 0 || n < 0 || k > n) return 0;
  int r = 1;
  for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
  return r;
}

FQ_HD constexpr int cfact(int n) {
  int r = 1;
  for (int i = 2; i <= n; ++i) r *= i;
  return r;
}

FQ_HD constexpr int cpopcount(unsigned x) {
  int c = 0;
  while (x) {
    c += int(x & 1u);
    x >>= 1;
  }
  return c;
}

// Colex rank of a strictly increasing tuple.
FQ_HD constexpr int colex_rank(const int* c, int k) {
  int r = 0;
  for (int i = 0; i < k; ++i) r += cbinom(c[i], i + 1);
  return r;
}

// The S-subsets of {0..M-1} in colex order (= increasing bitmask order).
template <int M, int S>
struct Subsets {
  static constexpr int count = cbinom(M, S);
  static constexpr int cnt1 = count > 0 ? count : 1;
  static constexpr int s1 = S > 0 ? S : 1;
  int v[cnt1][s1];
  unsigned mask[cnt1];
  FQ_HD constexpr Subsets() : v{}, mask{} {
    int idx = 0;
    if (S >= 0 && S <= M) {
      for (unsigned m = 0; m < (1u << M); ++m) {
        if (cpopcount(m) != S) continue;
        int p = 0;
        for (int b = 0; b < M; ++b)
          if (m & (1u << b)) v[idx][p++] = b;
        mask[idx] = m;
        ++idx;
      }
    }
  }
};

// Rank among S-subsets of {0..M-1} of the subset given by a bitmask.
FQ_HD constexpr int mask_rank(unsigned m) {
  int r = 0, i = 0;
  for (int b = 0; b < 32; ++b)
    if (m & (1u << b)) {
      r += cbinom(b, i + 1);
      ++i;
    }
  return r;
}

// Position of vertex v inside the subset `m` (number of members below v).
FQ_HD constexpr int pos_in(unsigned m, int v) { return cpopcount(m & ((1u << v) - 1u)); }

// Packed upper-triangular index of (i, j), i <= j, in an L x L symmetric matrix.
FQ_HD constexpr int packed_index(int i, int j, int L) { return i * L - (i * (i - 1)) / 2 + (j - i); }

}  // namespace fq
