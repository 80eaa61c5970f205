// Per-cell geometry and Whitney element matrices, device side.
//
// Kernel (a): the Regge metric of a cell from its signed squared edge lengths,
// with inverse and determinant, always in FP64:
//   G_ii = s_{0,i+1},  G_ij = (s_{0,i+1} + s_{0,j+1} - s_{i+1,j+1}) / 2
//   (regge/src/lengths/simplex.rs:308-326), vol = sqrt(|det G|)/n!
//   (regge/src/lib.rs:26-28), G^{-1} (metric/src/lib.rs:250-257).
//
// Kernel (b): the element matrices of the four Whitney pairings
// (formoniq/src/operators.rs:58-212). They are written here through the Gramian
// of the barycentric differentials,
//   B = L G^{-1} L^T,   L = unit_difbarys (simplicial/src/atlas.rs:174-182),
// whose j-th compound H_j = Lambda^j B (entries: j x j minors of B on colex
// vertex subsets) equals the reference's blade Gramian D Lambda^j(G^{-1}) D^T
// (operators.rs:90-91) by Cauchy-Binet. With Q = (I + 11^T)/((n+1)(n+2))
// (atlas.rs:198-204) and the deletion formula W_s = k! sum_p (-1)^p
// lambda_{s_p} dlambda_{s\s_p} (derham/src/interpolate/form.rs:186-232):
//   mass_k[s,t]      = vol (k!)^2 sum_{p,q} (-1)^{p+q} H_k[s\s_p, t\t_q] Q[s_p,t_q]
//   dif_both_k[r,r'] = vol (k!)^2 H_k[r, r']                (dW_r = k! dlambda_r)
//   dif_test_k[r,t]  = vol/(n+1) (k!)^2 sum_q (-1)^q H_k[t\t_q, r]
//   dif_trial_k      = dif_test_k^T
// which are the reference's sandwiches d M d^T and d M evaluated in closed form.
#pragma once

#include <cstdint>
#include <type_traits>
#include <utility>

#include "fq_combinatorics.cuh"
#include "fq_df64.cuh"

namespace fq {

template <typename F, int... I>
FQ_HDI void static_for_impl(F&& f, std::integer_sequence<int, I...>) {
  (f(std::integral_constant<int, I>{}), ...);
}
template <int N, typename F>
FQ_HDI void static_for(F&& f) {
  static_for_impl(f, std::make_integer_sequence<int, N>{});
}

template <int M, int S>
struct Tab {
  static constexpr Subsets<M, S> v{};
};

// Local edge index of vertices (a, b), a < b: colex rank C(b,2) + a
// (simplicial/src/topology/simplex.rs:209-211).
FQ_HD constexpr int edge_index(int a, int b) { return (b * (b - 1)) / 2 + a; }

// ---------------------------------------------------------------------------
// Arithmetic that differs per type: exact doubling, reciprocal
// ---------------------------------------------------------------------------
template <typename T>
FQ_HDI T twice(T x) {
  return x + x;
}
FQ_HDI df64 twice(df64 x) { return df64(f_mul(x.hi, 2.f), f_mul(x.lo, 2.f)); }  // exact
template <typename T>
FQ_HDI T halve(T x) {
  return x * T(0.5);
}
FQ_HDI df64 halve(df64 x) { return df64(f_mul(x.hi, 0.5f), f_mul(x.lo, 0.5f)); }  // exact (no underflow here)
template <typename T>
FQ_HDI T recip(T x) {
  return T(1) / x;
}
// Float-float reciprocal: the FP32 reciprocal of the leading part refined by one
// Newton-Raphson step r = q + q (1 - a q) carried out in float-float (the
// division of Bailey's double-double arithmetic); the step squares the 2^-24
// error of q to about 2^-48.
FQ_HDI df64 recip(df64 a) {
  const df64 q(1.0f / a.hi, 0.f);
  const df64 e = df64(1.f, 0.f) - a * q;
  return q + q * e;
}

// ---------------------------------------------------------------------------
// kernel (a): Gram matrix, determinant, inverse (FP64)
// ---------------------------------------------------------------------------
template <int N>
struct Metric {
  double ginv[N > 0 ? N : 1][N > 0 ? N : 1];
  double det;
};

template <int N>
FQ_HDI void regge_metric(const double* s, double (&g)[N > 0 ? N : 1][N > 0 ? N : 1]) {
#pragma unroll
  for (int i = 0; i < N; ++i) g[i][i] = s[edge_index(0, i + 1)];
#pragma unroll
  for (int i = 0; i < N; ++i)
#pragma unroll
    for (int j = i + 1; j < N; ++j) {
      const double v = 0.5 * (s[edge_index(0, i + 1)] + s[edge_index(0, j + 1)] - s[edge_index(i + 1, j + 1)]);
      g[i][j] = v;
      g[j][i] = v;
    }
}

// Symmetric inverse by cofactors (N <= 3) and by the 2x2-minor Laplace
// expansion (N = 4). Returns det.
template <int N>
FQ_HDI double sym_inverse(const double (&a)[N > 0 ? N : 1][N > 0 ? N : 1],
                                              double (&inv)[N > 0 ? N : 1][N > 0 ? N : 1]) {
  if constexpr (N == 0) {
    return 1.0;
  } else if constexpr (N == 1) {
    inv[0][0] = 1.0 / a[0][0];
    return a[0][0];
  } else if constexpr (N == 2) {
    const double det = a[0][0] * a[1][1] - a[0][1] * a[0][1];
    const double r = 1.0 / det;
    inv[0][0] = a[1][1] * r;
    inv[1][1] = a[0][0] * r;
    inv[0][1] = inv[1][0] = -a[0][1] * r;
    return det;
  } else if constexpr (N == 3) {
    const double c00 = a[1][1] * a[2][2] - a[1][2] * a[1][2];
    const double c01 = a[0][2] * a[1][2] - a[0][1] * a[2][2];
    const double c02 = a[0][1] * a[1][2] - a[0][2] * a[1][1];
    const double c11 = a[0][0] * a[2][2] - a[0][2] * a[0][2];
    const double c12 = a[0][1] * a[0][2] - a[0][0] * a[1][2];
    const double c22 = a[0][0] * a[1][1] - a[0][1] * a[0][1];
    const double det = a[0][0] * c00 + a[0][1] * c01 + a[0][2] * c02;
    const double r = 1.0 / det;
    inv[0][0] = c00 * r;
    inv[1][1] = c11 * r;
    inv[2][2] = c22 * r;
    inv[0][1] = inv[1][0] = c01 * r;
    inv[0][2] = inv[2][0] = c02 * r;
    inv[1][2] = inv[2][1] = c12 * r;
    return det;
  } else {
    static_assert(N == 4, "dimension above 4");
    const double s0 = a[0][0] * a[1][1] - a[1][0] * a[0][1];
    const double s1 = a[0][0] * a[1][2] - a[1][0] * a[0][2];
    const double s2 = a[0][0] * a[1][3] - a[1][0] * a[0][3];
    const double s3 = a[0][1] * a[1][2] - a[1][1] * a[0][2];
    const double s4 = a[0][1] * a[1][3] - a[1][1] * a[0][3];
    const double s5 = a[0][2] * a[1][3] - a[1][2] * a[0][3];
    const double c5 = a[2][2] * a[3][3] - a[3][2] * a[2][3];
    const double c4 = a[2][1] * a[3][3] - a[3][1] * a[2][3];
    const double c3 = a[2][1] * a[3][2] - a[3][1] * a[2][2];
    const double c2 = a[2][0] * a[3][3] - a[3][0] * a[2][3];
    const double c1 = a[2][0] * a[3][2] - a[3][0] * a[2][2];
    const double c0 = a[2][0] * a[3][1] - a[3][0] * a[2][1];
    const double det = s0 * c5 - s1 * c4 + s2 * c3 + s3 * c2 - s4 * c1 + s5 * c0;
    const double r = 1.0 / det;
    inv[0][0] = (a[1][1] * c5 - a[1][2] * c4 + a[1][3] * c3) * r;
    inv[0][1] = (-a[0][1] * c5 + a[0][2] * c4 - a[0][3] * c3) * r;
    inv[0][2] = (a[3][1] * s5 - a[3][2] * s4 + a[3][3] * s3) * r;
    inv[0][3] = (-a[2][1] * s5 + a[2][2] * s4 - a[2][3] * s3) * r;
    inv[1][1] = (a[0][0] * c5 - a[0][2] * c2 + a[0][3] * c1) * r;
    inv[1][2] = (-a[3][0] * s5 + a[3][2] * s2 - a[3][3] * s1) * r;
    inv[1][3] = (a[2][0] * s5 - a[2][2] * s2 + a[2][3] * s1) * r;
    inv[2][2] = (a[3][0] * s4 - a[3][1] * s2 + a[3][3] * s0) * r;
    inv[2][3] = (-a[2][0] * s4 + a[2][1] * s2 - a[2][3] * s0) * r;
    inv[3][3] = (a[2][0] * s3 - a[2][1] * s1 + a[2][2] * s0) * r;
    inv[1][0] = inv[0][1];
    inv[2][0] = inv[0][2];
    inv[3][0] = inv[0][3];
    inv[2][1] = inv[1][2];
    inv[3][1] = inv[1][3];
    inv[3][2] = inv[2][3];
    return det;
  }
}

// The same three steps in an arithmetic type T (float-float in FQ_FP64, where
// the FP64 pipe would otherwise bound the kernel): metric from lengths, inverse
// by cofactors with det, and below the barycentric Gramian.
template <int N, typename T>
FQ_HDI void regge_metric_t(const T* s, T (&g)[N > 0 ? N : 1][N > 0 ? N : 1]) {
#pragma unroll
  for (int i = 0; i < N; ++i) g[i][i] = s[edge_index(0, i + 1)];
#pragma unroll
  for (int i = 0; i < N; ++i)
#pragma unroll
    for (int j = i + 1; j < N; ++j) {
      const T v = halve(s[edge_index(0, i + 1)] + s[edge_index(0, j + 1)] - s[edge_index(i + 1, j + 1)]);
      g[i][j] = v;
      g[j][i] = v;
    }
}

template <int N, typename T>
FQ_HDI T sym_inverse_t(const T (&a)[N > 0 ? N : 1][N > 0 ? N : 1], T (&inv)[N > 0 ? N : 1][N > 0 ? N : 1]) {
  if constexpr (N == 0) {
    return T(1);
  } else if constexpr (N == 1) {
    inv[0][0] = recip(a[0][0]);
    return a[0][0];
  } else if constexpr (N == 2) {
    const T det = a[0][0] * a[1][1] - a[0][1] * a[0][1];
    const T r = recip(det);
    inv[0][0] = a[1][1] * r;
    inv[1][1] = a[0][0] * r;
    inv[0][1] = inv[1][0] = -(a[0][1] * r);
    return det;
  } else if constexpr (N == 3) {
    const T c00 = a[1][1] * a[2][2] - a[1][2] * a[1][2];
    const T c01 = a[0][2] * a[1][2] - a[0][1] * a[2][2];
    const T c02 = a[0][1] * a[1][2] - a[0][2] * a[1][1];
    const T c11 = a[0][0] * a[2][2] - a[0][2] * a[0][2];
    const T c12 = a[0][1] * a[0][2] - a[0][0] * a[1][2];
    const T c22 = a[0][0] * a[1][1] - a[0][1] * a[0][1];
    const T det = a[0][0] * c00 + a[0][1] * c01 + a[0][2] * c02;
    const T r = recip(det);
    inv[0][0] = c00 * r;
    inv[1][1] = c11 * r;
    inv[2][2] = c22 * r;
    inv[0][1] = inv[1][0] = c01 * r;
    inv[0][2] = inv[2][0] = c02 * r;
    inv[1][2] = inv[2][1] = c12 * r;
    return det;
  } else {
    static_assert(N == 4, "dimension above 4");
    const T s0 = a[0][0] * a[1][1] - a[1][0] * a[0][1];
    const T s1 = a[0][0] * a[1][2] - a[1][0] * a[0][2];
    const T s2 = a[0][0] * a[1][3] - a[1][0] * a[0][3];
    const T s3 = a[0][1] * a[1][2] - a[1][1] * a[0][2];
    const T s4 = a[0][1] * a[1][3] - a[1][1] * a[0][3];
    const T s5 = a[0][2] * a[1][3] - a[1][2] * a[0][3];
    const T c5 = a[2][2] * a[3][3] - a[3][2] * a[2][3];
    const T c4 = a[2][1] * a[3][3] - a[3][1] * a[2][3];
    const T c3 = a[2][1] * a[3][2] - a[3][1] * a[2][2];
    const T c2 = a[2][0] * a[3][3] - a[3][0] * a[2][3];
    const T c1 = a[2][0] * a[3][2] - a[3][0] * a[2][2];
    const T c0 = a[2][0] * a[3][1] - a[3][0] * a[2][1];
    const T det = s0 * c5 - s1 * c4 + s2 * c3 + s3 * c2 - s4 * c1 + s5 * c0;
    const T r = recip(det);
    inv[0][0] = (a[1][1] * c5 - a[1][2] * c4 + a[1][3] * c3) * r;
    inv[0][1] = (a[0][2] * c4 - a[0][1] * c5 - a[0][3] * c3) * r;
    inv[0][2] = (a[3][1] * s5 - a[3][2] * s4 + a[3][3] * s3) * r;
    inv[0][3] = (a[2][2] * s4 - a[2][1] * s5 - a[2][3] * s3) * r;
    inv[1][1] = (a[0][0] * c5 - a[0][2] * c2 + a[0][3] * c1) * r;
    inv[1][2] = (a[3][2] * s2 - a[3][0] * s5 - a[3][3] * s1) * r;
    inv[1][3] = (a[2][0] * s5 - a[2][2] * s2 + a[2][3] * s1) * r;
    inv[2][2] = (a[3][0] * s4 - a[3][1] * s2 + a[3][3] * s0) * r;
    inv[2][3] = (a[2][1] * s2 - a[2][0] * s4 - a[2][3] * s0) * r;
    inv[3][3] = (a[2][0] * s3 - a[2][1] * s1 + a[2][2] * s0) * r;
    inv[1][0] = inv[0][1];
    inv[2][0] = inv[0][2];
    inv[3][0] = inv[0][3];
    inv[2][1] = inv[1][2];
    inv[3][1] = inv[1][3];
    inv[3][2] = inv[2][3];
    return det;
  }
}

// ---------------------------------------------------------------------------
// Barycentric Gramian B and its compounds H_j = Lambda^j B
// ---------------------------------------------------------------------------
template <int N, typename T>
struct Bary {
  T b[N + 1][N + 1];
  T rdet;  // 1 / det G
};

// B from an inverse metric already in T (the float-float path).
template <int N, typename T>
FQ_HDI void bary_gramian_t(const T (&ginv)[N > 0 ? N : 1][N > 0 ? N : 1], Bary<N, T>& B) {
  T col[N > 0 ? N : 1];
  T tot = T(0);
#pragma unroll
  for (int j = 0; j < N; ++j) {
    T c = T(0);
#pragma unroll
    for (int i = 0; i < N; ++i) c = c + ginv[i][j];
    col[j] = c;
    tot = tot + c;
  }
  B.b[0][0] = tot;
#pragma unroll
  for (int j = 0; j < N; ++j) {
    B.b[0][j + 1] = -col[j];
    B.b[j + 1][0] = -col[j];
  }
#pragma unroll
  for (int i = 0; i < N; ++i)
#pragma unroll
    for (int j = 0; j < N; ++j) B.b[i + 1][j + 1] = ginv[i][j];
}

// B from an IEEE-double inverse metric: the unique entries are converted to T
// once and the rest is built in T.
template <int N, typename T>
FQ_HDI void bary_gramian(const double (&ginv)[N > 0 ? N : 1][N > 0 ? N : 1], Bary<N, T>& B) {
  T gt[N > 0 ? N : 1][N > 0 ? N : 1];
#pragma unroll
  for (int i = 0; i < N; ++i)
#pragma unroll
    for (int j = i; j < N; ++j) {
      gt[i][j] = T(ginv[i][j]);
      gt[j][i] = gt[i][j];
    }
  bary_gramian_t<N, T>(gt, B);
}

// Sums and differences inside the element programs (2 x 2 minors of B, the
// pullback and sandwich sums). In float-float they use Dekker's add: its error
// is bounded by the magnitudes that formed each entry, and the element
// tolerance is relative to the element matrix, so the accurate add's second
// TwoSum buys nothing here. The metric, its inverse and determinant
// (cell_bary) and the 3 x 3 and 4 x 4 minors of B, where cancellation is the
// rule, keep the accurate add. In FP32 and IEEE FP64 these are the plain
// operations.
template <typename T>
FQ_HDI T eadd(T a, T b) {
  return a + b;
}
template <typename T>
FQ_HDI T esub(T a, T b) {
  return a - b;
}
FQ_HDI df64 eadd(df64 a, df64 b) { return dd_add_dekker(a, b); }
FQ_HDI df64 esub(df64 a, df64 b) { return dd_add_dekker(a, -b); }

// The members of a compile-time vertex mask, increasing.
template <unsigned M, int J>
struct MaskList {
  int v[J > 0 ? J : 1];
  FQ_HD constexpr MaskList() : v{} {
    int p = 0;
    for (int b = 0; b < 32; ++b)
      if (M & (1u << b)) v[p++] = b;
  }
};

// det of B restricted to rows R, cols C (J x J, J <= 4), index sets compile-time.
template <int N, int J, unsigned RM, unsigned CM, typename T>
FQ_HDI T minor_det(const Bary<N, T>& B) {
  if constexpr (J == 0) {
    return T(1);
  } else {
    constexpr MaskList<RM, J> rl{};
    constexpr MaskList<CM, J> cl{};
    if constexpr (J == 1) {
      return B.b[rl.v[0]][cl.v[0]];
    } else if constexpr (J == 2) {
      return esub(B.b[rl.v[0]][cl.v[0]] * B.b[rl.v[1]][cl.v[1]], B.b[rl.v[0]][cl.v[1]] * B.b[rl.v[1]][cl.v[0]]);
    } else if constexpr (J == 3) {
      constexpr int r0 = rl.v[0], r1 = rl.v[1], r2 = rl.v[2];
      constexpr int c0 = cl.v[0], c1 = cl.v[1], c2 = cl.v[2];
      // 3 x 3 minors of the rank-n B cancel strongly on distorted cells: accurate adds
      const T m0 = B.b[r1][c1] * B.b[r2][c2] - B.b[r1][c2] * B.b[r2][c1];
      const T m1 = B.b[r1][c0] * B.b[r2][c2] - B.b[r1][c2] * B.b[r2][c0];
      const T m2 = B.b[r1][c0] * B.b[r2][c1] - B.b[r1][c1] * B.b[r2][c0];
      return B.b[r0][c0] * m0 - B.b[r0][c1] * m1 + B.b[r0][c2] * m2;
    } else {
      static_assert(J == 4, "compound above 4");
      constexpr int r0 = rl.v[0], r1 = rl.v[1], r2 = rl.v[2], r3 = rl.v[3];
      constexpr int c0 = cl.v[0], c1 = cl.v[1], c2 = cl.v[2], c3 = cl.v[3];
      const T s0 = B.b[r0][c0] * B.b[r1][c1] - B.b[r1][c0] * B.b[r0][c1];
      const T s1 = B.b[r0][c0] * B.b[r1][c2] - B.b[r1][c0] * B.b[r0][c2];
      const T s2 = B.b[r0][c0] * B.b[r1][c3] - B.b[r1][c0] * B.b[r0][c3];
      const T s3 = B.b[r0][c1] * B.b[r1][c2] - B.b[r1][c1] * B.b[r0][c2];
      const T s4 = B.b[r0][c1] * B.b[r1][c3] - B.b[r1][c1] * B.b[r0][c3];
      const T s5 = B.b[r0][c2] * B.b[r1][c3] - B.b[r1][c2] * B.b[r0][c3];
      const T k5 = B.b[r2][c2] * B.b[r3][c3] - B.b[r3][c2] * B.b[r2][c3];
      const T k4 = B.b[r2][c1] * B.b[r3][c3] - B.b[r3][c1] * B.b[r2][c3];
      const T k3 = B.b[r2][c1] * B.b[r3][c2] - B.b[r3][c1] * B.b[r2][c2];
      const T k2 = B.b[r2][c0] * B.b[r3][c3] - B.b[r3][c0] * B.b[r2][c3];
      const T k1 = B.b[r2][c0] * B.b[r3][c2] - B.b[r3][c0] * B.b[r2][c2];
      const T k0 = B.b[r2][c0] * B.b[r3][c1] - B.b[r3][c0] * B.b[r2][c1];
      return s0 * k5 - s1 * k4 + s2 * k3 + s3 * k2 - s4 * k1 + s5 * k0;
    }
  }
}

// H_J packed symmetric (colex J-subsets of {0..N}).
template <int N, int J, typename T>
struct Blades {
  static constexpr int L = cbinom(N + 1, J);
  static constexpr int P = (L * (L + 1)) / 2;
  T h[P > 0 ? P : 1];
  template <int I, int K>
  FQ_HDI T at() const {
    if constexpr (I <= K)
      return h[packed_index(I, K, L)];
    else
      return h[packed_index(K, I, L)];
  }
};

// Top compound in closed form: with L the (n+1) x n matrix of the barycentric
// differentials, Cauchy-Binet gives Lambda^n B = (Lambda^n L)(Lambda^n G^{-1})
// (Lambda^n L)^T, where Lambda^n G^{-1} = 1 / det G and the n x n minor of L
// without row v is (-1)^v. So H_n[I][K] = (-1)^(o_I + o_K) / det G, o_I the
// vertex the n-subset I omits -- exact where the n x n minors of the rank-n B
// cancel to roundoff.
template <int N, int I, int K, typename T>
FQ_HDI T top_blade(const Bary<N, T>& B) {
  constexpr unsigned full = (1u << (N + 1)) - 1u;
  constexpr unsigned oi = full & ~Tab<N + 1, N>::v.mask[I];
  constexpr unsigned ok = full & ~Tab<N + 1, N>::v.mask[K];
  constexpr int parity = (cpopcount(oi - 1u) + cpopcount(ok - 1u)) % 2;  // o_I + o_K, from the omitted bits
  if constexpr (parity)
    return -B.rdet;
  else
    return B.rdet;
}

template <int N, int J, typename T>
FQ_HDI void compute_blades(const Bary<N, T>& B, Blades<N, J, T>& H) {
  constexpr int L = Blades<N, J, T>::L;
  if constexpr (J == N && N >= 1) {
    static_for<L>([&](auto I) {
      static_for<L>([&](auto K) {
        constexpr int i = decltype(I)::value, k = decltype(K)::value;
        if constexpr (i <= k) H.h[packed_index(i, k, L)] = top_blade<N, i, k, T>(B);
      });
    });
  } else if constexpr (J > N) {
    // Lambda^{n+1} B = det B = 0: the barycentric differentials sum to zero.
#pragma unroll
    for (int i = 0; i < Blades<N, J, T>::P; ++i) H.h[i] = T(0);
  } else {
    static_for<L>([&](auto I) {
      static_for<L>([&](auto K) {
        if constexpr (int(decltype(I)::value) <= int(decltype(K)::value)) {
          constexpr unsigned rm = Tab<N + 1, J>::v.mask[decltype(I)::value];
          constexpr unsigned cm = Tab<N + 1, J>::v.mask[decltype(K)::value];
          H.h[packed_index(decltype(I)::value, decltype(K)::value, L)] = minor_det<N, J, rm, cm, T>(B);
        }
      });
    });
  }
}

// Single H_J entry on the fly (no storage), for blocks read once.
template <int N, int J, int I, int K, typename T>
FQ_HDI T blade_entry(const Bary<N, T>& B) {
  if constexpr (J > N) {
    return T(0);
  } else if constexpr (J == N && N >= 1) {
    return top_blade<N, I, K, T>(B);
  } else {
    constexpr unsigned rm = Tab<N + 1, J>::v.mask[I];
    constexpr unsigned cm = Tab<N + 1, J>::v.mask[K];
    return minor_det<N, J, rm, cm, T>(B);
  }
}

// ---------------------------------------------------------------------------
// Element entries
// ---------------------------------------------------------------------------
// mass_k[s, t] / (vol (k!)^2 / ((n+1)(n+2))): s, t are the I-th and K-th
// (k+1)-subsets of {0..n}.
template <int N, int KG, int I, int K, typename T>
FQ_HDI T mass_sum(const Blades<N, KG, T>& H) {
  constexpr unsigned ms = Tab<N + 1, KG + 1>::v.mask[I];
  constexpr unsigned mt = Tab<N + 1, KG + 1>::v.mask[K];
  T acc = T(0);
  static_for<KG + 1>([&](auto P) {
    constexpr int p = decltype(P)::value;
    constexpr int vs = Tab<N + 1, KG + 1>::v.v[I][p];
    constexpr int ra = mask_rank(ms & ~(1u << vs));
    static_for<KG + 1>([&](auto Q) {
      constexpr int q = decltype(Q)::value;
      constexpr int vt = Tab<N + 1, KG + 1>::v.v[K][q];
      constexpr int rb = mask_rank(mt & ~(1u << vt));
      constexpr int sgn = ((p + q) % 2) ? -1 : 1;
      constexpr int w = (vs == vt) ? 2 : 1;  // (1 + delta) of Q
      constexpr int coef = sgn * w;
      const T h = H.template at<ra, rb>();
      if constexpr (coef == 1)
        acc = eadd(acc, h);
      else if constexpr (coef == -1)
        acc = esub(acc, h);
      else if constexpr (coef == 2)
        acc = eadd(acc, twice(h));
      else
        acc = esub(acc, twice(h));
    });
  });
  return acc;
}

// dif_test_k[r, t] / (vol (k!)^2 / (n+1)): r the R-th k-subset, t the C-th
// (k+1)-subset.
template <int N, int KG, int R, int C, typename T>
FQ_HDI T dif_test_sum(const Blades<N, KG, T>& H) {
  constexpr unsigned mt = Tab<N + 1, KG + 1>::v.mask[C];
  T acc = T(0);
  static_for<KG + 1>([&](auto Q) {
    constexpr int q = decltype(Q)::value;
    constexpr int vt = Tab<N + 1, KG + 1>::v.v[C][q];
    constexpr int rb = mask_rank(mt & ~(1u << vt));
    const T h = H.template at<rb, R>();
    if constexpr (q % 2)
      acc = esub(acc, h);
    else
      acc = eadd(acc, h);
  });
  return acc;
}

}  // namespace fq
