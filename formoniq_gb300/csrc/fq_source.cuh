// The Galerkin load of a source form on the GPU: SourceForm::element
// (formoniq/src/operators.rs:598-635) summed by assemble_vector
// (formoniq/src/galerkin.rs:279-312).
//
//   l_s = integral_K <f, W_s>_{Lambda^k g^{-1}} vol = vol sum_q w_q <f(x_q), W_s(x_q)>
//
// with the Grundmann-Moeller rule of the requested degree on the cell, weights
// normalised to sum 1 (CellQuadrature::integrate, operators.rs:246-261), and
// W_s = k! sum_p (-1)^p lambda_{s_p} dlambda_{s\s_p} (derham/src/interpolate/form.rs:108-112).
//
// The source's values come in the cell's reference frame (derham/src/section.rs:50-66):
// components on dxi^J, xi_j = lambda_{j+1}, J the colex k-subsets of {0..n-1}.
// Since dxi^J = dlambda_{J+1}, the pairing is a row of the blade Gramian
// H_k = Lambda^k B the element programs already build,
//   <f, dlambda_t> = sum_J f_J H_k[J+1, t],
// so with the node moments m_v[J] = sum_q w_q lambda_q[v] f_q[J]
//   l_s = vol k! sum_p (-1)^p sum_J H_k[J+1, s\s_p] m_{s_p}[J].
// Each H_k entry is formed once and used for the n+1-k faces s = t + {v}.
//
// A flat ambient form (Pullback::identity, derham/src/section.rs:95-140) is
// pulled back through the cell's affine map: f_J = sum_A w_A det(E[A, J]),
// E = [x_{v_1} - x_{v_0}, ..., x_{v_n} - x_{v_0}]; by linearity the moments are
// taken on the ambient components first and pulled back once per cell.
//
// Layout: the values are cell-major [ncells][nq][ncomp] (what a caller writes
// after evaluating its field at the nodes); a block stages its 128 cells' values
// for a chunk of nodes in shared memory with coalesced streaming loads, then
// every thread reads its own cell's row (odd row stride: no bank conflicts).
// The element vectors go to entry-major slots [local face][cell] and the
// incidence gather of the matrix-free operator sums them per degree of freedom
// in cell order.
#pragma once

#include "fq_element_kernel.cuh"

namespace fq {

constexpr int kSourceThreads = 128;
constexpr int kSourceStageDoubles = 47;  // per thread: 128 x 47 x 8 B = 47 KiB of shared memory

struct SourceArgs {
  int64_t ncells = 0;
  const double* lengths = nullptr;      // [N1]
  const int32_t* cell_edges = nullptr;  // [C(n+1,2)][ncells]
  const int32_t* cell_verts = nullptr;  // [n+1][ncells] vertex kidx (ambient values)
  const int32_t* vertex_ids = nullptr;  // [N0] vertex id of each vertex kidx (ambient values)
  const double* coords = nullptr;       // [vertex id][adim] (ambient values)
  const double* values = nullptr;       // [ncells][nq][ncomp]
  const double* wlam = nullptr;         // [nq][n+1]: w_q lambda_q[v]
  int nq = 0;
  int chunk = 0;   // nodes staged at a time
  int stride = 0;  // doubles per thread row in shared memory (odd)
  df64* contrib = nullptr;  // [C(n+1,k+1)][ncells]
  int* status = nullptr;    // bit 0: a singular or non-finite cell metric
  int grid = 0;
};

// det of E[rows AM][cols JM] (J x J, J <= 4), index sets compile-time.
template <int J, unsigned AM, unsigned JM, int ADIM, int N>
FQ_HDI double edge_minor(const double (&E)[ADIM][N]) {
  if constexpr (J == 0) {
    return 1.0;
  } else {
    constexpr MaskList<AM, J> r{};
    constexpr MaskList<JM, J> c{};
    if constexpr (J == 1) {
      return E[r.v[0]][c.v[0]];
    } else if constexpr (J == 2) {
      return E[r.v[0]][c.v[0]] * E[r.v[1]][c.v[1]] - E[r.v[0]][c.v[1]] * E[r.v[1]][c.v[0]];
    } else if constexpr (J == 3) {
      const double m0 = E[r.v[1]][c.v[1]] * E[r.v[2]][c.v[2]] - E[r.v[1]][c.v[2]] * E[r.v[2]][c.v[1]];
      const double m1 = E[r.v[1]][c.v[0]] * E[r.v[2]][c.v[2]] - E[r.v[1]][c.v[2]] * E[r.v[2]][c.v[0]];
      const double m2 = E[r.v[1]][c.v[0]] * E[r.v[2]][c.v[1]] - E[r.v[1]][c.v[1]] * E[r.v[2]][c.v[0]];
      return E[r.v[0]][c.v[0]] * m0 - E[r.v[0]][c.v[1]] * m1 + E[r.v[0]][c.v[2]] * m2;
    } else {
      static_assert(J == 4, "pullback above grade 4");
      // Laplace expansion along the first two rows
      const double s0 = E[r.v[0]][c.v[0]] * E[r.v[1]][c.v[1]] - E[r.v[1]][c.v[0]] * E[r.v[0]][c.v[1]];
      const double s1 = E[r.v[0]][c.v[0]] * E[r.v[1]][c.v[2]] - E[r.v[1]][c.v[0]] * E[r.v[0]][c.v[2]];
      const double s2 = E[r.v[0]][c.v[0]] * E[r.v[1]][c.v[3]] - E[r.v[1]][c.v[0]] * E[r.v[0]][c.v[3]];
      const double s3 = E[r.v[0]][c.v[1]] * E[r.v[1]][c.v[2]] - E[r.v[1]][c.v[1]] * E[r.v[0]][c.v[2]];
      const double s4 = E[r.v[0]][c.v[1]] * E[r.v[1]][c.v[3]] - E[r.v[1]][c.v[1]] * E[r.v[0]][c.v[3]];
      const double s5 = E[r.v[0]][c.v[2]] * E[r.v[1]][c.v[3]] - E[r.v[1]][c.v[2]] * E[r.v[0]][c.v[3]];
      const double k5 = E[r.v[2]][c.v[2]] * E[r.v[3]][c.v[3]] - E[r.v[3]][c.v[2]] * E[r.v[2]][c.v[3]];
      const double k4 = E[r.v[2]][c.v[1]] * E[r.v[3]][c.v[3]] - E[r.v[3]][c.v[1]] * E[r.v[2]][c.v[3]];
      const double k3 = E[r.v[2]][c.v[1]] * E[r.v[3]][c.v[2]] - E[r.v[3]][c.v[1]] * E[r.v[2]][c.v[2]];
      const double k2 = E[r.v[2]][c.v[0]] * E[r.v[3]][c.v[3]] - E[r.v[3]][c.v[0]] * E[r.v[2]][c.v[3]];
      const double k1 = E[r.v[2]][c.v[0]] * E[r.v[3]][c.v[2]] - E[r.v[3]][c.v[0]] * E[r.v[2]][c.v[2]];
      const double k0 = E[r.v[2]][c.v[0]] * E[r.v[3]][c.v[1]] - E[r.v[3]][c.v[0]] * E[r.v[2]][c.v[1]];
      return s0 * k5 - s1 * k4 + s2 * k3 + s3 * k2 - s4 * k1 + s5 * k0;
    }
  }
}

// One thread per cell; ADIM = 0: values in the cell's reference frame, else
// ambient components of a flat form on dx^A (A colex k-subsets of ADIM axes).
template <int N, int K, int ADIM>
__global__ void __launch_bounds__(kSourceThreads) source_cell_kernel(SourceArgs a) {
  constexpr int NE = cbinom(N + 1, 2);
  constexpr int C = cbinom(N, K);                   // reference-frame components
  constexpr int CIN = ADIM > 0 ? cbinom(ADIM, K) : C;  // components of the input values
  constexpr int LF = cbinom(N + 1, K + 1);          // local faces of grade K
  constexpr int LT = cbinom(N + 1, K);              // K-subsets of the cell's vertices
  extern __shared__ double stage[];
  const int64_t nc = a.ncells;
  const int nq = a.nq;
  const int64_t per = int64_t(nq) * CIN;
  for (int64_t base = int64_t(blockIdx.x) * blockDim.x; base < nc; base += int64_t(gridDim.x) * blockDim.x) {
    const int nb = int(nc - base < int64_t(blockDim.x) ? nc - base : int64_t(blockDim.x));
    const int64_t cell = base + threadIdx.x;
    // moments of the input components: mi[v][A] = sum_q w_q lambda_q[v] f_q[A]
    df64 mi[N + 1][CIN];
#pragma unroll
    for (int v = 0; v <= N; ++v)
#pragma unroll
      for (int c = 0; c < CIN; ++c) mi[v][c] = df64(0);
    for (int q0 = 0; q0 < nq; q0 += a.chunk) {
      const int qn = nq - q0 < a.chunk ? nq - q0 : a.chunk;
      const int run = qn * CIN;
      __syncthreads();  // the previous chunk is consumed
      for (int i = threadIdx.x; i < nb * run; i += blockDim.x) {
        const int c = i / run;
        stage[c * a.stride + (i - c * run)] = __ldcs(a.values + (base + c) * per + int64_t(q0) * CIN + (i - c * run));
      }
      __syncthreads();
      if (cell < nc) {
        const double* row = stage + threadIdx.x * a.stride;
        for (int q = 0; q < qn; ++q) {
          df64 f[CIN];
#pragma unroll
          for (int c = 0; c < CIN; ++c) f[c] = df64(row[q * CIN + c]);
#pragma unroll
          for (int v = 0; v <= N; ++v) {
            const df64 wl(__ldg(a.wlam + (q0 + q) * (N + 1) + v));
#pragma unroll
            for (int c = 0; c < CIN; ++c) mi[v][c] = mi[v][c] + wl * f[c];
          }
        }
      }
    }
    if (cell >= nc) continue;  // only in the block's last pass: no barrier follows
    // reference-frame moments
    df64 m[N + 1][C];
    if constexpr (ADIM > 0) {
      double E[ADIM][N];
      {
        const int32_t v0 = __ldg(a.vertex_ids + __ldg(a.cell_verts + cell));
        double x0[ADIM];
#pragma unroll
        for (int d = 0; d < ADIM; ++d) x0[d] = __ldg(a.coords + int64_t(v0) * ADIM + d);
#pragma unroll
        for (int j = 0; j < N; ++j) {
          const int32_t vj = __ldg(a.vertex_ids + __ldg(a.cell_verts + int64_t(j + 1) * nc + cell));
#pragma unroll
          for (int d = 0; d < ADIM; ++d) E[d][j] = __ldg(a.coords + int64_t(vj) * ADIM + d) - x0[d];
        }
      }
#pragma unroll
      for (int v = 0; v <= N; ++v)
#pragma unroll
        for (int j = 0; j < C; ++j) m[v][j] = df64(0);
      static_for<C>([&](auto JC) {
        constexpr int j = decltype(JC)::value;
        constexpr unsigned jm = Tab<N, K>::v.mask[j];
        static_for<CIN>([&](auto AC) {
          constexpr int ai = decltype(AC)::value;
          constexpr unsigned am = Tab<ADIM, K>::v.mask[ai];
          const df64 d(edge_minor<K, am, jm, ADIM, N>(E));
#pragma unroll
          for (int v = 0; v <= N; ++v) m[v][j] = m[v][j] + d * mi[v][ai];
        });
      });
    } else {
#pragma unroll
      for (int v = 0; v <= N; ++v)
#pragma unroll
        for (int j = 0; j < C; ++j) m[v][j] = mi[v][j];
    }
    // the cell's metric and barycentric Gramian
    double s[NE > 0 ? NE : 1];
#pragma unroll
    for (int e = 0; e < NE; ++e) s[e] = __ldg(a.lengths + __ldg(a.cell_edges + int64_t(e) * nc + cell));
    Bary<N, df64> B;
    bool bad = false;
    const df64 vol = cell_bary<N, df64>(s, B, bad);
    if (bad) atomicOr(a.status, 1);
    df64 acc[LF];
#pragma unroll
    for (int i = 0; i < LF; ++i) acc[i] = df64(0);
    static_for<LT>([&](auto TC) {
      constexpr int t = decltype(TC)::value;
      constexpr unsigned tm = Tab<N + 1, K>::v.mask[t];
      static_for<C>([&](auto JC) {
        constexpr int j = decltype(JC)::value;
        constexpr int r = mask_rank(Tab<N, K>::v.mask[j] << 1);  // J + 1 among the k-subsets of {0..n}
        const df64 h = blade_entry<N, K, r, t>(B);
        static_for<N + 1>([&](auto VC) {
          constexpr int v = decltype(VC)::value;
          if constexpr (!(tm & (1u << v))) {
            constexpr unsigned sm = tm | (1u << v);
            constexpr int si = mask_rank(sm);
            if constexpr (pos_in(sm, v) % 2 == 0)
              acc[si] = acc[si] + h * m[v][j];
            else
              acc[si] = acc[si] - h * m[v][j];
          }
        });
      });
    });
    const df64 scale = vol * df64(double(cfact(K)));
#pragma unroll
    for (int i = 0; i < LF; ++i) a.contrib[int64_t(i) * nc + cell] = acc[i] * scale;
  }
}

template <int N, int K, int ADIM>
void launch_source_one(const SourceArgs& a, cudaStream_t st) {
  const int64_t need = (a.ncells + kSourceThreads - 1) / kSourceThreads;
  const unsigned blocks = unsigned(a.grid > 0 && need > a.grid ? a.grid : need);
  const size_t smem = size_t(kSourceThreads) * a.stride * sizeof(double);
  source_cell_kernel<N, K, ADIM><<<blocks, kSourceThreads, smem, st>>>(a);
}

// Every grade and ambient dimension of cell dimension N (one translation unit
// per N). Returns -1 for an unsupported (K, adim).
template <int N>
int launch_source_cells(int K, int adim, const SourceArgs& a, cudaStream_t st) {
  int r = -1;
  if (a.ncells <= 0) return 0;
  static_for<N + 1>([&](auto KC) {
    constexpr int k = decltype(KC)::value;
    if (k != K) return;
    if (adim == 0) {
      launch_source_one<N, k, 0>(a, st);
      r = 0;
    }
    static_for<5>([&](auto DC) {
      constexpr int d = decltype(DC)::value;
      if constexpr (d >= N && d >= 1) {
        if (adim == d) {
          launch_source_one<N, k, d>(a, st);
          r = 0;
        }
      }
    });
  });
  return r;
}

}  // namespace fq
