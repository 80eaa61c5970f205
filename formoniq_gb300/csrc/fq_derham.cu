// The de Rham map R: L^2 Lambda^k -> C^k on the GPU (derham/src/project.rs:53-96).
//
// (R w)_s = integral over the k-simplex s of w = (1/k!) sum_q w_q <w(x_q), v_1 ^ ... ^ v_k>,
// v_i = x_{s_i} - x_{s_0}, with the Grundmann-Moeller rule of the requested
// degree on the reference k-simplex (simplicial/src/atlas/quadrature.rs:38-82,
// weights normalised to sum 1). The pairing with the tangent blade is
// sum_I w_I det(V_I) over the k-subsets I of the ambient axes (colex order),
// metric-free as in the reference.
//
// A field is caller code, so it does not cross the C ABI: the library emits the
// quadrature nodes of every k-simplex (fq_derham_nodes), the caller evaluates
// its form there -- on the device, with the same resident layout -- and the
// library reduces the values against the tangent blades (fq_derham_reduce).
#include <algorithm>
#include <cmath>
#include <functional>
#include <vector>

#include "fq_combinatorics.cuh"
#include "fq_internal.h"

namespace fq {

constexpr int kMaxAmbient = 4;

// Grundmann-Moeller rule of index s = degree / 2 on the k-simplex: barycentric
// points (k+1 coordinates each) and weights normalised to sum 1.
void gm_rule(int k, int degree, std::vector<double>& pts, std::vector<double>& w) {
  const int s = degree / 2, d = 2 * s + 1;
  pts.clear();
  w.clear();
  auto fact = [](int n) {
    double f = 1.0;
    for (int i = 2; i <= n; ++i) f *= i;
    return f;
  };
  for (int i = 0; i <= s; ++i) {
    const double den = double(d + k - 2 * i);
    const double wi = (i % 2 ? -1.0 : 1.0) * std::pow(2.0, -2.0 * s) * std::pow(den, d) / (fact(i) * fact(d + k - i));
    // compositions of s - i into k + 1 non-negative parts, in lexicographic order
    std::vector<int> beta(size_t(k + 1), 0);
    const int total = s - i;
    std::vector<std::vector<int>> comps;
    std::function<void(int, int)> rec = [&](int pos, int left) {
      if (pos == k) {
        beta[size_t(k)] = left;
        comps.push_back(beta);
        return;
      }
      for (int b = left; b >= 0; --b) {
        beta[size_t(pos)] = b;
        rec(pos + 1, left - b);
      }
    };
    rec(0, total);
    for (const auto& c : comps) {
      for (int j = 0; j <= k; ++j) pts.push_back((2.0 * c[size_t(j)] + 1.0) / den);
      w.push_back(wi);
    }
  }
  double sum = 0.0;
  for (double x : w) sum += x;
  for (double& x : w) x /= sum;
}

namespace {

struct DerhamArgs {
  int64_t nsimp;
  int k, adim, nq, ncomp;
  const int32_t* verts;    // [nsimp][k+1]
  const double* coords;    // [N0][adim]
  const double* bary;      // [nq][k+1]
  const double* weights;   // [nq]
  const double* values;    // [nsimp][nq][ncomp]
  double* nodes;           // [nsimp][nq][adim]
  double* out;             // [nsimp]
  double inv_kfact;
};

__global__ void derham_nodes_kernel(DerhamArgs a) {
  const int64_t total = a.nsimp * a.nq;
  for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < total; t += int64_t(gridDim.x) * blockDim.x) {
    const int64_t s = t / a.nq;
    const int q = int(t - s * a.nq);
    for (int c = 0; c < a.adim; ++c) {
      double x = 0.0;
      for (int i = 0; i <= a.k; ++i) x += a.bary[q * (a.k + 1) + i] * a.coords[int64_t(a.verts[s * (a.k + 1) + i]) * a.adim + c];
      a.nodes[t * a.adim + c] = x;
    }
  }
}

// det of the k x k matrix m (row-major), k <= 4, Gaussian elimination with
// partial pivoting
__device__ double small_det(double m[kMaxAmbient][kMaxAmbient], int k) {
  double det = 1.0;
  for (int c = 0; c < k; ++c) {
    int p = c;
    for (int r = c + 1; r < k; ++r)
      if (fabs(m[r][c]) > fabs(m[p][c])) p = r;
    if (m[p][c] == 0.0) return 0.0;
    if (p != c) {
      for (int j = 0; j < k; ++j) {
        const double tmp = m[c][j];
        m[c][j] = m[p][j];
        m[p][j] = tmp;
      }
      det = -det;
    }
    det *= m[c][c];
    for (int r = c + 1; r < k; ++r) {
      const double f = m[r][c] / m[c][c];
      for (int j = c; j < k; ++j) m[r][j] -= f * m[c][j];
    }
  }
  return det;
}

__global__ void derham_reduce_kernel(DerhamArgs a) {
  for (int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; s < a.nsimp; s += int64_t(gridDim.x) * blockDim.x) {
    const int k = a.k, n = a.adim;
    double V[kMaxAmbient][kMaxAmbient];  // V[axis][i] = x_{s_{i+1}} - x_{s_0}
    const int64_t v0 = a.verts[s * (k + 1)];
    for (int i = 0; i < k; ++i) {
      const int64_t vi = a.verts[s * (k + 1) + i + 1];
      for (int c = 0; c < n; ++c) V[c][i] = a.coords[vi * n + c] - a.coords[v0 * n + c];
    }
    // tangent blade components det(V_I), I the k-subsets of the axes in colex order
    double blade[6];
    int nb = 0;
    for (int r = 0; r < a.ncomp; ++r) {
      // the r-th k-subset of the axes in colex order (rank = sum_j C(sub_j, j))
      int sub[kMaxAmbient];
      int rem = r;
      for (int j = k; j >= 1; --j) {
        int c = j - 1;
        while (cbinom(c + 1, j) <= rem) ++c;
        sub[j - 1] = c;
        rem -= cbinom(c, j);
      }
      double m[kMaxAmbient][kMaxAmbient];
      for (int i = 0; i < k; ++i)
        for (int j = 0; j < k; ++j) m[i][j] = V[sub[i]][j];
      blade[nb++] = k == 0 ? 1.0 : small_det(m, k);
    }
    double acc = 0.0;
    for (int q = 0; q < a.nq; ++q) {
      double pair = 0.0;
      const double* v = a.values + (s * a.nq + q) * a.ncomp;
      for (int r = 0; r < a.ncomp; ++r) pair += v[r] * blade[r];
      acc += a.weights[q] * pair;
    }
    a.out[s] = acc * a.inv_kfact;
  }
}

int grid_for_n(int64_t n) { return int(std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 16))); }

}  // namespace

static fq_status derham_setup(fq_ctx* ctx, fq_mesh* m, int adim, int grade, int degree, DerhamArgs& a,
                              DevBuf& rule) {
  if (grade < 0 || grade > m->dim) return set_error(ctx, FQ_INVALID_ARG, "grade out of range");
  if (adim < grade || adim < 1 || adim > kMaxAmbient)
    return set_error(ctx, FQ_UNSUPPORTED, "ambient dimension must be in [max(1, grade), 4]");
  if (degree < 0 || degree > 21) return set_error(ctx, FQ_INVALID_ARG, "quadrature degree outside 0..21");
  std::vector<double> pts, w;
  gm_rule(grade, degree, pts, w);
  std::vector<double> blob(pts);
  blob.insert(blob.end(), w.begin(), w.end());
  FQ_TRY(rule.alloc(ctx, blob.size() * 8));
  FQ_CUDA(ctx, cudaMemcpyAsync(rule.p, blob.data(), blob.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
  a.nsimp = m->nsimp[grade];
  a.k = grade;
  a.adim = adim;
  a.nq = int(w.size());
  a.ncomp = cbinom(adim, grade);
  FQ_TRY(device_skeleton(ctx, m, grade, &a.verts));
  a.bary = rule.as<double>();
  a.weights = rule.as<double>() + pts.size();
  double kf = 1.0;
  for (int i = 2; i <= grade; ++i) kf *= i;
  a.inv_kfact = 1.0 / kf;
  return FQ_OK;
}

}  // namespace fq

using namespace fq;

extern "C" {

int fq_derham_npoints(int grade, int degree) {
  if (grade < 0 || grade > 4 || degree < 0 || degree > 21) return 0;
  std::vector<double> p, w;
  gm_rule(grade, degree, p, w);
  return int(w.size());
}

fq_status fq_derham_nodes(fq_ctx* ctx, fq_mesh* m, const double* coords, int adim, int grade, int degree,
                          double* nodes) {
  if (!ctx || !m || !coords || !nodes) return FQ_INVALID_ARG;
  FQ_GUARD_BEGIN
  DerhamArgs a{};
  DevBuf rule;
  FQ_TRY(derham_setup(ctx, m, adim, grade, degree, a, rule));
  a.coords = coords;
  a.nodes = nodes;
  if (a.nsimp > 0) {
    derham_nodes_kernel<<<grid_for_n(a.nsimp * a.nq), 256, 0, ctx->stream>>>(a);
    ctx->launches++;
  }
  FQ_CUDA(ctx, cudaGetLastError());
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return FQ_OK;
  FQ_GUARD_END(ctx)
}

fq_status fq_derham_reduce(fq_ctx* ctx, fq_mesh* m, const double* coords, int adim, int grade, int degree,
                           const double* values, double* cochain) {
  if (!ctx || !m || !coords || !values || !cochain) return FQ_INVALID_ARG;
  FQ_GUARD_BEGIN
  DerhamArgs a{};
  DevBuf rule;
  FQ_TRY(derham_setup(ctx, m, adim, grade, degree, a, rule));
  a.coords = coords;
  a.values = values;
  a.out = cochain;
  if (a.nsimp > 0) {
    derham_reduce_kernel<<<grid_for_n(a.nsimp), 256, 0, ctx->stream>>>(a);
    ctx->launches++;
  }
  FQ_CUDA(ctx, cudaGetLastError());
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return FQ_OK;
  FQ_GUARD_END(ctx)
}

}  // extern "C"
