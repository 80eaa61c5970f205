// Device builders of the sparse maps the HX preconditioner and the coboundary
// API need, from the device skeletons of the mesh:
//   - the coboundary D_k (HilbertComplex::dif, whitney_complex.rs:417-423, the
//     relative one :640-643): row = (k+1)-simplex, entries (-1)^p at its faces
//     s \ s_p (found by binary search in the colex k-skeleton), columns sorted;
//   - the vector-nodal interpolation Pi_j of formoniq/src/hx.rs
//     (vector_nodal_prolongation): row = j-face, entries
//     factor * det(E_I) at (node * m + slot + I) for every vertex node of the face
//     and every colex j-subset I of the lattice axes, E the face's lattice edge
//     vectors at unit spacing (scaled per axis set on the device afterwards);
//   - transposes by a stable sort of the entries by target row, so a target
//     row lists its entries in source-row order.
// One thread per row; a row holds at most 5 x 6 entries, sorted in registers.
#include <cub/cub.cuh>

#include <algorithm>
#include <vector>

#include "fq_hx.h"

namespace fq {

namespace {

constexpr int TB = 256;
int grid_n(int64_t n) { return int(std::max<int64_t>(1, std::min<int64_t>((n + TB - 1) / TB, 152 * 32))); }

__device__ int64_t find_tuple(const int32_t* sk, int64_t n, const int32_t* tup, int w) {
  int64_t lo = 0, hi = n - 1;
  while (lo <= hi) {
    const int64_t mid = (lo + hi) >> 1;
    int cmp = 0;
    for (int i = w - 1; i >= 0; --i) {
      const int32_t a = sk[mid * w + i];
      if (a != tup[i]) {
        cmp = a < tup[i] ? -1 : 1;
        break;
      }
    }
    if (cmp == 0) return mid;
    if (cmp < 0)
      lo = mid + 1;
    else
      hi = mid - 1;
  }
  return -1;
}

// coboundary row of (k+1)-simplex s: fills up to k+2 (col, sign) pairs, sorted
__device__ int coboundary_row(const int32_t* hi, const int32_t* lo, int64_t nlo, const int32_t* lomap, int k,
                              int64_t s, int32_t* col, double* val) {
  const int w = k + 2;
  int ne = 0;
  for (int p = 0; p < w; ++p) {
    int32_t tup[5];
    int q = 0;
    for (int i = 0; i < w; ++i)
      if (i != p) tup[q++] = hi[s * w + i];
    int64_t c = find_tuple(lo, nlo, tup, w - 1);
    if (c >= 0 && lomap) c = lomap[c];
    if (c < 0) continue;
    int j = ne++;
    while (j > 0 && col[j - 1] > int32_t(c)) {
      col[j] = col[j - 1];
      val[j] = val[j - 1];
      --j;
    }
    col[j] = int32_t(c);
    val[j] = (p % 2) ? -1.0 : 1.0;
  }
  return ne;
}

__global__ void coboundary_count_kernel(const int32_t* hi, int64_t nhi, const int32_t* himap, const int32_t* lo,
                                        int64_t nlo, const int32_t* lomap, int k, int32_t* count) {
  for (int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; s < nhi; s += int64_t(gridDim.x) * blockDim.x) {
    const int64_t r = himap ? himap[s] : s;
    if (r < 0) continue;
    int32_t col[5];
    double val[5];
    count[r] = coboundary_row(hi, lo, nlo, lomap, k, s, col, val);
  }
}

__global__ void coboundary_fill_kernel(const int32_t* hi, int64_t nhi, const int32_t* himap, const int32_t* lo,
                                       int64_t nlo, const int32_t* lomap, int k, const int32_t* rp, int32_t* ci,
                                       double* v) {
  for (int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; s < nhi; s += int64_t(gridDim.x) * blockDim.x) {
    const int64_t r = himap ? himap[s] : s;
    if (r < 0) continue;
    int32_t col[5];
    double val[5];
    const int ne = coboundary_row(hi, lo, nlo, lomap, k, s, col, val);
    const int32_t o = rp[r];
    for (int e = 0; e < ne; ++e) {
      ci[o + e] = col[e];
      v[o + e] = val[e];
    }
  }
}

struct NodalArgs {
  const int32_t* skel;  // [N_j][j+1]
  const int32_t* map;   // relative: face -> row or -1; null: identity
  int64_t nfaces;
  int j, n, nbox, bc, mslots, slot, ncomp;
  int subsets[6][4];    // colex j-subsets of the axes
  uint8_t masks[6];     // their axis bit masks
  double factor;        // 1 / (j+1)!
};

__device__ int64_t node_index_d(const int* c, int n, int nbox, int bc) {
  int64_t idx = 0, stride = 1;
  for (int a = 0; a < n; ++a) {
    if (bc == FQ_RELATIVE) {
      if (c[a] <= 0 || c[a] >= nbox) return -1;
      idx += int64_t(c[a] - 1) * stride;
      stride *= (nbox - 1);
    } else {
      idx += int64_t(c[a]) * stride;
      stride *= (nbox + 1);
    }
  }
  return idx;
}

__device__ void lattice_coords_d(int64_t v, int n, int nbox, int* c) {
  for (int a = 0; a < n; ++a) {
    c[a] = int(v % (nbox + 1));
    v /= (nbox + 1);
  }
}

__device__ double det_small(double m[4][4], int j) {
  if (j == 0) return 1.0;
  if (j == 1) return m[0][0];
  if (j == 2) return m[0][0] * m[1][1] - m[0][1] * m[1][0];
  if (j == 3)
    return m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) - m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
           m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
  double d = 0.0;
  for (int col = 0; col < 4; ++col) {
    double sub[4][4];
    for (int r = 1; r < 4; ++r) {
      int q = 0;
      for (int cc = 0; cc < 4; ++cc)
        if (cc != col) sub[r - 1][q++] = m[r][cc];
    }
    const double s3 = sub[0][0] * (sub[1][1] * sub[2][2] - sub[1][2] * sub[2][1]) -
                      sub[0][1] * (sub[1][0] * sub[2][2] - sub[1][2] * sub[2][0]) +
                      sub[0][2] * (sub[1][0] * sub[2][1] - sub[1][1] * sub[2][0]);
    d += ((col % 2) ? -1.0 : 1.0) * m[0][col] * s3;
  }
  return d;
}

// the entries of one face's row, sorted by column
__device__ int nodal_row(const NodalArgs& a, int64_t s, int64_t* col, double* val, uint8_t* msk) {
  const int w = a.j + 1;
  const int32_t* vs = a.skel + s * w;
  int c0[4], ci[4];
  lattice_coords_d(vs[0], a.n, a.nbox, c0);
  double E[4][4] = {};
  for (int i = 1; i <= a.j; ++i) {
    lattice_coords_d(vs[i], a.n, a.nbox, ci);
    for (int ax = 0; ax < a.n; ++ax) E[ax][i - 1] = double(ci[ax] - c0[ax]);
  }
  double comp[6];
  for (int q = 0; q < a.ncomp; ++q) {
    double sub[4][4] = {};
    for (int r = 0; r < a.j; ++r)
      for (int cc = 0; cc < a.j; ++cc) sub[r][cc] = E[a.subsets[q][r]][cc];
    comp[q] = a.j == 0 ? 1.0 : det_small(sub, a.j);
  }
  int ne = 0;
  for (int i = 0; i < w; ++i) {
    int cv[4];
    lattice_coords_d(vs[i], a.n, a.nbox, cv);
    const int64_t node = node_index_d(cv, a.n, a.nbox, a.bc);
    if (node < 0) continue;
    for (int q = 0; q < a.ncomp; ++q) {
      const double v = a.factor * comp[q];
      if (v == 0.0) continue;
      const int64_t c = node * a.mslots + a.slot + q;
      int e = ne++;
      while (e > 0 && (col[e - 1] > c || (col[e - 1] == c && val[e - 1] > v))) {
        col[e] = col[e - 1];
        val[e] = val[e - 1];
        msk[e] = msk[e - 1];
        --e;
      }
      col[e] = c;
      val[e] = v;
      msk[e] = a.masks[q];
    }
  }
  return ne;
}

__global__ void nodal_count_kernel(NodalArgs a, int32_t* count) {
  for (int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; s < a.nfaces;
       s += int64_t(gridDim.x) * blockDim.x) {
    const int64_t r = a.map ? a.map[s] : s;
    if (r < 0) continue;
    int64_t col[30];
    double val[30];
    uint8_t msk[30];
    count[r] = nodal_row(a, s, col, val, msk);
  }
}

__global__ void nodal_fill_kernel(NodalArgs a, const int32_t* rp, int32_t* ci, double* v, uint8_t* mask) {
  for (int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; s < a.nfaces;
       s += int64_t(gridDim.x) * blockDim.x) {
    const int64_t r = a.map ? a.map[s] : s;
    if (r < 0) continue;
    int64_t col[30];
    double val[30];
    uint8_t msk[30];
    const int ne = nodal_row(a, s, col, val, msk);
    const int32_t o = rp[r];
    for (int e = 0; e < ne; ++e) {
      ci[o + e] = int32_t(col[e]);
      v[o + e] = val[e];
      mask[o + e] = msk[e];
    }
  }
}

__global__ void row_of_kernel(const int32_t* rp, int64_t nrows, int32_t* row) {
  for (int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; r < nrows; r += int64_t(gridDim.x) * blockDim.x)
    for (int32_t e = rp[r]; e < rp[r + 1]; ++e) row[e] = int32_t(r);
}

// target row of an entry: its column, or for a vector-nodal map (node, component)
__global__ void target_keys_kernel(const int32_t* ci, int64_t nnz, int mslots, int slot, int ncomp, uint32_t* key,
                                   uint32_t* idx) {
  for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < nnz; e += int64_t(gridDim.x) * blockDim.x) {
    const int32_t c = ci[e];
    key[e] = mslots > 0 ? uint32_t((c / mslots) * ncomp + (c % mslots - slot)) : uint32_t(c);
    idx[e] = uint32_t(e);
  }
}

__global__ void lower_bound_u32_kernel(const uint32_t* keys, int64_t n, int64_t nrows, int32_t* ptr) {
  for (int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; r <= nrows; r += int64_t(gridDim.x) * blockDim.x) {
    int64_t lo = 0, hi = n;
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (keys[mid] < uint32_t(r))
        lo = mid + 1;
      else
        hi = mid;
    }
    ptr[r] = int32_t(lo);
  }
}

__global__ void transpose_gather_kernel(const uint32_t* idx, const int32_t* row, const double* v, const uint8_t* mask,
                                        int64_t nnz, int32_t* tci, double* tv, uint8_t* tmask) {
  for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < nnz; t += int64_t(gridDim.x) * blockDim.x) {
    const uint32_t e = idx[t];
    tci[t] = row[e];
    tv[t] = v[e];
    if (tmask) tmask[t] = mask[e];
  }
}

int bits_of(int64_t v) {
  int b = 1;
  while (b < 32 && (int64_t(1) << b) <= v) ++b;
  return b;
}

fq_status scan_counts(fq_ctx* ctx, DevBuf& count, int64_t nrows, DevBuf& rp, int64_t* nnz) {
  cudaStream_t st = ctx->stream;
  FQ_TRY(rp.alloc(ctx, (nrows + 1) * 4));
  size_t tb = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, tb, count.as<int32_t>(), rp.as<int32_t>(), int(nrows + 1), st);
  DevBuf tmp;
  FQ_TRY(tmp.alloc(ctx, std::max<size_t>(tb, 16)));
  FQ_CUDA(ctx, cub::DeviceScan::ExclusiveSum(tmp.p, tb, count.as<int32_t>(), rp.as<int32_t>(), int(nrows + 1), st));
  int32_t total = 0;
  FQ_CUDA(ctx, cudaMemcpyAsync(&total, rp.as<int32_t>() + nrows, 4, cudaMemcpyDeviceToHost, st));
  FQ_CUDA(ctx, cudaStreamSynchronize(st));
  *nnz = total;
  return FQ_OK;
}

void adopt(DCsr& d, int64_t nr, int64_t nc, int64_t nnz, DevBuf&& rp, DevBuf&& ci, DevBuf&& v) {
  d.nrows = nr;
  d.ncols = nc;
  d.nnz = nnz;
  d.own_rp = std::move(rp);
  d.own_ci = std::move(ci);
  d.own_v64 = std::move(v);
  d.rp = d.own_rp.as<int32_t>();
  d.ci = d.own_ci.as<int32_t>();
  d.v64 = d.own_v64.as<double>();
  d.v32 = nullptr;
  d.own_v32.release();
}

}  // namespace

fq_status device_skeleton(fq_ctx* ctx, fq_mesh* m, int k, const int32_t** out) {
  if (!m->skel_dev[k].p) {
    const size_t bytes = std::max<size_t>(m->skel[k].size(), 1) * 4;
    FQ_TRY(m->skel_dev[k].alloc(ctx, bytes));
    if (!m->skel[k].empty())
      FQ_CUDA(ctx, cudaMemcpyAsync(m->skel_dev[k].p, m->skel[k].data(), m->skel[k].size() * 4,
                                   cudaMemcpyHostToDevice, ctx->stream));
  }
  *out = m->skel_dev[k].as<int32_t>();
  return FQ_OK;
}

// A^T (mslots == 0) or, for a vector-nodal map, its (node, component) reading;
// stable: a target row lists its entries in source-row order.
fq_status device_transpose(fq_ctx* ctx, const DCsr& a, const uint8_t* mask, int64_t nt_rows, int mslots, int slot,
                           int ncomp, DCsr& out, DevBuf* out_mask) {
  cudaStream_t st = ctx->stream;
  const int64_t nnz = a.nnz;
  DevBuf row, key, key2, idx, idx2, tmp, rp, ci, v;
  FQ_TRY(row.alloc(ctx, std::max<int64_t>(nnz, 1) * 4));
  FQ_TRY(key.alloc(ctx, std::max<int64_t>(nnz, 1) * 4));
  FQ_TRY(key2.alloc(ctx, std::max<int64_t>(nnz, 1) * 4));
  FQ_TRY(idx.alloc(ctx, std::max<int64_t>(nnz, 1) * 4));
  FQ_TRY(idx2.alloc(ctx, std::max<int64_t>(nnz, 1) * 4));
  FQ_TRY(rp.alloc(ctx, (nt_rows + 1) * 4));
  FQ_TRY(ci.alloc(ctx, std::max<int64_t>(nnz, 1) * 4));
  FQ_TRY(v.alloc(ctx, std::max<int64_t>(nnz, 1) * 8));
  if (out_mask) FQ_TRY(out_mask->alloc(ctx, std::max<int64_t>(nnz, 1)));
  if (nnz > 0) {
    row_of_kernel<<<grid_n(a.nrows), TB, 0, st>>>(a.rp, a.nrows, row.as<int32_t>());
    target_keys_kernel<<<grid_n(nnz), TB, 0, st>>>(a.ci, nnz, mslots, slot, ncomp, key.as<uint32_t>(),
                                                   idx.as<uint32_t>());
    const int bits = bits_of(std::max<int64_t>(nt_rows, 1));
    size_t tb = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, tb, key.as<uint32_t>(), key2.as<uint32_t>(), idx.as<uint32_t>(),
                                    idx2.as<uint32_t>(), int(nnz), 0, bits, st);
    FQ_TRY(tmp.alloc(ctx, std::max<size_t>(tb, 16)));
    FQ_CUDA(ctx, cub::DeviceRadixSort::SortPairs(tmp.p, tb, key.as<uint32_t>(), key2.as<uint32_t>(),
                                                 idx.as<uint32_t>(), idx2.as<uint32_t>(), int(nnz), 0, bits, st));
    transpose_gather_kernel<<<grid_n(nnz), TB, 0, st>>>(idx2.as<uint32_t>(), row.as<int32_t>(), a.v64, mask, nnz,
                                                        ci.as<int32_t>(), v.as<double>(),
                                                        out_mask ? out_mask->as<uint8_t>() : nullptr);
    ctx->launches += 3;
  }
  lower_bound_u32_kernel<<<grid_n(nt_rows + 1), TB, 0, st>>>(key2.as<uint32_t>(), nnz, nt_rows, rp.as<int32_t>());
  ctx->launches++;
  FQ_CUDA(ctx, cudaStreamSynchronize(st));
  adopt(out, nt_rows, a.nrows, nnz, std::move(rp), std::move(ci), std::move(v));
  return FQ_OK;
}

fq_status coboundary_device(fq_ctx* ctx, fq_mesh* m, int k, int bc, DCsr& D) {
  cudaStream_t st = ctx->stream;
  const int64_t nr = bc == FQ_RELATIVE ? m->ninterior[k + 1] : m->nsimp[k + 1];
  const int64_t nc = bc == FQ_RELATIVE ? m->ninterior[k] : m->nsimp[k];
  const int32_t *hi = nullptr, *lo = nullptr;
  FQ_TRY(device_skeleton(ctx, m, k + 1, &hi));
  FQ_TRY(device_skeleton(ctx, m, k, &lo));
  const int32_t* himap = bc == FQ_RELATIVE ? m->interior_dev[k + 1].as<int32_t>() : nullptr;
  const int32_t* lomap = bc == FQ_RELATIVE ? m->interior_dev[k].as<int32_t>() : nullptr;
  DevBuf count, rp, ci, v;
  FQ_TRY(count.alloc(ctx, (nr + 1) * 4));
  FQ_CUDA(ctx, cudaMemsetAsync(count.p, 0, (nr + 1) * 4, st));
  coboundary_count_kernel<<<grid_n(m->nsimp[k + 1]), TB, 0, st>>>(hi, m->nsimp[k + 1], himap, lo, m->nsimp[k], lomap,
                                                                   k, count.as<int32_t>());
  int64_t nnz = 0;
  FQ_TRY(scan_counts(ctx, count, nr, rp, &nnz));
  FQ_TRY(ci.alloc(ctx, std::max<int64_t>(nnz, 1) * 4));
  FQ_TRY(v.alloc(ctx, std::max<int64_t>(nnz, 1) * 8));
  coboundary_fill_kernel<<<grid_n(m->nsimp[k + 1]), TB, 0, st>>>(hi, m->nsimp[k + 1], himap, lo, m->nsimp[k], lomap,
                                                                  k, rp.as<int32_t>(), ci.as<int32_t>(),
                                                                  v.as<double>());
  ctx->launches += 2;
  FQ_CUDA(ctx, cudaStreamSynchronize(st));
  FQ_CUDA(ctx, cudaGetLastError());
  adopt(D, nr, nc, nnz, std::move(rp), std::move(ci), std::move(v));
  return FQ_OK;
}

fq_status vector_nodal_device(fq_ctx* ctx, fq_mesh* m, int j, int bc, int mslots, int slot, DCsr& Pi, DCsr& Pit) {
  cudaStream_t st = ctx->stream;
  const int n = m->dim, nb = m->kuhn_nbox;
  NodalArgs a{};
  FQ_TRY(device_skeleton(ctx, m, j, &a.skel));
  a.map = bc == FQ_RELATIVE ? m->interior_dev[j].as<int32_t>() : nullptr;
  a.nfaces = m->nsimp[j];
  a.j = j;
  a.n = n;
  a.nbox = nb;
  a.bc = bc;
  a.mslots = mslots;
  a.slot = slot;
  // colex j-subsets of the axes: increasing bit masks read colex
  std::vector<unsigned> subs;
  for (unsigned mask = 0; mask < (1u << n); ++mask)
    if (__builtin_popcount(mask) == j) subs.push_back(mask);
  std::sort(subs.begin(), subs.end(), [](unsigned x, unsigned y) {
    for (int b = 3; b >= 0; --b) {
      const unsigned bx = (x >> b) & 1u, by = (y >> b) & 1u;
      if (bx != by) return bx < by;
    }
    return false;
  });
  a.ncomp = int(subs.size());
  for (int q = 0; q < a.ncomp; ++q) {
    int p = 0;
    for (int ax = 0; ax < n; ++ax)
      if (subs[size_t(q)] & (1u << ax)) a.subsets[q][p++] = ax;
    a.masks[q] = uint8_t(subs[size_t(q)]);
  }
  double fact = 1.0;
  for (int i = 2; i <= j + 1; ++i) fact *= i;
  a.factor = 1.0 / fact;
  const int64_t nrows = bc == FQ_RELATIVE ? m->ninterior[j] : m->nsimp[j];
  int64_t n0 = 1;
  for (int ax = 0; ax < n; ++ax) n0 *= bc == FQ_RELATIVE ? std::max(nb - 1, 0) : nb + 1;
  DevBuf count, rp, ci, v;
  FQ_TRY(count.alloc(ctx, (nrows + 1) * 4));
  FQ_CUDA(ctx, cudaMemsetAsync(count.p, 0, (nrows + 1) * 4, st));
  nodal_count_kernel<<<grid_n(a.nfaces), TB, 0, st>>>(a, count.as<int32_t>());
  int64_t nnz = 0;
  FQ_TRY(scan_counts(ctx, count, nrows, rp, &nnz));
  FQ_TRY(ci.alloc(ctx, std::max<int64_t>(nnz, 1) * 4));
  FQ_TRY(v.alloc(ctx, std::max<int64_t>(nnz, 1) * 8));
  FQ_TRY(Pi.own_mask.alloc(ctx, std::max<int64_t>(nnz, 1)));
  nodal_fill_kernel<<<grid_n(a.nfaces), TB, 0, st>>>(a, rp.as<int32_t>(), ci.as<int32_t>(), v.as<double>(),
                                                     Pi.own_mask.as<uint8_t>());
  ctx->launches += 2;
  adopt(Pi, nrows, n0 * mslots, nnz, std::move(rp), std::move(ci), std::move(v));
  // scalable: lattice values kept as the base, scaled into v64 by the spacing
  FQ_TRY(Pi.own_base.alloc(ctx, std::max<int64_t>(nnz, 1) * 8));
  if (nnz) FQ_CUDA(ctx, cudaMemcpyAsync(Pi.own_base.p, Pi.v64, nnz * 8, cudaMemcpyDeviceToDevice, st));
  Pi.scalable = true;
  FQ_TRY(device_transpose(ctx, Pi, Pi.own_mask.as<uint8_t>(), n0 * a.ncomp, mslots, slot, a.ncomp, Pit,
                          &Pit.own_mask));
  FQ_TRY(Pit.own_base.alloc(ctx, std::max<int64_t>(nnz, 1) * 8));
  if (nnz) FQ_CUDA(ctx, cudaMemcpyAsync(Pit.own_base.p, Pit.v64, nnz * 8, cudaMemcpyDeviceToDevice, st));
  Pit.scalable = true;
  FQ_CUDA(ctx, cudaStreamSynchronize(st));
  FQ_CUDA(ctx, cudaGetLastError());
  return FQ_OK;
}

}  // namespace fq
