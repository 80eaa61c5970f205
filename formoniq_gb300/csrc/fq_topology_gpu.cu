// Mesh topology built on the device: the colex skeletons of Complex::from_cells
// (simplicial/src/topology/complex.rs:278-336, skeleton.rs:50-83), the cell ->
// face incidence, the boundary subcomplex of the relative complex
// (complex.rs:140-151, whitney_complex.rs:523-566) and the interior numbering.
//
// Per grade k every cell lists its k-faces (local faces in colex order, the
// increasing bit masks over its sorted vertices); the face tuples are sorted
// colex by a stable LSD radix sort over their vertices (smallest vertex first,
// largest last, so the largest is the primary key and ties keep list order, as
// the reference's sort of the skeleton does), duplicates collapse to one kidx by
// a scan, and the cell -> face table is the scan scattered back. A facet in one
// cell only is a boundary facet; a lower face is on the boundary when some
// boundary facet of a cell containing it contains it. The host keeps copies of
// the skeletons, flags and maps for its own builders (coboundaries, transfer
// maps, the orientation).
#include <cub/cub.cuh>

#include <algorithm>
#include <vector>

#include "fq_internal.h"

namespace fq {

namespace {

constexpr int TB = 256;
int grid_n(int64_t n) { return int(std::max<int64_t>(1, std::min<int64_t>((n + TB - 1) / TB, 152 * 32))); }

// Sort each cell's vertices; flag negative indices (bit 0) and repeated
// vertices (bit 1); track the largest vertex and mark used ones.
__global__ void cells_prepare_kernel(int32_t* cells, int64_t nc, int nv, int* flags, int* maxv) {
  for (int64_t c = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; c < nc; c += int64_t(gridDim.x) * blockDim.x) {
    int32_t v[5];
    for (int i = 0; i < nv; ++i) v[i] = cells[c * nv + i];
    for (int i = 1; i < nv; ++i)
      for (int j = i; j > 0 && v[j - 1] > v[j]; --j) {
        const int32_t t = v[j];
        v[j] = v[j - 1];
        v[j - 1] = t;
      }
    int m = -1;
    for (int i = 0; i < nv; ++i) {
      if (v[i] < 0) atomicOr(flags, 1);
      if (i > 0 && v[i] == v[i - 1]) atomicOr(flags, 2);
      cells[c * nv + i] = v[i];
      m = v[i] > m ? v[i] : m;
    }
    atomicMax(maxv, m);
  }
}

__global__ void mark_used_kernel(const int32_t* cells, int64_t n, int32_t nverts, int32_t* used) {
  for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < n; t += int64_t(gridDim.x) * blockDim.x) {
    const int32_t v = cells[t];
    if (v >= 0 && v < nverts) used[v] = 1;
  }
}

// faces[(c * nloc + l) * w + i]: vertex i of local face l (the l-th w-subset of
// the cell's vertex positions in increasing mask order) of cell c.
__global__ void list_faces_kernel(const int32_t* cells, int64_t nc, int nv, int w, const uint8_t* local_masks, int nloc,
                                  int32_t* faces) {
  const int64_t total = nc * nloc;
  for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < total; t += int64_t(gridDim.x) * blockDim.x) {
    const int64_t c = t / nloc;
    const unsigned mask = local_masks[t - c * nloc];
    int p = 0;
    for (int b = 0; b < nv; ++b)
      if (mask & (1u << b)) faces[t * w + p++] = cells[c * nv + b];
  }
}

__global__ void iota_kernel(uint32_t* idx, int64_t n) {
  for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < n; t += int64_t(gridDim.x) * blockDim.x)
    idx[t] = uint32_t(t);
}

__global__ void digit_kernel(const int32_t* tup, int w, int i, const uint32_t* idx, int64_t n, uint32_t* key) {
  for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < n; t += int64_t(gridDim.x) * blockDim.x)
    key[t] = uint32_t(tup[int64_t(idx[t]) * w + i]);
}

// new[t] = 1 where the t-th sorted tuple differs from the one before
__global__ void new_flags_kernel(const int32_t* tup, int w, const uint32_t* idx, int64_t n, int32_t* flag) {
  for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < n; t += int64_t(gridDim.x) * blockDim.x) {
    int f = t == 0;
    if (!f) {
      const int32_t* a = tup + int64_t(idx[t]) * w;
      const int32_t* b = tup + int64_t(idx[t - 1]) * w;
      for (int i = 0; i < w; ++i) f |= a[i] != b[i];
    }
    flag[t] = f;
  }
}

// kidx of the t-th sorted tuple = inclusive count of new tuples - 1: written to
// the listing position (cell-major) and, for the first of a run, the skeleton.
__global__ void kidx_kernel(const int32_t* tup, int w, const uint32_t* idx, const int32_t* incl, const int32_t* flag,
                            int64_t n, int32_t* cf, int32_t* skel) {
  for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < n; t += int64_t(gridDim.x) * blockDim.x) {
    const int32_t k = incl[t] - 1;
    cf[idx[t]] = k;
    if (flag[t])
      for (int i = 0; i < w; ++i) skel[int64_t(k) * w + i] = tup[int64_t(idx[t]) * w + i];
  }
}

// entry-major copy [l][c] of the cell-major table [c][l]
__global__ void transpose_cf_kernel(const int32_t* cf, int64_t nc, int nloc, int32_t* em) {
  const int64_t total = nc * nloc;
  for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < total; t += int64_t(gridDim.x) * blockDim.x) {
    const int64_t c = t / nloc;
    const int l = int(t - c * nloc);
    em[int64_t(l) * nc + c] = cf[t];
  }
}

__global__ void count_kernel(const int32_t* cf, int64_t n, int32_t* count) {
  for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < n; t += int64_t(gridDim.x) * blockDim.x)
    atomicAdd(count + cf[t], 1);
}

__global__ void facet_boundary_kernel(const int32_t* count, int64_t n, uint8_t* bnd) {
  for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < n; t += int64_t(gridDim.x) * blockDim.x)
    bnd[t] = count[t] == 1 ? 1 : 0;
}

// A local k-face of a cell lies on the boundary when a boundary local facet of
// the same cell contains it (facet l omits one vertex position; colex facet
// masks are the nv masks with one bit cleared).
__global__ void lower_boundary_kernel(const int32_t* cf_facet, const uint8_t* facet_bnd, const int32_t* cf_k,
                                      const uint8_t* local_masks, int64_t nc, int nv, int nloc_k,
                                      const uint8_t* facet_masks, uint8_t* bnd_k) {
  const int64_t total = nc * nloc_k;
  for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < total; t += int64_t(gridDim.x) * blockDim.x) {
    const int64_t c = t / nloc_k;
    const unsigned lm = local_masks[t - c * nloc_k];
    for (int f = 0; f < nv; ++f) {
      const unsigned fm = facet_masks[f];
      if ((lm & ~fm) == 0 && facet_bnd[cf_facet[c * nv + f]]) {
        bnd_k[cf_k[t]] = 1;
        break;
      }
    }
  }
}

__global__ void not_flags_kernel(const uint8_t* bnd, int64_t n, int32_t* out) {
  for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < n; t += int64_t(gridDim.x) * blockDim.x)
    out[t] = bnd[t] ? 0 : 1;
}

__global__ void interior_map_kernel(const uint8_t* bnd, const int32_t* excl, int64_t n, int32_t* map) {
  for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < n; t += int64_t(gridDim.x) * blockDim.x)
    map[t] = bnd[t] ? -1 : excl[t];
}

int bits_for(int64_t v) {
  int b = 1;
  while (b < 31 && (int64_t(1) << b) <= v) ++b;
  return b;
}

// Colex order of n tuples of width w (vertex indices < 2^vb): stable LSD radix
// sort, one CUB pass per vertex position. Returns the permutation in idx.
fq_status colex_sort(fq_ctx* ctx, const int32_t* tup, int w, int64_t n, int vb, DevBuf& idx) {
  cudaStream_t st = ctx->stream;
  DevBuf idx2, key, key2, tmp;
  FQ_TRY(idx.alloc(ctx, std::max<int64_t>(n, 1) * 4));
  FQ_TRY(idx2.alloc(ctx, std::max<int64_t>(n, 1) * 4));
  FQ_TRY(key.alloc(ctx, std::max<int64_t>(n, 1) * 4));
  FQ_TRY(key2.alloc(ctx, std::max<int64_t>(n, 1) * 4));
  iota_kernel<<<grid_n(n), TB, 0, st>>>(idx.as<uint32_t>(), n);
  size_t tmp_bytes = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, key.as<uint32_t>(), key2.as<uint32_t>(), idx.as<uint32_t>(),
                                  idx2.as<uint32_t>(), int(n), 0, vb, st);
  FQ_TRY(tmp.alloc(ctx, std::max<size_t>(tmp_bytes, 16)));
  for (int i = 0; i < w; ++i) {
    digit_kernel<<<grid_n(n), TB, 0, st>>>(tup, w, i, idx.as<uint32_t>(), n, key.as<uint32_t>());
    FQ_CUDA(ctx, cub::DeviceRadixSort::SortPairs(tmp.p, tmp_bytes, key.as<uint32_t>(), key2.as<uint32_t>(),
                                                 idx.as<uint32_t>(), idx2.as<uint32_t>(), int(n), 0, vb, st));
    std::swap(idx, idx2);
  }
  ctx->launches += 1 + 2 * uint64_t(w);
  return FQ_OK;
}

// Unique tuples in colex order: kidx per listing position (cf) and the skeleton.
fq_status unique_tuples(fq_ctx* ctx, const int32_t* tup, int w, int64_t n, int vb, DevBuf& cf, DevBuf& skel,
                        int64_t* nunique) {
  cudaStream_t st = ctx->stream;
  DevBuf idx, flag, incl, tmp;
  FQ_TRY(colex_sort(ctx, tup, w, n, vb, idx));
  FQ_TRY(flag.alloc(ctx, std::max<int64_t>(n, 1) * 4));
  FQ_TRY(incl.alloc(ctx, std::max<int64_t>(n, 1) * 4));
  new_flags_kernel<<<grid_n(n), TB, 0, st>>>(tup, w, idx.as<uint32_t>(), n, flag.as<int32_t>());
  size_t tmp_bytes = 0;
  cub::DeviceScan::InclusiveSum(nullptr, tmp_bytes, flag.as<int32_t>(), incl.as<int32_t>(), int(n), st);
  FQ_TRY(tmp.alloc(ctx, std::max<size_t>(tmp_bytes, 16)));
  FQ_CUDA(ctx, cub::DeviceScan::InclusiveSum(tmp.p, tmp_bytes, flag.as<int32_t>(), incl.as<int32_t>(), int(n), st));
  int32_t nu = 0;
  FQ_CUDA(ctx, cudaMemcpyAsync(&nu, incl.as<int32_t>() + (n - 1), 4, cudaMemcpyDeviceToHost, st));
  FQ_CUDA(ctx, cudaStreamSynchronize(st));
  FQ_TRY(cf.alloc(ctx, std::max<int64_t>(n, 1) * 4));
  FQ_TRY(skel.alloc(ctx, std::max<int64_t>(int64_t(nu) * w, 1) * 4));
  kidx_kernel<<<grid_n(n), TB, 0, st>>>(tup, w, idx.as<uint32_t>(), incl.as<int32_t>(), flag.as<int32_t>(), n,
                                        cf.as<int32_t>(), skel.as<int32_t>());
  ctx->launches += 3;
  *nunique = nu;
  return FQ_OK;
}

std::vector<uint8_t> local_masks_of(int nv, int w) {
  std::vector<uint8_t> out;
  for (unsigned mask = 0; mask < (1u << nv); ++mask)
    if (cpopcount(mask) == w) out.push_back(uint8_t(mask));
  return out;
}

template <typename T>
fq_status download(fq_ctx* ctx, const DevBuf& d, int64_t n, std::vector<T>& out) {
  out.resize(size_t(std::max<int64_t>(n, 0)));
  if (n > 0) FQ_CUDA(ctx, cudaMemcpyAsync(out.data(), d.p, size_t(n) * sizeof(T), cudaMemcpyDeviceToHost, ctx->stream));
  return FQ_OK;
}

}  // namespace

fq_status build_topology(fq_ctx* ctx, fq_mesh* m, int dim, int64_t ncells_in, const int32_t* cells_in) {
  cudaStream_t st = ctx->stream;
  const int nv = dim + 1;
  if (ncells_in * nv >= (int64_t(1) << 31)) return set_error(ctx, FQ_UNSUPPORTED, "mesh too large for 32-bit tables");
  // raw cells: sort vertices, validate, colex order and dedup (Skeleton::new)
  DevBuf raw, words, used;
  FQ_TRY(raw.alloc(ctx, size_t(ncells_in) * nv * 4));
  FQ_TRY(words.alloc(ctx, 16));
  FQ_CUDA(ctx, cudaMemcpyAsync(raw.p, cells_in, size_t(ncells_in) * nv * 4, cudaMemcpyHostToDevice, st));
  const int init[2] = {0, -1};
  FQ_CUDA(ctx, cudaMemcpyAsync(words.p, init, 8, cudaMemcpyHostToDevice, st));
  cells_prepare_kernel<<<grid_n(ncells_in), TB, 0, st>>>(raw.as<int32_t>(), ncells_in, nv, words.as<int>(),
                                                         words.as<int>() + 1);
  int hw[2] = {0, 0};
  FQ_CUDA(ctx, cudaMemcpyAsync(hw, words.p, 8, cudaMemcpyDeviceToHost, st));
  FQ_CUDA(ctx, cudaStreamSynchronize(st));
  if (hw[0] & 1) return set_error(ctx, FQ_INVALID_ARG, "negative vertex index");
  if (hw[0] & 2) return set_error(ctx, FQ_INVALID_ARG, "a cell repeats a vertex (degenerate simplex)");
  const int64_t nverts = int64_t(hw[1]) + 1;
  {
    FQ_TRY(used.alloc(ctx, std::max<int64_t>(nverts, 1) * 4));
    FQ_CUDA(ctx, cudaMemsetAsync(used.p, 0, std::max<int64_t>(nverts, 1) * 4, st));
    mark_used_kernel<<<grid_n(ncells_in * nv), TB, 0, st>>>(raw.as<int32_t>(), ncells_in * nv, int32_t(nverts),
                                                            used.as<int32_t>());
    DevBuf sum, tmp;
    FQ_TRY(sum.alloc(ctx, 8));
    size_t tb = 0;
    cub::DeviceReduce::Sum(nullptr, tb, used.as<int32_t>(), sum.as<int32_t>(), int(nverts), st);
    FQ_TRY(tmp.alloc(ctx, std::max<size_t>(tb, 16)));
    FQ_CUDA(ctx, cub::DeviceReduce::Sum(tmp.p, tb, used.as<int32_t>(), sum.as<int32_t>(), int(nverts), st));
    int32_t nused = 0;
    FQ_CUDA(ctx, cudaMemcpyAsync(&nused, sum.p, 4, cudaMemcpyDeviceToHost, st));
    FQ_CUDA(ctx, cudaStreamSynchronize(st));
    if (nused != nverts) return set_error(ctx, FQ_INVALID_ARG, "mesh vertices must be contiguous and fully used");
    ctx->launches += 3;
  }
  const int vb = bits_for(nverts);
  DevBuf cell_cf, cells;
  int64_t ncells = 0;
  FQ_TRY(unique_tuples(ctx, raw.as<int32_t>(), nv, ncells_in, vb, cell_cf, cells, &ncells));
  raw.release();
  m->dim = dim;
  m->ncells = ncells;

  // every grade: faces listed per cell, sorted, numbered
  DevBuf cfk[5];
  std::vector<uint8_t> lmask[5];
  for (int k = 0; k <= dim; ++k) {
    const int w = k + 1;
    lmask[k] = local_masks_of(nv, w);
    const int nloc = int(lmask[k].size());
    const int64_t nf = ncells * nloc;
    DevBuf dmask, faces, skel;
    FQ_TRY(dmask.alloc(ctx, 16));
    FQ_CUDA(ctx, cudaMemcpyAsync(dmask.p, lmask[k].data(), lmask[k].size(), cudaMemcpyHostToDevice, st));
    FQ_TRY(faces.alloc(ctx, std::max<int64_t>(nf * w, 1) * 4));
    list_faces_kernel<<<grid_n(nf), TB, 0, st>>>(cells.as<int32_t>(), ncells, nv, w, dmask.as<uint8_t>(), nloc,
                                                 faces.as<int32_t>());
    ctx->launches++;
    int64_t nk = 0;
    FQ_TRY(unique_tuples(ctx, faces.as<int32_t>(), w, nf, vb, cfk[k], skel, &nk));
    m->nsimp[k] = nk;
    FQ_TRY(m->cell_faces[k].alloc(ctx, std::max<int64_t>(nf, 1) * 4));
    transpose_cf_kernel<<<grid_n(nf), TB, 0, st>>>(cfk[k].as<int32_t>(), ncells, nloc, m->cell_faces[k].as<int32_t>());
    ctx->launches++;
    FQ_TRY(download(ctx, skel, nk * w, m->skel[k]));
    FQ_TRY(download(ctx, cfk[k], nf, m->cell_faces_host[k]));
    // the device skeleton is kept for kernels that need vertex tuples
    m->skel_dev[k] = std::move(skel);
  }
  for (int k = dim + 1; k < 6; ++k) m->nsimp[k] = 0;

  // boundary: facets in one cell, then the faces of boundary facets
  DevBuf bnd[5];
  for (int k = 0; k <= dim; ++k) {
    FQ_TRY(bnd[k].alloc(ctx, std::max<int64_t>(m->nsimp[k], 1)));
    FQ_CUDA(ctx, cudaMemsetAsync(bnd[k].p, 0, std::max<int64_t>(m->nsimp[k], 1), st));
  }
  if (dim >= 1) {
    const int f = dim - 1;
    DevBuf count;
    FQ_TRY(count.alloc(ctx, std::max<int64_t>(m->nsimp[f], 1) * 4));
    FQ_CUDA(ctx, cudaMemsetAsync(count.p, 0, std::max<int64_t>(m->nsimp[f], 1) * 4, st));
    count_kernel<<<grid_n(ncells * nv), TB, 0, st>>>(cfk[f].as<int32_t>(), ncells * nv, count.as<int32_t>());
    facet_boundary_kernel<<<grid_n(m->nsimp[f]), TB, 0, st>>>(count.as<int32_t>(), m->nsimp[f], bnd[f].as<uint8_t>());
    ctx->launches += 2;
    // facet masks in colex order (the local facets of a cell)
    DevBuf fmask;
    FQ_TRY(fmask.alloc(ctx, 16));
    FQ_CUDA(ctx, cudaMemcpyAsync(fmask.p, lmask[f].data(), lmask[f].size(), cudaMemcpyHostToDevice, st));
    for (int k = 0; k < f; ++k) {
      const int nloc = int(lmask[k].size());
      DevBuf dmask;
      FQ_TRY(dmask.alloc(ctx, 16));
      FQ_CUDA(ctx, cudaMemcpyAsync(dmask.p, lmask[k].data(), lmask[k].size(), cudaMemcpyHostToDevice, st));
      lower_boundary_kernel<<<grid_n(ncells * nloc), TB, 0, st>>>(
          cfk[f].as<int32_t>(), bnd[f].as<uint8_t>(), cfk[k].as<int32_t>(), dmask.as<uint8_t>(), ncells, nv, nloc,
          fmask.as<uint8_t>(), bnd[k].as<uint8_t>());
      ctx->launches++;
      FQ_CUDA(ctx, cudaStreamSynchronize(st));
    }
  }
  // interior numbering
  for (int k = 0; k <= dim; ++k) {
    const int64_t n = m->nsimp[k];
    DevBuf ones, excl, tmp;
    FQ_TRY(ones.alloc(ctx, (n + 1) * 4));
    FQ_TRY(excl.alloc(ctx, (n + 1) * 4));
    FQ_CUDA(ctx, cudaMemsetAsync(ones.p, 0, (n + 1) * 4, st));
    not_flags_kernel<<<grid_n(n), TB, 0, st>>>(bnd[k].as<uint8_t>(), n, ones.as<int32_t>());
    size_t tb = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, tb, ones.as<int32_t>(), excl.as<int32_t>(), int(n + 1), st);
    FQ_TRY(tmp.alloc(ctx, std::max<size_t>(tb, 16)));
    FQ_CUDA(ctx, cub::DeviceScan::ExclusiveSum(tmp.p, tb, ones.as<int32_t>(), excl.as<int32_t>(), int(n + 1), st));
    FQ_TRY(m->interior_dev[k].alloc(ctx, std::max<int64_t>(n, 1) * 4));
    interior_map_kernel<<<grid_n(n), TB, 0, st>>>(bnd[k].as<uint8_t>(), excl.as<int32_t>(), n,
                                                  m->interior_dev[k].as<int32_t>());
    ctx->launches += 2;
    int32_t cnt = 0;
    FQ_CUDA(ctx, cudaMemcpyAsync(&cnt, excl.as<int32_t>() + n, 4, cudaMemcpyDeviceToHost, st));
    FQ_TRY(download(ctx, bnd[k], n, m->boundary[k]));
    FQ_TRY(download(ctx, m->interior_dev[k], n, m->interior_map[k]));
    FQ_CUDA(ctx, cudaStreamSynchronize(st));
    m->ninterior[k] = cnt;
  }
  FQ_CUDA(ctx, cudaStreamSynchronize(st));
  FQ_CUDA(ctx, cudaGetLastError());
  return FQ_OK;
}

}  // namespace fq
