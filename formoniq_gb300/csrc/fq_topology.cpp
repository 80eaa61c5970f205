// Mesh topology on the host: the colex skeletons of Complex::from_cells
// (simplicial/src/topology/complex.rs:278-336, skeleton.rs:50-83), the cell ->
// face incidence the scatter needs, the boundary subcomplex of the relative
// complex (complex.rs:140-151, whitney_complex.rs:523-566) and a coherent
// orientation (topology/orientation.rs). The Kuhn mesher
// (simplicial/src/mesher/grid.rs:77-98) and the vertex placement of
// CartesianGrid (regge/src/mesher/cartesian.rs:158-226) live here too.
//
// Built once per mesh and cached; the hot path never touches it.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "fq_internal.h"

namespace fq {
namespace {

int ibinom(int n, int k) { return cbinom(n, k); }

// LSD radix sort of (key, idx) pairs on the low `bits` of key; stable.
void radix_sort_pairs(std::vector<uint64_t>& key, std::vector<uint32_t>& idx, int bits) {
  const size_t n = key.size();
  std::vector<uint64_t> k2(n);
  std::vector<uint32_t> i2(n);
  const int D = 11;
  for (int shift = 0; shift < bits; shift += D) {
    std::vector<size_t> cnt((1u << D) + 1, 0);
    const uint64_t mask = (1ull << D) - 1;
    for (size_t t = 0; t < n; ++t) cnt[((key[t] >> shift) & mask) + 1]++;
    for (size_t d = 0; d < (1u << D); ++d) cnt[d + 1] += cnt[d];
    for (size_t t = 0; t < n; ++t) {
      const size_t pos = cnt[(key[t] >> shift) & mask]++;
      k2[pos] = key[t];
      i2[pos] = idx[t];
    }
    key.swap(k2);
    idx.swap(i2);
  }
}

int bits_for(uint64_t v) {
  int b = 0;
  while ((1ull << b) <= v && b < 63) ++b;
  return std::max(b, 1);
}

// Sort tuples (rows of width w) colex and return the permutation. Keys pack
// the vertices with the largest most significant; 64-bit radix when they fit.
std::vector<uint32_t> colex_order(const std::vector<int32_t>& tup, int w, int64_t count, int64_t nverts) {
  std::vector<uint32_t> idx(static_cast<size_t>(count));
  std::iota(idx.begin(), idx.end(), 0u);
  const int vb = bits_for(uint64_t(std::max<int64_t>(nverts, 1)));
  if (vb * w <= 64) {
    std::vector<uint64_t> key(static_cast<size_t>(count));
    for (int64_t t = 0; t < count; ++t) {
      uint64_t k = 0;
      for (int i = w - 1; i >= 0; --i) k = (k << vb) | uint64_t(tup[t * w + i]);
      key[t] = k;
    }
    radix_sort_pairs(key, idx, vb * w);
  } else {
    std::sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) {
      for (int i = w - 1; i >= 0; --i) {
        const int32_t x = tup[int64_t(a) * w + i], y = tup[int64_t(b) * w + i];
        if (x != y) return x < y;
      }
      return a < b;
    });
  }
  return idx;
}

}  // namespace

// Build every skeleton and the cell -> face tables from raw cells.
fq_status build_topology(fq_ctx* ctx, fq_mesh* m, int dim, int64_t ncells_in, const int32_t* cells_in) {
  const int nv = dim + 1;
  // sort each cell's vertices, then the cells colex, dedup (Skeleton::new)
  std::vector<int32_t> raw(cells_in, cells_in + ncells_in * nv);
  int64_t maxv = -1;
  for (int64_t c = 0; c < ncells_in; ++c) {
    std::sort(&raw[c * nv], &raw[c * nv] + nv);
    for (int i = 0; i < nv; ++i) {
      if (raw[c * nv + i] < 0) return set_error(ctx, FQ_INVALID_ARG, "negative vertex index");
      if (i > 0 && raw[c * nv + i] == raw[c * nv + i - 1])
        return set_error(ctx, FQ_INVALID_ARG, "a cell repeats a vertex (degenerate simplex)");
      maxv = std::max<int64_t>(maxv, raw[c * nv + i]);
    }
  }
  const int64_t nverts = maxv + 1;
  std::vector<uint8_t> used(static_cast<size_t>(std::max<int64_t>(nverts, 0)), 0);
  for (auto v : raw) used[v] = 1;
  for (auto u : used)
    if (!u) return set_error(ctx, FQ_INVALID_ARG, "mesh vertices must be contiguous and fully used");
  auto order = colex_order(raw, nv, ncells_in, nverts);
  std::vector<int32_t> cells;
  cells.reserve(raw.size());
  for (int64_t t = 0; t < ncells_in; ++t) {
    const int32_t* c = &raw[int64_t(order[t]) * nv];
    if (!cells.empty() && std::equal(c, c + nv, cells.end() - nv)) continue;
    cells.insert(cells.end(), c, c + nv);
  }
  const int64_t ncells = int64_t(cells.size()) / nv;
  m->dim = dim;
  m->ncells = ncells;
  for (int k = 0; k <= dim; ++k) {
    const int nloc = ibinom(nv, k + 1);
    const int w = k + 1;
    // local k-faces of the cell in colex order: increasing bitmask order
    std::vector<std::vector<int>> locals;
    for (unsigned mask = 0; mask < (1u << nv); ++mask) {
      if (cpopcount(mask) != w) continue;
      std::vector<int> l;
      for (int b = 0; b < nv; ++b)
        if (mask & (1u << b)) l.push_back(b);
      locals.push_back(l);
    }
    const int64_t nf = ncells * nloc;
    std::vector<int32_t> faces(static_cast<size_t>(nf * w));
    for (int64_t c = 0; c < ncells; ++c)
      for (int l = 0; l < nloc; ++l)
        for (int i = 0; i < w; ++i) faces[(c * nloc + l) * w + i] = cells[c * nv + locals[l][i]];
    auto ord = colex_order(faces, w, nf, nverts);
    std::vector<int32_t>& sk = m->skel[k];
    sk.clear();
    std::vector<int32_t> cf(static_cast<size_t>(nf));
    int64_t kidx = -1;
    for (int64_t t = 0; t < nf; ++t) {
      const int32_t* f = &faces[int64_t(ord[t]) * w];
      if (kidx < 0 || !std::equal(f, f + w, sk.end() - w)) {
        sk.insert(sk.end(), f, f + w);
        ++kidx;
      }
      cf[ord[t]] = int32_t(kidx);
    }
    m->nsimp[k] = kidx + 1;
    m->cell_faces_host[k] = cf;
    // upload entry-major [local][cell]
    std::vector<int32_t> em(static_cast<size_t>(nf));
    for (int64_t c = 0; c < ncells; ++c)
      for (int l = 0; l < nloc; ++l) em[int64_t(l) * ncells + c] = cf[c * nloc + l];
    FQ_TRY(m->cell_faces[k].alloc(ctx, em.size() * sizeof(int32_t)));
    FQ_CUDA(ctx, cudaMemcpyAsync(m->cell_faces[k].p, em.data(), em.size() * sizeof(int32_t),
                                 cudaMemcpyHostToDevice, ctx->stream));
    FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (k == dim - 1 && dim >= 1) {
      // boundary facets: in exactly one cell
      std::vector<int32_t> count(static_cast<size_t>(m->nsimp[k]), 0);
      for (int64_t t = 0; t < nf; ++t) count[cf[t]]++;
      m->boundary[k].assign(static_cast<size_t>(m->nsimp[k]), 0);
      for (int64_t f = 0; f < m->nsimp[k]; ++f)
        if (count[f] == 1) m->boundary[k][f] = 1;
    }
  }
  for (int k = dim + 1; k < 6; ++k) m->nsimp[k] = 0;
  // boundary simplices of lower grade: faces of boundary facets
  for (int k = 0; k <= dim; ++k)
    if (m->boundary[k].empty()) m->boundary[k].assign(static_cast<size_t>(m->nsimp[k]), 0);
  if (dim >= 1) {
    const int fw = dim;  // facet width
    // map vertex tuple -> kidx per grade via binary search in the colex skeleton
    for (int64_t f = 0; f < m->nsimp[dim - 1]; ++f) {
      if (!m->boundary[dim - 1][f]) continue;
      const int32_t* fv = &m->skel[dim - 1][f * fw];
      for (int k = 0; k < dim - 1; ++k) {
        const int w = k + 1;
        for (unsigned mask = 0; mask < (1u << fw); ++mask) {
          if (cpopcount(mask) != w) continue;
          int32_t tup[5];
          int p = 0;
          for (int b = 0; b < fw; ++b)
            if (mask & (1u << b)) tup[p++] = fv[b];
          const int32_t* sk = m->skel[k].data();
          int64_t lo = 0, hi = m->nsimp[k] - 1;
          while (lo <= hi) {
            const int64_t mid = (lo + hi) / 2;
            int cmp = 0;
            for (int i = w - 1; i >= 0; --i)
              if (sk[mid * w + i] != tup[i]) {
                cmp = sk[mid * w + i] < tup[i] ? -1 : 1;
                break;
              }
            if (cmp == 0) {
              m->boundary[k][mid] = 1;
              break;
            }
            if (cmp < 0)
              lo = mid + 1;
            else
              hi = mid - 1;
          }
        }
      }
    }
  }
  for (int k = 0; k <= dim; ++k) {
    auto& im = m->interior_map[k];
    im.assign(static_cast<size_t>(m->nsimp[k]), -1);
    int64_t cnt = 0;
    for (int64_t i = 0; i < m->nsimp[k]; ++i)
      if (!m->boundary[k][i]) im[i] = int32_t(cnt++);
    m->ninterior[k] = cnt;
    FQ_TRY(m->interior_dev[k].alloc(ctx, std::max<size_t>(im.size(), 1) * sizeof(int32_t)));
    if (!im.empty())
      FQ_CUDA(ctx, cudaMemcpyAsync(m->interior_dev[k].p, im.data(), im.size() * sizeof(int32_t),
                                   cudaMemcpyHostToDevice, ctx->stream));
  }
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return FQ_OK;
}

// Kuhn cells of the cube: per box (axis 0 fastest) and per axis permutation,
// the chain origin, origin + s_a1, ... with strides s_a = (N+1)^a.
std::vector<int32_t> kuhn_cells(int dim, int nbox) {
  std::vector<int64_t> stride(dim);
  int64_t s = 1;
  for (int a = 0; a < dim; ++a) {
    stride[a] = s;
    s *= (nbox + 1);
  }
  int64_t nboxes = 1;
  for (int a = 0; a < dim; ++a) nboxes *= nbox;
  std::vector<int> perm(dim);
  std::iota(perm.begin(), perm.end(), 0);
  std::vector<std::vector<int>> perms;
  do perms.push_back(perm);
  while (std::next_permutation(perm.begin(), perm.end()));
  std::vector<int32_t> out;
  out.reserve(static_cast<size_t>(nboxes * int64_t(perms.size()) * (dim + 1)));
  for (int64_t b = 0; b < nboxes; ++b) {
    int64_t rem = b, origin = 0;
    for (int a = 0; a < dim; ++a) {
      origin += (rem % nbox) * stride[a];
      rem /= nbox;
    }
    for (const auto& p : perms) {
      int64_t v = origin;
      out.push_back(int32_t(v));
      for (int i = 0; i < dim; ++i) {
        v += stride[p[i]];
        out.push_back(int32_t(v));
      }
    }
  }
  return out;
}

namespace {
uint64_t splitmix64(uint64_t x) {
  uint64_t z = x + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
}  // namespace

// Uniform on [-1, 1) from (seed, counter): the 53 high bits of splitmix64.
double uniform_pm1(uint64_t seed, uint64_t counter) {
  const uint64_t key = splitmix64(seed ^ splitmix64(counter));
  return double(key >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

// Coherent orientation by breadth-first propagation over shared facets: two
// cells sharing a facet induce opposite orientations on it.
void compute_orientation(fq_mesh* m, const std::vector<int32_t>& facet_of_cell) {
  const int n = m->dim;
  const int nloc = n + 1;
  const int64_t nc = m->ncells;
  std::vector<int64_t> owner(static_cast<size_t>(m->nsimp[n - 1]), -1);
  std::vector<int64_t> other(static_cast<size_t>(nc * nloc), -1);
  for (int64_t c = 0; c < nc; ++c)
    for (int l = 0; l < nloc; ++l) {
      const int32_t f = facet_of_cell[c * nloc + l];
      if (owner[f] < 0) {
        owner[f] = c * nloc + l;
      } else {
        other[c * nloc + l] = owner[f];
        other[owner[f]] = c * nloc + l;
      }
    }
  // local facet l (colex) omits vertex position n - l: boundary sign (-1)^(n-l)
  auto lsign = [&](int l) { return ((n - l) % 2) ? -1 : 1; };
  m->orientation.assign(static_cast<size_t>(nc), 0);
  std::vector<int64_t> stack;
  for (int64_t root = 0; root < nc; ++root) {
    if (m->orientation[root]) continue;
    m->orientation[root] = 1;
    stack.push_back(root);
    while (!stack.empty()) {
      const int64_t c = stack.back();
      stack.pop_back();
      for (int l = 0; l < nloc; ++l) {
        const int64_t o = other[c * nloc + l];
        if (o < 0) continue;
        const int64_t oc = o / nloc;
        const int ol = int(o % nloc);
        const int want = -m->orientation[c] * lsign(l) * lsign(ol);
        if (!m->orientation[oc]) {
          m->orientation[oc] = int8_t(want);
          stack.push_back(oc);
        }
      }
    }
  }
}

}  // namespace fq
