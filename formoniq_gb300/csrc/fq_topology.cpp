// Host parts of the mesh topology: the Kuhn mesher
// (simplicial/src/mesher/grid.rs:77-98, with the vertex numbering of
// CartesianGrid, regge/src/mesher/cartesian.rs:158-226), the seeded uniform
// numbers of the synthetic meshes, and a coherent orientation
// (topology/orientation.rs), computed on demand. The skeletons, incidence and
// boundary are built on the device (fq_topology_gpu.cu).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "fq_internal.h"

namespace fq {

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
