// Symbolic analysis of the sparse direct solver (host, once per pattern):
// nested dissection of the Kuhn vertex lattice, the fronts, the assembly and
// extend-add maps, the level schedule. The numeric phase is fq_sparse_lu.cu.
#include <algorithm>
#include <cstring>
#include <numeric>

#include "fq_sparse_lu.h"

namespace fq {

namespace {

struct NdNode {
  int parent = -1, depth = 0;
  int child[2] = {-1, -1};
  int lo[4] = {0, 0, 0, 0}, hi[4] = {0, 0, 0, 0};
  int axis = -1, mid = 0;  // separator plane (axis < 0: a leaf)
};

constexpr int kLeafVertices = 8;  // a box of at most this many lattice points is a leaf
constexpr int kMaxFrontRows = 46000;

// The dissection tree of the lattice box [0, nbox]^dim (pre-order: a node
// before its children).
void build_tree(int dim, int nbox, std::vector<NdNode>& nodes) {
  struct Item {
    int lo[4], hi[4], parent, depth, slot;
  };
  std::vector<Item> stack;
  Item root{};
  for (int a = 0; a < dim; ++a) {
    root.lo[a] = 0;
    root.hi[a] = nbox;
  }
  root.parent = -1;
  root.depth = 0;
  root.slot = 0;
  stack.push_back(root);
  while (!stack.empty()) {
    Item it = stack.back();
    stack.pop_back();
    const int id = int(nodes.size());
    NdNode nd;
    nd.parent = it.parent;
    nd.depth = it.depth;
    int64_t nv = 1;
    int best = -1, ext = 0;
    for (int a = 0; a < dim; ++a) {
      nd.lo[a] = it.lo[a];
      nd.hi[a] = it.hi[a];
      const int e = it.hi[a] - it.lo[a] + 1;
      nv *= e;
      if (e > ext) {
        ext = e;
        best = a;
      }
    }
    if (it.parent >= 0) nodes[it.parent].child[it.slot] = id;
    if (nv <= kLeafVertices || ext < 3) {
      nodes.push_back(nd);
      continue;
    }
    nd.axis = best;
    nd.mid = (it.lo[best] + it.hi[best]) / 2;
    nodes.push_back(nd);
    Item l = it, r = it;
    l.hi[best] = nd.mid - 1;
    r.lo[best] = nd.mid + 1;
    l.parent = r.parent = id;
    l.depth = r.depth = it.depth + 1;
    l.slot = 0;
    r.slot = 1;
    stack.push_back(r);  // the left child is built first
    stack.push_back(l);
  }
}

// Every lattice point of the box lo..hi (inclusive), as a vertex id
// sum_a c_a (nbox+1)^a.
template <typename F>
void for_box(int dim, int nbox, const int* lo, const int* hi, F&& fn) {
  int c[4] = {0, 0, 0, 0};
  for (int a = 0; a < dim; ++a) {
    if (hi[a] < lo[a]) return;
    c[a] = lo[a];
  }
  while (true) {
    int64_t v = 0, stride = 1;
    for (int a = 0; a < dim; ++a) {
      v += c[a] * stride;
      stride *= nbox + 1;
    }
    fn(v);
    int a = 0;
    while (a < dim) {
      if (++c[a] <= hi[a]) break;
      c[a] = lo[a];
      ++a;
    }
    if (a == dim) break;
  }
}

}  // namespace

fq_status sparse_lu_analyse_host(fq_ctx* ctx, SparseLu& lu, int dim, int nbox, int64_t n, const int32_t* rp,
                                 const int32_t* ci, const int32_t* dof_vertices, SparseLuMaps& mp) {
  if (dim < 1 || dim > 4 || nbox < 1) return set_error(ctx, FQ_UNSUPPORTED, "sparse LU: needs a Kuhn lattice mesh");
  if (n <= 0) return set_error(ctx, FQ_INVALID_ARG, "sparse LU: empty system");
  if (n > (int64_t(1) << 30)) return set_error(ctx, FQ_UNSUPPORTED, "sparse LU: too many unknowns");
  std::vector<NdNode> nodes;
  build_tree(dim, nbox, nodes);
  const int nn = int(nodes.size());
  int64_t nverts = 1;
  for (int a = 0; a < dim; ++a) nverts *= nbox + 1;
  std::vector<int32_t> vnode(static_cast<size_t>(nverts), -1);
  for (int x = 0; x < nn; ++x) {
    const NdNode& nd = nodes[x];
    if (nd.axis < 0) {
      for_box(dim, nbox, nd.lo, nd.hi, [&](int64_t v) { vnode[v] = x; });
    } else {
      int lo[4], hi[4];
      std::memcpy(lo, nd.lo, sizeof lo);
      std::memcpy(hi, nd.hi, sizeof hi);
      lo[nd.axis] = hi[nd.axis] = nd.mid;
      for_box(dim, nbox, lo, hi, [&](int64_t v) { vnode[v] = x; });
    }
  }
  // Euler-tour intervals for the ancestor test; post-order
  std::vector<int> tin(nn), tout(nn), post;
  post.reserve(nn);
  {
    int clock = 0;
    std::vector<std::pair<int, int>> st{{0, 0}};
    while (!st.empty()) {
      auto& top = st.back();
      const int x = top.first;
      if (top.second == 0) tin[x] = clock++;
      if (top.second < 2) {
        const int c = nodes[x].child[top.second++];
        if (c >= 0) st.push_back({c, 0});
      } else {
        tout[x] = clock++;
        post.push_back(x);
        st.pop_back();
      }
    }
  }
  auto is_ancestor = [&](int a, int x) { return tin[a] <= tin[x] && tout[x] <= tout[a]; };
  // unknown -> node: the deepest node among its vertices' nodes; none: the root
  std::vector<int32_t> dnode(static_cast<size_t>(n));
  for (int64_t i = 0; i < n; ++i) {
    int best = 0, bd = -1;
    for (int q = 0; q < 5; ++q) {
      const int32_t v = dof_vertices[i * 5 + q];
      if (v < 0) continue;
      if (v >= nverts) return set_error(ctx, FQ_INVALID_ARG, "sparse LU: vertex outside the lattice");
      const int x = vnode[v];
      if (nodes[x].depth > bd) {
        bd = nodes[x].depth;
        best = x;
      }
    }
    for (int q = 0; q < 5; ++q) {
      const int32_t v = dof_vertices[i * 5 + q];
      if (v >= 0 && !is_ancestor(vnode[v], best))
        return set_error(ctx, FQ_UNSUPPORTED, "sparse LU: a simplex spans two dissection branches (not a Kuhn mesh)");
    }
    dnode[i] = best;
  }
  // elimination positions: nodes in post-order, unknowns in index order
  std::vector<int64_t> cnt(static_cast<size_t>(nn) + 1, 0);
  for (int64_t i = 0; i < n; ++i) cnt[dnode[i]]++;
  std::vector<int64_t> start(nn, 0);
  {
    int64_t acc = 0;
    for (int x : post) {
      start[x] = acc;
      acc += cnt[x];
    }
  }
  std::vector<int32_t> pos(static_cast<size_t>(n)), dof_at(static_cast<size_t>(n));
  {
    std::vector<int64_t> fill(start);
    for (int64_t i = 0; i < n; ++i) {
      const int64_t p = fill[dnode[i]]++;
      pos[i] = int32_t(p);
      dof_at[p] = int32_t(i);
    }
  }
  std::vector<int32_t> pnode(static_cast<size_t>(n));  // node of an elimination position
  for (int64_t i = 0; i < n; ++i) pnode[pos[i]] = dnode[i];
  // update sets, children first
  std::vector<std::vector<int32_t>> U(nn);
  std::vector<int32_t> cand;
  for (int x : post) {
    cand.clear();
    const int dx = nodes[x].depth;
    for (int64_t p = start[x]; p < start[x] + cnt[x]; ++p) {
      const int32_t i = dof_at[p];
      for (int32_t s = rp[i]; s < rp[i + 1]; ++s) {
        const int32_t j = ci[s];
        if (j < 0 || j >= n) return set_error(ctx, FQ_INVALID_ARG, "sparse LU: column index out of range");
        const int y = dnode[j];
        if (y == x) continue;
        if (nodes[y].depth < dx) {
          if (!is_ancestor(y, x)) return set_error(ctx, FQ_UNSUPPORTED, "sparse LU: coupling across dissection branches");
          cand.push_back(pos[j]);
        } else if (!is_ancestor(x, y)) {
          return set_error(ctx, FQ_UNSUPPORTED, "sparse LU: coupling across dissection branches");
        }
      }
    }
    for (int c : nodes[x].child)
      if (c >= 0)
        for (int32_t p : U[c])
          if (pnode[p] != x) cand.push_back(p);
    std::sort(cand.begin(), cand.end());
    cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
    U[x] = cand;
  }
  // levels
  std::vector<int> level(nn, 0);
  int nlev = 0;
  for (int x : post) {
    int l = 0;
    for (int c : nodes[x].child)
      if (c >= 0) l = std::max(l, level[c] + 1);
    level[x] = l;
    nlev = std::max(nlev, l + 1);
  }
  lu.n = n;
  lu.nnz = rp[n];
  lu.nfronts = nn;
  lu.nlevels = nlev;
  lu.front_m.assign(nn, 0);
  lu.front_f.assign(nn, 0);
  lu.front_off.assign(nn, 0);
  lu.front_start.assign(nn, 0);
  lu.parent.assign(nn, -1);
  lu.child0.assign(nn, -1);
  lu.child1.assign(nn, -1);
  for (int x = 0; x < nn; ++x) {
    lu.child0[x] = nodes[x].child[0];
    lu.child1[x] = nodes[x].child[1];
  }
  lu.level_ptr.assign(nlev + 1, 0);
  for (int x = 0; x < nn; ++x) lu.level_ptr[level[x] + 1]++;
  for (int l = 0; l < nlev; ++l) lu.level_ptr[l + 1] += lu.level_ptr[l];
  lu.level_fronts.assign(nn, 0);
  {
    std::vector<int32_t> fill(lu.level_ptr.begin(), lu.level_ptr.end() - 1);
    for (int x : post) lu.level_fronts[fill[level[x]]++] = x;
  }
  std::vector<FrontDesc> fd(nn);
  int64_t off = 0, toff = 0, eoff = 0, uoff = 0, roff = 0;
  double flops = 0.0;
  for (int l = 0; l < nlev; ++l) {
    for (int32_t q = lu.level_ptr[l]; q < lu.level_ptr[l + 1]; ++q) {
      const int x = lu.level_fronts[q];
      const int64_t f = cnt[x], u = int64_t(U[x].size()), m = f + u;
      if (m > kMaxFrontRows) return set_error(ctx, FQ_UNSUPPORTED, "sparse LU: a front beyond 46,000 rows");
      lu.front_m[x] = int32_t(m);
      lu.front_f[x] = int32_t(f);
      lu.front_off[x] = off;
      lu.front_start[x] = start[x];
      lu.parent[x] = nodes[x].parent;
      FrontDesc& d = fd[x];
      d.off = off;
      d.tile_off = toff;
      d.start = start[x];
      d.ea_off = eoff;
      d.uvec_off = uoff;
      d.roff = roff;
      d.m = int32_t(m);
      d.f = int32_t(f);
      d.parent = nodes[x].parent;
      d.child0 = nodes[x].child[0];
      d.child1 = nodes[x].child[1];
      d.pad = 0;
      const int64_t tiles = (f + kTile - 1) / kTile;
      off += m * m;
      toff += tiles * 2 * int64_t(kTile) * kTile;
      eoff += u;
      uoff += u;
      roff += m;
      const double df = double(f), du = double(u);
      flops += 2.0 / 3.0 * df * df * df + 2.0 * df * df * du + 2.0 * df * du * du;
    }
  }
  // tournament candidate sets of the widest level (fronts x leaves of 256 rows)
  lu.tourn_sets = 0;
  for (int l = 0; l < nlev; ++l) {
    int64_t maxf = 0;
    for (int32_t q = lu.level_ptr[l]; q < lu.level_ptr[l + 1]; ++q) maxf = std::max<int64_t>(maxf, cnt[lu.level_fronts[q]]);
    lu.tourn_sets = std::max<int64_t>(lu.tourn_sets, int64_t(lu.level_ptr[l + 1] - lu.level_ptr[l]) *
                                                         std::max<int64_t>(1, (maxf + 2 * kTile - 1) / (2 * kTile)));
  }
  lu.pool_elems = std::max<int64_t>(off, 1);
  lu.tile_elems = std::max<int64_t>(toff, 1);
  lu.uvec_elems = std::max<int64_t>(uoff, 1);
  lu.row_elems = std::max<int64_t>(roff, 1);
  lu.flops = flops;
  // front-local index of an elimination position
  auto local = [&](int x, int32_t p) -> int64_t {
    if (p >= start[x] && p < start[x] + cnt[x]) return p - start[x];
    auto it = std::lower_bound(U[x].begin(), U[x].end(), p);
    if (it == U[x].end() || *it != p) return -1;
    return cnt[x] + (it - U[x].begin());
  };
  // extend-add maps and update rows
  std::vector<int32_t> ea(static_cast<size_t>(std::max<int64_t>(eoff, 1))),
      ur(static_cast<size_t>(std::max<int64_t>(eoff, 1)));
  for (int x = 0; x < nn; ++x) {
    const int p = nodes[x].parent;
    for (size_t t = 0; t < U[x].size(); ++t) {
      ur[fd[x].ea_off + t] = U[x][t];
      const int64_t li = p >= 0 ? local(p, U[x][t]) : -1;
      if (p < 0 || li < 0) return set_error(ctx, FQ_CUDA_ERROR, "sparse LU: update unknown missing from the parent front");
      ea[fd[x].ea_off + t] = int32_t(li);
    }
  }
  // the extend-add maps inverted: per front row, its index among each child's
  // update unknowns (a child's map is one to one)
  std::vector<int32_t> rinv(static_cast<size_t>(2 * std::max<int64_t>(roff, 1)), -1);
  for (int x = 0; x < nn; ++x)
    for (int which = 0; which < 2; ++which) {
      const int c = nodes[x].child[which];
      if (c < 0) continue;
      for (int64_t t = 0; t < int64_t(U[c].size()); ++t) {
        const int64_t li = ea[fd[c].ea_off + t];
        if (li < 0 || li >= fd[x].m) return set_error(ctx, FQ_CUDA_ERROR, "sparse LU: an update row outside its parent");
        int32_t& slot = rinv[size_t(2 * (fd[x].roff + li) + which)];
        if (slot != -1) return set_error(ctx, FQ_CUDA_ERROR, "sparse LU: two update rows of a child on one parent row");
        slot = int32_t(t);
      }
    }
  // assembly map, grouped by level
  const int64_t nz = rp[n];
  std::vector<int64_t> aptr(nlev + 1, 0);
  std::vector<int32_t> sfront(static_cast<size_t>(std::max<int64_t>(nz, 1)));
  for (int64_t i = 0; i < n; ++i)
    for (int32_t s = rp[i]; s < rp[i + 1]; ++s) {
      const int32_t pi = pos[i], pj = pos[ci[s]];
      const int x = pnode[std::min(pi, pj)];
      sfront[s] = x;
      aptr[level[x] + 1]++;
    }
  for (int l = 0; l < nlev; ++l) aptr[l + 1] += aptr[l];
  std::vector<int32_t> aslot(static_cast<size_t>(std::max<int64_t>(nz, 1)));
  std::vector<int64_t> aoff(static_cast<size_t>(std::max<int64_t>(nz, 1)));
  std::vector<int32_t> arow(static_cast<size_t>(std::max<int64_t>(nz, 1)));
  {
    std::vector<int64_t> fill(aptr.begin(), aptr.end() - 1);
    for (int64_t i = 0; i < n; ++i)
      for (int32_t s = rp[i]; s < rp[i + 1]; ++s) {
        const int x = sfront[s];
        const int64_t lr = local(x, pos[i]), lc = local(x, pos[ci[s]]);
        if (lr < 0 || lc < 0) return set_error(ctx, FQ_CUDA_ERROR, "sparse LU: a slot outside its front");
        const int64_t q = fill[level[x]]++;
        aslot[q] = int32_t(s);
        arow[q] = int32_t(i);
        aoff[q] = fd[x].off + lc * fd[x].m + lr;
      }
  }
  lu.asm_ptr_h = aptr;
  // every index the kernels form stays inside its buffer
  for (int x = 0; x < nn; ++x) {
    const FrontDesc& d = fd[x];
    if (d.f > d.m || d.m < 0 || d.off + int64_t(d.m) * d.m > lu.pool_elems ||
        d.tile_off + ((int64_t(d.f) + kTile - 1) / kTile) * 2 * kTile * kTile > lu.tile_elems ||
        d.start + d.f > n || d.ea_off + (d.m - d.f) > std::max<int64_t>(eoff, 1) ||
        d.uvec_off + (d.m - d.f) > lu.uvec_elems || d.roff < 0 || d.roff + d.m > lu.row_elems)
      return set_error(ctx, FQ_CUDA_ERROR, "sparse LU: a front's ranges overrun their stores");
    for (int which = 0; which < 2; ++which) {
      const int c = which == 0 ? d.child0 : d.child1;
      if (c >= 0 && (c >= nn || fd[c].parent != x))
        return set_error(ctx, FQ_CUDA_ERROR, "sparse LU: a child that does not name its parent");
      for (int64_t i = 0; i < d.m; ++i) {
        const int32_t t = rinv[size_t(2 * (d.roff + i) + which)];
        if (t != -1 && (c < 0 || t < 0 || t >= fd[c].m - fd[c].f))
          return set_error(ctx, FQ_CUDA_ERROR, "sparse LU: an inverted update map entry outside its child");
      }
    }
    const int p = d.parent;
    if (d.m > d.f && p < 0) return set_error(ctx, FQ_CUDA_ERROR, "sparse LU: the root has update unknowns");
    for (int64_t t = 0; t < d.m - d.f; ++t)
      if (ea[d.ea_off + t] < 0 || ea[d.ea_off + t] >= fd[p].m || ur[d.ea_off + t] < 0 || ur[d.ea_off + t] >= n)
        return set_error(ctx, FQ_CUDA_ERROR, "sparse LU: an update map entry outside its parent front");
  }
  for (int64_t q = 0; q < nz; ++q)
    if (aoff[q] < 0 || aoff[q] >= lu.pool_elems || aslot[q] < 0 || aslot[q] >= nz || arow[q] < 0 || arow[q] >= n)
      return set_error(ctx, FQ_CUDA_ERROR, "sparse LU: an assembly offset outside the pool");
  mp.pos = std::move(pos);
  mp.fd = std::move(fd);
  mp.aslot = std::move(aslot);
  mp.arow = std::move(arow);
  mp.aoff = std::move(aoff);
  mp.ea = std::move(ea);
  mp.ur = std::move(ur);
  mp.rinv = std::move(rinv);
  return FQ_OK;
}

fq_status sparse_lu_analyse(fq_ctx* ctx, SparseLu& lu, int dim, int nbox, int64_t n, const int32_t* rp,
                            const int32_t* ci, const int32_t* dof_vertices) {
  SparseLuMaps mp;
  FQ_TRY(sparse_lu_analyse_host(ctx, lu, dim, nbox, n, rp, ci, dof_vertices, mp));
  const int nn = lu.nfronts;
  cudaStream_t st = ctx->stream;
  FQ_TRY(lu.perm.alloc(ctx, size_t(n) * 4));
  FQ_TRY(lu.fronts.alloc(ctx, sizeof(FrontDesc) * nn));
  FQ_TRY(lu.level_list.alloc(ctx, size_t(nn) * 4));
  FQ_TRY(lu.asm_slot.alloc(ctx, mp.aslot.size() * 4));
  FQ_TRY(lu.asm_off.alloc(ctx, mp.aoff.size() * 8));
  FQ_TRY(lu.asm_row.alloc(ctx, mp.arow.size() * 4));
  FQ_TRY(lu.ea_map.alloc(ctx, mp.ea.size() * 4));
  FQ_TRY(lu.urows.alloc(ctx, mp.ur.size() * 4));
  FQ_TRY(lu.rinv.alloc(ctx, mp.rinv.size() * 4));
  FQ_CUDA(ctx, cudaMemcpyAsync(lu.perm.p, mp.pos.data(), size_t(n) * 4, cudaMemcpyHostToDevice, st));
  FQ_CUDA(ctx, cudaMemcpyAsync(lu.fronts.p, mp.fd.data(), sizeof(FrontDesc) * nn, cudaMemcpyHostToDevice, st));
  FQ_CUDA(ctx, cudaMemcpyAsync(lu.level_list.p, lu.level_fronts.data(), size_t(nn) * 4, cudaMemcpyHostToDevice, st));
  FQ_CUDA(ctx, cudaMemcpyAsync(lu.asm_slot.p, mp.aslot.data(), mp.aslot.size() * 4, cudaMemcpyHostToDevice, st));
  FQ_CUDA(ctx, cudaMemcpyAsync(lu.asm_off.p, mp.aoff.data(), mp.aoff.size() * 8, cudaMemcpyHostToDevice, st));
  FQ_CUDA(ctx, cudaMemcpyAsync(lu.asm_row.p, mp.arow.data(), mp.arow.size() * 4, cudaMemcpyHostToDevice, st));
  FQ_CUDA(ctx, cudaMemcpyAsync(lu.ea_map.p, mp.ea.data(), mp.ea.size() * 4, cudaMemcpyHostToDevice, st));
  FQ_CUDA(ctx, cudaMemcpyAsync(lu.urows.p, mp.ur.data(), mp.ur.size() * 4, cudaMemcpyHostToDevice, st));
  FQ_CUDA(ctx, cudaMemcpyAsync(lu.rinv.p, mp.rinv.data(), mp.rinv.size() * 4, cudaMemcpyHostToDevice, st));
  FQ_CUDA(ctx, cudaStreamSynchronize(st));  // the host maps go out of scope
  return FQ_OK;
}

fq_status layout_dof_vertices(fq_ctx* ctx, const fq_mesh* m, int kind, int grade, int bc, int64_t nrows,
                              std::vector<int32_t>& out) {
  const Layout lay = make_layout(m->dim, kind, grade);
  out.assign(size_t(nrows) * 5, -1);
  int64_t row = 0;
  for (int b = 0; b < lay.nblocks; ++b) {
    const int g = lay.block_grade[b];
    if (g < 0 || g > m->dim) continue;
    for (int64_t s = 0; s < m->nsimp[g]; ++s) {
      if (bc == FQ_RELATIVE && m->boundary[g][s]) continue;
      if (row >= nrows) return set_error(ctx, FQ_INVALID_ARG, "sparse LU: layout larger than the system");
      for (int q = 0; q <= g; ++q) out[size_t(row) * 5 + q] = m->skel[g][size_t(s) * (g + 1) + q];
      ++row;
    }
  }
  return FQ_OK;
}

}  // namespace fq
