// Kernel (c) and its set-up: the scatter of per-cell element entries into a
// precomputed CSR pattern, atomic-free.
//
// The reference assembles by pushing every nonzero element entry as a COO
// triplet in cell order and letting the COO -> CSR conversion sum duplicates
// (formoniq/src/galerkin.rs:138-188). Here the (row, col) of every element entry
// is known before any value exists, so the set-up sorts the contributions once
// by (row, col) -- a stable radix sort, so within a slot they stay in cell order,
// the reference's summation order -- and the hot loop is then
//   element kernel:  values of every cell, entry-major (coalesced stores)
//   scatter kernel:  one thread per CSR slot sums its run of contributions
// with no atomics and a deterministic summation order. A slot whose every
// contribution is exactly 0.0 does not exist in the reference (the `val != 0.0`
// rule, galerkin.rs:173); such slots are flagged and compacted away.
#include <cub/cub.cuh>

#include <algorithm>
#include <cstdio>
#include <vector>

#include "fq_df64.cuh"
#include "fq_element_kernel.cuh"
#include "fq_internal.h"

namespace fq {

// ---------------------------------------------------------------------------
// Local layouts
// ---------------------------------------------------------------------------
Layout make_layout(int n, int kind, int K) {
  Layout L;
  auto push_grade = [&](int grade, int block, bool row, bool col) {
    const int cnt = (grade >= 0 && grade <= n) ? cbinom(n + 1, grade + 1) : 0;
    for (int l = 0; l < cnt; ++l) {
      if (row) {
        L.row_grade.push_back(grade);
        L.row_face.push_back(l);
        L.row_block.push_back(block);
      }
      if (col) {
        L.col_grade.push_back(grade);
        L.col_face.push_back(l);
        L.col_block.push_back(block);
      }
    }
  };
  bool sym = true;
  switch (kind) {
    case EK_MASS:
    case EK_HDIF:
      push_grade(K, 0, true, true);
      L.block_grade = {K};
      break;
    case EK_DIF_BOTH:
      push_grade(K - 1, 0, true, true);
      L.block_grade = {K - 1};
      break;
    case EK_DIF_TEST:
      push_grade(K - 1, 0, true, false);
      push_grade(K, 0, false, true);
      L.block_grade = {K - 1};
      sym = false;
      break;
    case EK_DIF_TRIAL:
      push_grade(K, 0, true, false);
      push_grade(K - 1, 0, false, true);
      L.block_grade = {K};
      sym = false;
      break;
    case EK_KKT:
      push_grade(K - 1, 0, true, true);  // kkt_sigma_local(n, K) dofs
      push_grade(K, 1, true, true);
      L.block_grade = {K - 1, K};
      break;
    case EK_DIRAC:
      for (int j = 0; j <= n; ++j) push_grade(j, j, true, true);
      for (int j = 0; j <= n; ++j) L.block_grade.push_back(j);
      break;
    default:
      break;
  }
  L.nblocks = int(L.block_grade.size());
  L.nrow_local = int(L.row_grade.size());
  L.ncol_local = int(L.col_grade.size());
  L.entry.assign(size_t(L.nrow_local) * L.ncol_local, -1);
  if (sym) {
    const int Lc = L.nrow_local;
    for (int i = 0; i < Lc; ++i)
      for (int j = 0; j < Lc; ++j) {
        const int a = std::min(i, j), b = std::max(i, j);
        bool zero = false;
        if (kind == EK_KKT && L.row_block[i] == 1 && L.row_block[j] == 1 && K == n) zero = true;  // dif_both(n+1)=0
        if (kind == EK_DIF_BOTH && K > n) zero = true;
        if (kind == EK_DIRAC && std::abs(L.row_grade[i] - L.row_grade[j]) >= 2) zero = true;
        if (!zero) L.entry[size_t(i) * Lc + j] = packed_index(a, b, Lc);
      }
    L.nent = (Lc * (Lc + 1)) / 2;
    if (kind == EK_KKT) {
      for (int i = 0; i < Lc; ++i) L.diag_entry.push_back(L.nent + i);
      L.nent += Lc;
    }
  } else {
    for (int i = 0; i < L.nrow_local; ++i)
      for (int j = 0; j < L.ncol_local; ++j) L.entry[size_t(i) * L.ncol_local + j] = i * L.ncol_local + j;
    L.nent = L.nrow_local * L.ncol_local;
  }
  return L;
}

// ---------------------------------------------------------------------------
// Plan construction (set-up, once per mesh and program)
// ---------------------------------------------------------------------------
struct KeyArgs {
  int64_t ncells;
  int lr, lc;
  const int32_t* entry;       // [lr*lc]
  const int32_t* row_src;     // per local row: pointer index into faces table
  const int32_t* col_src;
  const int64_t* row_off;     // per local row: global offset of its block
  const int64_t* col_off;
  const int32_t* const* faces;  // per (local row/col) : cell_faces[grade] + face*ncells
  const int32_t* const* rmaps;  // per local row: interior map or null
  const int32_t* const* cmaps;
  int64_t ncols;
  uint64_t sentinel;
  uint64_t* keys;
  int32_t* vals;
};

__global__ void plan_keys_kernel(KeyArgs a) {
  const int64_t per = int64_t(a.lr) * a.lc;
  const int64_t total = a.ncells * per;
  for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < total; t += int64_t(gridDim.x) * blockDim.x) {
    const int64_t c = t / per;
    const int rem = int(t - c * per);
    const int i = rem / a.lc, j = rem - (rem / a.lc) * a.lc;
    const int e = a.entry[rem];
    uint64_t key = a.sentinel;
    int32_t val = 0;
    if (e >= 0) {
      int64_t gi = a.faces[a.row_src[i]][c];
      int64_t gj = a.faces[a.col_src[j]][c];
      if (a.rmaps[i]) gi = a.rmaps[i][gi];
      if (a.cmaps[j]) gj = a.cmaps[j][gj];
      if (gi >= 0 && gj >= 0) {
        key = uint64_t(gi + a.row_off[i]) * uint64_t(a.ncols) + uint64_t(gj + a.col_off[j]);
        val = int32_t(int64_t(e) * a.ncells + c);
      }
    }
    a.keys[t] = key;
    a.vals[t] = val;
  }
}

__global__ void plan_diag_keys_kernel(KeyArgs a, const int32_t* diag_entry) {
  const int64_t total = a.ncells * a.lr;
  for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < total; t += int64_t(gridDim.x) * blockDim.x) {
    const int64_t c = t / a.lr;
    const int i = int(t - c * a.lr);
    int64_t gi = a.faces[a.row_src[i]][c];
    if (a.rmaps[i]) gi = a.rmaps[i][gi];
    uint64_t key = a.sentinel;
    int32_t val = 0;
    if (gi >= 0) {
      key = uint64_t(gi + a.row_off[i]);
      val = int32_t(int64_t(diag_entry[i]) * a.ncells + c);
    }
    a.keys[t] = key;
    a.vals[t] = val;
  }
}

// ptr[r] = first position p in sorted keys with key[p] >= r * stride, r in [0, nrows].
__global__ void lower_bound_rows_kernel(const uint64_t* keys, int64_t nkeys, int64_t nrows, uint64_t stride,
                                        int32_t* ptr) {
  for (int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; r <= nrows; r += int64_t(gridDim.x) * blockDim.x) {
    const uint64_t target = uint64_t(r) * stride;
    int64_t lo = 0, hi = nkeys;
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (keys[mid] < target)
        lo = mid + 1;
      else
        hi = mid;
    }
    ptr[r] = int32_t(lo);
  }
}

void launch_lower_bound_rows(const uint64_t* keys, int64_t nkeys, int64_t nrows, uint64_t stride, int32_t* out,
                             cudaStream_t st) {
  const int64_t b = std::max<int64_t>(1, std::min<int64_t>((nrows + 256) / 256, 152 * 32));
  lower_bound_rows_kernel<<<unsigned(b), 256, 0, st>>>(keys, nkeys, nrows, stride, out);
}

__global__ void col_from_key_kernel(const uint64_t* ukeys, int64_t n, uint64_t ncols, int32_t* col) {
  for (int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; s < n; s += int64_t(gridDim.x) * blockDim.x)
    col[s] = int32_t(ukeys[s] % ncols);
}

// ---- symmetric plans: the upper slots and their mirrors ----
__global__ void upper_flags_kernel(const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ col,
                                   int64_t nrows, int32_t* flag) {
  for (int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; r < nrows; r += int64_t(gridDim.x) * blockDim.x)
    for (int32_t s = row_ptr[r]; s < row_ptr[r + 1]; ++s) flag[s] = col[s] >= r ? 1 : 0;
}

// For every upper slot: its index, its mirror (binary search of the row in the
// mirror row's sorted columns; -1 if absent) and its contribution count.
__global__ void upper_list_kernel(const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ col,
                                  const int32_t* __restrict__ slot_ptr, const int32_t* __restrict__ flag,
                                  const int32_t* __restrict__ pos, int64_t nrows, int2* pair, int32_t* len) {
  for (int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; r < nrows; r += int64_t(gridDim.x) * blockDim.x)
    for (int32_t s = row_ptr[r]; s < row_ptr[r + 1]; ++s) {
      if (!flag[s]) continue;
      const int32_t c = col[s];
      int32_t lo = row_ptr[c], hi = row_ptr[c + 1];
      while (lo < hi) {
        const int32_t mid = (lo + hi) >> 1;
        if (col[mid] < int32_t(r))
          lo = mid + 1;
        else
          hi = mid;
      }
      const int32_t mirror = (lo < row_ptr[c + 1] && col[lo] == int32_t(r)) ? lo : -1;
      pair[pos[s]] = make_int2(s, mirror);
      len[pos[s]] = slot_ptr[s + 1] - slot_ptr[s];
    }
}

// One 16-byte record per upper slot with its first two contributions inline: the
// scatter then reaches the element values of most slots in two dependent loads
// (record, values) instead of three (pair and pointer, plan index, values).
__global__ void upper_rec_kernel(const int2* __restrict__ pair, const int32_t* __restrict__ up_ptr,
                                 const int32_t* __restrict__ up_perm, int64_t nup, int4* __restrict__ rec) {
  for (int64_t u = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; u < nup; u += int64_t(gridDim.x) * blockDim.x) {
    const int2 sm = pair[u];
    const int32_t b = up_ptr[u], e = up_ptr[u + 1];
    const int32_t p0 = e > b ? up_perm[b] : -1;
    const int32_t p1 = e - b == 2 ? up_perm[b + 1] : (e - b > 2 ? -(2 + (b + 1)) : -1);
    rec[u] = make_int4(sm.x, sm.y, p0, p1);
  }
}

// Slots with more than two contributions and their contributions past the first.
__global__ void upper_tail_kernel(const int32_t* __restrict__ up_ptr, int64_t nup,
                                  unsigned long long* __restrict__ out) {
  unsigned long long slots = 0, tail = 0;
  for (int64_t u = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; u < nup; u += int64_t(gridDim.x) * blockDim.x) {
    const int32_t c = up_ptr[u + 1] - up_ptr[u];
    if (c > 2) {
      slots += 1;
      tail += unsigned(c - 1);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    slots += __shfl_down_sync(0xffffffffu, slots, o);
    tail += __shfl_down_sync(0xffffffffu, tail, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(out, slots);
    atomicAdd(out + 1, tail);
  }
}

__global__ void upper_perm_kernel(const int2* __restrict__ pair, const int32_t* __restrict__ up_ptr,
                                  const int32_t* __restrict__ slot_ptr, const int32_t* __restrict__ perm, int64_t nup,
                                  int32_t* up_perm) {
  for (int64_t u = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; u < nup; u += int64_t(gridDim.x) * blockDim.x) {
    const int32_t s = pair[u].x, b = slot_ptr[s], e = slot_ptr[s + 1], o = up_ptr[u];
    for (int32_t t = b; t < e; ++t) up_perm[o + (t - b)] = perm[t];
  }
}

static int grid_for(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  return int(std::max<int64_t>(1, std::min<int64_t>(b, 152 * 32)));
}

static int bits_needed(uint64_t v) {
  int b = 1;
  while (b < 64 && (v >> b)) ++b;
  return b;
}

// Global block sizes and offsets for a layout under a boundary condition.
static std::vector<int64_t> block_offsets(const fq_mesh* m, const Layout& lay, int bc, int64_t* total) {
  std::vector<int64_t> off;
  int64_t acc = 0;
  for (int b = 0; b < lay.nblocks; ++b) {
    off.push_back(acc);
    const int g = lay.block_grade[b];
    int64_t sz = 0;
    if (g >= 0 && g <= m->dim) sz = bc == FQ_RELATIVE ? m->ninterior[g] : m->nsimp[g];
    acc += sz;
  }
  *total = acc;
  return off;
}

fq_status build_plan(fq_ctx* ctx, fq_mesh* m, Plan& plan, const Layout& lay) {
  cudaStream_t st = ctx->stream;
  const int64_t nc = m->ncells;
  // Row / column spaces. Column blocks follow the column grades.
  Layout colview = lay;
  int64_t nrows = 0, ncols = 0;
  auto roff = block_offsets(m, lay, plan.row_bc, &nrows);
  // Column blocks: same block structure, own grades (DIF_TEST/TRIAL have one
  // block each side with different grades).
  std::vector<int64_t> coff;
  {
    std::vector<int> cgrades;
    // distinct column blocks in order of appearance
    for (size_t j = 0; j < lay.col_block.size(); ++j) {
      const int b = lay.col_block[j];
      if (int(cgrades.size()) <= b) cgrades.resize(b + 1, -99);
      cgrades[b] = lay.col_grade[j];
    }
    int64_t acc = 0;
    for (size_t b = 0; b < cgrades.size(); ++b) {
      coff.push_back(acc);
      const int g = cgrades[b];
      int64_t sz = 0;
      if (g >= 0 && g <= m->dim) sz = plan.col_bc == FQ_RELATIVE ? m->ninterior[g] : m->nsimp[g];
      acc += sz;
    }
    ncols = acc;
  }
  plan.nrows = nrows;
  plan.ncols = ncols;
  plan.nent = lay.nent;
  const int lr = lay.nrow_local, lc = lay.ncol_local;

  // small device tables
  std::vector<const int32_t*> faces;
  std::vector<const int32_t*> rmaps(lr), cmaps(lc);
  std::vector<int32_t> row_src(lr), col_src(lc);
  std::vector<int64_t> row_off(lr), col_off(lc);
  for (int i = 0; i < lr; ++i) {
    const int g = lay.row_grade[i];
    row_src[i] = int32_t(faces.size());
    faces.push_back(m->cell_faces[g].as<int32_t>() + int64_t(lay.row_face[i]) * nc);
    rmaps[i] = plan.row_bc == FQ_RELATIVE ? m->interior_dev[g].as<int32_t>() : nullptr;
    row_off[i] = roff[lay.row_block[i]];
  }
  for (int j = 0; j < lc; ++j) {
    const int g = lay.col_grade[j];
    col_src[j] = int32_t(faces.size());
    faces.push_back(m->cell_faces[g].as<int32_t>() + int64_t(lay.col_face[j]) * nc);
    cmaps[j] = plan.col_bc == FQ_RELATIVE ? m->interior_dev[g].as<int32_t>() : nullptr;
    col_off[j] = coff[lay.col_block[j]];
  }
  // pack tables into one device buffer
  std::vector<char> blob;
  // Each table is copied with its exact size into a 16-byte aligned, zero-padded
  // slot; an empty table reads nothing.
  auto put = [&](const void* src, size_t bytes) {
    const size_t o = (blob.size() + 15) & ~size_t(15);
    blob.resize(o + bytes + 16, 0);
    if (bytes) memcpy(blob.data() + o, src, bytes);
    return o;
  };
  std::vector<int32_t> entry32(lay.entry.begin(), lay.entry.end());
  std::vector<int32_t> diag32(lay.diag_entry.begin(), lay.diag_entry.end());
  const size_t o_entry = put(entry32.data(), entry32.size() * 4);
  const size_t o_rsrc = put(row_src.data(), row_src.size() * 4);
  const size_t o_csrc = put(col_src.data(), col_src.size() * 4);
  const size_t o_roff = put(row_off.data(), row_off.size() * 8);
  const size_t o_coff = put(col_off.data(), col_off.size() * 8);
  const size_t o_faces = put(faces.data(), faces.size() * sizeof(void*));
  const size_t o_rmaps = put(rmaps.data(), rmaps.size() * sizeof(void*));
  const size_t o_cmaps = put(cmaps.data(), cmaps.size() * sizeof(void*));
  const size_t o_diag = put(diag32.data(), diag32.size() * 4);
  DevBuf tables;
  FQ_TRY(tables.alloc(ctx, blob.size()));
  FQ_CUDA(ctx, cudaMemcpyAsync(tables.p, blob.data(), blob.size(), cudaMemcpyHostToDevice, st));
  char* tb = tables.as<char>();

  KeyArgs ka;
  ka.ncells = nc;
  ka.lr = lr;
  ka.lc = lc;
  ka.entry = reinterpret_cast<const int32_t*>(tb + o_entry);
  ka.row_src = reinterpret_cast<const int32_t*>(tb + o_rsrc);
  ka.col_src = reinterpret_cast<const int32_t*>(tb + o_csrc);
  ka.row_off = reinterpret_cast<const int64_t*>(tb + o_roff);
  ka.col_off = reinterpret_cast<const int64_t*>(tb + o_coff);
  ka.faces = reinterpret_cast<const int32_t* const*>(tb + o_faces);
  ka.rmaps = reinterpret_cast<const int32_t* const*>(tb + o_rmaps);
  ka.cmaps = reinterpret_cast<const int32_t* const*>(tb + o_cmaps);
  ka.ncols = std::max<int64_t>(ncols, 1);
  ka.sentinel = uint64_t(std::max<int64_t>(nrows, 1)) * uint64_t(std::max<int64_t>(ncols, 1));
  const int end_bit = bits_needed(ka.sentinel);

  const int64_t total = nc * int64_t(lr) * lc;
  if (total >= (int64_t(1) << 31) || int64_t(lay.nent) * nc >= (int64_t(1) << 31))
    return set_error(ctx, FQ_UNSUPPORTED, "mesh too large for 32-bit scatter indices");
  DevBuf keys, keys2, vals, vals2;
  FQ_TRY(keys.alloc(ctx, std::max<int64_t>(total, 1) * 8));
  FQ_TRY(keys2.alloc(ctx, std::max<int64_t>(total, 1) * 8));
  FQ_TRY(vals.alloc(ctx, std::max<int64_t>(total, 1) * 4));
  FQ_TRY(vals2.alloc(ctx, std::max<int64_t>(total, 1) * 4));
  if (total > 0) {
    ka.keys = keys.as<uint64_t>();
    ka.vals = vals.as<int32_t>();
    plan_keys_kernel<<<grid_for(total, 256), 256, 0, st>>>(ka);
    ctx->launches++;
    size_t tmp_bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys.as<uint64_t>(), keys2.as<uint64_t>(),
                                    vals.as<int32_t>(), vals2.as<int32_t>(), int(total), 0, end_bit, st);
    DevBuf tmp;
    FQ_TRY(tmp.alloc(ctx, std::max<size_t>(tmp_bytes, 16)));
    FQ_CUDA(ctx, cub::DeviceRadixSort::SortPairs(tmp.p, tmp_bytes, keys.as<uint64_t>(), keys2.as<uint64_t>(),
                                                 vals.as<int32_t>(), vals2.as<int32_t>(), int(total), 0,
                                                 end_bit, st));
  }
  // run-length encode the sorted keys -> unique keys and counts
  DevBuf ukeys, counts, nruns;
  FQ_TRY(ukeys.alloc(ctx, std::max<int64_t>(total, 1) * 8));
  FQ_TRY(counts.alloc(ctx, (std::max<int64_t>(total, 1) + 1) * 4));
  FQ_TRY(nruns.alloc(ctx, 8));
  int64_t nruns_h = 0;
  if (total > 0) {
    size_t tmp_bytes = 0;
    cub::DeviceRunLengthEncode::Encode(nullptr, tmp_bytes, keys2.as<uint64_t>(), ukeys.as<uint64_t>(),
                                       counts.as<int32_t>(), nruns.as<int32_t>(), int(total), st);
    DevBuf tmp;
    FQ_TRY(tmp.alloc(ctx, std::max<size_t>(tmp_bytes, 16)));
    FQ_CUDA(ctx, cub::DeviceRunLengthEncode::Encode(tmp.p, tmp_bytes, keys2.as<uint64_t>(), ukeys.as<uint64_t>(),
                                                    counts.as<int32_t>(), nruns.as<int32_t>(), int(total), st));
    int32_t nr = 0;
    FQ_CUDA(ctx, cudaMemcpyAsync(&nr, nruns.p, 4, cudaMemcpyDeviceToHost, st));
    FQ_CUDA(ctx, cudaStreamSynchronize(st));
    nruns_h = nr;
    uint64_t lastkey = 0;
    if (nruns_h > 0) {
      FQ_CUDA(ctx, cudaMemcpyAsync(&lastkey, ukeys.as<uint64_t>() + (nruns_h - 1), 8, cudaMemcpyDeviceToHost, st));
      FQ_CUDA(ctx, cudaStreamSynchronize(st));
      if (lastkey == ka.sentinel) --nruns_h;
    }
  }
  plan.nslots = nruns_h;
  FQ_TRY(plan.slot_ptr.alloc(ctx, (nruns_h + 1) * 4));
  FQ_TRY(plan.col_idx.alloc(ctx, std::max<int64_t>(nruns_h, 1) * 4));
  FQ_TRY(plan.row_ptr.alloc(ctx, (nrows + 1) * 4));
  FQ_CUDA(ctx, cudaMemsetAsync(plan.slot_ptr.p, 0, 4, st));
  if (nruns_h > 0) {
    size_t tmp_bytes = 0;
    cub::DeviceScan::InclusiveSum(nullptr, tmp_bytes, counts.as<int32_t>(), plan.slot_ptr.as<int32_t>() + 1,
                                  int(nruns_h), st);
    DevBuf tmp;
    FQ_TRY(tmp.alloc(ctx, std::max<size_t>(tmp_bytes, 16)));
    FQ_CUDA(ctx, cub::DeviceScan::InclusiveSum(tmp.p, tmp_bytes, counts.as<int32_t>(),
                                               plan.slot_ptr.as<int32_t>() + 1, int(nruns_h), st));
    col_from_key_kernel<<<grid_for(nruns_h, 256), 256, 0, st>>>(ukeys.as<uint64_t>(), nruns_h, ka.ncols,
                                                                plan.col_idx.as<int32_t>());
    ctx->launches++;
  }
  lower_bound_rows_kernel<<<grid_for(nrows + 1, 256), 256, 0, st>>>(ukeys.as<uint64_t>(), nruns_h, nrows,
                                                                     uint64_t(ka.ncols), plan.row_ptr.as<int32_t>());
  ctx->launches++;
  int32_t ntrip = 0;
  FQ_CUDA(ctx, cudaMemcpyAsync(&ntrip, plan.slot_ptr.as<int32_t>() + nruns_h, 4, cudaMemcpyDeviceToHost, st));
  FQ_CUDA(ctx, cudaStreamSynchronize(st));
  plan.ntrip = ntrip;
  FQ_TRY(plan.perm.alloc(ctx, std::max<int64_t>(ntrip, 1) * 4));
  if (ntrip > 0)
    FQ_CUDA(ctx, cudaMemcpyAsync(plan.perm.p, vals2.p, size_t(ntrip) * 4, cudaMemcpyDeviceToDevice, st));

  // symmetric programs on one space: the upper half of the slots with mirrors
  const bool sym = plan.kind != EK_DIF_TEST && plan.kind != EK_DIF_TRIAL && plan.kind != EK_METRIC &&
                   plan.row_bc == plan.col_bc && nrows == ncols;
  if (sym && nruns_h > 0) {
    DevBuf flag, pos, len;
    FQ_TRY(flag.alloc(ctx, (nruns_h + 1) * 4));
    FQ_TRY(pos.alloc(ctx, (nruns_h + 1) * 4));
    FQ_CUDA(ctx, cudaMemsetAsync(flag.p, 0, (nruns_h + 1) * 4, st));
    upper_flags_kernel<<<grid_for(nrows, 256), 256, 0, st>>>(plan.row_ptr.as<int32_t>(), plan.col_idx.as<int32_t>(),
                                                             nrows, flag.as<int32_t>());
    size_t tmp_bytes = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, flag.as<int32_t>(), pos.as<int32_t>(), int(nruns_h + 1), st);
    DevBuf tmp;
    FQ_TRY(tmp.alloc(ctx, std::max<size_t>(tmp_bytes, 16)));
    FQ_CUDA(ctx, cub::DeviceScan::ExclusiveSum(tmp.p, tmp_bytes, flag.as<int32_t>(), pos.as<int32_t>(),
                                               int(nruns_h + 1), st));
    int32_t nup = 0;
    FQ_CUDA(ctx, cudaMemcpyAsync(&nup, pos.as<int32_t>() + nruns_h, 4, cudaMemcpyDeviceToHost, st));
    FQ_CUDA(ctx, cudaStreamSynchronize(st));
    plan.nup = nup;
    FQ_TRY(plan.up_pair.alloc(ctx, std::max<int64_t>(nup, 1) * 8));
    FQ_TRY(len.alloc(ctx, (int64_t(nup) + 1) * 4));
    FQ_TRY(plan.up_ptr.alloc(ctx, (int64_t(nup) + 1) * 4));
    FQ_CUDA(ctx, cudaMemsetAsync(len.p, 0, (int64_t(nup) + 1) * 4, st));
    upper_list_kernel<<<grid_for(nrows, 256), 256, 0, st>>>(
        plan.row_ptr.as<int32_t>(), plan.col_idx.as<int32_t>(), plan.slot_ptr.as<int32_t>(), flag.as<int32_t>(),
        pos.as<int32_t>(), nrows, plan.up_pair.as<int2>(), len.as<int32_t>());
    tmp_bytes = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, len.as<int32_t>(), plan.up_ptr.as<int32_t>(), int(nup + 1), st);
    DevBuf tmp2;
    FQ_TRY(tmp2.alloc(ctx, std::max<size_t>(tmp_bytes, 16)));
    FQ_CUDA(ctx, cub::DeviceScan::ExclusiveSum(tmp2.p, tmp_bytes, len.as<int32_t>(), plan.up_ptr.as<int32_t>(),
                                               int(nup + 1), st));
    int32_t ntu = 0;
    FQ_CUDA(ctx, cudaMemcpyAsync(&ntu, plan.up_ptr.as<int32_t>() + nup, 4, cudaMemcpyDeviceToHost, st));
    FQ_CUDA(ctx, cudaStreamSynchronize(st));
    plan.ntrip_up = ntu;
    FQ_TRY(plan.up_perm.alloc(ctx, std::max<int64_t>(ntu, 1) * 4));
    upper_perm_kernel<<<grid_for(nup, 256), 256, 0, st>>>(plan.up_pair.as<int2>(), plan.up_ptr.as<int32_t>(),
                                                         plan.slot_ptr.as<int32_t>(), plan.perm.as<int32_t>(), nup,
                                                         plan.up_perm.as<int32_t>());
    FQ_TRY(plan.up_rec.alloc(ctx, std::max<int64_t>(nup, 1) * 16));
    upper_rec_kernel<<<grid_for(nup, 256), 256, 0, st>>>(plan.up_pair.as<int2>(), plan.up_ptr.as<int32_t>(),
                                                        plan.up_perm.as<int32_t>(), nup, plan.up_rec.as<int4>());
    DevBuf tails;
    FQ_TRY(tails.alloc(ctx, 16));
    FQ_CUDA(ctx, cudaMemsetAsync(tails.p, 0, 16, st));
    upper_tail_kernel<<<grid_for(nup, 256), 256, 0, st>>>(plan.up_ptr.as<int32_t>(), nup,
                                                         tails.as<unsigned long long>());
    unsigned long long th[2] = {0, 0};
    FQ_CUDA(ctx, cudaMemcpyAsync(th, tails.p, 16, cudaMemcpyDeviceToHost, st));
    FQ_CUDA(ctx, cudaStreamSynchronize(st));
    plan.ntail_slots = int64_t(th[0]);
    plan.ntail = int64_t(th[1]);
    ctx->launches += 5;
  }

  // diagonal plan (preconditioner of the mixed system)
  if (!lay.diag_entry.empty()) {
    const int64_t dtotal = nc * lr;
    ka.sentinel = uint64_t(std::max<int64_t>(nrows, 1));
    ka.keys = keys.as<uint64_t>();
    ka.vals = vals.as<int32_t>();
    plan_diag_keys_kernel<<<grid_for(dtotal, 256), 256, 0, st>>>(ka, reinterpret_cast<const int32_t*>(tb + o_diag));
    ctx->launches++;
    size_t tmp_bytes = 0;
    const int dbits = bits_needed(ka.sentinel);
    cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys.as<uint64_t>(), keys2.as<uint64_t>(),
                                    vals.as<int32_t>(), vals2.as<int32_t>(), int(dtotal), 0, dbits, st);
    DevBuf tmp;
    FQ_TRY(tmp.alloc(ctx, std::max<size_t>(tmp_bytes, 16)));
    FQ_CUDA(ctx, cub::DeviceRadixSort::SortPairs(tmp.p, tmp_bytes, keys.as<uint64_t>(), keys2.as<uint64_t>(),
                                                 vals.as<int32_t>(), vals2.as<int32_t>(), int(dtotal), 0, dbits,
                                                 st));
    FQ_TRY(plan.diag_ptr.alloc(ctx, (nrows + 1) * 4));
    lower_bound_rows_kernel<<<grid_for(nrows + 1, 256), 256, 0, st>>>(keys2.as<uint64_t>(), dtotal, nrows, 1,
                                                                       plan.diag_ptr.as<int32_t>());
    ctx->launches++;
    int32_t nd = 0;
    FQ_CUDA(ctx, cudaMemcpyAsync(&nd, plan.diag_ptr.as<int32_t>() + nrows, 4, cudaMemcpyDeviceToHost, st));
    FQ_CUDA(ctx, cudaStreamSynchronize(st));
    plan.ndiag_trip = nd;
    FQ_TRY(plan.diag_perm.alloc(ctx, std::max<int64_t>(nd, 1) * 4));
    if (nd > 0)
      FQ_CUDA(ctx, cudaMemcpyAsync(plan.diag_perm.p, vals2.p, size_t(nd) * 4, cudaMemcpyDeviceToDevice, st));
  }
  FQ_CUDA(ctx, cudaStreamSynchronize(st));
  FQ_CUDA(ctx, cudaGetLastError());
  return FQ_OK;
}

// ---------------------------------------------------------------------------
// Hot loop: scatter
// ---------------------------------------------------------------------------
// The exact-zero test of the reference's `val != 0.0` rule on the bit pattern:
// integer instructions instead of an FP64 compare, +0.0 and -0.0 both zero.
__device__ __forceinline__ bool nonzero_bits(double v) { return (__double_as_longlong(v) << 1) != 0; }
__device__ __forceinline__ bool nonzero_bits(float v) { return (__float_as_int(v) << 1) != 0; }
__device__ __forceinline__ bool nonzero_bits(df64 v) { return nonzero_bits(v.hi) || nonzero_bits(v.lo); }
__device__ __forceinline__ double store_value(double v) { return v; }
__device__ __forceinline__ float store_value(float v) { return v; }
__device__ __forceinline__ double store_value(df64 v) { return v.to_double(); }

// Contributions of a slot whose loads a thread issues together.
constexpr int kScatterUnroll = 4;

// One thread per CSR slot; contributions summed in cell order. The plan
// indices of up to kScatterUnroll contributions are loaded together, then their
// element values, so a slot of up to four contributions (all of them on the 3D
// and 4D forms but the vertex masses) costs three dependent loads: slot_ptr,
// plan index, element value. E is the element type (df64, float or double), V
// the stored value type.
template <typename E, typename V>
__global__ void __launch_bounds__(256) scatter_kernel(const int32_t* __restrict__ slot_ptr,
                                                      const int32_t* __restrict__ perm, const E* __restrict__ elem,
                                                      V* __restrict__ values, uint8_t* __restrict__ zflag,
                                                      int* zero_count, int64_t nslots) {
  const int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (s >= nslots) return;
  const int b = __ldg(slot_ptr + s), e = __ldg(slot_ptr + s + 1);
  E acc = E(0);
  bool nz = false;
  for (int t = b; t < e; t += kScatterUnroll) {
    int p[kScatterUnroll];
#pragma unroll
    for (int u = 0; u < kScatterUnroll; ++u) p[u] = t + u < e ? __ldg(perm + t + u) : 0;
    E v[kScatterUnroll];
#pragma unroll
    for (int u = 0; u < kScatterUnroll; ++u) v[u] = t + u < e ? elem[p[u]] : E(0);
#pragma unroll
    for (int u = 0; u < kScatterUnroll; ++u)
      if (t + u < e) {
        acc += v[u];
        nz |= nonzero_bits(v[u]);
      }
  }
  values[s] = store_value(acc);
  if (zflag) zflag[s] = nz ? 0 : 1;
  if (!nz) atomicAdd(zero_count, 1);
}

// Symmetric plans: one thread per upper slot sums its contributions (in cell
// order, as scatter_kernel) and writes the value to the slot and its mirror.
// A mirror the pattern lacks (never, for a structurally symmetric program) sets
// status bit 2.
template <typename E, typename V>
__global__ void __launch_bounds__(256) scatter_sym_kernel(const int4* __restrict__ rec,
                                                          const int32_t* __restrict__ up_ptr,
                                                          const int32_t* __restrict__ perm,
                                                          const E* __restrict__ elem, V* __restrict__ values,
                                                          uint8_t* __restrict__ zflag, int* status, int64_t nup) {
  // The plan records are read once and the values written once per assembly:
  // streaming (evict-first) accesses, so that L2 keeps the element buffer the
  // element kernel has just written, which every gather reads. A record holds
  // the slot's first two contributions, so most slots need no plan index load.
  const int64_t u = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (u >= nup) return;
  const int4 r = __ldcs(rec + u);
  const E v0 = r.z >= 0 ? elem[r.z] : E(0);  // every slot has a contribution; guarded all the same
  const E v1 = r.w >= 0 ? elem[r.w] : E(0);
  E acc = v0;  // 0 + v0 is v0 (the element values are normalised float pairs)
  bool nz = nonzero_bits(v0);
  if (r.w >= 0) {
    acc += v1;
    nz |= nonzero_bits(v1);
  } else if (r.w < -1) {
    // more than two contributions: the rest, in order, from the plan
    const int e = __ldcs(up_ptr + u + 1);
    for (int t = -(r.w + 2); t < e; t += kScatterUnroll) {
      int p[kScatterUnroll];
#pragma unroll
      for (int k = 0; k < kScatterUnroll; ++k) p[k] = t + k < e ? __ldcs(perm + t + k) : 0;
      E v[kScatterUnroll];
#pragma unroll
      for (int k = 0; k < kScatterUnroll; ++k) v[k] = t + k < e ? elem[p[k]] : E(0);
#pragma unroll
      for (int k = 0; k < kScatterUnroll; ++k)
        if (t + k < e) {
          acc += v[k];
          nz |= nonzero_bits(v[k]);
        }
    }
  }
  const V out = store_value(acc);
  const uint8_t z = nz ? 0 : 1;
  __stcs(values + r.x, out);
  if (zflag) zflag[r.x] = z;
  int nzero = nz ? 0 : 1;
  if (r.y != r.x) {
    if (r.y >= 0) {
      __stcs(values + r.y, out);
      if (zflag) zflag[r.y] = z;
      nzero += nz ? 0 : 1;
    } else {
      atomicOr(status, 4);
    }
  }
  if (nzero) atomicAdd(status + 1, nzero);
}

// Symmetric plans, U upper slots per thread: a persistent grid walks the
// records in rounds of U * (grid threads); in a round, thread t handles the
// slots t, t + T, ..., t + (U-1) T (T = grid threads), so each of its U record
// loads is one coalesced warp transaction. All U records are loaded before any
// element value, and the next round's records are loaded before this round's
// gathers, so a thread keeps up to 2U record loads and 2U element gathers in
// flight where scatter_sym_kernel keeps one record, then two gathers. Every
// slot sums the same contributions in the same order as scatter_sym_kernel:
// the results are bit-identical.
template <typename E, typename V, int U>
__global__ void __launch_bounds__(256) scatter_sym_multi_kernel(const int4* __restrict__ rec,
                                                                const int32_t* __restrict__ up_ptr,
                                                                const int32_t* __restrict__ perm,
                                                                const E* __restrict__ elem, V* __restrict__ values,
                                                                uint8_t* __restrict__ zflag, int* status, int64_t nup) {
  const int64_t T = int64_t(gridDim.x) * blockDim.x;
  int nzero = 0;
  int4 nxt[U];
#pragma unroll
  for (int i = 0; i < U; ++i) {
    const int64_t u = int64_t(blockIdx.x) * blockDim.x + threadIdx.x + i * T;
    nxt[i] = u < nup ? __ldcs(rec + u) : make_int4(-1, -1, -1, -1);
  }
  for (int64_t t0 = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t0 < nup; t0 += U * T) {
    int4 r[U];
#pragma unroll
    for (int i = 0; i < U; ++i) r[i] = nxt[i];
    const int64_t t1 = t0 + U * T;
    if (t1 < nup) {
#pragma unroll
      for (int i = 0; i < U; ++i) {
        const int64_t u = t1 + i * T;
        nxt[i] = u < nup ? __ldcs(rec + u) : make_int4(-1, -1, -1, -1);
      }
    }
    E v0[U], v1[U];
#pragma unroll
    for (int i = 0; i < U; ++i) {
      v0[i] = r[i].z >= 0 ? elem[r[i].z] : E(0);
      v1[i] = r[i].w >= 0 ? elem[r[i].w] : E(0);
    }
#pragma unroll
    for (int i = 0; i < U; ++i) {
      if (r[i].x < 0) continue;  // past the end
      E acc = v0[i];
      bool nz = nonzero_bits(v0[i]);
      if (r[i].w >= 0) {
        acc += v1[i];
        nz |= nonzero_bits(v1[i]);
      } else if (r[i].w < -1) {
        const int e = __ldcs(up_ptr + (t0 + i * T) + 1);
        for (int t = -(r[i].w + 2); t < e; t += kScatterUnroll) {
          int p[kScatterUnroll];
#pragma unroll
          for (int k = 0; k < kScatterUnroll; ++k) p[k] = t + k < e ? __ldcs(perm + t + k) : 0;
          E v[kScatterUnroll];
#pragma unroll
          for (int k = 0; k < kScatterUnroll; ++k) v[k] = t + k < e ? elem[p[k]] : E(0);
#pragma unroll
          for (int k = 0; k < kScatterUnroll; ++k)
            if (t + k < e) {
              acc += v[k];
              nz |= nonzero_bits(v[k]);
            }
        }
      }
      const V out = store_value(acc);
      const uint8_t z = nz ? 0 : 1;
      __stcs(values + r[i].x, out);
      if (zflag) zflag[r[i].x] = z;
      nzero += nz ? 0 : 1;
      if (r[i].y != r[i].x) {
        if (r[i].y >= 0) {
          __stcs(values + r[i].y, out);
          if (zflag) zflag[r[i].y] = z;
          nzero += nz ? 0 : 1;
        } else {
          atomicOr(status, 4);
        }
      }
    }
  }
  if (nzero) atomicAdd(status + 1, nzero);
}

template <typename E>
__global__ void __launch_bounds__(256) scatter_diag_kernel(const int32_t* __restrict__ ptr,
                                                           const int32_t* __restrict__ perm,
                                                           const E* __restrict__ elem, double* __restrict__ out,
                                                           int64_t n) {
  const int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const int b = __ldg(ptr + s), e = __ldg(ptr + s + 1);
  E acc = E(0);
  for (int t = b; t < e; ++t) acc += elem[__ldg(perm + t)];
  out[s] = double(store_value(acc));
}

__global__ void df64_to_double_kernel(const df64* __restrict__ in, double* __restrict__ out, int64_t n) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    out[i] = in[i].to_double();
}

void launch_df64_to_double(const void* in, double* out, int64_t n, cudaStream_t st) {
  if (n <= 0) return;
  const int g = int(std::min<int64_t>((n + 255) / 256, 152 * 16));
  df64_to_double_kernel<<<g, 256, 0, st>>>(static_cast<const df64*>(in), out, n);
}

// The symmetric scatter with U slots per thread on a persistent grid of
// `bps` blocks of 256 threads per SM (bps 0: as many as are resident at once),
// at most enough blocks to give every thread one round.
template <typename E, typename V, int U>
static void launch_sym_multi(const Plan& plan, const E* elem, V* values, uint8_t* zero_flags, int* status, int bps,
                             cudaStream_t st) {
  static int sms = 0, resident = 0;  // per instantiation: the device's SMs and resident blocks of this kernel
  if (sms == 0) {
    int dev = 0, n = 152, r = 1;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, scatter_sym_multi_kernel<E, V, U>, 256, 0) != cudaSuccess)
      r = 1;
    resident = std::max(r, 1);
    sms = n;
  }
  const int per_sm = bps > 0 ? bps : resident;
  const int64_t need = (plan.nup + int64_t(256) * U - 1) / (int64_t(256) * U);
  const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>(need, int64_t(sms) * per_sm));
  scatter_sym_multi_kernel<E, V, U><<<unsigned(blocks), 256, 0, st>>>(plan.up_rec.as<int4>(), plan.up_ptr.as<int32_t>(),
                                                                        plan.up_perm.as<int32_t>(), elem, values,
                                                                        zero_flags, status, plan.nup);
}

template <typename E, typename V>
static bool launch_sym_shape(const Plan& plan, const E* elem, V* values, uint8_t* zero_flags, int* status,
                             ScatterShape shape, cudaStream_t st) {
  const int bps = shape.blocks_per_sm;
  switch (shape.slots_per_thread) {
    case 1: launch_sym_multi<E, V, 1>(plan, elem, values, zero_flags, status, bps, st); return true;
    case 2: launch_sym_multi<E, V, 2>(plan, elem, values, zero_flags, status, bps, st); return true;
    case 4: launch_sym_multi<E, V, 4>(plan, elem, values, zero_flags, status, bps, st); return true;
    case 8: launch_sym_multi<E, V, 8>(plan, elem, values, zero_flags, status, bps, st); return true;
    default: return false;
  }
}

void launch_scatter(const Plan& plan, const void* elem, void* values, uint8_t* zero_flags, int* status, int mode,
                    cudaStream_t st, ScatterShape shape) {
  if (plan.nslots == 0) return;
  int* zero_count = status + 1;
  if (plan.nup > 0) {
    if (shape.slots_per_thread < 0) shape.slots_per_thread = mode == FQ_FP64 ? 0 : 1;
    if (shape.slots_per_thread > 0) {
      bool done = false;
      if (mode == 1)
        done = launch_sym_shape(plan, static_cast<const float*>(elem), static_cast<float*>(values), zero_flags, status,
                                shape, st);
      else if (mode == 2)
        done = launch_sym_shape(plan, static_cast<const double*>(elem), static_cast<double*>(values), zero_flags,
                                status, shape, st);
      else
        done = launch_sym_shape(plan, static_cast<const df64*>(elem), static_cast<double*>(values), zero_flags,
                                status, shape, st);
      if (done) return;
    }
    const unsigned blocks = unsigned((plan.nup + 255) / 256);
    const int4* pr = plan.up_rec.as<int4>();
    const int32_t* up = plan.up_ptr.as<int32_t>();
    const int32_t* pm = plan.up_perm.as<int32_t>();
    if (mode == 1)
      scatter_sym_kernel<float, float><<<blocks, 256, 0, st>>>(pr, up, pm, static_cast<const float*>(elem),
                                                               static_cast<float*>(values), zero_flags, status,
                                                               plan.nup);
    else if (mode == 2)
      scatter_sym_kernel<double, double><<<blocks, 256, 0, st>>>(pr, up, pm, static_cast<const double*>(elem),
                                                                 static_cast<double*>(values), zero_flags, status,
                                                                 plan.nup);
    else
      scatter_sym_kernel<df64, double><<<blocks, 256, 0, st>>>(pr, up, pm, static_cast<const df64*>(elem),
                                                               static_cast<double*>(values), zero_flags, status,
                                                               plan.nup);
    return;
  }
  const int threads = 256;
  const unsigned blocks = unsigned((plan.nslots + threads - 1) / threads);
  const int32_t* sp = plan.slot_ptr.as<int32_t>();
  const int32_t* pm = plan.perm.as<int32_t>();
  if (mode == 1)
    scatter_kernel<float, float><<<blocks, threads, 0, st>>>(sp, pm, static_cast<const float*>(elem),
                                                             static_cast<float*>(values), zero_flags, zero_count,
                                                             plan.nslots);
  else if (mode == 2)
    scatter_kernel<double, double><<<blocks, threads, 0, st>>>(sp, pm, static_cast<const double*>(elem),
                                                               static_cast<double*>(values), zero_flags, zero_count,
                                                               plan.nslots);
  else
    scatter_kernel<df64, double><<<blocks, threads, 0, st>>>(sp, pm, static_cast<const df64*>(elem),
                                                             static_cast<double*>(values), zero_flags, zero_count,
                                                             plan.nslots);
}

void launch_scatter_diag(const Plan& plan, const void* elem, double* out, int mode, cudaStream_t st) {
  if (plan.nrows == 0) return;
  const int threads = 256;
  const unsigned blocks = unsigned((plan.nrows + threads - 1) / threads);
  const int32_t* dp = plan.diag_ptr.as<int32_t>();
  const int32_t* pm = plan.diag_perm.as<int32_t>();
  if (mode == 1)
    scatter_diag_kernel<float><<<blocks, threads, 0, st>>>(dp, pm, static_cast<const float*>(elem), out, plan.nrows);
  else if (mode == 2)
    scatter_diag_kernel<double><<<blocks, threads, 0, st>>>(dp, pm, static_cast<const double*>(elem), out,
                                                            plan.nrows);
  else
    scatter_diag_kernel<df64><<<blocks, threads, 0, st>>>(dp, pm, static_cast<const df64*>(elem), out, plan.nrows);
}

// ---------------------------------------------------------------------------
// Compaction of exact-zero slots (rare: unjittered meshes only)
// ---------------------------------------------------------------------------
__global__ void keep_kernel(const uint8_t* zflag, int64_t n, int32_t* keep) {
  const int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (s < n) keep[s] = zflag[s] ? 0 : 1;
  if (s == n) keep[s] = 0;
}

template <typename T>
__global__ void compact_kernel(const int32_t* pos, const uint8_t* zflag, const int32_t* col, const T* val,
                               int64_t n, int32_t* ncol, T* nval) {
  const int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (s >= n || zflag[s]) return;
  ncol[pos[s]] = col[s];
  nval[pos[s]] = val[s];
}

__global__ void compact_rows_kernel(const int32_t* pos, const int32_t* row_ptr, int64_t nrows, int32_t* nrow_ptr) {
  const int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (r <= nrows) nrow_ptr[r] = pos[row_ptr[r]];
}

fq_status compact_csr(fq_ctx* ctx, fq_matrix* m, int64_t nzero) {
  cudaStream_t st = ctx->stream;
  const Plan& p = *m->plan;
  const int64_t n = p.nslots;
  const size_t w = m->precision == FQ_FP32 ? 4 : 8;
  DevBuf keep, pos;
  FQ_TRY(keep.alloc(ctx, (n + 1) * 4));
  FQ_TRY(pos.alloc(ctx, (n + 1) * 4));
  keep_kernel<<<unsigned((n + 256) / 256), 256, 0, st>>>(m->zero_flags.as<uint8_t>(), n, keep.as<int32_t>());
  size_t tmp_bytes = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, keep.as<int32_t>(), pos.as<int32_t>(), int(n + 1), st);
  DevBuf tmp;
  FQ_TRY(tmp.alloc(ctx, std::max<size_t>(tmp_bytes, 16)));
  FQ_CUDA(ctx, cub::DeviceScan::ExclusiveSum(tmp.p, tmp_bytes, keep.as<int32_t>(), pos.as<int32_t>(), int(n + 1), st));
  const int64_t nnz = n - nzero;
  if (m->col_idx.bytes < size_t(std::max<int64_t>(nnz, 1)) * 4) FQ_TRY(m->col_idx.alloc(ctx, std::max<int64_t>(nnz, 1) * 4));
  if (m->row_ptr.bytes < size_t(p.nrows + 1) * 4) FQ_TRY(m->row_ptr.alloc(ctx, (p.nrows + 1) * 4));
  if (m->values.bytes < size_t(std::max<int64_t>(nnz, 1)) * w) FQ_TRY(m->values.alloc(ctx, std::max<int64_t>(nnz, 1) * w));
  if (w == 4)
    compact_kernel<float><<<unsigned((n + 255) / 256), 256, 0, st>>>(
        pos.as<int32_t>(), m->zero_flags.as<uint8_t>(), p.col_idx.as<int32_t>(), m->full_values.as<float>(), n,
        m->col_idx.as<int32_t>(), m->values.as<float>());
  else
    compact_kernel<double><<<unsigned((n + 255) / 256), 256, 0, st>>>(
        pos.as<int32_t>(), m->zero_flags.as<uint8_t>(), p.col_idx.as<int32_t>(), m->full_values.as<double>(), n,
        m->col_idx.as<int32_t>(), m->values.as<double>());
  compact_rows_kernel<<<unsigned((p.nrows + 256) / 256), 256, 0, st>>>(pos.as<int32_t>(), p.row_ptr.as<int32_t>(),
                                                                      p.nrows, m->row_ptr.as<int32_t>());
  ctx->launches += 3;
  FQ_CUDA(ctx, cudaStreamSynchronize(st));
  m->nnz = nnz;
  m->rp = m->row_ptr.as<int32_t>();
  m->ci = m->col_idx.as<int32_t>();
  m->compacted = true;
  return FQ_OK;
}

// ---------------------------------------------------------------------------
// Element pass and assembly driver
// ---------------------------------------------------------------------------
// The type of the element buffer a program writes, as a precision mode: the 4D
// Dirac program (all five grades coupled, 31 local dofs) runs in IEEE double
// in FQ_FP64 too (no configuration needs it fast and its float-float build is
// large), so its buffer holds doubles, and its scatter must read doubles.
int element_buffer_mode(int n, int kind, int mode) {
  return (n == 4 && kind == EK_DIRAC && mode == FQ_FP64) ? FQ_FP64_IEEE : mode;
}

template <int N>
static int launch_dim(int grade, int kind, int mode, const ElemArgs& a, cudaStream_t st) {
  if (kind == EK_METRIC || mode == 2 || (N == 4 && kind == EK_DIRAC)) return launch_typed<N, double>(grade, kind, a, st);
  if (mode == 1) return launch_typed<N, float>(grade, kind, a, st);
  return launch_typed<N, df64>(grade, kind, a, st);
}

int launch_element(int n, int grade, int kind, int mode, const ElemArgs& a, cudaStream_t st) {
  switch (n) {
    case 0:
      return launch_dim<0>(grade, kind, mode, a, st);
    case 1:
      return launch_dim<1>(grade, kind, mode, a, st);
    case 2:
      return launch_dim<2>(grade, kind, mode, a, st);
    case 3:
      return launch_dim<3>(grade, kind, mode, a, st);
    case 4:
      return launch_dim<4>(grade, kind, mode, a, st);
    default:
      return -1;
  }
}

int launch_element_multi(int n, int mode, const ElemMultiArgs& a, cudaStream_t st) {
  auto typed = [&](auto tag) -> int {
    using T = decltype(tag);
    switch (n) {
      case 1:
        return launch_multi_typed<1, T>(a, st);
      case 2:
        return launch_multi_typed<2, T>(a, st);
      case 3:
        return launch_multi_typed<3, T>(a, st);
      default:
        return -1;
    }
  };
  if (mode == FQ_FP32) return typed(float());
  if (mode == FQ_FP64_IEEE) return typed(double());
  return typed(df64());
}

fq_status element_pass(fq_ctx* ctx, fq_mesh* m, int kind, int grade, int mode, double param, DevBuf& buf,
                       int nent) {
  if (!m->has_lengths) return set_error(ctx, FQ_INVALID_ARG, "mesh has no edge lengths");
  const size_t need = size_t(std::max(nent, 1)) * size_t(std::max<int64_t>(m->ncells, 1)) * (mode == 1 ? 4 : 8);
  if (buf.bytes < need) FQ_TRY(buf.alloc(ctx, need));
  ElemArgs a;
  a.ncells = m->ncells;
  a.lengths = m->lengths.as<double>();
  a.cell_edges = m->dim >= 1 ? m->cell_faces[1].as<int32_t>() : nullptr;
  a.out = buf.p;
  a.ginv_out = a.det_out = a.vol_out = nullptr;
  a.param = param;
  a.status = ctx->status.as<int>();
  a.nent = nent;
  if (launch_element(m->dim, grade, kind, mode, a, ctx->stream) != 0)
    return set_error(ctx, FQ_UNSUPPORTED, "no element program for this dimension/grade");
  ctx->launches++;
  FQ_CUDA(ctx, cudaGetLastError());
  return FQ_OK;
}

fq_status get_plan(fq_ctx* ctx, fq_mesh* m, int kind, int grade, int row_bc, int col_bc, Plan** out) {
  auto key = std::make_tuple(kind, grade, row_bc, col_bc);
  auto it = m->plans.find(key);
  if (it != m->plans.end()) {
    *out = it->second.get();
    return FQ_OK;
  }
  auto plan = std::make_unique<Plan>();
  plan->kind = kind;
  plan->grade = grade;
  plan->row_bc = row_bc;
  plan->col_bc = col_bc;
  Layout lay = make_layout(m->dim, kind, grade);
  FQ_TRY(build_plan(ctx, m, *plan, lay));
  *out = plan.get();
  m->plans[key] = std::move(plan);
  return FQ_OK;
}

// Queues the element pass and the scatter of m on the context's stream: status
// bits go to ctx->status[0], the count of all-zero slots to ctx->status[1]. With
// `ev` (four events) the two kernels are bracketed for profiling. Per-slot
// zero flags are written only `with_flags` (the rare re-assembly that a
// nonzero count triggers, assemble_flagged).
static fq_status assemble_launch(fq_ctx* ctx, fq_matrix* m, cudaEvent_t* ev, bool with_flags = false) {
  fq_mesh* mesh = m->mesh;
  Plan& p = *m->plan;
  const int mode = m->precision;
  const size_t w = mode == FQ_FP32 ? 4 : 8;
  if (m->full_values.bytes < size_t(std::max<int64_t>(p.nslots, 1)) * w)
    FQ_TRY(m->full_values.alloc(ctx, std::max<int64_t>(p.nslots, 1) * w));
  if (m->zero_flags.bytes < size_t(std::max<int64_t>(p.nslots, 1)))
    FQ_TRY(m->zero_flags.alloc(ctx, std::max<int64_t>(p.nslots, 1)));
  int* zc = ctx->status.as<int>();
  if (ev) FQ_CUDA(ctx, cudaEventRecord(ev[0], ctx->stream));
  if (p.nslots > 0 || p.ndiag_trip > 0) FQ_TRY(element_pass(ctx, mesh, m->kind, m->grade, mode, m->param, mesh->elem, p.nent));
  if (ev) FQ_CUDA(ctx, cudaEventRecord(ev[1], ctx->stream));
  if (ev) FQ_CUDA(ctx, cudaEventRecord(ev[2], ctx->stream));
  launch_scatter(p, mesh->elem.p, m->full_values.p, with_flags ? m->zero_flags.as<uint8_t>() : nullptr, zc,
                 element_buffer_mode(mesh->dim, m->kind, mode), ctx->stream, ctx->scatter_shape);
  if (ev) FQ_CUDA(ctx, cudaEventRecord(ev[3], ctx->stream));
  if (p.nslots > 0) ctx->launches++;
  return FQ_OK;
}

// Matrices per multi-program element pass of a device multi-matrix assembly.
// Measured on the 3D 32^3 step of four forms: one pass 0.181 ms per step, two
// passes of two 0.187 ms (each runs the multi-program kernel's register
// allocation; fewer live element buffers only partly make up for it).
constexpr int kMultiChunk = kMultiPrograms;

// Whether the matrices can share one multi-program element pass: 2 to
// kMultiPrograms mass / dif_both matrices of one mesh of dimension 1-3 in one
// precision, each with slots.
static bool multi_fusable(fq_matrix* const* mats, int count) {
  if (count < 2 || count > kMultiPrograms || !mats[0]->plan) return false;
  const fq_mesh* mesh = mats[0]->mesh;
  const int mode = mats[0]->precision;
  if (mesh->dim < 1 || mesh->dim > 3 || !mesh->has_lengths) return false;
  for (int i = 0; i < count; ++i) {
    const fq_matrix* m = mats[i];
    if (!m->plan || m->mesh != mesh || m->precision != mode || m->plan->nslots <= 0) return false;
    if (!(m->kind == EK_MASS || (m->kind == EK_DIF_BOTH && m->grade >= 1)) || m->grade > mesh->dim) return false;
    if (element_buffer_mode(mesh->dim, m->kind, mode) != mode) return false;
  }
  return true;
}

// The multi-program element pass of fusable matrices into their own buffers.
static fq_status multi_element_pass(fq_ctx* ctx, fq_matrix* const* mats, int count) {
  fq_mesh* mesh = mats[0]->mesh;
  const int mode = mats[0]->precision;
  const size_t w = mode == FQ_FP32 ? 4 : 8;
  ElemMultiArgs a{};
  a.ncells = mesh->ncells;
  a.lengths = mesh->lengths.as<double>();
  a.cell_edges = mesh->cell_faces[1].as<int32_t>();
  a.status = ctx->status.as<int>();
  a.nprog = count;
  for (int i = 0; i < count; ++i) {
    fq_matrix* m = mats[i];
    const size_t need = size_t(std::max(m->plan->nent, 1)) * size_t(std::max<int64_t>(mesh->ncells, 1)) * w;
    if (m->elem.bytes < need) FQ_TRY(m->elem.alloc(ctx, need));
    a.kind[i] = m->kind;
    a.grade[i] = m->grade;
    a.nent[i] = m->plan->nent;
    a.out[i] = m->elem.p;
  }
  if (launch_element_multi(mesh->dim, mode, a, ctx->stream) != 0)
    return set_error(ctx, FQ_UNSUPPORTED, "no multi-program element pass for this dimension");
  ctx->launches++;
  FQ_CUDA(ctx, cudaGetLastError());
  return FQ_OK;
}

// The scatter of a matrix whose element pass has run into `elem`.
static fq_status scatter_launch(fq_ctx* ctx, fq_matrix* m, const void* elem, cudaEvent_t* ev) {
  Plan& p = *m->plan;
  const int mode = m->precision;
  const size_t w = mode == FQ_FP32 ? 4 : 8;
  if (m->full_values.bytes < size_t(std::max<int64_t>(p.nslots, 1)) * w)
    FQ_TRY(m->full_values.alloc(ctx, std::max<int64_t>(p.nslots, 1) * w));
  if (m->zero_flags.bytes < size_t(std::max<int64_t>(p.nslots, 1)))
    FQ_TRY(m->zero_flags.alloc(ctx, std::max<int64_t>(p.nslots, 1)));
  if (ev) FQ_CUDA(ctx, cudaEventRecord(ev[2], ctx->stream));
  launch_scatter(p, elem, m->full_values.p, nullptr, ctx->status.as<int>(),
                 element_buffer_mode(m->mesh->dim, m->kind, mode), ctx->stream, ctx->scatter_shape);
  if (ev) FQ_CUDA(ctx, cudaEventRecord(ev[3], ctx->stream));
  if (p.nslots > 0) ctx->launches++;
  return FQ_OK;
}

static fq_status accumulate_profile(fq_ctx* ctx, cudaEvent_t* ev) {
  float a = 0.f, b = 0.f;
  FQ_CUDA(ctx, cudaEventElapsedTime(&a, ev[0], ev[1]));
  FQ_CUDA(ctx, cudaEventElapsedTime(&b, ev[2], ev[3]));
  ctx->prof_ms[0] += a;
  ctx->prof_ms[1] += b;
  ctx->prof_n[0] += 1;
  ctx->prof_n[1] += 1;
  return FQ_OK;
}

// After the stream has drained: the scatter output becomes the matrix values,
// or, when `nzero` slots summed exact zeros only, the compacted CSR.
static fq_status assemble_adopt(fq_ctx* ctx, fq_matrix* m, int64_t nzero) {
  Plan& p = *m->plan;
  if (nzero > 0) return compact_csr(ctx, m, nzero);
  m->nnz = p.nslots;
  m->rp = p.row_ptr.as<int32_t>();
  m->ci = p.col_idx.as<int32_t>();
  m->compacted = false;
  // values live in full_values: swap roles to avoid a copy
  std::swap(m->values, m->full_values);
  return FQ_OK;
}

static fq_status check_status_words(fq_ctx* ctx) {
  if (ctx->host_status[0] & 4) return set_error(ctx, FQ_CUDA_ERROR, "symmetric plan without a mirror slot");
  if (ctx->host_status[0] & 2) return set_error(ctx, FQ_INVALID_ARG, "element program wrote outside its layout");
  if (ctx->host_status[0] & 1) return set_error(ctx, FQ_DEGENERATE_CELL, "a cell metric is singular or not finite");
  return FQ_OK;
}

// The rare path: some slot summed exact zeros only. m is assembled again with
// per-slot flags and the count of its all-zero slots is returned.
static fq_status assemble_flagged(fq_ctx* ctx, fq_matrix* m, int64_t* nzero) {
  FQ_CUDA(ctx, cudaMemsetAsync(ctx->status.p, 0, 8 * sizeof(int), ctx->stream));
  FQ_TRY(assemble_launch(ctx, m, nullptr, true));
  FQ_CUDA(ctx, cudaMemcpyAsync(ctx->host_status, ctx->status.p, 8 * sizeof(int), cudaMemcpyDeviceToHost,
                               ctx->stream));
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  FQ_TRY(check_status_words(ctx));
  *nzero = ctx->host_status[1];
  return FQ_OK;
}

// Element pass + scatter (+ compaction when needed) into m.
fq_status assemble_into(fq_ctx* ctx, fq_matrix* m) {
  FQ_CUDA(ctx, cudaMemsetAsync(ctx->status.p, 0, 8 * sizeof(int), ctx->stream));
  cudaEvent_t* ev = ctx->profiling && ctx->ev[0] ? ctx->ev : nullptr;
  FQ_TRY(assemble_launch(ctx, m, ev));
  FQ_CUDA(ctx, cudaMemcpyAsync(ctx->host_status, ctx->status.p, 8 * sizeof(int), cudaMemcpyDeviceToHost,
                               ctx->stream));
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (ev) FQ_TRY(accumulate_profile(ctx, ev));
  FQ_TRY(check_status_words(ctx));
  int64_t nzero = 0;
  if (ctx->host_status[1] > 0) FQ_TRY(assemble_flagged(ctx, m, &nzero));
  return assemble_adopt(ctx, m, nzero);
}


// Several matrices queued back to back with one read of the status words. The
// element buffer of a mesh is reused in stream order; when some slot summed
// exact zeros only (rare), every matrix is assembled again with flags.
fq_status assemble_many(fq_ctx* ctx, fq_matrix* const* mats, int count) {
  const bool prof = ctx->profiling && ctx->ev[0];
  if (prof) {
    while (ctx->prof_events.size() < size_t(count) * 4) {
      cudaEvent_t e;
      FQ_CUDA(ctx, cudaEventCreate(&e));
      ctx->prof_events.push_back(e);
    }
  }
  FQ_CUDA(ctx, cudaMemsetAsync(ctx->status.p, 0, 8 * sizeof(int), ctx->stream));
  for (int i0 = 0; i0 < count; i0 += kMultiChunk) {
    const int nc = std::min(kMultiChunk, count - i0);
    if (multi_fusable(mats + i0, nc)) {
      // one element pass for the chunk (the metric once per cell), then its scatters;
      // the pass's time is the chunk's first matrix's element time, the others' zero
      cudaEvent_t* ev = prof ? ctx->prof_events.data() + 4 * i0 : nullptr;
      if (ev) FQ_CUDA(ctx, cudaEventRecord(ev[0], ctx->stream));
      FQ_TRY(multi_element_pass(ctx, mats + i0, nc));
      if (ev) FQ_CUDA(ctx, cudaEventRecord(ev[1], ctx->stream));
      for (int i = i0; i < i0 + nc; ++i) {
        cudaEvent_t* e = prof ? ctx->prof_events.data() + 4 * i : nullptr;
        if (e && i > i0) {
          FQ_CUDA(ctx, cudaEventRecord(e[0], ctx->stream));
          FQ_CUDA(ctx, cudaEventRecord(e[1], ctx->stream));
        }
        FQ_TRY(scatter_launch(ctx, mats[i], mats[i]->elem.p, e));
      }
    } else {
      for (int i = i0; i < i0 + nc; ++i)
        if (mats[i]->plan) FQ_TRY(assemble_launch(ctx, mats[i], prof ? ctx->prof_events.data() + 4 * i : nullptr));
    }
  }
  FQ_CUDA(ctx, cudaMemcpyAsync(ctx->host_status, ctx->status.p, 8 * sizeof(int), cudaMemcpyDeviceToHost,
                               ctx->stream));
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (prof)
    for (int i = 0; i < count; ++i)
      if (mats[i]->plan) FQ_TRY(accumulate_profile(ctx, ctx->prof_events.data() + 4 * i));
  FQ_TRY(check_status_words(ctx));
  const bool any_zero = ctx->host_status[1] > 0;
  for (int i = 0; i < count; ++i) {
    fq_matrix* m = mats[i];
    if (!m->plan) continue;
    int64_t nzero = 0;
    if (any_zero && m->plan->nslots > 0) FQ_TRY(assemble_flagged(ctx, m, &nzero));
    FQ_TRY(assemble_adopt(ctx, m, nzero));
  }
  return FQ_OK;
}

// The host-buffer form of assemble_many for one mesh: the lengths go up once,
// and the values of every matrix come down on a second stream while the next
// matrix's kernels run (the copy of matrix i waits on an event after its
// scatter). A matrix that was compacted before, or that compacts now, is
// downloaded after the status read instead (its value count is known only then).
fq_status assemble_host_many(fq_ctx* ctx, fq_mesh* mesh, const double* lengths, fq_matrix* const* mats,
                             void* const* out, int count) {
  cudaStream_t st = ctx->stream;
  if (!ctx->copy_stream) FQ_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
  while (ctx->copy_events.size() < size_t(count) + 1) {
    cudaEvent_t e;
    FQ_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    ctx->copy_events.push_back(e);
  }
  const int64_t ne = mesh->dim >= 1 ? mesh->nsimp[1] : 0;
  if (mesh->lengths.bytes < size_t(std::max<int64_t>(ne, 1)) * 8)
    FQ_TRY(mesh->lengths.alloc(ctx, std::max<int64_t>(ne, 1) * 8));
  if (ne > 0) FQ_CUDA(ctx, cudaMemcpyAsync(mesh->lengths.p, lengths, ne * 8, cudaMemcpyHostToDevice, st));
  mesh->has_lengths = true;
  FQ_CUDA(ctx, cudaMemsetAsync(ctx->status.p, 0, 8 * sizeof(int), st));
  std::vector<char> streamed(size_t(count), 0);
  // per matrix (no multi-program pass): the first download starts after the
  // first matrix's scatter, not after one pass over every program
  for (int i = 0; i < count; ++i) {
    fq_matrix* m = mats[i];
    if (!m->plan) continue;
    FQ_TRY(assemble_launch(ctx, m, nullptr));
    if (!m->compacted && m->plan->nslots > 0) {
      const size_t w = m->precision == FQ_FP32 ? 4 : 8;
      FQ_CUDA(ctx, cudaEventRecord(ctx->copy_events[i], st));
      FQ_CUDA(ctx, cudaStreamWaitEvent(ctx->copy_stream, ctx->copy_events[i], 0));
      FQ_CUDA(ctx, cudaMemcpyAsync(out[i], m->full_values.p, size_t(m->plan->nslots) * w, cudaMemcpyDeviceToHost,
                                   ctx->copy_stream));
      streamed[i] = 1;
    }
  }
  // the caller's stream resumes after the downloads
  FQ_CUDA(ctx, cudaEventRecord(ctx->copy_events[count], ctx->copy_stream));
  FQ_CUDA(ctx, cudaStreamWaitEvent(st, ctx->copy_events[count], 0));
  FQ_CUDA(ctx, cudaMemcpyAsync(ctx->host_status, ctx->status.p, 8 * sizeof(int), cudaMemcpyDeviceToHost, st));
  FQ_CUDA(ctx, cudaStreamSynchronize(st));
  FQ_TRY(check_status_words(ctx));
  const bool any_zero = ctx->host_status[1] > 0;
  for (int i = 0; i < count; ++i) {
    fq_matrix* m = mats[i];
    if (!m->plan) continue;
    int64_t nzero = 0;
    if (any_zero && m->plan->nslots > 0) FQ_TRY(assemble_flagged(ctx, m, &nzero));
    FQ_TRY(assemble_adopt(ctx, m, nzero));
    if ((!streamed[i] || nzero > 0) && m->nnz > 0) {
      const size_t w = m->precision == FQ_FP32 ? 4 : 8;
      FQ_CUDA(ctx, cudaMemcpyAsync(out[i], m->values.p, size_t(m->nnz) * w, cudaMemcpyDeviceToHost, st));
      FQ_CUDA(ctx, cudaStreamSynchronize(st));
    }
  }
  return FQ_OK;
}

}  // namespace fq
