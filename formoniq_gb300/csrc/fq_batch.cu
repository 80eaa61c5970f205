// Batched assembly: many meshes of uneven size, dimension and degree assembled
// together.
//
// No counterpart in the reference (one mesh per assemble_matrix call,
// galerkin.rs:138-188). The batch keeps, per mesh, the scatter plan of its
// element program (built by the same plan builder as a single assembly) and
// slices of two batch-wide buffers: element values and CSR values. One
// assembly of the batch is a CUDA graph of
//   - one element launch per (dimension, degree) class present: a grid-stride
//     kernel over the concatenated cells of the class, each thread finding its
//     mesh by binary search over the class's cell offsets (a class shares one
//     kernel instance: register allocation is per kernel, so one launch over
//     all classes would run every program at the heaviest program's occupancy);
//   - one scatter launch over the concatenated CSR slots of all meshes:
//     `tps` threads per slot, or warp-staged (tps = 0: a warp gathers the
//     contributions of its 32 slots into shared memory, then each lane sums
//     its slot in order).
// The grid sizes and `tps` come from a tuner that times the candidates on the
// batch itself. Per mesh, the element values and the summation order of every
// slot are those of a single assembly (with tps = 0 or 1 bit for bit).
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <memory>
#include <vector>

#include "fq_df64.cuh"
#include "fq_internal.h"

namespace fq {

fq_status get_plan(fq_ctx* ctx, fq_mesh* m, int kind, int grade, int row_bc, int col_bc, Plan** out);
bool batch_fused_supported(int kind, int dim, int grade);
void launch_batch_fused_hdif(const ElemFusedEntry* ent, int n, int64_t total, int grid, int* status,
                             cudaStream_t st);
int batch_fused_registers();

struct ScatterBatchEntry {
  int64_t begin, nslots;
  const int32_t* slot_ptr;
  const int32_t* perm;
  const df64* elem;
  double* values;
};

// Symmetric plans: the upper slots of each mesh (index, mirror) and their
// contributions, in a batch index space padded per mesh to a multiple of 32.
struct ScatterSymEntry {
  int64_t begin, nup;
  const int2* pair;
  const int32_t* up_ptr;
  const int32_t* perm;
  const df64* elem;
  double* values;
};

namespace {

__device__ __forceinline__ bool nz_bits(float v) { return (__float_as_int(v) << 1) != 0; }

// tps = -1: one thread per upper slot of every mesh, the value written to the
// slot and its mirror; per slot the summation of the single-mesh scatter.
__global__ void __launch_bounds__(256) scatter_batch_sym_kernel(const ScatterSymEntry* __restrict__ tab, int ntab,
                                                                int64_t total, int* status) {
  for (int64_t g = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; g < total;
       g += int64_t(gridDim.x) * blockDim.x) {
    int lo = 0, hi = ntab - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (tab[mid].begin <= g)
        lo = mid;
      else
        hi = mid - 1;
    }
    const ScatterSymEntry& e = tab[lo];
    const int64_t u = g - e.begin;
    if (u >= e.nup) continue;  // padding between meshes
    const int2 sm = __ldg(e.pair + u);
    const int b = __ldg(e.up_ptr + u), en = __ldg(e.up_ptr + u + 1);
    df64 acc(0.f, 0.f);
    bool nz = false;
    for (int t = b; t < en; ++t) {
      const df64 v = e.elem[__ldg(e.perm + t)];
      acc += v;
      nz |= nz_bits(v.hi) || nz_bits(v.lo);
    }
    const double out = acc.to_double();
    e.values[sm.x] = out;
    int nzero = nz ? 0 : 1;
    if (sm.y != sm.x) {
      if (sm.y >= 0) {
        e.values[sm.y] = out;
        nzero += nz ? 0 : 1;
      } else {
        atomicOr(status, 4);
      }
    }
    if (nzero) atomicAdd(status + 1, nzero);
  }
}

// tps lanes per slot (tps divides 32), contributions strided over the lanes and
// combined in a fixed shuffle order.
template <int TPS>
__global__ void __launch_bounds__(256) scatter_batch_kernel(const ScatterBatchEntry* __restrict__ tab, int ntab,
                                                            int64_t total, int* zero_count) {
  const int lane = threadIdx.x % TPS;
  const int64_t groups_per_grid = int64_t(gridDim.x) * (blockDim.x / TPS);
  for (int64_t base = int64_t(blockIdx.x) * (blockDim.x / TPS); base < total; base += groups_per_grid) {
    const int64_t g = base + threadIdx.x / TPS;
    const bool valid = g < total;
    df64 acc(0.f, 0.f);
    bool nz = false;
    int lo = 0;
    bool live = valid;
    if (valid) {
      int hi = ntab - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (tab[mid].begin <= g)
          lo = mid;
        else
          hi = mid - 1;
      }
      // each mesh's range is padded to a multiple of 32: a padding index has no slot
      live = g - tab[lo].begin < tab[lo].nslots;
    }
    if (live) {
      const ScatterBatchEntry& e = tab[lo];
      const int64_t s = g - e.begin;
      const int b = __ldg(e.slot_ptr + s), en = __ldg(e.slot_ptr + s + 1);
      for (int t = b + lane; t < en; t += TPS) {
        const df64 v = e.elem[__ldg(e.perm + t)];
        acc += v;
        nz |= nz_bits(v.hi) || nz_bits(v.lo);
      }
    }
    if constexpr (TPS > 1) {
#pragma unroll
      for (int o = TPS / 2; o > 0; o >>= 1) {
        const df64 other(__shfl_down_sync(0xffffffffu, acc.hi, o, TPS), __shfl_down_sync(0xffffffffu, acc.lo, o, TPS));
        const int onz = __shfl_down_sync(0xffffffffu, int(nz), o, TPS);
        acc += other;
        nz = nz || onz;
      }
    }
    if (live && lane == 0) {
      const ScatterBatchEntry& e = tab[lo];
      e.values[g - e.begin] = acc.to_double();
      if (!nz) atomicAdd(zero_count, 1);
    }
  }
}

// Warp-staged form (tps = 0): each mesh's slot range starts at a multiple of 32
// in the batch index space, so a warp's 32 slots belong to one mesh; staging and
// summation order are those of the single-mesh scatter.
constexpr int kBatchStage = 256;

__global__ void __launch_bounds__(256) scatter_batch_warp_kernel(const ScatterBatchEntry* __restrict__ tab, int ntab,
                                                                 int64_t total, int* zero_count) {
  __shared__ df64 stage[8][kBatchStage];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t warps_per_grid = int64_t(gridDim.x) * 8;
  for (int64_t w = int64_t(blockIdx.x) * 8 + warp; w * 32 < total; w += warps_per_grid) {
    const int64_t g0 = w * 32;
    int lo = 0, hi = ntab - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (tab[mid].begin <= g0)
        lo = mid;
      else
        hi = mid - 1;
    }
    const ScatterBatchEntry& en = tab[lo];
    const int64_t s0 = g0 - en.begin;
    if (s0 >= en.nslots) continue;  // padding between meshes (uniform over the warp)
    const int64_t s = s0 + lane;
    const int64_t slast = min(s0 + 32, en.nslots);
    const int tb = __ldg(en.slot_ptr + s0), te = __ldg(en.slot_ptr + slast);
    const int count = te - tb;
    int b = 0, e = 0;
    if (s < en.nslots) {
      b = __ldg(en.slot_ptr + s) - tb;
      e = __ldg(en.slot_ptr + s + 1) - tb;
    }
    df64 acc(0.f, 0.f);
    bool nz = false;
    if (count <= kBatchStage) {
      df64* st = stage[warp];
      int t = lane;
      for (; t + 96 < count; t += 128) {
        const int p0 = __ldg(en.perm + tb + t), p1 = __ldg(en.perm + tb + t + 32);
        const int p2 = __ldg(en.perm + tb + t + 64), p3 = __ldg(en.perm + tb + t + 96);
        const df64 v0 = en.elem[p0], v1 = en.elem[p1], v2 = en.elem[p2], v3 = en.elem[p3];
        st[t] = v0;
        st[t + 32] = v1;
        st[t + 64] = v2;
        st[t + 96] = v3;
      }
      for (; t < count; t += 32) st[t] = en.elem[__ldg(en.perm + tb + t)];
      __syncwarp();
      for (int q = b; q < e; ++q) {
        const df64 v = st[q];
        acc += v;
        nz |= nz_bits(v.hi) || nz_bits(v.lo);
      }
      __syncwarp();
    } else {
      for (int q = b; q < e; ++q) {
        const df64 v = en.elem[__ldg(en.perm + tb + q)];
        acc += v;
        nz |= nz_bits(v.hi) || nz_bits(v.lo);
      }
    }
    if (s < en.nslots) {
      en.values[s] = acc.to_double();
      if (!nz) atomicAdd(zero_count, 1);
    }
  }
}

void launch_scatter_batch_sym(const ScatterSymEntry* tab, int ntab, int64_t total, int grid, int* status,
                              cudaStream_t st) {
  if (total <= 0) return;
  const int64_t need = (total + 255) / 256;
  const unsigned blocks = unsigned(grid > 0 ? std::min<int64_t>(grid, need) : need);
  scatter_batch_sym_kernel<<<blocks, 256, 0, st>>>(tab, ntab, total, status);
}

void launch_scatter_batch(const ScatterBatchEntry* tab, int ntab, int64_t total, int tps, int grid, int* zc,
                          cudaStream_t st) {
  if (total <= 0) return;
  const int threads = 256;
  if (tps == 0) {
    const int64_t need = (total + threads - 1) / threads;
    const unsigned blocks = unsigned(grid > 0 ? std::min<int64_t>(grid, need) : need);
    scatter_batch_warp_kernel<<<blocks, threads, 0, st>>>(tab, ntab, total, zc);
    return;
  }
  const int64_t need = (total * tps + threads - 1) / threads;
  const unsigned blocks = unsigned(grid > 0 ? std::min<int64_t>(grid, need) : need);
  switch (tps) {
    case 2:
      scatter_batch_kernel<2><<<blocks, threads, 0, st>>>(tab, ntab, total, zc);
      break;
    case 4:
      scatter_batch_kernel<4><<<blocks, threads, 0, st>>>(tab, ntab, total, zc);
      break;
    default:
      scatter_batch_kernel<1><<<blocks, threads, 0, st>>>(tab, ntab, total, zc);
      break;
  }
}

}  // namespace
}  // namespace fq

using namespace fq;

struct fq_batch {
  fq_ctx* ctx = nullptr;
  int kind = 0;
  struct Member {
    fq_mesh* mesh = nullptr;
    int grade = 0;
    Plan* plan = nullptr;
    int64_t elem_off = 0, val_off = 0;  // element offset in df64 units, value offset in doubles
  };
  std::vector<Member> members;
  struct Class {
    int dim = 0, grade = 0;
    int64_t total = 0;
    DevBuf table;  // ElemBatchEntry[]
    int n = 0;
    int nent = 0;  // element entries per cell of the class's program
    int grid = 0;  // tuned CTAs (0 = one thread per cell)
  };
  std::vector<Class> classes;
  DevBuf elem, values, stable, flags, symtable;
  int64_t total_cells = 0, total_slots = 0, max_slots = 0;  // total_slots: padded batch index space
  int64_t real_slots = 0;
  int64_t total_up = 0;  // padded upper-slot index space (0: some plan is not symmetric)
  int tps = 1, sgrid = 0;  // tps 0: warp-staged scatter, -1: symmetric
  // the element pass as one fused launch over every class (fq_batch_fused.cu)
  bool fused = false;
  int fgrid = 0;
  DevBuf ftable;  // ElemFusedEntry[], members in order
  cudaGraphExec_t graph = nullptr;
  ~fq_batch() {
    if (graph) cudaGraphExecDestroy(graph);
  }
};

namespace {

fq_status enqueue_batch(fq_batch* B) {
  fq_ctx* ctx = B->ctx;
  cudaStream_t st = ctx->stream;
  if (B->fused)
    launch_batch_fused_hdif(B->ftable.as<ElemFusedEntry>(), int(B->members.size()), B->total_cells, B->fgrid,
                            ctx->status.as<int>(), st);
  for (auto& c : B->classes) {
    if (B->fused) break;
    ElemArgs a;
    a.ncells = 0;
    a.lengths = nullptr;
    a.cell_edges = nullptr;
    a.out = nullptr;
    a.ginv_out = a.det_out = a.vol_out = nullptr;
    a.param = 0.0;
    a.status = ctx->status.as<int>();
    a.nent = c.nent;
    a.batch = c.table.as<ElemBatchEntry>();
    a.nbatch = c.n;
    a.total = c.total;
    a.grid = c.grid;
    if (launch_element(c.dim, c.grade, B->kind, FQ_FP64, a, st) != 0)
      return set_error(ctx, FQ_UNSUPPORTED, "no element program for this dimension/grade");
  }
  if (B->tps == -1)
    launch_scatter_batch_sym(B->symtable.as<ScatterSymEntry>(), int(B->members.size()), B->total_up, B->sgrid,
                             ctx->status.as<int>(), st);
  else
    launch_scatter_batch(B->stable.as<ScatterBatchEntry>(), int(B->members.size()), B->total_slots, B->tps,
                         B->sgrid, ctx->status.as<int>() + 1, st);
  return FQ_OK;
}

fq_status capture(fq_batch* B) {
  fq_ctx* ctx = B->ctx;
  if (B->graph) {
    cudaGraphExecDestroy(B->graph);
    B->graph = nullptr;
  }
  cudaGraph_t g = nullptr;
  if (cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    return FQ_OK;  // uncapturable stream: direct launches
  }
  fq_status s = enqueue_batch(B);
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
  if (s != FQ_OK) {
    if (g) cudaGraphDestroy(g);
    return s;
  }
  if (e == cudaSuccess) {
    e = cudaGraphInstantiate(&B->graph, g, 0);
    cudaGraphDestroy(g);
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    B->graph = nullptr;
  }
  return FQ_OK;
}

fq_status check_status(fq_ctx* ctx) {
  FQ_CUDA(ctx, cudaMemcpyAsync(ctx->host_status, ctx->status.p, 8 * sizeof(int), cudaMemcpyDeviceToHost,
                               ctx->stream));
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (ctx->host_status[0] & 4) return set_error(ctx, FQ_CUDA_ERROR, "symmetric plan without a mirror slot");
  if (ctx->host_status[0] & 2) return set_error(ctx, FQ_INVALID_ARG, "element program wrote outside its layout");
  if (ctx->host_status[0] & 1) return set_error(ctx, FQ_DEGENERATE_CELL, "a cell metric is singular or not finite");
  if (ctx->host_status[1] > 0)
    return set_error(ctx, FQ_UNSUPPORTED,
                     "some slots summed exact zeros only (the reference drops them): assemble those meshes alone");
  return FQ_OK;
}

float time_once(fq_batch* B, int reps) {
  fq_ctx* ctx = B->ctx;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  enqueue_batch(B);  // warm-up
  cudaEventRecord(a, ctx->stream);
  for (int r = 0; r < reps; ++r) enqueue_batch(B);
  cudaEventRecord(b, ctx->stream);
  cudaEventSynchronize(b);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return ms / float(std::max(reps, 1));
}

}  // namespace

extern "C" {

fq_status fq_batch_create(fq_ctx* ctx, int nmeshes, fq_mesh* const* meshes, const int* grades, int form,
                          fq_batch** out) {
  if (!ctx || !out || nmeshes < 1 || !meshes || !grades) return FQ_INVALID_ARG;
  int kind = 0;
  if (form == FQ_BATCH_MASS)
    kind = EK_MASS;
  else if (form == FQ_BATCH_HDIF)
    kind = EK_HDIF;
  else
    return set_error(ctx, FQ_INVALID_ARG, "unknown batch form");
  auto B = std::make_unique<fq_batch>();
  B->ctx = ctx;
  B->kind = kind;
  std::map<std::pair<int, int>, std::vector<int>> byclass;
  int64_t eoff = 0, voff = 0;
  for (int i = 0; i < nmeshes; ++i) {
    fq_mesh* m = meshes[i];
    if (!m || m->ctx != ctx) return set_error(ctx, FQ_INVALID_ARG, "batch meshes must belong to the context");
    if (!m->has_lengths) return set_error(ctx, FQ_INVALID_ARG, "mesh has no edge lengths");
    if (grades[i] < 0 || grades[i] > m->dim) return set_error(ctx, FQ_INVALID_ARG, "grade out of range");
    fq_batch::Member mb;
    mb.mesh = m;
    mb.grade = grades[i];
    FQ_TRY(get_plan(ctx, m, kind, grades[i], FQ_ABSOLUTE, FQ_ABSOLUTE, &mb.plan));
    mb.elem_off = eoff;
    mb.val_off = voff;
    eoff += (int64_t(mb.plan->nent) * m->ncells + 31) & ~int64_t(31);
    voff += (mb.plan->nslots + 31) & ~int64_t(31);
    B->total_cells += m->ncells;
    B->max_slots = std::max(B->max_slots, mb.plan->nslots);
    byclass[{m->dim, grades[i]}].push_back(i);
    B->members.push_back(mb);
  }
  FQ_TRY(B->elem.alloc(ctx, std::max<int64_t>(eoff, 1) * 8));
  FQ_TRY(B->values.alloc(ctx, std::max<int64_t>(voff, 1) * 8));
  FQ_TRY(B->flags.alloc(ctx, std::max<int64_t>(B->max_slots, 1)));
  // element tables per class
  for (auto& kv : byclass) {
    fq_batch::Class c;
    c.dim = kv.first.first;
    c.grade = kv.first.second;
    std::vector<ElemBatchEntry> tab;
    for (int i : kv.second) {
      const auto& mb = B->members[i];
      ElemBatchEntry e;
      e.begin = c.total;
      e.ncells = mb.mesh->ncells;
      e.lengths = mb.mesh->lengths.as<double>();
      e.cell_edges = mb.mesh->dim >= 1 ? mb.mesh->cell_faces[1].as<int32_t>() : nullptr;
      e.out = B->elem.as<df64>() + mb.elem_off;
      tab.push_back(e);
      c.total += e.ncells;
    }
    c.n = int(tab.size());
    c.nent = B->members[kv.second.front()].plan->nent;
    FQ_TRY(c.table.alloc(ctx, tab.size() * sizeof(ElemBatchEntry)));
    FQ_CUDA(ctx, cudaMemcpyAsync(c.table.p, tab.data(), tab.size() * sizeof(ElemBatchEntry), cudaMemcpyHostToDevice,
                                 ctx->stream));
    B->classes.push_back(std::move(c));
  }
  // scatter table over all meshes
  std::vector<ScatterBatchEntry> st;
  for (auto& mb : B->members) {
    ScatterBatchEntry e;
    e.begin = B->total_slots;  // a multiple of 32: warps never straddle meshes
    e.nslots = mb.plan->nslots;
    e.slot_ptr = mb.plan->slot_ptr.as<int32_t>();
    e.perm = mb.plan->perm.as<int32_t>();
    e.elem = B->elem.as<df64>() + mb.elem_off;
    e.values = B->values.as<double>() + mb.val_off;
    st.push_back(e);
    B->total_slots += (e.nslots + 31) & ~int64_t(31);
    B->real_slots += e.nslots;
  }
  FQ_TRY(B->stable.alloc(ctx, st.size() * sizeof(ScatterBatchEntry)));
  FQ_CUDA(ctx, cudaMemcpyAsync(B->stable.p, st.data(), st.size() * sizeof(ScatterBatchEntry), cudaMemcpyHostToDevice,
                               ctx->stream));
  // the symmetric table, when every member's plan has one
  bool all_sym = true;
  for (auto& mb : B->members) all_sym = all_sym && mb.plan->nup > 0;
  if (all_sym && !B->members.empty()) {
    std::vector<ScatterSymEntry> sy;
    for (auto& mb : B->members) {
      ScatterSymEntry e;
      e.begin = B->total_up;
      e.nup = mb.plan->nup;
      e.pair = mb.plan->up_pair.as<int2>();
      e.up_ptr = mb.plan->up_ptr.as<int32_t>();
      e.perm = mb.plan->up_perm.as<int32_t>();
      e.elem = B->elem.as<df64>() + mb.elem_off;
      e.values = B->values.as<double>() + mb.val_off;
      sy.push_back(e);
      B->total_up += (e.nup + 31) & ~int64_t(31);
    }
    FQ_TRY(B->symtable.alloc(ctx, sy.size() * sizeof(ScatterSymEntry)));
    FQ_CUDA(ctx, cudaMemcpyAsync(B->symtable.p, sy.data(), sy.size() * sizeof(ScatterSymEntry),
                                 cudaMemcpyHostToDevice, ctx->stream));
  }
  FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  FQ_TRY(capture(B.get()));
  *out = B.release();
  return FQ_OK;
}

fq_status fq_batch_tune(fq_batch* B, int reps) {
  if (!B) return FQ_INVALID_ARG;
  fq_ctx* ctx = B->ctx;
  reps = std::max(reps, 1);
  int dev_sms = 152;
  cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, ctx->device);
  // element stage: CTAs per SM of each class's grid-stride launch (0 = one thread per cell)
  const int per_sm[] = {0, 2, 4, 8, 16};
  for (auto& c : B->classes) {
    float best = 1e30f;
    int pick = 0;
    for (int ps : per_sm) {
      c.grid = ps * dev_sms;
      const float t = time_once(B, reps);
      if (t < best) {
        best = t;
        pick = c.grid;
      }
    }
    c.grid = pick;
  }
  // scatter stage: threads per slot and CTAs per SM
  float best = 1e30f;
  int btps = 1, bgrid = 0;
  for (int tps : {-1, 0, 1, 2, 4})
    for (int ps : per_sm) {
      if (tps == -1 && B->total_up == 0) continue;
      B->tps = tps;
      B->sgrid = ps * dev_sms;
      const float t = time_once(B, reps);
      if (t < best) {
        best = t;
        btps = tps;
        bgrid = B->sgrid;
      }
    }
  B->tps = btps;
  B->sgrid = bgrid;
  FQ_CUDA(ctx, cudaMemsetAsync(ctx->status.p, 0, 8 * sizeof(int), ctx->stream));
  FQ_TRY(capture(B));
  return FQ_OK;
}

fq_status fq_batch_set_launch(fq_batch* B, int element_grid, int scatter_tps, int scatter_grid) {
  if (!B || (scatter_tps != -1 && scatter_tps != 0 && scatter_tps != 1 && scatter_tps != 2 && scatter_tps != 4))
    return FQ_INVALID_ARG;
  if (scatter_tps == -1 && B->total_up == 0) return set_error(B->ctx, FQ_UNSUPPORTED, "no symmetric plans in batch");
  for (auto& c : B->classes) c.grid = element_grid;
  B->tps = scatter_tps;
  B->sgrid = scatter_grid;
  return capture(B);
}

fq_status fq_batch_set_element_launch(fq_batch* B, int fused, int grid) {
  if (!B || grid < 0) return FQ_INVALID_ARG;
  fq_ctx* ctx = B->ctx;
  if (fused) {
    for (auto& mb : B->members)
      if (!batch_fused_supported(B->kind, mb.mesh->dim, mb.grade))
        return set_error(ctx, FQ_UNSUPPORTED, "the fused element launch covers hdif_gram batches of dimensions 2-4");
    if (!B->ftable.p) {
      std::vector<ElemFusedEntry> tab;
      int64_t begin = 0;
      for (auto& mb : B->members) {
        ElemFusedEntry e{};
        e.begin = begin;
        e.ncells = mb.mesh->ncells;
        e.lengths = mb.mesh->lengths.as<double>();
        e.cell_edges = mb.mesh->cell_faces[1].as<int32_t>();
        e.out = B->elem.as<df64>() + mb.elem_off;
        e.nent = int(mb.plan->nent);
        e.dim = mb.mesh->dim;
        e.grade = mb.grade;
        tab.push_back(e);
        begin += e.ncells;
      }
      FQ_TRY(B->ftable.alloc(ctx, std::max<size_t>(tab.size(), 1) * sizeof(ElemFusedEntry)));
      if (!tab.empty())
        FQ_CUDA(ctx, cudaMemcpyAsync(B->ftable.p, tab.data(), tab.size() * sizeof(ElemFusedEntry),
                                     cudaMemcpyHostToDevice, ctx->stream));
      FQ_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
  }
  B->fused = fused != 0;
  B->fgrid = grid;
  return capture(B);
}

int fq_batch_fused_registers(void) { return batch_fused_registers(); }

fq_status fq_batch_assemble(fq_batch* B, int check) {
  if (!B) return FQ_INVALID_ARG;
  fq_ctx* ctx = B->ctx;
  FQ_CUDA(ctx, cudaMemsetAsync(ctx->status.p, 0, 8 * sizeof(int), ctx->stream));
  if (B->graph) {
    FQ_CUDA(ctx, cudaGraphLaunch(B->graph, ctx->stream));
  } else {
    FQ_TRY(enqueue_batch(B));
  }
  ctx->launches += B->classes.size() + 1;
  return check ? check_status(ctx) : FQ_OK;
}

fq_status fq_batch_assemble_per_mesh(fq_batch* B, int check) {
  if (!B) return FQ_INVALID_ARG;
  fq_ctx* ctx = B->ctx;
  cudaStream_t st = ctx->stream;
  FQ_CUDA(ctx, cudaMemsetAsync(ctx->status.p, 0, 8 * sizeof(int), st));
  for (auto& mb : B->members) {
    ElemArgs a;
    a.ncells = mb.mesh->ncells;
    a.lengths = mb.mesh->lengths.as<double>();
    a.cell_edges = mb.mesh->dim >= 1 ? mb.mesh->cell_faces[1].as<int32_t>() : nullptr;
    a.out = B->elem.as<df64>() + mb.elem_off;
    a.ginv_out = a.det_out = a.vol_out = nullptr;
    a.param = 0.0;
    a.status = ctx->status.as<int>();
    a.nent = mb.plan->nent;
    if (launch_element(mb.mesh->dim, mb.grade, B->kind, FQ_FP64, a, st) != 0)
      return set_error(ctx, FQ_UNSUPPORTED, "no element program for this dimension/grade");
    launch_scatter(*mb.plan, a.out, B->values.as<double>() + mb.val_off, B->flags.as<uint8_t>(),
                   ctx->status.as<int>(), FQ_FP64, st);
    ctx->launches += 2;
  }
  return check ? check_status(ctx) : FQ_OK;
}

fq_status fq_batch_info(const fq_batch* B, int64_t* total_cells, int64_t* total_slots, int* nclasses,
                        int* launches) {
  if (!B) return FQ_INVALID_ARG;
  if (total_cells) *total_cells = B->total_cells;
  if (total_slots) *total_slots = B->real_slots;
  if (nclasses) *nclasses = int(B->classes.size());
  if (launches) *launches = int(B->classes.size()) + 1;
  return FQ_OK;
}

fq_status fq_batch_launch_config(const fq_batch* B, int* scatter_tps, int* scatter_grid, int* element_grids,
                                 int max_classes) {
  if (!B) return FQ_INVALID_ARG;
  if (scatter_tps) *scatter_tps = B->tps;
  if (scatter_grid) *scatter_grid = B->sgrid;
  if (element_grids)
    for (int i = 0; i < max_classes && i < int(B->classes.size()); ++i) element_grids[i] = B->classes[i].grid;
  return FQ_OK;
}

fq_status fq_batch_matrix(const fq_batch* B, int i, int64_t* nrows, int64_t* nnz, const int32_t** row_ptr,
                          const int32_t** col_idx, const double** values) {
  if (!B || i < 0 || i >= int(B->members.size())) return FQ_INVALID_ARG;
  const auto& mb = B->members[i];
  if (nrows) *nrows = mb.plan->nrows;
  if (nnz) *nnz = mb.plan->nslots;
  if (row_ptr) *row_ptr = mb.plan->row_ptr.as<int32_t>();
  if (col_idx) *col_idx = mb.plan->col_idx.as<int32_t>();
  if (values) *values = B->values.as<double>() + mb.val_off;
  return FQ_OK;
}

fq_status fq_batch_copy_to_host(const fq_batch* B, int i, int32_t* row_ptr, int32_t* col_idx, double* values) {
  if (!B || i < 0 || i >= int(B->members.size())) return FQ_INVALID_ARG;
  fq_ctx* ctx = B->ctx;
  const auto& mb = B->members[i];
  cudaStream_t st = ctx->stream;
  if (row_ptr)
    FQ_CUDA(ctx, cudaMemcpyAsync(row_ptr, mb.plan->row_ptr.p, (mb.plan->nrows + 1) * 4, cudaMemcpyDeviceToHost, st));
  if (mb.plan->nslots > 0) {
    if (col_idx)
      FQ_CUDA(ctx, cudaMemcpyAsync(col_idx, mb.plan->col_idx.p, mb.plan->nslots * 4, cudaMemcpyDeviceToHost, st));
    if (values)
      FQ_CUDA(ctx, cudaMemcpyAsync(values, B->values.as<double>() + mb.val_off, mb.plan->nslots * 8,
                                   cudaMemcpyDeviceToHost, st));
  }
  FQ_CUDA(ctx, cudaStreamSynchronize(st));
  return FQ_OK;
}

void fq_batch_destroy(fq_batch* B) {
  if (!B) return;
  cudaStreamSynchronize(B->ctx->stream);
  delete B;
}

}  // extern "C"
