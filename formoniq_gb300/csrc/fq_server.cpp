// Serving: a continuously batched request loop over solve requests.
//
// No counterpart in the reference, which solves one problem per call. A server
// owns `lanes` lanes; each lane is a host thread with its own context (CUDA
// stream), so the device work of requests on different lanes overlaps. Requests
// wait in arrival order; the head request is admitted as soon as a lane is free
// and the HBM it is estimated to need fits the server budget next to what the
// running requests and the lanes' resident meshes hold (a request is always
// admitted when nothing runs). Meshes, scatter plans, assembled operators,
// preconditioner hierarchies and Krylov workspaces stay resident on their lane
// between requests, keyed by mesh shape; a request whose mesh is resident on
// some free lane goes there. A lane drops its resident meshes when the budget
// needs the room.
//
// Work inside a request is deterministic (fixed-order reductions, stable
// sorts), so a request's result does not depend on which lane ran it or on what
// ran beside it.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <tuple>
#include <vector>

#include "fq_internal.h"

namespace fq {
double uniform_pm1(uint64_t seed, uint64_t counter);
}

using namespace fq;
using Clock = std::chrono::steady_clock;

namespace {

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

int binom(int n, int k) {
  if (k < 0 || k > n) return 0;
  int r = 1;
  for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
  return r;
}

int64_t kuhn_cells_count(int n, int nb) {
  int64_t c = 1;
  for (int i = 2; i <= n; ++i) c *= i;
  for (int a = 0; a < n; ++a) c *= nb;
  return c;
}

// Bytes a request may hold at its peak: the scatter-plan build sorts 24 bytes
// per element triplet; plan, operator and Krylov vectors stay below that. A
// Dirac request adds the sparse direct solver's fronts: measured on Minkowski
// Kuhn boxes of 1e3 to 3e5 cells, about 1,100 cells^(4/3) bytes in FP32, twice
// that when the factors fall back to FP64.
uint64_t estimate_bytes(const fq_request& r) {
  const int n = r.dim;
  int L = 0;
  if (r.kind == FQ_REQ_DIRAC)
    L = (1 << (n + 1)) - 1;
  else
    L = binom(n + 1, r.grade) + binom(n + 1, r.grade + 1);
  const double cells = double(kuhn_cells_count(n, r.nbox));
  uint64_t est = uint64_t(40) * uint64_t(cells) * uint64_t(L) * uint64_t(L) + (uint64_t(32) << 20);
  if (r.kind == FQ_REQ_DIRAC) est += uint64_t(2.0 * 1100.0 * std::pow(cells, 4.0 / 3.0));
  return est;
}

// Counter-based N(0,1) (Box-Muller on two splitmix64 uniforms).
double seeded_normal(uint64_t seed, uint64_t i) {
  const double u1 = 0.5 * (uniform_pm1(seed ^ 0x9e3779b97f4a7c15ull, 2 * i) + 1.0);
  const double u2 = 0.5 * (uniform_pm1(seed ^ 0x9e3779b97f4a7c15ull, 2 * i + 1) + 1.0);
  const double r = std::sqrt(-2.0 * std::log(std::max(u1, 1e-300)));
  return r * std::cos(6.283185307179586 * u2);
}

struct Job {
  uint64_t ticket = 0;
  fq_request req{};
  Clock::time_point arrival, start, end;
  fq_result res{};
  bool done = false;
  uint64_t est = 0;
};

using MeshKey = std::tuple<int, int, int>;  // dim, nbox, minkowski

struct MeshEntry {
  fq_mesh* mesh = nullptr;
  std::map<std::tuple<int, int, int>, fq_mixed*> mixed;  // grade, bc, precision
  uint64_t last_use = 0;
};

}  // namespace

struct fq_server {
  int device = 0;
  int nlanes = 0;
  uint64_t budget = 0;
  bool cache = true;
  Clock::time_point epoch;

  struct Lane {
    int id = 0;
    fq_ctx* ctx = nullptr;
    std::thread th;
    std::map<MeshKey, MeshEntry> meshes;
    uint64_t held = 0;      // bytes resident while idle
    Job* job = nullptr;     // running request
    uint64_t use_clock = 0;
  };
  std::vector<std::unique_ptr<Lane>> lanes;

  std::mutex mu;
  std::condition_variable cv;
  std::deque<Job*> pending;                        // arrival order
  std::map<uint64_t, std::unique_ptr<Job>> jobs;   // by ticket
  uint64_t next_ticket = 1;
  bool stopping = false;
  fq_status init_status = FQ_OK;
  int ready = 0;
  fq_server_stats stats{};

  uint64_t committed() const {
    uint64_t c = 0;
    for (auto& l : lanes) c += l->held + (l->job ? l->job->est : 0);
    return c;
  }
  bool any_running() const {
    for (auto& l : lanes)
      if (l->job) return true;
    return false;
  }
  static MeshKey key_of(const fq_request& r) { return MeshKey{r.dim, r.nbox, r.minkowski}; }
};

namespace {

void clear_lane_cache(fq_server::Lane& L) {
  for (auto& kv : L.meshes) {
    for (auto& mx : kv.second.mixed) fq_mixed_destroy(mx.second);
    fq_mesh_destroy(kv.second.mesh);
  }
  L.meshes.clear();
}

fq_status set_request_lengths(fq_mesh* m, const fq_request& r) {
  if (r.lengths) return fq_mesh_set_lengths_sq(m, r.lengths, 0);
  if (!r.minkowski) return fq_mesh_kuhn_lengths(m, nullptr, nullptr, r.jitter, r.seed);
  // Minkowski: axis 0 timelike with time scale 0.7, then a relative length
  // jitter that keeps every sign (no edge becomes null)
  const int n = m->dim, nb = m->kuhn_nbox;
  int64_t nv = 1;
  for (int a = 0; a < n; ++a) nv *= (nb + 1);
  std::vector<double> x(size_t(nv * n));
  for (int64_t v = 0; v < nv; ++v) {
    int64_t rem = v;
    for (int a = 0; a < n; ++a) {
      const int64_t c = rem % (nb + 1);
      rem /= (nb + 1);
      x[v * n + a] = double(c) / double(nb) * (a == 0 ? 0.7 : 1.0);
    }
  }
  const auto& e = m->skel[1];
  std::vector<double> len(size_t(m->nsimp[1]));
  for (int64_t i = 0; i < m->nsimp[1]; ++i) {
    const int32_t u = e[i * 2], w = e[i * 2 + 1];
    double s = 0.0;
    for (int a = 0; a < n; ++a) {
      const double d = x[size_t(w) * n + a] - x[size_t(u) * n + a];
      s += (a == 0 ? -1.0 : 1.0) * d * d;
    }
    len[i] = s * (1.0 + r.jitter * uniform_pm1(r.seed, uint64_t(i)));
  }
  return fq_mesh_set_lengths_sq(m, len.data(), 0);
}

void run_job(fq_server* S, fq_server::Lane& L, Job& J) {
  const fq_request& r = J.req;
  fq_result& res = J.res;
  res.lane = L.id;
  fq_ctx* ctx = L.ctx;
  fq_status s = FQ_OK;
  const MeshKey key = fq_server::key_of(r);
  MeshEntry* ent = nullptr;
  auto it = L.meshes.find(key);
  if (it != L.meshes.end()) {
    ent = &it->second;
    res.cache_hit = 1;
  } else {
    fq_mesh* m = nullptr;
    s = fq_mesh_kuhn_cube(ctx, r.dim, r.nbox, &m);
    if (s == FQ_OK) {
      ent = &L.meshes[key];
      ent->mesh = m;
    }
  }
  if (s == FQ_OK) {
    ent->last_use = ++L.use_clock;
    s = set_request_lengths(ent->mesh, r);
  }
  std::vector<double> sol;
  fq_mesh* m = ent ? ent->mesh : nullptr;
  if (s == FQ_OK && r.kind == FQ_REQ_HODGE) {
    const int k = r.grade;
    if (k < 0 || k > r.dim) {
      s = set_error(ctx, FQ_INVALID_ARG, "grade out of range");
    } else {
      const int64_t nk = m->nsimp[k], nkm = k >= 1 ? m->nsimp[k - 1] : 0;
      std::vector<double> src;
      const double* sp = r.source;
      if (!sp) {
        src.resize(size_t(nk));
        for (int64_t i = 0; i < nk; ++i) src[i] = seeded_normal(r.seed, uint64_t(i));
        sp = src.data();
      }
      const auto mk = std::make_tuple(k, r.bc, r.opts.precision);
      fq_mixed* P = nullptr;
      auto pit = ent->mixed.find(mk);
      if (pit != ent->mixed.end()) {
        P = pit->second;
        s = fq_mixed_reassemble(P);
      } else {
        s = fq_mixed_create(ctx, m, k, fq_bc(r.bc), r.opts.precision, &P);
        if (s == FQ_OK) ent->mixed[mk] = P;
      }
      if (s == FQ_OK) {
        sol.assign(size_t(nkm + nk), 0.0);
        double p[1] = {0.0};
        s = fq_mixed_solve(P, sp, sol.data(), sol.data() + nkm, p, &r.opts, &res.report);
      }
    }
  } else if (s == FQ_OK) {
    int64_t nfull = 0;
    for (int j = 0; j <= r.dim; ++j) nfull += m->nsimp[j];
    std::vector<double> load;
    const double* lp = r.source;
    if (!lp) {
      load.resize(size_t(nfull));
      for (int64_t i = 0; i < nfull; ++i) load[i] = seeded_normal(r.seed, uint64_t(i));
      lp = load.data();
    }
    sol.assign(size_t(nfull), 0.0);
    s = fq_solve_dirac_source(ctx, m, r.mass_term, lp, nullptr, sol.data(), &r.opts, &res.report);
  }
  if (s == FQ_OK || s == FQ_NOT_CONVERGED) {
    double cs = 0.0;
    for (double v : sol) cs += v * v;
    res.checksum = cs;
    res.ndofs = sol.size();
    if (r.solution) std::memcpy(r.solution, sol.data(), sol.size() * sizeof(double));
  }
  res.status = s;
  if (!S->cache) clear_lane_cache(L);
}

void lane_main(fq_server* S, fq_server::Lane* L) {
  fq_status s = fq_ctx_create(S->device, nullptr, S->budget, &L->ctx);
  // No dense direct fallback in lanes: cuSOLVER's handle set-up and tear-down
  // allocate and free device memory synchronously, which invalidates the graph
  // captures other lanes run concurrently (their requests then fail with CUDA
  // errors). Lanes keep the MINRES result, as the serving stream's iteration
  // caps intend.
  if (s == FQ_OK) L->ctx->dense_fallback = false;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (s != FQ_OK && S->init_status == FQ_OK) S->init_status = s;
    S->ready++;
  }
  S->cv.notify_all();
  if (s != FQ_OK) return;
  std::unique_lock<std::mutex> lk(S->mu);
  for (;;) {
    if (S->stopping && S->pending.empty()) break;
    Job* J = S->pending.empty() ? nullptr : S->pending.front();
    const auto now = Clock::now();
    if (!J) {
      S->cv.wait(lk);
      continue;
    }
    if (J->arrival > now) {
      S->cv.wait_until(lk, J->arrival);
      continue;
    }
    // resident-mesh affinity: leave the head request to a free lane that holds its mesh
    const MeshKey key = fq_server::key_of(J->req);
    const bool mine = L->meshes.count(key) > 0;
    if (!mine) {
      bool other = false;
      for (auto& o : S->lanes)
        if (o.get() != L && !o->job && o->ctx && o->meshes.count(key)) other = true;
      if (other) {
        S->cv.wait_for(lk, std::chrono::microseconds(200));
        continue;
      }
    }
    // HBM admission
    bool evict = false;
    uint64_t c = S->committed();
    if (S->any_running() && c + J->est > S->budget) {
      if (!mine && L->held > 0 && c - L->held + J->est <= S->budget) {
        evict = true;
      } else {
        S->cv.wait(lk);
        continue;
      }
    }
    S->pending.pop_front();
    L->job = J;
    J->start = Clock::now();
    if (evict) {
      S->stats.evictions += L->meshes.size();
      L->held = 0;
    }
    lk.unlock();
    if (evict) clear_lane_cache(*L);
    run_job(S, *L, *J);
    lk.lock();
    J->end = Clock::now();
    J->res.queue_ms = ms_between(J->arrival, J->start);
    J->res.run_ms = ms_between(J->start, J->end);
    J->res.latency_ms = ms_between(J->arrival, J->end);
    J->res.start_ms = ms_between(S->epoch, J->start);
    J->res.end_ms = ms_between(S->epoch, J->end);
    J->done = true;
    L->job = nullptr;
    L->held = L->ctx->in_use;
    S->stats.completed++;
    S->stats.cache_hits += uint64_t(J->res.cache_hit);
    S->stats.busy_ms += J->res.run_ms;
    S->stats.peak_committed_bytes = std::max<uint64_t>(S->stats.peak_committed_bytes, S->committed() + J->est);
    S->cv.notify_all();
  }
  lk.unlock();
  clear_lane_cache(*L);
  fq_ctx_destroy(L->ctx);
  L->ctx = nullptr;
}

}  // namespace

extern "C" {

fq_status fq_server_create(int device, int lanes, uint64_t hbm_budget, int cache, fq_server** out) {
  if (!out || lanes < 1 || lanes > 64) return FQ_INVALID_ARG;
  auto* S = new (std::nothrow) fq_server();
  if (!S) return FQ_OOM_BUDGET;
  S->device = device;
  S->nlanes = lanes;
  S->budget = hbm_budget ? hbm_budget : (uint64_t(200) << 30);
  S->cache = cache != 0;
  S->epoch = Clock::now();
  for (int i = 0; i < lanes; ++i) {
    S->lanes.emplace_back(new fq_server::Lane());
    S->lanes.back()->id = i;
  }
  for (auto& L : S->lanes) L->th = std::thread(lane_main, S, L.get());
  {
    std::unique_lock<std::mutex> lk(S->mu);
    S->cv.wait(lk, [&] { return S->ready == lanes; });
  }
  if (S->init_status != FQ_OK) {
    fq_status s = S->init_status;
    fq_server_destroy(S);
    return s;
  }
  *out = S;
  return FQ_OK;
}

fq_status fq_server_submit(fq_server* S, const fq_request* req, uint64_t* ticket) {
  if (!S || !req || !ticket) return FQ_INVALID_ARG;
  if (req->kind != FQ_REQ_HODGE && req->kind != FQ_REQ_DIRAC) return FQ_INVALID_ARG;
  if (req->dim < 1 || req->dim > 4 || req->nbox < 1) return FQ_INVALID_ARG;
  auto J = std::make_unique<Job>();
  J->req = *req;
  const auto now = Clock::now();
  const auto at = S->epoch + std::chrono::duration_cast<Clock::duration>(
                                 std::chrono::duration<double, std::milli>(std::max(req->arrival_ms, 0.0)));
  J->arrival = req->arrival_ms >= 0.0 ? std::max(at, now) : now;
  J->est = estimate_bytes(*req);
  std::lock_guard<std::mutex> lk(S->mu);
  if (S->stopping) return FQ_INVALID_ARG;
  J->ticket = S->next_ticket++;
  *ticket = J->ticket;
  // arrival order (stable for equal times)
  auto pos = std::upper_bound(S->pending.begin(), S->pending.end(), J->arrival,
                              [](Clock::time_point t, const Job* j) { return t < j->arrival; });
  S->pending.insert(pos, J.get());
  S->stats.submitted++;
  S->jobs[J->ticket] = std::move(J);
  S->cv.notify_all();
  return FQ_OK;
}

fq_status fq_server_wait(fq_server* S, uint64_t ticket, fq_result* out) {
  if (!S || !out) return FQ_INVALID_ARG;
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->jobs.find(ticket);
  if (it == S->jobs.end()) return FQ_INVALID_ARG;
  Job* J = it->second.get();
  S->cv.wait(lk, [&] { return J->done; });
  *out = J->res;
  S->jobs.erase(it);
  return FQ_OK;
}

fq_status fq_server_get_stats(fq_server* S, fq_server_stats* out) {
  if (!S || !out) return FQ_INVALID_ARG;
  std::lock_guard<std::mutex> lk(S->mu);
  *out = S->stats;
  out->resident_bytes = 0;
  for (auto& L : S->lanes) out->resident_bytes += L->held;
  return FQ_OK;
}

void fq_server_destroy(fq_server* S) {
  if (!S) return;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stopping = true;
  }
  S->cv.notify_all();
  for (auto& L : S->lanes)
    if (L->th.joinable()) L->th.join();
  delete S;
}

}  // extern "C"
