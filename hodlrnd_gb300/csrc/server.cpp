// Request loop (serving): solves of different geometries, sizes and
// right-hand-side counts arrive at any time; each is admitted as soon as a
// slot is free and its predicted device bytes fit the budget next to what is
// already resident, runs on its own CUDA stream (one per geometry), and
// completes independently.  Geometries submitted with a key stay resident
// (tree, factors and work vectors on the device) for later requests until the
// budget needs their memory (least recently used first).
//
// The reference has no counterpart: HODLRdD_matrix is built and solved by its
// caller, one instance at a time (HODLRnD include/HDD_matrix.hpp:20-62).
//
// Admission uses hodlr_predict_bytes: the tree, lists and near field are
// counted exactly on the host; far-block ranks come from a prior rank model
// scaled by a correction learned from the builds this server has finished
// (the ratio of measured to predicted far bytes, per dimension and kernel).
//
// With hodlr_server_params.simulate set, workers do not touch the GPU: a
// build "takes" 1 ms per 10^4 points and reports its predicted bytes, a solve
// "takes" 0.5 ms per right-hand side and returns x = b.  That mode drives the
// admission, eviction and ordering logic on machines without a GPU.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/hodlrnd.h"
#include "tree.hpp"

namespace hodlr {
void set_thread_error(const std::string& msg);  // engine.cu: hodlr_last_error(NULL)
}
cudaStream_t ctx_stream(const hodlr_ctx* ctx);  // engine.cu: the context's stream

namespace {

using Clock = std::chrono::steady_clock;

double seconds_since(Clock::time_point t0) {
  return std::chrono::duration<double>(Clock::now() - t0).count();
}

int fail(int code, const std::string& msg) {
  hodlr::set_thread_error(msg);
  return code;
}

// ---- byte predictor ---------------------------------------------------------

// Prior rank of an admissible block of min(m, n) = k points: ranks grow with
// log(1/eps) and, for the kernels here, roughly like log(1/eps)^(ndim-1)
// (the number of terms of a d-dimensional multipole expansion to that
// accuracy), capped by k.  Constants fitted to the 2D / 3D / 4D cases of the
// test suite; the server corrects them from what it measures.
double prior_rank(int ndim, double eps, int64_t k) {
  const double digits = std::max(1.0, std::log10(1.0 / eps));
  const double r = 2.0 + 1.5 * digits * std::pow(double(std::max(ndim - 1, 1)), 1.5);
  return std::min(double(k), std::ceil(r));
}

// ACA workspace of a build in the request loop (MiB): builds run side by
// side, so each keeps its transient workspace small.
constexpr int kServerAcaMiB = 4096;

struct Prediction {
  uint64_t near_bytes = 0, far_bytes = 0, vector_bytes = 0, build_bytes = 0;
  int64_t far_blocks = 0;
  uint64_t total(double far_scale) const {
    return near_bytes + uint64_t(double(far_bytes) * far_scale) + vector_bytes + build_bytes;
  }
};

int predict(const hodlr_params& p, const double* pts, int64_t n, const double* lo, const double* hi,
            Prediction* out) {
  hodlr::TreeParams tp;
  tp.ndim = p.ndim;
  tp.nmax = p.nmax;
  tp.dprime = p.dprime;
  hodlr::Tree t;
  const std::string err = hodlr::build_tree(tp, pts, n, lo, hi, t);
  if (!err.empty()) return fail(HODLR_ERR_TREE, err);
  const std::vector<hodlr::FarBlock> far = hodlr::far_blocks(t);
  const hodlr::NearList nl = hodlr::near_blocks(t);
  const int L = t.levels - 1;
  Prediction pr;
  double near_entries = 0;
  for (int64_t k = 0; k + 1 < int64_t(nl.leaf_ptr.size()); k++)
    for (int64_t q = nl.leaf_ptr[size_t(k)]; q < nl.leaf_ptr[size_t(k + 1)]; q++)
      near_entries += double(t.count[size_t(t.gid(L, k))]) * double(t.count[size_t(t.gid(L, nl.src[size_t(q)]))]);
  // stored factors, plus the FP64 factors a reduced-precision operator keeps for its FP64 check
  const double fesz = (p.precision == HODLR_PREC_FP64 ? 8.0 : p.precision == HODLR_PREC_BF16_FACTORS ? 2.0 : 4.0) +
                      (p.precision != HODLR_PREC_FP64 && p.fp64_check != HODLR_FP64_CHECK_OFF ? 8.0 : 0.0);
  double far_entries = 0, sum_mn = 0;
  for (const hodlr::FarBlock& b : far) {
    const double m = double(t.count[size_t(t.gid(b.level, b.t))]);
    const double nn = double(t.count[size_t(t.gid(b.level, b.s))]);
    if (m == 0 || nn == 0) continue;
    pr.far_blocks++;
    const double r = prior_rank(p.ndim, p.eps_aca, int64_t(std::min(m, nn)));
    far_entries += (r >= std::min(m, nn) - 1) ? m * nn : r * (m + nn);
    sum_mn += m + nn;
  }
  pr.near_bytes = uint64_t(near_entries * 8.0 * (p.precision == HODLR_PREC_MIXED ? 1.5 : 1.0));
  pr.far_bytes = uint64_t(far_entries * fesz);
  // vectors: [x | z] buffers, per-level output slots, solver vectors, Krylov basis,
  // points, permutation and per-level point maps; plan records per far block
  const double restart = p.restart > 0 ? p.restart : 100;
  const double vb = p.precision == HODLR_PREC_MIXED ? 4.0 : 8.0;
  const double nd = double(n);
  pr.vector_bytes = uint64_t(nd * (2 * 8 + 8 * double(t.levels) + 7 * 8) + (restart + 1) * nd * vb +
                             nd * (8.0 * p.ndim + 8 + 4.0 * t.levels) + double(pr.far_blocks) * 96.0);
  // ACA workspace during the build: FP64 factors of the blocks of one launch,
  // bounded by kServerAcaMiB (the server's builds set aca_workspace_mib), and
  // the growth arena of an eighth of that
  const double ws_cap = double(kServerAcaMiB) * 1048576.0;
  pr.build_bytes = uint64_t(std::min(ws_cap, 8.0 * (far_entries + 0.25 * sum_mn)) + ws_cap / 8);
  *out = pr;
  return HODLR_OK;
}

// ---- server -----------------------------------------------------------------

struct Geometry {
  uint64_t key = 0;
  hodlr_ctx* ctx = nullptr;
  hodlr_op* op = nullptr;
  uint64_t bytes = 0;   // reserved while resident
  int busy = 0;
  uint64_t last_use = 0;
  int64_t n = 0;
  int ndim = 0;
};

struct Job {
  uint64_t ticket = 0;
  uint64_t key = 0;
  hodlr_params params{};
  hodlr_kernel_desc kernel{};
  std::vector<double> points, lo, hi, b;
  int64_t n = 0, nrhs = 0;
  Clock::time_point t_submit;
  Prediction pred;
  bool has_pred = false;   // pred computed (points given and no resident operator expected)
  uint64_t predicted = 0;  // bytes reserved at admission for a build
};

struct Done {
  hodlr_result res{};
  std::vector<double> x;
  bool ready = false;
};

}  // namespace

struct hodlr_server {
  hodlr_server_params p{};
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<std::unique_ptr<Job>> queue;
  std::unordered_map<uint64_t, std::unique_ptr<Geometry>> resident;
  std::map<uint64_t, Done> done;
  uint64_t next_ticket = 1, tick = 0;
  uint64_t used = 0;  // resident + reserved for running requests
  int running = 0;
  bool stop = false;
  std::map<int, double> far_scale;  // learned: key ndim * 16 + kernel kind
  std::set<uint64_t> building;      // keys whose build is running
  hodlr_server_stats st{};
  std::vector<std::thread> workers;
  cudaEvent_t t0_event = nullptr;   // recorded at creation: the origin of the requests' device times

  double scale_for(int ndim, int kind) {
    auto it = far_scale.find(ndim * 16 + kind);
    return it == far_scale.end() ? 1.0 : it->second;
  }
};

namespace {

uint64_t solve_extra_bytes(const Job& j) { return j.nrhs > 1 ? uint64_t(j.n) * uint64_t(j.nrhs) * 16 : 0; }

// Evicts idle resident geometries, least recently used first, until `need`
// more bytes fit or none is left.  Called with the lock held; the operator is
// destroyed outside the lock by the caller (returned in `victims`).
void evict_for(hodlr_server* s, uint64_t need, std::vector<std::unique_ptr<Geometry>>& victims) {
  while (s->used + need > s->p.memory_budget_bytes) {
    Geometry* best = nullptr;
    for (auto& kv : s->resident)
      if (!kv.second->busy && (!best || kv.second->last_use < best->last_use)) best = kv.second.get();
    if (!best) return;
    s->used -= best->bytes;
    s->st.evictions++;
    auto it = s->resident.find(best->key);
    victims.push_back(std::move(it->second));
    s->resident.erase(it);
  }
}

struct Admitted {
  std::unique_ptr<Job> job;
  Geometry* geo = nullptr;  // resident geometry to reuse, or null to build
  uint64_t reserved = 0;
};

// Picks the first queued request that can run now (FIFO among those that
// fit).  Lock held.
bool admit(hodlr_server* s, Admitted& a, std::vector<std::unique_ptr<Geometry>>& victims) {
  std::set<uint64_t> blocked;  // keys of earlier requests still queued: later ones must not overtake them
  size_t q = 0;
  while (q < s->queue.size()) {
    Job& j = *s->queue[q];
    if (j.key && blocked.count(j.key)) {
      q++;
      continue;
    }
    const uint64_t extra = solve_extra_bytes(j);
    auto g = j.key ? s->resident.find(j.key) : s->resident.end();
    if (g != s->resident.end()) {
      if (g->second->busy) {  // one request at a time per operator
        blocked.insert(j.key);
        q++;
        continue;
      }
      g->second->busy = 1;  // protect it from eviction below
      evict_for(s, extra, victims);
      if (s->used + extra > s->p.memory_budget_bytes) {
        g->second->busy = 0;
        blocked.insert(j.key);
        q++;
        continue;
      }
      s->used += extra;
      a.geo = g->second.get();
      a.reserved = extra;
      a.job = std::move(s->queue[q]);
      s->queue.erase(s->queue.begin() + long(q));
      s->st.resident_hits++;
      return true;
    }
    if (j.key && s->building.count(j.key)) {  // wait for that build, then reuse it
      q++;
      continue;
    }
    if (j.points.empty()) {
      // submitted against a resident key that has been evicted since
      Done& d = s->done[j.ticket];
      d.res.status = HODLR_ERR_STATE;
      std::strncpy(d.res.message, "the geometry is no longer resident; submit it again with its points",
                   sizeof(d.res.message) - 1);
      d.ready = true;
      s->queue.erase(s->queue.begin() + long(q));
      s->cv_done.notify_all();
      continue;
    }
    if (!j.has_pred) {  // the resident operator it expected is gone: predict now
      if (predict(j.params, j.points.data(), j.n, j.lo.data(), j.hi.data(), &j.pred) == HODLR_OK) j.has_pred = true;
    }
    const uint64_t need = j.pred.total(s->scale_for(j.params.ndim, j.kernel.kind)) + extra;
    if (!j.has_pred || need > s->p.memory_budget_bytes) {  // can never fit
      Done& d = s->done[j.ticket];
      d.res.status = j.has_pred ? HODLR_ERR_BUDGET : HODLR_ERR_TREE;
      d.res.predicted_bytes = need;
      std::strncpy(d.res.message,
                   j.has_pred ? "predicted device bytes exceed the server's memory budget" : "the tree cannot be built",
                   sizeof(d.res.message) - 1);
      d.ready = true;
      s->st.rejected++;
      s->queue.erase(s->queue.begin() + long(q));
      s->cv_done.notify_all();
      continue;
    }
    evict_for(s, need, victims);
    if (s->used + need > s->p.memory_budget_bytes) {
      if (j.key) blocked.insert(j.key);
      q++;
      continue;
    }
    s->used += need;
    j.predicted = need;
    if (j.key) s->building.insert(j.key);
    a.reserved = need;
    a.job = std::move(s->queue[q]);
    s->queue.erase(s->queue.begin() + long(q));
    return true;
  }
  return false;
}

void destroy_geometry(Geometry* g) {
  if (!g) return;
  if (g->op) hodlr_op_destroy(g->op);
  if (g->ctx) hodlr_ctx_destroy(g->ctx);
  g->op = nullptr;
  g->ctx = nullptr;
}

// Runs one admitted request outside the lock; returns the result and leaves
// a built geometry in `built` (null when the request used a resident one).
void execute(hodlr_server* s, Admitted& a, Done& d, std::unique_ptr<Geometry>& built, double t_admit) {
  Job& j = *a.job;
  hodlr_result& r = d.res;
  r.t_queue_s = t_admit;
  r.predicted_bytes = a.geo ? 0 : a.reserved - solve_extra_bytes(j) - j.pred.build_bytes;
  r.predicted_build_bytes = a.geo ? 0 : j.pred.build_bytes;
  d.x.assign(size_t(j.n * j.nrhs), 0.0);
  Geometry* g = a.geo;
  const auto t0 = Clock::now();
  cudaEvent_t ev[2] = {nullptr, nullptr};
  auto mark = [&](int k) {  // event k on the geometry's stream (device times of the request)
    if (s->p.simulate || !s->t0_event || !g || !g->ctx) return;
    if (cudaSetDevice(s->p.device) != cudaSuccess || cudaEventCreate(&ev[k]) != cudaSuccess) {
      ev[k] = nullptr;
      return;
    }
    cudaEventRecord(ev[k], ctx_stream(g->ctx));
  };
  if (!g) {
    built.reset(new Geometry());
    g = built.get();
    g->key = j.key;
    g->n = j.n;
    g->ndim = j.params.ndim;
    r.built = 1;
    if (s->p.simulate) {
      std::this_thread::sleep_for(std::chrono::microseconds(int64_t(1e3 * double(j.n) / 1e4)));
      g->bytes = a.reserved - solve_extra_bytes(j) - j.pred.build_bytes;
    } else {
      hodlr_params p = j.params;
      p.device = s->p.device;
      p.device_budget_bytes = 0;  // admission already accounted for it
      if (p.aca_workspace_mib == 0) p.aca_workspace_mib = kServerAcaMiB;
      int rc = hodlr_ctx_create(&p, &g->ctx);
      if (rc == HODLR_OK) mark(0);
      if (rc == HODLR_OK)
        rc = hodlr_build(g->ctx, j.points.data(), j.n, j.lo.data(), j.hi.data(), &j.kernel, &g->op);
      if (rc != HODLR_OK) {
        r.status = rc;
        std::strncpy(r.message, hodlr_last_error(g->ctx), sizeof(r.message) - 1);
        destroy_geometry(g);
        built.reset();
        r.t_total_s = seconds_since(j.t_submit);
        return;
      }
      hodlr_stats stv;
      hodlr_stats_get(g->op, &stv);
      g->bytes = stv.device_bytes;
    }
    r.actual_bytes = g->bytes;
  } else {
    r.actual_bytes = g->bytes;
    mark(0);
  }
  const auto t1 = Clock::now();
  r.t_build_s = std::chrono::duration<double>(t1 - t0).count();
  if (s->p.simulate) {
    std::this_thread::sleep_for(std::chrono::microseconds(500 * j.nrhs));
    d.x = j.b;
    r.status = HODLR_OK;
    r.iterations = j.nrhs;
  } else {
    hodlr_solve_info info;
    const int rc = hodlr_solve(g->op, j.b.data(), d.x.data(), j.nrhs, &info);
    r.status = rc;
    r.iterations = info.iterations;
    r.rel_residual = info.rel_residual;
    if (rc != HODLR_OK) std::strncpy(r.message, hodlr_last_error(g->ctx), sizeof(r.message) - 1);
    mark(1);
    if (ev[0] && ev[1] && cudaEventSynchronize(ev[1]) == cudaSuccess) {
      float a0 = 0.f, a1 = 0.f;
      if (cudaEventElapsedTime(&a0, s->t0_event, ev[0]) == cudaSuccess &&
          cudaEventElapsedTime(&a1, s->t0_event, ev[1]) == cudaSuccess) {
        r.t_device_start_s = 1e-3 * double(a0);
        r.t_device_end_s = 1e-3 * double(a1);
      }
    }
    for (cudaEvent_t e : ev)
      if (e) cudaEventDestroy(e);
  }
  r.t_solve_s = seconds_since(t1);
  r.t_total_s = seconds_since(j.t_submit);
}

// The operator of a request is kept resident when its build succeeded,
// whatever the solve's outcome (non-convergence included).
bool g_built_ok(const hodlr_result& r) { return r.built == 1 && r.actual_bytes > 0; }

void worker(hodlr_server* s) {
  std::unique_lock<std::mutex> lock(s->mu);
  for (;;) {
    Admitted a;
    std::vector<std::unique_ptr<Geometry>> victims;
    while (!s->stop && !(s->running < s->p.slots && admit(s, a, victims))) {
      if (!victims.empty()) break;
      s->cv_work.wait(lock);
    }
    if (!victims.empty() && !a.job) {
      lock.unlock();
      for (auto& v : victims) destroy_geometry(v.get());
      victims.clear();
      lock.lock();
      continue;
    }
    if (!a.job) return;  // stopping and nothing admitted
    s->running++;
    const double t_admit = seconds_since(a.job->t_submit);
    lock.unlock();
    for (auto& v : victims) destroy_geometry(v.get());
    Done d;
    std::unique_ptr<Geometry> built;
    execute(s, a, d, built, t_admit);
    lock.lock();
    s->running--;
    Job& j = *a.job;
    const uint64_t extra = solve_extra_bytes(j);
    if (a.geo) {
      s->used -= extra;
      a.geo->busy = 0;
      a.geo->last_use = ++s->tick;
    } else {
      s->used -= a.reserved;
      if (j.key) s->building.erase(j.key);
      if (built) {
        // learn: measured / predicted far bytes for this dimension and kernel
        if (!s->p.simulate && j.pred.far_bytes > 0) {
          const double fixed = double(j.pred.near_bytes + j.pred.vector_bytes);
          const double ratio = std::max(0.05, (double(built->bytes) - fixed) / double(j.pred.far_bytes));
          double& f = s->far_scale[j.params.ndim * 16 + j.kernel.kind];
          if (f == 0.0) f = ratio;
          else f = 0.5 * f + 0.5 * ratio;
        }
        s->st.builds++;
        if (j.key && g_built_ok(d.res)) {
          built->busy = 0;
          built->last_use = ++s->tick;
          s->used += built->bytes;
          s->resident[j.key] = std::move(built);
        }
      }
    }
    if (built) {  // not kept: free it outside the lock
      lock.unlock();
      destroy_geometry(built.get());
      built.reset();
      lock.lock();
    }
    s->st.completed++;
    s->st.rhs_solved += uint64_t(j.nrhs);
    s->done[j.ticket] = std::move(d);
    s->done[j.ticket].ready = true;
    s->cv_done.notify_all();
    s->cv_work.notify_all();
  }
}

}  // namespace

extern "C" {

int hodlr_predict_bytes(const hodlr_params* params, const double* points, int64_t n, const double* box_lo,
                        const double* box_hi, uint64_t* bytes) {
  if (!params || !points || !box_lo || !box_hi || !bytes || n < 1)
    return fail(HODLR_ERR_INVALID, "hodlr_predict_bytes: bad argument");
  Prediction pr;
  const int rc = predict(*params, points, n, box_lo, box_hi, &pr);
  if (rc != HODLR_OK) return rc;
  *bytes = pr.total(1.0);
  return HODLR_OK;
}

int hodlr_server_create(const hodlr_server_params* params, hodlr_server** out) {
  if (!params || !out) return fail(HODLR_ERR_INVALID, "hodlr_server_create: null argument");
  *out = nullptr;
  if (params->slots < 0 || params->slots > 64) return fail(HODLR_ERR_INVALID, "slots must be in 0..64");
  hodlr_server* s = new hodlr_server();
  s->p = *params;
  if (s->p.slots == 0) s->p.slots = 4;
  if (s->p.memory_budget_bytes == 0) s->p.memory_budget_bytes = uint64_t(150) << 30;
  if (!s->p.simulate) {
    cudaError_t e = cudaSetDevice(s->p.device);
    if (e == cudaSuccess) e = cudaEventCreate(&s->t0_event);
    if (e == cudaSuccess) e = cudaEventRecord(s->t0_event, nullptr);
    if (e == cudaSuccess) e = cudaEventSynchronize(s->t0_event);
    if (e != cudaSuccess) {
      if (s->t0_event) cudaEventDestroy(s->t0_event);
      delete s;
      return fail(HODLR_ERR_CUDA, std::string("hodlr_server_create: ") + cudaGetErrorString(e));
    }
  }
  for (int i = 0; i < s->p.slots; i++) s->workers.emplace_back(worker, s);
  *out = s;
  return HODLR_OK;
}

int hodlr_server_submit(hodlr_server* s, const hodlr_request* req, uint64_t* ticket) {
  if (!s || !req || !ticket) return fail(HODLR_ERR_INVALID, "hodlr_server_submit: null argument");
  const hodlr_params& p = req->params;
  if (req->n < 1 || req->nrhs < 1 || !req->b || p.ndim < 1 || p.ndim > hodlr::kMaxDim)
    return fail(HODLR_ERR_INVALID, "hodlr_server_submit: bad request (n, nrhs, b or ndim)");
  std::unique_ptr<Job> j(new Job());
  j->key = req->geometry_key;
  j->params = p;
  j->kernel = req->kernel;
  j->n = req->n;
  j->nrhs = req->nrhs;
  j->b.assign(req->b, req->b + req->n * req->nrhs);
  j->t_submit = Clock::now();
  if (req->points) {
    if (!req->box_lo || !req->box_hi) return fail(HODLR_ERR_INVALID, "hodlr_server_submit: points without a box");
    j->points.assign(req->points, req->points + req->n * p.ndim);
    j->lo.assign(req->box_lo, req->box_lo + p.ndim);
    j->hi.assign(req->box_hi, req->box_hi + p.ndim);
    // the prediction (a host tree build) is skipped when the key's operator is
    // resident, being built or queued for a build: the request will reuse it
    bool reuse = false;
    if (j->key) {
      std::lock_guard<std::mutex> lock(s->mu);
      reuse = s->resident.count(j->key) || s->building.count(j->key);
      for (const auto& q : s->queue)
        if (q->key == j->key && !q->points.empty()) reuse = true;
    }
    if (!reuse) {
      const int rc = predict(p, j->points.data(), j->n, j->lo.data(), j->hi.data(), &j->pred);
      if (rc != HODLR_OK) return rc;
      j->has_pred = true;
    }
  } else if (!j->key) {
    return fail(HODLR_ERR_INVALID, "hodlr_server_submit: points are needed without a geometry key");
  }
  std::lock_guard<std::mutex> lock(s->mu);
  if (s->stop) return fail(HODLR_ERR_STATE, "hodlr_server_submit: the server is shutting down");
  j->ticket = s->next_ticket++;
  *ticket = j->ticket;
  s->done[j->ticket] = Done();
  s->st.submitted++;
  s->queue.push_back(std::move(j));
  s->cv_work.notify_all();
  return HODLR_OK;
}

int hodlr_server_wait(hodlr_server* s, uint64_t ticket, double timeout_s, double* x, hodlr_result* result) {
  if (!s) return fail(HODLR_ERR_INVALID, "hodlr_server_wait: null server");
  std::unique_lock<std::mutex> lock(s->mu);
  auto it = s->done.find(ticket);
  if (it == s->done.end()) return fail(HODLR_ERR_INVALID, "hodlr_server_wait: unknown ticket");
  const auto deadline = Clock::now() + std::chrono::duration_cast<Clock::duration>(
                                           std::chrono::duration<double>(timeout_s < 0 ? 1e9 : timeout_s));
  while (!it->second.ready) {
    if (s->cv_done.wait_until(lock, deadline) == std::cv_status::timeout && !it->second.ready)
      return fail(HODLR_ERR_TIMEOUT, "hodlr_server_wait: not finished yet");
    it = s->done.find(ticket);
  }
  Done d = std::move(it->second);
  s->done.erase(it);
  lock.unlock();
  if (result) *result = d.res;
  if (x && !d.x.empty()) std::memcpy(x, d.x.data(), d.x.size() * sizeof(double));
  return d.res.status;
}

int hodlr_server_stats_get(hodlr_server* s, hodlr_server_stats* out) {
  if (!s || !out) return fail(HODLR_ERR_INVALID, "hodlr_server_stats_get: null argument");
  std::lock_guard<std::mutex> lock(s->mu);
  *out = s->st;
  out->queued = int64_t(s->queue.size());
  out->running = s->running;
  out->resident = int64_t(s->resident.size());
  out->used_bytes = s->used;
  return HODLR_OK;
}

int hodlr_server_destroy(hodlr_server* s) {
  if (!s) return HODLR_OK;
  {
    std::unique_lock<std::mutex> lock(s->mu);
    // finish what was submitted, then stop
    s->cv_done.wait(lock, [s] { return s->queue.empty() && s->running == 0; });
    s->stop = true;
    s->cv_work.notify_all();
  }
  for (auto& t : s->workers) t.join();
  for (auto& kv : s->resident) destroy_geometry(kv.second.get());
  if (s->t0_event) cudaEventDestroy(s->t0_event);
  delete s;
  return HODLR_OK;
}

}  // extern "C"
