// C ABI of the GB300 HODLRnD engine (include/hodlrnd.h): build pipeline,
// operator application and solves.  One process, one GPU; all device memory
// of an operator is owned by its hodlr_op.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/hodlrnd.h"
#include "aca.h"
#include "dtree.h"
#include "gmres.h"
#include "matvec.h"
#include "par.h"
#include "tc.h"
#include "tree.hpp"

using namespace hodlr;

namespace {
thread_local std::string g_thread_err;
}

namespace hodlr {
void set_thread_error(const std::string& msg) { g_thread_err = msg; }
}  // namespace hodlr

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Failure {
  int code;
  std::string msg;
};

void check_cuda(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return;
  const int code = (e == cudaErrorMemoryAllocation) ? HODLR_ERR_OOM : HODLR_ERR_CUDA;
  throw Failure{code, std::string(what) + ": " + cudaGetErrorString(e)};
}
#define CK(x) check_cuda((x), #x)

// Device allocation tracked against the context's budget.
struct DevMem {
  uint64_t used = 0, budget = 0;
  std::vector<std::pair<void*, size_t>> blocks;
  void* alloc(size_t bytes, const char* what) {
    if (bytes == 0) bytes = 16;
    if (budget && used + bytes > budget)
      throw Failure{HODLR_ERR_BUDGET, std::string(what) + ": device budget of " + std::to_string(budget) +
                                          " bytes exceeded (" + std::to_string(used + bytes) + " needed)"};
    void* p = nullptr;
    check_cuda(cudaMalloc(&p, bytes), what);
    used += bytes;
    blocks.push_back({p, bytes});
    return p;
  }
  template <typename T>
  T* alloc_n(size_t n, const char* what) {
    return static_cast<T*>(alloc(n * sizeof(T), what));
  }
  void release(void* p) {
    for (size_t i = 0; i < blocks.size(); i++)
      if (blocks[i].first == p) {
        cudaFree(p);
        used -= blocks[i].second;
        blocks.erase(blocks.begin() + long(i));
        return;
      }
  }
  void release_all() {
    for (auto& b : blocks) cudaFree(b.first);
    blocks.clear();
    used = 0;
  }
};

template <typename T>
T* upload(DevMem& mem, const std::vector<T>& v, cudaStream_t st, const char* what) {
  T* d = mem.alloc_n<T>(std::max<size_t>(v.size(), 1), what);
  if (!v.empty()) CK(cudaMemcpyAsync(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st));
  return d;
}

uint64_t block_seed(int64_t level, int64_t t, int64_t s) {
  // the same mixing as the CPU oracle's per-block mode
  uint64_t h = 0x243F6A8885A308D3ull;
  const uint64_t v[3] = {uint64_t(level), uint64_t(t), uint64_t(s)};
  for (int i = 0; i < 3; i++) {
    h ^= v[i] + 0x9E3779B97F4A7C15ull + (h << 6) + (h >> 2);
    h *= 0xD6E8FEB86659FD93ull;
    h ^= h >> 32;
  }
  return h;
}

// CUDA events around operator launches (hodlr_trace_*).
struct Tracer {
  bool on = false;
  std::vector<cudaEvent_t> pool;
  std::vector<std::pair<int, size_t>> pending;  // kind, index of the start event (stop = +1)
  size_t used = 0;
  uint64_t launches[HODLR_TRACE_KINDS] = {};
  double ms[HODLR_TRACE_KINDS] = {};
  double bytes[HODLR_TRACE_KINDS] = {};
  void start(int kind, cudaStream_t st) {
    if (!on) return;
    while (pool.size() < used + 2) {
      cudaEvent_t e;
      check_cuda(cudaEventCreate(&e), "cudaEventCreate");
      pool.push_back(e);
    }
    check_cuda(cudaEventRecord(pool[used], st), "cudaEventRecord");
    pending.push_back({kind, used});
    used += 2;
  }
  void stop(cudaStream_t st) {
    if (!on || pending.empty()) return;
    check_cuda(cudaEventRecord(pool[pending.back().second + 1], st), "cudaEventRecord");
  }
  void harvest() {
    for (auto& p : pending) {
      check_cuda(cudaEventSynchronize(pool[p.second + 1]), "cudaEventSynchronize");
      float t = 0.f;
      check_cuda(cudaEventElapsedTime(&t, pool[p.second], pool[p.second + 1]), "cudaEventElapsedTime");
      launches[p.first]++;
      ms[p.first] += double(t);
    }
    pending.clear();
    used = 0;
  }
  void reset() {
    pending.clear();
    used = 0;
    for (int k = 0; k < HODLR_TRACE_KINDS; k++) {
      launches[k] = 0;
      ms[k] = 0.0;
    }
  }
  ~Tracer() {
    for (cudaEvent_t e : pool) cudaEventDestroy(e);
  }
};

// Device side of one way of applying the operator (a plan).
struct Plan {
  Prec a_near = Prec::kD, a_far = Prec::kD;
  Panel* panels_near = nullptr;
  Seg* segs_near = nullptr;
  Item* small_near = nullptr;  // items of panels with at most 32 rows
  Item* big_near = nullptr;    // items of larger panels (row tiles)
  int nsmall_near = 0, nbig_near = 0;
  Panel* panels_far = nullptr;
  Seg* segs_far = nullptr;
  Item* small_far = nullptr;
  Item* big_far = nullptr;
  int nsmall_far = 0, nbig_far = 0;
  ZBlock* zb = nullptr;
  int nzb = 0;
  ZItem* zitems = nullptr;
  int nzitems = 0;
  ZFix* zfix = nullptr;
  int nzfix = 0;
  PanelFix* pfix_far = nullptr;
  int npfix_far = 0;
  PanelFix* pfix_near = nullptr;  // near panels above 32 rows split over items (share ypart with the far ones)
  int npfix_near = 0;
  int64_t nypart_near = 0;
  // small items stream their segments as one byte run (small_items_contiguous)
  bool contig_near = false, contig_far = false;
  int64_t nzpart = 0, nypart = 0;  // partial-sum scratch (elements of the vector type)
  void* zpart = nullptr;
  void* ypart = nullptr;
  // host copies of the arrays above, kept for operators of a batch (merged
  // into the batch's plan)
  struct Host {
    std::vector<Panel> panels_near, panels_far;
    std::vector<Seg> segs_near, segs_far;
    std::vector<Item> small_near, big_near, small_far, big_far;
    std::vector<PanelFix> pfix_near, pfix_far;
    std::vector<ZBlock> zb;
    std::vector<ZItem> zitems;
    std::vector<ZFix> zfix;
  };
  std::shared_ptr<Host> host;
};

}  // namespace

struct hodlr_ctx {
  hodlr_params p;
  std::string err;
  cudaStream_t stream = nullptr;
};

struct hodlr_op {
  hodlr_ctx* ctx = nullptr;
  bool keep_host_plans = false;  // set for the operators of a batch
  std::vector<double> box_lo, box_hi;  // the build's bounding box (kept for hodlr_op_save)
  std::vector<void*> far_chunks; // factor chunks written by the ACA batches (freed by relayout_far)
  bool batch_owned = false;      // freed by hodlr_batch_destroy only
  bool relaxed = false;  // FP32 factors: matvecs use relaxed accumulation (set by the solver)
  unsigned int* h_waits = nullptr;  // pinned: streaming-kernel wait give-ups (read_stream_timeouts)
  unsigned int waits_seen = 0;
  hodlr_params p;
  hodlr_kernel_desc kd;
  Tree tree;
  std::vector<FarBlock> far;
  NearList near;
  std::vector<int32_t> rank, dense;
  std::vector<const void*> uptr, vptr;  // stored factors (or dense tile) of each far block
  // FP32 / BF16 V factors after the relayout: the low-rank blocks of one source
  // node share row-major chunks of at most 128 columns.  Per block: the row
  // stride of its chunk (elements; 0: its own vpad(rank)), its z scales (BF16)
  // and the position of its z in the input buffer [x | z].
  struct VChunk {
    const void* V;          // n x w, row major
    int64_t x_off, zbase;   // source node's first tree position; z position of column 0
    int32_t n, w;
    const float* zscale;    // BF16: w scales
  };
  std::vector<VChunk> vchunks;
  std::vector<int64_t> vstride, zpos;
  std::vector<int32_t> vchunk_of;  // the chunk of each low-rank block (-1: none)
  std::vector<const float*> zsptr;
  // reduced-precision operators with the FP64 check: the FP64 factors of
  // every far block and the FP64 operator's plan (the refinement residuals)
  bool has_ref = false;
  std::vector<const void*> uptr64, vptr64;
  Plan plan_ref;
  // tensor-core products for 64 right-hand sides (BF16 factors; built on first use)
  struct TcPlan {
    // one launch per (family, small / big, rows bucket): items of at most
    // `rows` output rows, so each launch holds just the tensor memory and
    // shared memory its items need
    struct Run {
      const void* items;  // Item (panels) or TcZGroup (z)
      int n, rows, big;
    };
    bool built = false;
    std::vector<Run> near, far, z;
    PanelFix *fix_near = nullptr, *fix_far = nullptr;
    int nfix_near = 0, nfix_far = 0;
    TcZEntry* ze = nullptr;
    TcZFix* zfix = nullptr;  // split z groups
    TcZRow* zrows = nullptr;
    int nzfix = 0, zfix_rows = 0;
    uint32_t* in = nullptr;  // [x | z], 64 right-hand sides, packed BF16 pairs
    float *y = nullptr, *part_near = nullptr, *part_far = nullptr, *zpart = nullptr;
    unsigned int* status = nullptr;
    unsigned int* h_status = nullptr;
  } tc;
  int64_t n = 0, zlen = 0;
  int nslots = 0;
  DevMem mem;
  double* d_pts = nullptr;  // ndim x n, tree order
  int64_t* d_perm = nullptr;
  int32_t* d_lmap = nullptr;  // levels x n: reference order of each node's points (tree positions)
  Plan plan64;        // FP64 operator, or the FP64-vector operator of MIXED (FP32 far factors)
  Plan plan32;        // MIXED inner operator (all FP32)
  // work vectors
  double* d_in64 = nullptr;  // [x | z], n + zlen
  void* d_in2 = nullptr;     // [x | z] as (hi, lo) FP32 pairs: FP32 factors with FP64 vectors
  double* d_y64 = nullptr;   // nslots x n
  float* d_in32 = nullptr;
  float* d_y32 = nullptr;
  double* d_b64 = nullptr;   // tree-order right-hand side / solution / residual
  double* d_x64 = nullptr;
  double* d_r64 = nullptr;
  float* d_r32 = nullptr;
  float* d_d32 = nullptr;
  double* d_rref = nullptr;  // FP64 check: the refinement residual and correction, n each
  double* d_dref = nullptr;
  double* d_io = nullptr;    // caller-order staging, n
  double* d_io2 = nullptr;
  double* d_hb = nullptr;    // host-API staging of one right-hand side and its solution
  double* d_hx = nullptr;
  double* d_part = nullptr;  // kVecCtas partials
  double* d_scal = nullptr;  // scalars
  double* h_scal = nullptr;  // pinned
  GmresWork<double> g64;
  GmresWork<float> g32;
  hodlr_stats st;
  Tracer tr;
  ~hodlr_op() {
    gmres_free(g64);
    gmres_free(g32);
    if (h_scal) cudaFreeHost(h_scal);
    if (h_waits) cudaFreeHost(h_waits);
    if (tc.h_status) cudaFreeHost(tc.h_status);
    mem.release_all();
  }
};

namespace {

int fail(hodlr_ctx* ctx, int code, const std::string& msg) {
  g_thread_err = msg;
  if (ctx) ctx->err = msg;
  return code;
}

// ---------------------------------------------------------------- build steps

// For every level, the tree positions of each node's points listed in the
// reference's order (increasing caller index; cluster::binary_clustering keeps
// the parent's order, HDD_clusters.hpp:124-127).  Within a leaf that is the
// tree order itself; a non-leaf node's tree range is grouped by leaf instead.
std::vector<int32_t> reference_order_map(const Tree& t) {
  const int64_t n = t.n;
  const int L = t.levels - 1, d = t.p.ndim;
  std::vector<int32_t> map(size_t(n) * size_t(t.levels));
  std::vector<int64_t> inv(static_cast<size_t>(n)), leaf_of(static_cast<size_t>(n));
  for (int64_t q = 0; q < n; q++) inv[size_t(t.perm[size_t(q)])] = q;
  for (int64_t k = 0; k < t.level_size[size_t(L)]; k++) {
    const int64_t g = t.gid(L, k);
    for (int64_t q = t.begin[size_t(g)]; q < t.begin[size_t(g)] + t.count[size_t(g)]; q++) leaf_of[size_t(q)] = k;
  }
  for (int l = 0; l <= L; l++) {
    std::vector<int64_t> cur(static_cast<size_t>(t.level_size[size_t(l)]));
    for (int64_t k = 0; k < t.level_size[size_t(l)]; k++) cur[size_t(k)] = t.begin[size_t(t.gid(l, k))];
    int32_t* out = map.data() + size_t(l) * size_t(n);
    const int shift = d * (L - l);
    for (int64_t i = 0; i < n; i++) {  // caller order
      const int64_t q = inv[size_t(i)];
      const int64_t node = leaf_of[size_t(q)] >> shift;
      out[cur[size_t(node)]++] = int32_t(q);
    }
  }
  return map;
}

struct NearTiles {
  std::vector<TileDesc> tiles;
  int64_t total = 0;
};

NearTiles near_tiles(const Tree& t, const NearList& nl, int esz) {
  NearTiles out;
  const int L = t.levels - 1;
  for (int64_t k = 0; k + 1 < int64_t(nl.leaf_ptr.size()); k++)
    for (int64_t q = nl.leaf_ptr[size_t(k)]; q < nl.leaf_ptr[size_t(k + 1)]; q++) {
      const int64_t s = nl.src[size_t(q)];
      const int64_t gt = t.gid(L, k), gs = t.gid(L, s);
      TileDesc d;
      d.t_begin = t.begin[size_t(gt)];
      d.s_begin = t.begin[size_t(gs)];
      d.m = int32_t(t.count[size_t(gt)]);
      d.n = int32_t(t.count[size_t(gs)]);
      d.off = out.total;
      out.total += (stored_elems(d.m, d.n, esz) + 3) / 4 * 4;
      out.tiles.push_back(d);
    }
  return out;
}

// Columns one panel item takes before its panel chunk is split over items:
// far panels above 32 rows are many (one per node and level), near ones are
// few (leaves above 32 points) and get more, smaller items.
constexpr int kPanelCols = 256;
// factor bytes per leaf-panel item, about (HODLR_TUNE_SMALL_ITEM_BYTES overrides it for tuning runs)
#ifndef HODLR_TUNE_SMALL_ITEM_BYTES
#define HODLR_TUNE_SMALL_ITEM_BYTES (48 * 1024)
#endif
constexpr int64_t kSmallItemBytes = HODLR_TUNE_SMALL_ITEM_BYTES;
constexpr int kNearPanelCols = 48;

// Runs of consecutive segments [begin, end) with about `max_cols` columns each.
std::vector<std::pair<int32_t, int32_t>> column_groups(const std::vector<Seg>& segs, int64_t begin, int64_t end,
                                                       int max_cols) {
  std::vector<std::pair<int32_t, int32_t>> groups;
  int32_t gb = int32_t(begin), cols = 0;
  for (int64_t q = begin; q < end; q++) {
    if (cols > 0 && cols + segs[size_t(q)].K > max_cols) {
      groups.push_back({gb, int32_t(q)});
      gb = int32_t(q);
      cols = 0;
    }
    cols += segs[size_t(q)].K;
  }
  groups.push_back({gb, int32_t(end)});
  return groups;
}

void build_near_plan(hodlr_op* op, const NearTiles& nt, const void* base, Prec a, Plan& plan, cudaStream_t st) {
  const Tree& t = op->tree;
  const int L = t.levels - 1;
  std::vector<Panel> panels;
  std::vector<Seg> segs;
  std::vector<Item> small, big;
  std::vector<PanelFix> pfix;
  int64_t nypart = 0;
  const size_t esz = a == Prec::kD ? 8 : 4;
  size_t q = 0;
  for (int64_t k = 0; k + 1 < int64_t(op->near.leaf_ptr.size()); k++) {
    const int64_t b = op->near.leaf_ptr[size_t(k)], e = op->near.leaf_ptr[size_t(k + 1)];
    if (b == e) continue;
    Panel p;
    p.row_begin = t.begin[size_t(t.gid(L, k))];
    p.m = int32_t(t.count[size_t(t.gid(L, k))]);
    p.slot = 0;
    p.yoff = p.row_begin;
    p.seg_begin = int64_t(segs.size());
    for (int64_t z = b; z < e; z++, q++) {
      const TileDesc& d = nt.tiles[q];
      Seg s;
      s.A = static_cast<const char*>(base) + size_t(d.off) * esz;
      s.cscale = nullptr;
      s.in_off = d.s_begin;
      s.K = d.n;
      s.pad = 0;
      segs.push_back(s);
    }
    p.seg_end = int64_t(segs.size());
    const int np = int(panels.size());
    panels.push_back(p);
    if (p.m <= 32) {
      small.push_back({np, 0, int32_t(p.seg_begin), int32_t(p.seg_end), -1});
    } else {
      // as for far panels: runs of about kPanelCols columns per item, partial
      // row blocks added by the fix-up kernel
      const std::vector<std::pair<int32_t, int32_t>> groups = column_groups(segs, p.seg_begin, p.seg_end, kNearPanelCols);
      const int rows = rows_per_item(a);
      for (int c = 0; c < int((p.m + rows - 1) / rows); c++) {
        if (groups.size() == 1) {
          big.push_back({np, c, groups[0].first, groups[0].second, -1});
          continue;
        }
        pfix.push_back({np, c, int32_t(nypart), int32_t(groups.size())});
        for (auto& g : groups) big.push_back({np, c, g.first, g.second, int32_t(nypart++)});
      }
    }
  }
  plan.contig_near = small_items_contiguous(panels, segs, small, int(esz));
  plan.pfix_near = upload(op->mem, pfix, st, "near panel fix-ups");
  plan.npfix_near = int(pfix.size());
  plan.nypart_near = nypart * rows_per_item(a);
  plan.a_near = a;
  plan.panels_near = upload(op->mem, panels, st, "near panels");
  plan.segs_near = upload(op->mem, segs, st, "near segments");
  plan.small_near = upload(op->mem, small, st, "near items");
  plan.big_near = upload(op->mem, big, st, "near items");
  plan.nsmall_near = int(small.size());
  plan.nbig_near = int(big.size());
  if (op->keep_host_plans) {
    if (!plan.host) plan.host = std::make_shared<Plan::Host>();
    plan.host->panels_near = panels;
    plan.host->segs_near = segs;
    plan.host->small_near = small;
    plan.host->big_near = big;
    plan.host->pfix_near = pfix;
  }
}

// Far-field plan from the per-block storage pointers.
void build_far_plan(hodlr_op* op, const std::vector<const void*>& uptr, const std::vector<const void*>& vptr, Prec a,
                    Plan& plan, cudaStream_t st) {
  const Tree& t = op->tree;
  std::vector<Panel> panels;
  std::vector<Seg> segs;
  std::vector<Item> small, big;
  std::vector<ZBlock> zb;
  std::vector<PanelFix> pfix;
  int64_t nypart = 0;
  int64_t zoff = op->n;
  // FP32 / BF16 after the relayout: z = V^T x per chunk of source-node columns
  const bool chunks = a != Prec::kD && !op->vchunks.empty();
  size_t b = 0;
  while (b < op->far.size()) {
    const int l = op->far[b].level;
    const int64_t tk = op->far[b].t;
    size_t e = b;
    while (e < op->far.size() && op->far[e].level == l && op->far[e].t == tk) e++;
    const int64_t gt = t.gid(l, tk);
    Panel p;
    p.row_begin = t.begin[size_t(gt)];
    p.m = int32_t(t.count[size_t(gt)]);
    p.slot = l;
    p.yoff = int64_t(l) * op->n + p.row_begin;
    p.seg_begin = int64_t(segs.size());
    for (size_t q = b; q < e; q++) {
      const int64_t gs = t.gid(l, op->far[q].s);
      const int32_t ns = int32_t(t.count[size_t(gs)]);
      Seg s;
      s.pad = 0;
      s.cscale = nullptr;
      if (op->dense[q]) {
        s.A = uptr[q];
        s.in_off = t.begin[size_t(gs)];
        s.K = ns;
        if (a == Prec::kB)
          s.cscale = reinterpret_cast<const float*>(static_cast<const char*>(uptr[q]) +
                                                    far_u_data_bytes(p.m, ns, 0, true, a));
        segs.push_back(s);
      } else if (op->rank[q] > 0 && chunks) {
        s.A = uptr[q];
        s.in_off = op->zpos[q];
        s.K = op->rank[q];
        segs.push_back(s);
      } else if (op->rank[q] > 0) {
        ZBlock z;
        z.V = vptr[q];
        z.x_off = t.begin[size_t(gs)];
        z.z_off = zoff;
        z.n = ns;
        z.r = op->rank[q];
        z.zscale = a == Prec::kB ? reinterpret_cast<const float*>(static_cast<const char*>(vptr[q]) +
                                                                  far_v_data_bytes(ns, z.r, false, a))
                                 : nullptr;
        zb.push_back(z);
        s.A = uptr[q];
        s.in_off = zoff;
        s.K = op->rank[q];
        segs.push_back(s);
        zoff += op->rank[q];
      }
    }
    p.seg_end = int64_t(segs.size());
    if (p.seg_end > p.seg_begin) {
      const int np = int(panels.size());
      panels.push_back(p);
      if (p.m <= 32) {
        // one warp per leaf panel, or per run of about kSmallItemBytes of its
        // factors when it has more (partial rows added by the fix-up kernel):
        // a few panels with very long interaction lists would otherwise keep
        // single warps busy long after the rest
        const int max_cols = int(std::max<int64_t>(64, kSmallItemBytes / (int64_t(p.m) * prec_size(a))));
        const std::vector<std::pair<int32_t, int32_t>> groups = column_groups(segs, p.seg_begin, p.seg_end, max_cols);
        if (groups.size() == 1) {
          small.push_back({np, 0, int32_t(p.seg_begin), int32_t(p.seg_end), -1});
        } else {
          pfix.push_back({np, 0, int32_t(nypart), int32_t(groups.size())});
          for (auto& g : groups) small.push_back({np, 0, g.first, g.second, int32_t(nypart++)});
        }
      } else {
        const std::vector<std::pair<int32_t, int32_t>> groups = column_groups(segs, p.seg_begin, p.seg_end, kPanelCols);
        const int rows = rows_per_item(a);
        const int chunks = int((p.m + rows - 1) / rows);
        for (int c = 0; c < chunks; c++) {
          if (groups.size() == 1) {
            big.push_back({np, c, groups[0].first, groups[0].second, -1});
            continue;
          }
          pfix.push_back({np, c, int32_t(nypart), int32_t(groups.size())});
          for (auto& g : groups) big.push_back({np, c, g.first, g.second, int32_t(nypart++)});
        }
      }
    }
    b = e;
  }
  if (chunks) {
    for (const hodlr_op::VChunk& c : op->vchunks) {
      ZBlock z;
      z.V = c.V;
      z.x_off = c.x_off;
      z.z_off = c.zbase;
      z.n = c.n;
      z.r = c.w;  // the chunk's columns, padding included (its padding columns give z = 0)
      z.zscale = c.zscale;
      zb.push_back(z);
      zoff = std::max(zoff, c.zbase + c.w);
    }
  }
  // the input buffers hold the longest z of the operator's plans
  op->zlen = std::max(op->zlen, zoff - op->n);
  plan.a_far = a;
  // FP64 far factors stay where the ACA batches put them, so whether a panel's
  // blocks follow one another depends on the batch split (and differs for an
  // operator read from a file): their panels always take the direct-load
  // kernel, whose results do not depend on the layout.  FP32 and BF16 factors
  // are laid out in panel order (relayout_far).
  plan.contig_far = a != Prec::kD && small_items_contiguous(panels, segs, small, prec_size(a));
  plan.panels_far = upload(op->mem, panels, st, "far panels");
  plan.segs_far = upload(op->mem, segs, st, "far segments");
  plan.small_far = upload(op->mem, small, st, "far items");
  plan.big_far = upload(op->mem, big, st, "far items");
  plan.nsmall_far = int(small.size());
  plan.nbig_far = int(big.size());
  // V^T x items: up to 32 sixteen-byte loads of columns by a run of rows of
  // about kZItemBytes; blocks with more rows split into partial sums
  std::vector<ZItem> zit;
  std::vector<ZFix> zfix;
  int64_t nzpart = 0;
  const int esz = prec_size(a);
  const int cmax = std::min(32 * (16 / esz), kZPart);  // BF16: 128 of the 256 a warp could load
  for (size_t q = 0; q < zb.size(); q++) {
    const int n = zb[q].n, r = zb[q].r;
    const int rp = int(vpad(r, esz));
    for (int k0 = 0; k0 < rp; k0 += cmax) {
      const int nk = std::min(cmax, rp - k0);
      const int rows = std::max(1, kZItemBytes / (nk * esz));
      const int groups = (n + rows - 1) / rows;
      if (groups == 1) {
        zit.push_back({int32_t(q), k0, nk, 0, n, -1, 0, 0});
        z_item_stages(zit.back(), r, esz);
        continue;
      }
      for (int c = 0; c < nk && k0 + c < r; c++) zfix.push_back({zb[q].z_off + k0 + c, int32_t(nzpart + c), groups});
      for (int g = 0; g < groups; g++) {
        zit.push_back({int32_t(q), k0, nk, g * rows, std::min(n, (g + 1) * rows), int32_t(nzpart), 0, 0});
        z_item_stages(zit.back(), r, esz);
        nzpart += kZPart;
      }
    }
  }
  plan.zb = upload(op->mem, zb, st, "far z blocks");
  plan.nzb = int(zb.size());
  plan.zitems = upload(op->mem, zit, st, "far z items");
  plan.nzitems = int(zit.size());
  plan.zfix = upload(op->mem, zfix, st, "far z fix-ups");
  plan.nzfix = int(zfix.size());
  plan.pfix_far = upload(op->mem, pfix, st, "far panel fix-ups");
  plan.npfix_far = int(pfix.size());
  plan.nzpart = nzpart;
  plan.nypart = nypart * rows_per_item(a);
  if (op->keep_host_plans) {
    if (!plan.host) plan.host = std::make_shared<Plan::Host>();
    plan.host->panels_far = panels;
    plan.host->segs_far = segs;
    plan.host->small_far = small;
    plan.host->big_far = big;
    plan.host->pfix_far = pfix;
    plan.host->zb = zb;
    plan.host->zitems = zit;
    plan.host->zfix = zfix;
  }
}

// Element type of the far-field storage.
Prec far_prec(const hodlr_params& p) {
  return p.precision == HODLR_PREC_FP64 ? Prec::kD : p.precision == HODLR_PREC_BF16_FACTORS ? Prec::kB : Prec::kF;
}

// Batches of at least kAcaRunMin blocks (run_aca) are compacted kind by
// kind while the other kinds are still being compressed.
constexpr size_t kAcaRunMin = size_t(1) << 18;
constexpr size_t kAcaCtrBytes = 32;  // the arena counter, then the kinds' queue counters (from byte 16)

// Events without timing, destroyed with the set.
struct EventSet {
  std::vector<cudaEvent_t> e;
  explicit EventSet(int n) : e(size_t(n), nullptr) {
    for (cudaEvent_t& x : e) check_cuda(cudaEventCreateWithFlags(&x, cudaEventDisableTiming), "cudaEventCreate");
  }
  ~EventSet() {
    for (cudaEvent_t x : e)
      if (x) cudaEventDestroy(x);
  }
};

// ACA of every far block of the given operators (one, or the instances of a
// batch: their blocks share every launch), in workspace-bounded batches;
// compacted factors go to chunks of each operator's memory (FP64 or FP32;
// one per batch and team kind) and op->uptr / op->vptr record where.  With
// several operators their points and reference-order maps are concatenated
// for the launches, and each block carries its operator's kernel scale.
void run_aca(const std::vector<hodlr_op*>& ops, cudaStream_t st) {
  const size_t nops = ops.size();
  hodlr_op* op0 = ops[0];
  const bool joint = nops > 1;
  std::vector<int64_t> pbase(nops, 0), lbase(nops, 0), boff(nops + 1, 0);
  for (size_t j = 0; j < nops; j++) {
    hodlr_op* op = ops[j];
    const size_t nb = op->far.size();
    op->rank.assign(nb, 0);
    op->dense.assign(nb, 0);
    op->uptr.assign(nb, nullptr);
    op->vptr.assign(nb, nullptr);
    op->uptr64.assign(op->has_ref ? nb : 0, nullptr);
    op->vptr64.assign(op->has_ref ? nb : 0, nullptr);
    boff[j + 1] = boff[j] + int64_t(nb);
    if (j + 1 < nops) {
      pbase[j + 1] = pbase[j] + op->n;
      lbase[j + 1] = lbase[j] + int64_t(op->tree.levels) * op->n;
    }
  }
  const size_t nb = size_t(boff[nops]);
  if (nb == 0) return;
  const int ndim = op0->p.ndim;
  const Prec fp = far_prec(op0->p);
  const int cap0 = op0->p.rank_cap > 0 ? op0->p.rank_cap : 64;
  bool any_ref = false;  // some operator keeps an FP64 copy of its far field
  for (const hodlr_op* op : ops) any_ref = any_ref || op->has_ref;
  // global block g = boff[j] + b: operator j, its far block b
  std::vector<int32_t> job(nb), cap(nb), mm(nb), nn(nb);
  std::vector<int64_t> tb(nb), sb(nb), tmap(nb), smap(nb);
#pragma omp parallel for schedule(static) num_threads(par_threads(int64_t(nb)))
  for (int64_t gi = 0; gi < int64_t(nb); gi++) {
    const size_t g = size_t(gi);
    // the operator holding g: the last j with boff[j] <= g (empty operators skipped)
    const size_t j = size_t(std::upper_bound(boff.begin(), boff.end(), gi) - boff.begin()) - 1;
    const hodlr_op* op = ops[j];
    const Tree& t = op->tree;
    const FarBlock& f = op->far[g - size_t(boff[j])];
    const int64_t gt = t.gid(f.level, f.t), gs = t.gid(f.level, f.s);
    job[g] = int32_t(j);
    mm[g] = int32_t(t.count[size_t(gt)]);
    nn[g] = int32_t(t.count[size_t(gs)]);
    tb[g] = pbase[j] + t.begin[size_t(gt)];
    sb[g] = pbase[j] + t.begin[size_t(gs)];
    tmap[g] = lbase[j] + int64_t(f.level) * op->n + t.begin[size_t(gt)];
    smap[g] = lbase[j] + int64_t(f.level) * op->n + t.begin[size_t(gs)];
    cap[g] = std::min({mm[g], nn[g], cap0});
  }
  auto ws_need = [&](size_t g) { return uint64_t(cap[g]) * uint64_t(mm[g] + nn[g]); };
  // Scratch of one batch: the FP64 workspace is bounded (its size below); a
  // single block that needs more grows it.  Not counted against the
  // operators' memory: it is freed when the build returns.
  const size_t max_batch = size_t(1) << 23;
  struct Scratch {
    void* p = nullptr;
    size_t bytes = 0;
    ~Scratch() {
      if (p) cudaFree(p);
    }
    void ensure(size_t need, cudaStream_t st, const char* what) {
      if (need <= bytes) return;
      check_cuda(cudaStreamSynchronize(st), what);
      if (p) cudaFree(p);
      p = nullptr;
      bytes = 0;
      check_cuda(cudaMalloc(&p, need), what);
      bytes = need;
    }
  };
  Scratch s_ws, s_bits, s_lists, s_desc, s_out, s_idx, s_cd, s_pts, s_lmap, s_ctr;
  // FP64 workspace of one launch: a quarter of the free device memory,
  // between 4 and 64 GiB, so that most operators are compressed by one
  // launch per team kind; a growth arena of an eighth of it on top
  size_t free_b = 0, total_b = 0;
  check_cuda(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
  const uint64_t ws_doubles =
      op0->p.aca_workspace_mib > 0
          ? std::max<uint64_t>(uint64_t(1) << 17, uint64_t(op0->p.aca_workspace_mib) << 17)
          : std::min<uint64_t>(uint64_t(1) << 33, std::max<uint64_t>(uint64_t(1) << 29, uint64_t(free_b) / 4 / 8));
  const uint64_t arena_doubles = ws_doubles / 8;
  const uint64_t bits_room = ws_doubles / 8, list_room = ws_doubles / 8;
  const size_t nslot = std::min(nb, max_batch);
  s_desc.ensure(nslot * sizeof(AcaBlockDesc), st, "ACA descriptors");
  s_out.ensure(nslot * sizeof(AcaOut), st, "ACA results");
  s_idx.ensure(nslot * sizeof(int32_t), st, "ACA team lists");
  const size_t max_cd = size_t(1) << 20;  // compaction descriptors per launch
  s_cd.ensure(std::min(nslot, max_cd) * sizeof(CompactDesc), st, "compaction descriptors");
  // the growth arena's counter (bytes 0..7), then the work-queue counters of
  // the team kinds (from byte 16)
  s_ctr.ensure(kAcaCtrBytes, st, "ACA counters");
  int sms = 0;
  check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, op0->p.device), "cudaDeviceGetAttribute");
  AcaBlockDesc* d_desc = static_cast<AcaBlockDesc*>(s_desc.p);
  AcaOut* d_out = static_cast<AcaOut*>(s_out.p);
  int32_t* d_lists_idx = static_cast<int32_t*>(s_idx.p);
  CompactDesc* d_cd = static_cast<CompactDesc*>(s_cd.p);
  // points and reference-order maps of the launches
  PointsDev P{op0->d_pts, op0->n};
  const int32_t* d_lmap = op0->d_lmap;
  if (joint) {
    const int64_t ntot = pbase[nops - 1] + ops[nops - 1]->n;
    s_pts.ensure(size_t(ntot) * size_t(ndim) * sizeof(double), st, "batch points");
    double* jp = static_cast<double*>(s_pts.p);
    std::vector<int32_t> jl;
    jl.reserve(size_t(lbase[nops - 1] + int64_t(ops[nops - 1]->tree.levels) * ops[nops - 1]->n));
    for (size_t j = 0; j < nops; j++) {
      for (int k = 0; k < ndim; k++)
        CK(cudaMemcpyAsync(jp + int64_t(k) * ntot + pbase[j], ops[j]->d_pts + int64_t(k) * ops[j]->n,
                           sizeof(double) * size_t(ops[j]->n), cudaMemcpyDeviceToDevice, st));
      for (int32_t v : reference_order_map(ops[j]->tree)) jl.push_back(int32_t(v + pbase[j]));
    }
    s_lmap.ensure(jl.size() * sizeof(int32_t), st, "batch reference-order maps");
    CK(cudaMemcpyAsync(s_lmap.p, jl.data(), jl.size() * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));
    P = PointsDev{jp, ntot};
    d_lmap = static_cast<const int32_t*>(s_lmap.p);
  }
  // large blocks first keeps the CTA-team launch ahead of the warp teams: a
  // stable counting sort by max(m, n), descending (the sizes are node sizes);
  // threads count and place contiguous shares, with at most 64 MB of counters
  std::vector<size_t> todo(nb);
  {
    int32_t kmax = 0;
#pragma omp parallel for schedule(static) reduction(max : kmax) num_threads(par_threads(int64_t(nb)))
    for (int64_t g = 0; g < int64_t(nb); g++) kmax = std::max(kmax, std::max(mm[size_t(g)], nn[size_t(g)]));
    const size_t K = size_t(kmax) + 1;
    const int T = int(std::max<int64_t>(1, std::min<int64_t>(par_threads(int64_t(nb)), (int64_t(8) << 20) / int64_t(K))));
    std::vector<uint64_t> cnt(size_t(T) * K, 0);
    auto key = [&](size_t g) { return size_t(kmax - std::max(mm[g], nn[g])); };
#pragma omp parallel num_threads(T)
    {
      const int t = omp_get_thread_num();
      int64_t b, e;
      par_share(int64_t(nb), t, T, b, e);
      uint64_t* c = cnt.data() + size_t(t) * K;
      for (int64_t g = b; g < e; g++) c[key(size_t(g))]++;
#pragma omp barrier
#pragma omp single
      {
        uint64_t s = 0;  // (key, thread) order
        for (size_t k = 0; k < K; k++)
          for (int u = 0; u < T; u++) {
            const uint64_t v = cnt[size_t(u) * K + k];
            cnt[size_t(u) * K + k] = s;
            s += v;
          }
      }
      for (int64_t g = b; g < e; g++) todo[c[key(size_t(g))]++] = size_t(g);
    }
  }
  // budgets of the blocks in that order (prefix sums): FP64 workspace, pivot
  // bitmap words and pivot list entries
  auto bits_need = [&](size_t g) { return uint64_t((mm[g] + 31) / 32 + (nn[g] + 31) / 32); };
  auto list_need = [&](size_t g) { return uint64_t(2 * (std::min(mm[g], nn[g]) + 2)); };
  // (the sizes gathered into that order once, so that these passes and the
  // batches' read them in sequence)
  std::vector<int32_t> om(nb), on(nb), ocap(nb);
#pragma omp parallel for schedule(static) num_threads(par_threads(int64_t(nb)))
  for (int64_t i = 0; i < int64_t(nb); i++) {
    const size_t g = todo[size_t(i)];
    om[size_t(i)] = mm[g];
    on[size_t(i)] = nn[g];
    ocap[size_t(i)] = cap[g];
  }
  std::vector<uint64_t> pw(nb + 1), pbits(nb + 1), plist(nb + 1);
  par_exclusive_scan(int64_t(nb), pw.data(), [&](int64_t i) {
    return uint64_t(ocap[size_t(i)]) * uint64_t(om[size_t(i)] + on[size_t(i)]);
  });
  par_exclusive_scan(int64_t(nb), pbits.data(), [&](int64_t i) {
    return uint64_t((om[size_t(i)] + 31) / 32 + (on[size_t(i)] + 31) / 32);
  });
  par_exclusive_scan(int64_t(nb), plist.data(), [&](int64_t i) {
    return uint64_t(2 * (std::min(om[size_t(i)], on[size_t(i)]) + 2));
  });

  KernelDev K{op0->kd.kind, op0->kd.scale, op0->kd.diag};
  // every kernel of the launches below loaded now, while the GPU is idle
  check_cuda(aca_preload(ndim), "ACA kernels");
  check_cuda(compact_preload(ndim), "compaction kernels");
  struct Events {
    cudaEvent_t e[2] = {nullptr, nullptr};
    ~Events() {
      for (cudaEvent_t x : e)
        if (x) cudaEventDestroy(x);
    }
  } evs;
  check_cuda(cudaEventCreate(&evs.e[0]), "cudaEventCreate");
  check_cuda(cudaEventCreate(&evs.e[1]), "cudaEventCreate");
  cudaEvent_t ev_a0 = evs.e[0], ev_a1 = evs.e[1];
  // side streams of the ACA team kinds (one each), with their join events
  struct Side {
    cudaStream_t s[kAcaTeamKinds] = {};
    cudaEvent_t e[kAcaTeamKinds] = {};
    cudaStream_t cs = nullptr;              // compaction stream
    cudaEvent_t c0 = nullptr, c1 = nullptr;  // compaction launch timing
    ~Side() {
      if (cs) cudaStreamSynchronize(cs);
      for (int k = 0; k < kAcaTeamKinds; k++) {
        if (s[k]) cudaStreamSynchronize(s[k]);
        if (e[k]) cudaEventDestroy(e[k]);
        if (s[k]) cudaStreamDestroy(s[k]);
      }
      if (c0) cudaEventDestroy(c0);
      if (c1) cudaEventDestroy(c1);
      if (cs) cudaStreamDestroy(cs);
    }
  } side;
  for (int k = 0; k < kAcaTeamKinds; k++) {
    check_cuda(cudaStreamCreateWithFlags(&side.s[k], cudaStreamNonBlocking), "cudaStreamCreate");
    check_cuda(cudaEventCreateWithFlags(&side.e[k], cudaEventDisableTiming), "cudaEventCreate");
  }
  check_cuda(cudaStreamCreateWithFlags(&side.cs, cudaStreamNonBlocking), "cudaStreamCreate");
  check_cuda(cudaEventCreate(&side.c0), "cudaEventCreate");
  check_cuda(cudaEventCreate(&side.c1), "cudaEventCreate");
  double t_kernel = 0.0, t_compact = 0.0;
  // device times shared by every operator of the launch
  struct Report {
    const std::vector<hodlr_op*>& ops;
    double &tk, &tc;
    ~Report() {
      for (hodlr_op* op : ops) {
        op->st.t_aca_kernel_s = tk;
        op->st.t_compact_s = tc;
      }
    }
  } report{ops, t_kernel, t_compact};
  size_t pos = 0;
  std::vector<size_t> retry;
  std::vector<AcaBlockDesc> desc;
  std::vector<AcaOut> out;
  std::vector<CompactDesc> cds;
  while (pos < todo.size() || !retry.empty()) {
    // next batch
    std::vector<size_t> batch;
    size_t pos0 = 0;      // a run of the size order: its first position there
    bool in_order = false;  // (else a list of blocks to retry)
    uint64_t acc_w = 0, acc_b = 0, acc_l = 0;
    auto take = [&](size_t g) {
      const uint64_t w = ws_need(g), bw = bits_need(g), lw = list_need(g);
      if (!batch.empty() && (acc_w + w > ws_doubles || acc_b + bw > bits_room || acc_l + lw > list_room ||
                             batch.size() >= max_batch))
        return false;
      batch.push_back(g);
      acc_w += w;
      acc_b += bw;
      acc_l += lw;
      return true;
    };
    if (!retry.empty()) {
      std::vector<size_t> rest;
      for (size_t g : retry)
        if (!take(g)) rest.push_back(g);
      retry.swap(rest);
    } else {
      // the longest run from pos within every budget (at least one block):
      // the prefix sums are monotone, so a binary search finds its end
      auto fits = [&](size_t e) {
        return pw[e] - pw[pos] <= ws_doubles && pbits[e] - pbits[pos] <= bits_room &&
               plist[e] - plist[pos] <= list_room && e - pos <= max_batch;
      };
      size_t lo = pos + 1, hi = todo.size();  // fits(lo) is not required: one block always goes
      while (lo < hi) {
        const size_t mid = lo + (hi - lo + 1) / 2;
        if (fits(mid))
          lo = mid;
        else
          hi = mid - 1;
      }
      batch.assign(todo.begin() + int64_t(pos), todo.begin() + int64_t(lo));
      pos0 = pos;
      in_order = true;
      pos = lo;
    }
    // descriptors: per-block sizes and teams (parallel: the blocks are visited
    // in size order, so their arrays are read at random), offsets by a prefix
    // sum, then the descriptors (parallel again)
    const size_t nq = batch.size();
    const int tq = par_threads(int64_t(nq));
    desc.resize(nq);
    out.resize(nq);
    std::vector<uint64_t> qw(nq + 1), qb(nq + 1), ql(nq + 1);
    std::vector<int8_t> qteam(nq);
    if (in_order) {  // the size order's prefix sums, from the batch's start
#pragma omp parallel for schedule(static) num_threads(tq)
      for (int64_t q = 0; q <= int64_t(nq); q++) {
        const size_t i = pos0 + size_t(q);
        qw[size_t(q)] = pw[i] - pw[pos0];
        qb[size_t(q)] = pbits[i] - pbits[pos0];
        ql[size_t(q)] = plist[i] - plist[pos0];
        if (q < int64_t(nq)) qteam[size_t(q)] = int8_t(aca_team(om[i], on[i]));
      }
    } else {
      par_exclusive_scan(int64_t(nq), qw.data(), [&](int64_t q) { return ws_need(batch[size_t(q)]); });
      par_exclusive_scan(int64_t(nq), qb.data(), [&](int64_t q) { return bits_need(batch[size_t(q)]); });
      par_exclusive_scan(int64_t(nq), ql.data(), [&](int64_t q) { return list_need(batch[size_t(q)]); });
#pragma omp parallel for schedule(static) num_threads(tq)
      for (int64_t q = 0; q < int64_t(nq); q++) {
        const size_t g = batch[size_t(q)];
        qteam[size_t(q)] = int8_t(aca_team(mm[g], nn[g]));
      }
    }
    const uint64_t ow = qw[nq], ob = qb[nq], ol = ql[nq];
    s_ws.ensure((ow + arena_doubles) * 8, st, "ACA workspace");
    s_bits.ensure(std::max<uint64_t>(ob, 1) * 4, st, "ACA bitmaps");
    s_lists.ensure(std::max<uint64_t>(ol, 1) * 4, st, "ACA index lists");
    double* ws = static_cast<double*>(s_ws.p);
    AcaArgs a;
    a.lmap = d_lmap;
    a.P = P;
    a.K = K;
    a.tol = op0->p.eps_aca;
    a.blocks = d_desc;
    a.ws = ws;
    a.bits = static_cast<uint32_t*>(s_bits.p);
    a.lists = static_cast<int32_t*>(s_lists.p);
    a.out = d_out;
    // one persistent launch per team kind: teams take their blocks from the
    // kind's work queue; blocks whose rank outgrows their columns continue in
    // the arena
    a.queue = reinterpret_cast<unsigned int*>(static_cast<char*>(s_ctr.p) + 16);
    a.arena_used = static_cast<unsigned long long*>(s_ctr.p);
    a.arena_off = int64_t(ow);
    a.arena_size = arena_doubles;
    a.max_ctas = sms * 16;
    CK(cudaMemsetAsync(s_ctr.p, 0, kAcaCtrBytes, st));
    // Runs of the batch: in a batch in size order each team kind holds one
    // consecutive run (largest kind first).  The runs are launched in that
    // order, each as soon as its descriptors are on the device (the large
    // blocks' long compression starts first and the small kinds fill its
    // tail), and each run is compacted (on the compaction stream) once its
    // launch is done, the last-launched first.  Other batches (retries, small
    // batches) are one run of every kind.
    struct Run {
      size_t b, e;
      int kind;  // -1: every kind
    };
    std::vector<Run> runs;
    bool by_kind = nq >= kAcaRunMin;
    for (size_t q = 1; by_kind && q < nq; q++) by_kind = qteam[q] <= qteam[q - 1];
    if (by_kind) {
      size_t cnt[kAcaTeamKinds] = {};
      for (int8_t t : qteam) cnt[size_t(t)]++;
      size_t b0 = 0;
      for (int k = kAcaTeamKinds - 1; k >= 0; k--) {
        if (cnt[k] > 0) runs.push_back({b0, b0 + cnt[k], k});
        b0 += cnt[k];
      }
    } else {
      runs.push_back({0, nq, -1});
    }
    EventSet rev(2 * kAcaTeamKinds);
    auto ev_copy = [&](size_t r) { return rev.e[r]; };
    auto ev_done = [&](int k) { return rev.e[size_t(kAcaTeamKinds + k)]; };
    std::vector<int32_t> lst(nq);
    for (size_t r = 0; r < runs.size(); r++) {
      const size_t q0 = runs[r].b, nw = runs[r].e - q0;
      const int tw = par_threads(int64_t(nw));
#pragma omp parallel for schedule(static) num_threads(tw)
      for (int64_t q = int64_t(q0); q < int64_t(q0 + nw); q++) {
        const size_t g = batch[size_t(q)];
        const hodlr_op* op = ops[size_t(job[g])];
        const FarBlock& f = op->far[size_t(int64_t(g) - boff[size_t(job[g])])];
        AcaBlockDesc& d = desc[size_t(q)];
        d.t_map = tmap[g];
        d.s_map = smap[g];
        d.m = mm[g];
        d.n = nn[g];
        d.cap = cap[g];
        // the pivot lists hold every rank the block can reach, also after it grows into the arena
        d.lcap = std::min(mm[g], nn[g]);
        d.ws = int64_t(qw[size_t(q)]);
        d.bits = int64_t(qb[size_t(q)]);
        d.lists = int64_t(ql[size_t(q)]);
        d.seed = block_seed(f.level, f.t, f.s);
        d.kscale = joint ? op->kd.scale : 0.0;
      }
      // the run's index list: the team kinds one after another (largest
      // teams first), each kind's blocks in batch order (a stable partition)
      AcaLists al;
      for (int k = 0; k < kAcaTeamKinds; k++) {
        al.list[k] = d_lists_idx;
        al.n[k] = 0;
      }
      if (runs[r].kind >= 0) {
#pragma omp parallel for schedule(static) num_threads(tw)
        for (int64_t q = int64_t(q0); q < int64_t(q0 + nw); q++) lst[size_t(q)] = int32_t(q);
        al.list[runs[r].kind] = d_lists_idx + q0;
        al.n[runs[r].kind] = int(nw);
      } else {
        std::vector<uint64_t> lofs(nw), lcount;
        par_group_offsets(
            int64_t(nw), kAcaTeamKinds, lofs.data(), lcount,
            [&](int64_t i) { return kAcaTeamKinds - 1 - int(qteam[q0 + size_t(i)]); },
            [](int64_t) { return uint64_t(1); });
        size_t lpos[kAcaTeamKinds];
        size_t base = q0;
        for (int k = kAcaTeamKinds - 1; k >= 0; k--) {
          lpos[k] = base;
          al.list[k] = d_lists_idx + base;
          al.n[k] = int(lcount[size_t(kAcaTeamKinds - 1 - k)]);
          base += size_t(al.n[k]);
        }
#pragma omp parallel for schedule(static) num_threads(tw)
        for (int64_t i = 0; i < int64_t(nw); i++)
          lst[lpos[qteam[q0 + size_t(i)]] + lofs[size_t(i)]] = int32_t(q0 + size_t(i));
      }
      CK(cudaMemcpyAsync(d_desc + q0, desc.data() + q0, nw * sizeof(AcaBlockDesc), cudaMemcpyHostToDevice, st));
      CK(cudaMemcpyAsync(d_lists_idx + q0, lst.data() + q0, nw * sizeof(int32_t), cudaMemcpyHostToDevice, st));
      if (r == 0) CK(cudaEventRecord(ev_a0, st));  // the launches' span starts here
      CK(cudaEventRecord(ev_copy(r), st));
      for (int k = 0; k < kAcaTeamKinds; k++) {
        if (runs[r].kind >= 0 && k != runs[r].kind) continue;
        CK(cudaStreamWaitEvent(side.s[k], ev_copy(r), 0));
        CK(launch_aca_kind(ndim, a, al, k, side.s[k]));
        CK(cudaEventRecord(ev_done(k), side.s[k]));
      }
    }
    // the main stream joins every kind's launch
    for (int k = 0; k < kAcaTeamKinds; k++) {
      CK(cudaEventRecord(side.e[k], side.s[k]));
      CK(cudaStreamWaitEvent(st, side.e[k], 0));
    }
    CK(cudaEventRecord(ev_a1, st));
    // compaction of each run once its launch is done (the last-launched
    // first), on the compaction stream
    cudaStream_t cs = side.cs;
    const bool ref64 = fp != Prec::kD && any_ref, dual = ref64 && fp == Prec::kF;
    for (size_t rr = runs.size(); rr-- > 0;) {
      const size_t q0 = runs[rr].b, nw = runs[rr].e - q0;
      const int tw = par_threads(int64_t(nw));
      for (int k = 0; k < kAcaTeamKinds; k++)
        if (runs[rr].kind < 0 || k == runs[rr].kind) CK(cudaStreamWaitEvent(cs, ev_done(k), 0));
      // into pageable memory: returns once the run's results are here
      CK(cudaMemcpyAsync(out.data() + q0, d_out + q0, nw * sizeof(AcaOut), cudaMemcpyDeviceToHost, cs));
      CK(cudaStreamSynchronize(cs));
      // Per block of the run, in one pass: its results into its operator,
      // its operator, its stored bytes (FP32/BF16 and FP64 copies) and
      // whether it is compacted (dense or rank > 0).  Blocks that outgrew
      // their columns go back with 4x the columns.
      std::vector<int32_t> bjob(nw);
      std::vector<uint64_t> bsz(nw), bsz64(ref64 ? nw : 0);
      std::vector<uint8_t> bkeep(nw), bkeep64(ref64 ? nw : 0);
      int64_t novf = 0;
#pragma omp parallel for schedule(static) reduction(+ : novf) num_threads(tw)
      for (int64_t ii = 0; ii < int64_t(nw); ii++) {
        const size_t i = size_t(ii), q = q0 + i, g = batch[q];
        bjob[i] = job[g];
        bsz[i] = 0;
        bkeep[i] = 0;
        if (ref64) {
          bsz64[i] = 0;
          bkeep64[i] = 0;
        }
        if (out[q].flags & kAcaOverflow) {
          cap[g] = std::min(std::min(mm[g], nn[g]), cap[g] * 4);
          novf++;
          continue;
        }
        hodlr_op* op = ops[size_t(job[g])];
        const size_t b = size_t(int64_t(g) - boff[size_t(job[g])]);
        const int32_t r = out[q].rank;
        const int8_t dn = (out[q].flags & kAcaDense) ? 1 : 0;
        op->rank[b] = r;
        op->dense[b] = dn;
        bsz[i] = far_u_bytes(mm[g], nn[g], r, dn, fp) + far_v_bytes(nn[g], r, dn, fp);
        bkeep[i] = (dn || r > 0) ? 1 : 0;
        if (ref64 && op->has_ref) {
          bsz64[i] = far_u_bytes(mm[g], nn[g], r, dn, Prec::kD) + far_v_bytes(nn[g], r, dn, Prec::kD);
          bkeep64[i] = bkeep[i];
        }
      }
      if (novf > 0)
        for (size_t q = q0; q < q0 + nw; q++)
          if (out[q].flags & kAcaOverflow) retry.push_back(batch[q]);
      auto job_of = [&](int64_t i) { return int(bjob[size_t(i)]); };
      // byte offsets within each operator's chunk of this run (batch order)
      // and the position among the blocks compacted
      std::vector<uint64_t> bytes, off(nw), kidx(nw + 1);
      par_group_offsets(int64_t(nw), int(nops), off.data(), bytes, job_of, [&](int64_t i) { return bsz[size_t(i)]; });
      par_exclusive_scan(int64_t(nw), kidx.data(), [&](int64_t i) { return uint64_t(bkeep[size_t(i)]); });
      cds.resize(size_t(kidx[nw]));
      // the FP64 copy of the same blocks, for operators that keep one: with
      // FP32 factors both copies come from one compaction pass (the entries of
      // a dense tile are evaluated once)
      std::vector<uint64_t> bytes64, off64, kidx64;
      if (ref64) {
        off64.resize(nw);
        kidx64.resize(nw + 1);
        par_group_offsets(int64_t(nw), int(nops), off64.data(), bytes64, job_of,
                          [&](int64_t i) { return bsz64[size_t(i)]; });
        par_exclusive_scan(int64_t(nw), kidx64.data(), [&](int64_t i) { return uint64_t(bkeep64[size_t(i)]); });
      }
      std::vector<char*> chunk(nops, nullptr), chunk64(nops, nullptr);
      for (size_t j = 0; j < nops; j++) {
        if (bytes[j] > 0) {
          chunk[j] = static_cast<char*>(ops[j]->mem.alloc(bytes[j], "far-field factors"));
          ops[j]->far_chunks.push_back(chunk[j]);
          CK(cudaMemsetAsync(chunk[j], 0, bytes[j], cs));  // tile padding rows must read as zero
        }
        if (ref64 && bytes64[j] > 0) {
          chunk64[j] = static_cast<char*>(ops[j]->mem.alloc(bytes64[j], "far-field factors (FP64 reference)"));
          CK(cudaMemsetAsync(chunk64[j], 0, bytes64[j], cs));
        }
      }
#pragma omp parallel for schedule(static) num_threads(tw)
      for (int64_t ii = 0; ii < int64_t(nw); ii++) {
        const size_t i = size_t(ii), q = q0 + i;
        const size_t g = batch[q];
        if (out[q].flags & kAcaOverflow) continue;
        hodlr_op* op = ops[size_t(job[g])];
        const size_t b = size_t(int64_t(g) - boff[size_t(job[g])]);
        char* ch = chunk[size_t(job[g])];
        CompactDesc c;
        c.t_begin = tb[g];
        c.s_begin = sb[g];
        c.t_map = desc[q].t_map;
        c.s_map = desc[q].s_map;
        c.ws = out[q].cap ? out[q].ws : desc[q].ws;
        const int32_t rk = std::max(op->rank[b], 0);
        c.u_dst = ch + off[i];
        c.v_dst = ch + off[i] + far_u_bytes(mm[g], nn[g], rk, op->dense[b], fp);
        c.s_dst = nullptr;
        if (fp == Prec::kB)
          c.s_dst = reinterpret_cast<float*>(op->dense[b]
                                                 ? ch + off[i] + far_u_data_bytes(mm[g], nn[g], rk, true, fp)
                                                 : static_cast<char*>(c.v_dst) + far_v_data_bytes(nn[g], rk, false, fp));
        c.m = mm[g];
        c.n = nn[g];
        c.rank = op->rank[b];
        c.dense = op->dense[b];
        c.cap = out[q].cap ? out[q].cap : desc[q].cap;
        c.pad = 0;
        c.kscale = desc[q].kscale;
        c.u64_dst = c.v64_dst = nullptr;
        if (dual && kidx64[i + 1] > kidx64[i]) {
          char* ch64 = chunk64[size_t(job[g])];
          c.u64_dst = ch64 + off64[i];
          c.v64_dst = ch64 + off64[i] + far_u_bytes(mm[g], nn[g], rk, op->dense[b], Prec::kD);
          op->uptr64[b] = c.u64_dst;
          op->vptr64[b] = c.v64_dst;
        }
        op->uptr[b] = c.u_dst;
        op->vptr[b] = c.v_dst;
        if (kidx[i + 1] > kidx[i]) cds[size_t(kidx[i])] = c;
      }
      auto compact = [&](const std::vector<CompactDesc>& v, Prec to) {
        for (size_t b0 = 0; b0 < v.size(); b0 += max_cd) {
          const size_t k = std::min(max_cd, v.size() - b0);
          CK(cudaMemcpyAsync(d_cd, v.data() + b0, k * sizeof(CompactDesc), cudaMemcpyHostToDevice, cs));
          CK(cudaEventRecord(side.c0, cs));
          CK(launch_compact(ndim, P, K, ws, d_lmap, d_cd, int(k), to, cs));
          CK(cudaEventRecord(side.c1, cs));
          CK(cudaStreamSynchronize(cs));  // d_cd is refilled next
          float ms = 0.f;
          CK(cudaEventElapsedTime(&ms, side.c0, side.c1));
          t_compact += 1e-3 * double(ms);
        }
      };
      compact(cds, fp);
      // BF16 factors: the FP64 copy in a pass of its own
      if (ref64 && !dual) {
        bool any = false;
        for (size_t j = 0; j < nops; j++) any = any || chunk64[j] != nullptr;
        if (any) {
          std::vector<CompactDesc> cd64(static_cast<size_t>(kidx64[nw]));
#pragma omp parallel for schedule(static) num_threads(tw)
          for (int64_t ii = 0; ii < int64_t(nw); ii++) {
            const size_t i = size_t(ii), q = q0 + i;
            if (kidx64[i + 1] == kidx64[i]) continue;  // not kept (no FP64 copy, overflow, or rank 0)
            const size_t g = batch[q];
            hodlr_op* op = ops[size_t(job[g])];
            const size_t b = size_t(int64_t(g) - boff[size_t(job[g])]);
            char* ch = chunk64[size_t(job[g])];
            CompactDesc c;
            c.t_begin = tb[g];
            c.s_begin = sb[g];
            c.t_map = desc[q].t_map;
            c.s_map = desc[q].s_map;
            c.ws = out[q].cap ? out[q].ws : desc[q].ws;
            c.u_dst = ch + off64[i];
            c.v_dst = ch + off64[i] + far_u_bytes(mm[g], nn[g], op->rank[b], op->dense[b], Prec::kD);
            c.s_dst = nullptr;
            c.m = mm[g];
            c.n = nn[g];
            c.rank = op->rank[b];
            c.dense = op->dense[b];
            c.cap = out[q].cap ? out[q].cap : desc[q].cap;
            c.pad = 0;
            c.kscale = desc[q].kscale;
            c.u64_dst = c.v64_dst = nullptr;
            op->uptr64[b] = c.u_dst;
            op->vptr64[b] = c.v_dst;
            cd64[size_t(kidx64[i])] = c;
          }
          compact(cd64, Prec::kD);
        }
      }
    }
    CK(cudaStreamSynchronize(cs));
    CK(cudaStreamSynchronize(st));
    {
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, ev_a0, ev_a1));
      t_kernel += 1e-3 * double(ms);
    }
  }
}

void compute_stats(hodlr_op* op) {
  hodlr_stats& s = op->st;
  const Tree& t = op->tree;
  s.n = op->n;
  s.depth = t.levels - 1;
  s.n_leaves = t.level_size.back();
  s.n_far_blocks = int64_t(op->far.size());
  s.n_near_blocks = int64_t(op->near.src.size());
  s.n_dense_far_blocks = 0;
  s.max_rank = 0;
  s.far_entries = s.dense_far_entries = s.near_entries = 0;
  s.aca_entries = 0;
  double flop = 0.0;
  const int L = t.levels - 1;
  for (int64_t k = 0; k < t.level_size[size_t(L)]; k++) {
    const int64_t g = t.gid(L, k);
    if (t.count[size_t(g)] == 0) continue;
    double f = 0.0;
    for (int64_t q = op->near.leaf_ptr[size_t(k)]; q < op->near.leaf_ptr[size_t(k + 1)]; q++)
      f += double(t.count[size_t(t.gid(L, op->near.src[size_t(q)]))]);
    flop += f * double(t.count[size_t(g)]);
    s.near_entries += f * double(t.count[size_t(g)]);
  }
  for (size_t b = 0; b < op->far.size(); b++) {
    const double m = double(t.count[size_t(t.gid(op->far[b].level, op->far[b].t))]);
    const double n = double(t.count[size_t(t.gid(op->far[b].level, op->far[b].s))]);
    flop += double(op->rank[b]) * (m + n);
    // the ACA generates one residual row and column per step, one more for the stopping step
    s.aca_entries += double(op->rank[b] + 1) * (m + n);
    s.max_rank = std::max<int64_t>(s.max_rank, op->rank[b]);
    if (op->dense[b]) {
      s.n_dense_far_blocks++;
      s.dense_far_entries += m * n;
    } else {
      s.far_entries += double(op->rank[b]) * (m + n);
    }
  }
  s.n_flop = flop;
  s.memory_gb = 8e-9 * flop;
  s.compression_ratio = flop / (double(op->n) * double(op->n));
  const double fesz = double(prec_size(far_prec(op->p)));
  s.near_bytes = uint64_t(s.near_entries * 8.0 * (op->p.precision == HODLR_PREC_MIXED ? 1.5 : 1.0));
  s.far_bytes = uint64_t((s.far_entries + s.dense_far_entries) * fesz);
  s.device_bytes = op->mem.used;
  // Algorithmic bytes per launch of each operator kernel: stored matrix
  // entries once, plus each vector once (re-reads of x are not counted).
  // BF16 factors add their FP32 scales: one per z column, one per dense-tile column.
  double lr_rows = 0.0, lr_cols = 0.0, zsum = 0.0, dense_cols = 0.0;
  for (size_t b = 0; b < op->far.size(); b++) {
    if (op->dense[b]) dense_cols += double(t.count[size_t(t.gid(op->far[b].level, op->far[b].s))]);
    if (op->dense[b] || op->rank[b] == 0) continue;
    const double m = double(t.count[size_t(t.gid(op->far[b].level, op->far[b].t))]);
    const double n = double(t.count[size_t(t.gid(op->far[b].level, op->far[b].s))]);
    lr_rows += double(op->rank[b]) * m;
    lr_cols += double(op->rank[b]) * n;
    zsum += double(op->rank[b]);
  }
  const double N = double(op->n), slots = double(op->nslots);
  const double ss = far_prec(op->p) == Prec::kB ? 4.0 : 0.0;
  for (int v = 0; v < 2; v++) {  // v = 0: FP64 vectors, 1: FP32 vectors
    const double sx = v == 0 ? 8.0 : 4.0, snear = v == 0 ? 8.0 : 4.0;
    const int kb = v == 0 ? HODLR_TRACE_ZGEMV_FP64 : HODLR_TRACE_ZGEMV_FP32;
    op->tr.bytes[kb + 0] = lr_cols * fesz + zsum * (sx + ss) + N * sx;
    op->tr.bytes[kb + 1] = s.near_entries * snear + 2.0 * N * sx;
    op->tr.bytes[kb + 2] = (lr_rows + s.dense_far_entries) * fesz + dense_cols * ss + zsum * sx + N * sx +
                           N * (slots - 1.0) * sx;
    op->tr.bytes[kb + 3] = N * slots * sx + N * sx;
  }
  if (op->has_ref) {  // the FP64 operator of the refinement residuals
    const int kb = HODLR_TRACE_ZGEMV_REF;
    op->tr.bytes[kb + 0] = lr_cols * 8.0 + zsum * 8.0 + N * 8.0;
    op->tr.bytes[kb + 1] = s.near_entries * 8.0 + 2.0 * N * 8.0;
    op->tr.bytes[kb + 2] = (lr_rows + s.dense_far_entries) * 8.0 + zsum * 8.0 + N * 8.0 + N * (slots - 1.0) * 8.0;
    op->tr.bytes[kb + 3] = N * slots * 8.0 + N * 8.0;
  }
}

// ---------------------------------------------------------------- apply

template <typename T>
struct PrecOf;
template <>
struct PrecOf<double> {
  static constexpr Prec v = Prec::kD;
};
template <>
struct PrecOf<float> {
  static constexpr Prec v = Prec::kF;
};

// y = A x, tree order, nrhs = 1; x may alias nothing in the op's buffers.
template <typename T>
cudaError_t apply_tree(hodlr_op* op, const Plan& plan, const T* x, T* y, T* in, T* yslots, cudaStream_t st,
                       const int64_t* out_perm = nullptr) {
  const int64_t n = op->n, ldin = n + op->zlen;
  cudaError_t e = cudaMemcpyAsync(in, x, sizeof(T) * size_t(n), cudaMemcpyDeviceToDevice, st);
  if (e != cudaSuccess) return e;
  if (op->nslots > 1) {
    e = cudaMemsetAsync(yslots + n, 0, sizeof(T) * size_t(n) * size_t(op->nslots - 1), st);
    if (e != cudaSuccess) return e;
  }
  const Prec px = PrecOf<T>::v;
  const int kb = &plan == &op->plan_ref ? HODLR_TRACE_ZGEMV_REF
                 : px == Prec::kD       ? HODLR_TRACE_ZGEMV_FP64
                                        : HODLR_TRACE_ZGEMV_FP32;
  Tracer& tr = op->tr;
  if (plan.nzb > 0) tr.start(kb + 0, st);
  // FP32 or BF16 factors with FP64 vectors: compensated (or, while the solver
  // allows it, relaxed) FP32 accumulation on split inputs
  const bool df = plan.a_far != Prec::kD && px == Prec::kD;
  const Accum acc = !df                       ? Accum::kByType
                    : op->relaxed || op->p.relax == HODLR_RELAX_ALWAYS ? Accum::kRelaxed
                                                                       : Accum::kCompensated;
  void* fin = in;
  if (df) {
    fin = op->d_in2;
    if ((e = launch_split(reinterpret_cast<const double*>(in), fin, n, st)) != cudaSuccess) return e;
  }
  if ((e = launch_zgemv(plan.a_far, px, plan.zb, plan.zitems, plan.nzitems, plan.zfix, plan.nzfix, plan.zpart, fin, ldin,
                        1, st, acc)) != cudaSuccess)
    return e;
  if (plan.nzb > 0) tr.stop(st);
  tr.start(kb + 1, st);
  if ((e = launch_panels(plan.a_near, px, plan.panels_near, plan.segs_near, plan.small_near, plan.nsmall_near,
                         plan.big_near, plan.nbig_near, plan.pfix_near, plan.npfix_near, plan.ypart, in, ldin, yslots, n,
                         op->nslots, 1, st, Accum::kByType, plan.contig_near)) != cudaSuccess)
    return e;
  tr.stop(st);
  const bool far = plan.nsmall_far + plan.nbig_far > 0;
  if (far) tr.start(kb + 2, st);
  if ((e = launch_panels(plan.a_far, px, plan.panels_far, plan.segs_far, plan.small_far, plan.nsmall_far, plan.big_far,
                         plan.nbig_far, plan.pfix_far, plan.npfix_far, plan.ypart, fin, ldin, yslots, n, op->nslots, 1,
                         st, acc, plan.contig_far)) != cudaSuccess)
    return e;
  if (far) tr.stop(st);
  tr.start(kb + 3, st);
  e = launch_combine(px, yslots, n, op->nslots, n, 1, out_perm, y, px, n, st);
  tr.stop(st);
  if (tr.used > 8192) tr.harvest();
  return e;
}

__global__ void axpy_d_kernel(double* x, const double* d, int64_t n) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    x[i] = x[i] + d[i];
}

__global__ void axpy_f2d_kernel(double* x, const float* d, int64_t n) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    x[i] = x[i] + double(d[i]);
}

// Default threshold of relaxed products: residual estimate below tol times this.
constexpr double kRelaxFactor = 1e5;

Ortho ortho_of(const hodlr_params& p) {
  if (p.ortho == HODLR_ORTHO_MGS) return Ortho::kMGS;
  if (p.ortho == HODLR_ORTHO_CGS2) return Ortho::kCGS2;
  return p.precision == HODLR_PREC_FP64 ? Ortho::kMGS : Ortho::kCGS2;
}

// Solve in tree order on device buffers b, x (one right-hand side).
// Reduced-precision operators keep the FP64 far field unless the FP64 check is off.
bool wants_ref(const hodlr_params& p) {
  return p.precision != HODLR_PREC_FP64 && p.fp64_check != HODLR_FP64_CHECK_OFF;
}

// |b - A x| / |b| with the FP64-vector operator of `plan` (plan64: the stored
// operator, compensated products unless relaxed ones are forced; plan_ref:
// the FP64 operator); the residual vector is left in op->d_r64.  Tree order.
double true_residual(hodlr_op* op, const Plan& plan, const double* b, const double* x, cudaStream_t st) {
  CK(apply_tree<double>(op, plan, x, op->d_io2, op->d_in64, op->d_y64, st));
  CK(vec_sub_norm2<double>(b, op->d_io2, op->d_r64, op->n, op->d_part, op->d_scal + 1, st));
  CK(vec_norm2<double>(b, op->n, op->d_part, op->d_scal + 2, st));
  CK(cudaMemcpyAsync(op->h_scal, op->d_scal, sizeof(double) * 3, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return op->h_scal[1] / (op->h_scal[2] == 0.0 ? 1.0 : op->h_scal[2]);
}

// Iterative refinement with the FP64 operator around solves with the stored
// one: while |b - A64 x| / |b| > tol, solve A_stored d = r (r = b - A64 x,
// from d = 0, to a relative residual that leaves a 0.3 margin below tol)
// and x += d.  Each sweep multiplies the FP64 residual by about
// max(its inner tolerance, |A_stored^-1 (A64 - A_stored)|): far below 1 for
// FP32 factors (one sweep), about 1e-3 x the conditioning for BF16.
// `inner` runs the stored-operator solve of A d = r into d; returns the
// FP64 residual, counts sweeps and inner iterations.
double refine(hodlr_op* op, const double* b, double* x, double tol, int max_sweeps, int64_t max_iter, cudaStream_t st,
              const std::function<int64_t(const double* r, double* d, double sweep_tol, int64_t its_left)>& inner,
              int* sweeps, int64_t* its) {
  double res = true_residual(op, op->plan_ref, b, x, st);
  while (res > tol && *sweeps < max_sweeps && *its < max_iter) {
    // the correction's own stopping point, relative to |r|
    const double sweep_tol = std::min(0.5, 0.3 * tol / res);
    CK(cudaMemcpyAsync(op->d_rref, op->d_r64, sizeof(double) * size_t(op->n), cudaMemcpyDeviceToDevice, st));
    *its += inner(op->d_rref, op->d_dref, sweep_tol, max_iter - *its);
    axpy_d_kernel<<<kVecCtas, 256, 0, st>>>(x, op->d_dref, op->n);
    CK(cudaGetLastError());
    (*sweeps)++;
    res = true_residual(op, op->plan_ref, b, x, st);
  }
  return res;
}

// The stored-operator residual a solve without the FP64 check stops at.
double stored_stop(const hodlr_params& p, double tol) { return tol * (p.stored_margin > 0 ? p.stored_margin : 1.0); }

void solve_tree(hodlr_op* op, const double* b, double* x, cudaStream_t st, hodlr_solve_info* info) {
  const hodlr_params& p = op->p;
  const double tol = p.tol > 0 ? p.tol : p.eps_aca;
  const int64_t max_iter = p.max_iter > 0 ? p.max_iter : op->n;
  const int restart = p.restart > 0 ? p.restart : 100;
  const int max_outer = p.max_outer > 0 ? p.max_outer : 10;
  const double t0 = now_s();
  const bool ref = op->has_ref;
  double stop = ref ? tol : stored_stop(p, tol);
  if (p.precision != HODLR_PREC_MIXED) {
    // HODLRdD_matrix::solve: x0 = b, iterSolver(100, N, eps_ACA) (HDD_matrix.hpp:51-62);
    // with FP32 or BF16 factors the same FP64 GMRES runs on the stored operator
    CK(cudaMemcpyAsync(x, b, sizeof(double) * size_t(op->n), cudaMemcpyDeviceToDevice, st));
    TreeMatvec<double> A = [op, st](const double* xi, double* yo) {
      return apply_tree<double>(op, op->plan64, xi, yo, op->d_in64, op->d_y64, st);
    };
    // FP32 or BF16 factors: relaxed accumulation once the residual estimate is below
    // relax_below (tol * 1e5) -- an inexact Krylov method may take products with relative
    // error up to about tol / |r_k| (Simoncini and Szyld, SIAM J. Sci.
    // Comput. 25 (2003); Bouras and Fraysse, SIAM J. Matrix Anal. Appl. 26
    // (2005)), and relaxed products are accurate to about 1e-6 -- then the
    // true residual decides (with the FP64 operator, or with compensated
    // products on the stored one), and GMRES continues while it is above tol.
    const bool reduced = p.precision != HODLR_PREC_FP64;
    const bool relax = reduced && p.relax != HODLR_RELAX_OFF;
    // With the FP64 check the FP64 operator decides every sweep's end, so the
    // inner solves may take relaxed products from the first iteration on (fewer
    // bytes of work per product; measured 6% faster per solve at N = 262144,
    // solutions within 2.4e-9 of the FP64 operator)
    const double relax_at =
        p.relax_below > 0 ? p.relax_below : (ref ? 1.0 : std::min(1.0, tol * kRelaxFactor));
    std::function<void(double)> progress;
    if (relax) progress = [op, relax_at](double res) { op->relaxed = res < relax_at; };
    // The first solve's target on the stored operator: tol (FP32 factors, whose
    // rounding is about tol at eps_aca 1e-8), or inner_tol for BF16 factors
    // (about 1e-3 from the FP64 operator: refinement sweeps take it from there).
    const double first_tol = !ref || p.precision != HODLR_PREC_BF16_FACTORS
                                 ? stop
                                 : std::max(stop, p.inner_tol > 0 ? p.inner_tol : 1e-4);
    op->relaxed = false;
    GmresResult r;
    const cudaError_t ge =
        gmres_solve<double>(op->g64, A, b, x, false, restart, max_iter, first_tol, st, &r, ortho_of(p), progress);
    op->relaxed = false;
    CK(ge);
    int64_t its = r.iterations;
    int sweeps = 1;
    double res = r.resid, res_stored = r.resid;
    bool conv = r.converged;
    if (reduced && !ref && conv) {
      // no FP64 operator: the stored operator's true residual with compensated products
      for (;;) {
        res = res_stored = true_residual(op, op->plan64, b, x, st);
        if (res <= stop || sweeps >= 4 || its >= max_iter) break;
        GmresResult r2;
        CK(gmres_solve<double>(op->g64, A, b, x, false, restart, max_iter - its, stop, st, &r2, ortho_of(p)));
        its += r2.iterations;
        sweeps++;
      }
      conv = res <= stop;
    } else if (ref) {
      res_stored = true_residual(op, op->plan64, b, x, st);
      auto inner = [&](const double* rr, double* d, double sweep_tol, int64_t left) -> int64_t {
        GmresResult r2;
        op->relaxed = false;
        const cudaError_t e =
            gmres_solve<double>(op->g64, A, rr, d, true, restart, left, sweep_tol, st, &r2, ortho_of(p), progress);
        op->relaxed = false;
        CK(e);
        return r2.iterations;
      };
      res = refine(op, b, x, stop, max_outer + 1, max_iter, st, inner, &sweeps, &its);
      conv = res <= stop;
    }
    CK(cudaStreamSynchronize(st));
    info->iterations = its;
    info->outer_iterations = sweeps;
    info->rel_residual = res;
    info->rel_residual_stored = reduced ? res_stored : res;
    info->converged = conv ? 1 : 0;
  } else {
    // FP64 iterative refinement around FP32 GMRES on the FP32 operator; the
    // refinement residual with the FP64 operator (FP64 check) or with the
    // FP64-vector stored operator (FP64 near field, FP32 far factors)
    const double inner_tol = p.inner_tol > 0 ? p.inner_tol : 1e-4;
    TreeMatvec<float> A32 = [op, st](const float* xi, float* yo) {
      return apply_tree<float>(op, op->plan32, xi, yo, op->d_in32, op->d_y32, st);
    };
    const Plan& R = ref ? op->plan_ref : op->plan64;
    const int64_t n = op->n;
    CK(cudaMemsetAsync(x, 0, sizeof(double) * size_t(n), st));
    CK(cudaMemcpyAsync(op->d_r64, b, sizeof(double) * size_t(n), cudaMemcpyDeviceToDevice, st));
    CK(vec_norm2<double>(b, n, op->d_part, op->d_scal + 2, st));
    CK(vec_norm2<double>(op->d_r64, n, op->d_part, op->d_scal + 1, st));
    CK(cudaMemcpyAsync(op->h_scal, op->d_scal, sizeof(double) * 3, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    double normb = op->h_scal[2] == 0.0 ? 1.0 : op->h_scal[2];
    double rel = op->h_scal[1] / normb;
    int64_t inner_total = 0;
    int outer = 0;
    while (rel > stop && outer < max_outer && inner_total < max_iter) {
      CK(launch_gather(op->d_r64, Prec::kD, n, nullptr, n, 1, op->d_r32, Prec::kF, n, st));
      GmresResult r;
      // The first sweep stops at inner_tol; a later sweep aims below what the
      // remaining reduction needs (stop |b| / |r|, with a 0.3 margin) so that
      // it ends the solve instead of leaving a residual just above the target.
      double sweep_tol = inner_tol;
      if (outer > 0) sweep_tol = std::min(inner_tol, 0.3 * stop / rel);
      CK(gmres_solve<float>(op->g32, A32, op->d_r32, op->d_d32, true, restart, max_iter - inner_total,
                            std::max(sweep_tol, stop), st, &r, ortho_of(p)));
      inner_total += r.iterations;
      axpy_f2d_kernel<<<kVecCtas, 256, 0, st>>>(x, op->d_d32, n);
      CK(cudaGetLastError());
      rel = true_residual(op, R, b, x, st);
      outer++;
    }
    info->iterations = inner_total;
    info->outer_iterations = outer;
    info->rel_residual = rel;
    info->rel_residual_stored = ref ? true_residual(op, op->plan64, b, x, st) : rel;
    info->converged = rel <= stop ? 1 : 0;
  }
  info->stop_tol = stop;
  info->seconds = now_s() - t0;
}

}  // namespace

// The stream of a context (the request loop times its requests' GPU work on it).
cudaStream_t ctx_stream(const hodlr_ctx* ctx) { return ctx ? ctx->stream : nullptr; }

namespace {

int guarded(hodlr_ctx* ctx, const std::function<int()>& f) {
  try {
    return f();
  } catch (const Failure& e) {
    return fail(ctx, e.code, e.msg);
  } catch (const std::bad_alloc&) {
    return fail(ctx, HODLR_ERR_OOM, "host allocation failed");
  } catch (const std::exception& e) {
    return fail(ctx, HODLR_ERR_INVALID, e.what());
  }
}

// Runs f(i, stream) for i < n on host threads, each with the device set and
// its own non-blocking stream (synchronised before the thread ends): the
// per-instance parts of a batch build are independent, and their host work
// (plans, allocations) dominates for small instances.  The first failure is
// rethrown once every thread has finished.
template <class F>
void for_each_instance(int n, int device, F f) {
  const int T = std::max(1, std::min(n, std::min(omp_get_max_threads(), 16)));
  std::vector<Failure> errs(size_t(T), Failure{HODLR_OK, std::string()});
  std::atomic<int> next{0};
  auto worker = [&](int t) {
    Failure& err = errs[size_t(t)];
    cudaStream_t s = nullptr;
    try {
      check_cuda(cudaSetDevice(device), "cudaSetDevice");
      check_cuda(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "cudaStreamCreate");
      for (int i = next++; i < n; i = next++) f(i, s);
    } catch (const Failure& e) {
      err = e;
    } catch (const std::bad_alloc&) {
      err = Failure{HODLR_ERR_OOM, "host allocation failed"};
    } catch (const std::exception& e) {
      err = Failure{HODLR_ERR_INVALID, e.what()};
    }
    if (s) {
      cudaStreamSynchronize(s);
      cudaStreamDestroy(s);
    }
  };
#pragma omp parallel num_threads(T)
  worker(omp_get_thread_num());
  for (const Failure& e : errs)
    if (e.code != HODLR_OK) throw e;
}

}  // namespace

// ================================================================= C ABI


// State carried from build_prepare to build_finish.
struct BuildState {
  NearTiles nt, nt32;
  double* near64 = nullptr;
  float* near32 = nullptr;
  double t0 = 0.0, t2 = 0.0;
};

// Tree, lists, points and the near field of `op` (op->p, op->kd, op->n set).
void build_prepare(hodlr_op* op, const double* points, const double* box_lo, const double* box_hi, cudaStream_t st,
                   BuildState& bs) {
  const int64_t n = op->n;
  op->box_lo.assign(box_lo, box_lo + op->p.ndim);
  op->box_hi.assign(box_hi, box_hi + op->p.ndim);
  const double t0 = bs.t0 = now_s();
  TreeParams tp;
  tp.ndim = op->p.ndim;
  tp.nmax = op->p.nmax;
  tp.dprime = op->p.dprime;
  // the tree, its lists, the points in tree order, the permutation and the
  // reference-order maps, built on the device
  const int d = op->p.ndim;
  op->d_pts = op->mem.alloc_n<double>(size_t(n) * size_t(d), "points");
  op->d_perm = op->mem.alloc_n<int64_t>(size_t(n), "permutation");
  DeviceTreeOut dto;
  dto.d_pts = op->d_pts;
  dto.d_perm = op->d_perm;
  dto.alloc_lmap = [op](size_t k) { return op->mem.alloc_n<int32_t>(k, "reference-order map"); };
  const DeviceTreeStatus ds = build_tree_device(tp, points, n, box_lo, box_hi, op->tree, dto, st);
  if (ds.code != 0) throw Failure{ds.code, "hodlr_build: " + ds.msg};
  op->d_lmap = dto.d_lmap;
  op->far = far_blocks(op->tree);
  op->near = near_blocks(op->tree);
  op->nslots = op->tree.levels;
  const double t1 = now_s();
  op->st.t_tree_s = t1 - t0;
  // near field
  bs.nt = near_tiles(op->tree, op->near, 8);
  const NearTiles& nt = bs.nt;
  PointsDev P{op->d_pts, n};
  KernelDev K{op->kd.kind, op->kd.scale, op->kd.diag};
  TileDesc* d_tiles = upload(op->mem, nt.tiles, st, "near tile descriptors");
  double* near64 = bs.near64 = op->mem.alloc_n<double>(size_t(std::max<int64_t>(nt.total, 1)), "near field (FP64)");
  CK(cudaMemsetAsync(near64, 0, sizeof(double) * size_t(std::max<int64_t>(nt.total, 1)), st));
  CK(launch_assemble(d, P, K, d_tiles, int(nt.tiles.size()), near64, Prec::kD, st));
  if (op->p.precision == HODLR_PREC_MIXED) {
    bs.nt32 = near_tiles(op->tree, op->near, 4);
    const NearTiles& nt32 = bs.nt32;
    TileDesc* d_tiles32 = upload(op->mem, nt32.tiles, st, "near tile descriptors");
    float* near32 = bs.near32 = op->mem.alloc_n<float>(size_t(std::max<int64_t>(nt32.total, 1)), "near field (FP32)");
    CK(cudaMemsetAsync(near32, 0, sizeof(float) * size_t(std::max<int64_t>(nt32.total, 1)), st));
    CK(launch_assemble(d, P, K, d_tiles32, int(nt32.tiles.size()), near32, Prec::kF, st));
    CK(cudaStreamSynchronize(st));
    op->mem.release(d_tiles32);
  }
  CK(cudaStreamSynchronize(st));
  op->mem.release(d_tiles);
  bs.t2 = now_s();
  const double t2 = bs.t2;
  op->st.t_near_s = t2 - t1;
}

// FP32 far field: moves every block's U (or dense tile) into one buffer in
// the far plan's panel order -- the segments of a panel then sit back to
// back, each padded to 16 bytes, so the leaf-panel kernel streams a panel
// with one bulk copy per stage -- and every V into a second buffer; the ACA
// batches' chunks are freed.
void relayout_far(hodlr_op* op, cudaStream_t st) {
  const size_t nb = op->far.size();
  if (nb == 0 || op->p.precision == HODLR_PREC_FP64) return;
  const Prec fp = far_prec(op->p);
  std::vector<uint64_t> uoff(nb, 0);
  uint64_t ubytes = 0;
  const Tree& t = op->tree;
  // op->far is grouped by (level, target): the plan's panel order
  for (size_t q = 0; q < nb; q++) {
    const int l = op->far[q].level;
    const int64_t m = t.count[size_t(t.gid(l, op->far[q].t))], n = t.count[size_t(t.gid(l, op->far[q].s))];
    if (!op->dense[q] && op->rank[q] <= 0) continue;
    uoff[q] = ubytes;
    ubytes += far_u_bytes(m, n, op->rank[q], op->dense[q], fp);
  }
  char* fu = static_cast<char*>(op->mem.alloc(std::max<uint64_t>(ubytes, 16), "far-field factors (panel order)"));
  std::vector<CopyDesc> cd;
  cd.reserve(nb);
  for (size_t q = 0; q < nb; q++) {
    const int l = op->far[q].level;
    const int64_t m = t.count[size_t(t.gid(l, op->far[q].t))], n = t.count[size_t(t.gid(l, op->far[q].s))];
    if (!op->dense[q] && op->rank[q] <= 0) continue;
    cd.push_back({op->uptr[q], fu + uoff[q], far_u_bytes(m, n, op->rank[q], op->dense[q], fp)});
    op->uptr[q] = fu + uoff[q];
  }
  // V: the low-rank blocks of each source node (level, s), in far-block order,
  // packed side by side into row-major chunks of at most kVChunkCols columns
  // (each block its vpad(rank) columns; a wider block gets a chunk of its
  // own), so that z = V^T x reads one contiguous run per chunk.  BF16 chunks
  // keep their w z scales after the values.
  const int esz = prec_size(fp);
  const int kVChunkCols = std::min(32 * (16 / esz), kZPart);
  std::vector<size_t> lr;
  for (size_t q = 0; q < nb; q++)
    if (!op->dense[q] && op->rank[q] > 0) lr.push_back(q);
  std::stable_sort(lr.begin(), lr.end(), [&](size_t a, size_t b) {
    return op->far[a].level != op->far[b].level ? op->far[a].level < op->far[b].level
                                                : op->far[a].s < op->far[b].s;
  });
  op->vstride.assign(nb, 0);
  op->zpos.assign(nb, 0);
  op->vchunk_of.assign(nb, -1);
  op->zsptr.assign(nb, nullptr);
  op->vchunks.clear();
  struct Place {
    size_t chunk;
    int32_t coff;
  };
  std::vector<Place> place(nb, Place{0, 0});
  std::vector<uint64_t> cbyte;  // chunk offsets in the V array
  uint64_t vbytes = 0;
  int64_t zb = op->n;
  for (size_t i = 0; i < lr.size();) {
    const int l = op->far[lr[i]].level;
    const int64_t s_ = op->far[lr[i]].s;
    size_t e = i;
    while (e < lr.size() && op->far[lr[e]].level == l && op->far[lr[e]].s == s_) e++;
    const int64_t gs = t.gid(l, s_);
    const int32_t n = int32_t(t.count[size_t(gs)]);
    for (size_t k = i; k < e;) {
      hodlr_op::VChunk c{nullptr, t.begin[size_t(gs)], zb, n, 0, nullptr};
      while (k < e) {
        const int32_t w = int32_t(vpad(op->rank[lr[k]], esz));
        if (c.w > 0 && c.w + w > kVChunkCols) break;
        place[lr[k]] = Place{op->vchunks.size(), c.w};
        c.w += w;
        k++;
      }
      cbyte.push_back(vbytes);
      vbytes += round16(uint64_t(n) * uint64_t(c.w) * uint64_t(esz)) + (fp == Prec::kB ? round16(uint64_t(c.w) * 4) : 0);
      zb += c.w;
      op->vchunks.push_back(c);
    }
    i = e;
  }
  char* fv = static_cast<char*>(op->mem.alloc(std::max<uint64_t>(vbytes, 16), "far-field V factors (by source)"));
  CK(cudaMemsetAsync(fv, 0, std::max<uint64_t>(vbytes, 16), st));  // scale slots of padding columns
  for (size_t c = 0; c < op->vchunks.size(); c++) {
    hodlr_op::VChunk& C = op->vchunks[c];
    C.V = fv + cbyte[c];
    if (fp == Prec::kB)
      C.zscale = reinterpret_cast<const float*>(fv + cbyte[c] + round16(uint64_t(C.n) * uint64_t(C.w) * uint64_t(esz)));
  }
  std::vector<RowCopy> rc;
  rc.reserve(lr.size() * (fp == Prec::kB ? 2 : 1));
  for (size_t q : lr) {
    const hodlr_op::VChunk& C = op->vchunks[place[q].chunk];
    const int32_t r = op->rank[q], w = int32_t(vpad(r, esz)), coff = place[q].coff;
    char* dst = static_cast<char*>(const_cast<void*>(C.V)) + int64_t(coff) * esz;
    rc.push_back({op->vptr[q], dst, int64_t(w) * esz, int64_t(C.w) * esz, int32_t(w * esz), C.n});
    if (fp == Prec::kB) {
      const char* s_scale = static_cast<const char*>(op->vptr[q]) + far_v_data_bytes(C.n, r, false, fp);
      float* d_scale = const_cast<float*>(C.zscale) + coff;
      rc.push_back({s_scale, d_scale, 0, 0, int32_t(round16(uint64_t(r) * 4)), 1});
      op->zsptr[q] = d_scale;
    }
    op->vptr[q] = dst;
    op->vchunk_of[q] = int32_t(place[q].chunk);
    op->vstride[q] = C.w;
    op->zpos[q] = C.zbase + coff;
  }
  // descriptors in slices of 2^20 (one CTA each)
  const size_t slice = size_t(1) << 20;
  CopyDesc* d_cd = op->mem.alloc_n<CopyDesc>(std::min(cd.size(), slice) + 1, "relayout descriptors");
  for (size_t b = 0; b < cd.size(); b += slice) {
    const size_t k = std::min(slice, cd.size() - b);
    CK(cudaMemcpyAsync(d_cd, cd.data() + b, k * sizeof(CopyDesc), cudaMemcpyHostToDevice, st));
    CK(launch_copy16(d_cd, int(k), st));
    CK(cudaStreamSynchronize(st));
  }
  RowCopy* d_rc = op->mem.alloc_n<RowCopy>(std::min(rc.size(), slice) + 1, "relayout descriptors");
  for (size_t b = 0; b < rc.size(); b += slice) {
    const size_t k = std::min(slice, rc.size() - b);
    CK(cudaMemcpyAsync(d_rc, rc.data() + b, k * sizeof(RowCopy), cudaMemcpyHostToDevice, st));
    CK(launch_copy_rows(d_rc, int(k), st));
    CK(cudaStreamSynchronize(st));
  }
  op->mem.release(d_rc);
  op->mem.release(d_cd);
  for (void* c : op->far_chunks) op->mem.release(c);
  op->far_chunks.clear();
}

// Plans, work vectors and statistics, once the far blocks are compressed.
void build_finish(hodlr_op* op, BuildState& bs, cudaStream_t st) {
  const int64_t n = op->n;
  relayout_far(op, st);
  const std::vector<const void*>& uptr = op->uptr;
  const std::vector<const void*>& vptr = op->vptr;
  // plans
  const Prec fp = far_prec(op->p);
  build_near_plan(op, bs.nt, bs.near64, Prec::kD, op->plan64, st);
  build_far_plan(op, uptr, vptr, fp, op->plan64, st);
  if (op->p.precision == HODLR_PREC_MIXED) {
    build_near_plan(op, bs.nt32, bs.near32, Prec::kF, op->plan32, st);
    op->plan32.a_far = Prec::kF;
    op->plan32.contig_far = op->plan64.contig_far;
    op->plan32.panels_far = op->plan64.panels_far;
    op->plan32.segs_far = op->plan64.segs_far;
    op->plan32.small_far = op->plan64.small_far;
    op->plan32.big_far = op->plan64.big_far;
    op->plan32.nsmall_far = op->plan64.nsmall_far;
    op->plan32.nbig_far = op->plan64.nbig_far;
    op->plan32.zb = op->plan64.zb;
    op->plan32.nzb = op->plan64.nzb;
    op->plan32.zitems = op->plan64.zitems;
    op->plan32.nzitems = op->plan64.nzitems;
    op->plan32.zfix = op->plan64.zfix;
    op->plan32.nzfix = op->plan64.nzfix;
    op->plan32.pfix_far = op->plan64.pfix_far;
    op->plan32.npfix_far = op->plan64.npfix_far;
    op->plan32.nzpart = op->plan64.nzpart;
    op->plan32.nypart = std::max(op->plan64.nypart, op->plan32.nypart_near);
    op->plan32.zpart = op->mem.alloc(size_t(std::max<int64_t>(op->plan32.nzpart, 1)) * 4, "z partial sums (FP32)");
    op->plan32.ypart = op->mem.alloc(size_t(std::max<int64_t>(op->plan32.nypart, 1)) * 4, "row partial sums (FP32)");
  }
  op->plan64.nypart = std::max(op->plan64.nypart, op->plan64.nypart_near);
  op->plan64.zpart = op->mem.alloc(size_t(std::max<int64_t>(op->plan64.nzpart, 1)) * 8, "z partial sums");
  op->plan64.ypart = op->mem.alloc(size_t(std::max<int64_t>(op->plan64.nypart, 1)) * 8, "row partial sums");
  if (op->has_ref) {
    // the FP64 operator: the FP64 near field of plan64, the FP64 far factors
    Plan& r = op->plan_ref;
    build_far_plan(op, op->uptr64, op->vptr64, Prec::kD, r, st);
    r.a_near = op->plan64.a_near;
    r.panels_near = op->plan64.panels_near;
    r.segs_near = op->plan64.segs_near;
    r.small_near = op->plan64.small_near;
    r.big_near = op->plan64.big_near;
    r.nsmall_near = op->plan64.nsmall_near;
    r.nbig_near = op->plan64.nbig_near;
    r.pfix_near = op->plan64.pfix_near;
    r.npfix_near = op->plan64.npfix_near;
    r.nypart_near = op->plan64.nypart_near;
    r.contig_near = op->plan64.contig_near;
    r.nypart = std::max(r.nypart, r.nypart_near);
    r.zpart = op->mem.alloc(size_t(std::max<int64_t>(r.nzpart, 1)) * 8, "z partial sums (FP64 reference)");
    r.ypart = op->mem.alloc(size_t(std::max<int64_t>(r.nypart, 1)) * 8, "row partial sums (FP64 reference)");
  }
  // work vectors; the input buffers [x | z] end in 16 bytes of padding,
  // which the streaming V^T x stage copies may read (a run of inputs is
  // copied from the 16-byte boundary below it to the one above it)
  const int64_t ldin = n + op->zlen;
  op->d_in64 = static_cast<double*>(op->mem.alloc(size_t(ldin) * 8 + 16, "matvec input"));
  if (op->p.precision != HODLR_PREC_FP64)
    op->d_in2 = op->mem.alloc(size_t(ldin) * 8 + 16, "matvec input (FP32 pairs)");
  op->d_y64 = op->mem.alloc_n<double>(size_t(n) * size_t(op->nslots), "matvec slots");
  op->d_b64 = op->mem.alloc_n<double>(size_t(n), "rhs");
  op->d_x64 = op->mem.alloc_n<double>(size_t(n), "solution");
  op->d_r64 = op->mem.alloc_n<double>(size_t(n), "residual");
  op->d_io = op->mem.alloc_n<double>(size_t(n), "staging");
  if (op->has_ref) {
    op->d_rref = op->mem.alloc_n<double>(size_t(n), "refinement residual");
    op->d_dref = op->mem.alloc_n<double>(size_t(n), "refinement correction");
  }
  op->d_io2 = op->mem.alloc_n<double>(size_t(n), "staging");
  op->d_hb = op->mem.alloc_n<double>(size_t(n), "host staging");
  op->d_hx = op->mem.alloc_n<double>(size_t(n), "host staging");
  op->d_part = op->mem.alloc_n<double>(size_t(kVecCtas), "partials");
  op->d_scal = op->mem.alloc_n<double>(8, "scalars");
  CK(cudaMallocHost(&op->h_scal, sizeof(double) * 8));
  CK(cudaMallocHost(&op->h_waits, sizeof(unsigned int)));
  CK(read_stream_timeouts(op->h_waits, st));
  CK(cudaStreamSynchronize(st));
  op->waits_seen = *op->h_waits;
  const int restart = op->p.restart > 0 ? op->p.restart : 100;
  if (op->p.precision == HODLR_PREC_MIXED) {
    op->d_in32 = static_cast<float*>(op->mem.alloc(size_t(ldin) * 4 + 16, "matvec input (FP32)"));
    op->d_y32 = op->mem.alloc_n<float>(size_t(n) * size_t(op->nslots), "matvec slots (FP32)");
    op->d_r32 = op->mem.alloc_n<float>(size_t(n), "residual (FP32)");
    op->d_d32 = op->mem.alloc_n<float>(size_t(n), "correction (FP32)");
    CK(gmres_alloc<float>(op->g32, n, restart));
  } else {
    CK(gmres_alloc<double>(op->g64, n, restart));
  }
  CK(cudaStreamSynchronize(st));
  op->st.t_build_s = now_s() - bs.t0;
  compute_stats(op);
}


// ---- batches ---------------------------------------------------------------
// The operators of a batch are built together (their far blocks share the ACA
// launches) and keep their own storage; the batch adds one merged plan over
// all of them, so that a matvec of every instance is one launch per phase,
// and a CUDA graph of that launch sequence per (x, y, nrhs).
struct hodlr_batch {
  hodlr_ctx* ctx = nullptr;
  std::vector<hodlr_op*> ops;
  Prec vec = Prec::kD;  // vector type of hodlr_batch_matvec_device
  bool df = false;      // FP32 factors with FP64 vectors (compensated accumulation)
  DevMem mem;
  Plan plan;
  int64_t ld_in = 0, ycol = 0, total_n = 0, max_n = 0;
  std::vector<int64_t> offsets;  // instance i: rows offsets[i] .. offsets[i+1] of the caller's vectors
  BatchInst* d_inst = nullptr;
  void* d_in = nullptr;   // [x | z] of every instance, vector type
  void* d_in2 = nullptr;  // the same as (hi, lo) FP32 pairs (df)
  void* d_y = nullptr;    // output slots of every instance
  // several right-hand sides (FP32 vectors): nchunks_mr chunks of kMR columns
  int nchunks_mr = 0;
  float *d_in_mr = nullptr, *d_y_mr = nullptr, *d_zpart_mr = nullptr, *d_ypart_mr = nullptr;
  struct Graph {
    const void* x;
    void* y;
    int64_t nrhs;
    cudaGraph_t graph;
    cudaGraphExec_t exec;
    uint64_t kernels;
  };
  std::vector<Graph> graphs;
  ~hodlr_batch() {
    for (Graph& g : graphs) {
      cudaGraphExecDestroy(g.exec);
      cudaGraphDestroy(g.graph);
    }
    for (hodlr_op* op : ops) delete op;
    mem.release_all();
  }
};

namespace {

// The merged plan of the batch (vector type b.vec): every instance's items,
// segments and panels with their offsets moved to the instance's place in the
// batch's input buffer, output slots and partial-sum scratch.
void build_batch_plan(hodlr_batch& b, cudaStream_t st) {
  Plan::Host h;
  const bool f32 = b.vec == Prec::kF;
  const size_t nops = b.ops.size();
  // where each instance's records go in the merged arrays (prefix sums over
  // the instances), then the records themselves, instances in parallel
  struct Base {
    int64_t panels_near = 0, segs_near = 0, small_near = 0, big_near = 0, pfix_near = 0, near_parts = 0;
    int64_t panels_far = 0, segs_far = 0, small_far = 0, big_far = 0, pfix_far = 0, far_parts = 0;
    int64_t zb = 0, zitems = 0, zfix = 0, zpart = 0, in = 0, y = 0, x = 0;
  };
  std::vector<Base> base(nops + 1);
  std::vector<BatchInst> inst(nops);
  b.offsets.assign(1, 0);
  bool contig_near = true, contig_far = true;
  for (size_t j = 0; j < nops; j++) {
    const hodlr_op* op = b.ops[j];
    const Plan& pn = f32 ? op->plan32 : op->plan64;  // near field and scratch sizes
    const Plan::Host& hn = *pn.host;
    const Plan::Host& hf = *op->plan64.host;  // far field (shared by both vector types)
    const Base& a = base[j];
    Base& e = base[j + 1];
    BatchInst& I = inst[j];
    I.n = op->n;
    I.x_base = a.x;
    I.in_base = a.in;
    I.y_base = a.y;
    I.perm = op->d_perm;
    I.nslots = op->nslots;
    I.pad = 0;
    e.panels_near = a.panels_near + int64_t(hn.panels_near.size());
    e.segs_near = a.segs_near + int64_t(hn.segs_near.size());
    e.small_near = a.small_near + int64_t(hn.small_near.size());
    e.big_near = a.big_near + int64_t(hn.big_near.size());
    e.pfix_near = a.pfix_near + int64_t(hn.pfix_near.size());
    e.near_parts = a.near_parts + pn.nypart_near / rows_per_item(pn.a_near);
    e.panels_far = a.panels_far + int64_t(hf.panels_far.size());
    e.segs_far = a.segs_far + int64_t(hf.segs_far.size());
    e.small_far = a.small_far + int64_t(hf.small_far.size());
    e.big_far = a.big_far + int64_t(hf.big_far.size());
    e.pfix_far = a.pfix_far + int64_t(hf.pfix_far.size());
    int64_t op_far_parts = 0;
    for (const PanelFix& f : hf.pfix_far) op_far_parts += f.count;
    e.far_parts = a.far_parts + op_far_parts;
    e.zb = a.zb + int64_t(hf.zb.size());
    e.zitems = a.zitems + int64_t(hf.zitems.size());
    e.zfix = a.zfix + int64_t(hf.zfix.size());
    e.zpart = a.zpart + op->plan64.nzpart;
    e.in = a.in + op->n + op->zlen;
    e.y = a.y + int64_t(op->nslots) * op->n;
    e.x = a.x + op->n;
    b.offsets.push_back(e.x);
    b.max_n = std::max(b.max_n, op->n);
    // the merged items reference the same factor bytes, so their layout
    // test is each instance's own
    contig_near = contig_near && pn.contig_near;
    contig_far = contig_far && op->plan64.contig_far;
  }
  const Base& tot = base[nops];
  h.panels_near.resize(size_t(tot.panels_near));
  h.segs_near.resize(size_t(tot.segs_near));
  h.small_near.resize(size_t(tot.small_near));
  h.big_near.resize(size_t(tot.big_near));
  h.pfix_near.resize(size_t(tot.pfix_near));
  h.panels_far.resize(size_t(tot.panels_far));
  h.segs_far.resize(size_t(tot.segs_far));
  h.small_far.resize(size_t(tot.small_far));
  h.big_far.resize(size_t(tot.big_far));
  h.pfix_far.resize(size_t(tot.pfix_far));
  h.zb.resize(size_t(tot.zb));
  h.zitems.resize(size_t(tot.zitems));
  h.zfix.resize(size_t(tot.zfix));
  auto shift_item = [](Item it, int64_t panel_base, int64_t seg_base, int64_t part_base) {
    it.panel += int32_t(panel_base);
    it.seg_b += int32_t(seg_base);
    it.seg_e += int32_t(seg_base);
    if (it.part >= 0) it.part += int32_t(part_base);
    return it;
  };
#pragma omp parallel for schedule(dynamic, 1) num_threads(std::max(1, std::min<int>(int(nops), 16)))
  for (int64_t jj = 0; jj < int64_t(nops); jj++) {
    const size_t j = size_t(jj);
    const hodlr_op* op = b.ops[j];
    const Plan& pn = f32 ? op->plan32 : op->plan64;
    const Plan::Host& hn = *pn.host;
    const Plan::Host& hf = *op->plan64.host;
    const Base& a = base[j];
    // near field
    for (size_t k = 0; k < hn.panels_near.size(); k++) {
      Panel p = hn.panels_near[k];
      p.seg_begin += a.segs_near;
      p.seg_end += a.segs_near;
      p.yoff += a.y;
      h.panels_near[size_t(a.panels_near) + k] = p;
    }
    for (size_t k = 0; k < hn.segs_near.size(); k++) {
      Seg sg = hn.segs_near[k];
      sg.in_off += a.in;
      h.segs_near[size_t(a.segs_near) + k] = sg;
    }
    for (size_t k = 0; k < hn.small_near.size(); k++)
      h.small_near[size_t(a.small_near) + k] = shift_item(hn.small_near[k], a.panels_near, a.segs_near, a.near_parts);
    for (size_t k = 0; k < hn.big_near.size(); k++)
      h.big_near[size_t(a.big_near) + k] = shift_item(hn.big_near[k], a.panels_near, a.segs_near, a.near_parts);
    for (size_t k = 0; k < hn.pfix_near.size(); k++) {
      PanelFix f = hn.pfix_near[k];
      f.panel += int32_t(a.panels_near);
      f.part += int32_t(a.near_parts);
      h.pfix_near[size_t(a.pfix_near) + k] = f;
    }
    // far field
    for (size_t k = 0; k < hf.panels_far.size(); k++) {
      Panel p = hf.panels_far[k];
      p.seg_begin += a.segs_far;
      p.seg_end += a.segs_far;
      p.yoff += a.y;
      h.panels_far[size_t(a.panels_far) + k] = p;
    }
    for (size_t k = 0; k < hf.segs_far.size(); k++) {
      Seg sg = hf.segs_far[k];
      sg.in_off += a.in;
      h.segs_far[size_t(a.segs_far) + k] = sg;
    }
    for (size_t k = 0; k < hf.small_far.size(); k++)
      h.small_far[size_t(a.small_far) + k] = shift_item(hf.small_far[k], a.panels_far, a.segs_far, a.far_parts);
    for (size_t k = 0; k < hf.big_far.size(); k++)
      h.big_far[size_t(a.big_far) + k] = shift_item(hf.big_far[k], a.panels_far, a.segs_far, a.far_parts);
    for (size_t k = 0; k < hf.pfix_far.size(); k++) {
      PanelFix f = hf.pfix_far[k];
      f.panel += int32_t(a.panels_far);
      f.part += int32_t(a.far_parts);
      h.pfix_far[size_t(a.pfix_far) + k] = f;
    }
    // V^T x
    for (size_t k = 0; k < hf.zb.size(); k++) {
      ZBlock z = hf.zb[k];
      z.x_off += a.in;
      z.z_off += a.in;
      h.zb[size_t(a.zb) + k] = z;
    }
    for (size_t k = 0; k < hf.zitems.size(); k++) {
      ZItem it = hf.zitems[k];
      it.zb += int32_t(a.zb);
      if (it.part >= 0) it.part += int32_t(a.zpart);
      h.zitems[size_t(a.zitems) + k] = it;
    }
    for (size_t k = 0; k < hf.zfix.size(); k++) {
      ZFix f = hf.zfix[k];
      f.zpos += a.in;
      f.part += int32_t(a.zpart);
      h.zfix[size_t(a.zfix) + k] = f;
    }
  }
  const int64_t in_base = tot.in, y_base = tot.y, x_base = tot.x, zpart = tot.zpart;
  const int64_t near_parts = tot.near_parts, far_parts = tot.far_parts;
  if (in_base > (int64_t(1) << 31) || zpart > (int64_t(1) << 31))
    throw Failure{HODLR_ERR_INVALID, "hodlr_build_batch: the batch is too large for one merged plan"};
  b.ld_in = in_base;
  b.ycol = y_base;
  b.total_n = x_base;
  Plan& p = b.plan;
  const Plan& p0 = f32 ? b.ops[0]->plan32 : b.ops[0]->plan64;
  p.a_near = p0.a_near;
  p.a_far = b.ops[0]->plan64.a_far;
  p.panels_near = upload(b.mem, h.panels_near, st, "batch near panels");
  p.segs_near = upload(b.mem, h.segs_near, st, "batch near segments");
  p.small_near = upload(b.mem, h.small_near, st, "batch near items");
  p.big_near = upload(b.mem, h.big_near, st, "batch near items");
  p.nsmall_near = int(h.small_near.size());
  p.nbig_near = int(h.big_near.size());
  p.pfix_near = upload(b.mem, h.pfix_near, st, "batch near fix-ups");
  p.npfix_near = int(h.pfix_near.size());
  p.panels_far = upload(b.mem, h.panels_far, st, "batch far panels");
  p.contig_near = contig_near;
  p.contig_far = p.a_far != Prec::kD && contig_far;
  p.segs_far = upload(b.mem, h.segs_far, st, "batch far segments");
  p.small_far = upload(b.mem, h.small_far, st, "batch far items");
  p.big_far = upload(b.mem, h.big_far, st, "batch far items");
  p.nsmall_far = int(h.small_far.size());
  p.nbig_far = int(h.big_far.size());
  p.pfix_far = upload(b.mem, h.pfix_far, st, "batch far fix-ups");
  p.npfix_far = int(h.pfix_far.size());
  p.zb = upload(b.mem, h.zb, st, "batch z blocks");
  p.nzb = int(h.zb.size());
  p.zitems = upload(b.mem, h.zitems, st, "batch z items");
  p.nzitems = int(h.zitems.size());
  p.zfix = upload(b.mem, h.zfix, st, "batch z fix-ups");
  p.nzfix = int(h.zfix.size());
  const size_t vsz = f32 ? 4 : 8;
  p.nzpart = zpart;
  p.nypart = std::max(near_parts * rows_per_item(p.a_near), far_parts * rows_per_item(p.a_far));
  p.zpart = b.mem.alloc(size_t(std::max<int64_t>(p.nzpart, 1)) * vsz, "batch z partial sums");
  p.ypart = b.mem.alloc(size_t(std::max<int64_t>(p.nypart, 1)) * vsz, "batch row partial sums");
  b.d_inst = upload(b.mem, inst, st, "batch instances");
  b.d_in = b.mem.alloc(size_t(b.ld_in) * vsz + 16, "batch matvec input");
  if (b.df) b.d_in2 = b.mem.alloc(size_t(b.ld_in) * 8 + 16, "batch matvec input (FP32 pairs)");
  b.d_y = b.mem.alloc(size_t(b.ycol) * vsz, "batch matvec slots");
  CK(cudaStreamSynchronize(st));
}

// One column: x (caller order, all instances) -> y.
void batch_apply(hodlr_batch& b, const void* x, void* y, cudaStream_t st) {
  const Plan& p = b.plan;
  const size_t vsz = b.vec == Prec::kF ? 4 : 8;
  CK(launch_batch_gather(b.vec, b.d_inst, int(b.ops.size()), b.max_n, x, b.d_in, st));
  CK(cudaMemsetAsync(b.d_y, 0, size_t(b.ycol) * vsz, st));
  void* fin = b.d_in;
  Accum acc = Accum::kByType;
  if (b.df) {
    fin = b.d_in2;
    acc = Accum::kCompensated;
    CK(launch_split(static_cast<const double*>(b.d_in), fin, b.ld_in, st));
  }
  CK(launch_zgemv(p.a_far, b.vec, p.zb, p.zitems, p.nzitems, p.zfix, p.nzfix, p.zpart, fin, b.ld_in, 1, st, acc));
  CK(launch_panels(p.a_near, b.vec, p.panels_near, p.segs_near, p.small_near, p.nsmall_near, p.big_near, p.nbig_near,
                   p.pfix_near, p.npfix_near, p.ypart, b.d_in, b.ld_in, b.d_y, b.ycol, 1, 1, st, Accum::kByType,
                   p.contig_near));
  CK(launch_panels(p.a_far, b.vec, p.panels_far, p.segs_far, p.small_far, p.nsmall_far, p.big_far, p.nbig_far,
                   p.pfix_far, p.npfix_far, p.ypart, fin, b.ld_in, b.d_y, b.ycol, 1, 1, st, acc, p.contig_far));
  CK(launch_batch_combine(b.vec, b.d_inst, int(b.ops.size()), b.max_n, b.d_y, y, st));
}

// All columns at once with FP32 vectors: chunks of kMR right-hand sides, each
// factor byte read once per chunk (kernels of the multi-RHS family).
// Work buffers of nch chunks (allocated outside any stream capture).
void ensure_mr_buffers(hodlr_batch& b, int nch) {
  const Plan& p = b.plan;
  if (nch > b.nchunks_mr) {
    for (void* q : {static_cast<void*>(b.d_in_mr), static_cast<void*>(b.d_y_mr), static_cast<void*>(b.d_zpart_mr),
                    static_cast<void*>(b.d_ypart_mr)})
      if (q) b.mem.release(q);
    const size_t c = size_t(nch) * kMR * sizeof(float);
    b.d_in_mr = static_cast<float*>(b.mem.alloc(size_t(b.ld_in) * c, "batch multi-RHS input"));
    b.d_y_mr = static_cast<float*>(b.mem.alloc(size_t(b.ycol) * c, "batch multi-RHS slots"));
    b.d_zpart_mr =
        static_cast<float*>(b.mem.alloc(size_t(std::max<int64_t>(p.nzpart, 1)) * c, "batch multi-RHS z partial sums"));
    b.d_ypart_mr = static_cast<float*>(
        b.mem.alloc(size_t(std::max<int64_t>(p.nypart, 1)) * c, "batch multi-RHS row partial sums"));
    b.nchunks_mr = nch;
  }
}

void batch_apply_mr(hodlr_batch& b, const float* x, float* y, int64_t nrhs, cudaStream_t st) {
  const Plan& p = b.plan;
  const int nch = int((nrhs + kMR - 1) / kMR);
  if (nch > b.nchunks_mr) throw Failure{HODLR_ERR_STATE, "batch multi-RHS buffers were not allocated"};
  const int count = int(b.ops.size());
  CK(launch_batch_gather_mr(b.d_inst, count, b.max_n, x, b.total_n, int(nrhs), b.d_in_mr, b.ld_in, nch, st));
  CK(cudaMemsetAsync(b.d_y_mr, 0, size_t(b.ycol) * size_t(nch) * kMR * sizeof(float), st));
  const int64_t zld = std::max<int64_t>(p.nzpart, 1), yld = std::max<int64_t>(p.nypart, 1);
  CK(launch_zgemv_mr(p.zb, p.zitems, p.nzitems, p.zfix, p.nzfix, b.d_zpart_mr, zld, b.d_in_mr, b.ld_in, nch, st));
  CK(launch_panels_mr(p.panels_near, p.segs_near, p.small_near, p.nsmall_near, p.big_near, p.nbig_near, p.pfix_near,
                      p.npfix_near, b.d_ypart_mr, yld, b.d_in_mr, b.ld_in, b.d_y_mr, b.ycol, nch, st));
  CK(launch_panels_mr(p.panels_far, p.segs_far, p.small_far, p.nsmall_far, p.big_far, p.nbig_far, p.pfix_far,
                      p.npfix_far, b.d_ypart_mr, yld, b.d_in_mr, b.ld_in, b.d_y_mr, b.ycol, nch, st));
  CK(launch_batch_combine_mr(b.d_inst, count, b.max_n, b.d_y_mr, b.ycol, y, b.total_n, int(nrhs), nch, st));
}

// ---- tensor-core products for 64 right-hand sides ---------------------------

// Rows buckets of the tensor-core launches: 16, 32, 64, 128, 256.
int tc_bucket(int rows) {
  int b = 16;
  while (b < rows) b <<= 1;
  return b;
}

// Items of the tensor-core panel kernels for one family of panels: per panel,
// its row tiles (one for panels of at most 32 rows) times runs of whole
// segments of at most kTcColsPerItem columns (a longer segment alone) and at
// most kTcMaxSegs segments -- a CTA works through an item's columns one
// 16-column step after another, so long items would leave most SMs idle at
// the end of a launch.  Runs after the first write partial row blocks that a
// fix-up adds in order.  Items are listed by launch: small then big panels,
// each by rows bucket; runs[] gets one entry per non-empty launch (offsets
// into the items until the array is uploaded).
constexpr int kTcColsPerItem = 256;
void tc_panel_items(const std::vector<Panel>& panels, const std::vector<Seg>& segs, std::vector<Item>& items, std::vector<hodlr_op::TcPlan::Run>& runs, std::vector<PanelFix>& fix,
                    int& nparts) {
  std::vector<Item> by[2][5];  // [big][bucket]
  std::vector<std::pair<int32_t, int32_t>> cut;
  for (size_t pi = 0; pi < panels.size(); pi++) {
    const Panel& P = panels[pi];
    const int64_t ns = P.seg_end - P.seg_begin;
    if (ns <= 0 || P.m <= 0) continue;
    cut.clear();
    int64_t start = P.seg_begin, cols = 0;
    for (int64_t q = P.seg_begin; q < P.seg_end; q++) {
      const int64_t K = segs[size_t(q)].K;
      if (q > start && (cols + K > kTcColsPerItem || q - start >= kTcMaxSegs)) {
        cut.push_back({int32_t(start), int32_t(q)});
        start = q;
        cols = 0;
      }
      cols += K;
    }
    cut.push_back({int32_t(start), int32_t(P.seg_end)});
    const int nruns = int(cut.size());
    const bool is_big = P.m > 32;
    const int tiles = is_big ? int((P.m + kTcRows - 1) / kTcRows) : 1;
    for (int tl = 0; tl < tiles; tl++) {
      const int rows = is_big ? std::min<int>(kTcRows, P.m - tl * kTcRows) : P.m;
      int bk = 0;
      while ((16 << bk) < rows) bk++;
      if (nruns > 1) fix.push_back({int32_t(pi), tl, nparts, nruns});
      for (int q = 0; q < nruns; q++) {
        Item it;
        it.panel = int32_t(pi);
        it.chunk = tl;
        it.seg_b = cut[size_t(q)].first;
        it.seg_e = cut[size_t(q)].second;
        it.part = nruns > 1 ? nparts++ : -1;
        by[is_big][bk].push_back(it);
      }
    }
  }
  for (int big = 0; big < 2; big++)
    for (int bk = 0; bk < 5; bk++) {
      const std::vector<Item>& v = by[big][bk];
      if (v.empty()) continue;
      runs.push_back({reinterpret_cast<const void*>(items.size()), int(v.size()), 16 << bk, big});
      items.insert(items.end(), v.begin(), v.end());
    }
}

void build_tc_plan(hodlr_op* op, cudaStream_t st) {
  hodlr_op::TcPlan& T = op->tc;
  if (T.built) return;
  if (!op->plan64.host) throw Failure{HODLR_ERR_STATE, "the operator keeps no host plan for the tensor-core path"};
  const Plan::Host& h = *op->plan64.host;
  std::vector<Item> ni, fi;
  std::vector<PanelFix> fxn, fxf;
  int pn = 0, pf = 0;
  tc_panel_items(h.panels_near, h.segs_near, ni, T.near, fxn, pn);
  tc_panel_items(h.panels_far, h.segs_far, fi, T.far, fxf, pf);
  // z groups: the rows of z by source node, at most kTcRows rows per group.
  // Rows are (z block, k0, nk) runs: with source chunks each low-rank block's
  // own columns of its chunk (its padding columns skipped), else every column
  // of each z block.  A node is its first point and its size: a node and its
  // first child start at the same point.
  struct ZRun {
    int32_t zb, k0, nk;
  };
  std::vector<ZRun> runs;
  if (!op->vchunk_of.empty()) {
    for (size_t q = 0; q < op->far.size(); q++) {
      const int32_t c = op->vchunk_of[q];
      if (c < 0) continue;
      runs.push_back({c, int32_t(op->zpos[q] - op->vchunks[size_t(c)].zbase), op->rank[q]});
    }
  } else {
    for (size_t q = 0; q < h.zb.size(); q++) runs.push_back({int32_t(q), 0, h.zb[q].r});
  }
  auto same_source = [&](const ZBlock& a, const ZBlock& b) { return a.x_off == b.x_off && a.n == b.n; };
  std::stable_sort(runs.begin(), runs.end(), [&](const ZRun& x, const ZRun& y) {
    const ZBlock &a = h.zb[size_t(x.zb)], &b = h.zb[size_t(y.zb)];
    if (a.x_off != b.x_off) return a.x_off < b.x_off;
    if (a.n != b.n) return a.n < b.n;
    return x.zb != y.zb ? x.zb < y.zb : x.k0 < y.k0;
  });
  std::vector<TcZGroup> zg;
  std::vector<TcZEntry> ze;
  for (size_t q = 0; q < runs.size();) {
    const ZBlock& z0 = h.zb[size_t(runs[q].zb)];
    TcZGroup g{z0.x_off, z0.n, int32_t(ze.size()), int32_t(ze.size()), 0, -1, 0};
    while (q < runs.size() && same_source(h.zb[size_t(runs[q].zb)], z0)) {
      const ZRun& R = runs[q];
      for (int32_t k0 = 0; k0 < R.nk;) {
        const int32_t take = std::min(R.nk - k0, kTcRows - g.rows);
        ze.push_back({R.zb, R.k0 + k0, take});
        g.rows += take;
        k0 += take;
        if (g.rows == kTcRows) {  // close the group, continue with a new one on the same source
          g.e_end = int32_t(ze.size());
          zg.push_back(g);
          g = TcZGroup{z0.x_off, z0.n, int32_t(ze.size()), int32_t(ze.size()), 0, -1, 0};
        }
      }
      q++;
    }
    if (g.rows > 0) {
      g.e_end = int32_t(ze.size());
      zg.push_back(g);
    }
  }
  // groups over more than kTcZCols points: column runs writing partial sums,
  // added into z (and scaled) by a fix-up
  std::vector<TcZFix> zfix;
  std::vector<TcZRow> zrows;
  int zparts = 0;
  {
    std::vector<TcZGroup> split;
    for (const TcZGroup& g : zg) {
      if (g.n <= kTcZCols) {
        split.push_back(g);
        continue;
      }
      const int runs = (g.n + kTcZCols - 1) / kTcZCols;
      zfix.push_back({zparts, runs, g.rows, int32_t(zrows.size())});
      T.zfix_rows = std::max(T.zfix_rows, g.rows);
      for (int32_t e = g.e_begin; e < g.e_end; e++) {
        const TcZEntry& E = ze[size_t(e)];
        const ZBlock& Z = h.zb[size_t(E.zb)];
        for (int32_t k = E.k0; k < E.k0 + E.nk; k++) zrows.push_back({Z.z_off + k, Z.zscale ? Z.zscale + k : nullptr});
      }
      for (int c = 0; c < runs; c++) {
        TcZGroup r = g;
        r.x_off = g.x_off + int64_t(c) * kTcZCols;
        r.col0 = c * kTcZCols;
        r.n = std::min(kTcZCols, g.n - c * kTcZCols);
        r.part = zparts++;
        split.push_back(r);
      }
    }
    zg.swap(split);
  }
  // z groups by rows bucket
  std::vector<TcZGroup> zgs;
  for (int bk = 0; bk < 5; bk++) {
    const size_t b0 = zgs.size();
    for (const TcZGroup& g : zg)
      if (tc_bucket(g.rows) == (16 << bk)) zgs.push_back(g);
    if (zgs.size() > b0)
      T.z.push_back({reinterpret_cast<const void*>(b0), int(zgs.size() - b0), 16 << bk, 0});
  }
  const Item* d_ni = upload(op->mem, ni, st, "tensor-core near items");
  const Item* d_fi = upload(op->mem, fi, st, "tensor-core far items");
  const TcZGroup* d_zg = upload(op->mem, zgs, st, "tensor-core z groups");
  for (auto& r : T.near) r.items = d_ni + reinterpret_cast<size_t>(r.items);
  for (auto& r : T.far) r.items = d_fi + reinterpret_cast<size_t>(r.items);
  for (auto& r : T.z) r.items = d_zg + reinterpret_cast<size_t>(r.items);
  T.fix_near = upload(op->mem, fxn, st, "tensor-core near fix-ups");
  T.fix_far = upload(op->mem, fxf, st, "tensor-core far fix-ups");
  T.nfix_near = int(fxn.size());
  T.nfix_far = int(fxf.size());
  T.ze = upload(op->mem, ze, st, "tensor-core z entries");
  T.zfix = upload(op->mem, zfix, st, "tensor-core z fix-ups");
  T.zrows = upload(op->mem, zrows, st, "tensor-core z rows");
  T.nzfix = int(zfix.size());
  T.zpart = op->mem.alloc_n<float>(size_t(std::max(zparts, 1)) * kTcRows * kTcRhs, "tensor-core z partial sums");
  const int64_t n = op->n;
  T.in = op->mem.alloc_n<uint32_t>(size_t(n + op->zlen) * kTcRhs, "tensor-core input (64 right-hand sides)");
  T.y = op->mem.alloc_n<float>(size_t(n) * size_t(op->nslots) * kTcRhs, "tensor-core output slots");
  T.part_near = op->mem.alloc_n<float>(size_t(std::max(pn, 1)) * kTcRows * kTcRhs, "tensor-core partial rows");
  T.part_far = op->mem.alloc_n<float>(size_t(std::max(pf, 1)) * kTcRows * kTcRhs, "tensor-core partial rows");
  T.status = op->mem.alloc_n<unsigned int>(1, "tensor-core status");
  CK(cudaMemsetAsync(T.status, 0, sizeof(unsigned int), st));
  CK(cudaMallocHost(&T.h_status, sizeof(unsigned int)));
  CK(cudaStreamSynchronize(st));
  T.built = true;
}

// Y = A X for up to 64 columns of X (caller order, column major, FP32).
void apply_tc(hodlr_op* op, const float* x, int64_t ldx, float* y, int64_t ldy, int nrhs, cudaStream_t st) {
  hodlr_op::TcPlan& T = op->tc;
  const Plan& P = op->plan64;
  const int64_t n = op->n;
  CK(launch_tc_gather(x, ldx, nrhs, op->d_perm, n, T.in, st));
  CK(cudaMemsetAsync(T.y, 0, sizeof(float) * size_t(n) * size_t(op->nslots) * kTcRhs, st));
  TcLaunch a{};
  a.in = T.in;
  a.y = T.y;
  a.n = n;
  a.status = T.status;
  // z = V^T x, grouped by source node
  a.zb = P.zb;
  a.zentries = T.ze;
  a.part = T.zpart;
  for (const auto& r : T.z) {
    a.zgroups = static_cast<const TcZGroup*>(r.items);
    a.nz = r.n;
    a.nmax = r.rows;
    CK(launch_tc(kTcZ, a, st));
  }
  CK(launch_tc_zfix(T.zfix, T.nzfix, T.zfix_rows, T.zrows, T.zpart, T.in, st));
  a.nz = 0;
  // near field (FP64 tiles, three BF16 terms), then the far field (BF16)
  a.panels = P.panels_near;
  a.segs = P.segs_near;
  a.part = T.part_near;
  for (const auto& r : T.near) {
    a.items = static_cast<const Item*>(r.items), a.nitems = r.n, a.big = r.big, a.nmax = r.rows;
    CK(launch_tc(kTcNear, a, st));
  }
  CK(launch_tc_fix(P.panels_near, T.fix_near, T.nfix_near, T.part_near, T.y, st));
  a.panels = P.panels_far;
  a.segs = P.segs_far;
  a.part = T.part_far;
  for (const auto& r : T.far) {
    a.items = static_cast<const Item*>(r.items), a.nitems = r.n, a.big = r.big, a.nmax = r.rows;
    CK(launch_tc(kTcFar, a, st));
  }
  CK(launch_tc_fix(P.panels_far, T.fix_far, T.nfix_far, T.part_far, T.y, st));
  CK(launch_tc_combine(T.y, op->nslots, n, op->d_perm, y, ldy, nrhs, st));
}

// Why the parameters cannot be used (null when they can): the checks of
// hodlr_ctx_create, applied again to the parameters read from an operator file.
const char* params_problem(const hodlr_params& p) {
  if (p.ndim < 1 || p.ndim > kMaxDim) return "ndim must be in 1..8";
  if (p.nmax < 1) return "nmax must be positive";
  if (p.dprime < -1 || p.dprime > p.ndim - 1) return "dprime must be in -1..ndim-1";
  if (!(p.eps_aca > 0.0) || !(p.eps_aca < 1.0))
    return "eps_aca must be in (0, 1) (values >= 1 select a fixed rank in the reference, which this engine does "
           "not support)";
  if (p.precision != HODLR_PREC_FP64 && p.precision != HODLR_PREC_MIXED && p.precision != HODLR_PREC_FP32_FACTORS &&
      p.precision != HODLR_PREC_BF16_FACTORS)
    return "unknown precision";
  if (p.restart < 0 || p.restart > 1000) return "restart must be in 0..1000";
  if (p.ortho < HODLR_ORTHO_AUTO || p.ortho > HODLR_ORTHO_CGS2) return "unknown orthogonalisation";
  if (p.relax != HODLR_RELAX_AUTO && p.relax != HODLR_RELAX_OFF && p.relax != HODLR_RELAX_ALWAYS)
    return "relax must be HODLR_RELAX_AUTO, _OFF or _ALWAYS";
  if (p.fp64_check != HODLR_FP64_CHECK_AUTO && p.fp64_check != HODLR_FP64_CHECK_OFF)
    return "fp64_check must be HODLR_FP64_CHECK_AUTO or _OFF";
  if (p.aca_workspace_mib < 0) return "aca_workspace_mib must not be negative";
  return nullptr;
}

}  // namespace

extern "C" {

void hodlr_params_default(hodlr_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->ndim = 2;
  p->nmax = 64;
  p->dprime = 0;
  p->restart = 100;
  p->eps_aca = 1e-10;
  p->tol = 0.0;
  p->max_iter = 0;
  p->precision = HODLR_PREC_FP64;
  p->device = 0;
}

const char* hodlr_last_error(const hodlr_ctx* ctx) {
  if (ctx) return ctx->err.c_str();
  return g_thread_err.c_str();
}

int hodlr_ctx_create(const hodlr_params* params, hodlr_ctx** out) {
  if (!params || !out) return fail(nullptr, HODLR_ERR_INVALID, "hodlr_ctx_create: null argument");
  *out = nullptr;
  const hodlr_params& p = *params;
  const char* why = params_problem(p);
  if (why) return fail(nullptr, HODLR_ERR_INVALID, why);
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0)
    return fail(nullptr, HODLR_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
  if (p.device < 0 || p.device >= ndev) return fail(nullptr, HODLR_ERR_INVALID, "device ordinal out of range");
  if ((e = cudaSetDevice(p.device)) != cudaSuccess)
    return fail(nullptr, HODLR_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
  hodlr_ctx* c = new hodlr_ctx();
  c->p = p;
  if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess) {
    delete c;
    return fail(nullptr, HODLR_ERR_CUDA, std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
  }
  *out = c;
  return HODLR_OK;
}

int hodlr_ctx_destroy(hodlr_ctx* ctx) {
  if (!ctx) return HODLR_OK;
  cudaSetDevice(ctx->p.device);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return HODLR_OK;
}

int hodlr_build(hodlr_ctx* ctx, const double* points, int64_t n, const double* box_lo, const double* box_hi,
                const hodlr_kernel_desc* kernel, hodlr_op** out) {
  if (!ctx || !points || !box_lo || !box_hi || !kernel || !out)
    return fail(ctx, HODLR_ERR_INVALID, "hodlr_build: null argument");
  *out = nullptr;
  if (n < 1) return fail(ctx, HODLR_ERR_INVALID, "hodlr_build: need at least one point");
  if (n > (int64_t(1) << 31) - 1) return fail(ctx, HODLR_ERR_INVALID, "hodlr_build: at most 2^31-1 points");
  if (kernel->kind < HODLR_KERNEL_INV_R || kernel->kind > HODLR_KERNEL_EXP_NEG_R)
    return fail(ctx, HODLR_ERR_INVALID, "hodlr_build: unknown kernel kind");
  std::unique_ptr<hodlr_op> op(new hodlr_op());
  op->ctx = ctx;
  op->p = ctx->p;
  op->has_ref = wants_ref(op->p);
  op->keep_host_plans = op->p.precision == HODLR_PREC_BF16_FACTORS;  // the tensor-core plan is built from them
  op->kd = *kernel;
  op->n = n;
  op->mem.budget = ctx->p.device_budget_bytes;
  std::memset(&op->st, 0, sizeof(op->st));
  return guarded(ctx, [&]() -> int {
    CK(cudaSetDevice(ctx->p.device));
    cudaStream_t st = ctx->stream;
    BuildState bs;
    build_prepare(op.get(), points, box_lo, box_hi, st, bs);
    std::vector<hodlr_op*> one{op.get()};
    run_aca(one, st);
    op->st.t_aca_s = now_s() - bs.t2;
    build_finish(op.get(), bs, st);
    *out = op.release();
    return HODLR_OK;
  });
}

int hodlr_op_destroy(hodlr_op* op) {
  if (!op) return HODLR_OK;
  if (op->batch_owned)
    return fail(op->ctx, HODLR_ERR_STATE, "hodlr_op_destroy: the operator belongs to a batch (hodlr_batch_destroy)");
  cudaSetDevice(op->p.device);
  cudaStreamSynchronize(op->ctx->stream);
  delete op;
  return HODLR_OK;
}

// After a synchronised matvec or solve on `st`: a streaming kernel that gave
// up waiting for its copies left results that must not be used.
void check_stream_waits(hodlr_op* op, cudaStream_t st) {
  CK(read_stream_timeouts(op->h_waits, st));
  CK(cudaStreamSynchronize(st));
  if (*op->h_waits != op->waits_seen) {
    op->waits_seen = *op->h_waits;
    throw Failure{HODLR_ERR_DEVICE, "a matvec kernel gave up waiting for its bulk copies; the results are invalid"};
  }
}

int hodlr_matvec_device(hodlr_op* op, const double* d_x, double* d_y, int64_t nrhs, void* stream) {
  if (!op || !d_x || !d_y) return fail(op ? op->ctx : nullptr, HODLR_ERR_INVALID, "hodlr_matvec_device: null argument");
  if (nrhs < 1) return fail(op->ctx, HODLR_ERR_INVALID, "hodlr_matvec_device: nrhs must be positive");
  return guarded(op->ctx, [&]() -> int {
    CK(cudaSetDevice(op->p.device));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int64_t n = op->n;
    for (int64_t c = 0; c < nrhs; c++) {
      // gather into tree order; the combine step scatters back to the caller's order
      CK(launch_gather(d_x + c * n, Prec::kD, n, op->d_perm, n, 1, op->d_io, Prec::kD, n, st));
      CK(apply_tree<double>(op, op->plan64, op->d_io, d_y + c * n, op->d_in64, op->d_y64, st, op->d_perm));
    }
    return HODLR_OK;
  });
}

int hodlr_matvec(hodlr_op* op, const double* x, double* y, int64_t nrhs) {
  if (!op || !x || !y) return fail(op ? op->ctx : nullptr, HODLR_ERR_INVALID, "hodlr_matvec: null argument");
  if (nrhs < 1) return fail(op->ctx, HODLR_ERR_INVALID, "hodlr_matvec: nrhs must be positive");
  return guarded(op->ctx, [&]() -> int {
    CK(cudaSetDevice(op->p.device));
    cudaStream_t st = op->ctx->stream;
    const int64_t n = op->n;
    const double t0 = now_s();
    for (int64_t c = 0; c < nrhs; c++) {
      CK(cudaMemcpyAsync(op->d_b64, x + c * n, sizeof(double) * size_t(n), cudaMemcpyHostToDevice, st));
      const int rc = hodlr_matvec_device(op, op->d_b64, op->d_x64, 1, st);
      if (rc != HODLR_OK) return rc;
      CK(cudaMemcpyAsync(y + c * n, op->d_x64, sizeof(double) * size_t(n), cudaMemcpyDeviceToHost, st));
    }
    CK(cudaStreamSynchronize(st));
    op->st.t_matvec_s = (now_s() - t0) / double(nrhs);
    check_stream_waits(op, st);
    return HODLR_OK;
  });
}

int hodlr_solve_device(hodlr_op* op, const double* d_b, double* d_x, int64_t nrhs, void* stream,
                       hodlr_solve_info* info) {
  if (!op || !d_b || !d_x) return fail(op ? op->ctx : nullptr, HODLR_ERR_INVALID, "hodlr_solve_device: null argument");
  if (nrhs < 1) return fail(op->ctx, HODLR_ERR_INVALID, "hodlr_solve_device: nrhs must be positive");
  hodlr_solve_info local;
  if (!info) info = &local;
  std::memset(info, 0, sizeof(*info));
  return guarded(op->ctx, [&]() -> int {
    CK(cudaSetDevice(op->p.device));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int64_t n = op->n;
    bool all_conv = true;
    double worst = 0.0;
    hodlr_solve_info one;
    for (int64_t c = 0; c < nrhs; c++) {
      CK(launch_gather(d_b + c * n, Prec::kD, n, op->d_perm, n, 1, op->d_b64, Prec::kD, n, st));
      std::memset(&one, 0, sizeof(one));
      solve_tree(op, op->d_b64, op->d_x64, st, &one);
      CK(launch_gather(op->d_x64, Prec::kD, n, nullptr, n, 1, op->d_io, Prec::kD, n, st));
      // scatter: x_caller[perm[i]] = x_tree[i]
      CK(launch_combine(Prec::kD, op->d_io, n, 1, n, 1, op->d_perm, d_x + c * n, Prec::kD, n, st));
      info->iterations += one.iterations;
      info->outer_iterations += one.outer_iterations;
      info->seconds += one.seconds;
      worst = std::max(worst, one.rel_residual);
      all_conv = all_conv && one.converged;
    }
    CK(cudaStreamSynchronize(st));
    check_stream_waits(op, st);
    info->rel_residual = worst;
    info->converged = all_conv ? 1 : 0;
    info->stop_tol = one.stop_tol;
    info->rel_residual_stored = std::max(info->rel_residual_stored, one.rel_residual_stored);
    return all_conv ? HODLR_OK : fail(op->ctx, HODLR_ERR_NOT_CONVERGED, "GMRES did not reach the tolerance");
  });
}

int hodlr_solve(hodlr_op* op, const double* b, double* x, int64_t nrhs, hodlr_solve_info* info) {
  if (!op || !b || !x) return fail(op ? op->ctx : nullptr, HODLR_ERR_INVALID, "hodlr_solve: null argument");
  if (nrhs < 1) return fail(op->ctx, HODLR_ERR_INVALID, "hodlr_solve: nrhs must be positive");
  hodlr_solve_info local;
  if (!info) info = &local;
  std::memset(info, 0, sizeof(*info));
  return guarded(op->ctx, [&]() -> int {
    CK(cudaSetDevice(op->p.device));
    cudaStream_t st = op->ctx->stream;
    const int64_t n = op->n;
    const bool staged = nrhs == 1;
    double* db = staged ? op->d_hb : op->mem.alloc_n<double>(size_t(n * nrhs), "solve rhs");
    double* dx = staged ? op->d_hx : op->mem.alloc_n<double>(size_t(n * nrhs), "solve solution");
    CK(cudaMemcpyAsync(db, b, sizeof(double) * size_t(n * nrhs), cudaMemcpyHostToDevice, st));
    const int rc = hodlr_solve_device(op, db, dx, nrhs, st, info);
    cudaMemcpyAsync(x, dx, sizeof(double) * size_t(n * nrhs), cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    if (!staged) {
      op->mem.release(db);
      op->mem.release(dx);
    }
    return rc;
  });
}

int hodlr_matvec_tc_device(hodlr_op* op, const float* d_x, float* d_y, int64_t nrhs, void* stream) {
  if (!op || !d_x || !d_y) return fail(op ? op->ctx : nullptr, HODLR_ERR_INVALID, "hodlr_matvec_tc_device: null argument");
  if (nrhs < 1) return fail(op->ctx, HODLR_ERR_INVALID, "hodlr_matvec_tc_device: nrhs must be positive");
  if (op->p.precision != HODLR_PREC_BF16_FACTORS)
    return fail(op->ctx, HODLR_ERR_INVALID, "hodlr_matvec_tc_device: the operator must store BF16 factors");
  return guarded(op->ctx, [&]() -> int {
    CK(cudaSetDevice(op->p.device));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    build_tc_plan(op, st);
    const int64_t n = op->n;
    for (int64_t c = 0; c < nrhs; c += kTcRhs) {
      const int k = int(std::min<int64_t>(kTcRhs, nrhs - c));
      apply_tc(op, d_x + c * n, n, d_y + c * n, n, k, st);
    }
    CK(cudaMemcpyAsync(op->tc.h_status, op->tc.status, sizeof(unsigned int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (*op->tc.h_status != 0) {
      CK(cudaMemsetAsync(op->tc.status, 0, sizeof(unsigned int), st));
      throw Failure{HODLR_ERR_DEVICE, "a tensor-core kernel gave up waiting for its MMAs; the results are invalid"};
    }
    return HODLR_OK;
  });
}

int hodlr_set_relax(hodlr_op* op, int32_t relax, double relax_below) {
  if (!op) return fail(nullptr, HODLR_ERR_INVALID, "hodlr_set_relax: null argument");
  if (relax != HODLR_RELAX_AUTO && relax != HODLR_RELAX_OFF && relax != HODLR_RELAX_ALWAYS)
    return fail(op->ctx, HODLR_ERR_INVALID, "hodlr_set_relax: relax must be HODLR_RELAX_AUTO, _OFF or _ALWAYS");
  op->p.relax = relax;
  op->p.relax_below = relax_below;
  return HODLR_OK;
}

int hodlr_set_solver(hodlr_op* op, int32_t restart, double tol, int64_t max_iter, double inner_tol,
                     int32_t max_outer) {
  if (!op) return fail(nullptr, HODLR_ERR_INVALID, "hodlr_set_solver: null argument");
  if (restart < 0 || restart > 1000) return fail(op->ctx, HODLR_ERR_INVALID, "hodlr_set_solver: restart in 0..1000");
  return guarded(op->ctx, [&]() -> int {
    CK(cudaSetDevice(op->p.device));
    op->p.restart = restart;
    op->p.tol = tol;
    op->p.max_iter = max_iter;
    op->p.inner_tol = inner_tol;
    op->p.max_outer = max_outer;
    const int r = restart > 0 ? restart : 100;
    if (op->p.precision == HODLR_PREC_MIXED) {
      if (r > op->g32.restart) CK(gmres_alloc<float>(op->g32, op->n, r));
    } else if (r > op->g64.restart) {
      CK(gmres_alloc<double>(op->g64, op->n, r));
    }
    return HODLR_OK;
  });
}

int hodlr_stats_get(const hodlr_op* op, hodlr_stats* out) {
  if (!op || !out) return fail(nullptr, HODLR_ERR_INVALID, "hodlr_stats_get: null argument");
  *out = op->st;
  return HODLR_OK;
}

int hodlr_get_permutation(const hodlr_op* op, int64_t* perm) {
  if (!op || !perm) return fail(nullptr, HODLR_ERR_INVALID, "hodlr_get_permutation: null argument");
  std::memcpy(perm, op->tree.perm.data(), sizeof(int64_t) * size_t(op->n));
  return HODLR_OK;
}

int hodlr_get_blocks(const hodlr_op* op, int32_t* level, int64_t* target, int64_t* source, int32_t* rank) {
  if (!op) return fail(nullptr, HODLR_ERR_INVALID, "hodlr_get_blocks: null argument");
  for (size_t b = 0; b < op->far.size(); b++) {
    if (level) level[b] = op->far[b].level;
    if (target) target[b] = op->far[b].t;
    if (source) source[b] = op->far[b].s;
    if (rank) rank[b] = op->rank[b];
  }
  return HODLR_OK;
}

int hodlr_get_block(const hodlr_op* op, int64_t b, int32_t* m, int32_t* n, int32_t* rank, int32_t* dense, double* U,
                    double* V) {
  if (!op) return fail(nullptr, HODLR_ERR_INVALID, "hodlr_get_block: null argument");
  if (b < 0 || b >= int64_t(op->far.size())) return fail(op->ctx, HODLR_ERR_INVALID, "hodlr_get_block: no such block");
  return guarded(op->ctx, [&]() -> int {
    const Tree& t = op->tree;
    const int32_t mm = int32_t(t.count[size_t(t.gid(op->far[b].level, op->far[b].t))]);
    const int32_t nn = int32_t(t.count[size_t(t.gid(op->far[b].level, op->far[b].s))]);
    if (m) *m = mm;
    if (n) *n = nn;
    if (rank) *rank = op->rank[size_t(b)];
    if (dense) *dense = op->dense[size_t(b)];
    const Prec fp = far_prec(op->p);
    const int esz = prec_size(fp);
    // stored values (FP64, FP32 or BF16 bits) of `count` elements as doubles
    auto to_double = [&](const void* src, size_t count) {
      std::vector<double> out(count);
      if (fp == Prec::kD) {
        CK(cudaMemcpy(out.data(), src, count * 8, cudaMemcpyDeviceToHost));
      } else if (fp == Prec::kF) {
        std::vector<float> t32(count);
        CK(cudaMemcpy(t32.data(), src, count * 4, cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < count; i++) out[i] = double(t32[i]);
      } else {
        std::vector<uint16_t> t16(count);
        CK(cudaMemcpy(t16.data(), src, count * 2, cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < count; i++) {
          const uint32_t bits = uint32_t(t16[i]) << 16;
          float f;
          std::memcpy(&f, &bits, 4);
          out[i] = double(f);
        }
      }
      return out;
    };
    auto scales = [&](const void* at, size_t count) {
      std::vector<float> s(count);
      CK(cudaMemcpy(s.data(), at, count * 4, cudaMemcpyDeviceToHost));
      return s;
    };
    // copy a stored rows x cols matrix (tiled layout, matvec.h) to a dense column-major dst
    auto fetch = [&](const void* src, size_t rows, size_t cols, double* dst) {
      if (!dst || !src || rows * cols == 0) return;
      const std::vector<double> tmp = to_double(src, size_t(stored_elems(int64_t(rows), int64_t(cols), esz)));
      for (size_t c = 0; c < cols; c++)
        for (size_t r = 0; r < rows; r++)
          dst[c * rows + r] = tmp[size_t(elem_offset(int64_t(r), int64_t(c), int64_t(rows), int64_t(cols), esz))];
    };
    CK(cudaSetDevice(op->p.device));
    CK(cudaStreamSynchronize(op->ctx->stream));
    const char* ub = static_cast<const char*>(op->uptr[size_t(b)]);
    if (op->dense[size_t(b)]) {
      fetch(ub, size_t(mm), size_t(nn), U);
      if (U && ub && fp == Prec::kB) {  // BF16: A = A' diag(column scales)
        const std::vector<float> cs = scales(ub + far_u_data_bytes(mm, nn, 0, true, fp), size_t(nn));
        for (size_t c = 0; c < size_t(nn); c++)
          for (size_t r = 0; r < size_t(mm); r++) U[c * size_t(mm) + r] *= double(cs[c]);
      }
    } else {
      const size_t r = size_t(std::max(op->rank[size_t(b)], 0));
      fetch(ub, size_t(mm), r, U);
      const char* vb = static_cast<const char*>(op->vptr[size_t(b)]);
      if (U && vb && r > 0 && fp == Prec::kB) {  // BF16: U V^T = U' diag(z scales) V'^T
        const char* zsb = op->zsptr.empty() || !op->zsptr[size_t(b)]
                              ? vb + far_v_data_bytes(nn, int64_t(r), false, fp)
                              : reinterpret_cast<const char*>(op->zsptr[size_t(b)]);
        const std::vector<float> zs = scales(zsb, r);
        for (size_t k = 0; k < r; k++)
          for (size_t i = 0; i < size_t(mm); i++) U[k * size_t(mm) + i] *= double(zs[k]);
      }
      if (V && vb && r > 0) {  // V is row major, nn x vpad(r), rows `stride` elements apart
        const size_t rp = size_t(vpad(int64_t(r), esz));
        const size_t stride = op->vstride.empty() || op->vstride[size_t(b)] == 0 ? rp : size_t(op->vstride[size_t(b)]);
        const std::vector<double> tmp = to_double(vb, (size_t(nn) - 1) * stride + rp);
        for (size_t k = 0; k < r; k++)
          for (size_t j = 0; j < size_t(nn); j++) V[k * size_t(nn) + j] = tmp[j * stride + k];
      }
    }
    return HODLR_OK;
  });
}

int hodlr_trace_enable(hodlr_op* op, int on) {
  if (!op) return fail(nullptr, HODLR_ERR_INVALID, "hodlr_trace_enable: null argument");
  return guarded(op->ctx, [&]() -> int {
    if (on) op->tr.reset();
    op->tr.on = on != 0;
    return HODLR_OK;
  });
}

int hodlr_trace_get(hodlr_op* op, hodlr_trace* out) {
  if (!op || !out) return fail(nullptr, HODLR_ERR_INVALID, "hodlr_trace_get: null argument");
  return guarded(op->ctx, [&]() -> int {
    CK(cudaSetDevice(op->p.device));
    op->tr.harvest();
    for (int k = 0; k < HODLR_TRACE_KINDS; k++) {
      out->launches[k] = op->tr.launches[k];
      out->total_ms[k] = op->tr.ms[k];
      out->bytes_per_launch[k] = op->tr.bytes[k];
    }
    return HODLR_OK;
  });
}

uint64_t hodlr_kernel_launches(void) { return g_kernel_launches.load(); }

// ---------------------------------------------------------------- host-only tree

struct hodlr_tree {
  Tree t;
  std::vector<FarBlock> far;
  NearList near;
};

int hodlr_tree_build(const hodlr_params* params, const double* points, int64_t n, const double* box_lo,
                     const double* box_hi, hodlr_tree** out) {
  if (!params || !points || !box_lo || !box_hi || !out)
    return fail(nullptr, HODLR_ERR_INVALID, "hodlr_tree_build: null argument");
  *out = nullptr;
  try {
    std::unique_ptr<hodlr_tree> tr(new hodlr_tree());
    TreeParams tp;
    tp.ndim = params->ndim;
    tp.nmax = params->nmax;
    tp.dprime = params->dprime;
    const std::string err = build_tree(tp, points, n, box_lo, box_hi, tr->t);
    if (!err.empty())
      return fail(nullptr, err.find("exceeds") != std::string::npos ? HODLR_ERR_TREE : HODLR_ERR_INVALID,
                  "hodlr_tree_build: " + err);
    tr->far = far_blocks(tr->t);
    tr->near = near_blocks(tr->t);
    *out = tr.release();
    return HODLR_OK;
  } catch (const std::exception& e) {
    return fail(nullptr, HODLR_ERR_INVALID, e.what());
  }
}

int hodlr_tree_build_device(const hodlr_params* params, const double* points, int64_t n, const double* box_lo,
                            const double* box_hi, hodlr_tree** out) {
  if (!params || !points || !box_lo || !box_hi || !out)
    return fail(nullptr, HODLR_ERR_INVALID, "hodlr_tree_build_device: null argument");
  *out = nullptr;
  cudaStream_t st = nullptr;
  try {
    check_cuda(cudaSetDevice(params->device), "cudaSetDevice");
    check_cuda(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
    std::unique_ptr<hodlr_tree> tr(new hodlr_tree());
    TreeParams tp;
    tp.ndim = params->ndim;
    tp.nmax = params->nmax;
    tp.dprime = params->dprime;
    DeviceTreeOut dto;  // the host arrays only
    const DeviceTreeStatus ds = build_tree_device(tp, points, n, box_lo, box_hi, tr->t, dto, st);
    cudaStreamDestroy(st);
    st = nullptr;
    if (ds.code != 0) return fail(nullptr, ds.code, "hodlr_tree_build_device: " + ds.msg);
    tr->far = far_blocks(tr->t);
    tr->near = near_blocks(tr->t);
    *out = tr.release();
    return HODLR_OK;
  } catch (const Failure& f) {
    if (st) cudaStreamDestroy(st);
    return fail(nullptr, f.code, "hodlr_tree_build_device: " + f.msg);
  } catch (const std::exception& e) {
    if (st) cudaStreamDestroy(st);
    return fail(nullptr, HODLR_ERR_INVALID, e.what());
  }
}

int hodlr_tree_sizes(const hodlr_tree* tr, int64_t* sizes) {
  if (!tr || !sizes) return fail(nullptr, HODLR_ERR_INVALID, "hodlr_tree_sizes: null argument");
  sizes[0] = tr->t.levels;
  sizes[1] = tr->t.level_off.back();
  sizes[2] = int64_t(tr->t.nbr.size());
  sizes[3] = int64_t(tr->t.intr.size());
  sizes[4] = int64_t(tr->far.size());
  sizes[5] = int64_t(tr->near.src.size());
  return HODLR_OK;
}

int hodlr_tree_get(const hodlr_tree* tr, int64_t* level_sizes, int64_t* node_counts, int64_t* nbr_ptr, int64_t* nbr,
                   int64_t* intr_ptr, int64_t* intr, int64_t* leaf_perm) {
  if (!tr) return fail(nullptr, HODLR_ERR_INVALID, "hodlr_tree_get: null argument");
  const Tree& t = tr->t;
  if (level_sizes) std::copy(t.level_size.begin(), t.level_size.end(), level_sizes);
  if (node_counts) std::copy(t.count.begin(), t.count.end(), node_counts);
  if (nbr_ptr) std::copy(t.nbr_ptr.begin(), t.nbr_ptr.end(), nbr_ptr);
  if (nbr) std::copy(t.nbr.begin(), t.nbr.end(), nbr);
  if (intr_ptr) std::copy(t.intr_ptr.begin(), t.intr_ptr.end(), intr_ptr);
  if (intr) std::copy(t.intr.begin(), t.intr.end(), intr);
  if (leaf_perm) std::copy(t.perm.begin(), t.perm.end(), leaf_perm);
  return HODLR_OK;
}

int hodlr_tree_destroy(hodlr_tree* tr) {
  delete tr;
  return HODLR_OK;
}


int hodlr_build_batch(hodlr_ctx* ctx, int32_t count, const double* const* points, const int64_t* n,
                      const double* box_lo, const double* box_hi, const hodlr_kernel_desc* kernels,
                      hodlr_batch** out) {
  if (!ctx || !points || !n || !box_lo || !box_hi || !kernels || !out)
    return fail(ctx, HODLR_ERR_INVALID, "hodlr_build_batch: null argument");
  *out = nullptr;
  if (count < 1) return fail(ctx, HODLR_ERR_INVALID, "hodlr_build_batch: count must be positive");
  for (int32_t i = 0; i < count; i++) {
    if (!points[i] || n[i] < 1 || n[i] > (int64_t(1) << 31) - 1)
      return fail(ctx, HODLR_ERR_INVALID, "hodlr_build_batch: instance " + std::to_string(i) + ": bad points or n");
    if (kernels[i].kind != kernels[0].kind || kernels[i].diag != kernels[0].diag || kernels[i].scale == 0.0)
      return fail(ctx, HODLR_ERR_INVALID,
                  "hodlr_build_batch: instances must share the kernel kind and diagonal and have nonzero scales");
  }
  if (kernels[0].kind < HODLR_KERNEL_INV_R || kernels[0].kind > HODLR_KERNEL_EXP_NEG_R)
    return fail(ctx, HODLR_ERR_INVALID, "hodlr_build_batch: unknown kernel kind");
  if (ctx->p.precision == HODLR_PREC_BF16_FACTORS)
    return fail(ctx, HODLR_ERR_INVALID, "hodlr_build_batch: batches store FP64 or FP32 factors");
  std::unique_ptr<hodlr_batch> b(new hodlr_batch());
  b->ctx = ctx;
  b->vec = ctx->p.precision == HODLR_PREC_MIXED ? Prec::kF : Prec::kD;
  b->df = ctx->p.precision == HODLR_PREC_FP32_FACTORS;
  return guarded(ctx, [&]() -> int {
    CK(cudaSetDevice(ctx->p.device));
    cudaStream_t st = ctx->stream;
    const int d = ctx->p.ndim;
    std::vector<BuildState> bs(static_cast<size_t>(count));
    for (int32_t i = 0; i < count; i++) {
      hodlr_op* op = new hodlr_op();
      b->ops.push_back(op);
      op->ctx = ctx;
      op->p = ctx->p;
      op->has_ref = wants_ref(op->p);
      op->kd = kernels[i];
      op->n = n[i];
      op->keep_host_plans = true;
      op->batch_owned = true;
      std::memset(&op->st, 0, sizeof(op->st));
    }
    CK(cudaStreamSynchronize(st));
    for_each_instance(count, ctx->p.device, [&](int i, cudaStream_t s) {
      build_prepare(b->ops[size_t(i)], points[i], box_lo + size_t(i) * d, box_hi + size_t(i) * d, s, bs[size_t(i)]);
    });
    const double ta = now_s();
    run_aca(b->ops, st);
    const double t_aca = now_s() - ta;
    CK(cudaStreamSynchronize(st));
    for_each_instance(count, ctx->p.device, [&](int i, cudaStream_t s) {
      b->ops[size_t(i)]->st.t_aca_s = t_aca;
      build_finish(b->ops[size_t(i)], bs[size_t(i)], s);
    });
    build_batch_plan(*b, st);
    *out = b.release();
    return HODLR_OK;
  });
}

int hodlr_batch_offsets(const hodlr_batch* b, int64_t* offsets) {
  if (!b || !offsets) return fail(nullptr, HODLR_ERR_INVALID, "hodlr_batch_offsets: null argument");
  std::copy(b->offsets.begin(), b->offsets.end(), offsets);
  return HODLR_OK;
}

int hodlr_batch_op(hodlr_batch* b, int32_t i, hodlr_op** op) {
  if (!b || !op) return fail(nullptr, HODLR_ERR_INVALID, "hodlr_batch_op: null argument");
  if (i < 0 || i >= int32_t(b->ops.size())) return fail(b->ctx, HODLR_ERR_INVALID, "hodlr_batch_op: index out of range");
  *op = b->ops[size_t(i)];
  return HODLR_OK;
}

int hodlr_batch_matvec_device(hodlr_batch* b, const void* d_x, void* d_y, int64_t nrhs, void* stream) {
  if (!b || !d_x || !d_y) return fail(b ? b->ctx : nullptr, HODLR_ERR_INVALID, "hodlr_batch_matvec_device: null argument");
  if (nrhs < 1) return fail(b->ctx, HODLR_ERR_INVALID, "hodlr_batch_matvec_device: nrhs must be positive");
  return guarded(b->ctx, [&]() -> int {
    CK(cudaSetDevice(b->ctx->p.device));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    hodlr_batch::Graph* g = nullptr;
    for (hodlr_batch::Graph& q : b->graphs)
      if (q.x == d_x && q.y == d_y && q.nrhs == nrhs) g = &q;
    if (!g) {
      // capture every column's launch sequence once on the batch's own stream
      const size_t vsz = b->vec == Prec::kF ? 4 : 8;
      cudaStream_t cs = b->ctx->stream;
      if (b->vec == Prec::kF) ensure_mr_buffers(*b, int((nrhs + kMR - 1) / kMR));
      CK(cudaStreamSynchronize(cs));
      const uint64_t k0 = g_kernel_launches.load();
      hodlr_batch::Graph ng{d_x, d_y, nrhs, nullptr, nullptr, 0};
      CK(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
      try {
        if (b->vec == Prec::kF) {
          batch_apply_mr(*b, static_cast<const float*>(d_x), static_cast<float*>(d_y), nrhs, cs);
        } else {
          for (int64_t c = 0; c < nrhs; c++)
            batch_apply(*b, static_cast<const char*>(d_x) + size_t(c * b->total_n) * vsz,
                        static_cast<char*>(d_y) + size_t(c * b->total_n) * vsz, cs);
        }
      } catch (...) {
        cudaGraph_t dead = nullptr;
        cudaStreamEndCapture(cs, &dead);
        if (dead) cudaGraphDestroy(dead);
        throw;
      }
      CK(cudaStreamEndCapture(cs, &ng.graph));
      ng.kernels = g_kernel_launches.load() - k0;
      CK(cudaGraphInstantiate(&ng.exec, ng.graph, 0));
      b->graphs.push_back(ng);
      g = &b->graphs.back();
    } else {
      count_launches(g->kernels);
    }
    CK(cudaGraphLaunch(g->exec, st));
    return HODLR_OK;
  });
}

int hodlr_batch_destroy(hodlr_batch* b) {
  if (!b) return HODLR_OK;
  cudaSetDevice(b->ctx->p.device);
  cudaStreamSynchronize(b->ctx->stream);
  delete b;
  return HODLR_OK;
}


// ---- operator files ----------------------------------------------------------
// Layout (host byte order): magic "HODLRGB\0", u32 version, hodlr_params,
// hodlr_kernel_desc, i64 n, the n x ndim points (caller order), the box
// (2 x ndim), i64 far-block count, per block i32 rank and i32 dense, then per
// block its stored U (or dense tile) and V bytes, in far-block order, each as
// the engine stores them (FP64, FP32 or BF16 with its scales).  Loading
// rebuilds the tree, lists and near field from the points (deterministic) and
// takes the far field from the file instead of running ACA.
namespace {
constexpr char kOpMagic[8] = {'H', 'O', 'D', 'L', 'R', 'G', 'B', 0};
constexpr uint32_t kOpVersion = 2;  // 2: hodlr_params with fp64_check, the FP64 factors of the check

struct OpFile {
  std::FILE* f = nullptr;
  ~OpFile() {
    if (f) std::fclose(f);
  }
};

uint64_t block_u_bytes(int64_t m, int64_t n, int32_t rank, int32_t dense, Prec p) {
  return far_u_bytes(m, n, rank, dense != 0, p);
}
uint64_t block_v_bytes(int64_t n, int32_t rank, int32_t dense, Prec p) { return far_v_bytes(n, rank, dense != 0, p); }
}  // namespace

int hodlr_op_save(const hodlr_op* op, const double* points, const char* path) {
  if (!op || !points || !path) return fail(op ? op->ctx : nullptr, HODLR_ERR_INVALID, "hodlr_op_save: null argument");
  return guarded(op->ctx, [&]() -> int {
    CK(cudaSetDevice(op->p.device));
    OpFile fh;
    fh.f = std::fopen(path, "wb");
    if (!fh.f) throw Failure{HODLR_ERR_IO, std::string("hodlr_op_save: cannot create ") + path};
    auto put = [&](const void* p, size_t bytes) {
      if (bytes && std::fwrite(p, 1, bytes, fh.f) != bytes)
        throw Failure{HODLR_ERR_IO, std::string("hodlr_op_save: write failed: ") + path};
    };
    const int d = op->p.ndim;
    put(kOpMagic, 8);
    put(&kOpVersion, 4);
    put(&op->p, sizeof(op->p));
    put(&op->kd, sizeof(op->kd));
    put(&op->n, 8);
    put(points, sizeof(double) * size_t(op->n) * size_t(d));
    put(op->box_lo.data(), sizeof(double) * size_t(d));
    put(op->box_hi.data(), sizeof(double) * size_t(d));
    const int64_t nb = int64_t(op->far.size());
    put(&nb, 8);
    put(op->rank.data(), 4 * size_t(nb));
    put(op->dense.data(), 4 * size_t(nb));
    const Prec esz = far_prec(op->p);
    const Tree& t = op->tree;
    std::vector<char> buf;
    for (int64_t q = 0; q < nb; q++) {
      const FarBlock& fb = op->far[size_t(q)];
      const int64_t m = t.count[size_t(t.gid(fb.level, fb.t))], n = t.count[size_t(t.gid(fb.level, fb.s))];
      const int32_t r = op->rank[size_t(q)], dn = op->dense[size_t(q)];
      if (!dn && r <= 0) continue;
      const uint64_t bu = block_u_bytes(m, n, r, dn, esz), bv = block_v_bytes(n, r, dn, esz);
      buf.assign(bu + bv, 0);
      CK(cudaMemcpy(buf.data(), op->uptr[size_t(q)], bu, cudaMemcpyDeviceToHost));
      const int64_t stride = op->vstride.empty() ? 0 : op->vstride[size_t(q)];
      if (bv && stride == 0) {
        CK(cudaMemcpy(buf.data() + bu, op->vptr[size_t(q)], bv, cudaMemcpyDeviceToHost));
      } else if (bv) {  // a block of a source chunk: its rows, then (BF16) its z scales
        const int es = prec_size(esz);
        const size_t row = size_t(vpad(r, es)) * size_t(es);
        CK(cudaMemcpy2D(buf.data() + bu, row, op->vptr[size_t(q)], size_t(stride) * size_t(es), row, size_t(n),
                        cudaMemcpyDeviceToHost));
        if (esz == Prec::kB)
          CK(cudaMemcpy(buf.data() + bu + far_v_data_bytes(n, r, false, esz), op->zsptr[size_t(q)],
                        size_t(r) * 4, cudaMemcpyDeviceToHost));
      }
      put(buf.data(), bu + bv);
    }
    if (op->has_ref)  // the FP64 factors of the FP64 check, in the same order
      for (int64_t q = 0; q < nb; q++) {
        const FarBlock& fb = op->far[size_t(q)];
        const int64_t m = t.count[size_t(t.gid(fb.level, fb.t))], n = t.count[size_t(t.gid(fb.level, fb.s))];
        const int32_t r = op->rank[size_t(q)], dn = op->dense[size_t(q)];
        if (!dn && r <= 0) continue;
        const uint64_t bu = block_u_bytes(m, n, r, dn, Prec::kD), bv = block_v_bytes(n, r, dn, Prec::kD);
        buf.resize(bu + bv);
        CK(cudaMemcpy(buf.data(), op->uptr64[size_t(q)], bu, cudaMemcpyDeviceToHost));
        if (bv) CK(cudaMemcpy(buf.data() + bu, op->vptr64[size_t(q)], bv, cudaMemcpyDeviceToHost));
        put(buf.data(), bu + bv);
      }
    if (std::fflush(fh.f) != 0) throw Failure{HODLR_ERR_IO, std::string("hodlr_op_save: write failed: ") + path};
    return HODLR_OK;
  });
}

int hodlr_op_load(hodlr_ctx* ctx, const char* path, hodlr_op** out) {
  if (!ctx || !path || !out) return fail(ctx, HODLR_ERR_INVALID, "hodlr_op_load: null argument");
  *out = nullptr;
  std::unique_ptr<hodlr_op> op(new hodlr_op());
  return guarded(ctx, [&]() -> int {
    CK(cudaSetDevice(ctx->p.device));
    cudaStream_t st = ctx->stream;
    OpFile fh;
    fh.f = std::fopen(path, "rb");
    if (!fh.f) throw Failure{HODLR_ERR_IO, std::string("hodlr_op_load: cannot open ") + path};
    auto get = [&](void* p, size_t bytes) {
      if (bytes && std::fread(p, 1, bytes, fh.f) != bytes)
        throw Failure{HODLR_ERR_IO, std::string("hodlr_op_load: truncated file: ") + path};
    };
    char magic[8];
    uint32_t version = 0;
    get(magic, 8);
    get(&version, 4);
    if (std::memcmp(magic, kOpMagic, 8) != 0 || version != kOpVersion)
      throw Failure{HODLR_ERR_IO, std::string("hodlr_op_load: not an operator file of this version: ") + path};
    op->ctx = ctx;
    get(&op->p, sizeof(op->p));
    get(&op->kd, sizeof(op->kd));
    get(&op->n, 8);
    op->p.device = ctx->p.device;
    op->mem.budget = ctx->p.device_budget_bytes;
    const int d = op->p.ndim;
    const char* why = params_problem(op->p);
    if (why || op->n < 1 || op->n > (int64_t(1) << 31) - 1 || op->kd.kind < HODLR_KERNEL_INV_R ||
        op->kd.kind > HODLR_KERNEL_EXP_NEG_R || !std::isfinite(op->kd.scale) || !std::isfinite(op->kd.diag))
      throw Failure{HODLR_ERR_IO, std::string("hodlr_op_load: corrupt header (") +
                                      (why ? why : "point count or kernel out of range") + "): " + path};
    op->keep_host_plans = op->p.precision == HODLR_PREC_BF16_FACTORS;  // for the tensor-core plan
    std::memset(&op->st, 0, sizeof(op->st));
    std::vector<double> pts(size_t(op->n) * size_t(d)), lo(static_cast<size_t>(d)), hi(static_cast<size_t>(d));
    get(pts.data(), sizeof(double) * pts.size());
    get(lo.data(), sizeof(double) * size_t(d));
    get(hi.data(), sizeof(double) * size_t(d));
    BuildState bs;
    build_prepare(op.get(), pts.data(), lo.data(), hi.data(), st, bs);
    int64_t nb = 0;
    get(&nb, 8);
    if (nb != int64_t(op->far.size()))
      throw Failure{HODLR_ERR_IO, std::string("hodlr_op_load: far-block count does not match the tree: ") + path};
    op->rank.assign(size_t(nb), 0);
    op->dense.assign(size_t(nb), 0);
    get(op->rank.data(), 4 * size_t(nb));
    get(op->dense.data(), 4 * size_t(nb));
    const Prec esz = far_prec(op->p);
    const Tree& t = op->tree;
    // one chunk in the compaction layout (each block's U then V, 16-byte aligned)
    std::vector<uint64_t> off(size_t(nb), 0);
    uint64_t total = 0;
    for (int64_t q = 0; q < nb; q++) {
      const FarBlock& fb = op->far[size_t(q)];
      const int64_t m = t.count[size_t(t.gid(fb.level, fb.t))], n = t.count[size_t(t.gid(fb.level, fb.s))];
      const int32_t r = op->rank[size_t(q)], dn = op->dense[size_t(q)];
      if (r < 0 || r > std::min(m, n) || (dn != 0 && dn != 1))
        throw Failure{HODLR_ERR_IO, std::string("hodlr_op_load: corrupt block table: ") + path};
      off[size_t(q)] = total;
      if (!dn && r <= 0) continue;
      total += block_u_bytes(m, n, r, dn, esz) + block_v_bytes(n, r, dn, esz);
    }
    std::vector<char> host(std::max<uint64_t>(total, 16), 0);
    op->uptr.assign(size_t(nb), nullptr);
    op->vptr.assign(size_t(nb), nullptr);
    char* chunk = static_cast<char*>(op->mem.alloc(std::max<uint64_t>(total, 16), "far-field factors"));
    op->far_chunks.push_back(chunk);
    for (int64_t q = 0; q < nb; q++) {
      const FarBlock& fb = op->far[size_t(q)];
      const int64_t m = t.count[size_t(t.gid(fb.level, fb.t))], n = t.count[size_t(t.gid(fb.level, fb.s))];
      const int32_t r = op->rank[size_t(q)], dn = op->dense[size_t(q)];
      if (!dn && r <= 0) continue;
      const uint64_t bu = block_u_bytes(m, n, r, dn, esz), bv = block_v_bytes(n, r, dn, esz);
      const uint64_t vo = off[size_t(q)] + bu;
      get(host.data() + off[size_t(q)], bu);
      if (bv) get(host.data() + vo, bv);
      op->uptr[size_t(q)] = chunk + off[size_t(q)];
      op->vptr[size_t(q)] = dn ? nullptr : chunk + vo;
    }
    CK(cudaMemcpyAsync(chunk, host.data(), std::max<uint64_t>(total, 16), cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));
    op->has_ref = wants_ref(op->p);
    if (op->has_ref) {  // the FP64 factors of the FP64 check
      uint64_t total64 = 0;
      std::vector<uint64_t> off64(size_t(nb), 0);
      for (int64_t q = 0; q < nb; q++) {
        const FarBlock& fb = op->far[size_t(q)];
        const int64_t m = t.count[size_t(t.gid(fb.level, fb.t))], n = t.count[size_t(t.gid(fb.level, fb.s))];
        const int32_t r = op->rank[size_t(q)], dn = op->dense[size_t(q)];
        off64[size_t(q)] = total64;
        if (!dn && r <= 0) continue;
        total64 += block_u_bytes(m, n, r, dn, Prec::kD) + block_v_bytes(n, r, dn, Prec::kD);
      }
      std::vector<char> h64(std::max<uint64_t>(total64, 16), 0);
      char* c64 = static_cast<char*>(op->mem.alloc(std::max<uint64_t>(total64, 16), "far-field factors (FP64 reference)"));
      op->uptr64.assign(size_t(nb), nullptr);
      op->vptr64.assign(size_t(nb), nullptr);
      for (int64_t q = 0; q < nb; q++) {
        const FarBlock& fb = op->far[size_t(q)];
        const int64_t m = t.count[size_t(t.gid(fb.level, fb.t))], n = t.count[size_t(t.gid(fb.level, fb.s))];
        const int32_t r = op->rank[size_t(q)], dn = op->dense[size_t(q)];
        if (!dn && r <= 0) continue;
        const uint64_t bu = block_u_bytes(m, n, r, dn, Prec::kD), bv = block_v_bytes(n, r, dn, Prec::kD);
        get(h64.data() + off64[size_t(q)], bu + bv);
        op->uptr64[size_t(q)] = c64 + off64[size_t(q)];
        op->vptr64[size_t(q)] = dn ? nullptr : c64 + off64[size_t(q)] + bu;
      }
      CK(cudaMemcpyAsync(c64, h64.data(), std::max<uint64_t>(total64, 16), cudaMemcpyHostToDevice, st));
      CK(cudaStreamSynchronize(st));
    }
    char extra;
    if (std::fread(&extra, 1, 1, fh.f) == 1)
      throw Failure{HODLR_ERR_IO, std::string("hodlr_op_load: trailing bytes: ") + path};
    op->st.t_aca_s = 0.0;
    build_finish(op.get(), bs, st);
    *out = op.release();
    return HODLR_OK;
  });
}

}  // extern "C"
