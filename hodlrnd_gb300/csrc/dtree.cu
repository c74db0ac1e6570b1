// The 2^d tree and its interaction lists on the device (see dtree.h).
#include "dtree.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/hodlrnd.h"
#include "device.cuh"

namespace hodlr {
namespace {

constexpr int kSplitThreads = 512;
constexpr int kSplitWarps = kSplitThreads / 32;
constexpr int kMaxFan = 1 << kMaxDim;  // 256

struct CudaError {
  cudaError_t e;
  const char* what;
};
void ck(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw CudaError{e, what};
}

// Temporary device buffers of one build, freed when it returns.
struct Scratch {
  std::vector<void*> ptrs;
  template <typename T>
  T* alloc(size_t n, const char* what) {
    void* p = nullptr;
    ck(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)), what);
    ptrs.push_back(p);
    return static_cast<T*>(p);
  }
  ~Scratch() {
    for (void* p : ptrs) cudaFree(p);
  }
};

// Child boxes of a level (cluster ctor + compute_cluster_center,
// HDD_clusters.hpp:25-37,70-79; children halve the parent at its midpoint,
// dimension 0 the most significant bit of the child index).  One thread per
// child; every operation rounds once, in the host's order.
__global__ void child_boxes_kernel(int d, int fan, int64_t C, const double* __restrict__ plo,
                                   const double* __restrict__ phi, double* __restrict__ lo, double* __restrict__ hi,
                                   double* __restrict__ center, double* __restrict__ L) {
  const int64_t g = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (g >= C) return;
  const int64_t p = g / fan;
  const int c = int(g % fan);
  double Lv = 0.0;
  for (int k = 0; k < d; k++) {
    const double a = plo[p * d + k], b = phi[p * d + k];
    const double mid = __dmul_rn(0.5, __dadd_rn(a, b));
    const bool upper = (c >> (d - 1 - k)) & 1;
    const double l = upper ? mid : a, h = upper ? b : mid;
    lo[g * d + k] = l;
    hi[g * d + k] = h;
    center[g * d + k] = __dmul_rn(0.5, __dadd_rn(l, h));
    const double side = fabs(__dsub_rn(l, h));
    if (k == 0 || side > Lv) Lv = side;
  }
  L[g] = Lv;
}

// Stable partition of each parent's points among its children (one CTA per
// parent): pass 1 counts the points per child and writes the children's
// ranges; pass 2 moves the points, tile by tile, to their child's range in
// their current order (lanes of equal child ranked by __match_any_sync,
// warps in order, tiles in order).  x < mid goes to the lower half
// (HDD_clusters.hpp:124-127).
__global__ void __launch_bounds__(kSplitThreads) split_kernel(int d, int fan, const double* __restrict__ pts,
                                                              const int64_t* __restrict__ pbegin,
                                                              const int64_t* __restrict__ pcount,
                                                              const double* __restrict__ plo,
                                                              const double* __restrict__ phi,
                                                              const int32_t* __restrict__ perm_in,
                                                              int32_t* __restrict__ perm_out,
                                                              int64_t* __restrict__ cbegin,
                                                              int64_t* __restrict__ ccount,
                                                              unsigned long long* __restrict__ maxc) {
  __shared__ int cnt[kMaxFan];
  __shared__ int run[kMaxFan];
  __shared__ int wcnt[kSplitWarps][kMaxFan];
  const int64_t p = blockIdx.x;
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int64_t b = pbegin[p], e = b + pcount[p];
  double mid[kMaxDim];
  for (int k = 0; k < d; k++) mid[k] = __dmul_rn(0.5, __dadd_rn(plo[p * d + k], phi[p * d + k]));
  auto child = [&](int64_t i) {
    const double* x = pts + int64_t(perm_in[i]) * d;
    int c = 0;
    for (int k = 0; k < d; k++) c = (c << 1) | (x[k] < mid[k] ? 0 : 1);
    return c;
  };
  for (int c = t; c < fan; c += kSplitThreads) cnt[c] = 0;
  for (int q = t; q < kSplitWarps * fan; q += kSplitThreads) wcnt[q / fan][q % fan] = 0;
  __syncthreads();
  for (int64_t i = b + t; i < e; i += kSplitThreads) atomicAdd(&cnt[child(i)], 1);
  __syncthreads();
  if (t == 0) {
    int acc = 0;
    unsigned long long mx = 0;
    for (int c = 0; c < fan; c++) {
      run[c] = acc;
      cbegin[p * fan + c] = b + acc;
      ccount[p * fan + c] = cnt[c];
      mx = max(mx, (unsigned long long)cnt[c]);
      acc += cnt[c];
    }
    atomicMax(maxc, mx);
  }
  __syncthreads();
  const unsigned lt = (1u << lane) - 1u;
  for (int64_t base = b; base < e; base += kSplitThreads) {
    const int64_t i = base + t;
    const bool valid = i < e;
    const int c = valid ? child(i) : 0x10000 + lane;  // invalid lanes: keys of their own
    const unsigned same = __match_any_sync(0xffffffffu, c);
    const int rank = __popc(same & lt);
    if (valid && rank == 0) wcnt[warp][c] = __popc(same);
    __syncthreads();
    if (valid) {
      int off = run[c] + rank;
      for (int w = 0; w < warp; w++) off += wcnt[w][c];
      perm_out[b + off] = perm_in[i];
    }
    __syncthreads();
    for (int cc = t; cc < fan; cc += kSplitThreads) {
      int tot = 0;
      for (int w = 0; w < kSplitWarps; w++) {
        tot += wcnt[w][cc];
        wcnt[w][cc] = 0;
      }
      run[cc] += tot;
    }
    __syncthreads();
  }
}

// interaction_type (HDD_clusters.hpp:142-162) and Node::is_admissible
// (HDD_node.hpp:24-31) as tree.cpp evaluates them, one rounding per operation.
__device__ bool admissible(int d, int dprime, const double* __restrict__ center, const double* __restrict__ L,
                           int64_t me, int64_t other) {
  const double* ca = center + me * d;
  const double* cb = center + other * d;
  double dist = fabs(__dsub_rn(ca[0], cb[0]));
  for (int k = 0; k < d; k++) {
    const double v = fabs(__dsub_rn(ca[k], cb[k]));
    if (v > dist) dist = v;
  }
  if (dist < __dmul_rn(1.5, L[me])) {
    const double Lm = L[me] > L[other] ? L[me] : L[other];  // std::max(L[a], L[b])
    double e = 0.0;
    for (int k = 0; k < d; k++) {
      const double q = __dsub_rn(ca[k], cb[k]);
      e = __dadd_rn(e, __dmul_rn(q, q));
    }
    double dp = __ddiv_rn(__dsqrt_rn(e), Lm);
    dp = __dmul_rn(dp, dp);
    const int type = double(d) + 1 > dp ? int(double(d) - round(dp)) : -1;
    if (type > dprime) return false;
  }
  return true;
}

// Node::get_interaction_list (HDD_node.hpp:150-180) for every node k of the
// new level: its siblings, then the children of each of the parent's
// neighbours, in order; admissible pairs go to the interaction list, the rest
// to the neighbour list.  fill = false counts, fill = true writes at the
// scanned offsets.
template <bool kFill>
__global__ void lists_kernel(int d, int dprime, int fan, int64_t C, const double* __restrict__ center,
                             const double* __restrict__ L, const int64_t* __restrict__ pn_ptr,
                             const int64_t* __restrict__ pn, int64_t* __restrict__ nb_cnt_or_ptr,
                             int64_t* __restrict__ in_cnt_or_ptr, int64_t* __restrict__ nb,
                             int64_t* __restrict__ in) {
  const int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (k >= C) return;
  const int64_t pk = k / fan;
  int64_t qn = kFill ? nb_cnt_or_ptr[k] : 0, qi = kFill ? in_cnt_or_ptr[k] : 0;
  auto take = [&](int64_t o) {
    if (admissible(d, dprime, center, L, k, o)) {
      if (kFill) in[qi] = o;
      qi++;
    } else {
      if (kFill) nb[qn] = o;
      qn++;
    }
  };
  for (int c = 0; c < fan; c++) {
    const int64_t sib = pk * fan + c;
    if (sib != k) take(sib);
  }
  for (int64_t q = pn_ptr[pk]; q < pn_ptr[pk + 1]; q++)
    for (int c = 0; c < fan; c++) take(pn[q] * fan + c);
  if (!kFill) {
    nb_cnt_or_ptr[k] = qn;
    in_cnt_or_ptr[k] = qi;
  }
}

// Exclusive scan of n int64 counts into out[0..n] (out[n] = total), in place
// allowed: per 1024-element block a local scan and the block sum, one CTA
// scanning the block sums, then the block offsets added.
constexpr int kScanBlock = 1024;
__device__ int64_t block_incl_scan(int64_t v, int64_t* warp_tot) {
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t u = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += u;
  }
  if (lane == 31) warp_tot[w] = v;
  __syncthreads();
  if (w == 0) {
    int64_t s = lane < int(blockDim.x >> 5) ? warp_tot[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t u = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += u;
    }
    warp_tot[lane] = s;
  }
  __syncthreads();
  if (w > 0) v += warp_tot[w - 1];
  __syncthreads();
  return v;
}
__global__ void __launch_bounds__(kScanBlock) scan_blocks_kernel(const int64_t* __restrict__ in, int64_t n,
                                                                 int64_t* __restrict__ out, int64_t* __restrict__ sums) {
  __shared__ int64_t wt[32];
  const int64_t i = blockIdx.x * int64_t(kScanBlock) + threadIdx.x;
  const int64_t v = i < n ? in[i] : 0;
  const int64_t incl = block_incl_scan(v, wt);
  if (i < n) out[i] = incl - v;
  if (threadIdx.x == kScanBlock - 1) sums[blockIdx.x] = incl;
}
__global__ void __launch_bounds__(kScanBlock) scan_sums_kernel(int64_t* __restrict__ sums, int64_t nb,
                                                               int64_t* __restrict__ total) {
  __shared__ int64_t wt[32];
  int64_t carry = 0;
  for (int64_t base = 0; base < nb; base += kScanBlock) {
    const int64_t i = base + threadIdx.x;
    const int64_t v = i < nb ? sums[i] : 0;
    const int64_t incl = block_incl_scan(v, wt);
    if (i < nb) sums[i] = carry + incl - v;
    carry += wt[31];  // the tile's total (warp 0 scanned the 32 warp totals)
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}
__global__ void __launch_bounds__(kScanBlock) scan_add_kernel(int64_t* __restrict__ out, int64_t n,
                                                              const int64_t* __restrict__ sums) {
  const int64_t i = blockIdx.x * int64_t(kScanBlock) + threadIdx.x;
  if (i < n) out[i] += sums[blockIdx.x];
}

__global__ void gather_soa_kernel(int d, int64_t n, const double* __restrict__ pts, const int32_t* __restrict__ perm,
                                  double* __restrict__ soa, int64_t* __restrict__ perm64) {
  const int64_t q = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (q >= n) return;
  const int32_t i = perm[q];
  for (int k = 0; k < d; k++) soa[int64_t(k) * n + q] = pts[int64_t(i) * d + k];
  perm64[q] = i;
}
__global__ void inverse_kernel(int64_t n, const int32_t* __restrict__ perm, int32_t* __restrict__ inv) {
  const int64_t q = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (q < n) inv[perm[q]] = int32_t(q);
}
__global__ void lmap_kernel(int64_t n, const int32_t* __restrict__ perm_l, const int32_t* __restrict__ inv,
                            int32_t* __restrict__ out) {
  const int64_t j = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (j < n) out[j] = inv[perm_l[j]];
}

unsigned blocks_for(int64_t n, int t) { return unsigned((n + t - 1) / t); }

// out[0..n] = exclusive scan of cnt (out may alias cnt); returns the total.
int64_t scan(Scratch& s, const int64_t* cnt, int64_t n, int64_t* out, cudaStream_t st) {
  const int64_t nb = std::max<int64_t>(1, (n + kScanBlock - 1) / kScanBlock);
  int64_t* sums = s.alloc<int64_t>(size_t(nb), "tree scan");
  count_launches(3);
  scan_blocks_kernel<<<unsigned(nb), kScanBlock, 0, st>>>(cnt, n, out, sums);
  scan_sums_kernel<<<1, kScanBlock, 0, st>>>(sums, nb, out + n);
  scan_add_kernel<<<unsigned(nb), kScanBlock, 0, st>>>(out, n, sums);
  ck(cudaGetLastError(), "tree scan");
  int64_t total = 0;
  ck(cudaMemcpyAsync(&total, out + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st), "tree scan");
  ck(cudaStreamSynchronize(st), "tree scan");
  return total;
}

template <typename T>
void to_host(std::vector<T>& dst, size_t at, const T* src, size_t n, cudaStream_t st) {
  if (n == 0) return;
  if (dst.size() < at + n) dst.resize(at + n);
  ck(cudaMemcpyAsync(dst.data() + at, src, n * sizeof(T), cudaMemcpyDeviceToHost, st), "tree to host");
}

}  // namespace

DeviceTreeStatus build_tree_device(const TreeParams& p, const double* points, int64_t n, const double* box_lo,
                                   const double* box_hi, Tree& t, DeviceTreeOut& out, cudaStream_t st) {
  DeviceTreeStatus res;
  if (p.ndim < 1 || p.ndim > kMaxDim) return {HODLR_ERR_INVALID, "ndim must be in 1..8"};
  if (p.nmax < 1) return {HODLR_ERR_INVALID, "nmax must be positive"};
  if (p.dprime < -1 || p.dprime > p.ndim - 1) return {HODLR_ERR_INVALID, "dprime must be in -1..ndim-1"};
  if (n < 1) return {HODLR_ERR_INVALID, "need at least one point"};
  if (n > (int64_t(1) << 31) - 1) return {HODLR_ERR_INVALID, "at most 2^31-1 points"};
  const int d = p.ndim;
  const int fan = 1 << d;
  try {
    Scratch s;
    t = Tree();
    t.p = p;
    t.n = n;
    // level 0: the root with the caller's box (set_box on the host: the same rounding as tree.cpp)
    std::vector<double> rlo(box_lo, box_lo + d), rhi(box_hi, box_hi + d), rc(static_cast<size_t>(d));
    double rL = std::fabs(rlo[0] - rhi[0]);
    for (int k = 0; k < d; k++) {
      if (std::fabs(rlo[k] - rhi[k]) > rL) rL = std::fabs(rlo[k] - rhi[k]);
      rc[size_t(k)] = 0.5 * (rlo[size_t(k)] + rhi[size_t(k)]);
    }
    double* d_aos = s.alloc<double>(size_t(n) * d, "tree points");
    ck(cudaMemcpyAsync(d_aos, points, sizeof(double) * size_t(n) * d, cudaMemcpyHostToDevice, st), "tree points");
    struct Level {
      int64_t size = 0;
      int64_t *begin = nullptr, *count = nullptr;
      double *lo = nullptr, *hi = nullptr, *center = nullptr, *L = nullptr;
      int64_t *nb_ptr = nullptr, *in_ptr = nullptr, *nb = nullptr, *in = nullptr;
      int64_t nnb = 0, nin = 0;
      int32_t* perm = nullptr;  // the points' order after this level's split
    };
    std::vector<Level> lv(1);
    {
      Level& r = lv[0];
      r.size = 1;
      r.begin = s.alloc<int64_t>(1, "tree nodes");
      r.count = s.alloc<int64_t>(1, "tree nodes");
      r.lo = s.alloc<double>(size_t(d), "tree boxes");
      r.hi = s.alloc<double>(size_t(d), "tree boxes");
      r.center = s.alloc<double>(size_t(d), "tree boxes");
      r.L = s.alloc<double>(1, "tree boxes");
      r.nb_ptr = s.alloc<int64_t>(2, "tree lists");
      r.in_ptr = s.alloc<int64_t>(2, "tree lists");
      r.nb = s.alloc<int64_t>(1, "tree lists");
      r.in = s.alloc<int64_t>(1, "tree lists");
      r.perm = s.alloc<int32_t>(size_t(n), "tree permutation");
      const int64_t zero[2] = {0, 0}, cnt = n;
      ck(cudaMemcpyAsync(r.begin, zero, sizeof(int64_t), cudaMemcpyHostToDevice, st), "tree root");
      ck(cudaMemcpyAsync(r.count, &cnt, sizeof(int64_t), cudaMemcpyHostToDevice, st), "tree root");
      ck(cudaMemcpyAsync(r.lo, rlo.data(), sizeof(double) * d, cudaMemcpyHostToDevice, st), "tree root");
      ck(cudaMemcpyAsync(r.hi, rhi.data(), sizeof(double) * d, cudaMemcpyHostToDevice, st), "tree root");
      ck(cudaMemcpyAsync(r.center, rc.data(), sizeof(double) * d, cudaMemcpyHostToDevice, st), "tree root");
      ck(cudaMemcpyAsync(r.L, &rL, sizeof(double), cudaMemcpyHostToDevice, st), "tree root");
      ck(cudaMemcpyAsync(r.nb_ptr, zero, sizeof(zero), cudaMemcpyHostToDevice, st), "tree root");
      ck(cudaMemcpyAsync(r.in_ptr, zero, sizeof(zero), cudaMemcpyHostToDevice, st), "tree root");
      std::vector<int32_t> id(static_cast<size_t>(n));
      for (int64_t i = 0; i < n; i++) id[size_t(i)] = int32_t(i);
      ck(cudaMemcpyAsync(r.perm, id.data(), sizeof(int32_t) * size_t(n), cudaMemcpyHostToDevice, st), "tree root");
      ck(cudaStreamSynchronize(st), "tree root");
    }
    unsigned long long* d_maxc = s.alloc<unsigned long long>(1, "tree counter");
    int64_t maxc = n;
    // Tree::Tree: split the whole last level while any node holds more than
    // Nmax points (HDD_tree.hpp:43-69); empty nodes are split too
    while (maxc > p.nmax) {
      const Level& P = lv.back();
      if (P.size > kMaxLevelNodes / fan)
        return {HODLR_ERR_TREE, "tree exceeds " + std::to_string(kMaxLevelNodes) +
                                    " nodes on one level (points too clustered for Nmax; the reference would run out "
                                    "of memory)"};
      Level c;
      c.size = P.size * fan;
      const size_t C = size_t(c.size);
      c.begin = s.alloc<int64_t>(C, "tree nodes");
      c.count = s.alloc<int64_t>(C, "tree nodes");
      c.lo = s.alloc<double>(C * d, "tree boxes");
      c.hi = s.alloc<double>(C * d, "tree boxes");
      c.center = s.alloc<double>(C * d, "tree boxes");
      c.L = s.alloc<double>(C, "tree boxes");
      c.perm = s.alloc<int32_t>(size_t(n), "tree permutation");
      ck(cudaMemsetAsync(d_maxc, 0, sizeof(unsigned long long), st), "tree split");
      count_launches(2);
      child_boxes_kernel<<<blocks_for(c.size, 256), 256, 0, st>>>(d, fan, c.size, P.lo, P.hi, c.lo, c.hi, c.center,
                                                                   c.L);
      split_kernel<<<unsigned(P.size), kSplitThreads, 0, st>>>(d, fan, d_aos, P.begin, P.count, P.lo, P.hi, P.perm,
                                                              c.perm, c.begin, c.count, d_maxc);
      ck(cudaGetLastError(), "tree split");
      unsigned long long mx = 0;
      ck(cudaMemcpyAsync(&mx, d_maxc, sizeof(mx), cudaMemcpyDeviceToHost, st), "tree split");
      ck(cudaStreamSynchronize(st), "tree split");
      maxc = int64_t(mx);
      // a level that still holds too many points and is already too wide
      // fails on the next split: the host build reaches the same refusal
      if (maxc > p.nmax && c.size > kMaxLevelNodes / fan)
        return {HODLR_ERR_TREE, "tree exceeds " + std::to_string(kMaxLevelNodes) +
                                    " nodes on one level (points too clustered for Nmax; the reference would run out "
                                    "of memory)"};
      // interaction and neighbour lists of the new level
      c.nb_ptr = s.alloc<int64_t>(C + 1, "tree lists");
      c.in_ptr = s.alloc<int64_t>(C + 1, "tree lists");
      count_launches(1);
      lists_kernel<false><<<blocks_for(c.size, 128), 128, 0, st>>>(d, p.dprime, fan, c.size, c.center, c.L, P.nb_ptr,
                                                                   P.nb, c.nb_ptr, c.in_ptr, nullptr, nullptr);
      ck(cudaGetLastError(), "tree lists");
      c.nnb = scan(s, c.nb_ptr, c.size, c.nb_ptr, st);
      c.nin = scan(s, c.in_ptr, c.size, c.in_ptr, st);
      c.nb = s.alloc<int64_t>(size_t(c.nnb), "tree lists");
      c.in = s.alloc<int64_t>(size_t(c.nin), "tree lists");
      count_launches(1);
      lists_kernel<true><<<blocks_for(c.size, 128), 128, 0, st>>>(d, p.dprime, fan, c.size, c.center, c.L, P.nb_ptr,
                                                                  P.nb, c.nb_ptr, c.in_ptr, c.nb, c.in);
      ck(cudaGetLastError(), "tree lists");
      lv.push_back(c);
    }
    // the host tree: node arrays level by level, lists with global offsets
    const int levels = int(lv.size());
    t.levels = levels;
    t.level_size.clear();
    t.level_off = {0};
    for (const Level& l : lv) {
      t.level_size.push_back(l.size);
      t.level_off.push_back(t.level_off.back() + l.size);
    }
    const size_t nodes = size_t(t.level_off.back());
    t.begin.resize(nodes);
    t.count.resize(nodes);
    t.lo.resize(nodes * d);
    t.hi.resize(nodes * d);
    t.center.resize(nodes * d);
    t.L.resize(nodes);
    t.nbr_ptr.assign(nodes + 1, 0);
    t.intr_ptr.assign(nodes + 1, 0);
    std::vector<std::vector<int64_t>> nbp(static_cast<size_t>(levels)), inp(static_cast<size_t>(levels));
    size_t tot_nb = 0, tot_in = 0;
    for (int l = 0; l < levels; l++) {
      const Level& L = lv[size_t(l)];
      const size_t off = size_t(t.level_off[size_t(l)]), sz = size_t(L.size);
      to_host(t.begin, off, L.begin, sz, st);
      to_host(t.count, off, L.count, sz, st);
      to_host(t.lo, off * d, L.lo, sz * d, st);
      to_host(t.hi, off * d, L.hi, sz * d, st);
      to_host(t.center, off * d, L.center, sz * d, st);
      to_host(t.L, off, L.L, sz, st);
      nbp[size_t(l)].resize(sz + 1);
      inp[size_t(l)].resize(sz + 1);
      to_host(nbp[size_t(l)], 0, L.nb_ptr, sz + 1, st);
      to_host(inp[size_t(l)], 0, L.in_ptr, sz + 1, st);
      tot_nb += size_t(L.nnb);
      tot_in += size_t(L.nin);
    }
    t.nbr.resize(tot_nb);
    t.intr.resize(tot_in);
    {
      size_t onb = 0, oin = 0;
      for (int l = 0; l < levels; l++) {
        const Level& L = lv[size_t(l)];
        to_host(t.nbr, onb, L.nb, size_t(L.nnb), st);
        to_host(t.intr, oin, L.in, size_t(L.nin), st);
        onb += size_t(L.nnb);
        oin += size_t(L.nin);
      }
    }
    std::vector<int32_t> perm32(static_cast<size_t>(n));
    to_host(perm32, 0, lv.back().perm, size_t(n), st);
    // the device arrays of the engine: points in tree order, the permutation,
    // and per level the reference order (each level's order mapped to tree positions)
    if (out.d_pts && out.d_perm) {
      count_launches(1);
      gather_soa_kernel<<<blocks_for(n, 256), 256, 0, st>>>(d, n, d_aos, lv.back().perm, out.d_pts, out.d_perm);
      ck(cudaGetLastError(), "tree points");
    }
    if (out.alloc_lmap) {
      out.d_lmap = out.alloc_lmap(size_t(levels) * size_t(n));
      int32_t* inv = s.alloc<int32_t>(size_t(n), "tree inverse permutation");
      count_launches(1 + uint64_t(levels));
      inverse_kernel<<<blocks_for(n, 256), 256, 0, st>>>(n, lv.back().perm, inv);
      for (int l = 0; l < levels; l++)
        lmap_kernel<<<blocks_for(n, 256), 256, 0, st>>>(n, lv[size_t(l)].perm, inv, out.d_lmap + size_t(l) * n);
      ck(cudaGetLastError(), "tree reference-order maps");
    }
    ck(cudaStreamSynchronize(st), "tree to host");
    {
      size_t onb = 0, oin = 0;
      for (int l = 0; l < levels; l++) {
        const size_t off = size_t(t.level_off[size_t(l)]);
        for (int64_t k = 0; k < lv[size_t(l)].size; k++) {
          t.nbr_ptr[off + size_t(k) + 1] = int64_t(onb) + nbp[size_t(l)][size_t(k) + 1];
          t.intr_ptr[off + size_t(k) + 1] = int64_t(oin) + inp[size_t(l)][size_t(k) + 1];
        }
        onb += size_t(lv[size_t(l)].nnb);
        oin += size_t(lv[size_t(l)].nin);
      }
    }
    t.perm.assign(perm32.begin(), perm32.end());
  } catch (const CudaError& e) {
    return {e.e == cudaErrorMemoryAllocation ? HODLR_ERR_OOM : HODLR_ERR_CUDA,
            std::string(e.what) + ": " + cudaGetErrorString(e.e)};
  }
  return res;
}

}  // namespace hodlr
