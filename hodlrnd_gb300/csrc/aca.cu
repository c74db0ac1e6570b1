// Batched partially pivoted ACA on the GPU: one team (a warp for small
// blocks, a CTA for large ones) compresses one admissible block.
//
// Restates LowRankMat::ACA_FAST (HODLRnD include/LowRank_matrix.hpp:64-377;
// ACA_MEM_EFF :379-660 runs the same loop) step for step:
//  * start at local row 0; generate the residual row, pick the first
//    largest |entry| among the remaining columns (maxAbsVector,
//    include/kernel_function.hpp:55-68);
//  * while that pivot is below eps_ACA in absolute value, retry with another
//    row (10 tries): the last/first remaining row while the rank is below 3,
//    then alternately a random remaining row and the midpoint of the widest
//    gap between used rows (:144-216); the same for columns (:245-316),
//    including the column branch that dereferences remaining_col_ind.end(),
//    which with libstdc++ yields the number of remaining columns (:258);
//  * gamma = 1 / row pivot, u = gamma * column, v = row; the squared
//    Frobenius estimate gains gamma^2 |row|^2 |col|^2 + 2 sum_k |u_k.u| |v_k.v|
//    (:326-338);
//  * stop when r (m+n) |row| |col| <= |column pivot| eps |S|^2 or r reaches
//    min(m, n); a block whose rank reaches min(m, n) - 1 is kept dense
//    (:341-363).
// The reference draws its random rows from the process-wide rand(); here each
// block has its own splitmix64 stream seeded from (level, target, source), so
// blocks can run in any order (the CPU oracle does the same in rng_mode 1).
//
// Residual rows/columns are formed with one rounding per operation
// (__dsub_rn/__dmul_rn) in the same order as the reference, so the factors
// match the oracle bit for bit; only the norm reductions are summed in a
// different order.
//
// Rows and columns are indexed in the reference's order of the node's points
// (by caller index; a non-leaf node's tree-order range is grouped by leaf
// instead), so the pivots, the restarts and hence the factors follow the
// reference; the compaction step scatters the factors into tree order.
//
// Workspace per block: U (m x cap) and V (n x cap) FP64 column major, a
// bitmap of remaining rows and one of remaining columns, the lists of used
// row and column indices.  A block whose rank would exceed cap reports
// kAcaOverflow and is rerun by the host with a larger cap.
#include "aca.h"
#include "device.cuh"

namespace hodlr {

namespace {

constexpr int kMaxTries = 10;
constexpr int kNormChunk = 512;  // norm-estimate terms a CTA team holds in shared memory at once

__device__ __forceinline__ int rng_next(uint64_t& s) {
  s += 0x9E3779B97F4A7C15ull;
  uint64_t z = s;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return int(z >> 33);
}

// Shared memory of one staged team (blocks of at most T rows and columns):
// U (T x T), V (T x T), the target and source coordinates (D x T each), then
// the target and source tree positions, the used-row and used-column lists
// and the two bitmaps.
__host__ __device__ constexpr int staged_team_bytes(int T, int D) {
  return (2 * T * T + 2 * D * T) * 8 + (2 * T + 2 * (T + 2) + 2) * 4;
}

template <int D, class Team, bool S = false>
struct AcaTeam {
  const AcaArgs& a;
  const AcaBlockDesc& B;
  Team tm;
  int m, n, cap, nwr, nwc;
  double *U, *V;
  uint32_t *rb, *cb;
  int32_t *rl, *cl;
  KernelDev K;
  // staged teams: coordinates (target, source; SoA with strides m, n) and tree positions
  double *xt = nullptr, *xs = nullptr;
  int32_t *it = nullptr, *is = nullptr;

  __device__ AcaTeam(const AcaArgs& a_, const AcaBlockDesc& B_, Team tm_, unsigned char* sm = nullptr)
      : a(a_), B(B_), tm(tm_) {
    K = a.K;
    if (B.kscale != 0.0) K.scale = B.kscale;
    m = B.m;
    n = B.n;
    cap = B.cap;
    nwr = int((m + 31) >> 5);
    nwc = int((n + 31) >> 5);
    if constexpr (S) {
      // cap <= min(m, n) <= T: every piece fits the team's share (staged_team_bytes)
      constexpr int T = Team::kSize;
      double* d = reinterpret_cast<double*>(sm);
      U = d;
      V = U + T * T;
      xt = V + T * T;
      xs = xt + D * T;
      it = reinterpret_cast<int32_t*>(xs + D * T);
      is = it + T;
      rl = is + T;
      cl = rl + T + 2;
      rb = reinterpret_cast<uint32_t*>(cl + T + 2);
      cb = rb + 1;
    } else {
      U = a.ws + B.ws;
      V = U + int64_t(m) * cap;
      rb = a.bits + B.bits;
      cb = rb + nwr;
      rl = a.lists + B.lists;
      cl = rl + (B.lcap > 0 ? B.lcap : cap) + 2;  // room for the rank the block may grow to
    }
  }

  // staged teams: the block's points (tree positions and coordinates) into shared memory
  __device__ void stage_points() {
    for (int i = tm.tid(); i < m; i += Team::kSize) {
      const int32_t p = a.lmap[B.t_map + i];
      it[i] = p;
#pragma unroll
      for (int k = 0; k < D; k++) xt[k * m + i] = a.P.x[k * a.P.ld + p];
    }
    for (int j = tm.tid(); j < n; j += Team::kSize) {
      const int32_t p = a.lmap[B.s_map + j];
      is[j] = p;
#pragma unroll
      for (int k = 0; k < D; k++) xs[k * n + j] = a.P.x[k * a.P.ld + p];
    }
    tm.sync();
  }

  // A larger workspace from the growth arena: 4 x the columns (at most
  // min(m, n)), the r columns computed so far copied over.  False when there
  // is no arena or it is full.
  __device__ bool grow(int r, AcaOut* out) {
    if (S || !a.arena_used) return false;
    const int ncap = min(min(m, n), cap * 4);
    if (ncap <= cap) return false;
    const uint64_t need = uint64_t(ncap) * uint64_t(m + n);
    double got = -1.0;  // arena offset (doubles; exact below 2^53), or -1
    if (tm.tid() == 0) {
      const unsigned long long off = atomicAdd(a.arena_used, (unsigned long long)need);
      if (off + need <= a.arena_size) got = double(off);
    }
    got = tm.bcast(got);
    if (got < 0.0) return false;
    const int64_t ws = a.arena_off + int64_t(got);
    double* nu = a.ws + ws;
    double* nv = nu + int64_t(m) * ncap;
    for (int64_t e = tm.tid(); e < int64_t(m) * r; e += Team::kSize) nu[e] = U[e];
    for (int64_t e = tm.tid(); e < int64_t(n) * r; e += Team::kSize) nv[e] = V[e];
    tm.sync();
    U = nu;
    V = nv;
    cap = ncap;
    if (tm.tid() == 0) {
      out->cap = ncap;
      out->ws = ws;
    }
    return true;
  }

  // staged teams: U and V of a low-rank result to the block's workspace
  // (the layout the compaction reads: U m x cap, then V n x cap, column major)
  __device__ void write_factors(int r) {
    double* gu = a.ws + B.ws;
    double* gv = gu + int64_t(m) * cap;
    for (int e = tm.tid(); e < m * r; e += Team::kSize) gu[e] = U[e];
    for (int e = tm.tid(); e < n * r; e += Team::kSize) gv[e] = V[e];
  }

  __device__ void init_bits(uint32_t* bits, int nw, int size) {
    for (int w = tm.tid(); w < nw; w += Team::kSize) {
      const int lo = w * 32, hi = min(size, lo + 32);
      bits[w] = (hi - lo == 32) ? 0xffffffffu : ((1u << (hi - lo)) - 1u);
    }
  }

  // std::set::erase; returns whether the index was present.
  __device__ bool erase(uint32_t* bits, int idx) {
    const uint32_t w = bits[idx >> 5];
    const bool was = (w >> (idx & 31)) & 1u;
    tm.sync();
    if (tm.tid() == 0 && was) bits[idx >> 5] = w & ~(1u << (idx & 31));
    tm.sync();
    return was;
  }

  // *begin(); 0 for an empty set (libstdc++ reads the node count there).
  __device__ int first(const uint32_t* bits, int nw) {
    int r = 0;
    if (tm.tid() == 0)
      for (int w = 0; w < nw; w++)
        if (bits[w]) {
          r = w * 32 + __ffs(bits[w]) - 1;
          break;
        }
    return tm.bcast(r);
  }
  // *--end()
  __device__ int last(const uint32_t* bits, int nw) {
    int r = 0;
    if (tm.tid() == 0)
      for (int w = nw - 1; w >= 0; w--)
        if (bits[w]) {
          r = w * 32 + 31 - __clz(bits[w]);
          break;
        }
    return tm.bcast(r);
  }
  // std::advance(begin(), k)
  __device__ int kth(const uint32_t* bits, int nw, int k) {
    int r = 0;
    if (tm.tid() == 0)
      for (int w = 0; w < nw; w++) {
        uint32_t b = bits[w];
        const int c = __popc(b);
        if (k < c) {
          for (; k > 0; k--) b &= b - 1;
          r = w * 32 + __ffs(b) - 1;
          break;
        }
        k -= c;
      }
    return tm.bcast(r);
  }
  // Midpoint of the widest gap between consecutive sorted used indices; the
  // first widest gap wins, and an all-zero gap list yields the smallest index
  // (LowRank_matrix.hpp:181-198).
  __device__ int gap_mid(const int32_t* list, int len) {
    int r = 0;
    if (tm.tid() == 0) {
      int lo = list[0];
      for (int q = 1; q < len; q++) lo = min(lo, list[q]);
      int best_gap = 0, best_a = lo;
      for (int q = 0; q < len; q++) {
        const int av = list[q];
        int succ = 0x7fffffff;
        for (int z = 0; z < len; z++)
          if (list[z] > av && list[z] < succ) succ = list[z];
        if (succ == 0x7fffffff) continue;
        const int g = succ - av;
        if (g > best_gap || (g == best_gap && av < best_a && g > 0)) {
          best_gap = g;
          best_a = av;
        }
      }
      r = best_a + best_gap / 2;
    }
    return tm.bcast(r);
  }

  // Residual row i0 into V[:, r]; argmax over the remaining columns.
  __device__ void gen_row(int i0, int r, int nc, double& mx, int& piv, double& sq) {
    double xi[D];
    int64_t pi;
    if constexpr (S) {
      pi = it[i0];
#pragma unroll
      for (int k = 0; k < D; k++) xi[k] = xt[k * m + i0];
    } else {
      pi = a.lmap[B.t_map + i0];
      load_point<D>(a.P, pi, xi);
    }
    double ba = -1.0, bv = 0.0, v0 = 0.0, s = 0.0;
    int bi = 0x7fffffff;
    for (int j = tm.tid(); j < n; j += Team::kSize) {
      double val;
      if constexpr (S)
        val = kernel_entry_xy<D>(K, pi == is[j], xi, xs + j, n);
      else
        val = kernel_entry<D>(a.P, K, pi, a.lmap[B.s_map + j], xi);
      for (int k = 0; k < r; k++) val = __dsub_rn(val, __dmul_rn(U[i0 + int64_t(k) * m], V[j + int64_t(k) * n]));
      V[j + int64_t(r) * n] = val;
      s += val * val;
      if (j == 0) v0 = val;
      if ((cb[j >> 5] >> (j & 31)) & 1u) {
        const double av = fabs(val);
        if (av > ba) {
          ba = av;
          bi = j;
          bv = val;
        }
      }
    }
    sq = s;
    tm.argmax(ba, bi, bv);
    if (nc == 0) {
      piv = 0;
      mx = tm.bcast(v0);
    } else {
      piv = bi;
      mx = bv;
    }
    tm.sync();
  }

  // Residual column j0 into U[:, r]; argmax over the remaining rows.
  __device__ void gen_col(int j0, int r, int nr, double& mx, int& piv, double& sq) {
    double ba = -1.0, bv = 0.0, v0 = 0.0, s = 0.0;
    int bi = 0x7fffffff;
    const int64_t pj = S ? int64_t(is[j0]) : int64_t(a.lmap[B.s_map + j0]);
    for (int i = tm.tid(); i < m; i += Team::kSize) {
      // A(i, j0) with the target point first, as getCol evaluates it
      // (getMatrixEntry(sources[j], k), kernel_function.hpp:32-40).
      double xi[D];
      double val;
      if constexpr (S) {
#pragma unroll
        for (int k = 0; k < D; k++) xi[k] = xt[k * m + i];
        val = kernel_entry_xy<D>(K, it[i] == pj, xi, xs + j0, n);
      } else {
        const int64_t pi = a.lmap[B.t_map + i];
        load_point<D>(a.P, pi, xi);
        val = kernel_entry<D>(a.P, K, pi, pj, xi);
      }
      for (int k = 0; k < r; k++) val = __dsub_rn(val, __dmul_rn(V[j0 + int64_t(k) * n], U[i + int64_t(k) * m]));
      U[i + int64_t(r) * m] = val;
      s += val * val;
      if (i == 0) v0 = val;
      if ((rb[i >> 5] >> (i & 31)) & 1u) {
        const double av = fabs(val);
        if (av > ba) {
          ba = av;
          bi = i;
          bv = val;
        }
      }
    }
    sq = s;
    tm.argmax(ba, bi, bv);
    if (nr == 0) {
      piv = 0;
      mx = tm.bcast(v0);
    } else {
      piv = bi;
      mx = bv;
    }
    tm.sync();
  }

  // mnorm += 2 |u_k . u_r| |v_k . v_r| for k < r, in order of k (LowRank_matrix.hpp:335-338).
  // A CTA team gives each dot product pair to one warp (a warp reduction, no
  // barrier), writes the terms to shared memory and adds them in order after
  // one barrier per kNormChunk columns; warp and sub-warp teams reduce each
  // pair across the team.
  __device__ void norm_update(int r, double& mnorm) {
    if constexpr (Team::kSize > 32) {
      constexpr int W = Team::kSize / 32;
      const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
      for (int k0 = 0; k0 < r; k0 += kNormChunk) {
        const int kn = min(kNormChunk, r - k0);
        for (int kk = w; kk < kn; kk += W) {
          const int k = k0 + kk;
          double du = 0.0, dv = 0.0;
          for (int i = lane; i < m; i += 32) du += U[i + int64_t(k) * m] * U[i + int64_t(r) * m];
          for (int j = lane; j < n; j += 32) dv += V[j + int64_t(k) * n] * V[j + int64_t(r) * n];
          du = WarpTeam().sum(du);
          dv = WarpTeam().sum(dv);
          if (lane == 0) tm.terms[kk] = __dmul_rn(__dmul_rn(2.0, fabs(du)), fabs(dv));
        }
        __syncthreads();
        for (int kk = 0; kk < kn; kk++) mnorm += tm.terms[kk];
        __syncthreads();
      }
    } else {
      for (int k = 0; k < r; k++) {
        double du = 0.0, dv = 0.0;
        for (int i = tm.tid(); i < m; i += Team::kSize) du += U[i + int64_t(k) * m] * U[i + int64_t(r) * m];
        for (int j = tm.tid(); j < n; j += Team::kSize) dv += V[j + int64_t(k) * n] * V[j + int64_t(r) * n];
        du = tm.sum(du);
        dv = tm.sum(dv);
        mnorm += __dmul_rn(__dmul_rn(2.0, fabs(du)), fabs(dv));
      }
    }
  }

  __device__ void run(AcaOut* out) {
    const double tol = a.tol;
    if constexpr (S) stage_points();
    init_bits(rb, nwr, m);
    init_bits(cb, nwc, n);
    tm.sync();
    int nr = m, nc = n;
    if (erase(rb, 0)) nr--;
    if (tm.tid() == 0) rl[0] = 0;
    int nrow = 1, ncol = 0, r = 0;
    uint64_t rng = B.seed;
    double mx = 0.0, gamma = 0.0, mnorm = 0.0, row_norm = 0.0, col_norm = 0.0;
    int piv = 0, cur_row = 0, flags = 0;
    const int mn = min(m, n);
    if (tm.tid() == 0) {
      out->cap = 0;
      out->ws = 0;
    }
    do {
      if (r >= cap && !grow(r, out)) {
        flags |= kAcaOverflow;
        break;
      }
      double rsq_p = 0.0, csq_p = 0.0;
      gen_row(cur_row, r, nc, mx, piv, rsq_p);
      int count = 0;
      bool at_end = false, use_rand = true;
      while (fabs(mx) < tol && count < kMaxTries && nc > 0 && nr > 0) {
        int nrw;
        if (r < 3) {
          nrw = at_end ? last(rb, nwr) : first(rb, nwr);
          at_end = !at_end;
        } else {
          if (use_rand) {
            int k = 0;
            if (tm.tid() == 0) k = int(int64_t(rng_next(rng)) % int64_t(nr));
            nrw = kth(rb, nwr, tm.bcast(k));
          } else {
            nrw = gap_mid(rl, nrow - 1);
          }
          use_rand = !use_rand;
        }
        if (tm.tid() == 0) rl[nrow - 1] = nrw;
        if (erase(rb, nrw)) nr--;
        cur_row = nrw;
        gen_row(cur_row, r, nc, mx, piv, rsq_p);
        count++;
      }
      if (count == kMaxTries || nc == 0 || nr == 0) break;
      count = 0;
      if (tm.tid() == 0) cl[ncol] = piv;
      ncol++;
      if (erase(cb, piv)) nc--;
      gamma = __ddiv_rn(1.0, mx);
      int cur_col = piv;
      gen_col(cur_col, r, nr, mx, piv, csq_p);
      while (fabs(mx) < tol && count < kMaxTries && nc > 0 && nr > 0) {
        int ncl;
        if (ncol - 1 < 3) {
          ncl = at_end ? nc : first(cb, nwc);
          at_end = !at_end;
        } else {
          if (use_rand) {
            int k = 0;
            if (tm.tid() == 0) k = int(int64_t(rng_next(rng)) % int64_t(nc));
            ncl = kth(cb, nwc, tm.bcast(k));
          } else {
            ncl = gap_mid(cl, ncol - 1);
          }
          use_rand = !use_rand;
        }
        if (tm.tid() == 0) cl[ncol - 1] = ncl;
        if (erase(cb, ncl)) nc--;
        cur_col = ncl;
        gen_col(cur_col, r, nr, mx, piv, csq_p);
        count++;
      }
      if (tm.tid() == 0) rl[nrow] = piv;
      nrow++;
      if (erase(rb, piv)) nr--;
      cur_row = piv;
      // u_r = gamma * col; v_r = row (already in V[:, r])
      for (int i = tm.tid(); i < m; i += Team::kSize)
        U[i + int64_t(r) * m] = __dmul_rn(gamma, U[i + int64_t(r) * m]);
      tm.sync();
      const double rsq = tm.sum(rsq_p), csq = tm.sum(csq_p);
      row_norm = sqrt(rsq);
      col_norm = sqrt(csq);
      mnorm += fabs(__dmul_rn(__dmul_rn(__dmul_rn(gamma, gamma), rsq), csq));
      norm_update(r, mnorm);
      r++;
    } while (__dmul_rn(__dmul_rn(double(int(int64_t(r) * (m + n))), row_norm), col_norm) >
                 __dmul_rn(__dmul_rn(fabs(mx), tol), mnorm) &&
             r < mn);
    int rank = r;
    if (!(flags & kAcaOverflow) && r >= mn - 1) {
      flags |= kAcaDense;
      rank = mn;
    }
    if constexpr (S)
      if (!(flags & (kAcaOverflow | kAcaDense))) write_factors(r);
    if (tm.tid() == 0) {
      out->rank = rank;
      out->flags = flags;
    }
  }
};

// Next list position of a team: its static index (first pass) or, with a
// work queue, the next value of the kind's counter (blocks are taken in list
// order, largest first, so teams finish close together).  Team-uniform.
template <class Team>
__device__ __forceinline__ int next_item(const AcaArgs& a, int kind, int first, int& pass, const Team& tm) {
  if (!a.queue) return pass++ == 0 ? first : 0x7fffffff;
  int v = 0;
  if (tm.tid() == 0) v = int(atomicAdd(a.queue + kind, 1u));
  return tm.bcast(v);
}

template <int D>
__global__ void __launch_bounds__(128) aca_warp_kernel(AcaArgs a, const int32_t* __restrict__ list, int count) {
  WarpTeam tm;
  int pass = 0;
  for (;;) {
    const int q = next_item(a, kAcaTeamWarp, blockIdx.x * 4 + (threadIdx.x >> 5), pass, tm);
    if (q >= count) return;
    const int b = list[q];
    AcaTeam<D, WarpTeam> t(a, a.blocks[b], tm);
    t.run(a.out + b);
  }
}

template <int D>
__global__ void __launch_bounds__(256) aca_cta_kernel(AcaArgs a, const int32_t* __restrict__ list, int count) {
  __shared__ double red[256 / 32 + 1];
  __shared__ double terms[kNormChunk];
  __shared__ int redi[256 / 32 + 1];
  CtaTeam<256> tm{red, redi, terms};
  int pass = 0;
  for (;;) {
    const int q = next_item(a, kAcaTeamCta, int(blockIdx.x), pass, tm);
    if (q >= count) return;
    const int b = list[q];
    AcaTeam<D, CtaTeam<256>> t(a, a.blocks[b], tm);
    t.run(a.out + b);
    tm.sync();
  }
}

// Teams of T = 8 or 16 lanes, 128 / T per CTA, each on one block of at most
// T rows and columns held in shared memory.
template <int D, int T>
__global__ void __launch_bounds__(128) aca_sub_kernel(AcaArgs a, const int32_t* __restrict__ list, int count) {
  extern __shared__ __align__(16) unsigned char asm_[];
  constexpr int kTeams = 128 / T;
  constexpr int kind = T == 8 ? kAcaTeam8 : kAcaTeam16;
  const int tl = threadIdx.x / T;
  SubTeam<T> tm;
  int pass = 0;
  for (;;) {
    const int q = next_item(a, kind, blockIdx.x * kTeams + tl, pass, tm);
    if (q >= count) return;
    const int b = list[q];
    AcaTeam<D, SubTeam<T>, true> t(a, a.blocks[b], tm, asm_ + tl * staged_team_bytes(T, D));
    t.run(a.out + b);
    tm.sync();  // the team's shared memory is reused by its next block
  }
}

// CTAs of a launch: one per team's share of the list, or with work queues
// at most a.max_ctas (the teams loop over the queue).
unsigned aca_grid(const AcaArgs& a, int count, int teams_per_cta) {
  const int need = (count + teams_per_cta - 1) / teams_per_cta;
  return unsigned(a.queue && a.max_ctas > 0 ? min(need, a.max_ctas) : need);
}

template <int D, int T>
void launch_sub(const AcaArgs& a, const int32_t* list, int count, cudaStream_t st) {
  constexpr int kTeams = 128 / T;
  constexpr int bytes = kTeams * staged_team_bytes(T, D);
  static_assert(bytes <= 227 * 1024, "staged ACA teams exceed the shared memory of a CTA");
  if (bytes > 48 * 1024) cudaFuncSetAttribute(aca_sub_kernel<D, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  aca_sub_kernel<D, T><<<aca_grid(a, count, kTeams), 128, bytes, st>>>(a, list, count);
}

template <int D>
void launch_kind(const AcaArgs& a, const AcaLists& L, int kind, cudaStream_t st) {
  if (L.n[kind] <= 0) return;
  switch (kind) {
    case kAcaTeamCta:
      aca_cta_kernel<D><<<aca_grid(a, L.n[kAcaTeamCta], 1), 256, 0, st>>>(a, L.list[kAcaTeamCta], L.n[kAcaTeamCta]);
      break;
    case kAcaTeamWarp:
      aca_warp_kernel<D><<<aca_grid(a, L.n[kAcaTeamWarp], 4), 128, 0, st>>>(a, L.list[kAcaTeamWarp],
                                                                            L.n[kAcaTeamWarp]);
      break;
    case kAcaTeam16: launch_sub<D, 16>(a, L.list[kAcaTeam16], L.n[kAcaTeam16], st); break;
    case kAcaTeam8: launch_sub<D, 8>(a, L.list[kAcaTeam8], L.n[kAcaTeam8], st); break;
  }
}

// The launches' kernels, loaded before the first launch: with lazy module
// loading, loading a kernel while others run waits for them, which would
// serialise the team kinds' concurrent launches.
template <int D>
cudaError_t preload_d() {
  cudaFuncAttributes fa;
  cudaError_t e = cudaFuncGetAttributes(&fa, aca_cta_kernel<D>);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, aca_warp_kernel<D>);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, aca_sub_kernel<D, 16>);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, aca_sub_kernel<D, 8>);
  return e;
}

template <int D>
void launch_d(const AcaArgs& a, const AcaLists& L, cudaStream_t st) {
  for (int k : {kAcaTeamCta, kAcaTeamWarp, kAcaTeam16, kAcaTeam8}) launch_kind<D>(a, L, k, st);
}

}  // namespace

int aca_team(int m, int n) {
  const int mx = m > n ? m : n;
  if (mx <= 8) return kAcaTeam8;
  if (mx <= 16) return kAcaTeam16;
  if (mx <= 256) return kAcaTeamWarp;
  return kAcaTeamCta;
}

cudaError_t aca_preload(int ndim) {
  switch (ndim) {
    case 1: return preload_d<1>();
    case 2: return preload_d<2>();
    case 3: return preload_d<3>();
    case 4: return preload_d<4>();
    case 5: return preload_d<5>();
    case 6: return preload_d<6>();
    case 7: return preload_d<7>();
    case 8: return preload_d<8>();
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_aca_kind(int ndim, const AcaArgs& a, const AcaLists& L, int kind, cudaStream_t st) {
  if (kind < 0 || kind >= kAcaTeamKinds) return cudaErrorInvalidValue;
  if (L.n[kind] <= 0) return cudaSuccess;
  count_launches(1);
  switch (ndim) {
    case 1: launch_kind<1>(a, L, kind, st); break;
    case 2: launch_kind<2>(a, L, kind, st); break;
    case 3: launch_kind<3>(a, L, kind, st); break;
    case 4: launch_kind<4>(a, L, kind, st); break;
    case 5: launch_kind<5>(a, L, kind, st); break;
    case 6: launch_kind<6>(a, L, kind, st); break;
    case 7: launch_kind<7>(a, L, kind, st); break;
    case 8: launch_kind<8>(a, L, kind, st); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_aca(int ndim, const AcaArgs& a, const AcaLists& L, cudaStream_t st) {
  uint64_t k = 0;
  for (int q = 0; q < kAcaTeamKinds; q++) k += uint64_t(L.n[q] > 0);
  count_launches(k);
  switch (ndim) {
    case 1: launch_d<1>(a, L, st); break;
    case 2: launch_d<2>(a, L, st); break;
    case 3: launch_d<3>(a, L, st); break;
    case 4: launch_d<4>(a, L, st); break;
    case 5: launch_d<5>(a, L, st); break;
    case 6: launch_d<6>(a, L, st); break;
    case 7: launch_d<7>(a, L, st); break;
    case 8: launch_d<8>(a, L, st); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace hodlr
