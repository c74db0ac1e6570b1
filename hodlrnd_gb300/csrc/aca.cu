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

__device__ __forceinline__ int rng_next(uint64_t& s) {
  s += 0x9E3779B97F4A7C15ull;
  uint64_t z = s;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return int(z >> 33);
}

template <int D, class Team>
struct AcaTeam {
  const AcaArgs& a;
  const AcaBlockDesc& B;
  Team tm;
  int m, n, cap, nwr, nwc;
  double *U, *V;
  uint32_t *rb, *cb;
  int32_t *rl, *cl;
  KernelDev K;

  __device__ AcaTeam(const AcaArgs& a_, const AcaBlockDesc& B_, Team tm_) : a(a_), B(B_), tm(tm_) {
    K = a.K;
    if (B.kscale != 0.0) K.scale = B.kscale;
    m = B.m;
    n = B.n;
    cap = B.cap;
    nwr = int((m + 31) >> 5);
    nwc = int((n + 31) >> 5);
    U = a.ws + B.ws;
    V = U + int64_t(m) * cap;
    rb = a.bits + B.bits;
    cb = rb + nwr;
    rl = a.lists + B.lists;
    cl = rl + cap + 2;
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
    const int64_t pi = a.lmap[B.t_map + i0];
    load_point<D>(a.P, pi, xi);
    double ba = -1.0, bv = 0.0, v0 = 0.0, s = 0.0;
    int bi = 0x7fffffff;
    for (int j = tm.tid(); j < n; j += Team::kSize) {
      double val = kernel_entry<D>(a.P, K, pi, a.lmap[B.s_map + j], xi);
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
    const int64_t pj = a.lmap[B.s_map + j0];
    for (int i = tm.tid(); i < m; i += Team::kSize) {
      // A(i, j0) with the target point first, as getCol evaluates it
      // (getMatrixEntry(sources[j], k), kernel_function.hpp:32-40).
      double xi[D];
      const int64_t pi = a.lmap[B.t_map + i];
      load_point<D>(a.P, pi, xi);
      double val = kernel_entry<D>(a.P, K, pi, pj, xi);
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

  __device__ void run(AcaOut* out) {
    const double tol = a.tol;
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
    do {
      if (r >= cap) {
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
      for (int k = 0; k < r; k++) {
        double du = 0.0, dv = 0.0;
        for (int i = tm.tid(); i < m; i += Team::kSize) du += U[i + int64_t(k) * m] * U[i + int64_t(r) * m];
        for (int j = tm.tid(); j < n; j += Team::kSize) dv += V[j + int64_t(k) * n] * V[j + int64_t(r) * n];
        du = tm.sum(du);
        dv = tm.sum(dv);
        mnorm += __dmul_rn(__dmul_rn(2.0, fabs(du)), fabs(dv));
      }
      r++;
    } while (__dmul_rn(__dmul_rn(double(int(int64_t(r) * (m + n))), row_norm), col_norm) >
                 __dmul_rn(__dmul_rn(fabs(mx), tol), mnorm) &&
             r < mn);
    int rank = r;
    if (!(flags & kAcaOverflow) && r >= mn - 1) {
      flags |= kAcaDense;
      rank = mn;
    }
    if (tm.tid() == 0) {
      out->rank = rank;
      out->flags = flags;
    }
  }
};

template <int D>
__global__ void __launch_bounds__(128) aca_warp_kernel(AcaArgs a, const int32_t* __restrict__ list, int count) {
  const int team = blockIdx.x * 4 + (threadIdx.x >> 5);
  if (team >= count) return;
  const int b = list[team];
  AcaTeam<D, WarpTeam> t(a, a.blocks[b], WarpTeam());
  t.run(a.out + b);
}

template <int D>
__global__ void __launch_bounds__(256) aca_cta_kernel(AcaArgs a, const int32_t* __restrict__ list, int count) {
  __shared__ double red[256 / 32 + 1];
  __shared__ int redi[256 / 32 + 1];
  const int b = list[blockIdx.x];
  CtaTeam<256> tm{red, redi};
  AcaTeam<D, CtaTeam<256>> t(a, a.blocks[b], tm);
  t.run(a.out + b);
}

template <int D>
void launch_d(const AcaArgs& a, const int32_t* warp_list, int nwarp, const int32_t* cta_list, int ncta,
              cudaStream_t st) {
  if (nwarp > 0) aca_warp_kernel<D><<<unsigned((nwarp + 3) / 4), 128, 0, st>>>(a, warp_list, nwarp);
  if (ncta > 0) aca_cta_kernel<D><<<unsigned(ncta), 256, 0, st>>>(a, cta_list, ncta);
}

}  // namespace

cudaError_t launch_aca(int ndim, const AcaArgs& a, const int32_t* warp_list, int nwarp, const int32_t* cta_list,
                       int ncta, cudaStream_t st) {
  count_launches(uint64_t(nwarp > 0) + uint64_t(ncta > 0));
  switch (ndim) {
    case 1: launch_d<1>(a, warp_list, nwarp, cta_list, ncta, st); break;
    case 2: launch_d<2>(a, warp_list, nwarp, cta_list, ncta, st); break;
    case 3: launch_d<3>(a, warp_list, nwarp, cta_list, ncta, st); break;
    case 4: launch_d<4>(a, warp_list, nwarp, cta_list, ncta, st); break;
    case 5: launch_d<5>(a, warp_list, nwarp, cta_list, ncta, st); break;
    case 6: launch_d<6>(a, warp_list, nwarp, cta_list, ncta, st); break;
    case 7: launch_d<7>(a, warp_list, nwarp, cta_list, ncta, st); break;
    case 8: launch_d<8>(a, warp_list, nwarp, cta_list, ncta, st); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace hodlr
