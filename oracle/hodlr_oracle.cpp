// HODLRnD CPU oracle -- TEST INFRASTRUCTURE ONLY.
//
// A plain C++ restatement of the reference's hot path, used by tests/ to
// check the GPU engine and by bench.py's CPU-baseline leg.  The GPU product
// never links, loads or calls this file.  Each function names the reference
// code it restates (paths relative to the HODLRnD project root):
//
//   tree + 2^d clustering ...... include/HDD_tree.hpp:23-74,
//                                include/HDD_clusters.hpp:22-41,70-133
//   admissibility, lists ....... include/HDD_node.hpp:24-31,150-180,
//                                include/HDD_clusters.hpp:142-162,
//                                include/points_dt.hpp:20-39
//   partially pivoted ACA ...... include/LowRank_matrix.hpp:64-377 (the loop
//                                is shared with ACA_MEM_EFF :379-660)
//   leaf dense blocks .......... include/HDD_node.hpp:118-148,
//                                include/kernel_function.hpp:43-53
//   matvec ..................... include/HDD_tree.hpp:86-107,
//                                include/HDD_node.hpp:82-99,223-254
//   restarted GMRES ............ include/GMRES.hpp:83-146,160-305
//   statistics ................. include/HDD_node.hpp:182-220,
//                                include/HDD_matrix.hpp:69-85
//
// Parity pins: the restatement is compared, in tests/, with the reference's
// own headers compiled in place (oracle/ref_driver.cpp) -- identical trees,
// lists and ranks, and bit-identical GMRES on a dense operator -- and with
// the reference's golden pair data/x_10000.bin / data/rhs_10000.bin.
//
// Deliberate, documented differences from the reference:
//  * Every admissible block is stored as U V^T.  The reference stores blocks
//    with more than 2*Nmax columns as a skeleton A(:,J) A(I,J)^-1 A(I,:)
//    (LowRank_matrix.hpp:27-35,40-59,685-698); both are the same cross
//    approximation, so the matvecs agree to rounding.
//  * rng_mode 1 (per block): the restart heuristic's rand() calls
//    (LowRank_matrix.hpp:175,274) draw from a per-block counter-based
//    generator keyed by (level, target, source) instead of the process-wide
//    rand() stream, so that blocks can be compressed in any order.  rng_mode
//    0 calls the C library's rand() in the reference's block order and
//    reproduces the reference exactly.
//  * Dereferencing remaining_col_ind.end() (LowRank_matrix.hpp:258) is
//    undefined behaviour; with libstdc++ it reads the set's node count, and
//    the restatement uses that value (it is always a valid column index
//    there, because the failed pivot column was already removed).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const int kMaxDim = 8;

struct Params {
  int32_t ndim, nmax, dprime, kind;
  double eps, scale, diag;
  int32_t rng_mode, threads;
};

struct TNode {
  int64_t count = 0;
  double lo[kMaxDim], hi[kMaxDim], center[kMaxDim];
  double L = 0.0;
  std::vector<int64_t> pts;  // original point indices, in reference order
  std::vector<int64_t> nbr, intr;
};

struct Block {
  int level;
  int64_t t, s;
  int rank = 0;
  bool dense = false;
  std::vector<double> U, V;  // U: m x rank, V: n x rank, column major
};

struct Oracle {
  Params p;
  int64_t n = 0;
  std::vector<double> pts;  // n x ndim row major
  std::vector<std::vector<TNode>> lv;
  std::vector<Block> blocks;
  // leaf near field: per leaf, the dense self block and one per neighbour
  std::vector<std::vector<std::vector<double>>> near;  // [leaf][0=self,1..] m x n col major
  std::vector<std::vector<int64_t>> near_src;          // [leaf][k] source leaf id
  double t_tree = 0, t_init = 0, t_mv = 0;
};

// ---------------------------------------------------------------- kernel
// Entry k(x_i, x_j): d2 accumulated in dimension order, r = sqrt(d2).
inline double entry(const Oracle& o, int64_t i, int64_t j) {
  if (i == j) return o.p.diag;
  const double* a = &o.pts[size_t(i) * size_t(o.p.ndim)];
  const double* b = &o.pts[size_t(j) * size_t(o.p.ndim)];
  double d2 = 0.0;
  for (int k = 0; k < o.p.ndim; k++) {
    const double t = a[k] - b[k];
    d2 = d2 + t * t;
  }
  switch (o.p.kind) {
    case 1: return o.p.scale / std::sqrt(d2);
    case 2: return o.p.scale / d2;
    case 3: return o.p.scale * std::log(std::sqrt(d2));
    case 4: return o.p.scale * std::exp(-std::sqrt(d2));
  }
  return 0.0;
}

// ---------------------------------------------------------------- geometry
// interaction_type (HDD_clusters.hpp:142-162).
int interaction_type(const TNode& A, const TNode& B, int ndim) {
  const double L = std::max(A.L, B.L);
  double e = 0.0;
  for (int k = 0; k < ndim; k++) e += (A.center[k] - B.center[k]) * (A.center[k] - B.center[k]);
  e = std::sqrt(e);
  double dp = e / L;
  dp *= dp;
  int type = ndim;
  if (double(ndim) + 1 > dp)
    type = int(double(type) - std::round(dp));
  else
    type = -1;
  return type;
}

// Node::is_admissible (HDD_node.hpp:24-31): near iff the max-norm centre
// distance is below 1.5 L_self and the interaction type exceeds d'.
bool admissible(const TNode& self, const TNode& other, const Params& p) {
  double dist = std::fabs(self.center[0] - other.center[0]);
  for (int k = 0; k < p.ndim; k++) {
    const double t = std::fabs(self.center[k] - other.center[k]);
    if (t > dist) dist = t;
  }
  if (dist < 1.5 * self.L)
    if (interaction_type(self, other, p.ndim) > p.dprime) return false;
  return true;
}

void set_box(TNode& nd, const double* lo, const double* hi, int ndim) {
  nd.L = std::fabs(lo[0] - hi[0]);
  for (int k = 0; k < ndim; k++) {
    nd.lo[k] = lo[k];
    nd.hi[k] = hi[k];
    if (std::fabs(lo[k] - hi[k]) > nd.L) nd.L = std::fabs(lo[k] - hi[k]);
    nd.center[k] = 0.5 * (lo[k] + hi[k]);
  }
}

// Tree::Tree (HDD_tree.hpp:23-74) with cluster::level_clustering
// (HDD_clusters.hpp:80-133): every node of the last level is split into 2^d
// children, child c taking bit (d-1-k) of c from dimension k (x < mid goes to
// the lower half); splitting continues while any node holds more than Nmax
// points.  Children of node k are nodes k*2^d .. k*2^d+2^d-1 of the next level.
void build_tree(Oracle& o, const double* lo, const double* hi) {
  const int d = o.p.ndim;
  const int64_t fan = int64_t(1) << d;
  o.lv.clear();
  o.lv.emplace_back(1);
  TNode& root = o.lv[0][0];
  set_box(root, lo, hi, d);  // root box from the caller (HDD_matrix.hpp:20-33)
  root.count = o.n;
  root.pts.resize(size_t(o.n));
  for (int64_t i = 0; i < o.n; i++) root.pts[size_t(i)] = i;
  int64_t maxc = o.n;
  while (maxc > o.p.nmax) {
    const std::vector<TNode>& par = o.lv.back();
    if (par.size() * size_t(fan) > (size_t(1) << 22)) throw std::runtime_error("tree too wide");
    std::vector<TNode> ch(par.size() * size_t(fan));
    for (size_t pk = 0; pk < par.size(); pk++) {
      const TNode& P = par[pk];
      double mid[kMaxDim];
      for (int k = 0; k < d; k++) mid[k] = 0.5 * (P.lo[k] + P.hi[k]);
      for (int64_t c = 0; c < fan; c++) {
        double lo[kMaxDim], hi[kMaxDim];
        for (int k = 0; k < d; k++) {
          const bool upper = (c >> (d - 1 - k)) & 1;
          lo[k] = upper ? mid[k] : P.lo[k];
          hi[k] = upper ? P.hi[k] : mid[k];
        }
        set_box(ch[pk * size_t(fan) + size_t(c)], lo, hi, d);
      }
      for (int64_t q : P.pts) {
        const double* x = &o.pts[size_t(q) * size_t(d)];
        int64_t c = 0;
        for (int k = 0; k < d; k++) c = (c << 1) | (x[k] < mid[k] ? 0 : 1);
        ch[pk * size_t(fan) + size_t(c)].pts.push_back(q);
      }
    }
    for (auto& nd : ch) nd.count = int64_t(nd.pts.size());
    o.lv.push_back(std::move(ch));
    // lists for the new level (Node::get_interaction_list, HDD_node.hpp:150-180)
    std::vector<TNode>& cur = o.lv.back();
    const std::vector<TNode>& parl = o.lv[o.lv.size() - 2];
    for (size_t k = 0; k < cur.size(); k++) {
      TNode& me = cur[k];
      const int64_t pk = int64_t(k) / fan;
      for (int64_t c = 0; c < fan; c++) {
        const int64_t sib = pk * fan + c;
        if (sib == int64_t(k)) continue;
        (admissible(me, cur[size_t(sib)], o.p) ? me.intr : me.nbr).push_back(sib);
      }
      for (int64_t q : parl[size_t(pk)].nbr)
        for (int64_t c = 0; c < fan; c++) {
          const int64_t oth = q * fan + c;
          (admissible(me, cur[size_t(oth)], o.p) ? me.intr : me.nbr).push_back(oth);
        }
    }
    maxc = cur[0].count;
    for (auto& nd : cur)
      if (nd.count > maxc) maxc = nd.count;
  }
}

// ---------------------------------------------------------------- ACA
struct Rng {
  int mode;
  uint64_t state;
  int next() {
    if (mode == 0) return std::rand();
    state += 0x9E3779B97F4A7C15ull;
    uint64_t z = state;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return int(z >> 33);
  }
};

}  // namespace

extern "C" uint64_t orc_block_seed(int64_t level, int64_t t, int64_t s) {
  uint64_t h = 0x243F6A8885A308D3ull;
  const uint64_t v[3] = {uint64_t(level), uint64_t(t), uint64_t(s)};
  for (int i = 0; i < 3; i++) {
    h ^= v[i] + 0x9E3779B97F4A7C15ull + (h << 6) + (h >> 2);
    h *= 0xD6E8FEB86659FD93ull;
    h ^= h >> 32;
  }
  return h;
}

namespace {

// Ordered set of remaining local indices, kept as flags plus a count; the
// queries mirror the std::set operations the reference uses.
struct Remaining {
  std::vector<char> f;
  int64_t cnt;
  explicit Remaining(int64_t n) : f(size_t(n), 1), cnt(n) {}
  void erase(int64_t i) {
    if (i >= 0 && i < int64_t(f.size()) && f[size_t(i)]) {
      f[size_t(i)] = 0;
      --cnt;
    }
  }
  int64_t first() const {  // *begin(); an empty libstdc++ set yields its node count, 0
    for (size_t i = 0; i < f.size(); i++)
      if (f[i]) return int64_t(i);
    return 0;
  }
  int64_t last() const {  // *--end()
    for (size_t i = f.size(); i-- > 0;)
      if (f[i]) return int64_t(i);
    return 0;
  }
  int64_t kth(int64_t k) const {  // std::advance(begin(), k)
    for (size_t i = 0; i < f.size(); i++)
      if (f[i] && k-- == 0) return int64_t(i);
    return 0;
  }
};

// kernel_function::maxAbsVector (kernel_function.hpp:55-68): first index of
// largest |v| over the allowed set; an empty set yields index 0.
void max_abs(const std::vector<double>& v, const Remaining& R, double& mx, int64_t& idx) {
  idx = R.first();
  mx = v[size_t(idx)];
  for (size_t i = size_t(idx); i < R.f.size(); i++)
    if (R.f[i] && std::fabs(v[i]) > std::fabs(mx)) {
      idx = int64_t(i);
      mx = v[i];
    }
}

// midpoint of the widest gap between already used indices
// (LowRank_matrix.hpp:181-198 / :280-297)
int64_t gap_mid(const std::vector<int64_t>& used) {
  std::vector<int64_t> s(used);
  std::sort(s.begin(), s.end());
  int64_t best = 0, idx = 0;
  for (size_t i = 0; i + 1 < s.size(); i++) {
    const int64_t g = s[i + 1] - s[i];
    if (g > best) {
      idx = int64_t(i);
      best = g;
    }
  }
  return s[size_t(idx)] + int64_t(int(best) / 2);
}

// LowRankMat::ACA_FAST loop (LowRank_matrix.hpp:64-377).
void aca(const Oracle& o, const std::vector<int64_t>& rows, const std::vector<int64_t>& cols, Rng& rng,
         Block& B) {
  const double tol = o.p.eps;
  const int64_t m = int64_t(rows.size()), n = int64_t(cols.size());
  const double mn = double(std::min(m, n));
  Remaining rr(m), rc(n);
  std::vector<int64_t> row_ind, col_ind;
  std::vector<std::vector<double>> u, v;
  std::vector<double> row(static_cast<size_t>(n)), col(static_cast<size_t>(m));
  row_ind.push_back(0);
  rr.erase(0);
  double mx = 0, gamma = 0, mnorm = 0, row_norm = 0, col_norm = 0;
  int64_t pivot = 0;
  int r = 0;
  const int max_tries = 10;

  auto gen_row = [&](int64_t i) {
    for (int64_t j = 0; j < n; j++) row[size_t(j)] = entry(o, rows[size_t(i)], cols[size_t(j)]);
    for (int k = 0; k < r; k++) {
      const double a = u[size_t(k)][size_t(i)];
      for (int64_t j = 0; j < n; j++) row[size_t(j)] = row[size_t(j)] - a * v[size_t(k)][size_t(j)];
    }
  };
  auto gen_col = [&](int64_t j) {
    for (int64_t i = 0; i < m; i++) col[size_t(i)] = entry(o, rows[size_t(i)], cols[size_t(j)]);
    for (int k = 0; k < r; k++) {
      const double a = v[size_t(k)][size_t(j)];
      for (int64_t i = 0; i < m; i++) col[size_t(i)] = col[size_t(i)] - a * u[size_t(k)][size_t(i)];
    }
  };

  do {
    gen_row(row_ind.back());
    max_abs(row, rc, mx, pivot);
    int count = 0;
    bool at_end = false, use_rand = true;
    while (std::fabs(mx) < tol && count < max_tries && rc.cnt > 0 && rr.cnt > 0) {
      row_ind.pop_back();
      int64_t nr;
      if (r < 3) {
        nr = at_end ? rr.last() : rr.first();
        at_end = !at_end;
      } else {
        if (use_rand)
          nr = rr.kth(int64_t(rng.next()) % rr.cnt);
        else
          nr = gap_mid(row_ind);
        use_rand = !use_rand;
      }
      row_ind.push_back(nr);
      rr.erase(nr);
      gen_row(nr);
      max_abs(row, rc, mx, pivot);
      count++;
    }
    if (count == max_tries || rc.cnt == 0 || rr.cnt == 0) break;
    count = 0;
    col_ind.push_back(pivot);
    rc.erase(pivot);
    gamma = 1.0 / mx;
    gen_col(col_ind.back());
    max_abs(col, rr, mx, pivot);
    while (std::fabs(mx) < tol && count < max_tries && rc.cnt > 0 && rr.cnt > 0) {
      col_ind.pop_back();
      int64_t nc;
      if (col_ind.size() < 3) {
        nc = at_end ? rc.cnt : rc.first();
        at_end = !at_end;
      } else {
        if (use_rand)
          nc = rc.kth(int64_t(rng.next()) % rc.cnt);
        else
          nc = gap_mid(col_ind);
        use_rand = !use_rand;
      }
      col_ind.push_back(nc);
      rc.erase(nc);
      gen_col(nc);
      max_abs(col, rr, mx, pivot);
      count++;
    }
    row_ind.push_back(pivot);
    rr.erase(pivot);
    std::vector<double> un(static_cast<size_t>(m));
    for (int64_t i = 0; i < m; i++) un[size_t(i)] = gamma * col[size_t(i)];
    u.push_back(std::move(un));
    v.push_back(row);
    double rsq = 0.0, csq = 0.0;
    for (int64_t j = 0; j < n; j++) rsq += row[size_t(j)] * row[size_t(j)];
    row_norm = std::sqrt(rsq);
    for (int64_t i = 0; i < m; i++) csq += col[size_t(i)] * col[size_t(i)];
    col_norm = std::sqrt(csq);
    mnorm += std::fabs(gamma * gamma * rsq * csq);
    for (int k = 0; k < r; k++) {
      double du = 0.0, dv = 0.0;
      for (int64_t i = 0; i < m; i++) du += u[size_t(k)][size_t(i)] * u.back()[size_t(i)];
      for (int64_t j = 0; j < n; j++) dv += v[size_t(k)][size_t(j)] * v.back()[size_t(j)];
      mnorm += 2.0 * std::fabs(du) * std::fabs(dv);
    }
    r++;
  } while (double(int(r * (m + n))) * row_norm * col_norm > std::fabs(mx) * tol * mnorm && r < mn);

  if (r >= mn - 1) {
    // trivial full-rank representation (LowRank_matrix.hpp:348-363)
    B.dense = true;
    if (m < n) {
      B.rank = int(m);
      B.U.assign(size_t(m * m), 0.0);
      for (int64_t i = 0; i < m; i++) B.U[size_t(i * m + i)] = 1.0;
      B.V.resize(size_t(n * m));
      for (int64_t i = 0; i < m; i++)
        for (int64_t j = 0; j < n; j++) B.V[size_t(i * n + j)] = entry(o, rows[size_t(i)], cols[size_t(j)]);
    } else {
      B.rank = int(n);
      B.U.resize(size_t(m * n));
      for (int64_t j = 0; j < n; j++)
        for (int64_t i = 0; i < m; i++) B.U[size_t(j * m + i)] = entry(o, rows[size_t(i)], cols[size_t(j)]);
      B.V.assign(size_t(n * n), 0.0);
      for (int64_t j = 0; j < n; j++) B.V[size_t(j * n + j)] = 1.0;
    }
  } else {
    B.rank = r;
    B.U.resize(size_t(m * r));
    B.V.resize(size_t(n * r));
    for (int k = 0; k < r; k++) {
      std::memcpy(&B.U[size_t(k * m)], u[size_t(k)].data(), size_t(m) * sizeof(double));
      std::memcpy(&B.V[size_t(k * n)], v[size_t(k)].data(), size_t(n) * sizeof(double));
    }
  }
}

// Tree::Initialise_tree / Node::Initialize_node (HDD_tree.hpp:76-83,
// HDD_node.hpp:118-148): one ACA per (node, far partner) pair, dense blocks
// for the leaf itself and its neighbours.
void assemble(Oracle& o) {
  o.blocks.clear();
  for (size_t l = 0; l < o.lv.size(); l++)
    for (size_t k = 0; k < o.lv[l].size(); k++) {
      const TNode& me = o.lv[l][k];
      if (me.count == 0) continue;
      for (int64_t s : me.intr)
        if (o.lv[l][size_t(s)].count != 0) {
          Block b;
          b.level = int(l);
          b.t = int64_t(k);
          b.s = s;
          o.blocks.push_back(std::move(b));
        }
    }
  const int64_t nb = int64_t(o.blocks.size());
  if (o.p.rng_mode == 0) {
    Rng rng{0, 0};
    for (int64_t b = 0; b < nb; b++) {
      Block& B = o.blocks[size_t(b)];
      aca(o, o.lv[size_t(B.level)][size_t(B.t)].pts, o.lv[size_t(B.level)][size_t(B.s)].pts, rng, B);
    }
  } else {
#pragma omp parallel for schedule(dynamic, 16) num_threads(o.p.threads > 0 ? o.p.threads : 1)
    for (int64_t b = 0; b < nb; b++) {
      Block& B = o.blocks[size_t(b)];
      Rng rng{1, orc_block_seed(B.level, B.t, B.s)};
      aca(o, o.lv[size_t(B.level)][size_t(B.t)].pts, o.lv[size_t(B.level)][size_t(B.s)].pts, rng, B);
    }
  }
  const std::vector<TNode>& leaves = o.lv.back();
  o.near.assign(leaves.size(), {});
  o.near_src.assign(leaves.size(), {});
  const int64_t nl = int64_t(leaves.size());
#pragma omp parallel for schedule(dynamic, 16) num_threads(o.p.threads > 0 ? o.p.threads : 1)
  for (int64_t k = 0; k < nl; k++) {
    const TNode& me = leaves[size_t(k)];
    if (me.count == 0) continue;
    std::vector<int64_t> srcs{k};
    for (int64_t s : me.nbr)
      if (leaves[size_t(s)].count != 0) srcs.push_back(s);
    for (int64_t s : srcs) {
      const TNode& so = leaves[size_t(s)];
      std::vector<double> D(static_cast<size_t>(me.count * so.count));
      for (int64_t i = 0; i < me.count; i++)
        for (int64_t j = 0; j < so.count; j++)
          D[size_t(j * me.count + i)] = entry(o, me.pts[size_t(i)], so.pts[size_t(j)]);
      o.near[size_t(k)].push_back(std::move(D));
      o.near_src[size_t(k)].push_back(s);
    }
  }
}

// y += D x with D m x n column major (column by column, as the Eigen GEMV).
inline void gemv_acc(const double* D, int64_t m, int64_t n, const double* x, double* y) {
  for (int64_t j = 0; j < n; j++) {
    const double xj = x[j];
    for (int64_t i = 0; i < m; i++) y[i] = y[i] + D[j * m + i] * xj;
  }
}

// Tree::mat_vec (HDD_tree.hpp:86-107): gather x per node, node potentials
// (dense leaf blocks first, then every far block as U (V^T x)), then
// scatter-add the potentials level by level, node by node.
void matvec(const Oracle& o, const double* x, double* y) {
  std::vector<std::vector<std::vector<double>>> pot(o.lv.size());
  std::vector<std::vector<std::vector<double>>> chg(o.lv.size());
  for (size_t l = 0; l < o.lv.size(); l++) {
    pot[l].resize(o.lv[l].size());
    chg[l].resize(o.lv[l].size());
    for (size_t k = 0; k < o.lv[l].size(); k++) {
      const TNode& nd = o.lv[l][k];
      pot[l][k].assign(size_t(nd.count), 0.0);
      chg[l][k].resize(size_t(nd.count));
      for (int64_t i = 0; i < nd.count; i++) chg[l][k][size_t(i)] = x[nd.pts[size_t(i)]];
    }
  }
  // block index ranges per (level, node)
  std::vector<std::vector<int64_t>> bstart(o.lv.size());
  for (size_t l = 0; l < o.lv.size(); l++) bstart[l].assign(o.lv[l].size() + 1, 0);
  {
    std::vector<std::vector<int64_t>> cnt(o.lv.size());
    for (size_t l = 0; l < o.lv.size(); l++) cnt[l].assign(o.lv[l].size(), 0);
    for (const Block& B : o.blocks) cnt[size_t(B.level)][size_t(B.t)]++;
    int64_t acc = 0;
    for (size_t l = 0; l < o.lv.size(); l++)
      for (size_t k = 0; k < o.lv[l].size(); k++) {
        bstart[l][k] = acc;
        acc += cnt[l][k];
      }
  }
  const size_t leaf_l = o.lv.size() - 1;
  for (size_t l = 0; l < o.lv.size(); l++) {
    const int64_t nn = int64_t(o.lv[l].size());
#pragma omp parallel for schedule(dynamic, 16) num_threads(o.p.threads > 0 ? o.p.threads : 1)
    for (int64_t k = 0; k < nn; k++) {
      const TNode& nd = o.lv[l][size_t(k)];
      if (nd.count == 0) continue;
      std::vector<double>& P = pot[l][size_t(k)];
      std::vector<double> tmp;
      if (l == leaf_l) {
        for (size_t q = 0; q < o.near[size_t(k)].size(); q++) {
          const int64_t s = o.near_src[size_t(k)][q];
          const std::vector<double>& q_s = chg[l][size_t(s)];
          tmp.assign(size_t(nd.count), 0.0);
          gemv_acc(o.near[size_t(k)][q].data(), nd.count, int64_t(q_s.size()), q_s.data(), tmp.data());
          for (int64_t i = 0; i < nd.count; i++) P[size_t(i)] = P[size_t(i)] + tmp[size_t(i)];
        }
      }
      int64_t b = bstart[l][size_t(k)];
      for (int64_t s : nd.intr) {
        const TNode& so = o.lv[l][size_t(s)];
        if (so.count == 0) continue;
        const Block& B = o.blocks[size_t(b++)];
        const std::vector<double>& q_s = chg[l][size_t(s)];
        std::vector<double> z(static_cast<size_t>(B.rank));
        for (int c = 0; c < B.rank; c++) {
          double acc = 0.0;
          for (int64_t j = 0; j < so.count; j++) acc += B.V[size_t(c * so.count + j)] * q_s[size_t(j)];
          z[size_t(c)] = acc;
        }
        tmp.assign(size_t(nd.count), 0.0);
        gemv_acc(B.U.data(), nd.count, B.rank, z.data(), tmp.data());
        for (int64_t i = 0; i < nd.count; i++) P[size_t(i)] = P[size_t(i)] + tmp[size_t(i)];
      }
    }
  }
  for (int64_t i = 0; i < o.n; i++) y[i] = 0.0;
  for (size_t l = 0; l < o.lv.size(); l++)
    for (size_t k = 0; k < o.lv[l].size(); k++) {
      const TNode& nd = o.lv[l][k];
      for (int64_t i = 0; i < nd.count; i++) y[nd.pts[size_t(i)]] += pot[l][k][size_t(i)];
    }
}

// ---------------------------------------------------------------- GMRES
// iterSolver::GMRES (GMRES.hpp:160-305) with the real-valued plane rotations
// (:83-103,124-129) and Update (:132-146).  x holds x0 on entry.
template <typename Op>
int gmres(Op&& A, int64_t n, const double* b, double* x, int restart, int max_iter, double tol, double* resid_out) {
  auto norm = [&](const std::vector<double>& v) {
    double s = 0.0;
    for (double t : v) s += t * t;
    return std::sqrt(s);
  };
  const int m = restart;
  std::vector<double> H(static_cast<size_t>((m + 1) * m), 0.0);
  auto h = [&](int i, int j) -> double& { return H[size_t(j * (m + 1) + i)]; };
  std::vector<double> s(static_cast<size_t>(m + 1), 0.0), cs(static_cast<size_t>(m + 1), 0.0), sn(static_cast<size_t>(m + 1), 0.0);
  std::vector<double> bv(b, b + n), w(static_cast<size_t>(n)), r(static_cast<size_t>(n)), tmp(static_cast<size_t>(n));
  double normb = norm(bv);
  A(x, tmp.data());
  for (int64_t t = 0; t < n; t++) r[size_t(t)] = b[t] - tmp[size_t(t)];
  double beta = norm(r);
  if (normb == 0.0) normb = 1;
  double resid = beta / normb;
  if (resid <= tol) {
    *resid_out = resid;
    return 0;
  }
  auto rot = [](double& dx, double& dy, double c, double sgn) {
    const double t = c * dx + sgn * dy;
    dy = (-sgn) * dx + c * dy;
    dx = t;
  };
  auto gen = [](double dx, double dy, double& c, double& sg) {
    if (dy == 0.0) {
      c = 1.0;
      sg = 0.0;
    } else if (std::fabs(dy) > std::fabs(dx)) {
      const double t = dx / dy;
      sg = 1.0 / std::sqrt(1.0 + t * t);
      c = t * sg;
    } else {
      const double t = dy / dx;
      c = 1.0 / std::sqrt(1.0 + t * t);
      sg = t * c;
    }
  };
  std::vector<std::vector<double>> v(static_cast<size_t>(m + 1), std::vector<double>(static_cast<size_t>(n)));
  auto update = [&](int k) {
    std::vector<double> y(s);
    for (int i = k; i >= 0; i--) {
      y[size_t(i)] /= h(i, i);
      for (int j = i - 1; j >= 0; j--) y[size_t(j)] -= h(j, i) * y[size_t(i)];
    }
    for (int j = 0; j <= k; j++)
      for (int64_t t = 0; t < n; t++) x[t] = x[t] + v[size_t(j)][size_t(t)] * y[size_t(j)];
  };
  int j = 1;
  while (j <= max_iter) {
    const double ib = 1.0 / beta;
    for (int64_t t = 0; t < n; t++) v[0][size_t(t)] = r[size_t(t)] * ib;
    std::fill(s.begin(), s.end(), 0.0);
    s[0] = beta;
    for (int i = 0; i < m && j <= max_iter; i++, j++) {
      A(v[size_t(i)].data(), w.data());
      for (int k = 0; k <= i; k++) {
        double d = 0.0;
        for (int64_t t = 0; t < n; t++) d += w[size_t(t)] * v[size_t(k)][size_t(t)];
        h(k, i) = d;
        for (int64_t t = 0; t < n; t++) w[size_t(t)] = w[size_t(t)] - d * v[size_t(k)][size_t(t)];
      }
      h(i + 1, i) = norm(w);
      const double ih = 1.0 / h(i + 1, i);
      for (int64_t t = 0; t < n; t++) v[size_t(i + 1)][size_t(t)] = ih * w[size_t(t)];
      for (int k = 0; k < i; k++) rot(h(k, i), h(k + 1, i), cs[size_t(k)], sn[size_t(k)]);
      gen(h(i, i), h(i + 1, i), cs[size_t(i)], sn[size_t(i)]);
      rot(h(i, i), h(i + 1, i), cs[size_t(i)], sn[size_t(i)]);
      rot(s[size_t(i)], s[size_t(i + 1)], cs[size_t(i)], sn[size_t(i)]);
      resid = std::fabs(s[size_t(i + 1)]) / normb;
      if (resid < tol) {
        update(i);
        *resid_out = resid;
        return j;
      }
    }
    update(m - 1);
    A(x, tmp.data());
    for (int64_t t = 0; t < n; t++) r[size_t(t)] = b[t] - tmp[size_t(t)];
    beta = norm(r);
    resid = beta / normb;
    if (resid < tol) {
      *resid_out = resid;
      return j;
    }
  }
  *resid_out = resid;
  return max_iter;
}

double now_s() {
#ifdef _OPENMP
  return omp_get_wtime();
#else
  return 0.0;
#endif
}

}  // namespace

// ---------------------------------------------------------------- C API
extern "C" {

struct orc_params {
  int32_t ndim, nmax, dprime, kind;
  double eps, scale, diag;
  int32_t rng_mode, threads;
};

void* orc_build(const orc_params* prm, const double* pts, int64_t n, const double* lo, const double* hi,
                int32_t with_operators) {
  if (!prm || prm->ndim < 1 || prm->ndim > kMaxDim || n < 1) return nullptr;
  Oracle* o = new Oracle();
  std::memcpy(&o->p, prm, sizeof(Params));
  o->n = n;
  o->pts.assign(pts, pts + size_t(n) * size_t(prm->ndim));
  if (o->p.rng_mode == 0) std::srand(1);
  double t0 = now_s();
  try {
    build_tree(*o, lo, hi);
  } catch (const std::exception&) {
    delete o;
    return nullptr;
  }
  o->t_tree = now_s() - t0;
  if (with_operators) {
    t0 = now_s();
    assemble(*o);
    o->t_init = now_s() - t0;
  }
  return o;
}

void orc_free(void* h) { delete static_cast<Oracle*>(h); }

int64_t orc_num_levels(void* h) { return int64_t(static_cast<Oracle*>(h)->lv.size()); }
int64_t orc_level_size(void* h, int64_t l) { return int64_t(static_cast<Oracle*>(h)->lv[size_t(l)].size()); }

// sizes[0] = total nodes, [1] = total neighbour entries, [2] = total interaction entries
void orc_structure_sizes(void* h, int64_t* sizes) {
  Oracle* o = static_cast<Oracle*>(h);
  sizes[0] = sizes[1] = sizes[2] = 0;
  for (auto& L : o->lv)
    for (auto& nd : L) {
      sizes[0]++;
      sizes[1] += int64_t(nd.nbr.size());
      sizes[2] += int64_t(nd.intr.size());
    }
}

void orc_get_structure(void* h, int64_t* counts, int64_t* nbr_ptr, int64_t* nbr, int64_t* intr_ptr, int64_t* intr,
                       int64_t* leaf_perm) {
  Oracle* o = static_cast<Oracle*>(h);
  int64_t q = 0, a = 0, b = 0;
  nbr_ptr[0] = intr_ptr[0] = 0;
  for (auto& L : o->lv)
    for (auto& nd : L) {
      counts[q] = nd.count;
      for (int64_t t : nd.nbr) nbr[a++] = t;
      for (int64_t t : nd.intr) intr[b++] = t;
      nbr_ptr[q + 1] = a;
      intr_ptr[q + 1] = b;
      q++;
    }
  int64_t p = 0;
  for (auto& nd : o->lv.back())
    for (int64_t t : nd.pts) leaf_perm[p++] = t;
}

int64_t orc_num_blocks(void* h) { return int64_t(static_cast<Oracle*>(h)->blocks.size()); }

void orc_get_blocks(void* h, int64_t* level, int64_t* t, int64_t* s, int64_t* rank, int64_t* dense) {
  Oracle* o = static_cast<Oracle*>(h);
  for (size_t b = 0; b < o->blocks.size(); b++) {
    level[b] = o->blocks[b].level;
    t[b] = o->blocks[b].t;
    s[b] = o->blocks[b].s;
    rank[b] = o->blocks[b].rank;
    dense[b] = o->blocks[b].dense ? 1 : 0;
  }
}

// Copies block b's factors: U (m x rank) then V (n x rank), column major.
void orc_get_block_factors(void* h, int64_t b, double* U, double* V) {
  Oracle* o = static_cast<Oracle*>(h);
  const Block& B = o->blocks[size_t(b)];
  std::memcpy(U, B.U.data(), B.U.size() * sizeof(double));
  std::memcpy(V, B.V.data(), B.V.size() * sizeof(double));
}

void orc_matvec(void* h, const double* x, double* y) {
  Oracle* o = static_cast<Oracle*>(h);
  double t0 = now_s();
  matvec(*o, x, y);
  o->t_mv = now_s() - t0;
}

int32_t orc_gmres(void* h, const double* b, double* x, int32_t restart, int32_t max_iter, double tol,
                  double* resid) {
  Oracle* o = static_cast<Oracle*>(h);
  return gmres([&](const double* in, double* out) { matvec(*o, in, out); }, o->n, b, x, restart,
               max_iter > 0 ? max_iter : int(o->n), tol, resid);
}

// out: n_flop, max_rank, t_tree, t_init, t_matvec (Node::compute_flop_count /
// find_max_rank, HDD_node.hpp:182-220)
void orc_stats(void* h, double* out) {
  Oracle* o = static_cast<Oracle*>(h);
  double flop = 0.0;
  int64_t maxr = 0;
  const size_t leaf_l = o->lv.size() - 1;
  for (size_t k = 0; k < o->lv[leaf_l].size(); k++) {
    const TNode& nd = o->lv[leaf_l][k];
    if (nd.count == 0) continue;
    double f = double(nd.count);
    for (int64_t s : nd.nbr)
      if (o->lv[leaf_l][size_t(s)].count != 0) f += double(o->lv[leaf_l][size_t(s)].count);
    flop += f * double(nd.count);
  }
  for (const Block& B : o->blocks) {
    const int64_t m = o->lv[size_t(B.level)][size_t(B.t)].count, n = o->lv[size_t(B.level)][size_t(B.s)].count;
    flop += double(B.rank) * double(m + n);
    if (B.rank > maxr) maxr = B.rank;
  }
  out[0] = flop;
  out[1] = double(maxr);
  out[2] = o->t_tree;
  out[3] = o->t_init;
  out[4] = o->t_mv;
}

// Dense FP64 oracle: y[r] = sum_j A(rows[r], j) x_j for the listed rows
// (all rows when rows == NULL), each row summed in column order.
void orc_dense_matvec(const orc_params* prm, const double* pts, int64_t n, const double* x, const int64_t* rows,
                      int64_t nrows, double* y) {
  Oracle o;
  std::memcpy(&o.p, prm, sizeof(Params));
  o.n = n;
  o.pts.assign(pts, pts + size_t(n) * size_t(prm->ndim));
  const int64_t nr = rows ? nrows : n;
#pragma omp parallel for schedule(dynamic, 8) num_threads(prm->threads > 0 ? prm->threads : 1)
  for (int64_t r = 0; r < nr; r++) {
    const int64_t i = rows ? rows[r] : r;
    double acc = 0.0;
    for (int64_t j = 0; j < n; j++) acc += entry(o, i, j) * x[j];
    y[r] = acc;
  }
}

// GMRES restatement on the dense kernel matrix (pins against the reference's
// iterSolver on the same operator).  The dense GEMV accumulates column by
// column, as eigen_min does.
int32_t orc_dense_gmres(const orc_params* prm, const double* pts, int64_t n, const double* b, double* x,
                        int32_t restart, int32_t max_iter, double tol, double* resid) {
  Oracle o;
  std::memcpy(&o.p, prm, sizeof(Params));
  o.n = n;
  o.pts.assign(pts, pts + size_t(n) * size_t(prm->ndim));
  std::vector<double> A(static_cast<size_t>(n * n));
  for (int64_t j = 0; j < n; j++)
    for (int64_t i = 0; i < n; i++) A[size_t(j * n + i)] = entry(o, i, j);
  auto op = [&](const double* in, double* out) {
    for (int64_t i = 0; i < n; i++) out[i] = 0.0;
    gemv_acc(A.data(), n, n, in, out);
  };
  return gmres(op, n, b, x, restart, max_iter > 0 ? max_iter : int(n), tol, resid);
}

}  // extern "C"
