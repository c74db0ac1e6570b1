// Host-side 2^d tree (see tree.hpp).  Compiled with -ffp-contract=off: the
// box midpoints, centres and admissibility distances must round exactly as
// the reference's scalar code does, since a point on a split plane or a
// centre distance at a threshold decides the structure.
#include "tree.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace hodlr {

namespace {

void set_box(Tree& t, int64_t g, const double* lo, const double* hi) {
  const int d = t.p.ndim;
  double L = std::fabs(lo[0] - hi[0]);  // cluster ctor, HDD_clusters.hpp:25-37
  for (int k = 0; k < d; k++) {
    t.lo[size_t(g * d + k)] = lo[k];
    t.hi[size_t(g * d + k)] = hi[k];
    if (std::fabs(lo[k] - hi[k]) > L) L = std::fabs(lo[k] - hi[k]);
    t.center[size_t(g * d + k)] = 0.5 * (lo[k] + hi[k]);  // compute_cluster_center, :70-79
  }
  t.L[size_t(g)] = L;
}

// interaction_type (HDD_clusters.hpp:142-162): d - round((|c_a - c_b|_2 / L)^2)
// when that ratio is below d + 1, else -1; L is the larger box side.
int interaction_type(const Tree& t, int64_t a, int64_t b) {
  const int d = t.p.ndim;
  const double L = std::max(t.L[size_t(a)], t.L[size_t(b)]);
  const double* ca = &t.center[size_t(a * d)];
  const double* cb = &t.center[size_t(b * d)];
  double e = 0.0;
  for (int k = 0; k < d; k++) e += (ca[k] - cb[k]) * (ca[k] - cb[k]);
  double dp = std::sqrt(e) / L;
  dp *= dp;
  if (double(d) + 1 > dp) return int(double(d) - std::round(dp));
  return -1;
}

// Node::is_admissible (HDD_node.hpp:24-31): a pair is near when the max-norm
// distance of the centres is below 1.5 times the own box side and the
// interaction type exceeds d'.
bool admissible(const Tree& t, int64_t me, int64_t other) {
  const int d = t.p.ndim;
  const double* ca = &t.center[size_t(me * d)];
  const double* cb = &t.center[size_t(other * d)];
  double dist = std::fabs(ca[0] - cb[0]);
  for (int k = 0; k < d; k++) {
    const double v = std::fabs(ca[k] - cb[k]);
    if (v > dist) dist = v;
  }
  if (dist < 1.5 * t.L[size_t(me)])
    if (interaction_type(t, me, other) > t.p.dprime) return false;
  return true;
}

}  // namespace

std::string build_tree(const TreeParams& p, const double* pts, int64_t n, const double* box_lo, const double* box_hi,
                       Tree& t) {
  if (p.ndim < 1 || p.ndim > kMaxDim) return "ndim must be in 1..8";
  if (p.nmax < 1) return "nmax must be positive";
  if (p.dprime < -1 || p.dprime > p.ndim - 1) return "dprime must be in -1..ndim-1";
  if (n < 1) return "need at least one point";
  const int d = p.ndim;
  const int64_t fan = int64_t(1) << d;
  t = Tree();
  t.p = p;
  t.n = n;
  t.level_size = {1};
  t.level_off = {0, 1};
  t.begin = {0};
  t.count = {n};
  t.lo.assign(size_t(d), 0.0);
  t.hi.assign(size_t(d), 0.0);
  t.center.assign(size_t(d), 0.0);
  t.L.assign(1, 0.0);
  set_box(t, 0, box_lo, box_hi);
  t.nbr_ptr = {0, 0};
  t.intr_ptr = {0, 0};
  t.perm.resize(size_t(n));
  for (int64_t i = 0; i < n; i++) t.perm[size_t(i)] = i;

  std::vector<int64_t> next(static_cast<size_t>(n));
  std::vector<uint16_t> child_of(static_cast<size_t>(n));
  int64_t maxc = n;
  int l = 0;
  // Tree::Tree: split the whole last level while any node holds more than Nmax
  // points (HDD_tree.hpp:43-69); empty nodes are split too.
  while (maxc > p.nmax) {
    const int64_t P = t.level_size[size_t(l)];
    if (P > kMaxLevelNodes / fan)
      return "tree exceeds " + std::to_string(kMaxLevelNodes) +
             " nodes on one level (points too clustered for Nmax; the reference would run out of memory)";
    const int64_t C = P * fan;
    const int64_t poff = t.level_off[size_t(l)], coff = poff + P;
    t.level_size.push_back(C);
    t.level_off.push_back(coff + C);
    t.begin.resize(size_t(coff + C));
    t.count.resize(size_t(coff + C));
    t.lo.resize(size_t((coff + C) * d));
    t.hi.resize(size_t((coff + C) * d));
    t.center.resize(size_t((coff + C) * d));
    t.L.resize(size_t(coff + C));
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t pk = 0; pk < P; pk++) {
      const int64_t pg = poff + pk;
      double mid[kMaxDim];
      for (int k = 0; k < d; k++) mid[k] = 0.5 * (t.lo[size_t(pg * d + k)] + t.hi[size_t(pg * d + k)]);
      // children boxes: cluster::binary_clustering halves dimension 0 first,
      // so dimension 0 is the most significant bit of the child index
      for (int64_t c = 0; c < fan; c++) {
        double lo[kMaxDim], hi[kMaxDim];
        for (int k = 0; k < d; k++) {
          const bool upper = (c >> (d - 1 - k)) & 1;
          lo[k] = upper ? mid[k] : t.lo[size_t(pg * d + k)];
          hi[k] = upper ? t.hi[size_t(pg * d + k)] : mid[k];
        }
        set_box(t, coff + pk * fan + c, lo, hi);
      }
      // stable counting sort of the parent's range by child (x < mid -> lower)
      const int64_t b = t.begin[size_t(pg)], e = b + t.count[size_t(pg)];
      std::vector<int64_t> cnt(static_cast<size_t>(fan), 0);
      for (int64_t i = b; i < e; i++) {
        const double* x = &pts[size_t(t.perm[size_t(i)] * d)];
        int c = 0;
        for (int k = 0; k < d; k++) c = (c << 1) | (x[k] < mid[k] ? 0 : 1);
        child_of[size_t(i)] = uint16_t(c);
        cnt[size_t(c)]++;
      }
      int64_t acc = b;
      for (int64_t c = 0; c < fan; c++) {
        t.begin[size_t(coff + pk * fan + c)] = acc;
        t.count[size_t(coff + pk * fan + c)] = cnt[size_t(c)];
        const int64_t tmp = cnt[size_t(c)];
        cnt[size_t(c)] = acc;
        acc += tmp;
      }
      for (int64_t i = b; i < e; i++) next[size_t(cnt[child_of[size_t(i)]]++)] = t.perm[size_t(i)];
    }
    // every point lies in exactly one parent range, so next is a full permutation
    t.perm.swap(next);
    l++;

    // interaction and neighbour lists of the new level (Node::get_interaction_list,
    // HDD_node.hpp:150-180): the siblings, then the children of each of the
    // parent's neighbours, in order.
    std::vector<std::vector<int64_t>> nb(static_cast<size_t>(C)), in(static_cast<size_t>(C));
    const int64_t* pn_ptr = t.nbr_ptr.data();
    const int64_t* pn = t.nbr.data();
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t k = 0; k < C; k++) {
      const int64_t me = coff + k, pk = k / fan, pg = poff + pk;
      for (int64_t c = 0; c < fan; c++) {
        const int64_t sib = pk * fan + c;
        if (sib == k) continue;
        (admissible(t, me, coff + sib) ? in : nb)[size_t(k)].push_back(sib);
      }
      for (int64_t q = pn_ptr[pg]; q < pn_ptr[pg + 1]; q++)
        for (int64_t c = 0; c < fan; c++) {
          const int64_t o = pn[q] * fan + c;
          (admissible(t, me, coff + o) ? in : nb)[size_t(k)].push_back(o);
        }
    }
    for (int64_t k = 0; k < C; k++) {
      t.nbr.insert(t.nbr.end(), nb[size_t(k)].begin(), nb[size_t(k)].end());
      t.intr.insert(t.intr.end(), in[size_t(k)].begin(), in[size_t(k)].end());
      t.nbr_ptr.push_back(int64_t(t.nbr.size()));
      t.intr_ptr.push_back(int64_t(t.intr.size()));
    }
    maxc = 0;
    for (int64_t k = 0; k < C; k++) maxc = std::max(maxc, t.count[size_t(coff + k)]);
  }
  t.levels = l + 1;
  return "";
}

std::vector<FarBlock> far_blocks(const Tree& t) {
  std::vector<FarBlock> out;
  for (int l = 0; l < t.levels; l++)
    for (int64_t k = 0; k < t.level_size[size_t(l)]; k++) {
      const int64_t g = t.gid(l, k);
      if (t.count[size_t(g)] == 0) continue;
      for (int64_t q = t.intr_ptr[size_t(g)]; q < t.intr_ptr[size_t(g + 1)]; q++) {
        const int64_t s = t.intr[size_t(q)];
        if (t.count[size_t(t.gid(l, s))] != 0) out.push_back({l, k, s});
      }
    }
  return out;
}

NearList near_blocks(const Tree& t) {
  NearList nl;
  const int l = t.levels - 1;
  const int64_t P = t.level_size[size_t(l)];
  nl.leaf_ptr.assign(size_t(P + 1), 0);
  for (int64_t k = 0; k < P; k++) {
    const int64_t g = t.gid(l, k);
    if (t.count[size_t(g)] != 0) {
      nl.src.push_back(k);
      for (int64_t q = t.nbr_ptr[size_t(g)]; q < t.nbr_ptr[size_t(g + 1)]; q++) {
        const int64_t s = t.nbr[size_t(q)];
        if (t.count[size_t(t.gid(l, s))] != 0) nl.src.push_back(s);
      }
    }
    nl.leaf_ptr[size_t(k + 1)] = int64_t(nl.src.size());
  }
  return nl;
}

}  // namespace hodlr
