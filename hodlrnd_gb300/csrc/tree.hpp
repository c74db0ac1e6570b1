// Host-side 2^d tree, admissibility and interaction lists.
//
// Restates the reference's clustering rules (HODLRnD include/HDD_tree.hpp:23-74,
// include/HDD_clusters.hpp:22-41,70-162, include/HDD_node.hpp:24-31,150-180)
// with a flat, level-by-level layout: points are permuted into tree order so
// that every node at every level owns a contiguous range [begin, begin+count).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace hodlr {

constexpr int kMaxDim = 8;
// Refuse trees whose widest level would hold more nodes than this (clustered
// or duplicated points can make the reference's "split while any node holds
// more than Nmax points" rule run away).
constexpr int64_t kMaxLevelNodes = int64_t(1) << 26;

struct TreeParams {
  int ndim = 2, nmax = 64, dprime = 0;
};

struct Tree {
  TreeParams p;
  int64_t n = 0;
  int levels = 0;                      // number of levels; leaves are level levels-1
  std::vector<int64_t> level_size;     // nodes per level (2^(d*l))
  std::vector<int64_t> level_off;      // first global node index of each level (size levels+1)
  std::vector<int64_t> begin, count;   // per global node: tree-order range
  std::vector<double> lo, hi, center;  // per global node, ndim each
  std::vector<double> L;               // per global node: largest box side
  std::vector<int64_t> nbr_ptr, nbr;   // per global node (CSR); entries are node ids within the level
  std::vector<int64_t> intr_ptr, intr;
  std::vector<int64_t> perm;           // tree position -> caller index

  int64_t gid(int l, int64_t k) const { return level_off[size_t(l)] + k; }
};

// Returns an empty string on success, else an error message.
std::string build_tree(const TreeParams& p, const double* pts, int64_t n, const double* box_lo, const double* box_hi,
                       Tree& t);

// A far block (target node t, source node s at one level), in the
// reference's assembly order.
struct FarBlock {
  int level;
  int64_t t, s;  // node ids within the level
};

std::vector<FarBlock> far_blocks(const Tree& t);

// Near blocks of the non-empty leaves: for each leaf (in order) itself then
// each non-empty neighbour (HDD_node.hpp:136-144,227-240).
struct NearList {
  std::vector<int64_t> leaf_ptr;  // per leaf (CSR into src)
  std::vector<int64_t> src;       // source leaf ids
};

NearList near_blocks(const Tree& t);

}  // namespace hodlr
