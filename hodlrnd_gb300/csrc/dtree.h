// The 2^d tree and its interaction lists built on the device (dtree.cu).
//
// Same rules and the same arrays, bit for bit, as the host restatement
// (tree.cpp: HODLRnD include/HDD_tree.hpp:23-74, include/HDD_clusters.hpp:
// 22-41,70-162, include/HDD_node.hpp:24-31,150-180): every level splits all
// nodes of the last level at their box midpoints; the points of a parent are
// partitioned among its children stably (one CTA per parent); child boxes,
// centres and sides are formed with the host's operations in the host's
// order (one rounding each, no contraction); and each new node's candidates
// -- its siblings, then the children of its parent's neighbours -- are split
// into neighbours and interaction partners by the reference's admissibility
// rule, counted, scanned and written in order.
//
// The level-l order of the points (each level-l node's points by increasing
// caller index) is exactly the reference order the ACA walks, so the
// reference-order map of every level falls out of the build as well.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <functional>
#include <string>

#include "tree.hpp"

namespace hodlr {

struct DeviceTreeOut {
  double* d_pts = nullptr;     // ndim x n doubles (caller's): the points in tree order, structure of arrays
  int64_t* d_perm = nullptr;   // n (caller's): tree position -> caller index
  // called once the depth is known: device memory for levels x n int32 (the
  // reference-order maps, written by the build); may be null to skip them
  std::function<int32_t*(size_t)> alloc_lmap;
  int32_t* d_lmap = nullptr;   // what alloc_lmap returned
};

// code: 0 on success, else an HODLR_ERR_* value with msg set.
struct DeviceTreeStatus {
  int code = 0;
  std::string msg;
};

// points: host, n x ndim row major (caller order).  Fills t as build_tree
// does; writes out's device arrays.  Synchronous on st.
DeviceTreeStatus build_tree_device(const TreeParams& p, const double* points, int64_t n, const double* box_lo,
                                   const double* box_hi, Tree& t, DeviceTreeOut& out, cudaStream_t st);

}  // namespace hodlr
