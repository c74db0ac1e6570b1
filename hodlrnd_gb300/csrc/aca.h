// Batched ACA launch interface (aca.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "device.cuh"

namespace hodlr {

enum : int32_t { kAcaDense = 1, kAcaOverflow = 2 };

// One admissible block in an ACA launch.
struct AcaBlockDesc {
  int64_t t_map, s_map;      // offsets into AcaArgs::lmap of the target (rows) and source (columns) node
  int32_t m, n;              // rows, columns
  int32_t cap;               // workspace columns
  int32_t pad;
  int64_t ws;                // offset (doubles) of U (m x cap) followed by V (n x cap)
  int64_t bits;              // offset (words) of the row bitmap followed by the column bitmap
  int64_t lists;             // offset (int32) of the used-row list (cap+2) then the used-column list (cap+2)
  uint64_t seed;             // restart-heuristic generator seed
  double kscale;             // kernel scale of this block's operator; 0: AcaArgs::K.scale (batched builds
                             // run blocks of several operators in one launch)
};

struct AcaOut {
  int32_t rank;   // rank, or min(m, n) for a block kept dense
  int32_t flags;  // kAcaDense | kAcaOverflow
};

struct AcaArgs {
  // lmap[l * n + begin + k] = tree position of the k-th point of the level-l
  // node starting at tree position `begin`, in the reference's order (points
  // of a node by increasing caller index, HDD_clusters.hpp:124-127).
  const int32_t* lmap;
  PointsDev P;
  KernelDev K;
  double tol;
  const AcaBlockDesc* blocks;
  double* ws;
  uint32_t* bits;
  int32_t* lists;
  AcaOut* out;
};

// warp_list / cta_list: indices into a.blocks compressed by one warp / one
// 256-thread CTA each.  Asynchronous on st.
cudaError_t launch_aca(int ndim, const AcaArgs& a, const int32_t* warp_list, int nwarp, const int32_t* cta_list,
                       int ncta, cudaStream_t st);

}  // namespace hodlr
