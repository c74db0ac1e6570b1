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
  int32_t lcap;              // the largest rank the pivot lists hold (0: cap); a block that may grow into
                             // the arena needs min(m, n)
  int64_t ws;                // offset (doubles) of U (m x cap) followed by V (n x cap)
  int64_t bits;              // offset (words) of the row bitmap followed by the column bitmap
  int64_t lists;             // offset (int32) of the used-row list (lcap+2) then the used-column list (lcap+2)
  uint64_t seed;             // restart-heuristic generator seed
  double kscale;             // kernel scale of this block's operator; 0: AcaArgs::K.scale (batched builds
                             // run blocks of several operators in one launch)
};

struct AcaOut {
  int32_t rank;   // rank, or min(m, n) for a block kept dense
  int32_t flags;  // kAcaDense | kAcaOverflow
  int32_t cap;    // workspace columns of the result (0: the descriptor's)
  int32_t pad;
  int64_t ws;     // offset (doubles, from AcaArgs::ws) of the result's U and V when cap != 0
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
  // Growth arena: a block whose rank reaches its workspace columns takes a
  // workspace of 4 x the columns (at most min(m, n)) from ws + arena_off on,
  // bumping *arena_used (doubles); when the arena is full it reports
  // kAcaOverflow instead.  arena_used == nullptr: no arena (overflow at once).
  int64_t arena_off;
  uint64_t arena_size;
  unsigned long long* arena_used;
  // Work queues: with queue != nullptr every team takes its next block from
  // queue[kind] (an atomic counter the caller zeroes) until the list is done,
  // and a launch has at most max_ctas CTAs.
  unsigned int* queue;
  int max_ctas;
};

// Team kinds: 8 or 16 lanes of a warp (blocks of at most 8 or 16 rows and
// columns, held in shared memory), a warp (at most 256), a 256-thread CTA.
enum : int { kAcaTeam8 = 0, kAcaTeam16 = 1, kAcaTeamWarp = 2, kAcaTeamCta = 3, kAcaTeamKinds = 4 };
// The team kind that compresses an m x n block.  The team size sets the
// order in which the norms of the stopping rule are summed, so every caller
// that must reproduce hodlr_build's factors picks teams with this.
int aca_team(int m, int n);

// list[k]: indices into a.blocks compressed by teams of kind k (n[k] of them)
struct AcaLists {
  const int32_t* list[kAcaTeamKinds];
  int n[kAcaTeamKinds];
};
// Asynchronous on st.
cudaError_t launch_aca(int ndim, const AcaArgs& a, const AcaLists& lists, cudaStream_t st);
// The team kind `kind` alone (its list in lists), asynchronous on st: the kinds
// touch disjoint blocks and may run on different streams at once.
cudaError_t launch_aca_kind(int ndim, const AcaArgs& a, const AcaLists& lists, int kind, cudaStream_t st);
// Loads the ACA kernels of points in ndim dimensions (before launches that
// should run concurrently).
cudaError_t aca_preload(int ndim);

}  // namespace hodlr
