// Tensor-core products of the HODLR operator for 64 right-hand sides at once
// (tcgen05.cu).
//
// Vectors are "point major": entry p of a 64-column block sits at
// v[p * 64 .. p * 64 + 63], for the inputs [x | z] (tree positions, then the
// z values of the low-rank blocks) and for the FP32 output slots.  Inputs are
// stored split once: each value as a packed pair of BF16 words, the high part
// in the low half-word and the rest in the high half-word (x = hi + lo to
// about 2^-17 relative).  Each product is D (128 x N) = A (128 x K) B^T on the
// tensor cores: A holds the 64 right-hand sides' high parts (rows 0-63) and
// low parts (rows 64-127), B the factor columns (N output rows, K input
// columns in steps of 32), D the FP32 accumulator in tensor memory; the
// result is D_hi + D_lo.  BF16 factors times their input scale (BF16 dense
// tiles) are split into two BF16 terms, FP64 near-field entries into three
// (about 2^-24 relative).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "matvec.h"

namespace hodlr {

constexpr int kTcRhs = 64;     // right-hand sides per block
constexpr int kTcMaxSegs = 256;  // segments of one panel item (the host splits longer items)
// Output rows of one item: panels above 32 rows go in items of 64 rows, and z
// groups hold at most 64 rows -- so a CTA holds at most 64 tensor-memory
// columns and 8 CTAs share an SM.  Split items' partial sums are blocks of
// kTcRows rows.
constexpr int kTcRows = 64;

// kind of product: z = V^T x (one item per low-rank block), near-field panels
// (FP64 tiles), far-field panels (BF16 dense tiles and U factors)
enum TcKind { kTcZ = 0, kTcNear = 1, kTcFar = 2 };

// z = V^T x for the low-rank blocks with one source node, grouped: the
// group's rows are rows k0 .. k0 + nk - 1 of z_b for each of its entries
// (at most 256 rows in all), and its columns the source node's points.
struct TcZEntry {
  int32_t zb;      // index into the z blocks
  int32_t k0, nk;  // rows (columns of V) of z_b in this group
};
struct TcZGroup {
  int64_t x_off;   // first point of the group's columns (of the source node)
  int32_t n;       // columns: all points of the source node, or a run of at most kTcZCols of them
  int32_t e_begin, e_end;  // entries
  int32_t rows;    // sum of nk
  int32_t part;    // < 0: the group writes z; else its partial sums go to part block `part` (a fix-up adds them)
  int32_t col0;    // the first column's point within the source node (its row of V): 0 unless a column run
};
// A source node with more points than kTcZCols is split into column runs
// whose partial sums (blocks of kTcRows rows x 64) a fix-up adds into z.
constexpr int kTcZCols = 256;
struct TcZRow {        // row i of a split group: where its z goes
  int64_t zpos;
  const float* zscale;  // the row's z scale (BF16), or null
};
struct TcZFix {
  int32_t part, count;  // part blocks part .. part + count - 1
  int32_t rows, row0;   // rows, and their first entry in the TcZRow table
};

struct TcLaunch {
  uint32_t* in;     // [x | z], point major, packed BF16 pairs
  float* y;         // output slots, point major: slot s of row p at (s * n + p) * 64
  float* part;      // partial row blocks of split panels: (part * rows_per_item + i) * 64
  int64_t n;        // points (rows of one slot)
  unsigned int* status;  // wait give-ups
  // panels (near, far)
  const Panel* panels;
  const Seg* segs;
  const Item* items;
  int nitems;
  int big;          // items are 64-row chunks of panels above 32 rows
  // z products: blocks, groups by source node, group entries
  const ZBlock* zb;
  const TcZGroup* zgroups;
  const TcZEntry* zentries;
  int nz;           // groups
  int nmax;         // largest output row count of the launch's items (N before padding)
};

// One launch per kind (and small / big items); asynchronous on st.
cudaError_t launch_tc(TcKind kind, const TcLaunch& a, cudaStream_t st);
// in[p * 64 + r] = split(x[perm[p] + r * ld_x]) (x in caller order, column major FP32), p < n,
// r < nrhs (<= 64); columns r >= nrhs are zero
cudaError_t launch_tc_gather(const float* x, int64_t ld_x, int nrhs, const int64_t* perm, int64_t n, uint32_t* in,
                             cudaStream_t st);
// y_out[perm[p] + r * ld_out] = sum over slots s of y[(s * n + p) * 64 + r], r < nrhs
cudaError_t launch_tc_combine(const float* y, int nslots, int64_t n, const int64_t* perm, float* out,
                              int64_t ld_out, int nrhs, cudaStream_t st);
// z of split z groups: in[zpos * 64 + r] = zscale * sum over the group's part blocks
cudaError_t launch_tc_zfix(const TcZFix* fix, int nfix, int max_rows, const TcZRow* rows, const float* zpart,
                           uint32_t* in, cudaStream_t st);
// adds split panels' partial row blocks (kTcRows rows each) into their output rows
cudaError_t launch_tc_fix(const Panel* panels, const PanelFix* fix, int nfix, const float* part, float* y,
                          cudaStream_t st);

}  // namespace hodlr
