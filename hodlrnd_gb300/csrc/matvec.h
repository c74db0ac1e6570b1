// HODLR matvec launch interface (matvec.cu).
//
// The operator is applied in tree order in two phases:
//   phase 1: z_b = V_b^T x_s for every low-rank far block b (warp per block);
//   phase 2: for every "panel" -- the rows of one node at one level, or of one
//            leaf for the near field -- y_slot[rows] = sum over its segments of
//            M_seg * in[seg], where a segment is a dense leaf block (input x_s),
//            a far block kept dense (input x_s) or a factor U_b (input z_b).
// Each level's far panels write their own output slot and the near field
// writes slot 0, so no two warps update the same output; the slots are then
// summed in a fixed order (deterministic, no atomics).  This replaces the
// reference's serial gather / per-node GEMV / scatter-add (HODLRnD
// include/HDD_tree.hpp:86-107, include/HDD_node.hpp:82-99,223-254,
// include/LowRank_matrix.hpp:40-63).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "device.cuh"

namespace hodlr {

struct Panel {
  int64_t row_begin;  // tree position of the first row
  int64_t seg_begin, seg_end;
  int32_t m;          // rows
  int32_t slot;       // output slot
  int64_t yoff;       // offset of the first row's output in a column of the slots (slot * ld_y + row_begin
                      // for one operator; the instance's base added in a batch plan)
};

// Storage of an m x K matrix (near tiles, dense far blocks, factors U and V).
// With m <= 32 it is plain column major.  Larger matrices are read 16 bytes
// per lane, 32 lanes per warp, so they are cut into row tiles of
// tile_rows(esz) = 512 / esz rows (128 FP32, 64 FP64), each tile stored
// column major on its own with its height rounded up to a multiple of
// height_quantum(esz) rows (zero padding; 4, or 8 for BF16 so that every
// column starts on 16 bytes): a warp working on one tile then streams one
// contiguous region.
__host__ __device__ inline int64_t tile_rows(int esz) { return 512 / esz; }
__host__ __device__ inline int64_t height_quantum(int esz) { return esz < 4 ? 16 / esz : 4; }
__host__ __device__ inline int64_t tile_height(int64_t m, int64_t t, int esz) {
  const int64_t T = tile_rows(esz), q = height_quantum(esz);
  int64_t rows = m - t * T;
  if (rows > T) rows = T;
  return (rows + q - 1) / q * q;
}
__host__ __device__ inline int64_t stored_elems(int64_t m, int64_t K, int esz) {
  if (m <= 32) return m * K;
  const int64_t T = tile_rows(esz), full = m / T, rem = m - full * T, q = height_quantum(esz);
  return (full * T + (rem + q - 1) / q * q) * K;
}
__host__ __device__ inline int64_t elem_offset(int64_t i, int64_t k, int64_t m, int64_t K, int esz) {
  if (m <= 32) return k * m + i;
  const int64_t T = tile_rows(esz), t = i / T;
  return t * T * K + k * tile_height(m, t, esz) + (i - t * T);
}

struct Seg {
  const void* A;   // m x K, stored as above
  int64_t in_off;  // offset of the K inputs in the input buffer
  int32_t K;
  int32_t pad;
  const float* cscale;  // BF16 dense tiles: the K column scales (input j is multiplied by cscale[j]); else null
};

// One warp's share of phase 2: rows chunk * kRowsPerItem(prec) ... of the
// panel (all of them when m <= 32) times segments [seg_b, seg_e).  A panel
// chunk whose columns are split over several items writes partial sums
// (part >= 0: rows at ypart[part * rows_per_item]) that a fix-up pass adds
// in a fixed order; otherwise part < 0 and the item writes its output slot.
struct Item {
  int32_t panel;
  int32_t chunk;
  int32_t seg_b, seg_e;
  int32_t part;
};

// Sum of `count` partial row blocks (parts part .. part+count-1) into the
// output slot of rows chunk * rows_per_item .. of the panel.
struct PanelFix {
  int32_t panel;
  int32_t chunk;
  int32_t part;
  int32_t count;
}; 


// V factors are stored row major, n x vpad(r): each row's r values padded to a
// multiple of one 16-byte load.
__host__ __device__ inline int64_t vpad(int64_t r, int esz) {
  const int64_t c = 16 / esz;
  return (r + c - 1) / c * c;
}

struct ZBlock {
  const void* V;   // n x vpad(r), row major
  int64_t x_off;   // tree position of the source node
  int64_t z_off;   // offset of z_b in the input buffer
  int32_t n, r;
  const float* zscale;  // BF16: the r column scales of z; else null
};

// One warp's share of phase 1: columns [k0, k0 + nk) of block zb (all of
// them for blocks with n <= 32, at most kZCols for larger ones).
struct ZItem {
  int32_t zb;
  int32_t k0, nk;  // (padded) columns k0 .. k0 + nk - 1, at most 32 loads of 16 bytes
  int32_t j0, j1;  // rows j0 .. j1 - 1
  int32_t part;    // < 0: write z; else partial sums at zpart[part + c], c < nk
  int32_t R, nst;  // items of whole rows (staged): V rows per ring stage, stage count; else 0, 0
};
// Sets R and nst of an item of block rank r stored with esz-byte elements.
void z_item_stages(ZItem& it, int r, int esz);
constexpr int kZPart = 128;          // partial-sum stride of one item (>= any nk)
// V bytes one item reads at most (when the block has that many); HODLR_TUNE_Z_ITEM_BYTES
// overrides it for tuning runs
#ifndef HODLR_TUNE_Z_ITEM_BYTES
#define HODLR_TUNE_Z_ITEM_BYTES (1 << 17)
#endif
constexpr int kZItemBytes = HODLR_TUNE_Z_ITEM_BYTES;

// z[zpos] = sum_{q < count} zpart[part + q * kZPart]
struct ZFix {
  int64_t zpos;
  int32_t part;
  int32_t count;
};

// Element types: A = stored matrix, X = vectors, ACC = accumulation.
enum class Prec { kD, kF, kB };  // double, float, bfloat16 (far-field storage only)

__host__ __device__ inline int prec_size(Prec p) { return p == Prec::kD ? 8 : p == Prec::kF ? 4 : 2; }

// Storage of one far block (m x n, rank r, or dense), 16-byte aligned pieces:
// U (or the dense tile), then for BF16 a dense tile's n FP32 column scales;
// V, then for BF16 the r FP32 column scales of z (the product of U's and V's
// column scales).  BF16 thus stores every factor per-column scaled.
__host__ __device__ inline uint64_t round16(uint64_t b) { return (b + 15) / 16 * 16; }
__host__ __device__ inline uint64_t far_u_data_bytes(int64_t m, int64_t n, int64_t r, bool dense, Prec p) {
  const int esz = prec_size(p);
  return round16(uint64_t(stored_elems(m, dense ? n : r, esz)) * uint64_t(esz));
}
__host__ __device__ inline uint64_t far_u_bytes(int64_t m, int64_t n, int64_t r, bool dense, Prec p) {
  return far_u_data_bytes(m, n, r, dense, p) + ((p == Prec::kB && dense) ? round16(uint64_t(n) * 4) : 0);
}
__host__ __device__ inline uint64_t far_v_data_bytes(int64_t n, int64_t r, bool dense, Prec p) {
  const int esz = prec_size(p);
  return dense ? 0 : round16(uint64_t(n) * uint64_t(vpad(r, esz)) * uint64_t(esz));
}
__host__ __device__ inline uint64_t far_v_bytes(int64_t n, int64_t r, bool dense, Prec p) {
  return far_v_data_bytes(n, r, dense, p) + ((p == Prec::kB && !dense) ? round16(uint64_t(r) * 4) : 0);
}

// in:   input buffer [x (ld_in rows of x) | z], nrhs columns with leading dimension ld_in
// y:    output slots, slot s of column c at y + (c * nslots + s) * ld_y
// zpart / ypart: scratch of the vector precision (one column of partials).
// acc, for FP32 matrices with FP64 vectors: the input buffer `in` holds each
// FP64 value split into an (hi, lo) FP32 pair (launch_split), z is written in
// the same form, outputs and partial sums stay FP64, and products are summed
// * kCompensated: in compensated FP32 (FP64-level accuracy on the FP32 pipe);
// * kRelaxed: in plain FP32 from the high parts (about 1e-6 relative).
// Other type pairs ignore it.
enum class Accum { kByType, kCompensated, kRelaxed };
cudaError_t launch_zgemv(Prec a, Prec x, const ZBlock* zb, const ZItem* items, int nitems, const ZFix* fix, int nfix,
                         void* zpart, void* in, int64_t ld_in, int nrhs, cudaStream_t st,
                         Accum acc = Accum::kByType);
// `small` items belong to panels of at most 32 rows, `big` ones to larger panels.
// contig: every small item's segments lie in memory in segment order, each
// after the end of the previous one (small_items_contiguous), so that the
// item's factors can be streamed as one byte run.
cudaError_t launch_panels(Prec a, Prec x, const Panel* panels, const Seg* segs, const Item* small, int nsmall,
                          const Item* big, int nbig, const PanelFix* fix, int nfix, void* ypart, const void* in,
                          int64_t ld_in, void* y, int64_t ld_y, int nslots, int nrhs, cudaStream_t st,
                          Accum acc = Accum::kByType, bool contig = false);
// Whether the segments of every small item (panels of at most 32 rows) with
// esz-byte elements follow one another in memory, as launch_panels' contig asks.
bool small_items_contiguous(const std::vector<Panel>& panels, const std::vector<Seg>& segs,
                            const std::vector<Item>& small, int esz);
// Copy of `bytes` (a multiple of 16) from src to dst, both 16-byte aligned.
struct CopyDesc {
  const void* src;
  void* dst;
  uint64_t bytes;
};
cudaError_t launch_copy16(const CopyDesc* d, int n, cudaStream_t st);
// rows x row_bytes from src (rows src_pitch bytes apart) to dst (dst_pitch
// apart); row_bytes, the pitches and both addresses multiples of 16 bytes.
struct RowCopy {
  const void* src;
  void* dst;
  int64_t src_pitch, dst_pitch;
  int32_t row_bytes, rows;
};
cudaError_t launch_copy_rows(const RowCopy* d, int n, cudaStream_t st);

// One instance of a batch of operators: its n rows sit at x_base in the
// caller's concatenated vectors, at in_base in the batch's input buffer and
// at y_base in the batch's output slots (nslots slots of n rows each).
struct BatchInst {
  int64_t n, x_base, in_base, y_base;
  const int64_t* perm;  // tree position -> caller index within the instance
  int32_t nslots, pad;
};
// in[in_base + r] = x[x_base + perm[r]] for every instance (vectors of type x)
cudaError_t launch_batch_gather(Prec x, const BatchInst* inst, int count, int64_t max_n, const void* src, void* in,
                                cudaStream_t st);
// out[x_base + perm[r]] = sum over the instance's slots s of y[y_base + s n + r]
cudaError_t launch_batch_combine(Prec x, const BatchInst* inst, int count, int64_t max_n, const void* y, void* out,
                                 cudaStream_t st);

// ---- several right-hand sides: FP32 factors and vectors ---------------------
// A chunk of kMR right-hand sides is stored interleaved: entry e of a vector
// buffer holds the chunk's kMR values at e * kMR .. e * kMR + kMR - 1.
// Buffers hold nchunks chunks of ld entries each (grid.y runs over chunks);
// zpart / ypart hold zpart_ld / ypart_ld entries per chunk.
constexpr int kMR = 32;
cudaError_t launch_zgemv_mr(const ZBlock* zb, const ZItem* items, int nitems, const ZFix* fix, int nfix, float* zpart,
                            int64_t zpart_ld, float* in, int64_t ld_in, int nchunks, cudaStream_t st);
// output slots: ld_y entries per chunk, panel rows at P.yoff
cudaError_t launch_panels_mr(const Panel* panels, const Seg* segs, const Item* small, int nsmall, const Item* big,
                             int nbig, const PanelFix* fix, int nfix, float* ypart, int64_t ypart_ld, const float* in,
                             int64_t ld_in, float* y, int64_t ld_y, int nchunks, cudaStream_t st);
// x, out: caller order, column major total_n x k (FP32); chunk ch holds columns ch*kMR ..
cudaError_t launch_batch_gather_mr(const BatchInst* inst, int count, int64_t max_n, const float* x, int64_t total_n,
                                   int k, float* in, int64_t ld_in, int nchunks, cudaStream_t st);
cudaError_t launch_batch_combine_mr(const BatchInst* inst, int count, int64_t max_n, const float* y, int64_t ld_y,
                                    float* out, int64_t total_n, int k, int nchunks, cudaStream_t st);

// out[i] = (hi, lo) FP32 pair of x[i] (hi = x rounded to FP32, lo = the rest)
cudaError_t launch_split(const double* x, void* out, int64_t n, cudaStream_t st);

// Copies to `host` (pinned) the number of times a streaming kernel on this
// device gave up waiting for its bulk copies since the library was loaded
// (every wait is bounded); the value is valid once `st` has synchronised.
cudaError_t read_stream_timeouts(unsigned int* host, cudaStream_t st);
// rows handled by one big-panel item for stored element size `a`
inline int rows_per_item(Prec a) { return int(tile_rows(prec_size(a))); }
// out[perm[i] + c*ld_out] (or out[i + c*ld_out] when perm == NULL) =
//   sum_s y[(c*nslots + s)*ld_y + i], i < n
cudaError_t launch_combine(Prec x, const void* y, int64_t ld_y, int nslots, int64_t n, int nrhs, const int64_t* perm,
                           void* out, Prec out_prec, int64_t ld_out, cudaStream_t st);
// dst[i + c*ld_dst] = src[perm[i] + c*ld_src] (perm == NULL: identity), converting precision
cudaError_t launch_gather(const void* src, Prec sp, int64_t ld_src, const int64_t* perm, int64_t n, int nrhs, void* dst,
                          Prec dp, int64_t ld_dst, cudaStream_t st);

// Dense blocks from the kernel: tile t is out + off[t], m x n stored as above
// (the caller zeroes the padding), A(t_begin + i, s_begin + j).
struct TileDesc {
  int64_t t_begin, s_begin;
  int64_t off;  // element offset in the output array
  int32_t m, n;
};
cudaError_t launch_assemble(int ndim, const PointsDev& P, const KernelDev& K, const TileDesc* tiles, int ntiles,
                            void* out, Prec op, cudaStream_t st);

// Far-block compaction after ACA: for each listed block copy U (m x rank) and
// V (n x rank) out of its ACA workspace (FP64) into u_dst/v_dst in the stored
// precision and layout, or, for a block kept dense, evaluate its m x n block
// into u_dst (the caller zeroes the padding).
struct CompactDesc {
  int64_t t_begin, s_begin;
  int64_t t_map, s_map;  // offsets of the nodes' reference-order maps (low-rank blocks)
  int64_t ws;         // ACA workspace offset (doubles)
  void* u_dst;        // U or the dense tile
  void* v_dst;        // V (unused for dense blocks)
  int32_t m, n, rank, dense;
  int32_t cap;        // workspace columns (V starts after m * cap doubles)
  int32_t pad;
  double kscale;      // kernel scale for a dense block's entries; 0: the launch's K.scale
  float* s_dst;       // BF16: column scales of a dense tile, or z column scales of a low-rank block
  void* u64_dst;      // FP32 launches: the FP64 copy of U or of the dense tile as well (null: none)
  void* v64_dst;      // and of V
};
// U row i (reference order) lands on tree row lmap[t_map + i] - t_begin; V likewise.
cudaError_t launch_compact(int ndim, const PointsDev& P, const KernelDev& K, const double* ws, const int32_t* lmap,
                           const CompactDesc* blocks, int nblocks, Prec op, cudaStream_t st);
// Loads the compaction kernels (before launches that overlap running kernels:
// with lazy module loading a first launch would wait for those).
cudaError_t compact_preload(int ndim);

}  // namespace hodlr
