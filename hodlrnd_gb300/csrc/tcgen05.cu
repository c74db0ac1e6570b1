// Tensor-core (tcgen05) kernels of the engine, and the self-test of the
// operand layouts and descriptors they rely on (umma.cuh).
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/hodlrnd.h"
#include "device.cuh"
#include "tc.h"
#include "umma.cuh"

namespace hodlr {
void set_thread_error(const std::string& msg);  // engine.cu: hodlr_last_error(NULL)
}

namespace hodlr {
namespace {

// D (128 x N, FP32, row major) = A (128 x K) B^T (B: N x K), both BF16 row
// major in global memory: staged into shared memory in the K-major core-matrix
// layout, multiplied by K / 16 tcgen05.mma steps into tensor memory, read
// back by the four warps.  One CTA of 128 threads.
__global__ void __launch_bounds__(128) tc_selftest_kernel(const uint16_t* __restrict__ A,
                                                          const uint16_t* __restrict__ B, int N, int K,
                                                          uint32_t ncols, float* __restrict__ D,
                                                          unsigned int* __restrict__ status) {
  extern __shared__ __align__(1024) unsigned char tsm[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(tsm);
  uint32_t* slot = reinterpret_cast<uint32_t*>(tsm + 16);
  unsigned char* sa = tsm + 1024;
  unsigned char* sb = sa + 128 * K * 2;
  const int KG = K / 8;
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  for (int e = t; e < 128 * K; e += 128)
    *reinterpret_cast<uint16_t*>(sa + umma_kmajor_offset(uint32_t(e / K), uint32_t(e % K), uint32_t(KG))) = A[e];
  for (int e = t; e < N * K; e += 128)
    *reinterpret_cast<uint16_t*>(sb + umma_kmajor_offset(uint32_t(e / K), uint32_t(e % K), uint32_t(KG))) = B[e];
  if (t == 0) {
    mbar_init(bar, 1u);
    fence_mbar_init();
  }
  if (warp == 0) {
    tmem_alloc(slot, ncols);
    tmem_relinquish();
  }
  fence_proxy_async();  // the operands, written by this thread, visible to the tensor core
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *slot;
  if (t == 0) {
    const uint32_t idesc = umma_idesc_bf16(128, N);
    for (int s = 0; s < K / 16; s++)
      umma_bf16(tmem, umma_desc(sa + 256 * s, 128, uint32_t(KG) * 128),
                umma_desc(sb + 256 * s, 128, uint32_t(KG) * 128), idesc, s > 0 ? 1u : 0u);
    umma_commit(bar);
  }
  const bool ok = __syncthreads_and(mbar_wait(bar, 0u) ? 1 : 0);
  tc_fence_after();
  if (ok) {
    for (int c = 0; c < N; c += 16) {
      float v[16];
      tmem_ld16(tmem + (uint32_t(warp * 32) << 16) + uint32_t(c), v);
#pragma unroll
      for (int q = 0; q < 16; q++) D[int64_t(warp * 32 + lane) * N + c + q] = v[q];
    }
  } else if (t == 0) {
    atomicAdd(status, 1u);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, ncols);
}

// ---- HODLR products for 64 right-hand sides (tc.h) ------------------------
//
// One CTA of 128 threads works through items (persistent: item it, it +
// gridDim.x, ...).  An item is an output-row chunk (rows <= 64) and a
// sequence of input columns -- all columns of its segments, in order; for a
// z item, the rows of V.  Columns go in steps of 16: per step the CTA writes
// the A tile (the 16 columns' inputs for 64 right-hand sides, split hi / lo)
// and one or three B tiles (the columns' factor entries of the item's rows)
// into one of two shared-memory buffers, and thread 0 issues the MMAs into
// the item's tensor-memory accumulator and commits them to the buffer's
// mbarrier; the buffer is rewritten two steps later, after that mbarrier.
// Every wait is bounded (2 s): a give-up is counted in *status, the CTA
// finishes its item without the missing products, frees its tensor memory
// and returns.

constexpr int kTcThreads = 128;
constexpr int kStepK = 32;               // columns per step (two MMAs of K = 16)
constexpr int kTcA = 128 * kStepK * 2;  // bytes of one A tile (128 rows x kStepK BF16)

template <int KIND>
struct TcB;
template <>
struct TcB<kTcZ> {
  using T = uint16_t;
  static constexpr int kTerms = 1;
};
template <>
struct TcB<kTcFar> {
  using T = uint16_t;
  static constexpr int kTerms = 2;  // the entry times its input scale, in two BF16 terms
};
template <>
struct TcB<kTcNear> {
  using T = double;
  static constexpr int kTerms = 3;
};

// shared memory of a CTA for items of at most nmax rows
__host__ __device__ constexpr int tc_npad(int rows) { return (rows + 15) / 16 * 16; }
template <int KIND>
__host__ __device__ constexpr int tc_buf_bytes(int npad) {
  return kTcA + TcB<KIND>::kTerms * npad * kStepK * 2;
}
struct TcRow {  // z groups: one output row
  const uint16_t* v;  // V_b + k: entry j (column j) at v[j * vp]
  int64_t zpos;       // z position of the row
  float zscale;
  int32_t vp;
};
// panel items: the segments' first columns (kTcMaxSegs + 1 of them), then the
// segment records; z groups: the rows
constexpr int kTcStartBytes = (kTcMaxSegs + 1 + 31) / 32 * 32 * 4;
constexpr int kTcPanelTable = kTcStartBytes + kTcMaxSegs * int(sizeof(Seg));
template <int KIND>
__host__ __device__ constexpr int tc_table_bytes() {
  return KIND == kTcZ ? kTcRows * int(sizeof(TcRow)) : kTcPanelTable;
}
template <int KIND>
__host__ __device__ constexpr int tc_smem_bytes(int npad) {
  // header (barriers, tensor-memory slot, step table), the item's table, two buffers
  return 1024 + tc_table_bytes<KIND>() + 2 * tc_buf_bytes<KIND>(npad);
}

struct TcCol {
  const void* ptr;  // the column's entry of the item's first row (rows follow contiguously)
  int64_t pos;      // input position
  float scale;      // input scale (BF16 dense tiles), else 1
  int32_t valid;
};

template <int KIND>
__global__ void __launch_bounds__(kTcThreads) tc_kernel(TcLaunch a, int npad_max, uint32_t tcols) {
  using TB = typename TcB<KIND>::T;
  constexpr int kTerms = TcB<KIND>::kTerms;
  extern __shared__ __align__(1024) unsigned char tsm[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(tsm);        // 2 buffers
  uint32_t* slot = reinterpret_cast<uint32_t*>(tsm + 16);  // tensor-memory address
  TcCol* tab = reinterpret_cast<TcCol*>(tsm + 64);         // kStepK columns of the step being written
  int32_t* cstart = reinterpret_cast<int32_t*>(tsm + 1024);  // first column of each segment of the item
  Seg* sseg = reinterpret_cast<Seg*>(tsm + 1024 + kTcStartBytes);  // the item's segment records
  TcRow* zrow = reinterpret_cast<TcRow*>(tsm + 1024);        // z groups: the rows
  unsigned char* buf0 = tsm + 1024 + tc_table_bytes<KIND>();
  const int bufb = tc_buf_bytes<KIND>(npad_max);
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int nitems = KIND == kTcZ ? a.nz : a.nitems;
  if (t == 0) {
    mbar_init(bar, 1u);
    mbar_init(bar + 1, 1u);
    fence_mbar_init();
  }
  if (warp == 0) {
    tmem_alloc(slot, tcols);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *slot;
  uint32_t commits[2] = {0u, 0u};  // commits so far per buffer (phase of its next completion)
  bool alive = true;               // false after a wait gave up
  for (int item = blockIdx.x; item < nitems && alive; item += gridDim.x) {
    // ---- the item: rows, output, columns
    int rows, nseg = 1, qb = 0;
    int64_t C;
    int64_t out_base = 0;  // output row 0: index (in 64-entry rows) into y or part (panels)
    float* outp = nullptr;
    int row0 = 0, tile = 0, m = 0;
    int64_t zx = 0;
    int zpart = -1;
    if constexpr (KIND == kTcZ) {
      const TcZGroup G = a.zgroups[item];
      rows = G.rows;
      C = G.n;
      zx = G.x_off;
      zpart = G.part;
      out_base = 0;  // rows carry their z positions
      // row table: entry e covers rows re .. re + nk - 1 (prefix over entries by warp 0)
      const int ne = G.e_end - G.e_begin;  // <= kTcRows: every entry has a row
      if (warp == 0) {
        int32_t run = 0;
        for (int w0 = 0; w0 < ne; w0 += 32) {
          const int e = w0 + lane;
          int32_t k = e < ne ? a.zentries[G.e_begin + e].nk : 0;
          int32_t incl = k;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const int32_t v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
          }
          if (e < ne) cstart[e] = run + incl - k;  // shares the row table's space: rows are written after
          run += __shfl_sync(0xffffffffu, incl, 31);
        }
      }
      __syncthreads();
      TcRow rw[1];
      int nr = 0;
      for (int i = t; i < rows && nr < 1; i += kTcThreads, nr++) {
        int lo = 0, hi = ne - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (cstart[mid] <= i) lo = mid;
          else hi = mid - 1;
        }
        const TcZEntry E = a.zentries[G.e_begin + lo];
        const ZBlock Z = a.zb[E.zb];
        const int k = E.k0 + (i - cstart[lo]);
        rw[nr].vp = int32_t(vpad(Z.r, 2));
        rw[nr].v = static_cast<const uint16_t*>(Z.V) + int64_t(G.col0) * rw[nr].vp + k;  // V row col0, column k
        rw[nr].zpos = Z.z_off + k;
        rw[nr].zscale = Z.zscale ? __ldg(Z.zscale + k) : 1.f;
      }
      __syncthreads();  // the entry starts are read; the rows overwrite them
      nr = 0;
      for (int i = t; i < rows && nr < 1; i += kTcThreads, nr++) zrow[i] = rw[nr];
      __syncthreads();
    } else {
      const Item I = a.items[item];
      const Panel P = a.panels[I.panel];
      m = P.m;
      // big panels: rows row0 .. row0 + 63, inside one storage tile (its rows a multiple of 64)
      row0 = a.big ? I.chunk * kTcRows : 0;
      tile = int(row0 / tile_rows(int(sizeof(TB))));
      rows = a.big ? min(kTcRows, m - row0) : m;
      qb = I.seg_b;
      nseg = I.seg_e - I.seg_b;
      if (I.part < 0) {
        outp = a.y;
        out_base = P.yoff + row0;
      } else {
        outp = a.part;
        out_base = int64_t(I.part) * kTcRows;
      }
      // column starts of the segments (exclusive prefix sum), 32 at a time by warp 0
      if (warp == 0) {
        int32_t run = 0;
        for (int w0 = 0; w0 < nseg; w0 += 32) {
          const int q = w0 + lane;
          int32_t k = q < nseg ? a.segs[qb + q].K : 0;
          int32_t incl = k;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const int32_t v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
          }
          if (q < nseg) cstart[q] = run + incl - k;
          run += __shfl_sync(0xffffffffu, incl, 31);
        }
        if (lane == 0) cstart[nseg] = run;  // total (nseg <= kTcMaxSegs: host-checked)
      }
      for (int q = t; q < nseg; q += kTcThreads) sseg[q] = a.segs[qb + q];
      __syncthreads();
      C = cstart[nseg];
    }
    // the host gives every item at least one row and one column; an empty one is skipped
    if (rows <= 0) {
      __syncthreads();
      continue;
    }
    const int npad = tc_npad(rows);
    const uint32_t idesc = umma_idesc_bf16(128, npad);
    const int nsteps = int((C + kStepK - 1) / kStepK);
    for (int s = 0; s < nsteps && alive; s++) {
      const int b = s & 1;
      unsigned char* sa = buf0 + b * bufb;
      unsigned char* sb = sa + kTcA;
      // the buffer's previous MMAs (two steps ago, or of an earlier item) must be done
      if (commits[b] > 0) {
        const bool ok = __syncthreads_and(mbar_wait(bar + b, (commits[b] - 1u) & 1u) ? 1 : 0);
        if (!ok) {
          if (t == 0) atomicAdd(a.status, 1u);
          alive = false;
          break;
        }
        tc_fence_after();
      }
      // step table: column c = kStepK s + t of the item (threads 0 .. kStepK - 1)
      if (t < kStepK) {
        const int64_t c = int64_t(s) * kStepK + t;
        TcCol col{nullptr, 0, 1.f, 0};
        if (c < C) {
          col.valid = 1;
          if constexpr (KIND == kTcZ) {
            col.pos = zx + c;
          } else {
            // the last segment whose first column is <= c
            int lo = 0, hi = nseg - 1;
            while (lo < hi) {
              const int mid = (lo + hi + 1) >> 1;
              if (cstart[mid] <= c) lo = mid;
              else hi = mid - 1;
            }
            const Seg& S = sseg[lo];
            const int j = int(c - cstart[lo]);
            col.pos = S.in_off + j;
            if (S.cscale) col.scale = __ldg(S.cscale + j);
            const TB* A = static_cast<const TB*>(S.A);
            if (a.big) {
              const int esz = int(sizeof(TB));
              const int64_t T = tile_rows(esz), h = tile_height(m, tile, esz);
              col.ptr = A + int64_t(tile) * T * S.K + int64_t(j) * h + (row0 - int64_t(tile) * T);
            } else {
              col.ptr = A + int64_t(j) * m;
            }
          }
        }
        tab[t] = col;
      }
      __syncthreads();
      // A: thread t -> right-hand side r = t & 63, columns 16 h .. 16 h + 15 (h = t >> 6) from the
      // packed inputs (BF16 high part in the low half-word): high parts at row r, low parts at r + 64
      {
        const int r = t & 63, h = t >> 6;
        uint32_t w[16];
#pragma unroll
        for (int u = 0; u < 16; u++) {
          const TcCol& col = tab[16 * h + u];
          w[u] = col.valid ? a.in[col.pos * kTcRhs + r] : 0u;
        }
#pragma unroll
        for (int g = 0; g < 2; g++) {
          uint32_t hw[4], lw[4];
#pragma unroll
          for (int u = 0; u < 4; u++) {
            hw[u] = __byte_perm(w[8 * g + 2 * u], w[8 * g + 2 * u + 1], 0x5410);
            lw[u] = __byte_perm(w[8 * g + 2 * u], w[8 * g + 2 * u + 1], 0x7632);
          }
          const uint32_t k = uint32_t(16 * h + 8 * g);
          *reinterpret_cast<uint4*>(sa + umma_kmajor_offset(r, k, kStepK / 8)) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
          *reinterpret_cast<uint4*>(sa + umma_kmajor_offset(r + 64, k, kStepK / 8)) =
              make_uint4(lw[0], lw[1], lw[2], lw[3]);
        }
      }
      // B: chunk (row i, column group h of 8) -> 8 entries in kTerms BF16 terms; rows >= rows and
      // invalid columns are zero.  Every load of a chunk is issued before its entries are used.
      for (int ch = t; ch < npad * (kStepK / 8); ch += kTcThreads) {
        const int i = ch % npad, h = ch / npad;
        TB raw[8];
#pragma unroll
        for (int u = 0; u < 8; u++) {
          const TcCol& col = tab[8 * h + u];
          const bool ok = col.valid && i < rows;
          if constexpr (KIND == kTcZ) {
            // column c of the group = point c of the run: row i's V entry
            const int64_t c = int64_t(s) * kStepK + 8 * h + u;
            raw[u] = ok ? zrow[i].v[c * zrow[i].vp] : TB(0);
          } else {
            raw[u] = ok ? static_cast<const TB*>(col.ptr)[i] : TB(0);
          }
        }
        uint32_t wq[kTerms][4];
#pragma unroll
        for (int u = 0; u < 8; u += 2) {
          uint16_t e[kTerms][2];
#pragma unroll
          for (int d = 0; d < 2; d++) {
            if constexpr (KIND == kTcNear) {
              // three BF16 terms of the FP64 entry: a = t0 + t1 + t2 + O(2^-24 a)
              const float f = float(raw[u + d]);
              const uint16_t t0 = bf16_bits(f);
              const float r1 = f - bf16_value(t0);
              const uint16_t t1 = bf16_bits(r1);
              e[0][d] = t0;
              e[1 % kTerms][d] = t1;
              e[2 % kTerms][d] = bf16_bits(r1 - bf16_value(t1));
            } else if constexpr (KIND == kTcFar) {
              // the stored entry times its column's input scale (BF16 dense tiles; 1 otherwise)
              // in two BF16 terms (2^-16 relative)
              const float f = bf16_value(uint16_t(raw[u + d])) * tab[8 * h + u + d].scale;
              const uint16_t t0 = bf16_bits(f);
              e[0][d] = t0;
              e[1 % kTerms][d] = bf16_bits(f - bf16_value(t0));
            } else {
              e[0][d] = uint16_t(raw[u + d]);
            }
          }
#pragma unroll
          for (int q = 0; q < kTerms; q++) wq[q][u / 2] = uint32_t(e[q][0]) | (uint32_t(e[q][1]) << 16);
        }
#pragma unroll
        for (int q = 0; q < kTerms; q++)
          *reinterpret_cast<uint4*>(sb + q * npad * (kStepK * 2) + umma_kmajor_offset(i, 8 * h, kStepK / 8)) =
              make_uint4(wq[q][0], wq[q][1], wq[q][2], wq[q][3]);
      }
      fence_proxy_async();  // this thread's operand writes, visible to the tensor core
      tc_fence_before();
      __syncthreads();
      tc_fence_after();
      if (t == 0) {
        // K-major tiles with kStepK / 8 core matrices along K: leading offset 128 B, stride kStepK * 16 B;
        // each MMA consumes 16 columns (two core matrices, 256 B further along)
#pragma unroll
        for (int k = 0; k < kStepK / 16; k++) {
          const uint64_t da = umma_desc(sa + 256 * k, 128, kStepK * 16);
#pragma unroll
          for (int q = 0; q < kTerms; q++)
            umma_bf16(tmem, da, umma_desc(sb + q * npad * (kStepK * 2) + 256 * k, 128, kStepK * 16), idesc,
                      (s > 0 || k > 0 || q > 0) ? 1u : 0u);
        }
        umma_commit(bar + b);
      }
      commits[b]++;
    }
    if (!alive) break;
    // ---- epilogue: D = D_hi (lanes 0-63) + D_lo (lanes 64-127), 16 output rows at a time
    if (nsteps > 0) {
      const int b = (nsteps - 1) & 1;
      const bool ok = __syncthreads_and(mbar_wait(bar + b, (commits[b] - 1u) & 1u) ? 1 : 0);
      if (!ok) {
        if (t == 0) atomicAdd(a.status, 1u);
        alive = false;
        break;
      }
      tc_fence_after();
    }
    float* xch = reinterpret_cast<float*>(buf0);  // 64 x 16 FP32 (the buffers are idle now)
    for (int c0 = 0; c0 < npad; c0 += 16) {
      float v[16];
      if (nsteps > 0) {
        tmem_ld16(tmem + (uint32_t(warp * 32) << 16) + uint32_t(c0), v);
      } else {
#pragma unroll
        for (int q = 0; q < 16; q++) v[q] = 0.f;
      }
      if (warp >= 2) {
#pragma unroll
        for (int q = 0; q < 16; q++) xch[q * 64 + (t - 64)] = v[q];
      }
      __syncthreads();
      if (warp < 2) {
#pragma unroll
        for (int q = 0; q < 16; q++) {
          const int i = c0 + q;
          if (i < rows) {
            const float val = v[q] + xch[q * 64 + t];
            if constexpr (KIND == kTcZ) {
              if (zpart < 0)
                a.in[zrow[i].zpos * kTcRhs + t] = split_pack(val * zrow[i].zscale);
              else  // a column run of a split group: unscaled partial sums
                a.part[(int64_t(zpart) * kTcRows + i) * kTcRhs + t] = val;
            } else
              outp[(out_base + i) * kTcRhs + t] = val;
          }
        }
      }
      __syncthreads();
    }
    tc_fence_before();
  }
  // drain: the MMAs still in flight on either buffer (bounded), then free tensor memory
  for (int b = 0; b < 2; b++)
    if (commits[b] > 0) mbar_wait(bar + b, (commits[b] - 1u) & 1u);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tmem, tcols);
}

__global__ void tc_gather_kernel(const float* __restrict__ x, int64_t ld_x, int nrhs, const int64_t* __restrict__ perm,
                                 int64_t n, uint32_t* __restrict__ in) {
  const int64_t total = n * kTcRhs;
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < total; e += int64_t(gridDim.x) * blockDim.x) {
    const int64_t p = e / kTcRhs;
    const int r = int(e % kTcRhs);
    in[e] = split_pack(r < nrhs ? x[perm[p] + int64_t(r) * ld_x] : 0.f);
  }
}

__global__ void tc_combine_kernel(const float* __restrict__ y, int nslots, int64_t n, const int64_t* __restrict__ perm,
                                  float* __restrict__ out, int64_t ld_out, int nrhs) {
  const int64_t total = n * kTcRhs;
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < total; e += int64_t(gridDim.x) * blockDim.x) {
    const int64_t p = e / kTcRhs;
    const int r = int(e % kTcRhs);
    if (r >= nrhs) continue;
    float v = 0.f;
    for (int s = 0; s < nslots; s++) v += y[int64_t(s) * total + e];
    out[perm[p] + int64_t(r) * ld_out] = v;
  }
}

__global__ void tc_zfix_kernel(const TcZFix* __restrict__ fix, int nfix, int max_rows,
                               const TcZRow* __restrict__ rows, const float* __restrict__ zpart, uint32_t* __restrict__ in) {
  const int64_t total = int64_t(nfix) * max_rows * kTcRhs;
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < total; e += int64_t(gridDim.x) * blockDim.x) {
    const int f = int(e / (int64_t(max_rows) * kTcRhs));
    const int i = int((e / kTcRhs) % max_rows), r = int(e % kTcRhs);
    const TcZFix F = fix[f];
    if (i >= F.rows) continue;
    float v = 0.f;
    for (int q = 0; q < F.count; q++) v += zpart[(int64_t(F.part + q) * kTcRows + i) * kTcRhs + r];
    const TcZRow R = rows[F.row0 + i];
    in[R.zpos * kTcRhs + r] = split_pack(R.zscale ? v * *R.zscale : v);
  }
}

// One CTA per split item chunk: its rows x 64 sums of the partial blocks.
__global__ void tc_fix_kernel(const Panel* __restrict__ panels, const PanelFix* __restrict__ fix,
                              const float* __restrict__ part, float* __restrict__ y) {
  const PanelFix F = fix[blockIdx.x];
  const Panel P = panels[F.panel];
  const int row0 = P.m > 32 ? F.chunk * kTcRows : 0;
  const int rows = min(kTcRows, P.m - row0);
  for (int e = threadIdx.x; e < rows * kTcRhs; e += blockDim.x) {
    const int i = e / kTcRhs, r = e % kTcRhs;
    float v = 0.f;
    for (int q = 0; q < F.count; q++) v += part[(int64_t(F.part + q) * kTcRows + i) * kTcRhs + r];
    y[(P.yoff + row0 + i) * kTcRhs + r] = v;
  }
}

}  // namespace

template <int KIND>
static cudaError_t launch_tc_k(const TcLaunch& a, cudaStream_t st) {
  const int nitems = KIND == kTcZ ? a.nz : a.nitems;
  if (nitems <= 0) return cudaSuccess;
  const int npad = tc_npad(a.nmax);
  if (npad < 16 || npad > kTcRows) return cudaErrorInvalidValue;
  uint32_t tcols = 32;
  while (tcols < uint32_t(npad)) tcols <<= 1;
  const int smem = tc_smem_bytes<KIND>(npad);
  cudaError_t e = cudaFuncSetAttribute(tc_kernel<KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0, smem_sm = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess ||
      (e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess ||
      (e = cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev)) != cudaSuccess)
    return e;
  // resident CTAs per SM: threads (2048 / 128), shared memory (1 KB reserved
  // per CTA), and tensor memory (512 columns per SM shared by the CTAs)
  const int per_sm = std::max(1, std::min({2048 / kTcThreads, smem_sm / (smem + 1024), int(512 / tcols)}));
  const int grid = std::min(nitems, sms * per_sm);
  count_launches(1);
  tc_kernel<KIND><<<grid, kTcThreads, smem, st>>>(a, npad, tcols);
  return cudaGetLastError();
}

cudaError_t launch_tc(TcKind kind, const TcLaunch& a, cudaStream_t st) {
  switch (kind) {
    case kTcZ: return launch_tc_k<kTcZ>(a, st);
    case kTcNear: return launch_tc_k<kTcNear>(a, st);
    case kTcFar: return launch_tc_k<kTcFar>(a, st);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_tc_gather(const float* x, int64_t ld_x, int nrhs, const int64_t* perm, int64_t n, uint32_t* in,
                             cudaStream_t st) {
  count_launches(1);
  tc_gather_kernel<<<1216, 256, 0, st>>>(x, ld_x, nrhs, perm, n, in);
  return cudaGetLastError();
}

cudaError_t launch_tc_combine(const float* y, int nslots, int64_t n, const int64_t* perm, float* out, int64_t ld_out,
                              int nrhs, cudaStream_t st) {
  count_launches(1);
  tc_combine_kernel<<<1216, 256, 0, st>>>(y, nslots, n, perm, out, ld_out, nrhs);
  return cudaGetLastError();
}

cudaError_t launch_tc_zfix(const TcZFix* fix, int nfix, int max_rows, const TcZRow* rows, const float* zpart,
                           uint32_t* in, cudaStream_t st) {
  if (nfix <= 0) return cudaSuccess;
  count_launches(1);
  tc_zfix_kernel<<<1216, 256, 0, st>>>(fix, nfix, max_rows, rows, zpart, in);
  return cudaGetLastError();
}

cudaError_t launch_tc_fix(const Panel* panels, const PanelFix* fix, int nfix, const float* part, float* y,
                          cudaStream_t st) {
  if (nfix <= 0) return cudaSuccess;
  count_launches(1);
  tc_fix_kernel<<<nfix, 256, 0, st>>>(panels, fix, part, y);
  return cudaGetLastError();
}

}  // namespace hodlr

extern "C" int hodlr_tc_selftest(const uint16_t* A, const uint16_t* B, int32_t n, int32_t k, float* D) {
  using namespace hodlr;
  if (!A || !B || !D) {
    set_thread_error("hodlr_tc_selftest: null argument");
    return HODLR_ERR_INVALID;
  }
  if (n < 16 || n > 256 || n % 16 != 0 || k < 16 || k > 128 || k % 16 != 0) {
    set_thread_error("hodlr_tc_selftest: n must be a multiple of 16 in 16..256, k a multiple of 16 in 16..128");
    return HODLR_ERR_INVALID;
  }
  uint32_t ncols = 32;
  while (ncols < uint32_t(n)) ncols <<= 1;
  uint16_t *dA = nullptr, *dB = nullptr;
  float* dD = nullptr;
  unsigned int* dS = nullptr;
  unsigned int st = 0;
  const size_t smem = 1024 + size_t(128 + n) * size_t(k) * 2;
  cudaError_t e;
  auto done = [&](int rc, const std::string& msg) {
    cudaFree(dA);
    cudaFree(dB);
    cudaFree(dD);
    cudaFree(dS);
    if (rc != HODLR_OK) set_thread_error(msg);
    return rc;
  };
  if ((e = cudaMalloc(&dA, 128 * size_t(k) * 2)) || (e = cudaMalloc(&dB, size_t(n) * size_t(k) * 2)) ||
      (e = cudaMalloc(&dD, 128 * size_t(n) * 4)) || (e = cudaMalloc(&dS, 4)) || (e = cudaMemset(dS, 0, 4)) ||
      (e = cudaMemcpy(dA, A, 128 * size_t(k) * 2, cudaMemcpyHostToDevice)) ||
      (e = cudaMemcpy(dB, B, size_t(n) * size_t(k) * 2, cudaMemcpyHostToDevice)) ||
      (e = cudaFuncSetAttribute(tc_selftest_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem))))
    return done(HODLR_ERR_CUDA, std::string("hodlr_tc_selftest: ") + cudaGetErrorString(e));
  count_launches(1);
  tc_selftest_kernel<<<1, 128, smem>>>(dA, dB, n, k, ncols, dD, dS);
  if ((e = cudaGetLastError()) || (e = cudaDeviceSynchronize()) ||
      (e = cudaMemcpy(D, dD, 128 * size_t(n) * 4, cudaMemcpyDeviceToHost)) ||
      (e = cudaMemcpy(&st, dS, 4, cudaMemcpyDeviceToHost)))
    return done(HODLR_ERR_CUDA, std::string("hodlr_tc_selftest: ") + cudaGetErrorString(e));
  if (st != 0) return done(HODLR_ERR_DEVICE, "hodlr_tc_selftest: the MMA did not complete within the wait limit");
  return done(HODLR_OK, "");
}
