// HODLR matvec kernels (see matvec.h).
#include "device.cuh"
#include "matvec.h"

namespace hodlr {

namespace {

constexpr int kWarpsPerCta = 8;

template <typename T>
__device__ __forceinline__ T ldg(const T* p) {
  return __ldg(p);
}

template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
  using type = float4;
};
template <>
struct Vec16<double> {
  using type = double2;
};

template <typename TACC>
__device__ __forceinline__ TACC dot16(const float4& a, const TACC* x) {
  return TACC(a.x) * x[0] + TACC(a.y) * x[1] + TACC(a.z) * x[2] + TACC(a.w) * x[3];
}
template <typename TACC>
__device__ __forceinline__ TACC dot16(const double2& a, const TACC* x) {
  return TACC(a.x) * x[0] + TACC(a.y) * x[1];
}
__device__ __forceinline__ void axpy16(const float4& a, float s, float* acc) {
  acc[0] += a.x * s;
  acc[1] += a.y * s;
  acc[2] += a.z * s;
  acc[3] += a.w * s;
}
__device__ __forceinline__ void axpy16(const float4& a, double s, double* acc) {
  acc[0] += double(a.x) * s;
  acc[1] += double(a.y) * s;
  acc[2] += double(a.z) * s;
  acc[3] += double(a.w) * s;
}
__device__ __forceinline__ void axpy16(const double2& a, double s, double* acc) {
  acc[0] += a.x * s;
  acc[1] += a.y * s;
}

// Phase 1: z_b = V_b^T x_s.  A block with n <= 32 is one warp's item: lanes
// form groups of npad (next power of two >= n) that each take one column.  A
// larger block is split into items of up to kZCols columns; the warp strides
// over the n rows with independent accumulators per column, so a 32768-point
// block is spread over r / kZCols warps instead of one.
template <typename TA, typename TX, typename TACC>
__global__ void __launch_bounds__(256) zgemv_kernel(const ZBlock* __restrict__ zb, const ZItem* __restrict__ items,
                                                    int nitems, TX* in, int64_t ld_in) {
  const int w = blockIdx.x * kWarpsPerCta + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= nitems) return;
  const ZItem it = items[w];
  const ZBlock Z = zb[it.zb];
  const TA* V = static_cast<const TA*>(Z.V);
  const TX* x = in + blockIdx.y * ld_in + Z.x_off;
  TX* z = in + blockIdx.y * ld_in + Z.z_off;
  const int n = Z.n, r = Z.r;
  if (n <= 32) {
    int npad = 1;
    while (npad < n) npad <<= 1;
    const int slices = 32 / npad;
    const int j = lane & (npad - 1), c = lane / npad;
    const TACC xj = j < n ? TACC(x[j]) : TACC(0);
    for (int k0 = 0; k0 < r; k0 += slices) {
      const int k = k0 + c;
      TACC acc = (k < r && j < n) ? TACC(ldg(V + int64_t(k) * n + j)) * xj : TACC(0);
      for (int o = 1; o < npad; o <<= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if (j == 0 && k < r) z[k] = TX(acc);
    }
  } else {
    // 16 bytes per lane: RPL consecutive rows of kZCols columns
    constexpr int RPL = 16 / int(sizeof(TA));
    using VT = typename Vec16<TA>::type;
    const int64_t ldv = lead_dim(n);
    const int k0 = it.k0, nk = it.nk;
    TACC acc[kZCols];
#pragma unroll
    for (int c = 0; c < kZCols; c++) acc[c] = TACC(0);
    const TA* v = V + int64_t(k0) * ldv;
    for (int j = lane * RPL; j < n; j += 32 * RPL) {
      TACC xv[RPL];
#pragma unroll
      for (int q = 0; q < RPL; q++) xv[q] = (j + q < n) ? TACC(x[j + q]) : TACC(0);
#pragma unroll
      for (int c = 0; c < kZCols; c++)
        if (c < nk) {
          const VT a = __ldg(reinterpret_cast<const VT*>(v + int64_t(c) * ldv + j));
          acc[c] += dot16<TACC>(a, xv);
        }
    }
#pragma unroll
    for (int c = 0; c < kZCols; c++) {
      TACC a = acc[c];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
      if (lane == 0 && c < nk) z[k0 + c] = TX(a);
    }
  }
}

// Phase 2: one warp per (panel, 32-row chunk).
template <typename TA, typename TX, typename TACC>
__global__ void __launch_bounds__(256)
    panel_kernel(const Panel* __restrict__ panels, const Seg* __restrict__ segs, const Item* __restrict__ items,
                 int nitems, const TX* __restrict__ in, int64_t ld_in, TX* __restrict__ y, int64_t ld_y, int nslots) {
  const int w = blockIdx.x * kWarpsPerCta + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= nitems) return;
  const Item it = items[w];
  const Panel P = panels[it.panel];
  const int m = P.m;
  const TX* inc = in + blockIdx.y * ld_in;
  TX* yo = y + (int64_t(blockIdx.y) * nslots + P.slot) * ld_y + P.row_begin;
  if (m <= 32) {
    int mpad = 1;
    while (mpad < m) mpad <<= 1;
    const int slices = 32 / mpad;
    const int i = lane & (mpad - 1), sl = lane / mpad;
    TACC acc = 0;
    for (int64_t s = P.seg_begin; s < P.seg_end; s++) {
      const Seg S = segs[s];
      const TA* A = static_cast<const TA*>(S.A);
      const TX* x = inc + S.in_off;
      if (i < m) {
        int j = sl;
        TACC a1 = 0;
        for (; j + slices < S.K; j += 2 * slices) {
          acc += TACC(ldg(A + int64_t(j) * m + i)) * TACC(x[j]);
          a1 += TACC(ldg(A + int64_t(j + slices) * m + i)) * TACC(x[j + slices]);
        }
        if (j < S.K) acc += TACC(ldg(A + int64_t(j) * m + i)) * TACC(x[j]);
        acc += a1;
      }
    }
    for (int o = mpad; o < 32; o <<= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (sl == 0 && i < m) yo[i] = TX(acc);
  } else {
    // 16 bytes per lane: rows [i, i + RPL) of each column
    constexpr int RPL = 16 / int(sizeof(TA));
    using VT = typename Vec16<TA>::type;
    const int64_t ld = lead_dim(m);
    const int i = it.chunk * 32 * RPL + lane * RPL;
    const bool act = i < m;
    TACC a0[RPL], a1[RPL];
#pragma unroll
    for (int q = 0; q < RPL; q++) a0[q] = a1[q] = TACC(0);
    for (int64_t s = P.seg_begin; s < P.seg_end; s++) {
      const Seg S = segs[s];
      const TA* A = static_cast<const TA*>(S.A) + i;
      const TX* x = inc + S.in_off;
      if (act) {
        int j = 0;
        for (; j + 3 < S.K; j += 4) {
          const VT v0 = __ldg(reinterpret_cast<const VT*>(A + int64_t(j) * ld));
          const VT v1 = __ldg(reinterpret_cast<const VT*>(A + int64_t(j + 1) * ld));
          const VT v2 = __ldg(reinterpret_cast<const VT*>(A + int64_t(j + 2) * ld));
          const VT v3 = __ldg(reinterpret_cast<const VT*>(A + int64_t(j + 3) * ld));
          axpy16(v0, TACC(x[j]), a0);
          axpy16(v1, TACC(x[j + 1]), a1);
          axpy16(v2, TACC(x[j + 2]), a0);
          axpy16(v3, TACC(x[j + 3]), a1);
        }
        for (; j < S.K; j++) axpy16(__ldg(reinterpret_cast<const VT*>(A + int64_t(j) * ld)), TACC(x[j]), a0);
      }
    }
    if (act) {
#pragma unroll
      for (int q = 0; q < RPL; q++)
        if (i + q < m) yo[i + q] = TX(a0[q] + a1[q]);
    }
  }
}

template <typename TX, typename TO>
__global__ void combine_kernel(const TX* __restrict__ y, int64_t ld_y, int nslots, int64_t n,
                               const int64_t* __restrict__ perm, TO* __restrict__ out, int64_t ld_out) {
  const int c = blockIdx.y;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const TX* yc = y + int64_t(c) * nslots * ld_y + i;
    double acc = double(yc[0]);
    for (int s = 1; s < nslots; s++) acc += double(yc[int64_t(s) * ld_y]);
    out[(perm ? perm[i] : i) + c * ld_out] = TO(acc);
  }
}

template <typename TS, typename TD>
__global__ void gather_kernel(const TS* __restrict__ src, int64_t ld_src, const int64_t* __restrict__ perm, int64_t n,
                              TD* __restrict__ dst, int64_t ld_dst) {
  const int c = blockIdx.y;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    dst[i + c * ld_dst] = TD(src[(perm ? perm[i] : i) + c * ld_src]);
}

template <int D, typename TO>
__global__ void __launch_bounds__(256) assemble_kernel(PointsDev P, KernelDev K, const TileDesc* __restrict__ tiles,
                                                       int ntiles, TO* __restrict__ out) {
  const int w = blockIdx.x * kWarpsPerCta + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= ntiles) return;
  const TileDesc T = tiles[w];
  TO* o = out + T.off;
  const int64_t ld = lead_dim(T.m);
  const int64_t total = ld * T.n;
  for (int64_t e = lane; e < total; e += 32) {
    const int i = int(e % ld), j = int(e / ld);
    if (i >= T.m) {
      o[e] = TO(0);
      continue;
    }
    double xi[D];
    load_point<D>(P, T.t_begin + i, xi);
    o[e] = TO(kernel_entry<D>(P, K, T.t_begin + i, T.s_begin + j, xi));
  }
}

template <int D, typename TO>
__global__ void __launch_bounds__(256) compact_kernel(PointsDev P, KernelDev K, const double* __restrict__ ws,
                                                      const int32_t* __restrict__ lmap,
                                                      const CompactDesc* __restrict__ blocks, int nblocks) {
  const CompactDesc B = blocks[blockIdx.x];
  TO* u = static_cast<TO*>(B.u_dst);
  const int64_t ldu = lead_dim(B.m), ldv = lead_dim(B.n);
  if (B.dense) {
    const int64_t total = ldu * B.n;
    for (int64_t e = threadIdx.x; e < total; e += blockDim.x) {
      const int i = int(e % ldu), j = int(e / ldu);
      if (i >= B.m) {
        u[e] = TO(0);
        continue;
      }
      double xi[D];
      load_point<D>(P, B.t_begin + i, xi);
      u[e] = TO(kernel_entry<D>(P, K, B.t_begin + i, B.s_begin + j, xi));
    }
  } else {
    const double* U = ws + B.ws;
    for (int64_t e = threadIdx.x; e < (ldu - B.m) * B.rank; e += blockDim.x)
      u[B.m + (e % (ldu - B.m)) + (e / (ldu - B.m)) * ldu] = TO(0);
    const int64_t nu = int64_t(B.m) * B.rank;
    for (int64_t e = threadIdx.x; e < nu; e += blockDim.x) {
      const int i = int(e % B.m), k = int(e / B.m);
      u[(lmap[B.t_map + i] - B.t_begin) + int64_t(k) * ldu] = TO(U[e]);
    }
    // V follows U's full workspace (m x cap); its first rank columns are contiguous
    const double* Vw = ws + B.ws + int64_t(B.m) * B.cap;
    TO* v = static_cast<TO*>(B.v_dst);
    for (int64_t e = threadIdx.x; e < (ldv - B.n) * B.rank; e += blockDim.x)
      v[B.n + (e % (ldv - B.n)) + (e / (ldv - B.n)) * ldv] = TO(0);
    const int64_t nv = int64_t(B.n) * B.rank;
    for (int64_t e = threadIdx.x; e < nv; e += blockDim.x) {
      const int j = int(e % B.n), k = int(e / B.n);
      v[(lmap[B.s_map + j] - B.s_begin) + int64_t(k) * ldv] = TO(Vw[e]);
    }
  }
}

unsigned warps_grid(int64_t items) { return unsigned((items + kWarpsPerCta - 1) / kWarpsPerCta); }

unsigned vec_grid(int64_t n) {
  int64_t g = (n + 255) / 256;
  if (g > 152 * 8) g = 152 * 8;
  if (g < 1) g = 1;
  return unsigned(g);
}

}  // namespace

cudaError_t launch_zgemv(Prec a, Prec x, const ZBlock* zb, const ZItem* items, int nitems, void* in, int64_t ld_in,
                         int nrhs, cudaStream_t st) {
  if (nitems <= 0) return cudaSuccess;
  count_launches(1);
  dim3 g(warps_grid(nitems), unsigned(nrhs));
  if (a == Prec::kD && x == Prec::kD)
    zgemv_kernel<double, double, double><<<g, 256, 0, st>>>(zb, items, nitems, static_cast<double*>(in), ld_in);
  else if (a == Prec::kF && x == Prec::kD)
    zgemv_kernel<float, double, double><<<g, 256, 0, st>>>(zb, items, nitems, static_cast<double*>(in), ld_in);
  else if (a == Prec::kF && x == Prec::kF)
    zgemv_kernel<float, float, float><<<g, 256, 0, st>>>(zb, items, nitems, static_cast<float*>(in), ld_in);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

cudaError_t launch_panels(Prec a, Prec x, const Panel* panels, const Seg* segs, const Item* items, int nitems,
                          const void* in, int64_t ld_in, void* y, int64_t ld_y, int nslots, int nrhs,
                          cudaStream_t st) {
  if (nitems <= 0) return cudaSuccess;
  count_launches(1);
  dim3 g(warps_grid(nitems), unsigned(nrhs));
  if (a == Prec::kD && x == Prec::kD)
    panel_kernel<double, double, double><<<g, 256, 0, st>>>(panels, segs, items, nitems,
                                                            static_cast<const double*>(in), ld_in,
                                                            static_cast<double*>(y), ld_y, nslots);
  else if (a == Prec::kF && x == Prec::kD)
    panel_kernel<float, double, double><<<g, 256, 0, st>>>(panels, segs, items, nitems,
                                                           static_cast<const double*>(in), ld_in,
                                                           static_cast<double*>(y), ld_y, nslots);
  else if (a == Prec::kF && x == Prec::kF)
    panel_kernel<float, float, float><<<g, 256, 0, st>>>(panels, segs, items, nitems,
                                                         static_cast<const float*>(in), ld_in,
                                                         static_cast<float*>(y), ld_y, nslots);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

cudaError_t launch_combine(Prec x, const void* y, int64_t ld_y, int nslots, int64_t n, int nrhs, const int64_t* perm,
                           void* out, Prec out_prec, int64_t ld_out, cudaStream_t st) {
  count_launches(1);
  dim3 g(vec_grid(n), unsigned(nrhs));
  if (x == Prec::kD && out_prec == Prec::kD)
    combine_kernel<double, double><<<g, 256, 0, st>>>(static_cast<const double*>(y), ld_y, nslots, n, perm,
                                                      static_cast<double*>(out), ld_out);
  else if (x == Prec::kF && out_prec == Prec::kF)
    combine_kernel<float, float><<<g, 256, 0, st>>>(static_cast<const float*>(y), ld_y, nslots, n, perm,
                                                    static_cast<float*>(out), ld_out);
  else if (x == Prec::kF && out_prec == Prec::kD)
    combine_kernel<float, double><<<g, 256, 0, st>>>(static_cast<const float*>(y), ld_y, nslots, n, perm,
                                                     static_cast<double*>(out), ld_out);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

cudaError_t launch_gather(const void* src, Prec sp, int64_t ld_src, const int64_t* perm, int64_t n, int nrhs, void* dst,
                          Prec dp, int64_t ld_dst, cudaStream_t st) {
  count_launches(1);
  dim3 g(vec_grid(n), unsigned(nrhs));
  if (sp == Prec::kD && dp == Prec::kD)
    gather_kernel<double, double><<<g, 256, 0, st>>>(static_cast<const double*>(src), ld_src, perm, n,
                                                     static_cast<double*>(dst), ld_dst);
  else if (sp == Prec::kD && dp == Prec::kF)
    gather_kernel<double, float><<<g, 256, 0, st>>>(static_cast<const double*>(src), ld_src, perm, n,
                                                    static_cast<float*>(dst), ld_dst);
  else if (sp == Prec::kF && dp == Prec::kD)
    gather_kernel<float, double><<<g, 256, 0, st>>>(static_cast<const float*>(src), ld_src, perm, n,
                                                    static_cast<double*>(dst), ld_dst);
  else
    gather_kernel<float, float><<<g, 256, 0, st>>>(static_cast<const float*>(src), ld_src, perm, n,
                                                   static_cast<float*>(dst), ld_dst);
  return cudaGetLastError();
}

template <int D>
static void assemble_d(const PointsDev& P, const KernelDev& K, const TileDesc* tiles, int ntiles, void* out, Prec op,
                       cudaStream_t st) {
  if (op == Prec::kD)
    assemble_kernel<D, double><<<warps_grid(ntiles), 256, 0, st>>>(P, K, tiles, ntiles, static_cast<double*>(out));
  else
    assemble_kernel<D, float><<<warps_grid(ntiles), 256, 0, st>>>(P, K, tiles, ntiles, static_cast<float*>(out));
}

cudaError_t launch_assemble(int ndim, const PointsDev& P, const KernelDev& K, const TileDesc* tiles, int ntiles,
                            void* out, Prec op, cudaStream_t st) {
  if (ntiles <= 0) return cudaSuccess;
  count_launches(1);
  switch (ndim) {
    case 1: assemble_d<1>(P, K, tiles, ntiles, out, op, st); break;
    case 2: assemble_d<2>(P, K, tiles, ntiles, out, op, st); break;
    case 3: assemble_d<3>(P, K, tiles, ntiles, out, op, st); break;
    case 4: assemble_d<4>(P, K, tiles, ntiles, out, op, st); break;
    case 5: assemble_d<5>(P, K, tiles, ntiles, out, op, st); break;
    case 6: assemble_d<6>(P, K, tiles, ntiles, out, op, st); break;
    case 7: assemble_d<7>(P, K, tiles, ntiles, out, op, st); break;
    case 8: assemble_d<8>(P, K, tiles, ntiles, out, op, st); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template <int D>
static void compact_d(const PointsDev& P, const KernelDev& K, const double* ws, const int32_t* lmap,
                      const CompactDesc* blocks, int nblocks, Prec op, cudaStream_t st) {
  if (op == Prec::kD)
    compact_kernel<D, double><<<unsigned(nblocks), 256, 0, st>>>(P, K, ws, lmap, blocks, nblocks);
  else
    compact_kernel<D, float><<<unsigned(nblocks), 256, 0, st>>>(P, K, ws, lmap, blocks, nblocks);
}

cudaError_t launch_compact(int ndim, const PointsDev& P, const KernelDev& K, const double* ws, const int32_t* lmap,
                           const CompactDesc* blocks, int nblocks, Prec op, cudaStream_t st) {
  if (nblocks <= 0) return cudaSuccess;
  count_launches(1);
  switch (ndim) {
    case 1: compact_d<1>(P, K, ws, lmap, blocks, nblocks, op, st); break;
    case 2: compact_d<2>(P, K, ws, lmap, blocks, nblocks, op, st); break;
    case 3: compact_d<3>(P, K, ws, lmap, blocks, nblocks, op, st); break;
    case 4: compact_d<4>(P, K, ws, lmap, blocks, nblocks, op, st); break;
    case 5: compact_d<5>(P, K, ws, lmap, blocks, nblocks, op, st); break;
    case 6: compact_d<6>(P, K, ws, lmap, blocks, nblocks, op, st); break;
    case 7: compact_d<7>(P, K, ws, lmap, blocks, nblocks, op, st); break;
    case 8: compact_d<8>(P, K, ws, lmap, blocks, nblocks, op, st); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace hodlr
