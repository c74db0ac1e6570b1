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

// Accumulators.  Acc<float> and Acc<double> are plain sums.  Acc<DF> is a
// compensated FP32 accumulator: the running value is hi + lo, each product
// of an FP32 matrix entry with an FP64 input split as xh + xl is formed
// exactly with an FMA (p + e == v * xh), and each addition keeps its
// rounding error (TwoSum), following Ogita, Rump and Oishi, "Accurate sum
// and dot product", SIAM J. Sci. Comput. 26 (2005), algorithm Dot2.  The
// result is about as accurate as FP64 accumulation while using only the
// FP32 pipe (GB300's FP64 rate is far below what a streaming matvec needs).
struct DF {
  float hi, lo;
};

template <typename T>
struct Acc;

template <>
struct Acc<float> {
  using A = float;
  using X = float;
  static __device__ __forceinline__ X in(float v) { return v; }
  static __device__ __forceinline__ X in(double v) { return float(v); }
  static __device__ __forceinline__ A zero() { return 0.f; }
  static __device__ __forceinline__ void fma(A& a, float v, X x) { a += v * x; }
  static __device__ __forceinline__ A add(A a, A b) { return a + b; }
  static __device__ __forceinline__ A shfl_xor(A a, int o) { return __shfl_xor_sync(0xffffffffu, a, o); }
  static __device__ __forceinline__ X shfl(X x, int src) { return __shfl_sync(0xffffffffu, x, src); }
  static __device__ __forceinline__ double value(A a) { return double(a); }
};

template <>
struct Acc<double> {
  using A = double;
  using X = double;
  static __device__ __forceinline__ X in(float v) { return double(v); }
  static __device__ __forceinline__ X in(double v) { return v; }
  static __device__ __forceinline__ A zero() { return 0.0; }
  static __device__ __forceinline__ void fma(A& a, float v, X x) { a += double(v) * x; }
  static __device__ __forceinline__ void fma(A& a, double v, X x) { a += v * x; }
  static __device__ __forceinline__ A add(A a, A b) { return a + b; }
  static __device__ __forceinline__ A shfl_xor(A a, int o) { return __shfl_xor_sync(0xffffffffu, a, o); }
  static __device__ __forceinline__ X shfl(X x, int src) { return __shfl_sync(0xffffffffu, x, src); }
  static __device__ __forceinline__ double value(A a) { return a; }
};

template <>
struct Acc<DF> {
  using A = DF;
  using X = DF;
  static __device__ __forceinline__ X in(double v) {
    const float h = __double2float_rn(v);
    return DF{h, __double2float_rn(v - double(h))};
  }
  static __device__ __forceinline__ X in(float v) { return DF{v, 0.f}; }
  static __device__ __forceinline__ X in(float2 v) { return DF{v.x, v.y}; }
  static __device__ __forceinline__ A zero() { return DF{0.f, 0.f}; }
  // hi + lo renormalised (FastTwoSum) as an input pair
  static __device__ __forceinline__ float2 to_pair(A a) {
    const float s = __fadd_rn(a.hi, a.lo);
    return make_float2(s, __fsub_rn(a.lo, __fsub_rn(s, a.hi)));
  }
  // a += v * (x.hi + x.lo)
  static __device__ __forceinline__ void fma(A& a, float v, X x) {
    const float p = __fmul_rn(v, x.hi);
    float e = __fmaf_rn(v, x.hi, -p);
    e = __fmaf_rn(v, x.lo, e);
    const float s = __fadd_rn(a.hi, p);
    const float bb = __fsub_rn(s, a.hi);
    const float t = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    a.hi = s;
    a.lo = __fadd_rn(a.lo, __fadd_rn(t, e));
  }
  static __device__ __forceinline__ A add(A a, A b) {
    const float s = __fadd_rn(a.hi, b.hi);
    const float bb = __fsub_rn(s, a.hi);
    const float t = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
    return DF{s, __fadd_rn(__fadd_rn(a.lo, b.lo), t)};
  }
  static __device__ __forceinline__ A shfl_xor(A a, int o) {
    return DF{__shfl_xor_sync(0xffffffffu, a.hi, o), __shfl_xor_sync(0xffffffffu, a.lo, o)};
  }
  static __device__ __forceinline__ X shfl(X x, int src) {
    return DF{__shfl_sync(0xffffffffu, x.hi, src), __shfl_sync(0xffffffffu, x.lo, src)};
  }
  static __device__ __forceinline__ double value(A a) { return double(a.hi) + double(a.lo); }
};

// Element types of a launch: the input vector buffer [x | z] (TI) and the
// outputs and partial sums (TY).  Compensated accumulation reads its inputs
// pre-split into (hi, lo) FP32 pairs, so its hot loops use no FP64 operation.
template <typename TACC>
struct IO;
template <>
struct IO<float> {
  using TI = float;
  using TY = float;
  static __device__ __forceinline__ TI from_double(double v) { return float(v); }
};
template <>
struct IO<double> {
  using TI = double;
  using TY = double;
  static __device__ __forceinline__ TI from_double(double v) { return v; }
};
template <>
struct IO<DF> {
  using TI = float2;
  using TY = double;
  static __device__ __forceinline__ TI from_double(double v) {
    const float h = __double2float_rn(v);
    return make_float2(h, __double2float_rn(v - double(h)));
  }
};

// acc[q] += a[q] * x for the components of a 16-byte vector
template <typename TACC, typename X>
__device__ __forceinline__ void axpy16(const float4& a, X x, typename Acc<TACC>::A* acc) {
  Acc<TACC>::fma(acc[0], a.x, x);
  Acc<TACC>::fma(acc[1], a.y, x);
  Acc<TACC>::fma(acc[2], a.z, x);
  Acc<TACC>::fma(acc[3], a.w, x);
}
template <typename TACC, typename X>
__device__ __forceinline__ void axpy16(const double2& a, X x, typename Acc<TACC>::A* acc) {
  Acc<TACC>::fma(acc[0], a.x, x);
  Acc<TACC>::fma(acc[1], a.y, x);
}

template <typename T>
__device__ __forceinline__ T vzero();
template <>
__device__ __forceinline__ float4 vzero<float4>() {
  return make_float4(0.f, 0.f, 0.f, 0.f);
}
template <>
__device__ __forceinline__ double2 vzero<double2>() {
  return make_double2(0.0, 0.0);
}

template <typename TACC>
__device__ __forceinline__ typename IO<TACC>::TI to_input(typename Acc<TACC>::A a) {
  return typename IO<TACC>::TI(Acc<TACC>::value(a));
}
template <>
__device__ __forceinline__ float2 to_input<DF>(DF a) {
  return Acc<DF>::to_pair(a);
}

// Phase 1: z_b = V_b^T x_s with V_b stored row major (n x vpad(r)).  The
// CPL = 16 / sizeof(TA) columns of a 16-byte load belong to one lane; P lanes
// cover a row's nk columns and the warp's G = 32 / P lane groups take
// consecutive rows, so each load instruction of the warp reads G whole rows,
// one contiguous run.  Each lane keeps CPL running sums; the groups are added
// by shuffles once at the end.  A block with more rows than one item takes
// writes partial sums (zfix_kernel adds them in order).
template <typename TA, typename TACC>
__global__ void __launch_bounds__(256) zgemv_kernel(const ZBlock* __restrict__ zb, const ZItem* __restrict__ items,
                                                    int nitems, typename IO<TACC>::TY* __restrict__ zpart,
                                                    typename IO<TACC>::TI* in, int64_t ld_in) {
  using TX = typename IO<TACC>::TI;
  constexpr int CPL = 16 / int(sizeof(TA));
  using VT = typename Vec16<TA>::type;
  const int w = blockIdx.x * kWarpsPerCta + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= nitems) return;
  const ZItem it = items[w];
  const ZBlock Z = zb[it.zb];
  const int64_t rp = vpad(Z.r, int(sizeof(TA)));
  const TX* x = in + blockIdx.y * ld_in + Z.x_off;
  TX* z = in + blockIdx.y * ld_in + Z.z_off;
  const int lanes = (it.nk + CPL - 1) / CPL;
  int P = 1;
  while (P < lanes) P <<= 1;
  const int G = 32 / P, g = lane / P, p = lane % P;
  const bool cact = p < lanes;
  const TA* Vc = static_cast<const TA*>(Z.V) + it.k0 + p * CPL;
  using AC = Acc<TACC>;
  typename AC::A acc[CPL];
#pragma unroll
  for (int q = 0; q < CPL; q++) acc[q] = AC::zero();
  int j = it.j0 + g;
  for (; j + 3 * G < it.j1; j += 4 * G) {
    VT v[4];
    typename AC::X xs[4];
#pragma unroll
    for (int u = 0; u < 4; u++) {
      v[u] = cact ? __ldg(reinterpret_cast<const VT*>(Vc + int64_t(j + u * G) * rp)) : vzero<VT>();
      xs[u] = AC::in(x[j + u * G]);
    }
#pragma unroll
    for (int u = 0; u < 4; u++) axpy16<TACC>(v[u], xs[u], acc);
  }
  for (; j < it.j1; j += G) {
    const VT v = cact ? __ldg(reinterpret_cast<const VT*>(Vc + int64_t(j) * rp)) : vzero<VT>();
    axpy16<TACC>(v, AC::in(x[j]), acc);
  }
  for (int o = P; o < 32; o <<= 1)
#pragma unroll
    for (int q = 0; q < CPL; q++) acc[q] = AC::add(acc[q], AC::shfl_xor(acc[q], o));
  if (g == 0 && cact) {
#pragma unroll
    for (int q = 0; q < CPL; q++) {
      const int c = p * CPL + q;
      if (it.part < 0) {
        if (it.k0 + c < Z.r) z[it.k0 + c] = to_input<TACC>(acc[q]);
      } else {
        zpart[it.part + c] = typename IO<TACC>::TY(AC::value(acc[q]));
      }
    }
  }
}

template <typename TACC>
__global__ void zfix_kernel(const ZFix* __restrict__ fix, int nfix, const typename IO<TACC>::TY* __restrict__ zpart,
                            typename IO<TACC>::TI* in, int64_t ld_in) {
  using TY = typename IO<TACC>::TY;
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nfix) return;
  const ZFix F = fix[f];
  TY acc = TY(0);
  for (int q = 0; q < F.count; q++) acc += zpart[F.part + q * kZPart];
  in[blockIdx.y * ld_in + F.zpos] = IO<TACC>::from_double(double(acc));
}

// Phase 2, panels of at most 32 rows (leaves): lanes form 32 / mpad slices of
// mpad lanes (mpad = next power of two >= m), one lane per row; slice sl
// walks segments sl, sl + slices, ... of the item on its own, four columns
// per step, so a warp has several small tiles in flight at once.  The slices
// are added by shuffles at the end.
template <typename TA, typename TACC>
__global__ void __launch_bounds__(256)
    panel_small_kernel(const Panel* __restrict__ panels, const Seg* __restrict__ segs, const Item* __restrict__ items,
                       int nitems, const typename IO<TACC>::TI* __restrict__ in, int64_t ld_in,
                       typename IO<TACC>::TY* __restrict__ y, int64_t ld_y, int nslots) {
  using TX = typename IO<TACC>::TI;
  using TY = typename IO<TACC>::TY;
  const int w = blockIdx.x * kWarpsPerCta + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= nitems) return;
  const Item it = items[w];
  const Panel P = panels[it.panel];
  const int m = P.m;
  const TX* inc = in + blockIdx.y * ld_in;
  TY* yo = y + (int64_t(blockIdx.y) * nslots + P.slot) * ld_y + P.row_begin;
  int mpad = 1;
  while (mpad < m) mpad <<= 1;
  const int slices = 32 / mpad;
  const int i = lane & (mpad - 1), sl = lane / mpad;
  using AC = Acc<TACC>;
  typename AC::A a0 = AC::zero(), a1 = AC::zero();
  if (i < m) {
    for (int64_t s = it.seg_b + sl; s < it.seg_e; s += slices) {
      const Seg S = segs[s];
      const TA* A = static_cast<const TA*>(S.A) + i;
      const TX* x = inc + S.in_off;
      int j = 0;
      for (; j + 3 < S.K; j += 4) {
        const TA v0 = ldg(A + int64_t(j) * m), v1 = ldg(A + int64_t(j + 1) * m);
        const TA v2 = ldg(A + int64_t(j + 2) * m), v3 = ldg(A + int64_t(j + 3) * m);
        const TX x0 = x[j], x1 = x[j + 1], x2 = x[j + 2], x3 = x[j + 3];
        AC::fma(a0, v0, AC::in(x0));
        AC::fma(a1, v1, AC::in(x1));
        AC::fma(a0, v2, AC::in(x2));
        AC::fma(a1, v3, AC::in(x3));
      }
      for (; j < S.K; j++) AC::fma(a0, ldg(A + int64_t(j) * m), AC::in(x[j]));
    }
  }
  typename AC::A acc = AC::add(a0, a1);
  for (int o = mpad; o < 32; o <<= 1) acc = AC::add(acc, AC::shfl_xor(acc, o));
  if (sl == 0 && i < m) yo[i] = TY(AC::value(acc));
}

// Phase 2, panels of more than 32 rows: item chunk = row tile t of the
// panel; every segment's tile is streamed column by column, 16 bytes per
// lane (rows t*T + lane*RPL ..).  Input values come 32 at a time from one
// coalesced load and are broadcast by shuffle.
template <typename TA, typename TACC>
__global__ void __launch_bounds__(256)
    panel_tile_kernel(const Panel* __restrict__ panels, const Seg* __restrict__ segs, const Item* __restrict__ items,
                      int nitems, typename IO<TACC>::TY* __restrict__ ypart,
                      const typename IO<TACC>::TI* __restrict__ in, int64_t ld_in,
                      typename IO<TACC>::TY* __restrict__ y, int64_t ld_y, int nslots) {
  using TX = typename IO<TACC>::TI;
  using TY = typename IO<TACC>::TY;
  constexpr int RPL = 16 / int(sizeof(TA));
  constexpr int T = 32 * RPL;
  using VT = typename Vec16<TA>::type;
  const int w = blockIdx.x * kWarpsPerCta + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= nitems) return;
  const Item it = items[w];
  const Panel P = panels[it.panel];
  const int m = P.m;
  const TX* inc = in + blockIdx.y * ld_in;
  const int t = it.chunk;
  const int rows = min(T, m - t * T);
  const int64_t h = tile_height(m, t, int(sizeof(TA)));
  const bool act = lane * RPL < rows;
  using AC = Acc<TACC>;
  typename AC::A a0[RPL], a1[RPL];
#pragma unroll
  for (int q = 0; q < RPL; q++) a0[q] = a1[q] = AC::zero();
  for (int64_t s = it.seg_b; s < it.seg_e; s++) {
    const Seg S = segs[s];
    const TA* A = static_cast<const TA*>(S.A) + int64_t(t) * T * S.K + lane * RPL;
    const TX* x = inc + S.in_off;
    for (int j0 = 0; j0 < S.K; j0 += 32) {
      const int jn = min(32, S.K - j0);
      const typename AC::X xl = AC::in(lane < jn ? x[j0 + lane] : TX{});
      const TA* Aj = A + int64_t(j0) * h;
      int jj = 0;
      for (; jj + 3 < jn; jj += 4) {
        VT v[4];
#pragma unroll
        for (int u = 0; u < 4; u++)
          v[u] = act ? __ldg(reinterpret_cast<const VT*>(Aj + int64_t(jj + u) * h)) : vzero<VT>();
        axpy16<TACC>(v[0], AC::shfl(xl, jj), a0);
        axpy16<TACC>(v[1], AC::shfl(xl, jj + 1), a1);
        axpy16<TACC>(v[2], AC::shfl(xl, jj + 2), a0);
        axpy16<TACC>(v[3], AC::shfl(xl, jj + 3), a1);
      }
      for (; jj < jn; jj++) {
        const VT v = act ? __ldg(reinterpret_cast<const VT*>(Aj + int64_t(jj) * h)) : vzero<VT>();
        axpy16<TACC>(v, AC::shfl(xl, jj), a0);
      }
    }
  }
  if (act) {
    const int i = t * T + lane * RPL;
    TY* dst = it.part < 0 ? y + (int64_t(blockIdx.y) * nslots + P.slot) * ld_y + P.row_begin + i
                          : ypart + int64_t(it.part) * T + lane * RPL;
#pragma unroll
    for (int q = 0; q < RPL; q++)
      if (i + q < m) dst[q] = TY(AC::value(AC::add(a0[q], a1[q])));
  }
}

// Adds the partial row blocks of split panel chunks, in part order.
template <typename TX>
__global__ void __launch_bounds__(256) panel_fix_kernel(const Panel* __restrict__ panels,
                                                        const PanelFix* __restrict__ fix, int nfix, int rows,
                                                        const TX* __restrict__ ypart, TX* __restrict__ y, int64_t ld_y,
                                                        int nslots) {
  const int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  const int f = int(t / rows), q = int(t % rows);
  if (f >= nfix) return;
  const PanelFix F = fix[f];
  const Panel P = panels[F.panel];
  const int i = F.chunk * rows + q;
  if (i >= P.m) return;
  TX acc = TX(0);
  for (int g = 0; g < F.count; g++) acc += ypart[int64_t(F.part + g) * rows + q];
  y[(int64_t(blockIdx.y) * nslots + P.slot) * ld_y + P.row_begin + i] = acc;
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
  const int64_t total = int64_t(T.m) * T.n;
  for (int64_t e = lane; e < total; e += 32) {
    const int i = int(e % T.m), j = int(e / T.m);
    double xi[D];
    load_point<D>(P, T.t_begin + i, xi);
    o[elem_offset(i, j, T.m, T.n, int(sizeof(TO)))] = TO(kernel_entry<D>(P, K, T.t_begin + i, T.s_begin + j, xi));
  }
}

template <int D, typename TO>
__global__ void __launch_bounds__(256) compact_kernel(PointsDev P, KernelDev K, const double* __restrict__ ws,
                                                      const int32_t* __restrict__ lmap,
                                                      const CompactDesc* __restrict__ blocks, int nblocks) {
  const CompactDesc B = blocks[blockIdx.x];
  TO* u = static_cast<TO*>(B.u_dst);
  constexpr int esz = int(sizeof(TO));
  if (B.dense) {
    const int64_t total = int64_t(B.m) * B.n;
    for (int64_t e = threadIdx.x; e < total; e += blockDim.x) {
      const int i = int(e % B.m), j = int(e / B.m);
      double xi[D];
      load_point<D>(P, B.t_begin + i, xi);
      u[elem_offset(i, j, B.m, B.n, esz)] = TO(kernel_entry<D>(P, K, B.t_begin + i, B.s_begin + j, xi));
    }
  } else {
    const double* U = ws + B.ws;
    const int64_t nu = int64_t(B.m) * B.rank;
    for (int64_t e = threadIdx.x; e < nu; e += blockDim.x) {
      const int i = int(e % B.m), k = int(e / B.m);
      u[elem_offset(lmap[B.t_map + i] - B.t_begin, k, B.m, B.rank, esz)] = TO(U[e]);
    }
    // V follows U's full workspace (m x cap); stored row major, n x vpad(rank)
    const double* Vw = ws + B.ws + int64_t(B.m) * B.cap;
    TO* v = static_cast<TO*>(B.v_dst);
    const int64_t rp = vpad(B.rank, esz);
    const int64_t nv = int64_t(B.n) * B.rank;
    for (int64_t e = threadIdx.x; e < nv; e += blockDim.x) {
      const int j = int(e % B.n), k = int(e / B.n);
      v[(lmap[B.s_map + j] - B.s_begin) * rp + k] = TO(Vw[e]);
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

template <typename TA, typename TACC>
static void zgemv_t(const ZBlock* zb, const ZItem* items, int nitems, const ZFix* fix, int nfix, void* zpart, void* in,
                    int64_t ld_in, int nrhs, cudaStream_t st) {
  using TI = typename IO<TACC>::TI;
  using TY = typename IO<TACC>::TY;
  dim3 g(warps_grid(nitems), unsigned(nrhs));
  zgemv_kernel<TA, TACC><<<g, 256, 0, st>>>(zb, items, nitems, static_cast<TY*>(zpart), static_cast<TI*>(in), ld_in);
  if (nfix > 0) {
    dim3 gf(unsigned((nfix + 255) / 256), unsigned(nrhs));
    zfix_kernel<TACC><<<gf, 256, 0, st>>>(fix, nfix, static_cast<const TY*>(zpart), static_cast<TI*>(in), ld_in);
  }
}

cudaError_t launch_zgemv(Prec a, Prec x, const ZBlock* zb, const ZItem* items, int nitems, const ZFix* fix, int nfix,
                         void* zpart, void* in, int64_t ld_in, int nrhs, cudaStream_t st, bool df) {
  if (nitems <= 0) return cudaSuccess;
  count_launches(nfix > 0 ? 2 : 1);
  if (a == Prec::kD && x == Prec::kD)
    zgemv_t<double, double>(zb, items, nitems, fix, nfix, zpart, in, ld_in, nrhs, st);
  else if (a == Prec::kF && x == Prec::kD && df)
    zgemv_t<float, DF>(zb, items, nitems, fix, nfix, zpart, in, ld_in, nrhs, st);
  else if (a == Prec::kF && x == Prec::kF)
    zgemv_t<float, float>(zb, items, nitems, fix, nfix, zpart, in, ld_in, nrhs, st);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

template <typename TA, typename TACC>
static void panels_t(const Panel* panels, const Seg* segs, const Item* small, int nsmall, const Item* big, int nbig,
                     const PanelFix* fix, int nfix, void* ypart, const void* in, int64_t ld_in, void* y, int64_t ld_y,
                     int nslots, int nrhs, cudaStream_t st) {
  using TI = typename IO<TACC>::TI;
  using TY = typename IO<TACC>::TY;
  if (nbig > 0) {
    dim3 g(warps_grid(nbig), unsigned(nrhs));
    panel_tile_kernel<TA, TACC><<<g, 256, 0, st>>>(panels, segs, big, nbig, static_cast<TY*>(ypart),
                                                   static_cast<const TI*>(in), ld_in, static_cast<TY*>(y), ld_y, nslots);
  }
  if (nsmall > 0) {
    dim3 g(warps_grid(nsmall), unsigned(nrhs));
    panel_small_kernel<TA, TACC><<<g, 256, 0, st>>>(panels, segs, small, nsmall, static_cast<const TI*>(in), ld_in,
                                                    static_cast<TY*>(y), ld_y, nslots);
  }
  if (nfix > 0) {
    const int rows = int(tile_rows(int(sizeof(TA))));
    dim3 gf(unsigned((int64_t(nfix) * rows + 255) / 256), unsigned(nrhs));
    panel_fix_kernel<TY><<<gf, 256, 0, st>>>(panels, fix, nfix, rows, static_cast<const TY*>(ypart),
                                             static_cast<TY*>(y), ld_y, nslots);
  }
}

cudaError_t launch_panels(Prec a, Prec x, const Panel* panels, const Seg* segs, const Item* small, int nsmall,
                          const Item* big, int nbig, const PanelFix* fix, int nfix, void* ypart, const void* in,
                          int64_t ld_in, void* y, int64_t ld_y, int nslots, int nrhs, cudaStream_t st, bool df) {
  if (nsmall + nbig <= 0) return cudaSuccess;
  count_launches(uint64_t(nbig > 0) + uint64_t(nsmall > 0) + uint64_t(nfix > 0));
  if (a == Prec::kD && x == Prec::kD)
    panels_t<double, double>(panels, segs, small, nsmall, big, nbig, fix, nfix, ypart, in, ld_in, y, ld_y, nslots,
                             nrhs, st);
  else if (a == Prec::kF && x == Prec::kD && df)
    panels_t<float, DF>(panels, segs, small, nsmall, big, nbig, fix, nfix, ypart, in, ld_in, y, ld_y, nslots, nrhs,
                        st);
  else if (a == Prec::kF && x == Prec::kF)
    panels_t<float, float>(panels, segs, small, nsmall, big, nbig, fix, nfix, ypart, in, ld_in, y, ld_y, nslots, nrhs,
                           st);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

__global__ void split_kernel(const double* __restrict__ x, float2* __restrict__ out, int64_t n) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const double v = x[i];
    const float h = __double2float_rn(v);
    out[i] = make_float2(h, __double2float_rn(v - double(h)));
  }
}

cudaError_t launch_split(const double* x, void* out, int64_t n, cudaStream_t st) {
  count_launches(1);
  split_kernel<<<vec_grid(n), 256, 0, st>>>(x, static_cast<float2*>(out), n);
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
