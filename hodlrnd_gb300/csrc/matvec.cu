// HODLR matvec kernels (see matvec.h).
#include <cuda_bf16.h>

#include "bulk.cuh"
#include "device.cuh"
#include "matvec.h"

namespace hodlr {

__device__ unsigned int g_stream_timeouts = 0;

cudaError_t read_stream_timeouts(unsigned int* host, cudaStream_t st) {
  return cudaMemcpyFromSymbolAsync(host, g_stream_timeouts, sizeof(unsigned int), 0, cudaMemcpyDeviceToHost, st);
}

namespace {

constexpr int kWarpsPerCta = 8;

template <typename T>
__device__ __forceinline__ T ldg(const T* p) {
  return __ldg(p);
}

// BF16 storage element (bits only; arithmetic converts to FP32)
struct bf16 {
  unsigned short b;
};
template <>
__device__ __forceinline__ bf16 ldg<bf16>(const bf16* p) {
  return bf16{__ldg(reinterpret_cast<const unsigned short*>(p))};
}
__device__ __forceinline__ float bf2f(unsigned short b) { return __uint_as_float(uint32_t(b) << 16); }

template <typename T>
struct Vec16;
template <>
struct Vec16<bf16> {
  using type = uint4;  // 8 BF16 values
};
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
  static __device__ __forceinline__ A scale(A a, float s) { return a * s; }
  static __device__ __forceinline__ X xscale(X x, float s) { return x * s; }
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
  static __device__ __forceinline__ A scale(A a, float s) { return a * double(s); }
  static __device__ __forceinline__ X xscale(X x, float s) { return x * double(s); }
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
  static __device__ __forceinline__ void fma(A& a, bf16 v, X x) { fma(a, bf2f(v.b), x); }
  // (hi + lo) * s with the rounding error of hi * s kept (TwoProduct by FMA)
  static __device__ __forceinline__ A scale(A a, float s) {
    const float p = __fmul_rn(a.hi, s);
    return DF{p, __fmaf_rn(a.lo, s, __fmaf_rn(a.hi, s, -p))};
  }
  static __device__ __forceinline__ X xscale(X x, float s) { return scale(x, s); }
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

// Relaxed accumulation (Accum::kRelaxed): the inputs and outputs of DF
// (split FP64 inputs, FP64 outputs) with plain FP32 sums of the products of
// the FP32 factors with the inputs' high parts.  Cheaper, and accurate to
// about 1e-6 relative: what an inexact Krylov method may use once its
// residual has dropped far enough.
struct FH {};

template <>
struct Acc<FH> {
  using A = float;
  using X = float;
  static __device__ __forceinline__ X in(float2 v) { return v.x; }
  static __device__ __forceinline__ X in(float v) { return v; }
  static __device__ __forceinline__ A zero() { return 0.f; }
  static __device__ __forceinline__ void fma(A& a, float v, X x) { a = __fmaf_rn(v, x, a); }
  static __device__ __forceinline__ void fma(A& a, bf16 v, X x) { a = __fmaf_rn(bf2f(v.b), x, a); }
  static __device__ __forceinline__ A add(A a, A b) { return a + b; }
  static __device__ __forceinline__ A scale(A a, float s) { return a * s; }
  static __device__ __forceinline__ X xscale(X x, float s) { return x * s; }
  static __device__ __forceinline__ A shfl_xor(A a, int o) { return __shfl_xor_sync(0xffffffffu, a, o); }
  static __device__ __forceinline__ X shfl(X x, int src) { return __shfl_sync(0xffffffffu, x, src); }
  static __device__ __forceinline__ double value(A a) { return double(a); }
};

template <>
struct IO<FH> {
  using TI = float2;
  using TY = double;
  static __device__ __forceinline__ TI from_double(double v) { return IO<DF>::from_double(v); }
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

template <typename TACC, typename X>
__device__ __forceinline__ void axpy16(const uint4& a, X x, typename Acc<TACC>::A* acc) {
  Acc<TACC>::fma(acc[0], __uint_as_float(a.x << 16), x);
  Acc<TACC>::fma(acc[1], __uint_as_float(a.x & 0xffff0000u), x);
  Acc<TACC>::fma(acc[2], __uint_as_float(a.y << 16), x);
  Acc<TACC>::fma(acc[3], __uint_as_float(a.y & 0xffff0000u), x);
  Acc<TACC>::fma(acc[4], __uint_as_float(a.z << 16), x);
  Acc<TACC>::fma(acc[5], __uint_as_float(a.z & 0xffff0000u), x);
  Acc<TACC>::fma(acc[6], __uint_as_float(a.w << 16), x);
  Acc<TACC>::fma(acc[7], __uint_as_float(a.w & 0xffff0000u), x);
}

template <typename T>
__device__ __forceinline__ T vzero();
template <>
__device__ __forceinline__ uint4 vzero<uint4>() {
  return make_uint4(0u, 0u, 0u, 0u);
}
template <>
__device__ __forceinline__ float4 vzero<float4>() {
  return make_float4(0.f, 0.f, 0.f, 0.f);
}
template <>
__device__ __forceinline__ double2 vzero<double2>() {
  return make_double2(0.0, 0.0);
}

// Input value of column j of a segment: x_j, times the column scale of a BF16
// dense tile (cs non-null).
template <typename TACC, typename TX>
__device__ __forceinline__ typename Acc<TACC>::X seg_in(TX x, const float* cs, int j) {
  return cs ? Acc<TACC>::xscale(Acc<TACC>::in(x), __ldg(cs + j)) : Acc<TACC>::in(x);
}

// An input value back in the staged (hi, lo) form, after scaling.
template <typename TACC>
__device__ __forceinline__ float2 x_pair(typename Acc<TACC>::X x);
template <>
__device__ __forceinline__ float2 x_pair<DF>(DF x) {
  return make_float2(x.hi, x.lo);
}
template <>
__device__ __forceinline__ float2 x_pair<FH>(float x) {
  return make_float2(x, 0.f);
}

template <typename TACC>
__device__ __forceinline__ typename IO<TACC>::TI to_input(typename Acc<TACC>::A a) {
  return typename IO<TACC>::TI(Acc<TACC>::value(a));
}
template <>
__device__ __forceinline__ float2 to_input<DF>(DF a) {
  return Acc<DF>::to_pair(a);
}
template <>
__device__ __forceinline__ float2 to_input<FH>(float a) {
  return make_float2(a, 0.f);
}

// Phase 1: z_b = V_b^T x_s with V_b stored row major (n x vpad(r)).  The
// CPL = 16 / sizeof(TA) columns of a 16-byte load belong to one lane; P lanes
// cover a row's nk columns and the warp's G = 32 / P lane groups take
// consecutive rows, so each 16-byte read of the warp covers G whole rows.
// Each lane keeps CPL running sums, over rows g, g + G, g + 2G, ... of the
// item in that order; the groups are added by shuffles once at the end.  A
// block with more rows than one item takes writes partial sums (zfix_kernel
// adds them in order).
//
// An item that covers whole rows (k0 == 0, nk == vpad(r)) reads one
// contiguous run of V, and its inputs x[j0 .. j1) are contiguous too: both
// are staged through a per-warp ring of kZStages shared-memory stages by bulk
// copies, R rows per stage (R a multiple of G, so every lane's row order is
// the one above).  Other items (blocks of more than 128 FP32 or 64 FP64
// columns) load V directly.
// Ring shapes (stages x bytes) of the staged kernels; HODLR_TUNE_* override
// them at compile time for tuning runs.  Two stages per warp measured best on
// GB300 (the shared memory per warp, not the stage count, limits the warps
// per SM, and more warps hide more latency than deeper rings); V^T x stages
// of 4 KB (with V grouped by source node, whole-row runs are long) beat 2 KB
// by 2% per solve at N = 262144.
#ifndef HODLR_TUNE_Z_STAGES
#define HODLR_TUNE_Z_STAGES 2
#endif
#ifndef HODLR_TUNE_Z_BYTES
#define HODLR_TUNE_Z_BYTES 4096
#endif
#ifndef HODLR_TUNE_P_STAGES
#define HODLR_TUNE_P_STAGES 2
#endif
#ifndef HODLR_TUNE_P_BYTES
#define HODLR_TUNE_P_BYTES 4096
#endif
#ifndef HODLR_TUNE_S_STAGES
#define HODLR_TUNE_S_STAGES 2
#endif
#ifndef HODLR_TUNE_S_BYTES
#define HODLR_TUNE_S_BYTES 2048
#endif
#ifndef HODLR_TUNE_S_MINB
#define HODLR_TUNE_S_MINB 6  // leaf-panel CTAs per SM the register allocation must allow (no spills at 6)
#endif
#ifndef HODLR_TUNE_P_MINB
#define HODLR_TUNE_P_MINB 4
#endif
constexpr int kZWarps = 4;                      // warps per CTA of zgemv_kernel
constexpr int kZStages = HODLR_TUNE_Z_STAGES;   // ring stages per warp
constexpr int kZStageBytes = HODLR_TUNE_Z_BYTES;  // V bytes per stage
// input bytes per stage: at most kZStageBytes / 16 rows of 8 bytes, plus 2 x 15
// bytes of alignment slack, rounded to 16
constexpr int kZXBytes = (kZStageBytes / 16) * 8 + 32;
constexpr int kZWarpSmem = 64 + kZStages * (kZStageBytes + kZXBytes);
static_assert(kZWarpSmem % 16 == 0 && kZXBytes % 16 == 0, "bulk copy destinations must stay 16-byte aligned");

// The end of an item: acc[q] (column p * CPL + q of the item) is summed over
// the G = 32 / P lanes sharing p by a transposed butterfly -- while a lane
// holds several columns, each exchange hands half of them to the partner
// lane and keeps the other half -- so lane l ends with the total of column
// p * CPL + coff(l) + k in acc[k], k < w; lanes that differ only in the bits
// of the plain exchanges that follow hold the same totals, and the one with
// those bits clear writes them.
template <typename TA, typename TACC>
__device__ __forceinline__ void z_finish(typename Acc<TACC>::A* acc, int P, int lane, const ZItem& it,
                                         const ZBlock& Z, typename IO<TACC>::TI* z,
                                         typename IO<TACC>::TY* zpart) {
  using AC = Acc<TACC>;
  constexpr int CPL = 16 / int(sizeof(TA));
  int coff = 0, w = CPL, o = 16;
#pragma unroll
  for (int lv = 0; (CPL >> lv) > 1; lv++, o >>= 1) {
    if (o < P) break;
    const int half = CPL >> (lv + 1);
    const bool up = (lane & o) != 0;
#pragma unroll
    for (int k = 0; k < CPL / 2; k++) {
      if (k < half) {
        const typename AC::A send = up ? acc[k] : acc[k + half];
        const typename AC::A keep = up ? acc[k + half] : acc[k];
        acc[k] = AC::add(keep, AC::shfl_xor(send, o));
      }
    }
    if (up) coff += half;
    w = half;
  }
  bool writer = true;
  for (; o >= P; o >>= 1) {  // w == 1 here
    acc[0] = AC::add(acc[0], AC::shfl_xor(acc[0], o));
    if (lane & o) writer = false;
  }
  const int p = lane % P;
  if (!writer || p * CPL >= it.nk) return;
#pragma unroll
  for (int k = 0; k < CPL; k++) {
    if (k < w) {
      const int c = p * CPL + coff + k;  // column within the item
      typename AC::A v = acc[k];
      // BF16: z columns carry the product of U's and V's column scales
      if (sizeof(TA) == 2 && Z.zscale && it.k0 + c < Z.r) v = AC::scale(v, __ldg(Z.zscale + it.k0 + c));
      if (it.part < 0) {
        if (it.k0 + c < Z.r) z[it.k0 + c] = to_input<TACC>(v);
      } else {
        zpart[it.part + c] = typename IO<TACC>::TY(AC::value(v));
      }
    }
  }
}

template <typename TA, typename TACC>
__global__ void __launch_bounds__(kZWarps * 32) zgemv_kernel(const ZBlock* __restrict__ zb,
                                                           const ZItem* __restrict__ items, int nitems,
                                                           typename IO<TACC>::TY* __restrict__ zpart,
                                                           typename IO<TACC>::TI* in, int64_t ld_in) {
  using TX = typename IO<TACC>::TI;
  constexpr int CPL = 16 / int(sizeof(TA));
  using VT = typename Vec16<TA>::type;
  using AC = Acc<TACC>;
  extern __shared__ __align__(16) unsigned char zsm[];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int w = blockIdx.x * kZWarps + wid;
  if (w >= nitems) return;
  const ZItem it = items[w];
  const ZBlock Z = zb[it.zb];
  const int64_t rp = vpad(Z.r, int(sizeof(TA)));
  const TX* x = in + blockIdx.y * ld_in + Z.x_off;
  TX* z = in + blockIdx.y * ld_in + Z.z_off;
  const int lanes = (it.nk + CPL - 1) / CPL;
  const int P = lanes <= 1 ? 1 : 1 << (32 - __clz(lanes - 1));  // next power of two >= lanes
  const int G = 32 / P, g = lane / P, p = lane % P;
  const bool cact = p < lanes;
  typename AC::A acc[CPL];
#pragma unroll
  for (int q = 0; q < CPL; q++) acc[q] = AC::zero();
  if (it.nst > 0) {
    // rows of rowb = rp * sizeof(TA) bytes (16 .. 512, a multiple of 16); V
    // is 16-byte aligned (factor chunks are, and every block's V starts on a
    // 16-byte boundary), so every stage's source and size are too.  The input
    // run is copied from its 16-byte boundary below to the one above; the
    // input buffers carry 16 bytes of padding at their end for that.  R and
    // nst come from z_item_stages: R a multiple of G, at most
    // kZStageBytes / rowb rows.
    unsigned char* base = zsm + wid * kZWarpSmem;
    uint64_t* bar = reinterpret_cast<uint64_t*>(base);
    unsigned char* vbuf = base + 64;
    unsigned char* xbuf = vbuf + kZStages * kZStageBytes;
    const int rowb = int(rp) * int(sizeof(TA));
    const int R = it.R, nst = it.nst;
    const int nrows = it.j1 - it.j0;
    const TA* V = static_cast<const TA*>(Z.V) + int64_t(it.j0) * rp;
    const TX* xr = x + it.j0;
    if (lane == 0) {
#pragma unroll
      for (int s = 0; s < kZStages; s++) mbar_init(bar + s, 1);
      fence_mbar_init();
    }
    __syncwarp();
    auto issue = [&](int q) {  // lane 0
      const int s = q % kZStages;
      const int r0 = q * R, nr = min(R, nrows - r0);
      const uint32_t vb = uint32_t(nr) * uint32_t(rowb);
      const unsigned char* xs = reinterpret_cast<const unsigned char*>(xr + r0);
      const unsigned char* xa = static_cast<const unsigned char*>(align_down16(xs));
      const uint32_t xb = uint32_t((xs + size_t(nr) * sizeof(TX) - xa + 15) & ~size_t(15));
      fence_proxy_async();
      mbar_expect_tx(bar + s, vb + xb);
      bulk_g2s(vbuf + s * kZStageBytes, V + int64_t(r0) * rp, vb, bar + s);
      bulk_g2s(xbuf + s * kZXBytes, xa, xb, bar + s);
    };
    if (lane == 0)
      for (int q = 0; q < min(kZStages, nst); q++) issue(q);
    for (int q = 0; q < nst; q++) {
      const int s = q % kZStages;
      const bool ok = __all_sync(0xffffffffu, mbar_wait(bar + s, uint32_t(q / kZStages) & 1u));
      if (!ok) {
        // give up: count it, let the copies still in flight land, return
        if (lane == 0) atomicAdd(&g_stream_timeouts, 1u);
        for (int t = q; t < min(q + kZStages, nst); t++) mbar_wait(bar + t % kZStages, uint32_t(t / kZStages) & 1u);
        return;
      }
      const int r0 = q * R, nr = min(R, nrows - r0);
      const int xo = int((reinterpret_cast<uintptr_t>(xr + r0) & 15u) / sizeof(TX));
      const TX* xsm = reinterpret_cast<const TX*>(xbuf + s * kZXBytes) + xo;
      const unsigned char* vs = vbuf + s * kZStageBytes + p * 16;
      for (int i = g; i < nr; i += G) {
        const VT v = cact ? *reinterpret_cast<const VT*>(vs + i * rowb) : vzero<VT>();
        axpy16<TACC>(v, AC::in(xsm[i]), acc);
      }
      __syncwarp();
      if (lane == 0 && q + kZStages < nst) issue(q + kZStages);
    }
  } else {
    const TA* Vc = static_cast<const TA*>(Z.V) + it.k0 + p * CPL;
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
  }
  z_finish<TA, TACC>(acc, P, lane, it, Z, z, zpart);
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
// takes segments sl, sl + slices, ... of the item, each cut into pieces of at
// most cmax columns (a multiple of 16 bytes' worth of elements, so that every
// piece starts on a 16-byte boundary).  The warp runs in rounds: in round q
// every slice processes its q-th piece.  A piece (its m x c column-major
// block, rounded up to 16 bytes, and its input run, from the 16-byte boundary
// below to the one above) is staged in shared memory by bulk copies that the
// slice's first lane starts, kSStages rounds ahead; each round's mbarrier
// expects one arrival per slice.  Column j of a piece goes to accumulator
// j & 1; the slices are added by shuffles at the end.  For a BF16 dense tile
// the slice's lanes first multiply the staged inputs by the tile's column
// scales, in place (once per column rather than once per entry).
constexpr int kSWarps = 4;                     // warps per CTA of panel_small_kernel
constexpr int kSStages = HODLR_TUNE_S_STAGES;
constexpr int kSUBytes = HODLR_TUNE_S_BYTES;   // segment bytes per round (all slices)
// input bytes per round (all slices): twice as many for BF16, whose pieces
// hold more columns per byte of segment
template <typename TA>
__host__ __device__ constexpr int s_xbytes() { return sizeof(TA) == 2 ? 2 * kSUBytes : kSUBytes; }
template <typename TA>
__host__ __device__ constexpr int s_warp_smem() { return 64 + kSStages * (kSUBytes + s_xbytes<TA>()); }
// every slice's piece holds at least 16 bytes' worth of columns (cmax >= Q
// below) for any m <= 32 with these budgets
static_assert(kSUBytes >= 2048 && kSUBytes % 16 == 0, "leaf-panel stage too small");
static_assert(s_warp_smem<float>() % 16 == 0 && s_warp_smem<bf16>() % 16 == 0,
              "bulk copy destinations must stay 16-byte aligned");

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

template <typename TA, typename TACC>
__global__ void __launch_bounds__(kSWarps * 32, HODLR_TUNE_S_MINB)
    panel_small_kernel(const Panel* __restrict__ panels, const Seg* __restrict__ segs, const Item* __restrict__ items,
                       int nitems, const typename IO<TACC>::TI* __restrict__ in, int64_t ld_in,
                       typename IO<TACC>::TY* __restrict__ y, int64_t ld_y, int nslots,
                       typename IO<TACC>::TY* __restrict__ ypart) {
  using TX = typename IO<TACC>::TI;
  using TY = typename IO<TACC>::TY;
  using AC = Acc<TACC>;
  constexpr int esz = int(sizeof(TA));
  constexpr int Q = 16 / esz;  // piece columns are a multiple of Q
  constexpr int kSXBytes = s_xbytes<TA>(), kSWarpSmem = s_warp_smem<TA>();
  extern __shared__ __align__(16) unsigned char ssm[];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int w = blockIdx.x * kSWarps + wid;
  if (w >= nitems) return;
  const Item it = items[w];
  const Panel P = panels[it.panel];
  const int m = P.m;
  const TX* inc = in + blockIdx.y * ld_in;
  TY* yo = y + int64_t(blockIdx.y) * nslots * ld_y + P.yoff;
  int mpad = 1;
  while (mpad < m) mpad <<= 1;
  const int slices = 32 / mpad;
  const int i = lane & (mpad - 1), sl = lane / mpad;
  // per slice and round: ub bytes of segment, xb bytes of inputs; a piece of
  // c columns needs c*m*esz + 15 and c*sizeof(TX) + 32 bytes at most
  const int ub = kSUBytes / slices, xb = kSXBytes / slices;
  const int cmax = min((ub - 15) / (m * esz), (xb - 32) / int(sizeof(TX))) / Q * Q;  // >= Q: ub, xb >= 64 mpad
  unsigned char* base = ssm + wid * kSWarpSmem;
  uint64_t* bar = reinterpret_cast<uint64_t*>(base);
  unsigned char* stage0 = base + 64;
  // rounds = the largest piece count over the slices
  int npieces = 0;
  for (int64_t q = it.seg_b + sl; q < it.seg_e; q += slices) npieces += (segs[q].K + cmax - 1) / cmax;
  int rounds = npieces;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) rounds = max(rounds, __shfl_xor_sync(0xffffffffu, rounds, o));
  if (lane == 0) {
#pragma unroll
    for (int s = 0; s < kSStages; s++) mbar_init(bar + s, uint32_t(slices));
    fence_mbar_init();
  }
  __syncwarp();

  int64_t ps = it.seg_b + sl;  // producer cursor of this slice (used by its first lane)
  int pc = 0;
#define HODLR_SMALL_ISSUE(q_)                                                                                   \
  do {                                                                                                          \
    if (i != 0) break;                                                                                          \
    const int st_ = (q_) % kSStages;                                                                            \
    if (ps >= it.seg_e) {                                                                                       \
      mbar_arrive(bar + st_);                                                                                   \
      break;                                                                                                    \
    }                                                                                                           \
    const Seg S_ = segs[ps];                                                                                    \
    const int c_ = min(cmax, S_.K - pc);                                                                        \
    unsigned char* su_ = stage0 + st_ * (kSUBytes + kSXBytes) + sl * ub;                                        \
    unsigned char* sx_ = stage0 + st_ * (kSUBytes + kSXBytes) + kSUBytes + sl * xb;                             \
    /* pc is a multiple of Q, so the piece starts 16-byte aligned; the rounded                                 \
       size stays inside the block's storage (padded to 16 bytes) */                                            \
    const TA* A_ = static_cast<const TA*>(S_.A) + int64_t(pc) * m;                                              \
    const uint32_t bu_ = uint32_t((c_ * m * esz + 15) & ~15);                                                   \
    const unsigned char* xs_ = reinterpret_cast<const unsigned char*>(inc + S_.in_off + pc);                    \
    const unsigned char* xa_ = static_cast<const unsigned char*>(align_down16(xs_));                            \
    const uint32_t bx_ = uint32_t((xs_ + size_t(c_) * sizeof(TX) - xa_ + 15) & ~size_t(15));                    \
    fence_proxy_async();                                                                                        \
    mbar_expect_tx(bar + st_, bu_ + bx_);                                                                       \
    bulk_g2s(su_, A_, bu_, bar + st_);                                                                          \
    bulk_g2s(sx_, xa_, bx_, bar + st_);                                                                         \
    pc += c_;                                                                                                   \
    if (pc >= S_.K) {                                                                                           \
      ps += slices;                                                                                             \
      pc = 0;                                                                                                   \
    }                                                                                                           \
  } while (0)
  for (int q = 0; q < min(kSStages, rounds); q++) HODLR_SMALL_ISSUE(q);
  typename AC::A a0 = AC::zero(), a1 = AC::zero();
  int64_t cs = it.seg_b + sl;  // consumer cursor
  int cc = 0;
  for (int q = 0; q < rounds; q++) {
    const int st = q % kSStages;
    const bool ok = __all_sync(0xffffffffu, mbar_wait(bar + st, uint32_t(q / kSStages) & 1u));
    if (!ok) {
      if (lane == 0) atomicAdd(&g_stream_timeouts, 1u);
      for (int t = q; t < min(q + kSStages, rounds); t++) mbar_wait(bar + t % kSStages, uint32_t(t / kSStages) & 1u);
      return;
    }
    if constexpr (sizeof(TA) == 2) {
      // BF16 dense tile: the slice's lanes multiply the staged inputs by the
      // column scales once, in place, before the products
      if (cs < it.seg_e) {
        const Seg S = segs[cs];
        if (S.cscale) {
          const int c = min(cmax, S.K - cc);
          const int xo = int((reinterpret_cast<uintptr_t>(inc + S.in_off + cc) & 15u) / sizeof(TX));
          TX* sx = reinterpret_cast<TX*>(stage0 + st * (kSUBytes + kSXBytes) + kSUBytes + sl * xb) + xo;
          for (int j = i; j < c; j += mpad) sx[j] = x_pair<TACC>(seg_in<TACC>(sx[j], S.cscale, cc + j));
        }
      }
      __syncwarp();
    }
    if (cs < it.seg_e) {
      const Seg S = segs[cs];
      const int c = min(cmax, S.K - cc);
      const TA* su = reinterpret_cast<const TA*>(stage0 + st * (kSUBytes + kSXBytes) + sl * ub);
      const int xo = int((reinterpret_cast<uintptr_t>(inc + S.in_off + cc) & 15u) / sizeof(TX));
      const TX* sx = reinterpret_cast<const TX*>(stage0 + st * (kSUBytes + kSXBytes) + kSUBytes + sl * xb) + xo;
      if (i < m) {
        int j = 0;
        for (; j + 1 < c; j += 2) {
          AC::fma(a0, su[j * m + i], AC::in(sx[j]));
          AC::fma(a1, su[(j + 1) * m + i], AC::in(sx[j + 1]));
        }
        if (j < c) AC::fma(a0, su[j * m + i], AC::in(sx[j]));
      }
      cc += c;
      if (cc >= S.K) {
        cs += slices;
        cc = 0;
      }
    }
    __syncwarp();  // round q's stage is refilled for round q + kSStages
    if (q + kSStages < rounds) HODLR_SMALL_ISSUE(q + kSStages);
  }
#undef HODLR_SMALL_ISSUE
  typename AC::A acc = AC::add(a0, a1);
  for (int o = mpad; o < 32; o <<= 1) acc = AC::add(acc, AC::shfl_xor(acc, o));
  // a panel whose columns are split over several items: partial rows at
  // ypart[part * tile_rows], added in part order by panel_fix_kernel
  if (sl == 0 && i < m) {
    if (it.part < 0)
      yo[i] = TY(AC::value(acc));
    else
      ypart[int64_t(it.part) * tile_rows(int(sizeof(TA))) + i] = TY(AC::value(acc));
  }
}

// Phase 2, panels of at most 32 rows, when the segments of every item lie
// in memory in segment order (the far field after its relayout in panel
// order, the near field as assembled).  All segments of a panel have its m
// rows, so an item's factors form one run of m-row columns (after each
// segment up to 15 bytes of padding, and for a BF16 dense tile its column
// scales).  The run is streamed through a per-warp ring of kLStages stages;
// a stage is the bytes of a run of whole columns -- at most kLStageBytes, at
// most kLCols columns -- fetched by ONE bulk copy (from the 16-byte boundary
// at or below its first column), and the input values of those columns,
// gathered into the stage by the lanes with 4- or 8-byte asynchronous copies
// (cp.async) that complete on the stage's mbarrier.  Relaxed products read
// only the high part of a split input, so only that part is staged.  Both
// are issued kLStages - 1 stages ahead of the products, so neither the
// factor bytes nor the scattered inputs (read from L2: x and z are small)
// are waited for in the loop.
//
// The warp plans each stage together: lane k reads the record of the k-th
// next segment (one coalesced load per 32 segments; the first 32 of each
// plan are loaded one stage ahead), a warp scan places each segment's
// columns in the stage, and every lane then fills the stage's column table
// (the element offset of each column in the stage buffer) and starts the
// gathers of columns lane, lane + 32, ... (for BF16 dense tiles also the
// gathers of their column scales).  After the wait the lanes multiply the
// staged inputs of BF16 dense tiles by their scales, once per column.  The
// products then read only shared memory: lanes form slices of mpad lanes
// (one lane per row), slice sl takes the stage's columns sl, sl + slices,
// ..., column parity picks the accumulator.
#ifndef HODLR_TUNE_L_STAGES
#define HODLR_TUNE_L_STAGES 2
#endif
#ifndef HODLR_TUNE_L_BYTES
#define HODLR_TUNE_L_BYTES 4096
#endif
#ifndef HODLR_TUNE_L_COLS
#define HODLR_TUNE_L_COLS 128
#endif
#ifndef HODLR_TUNE_L_MINB
#define HODLR_TUNE_L_MINB 5
#endif
constexpr int kLWarps = 4;
constexpr int kLStages = HODLR_TUNE_L_STAGES;
constexpr int kLStageBytes = HODLR_TUNE_L_BYTES;  // factor bytes per stage at most
constexpr int kLCols = HODLR_TUNE_L_COLS;         // columns per stage at most
constexpr int kLHead = 64;                        // barriers and stage descriptors
static_assert(kLStages >= 2 && kLStages <= 4, "leaf ring: 2 to 4 stages");
static_assert(kLStageBytes % 16 == 0 && kLStageBytes >= 512 && kLStageBytes <= 65536,
              "leaf stage: a multiple of 16 bytes in 512 .. 65536 (column offsets are 16-bit)");
static_assert(kLCols % 32 == 0 && kLCols <= 1024, "leaf stage columns: a multiple of 32");
static_assert(32 + kLStages * 8 <= kLHead, "leaf ring header too small");
// The staged input of one column: the input element, or for relaxed products
// (which read only the high part of a split input) that high part alone.
template <typename TACC>
struct LeafX {
  using T = typename IO<TACC>::TI;
};
template <>
struct LeafX<FH> {
  using T = float;
};
// An input after scaling, in its staged form.
__device__ __forceinline__ void put_staged(float2& d, DF x) { d = make_float2(x.hi, x.lo); }
__device__ __forceinline__ void put_staged(float& d, float x) { d = x; }
__device__ __forceinline__ void put_staged(double& d, double x) { d = x; }
// stage: factor bytes | inputs (kLCols x TX) | column offsets (kLCols x u16) | BF16 scales (kLCols x f32)
template <typename TA, typename TX>
__host__ __device__ constexpr int l_stage_smem() {
  return kLStageBytes + kLCols * int(sizeof(TX)) + kLCols * 2 + (sizeof(TA) == 2 ? kLCols * 4 : 0);
}
template <typename TA, typename TX>
__host__ __device__ constexpr int l_warp_smem() { return kLHead + kLStages * l_stage_smem<TA, TX>(); }

__device__ __forceinline__ void cp_async_gather(void* dst, const void* src, int bytes) {
  if (bytes == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
// the stage's mbarrier also waits for this thread's earlier cp.async copies
// (its pending count is raised now and lowered when they land)
__device__ __forceinline__ void cp_async_arrive(uint64_t* bar) {
  asm volatile("cp.async.mbarrier.arrive.shared.b64 [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// The products of one staged stage for one lane (row i of slice sl): columns
// sl, sl + S, sl + 2S, ... of the stage, alternately into a0 and a1.  S (the
// slice count) is a compile-time constant so that the column strides are
// immediate offsets.
template <int S, typename TA, typename TX, typename TACC>
__device__ __forceinline__ void leaf_products(const TA* __restrict__ su, const TX* __restrict__ xs,
                                              const uint16_t* __restrict__ co, int C, int sl, int i,
                                              typename Acc<TACC>::A& a0, typename Acc<TACC>::A& a1) {
  using AC = Acc<TACC>;
  const TA* sui = su + i;
  const TX* px = xs + sl;
  const uint16_t* pc = co + sl;
  int c = sl;
  for (; c + 3 * S < C; c += 4 * S, px += 4 * S, pc += 4 * S) {
    const typename AC::X x0 = AC::in(px[0]), x1 = AC::in(px[S]), x2 = AC::in(px[2 * S]), x3 = AC::in(px[3 * S]);
    const TA v0 = sui[pc[0]], v1 = sui[pc[S]], v2 = sui[pc[2 * S]], v3 = sui[pc[3 * S]];
    AC::fma(a0, v0, x0);
    AC::fma(a1, v1, x1);
    AC::fma(a0, v2, x2);
    AC::fma(a1, v3, x3);
  }
  for (int k = 0; c < C; c += S, px += S, pc += S, k++) AC::fma((k & 1) ? a1 : a0, sui[pc[0]], AC::in(px[0]));
}

template <typename TA, typename TACC>
__global__ void __launch_bounds__(kLWarps * 32, HODLR_TUNE_L_MINB)
    panel_leaf_kernel(const Panel* __restrict__ panels, const Seg* __restrict__ segs, const Item* __restrict__ items,
                      int nitems, const typename IO<TACC>::TI* __restrict__ in, int64_t ld_in,
                      typename IO<TACC>::TY* __restrict__ y, int64_t ld_y, int nslots,
                      typename IO<TACC>::TY* __restrict__ ypart) {
  using TI = typename IO<TACC>::TI;
  using TX = typename LeafX<TACC>::T;
  using TY = typename IO<TACC>::TY;
  using AC = Acc<TACC>;
  constexpr int esz = int(sizeof(TA));
  constexpr bool kScaled = esz == 2;
  constexpr int kStage = l_stage_smem<TA, TX>(), kWarpSmem = l_warp_smem<TA, TX>();
  constexpr int kXOff = kLStageBytes, kOOff = kXOff + kLCols * int(sizeof(TX)), kSOff = kOOff + kLCols * 2;
  extern __shared__ __align__(16) unsigned char lsm[];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int w = blockIdx.x * kLWarps + wid;
  if (w >= nitems) return;
  const Item it = items[w];
  const Panel P = panels[it.panel];
  const int m = P.m;
  const int colb = m * esz;  // bytes per column
  const TI* inc = in + blockIdx.y * ld_in;
  TY* yo = y + int64_t(blockIdx.y) * nslots * ld_y + P.yoff;
  int mpad = 1;
  while (mpad < m) mpad <<= 1;
  const int slices = 32 / mpad;
  const int i = lane & (mpad - 1), sl = lane / mpad;
  unsigned char* base = lsm + wid * kWarpSmem;
  uint64_t* bar = reinterpret_cast<uint64_t*>(base);
  int2* meta = reinterpret_cast<int2*>(base + 32);  // per stage: column count, unused
  unsigned char* ring = base + kLHead;
  const int32_t qe = it.seg_e;
  const char* a0 = static_cast<const char*>(segs[it.seg_b].A);  // 16-byte aligned: every segment starts on 16 bytes
  if (lane == 0) {
#pragma unroll
    for (int s = 0; s < kLStages; s++) mbar_init(bar + s, 1u);
    fence_mbar_init();
  }
  __syncwarp();

  // next column to stage (the same in every lane): segment pq, column pj
  int32_t pq = it.seg_b, pj = 0;
  // lane k's record of segment rq + k, loaded a stage ahead of its use (the
  // first window of the next plan), so that its latency overlaps the products
  int32_t rq = -1, rK = 0, rso = 0;
  int64_t rino = 0;
  const float* rcs = nullptr;
  auto prefetch = [&]() {
    rq = pq;
    rK = 0;
    rso = 0;
    rino = 0;
    rcs = nullptr;
    if (pq + lane < qe) {
      const Seg S = segs[pq + lane];
      rK = S.K;
      rso = int32_t(static_cast<const char*>(S.A) - a0);
      rino = S.in_off;
      rcs = S.cscale;
    }
  };
  // Plans the stage from (pq, pj) into slot st and issues its copies; false
  // when every column is staged.  Warp-uniform.
  auto issue = [&](int st) -> bool {
    if (pq >= qe) return false;
    unsigned char* su = ring + st * kStage;
    TX* xs = reinterpret_cast<TX*>(su + kXOff);
    uint16_t* co = reinterpret_cast<uint16_t*>(su + kOOff);
    float* sc = reinterpret_cast<float*>(su + kSOff);
    int32_t sbase = 0, cols = 0, end = 0;
    bool first = true, more = true;
    while (more) {
      // lane k: segment pq + k, its first column to stage (pj for k = 0)
      const int32_t q = pq + lane;
      int32_t K = 0, so = 0;
      int64_t ino = 0;
      const float* cs = nullptr;
      if (pq == rq) {  // warp-uniform
        K = rK;
        so = rso;
        ino = rino;
        cs = rcs;
      } else if (q < qe) {
        const Seg S = segs[q];
        K = S.K;
        so = int32_t(static_cast<const char*>(S.A) - a0);
        ino = S.in_off;
        cs = S.cscale;
      }
      const int32_t j0 = lane == 0 ? pj : 0;
      const int32_t avail = max(K - j0, 0);
      if (first) sbase = (__shfl_sync(0xffffffffu, so + j0 * colb, 0)) & ~15;
      first = false;
      // columns of this segment whose end stays within the stage's bytes
      const int32_t room = sbase + kLStageBytes - so;
      int32_t fit = room >= colb * (j0 + 1) ? room / colb - j0 : 0;
      int32_t take = min(avail, fit);
      // segments after the first one that is not taken whole take nothing
      const unsigned part = __ballot_sync(0xffffffffu, take < avail || q >= qe);
      const int stop_at = part ? __ffs(part) - 1 : 32;  // first lane not taken whole
      if (lane > stop_at) take = 0;
      // the column cap: exclusive prefix sum of the takes
      int32_t pre = take;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int32_t v = __shfl_up_sync(0xffffffffu, pre, o);
        if (lane >= o) pre += v;
      }
      pre -= take;
      take = max(0, min(take, kLCols - cols - pre));
      // column table and gathers for this window: the taken columns in order
      int32_t incl = pre + take;  // columns before the end of this lane's share
      const int32_t total = __shfl_sync(0xffffffffu, incl, 31);
      const int32_t wcols = min(total, kLCols - cols);
      for (int c0 = 0; c0 < wcols; c0 += 32) {  // every lane takes part in the shuffles
        const int c = c0 + lane;
        // the lane k whose share holds column c: the shares with columns are
        // those of lanes 0, 1, ... in column order, so k is the number of
        // shares starting before column c0, plus the shares starting in
        // c0 .. c, minus one (one warp vote and one OR-reduction of the
        // share starts, no search)
        const bool owns = take > 0;
        const int k0 = __popc(__ballot_sync(0xffffffffu, owns && pre < c0));
        const uint32_t starts =
            __reduce_or_sync(0xffffffffu, owns && pre >= c0 && pre < c0 + 32 ? 1u << (pre - c0) : 0u);
        const int k = k0 - 1 + __popc(starts & (0xffffffffu >> (31 - lane)));
        const int32_t pk = __shfl_sync(0xffffffffu, pre, k);
        const int32_t jk = __shfl_sync(0xffffffffu, j0, k) + (c - pk);
        const int32_t sok = __shfl_sync(0xffffffffu, so, k);
        const int64_t ink = __shfl_sync(0xffffffffu, ino, k);
        unsigned long long csk = 0;
        if constexpr (kScaled) csk = __shfl_sync(0xffffffffu, reinterpret_cast<unsigned long long>(cs), k);
        if (c < wcols) {
          co[cols + c] = uint16_t((sok + jk * colb - sbase) / esz);
          // relaxed products stage only the high part (the first member) of a split input
          cp_async_gather(xs + cols + c, reinterpret_cast<const TX*>(inc + ink + jk), int(sizeof(TX)));
          if constexpr (kScaled) {
            if (csk)
              cp_async_gather(sc + cols + c, reinterpret_cast<const float*>(csk) + jk, 4);
            else
              sc[cols + c] = 1.f;
          }
        }
      }
      // the last lane with columns ends the stage's bytes and moves the cursor
      const unsigned has = __ballot_sync(0xffffffffu, take > 0);
      if (has) {
        const int kl = 31 - __clz(has);
        const int32_t e = __shfl_sync(0xffffffffu, so + (j0 + take) * colb, kl);
        const int32_t tk = __shfl_sync(0xffffffffu, take, kl), ak = __shfl_sync(0xffffffffu, avail, kl);
        const int32_t jl = __shfl_sync(0xffffffffu, j0, kl);
        end = e;
        if (tk < ak) {
          pq += kl;
          pj = jl + tk;
        } else {
          pq += kl + 1;
          pj = 0;
        }
      }
      cols += wcols;
      // another window of 32 segments only when all 32 were taken whole
      more = has == 0xffffffffu && stop_at == 32 && cols < kLCols && pq < qe;
    }
    cp_async_arrive(bar + st);
    if (lane == 0) meta[st] = make_int2(cols, 0);
    __syncwarp();
    if (lane == 0) {
      // end rounded up to 16 bytes stays inside the last segment's storage
      // (every segment occupies a multiple of 16 bytes), and end - sbase <= kLStageBytes
      const uint32_t bytes = uint32_t(((end + 15) & ~15) - sbase);
      fence_proxy_async();
      mbar_expect_tx(bar + st, bytes);
      bulk_g2s(su, a0 + sbase, bytes, bar + st);
    }
    return true;
  };

  int nissued = 0;
  prefetch();
  for (int s = 0; s < kLStages; s++) {
    if (!issue(s)) break;
    nissued++;
    prefetch();
  }
  typename AC::A a0acc = AC::zero(), a1acc = AC::zero();
  for (int k = 0; k < nissued; k++) {
    const int st = k % kLStages;
    const bool ok = __all_sync(0xffffffffu, mbar_wait(bar + st, uint32_t(k / kLStages) & 1u));
    if (!ok) {
      if (lane == 0) atomicAdd(&g_stream_timeouts, 1u);
      for (int t = k; t < nissued; t++) mbar_wait(bar + t % kLStages, uint32_t(t / kLStages) & 1u);
      cp_async_wait_all();
      return;
    }
    const int C = meta[st].x;
    const unsigned char* sb = ring + st * kStage;
    const TA* su = reinterpret_cast<const TA*>(sb);
    const TX* xs = reinterpret_cast<const TX*>(sb + kXOff);
    const uint16_t* co = reinterpret_cast<const uint16_t*>(sb + kOOff);
    const float* sc = reinterpret_cast<const float*>(sb + kSOff);
    if constexpr (kScaled) {
      // BF16: the staged inputs times their column scales, once per column
      // (lane c % 32 gathered column c and scales it), before the products
      TX* xw = const_cast<TX*>(xs);
      for (int c = lane; c < C; c += 32) put_staged(xw[c], AC::xscale(AC::in(xw[c]), sc[c]));
      __syncwarp();
    }
    if (i < m) {
      switch (slices) {
        case 32: leaf_products<32, TA, TX, TACC>(su, xs, co, C, sl, i, a0acc, a1acc); break;
        case 16: leaf_products<16, TA, TX, TACC>(su, xs, co, C, sl, i, a0acc, a1acc); break;
        case 8: leaf_products<8, TA, TX, TACC>(su, xs, co, C, sl, i, a0acc, a1acc); break;
        case 4: leaf_products<4, TA, TX, TACC>(su, xs, co, C, sl, i, a0acc, a1acc); break;
        case 2: leaf_products<2, TA, TX, TACC>(su, xs, co, C, sl, i, a0acc, a1acc); break;
        default: leaf_products<1, TA, TX, TACC>(su, xs, co, C, sl, i, a0acc, a1acc); break;
      }
    }
    __syncwarp();  // stage k's slot is refilled for stage k + kLStages
    if (issue(st)) {
      nissued++;
      prefetch();
    }
  }
  typename AC::A acc = AC::add(a0acc, a1acc);
  for (int o = mpad; o < 32; o <<= 1) acc = AC::add(acc, AC::shfl_xor(acc, o));
  if (sl == 0 && i < m) {
    if (it.part < 0)
      yo[i] = TY(AC::value(acc));
    else
      ypart[int64_t(it.part) * tile_rows(int(sizeof(TA))) + i] = TY(AC::value(acc));
  }
}

// Phase 2, panels of more than 32 rows: item chunk = row tile t of the
// panel (T = 512 / sizeof(TA) rows; a lane owns RPL = 16 / sizeof(TA) rows
// t*T + g*RPL ..).  A tile of rows <= 16 RPL rows needs fewer than 32 lanes
// per column: the warp then splits into slices of L lanes (L = the row
// groups rounded up to a power of two), slice sl taking the columns
// j = sl (mod 32 / L) of each segment, so that every lane has work (a
// 64-row BF16 tile keeps 8 lanes per column and 4 columns in flight).  Every
// segment's tile is h x K, column major with column stride h (h = the tile's
// row count rounded up to height_quantum rows), so a run of its columns is one contiguous byte
// range, and so is the run of their input values.  Both are staged through a
// per-warp ring of kPStages shared-memory stages by bulk copies, at most
// kPStageBytes of tile and kPCols columns per stage.  Within one stage a
// slice's k-th column goes to accumulator set k & 1; the slices' sums are
// added by shuffles at the end.  BF16 dense tiles: the warp multiplies the
// staged inputs by the column scales first, once, in place.
constexpr int kPWarps = 4;           // warps per CTA of panel_tile_kernel
constexpr int kPStages = HODLR_TUNE_P_STAGES;
constexpr int kPStageBytes = HODLR_TUNE_P_BYTES;
constexpr int kPCols = 64;           // columns per stage at most
constexpr int kPXBytes = kPCols * 8 + 32;
constexpr int kPWarpSmem = 64 + kPStages * (kPStageBytes + kPXBytes);
static_assert(kPWarpSmem % 16 == 0 && kPXBytes % 16 == 0, "bulk copy destinations must stay 16-byte aligned");

template <typename TA, typename TACC>
__global__ void __launch_bounds__(kPWarps * 32, HODLR_TUNE_P_MINB)
    panel_tile_kernel(const Panel* __restrict__ panels, const Seg* __restrict__ segs, const Item* __restrict__ items,
                      int nitems, typename IO<TACC>::TY* __restrict__ ypart,
                      const typename IO<TACC>::TI* __restrict__ in, int64_t ld_in,
                      typename IO<TACC>::TY* __restrict__ y, int64_t ld_y, int nslots) {
  using TX = typename IO<TACC>::TI;
  using TY = typename IO<TACC>::TY;
  constexpr int RPL = 16 / int(sizeof(TA));
  constexpr int T = 32 * RPL;
  using VT = typename Vec16<TA>::type;
  using AC = Acc<TACC>;
  extern __shared__ __align__(16) unsigned char psm[];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int w = blockIdx.x * kPWarps + wid;
  if (w >= nitems) return;
  const Item it = items[w];
  const Panel P = panels[it.panel];
  const int m = P.m;
  const TX* inc = in + blockIdx.y * ld_in;
  const int t = it.chunk;
  const int rows = min(T, m - t * T);
  const int64_t h = tile_height(m, t, int(sizeof(TA)));
  const int colb = int(h) * int(sizeof(TA));  // bytes per tile column: 16 .. 512, a multiple of 16
  const int cps = min(kPCols, kPStageBytes / colb);
  int lg = 1;  // lanes per slice
  while (lg * RPL < rows) lg <<= 1;
  const int slices = 32 / lg;
  const int g = lane & (lg - 1), sl = lane / lg;
  const bool act = g * RPL < rows;
  typename AC::A a0[RPL], a1[RPL];
#pragma unroll
  for (int q = 0; q < RPL; q++) a0[q] = a1[q] = AC::zero();

  unsigned char* base = psm + wid * kPWarpSmem;
  uint64_t* bar = reinterpret_cast<uint64_t*>(base);
  unsigned char* ubuf = base + 64;
  unsigned char* xbuf = ubuf + kPStages * kPStageBytes;
  if (lane == 0) {
#pragma unroll
    for (int s = 0; s < kPStages; s++) mbar_init(bar + s, 1);
    fence_mbar_init();
  }
  __syncwarp();
  // producer cursor (segment, first column); every lane keeps it, lane 0 issues
  int64_t ps = it.seg_b;
  int pc = 0, issued = 0;
#define HODLR_PANEL_ISSUE_NEXT()                                                                                  \
  do {                                                                                                            \
    while (ps < it.seg_e && pc >= segs[ps].K) {                                                                   \
      ps++;                                                                                                       \
      pc = 0;                                                                                                     \
    }                                                                                                             \
    if (ps >= it.seg_e) break;                                                                                    \
    const Seg S_ = segs[ps];                                                                                      \
    const int nc_ = min(cps, S_.K - pc);                                                                          \
    if (lane == 0) {                                                                                              \
      const int st_ = issued % kPStages;                                                                          \
      /* U tile t starts at element t*T*K: 16-byte aligned since T * sizeof(TA) = 512 */                          \
      const TA* src_ = static_cast<const TA*>(S_.A) + int64_t(t) * T * S_.K + int64_t(pc) * h;                    \
      const uint32_t ub_ = uint32_t(nc_) * uint32_t(colb);                                                        \
      const unsigned char* xs_ = reinterpret_cast<const unsigned char*>(inc + S_.in_off + pc);                    \
      const unsigned char* xa_ = static_cast<const unsigned char*>(align_down16(xs_));                            \
      const uint32_t xb_ = uint32_t((xs_ + size_t(nc_) * sizeof(TX) - xa_ + 15) & ~size_t(15));                   \
      fence_proxy_async();                                                                                        \
      mbar_expect_tx(bar + st_, ub_ + xb_);                                                                       \
      bulk_g2s(ubuf + st_ * kPStageBytes, src_, ub_, bar + st_);                                                  \
      bulk_g2s(xbuf + st_ * kPXBytes, xa_, xb_, bar + st_);                                                       \
    }                                                                                                             \
    pc += nc_;                                                                                                    \
    issued++;                                                                                                     \
  } while (0)
  for (int q = 0; q < kPStages; q++) HODLR_PANEL_ISSUE_NEXT();
  // consumer cursor
  int64_t cs = it.seg_b;
  int cc = 0;
  for (int q = 0; q < issued; q++) {
    while (cc >= segs[cs].K) {
      cs++;
      cc = 0;
    }
    const Seg S = segs[cs];
    const int nc = min(cps, S.K - cc);
    const int st = q % kPStages;
    const bool ok = __all_sync(0xffffffffu, mbar_wait(bar + st, uint32_t(q / kPStages) & 1u));
    if (!ok) {
      if (lane == 0) atomicAdd(&g_stream_timeouts, 1u);
      for (int u = q; u < issued; u++) mbar_wait(bar + u % kPStages, uint32_t(u / kPStages) & 1u);
      return;
    }
    const int xo = int((reinterpret_cast<uintptr_t>(inc + S.in_off + cc) & 15u) / sizeof(TX));
    const TX* xsm = reinterpret_cast<const TX*>(xbuf + st * kPXBytes) + xo;
    const unsigned char* us = ubuf + st * kPStageBytes + g * 16;
    if constexpr (sizeof(TA) == 2) {
      // BF16 dense tile: the staged inputs times the column scales, once, in place
      if (S.cscale) {
        TX* xw = const_cast<TX*>(xsm);
        for (int j = lane; j < nc; j += 32) xw[j] = x_pair<TACC>(seg_in<TACC>(xw[j], S.cscale, cc + j));
        __syncwarp();
      }
    }
#define HODLR_XIN(j_) AC::in(xsm[j_])
    // this slice's columns of the stage: segment columns cc + j, j = sl (mod slices)
    int j = (sl - cc) & (slices - 1);
    for (; j + slices < nc; j += 2 * slices) {
      const VT v0 = act ? *reinterpret_cast<const VT*>(us + j * colb) : vzero<VT>();
      const VT v1 = act ? *reinterpret_cast<const VT*>(us + (j + slices) * colb) : vzero<VT>();
      axpy16<TACC>(v0, HODLR_XIN(j), a0);
      axpy16<TACC>(v1, HODLR_XIN(j + slices), a1);
    }
    if (j < nc) {
      const VT v0 = act ? *reinterpret_cast<const VT*>(us + j * colb) : vzero<VT>();
      axpy16<TACC>(v0, HODLR_XIN(j), a0);
    }
#undef HODLR_XIN
    cc += nc;
    __syncwarp();
    HODLR_PANEL_ISSUE_NEXT();  // the next run, if any, into the stage just consumed
  }
#undef HODLR_PANEL_ISSUE_NEXT
#pragma unroll
  for (int q = 0; q < RPL; q++) {
    a0[q] = AC::add(a0[q], a1[q]);
    for (int o = lg; o < 32; o <<= 1) a0[q] = AC::add(a0[q], AC::shfl_xor(a0[q], o));
  }
  if (act && sl == 0) {
    const int i = t * T + g * RPL;
    TY* dst = it.part < 0 ? y + int64_t(blockIdx.y) * nslots * ld_y + P.yoff + i
                          : ypart + int64_t(it.part) * T + g * RPL;
#pragma unroll
    for (int q = 0; q < RPL; q++)
      if (i + q < m) dst[q] = TY(AC::value(a0[q]));
  }
}

// ---- direct-load variants, used for FP64 factors ----------------------------
// FP64 products run on GB300's FP64 pipe, whose rate (not the bytes in
// flight) bounds these kernels; plain loads with eight warps per CTA keep
// that pipe busier than the shared-memory staged versions above.  Lane
// layouts as described above for each phase; the node-panel variant keeps
// one column per warp step (no column slices), with columns alternating
// between the two accumulator sets.
template <typename TA, typename TACC>
__global__ void __launch_bounds__(256) zgemv_direct_kernel(const ZBlock* __restrict__ zb, const ZItem* __restrict__ items,
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

template <typename TA, typename TACC>
__global__ void __launch_bounds__(256)
    panel_small_direct_kernel(const Panel* __restrict__ panels, const Seg* __restrict__ segs, const Item* __restrict__ items,
                       int nitems, const typename IO<TACC>::TI* __restrict__ in, int64_t ld_in,
                       typename IO<TACC>::TY* __restrict__ y, int64_t ld_y, int nslots,
                       typename IO<TACC>::TY* __restrict__ ypart) {
  using TX = typename IO<TACC>::TI;
  using TY = typename IO<TACC>::TY;
  const int w = blockIdx.x * kWarpsPerCta + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= nitems) return;
  const Item it = items[w];
  const Panel P = panels[it.panel];
  const int m = P.m;
  const TX* inc = in + blockIdx.y * ld_in;
  TY* yo = y + int64_t(blockIdx.y) * nslots * ld_y + P.yoff;
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
  // a panel whose columns are split over several items: partial rows at
  // ypart[part * tile_rows], added in part order by panel_fix_kernel
  if (sl == 0 && i < m) {
    if (it.part < 0)
      yo[i] = TY(AC::value(acc));
    else
      ypart[int64_t(it.part) * tile_rows(int(sizeof(TA))) + i] = TY(AC::value(acc));
  }
}

template <typename TA, typename TACC>
__global__ void __launch_bounds__(256)
    panel_tile_direct_kernel(const Panel* __restrict__ panels, const Seg* __restrict__ segs, const Item* __restrict__ items,
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
    TY* dst = it.part < 0 ? y + int64_t(blockIdx.y) * nslots * ld_y + P.yoff + i
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
  y[int64_t(blockIdx.y) * nslots * ld_y + P.yoff + i] = acc;
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
  double* u64 = static_cast<double*>(B.u64_dst);  // the FP64 copy too, when asked for
  constexpr int esz = int(sizeof(TO));
  if (B.kscale != 0.0) K.scale = B.kscale;
  if (B.dense) {
    const int64_t total = int64_t(B.m) * B.n;
    for (int64_t e = threadIdx.x; e < total; e += blockDim.x) {
      const int i = int(e % B.m), j = int(e / B.m);
      double xi[D];
      load_point<D>(P, B.t_begin + i, xi);
      const double a = kernel_entry<D>(P, K, B.t_begin + i, B.s_begin + j, xi);
      u[elem_offset(i, j, B.m, B.n, esz)] = TO(a);
      if (u64) u64[elem_offset(i, j, B.m, B.n, 8)] = a;
    }
  } else {
    const double* U = ws + B.ws;
    const int64_t nu = int64_t(B.m) * B.rank;
    for (int64_t e = threadIdx.x; e < nu; e += blockDim.x) {
      const int i = int(e % B.m), k = int(e / B.m);
      const int64_t row = lmap[B.t_map + i] - B.t_begin;
      u[elem_offset(row, k, B.m, B.rank, esz)] = TO(U[e]);
      if (u64) u64[elem_offset(row, k, B.m, B.rank, 8)] = U[e];
    }
    // V follows U's full workspace (m x cap); stored row major, n x vpad(rank)
    const double* Vw = ws + B.ws + int64_t(B.m) * B.cap;
    TO* v = static_cast<TO*>(B.v_dst);
    double* v64 = static_cast<double*>(B.v64_dst);
    const int64_t rp = vpad(B.rank, esz), rp64 = vpad(B.rank, 8);
    const int64_t nv = int64_t(B.n) * B.rank;
    for (int64_t e = threadIdx.x; e < nv; e += blockDim.x) {
      const int j = int(e % B.n), k = int(e / B.n);
      const int64_t row = lmap[B.s_map + j] - B.s_begin;
      v[row * rp + k] = TO(Vw[e]);
      if (v64) v64[row * rp64 + k] = Vw[e];
    }
  }
}

// BF16 storage of the same blocks, every factor scaled per column.  A dense
// tile keeps, per column j, the FP32 scale c_j = max_i |A_ij| (in s_dst) and
// the BF16 entries A_ij / c_j (round to nearest even); a low-rank block keeps
// per column k the scales su_k = max_i |U_ik|, sv_k = max_j |V_jk| and
// U_ik / su_k, V_jk / sv_k in BF16, with su_k * sv_k (the scale of
// z_k = V_k^T x) in s_dst.  A zero column gets scale 1.  One warp per column.
__device__ __forceinline__ unsigned short to_bf16_bits(double v) {
  return __bfloat16_as_ushort(__float2bfloat16_rn(float(v)));
}
__device__ __forceinline__ double warp_max(double v) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

template <int D>
__global__ void __launch_bounds__(256) compact_bf16_kernel(PointsDev P, KernelDev K, const double* __restrict__ ws,
                                                           const int32_t* __restrict__ lmap,
                                                           const CompactDesc* __restrict__ blocks, int nblocks) {
  const CompactDesc B = blocks[blockIdx.x];
  unsigned short* u = static_cast<unsigned short*>(B.u_dst);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  if (B.kscale != 0.0) K.scale = B.kscale;
  if (B.dense) {
    for (int j = warp; j < B.n; j += nw) {
      double mx = 0.0;
      for (int i = lane; i < B.m; i += 32) {
        double xi[D];
        load_point<D>(P, B.t_begin + i, xi);
        mx = fmax(mx, fabs(kernel_entry<D>(P, K, B.t_begin + i, B.s_begin + j, xi)));
      }
      mx = warp_max(mx);
      const float sc = mx > 0.0 ? float(mx) : 1.0f;
      for (int i = lane; i < B.m; i += 32) {
        double xi[D];
        load_point<D>(P, B.t_begin + i, xi);
        u[elem_offset(i, j, B.m, B.n, 2)] = to_bf16_bits(kernel_entry<D>(P, K, B.t_begin + i, B.s_begin + j, xi) / sc);
      }
      if (lane == 0) B.s_dst[j] = sc;
    }
  } else {
    const double* Vw = ws + B.ws + int64_t(B.m) * B.cap;
    unsigned short* v = static_cast<unsigned short*>(B.v_dst);
    const int64_t rp = vpad(B.rank, 2);
    for (int k = warp; k < B.rank; k += nw) {
      const double* Uk = ws + B.ws + int64_t(k) * B.m;
      const double* Vk = Vw + int64_t(k) * B.n;
      double mu = 0.0, mv = 0.0;
      for (int i = lane; i < B.m; i += 32) mu = fmax(mu, fabs(Uk[i]));
      for (int j = lane; j < B.n; j += 32) mv = fmax(mv, fabs(Vk[j]));
      mu = warp_max(mu);
      mv = warp_max(mv);
      const float su = mu > 0.0 ? float(mu) : 1.0f, sv = mv > 0.0 ? float(mv) : 1.0f;
      for (int i = lane; i < B.m; i += 32)
        u[elem_offset(lmap[B.t_map + i] - B.t_begin, k, B.m, B.rank, 2)] = to_bf16_bits(Uk[i] / su);
      for (int j = lane; j < B.n; j += 32) v[(lmap[B.s_map + j] - B.s_begin) * rp + k] = to_bf16_bits(Vk[j] / sv);
      if (lane == 0) B.s_dst[k] = su * sv;
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

void z_item_stages(ZItem& it, int r, int esz) {
  const int rp = int(vpad(r, esz));
  it.R = it.nst = 0;
  if (it.k0 != 0 || it.nk != rp || it.j1 <= it.j0) return;
  const int lanes = (it.nk + 16 / esz - 1) / (16 / esz);
  int P = 1;
  while (P < lanes) P <<= 1;
  const int G = 32 / P, rowb = rp * esz;
  it.R = (kZStageBytes / rowb) / G * G;  // >= G: rowb <= 16 P, kZStageBytes >= 512
  it.nst = (it.j1 - it.j0 + it.R - 1) / it.R;
}

template <typename TA, typename TACC>
static void zgemv_t(const ZBlock* zb, const ZItem* items, int nitems, const ZFix* fix, int nfix, void* zpart, void* in,
                    int64_t ld_in, int nrhs, cudaStream_t st) {
  using TI = typename IO<TACC>::TI;
  using TY = typename IO<TACC>::TY;
  if constexpr (sizeof(TA) == 8) {  // FP64 storage: direct loads
    dim3 g(warps_grid(nitems), unsigned(nrhs));
    zgemv_direct_kernel<TA, TACC><<<g, 256, 0, st>>>(zb, items, nitems, static_cast<TY*>(zpart),
                                                     static_cast<TI*>(in), ld_in);
  } else {
    dim3 g(unsigned((nitems + kZWarps - 1) / kZWarps), unsigned(nrhs));
    cudaFuncSetAttribute(zgemv_kernel<TA, TACC>, cudaFuncAttributeMaxDynamicSharedMemorySize, kZWarps * kZWarpSmem);
    zgemv_kernel<TA, TACC><<<g, kZWarps * 32, kZWarps * kZWarpSmem, st>>>(zb, items, nitems, static_cast<TY*>(zpart),
                                                                           static_cast<TI*>(in), ld_in);
  }
  if (nfix > 0) {
    dim3 gf(unsigned((nfix + 255) / 256), unsigned(nrhs));
    zfix_kernel<TACC><<<gf, 256, 0, st>>>(fix, nfix, static_cast<const TY*>(zpart), static_cast<TI*>(in), ld_in);
  }
}

cudaError_t launch_zgemv(Prec a, Prec x, const ZBlock* zb, const ZItem* items, int nitems, const ZFix* fix, int nfix,
                         void* zpart, void* in, int64_t ld_in, int nrhs, cudaStream_t st, Accum acc) {
  if (nitems <= 0) return cudaSuccess;
  count_launches(nfix > 0 ? 2 : 1);
  if (a == Prec::kD && x == Prec::kD)
    zgemv_t<double, double>(zb, items, nitems, fix, nfix, zpart, in, ld_in, nrhs, st);
  else if (a == Prec::kF && x == Prec::kD && acc == Accum::kCompensated)
    zgemv_t<float, DF>(zb, items, nitems, fix, nfix, zpart, in, ld_in, nrhs, st);
  else if (a == Prec::kF && x == Prec::kD && acc == Accum::kRelaxed)
    zgemv_t<float, FH>(zb, items, nitems, fix, nfix, zpart, in, ld_in, nrhs, st);
  else if (a == Prec::kB && x == Prec::kD && acc == Accum::kRelaxed)
    zgemv_t<bf16, FH>(zb, items, nitems, fix, nfix, zpart, in, ld_in, nrhs, st);
  else if (a == Prec::kB && x == Prec::kD)
    zgemv_t<bf16, DF>(zb, items, nitems, fix, nfix, zpart, in, ld_in, nrhs, st);
  else if (a == Prec::kF && x == Prec::kF)
    zgemv_t<float, float>(zb, items, nitems, fix, nfix, zpart, in, ld_in, nrhs, st);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

// FP32 and BF16 storage: the bulk-copy staged kernels
template <typename TA, typename TACC>
static void panels_leaf(const Panel* panels, const Seg* segs, const Item* small, int nsmall, const void* in,
                        int64_t ld_in, void* ypart, void* y, int64_t ld_y, int nslots, int nrhs, cudaStream_t st) {
  using TI = typename IO<TACC>::TI;
  using TY = typename IO<TACC>::TY;
  using TX = typename LeafX<TACC>::T;
  dim3 g(unsigned((nsmall + kLWarps - 1) / kLWarps), unsigned(nrhs));
  cudaFuncSetAttribute(panel_leaf_kernel<TA, TACC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       kLWarps * l_warp_smem<TA, TX>());
  panel_leaf_kernel<TA, TACC><<<g, kLWarps * 32, kLWarps * l_warp_smem<TA, TX>(), st>>>(
      panels, segs, small, nsmall, static_cast<const TI*>(in), ld_in, static_cast<TY*>(y), ld_y, nslots,
      static_cast<TY*>(ypart));
}

template <typename TA, typename TACC>
static void panels_staged(const Panel* panels, const Seg* segs, const Item* small, int nsmall, const Item* big,
                          int nbig, const void* in, int64_t ld_in, void* ypart, void* y, int64_t ld_y, int nslots,
                          int nrhs, cudaStream_t st, bool contig) {
  using TI = typename IO<TACC>::TI;
  using TY = typename IO<TACC>::TY;
  if (nbig > 0) {
    dim3 g(unsigned((nbig + kPWarps - 1) / kPWarps), unsigned(nrhs));
    // above the default 48 KB of dynamic shared memory; set on every launch
    // (the attribute is per device and cheap to set)
    cudaFuncSetAttribute(panel_tile_kernel<TA, TACC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         kPWarps * kPWarpSmem);
    panel_tile_kernel<TA, TACC><<<g, kPWarps * 32, kPWarps * kPWarpSmem, st>>>(
        panels, segs, big, nbig, static_cast<TY*>(ypart), static_cast<const TI*>(in), ld_in, static_cast<TY*>(y), ld_y,
        nslots);
  }
  if (nsmall > 0 && contig) {
    panels_leaf<TA, TACC>(panels, segs, small, nsmall, in, ld_in, ypart, y, ld_y, nslots, nrhs, st);
  } else if (nsmall > 0) {
    dim3 g(unsigned((nsmall + kSWarps - 1) / kSWarps), unsigned(nrhs));
    cudaFuncSetAttribute(panel_small_kernel<TA, TACC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         kSWarps * s_warp_smem<TA>());
    panel_small_kernel<TA, TACC><<<g, kSWarps * 32, kSWarps * s_warp_smem<TA>(), st>>>(
        panels, segs, small, nsmall, static_cast<const TI*>(in), ld_in, static_cast<TY*>(y), ld_y, nslots,
        static_cast<TY*>(ypart));
  }
}

template <typename TA, typename TACC>
static void panels_t(const Panel* panels, const Seg* segs, const Item* small, int nsmall, const Item* big, int nbig,
                     const PanelFix* fix, int nfix, void* ypart, const void* in, int64_t ld_in, void* y, int64_t ld_y,
                     int nslots, int nrhs, cudaStream_t st, bool contig) {
  using TI = typename IO<TACC>::TI;
  using TY = typename IO<TACC>::TY;
  if constexpr (sizeof(TA) == 8) {  // FP64 storage: direct loads
    if (nbig > 0) {
      dim3 g(warps_grid(nbig), unsigned(nrhs));
      panel_tile_direct_kernel<TA, TACC><<<g, 256, 0, st>>>(panels, segs, big, nbig, static_cast<TY*>(ypart),
                                                            static_cast<const TI*>(in), ld_in, static_cast<TY*>(y),
                                                            ld_y, nslots);
    }
    if (nsmall > 0 && contig) {
      panels_leaf<TA, TACC>(panels, segs, small, nsmall, in, ld_in, ypart, y, ld_y, nslots, nrhs, st);
    } else if (nsmall > 0) {
      dim3 g(warps_grid(nsmall), unsigned(nrhs));
      panel_small_direct_kernel<TA, TACC><<<g, 256, 0, st>>>(panels, segs, small, nsmall, static_cast<const TI*>(in),
                                                             ld_in, static_cast<TY*>(y), ld_y, nslots,
                                                             static_cast<TY*>(ypart));
    }
  } else {
    panels_staged<TA, TACC>(panels, segs, small, nsmall, big, nbig, in, ld_in, ypart, y, ld_y, nslots, nrhs, st,
                            contig);
  }
  if (nfix > 0) {
    const int rows = int(tile_rows(int(sizeof(TA))));
    dim3 gf(unsigned((int64_t(nfix) * rows + 255) / 256), unsigned(nrhs));
    panel_fix_kernel<TY><<<gf, 256, 0, st>>>(panels, fix, nfix, rows, static_cast<const TY*>(ypart),
                                             static_cast<TY*>(y), ld_y, nslots);
  }
}


bool small_items_contiguous(const std::vector<Panel>& panels, const std::vector<Seg>& segs,
                            const std::vector<Item>& small, int esz) {
  for (const Item& it : small) {
    const int64_t m = panels[size_t(it.panel)].m;
    if (m < 1 || m > 32) return false;
    const char* a0 = static_cast<const char*>(segs[size_t(it.seg_b)].A);
    if (reinterpret_cast<uintptr_t>(a0) % 16 != 0) return false;
    const char* next = a0;  // end of the previous segment's columns
    for (int32_t q = it.seg_b; q < it.seg_e; q++) {
      const char* a = static_cast<const char*>(segs[size_t(q)].A);
      // each segment starts on 16 bytes after the previous one's data; offsets
      // from the item's first segment stay far below 2^31
      if (a < next || reinterpret_cast<uintptr_t>(a) % 16 != 0 || a - a0 > (int64_t(1) << 30)) return false;
      next = a + m * int64_t(segs[size_t(q)].K) * esz;
    }
  }
  return true;
}

cudaError_t launch_panels(Prec a, Prec x, const Panel* panels, const Seg* segs, const Item* small, int nsmall,
                          const Item* big, int nbig, const PanelFix* fix, int nfix, void* ypart, const void* in,
                          int64_t ld_in, void* y, int64_t ld_y, int nslots, int nrhs, cudaStream_t st, Accum acc,
                          bool contig) {
  if (nsmall + nbig <= 0) return cudaSuccess;
  count_launches(uint64_t(nbig > 0) + uint64_t(nsmall > 0) + uint64_t(nfix > 0));
  if (a == Prec::kD && x == Prec::kD)
    panels_t<double, double>(panels, segs, small, nsmall, big, nbig, fix, nfix, ypart, in, ld_in, y, ld_y, nslots,
                             nrhs, st, contig);
  else if (a == Prec::kF && x == Prec::kD && acc == Accum::kCompensated)
    panels_t<float, DF>(panels, segs, small, nsmall, big, nbig, fix, nfix, ypart, in, ld_in, y, ld_y, nslots, nrhs,
                        st, contig);
  else if (a == Prec::kF && x == Prec::kD && acc == Accum::kRelaxed)
    panels_t<float, FH>(panels, segs, small, nsmall, big, nbig, fix, nfix, ypart, in, ld_in, y, ld_y, nslots, nrhs,
                        st, contig);
  else if (a == Prec::kB && x == Prec::kD && acc == Accum::kRelaxed)
    panels_t<bf16, FH>(panels, segs, small, nsmall, big, nbig, fix, nfix, ypart, in, ld_in, y, ld_y, nslots, nrhs,
                       st, contig);
  else if (a == Prec::kB && x == Prec::kD)
    panels_t<bf16, DF>(panels, segs, small, nsmall, big, nbig, fix, nfix, ypart, in, ld_in, y, ld_y, nslots, nrhs,
                       st, contig);
  else if (a == Prec::kF && x == Prec::kF)
    panels_t<float, float>(panels, segs, small, nsmall, big, nbig, fix, nfix, ypart, in, ld_in, y, ld_y, nslots, nrhs,
                           st, contig);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

template <typename T>
__global__ void __launch_bounds__(256) batch_gather_kernel(const BatchInst* __restrict__ inst, const T* __restrict__ x,
                                                           T* __restrict__ in) {
  const BatchInst I = inst[blockIdx.y];
  for (int64_t r = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; r < I.n; r += int64_t(gridDim.x) * blockDim.x)
    in[I.in_base + r] = x[I.x_base + I.perm[r]];
}

template <typename T>
__global__ void __launch_bounds__(256) batch_combine_kernel(const BatchInst* __restrict__ inst, const T* __restrict__ y,
                                                            T* __restrict__ out) {
  const BatchInst I = inst[blockIdx.y];
  for (int64_t r = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; r < I.n; r += int64_t(gridDim.x) * blockDim.x) {
    const T* yc = y + I.y_base + r;
    double acc = double(yc[0]);
    for (int s = 1; s < I.nslots; s++) acc += double(yc[int64_t(s) * I.n]);
    out[I.x_base + I.perm[r]] = T(acc);
  }
}

namespace {
dim3 batch_grid(int count, int64_t max_n) {
  int64_t g = (max_n + 255) / 256;
  if (g > 64) g = 64;
  if (g < 1) g = 1;
  return dim3(unsigned(g), unsigned(count));
}
}  // namespace

cudaError_t launch_batch_gather(Prec x, const BatchInst* inst, int count, int64_t max_n, const void* src, void* in,
                                cudaStream_t st) {
  if (count <= 0) return cudaSuccess;
  count_launches(1);
  if (x == Prec::kD)
    batch_gather_kernel<double><<<batch_grid(count, max_n), 256, 0, st>>>(inst, static_cast<const double*>(src),
                                                                           static_cast<double*>(in));
  else
    batch_gather_kernel<float><<<batch_grid(count, max_n), 256, 0, st>>>(inst, static_cast<const float*>(src),
                                                                          static_cast<float*>(in));
  return cudaGetLastError();
}

cudaError_t launch_batch_combine(Prec x, const BatchInst* inst, int count, int64_t max_n, const void* y, void* out,
                                 cudaStream_t st) {
  if (count <= 0) return cudaSuccess;
  count_launches(1);
  if (x == Prec::kD)
    batch_combine_kernel<double><<<batch_grid(count, max_n), 256, 0, st>>>(inst, static_cast<const double*>(y),
                                                                            static_cast<double*>(out));
  else
    batch_combine_kernel<float><<<batch_grid(count, max_n), 256, 0, st>>>(inst, static_cast<const float*>(y),
                                                                           static_cast<float*>(out));
  return cudaGetLastError();
}

__global__ void __launch_bounds__(128) copy16_kernel(const CopyDesc* __restrict__ d) {
  const CopyDesc D = d[blockIdx.x];
  const int4* s = static_cast<const int4*>(D.src);
  int4* t = static_cast<int4*>(D.dst);
  for (uint64_t i = threadIdx.x; i < D.bytes / 16; i += blockDim.x) t[i] = s[i];
}

// One CTA per descriptor: 16-byte units of every row.
__global__ void __launch_bounds__(128) copy_rows_kernel(const RowCopy* __restrict__ d) {
  const RowCopy D = d[blockIdx.x];
  const int units = D.row_bytes / 16;
  const int64_t total = int64_t(units) * D.rows;
  for (int64_t e = threadIdx.x; e < total; e += blockDim.x) {
    const int64_t row = e / units, u = e - row * units;
    *reinterpret_cast<int4*>(static_cast<char*>(D.dst) + row * D.dst_pitch + u * 16) =
        *reinterpret_cast<const int4*>(static_cast<const char*>(D.src) + row * D.src_pitch + u * 16);
  }
}

cudaError_t launch_copy_rows(const RowCopy* d, int n, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  count_launches(1);
  copy_rows_kernel<<<unsigned(n), 128, 0, st>>>(d);
  return cudaGetLastError();
}

cudaError_t launch_copy16(const CopyDesc* d, int n, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  count_launches(1);
  copy16_kernel<<<unsigned(n), 128, 0, st>>>(d);
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
  else if (op == Prec::kB)
    compact_bf16_kernel<D><<<unsigned(nblocks), 256, 0, st>>>(P, K, ws, lmap, blocks, nblocks);
  else
    compact_kernel<D, float><<<unsigned(nblocks), 256, 0, st>>>(P, K, ws, lmap, blocks, nblocks);
}

template <int D>
static cudaError_t compact_preload_d() {
  cudaFuncAttributes fa;
  cudaError_t e = cudaFuncGetAttributes(&fa, compact_kernel<D, double>);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, compact_kernel<D, float>);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, compact_bf16_kernel<D>);
  return e;
}

cudaError_t compact_preload(int ndim) {
  switch (ndim) {
    case 1: return compact_preload_d<1>();
    case 2: return compact_preload_d<2>();
    case 3: return compact_preload_d<3>();
    case 4: return compact_preload_d<4>();
    case 5: return compact_preload_d<5>();
    case 6: return compact_preload_d<6>();
    case 7: return compact_preload_d<7>();
    case 8: return compact_preload_d<8>();
    default: return cudaErrorInvalidValue;
  }
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


// ============================================================================
// Several right-hand sides at once: FP32 factors, FP32 vectors, FP32 sums.
// A chunk of kMR right-hand sides is interleaved: entry e of a vector buffer
// holds its kMR values contiguously (byte offset e * 4 kMR), so one input row
// or z row is one 128-byte run that the bulk-copy engine stages next to the
// factor bytes, and every factor entry read from HBM feeds kMR FMAs.  The
// lane layouts are those of the single-vector kernels, each lane keeping kMR
// sums per matrix row or column it owns; grid.y runs over chunks.
// ============================================================================
namespace {

constexpr int kMWarps = 4;
constexpr int kMStages = 2;
constexpr int kMVBytes = 4096;                 // factor bytes per stage
constexpr int kMXBytes = 4096;                 // input bytes per stage (32 rows of kMR floats)
constexpr int kMRowBytes = kMR * 4;            // one interleaved entry
constexpr int kMWarpSmem = 64 + kMStages * (kMVBytes + kMXBytes);
static_assert(kMWarpSmem % 16 == 0, "bulk copy destinations must stay 16-byte aligned");

__device__ __forceinline__ void fma4x(float a, const float4& x, float* acc) {
  acc[0] = __fmaf_rn(a, x.x, acc[0]);
  acc[1] = __fmaf_rn(a, x.y, acc[1]);
  acc[2] = __fmaf_rn(a, x.z, acc[2]);
  acc[3] = __fmaf_rn(a, x.w, acc[3]);
}

// Lane c of a warp owns right-hand side c of the chunk (kMR = 32 = warp
// width): it reads its input value of a row with one conflict-free shared
// load, the row's factor values with broadcast 16-byte loads, and keeps one
// sum per output row or column it produces -- no cross-lane reductions, and
// every output row is one coalesced 128-byte store.

// z_b = V_b^T X_s: item = rows [j0, j1) of block zb (all columns); passes of
// kMCols columns (one pass unless r > kMCols); runs of whole V rows and their
// input rows staged by bulk copies in a ring of kMStages.
constexpr int kMCols = 64;

// acc[c] += V[i][c] x[i] over the stage's rows, NC4 groups of 4 columns
template <int NC4>
__device__ __forceinline__ void mr_rows(const unsigned char* vs, int rowb, const float* xs, int nr, int lane,
                                        float (&acc)[kMCols]) {
  for (int i = 0; i < nr; i++) {
    const float x = xs[i * kMR + lane];
    const float4* v4 = reinterpret_cast<const float4*>(vs + i * rowb);
#pragma unroll
    for (int c = 0; c < NC4; c++) {
      const float4 v = v4[c];
      acc[4 * c] = __fmaf_rn(v.x, x, acc[4 * c]);
      acc[4 * c + 1] = __fmaf_rn(v.y, x, acc[4 * c + 1]);
      acc[4 * c + 2] = __fmaf_rn(v.z, x, acc[4 * c + 2]);
      acc[4 * c + 3] = __fmaf_rn(v.w, x, acc[4 * c + 3]);
    }
  }
}

__global__ void __launch_bounds__(kMWarps * 32, 3)
    zgemv_mr_kernel(const ZBlock* __restrict__ zb, const ZItem* __restrict__ items, int nitems,
                    float* __restrict__ zpart, int64_t zpart_ld, float* in, int64_t ld_in) {
  extern __shared__ __align__(16) unsigned char msm[];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int w = blockIdx.x * kMWarps + wid;
  if (w >= nitems) return;
  const ZItem it = items[w];
  const ZBlock Z = zb[it.zb];
  const int64_t rp = vpad(Z.r, 4);
  float* inc = in + int64_t(blockIdx.y) * ld_in * kMR;
  float* zp = zpart + int64_t(blockIdx.y) * zpart_ld * kMR;
  unsigned char* base = msm + wid * kMWarpSmem;
  uint64_t* bar = reinterpret_cast<uint64_t*>(base);
  unsigned char* stage0 = base + 64;
  const int rowb = int(rp) * 4;  // 16 .. 512 bytes, a multiple of 16
  const int R = min(kMVBytes / rowb, kMXBytes / kMRowBytes);  // 0 only for rows above 4096 bytes
  const int nrows = it.j1 - it.j0;
  const int nst = (nrows + R - 1) / R;
  const float* V = static_cast<const float*>(Z.V) + int64_t(it.j0) * rp;
  const float* xr = inc + (Z.x_off + it.j0) * kMR;
  const int npass = (it.nk + kMCols - 1) / kMCols;
  float acc[kMCols];
  if (R == 0) {
    // rows wider than a stage (rank above 1024): direct loads
    for (int pass = 0; pass < npass; pass++) {
      const int c0 = it.k0 + pass * kMCols, ncol = min(kMCols, it.k0 + it.nk - c0);
#pragma unroll
      for (int c = 0; c < kMCols; c++) acc[c] = 0.f;
      for (int j = 0; j < nrows; j++) {
        const float x = xr[int64_t(j) * kMR + lane];
        const float* vj = V + int64_t(j) * rp + c0;
#pragma unroll
        for (int c = 0; c < kMCols; c++)
          if (c < ncol) acc[c] = __fmaf_rn(__ldg(vj + c), x, acc[c]);
      }
#pragma unroll
      for (int c = 0; c < kMCols; c++)
        if (c < ncol) {
          const int col = c0 + c;
          if (it.part < 0) {
            if (col < Z.r) inc[(Z.z_off + col) * kMR + lane] = acc[c];
          } else {
            zp[(int64_t(it.part) + col - it.k0) * kMR + lane] = acc[c];
          }
        }
    }
    return;
  }
  const int total = nst * npass;  // stages over all passes
  if (lane == 0) {
#pragma unroll
    for (int s = 0; s < kMStages; s++) mbar_init(bar + s, 1);
    fence_mbar_init();
  }
  __syncwarp();
  // stage q: pass q / nst, rows (q % nst) * R ..
#define HODLR_MR_ISSUE(q_)                                                                     \
  do {                                                                                         \
    const int s_ = (q_) % kMStages;                                                            \
    const int r0_ = ((q_) % nst) * R, nr_ = min(R, nrows - r0_);                               \
    unsigned char* st_ = stage0 + s_ * (kMVBytes + kMXBytes);                                  \
    fence_proxy_async();                                                                       \
    mbar_expect_tx(bar + s_, uint32_t(nr_) * uint32_t(rowb + kMRowBytes));                     \
    bulk_g2s(st_, V + int64_t(r0_) * rp, uint32_t(nr_ * rowb), bar + s_);                      \
    bulk_g2s(st_ + kMVBytes, xr + int64_t(r0_) * kMR, uint32_t(nr_ * kMRowBytes), bar + s_);    \
  } while (0)
  if (lane == 0)
    for (int q = 0; q < min(kMStages, total); q++) HODLR_MR_ISSUE(q);
  for (int q = 0; q < total; q++) {
    const int pass = q / nst, c0 = it.k0 + pass * kMCols;
    const int ncol4 = min(kMCols, it.k0 + it.nk - c0) / 4;
    if (q % nst == 0) {
#pragma unroll
      for (int c = 0; c < kMCols; c++) acc[c] = 0.f;
    }
    const int s = q % kMStages;
    const bool ok = __all_sync(0xffffffffu, mbar_wait(bar + s, uint32_t(q / kMStages) & 1u));
    if (!ok) {
      if (lane == 0) atomicAdd(&g_stream_timeouts, 1u);
      for (int t = q; t < min(q + kMStages, total); t++) mbar_wait(bar + t % kMStages, uint32_t(t / kMStages) & 1u);
      return;
    }
    const int nr = min(R, nrows - (q % nst) * R);
    const unsigned char* vs = stage0 + s * (kMVBytes + kMXBytes) + c0 * 4;
    const float* xs = reinterpret_cast<const float*>(stage0 + s * (kMVBytes + kMXBytes) + kMVBytes);
    switch (ncol4) {  // column count known at compile time: no per-row guards
#define HODLR_MR_CASE(k_) \
  case k_:                \
    mr_rows<k_>(vs, rowb, xs, nr, lane, acc); \
    break;
      HODLR_MR_CASE(1) HODLR_MR_CASE(2) HODLR_MR_CASE(3) HODLR_MR_CASE(4) HODLR_MR_CASE(5) HODLR_MR_CASE(6)
      HODLR_MR_CASE(7) HODLR_MR_CASE(8) HODLR_MR_CASE(9) HODLR_MR_CASE(10) HODLR_MR_CASE(11) HODLR_MR_CASE(12)
      HODLR_MR_CASE(13) HODLR_MR_CASE(14) HODLR_MR_CASE(15) HODLR_MR_CASE(16)
#undef HODLR_MR_CASE
      default:
        break;
    }
    __syncwarp();
    if (lane == 0 && q + kMStages < total) HODLR_MR_ISSUE(q + kMStages);
    if (q % nst == nst - 1) {  // end of a pass: columns c0 .. c0 + 4 ncol4
#pragma unroll
      for (int c = 0; c < kMCols; c++)
        if (c < 4 * ncol4) {
          const int col = c0 + c;
          if (it.part < 0) {
            if (col < Z.r) inc[(Z.z_off + col) * kMR + lane] = acc[c];
          } else {
            zp[(int64_t(it.part) + col - it.k0) * kMR + lane] = acc[c];
          }
        }
    }
  }
#undef HODLR_MR_ISSUE
}

// z row zpos (all kMR values) = sum of the item partials, in order.
__global__ void __launch_bounds__(256) zfix_mr_kernel(const ZFix* __restrict__ fix, int nfix,
                                                     const float* __restrict__ zpart, int64_t zpart_ld,
                                                     float* __restrict__ in, int64_t ld_in) {
  const int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  const int f = int(t / kMR), c = int(t % kMR);
  if (f >= nfix) return;
  const ZFix F = fix[f];
  const float* zp = zpart + int64_t(blockIdx.y) * zpart_ld * kMR;
  float acc = 0.f;
  for (int q = 0; q < F.count; q++) acc += zp[(int64_t(F.part) + int64_t(q) * kZPart) * kMR + c];
  in[int64_t(blockIdx.y) * ld_in * kMR + F.zpos * kMR + c] = acc;
}

// Leaf panels (m <= 32): one warp per item; lane c keeps m sums.  The item's
// segments are cut into pieces that are packed, in order, into stages of at
// most kMSUBytes of factor bytes (each piece 16-byte aligned, a multiple of 4
// columns unless it ends its segment) and kMSRows input rows; one lane issues
// the bulk copies of a stage, every lane replays the same packing to find the
// pieces.
constexpr int kMSUBytes = 4096;
constexpr int kMSRows = 32;
constexpr int kMSXBytes = kMSRows * kMRowBytes;
constexpr int kMSWarpSmem = 64 + kMStages * (kMSUBytes + kMSXBytes);
static_assert(kMSWarpSmem % 16 == 0, "bulk copy destinations must stay 16-byte aligned");

// acc[i] += U[i][j] x[j] over a piece's columns, rows 0 .. MP-1
template <int MP>
__device__ __forceinline__ void mr_cols(const float* ua, int m, const float* xr, int nc, float (&acc)[32]) {
  for (int j = 0; j < nc; j++) {
    const float x = xr[j * kMR];
#pragma unroll
    for (int i = 0; i < MP; i++) acc[i] = __fmaf_rn(ua[j * m + i], x, acc[i]);
  }
}

struct MrCursor {
  int64_t s;  // segment
  int c;      // first column of the next piece
};

// Next piece of a stage holding `used` factor bytes and `rows` input rows;
// false when the stage is full or the segments are done.
__device__ __forceinline__ bool mr_next_piece(const Seg* segs, int64_t seg_e, int m, MrCursor& cur, int used, int rows,
                                              int64_t& s, int& c0, int& nc, int& bytes) {
  if (cur.s >= seg_e) return false;
  const int K = segs[cur.s].K;
  int room_c = min((kMSUBytes - used) / (m * 4), kMSRows - rows);
  int c = min(K - cur.c, room_c);
  if (c < K - cur.c) c = c / 4 * 4;  // a piece that does not end its segment keeps 16-byte alignment
  if (c <= 0) return false;
  nc = c;
  bytes = (c * m * 4 + 15) & ~15;
  if (used + bytes > kMSUBytes) return false;
  s = cur.s;
  c0 = cur.c;
  cur.c += c;
  if (cur.c >= K) {
    cur.s++;
    cur.c = 0;
  }
  return true;
}

__global__ void __launch_bounds__(kMWarps * 32, 3)
    panel_small_mr_kernel(const Panel* __restrict__ panels, const Seg* __restrict__ segs,
                          const Item* __restrict__ items, int nitems, const float* __restrict__ in, int64_t ld_in,
                          float* __restrict__ y, int64_t ld_y, float* __restrict__ ypart, int64_t ypart_ld) {
  extern __shared__ __align__(16) unsigned char msm[];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int w = blockIdx.x * kMWarps + wid;
  if (w >= nitems) return;
  const Item it = items[w];
  const Panel P = panels[it.panel];
  const int m = P.m;
  int mp = 4;
  while (mp < m) mp <<= 1;
  const float* inc = in + int64_t(blockIdx.y) * ld_in * kMR;
  unsigned char* base = msm + wid * kMSWarpSmem;
  uint64_t* bar = reinterpret_cast<uint64_t*>(base);
  unsigned char* stage0 = base + 64;
  if (lane == 0) {
#pragma unroll
    for (int s = 0; s < kMStages; s++) mbar_init(bar + s, 1);
    fence_mbar_init();
  }
  __syncwarp();
  MrCursor pc{it.seg_b, 0}, cc{it.seg_b, 0};
  int issued = 0;
  // packs and issues the next stage; false when nothing is left
  // Packs and issues the next stage: per piece, lane 0 raises the stage's
  // transaction count (no arrival) and starts its two copies; the stage's one
  // arrival comes after the last piece, so the phase cannot complete before
  // every copy is accounted for.  ok_ is false when nothing is left.
#define HODLR_MRS_ISSUE(ok_)                                                                      \
  do {                                                                                            \
    const int st_ = issued % kMStages;                                                            \
    unsigned char* su_ = stage0 + st_ * (kMSUBytes + kMSXBytes);                                  \
    int used_ = 0, rows_ = 0, nc_, by_, c0_;                                                      \
    int64_t s_;                                                                                   \
    if (lane == 0) fence_proxy_async();                                                           \
    while (mr_next_piece(segs, it.seg_e, m, pc, used_, rows_, s_, c0_, nc_, by_)) {               \
      if (lane == 0) {                                                                            \
        const Seg S_ = segs[s_];                                                                  \
        mbar_expect_tx_only(bar + st_, uint32_t(by_ + nc_ * kMRowBytes));                         \
        bulk_g2s(su_ + used_, static_cast<const float*>(S_.A) + int64_t(c0_) * m, uint32_t(by_), bar + st_); \
        bulk_g2s(su_ + kMSUBytes + rows_ * kMRowBytes, inc + (S_.in_off + c0_) * kMR,            \
                 uint32_t(nc_ * kMRowBytes), bar + st_);                                          \
      }                                                                                           \
      used_ += by_;                                                                               \
      rows_ += nc_;                                                                               \
    }                                                                                             \
    ok_ = rows_ > 0;                                                                              \
    if (ok_) {                                                                                    \
      if (lane == 0) mbar_arrive(bar + st_);                                                      \
      issued++;                                                                                   \
    }                                                                                             \
  } while (0)
  bool more = true;
  for (int q = 0; q < kMStages && more; q++) HODLR_MRS_ISSUE(more);
  float acc[32];
#pragma unroll
  for (int i = 0; i < 32; i++) acc[i] = 0.f;
  for (int q = 0; q < issued; q++) {
    const int st = q % kMStages;
    const bool ok = __all_sync(0xffffffffu, mbar_wait(bar + st, uint32_t(q / kMStages) & 1u));
    if (!ok) {
      if (lane == 0) atomicAdd(&g_stream_timeouts, 1u);
      for (int t = q; t < issued; t++) mbar_wait(bar + t % kMStages, uint32_t(t / kMStages) & 1u);
      return;
    }
    const unsigned char* su = stage0 + st * (kMSUBytes + kMSXBytes);
    const float* xs = reinterpret_cast<const float*>(su + kMSUBytes);
    int used = 0, rows = 0, nc, by, c0;
    int64_t sg;
    while (mr_next_piece(segs, it.seg_e, m, cc, used, rows, sg, c0, nc, by)) {
      const float* ua = reinterpret_cast<const float*>(su + used);
      const float* xr = xs + rows * kMR + lane;
      // rows 0 .. mp-1 (mp = next power of two >= m, at least 4): sums of rows
      // m .. mp-1 read neighbouring bytes of the warp's stage and are never stored
      if (mp <= 4)
        mr_cols<4>(ua, m, xr, nc, acc);
      else if (mp <= 8)
        mr_cols<8>(ua, m, xr, nc, acc);
      else if (mp <= 16)
        mr_cols<16>(ua, m, xr, nc, acc);
      else
        mr_cols<32>(ua, m, xr, nc, acc);
      used += by;
      rows += nc;
    }
    __syncwarp();
    if (more) HODLR_MRS_ISSUE(more);  // into the stage just consumed (the ring is full while more)
  }
#undef HODLR_MRS_ISSUE
  // split panels: partial rows at the part's 128-row block of ypart (panel_fix_mr_kernel)
  float* yo = it.part < 0 ? y + int64_t(blockIdx.y) * ld_y * kMR + P.yoff * kMR
                          : ypart + int64_t(blockIdx.y) * ypart_ld * kMR + int64_t(it.part) * 128 * kMR;
#pragma unroll
  for (int i = 0; i < 32; i++)
    if (i < m) yo[int64_t(i) * kMR + lane] = acc[i];
}

// acc[i] += U[i][j] x[j] over a stage's columns: H4 groups of 4 rows (a full
// tile), or h4 of them checked per group (H4 == 0, the last tile)
template <int H4>
__device__ __forceinline__ void mr_tile(const unsigned char* us, int colb, const float* xs, int nc, int lane, int h4,
                                        float (&acc)[128]) {
  for (int j = 0; j < nc; j++) {
    const float x = xs[j * kMR + lane];
    const float4* u4 = reinterpret_cast<const float4*>(us + j * colb);
#pragma unroll
    for (int r = 0; r < 32; r++)
      if (H4 ? r < H4 : r < h4) {
        const float4 u = u4[r];
        acc[4 * r] = __fmaf_rn(u.x, x, acc[4 * r]);
        acc[4 * r + 1] = __fmaf_rn(u.y, x, acc[4 * r + 1]);
        acc[4 * r + 2] = __fmaf_rn(u.z, x, acc[4 * r + 2]);
        acc[4 * r + 3] = __fmaf_rn(u.w, x, acc[4 * r + 3]);
      }
  }
}

// Panels of more than 32 rows: item = row tile t (up to 128 rows) times a
// run of segments; lane c keeps the tile's row sums; runs of tile columns and
// their input rows are staged.
constexpr int kMTUBytes = 4096;
constexpr int kMTXBytes = 4096;  // 32 input rows
constexpr int kMTWarpSmem = 64 + kMStages * (kMTUBytes + kMTXBytes);
static_assert(kMTWarpSmem % 16 == 0, "bulk copy destinations must stay 16-byte aligned");

__global__ void __launch_bounds__(kMWarps * 32, 2)
    panel_tile_mr_kernel(const Panel* __restrict__ panels, const Seg* __restrict__ segs,
                         const Item* __restrict__ items, int nitems, float* __restrict__ ypart, int64_t ypart_ld,
                         const float* __restrict__ in, int64_t ld_in, float* __restrict__ y, int64_t ld_y) {
  constexpr int T = 128;
  extern __shared__ __align__(16) unsigned char msm[];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int w = blockIdx.x * kMWarps + wid;
  if (w >= nitems) return;
  const Item it = items[w];
  const Panel P = panels[it.panel];
  const int m = P.m;
  const float* inc = in + int64_t(blockIdx.y) * ld_in * kMR;
  const int t = it.chunk;
  const int rows = min(T, m - t * T);
  const int64_t h = tile_height(m, t, 4);
  const int colb = int(h) * 4;
  const int h4 = int(h) / 4;
  const int cps = min(kMTUBytes / colb, kMTXBytes / kMRowBytes);
  float acc[T];
#pragma unroll
  for (int i = 0; i < T; i++) acc[i] = 0.f;
  unsigned char* base = msm + wid * kMTWarpSmem;
  uint64_t* bar = reinterpret_cast<uint64_t*>(base);
  unsigned char* stage0 = base + 64;
  if (lane == 0) {
#pragma unroll
    for (int s = 0; s < kMStages; s++) mbar_init(bar + s, 1);
    fence_mbar_init();
  }
  __syncwarp();
  int64_t ps = it.seg_b;
  int pc = 0, issued = 0;
#define HODLR_MRT_ISSUE()                                                                          \
  do {                                                                                             \
    while (ps < it.seg_e && pc >= segs[ps].K) {                                                    \
      ps++;                                                                                        \
      pc = 0;                                                                                      \
    }                                                                                              \
    if (ps >= it.seg_e) break;                                                                     \
    const Seg S_ = segs[ps];                                                                       \
    const int nc_ = min(cps, S_.K - pc);                                                           \
    if (lane == 0) {                                                                               \
      const int st_ = issued % kMStages;                                                           \
      unsigned char* dst_ = stage0 + st_ * (kMTUBytes + kMTXBytes);                                \
      const float* src_ = static_cast<const float*>(S_.A) + int64_t(t) * T * S_.K + int64_t(pc) * h; \
      fence_proxy_async();                                                                         \
      mbar_expect_tx(bar + st_, uint32_t(nc_) * uint32_t(colb + kMRowBytes));                      \
      bulk_g2s(dst_, src_, uint32_t(nc_ * colb), bar + st_);                                       \
      bulk_g2s(dst_ + kMTUBytes, inc + (S_.in_off + pc) * kMR, uint32_t(nc_ * kMRowBytes), bar + st_); \
    }                                                                                              \
    pc += nc_;                                                                                     \
    issued++;                                                                                      \
  } while (0)
  for (int q = 0; q < kMStages; q++) HODLR_MRT_ISSUE();
  int64_t cs = it.seg_b;
  int cc = 0;
  for (int q = 0; q < issued; q++) {
    while (cc >= segs[cs].K) {
      cs++;
      cc = 0;
    }
    const int nc = min(cps, segs[cs].K - cc);
    const int st = q % kMStages;
    const bool ok = __all_sync(0xffffffffu, mbar_wait(bar + st, uint32_t(q / kMStages) & 1u));
    if (!ok) {
      if (lane == 0) atomicAdd(&g_stream_timeouts, 1u);
      for (int u = q; u < issued; u++) mbar_wait(bar + u % kMStages, uint32_t(u / kMStages) & 1u);
      return;
    }
    const unsigned char* us = stage0 + st * (kMTUBytes + kMTXBytes);
    const float* xs = reinterpret_cast<const float*>(us + kMTUBytes);
    if (h4 == T / 4)
      mr_tile<T / 4>(us, colb, xs, nc, lane, h4, acc);
    else
      mr_tile<0>(us, colb, xs, nc, lane, h4, acc);
    cc += nc;
    __syncwarp();
    HODLR_MRT_ISSUE();
  }
#undef HODLR_MRT_ISSUE
  float* dst = it.part < 0 ? y + int64_t(blockIdx.y) * ld_y * kMR + (P.yoff + int64_t(t) * T) * kMR
                           : ypart + int64_t(blockIdx.y) * ypart_ld * kMR + int64_t(it.part) * T * kMR;
#pragma unroll
  for (int i = 0; i < T; i++)
    if (i < rows) dst[int64_t(i) * kMR + lane] = acc[i];
}

__global__ void __launch_bounds__(256) panel_fix_mr_kernel(const Panel* __restrict__ panels,
                                                           const PanelFix* __restrict__ fix, int nfix,
                                                           const float* __restrict__ ypart, int64_t ypart_ld,
                                                           float* __restrict__ y, int64_t ld_y) {
  constexpr int rows = 128;
  const int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  const int64_t fq = t / kMR;
  const int c = int(t % kMR);
  const int f = int(fq / rows), q = int(fq % rows);
  if (f >= nfix) return;
  const PanelFix F = fix[f];
  const Panel P = panels[F.panel];
  const int i = F.chunk * rows + q;
  if (i >= P.m) return;
  const float* yp = ypart + int64_t(blockIdx.y) * ypart_ld * kMR;
  float acc = 0.f;
  for (int g = 0; g < F.count; g++) acc += yp[((int64_t(F.part) + g) * rows + q) * kMR + c];
  y[int64_t(blockIdx.y) * ld_y * kMR + (P.yoff + i) * kMR + c] = acc;
}

// in (chunk ch, interleaved) <- x (caller order, column major total_n x k)
__global__ void __launch_bounds__(256) batch_gather_mr_kernel(const BatchInst* __restrict__ inst,
                                                              const float* __restrict__ x, int64_t total_n, int k,
                                                              float* __restrict__ in, int64_t ld_in, int ch) {
  const BatchInst I = inst[blockIdx.y];
  float* inc = in + int64_t(ch) * ld_in * kMR;
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < I.n * kMR;
       e += int64_t(gridDim.x) * blockDim.x) {
    const int64_t r = e / kMR;
    const int c = int(e % kMR), col = ch * kMR + c;
    inc[(I.in_base + r) * kMR + c] = col < k ? x[int64_t(col) * total_n + I.x_base + I.perm[r]] : 0.f;
  }
}

__global__ void __launch_bounds__(256) batch_combine_mr_kernel(const BatchInst* __restrict__ inst,
                                                               const float* __restrict__ y, int64_t ld_y,
                                                               float* __restrict__ out, int64_t total_n, int k, int ch) {
  const BatchInst I = inst[blockIdx.y];
  const float* yc = y + int64_t(ch) * ld_y * kMR;
  for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < I.n * kMR;
       e += int64_t(gridDim.x) * blockDim.x) {
    const int64_t r = e / kMR;
    const int c = int(e % kMR), col = ch * kMR + c;
    if (col >= k) continue;
    double acc = double(yc[(I.y_base + r) * kMR + c]);
    for (int s = 1; s < I.nslots; s++) acc += double(yc[(I.y_base + int64_t(s) * I.n + r) * kMR + c]);
    out[int64_t(col) * total_n + I.x_base + I.perm[r]] = float(acc);
  }
}

}  // namespace

cudaError_t launch_zgemv_mr(const ZBlock* zb, const ZItem* items, int nitems, const ZFix* fix, int nfix, float* zpart,
                            int64_t zpart_ld, float* in, int64_t ld_in, int nchunks, cudaStream_t st) {
  if (nitems <= 0) return cudaSuccess;
  count_launches(nfix > 0 ? 2 : 1);
  cudaFuncSetAttribute(zgemv_mr_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kMWarps * kMWarpSmem);
  dim3 g(unsigned((nitems + kMWarps - 1) / kMWarps), unsigned(nchunks));
  zgemv_mr_kernel<<<g, kMWarps * 32, kMWarps * kMWarpSmem, st>>>(zb, items, nitems, zpart, zpart_ld, in, ld_in);
  if (nfix > 0) {
    dim3 gf(unsigned((int64_t(nfix) * kMR + 255) / 256), unsigned(nchunks));
    zfix_mr_kernel<<<gf, 256, 0, st>>>(fix, nfix, zpart, zpart_ld, in, ld_in);
  }
  return cudaGetLastError();
}

cudaError_t launch_panels_mr(const Panel* panels, const Seg* segs, const Item* small, int nsmall, const Item* big,
                             int nbig, const PanelFix* fix, int nfix, float* ypart, int64_t ypart_ld, const float* in,
                             int64_t ld_in, float* y, int64_t ld_y, int nchunks, cudaStream_t st) {
  if (nsmall + nbig <= 0) return cudaSuccess;
  count_launches(uint64_t(nbig > 0) + uint64_t(nsmall > 0) + uint64_t(nfix > 0));
  if (nbig > 0) {
    cudaFuncSetAttribute(panel_tile_mr_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kMWarps * kMTWarpSmem);
    dim3 g(unsigned((nbig + kMWarps - 1) / kMWarps), unsigned(nchunks));
    panel_tile_mr_kernel<<<g, kMWarps * 32, kMWarps * kMTWarpSmem, st>>>(panels, segs, big, nbig, ypart, ypart_ld, in,
                                                                          ld_in, y, ld_y);
  }
  if (nsmall > 0) {
    cudaFuncSetAttribute(panel_small_mr_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kMWarps * kMSWarpSmem);
    dim3 g(unsigned((nsmall + kMWarps - 1) / kMWarps), unsigned(nchunks));
    panel_small_mr_kernel<<<g, kMWarps * 32, kMWarps * kMSWarpSmem, st>>>(panels, segs, small, nsmall, in, ld_in, y,
                                                                           ld_y, ypart, ypart_ld);
  }
  if (nfix > 0) {
    dim3 gf(unsigned((int64_t(nfix) * 128 * kMR + 255) / 256), unsigned(nchunks));
    panel_fix_mr_kernel<<<gf, 256, 0, st>>>(panels, fix, nfix, ypart, ypart_ld, y, ld_y);
  }
  return cudaGetLastError();
}

cudaError_t launch_batch_gather_mr(const BatchInst* inst, int count, int64_t max_n, const float* x, int64_t total_n,
                                   int k, float* in, int64_t ld_in, int nchunks, cudaStream_t st) {
  if (count <= 0) return cudaSuccess;
  for (int ch = 0; ch < nchunks; ch++) {
    count_launches(1);
    batch_gather_mr_kernel<<<batch_grid(count, max_n * kMR), 256, 0, st>>>(inst, x, total_n, k, in, ld_in, ch);
  }
  return cudaGetLastError();
}

cudaError_t launch_batch_combine_mr(const BatchInst* inst, int count, int64_t max_n, const float* y, int64_t ld_y,
                                    float* out, int64_t total_n, int k, int nchunks, cudaStream_t st) {
  if (count <= 0) return cudaSuccess;
  for (int ch = 0; ch < nchunks; ch++) {
    count_launches(1);
    batch_combine_mr_kernel<<<batch_grid(count, max_n * kMR), 256, 0, st>>>(inst, y, ld_y, out, total_n, k, ch);
  }
  return cudaGetLastError();
}

}  // namespace hodlr
