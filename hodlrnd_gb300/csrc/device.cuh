// Device-side helpers shared by the HODLRnD GB300 kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

namespace hodlr {

// Process-wide count of this engine's kernel launches (hodlr_kernel_launches).
inline std::atomic<uint64_t> g_kernel_launches{0};
inline void count_launches(uint64_t k) { g_kernel_launches.fetch_add(k, std::memory_order_relaxed); }

// Kernel kinds (include/hodlrnd.h).
enum : int { kInvR = 1, kInvR2 = 2, kLogR = 3, kExpNegR = 4 };

struct KernelDev {
  int kind;
  double scale, diag;
};

// Points in tree order, structure of arrays: coordinate k of point i is
// x[k * ld + i].
struct PointsDev {
  const double* x;
  int64_t ld;
};

// One matrix entry A(i, j) for tree positions i, j (kernel_function::getRow /
// getCol / getMatrix + the user getMatrixEntry, include/kernel_function.hpp:20-53).
// d2 is accumulated in dimension order with one rounding per operation (the
// explicit _rn intrinsics keep the compiler from contracting into FMAs); sqrt
// and division are IEEE round-to-nearest on both sides, so the 1/r and 1/r^2
// entries are bit-identical to the scalar host code.  The log r and e^-r
// kinds call CUDA's log and exp, which need not round as the host's libm
// does: those entries agree to a few units in the last place.
template <int D>
__device__ __forceinline__ double kernel_entry(const PointsDev& P, const KernelDev& K, int64_t i, int64_t j,
                                               const double* xi) {
  if (i == j) return K.diag;
  double d2 = 0.0;
#pragma unroll
  for (int k = 0; k < D; k++) {
    const double t = __dsub_rn(xi[k], P.x[k * P.ld + j]);
    d2 = __dadd_rn(d2, __dmul_rn(t, t));
  }
  switch (K.kind) {
    case kInvR: return __ddiv_rn(K.scale, __dsqrt_rn(d2));
    case kInvR2: return __ddiv_rn(K.scale, d2);
    case kLogR: return __dmul_rn(K.scale, log(__dsqrt_rn(d2)));
    default: return __dmul_rn(K.scale, exp(-__dsqrt_rn(d2)));
  }
}

// The same entry from two staged coordinate vectors (stride ld between
// coordinates); same_point: the tree positions are equal (the diagonal).
template <int D>
__device__ __forceinline__ double kernel_entry_xy(const KernelDev& K, bool same_point, const double* xi,
                                                  const double* xj, int ld) {
  if (same_point) return K.diag;
  double d2 = 0.0;
#pragma unroll
  for (int k = 0; k < D; k++) {
    const double t = __dsub_rn(xi[k], xj[k * ld]);
    d2 = __dadd_rn(d2, __dmul_rn(t, t));
  }
  switch (K.kind) {
    case kInvR: return __ddiv_rn(K.scale, __dsqrt_rn(d2));
    case kInvR2: return __ddiv_rn(K.scale, d2);
    case kLogR: return __dmul_rn(K.scale, log(__dsqrt_rn(d2)));
    default: return __dmul_rn(K.scale, exp(-__dsqrt_rn(d2)));
  }
}

template <int D>
__device__ __forceinline__ void load_point(const PointsDev& P, int64_t i, double* xi) {
#pragma unroll
  for (int k = 0; k < D; k++) xi[k] = P.x[k * P.ld + i];
}

// a = hi + lo + e, |e| <= 2^-46 |a|: hi is a's sign, exponent and leading 24
// significand bits, lo the next 23 bits (truncated), both exact floats, built
// with integer operations only (GB300's FP64 pipe is far slower than its
// FP32 and integer pipes).  |a| < 2^-70 gives (0, 0), an absolute error below
// 8.5e-22; |a| >= 2^127 falls back to a rounding conversion.
__device__ __forceinline__ float2 split_d(double a) {
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(a));
  const unsigned hi32 = unsigned(b >> 32), lo32 = unsigned(b);
  const int e = int((hi32 >> 20) & 0x7ffu);
  if (e < 1023 - 70) return make_float2(0.f, 0.f);
  if (e > 1023 + 126) return make_float2(__double2float_rn(a), 0.f);
  const unsigned sign = hi32 & 0x80000000u;
  const unsigned m23 = ((hi32 & 0xfffffu) << 3) | (lo32 >> 29);
  const float hi = __uint_as_float(sign | (unsigned(e - 1023 + 127) << 23) | m23);
  // the next 23 bits r as a float (2^23 + r - 2^23, exact), times 2^(e - 1069)
  const float r = __fsub_rn(__uint_as_float(0x4B000000u | ((lo32 & 0x1fffffffu) >> 6)), 8388608.f);
  const float lo = __fmul_rn(r, __uint_as_float(unsigned(e - 1069 + 127) << 23));
  return make_float2(hi, __uint_as_float(__float_as_uint(lo) | sign));
}

// s + c += (a.x + a.y)(b.x + b.y)
__device__ __forceinline__ void dot2_add(float& s, float& c, float2 a, float2 b) {
  const float p = __fmul_rn(a.x, b.x);
  const float pe = __fmaf_rn(a.x, b.x, -p);
  const float t = __fmaf_rn(a.x, b.y, __fmaf_rn(a.y, b.x, pe));
  const float s2 = __fadd_rn(s, p);
  const float bb = __fsub_rn(s2, s);
  const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(s2, bb)), __fsub_rn(p, bb));
  s = s2;
  c = __fadd_rn(c, __fadd_rn(err, t));
}

// (s, c) + (s2, c2) as an unevaluated FP32 pair (TwoSum on the high parts).
__device__ __forceinline__ void pair_add(float& s, float& c, float s2, float c2) {
  const float t = __fadd_rn(s, s2);
  const float bb = __fsub_rn(t, s);
  const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bb)), __fsub_rn(s2, bb));
  s = t;
  c = __fadd_rn(__fadd_rn(c, c2), err);
}

// ---------------------------------------------------------------- teams
// A "team" is the group of threads that compresses one block: a warp, or a
// whole CTA.  All members call every team function (uniform control flow).

struct WarpTeam {
  static constexpr int kSize = 32;
  __device__ __forceinline__ int tid() const { return threadIdx.x & 31; }
  __device__ __forceinline__ void sync() const { __syncwarp(); }
  __device__ __forceinline__ double sum(double v) const {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
  }
  // Largest |v|, lowest index on ties (kernel_function::maxAbsVector keeps the
  // first maximum, include/kernel_function.hpp:55-68).
  __device__ __forceinline__ void argmax(double& a, int& i, double& v) const {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double a2 = __shfl_xor_sync(0xffffffffu, a, o);
      const int i2 = __shfl_xor_sync(0xffffffffu, i, o);
      const double v2 = __shfl_xor_sync(0xffffffffu, v, o);
      if (a2 > a || (a2 == a && i2 < i)) {
        a = a2;
        i = i2;
        v = v2;
      }
    }
  }
  __device__ __forceinline__ int bcast(int v) const { return __shfl_sync(0xffffffffu, v, 0); }
  __device__ __forceinline__ double bcast(double v) const { return __shfl_sync(0xffffffffu, v, 0); }
};

// T lanes of one warp (T = 8 or 16): lanes 0..T-1, T..2T-1, ... each form a
// team of their own.  Teams of one warp may follow different control flow
// (their blocks differ); every shuffle names only the team's lanes.
template <int T>
struct SubTeam {
  static constexpr int kSize = T;
  unsigned mask;
  __device__ __forceinline__ SubTeam() : mask(((1u << T) - 1u) << ((threadIdx.x & 31) & ~(T - 1))) {}
  __device__ __forceinline__ int tid() const { return threadIdx.x & (T - 1); }
  __device__ __forceinline__ void sync() const { __syncwarp(mask); }
  __device__ __forceinline__ double sum(double v) const {
#pragma unroll
    for (int o = T / 2; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o, T);
    return v;
  }
  __device__ __forceinline__ void argmax(double& a, int& i, double& v) const {
#pragma unroll
    for (int o = T / 2; o > 0; o >>= 1) {
      const double a2 = __shfl_xor_sync(mask, a, o, T);
      const int i2 = __shfl_xor_sync(mask, i, o, T);
      const double v2 = __shfl_xor_sync(mask, v, o, T);
      if (a2 > a || (a2 == a && i2 < i)) {
        a = a2;
        i = i2;
        v = v2;
      }
    }
  }
  __device__ __forceinline__ int bcast(int v) const { return __shfl_sync(mask, v, 0, T); }
  __device__ __forceinline__ double bcast(double v) const { return __shfl_sync(mask, v, 0, T); }
};

template <int NT>
struct CtaTeam {
  static constexpr int kSize = NT;
  static constexpr int kWarps = NT / 32;
  double* red;    // shared, kWarps + 1
  int* redi;      // shared, kWarps + 1
  double* terms;  // shared, kNormChunk: the norm estimate's terms of one pass (ACA)
  __device__ __forceinline__ int tid() const { return threadIdx.x; }
  __device__ __forceinline__ void sync() const { __syncthreads(); }
  __device__ __forceinline__ double sum(double v) const {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[w] = v;
    __syncthreads();
    if (w == 0) {
      v = lane < kWarps ? red[lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) red[kWarps] = v;
    }
    __syncthreads();
    v = red[kWarps];
    __syncthreads();
    return v;
  }
  __device__ __forceinline__ void argmax(double& a, int& i, double& v) const {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    WarpTeam().argmax(a, i, v);
    __shared__ double sa[kWarps + 1], sv[kWarps + 1];
    if (lane == 0) {
      sa[w] = a;
      sv[w] = v;
      redi[w] = i;
    }
    __syncthreads();
    if (w == 0) {
      a = lane < kWarps ? sa[lane] : -1.0;
      i = lane < kWarps ? redi[lane] : 0x7fffffff;
      v = lane < kWarps ? sv[lane] : 0.0;
      WarpTeam().argmax(a, i, v);
      if (lane == 0) {
        sa[kWarps] = a;
        sv[kWarps] = v;
        redi[kWarps] = i;
      }
    }
    __syncthreads();
    a = sa[kWarps];
    v = sv[kWarps];
    i = redi[kWarps];
    __syncthreads();
  }
  __device__ __forceinline__ int bcast(int v) const {
    if (threadIdx.x == 0) redi[kWarps] = v;
    __syncthreads();
    v = redi[kWarps];
    __syncthreads();
    return v;
  }
  __device__ __forceinline__ double bcast(double v) const {
    if (threadIdx.x == 0) red[kWarps] = v;
    __syncthreads();
    v = red[kWarps];
    __syncthreads();
    return v;
  }
};

__host__ __device__ inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

}  // namespace hodlr
