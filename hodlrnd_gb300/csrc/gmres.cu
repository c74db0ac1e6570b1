// Restarted GMRES on the device (see gmres.h).
#include "device.cuh"
#include "gmres.h"

#include <cmath>

namespace hodlr {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ double to_d(double v) { return v; }
__device__ __forceinline__ double to_d(float v) { return double(v); }

// a - h * b with one rounding per operation in FP64, rounded to T.
__device__ __forceinline__ double axmy(double a, double h, double b) { return __dsub_rn(a, __dmul_rn(h, b)); }

// Block-wide sum; every thread gets the result.
__device__ double block_sum(double v) {
  __shared__ double sh[kThreads / 32 + 1];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  if (wid == 0) {
    v = lane < kThreads / 32 ? sh[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) sh[kThreads / 32] = v;
  }
  __syncthreads();
  v = sh[kThreads / 32];
  __syncthreads();
  return v;
}

// Sum of the kVecCtas partials in a fixed order (each CTA gets the same value).
__device__ double reduce_parts(const double* part) {
  double v = 0.0;
  for (int i = threadIdx.x; i < kVecCtas; i += kThreads) v += part[i];
  return block_sum(v);
}

template <typename T>
__global__ void __launch_bounds__(kThreads) dot_partial_kernel(const T* a, const T* b, int64_t n, double* part) {
  double acc = 0.0;
  for (int64_t i = blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n; i += int64_t(kVecCtas) * kThreads)
    acc += to_d(a[i]) * to_d(b[i]);
  acc = block_sum(acc);
  if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

// partials of |sum_{s = s0}^{s1 - 1} y[s * n + i]|^2 over i
template <typename T>
__global__ void __launch_bounds__(kThreads) slots_partial_kernel(const T* y, int64_t n, int s0, int s1, double* part) {
  double acc = 0.0;
  for (int64_t i = blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n; i += int64_t(kVecCtas) * kThreads) {
    double v = 0.0;
    for (int s = s0; s < s1; s++) v += to_d(y[int64_t(s) * n + i]);
    acc += v * v;
  }
  acc = block_sum(acc);
  if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

// h = <w, v_k> from part_in; w -= h v_k; part_out = partials of <w, next>.
template <typename T>
__global__ void __launch_bounds__(kThreads)
    mgs_step_kernel(T* w, const T* vk, const T* next, int64_t n, const double* part_in, double* part_out, double* hout) {
  const double h = reduce_parts(part_in);
  if (blockIdx.x == 0 && threadIdx.x == 0) *hout = h;
  double acc = 0.0;
  for (int64_t i = blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n; i += int64_t(kVecCtas) * kThreads) {
    const T wi = T(axmy(to_d(w[i]), h, to_d(vk[i])));
    w[i] = wi;
    acc += to_d(wi) * to_d(next ? next[i] : wi);
  }
  acc = block_sum(acc);
  if (threadIdx.x == 0) part_out[blockIdx.x] = acc;
}

// Classical Gram-Schmidt, one pass (applied twice per Arnoldi step: CGS2).
// Its O(n * nv) products run on the FP32 pipe: GB300's FP64 pipe, not HBM,
// bounded the FP64 versions (84% FP64-pipe busy, 12% of DRAM bandwidth).
// Each FP64 value is split into two floats from its bits alone (split_d,
// device.cuh),
// products are formed as in Dot2 (Ogita, Rump and Oishi, SIAM J. Sci.
// Comput. 26 (2005)): the product of the high parts exactly by FMA, the cross
// terms rounded, every addition's error kept.  Dots and updates come out
// within about 1e-14 of the exact values (FP64 summation of the same terms
// is within n * 1.1e-16); only O(n) operations stay on the FP64 pipe.

__device__ __forceinline__ float2 split_t(double a) { return split_d(a); }
__device__ __forceinline__ float2 split_t(float a) { return make_float2(a, 0.f); }

// cgs_dots: part[j * kVecCtas + cta] = this CTA's share of <w, v_j> for
// j < nv and cta < kDotCtas.  Grid kDotCtas x ceil(nv / 8): CTA (cta, g)
// takes vectors 8g .. 8g + 7, so every group runs at once and each thread
// keeps eight loads in flight over about n / (kDotCtas * 256) elements; the
// CTA's sums are combined as FP32 pairs (the FP64 pipe would bound a
// reduction in FP64), and a partial's summation order depends only on cta.
constexpr int kDotGroup = 8;
constexpr int kDotCtas = 152;
template <typename T>
__global__ void __launch_bounds__(kThreads)
    cgs_dots_kernel(const T* __restrict__ w, const T* __restrict__ V, int64_t n, int nv, double* __restrict__ part) {
  constexpr int U = kDotGroup;
  __shared__ float shs[U][kThreads / 32], shc[U][kThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int j0 = blockIdx.y * U;
  const int jn = min(U, nv - j0);
  float as[U], ac[U];
#pragma unroll
  for (int u = 0; u < U; u++) as[u] = ac[u] = 0.f;
  for (int64_t i = blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n; i += int64_t(kDotCtas) * kThreads) {
    const float2 wi = split_t(w[i]);
#pragma unroll
    for (int u = 0; u < U; u++)
      if (u < jn) dot2_add(as[u], ac[u], split_t(V[int64_t(j0 + u) * n + i]), wi);
  }
#pragma unroll
  for (int u = 0; u < U; u++) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
      pair_add(as[u], ac[u], __shfl_xor_sync(0xffffffffu, as[u], o), __shfl_xor_sync(0xffffffffu, ac[u], o));
    if (lane == 0) {
      shs[u][wid] = as[u];
      shc[u][wid] = ac[u];
    }
  }
  __syncthreads();
  if (threadIdx.x < jn) {
    float vs = 0.f, vc = 0.f;
    for (int q = 0; q < kThreads / 32; q++) pair_add(vs, vc, shs[threadIdx.x][q], shc[threadIdx.x][q]);
    part[int64_t(j0 + threadIdx.x) * kVecCtas + blockIdx.x] = __dadd_rn(double(vs), double(vc));
  }
}

// Sum of the first kDotCtas partials in a fixed order (each CTA gets the same value).
__device__ double reduce_dot_parts(const double* part) {
  double v = 0.0;
  for (int i = threadIdx.x; i < kDotCtas; i += kThreads) v += part[i];
  return block_sum(v);
}

// One CTA per basis vector j: hc[j] = <w, v_j> from the partial sums (fixed
// order); the Hessenberg column gets hc (first pass) or hc added (second).
__global__ void __launch_bounds__(kThreads)
    cgs_reduce_kernel(const double* __restrict__ part, double* __restrict__ hc, double* __restrict__ hcol, int second) {
  const int j = blockIdx.x;
  const double v = reduce_dot_parts(part + int64_t(j) * kVecCtas);
  if (threadIdx.x == 0) {
    hc[j] = v;
    hcol[j] = second ? __dadd_rn(hcol[j], v) : v;
  }
}

// w -= sum_j hc[j] v_j: the sum of the products as above, then one FP64
// subtraction, rounded to T once; with part, also the partial sums of |w|^2
// for the normalisation (as FP32 pairs until one FP64 value per CTA).
// nv <= kMaxBasis (the restart length + 1).
constexpr int kMaxBasis = 1001;
template <typename T>
__global__ void __launch_bounds__(kThreads) cgs_update_kernel(T* __restrict__ w, const T* __restrict__ V, int64_t n,
                                                              int nv, const double* __restrict__ hc,
                                                              double* __restrict__ part) {
  __shared__ float2 hs[kMaxBasis];
  __shared__ float ps[kThreads / 32], pc[kThreads / 32];
  for (int j = threadIdx.x; j < nv; j += kThreads) hs[j] = split_d(hc[j]);
  __syncthreads();
  float ns = 0.f, nc = 0.f;
  for (int64_t i = blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n; i += int64_t(kVecCtas) * kThreads) {
    float s = 0.f, c = 0.f;
#pragma unroll 8
    for (int j = 0; j < nv; j++) dot2_add(s, c, split_t(V[int64_t(j) * n + i]), hs[j]);
    const T t = T(__dsub_rn(to_d(w[i]), __dadd_rn(double(s), double(c))));
    w[i] = t;
    const float2 ts = split_t(t);
    dot2_add(ns, nc, ts, ts);
  }
  if (part) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
      pair_add(ns, nc, __shfl_xor_sync(0xffffffffu, ns, o), __shfl_xor_sync(0xffffffffu, nc, o));
    if (lane == 0) {
      ps[wid] = ns;
      pc[wid] = nc;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      float vs = 0.f, vc = 0.f;
      for (int q = 0; q < kThreads / 32; q++) pair_add(vs, vc, ps[q], pc[q]);
      part[blockIdx.x] = __dadd_rn(double(vs), double(vc));
    }
  }
}

// h = sqrt(<w, w>) from part; v_next = (1 / h) * w (GMRES.hpp:241-242).
template <typename T>
__global__ void __launch_bounds__(kThreads)
    normalize_kernel(const T* w, T* vnext, int64_t n, const double* ih_ptr) {
  const double ih = *ih_ptr;
  for (int64_t i = blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n; i += int64_t(kVecCtas) * kThreads)
    vnext[i] = T(__dmul_rn(ih, to_d(w[i])));
}

// h = sqrt(<w, w>) from part into *hout and 1 / h into *ihout, once (one CTA):
// every CTA of normalize_kernel then multiplies by the same value without
// summing the partials and dividing itself.
__global__ void __launch_bounds__(kThreads) norm_recip_kernel(const double* part, double* hout, double* ihout) {
  const double h = sqrt(reduce_parts(part));
  if (threadIdx.x == 0) {
    *hout = h;
    *ihout = 1.0 / h;
  }
}

// v0 = r * (1 / beta) (GMRES.hpp:220); s = beta e_0.
template <typename T>
__global__ void __launch_bounds__(kThreads)
    start_cycle_kernel(const T* r, T* v0, int64_t n, const double* scal, double* s, int restart) {
  const double ib = 1.0 / scal[1];
  for (int64_t i = blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n; i += int64_t(kVecCtas) * kThreads)
    v0[i] = T(__dmul_rn(to_d(r[i]), ib));
  if (blockIdx.x == 0)
    for (int k = threadIdx.x; k <= restart; k += kThreads) s[k] = k == 0 ? scal[1] : 0.0;
}

__device__ __forceinline__ void apply_rot(double& dx, double& dy, double cs, double sn) {
  const double t = __dadd_rn(__dmul_rn(cs, dx), __dmul_rn(sn, dy));
  dy = __dadd_rn(__dmul_rn(-sn, dx), __dmul_rn(cs, dy));
  dx = t;
}

__device__ __forceinline__ void gen_rot(double dx, double dy, double& cs, double& sn) {
  if (dy == 0.0) {
    cs = 1.0;
    sn = 0.0;
  } else if (fabs(dy) > fabs(dx)) {
    const double t = dx / dy;
    sn = 1.0 / sqrt(__dadd_rn(1.0, __dmul_rn(t, t)));
    cs = __dmul_rn(t, sn);
  } else {
    const double t = dy / dx;
    cs = 1.0 / sqrt(__dadd_rn(1.0, __dmul_rn(t, t)));
    sn = __dmul_rn(t, cs);
  }
}

// Rotations for column i of H and the residual estimate (GMRES.hpp:244-250).
// The running entry stays in a register (H and rot do not alias), so the
// loads of the next entry and rotation are not held up by the stores.
__global__ void givens_kernel(double* __restrict__ H, int ldh, double* __restrict__ rot, int restart, int i,
                              double* __restrict__ scal) {
  double* cs = rot;
  double* sn = rot + (restart + 1);
  double* s = rot + 2 * (restart + 1);
  double* h = H + int64_t(i) * ldh;
  double hk = h[0];
  for (int k = 0; k < i; k++) {
    double hk1 = h[k + 1];
    apply_rot(hk, hk1, cs[k], sn[k]);
    h[k] = hk;
    hk = hk1;
  }
  double hi1 = h[i + 1];
  gen_rot(hk, hi1, cs[i], sn[i]);
  apply_rot(hk, hi1, cs[i], sn[i]);
  h[i] = hk;
  h[i + 1] = hi1;
  apply_rot(s[i], s[i + 1], cs[i], sn[i]);
  scal[0] = fabs(s[i + 1]) / scal[2];
}

// Update (GMRES.hpp:132-146): back substitution into y.
__global__ void backsolve_kernel(const double* H, int ldh, double* rot, int restart, int k) {
  const double* s = rot + 2 * (restart + 1);
  double* y = rot + 3 * (restart + 1);
  for (int i = 0; i <= k; i++) y[i] = s[i];
  for (int i = k; i >= 0; i--) {
    y[i] /= H[i + int64_t(i) * ldh];
    for (int j = i - 1; j >= 0; j--) y[j] = __dsub_rn(y[j], __dmul_rn(H[j + int64_t(i) * ldh], y[i]));
  }
}

// x += sum_j V_j y_j, accumulated j by j as the reference does.
template <typename T>
__global__ void __launch_bounds__(kThreads)
    update_x_kernel(T* x, const T* V, int64_t ldv, const double* rot, int restart, int k, int64_t n) {
  const double* y = rot + 3 * (restart + 1);
  for (int64_t i = blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n; i += int64_t(kVecCtas) * kThreads) {
    double xi = to_d(x[i]);
    for (int j = 0; j <= k; j++) xi = __dadd_rn(xi, __dmul_rn(to_d(V[j * ldv + i]), y[j]));
    x[i] = T(xi);
  }
}

// c = a - b and partial sums of |c|^2.
template <typename T>
__global__ void __launch_bounds__(kThreads) sub_norm_kernel(const T* a, const T* b, T* c, int64_t n, double* part) {
  double acc = 0.0;
  for (int64_t i = blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n; i += int64_t(kVecCtas) * kThreads) {
    const double v = __dsub_rn(to_d(a[i]), to_d(b[i]));
    const T tv = T(v);
    if (c) c[i] = tv;
    acc += to_d(tv) * to_d(tv);
  }
  acc = block_sum(acc);
  if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

__global__ void finish_norm_kernel(const double* part, double* dst) {
  const double v = reduce_parts(part);
  if (threadIdx.x == 0) *dst = sqrt(v);
}

template <typename T>
__global__ void fill_zero_kernel(T* x, int64_t n) {
  for (int64_t i = blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n; i += int64_t(kVecCtas) * kThreads) x[i] = T(0);
}

#define HODLR_TRY(x)                      \
  do {                                    \
    cudaError_t e_ = (x);                 \
    if (e_ != cudaSuccess) return e_;     \
  } while (0)

}  // namespace

template <typename T>
cudaError_t gmres_alloc(GmresWork<T>& W, int64_t n, int restart) {
  gmres_free(W);
  W.n = n;
  W.restart = restart;
  HODLR_TRY(cudaMalloc(&W.V, sizeof(T) * size_t(n) * size_t(restart + 1)));
  HODLR_TRY(cudaMalloc(&W.w, sizeof(T) * size_t(n)));
  HODLR_TRY(cudaMalloc(&W.r, sizeof(T) * size_t(n)));
  HODLR_TRY(cudaMalloc(&W.tmp, sizeof(T) * size_t(n)));
  HODLR_TRY(cudaMalloc(&W.H, sizeof(double) * size_t(restart + 1) * size_t(restart)));
  HODLR_TRY(cudaMemset(W.H, 0, sizeof(double) * size_t(restart + 1) * size_t(restart)));
  HODLR_TRY(cudaMalloc(&W.rot, sizeof(double) * 4 * size_t(restart + 1)));
  HODLR_TRY(cudaMemset(W.rot, 0, sizeof(double) * 4 * size_t(restart + 1)));
  HODLR_TRY(cudaMalloc(&W.part, sizeof(double) * 2 * kVecCtas));
  HODLR_TRY(cudaMalloc(&W.partk, sizeof(double) * kVecCtas * size_t(restart + 1)));
  HODLR_TRY(cudaMalloc(&W.hc, sizeof(double) * size_t(restart + 1)));
  HODLR_TRY(cudaMalloc(&W.scal, sizeof(double) * 8));
  HODLR_TRY(cudaMallocHost(&W.hscal, sizeof(double) * 8));
  return cudaSuccess;
}

template <typename T>
void gmres_free(GmresWork<T>& W) {
  cudaFree(W.V);
  cudaFree(W.w);
  cudaFree(W.r);
  cudaFree(W.tmp);
  cudaFree(W.H);
  cudaFree(W.rot);
  cudaFree(W.part);
  cudaFree(W.partk);
  cudaFree(W.hc);
  cudaFree(W.scal);
  if (W.hscal) cudaFreeHost(W.hscal);
  W = GmresWork<T>();
}

template <typename T>
cudaError_t vec_sub_norm2(const T* a, const T* b, T* c, int64_t n, double* part, double* dst, cudaStream_t st) {
  count_launches(1);
  sub_norm_kernel<T><<<kVecCtas, kThreads, 0, st>>>(a, b, c, n, part);
  count_launches(1);
  finish_norm_kernel<<<1, kThreads, 0, st>>>(part, dst);
  return cudaGetLastError();
}

template <typename T>
cudaError_t vec_norm2(const T* a, int64_t n, double* part, double* dst, cudaStream_t st) {
  count_launches(1);
  dot_partial_kernel<T><<<kVecCtas, kThreads, 0, st>>>(a, a, n, part);
  count_launches(1);
  finish_norm_kernel<<<1, kThreads, 0, st>>>(part, dst);
  return cudaGetLastError();
}

template <typename T>
cudaError_t slots_norm2(const T* y, int64_t n, int s0, int s1, double* part, double* dst, cudaStream_t st) {
  count_launches(1);
  slots_partial_kernel<T><<<kVecCtas, kThreads, 0, st>>>(y, n, s0, s1, part);
  count_launches(1);
  finish_norm_kernel<<<1, kThreads, 0, st>>>(part, dst);
  return cudaGetLastError();
}

template <typename T>
cudaError_t gmres_solve(GmresWork<T>& W, const TreeMatvec<T>& A, const T* b, T* x, bool x0_zero, int restart,
                        int64_t max_iter, double tol, cudaStream_t st, GmresResult* res, Ortho ortho,
                        const std::function<void(double)>& progress) {
  const int64_t n = W.n;
  if (restart > W.restart || restart < 1) return cudaErrorInvalidValue;
  const int m = restart, ldh = W.restart + 1;
  double* part0 = W.part;
  double* part1 = W.part + kVecCtas;
  auto host_scal = [&](int count) -> cudaError_t {
    HODLR_TRY(cudaMemcpyAsync(W.hscal, W.scal, sizeof(double) * size_t(count), cudaMemcpyDeviceToHost, st));
    return cudaStreamSynchronize(st);
  };
  // normb = |b|; r = b - A x; beta = |r| (GMRES.hpp:186-197)
  HODLR_TRY(vec_norm2<T>(b, n, part0, W.scal + 2, st));
  if (x0_zero) {
    count_launches(1);
    fill_zero_kernel<T><<<kVecCtas, kThreads, 0, st>>>(x, n);
    HODLR_TRY(vec_sub_norm2<T>(b, x, W.r, n, part0, W.scal + 1, st));
  } else {
    HODLR_TRY(A(x, W.tmp));
    HODLR_TRY(vec_sub_norm2<T>(b, W.tmp, W.r, n, part0, W.scal + 1, st));
  }
  HODLR_TRY(host_scal(3));
  if (W.hscal[2] == 0.0) {
    W.hscal[2] = 1.0;
    HODLR_TRY(cudaMemcpyAsync(W.scal + 2, W.hscal + 2, sizeof(double), cudaMemcpyHostToDevice, st));
  }
  double resid = W.hscal[1] / W.hscal[2];
  res->converged = false;
  if (resid <= tol) {
    res->iterations = 0;
    res->resid = resid;
    res->converged = true;
    return cudaSuccess;
  }
  int64_t j = 1;
  while (j <= max_iter) {
    count_launches(1);
    start_cycle_kernel<T><<<kVecCtas, kThreads, 0, st>>>(W.r, W.V, n, W.scal, W.rot + 2 * (W.restart + 1), W.restart);
    for (int i = 0; i < m && j <= max_iter; i++, j++) {
      T* vi = W.V + int64_t(i) * n;
      HODLR_TRY(A(vi, W.w));
      double* plast;
      if (ortho == Ortho::kMGS) {
        count_launches(1);
        dot_partial_kernel<T><<<kVecCtas, kThreads, 0, st>>>(W.w, W.V, n, part0);
        for (int k = 0; k <= i; k++) {
          const T* next = k < i ? W.V + int64_t(k + 1) * n : nullptr;
          double* pin = (k & 1) ? part1 : part0;
          double* pout = (k & 1) ? part0 : part1;
          count_launches(1);
          mgs_step_kernel<T><<<kVecCtas, kThreads, 0, st>>>(W.w, W.V + int64_t(k) * n, next, n, pin, pout,
                                                             W.H + k + int64_t(i) * ldh);
        }
        plast = (i & 1) ? part0 : part1;
      } else {
        // CGS2: two classical passes against v_0 .. v_i, |w|^2 from the second
        for (int pass = 0; pass < 2; pass++) {
          count_launches(3);
          cgs_dots_kernel<T><<<dim3(kDotCtas, unsigned((i + 1 + kDotGroup - 1) / kDotGroup)), kThreads, 0, st>>>(
              W.w, W.V, n, i + 1, W.partk);
          cgs_reduce_kernel<<<i + 1, kThreads, 0, st>>>(W.partk, W.hc, W.H + int64_t(i) * ldh, pass);
          cgs_update_kernel<T><<<kVecCtas, kThreads, 0, st>>>(W.w, W.V, n, i + 1, W.hc, pass == 1 ? part0 : nullptr);
        }
        plast = part0;
      }
      count_launches(2);
      norm_recip_kernel<<<1, kThreads, 0, st>>>(plast, W.H + (i + 1) + int64_t(i) * ldh, W.scal + 4);
      normalize_kernel<T><<<kVecCtas, kThreads, 0, st>>>(W.w, W.V + int64_t(i + 1) * n, n, W.scal + 4);
      count_launches(1);
      givens_kernel<<<1, 1, 0, st>>>(W.H, ldh, W.rot, W.restart, i, W.scal);
      HODLR_TRY(cudaGetLastError());
      HODLR_TRY(host_scal(1));
      resid = W.hscal[0];
      if (progress) progress(resid);
      if (resid < tol) {
        count_launches(1);
        backsolve_kernel<<<1, 1, 0, st>>>(W.H, ldh, W.rot, W.restart, i);
        count_launches(1);
        update_x_kernel<T><<<kVecCtas, kThreads, 0, st>>>(x, W.V, n, W.rot, W.restart, i, n);
        HODLR_TRY(cudaGetLastError());
        res->iterations = j;
        res->resid = resid;
        res->converged = true;
        return cudaStreamSynchronize(st);
      }
    }
    count_launches(1);
    backsolve_kernel<<<1, 1, 0, st>>>(W.H, ldh, W.rot, W.restart, m - 1);
    count_launches(1);
    update_x_kernel<T><<<kVecCtas, kThreads, 0, st>>>(x, W.V, n, W.rot, W.restart, m - 1, n);
    if (progress) progress(1.0);  // the restart's true residual
    HODLR_TRY(A(x, W.tmp));
    HODLR_TRY(vec_sub_norm2<T>(b, W.tmp, W.r, n, part0, W.scal + 1, st));
    HODLR_TRY(host_scal(2));
    resid = W.hscal[1] / W.hscal[2];
    if (resid < tol) {
      res->iterations = j;
      res->resid = resid;
      res->converged = true;
      return cudaSuccess;
    }
  }
  res->iterations = max_iter;
  res->resid = resid;
  return cudaSuccess;
}

template cudaError_t gmres_alloc<double>(GmresWork<double>&, int64_t, int);
template cudaError_t gmres_alloc<float>(GmresWork<float>&, int64_t, int);
template void gmres_free<double>(GmresWork<double>&);
template void gmres_free<float>(GmresWork<float>&);
template cudaError_t gmres_solve<double>(GmresWork<double>&, const TreeMatvec<double>&, const double*, double*, bool,
                                         int, int64_t, double, cudaStream_t, GmresResult*, Ortho,
                                         const std::function<void(double)>&);
template cudaError_t gmres_solve<float>(GmresWork<float>&, const TreeMatvec<float>&, const float*, float*, bool, int,
                                        int64_t, double, cudaStream_t, GmresResult*, Ortho,
                                        const std::function<void(double)>&);
template cudaError_t vec_sub_norm2<double>(const double*, const double*, double*, int64_t, double*, double*,
                                           cudaStream_t);
template cudaError_t vec_sub_norm2<float>(const float*, const float*, float*, int64_t, double*, double*, cudaStream_t);
template cudaError_t vec_norm2<double>(const double*, int64_t, double*, double*, cudaStream_t);
template cudaError_t slots_norm2<double>(const double*, int64_t, int, int, double*, double*, cudaStream_t);
template cudaError_t vec_norm2<float>(const float*, int64_t, double*, double*, cudaStream_t);

}  // namespace hodlr
