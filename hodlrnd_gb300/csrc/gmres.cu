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
// cgs_dots: part[j * kVecCtas + cta] = this CTA's share of <w, v_j> for
// j < nv.  Grid kVecCtas x ceil(nv / 8): CTA (cta, g) takes vectors
// 8g .. 8g + 7, so every group runs at once and each thread keeps eight
// loads in flight; a partial's summation order depends only on cta.
constexpr int kDotGroup = 8;
template <typename T>
__global__ void __launch_bounds__(kThreads)
    cgs_dots_kernel(const T* __restrict__ w, const T* __restrict__ V, int64_t n, int nv, double* __restrict__ part) {
  constexpr int U = kDotGroup;
  __shared__ double sh[U][kThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int j0 = blockIdx.y * U;
  const int jn = min(U, nv - j0);
  double acc[U];
#pragma unroll
  for (int u = 0; u < U; u++) acc[u] = 0.0;
  for (int64_t i = blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n; i += int64_t(kVecCtas) * kThreads) {
    const double wi = to_d(w[i]);
#pragma unroll
    for (int u = 0; u < U; u++)
      if (u < jn) acc[u] += to_d(V[int64_t(j0 + u) * n + i]) * wi;
  }
#pragma unroll
  for (int u = 0; u < U; u++) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc[u] += __shfl_xor_sync(0xffffffffu, acc[u], o);
    if (lane == 0) sh[u][wid] = acc[u];
  }
  __syncthreads();
  if (threadIdx.x < jn) {
    double v = 0.0;
    for (int q = 0; q < kThreads / 32; q++) v += sh[threadIdx.x][q];
    part[int64_t(j0 + threadIdx.x) * kVecCtas + blockIdx.x] = v;
  }
}

// One CTA per basis vector j: hc[j] = <w, v_j> from the partial sums (fixed
// order); the Hessenberg column gets hc (first pass) or hc added (second).
__global__ void __launch_bounds__(kThreads)
    cgs_reduce_kernel(const double* __restrict__ part, double* __restrict__ hc, double* __restrict__ hcol, int second) {
  const int j = blockIdx.x;
  const double v = reduce_parts(part + int64_t(j) * kVecCtas);
  if (threadIdx.x == 0) {
    hc[j] = v;
    hcol[j] = second ? __dadd_rn(hcol[j], v) : v;
  }
}

// w -= sum_j hc[j] v_j (in FP64, j in order, rounded to T once); with part,
// also the partial sums of |w|^2 for the normalisation.
template <typename T>
__global__ void __launch_bounds__(kThreads) cgs_update_kernel(T* __restrict__ w, const T* __restrict__ V, int64_t n,
                                                              int nv, const double* __restrict__ hc,
                                                              double* __restrict__ part) {
  double acc = 0.0;
  for (int64_t i = blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n; i += int64_t(kVecCtas) * kThreads) {
    double wi = to_d(w[i]);
#pragma unroll 8
    for (int j = 0; j < nv; j++) wi = axmy(wi, hc[j], to_d(V[int64_t(j) * n + i]));
    const T t = T(wi);
    w[i] = t;
    acc += to_d(t) * to_d(t);
  }
  if (part) {
    acc = block_sum(acc);
    if (threadIdx.x == 0) part[blockIdx.x] = acc;
  }
}

// h = sqrt(<w, w>) from part; v_next = (1 / h) * w (GMRES.hpp:241-242).
template <typename T>
__global__ void __launch_bounds__(kThreads)
    normalize_kernel(const T* w, T* vnext, int64_t n, const double* part, double* hout) {
  const double h = sqrt(reduce_parts(part));
  if (blockIdx.x == 0 && threadIdx.x == 0) *hout = h;
  const double ih = 1.0 / h;
  for (int64_t i = blockIdx.x * int64_t(kThreads) + threadIdx.x; i < n; i += int64_t(kVecCtas) * kThreads)
    vnext[i] = T(__dmul_rn(ih, to_d(w[i])));
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
__global__ void givens_kernel(double* H, int ldh, double* rot, int restart, int i, double* scal) {
  double* cs = rot;
  double* sn = rot + (restart + 1);
  double* s = rot + 2 * (restart + 1);
  double* h = H + int64_t(i) * ldh;
  for (int k = 0; k < i; k++) apply_rot(h[k], h[k + 1], cs[k], sn[k]);
  gen_rot(h[i], h[i + 1], cs[i], sn[i]);
  apply_rot(h[i], h[i + 1], cs[i], sn[i]);
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
          cgs_dots_kernel<T><<<dim3(kVecCtas, unsigned((i + 1 + kDotGroup - 1) / kDotGroup)), kThreads, 0, st>>>(
              W.w, W.V, n, i + 1, W.partk);
          cgs_reduce_kernel<<<i + 1, kThreads, 0, st>>>(W.partk, W.hc, W.H + int64_t(i) * ldh, pass);
          cgs_update_kernel<T><<<kVecCtas, kThreads, 0, st>>>(W.w, W.V, n, i + 1, W.hc, pass == 1 ? part0 : nullptr);
        }
        plast = part0;
      }
      count_launches(1);
      normalize_kernel<T><<<kVecCtas, kThreads, 0, st>>>(W.w, W.V + int64_t(i + 1) * n, n, plast,
                                                          W.H + (i + 1) + int64_t(i) * ldh);
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
template cudaError_t vec_norm2<float>(const float*, int64_t, double*, double*, cudaStream_t);

}  // namespace hodlr
