// Restarted GMRES on the device (gmres.cu).
//
// Follows iterSolver::GMRES (HODLRnD include/GMRES.hpp:160-305): modified
// Gram-Schmidt Arnoldi, real Givens rotations (:83-103,124-129), back
// substitution Update (:132-146), restart with a true residual, relative
// residual against |b|.  Vectors are of type T (double, or float for the
// inner solve of mixed precision); the Hessenberg matrix, the rotations, the
// least-squares right-hand side and every reduction are FP64.
//
// Orthogonalisation:
// * kMGS, the reference's modified Gram-Schmidt: each step is one kernel that
//   finishes the previous dot product from the per-CTA partial sums (fixed
//   order, so results are deterministic), applies w -= h v_k and accumulates
//   the partial sums of the next dot product -- i + 2 launches at step i;
// * kCGS2, classical Gram-Schmidt applied twice: per pass one kernel forms all
//   i + 1 dot products, one reduces them, one applies the update -- six
//   launches at any step, and the same orthogonality as MGS or better
//   (Giraud, Langou, Rozloznik, "The loss of orthogonality in the
//   Gram-Schmidt processes", Comput. Math. Appl. 50 (2005)).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <functional>

namespace hodlr {

constexpr int kVecCtas = 152 * 4;  // fixed grid of the vector kernels

template <typename T>
struct GmresWork {
  int64_t n = 0;
  int restart = 0;
  T* V = nullptr;  // (restart + 1) Krylov vectors of length n
  T* w = nullptr;
  T* r = nullptr;
  T* tmp = nullptr;
  double* H = nullptr;    // (restart + 1) x restart, column major
  double* rot = nullptr;  // cs, sn, s, y: 4 x (restart + 1)
  double* part = nullptr; // 2 x kVecCtas partial sums
  double* partk = nullptr; // (restart + 1) x kVecCtas partial sums (CGS2)
  double* hc = nullptr;    // restart + 1 projection coefficients of one CGS pass
  double* scal = nullptr; // device scalars: [0] resid, [1] beta, [2] normb
  double* hscal = nullptr;  // pinned host mirror of scal
};

template <typename T>
cudaError_t gmres_alloc(GmresWork<T>& W, int64_t n, int restart);
template <typename T>
void gmres_free(GmresWork<T>& W);

// y = A x in tree order, type T, asynchronous on the solver's stream.
template <typename T>
using TreeMatvec = std::function<cudaError_t(const T* x, T* y)>;

enum class Ortho { kMGS, kCGS2 };

struct GmresResult {
  int64_t iterations = 0;  // the reference's return value
  double resid = 0.0;      // last relative residual estimate
  bool converged = false;
};

// Solve A x = b.  x holds x0 on entry unless x0_zero (then x is overwritten
// with zeros first and the initial matvec is skipped).  `progress`, when
// set, is called with the residual estimate after every Arnoldi step and
// with 1.0 before the true residual of a restart (an inexact method can
// choose the accuracy of its next products from it).
template <typename T>
cudaError_t gmres_solve(GmresWork<T>& W, const TreeMatvec<T>& A, const T* b, T* x, bool x0_zero, int restart,
                        int64_t max_iter, double tol, cudaStream_t st, GmresResult* res, Ortho ortho = Ortho::kMGS,
                        const std::function<void(double)>& progress = {});

// Vector helpers shared with the iterative refinement.
// out = ||a - b||^2 partial + final into *dst (device double); c = a - b written when c != NULL.
template <typename T>
cudaError_t vec_sub_norm2(const T* a, const T* b, T* c, int64_t n, double* part, double* dst, cudaStream_t st);
template <typename T>
cudaError_t vec_norm2(const T* a, int64_t n, double* part, double* dst, cudaStream_t st);
// *dst = || sum_{s = s0}^{s1 - 1} y[s * n .. s * n + n) || (output slots of a matvec)
template <typename T>
cudaError_t slots_norm2(const T* y, int64_t n, int s0, int s1, double* part, double* dst, cudaStream_t st);

}  // namespace hodlr
