// hodlrnd_matrix.hpp -- header-only C++17 facade over the C ABI (hodlrnd.h)
// with the class and method names of HODLRnD's HODLRdD_matrix<Kernel>
// (include/HDD_matrix.hpp:10-89), so that reference user code keeps its shape:
//
//   Kernel* ker = ...;                             // provides gpu_kernel_desc()
//   std::vector<ptsnD>* gridPoints = ...;          // the reference's point type
//   hodlrnd::HODLRdD_matrix<Kernel> Kmat(ker, gridPoints, X, Y, params);
//   Kmat.Assemble_matrix_operators();
//   Vec b = Kmat * x;                              // operator*
//   Vec y = Kmat.solve(b);                         // GMRES, x0 = b
//   Kmat.print_matrix_statistics();
//
// Differences a reference user sees:
//  * the kernel describes itself with gpu_kernel_desc() (kind, scale, diag)
//    instead of answering getMatrixEntry(i, j) per entry -- the GPU engine
//    evaluates entries itself and never calls back into host code;
//  * Nmax, eps_ACA and INTERACTION_TYPE_ALLOWED are runtime fields of
//    hodlr_params instead of compile-time constants (include/myHeaders.hpp:35-48);
//    NDIM is taken from the point type;
//  * failures throw hodlrnd::Error carrying the C ABI's status and message.
// Points may be given as the reference's std::vector<ptsnD>* (any struct with
// a double x[NDIM] member, include/points_dt.hpp:9-13) or as a flat n x ndim
// row-major array; the box corners and vectors as any contiguous double
// container with size() and operator[] / data() (std::vector<double>, or
// Eigen::VectorXd as in the reference).
#pragma once

#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "hodlrnd.h"

namespace hodlrnd {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void check(int rc, const hodlr_ctx* ctx) {
  if (rc != HODLR_OK) throw Error(rc, hodlr_last_error(ctx));
}

inline hodlr_params default_params(int ndim) {
  hodlr_params p;
  hodlr_params_default(&p);
  p.ndim = ndim;
  return p;
}

// the NDIM of a ptsnD-like point type: the extent of its x[] member
template <class Pt>
constexpr int point_dim() {
  return int(std::extent<decltype(Pt::x)>::value);
}

template <class Box>
std::vector<double> to_std(const Box& b) {
  std::vector<double> v(size_t(b.size()));
  for (size_t k = 0; k < v.size(); k++) v[k] = double(b[k]);
  return v;
}

template <class Kernel>
class HODLRdD_matrix {
 public:
  // HODLRdD_matrix(Kernel*&, std::vector<ptsnD>*&, VectorXd x1, VectorXd x2)
  // (include/HDD_matrix.hpp:20-33): the reference's own argument shapes.  The
  // points are copied (the engine keeps them on the device).  params.ndim is
  // set from the point type; params defaults to the reference's constants.
  template <class Pt, class Box>
  HODLRdD_matrix(Kernel* kernel, std::vector<Pt>* gridPoints, const Box& x1, const Box& x2,
                 hodlr_params params = default_params(point_dim<Pt>()))
      : HODLRdD_matrix(kernel, flatten(gridPoints), to_std(x1), to_std(x2), with_ndim(params, point_dim<Pt>())) {}

  // points: n x ndim row major (the x[] of each ptsnD, one after another).
  HODLRdD_matrix(Kernel* kernel, const std::vector<double>& points, const std::vector<double>& x1,
                 const std::vector<double>& x2, const hodlr_params& params)
      : kernel_(kernel), points_(points), x1_(x1), x2_(x2), p_(params) {
    if (p_.ndim < 1 || x1.size() != size_t(p_.ndim) || x2.size() != size_t(p_.ndim) ||
        points.size() % size_t(p_.ndim) != 0)
      throw Error(HODLR_ERR_INVALID, "HODLRdD_matrix: points / box do not match ndim");
    n_ = int64_t(points.size() / size_t(p_.ndim));
    check(hodlr_ctx_create(&p_, &ctx_), nullptr);
  }
  HODLRdD_matrix(const HODLRdD_matrix&) = delete;
  HODLRdD_matrix& operator=(const HODLRdD_matrix&) = delete;
  ~HODLRdD_matrix() {
    hodlr_op_destroy(op_);
    hodlr_ctx_destroy(ctx_);
  }

  size_t get_size() const { return size_t(n_); }

  // Assemble_matrix_operators (include/HDD_matrix.hpp:39-41)
  void Assemble_matrix_operators() {
    hodlr_op_destroy(op_);
    op_ = nullptr;
    const hodlr_kernel_desc kd = kernel_->gpu_kernel_desc();
    check(hodlr_build(ctx_, points_.data(), n_, x1_.data(), x2_.data(), &kd, &op_), ctx_);
  }

  // operator* (include/HDD_matrix.hpp:43-47); Vec: std::vector<double>,
  // Eigen::VectorXd or any contiguous double vector constructible from a size
  template <class Vec>
  Vec operator*(const Vec& x) {
    need_op();
    need_size(size_t(x.size()));
    Vec y(x.size());
    check(hodlr_matvec(op_, x.data(), y.data(), 1), ctx_);
    return y;
  }

  // solve (include/HDD_matrix.hpp:51-62); the reference's GMRES iteration count
  // is in last_solve().iterations.
  template <class Vec>
  Vec solve(const Vec& b) {
    need_op();
    need_size(size_t(b.size()));
    Vec x(b.size());
    const int rc = hodlr_solve(op_, b.data(), x.data(), 1, &info_);
    if (rc != HODLR_OK && rc != HODLR_ERR_NOT_CONVERGED) check(rc, ctx_);
    return x;
  }
  const hodlr_solve_info& last_solve() const { return info_; }

  hodlr_stats statistics() const {
    hodlr_stats s;
    check(hodlr_stats_get(op_, &s), ctx_);
    return s;
  }

  // print_matrix_statistics (include/HDD_matrix.hpp:69-85)
  void print_matrix_statistics() const {
    const hodlr_stats s = statistics();
    std::printf("Memory (in GB) : %g\nNumber of FLOP : %g\nCompression Ratio : %g\n", s.memory_gb, s.n_flop,
                s.compression_ratio);
    std::printf("Maximum rank across the Tree : %lld\nTime to Initialize (in s) : %g\nMatrix-Vector time (in s) : %g\n",
                (long long)s.max_rank, s.t_build_s, s.t_matvec_s);
  }

  hodlr_op* handle() { return op_; }

 private:
  template <class Pt>
  static std::vector<double> flatten(const std::vector<Pt>* pts) {
    if (!pts) throw Error(HODLR_ERR_INVALID, "HODLRdD_matrix: null point vector");
    constexpr int d = point_dim<Pt>();
    std::vector<double> flat(pts->size() * size_t(d));
    for (size_t i = 0; i < pts->size(); i++)
      for (int k = 0; k < d; k++) flat[i * size_t(d) + size_t(k)] = (*pts)[i].x[k];
    return flat;
  }
  static hodlr_params with_ndim(hodlr_params p, int ndim) {
    p.ndim = ndim;
    return p;
  }
  void need_op() const {
    if (!op_) throw Error(HODLR_ERR_STATE, "call Assemble_matrix_operators() first");
  }
  void need_size(size_t n) const {
    if (n != size_t(n_)) throw Error(HODLR_ERR_INVALID, "vector length differs from the number of points");
  }
  Kernel* kernel_;
  std::vector<double> points_, x1_, x2_;
  hodlr_params p_;
  int64_t n_ = 0;
  hodlr_ctx* ctx_ = nullptr;
  hodlr_op* op_ = nullptr;
  hodlr_solve_info info_{};
};

// storedata::load_vec / save_vec (include/myHeaders.hpp:146-170) on
// std::vector<double>, through hodlr_vec_load / hodlr_vec_save (no cereal).
namespace storedata {
inline std::vector<double> load_vec(const std::string& fname) {
  int64_t n = 0;
  check(hodlr_vec_load(fname.c_str(), nullptr, 0, &n), nullptr);
  std::vector<double> x(static_cast<size_t>(n));
  check(hodlr_vec_load(fname.c_str(), x.data(), n, &n), nullptr);
  return x;
}
inline void save_vec(const std::string& fname, const std::vector<double>& x) {
  check(hodlr_vec_save(fname.c_str(), x.data(), int64_t(x.size())), nullptr);
}
}  // namespace storedata

}  // namespace hodlrnd
