// Test-oracle only.  Stand-in for the user-edited configuration header of
// HODLRnD (include/myHeaders.hpp:1-183).  The reference keeps its
// hyper-parameters as `const` globals that a user edits by hand
// (README.md:4-9); this header supplies the same globals from -D macros so
// that the reference's own headers (HDD_matrix.hpp, HDD_tree.hpp,
// HDD_node.hpp, HDD_clusters.hpp, LowRank_matrix.hpp, kernel_function.hpp,
// GMRES.hpp, points_dt.hpp) can be compiled unmodified, in place, once per
// configuration.  It defines the include guard `myHeaders_HPP` first, so the
// reference's own myHeaders.hpp is skipped when they include it.
//
// Everything here mirrors myHeaders.hpp's declarations (names, types and
// the double-precision branch :65-73); the bodies are restated.  cereal I/O
// (myHeaders.hpp:146-170) is not needed by the oracle and is left out.
#ifndef myHeaders_HPP
#define myHeaders_HPP

#include <iostream>
#include <chrono>
#include <ctime>
#include <set>
#include <string>
#include <vector>
#include <random>
#include <cmath>
#include <complex>
#include <iterator>
#include <math.h>
#include <iomanip>
#include <fstream>
#include <list>
#include <algorithm>
#include <numeric>
#include <stack>
#include <omp.h>

#define _USE_MATH_DEFINES
#include <Eigen/Dense>
#include <Eigen/Sparse>

#if !defined(REF_NDIM) || !defined(REF_NMAX) || !defined(REF_DPRIME) || !defined(REF_EPS)
#error "ref_config.hpp needs -DREF_NDIM -DREF_NMAX -DREF_DPRIME -DREF_EPS"
#endif

using std::string;
using namespace Eigen;

const std::string data_directory = "";
const double PI = 4.0 * atan(1);

const int nThreads = 1;
const int NDIM = REF_NDIM;
const int Nmax = REF_NMAX;
int numPoints = 10;
const int INTERACTION_TYPE_ALLOWED = REF_DPRIME;
const double eps_ACA = REF_EPS;
const int SYS_SIZE = 2 * Nmax;
size_t N = 1;

int mod(int a, int b) { return ((a % b + b) % b); }

using dtype = double;
using dtype_base = double;
using Mat = Eigen::MatrixXd;
using Vec = Eigen::VectorXd;
#define abs_(x) ((x < 0) ? (-x) : (x))
#define conj_(x) (x)

Eigen::VectorXd uniform_nodes(double a, double b, int n) {
  Eigen::VectorXd X(n);
  double l = (b - a);
  for (int k = 0; k < n; k++) X(k) = a + l / (double)(n - 1) * k;
  return X;
}

std::string inline getTimeStamp() { return std::string("\n"); }

namespace Vec_ops {
dtype_base inline relative_error(Vec& X_ori, Vec& X_comp) { return (X_ori - X_comp).norm() / X_ori.norm(); }
dtype inline dot_product(const Vec& x, const Vec& y) {
  dtype tmp = dtype(0.0);
  for (int i = 0; i < x.size(); i++) tmp += x(i) * y(i);
  return tmp;
}
}  // namespace Vec_ops

template <typename T>
void inline print_vec(std::vector<T>& vec_to_print) {
  for (auto it = vec_to_print.begin(); it != vec_to_print.end(); it++) {
    if (it != vec_to_print.begin()) std::cout << ", ";
    std::cout << *it;
  }
}

#endif
