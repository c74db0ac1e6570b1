// Test-oracle only: drives the reference HODLRnD headers, compiled unmodified
// from where they lie (see build_ref.py), on a seeded input file and dumps
// what the parity fixtures need: the tree (HDD_tree.hpp:23-74), the
// interaction/neighbour lists (HDD_node.hpp:150-180), every low-rank block's
// rank and representation (LowRank_matrix.hpp:22-36), one matvec
// (HDD_matrix.hpp:43-47), one GMRES solve set up exactly as
// HODLRdD_matrix::solve does (HDD_matrix.hpp:51-62) and the statistics of
// print_matrix_statistics (HDD_matrix.hpp:69-85).
//
// Modes (first argument):
//   hodlr  <in.bin> <out.bin>   build + matvec + solve on the input points
//   gmres  <in.bin> <out.bin>   iterSolver::GMRES (GMRES.hpp:160-305) on the
//                               dense kernel matrix, to pin the GMRES restatement
//   golden4d <out.bin>          kernel_4d_test (user_kernel.hpp:117-179) on its
//                               numPoints=10 grid: dense rows and the HODLR
//                               matvec of the x in data/x_10000.bin
//
// Private members are read through the explicit-instantiation access rule
// (an explicit instantiation may name private members), so the reference
// headers are not edited.
#include "ref_config.hpp"

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>

#include "HDD_matrix.hpp"
#include "points_dt.hpp"
#ifdef REF_WITH_USER_KERNELS
#include "user_kernel.hpp"
#endif

// ---------------------------------------------------------------- access
template <typename Tag, typename Tag::type M>
struct Rob {
  friend typename Tag::type get(Tag) { return M; }
};

// ---------------------------------------------------------------- I/O
struct Reader {
  std::vector<char> buf;
  size_t pos = 0;
  explicit Reader(const char* path) {
    FILE* f = std::fopen(path, "rb");
    if (!f) throw std::runtime_error(std::string("cannot open ") + path);
    std::fseek(f, 0, SEEK_END);
    long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    buf.resize(size_t(n));
    if (std::fread(buf.data(), 1, buf.size(), f) != buf.size()) throw std::runtime_error("short read");
    std::fclose(f);
  }
  template <typename T>
  T get() {
    T v;
    std::memcpy(&v, buf.data() + pos, sizeof(T));
    pos += sizeof(T);
    return v;
  }
  void get_array(double* dst, size_t n) {
    std::memcpy(dst, buf.data() + pos, n * sizeof(double));
    pos += n * sizeof(double);
  }
};

struct Writer {
  FILE* f;
  explicit Writer(const char* path) : f(std::fopen(path, "wb")) {
    if (!f) throw std::runtime_error(std::string("cannot open ") + path);
  }
  ~Writer() { std::fclose(f); }
  template <typename T>
  void put(const std::string& name, char code, const T* data, uint64_t n) {
    uint32_t len = uint32_t(name.size());
    std::fwrite(&len, 4, 1, f);
    std::fwrite(name.data(), 1, len, f);
    std::fwrite(&code, 1, 1, f);
    std::fwrite(&n, 8, 1, f);
    std::fwrite(data, sizeof(T), n, f);
  }
  void f64(const std::string& name, const std::vector<double>& v) { put(name, 'd', v.data(), v.size()); }
  void i64(const std::string& name, const std::vector<int64_t>& v) { put(name, 'q', v.data(), v.size()); }
};

// ---------------------------------------------------------------- kernel
// Kernel kinds shared with the restatement and the GPU engine:
//   1: scale / r   2: scale / r^2 (as scale / d2)   3: scale * log(r)   4: scale * exp(-r)
// with r = sqrt(d2), d2 = sum_k (x_ik - x_jk)^2 accumulated in dimension order,
// and A_ii = diag.
class cfg_kernel {
 public:
  std::vector<ptsnD>* gridPoints;
  int kind;
  double scale, diag;
  void get_points(std::vector<ptsnD>*& src) { src = gridPoints; }
  dtype_base getMatrixEntry(int i, int j) {
    if (i == j) return diag;
    const ptsnD& a = gridPoints->at(i);
    const ptsnD& b = gridPoints->at(j);
    double d2 = 0.0;
    for (int k = 0; k < NDIM; k++) {
      const double t = a.x[k] - b.x[k];
      d2 = d2 + t * t;
    }
    switch (kind) {
      case 1: return scale / std::sqrt(d2);
      case 2: return scale / d2;
      case 3: return scale * std::log(std::sqrt(d2));
      case 4: return scale * std::exp(-std::sqrt(d2));
    }
    return 0.0;
  }
};

typedef cfg_kernel K;
struct TagTree { typedef Tree<K>* HODLRdD_matrix<K>::*type; friend type get(TagTree); };
struct TagObj { typedef std::vector<std::vector<Node<K>*>> Tree<K>::*type; friend type get(TagObj); };
struct TagLevel { typedef int Tree<K>::*type; friend type get(TagLevel); };
struct TagSelf { typedef size_t Node<K>::*type; friend type get(TagSelf); };
struct TagLR { typedef LowRankMat<K>* Node<K>::*type; friend type get(TagLR); };
struct TagMem { typedef bool LowRankMat<K>::*type; friend type get(TagMem); };
template struct Rob<TagTree, &HODLRdD_matrix<K>::HODLRdD_tree>;
template struct Rob<TagObj, &Tree<K>::obj_arr>;
template struct Rob<TagLevel, &Tree<K>::level>;
template struct Rob<TagSelf, &Node<K>::self_id>;
template struct Rob<TagLR, &Node<K>::LR>;
template struct Rob<TagMem, &LowRankMat<K>::is_mem_efficient>;

struct Input {
  int64_t n = 0;
  int32_t ndim = 0, kind = 0, restart = 100, max_iter = 0;
  double scale = 0, diag = 0, tol = 0;
  std::vector<double> pts, lo, hi, x, b;
};

static Input read_input(const char* path) {
  Reader r(path);
  Input in;
  in.n = r.get<int64_t>();
  in.ndim = r.get<int32_t>();
  in.kind = r.get<int32_t>();
  in.scale = r.get<double>();
  in.diag = r.get<double>();
  in.restart = r.get<int32_t>();
  in.max_iter = r.get<int32_t>();
  in.tol = r.get<double>();
  if (in.ndim != NDIM) throw std::runtime_error("input NDIM does not match the compiled NDIM");
  in.pts.resize(size_t(in.n) * NDIM);
  r.get_array(in.pts.data(), in.pts.size());
  in.lo.resize(NDIM);
  in.hi.resize(NDIM);
  r.get_array(in.lo.data(), NDIM);
  r.get_array(in.hi.data(), NDIM);
  in.x.resize(size_t(in.n));
  in.b.resize(size_t(in.n));
  r.get_array(in.x.data(), in.x.size());
  r.get_array(in.b.data(), in.b.size());
  return in;
}

static Vec to_vec(const std::vector<double>& v) {
  Vec r(Index(v.size()));
  for (size_t i = 0; i < v.size(); i++) r(Index(i)) = v[i];
  return r;
}
static std::vector<double> from_vec(const Vec& v) {
  std::vector<double> r(size_t(v.size()));
  for (Index i = 0; i < v.size(); i++) r[size_t(i)] = v(i);
  return r;
}

static int mode_hodlr(const char* in_path, const char* out_path) {
  Input in = read_input(in_path);
  std::vector<ptsnD>* pts = new std::vector<ptsnD>(size_t(in.n));
  for (int64_t i = 0; i < in.n; i++) {
    for (int k = 0; k < NDIM; k++) (*pts)[size_t(i)].x[k] = in.pts[size_t(i) * NDIM + k];
    (*pts)[size_t(i)].id = size_t(i);
  }
  N = size_t(in.n);
  cfg_kernel* ker = new cfg_kernel();
  ker->gridPoints = pts;
  ker->kind = in.kind;
  ker->scale = in.scale;
  ker->diag = in.diag;
  Eigen::VectorXd X(NDIM), Y(NDIM);
  for (int k = 0; k < NDIM; k++) {
    X(k) = in.lo[size_t(k)];
    Y(k) = in.hi[size_t(k)];
  }
  double t0 = omp_get_wtime();
  HODLRdD_matrix<K> Kmat(ker, pts, X, Y);
  double t_tree = omp_get_wtime() - t0;
  t0 = omp_get_wtime();
  Kmat.Assemble_matrix_operators();
  double t_init = omp_get_wtime() - t0;

  Vec x = to_vec(in.x);
  t0 = omp_get_wtime();
  Vec y = Kmat * x;
  double t_mv = omp_get_wtime() - t0;

  // HODLRdD_matrix::solve (HDD_matrix.hpp:51-62) with the iteration count kept.
  Vec b = to_vec(in.b);
  Vec xs = b;
  HODLRdD_matrix<K>* mat_obj = &Kmat;
  int max_iter = in.max_iter > 0 ? in.max_iter : int(N);
  iterSolver<HODLRdD_matrix<K>> solver(in.restart, max_iter, in.tol);
  t0 = omp_get_wtime();
  int iters = solver.GMRES(mat_obj, xs, b);
  double t_solve = omp_get_wtime() - t0;
  double resid = solver.getResidual();

  Tree<K>* tree = Kmat.*get(TagTree());
  std::vector<std::vector<Node<K>*>>& obj = tree->*get(TagObj());
  const int levels = tree->*get(TagLevel());

  Writer w(out_path);
  std::vector<int64_t> level_sizes, node_counts, node_ids, nbr_ptr{0}, nbr, intr_ptr{0}, intr, leaf_perm;
  std::vector<int64_t> blk_level, blk_t, blk_s, blk_rank, blk_memeff;
  for (int l = 0; l < levels; l++) {
    level_sizes.push_back(int64_t(obj[size_t(l)].size()));
    for (size_t j = 0; j < obj[size_t(l)].size(); j++) {
      Node<K>* nd = obj[size_t(l)][j];
      node_counts.push_back(int64_t(nd->n_particles));
      node_ids.push_back(int64_t(nd->*get(TagSelf())));
      for (Node<K>* p : nd->my_neighbour_addr) nbr.push_back(int64_t(p->*get(TagSelf())));
      for (Node<K>* p : nd->my_intr_list_addr) intr.push_back(int64_t(p->*get(TagSelf())));
      nbr_ptr.push_back(int64_t(nbr.size()));
      intr_ptr.push_back(int64_t(intr.size()));
      if (l == levels - 1)
        for (size_t q : nd->my_cluster->index_of_points) leaf_perm.push_back(int64_t(q));
      if (nd->n_particles != 0) {
        LowRankMat<K>* LR = nd->*get(TagLR());
        for (int i = 0; i < nd->n_intraction; i++) {
          if (nd->my_intr_list_addr[size_t(i)]->n_particles == 0) continue;
          blk_level.push_back(l);
          blk_t.push_back(int64_t(nd->*get(TagSelf())));
          blk_s.push_back(int64_t(nd->my_intr_list_addr[size_t(i)]->*get(TagSelf())));
          blk_rank.push_back(LR[i].rank());
          blk_memeff.push_back((LR[i].*get(TagMem())) ? 1 : 0);
        }
      }
    }
  }
  double n_flop = 0.0;
  size_t max_rank = 0;
  tree->get_stat(n_flop, max_rank);
  w.i64("level_sizes", level_sizes);
  w.i64("node_counts", node_counts);
  w.i64("node_ids", node_ids);
  w.i64("nbr_ptr", nbr_ptr);
  w.i64("nbr", nbr);
  w.i64("intr_ptr", intr_ptr);
  w.i64("intr", intr);
  w.i64("leaf_perm", leaf_perm);
  w.i64("blk_level", blk_level);
  w.i64("blk_t", blk_t);
  w.i64("blk_s", blk_s);
  w.i64("blk_rank", blk_rank);
  w.i64("blk_memeff", blk_memeff);
  w.f64("y", from_vec(y));
  w.f64("x_solve", from_vec(xs));
  w.i64("gmres_iters", {int64_t(iters)});
  w.f64("gmres_resid", {resid});
  w.f64("stats", {n_flop, double(max_rank), t_tree, t_init, t_mv, t_solve});
  return 0;
}

// Dense operator for iterSolver: y = A x with A the kernel matrix, rows
// accumulated in column order like the eigen_min GEMV.
struct DenseOp {
  Mat A;
  Vec operator*(Vec x) { return A * x; }
};

static int mode_gmres(const char* in_path, const char* out_path) {
  Input in = read_input(in_path);
  std::vector<ptsnD>* pts = new std::vector<ptsnD>(size_t(in.n));
  for (int64_t i = 0; i < in.n; i++)
    for (int k = 0; k < NDIM; k++) (*pts)[size_t(i)].x[k] = in.pts[size_t(i) * NDIM + k];
  cfg_kernel ker;
  ker.gridPoints = pts;
  ker.kind = in.kind;
  ker.scale = in.scale;
  ker.diag = in.diag;
  DenseOp* op = new DenseOp();
  op->A = Mat(Index(in.n), Index(in.n));
  for (int64_t i = 0; i < in.n; i++)
    for (int64_t j = 0; j < in.n; j++) op->A(Index(i), Index(j)) = ker.getMatrixEntry(int(i), int(j));
  Vec b = to_vec(in.b);
  Vec xs = b;
  int max_iter = in.max_iter > 0 ? in.max_iter : int(in.n);
  iterSolver<DenseOp> solver(in.restart, max_iter, in.tol);
  int iters = solver.GMRES(op, xs, b);
  Writer w(out_path);
  w.f64("x_solve", from_vec(xs));
  w.i64("gmres_iters", {int64_t(iters)});
  w.f64("gmres_resid", {solver.getResidual()});
  return 0;
}

#ifdef REF_WITH_USER_KERNELS
// kernel_4d_test on its own grid (user_kernel.hpp:117-179), as include/main.cpp
// and include/generate_rhs.cpp use it with numPoints = 10.
static int mode_golden4d(const char* x_path, const char* out_path) {
  numPoints = 10;
  N = size_t(std::pow(numPoints, NDIM));
  std::vector<ptsnD>* gridPoints;
  kernel_4d_test* ker = new kernel_4d_test();
  ker->get_points(gridPoints);
  Reader r(x_path);
  Vec x{Index(N)};
  r.get_array(x.data(), N);
  kernel_function<kernel_4d_test>* kf = new kernel_function<kernel_4d_test>(ker);
  std::vector<size_t> all(N);
  for (size_t i = 0; i < N; i++) all[i] = i;
  std::vector<double> dense(N);
  for (size_t i = 0; i < N; i++) dense[i] = kf->getRow(int(i), all).dot(x);
  Eigen::VectorXd X(NDIM), Y(NDIM);
  for (int i = 0; i < NDIM; ++i) {
    X(i) = -1;
    Y(i) = 1;
  }
  HODLRdD_matrix<kernel_4d_test> Kmat(ker, gridPoints, X, Y);
  Kmat.Assemble_matrix_operators();
  Vec y = Kmat * x;
  Writer w(out_path);
  w.f64("dense", dense);
  w.f64("hodlr", from_vec(y));
  w.f64("kii", {ker->getMatrixEntry(0, 0)});
  std::vector<double> p;
  for (size_t i = 0; i < N; i++)
    for (int k = 0; k < NDIM; k++) p.push_back((*gridPoints)[i].x[k]);
  w.f64("points", p);
  return 0;
}
#endif

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: ref_driver hodlr|gmres <in> <out> | golden4d <x.bin> <out>\n");
    return 2;
  }
  try {
    std::string mode = argv[1];
    if (mode == "hodlr" && argc >= 4) return mode_hodlr(argv[2], argv[3]);
    if (mode == "gmres" && argc >= 4) return mode_gmres(argv[2], argv[3]);
#ifdef REF_WITH_USER_KERNELS
    if (mode == "golden4d" && argc >= 4) return mode_golden4d(argv[2], argv[3]);
#endif
  } catch (const std::exception& e) {
    std::fprintf(stderr, "ref_driver: %s\n", e.what());
    return 1;
  }
  std::fprintf(stderr, "ref_driver: bad arguments\n");
  return 2;
}
