/*
 * hodlrnd.h -- C ABI of the GB300 HODLRnD engine (libhodlrnd_gb300.so).
 *
 * The reference (HODLRnD) is a header-only C++ template library whose hot
 * path is: 2^d-tree clustering -> ACA compression of every admissible block
 * -> HODLR matvec -> restarted GMRES.  It has no binary interface; its users
 * call the class HODLRdD_matrix<Kernel>.  This header is the drop-in
 * boundary for that path: plain C types, host or device pointers and sizes,
 * status codes.  Each entry point names the reference interface it replaces
 * (paths relative to the HODLRnD project root).
 *
 * Conventions
 *  - Every function returns HODLR_OK (0) or a HODLR_ERR_* code; the message
 *    of the last failure is returned by hodlr_last_error().
 *  - Points are passed as n x ndim row-major doubles (the x[] field of the
 *    reference's ptsnD, include/points_dt.hpp:9-13).  Vectors are in the
 *    caller's point order; several right-hand sides are n x nrhs column-major.
 *  - The engine copies what it needs to the device and owns that memory until
 *    the matching *_destroy call.  Host buffers stay owned by the caller.
 *  - A context and the operators built from it must be used from one host
 *    thread at a time (the reference is single-threaded too).
 */
#ifndef HODLRND_H
#define HODLRND_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define HODLR_OK 0
#define HODLR_ERR_INVALID 1       /* bad argument */
#define HODLR_ERR_CUDA 2          /* a CUDA runtime call failed */
#define HODLR_ERR_OOM 3           /* device allocation failed */
#define HODLR_ERR_BUDGET 4        /* device_budget_bytes would be exceeded */
#define HODLR_ERR_NOT_CONVERGED 5 /* GMRES stopped at max_iter (result still written) */
#define HODLR_ERR_TREE 6          /* tree would exceed the node limit (degenerate input) */
#define HODLR_ERR_STATE 7         /* call out of order (e.g. matvec before build) */
#define HODLR_ERR_DEVICE 8        /* a device-side check failed (index or size out of range), or a
                                     streaming kernel gave up waiting (2 s) for its bulk copies.  The
                                     give-up count is kept per device: after one, the next matvec or
                                     solve of every operator on that device reports this code once */
#define HODLR_ERR_IO 9            /* a file could not be read or written, or is malformed */
#define HODLR_ERR_TIMEOUT 10      /* hodlr_server_wait: the request has not finished within the timeout */

/* ---- kernels --------------------------------------------------------- */
/* Entry A_ij for i != j with r = |x_i - x_j| (Euclidean, include/points_dt.hpp:31-39);
 * A_ii = diag.  These cover the reference's test kernels
 * (include/user_kernel.hpp:46-49,101-104,167-170) and the benchmark kernels. */
#define HODLR_KERNEL_INV_R 1     /* scale / r          */
#define HODLR_KERNEL_INV_R2 2    /* scale / r^2        */
#define HODLR_KERNEL_LOG_R 3     /* scale * log(r)     */
#define HODLR_KERNEL_EXP_NEG_R 4 /* scale * exp(-r)    */

typedef struct hodlr_kernel_desc {
  int32_t kind; /* HODLR_KERNEL_* */
  int32_t reserved;
  double scale;
  double diag;
} hodlr_kernel_desc;

/* ---- precision of the stored far-field factors ------------------------ */
#define HODLR_PREC_FP64 0  /* everything FP64 (the reference's arithmetic, include/myHeaders.hpp:66-72) */
#define HODLR_PREC_MIXED 1 /* far-field U, V in FP32; FP64 near field; solve = FP64 iterative
                              refinement around an FP32 inner GMRES */
#define HODLR_PREC_BF16_FACTORS 3 /* far-field U, V and dense far blocks in BF16 with one FP32 scale per
                                     column of U and V (folded into z) or per row of a dense block; products
                                     summed in FP32; FP64 near field; FP64 GMRES.  For loose eps_aca
                                     (about 1e-4): BF16 keeps 8 significant bits. */
#define HODLR_PREC_FP32_FACTORS 2 /* far-field U, V in FP32, every product accumulated in compensated
                                     FP32 (FP64-level accuracy); FP64 near field; FP64 GMRES as the
                                     reference's solve, on the FP32-stored operator */

/* ---- parameters -------------------------------------------------------- */
typedef struct hodlr_params {
  int32_t ndim;      /* NDIM (include/myHeaders.hpp:35), 1..8 */
  int32_t nmax;      /* Nmax (include/myHeaders.hpp:36): split while a node holds more points */
  int32_t dprime;    /* INTERACTION_TYPE_ALLOWED = d' (include/myHeaders.hpp:39), -1..ndim-1 */
  int32_t restart;   /* GMRES restart length; the reference uses 100 (include/HDD_matrix.hpp:54) */
  double eps_aca;    /* eps_ACA (include/myHeaders.hpp:47) */
  double tol;        /* GMRES relative-residual tolerance; <= 0 selects eps_aca (HDD_matrix.hpp:54) */
  int64_t max_iter;  /* GMRES iteration limit; <= 0 selects N (HDD_matrix.hpp:54) */
  int32_t precision; /* HODLR_PREC_* */
  int32_t device;    /* CUDA device ordinal */
  uint64_t device_budget_bytes; /* refuse a build whose device footprint would exceed this; 0 = no limit */
  int32_t rank_cap;  /* initial ACA workspace columns per block (0 = default); grown on demand */
  int32_t max_outer; /* MIXED: iterative-refinement sweeps (0 = default 10) */
  double inner_tol;  /* MIXED: relative-residual target of each FP32 inner GMRES (<= 0: default 1e-4) */
  int32_t ortho;     /* GMRES orthogonalisation, HODLR_ORTHO_* */
  int32_t relax;     /* FP32_FACTORS, BF16_FACTORS: HODLR_RELAX_AUTO, _OFF or _ALWAYS */
  double relax_below; /* FP32_FACTORS, BF16_FACTORS: relative residual estimate below which products
                         are relaxed (<= 0: the default -- from the first iteration when the FP64
                         check is on, tol * 1e5 when it is off) */
  int32_t fp64_check; /* FP32_FACTORS, BF16_FACTORS, MIXED: HODLR_FP64_CHECK_AUTO (on) or _OFF */
  int32_t aca_workspace_mib; /* FP64 workspace of one ACA launch, MiB (0: a quarter of the free device
                                memory, 4 to 64 GiB); blocks beyond it go to further launches.  Freed
                                when the build returns.  No counterpart in the reference. */
  double stored_margin; /* with the FP64 check off: a solve ends when the true residual with the stored
                           operator is at most tol * stored_margin (<= 0: 1) */
} hodlr_params;

/* FP32_FACTORS and BF16_FACTORS solves: once GMRES's residual estimate is
 * below relax_below, the matvecs sum the products in plain FP32 (about 1e-6
 * relative, which an inexact Krylov method tolerates at that residual)
 * instead of compensated FP32; the solve ends only when the true residual,
 * with compensated products, is at most tol (GMRES continues from x
 * otherwise).  HODLR_RELAX_OFF: compensated products throughout.
 * HODLR_RELAX_ALWAYS: plain FP32 sums for every product (matvecs, solves and
 * the true residual) -- FP32 accumulation, for loose tolerances (>= ~1e-5). */
#define HODLR_RELAX_AUTO 0
#define HODLR_RELAX_OFF 1
#define HODLR_RELAX_ALWAYS 2

/* Reduced-precision operators (FP32_FACTORS, BF16_FACTORS, MIXED) store
 * rounded far-field factors; rounding moves the stored operator away from the
 * FP64 one (about 1e-8 relative for FP32 factors at eps_aca 1e-8 and
 * N = 262144, about 1e-3 for BF16), so a stored-operator residual of tol says
 * little about the FP64 operator's.  With the FP64 check (the default) the
 * build also keeps the FP64 far factors (their bytes count in device_bytes),
 * and a solve is FP64 iterative refinement: GMRES on the stored operator,
 * then residuals b - A x with the FP64 operator, each followed by a stored-
 * operator GMRES solve of the correction, until the FP64 operator's residual
 * is at most tol.  HODLR_FP64_CHECK_OFF keeps only the stored factors and
 * ends on the stored operator's residual (see stored_margin). */
#define HODLR_FP64_CHECK_AUTO 0
#define HODLR_FP64_CHECK_OFF 1

/* GMRES orthogonalisation.  MGS is the reference's (include/GMRES.hpp:236-240)
 * and needs i + 2 kernel launches at Arnoldi step i; CGS2 (classical
 * Gram-Schmidt applied twice) needs six at any step and is as orthogonal.
 * AUTO: MGS for HODLR_PREC_FP64 (the reference's arithmetic), CGS2 otherwise. */
#define HODLR_ORTHO_AUTO 0
#define HODLR_ORTHO_MGS 1
#define HODLR_ORTHO_CGS2 2

/* Fill p with the reference's defaults: ndim 2, Nmax 64, d' 0, eps 1e-10,
 * restart 100, tol = eps, max_iter = N, FP64.  No counterpart in the
 * reference (its defaults are the constants in include/myHeaders.hpp:35-49). */
void hodlr_params_default(hodlr_params* p);

typedef struct hodlr_ctx hodlr_ctx;
typedef struct hodlr_op hodlr_op;

/* Create a context on params->device.  Replaces editing the compile-time
 * constants of include/myHeaders.hpp:32-49. */
int hodlr_ctx_create(const hodlr_params* params, hodlr_ctx** out);
int hodlr_ctx_destroy(hodlr_ctx* ctx);

/* Message of the last failure on this context (or, with ctx == NULL, of the
 * last failure on the calling thread).  Never NULL. */
const char* hodlr_last_error(const hodlr_ctx* ctx);

/* Build the operator: tree and interaction lists (HODLRdD_matrix ctor,
 * include/HDD_matrix.hpp:20-33 -> Tree::Tree, include/HDD_tree.hpp:23-74)
 * followed by Assemble_matrix_operators (include/HDD_matrix.hpp:39-41 ->
 * Tree::Initialise_tree / Node::Initialize_node, include/HDD_node.hpp:118-148):
 * ACA of every admissible block and the dense leaf blocks.
 * points: host, n x ndim row-major; box_lo/box_hi: host, ndim each (the
 * bounding box the reference takes as x1, x2). */
int hodlr_build(hodlr_ctx* ctx, const double* points, int64_t n, const double* box_lo, const double* box_hi,
                const hodlr_kernel_desc* kernel, hodlr_op** out);
int hodlr_op_destroy(hodlr_op* op);

/* Operator files.  hodlr_op_save writes the operator built from `points`
 * (the caller-order n x ndim array given to hodlr_build) with its parameters,
 * kernel, box, block ranks and compressed far field; hodlr_op_load rebuilds
 * the tree, lists and near field from the points and takes the far field from
 * the file (no ACA), on ctx's device.  Matvecs and solves of the loaded
 * operator equal the saved one's bit for bit.  Malformed files give
 * HODLR_ERR_IO.  No counterpart in the reference (it keeps no operator
 * beyond its process). */
int hodlr_op_save(const hodlr_op* op, const double* points, const char* path);
int hodlr_op_load(hodlr_ctx* ctx, const char* path, hodlr_op** out);

/* y = A x (HODLRdD_matrix::operator*, include/HDD_matrix.hpp:43-47).  Host
 * pointers, n x nrhs column-major, caller's point order. */
int hodlr_matvec(hodlr_op* op, const double* x, double* y, int64_t nrhs);

/* Same with device pointers on the given cudaStream_t (NULL = the legacy
 * default stream).  Asynchronous: returns once the work is queued. */
int hodlr_matvec_device(hodlr_op* op, const double* d_x, double* d_y, int64_t nrhs, void* stream);

typedef struct hodlr_solve_info {
  int64_t iterations;       /* total inner GMRES iterations (the reference's return value, GMRES.hpp:267,294,302) */
  int64_t outer_iterations; /* iterative-refinement sweeps (1 for FP64) */
  double rel_residual;      /* |b - A x| / |b| in FP64, with the FP64 operator (FP64, or reduced precision
                               with the FP64 check), else with the stored operator */
  int32_t converged;         /* rel_residual <= stop_tol */
  int32_t reserved;
  double seconds;
  double stop_tol;          /* the residual the solve had to reach (tol, or tol * stored_margin) */
  double rel_residual_stored; /* reduced precision: |b - A x| / |b| with the stored operator */
} hodlr_solve_info;

/* Solve A x = b (HODLRdD_matrix::solve, include/HDD_matrix.hpp:51-62 ->
 * iterSolver::GMRES, include/GMRES.hpp:160-305).  FP64: restarted GMRES with
 * x0 = b, as the reference.  MIXED: FP64 iterative refinement whose inner
 * solves are FP32 GMRES on the FP32-factor operator.  Host pointers. */
int hodlr_solve(hodlr_op* op, const double* b, double* x, int64_t nrhs, hodlr_solve_info* info);

/* Same with device pointers; synchronous with respect to the given stream. */
int hodlr_solve_device(hodlr_op* op, const double* d_b, double* d_x, int64_t nrhs, void* stream,
                       hodlr_solve_info* info);

/* Solver settings of an existing operator, as iterSolver takes them per solve
 * (restart, max_iter, tol: include/GMRES.hpp:56-63); restart/tol/max_iter
 * <= 0 select 100 / eps_aca / N, inner_tol and max_outer <= 0 the defaults. */
int hodlr_set_solver(hodlr_op* op, int32_t restart, double tol, int64_t max_iter, double inner_tol,
                     int32_t max_outer);
/* Relaxed-product settings (relax, relax_below of hodlr_params) for later
 * solves of an FP32_FACTORS operator.  No counterpart in the reference. */
int hodlr_set_relax(hodlr_op* op, int32_t relax, double relax_below);

typedef struct hodlr_stats {
  int64_t n, depth, n_leaves, n_far_blocks, n_dense_far_blocks, n_near_blocks, max_rank;
  double n_flop;            /* Node::compute_flop_count summed (include/HDD_node.hpp:182-202) */
  double memory_gb;         /* 8e-9 * n_flop, as print_matrix_statistics (include/HDD_matrix.hpp:69-85) */
  double compression_ratio; /* n_flop / N^2 */
  uint64_t near_bytes;      /* stored dense leaf blocks */
  uint64_t far_bytes;       /* stored far-field factors and dense far blocks */
  uint64_t device_bytes;    /* everything the operator holds on the device */
  double t_tree_s, t_aca_s, t_near_s, t_build_s, t_matvec_s;
  double far_entries;       /* sum over low-rank blocks of r (m + n) */
  double dense_far_entries; /* sum over dense far blocks of m n */
  double near_entries;      /* sum over near blocks of m n */
  double t_aca_kernel_s;    /* device time of the ACA launches (inside t_aca_s) */
  double t_compact_s;       /* device time of the factor compaction launches (inside t_aca_s) */
  double aca_entries;       /* kernel entries the ACA generated: sum over blocks of (r + 1)(m + n) */
} hodlr_stats;

/* print_matrix_statistics figures (include/HDD_matrix.hpp:69-85) plus byte counts. */
int hodlr_stats_get(const hodlr_op* op, hodlr_stats* out);

/* Leaf-order permutation: perm[k] = caller index of the k-th point in tree
 * order (the concatenated index_of_points of the leaves, HDD_clusters.hpp:26). */
int hodlr_get_permutation(const hodlr_op* op, int64_t* perm);

/* Far blocks in the reference's assembly order (level, target node, partner
 * in interaction-list order; include/HDD_tree.hpp:76-83, HDD_node.hpp:126-130).
 * Arrays of length n_far_blocks; rank is the reference's rank() (min(m,n)
 * for a block kept dense, LowRank_matrix.hpp:348-363). */
int hodlr_get_blocks(const hodlr_op* op, int32_t* level, int64_t* target, int64_t* source, int32_t* rank);

/* Factors of far block b (order of hodlr_get_blocks), converted to FP64:
 * U (m x rank) and V (n x rank) column major with A_b ~ U V^T, the L and R of
 * LowRankMat (include/LowRank_matrix.hpp:10,61); for a block kept dense
 * (*dense = 1) U receives the m x n block and V is not written.  m and n are
 * the point counts of the target and source nodes; pass NULL to only query. */
int hodlr_get_block(const hodlr_op* op, int64_t b, int32_t* m, int32_t* n, int32_t* rank, int32_t* dense, double* U,
                    double* V);

/* ---- tracing ------------------------------------------------------------
 * CUDA events around every kernel launch that applies the operator, so that
 * a caller can relate device time to the algorithmic bytes each launch must
 * move.  No counterpart in the reference, which only times whole phases with
 * omp_get_wtime (include/HDD_tree.hpp:77-81,95-99). */
#define HODLR_TRACE_KINDS 16
#define HODLR_TRACE_ZGEMV_FP64 0   /* z = V^T x, FP64 vectors (FP64 factors, or FP32 factors with
                                      compensated accumulation) */
#define HODLR_TRACE_NEAR_FP64 1    /* near-field leaf panels, FP64 vectors */
#define HODLR_TRACE_FAR_FP64 2     /* far-field panels (U z and dense far blocks), FP64 vectors */
#define HODLR_TRACE_COMBINE_FP64 3 /* sum of the per-level output slots */
#define HODLR_TRACE_ZGEMV_FP32 4   /* the same four for FP32 vectors (inner solve of HODLR_PREC_MIXED) */
#define HODLR_TRACE_NEAR_FP32 5
#define HODLR_TRACE_FAR_FP32 6
#define HODLR_TRACE_COMBINE_FP32 7
#define HODLR_TRACE_ZGEMV_REF 8    /* the same four for the FP64 operator kept by reduced-precision
                                      operators (the refinement residuals of the FP64 check) */
#define HODLR_TRACE_NEAR_REF 9
#define HODLR_TRACE_FAR_REF 10
#define HODLR_TRACE_COMBINE_REF 11

typedef struct hodlr_trace {
  uint64_t launches[HODLR_TRACE_KINDS];
  double total_ms[HODLR_TRACE_KINDS];         /* summed CUDA-event durations */
  double bytes_per_launch[HODLR_TRACE_KINDS]; /* algorithmic bytes one launch must move */
} hodlr_trace;

/* Enable (on != 0) or disable tracing; enabling clears the counters. */
int hodlr_trace_enable(hodlr_op* op, int on);
/* Wait for the traced launches and return the accumulated figures. */
int hodlr_trace_get(hodlr_op* op, hodlr_trace* out);
/* Number of kernels this library has launched in the process so far. */
uint64_t hodlr_kernel_launches(void);

/* ---- one block, no allocation -------------------------------------------
 * No counterpart in the reference.  For callers that cannot call cudaMalloc
 * where they need a block compressed (a framework that owns all device memory
 * through its own pool, a loop that cannot afford cudaMalloc's implicit
 * synchronisation): partially pivoted ACA of the single block
 * A(rows, cols), with the same kernel, pivoting, restarts and stopping rule as
 * hodlr_build, and with its bookkeeping in a fixed static device array (about
 * 136 KB per GPU, held until the process exits) instead of allocated memory.
 *  d_points  device, ndim x ld doubles, coordinate k of point i at k*ld + i
 *  d_rows    device, m point indices (the block's rows, in the order the ACA
 *            walks them; the reference walks a node's points by increasing index)
 *  d_cols    device, n point indices (columns)
 *  seed      the restart heuristic's random stream (hodlr_build seeds each
 *            block from its level, target and source node)
 *  cap       columns available in d_factors, at most HODLR_NOALLOC_MAX_RANK
 *  d_factors device, (m + n) * cap doubles: U (m x cap) then V (n x cap),
 *            column major; the first *rank columns hold U and V with A ~ U V^T
 *  *rank, *flags  on return (host): flags bit 0 = the block is to be kept dense
 *            (rank reached min(m,n) - 1; the factors are then not a
 *            representation), bit 1 = cap columns were not enough.
 * m and n above HODLR_NOALLOC_MAX_POINTS, or cap above HODLR_NOALLOC_MAX_RANK,
 * are rejected with HODLR_ERR_INVALID.  Every index in d_rows and d_cols must
 * be below ld (they address d_points; the device does not check them).  The
 * first call on a device (and the first after that device's context was
 * reset) looks the static array up with cudaGetSymbolAddress; that call should
 * come before any stream capture on the device.  All calls share the array:
 * calls whose GPU work overlaps (other streams or threads) race and must be
 * serialised.  Every call waits for its result: it synchronises `stream` and
 * copies the rank and flags back to the host. */
#define HODLR_NOALLOC_MAX_POINTS 16384
#define HODLR_NOALLOC_MAX_RANK 512
int hodlr_aca_block_noalloc(const double* d_points, int64_t ld, int32_t ndim, const int32_t* d_rows, int32_t m,
                            const int32_t* d_cols, int32_t n, const hodlr_kernel_desc* kernel, double eps_aca,
                            uint64_t seed, int32_t cap, double* d_factors, int32_t* rank, int32_t* flags,
                            void* stream);

/* Y = A X for several right-hand sides on the tensor cores: an operator with
 * BF16 far-field factors (HODLR_PREC_BF16_FACTORS), X and Y device arrays of
 * n x nrhs FP32, column major, caller's point order.  Blocks of 64 columns
 * go through tcgen05 MMAs (BF16 operands, FP32 accumulation in tensor
 * memory): every right-hand side split once into BF16 high and low parts (to
 * about 2^-17 relative), each BF16 factor entry times its input scale in two
 * BF16 terms, the FP64 near field in three -- the product differs from the
 * stored operator's single-RHS product by about 1e-5 relative, far below the
 * BF16 storage itself (about 1e-3).  The first call builds the tensor-core
 * plan and buffers (about (n + sum of ranks) x 256 bytes).  Synchronises
 * `stream`.  Replaces the mat-mat use of HODLRdD_matrix::operator*
 * (include/HDD_matrix.hpp:42-47). */
int hodlr_matvec_tc_device(hodlr_op* op, const float* d_x, float* d_y, int64_t nrhs, void* stream);

/* ---- tensor cores ---------------------------------------------------------
 * Self-test of the fifth-generation tensor-core path (tcgen05) the multi-RHS
 * products use: D = A B^T with A (128 x k) and B (n x k) BF16, row major,
 * given as their 16-bit patterns, D (128 x n) FP32 row major, accumulated in
 * tensor memory.  n a multiple of 16 in 16..256, k a multiple of 16 in 16..128.
 * Host pointers; synchronous.  No counterpart in the reference. */
int hodlr_tc_selftest(const uint16_t* A, const uint16_t* B, int32_t n, int32_t k, float* D);

/* ---- batches of independent operators ---------------------------------- */
/* No counterpart in the reference (one HODLRdD_matrix per caller,
 * include/HDD_matrix.hpp:20-62).  count operators built on ctx's parameters,
 * instance i from points[i] (n[i] x ndim, row major), box box_lo/hi +
 * i*ndim and kernels[i] (one kind and diagonal for all, scales may differ).
 * The far blocks of every instance are compressed together (they share each
 * ACA launch); each instance keeps its own storage and is an ordinary
 * operator (hodlr_batch_op: solve, matvec, statistics; owned by the batch).
 * The batch also holds one merged plan over all instances. */
typedef struct hodlr_batch hodlr_batch;
int hodlr_build_batch(hodlr_ctx* ctx, int32_t count, const double* const* points, const int64_t* n,
                      const double* box_lo, const double* box_hi, const hodlr_kernel_desc* kernels,
                      hodlr_batch** out);
/* offsets[0..count]: instance i occupies rows offsets[i] .. offsets[i+1]-1 of a batch vector. */
int hodlr_batch_offsets(const hodlr_batch* batch, int64_t* offsets);
int hodlr_batch_op(hodlr_batch* batch, int32_t i, hodlr_op** op);
/* Y = A X for every instance at once: X and Y are device arrays of
 * offsets[count] x nrhs (column major, each instance's rows in its caller's
 * order) of FP32 for HODLR_PREC_MIXED, FP64 otherwise.  Every column of every
 * instance is one launch per phase of the merged plan; the whole sequence is
 * captured as a CUDA graph on the first call with these (X, Y, nrhs) and
 * replayed on `stream` afterwards.  Asynchronous. */
int hodlr_batch_matvec_device(hodlr_batch* batch, const void* d_x, void* d_y, int64_t nrhs, void* stream);
int hodlr_batch_destroy(hodlr_batch* batch);

/* ---- request loop (serving) --------------------------------------------- */
/* No counterpart in the reference, which builds and solves one
 * HODLRdD_matrix at a time in its caller (include/HDD_matrix.hpp:20-62).
 *
 * A server owns `slots` worker threads.  Requests (a geometry -- points, box,
 * kernel, parameters -- and nrhs right-hand sides) are queued by
 * hodlr_server_submit, which copies every input and returns at once.  A
 * worker admits the first queued request whose predicted device bytes
 * (hodlr_predict_bytes, corrected by what earlier builds measured) fit in
 * memory_budget_bytes next to the resident geometries and the other running
 * requests, evicting idle resident geometries least recently used first.
 * Each geometry has its own CUDA stream, so running requests overlap on the
 * device.  A request with a nonzero geometry_key keeps its operator resident
 * after it finishes; a later request with the same key may pass points =
 * NULL and is solved on the resident operator (requests on one operator run
 * one at a time).  Results are bit-identical to solving the same request
 * alone: every kernel is deterministic and no work is shared between
 * requests.
 *
 * simulate = 1 runs the same admission and scheduling without a GPU (builds
 * and solves take a nominal time, x = b); it exists for capacity planning and
 * for testing the scheduler. */
typedef struct hodlr_server hodlr_server;

typedef struct hodlr_server_params {
  int32_t device;               /* CUDA device of every geometry */
  int32_t slots;                /* requests running at once (worker threads); 0 = 4 */
  uint64_t memory_budget_bytes; /* device bytes for resident and running geometries; 0 = 150 GiB */
  int32_t simulate;             /* 1: no GPU work (see above) */
  int32_t reserved;
} hodlr_server_params;

typedef struct hodlr_request {
  uint64_t geometry_key;     /* 0: do not keep the operator resident */
  hodlr_params params;       /* per-request parameters (params.device is ignored) */
  hodlr_kernel_desc kernel;
  const double* points;      /* n x ndim, row major; NULL to reuse the resident geometry_key */
  const double* box_lo;      /* ndim each; may be NULL with points == NULL */
  const double* box_hi;
  int64_t n;
  const double* b;           /* n x nrhs, column major, caller's point order */
  int64_t nrhs;
} hodlr_request;

typedef struct hodlr_result {
  int32_t status;            /* HODLR_OK, HODLR_ERR_NOT_CONVERGED, or the failure */
  int32_t built;             /* 1: this request built its operator; 0: it was resident */
  int64_t iterations;        /* GMRES iterations summed over the right-hand sides */
  double rel_residual;       /* worst over the right-hand sides */
  double t_queue_s;          /* submit -> admission */
  double t_build_s;          /* operator build (0 when resident) */
  double t_solve_s;          /* all right-hand sides, host copies included */
  double t_total_s;          /* submit -> completion */
  uint64_t predicted_bytes;  /* predicted footprint of the operator it built (0 when resident) */
  uint64_t actual_bytes;     /* the operator's device footprint */
  uint64_t predicted_build_bytes; /* transient build workspace reserved at admission beside it */
  double t_device_start_s;   /* the request's GPU work: first and last event on its geometry's stream, */
  double t_device_end_s;     /* seconds from the server's creation (0 with simulate) */
  char message[128];         /* failure message, empty on success */
} hodlr_result;

typedef struct hodlr_server_stats {
  uint64_t submitted, completed, rejected, builds, resident_hits, evictions, rhs_solved;
  int64_t queued, running, resident;
  uint64_t used_bytes;
} hodlr_server_stats;

int hodlr_server_create(const hodlr_server_params* params, hodlr_server** out);
int hodlr_server_submit(hodlr_server* server, const hodlr_request* request, uint64_t* ticket);
/* Waits up to timeout_s (< 0: no limit) for the request; on completion writes
 * x (n x nrhs, caller's order; may be NULL) and *result (may be NULL), forgets
 * the ticket and returns result->status.  HODLR_ERR_TIMEOUT if still running. */
int hodlr_server_wait(hodlr_server* server, uint64_t ticket, double timeout_s, double* x, hodlr_result* result);
int hodlr_server_stats_get(hodlr_server* server, hodlr_server_stats* out);
/* Finishes every submitted request, then frees the resident geometries. */
int hodlr_server_destroy(hodlr_server* server);

/* Predicted device bytes of hodlr_build + solves for these inputs: tree,
 * lists and near field exactly; far-block ranks from a prior model of rank
 * versus eps_aca, ndim and block size; plus the build's ACA workspace.  Host
 * only.  No counterpart in the reference (its print_matrix_statistics reports
 * the memory after the build, include/HDD_matrix.hpp:69-85). */
int hodlr_predict_bytes(const hodlr_params* params, const double* points, int64_t n, const double* box_lo,
                        const double* box_hi, uint64_t* bytes);

/* ---- vector files (host only) ------------------------------------------ */
/* storedata::load_vec / save_vec (include/myHeaders.hpp:146-170): a cereal
 * PortableBinary archive of one std::vector<double> -- a 1-byte endianness tag
 * (1 = little endian), a u64 element count, the float64 values -- read and
 * written without cereal.  hodlr_vec_load with x == NULL only stores the count
 * in *n; otherwise it fails with HODLR_ERR_INVALID when the file holds more
 * than cap values.  Both byte orders are read; files are written little endian.
 * Malformed files give HODLR_ERR_IO.  Errors: hodlr_last_error(NULL). */
int hodlr_vec_load(const char* path, double* x, int64_t cap, int64_t* n);
int hodlr_vec_save(const char* path, const double* x, int64_t n);

/* ---- host-only tree planning (no device needed) ------------------------ */
typedef struct hodlr_tree hodlr_tree;

/* Tree and lists only (include/HDD_tree.hpp:23-74, include/HDD_node.hpp:150-180). */
int hodlr_tree_build(const hodlr_params* params, const double* points, int64_t n, const double* box_lo,
                     const double* box_hi, hodlr_tree** out);
/* The same tree and lists built on the GPU params->device (what hodlr_build
 * uses): the points' stable partition among the children, the child boxes and
 * the admissibility tests run on the device with the host's rounding, so the
 * arrays equal hodlr_tree_build's bit for bit.  Errors: hodlr_last_error(NULL). */
int hodlr_tree_build_device(const hodlr_params* params, const double* points, int64_t n, const double* box_lo,
                            const double* box_hi, hodlr_tree** out);
/* sizes[0..5] = levels, nodes (all levels), neighbour entries, interaction entries,
 * far blocks (both nodes non-empty), near blocks (self + non-empty neighbours of non-empty leaves) */
int hodlr_tree_sizes(const hodlr_tree* tree, int64_t* sizes);
/* Node arrays run over all levels, level by level, nodes in reference order
 * (child c of node k is node k*2^ndim + c of the next level). */
int hodlr_tree_get(const hodlr_tree* tree, int64_t* level_sizes, int64_t* node_counts, int64_t* nbr_ptr,
                   int64_t* nbr, int64_t* intr_ptr, int64_t* intr, int64_t* leaf_perm);
int hodlr_tree_destroy(hodlr_tree* tree);

#ifdef __cplusplus
}
#endif
#endif /* HODLRND_H */
