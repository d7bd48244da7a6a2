/*
 * tapkee_gb300.h -- C ABI of the GB300 local-neighborhood operator.
 *
 * This library computes, on one GB300 GPU (sm_103a), the stage that the
 * reference (lisitsyn/tapkee 1.3.4) runs inside
 *   tapkee::with((method=KernelLocallyLinearEmbedding | KernelLocalTangentSpaceAlignment,
 *                 neighbors_method=Brute, num_neighbors=k, klle_shift=s)).embedUsing(X)
 * before its eigensolver: brute-force kNN under the linear kernel, the
 * connectivity check with its 2k retry, LLE reconstruction weights or LTSA
 * tangent bases, and the sparse alignment matrix M in CSR form.
 *
 * Conventions
 *   - X is points-major: point i occupies X[i*ldx .. i*ldx + D), which is the
 *     memory layout of the reference's D x N column-major DenseMatrix
 *     (defines/types.hpp:23). dtype is TK_F32 or TK_F64.
 *   - Every buffer is caller-owned. Pointers may be host memory (pageable or
 *     pinned) or device memory of the context's GPU; the library detects which.
 *   - Indices are int32 (the reference's IndexType, defines/types.hpp:19);
 *     CSR row pointers are int64, columns int32, values double.
 *   - No C++ exception crosses this boundary: every call returns a tk_status.
 *     tk_last_error() gives the message of the last failing call on a context.
 *   - One tk_ctx owns one CUDA stream and its scratch memory. Calls on one
 *     context are serialised by the caller; different contexts are independent.
 */
#ifndef TAPKEE_GB300_H
#define TAPKEE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. The C++ facade maps them onto the reference's exception types
 * (exceptions.hpp:14-91). */
typedef enum tk_status
{
    TK_OK = 0,
    TK_ERR_INVALID_ARG = 1,      /* wrong_parameter_error                          */
    TK_ERR_NO_DATA = 2,          /* no_data_error (N == 0)                         */
    TK_ERR_OOM = 3,              /* not_enough_memory_error                        */
    TK_ERR_CUDA = 4,             /* a CUDA runtime call failed                     */
    TK_ERR_TIMEOUT = 5,          /* a bounded device-side wait gave up             */
    TK_ERR_CANCELLED = 6,        /* cancelled_exception (cancel_function true)     */
    TK_ERR_BUFFER_TOO_SMALL = 7, /* output capacity below the required size       */
    TK_ERR_UNSUPPORTED = 8,      /* unsupported_method_error                       */
    TK_ERR_NO_DEVICE = 9,        /* no usable sm_103a device                       */
    TK_ERR_INTERNAL = 10,        /* an internal consistency check failed           */
    TK_ERR_NOT_CONVERGED = 11    /* eigendecomposition_error (the eigensolver did
                                    not reach its tolerance)                       */
} tk_status;

typedef enum tk_dtype
{
    TK_F32 = 0,
    TK_F64 = 1
} tk_dtype;

/* Method tags (defines/methods.hpp:74,82,90). */
typedef enum tk_method
{
    TK_METHOD_KLLE = 0,  /* KernelLocallyLinearEmbedding            */
    TK_METHOD_KLTSA = 1, /* KernelLocalTangentSpaceAlignment         */
    TK_METHOD_HLLE = 2   /* HessianLocallyLinearEmbedding           */
} tk_method;

/* Distance screening engine of the brute kNN. Both are followed by the same
 * exact FP64 re-rank and certification, so they return identical neighbours. */
typedef enum tk_screen
{
    TK_SCREEN_TENSOR = 0, /* tcgen05 tensor-core fp16 split GEMM (default) */
    TK_SCREEN_FP32 = 1    /* plain FP32 CUDA-core GEMM                     */
} tk_screen;

/* Log levels, mirroring utils/logging.hpp:89-144. */
typedef enum tk_log_level
{
    TK_LOG_INFO = 0,
    TK_LOG_WARNING = 1,
    TK_LOG_DEBUG = 2,
    TK_LOG_ERROR = 3,
    TK_LOG_BENCHMARK = 4
} tk_log_level;

typedef void (*tk_log_fn)(int level, const char* message, void* user);

typedef struct tk_ctx tk_ctx;

/* Parameters of the stage; the defaults are the reference keyword defaults
 * (defines/keywords.hpp). */
typedef struct tk_params
{
    int method;             /* tk_method; required                             keywords.hpp:35  */
    int num_neighbors;      /* default 5, must lie in [3, N)                   keywords.hpp:112 */
    int target_dimension;   /* default 2, must lie in [1, N)                   keywords.hpp:125 */
    double klle_shift;      /* default 1e-3                                    keywords.hpp:248 */
    double nullspace_shift; /* default 1e-9                                    keywords.hpp:235 */
    int check_connectivity; /* default 1                                       keywords.hpp:272 */
    int screen;             /* tk_screen, default TK_SCREEN_TENSOR                              */
    int (*cancel_function)(void); /* polled between stages; NULL = never cancel              */
} tk_params;

/* Statistics of one brute kNN call. */
typedef struct tk_knn_stats
{
    int64_t rows_uncertified; /* rows whose screened candidate list could not be
                                 certified and were recomputed exactly          */
    int32_t candidates;       /* candidates kept per row by the screen          */
    int32_t screen;           /* engine used                                    */
    int64_t tie_rows;         /* rows whose k-th and (k+1)-th nearest distances
                                 lie within 1e-12 relative: their sets follow
                                 the reference's nth_element partition           */
    int64_t extra_rows;       /* rows for which the reference returns k + 1
                                 neighbours (see tk_knn_extra_rows)             */
} tk_knn_stats;

/* Summary of the operator held by a context after tk_local_operator(). */
typedef struct tk_operator_info
{
    int64_t n;                /* number of points                                   */
    int32_t k;                /* neighbours per point actually used (after the
                                 clamp to N-1 and any connectivity doublings)       */
    int32_t method;           /* tk_method                                          */
    int32_t target_dimension; /* td (LTSA basis width)                              */
    int32_t connectivity_retries; /* how many times k was doubled                   */
    int64_t nnz;              /* non-zeros of M                                     */
    int64_t rows_uncertified; /* see tk_knn_stats                                   */
    float stage_ms[6];        /* device time per stage: knn, connectivity, weights,
                                 assembly, total, and the distance-screen kernel
                                 alone (last kNN pass)                               */
    int64_t tie_rows;         /* see tk_knn_stats (last kNN pass)                   */
    int64_t extra_rows;       /* see tk_knn_stats (last kNN pass)                   */
    float kernel_ms[8];       /* device time per kernel group (CUDA events): point
                                 preparation, distance screen, re-rank (with the
                                 exact fallback and tie selection), all of the last
                                 kNN pass; weights; reverse lists, row pass and CSR
                                 write of assembly; connectivity checks (all passes) */
} tk_operator_info;

/* ---- context -------------------------------------------------------------- */

/* Fills p with the reference defaults (method = TK_METHOD_KLLE). */
void tk_params_default(tk_params* p);

/* Creates a context on `device`. `stream` is a cudaStream_t to run on, or NULL
 * for a context-owned non-blocking stream. Fails with TK_ERR_NO_DEVICE unless the
 * device is compute capability 10.3. */
int tk_ctx_create(int device, void* stream, tk_ctx** out);
int tk_ctx_destroy(tk_ctx* ctx);

/* Message of the last failing call on ctx (never NULL). */
const char* tk_last_error(const tk_ctx* ctx);
const char* tk_status_string(int status);

/* Installs a log sink (utils/logging.hpp:119-137, set_logger_impl); NULL restores
 * the default (warnings and errors to stderr). */
int tk_set_log_callback(tk_ctx* ctx, tk_log_fn fn, void* user);

/* Library version string ("major.minor.patch"). */
const char* tk_version(void);

/* Number of CUDA kernels this library has launched in this process (all
 * contexts); a diagnostic for profiling and benchmarks. */
long long tk_kernel_launch_count(void);

/* ---- stage entry points ----------------------------------------------------- */

/* Brute-force k nearest neighbours of every point under the kernel-trick
 * distance sqrt(k(x,x) - 2 k(x,y) + k(y,y)) with the linear kernel.
 * Replaces find_neighbors_bruteforce_impl (neighbors/neighbors.hpp:119-149) with
 * KernelDistance (neighbors/neighbors.hpp:40-55) over eigen_kernel_callback
 * (callbacks/eigen_callbacks.hpp:34-46).
 * idx_out (N x k) receives, per row, the reference's neighbour set: the k
 * nearest other points ordered by (distance, index). Where the k-th and
 * (k+1)-th nearest distances tie (within 1e-12 relative; stats->tie_rows), the
 * row instead holds the first k records of the first k + 1 that libstdc++'s
 * std::nth_element(begin, begin + k + 1, end) leaves over the row's N records in
 * index order, minus the point itself, in that partition order -- the
 * reference's selection (neighbors/neighbors.hpp:135-146, distances_comparator
 * :28-34). d2_out (N x k, optional) receives the FP64 squared distances.
 * Requires 1 <= k <= N-1. */
int tk_knn_brute(tk_ctx* ctx, const void* X, int dtype, int64_t N, int D, int64_t ldx, int k, int screen,
                 int32_t* idx_out, double* d2_out, tk_knn_stats* stats);

/* The rows of the last brute kNN pass on ctx (tk_knn_brute, or the final pass of
 * tk_local_operator) for which the reference returns k + 1 neighbours: the point
 * has k + 1 or more exact duplicates and the partition leaves it outside the
 * first k + 1 records (neighbors/neighbors.hpp:140-146 then keeps all k + 1).
 * The first k of them are in idx_out, which is what the reference's weight and
 * connectivity routines read (they take k from the first row's list:
 * routines/locally_linear.hpp:96, neighbors/connected.hpp:27). Writes up to
 * `capacity` (row, (k+1)-th neighbour) pairs into rows[] / extra[] (host
 * memory; either may be NULL) and *count = the number of such rows. */
int tk_knn_extra_rows(tk_ctx* ctx, int32_t* rows, int32_t* extra, int64_t capacity, int64_t* count);

/* Reachability of every vertex from vertex 0 along kNN out-edges.
 * Replaces is_connected (neighbors/connected.hpp:19-62). *connected = 1 or 0. */
int tk_check_connected(tk_ctx* ctx, int64_t N, int k, const int32_t* idx, int* connected);

/* LLE reconstruction weights: per point, C = Gram of (neighbours - x) plus
 * klle_shift * trace(C) * I, w = C^{-1} 1 / sum. W_out is N x k, aligned with idx.
 * Replaces the per-point solve of linear_weight_matrix
 * (routines/locally_linear.hpp:107-131). */
int tk_lle_weights(tk_ctx* ctx, const void* X, int dtype, int64_t N, int D, int64_t ldx, const int32_t* idx,
                   int k, double klle_shift, double* W_out);

/* Reverse-mode derivative of tk_lle_weights with the neighbour sets held fixed:
 * given the weights W (N x k, from tk_lle_weights on the same X, idx, klle_shift)
 * and an upstream gradient dW = dL/dW (N x k), writes dX_out = dL/dX (N x D FP64,
 * row stride D). Per point it solves (C + klle_shift tr(C) I) mu = dW_i - (dW_i.w_i) 1
 * with the forward's solver and scatters -mu_a p - w_a q - 2 klle_shift (mu.w) z_a
 * (p = sum w_b z_b, q = sum mu_b z_b, z_a = x_{n_a} - x_i) to the neighbours and its
 * negated sum to the point. No counterpart in the reference (which does not
 * differentiate); it is the adjoint of the solve in linear_weight_matrix
 * (routines/locally_linear.hpp:117-131). */
int tk_lle_weights_grad(tk_ctx* ctx, const void* X, int dtype, int64_t N, int D, int64_t ldx, const int32_t* idx,
                        int k, double klle_shift, const double* W, const double* dW, double* dX_out);

/* LTSA tangent basis: per point, the eigenvectors of the td largest eigenvalues
 * of the double-centred neighbour Gram. V_out is N x k x td (sign of each vector
 * is arbitrary); the alignment block is P = (1/k) 1 1^T + V V^T.
 * Replaces the per-point part of tangent_weight_matrix
 * (routines/locally_linear.hpp:45-63, with centerMatrix utils/matrix.hpp:12-19). */
int tk_ltsa_basis(tk_ctx* ctx, const void* X, int dtype, int64_t N, int D, int64_t ldx, const int32_t* idx,
                  int k, int td, double* V_out);

/* Hessian LLE basis: per point, the product columns Yr (k x dp, dp = td (td+1)/2)
 * of the orthonormalised [1, V, v_j v_l] built from the LTSA tangent basis V;
 * the point's Hessian block is B = Yr Yr^T. Y_out is N x k x dp. Replaces the
 * per-point part of hessian_weight_matrix (routines/locally_linear.hpp:183-234).
 * td must be 1 or 2 (the reference places the product columns correctly only
 * for those, :208-214) and k > td + dp. */
int tk_hessian_basis(tk_ctx* ctx, const void* X, int dtype, int64_t N, int D, int64_t ldx, const int32_t* idx,
                     int k, int td, double* Y_out);

/* Sparse alignment matrix M in CSR (= CSC, M is symmetric), duplicates summed:
 *   TK_METHOD_KLLE : M = (I - W)^T (I - W) + shift I   from weights = W (N x k)
 *                    (triplets of routines/locally_linear.hpp:133-146)
 *   TK_METHOD_KLTSA: M = shift I + sum_i S_i^T (I - P_i) S_i from weights = V
 *                    (N x k x td) (triplets of routines/locally_linear.hpp:65-77)
 *   TK_METHOD_HLLE : M = sum_i S_i^T B_i S_i, B_i = Y_i Y_i^T, from weights = Y
 *                    (N x k x td(td+1)/2, tk_hessian_basis); shift unused
 *                    (triplets of routines/locally_linear.hpp:236-243)
 * followed by sparse_matrix_from_triplets (utils/sparse.hpp:16-21).
 * Columns are ascending within each row. Two-phase: with col_idx == NULL the
 * call only writes row_ptr (if non-NULL) and *nnz_io = nnz; with buffers whose
 * capacity *nnz_io is below nnz it returns TK_ERR_BUFFER_TOO_SMALL and sets
 * *nnz_io = nnz. */
int tk_assemble(tk_ctx* ctx, int method, int64_t N, int k, int td, const int32_t* idx, const double* weights,
                double shift, int64_t* row_ptr, int32_t* col_idx, double* vals, int64_t* nnz_io);

/* The dense eigenproblem pair of NPE (kind TK_PAIR_NPE, from the KLLE matrix M)
 * or LLTSA (kind TK_PAIR_LLTSA, from the KLTSA matrix M) for the linear
 * kernel: replaces construct_neighborhood_preserving_eigenproblem and
 * construct_lltsa_eigenproblem (routines/locally_linear.hpp:257-338). X is
 * points-major (N rows of D, row stride ldx), M is the CSR of tk_assemble /
 * tk_operator_copy (row_ptr: N + 1; col_idx, vals: row_ptr[N]). lhs and rhs are
 * D x D, column-major, written exactly as the reference leaves them:
 *   rhs = (U + U^T) / 2, U the upper triangle of sum_i x_i x_i^T (LLTSA: minus
 *         s s^T / N, s = sum_i x_i) -- off-diagonal entries halved;
 *   lhs = upper triangle of sum over nonzeros (i, j) of M_ij (x_i x_j^T + x_j
 *         x_i^T) (LLTSA: minus s s^T / N), lower triangle zero.
 * All pointers may be host or device memory. FP64 sums over fixed row blocks. */
#define TK_PAIR_NPE 0
#define TK_PAIR_LLTSA 1
int tk_eigenproblem_pair(tk_ctx* ctx, int kind, const void* X, int dtype, int64_t N, int D, int64_t ldx,
                         const int64_t* row_ptr, const int32_t* col_idx, const double* vals, double* lhs,
                         double* rhs);

/* Result summary of tk_smallest_eigenvectors. */
typedef struct tk_eig_info
{
    int32_t iterations;     /* filter + Rayleigh-Ritz rounds                      */
    int32_t block;          /* subspace width (32)                                 */
    int64_t matvecs;        /* block products with M                               */
    double spectrum_bound;  /* upper bound B of the spectrum used by the filter    */
    double max_residual;    /* max over returned pairs of ||M v - lambda v||       */
    int32_t converged;      /* 1 when every wanted pair met tol * B                */
    float ms;               /* wall time of the call                               */
} tk_eig_info;

/* The target_dimension smallest eigenpairs of the symmetric positive
 * semi-definite CSR matrix M after skipping the `skip` smallest: replaces
 * eigendecomposition(Arpack, SmallestEigenvalues, M, td) with skip = 1, the
 * last step of KLLE / KLTSA embed() (routines/eigendecomposition.hpp:31-50,
 * 252-266, 330-345; methods/kernel_locally_linear_embedding.hpp:27). M is the
 * CSR of tk_assemble / tk_operator_copy (row_ptr N + 1, col_idx and vals
 * row_ptr[N]); it must be symmetric (both triangles stored). Chebyshev-filtered
 * subspace iteration on the GPU; stops when every wanted pair has
 * ||M v - lambda v|| <= tol * B (tol <= 0: 1e-12), B an upper bound of the
 * spectrum, or after max_matvecs block products (<= 0: 200000), returning
 * TK_ERR_NOT_CONVERGED with the current iterate written. vectors is N x td
 * column-major (the reference's DenseMatrix), each vector's entry of largest
 * magnitude positive; values (td) ascending. Needs td + skip <= 14 and
 * N >= 128 (four block widths); smaller problems belong to a dense solver.
 * All pointers may be host or device memory; info may be NULL. */
int tk_smallest_eigenvectors(tk_ctx* ctx, int64_t N, const int64_t* row_ptr, const int32_t* col_idx,
                             const double* vals, int target_dimension, int skip, double tol, int64_t max_matvecs,
                             double* vectors, double* values, tk_eig_info* info);

/* The whole stage of KernelLocallyLinearEmbeddingImplementation::embed /
 * KernelLocalTangentSpaceAlignmentImplementation::embed up to the eigensolver
 * (methods/kernel_locally_linear_embedding.hpp:22-30,
 *  methods/kernel_local_tangent_space_alignment.hpp:22-30): parameter checks of
 * ImplementationBase (methods/base.hpp:31-49,82-88), find_neighbors with the k
 * clamp and connectivity retry (neighbors/neighbors.hpp:173-213), weights, and M.
 * The result stays on the device, owned by ctx, until the next call; read it
 * with tk_operator_copy / tk_operator_device_views. info may be NULL. */
int tk_local_operator(tk_ctx* ctx, const tk_params* params, const void* X, int dtype, int64_t N, int D,
                      int64_t ldx, tk_operator_info* info);

/* Copies the operator held by ctx into caller buffers (host or device; any may
 * be NULL): idx N x k, weights (N x k for KLLE, N x k x td for KLTSA),
 * row_ptr N+1, col_idx nnz, vals nnz. */
int tk_operator_copy(tk_ctx* ctx, int32_t* idx, double* weights, int64_t* row_ptr, int32_t* col_idx,
                     double* vals);

/* Device pointers of the operator held by ctx (valid until the next call on ctx). */
int tk_operator_device_views(tk_ctx* ctx, const int32_t** idx, const double** weights, const int64_t** row_ptr,
                             const int32_t** col_idx, const double** vals);

/* Information about the operator held by ctx. */
int tk_operator_get_info(const tk_ctx* ctx, tk_operator_info* info);

/* Failure-path self-test: one CTA waits, with the distance screen's own bounded
 * mbarrier wait (2 s limit), on a barrier that nothing arrives at. The wait
 * expires, the kernel records the device-side timeout and returns, and the call
 * returns TK_ERR_TIMEOUT with *outcome = 1 (2 would mean the wait completed).
 * The context stays usable. No counterpart in the reference. */
int tk_selftest_bounded_wait(tk_ctx* ctx, int* outcome);

/* Failure-path self-test of the connectivity check's grid barrier: a cooperative
 * launch whose CTA 0 returns without reaching the barrier. The other CTAs' waits
 * (2 s limit) expire, they record the device-side timeout and return, and the call
 * returns TK_ERR_TIMEOUT with *outcome = 1 (2 would mean the barrier completed).
 * The context stays usable. No counterpart in the reference. */
int tk_selftest_grid_barrier(tk_ctx* ctx, int* outcome);

/* Waits for all work queued on the context's stream. */
int tk_ctx_synchronize(tk_ctx* ctx);

/* ---- batches of independent problems ------------------------------------------ */

/* Many independent KLLE stages (the part of embed() that tk_local_operator runs,
 * without the connectivity retry) of uneven N, D and k, planned once and replayed
 * as one CUDA graph: one persistent tensor-core screen launch per group of
 * problems with the same padded dimension and candidate-list length, one launch
 * per stage for the rest. No counterpart in the reference, which embeds one data
 * set per call; each problem's result equals tk_local_operator's on it (the same
 * neighbours, weights within 1e-5, the same M structure). */
typedef struct tk_batch tk_batch;

typedef struct tk_batch_problem
{
    const void* X; /* device memory, points-major N x D, row stride ldx     */
    int dtype;     /* TK_F32 or TK_F64                                      */
    int64_t N;
    int D;         /* 1..128                                                */
    int64_t ldx;
    int k;         /* 1..min(56, N-1)                                       */
} tk_batch_problem;

/* Tile shapes of a batch (picked by the autotuner, tapkee_gb300/autotune.py). */
typedef struct tk_batch_tuning
{
    int screen_qt[2]; /* query blocks of 128 rows per screen work item for padded
                         dimension 64 (1 or 2) and 128 (1)                       */
    int lle_warps;    /* problems per block of the weight solve: 4 or 8 warps    */
    int wide_lists;   /* 1: 64 screened candidates per row for every k, else the
                         smallest list >= k + 8 (32 or 64)                        */
} tk_batch_tuning;

void tk_batch_tuning_default(tk_batch_tuning* tuning);

/* Plans the batch on ctx's device and stream, runs it once and captures it as a
 * CUDA graph. The X buffers must stay valid (their contents may change) for the
 * life of the batch. tuning may be NULL (defaults). */
int tk_batch_create(tk_ctx* ctx, const tk_batch_problem* problems, int count, double klle_shift,
                    double nullspace_shift, const tk_batch_tuning* tuning, tk_batch** out);
/* Replays the graph and waits for it; ms_out (may be NULL) = device time. */
int tk_batch_run(tk_batch* batch, float* ms_out);
int tk_batch_count(const tk_batch* batch);
/* n, k, nnz of problem p (caller numbering); rows_uncertified counts its screen group. */
int tk_batch_get_info(tk_batch* batch, int p, tk_operator_info* info);
/* Problem p's neighbours (N x k), weights (N x k), and M in CSR (N+1, nnz, nnz),
 * numbered within the problem. Host or device buffers; any may be NULL. */
int tk_batch_copy(tk_batch* batch, int p, int32_t* idx, double* weights, int64_t* row_ptr, int32_t* col_idx,
                  double* vals);
int tk_batch_destroy(tk_batch* batch);

/* ---- allocation-free entry point --------------------------------------------- */

/* Largest graph tk_check_connected_noalloc accepts, and the size of the static
 * device scratch that holds its BFS state (one instance per device). */
#define TK_NOALLOC_MAX_POINTS 2097152
#define TK_NOALLOC_SCRATCH_BYTES 17039616

/* Same result as tk_check_connected, without a context and without allocating
 * host or device memory. It has no counterpart in the reference: it exists for
 * callers that cannot allocate device memory at the point of the call (a process
 * whose free HBM is held by a caching allocator) or cannot accept the
 * device-wide synchronisation of a scratch buffer being freed and regrown.
 *   - idx (N x k) must already be device or managed memory of `device`;
 *     nothing is copied. stream is a cudaStream_t of `device` (NULL = default
 *     stream). The call waits for its own result on that stream.
 *   - N must not exceed TK_NOALLOC_MAX_POINTS; larger N returns
 *     TK_ERR_INVALID_ARG with a message naming the limit.
 *   - The first call on a device does the set-up (resolves the device address of
 *     the scratch array and loads the kernel): make it before any stream capture.
 *     The resolved address is kept for the life of the process; cudaDeviceReset
 *     destroys the array it points to, so a process that resets a device must not
 *     call this entry point on that device afterwards.
 *   - Every call on a device shares the one scratch array: calls that overlap in
 *     time on that device (other threads, other streams) race and must be
 *     serialised by the caller.
 *   - msg (msg_len bytes, may be NULL) receives the error message, "" on success. */
int tk_check_connected_noalloc(int device, void* stream, int64_t N, int k, const int32_t* idx, int* connected,
                               char* msg, size_t msg_len);

#ifdef __cplusplus
}
#endif

#endif /* TAPKEE_GB300_H */
