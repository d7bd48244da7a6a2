// tk_internal.h -- shared declarations of the GB300 local-neighborhood operator.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <unordered_map>

#include "../../include/tapkee_gb300.h"

namespace tk {

// Internal error carrying a tk_status; converted to a return code at the C ABI.
struct Error : public std::runtime_error
{
    int status;
    Error(int s, const std::string& msg) : std::runtime_error(msg), status(s) {}
};

#define TK_CUDA(call)                                                                                        \
    do                                                                                                       \
    {                                                                                                        \
        cudaError_t err__ = (call);                                                                          \
        if (err__ != cudaSuccess)                                                                            \
        {                                                                                                    \
            if (err__ == cudaErrorMemoryAllocation)                                                          \
                throw ::tk::Error(TK_ERR_OOM, std::string("out of device memory at ") + #call);             \
            throw ::tk::Error(TK_ERR_CUDA, std::string(cudaGetErrorString(err__)) + " at " + __FILE__ + ":" + \
                                               std::to_string(__LINE__));                                   \
        }                                                                                                    \
    } while (0)

// Counts every kernel launch of the library (exported as tk_kernel_launch_count).
extern std::atomic<long long> g_kernel_launches;
#define TK_CHECK_LAUNCH()                                                                                   \
    do                                                                                                      \
    {                                                                                                       \
        TK_CUDA(cudaGetLastError());                                                                        \
        ::tk::g_kernel_launches.fetch_add(1, std::memory_order_relaxed);                                    \
    } while (0)

// Device-side error word bits (written by kernels instead of trapping).
enum : unsigned
{
    DEV_ERR_TIMEOUT = 1u,       // a bounded spin-wait gave up
    DEV_ERR_OVERFLOW = 2u,      // a bounded buffer overflowed
    DEV_ERR_BOUNDS = 4u,        // an index check failed
    DEV_ERR_NONFINITE = 8u      // non-finite input where finite is required
};

// Grow-only named scratch arena of a context.
struct Scratch
{
    struct Buf
    {
        void* ptr = nullptr;
        size_t bytes = 0;
    };
    std::unordered_map<std::string, Buf> bufs;
    void* get(const std::string& name, size_t bytes);
    void release_all();
};

// Layout of the prepared (screening) copy of the point cloud.
struct Prepared
{
    int64_t N = 0;      // points
    int64_t Npad = 0;   // rows padded to the screening tile (multiple of 256)
    int D = 0;          // input dimension
    int Dp = 0;         // padded dimension (multiple of 64)
    float* xc = nullptr;        // Npad x Dp centred FP32 coordinates, sorted order
    float* nrm = nullptr;       // Npad squared norms of xc (+inf for padding rows)
    uint16_t* xh = nullptr;     // Npad x Dp fp16 high parts of scale*xc (tensor screen)
    uint16_t* xl = nullptr;     // Npad x Dp fp16 low parts
    uint16_t* xn = nullptr;     // Npad x 16 fp16: hi/lo of -|2^s xc|^2 / 2^14 (cols 0,1), tensor screen
    int32_t* perm = nullptr;    // sorted position -> original index
    float* rmax = nullptr;      // device scalars: [0] R = max |xc|, [1] fp16 scale exponent s
    float scale_log2 = 0.f;     // xh/xl hold xc * 2^scale_log2
    // set by the wide tensor screen and the seeded long-list passes: per sorted
    // row, the smallest screened value over the candidate tiles screened with
    // high parts only (FLT_MAX: none), and the relative error constant of those values
    float* far_val = nullptr;
    float c2_far = 0.f;
};

} // namespace tk

struct tk_ctx
{
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::string last_error;
    tk_log_fn log_fn = nullptr;
    void* log_user = nullptr;
    tk::Scratch scratch;
    unsigned* dev_err = nullptr;      // device error word
    unsigned* host_err = nullptr;     // pinned mirror
    int64_t* host_i64 = nullptr;      // pinned small readback area (16 entries)
    cudaEvent_t ev[12] = {};
    float screen_ms = 0.f;            // device time of the last distance screen
    // per-kernel timing marks of tk_local_operator (recorded only while marks_on,
    // so they never enter a captured graph); see tk::mark
    cudaEvent_t kev[10] = {};
    bool marks_on = false;
    int64_t knn_ties = 0;             // tie rows of the last brute kNN pass
    int64_t knn_extra = 0;            // rows of that pass with k + 1 reference neighbours
    int num_sms = 0;
    // operator held by the context
    tk_operator_info op{};
    bool op_valid = false;
};

namespace tk {

void log(tk_ctx* ctx, int level, const std::string& msg);

// Timing marks (tk_ctx::kev) of one tk_local_operator call, in stream order.
enum : int
{
    KM_PREP = 0,   // before the point preparation of the last kNN pass
    KM_SCREEN0,    // before its distance screen
    KM_SCREEN1,    // after the screen
    KM_RERANK,     // after the re-rank, fallback and tie selection
    KM_ASM0,       // assembly: start
    KM_ASM_REV,    // after the reverse lists
    KM_ASM_ROWS,   // after the row pass
    KM_ASM_END,    // after the CSR write
    KM_COUNT
};
inline void mark(tk_ctx* ctx, int m)
{
    if (ctx->marks_on)
        cudaEventRecord(ctx->kev[m], ctx->stream);
}

// ---- kernel launchers (one translation unit each) -------------------------

// prep.cu: centre, order spatially and lay out the point cloud for screening.
void prepare_points(tk_ctx* ctx, const void* X, int dtype, int64_t N, int D, int64_t ldx, bool tensor,
                    Prepared& out);

// knn_simt.cu / knn_tc.cu: screening, K candidates per row (sorted-space indices).
constexpr int KCAND_MAX = 64;
void screen_fp32(tk_ctx* ctx, const Prepared& P, int kc, int32_t* cand_idx, float* cand_val);
void screen_tensor(tk_ctx* ctx, Prepared& P, int kc, int k, int32_t* cand_idx, float* cand_val);

// ---- batches of independent problems -----------------------------------------

// One problem of a batch as the kernels see it.
struct BatchProb
{
    const void* X;     // device points, row stride ldx
    int dtype;
    int D;
    int64_t ldx;
    int64_t N;
    int k;
    int group;         // screen group
    int64_t row0;      // first stacked row in its screen group (multiple of 256)
    int64_t idx_off;   // element offset of its rows in the neighbour and weight tables
    int64_t out_row0;  // first row in the batch's output row space (problems ordered by k)
    int64_t hoff;      // first Morton bucket of the problem in its group's histogram
    int hbits;         // log2 of the problem's bucket count
};

// Problems stacked for one batched screen launch (same Dp and KC).
struct StackedScreen
{
    int Dp = 0, kc = 0, qt = 1;
    int kmax = 0;                     // largest k of the group's problems
    int64_t rows = 0;                 // stacked rows (multiple of 256)
    const uint16_t* xh = nullptr;     // rows x Dp fp16 hi / lo of 2^s (x - mean)
    const uint16_t* xl = nullptr;
    const uint16_t* xn = nullptr;     // rows x 16 fp16 norm column
    const float* nrm = nullptr;       // rows squared norms (+inf for padding)
    const int4* items = nullptr;      // (q0 / (qt 128), first tile, tiles, problem)
    int nitems = 0;
    const int64_t* prob_n = nullptr;  // per problem (batch numbering)
    const float* prob_scale = nullptr;
};
void screen_tensor_batch(tk_ctx* ctx, const StackedScreen& S, int32_t* cand_idx, float* cand_val);

// Where the rows handled by the re-rank live: one problem (rows in sorted order,
// perm maps them back) or a batch (stacked rows; row_prob gives each row's problem
// or -1 for padding).
struct RowSpace
{
    const void* X = nullptr;
    int dtype = 0;
    int64_t ldx = 0;
    int D = 0;
    int64_t N = 0;
    int k = 0;
    const int32_t* perm = nullptr;
    const float* R = nullptr;
    int32_t* idx_out = nullptr;
    double* d2_out = nullptr;
    const int32_t* row_prob = nullptr;  // batch only (perm then maps stacked rows to points)
    const BatchProb* probs = nullptr;
    const float* prob_R = nullptr;
    int32_t* idx_all = nullptr;
    const float* far_val = nullptr;  // per row: smallest far-tile screened value (wide screen)
    float c2_far = 0.f;
};
// Re-rank + certification + exact fallback of a batch group; the fallback reads
// its row count on the device (no host synchronisation).
// LLE weights of the rows of one k-group of a batch (uniform k; row g belongs to
// problem row_prob[g]); warps = warps per block of the solve kernel (4 or 8).
void lle_weights_batch(tk_ctx* ctx, const BatchProb* probs, const int32_t* row_prob, int64_t out_row0, int64_t rows,
                       const int32_t* idx, int k, double klle_shift, double* W, int warps);
// counts_out: 4 device counters (uncertified rows, tie rows, rows with k + 1
// reference neighbours, unused); max_n bounds the group's problem sizes.
void rerank_batch(tk_ctx* ctx, const RowSpace& S, int64_t rows, int64_t max_n, int kc, const int32_t* cand_idx,
                  const float* cand_val, const float* nrm, float eps_c1, float eps_c2, unsigned* counts_out);
bool tensor_screen_supported(int Dp);

// rerank.cu: exact FP64 re-rank, certification, exact fallback, and the
// reference's nth_element selection for tie rows. Returns the number of
// uncertified rows (device -> host read); sets ctx->knn_ties and ctx->knn_extra
// and leaves the extra rows as (row, (k + 1)-th neighbour) pairs in the scratch
// buffer "rerank.extra".
int64_t rerank(tk_ctx* ctx, const Prepared& P, const void* X, int dtype, int64_t ldx, int k, int kc,
               const int32_t* cand_idx, const float* cand_val, float eps_c1, float eps_c2, int32_t* idx_out,
               double* d2_out);

// connectivity.cu
bool check_connected(tk_ctx* ctx, int64_t N, int k, const int32_t* idx);
// One cooperative launch whose CTA 0 never reaches the BFS grid barrier: returns 1
// when the other CTAs' bounded waits expired as designed, 2 if the barrier
// completed, 0 otherwise.
int barrier_selftest(tk_ctx* ctx);

// lle.cu
void lle_weights(tk_ctx* ctx, const void* X, int dtype, int64_t N, int D, int64_t ldx, const int32_t* idx,
                 int k, double klle_shift, double* W);
// The same regularised solve with a per-point right-hand side rhs (N x k; NULL =
// ones) and, when normalize is false, the raw solution instead of weights.
void lle_solve(tk_ctx* ctx, const void* X, int dtype, int64_t N, int D, int64_t ldx, const int32_t* idx, int k,
               double klle_shift, const double* rhs, bool normalize, double* W);
// lle_pair.cu: the same solve, two points per warp, for float32 points with
// 16-byte aligned rows and k <= 16 (lle_solve dispatches to it).
bool lle_pair_supported(const void* X, int dtype, int64_t ldx, int k);
void lle_pair_solve(tk_ctx* ctx, const void* X, int64_t N, int D, int64_t ldx, const int32_t* idx, int k,
                    double klle_shift, const double* rhs, bool normalize, double* W);
// dL/dX (N x D, FP64, row stride D) of the weights W for upstream dL/dW = G.
void lle_weights_grad(tk_ctx* ctx, const void* X, int dtype, int64_t N, int D, int64_t ldx, const int32_t* idx, int k,
                      double klle_shift, const double* W, const double* G, double* gX);

// ltsa.cu
void ltsa_basis(tk_ctx* ctx, const void* X, int dtype, int64_t N, int D, int64_t ldx, const int32_t* idx,
                int k, int td, double* V);

// hessian.cu: the dp = td (td + 1) / 2 product columns Y (N x k x dp) of every
// point's orthonormalised Hessian basis; B = Y Y^T per point (td 1 or 2).
void hessian_basis(tk_ctx* ctx, const void* X, int dtype, int64_t N, int D, int64_t ldx, const int32_t* idx,
                   int k, int td, double* Y);

// Columns per (point, neighbour) of a method's weights: LLE 1, LTSA td, HLLE
// td (td + 1) / 2.
inline int weight_columns(int method, int td)
{
    return method == TK_METHOD_KLTSA ? td : (method == TK_METHOD_HLLE ? td * (td + 1) / 2 : 1);
}

// assemble.cu: the row phase (reverse adjacency, every row's sorted columns and
// values into a row scratch, row counts, row_ptr) returns nnz; the write phase
// then copies the rows into col_idx/vals (device pointers) from the state kept
// in the context's scratch.
// Exclusive scan of n int counters into n + 1 int64 offsets (deterministic).
void scan_to_offsets(tk_ctx* ctx, const int* in, int64_t n, int64_t* out);
// Reverse adjacency of an N x k neighbour table: rev[rptr[j] .. rptr[j+1]) holds
// the edge ids e = r k + a with idx[e] = j, ascending (so by source r). Entries
// outside [0, N) are skipped and raise DEV_ERR_BOUNDS. rptr: N + 1, rev: N k.
void reverse_lists(tk_ctx* ctx, int64_t N, int k, const int32_t* idx, int64_t* rptr, int32_t* rev);
// The row phase without reading nnz back (row_ptr[N] holds it on the device).
void assemble_rows_device(tk_ctx* ctx, int method, int64_t N, int k, int td, const int32_t* idx,
                          const double* weights, double shift, int64_t* row_ptr);
int64_t assemble_rows(tk_ctx* ctx, int method, int64_t N, int k, int td, const int32_t* idx, const double* weights,
                      double shift, int64_t* row_ptr);
void assemble_write(tk_ctx* ctx, int method, int64_t N, int k, int td, const int32_t* idx, const double* weights,
                    double shift, const int64_t* row_ptr, int32_t* col_idx, double* vals);

// pair.cu: the NPE / LLTSA dense eigenproblem pair (device pointers).
void eigenproblem_pair(tk_ctx* ctx, int kind, const void* X, int dtype, int64_t N, int D, int64_t ldx,
                       const int64_t* row_ptr, const int32_t* col_idx, const double* vals, double* lhs, double* rhs);

// knn_tc.cu: one bounded mbarrier wait that nothing satisfies (the screen's wait
// helper); returns 1 when it expired as designed, 2 if it completed.
int wait_selftest(tk_ctx* ctx);

// eigen.cu: smallest eigenpairs of a symmetric CSR matrix (device pointers;
// vectors N x td column-major, values td). eigen_block_width gives the subspace
// width for td + skip, 0 when unsupported.
int eigen_block_width(int td, int skip);
// Checks a caller's CSR row pointers (N + 1 entries, device) against nnz: entries in
// [0, nnz], non-decreasing; a violation raises DEV_ERR_BOUNDS for check_device_errors.
void check_csr_rows(tk_ctx* ctx, int64_t N, const int64_t* row_ptr, int64_t nnz);
void smallest_eigenvectors(tk_ctx* ctx, int64_t N, int64_t nnz, const int64_t* row_ptr, const int32_t* col_idx,
                           const double* vals, int td, int skip, double tol, int64_t max_matvecs, double* vectors,
                           double* values, tk_eig_info* info);

// Screening error model (see rerank.cu): |approx - exact| <= c1 (|x|^2 + R^2) + c2 |x| R.
void screen_error_model(int screen, int Dp, float* c1, float* c2);
// Relative error constant c2 of screened values formed from the fp16 high parts
// only (x.y ~ h_x.h_y): |a - d^2| <= c1 (|x|^2 + R^2) + c2 |x| R.
void screen_error_model_far(int Dp, float* c2);

} // namespace tk
