// eigen.cu -- the smallest eigenpairs of the sparse alignment matrix M.
//
// KLLE and KLTSA end embed() (methods/kernel_locally_linear_embedding.hpp:27,
// methods/kernel_local_tangent_space_alignment.hpp:27) with
// eigendecomposition(eigen_method, SmallestEigenvalues, M, td)
// (routines/eigendecomposition.hpp:330-345). With the default eigen_method,
// Arpack (defines/methods.hpp:198), that is ARPACK in "SM" mode whose operator
// solves with a SimplicialLDLT factor of M (routines/eigendecomposition.hpp:252-266,
// routines/matrix_operations.hpp:30-49, defines/types.hpp:40). It returns the
// td + skip smallest eigenpairs in increasing order and keeps the columns
// skip .. skip + td - 1 (routines/eigendecomposition.hpp:31-50).
//
// Here the same eigenpairs come from Chebyshev-filtered subspace iteration
// (Zhou, Saad, Tiago, Chelikowsky, J. Comput. Phys. 219, 2006) with the scaled
// three-term filter of Zhou & Saad (SIAM J. Matrix Anal. Appl. 29, 2007), run on
// M itself. Every step is then a sparse product with M on the GPU, and no
// factorisation is needed:
//   1. An upper bound B of the spectrum: the smaller of the Gershgorin bound and
//      a 40-step Lanczos estimate (largest Ritz value + last beta) widened by 5 %.
//   2. A block of BW = 32 vectors (td + skip <= 14), random, orthonormalised.
//   3. Repeat until every wanted pair has ||M x - theta x|| <= tol B:
//      - filter the block with a degree-m Chebyshev polynomial that damps
//        [a, B], where a is the largest Ritz value of the block, scaled to 1 at 0;
//      - orthonormalise it (Cholesky QR, twice);
//      - Rayleigh-Ritz with M.
//   The degree keeps the growth of the filter below 1e6 over the block, so the
//   Cholesky QR stays well conditioned.
// M's smallest eigenvalues are ~1e-9 .. 1e-6 of B, so products with M need more than
// FP32. They are accumulated in float-float (~2^-46 relative) on the FP32 pipes,
// because GB300's FP64 rate is a small fraction of its FP32 rate. The block is
// stored as float-float pairs; Gram matrices, rotations and residuals are FP64.
// Every reduction runs in a fixed order, so the result is the same on every run.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "eigen_host.h"
#include "ff.cuh"
#include "tk_internal.h"

namespace tk {
namespace {

constexpr int EG_THREADS = 256;
constexpr int GRAM_ROWS = 32;       // rows staged per step of the Gram kernel
constexpr int LANCZOS_STEPS = 40;
constexpr int DEG_MIN = 4, DEG_MAX = 32768;  // the growth limit, not DEG_MAX, sets the degree in practice
constexpr double GROWTH_LOG = 13.8;  // ln(1e6): the filter's largest gain over the block

__device__ __forceinline__ float2 split_ff(double x)
{
    const float h = (float)x;
    return make_float2(h, (float)(x - (double)h));
}

__device__ __forceinline__ double ff_d(float2 a)
{
    return (double)a.x + (double)a.y;
}

// A caller's CSR row pointers: every entry in [0, nnz] and non-decreasing, so
// that no row range reaches outside the column and value arrays. A violation
// raises DEV_ERR_BOUNDS (reads only rp[0..N]).
__global__ void k_check_rows(int64_t N, const int64_t* __restrict__ rp, int64_t nnz, unsigned* err)
{
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r <= N; r += (int64_t)gridDim.x * blockDim.x)
    {
        const int64_t a = rp[r];
        bool bad = a < 0 || a > nnz;
        if (r < N)
            bad = bad || rp[r + 1] < a;
        if (bad)
            atomicOr(err, DEV_ERR_BOUNDS);
    }
}

__global__ void k_vals_split(int64_t nnz, const double* __restrict__ v, float2* __restrict__ out)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nnz; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = split_ff(v[i]);
}

// Gershgorin bound max_r sum_p |M_rp|, one warp per row. Non-negative doubles
// order like their bit patterns, so the maximum goes through a 64-bit atomicMax.
__global__ void k_gershgorin(int64_t N, const int64_t* __restrict__ rp, const double* __restrict__ v,
                             unsigned long long* out)
{
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < N; r += nw)
    {
        double s = 0.0;
        for (int64_t p = rp[r] + lane; p < rp[r + 1]; p += 32)
            s += fabs(v[p]);
#pragma unroll
        for (int o = 16; o; o >>= 1)
            s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0)
            atomicMax(out, (unsigned long long)__double_as_longlong(s));
    }
}

__device__ __forceinline__ uint64_t mix64(uint64_t z)
{
    // splitmix64 finaliser (Steele, Lea, Flood, OOPSLA 2014)
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Uniform entries in [-1, 1) from a counter-based hash of (seed, element).
__global__ void k_init_block(int64_t n, uint64_t seed, float2* __restrict__ Y)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    {
        const uint64_t u = mix64(seed + 0x9E3779B97F4A7C15ull * (uint64_t)(i + 1));
        Y[i] = split_ff((double)(u >> 11) * 0x1.0p-52 - 1.0);
    }
}

// Out = alpha (M Y - c Y) + beta Old, row-major N x BW blocks of float-float
// pairs, one warp per row of M. The lanes form G = 32 / BW groups of BW lanes:
// group g takes the row's non-zeros g, g + G, ... and lane j of a group owns
// column j, so each non-zero reads one contiguous row of Y. The gathers of U
// non-zeros are issued before their products are accumulated, which keeps
// enough loads in flight to cover the L2 latency. Columns are checked against
// N; a bad one raises DEV_ERR_BOUNDS and is skipped.
template <int BW>
__global__ void __launch_bounds__(EG_THREADS, 4) k_cheb(int64_t N, const int64_t* __restrict__ rp,
                                                        const int32_t* __restrict__ col,
                                                        const float2* __restrict__ vff, const float2* __restrict__ Y,
                                                        const float2* __restrict__ Old, float2* __restrict__ Out,
                                                        float2 alpha, float2 negc, float2 beta, unsigned* err)
{
    constexpr int G = 32 / BW;
    constexpr int U = BW == 1 ? 1 : 8;
    const int lane = threadIdx.x & 31, g = lane / BW, j = lane % BW;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < N; r += nw)
    {
        const int64_t p0 = rp[r], p1 = rp[r + 1];
        ff acc = ff_zero();
        for (int64_t base = p0; base < p1; base += 32)
        {
            const int n = (int)min((int64_t)32, p1 - base);
            int cc = 0;
            float2 vv = make_float2(0.f, 0.f);
            if (lane < n)
            {
                cc = col[base + lane];
                vv = vff[base + lane];
                if (cc < 0 || (int64_t)cc >= N)
                {
                    atomicOr(err, DEV_ERR_BOUNDS);
                    cc = 0;
                    vv = make_float2(0.f, 0.f);
                }
            }
            for (int q0 = 0; q0 < n; q0 += G * U)
            {
                float2 y[U];
                float vh[U], vl[U];
#pragma unroll
                for (int u = 0; u < U; ++u)
                {
                    const int q = q0 + G * u + g;
                    const int cq = __shfl_sync(0xffffffffu, cc, q & 31);
                    vh[u] = __shfl_sync(0xffffffffu, vv.x, q & 31);
                    vl[u] = __shfl_sync(0xffffffffu, vv.y, q & 31);
                    y[u] = q < n ? Y[(int64_t)cq * BW + j] : make_float2(0.f, 0.f);
                }
#pragma unroll
                for (int u = 0; u < U; ++u)
                    acc = ff_fma(acc, vh[u], vl[u], y[u].x, y[u].y);
            }
        }
#pragma unroll
        for (int o = BW; o < 32; o <<= 1)
            acc = ff_add(acc, ff_shfl_xor(acc, o));
        if (g == 0)
        {
            const float2 yr = Y[r * BW + j];
            ff t = ff_fma(acc, negc.x, negc.y, yr.x, yr.y);
            t = ff_mul(t, ff{alpha.x, alpha.y});
            if (Old)
            {
                const float2 o = Old[r * BW + j];
                t = ff_fma(t, beta.x, beta.y, o.x, o.y);
            }
            Out[r * BW + j] = make_float2(t.hi, t.lo);
        }
    }
}

// Block partials of A^T B (BW x BW, FP64) over fixed row ranges.
template <int BW>
__global__ void __launch_bounds__(EG_THREADS) k_gram(int64_t N, const float2* __restrict__ A,
                                                     const float2* __restrict__ B, int64_t rows_per,
                                                     double* __restrict__ part)
{
    constexpr int NE = BW * BW;
    constexpr int EPT = (NE + EG_THREADS - 1) / EG_THREADS;
    __shared__ double as[GRAM_ROWS * BW], bs[GRAM_ROWS * BW];
    const int t = threadIdx.x;
    const int64_t r0 = (int64_t)blockIdx.x * rows_per, r1 = min(N, r0 + rows_per);
    double acc[EPT];
#pragma unroll
    for (int m = 0; m < EPT; ++m)
        acc[m] = 0.0;
    for (int64_t c0 = r0; c0 < r1; c0 += GRAM_ROWS)
    {
        const int nr = (int)min((int64_t)GRAM_ROWS, r1 - c0);
        __syncthreads();
        for (int q = t; q < nr * BW; q += EG_THREADS)
        {
            as[q] = ff_d(A[c0 * BW + q]);
            bs[q] = ff_d(B[c0 * BW + q]);
        }
        __syncthreads();
        for (int rr = 0; rr < nr; ++rr)
        {
#pragma unroll
            for (int m = 0; m < EPT; ++m)
            {
                const int e = t + EG_THREADS * m;
                if (e < NE)
                    acc[m] = fma(as[rr * BW + e / BW], bs[rr * BW + e % BW], acc[m]);
            }
        }
    }
#pragma unroll
    for (int m = 0; m < EPT; ++m)
    {
        const int e = t + EG_THREADS * m;
        if (e < NE)
            part[(int64_t)blockIdx.x * NE + e] = acc[m];
    }
}

// out[e] = sum over parts in order.
__global__ void k_sum_parts(int nparts, int ne, const double* __restrict__ part, double* __restrict__ out)
{
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += gridDim.x * blockDim.x)
    {
        double s = 0.0;
        for (int b = 0; b < nparts; ++b)
            s += part[(int64_t)b * ne + e];
        out[e] = s;
    }
}

// Out = In Q (Q row-major BW x BW, FP64), one thread per row.
template <int BW>
__global__ void __launch_bounds__(128) k_rotate(int64_t N, const float2* __restrict__ In, const double* __restrict__ Qg,
                                                float2* __restrict__ Out)
{
    __shared__ double Q[BW * BW];
    for (int q = threadIdx.x; q < BW * BW; q += blockDim.x)
        Q[q] = Qg[q];
    __syncthreads();
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < N; r += (int64_t)gridDim.x * blockDim.x)
    {
        double x[BW];
#pragma unroll
        for (int i = 0; i < BW; ++i)
            x[i] = ff_d(In[r * BW + i]);
#pragma unroll 4
        for (int jj = 0; jj < BW; ++jj)
        {
            double s = 0.0;
#pragma unroll
            for (int i = 0; i < BW; ++i)
                s = fma(x[i], Q[i * BW + jj], s);
            Out[r * BW + jj] = split_ff(s);
        }
    }
}

// Block partials of the column norms ||Z_j - theta_j X_j||^2. The grid stride is a
// multiple of BW, so each thread stays on one column.
template <int BW>
__global__ void __launch_bounds__(EG_THREADS) k_resid(int64_t N, const float2* __restrict__ X,
                                                      const float2* __restrict__ Z, const double* __restrict__ theta,
                                                      double* __restrict__ part)
{
    __shared__ double ws[EG_THREADS / 32][32];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const int j = t % BW;
    const double th = theta[j];
    double s = 0.0;
    const int64_t n = N * BW;
    for (int64_t e = blockIdx.x * (int64_t)EG_THREADS + t; e < n; e += (int64_t)gridDim.x * EG_THREADS)
    {
        const double d = ff_d(Z[e]) - th * ff_d(X[e]);
        s = fma(d, d, s);
    }
#pragma unroll
    for (int o = BW; o < 32; o <<= 1)
        s += __shfl_xor_sync(0xffffffffu, s, o);
    ws[w][lane] = s;
    __syncthreads();
    if (t < BW)
    {
        double a = 0.0;
        for (int q = 0; q < EG_THREADS / 32; ++q)
            a += ws[q][t % 32];
        part[(int64_t)blockIdx.x * BW + t] = a;
    }
}

// Per output column c (grid.y), block partials of (max |x|, lowest row with it).
template <int BW>
__global__ void __launch_bounds__(EG_THREADS) k_colmax(int64_t N, const float2* __restrict__ X, int col0,
                                                       double* __restrict__ pv, int64_t* __restrict__ pi)
{
    __shared__ double sv[EG_THREADS / 32];
    __shared__ int64_t si[EG_THREADS / 32];
    const int c = blockIdx.y, t = threadIdx.x, lane = t & 31, w = t >> 5;
    double bv = -1.0;
    int64_t bi = 0;
    for (int64_t r = blockIdx.x * (int64_t)EG_THREADS + t; r < N; r += (int64_t)gridDim.x * EG_THREADS)
    {
        const double a = fabs(ff_d(X[r * BW + col0 + c]));
        if (a > bv)
        {
            bv = a;
            bi = r;
        }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1)
    {
        const double ov = __shfl_xor_sync(0xffffffffu, bv, o);
        const int64_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov > bv || (ov == bv && oi < bi))
        {
            bv = ov;
            bi = oi;
        }
    }
    if (lane == 0)
    {
        sv[w] = bv;
        si[w] = bi;
    }
    __syncthreads();
    if (t == 0)
    {
        for (int q = 1; q < EG_THREADS / 32; ++q)
            if (sv[q] > bv || (sv[q] == bv && si[q] < bi))
            {
                bv = sv[q];
                bi = si[q];
            }
        pv[(int64_t)c * gridDim.x + blockIdx.x] = bv;
        pi[(int64_t)c * gridDim.x + blockIdx.x] = bi;
    }
}

struct Signs
{
    double s[32];
};

// out (column-major N x td) = sign_c * X[:, col0 + c].
template <int BW>
__global__ void k_write_vectors(int64_t N, const float2* __restrict__ X, int col0, int td, Signs sg,
                                double* __restrict__ out)
{
    const int64_t n = N * td;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    {
        const int c = (int)(e / N);
        const int64_t r = e - (int64_t)c * N;
        out[e] = sg.s[c] * ff_d(X[r * BW + col0 + c]);
    }
}

using eigen_host::chol_upper;
using eigen_host::inv_upper;
using eigen_host::jacobi_eig;

float2 host_ff(double x)
{
    const float h = (float)x;
    return make_float2(h, (float)(x - (double)h));
}

// ---------------------------------------------------------------- the solver

struct Csr
{
    int64_t N;
    const int64_t* rp;
    const int32_t* col;
    const float2* vff;
};

template <int BW>
class Filter
{
  public:
    Filter(tk_ctx* ctx, const Csr& A) : ctx_(ctx), A_(A)
    {
        const int64_t n = A.N;
        nparts_ = (int)std::max<int64_t>(1, std::min<int64_t>((n + 511) / 512, (int64_t)ctx->num_sms * 2));
        rows_per_ = (n + nparts_ - 1) / nparts_;
        // one resident wave of the product kernel (its rows are grid-strided)
        int per_sm = 1;
        TK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cheb<BW>, EG_THREADS, 0));
        spmm_grid_ = (int)std::max<int64_t>(1, std::min<int64_t>((n + 7) / 8, (int64_t)ctx->num_sms * std::max(per_sm, 1)));
        row_grid_ = (int)std::max<int64_t>(1, std::min<int64_t>((n + 127) / 128, (int64_t)ctx->num_sms * 8));
        el_grid_ = (int)std::max<int64_t>(1, std::min<int64_t>((n * BW + EG_THREADS - 1) / EG_THREADS,
                                                               (int64_t)ctx->num_sms * 8));
        // partials of the Gram (nparts_ x BW^2) and of the residual norms (el_grid_ x BW)
        const size_t np = std::max((size_t)nparts_ * BW * BW, (size_t)el_grid_ * BW);
        part_ = (double*)ctx->scratch.get("eig.part" + std::to_string(BW), sizeof(double) * np);
        small_ = (double*)ctx->scratch.get("eig.small" + std::to_string(BW), sizeof(double) * (BW * BW + BW));
    }
    // Out = alpha (M Y - c Y) + beta Old
    void cheb(const float2* Y, const float2* Old, float2* Out, double alpha, double c, double beta)
    {
        k_cheb<BW><<<spmm_grid_, EG_THREADS, 0, ctx_->stream>>>(A_.N, A_.rp, A_.col, A_.vff, Y, Old, Out,
                                                               host_ff(alpha), host_ff(-c), host_ff(beta),
                                                               ctx_->dev_err);
        TK_CHECK_LAUNCH();
    }
    // A^T B, BW x BW row-major on the host
    std::vector<double> gram(const float2* A, const float2* B)
    {
        k_gram<BW><<<nparts_, EG_THREADS, 0, ctx_->stream>>>(A_.N, A, B, rows_per_, part_);
        TK_CHECK_LAUNCH();
        k_sum_parts<<<1, EG_THREADS, 0, ctx_->stream>>>(nparts_, BW * BW, part_, small_);
        TK_CHECK_LAUNCH();
        std::vector<double> h(BW * BW);
        TK_CUDA(cudaMemcpyAsync(h.data(), small_, sizeof(double) * BW * BW, cudaMemcpyDeviceToHost, ctx_->stream));
        TK_CUDA(cudaStreamSynchronize(ctx_->stream));
        return h;
    }
    void rotate(const float2* In, const std::vector<double>& Q, float2* Out)
    {
        TK_CUDA(cudaMemcpyAsync(small_, Q.data(), sizeof(double) * BW * BW, cudaMemcpyHostToDevice, ctx_->stream));
        k_rotate<BW><<<row_grid_, 128, 0, ctx_->stream>>>(A_.N, In, small_, Out);
        TK_CHECK_LAUNCH();
        // the next upload to small_ must not overtake this launch
        TK_CUDA(cudaStreamSynchronize(ctx_->stream));
    }
    std::vector<double> residuals(const float2* X, const float2* Z, const std::vector<double>& theta)
    {
        TK_CUDA(cudaMemcpyAsync(small_ + BW * BW, theta.data(), sizeof(double) * BW, cudaMemcpyHostToDevice,
                                ctx_->stream));
        k_resid<BW><<<el_grid_, EG_THREADS, 0, ctx_->stream>>>(A_.N, X, Z, small_ + BW * BW, part_);
        TK_CHECK_LAUNCH();
        k_sum_parts<<<1, EG_THREADS, 0, ctx_->stream>>>(el_grid_, BW, part_, small_);
        TK_CHECK_LAUNCH();
        std::vector<double> h(BW);
        TK_CUDA(cudaMemcpyAsync(h.data(), small_, sizeof(double) * BW, cudaMemcpyDeviceToHost, ctx_->stream));
        TK_CUDA(cudaStreamSynchronize(ctx_->stream));
        for (double& v : h)
            v = std::sqrt(v);
        return h;
    }
    // In place: orthonormalise the columns of *Y (Cholesky QR, two passes, a
    // shifted first pass when the Gram matrix is numerically singular). tmp is
    // a spare block; *Y and tmp may be swapped.
    void orthonormalise(float2*& Y, float2*& tmp)
    {
        int passes = 2;
        for (int pass = 0; pass < passes; ++pass)
        {
            std::vector<double> G = gram(Y, Y), R;
            for (int i = 0; i < BW; ++i)
                for (int j = 0; j < i; ++j)
                    G[(size_t)i * BW + j] = G[(size_t)j * BW + i] = 0.5 * (G[(size_t)i * BW + j] + G[(size_t)j * BW + i]);
            if (!chol_upper(BW, G, R))
            {
                // shifted Cholesky QR (Fukaya, Kannan, Nakatsukasa, Yamamoto, Yanagisawa,
                // SIAM J. Sci. Comput. 42, 2020): s = 11 (N BW + BW (BW + 1)) u ||G||
                double tr = 0.0;
                for (int i = 0; i < BW; ++i)
                    tr += G[(size_t)i * BW + i];
                const double s = 11.0 * ((double)A_.N * BW + BW * (BW + 1)) * 0x1.0p-47 * tr;
                for (int i = 0; i < BW; ++i)
                    G[(size_t)i * BW + i] += s;
                if (!chol_upper(BW, G, R))
                    throw Error(TK_ERR_INTERNAL, "eigensolver: the block lost rank (Cholesky QR failed)");
                passes = std::min(passes + 1, 4);
            }
            rotate(Y, inv_upper(BW, R), tmp);
            std::swap(Y, tmp);
        }
    }
    int64_t n() const { return A_.N; }

  private:
    tk_ctx* ctx_;
    Csr A_;
    int nparts_ = 1;
    int64_t rows_per_ = 1;
    double* part_ = nullptr;
    double* small_ = nullptr;
    int spmm_grid_ = 1, row_grid_ = 1, el_grid_ = 1;
};

// Upper bound of the spectrum from LANCZOS_STEPS Lanczos steps (no
// re-orthogonalisation; only the largest Ritz value is used): theta_max + beta_last.
double lanczos_bound(tk_ctx* ctx, const Csr& A, uint64_t seed)
{
    Filter<1> F(ctx, A);
    const int64_t N = A.N;
    float2* v = (float2*)ctx->scratch.get("eig.lz_v", sizeof(float2) * (size_t)N);
    float2* vp = (float2*)ctx->scratch.get("eig.lz_vp", sizeof(float2) * (size_t)N);
    float2* w = (float2*)ctx->scratch.get("eig.lz_w", sizeof(float2) * (size_t)N);
    k_init_block<<<(int)std::min<int64_t>((N + 255) / 256, 4096), 256, 0, ctx->stream>>>(N, seed, v);
    TK_CHECK_LAUNCH();
    TK_CUDA(cudaMemsetAsync(vp, 0, sizeof(float2) * (size_t)N, ctx->stream));
    {
        const double nv = std::sqrt(F.gram(v, v)[0]);
        F.rotate(v, {1.0 / nv}, w);
        std::swap(v, w);
    }
    const int K = (int)std::min<int64_t>(LANCZOS_STEPS, N - 1);
    std::vector<double> al, be;
    double beta = 0.0;
    for (int i = 0; i < K; ++i)
    {
        F.cheb(v, nullptr, w, 1.0, 0.0, 0.0);
        const double alpha = F.gram(v, w)[0];
        F.cheb(v, vp, w, 1.0, alpha, -beta);
        const double nb = std::sqrt(std::max(0.0, F.gram(w, w)[0]));
        al.push_back(alpha);
        be.push_back(nb);
        beta = nb;
        if (!(nb > 1e-300) || nb <= 1e-14 * std::fabs(alpha))
            break;
        std::swap(vp, v);  // vp <- v
        F.rotate(w, {1.0 / nb}, v);
    }
    const int k = (int)al.size();
    std::vector<double> T((size_t)k * k, 0.0), wv, V;
    for (int i = 0; i < k; ++i)
    {
        T[(size_t)i * k + i] = al[i];
        if (i + 1 < k)
            T[(size_t)i * k + i + 1] = T[(size_t)(i + 1) * k + i] = be[i];
    }
    jacobi_eig(k, T, wv, V);
    return wv.back() + be.back();
}

template <int BW>
void run_solver(tk_ctx* ctx, const Csr& A, double bound, int td, int skip, double tol, int64_t max_matvecs,
                double* vectors, double* values, tk_eig_info* info)
{
    const int64_t N = A.N;
    const int want = td + skip;
    Filter<BW> F(ctx, A);
    const size_t bytes = sizeof(float2) * (size_t)N * BW;
    float2* buf[5];
    for (int i = 0; i < 5; ++i)
        buf[i] = (float2*)ctx->scratch.get("eig.blk" + std::to_string(BW) + "_" + std::to_string(i), bytes);
    float2* X = buf[0];
    float2* Ya = buf[1];
    float2* Yb = buf[2];
    float2* Z = buf[3];
    float2* T = buf[4];

    k_init_block<<<(int)std::min<int64_t>((N * BW + 255) / 256, 8192), 256, 0, ctx->stream>>>(N * BW, 0x7A9B3C1Dull, X);
    TK_CHECK_LAUNCH();
    F.orthonormalise(X, T);

    int64_t matvecs = 0;
    int iters = 0;
    std::vector<double> theta(BW, 0.0), res(BW, 0.0);
    bool converged = false;
    auto rayleigh_ritz = [&]() {
        F.cheb(X, nullptr, Z, 1.0, 0.0, 0.0);
        ++matvecs;
        std::vector<double> H = F.gram(X, Z), V;
        for (int i = 0; i < BW; ++i)
            for (int j = 0; j < i; ++j)
                H[(size_t)i * BW + j] = H[(size_t)j * BW + i] = 0.5 * (H[(size_t)i * BW + j] + H[(size_t)j * BW + i]);
        jacobi_eig(BW, H, theta, V);
        F.rotate(X, V, T);
        std::swap(X, T);
        F.rotate(Z, V, T);
        std::swap(Z, T);
        res = F.residuals(X, Z, theta);
        double worst = 0.0;
        for (int j = 0; j < want; ++j)
            worst = std::max(worst, res[j]);
        return worst;
    };
    // a device-side check (a column outside [0, N)) ends the iteration early;
    // the caller reports it
    auto device_error = [&]() {
        unsigned e = 0;
        TK_CUDA(cudaMemcpyAsync(&e, ctx->dev_err, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
        TK_CUDA(cudaStreamSynchronize(ctx->stream));
        return e != 0;
    };
    double worst = rayleigh_ritz();
    converged = worst <= tol * bound;
    while (!converged && matvecs < max_matvecs && !device_error())
    {
        if (theta[BW - 1] > bound)  // the estimate was low: fall back to a safe bound
            bound = 1.05 * theta[BW - 1];
        const double a = theta[BW - 1];
        const double lo = std::min(theta[0], 0.0);
        double e = 0.5 * (bound - a);
        if (!(e > 0.0))
            e = 1e-3 * std::max(std::fabs(bound), 1e-300);
        const double c = 0.5 * (bound + a);
        const double x0 = (c - lo) / e;
        const double rho = std::acosh(std::max(x0, 1.0 + 1e-15));
        int64_t m = (int64_t)(GROWTH_LOG / rho);
        // at most doubling the products spent so far: a cut that the block has not
        // resolved yet (or a cluster of null vectors filling it) cannot start a
        // filter far longer than the work that led to it
        m = std::min<int64_t>(m, std::max<int64_t>(64, matvecs));
        m = std::max<int64_t>(DEG_MIN, std::min<int64_t>(DEG_MAX, m));
        m = std::max<int64_t>(1, std::min<int64_t>(m, max_matvecs - matvecs - 1));
        // scaled Chebyshev filter, value 1 at lo
        const double sigma1 = e / (lo - c);
        double sigma = sigma1;
        float2* prev = X;
        float2* cur = Ya;
        F.cheb(X, nullptr, cur, sigma1 / e, c, 0.0);
        ++matvecs;
        for (int64_t i = 2; i <= m; ++i)
        {
            const double sn = 1.0 / (2.0 / sigma1 - sigma);
            float2* next = (prev != Yb && cur != Yb) ? Yb : (prev != Ya && cur != Ya) ? Ya : X;
            F.cheb(cur, prev, next, 2.0 * sn / e, c, -sigma * sn);
            ++matvecs;
            prev = cur;
            cur = next;
            sigma = sn;
        }
        // cur holds the filtered block; X, Ya, Yb are now a free permutation
        float2* spare = (cur != X) ? X : Ya;
        F.orthonormalise(cur, spare);
        // keep the roles: X = orthonormal block, Ya / Yb free
        float2* pool[3] = {X, Ya, Yb};
        X = cur;
        int fi = 0;
        float2* freeb[2];
        for (float2* p : pool)
            if (p != X && fi < 2)
                freeb[fi++] = p;
        Ya = freeb[0];
        Yb = freeb[1];
        worst = rayleigh_ritz();
        ++iters;
        converged = worst <= tol * bound;
        if (ctx->log_fn)
        {
            char msg[256];
            std::snprintf(msg, sizeof(msg),
                          "eigensolver round %d: degree %lld, cut %.3e, bound %.3e, smallest Ritz value %.6e, "
                          "largest wanted residual %.3e",
                          iters, (long long)m, a, bound, theta[0], worst);
            log(ctx, TK_LOG_DEBUG, msg);
        }
    }
    // signs: the entry of largest magnitude of each returned vector is positive
    const int nb = (int)std::max<int64_t>(1, std::min<int64_t>((N + EG_THREADS - 1) / EG_THREADS, 1024));
    double* pv = (double*)ctx->scratch.get("eig.colmax_v", sizeof(double) * (size_t)nb * td);
    int64_t* pi = (int64_t*)ctx->scratch.get("eig.colmax_i", sizeof(int64_t) * (size_t)nb * td);
    k_colmax<BW><<<dim3(nb, td), EG_THREADS, 0, ctx->stream>>>(N, X, skip, pv, pi);
    TK_CHECK_LAUNCH();
    std::vector<double> hv((size_t)nb * td);
    std::vector<int64_t> hi((size_t)nb * td);
    TK_CUDA(cudaMemcpyAsync(hv.data(), pv, sizeof(double) * hv.size(), cudaMemcpyDeviceToHost, ctx->stream));
    TK_CUDA(cudaMemcpyAsync(hi.data(), pi, sizeof(int64_t) * hi.size(), cudaMemcpyDeviceToHost, ctx->stream));
    TK_CUDA(cudaStreamSynchronize(ctx->stream));
    Signs sg{};
    std::vector<int64_t> arg(td, 0);
    for (int c = 0; c < td; ++c)
    {
        double bv = -1.0;
        int64_t bi = 0;
        for (int b = 0; b < nb; ++b)
        {
            const double v = hv[(size_t)c * nb + b];
            const int64_t i = hi[(size_t)c * nb + b];
            if (v > bv || (v == bv && i < bi))
            {
                bv = v;
                bi = i;
            }
        }
        arg[c] = bi;
    }
    // the sign of X[arg, skip + c]: read those entries back
    for (int c = 0; c < td; ++c)
    {
        float2 e;
        TK_CUDA(cudaMemcpyAsync(&e, X + arg[c] * BW + skip + c, sizeof(float2), cudaMemcpyDeviceToHost, ctx->stream));
        TK_CUDA(cudaStreamSynchronize(ctx->stream));
        sg.s[c] = ((double)e.x + (double)e.y) < 0.0 ? -1.0 : 1.0;
    }
    k_write_vectors<BW><<<(int)std::min<int64_t>((N * td + 255) / 256, 8192), 256, 0, ctx->stream>>>(N, X, skip, td,
                                                                                                    sg, vectors);
    TK_CHECK_LAUNCH();
    TK_CUDA(cudaMemcpyAsync(values, theta.data() + skip, sizeof(double) * td, cudaMemcpyHostToDevice, ctx->stream));
    double mres = 0.0;
    for (int j = skip; j < want; ++j)
        mres = std::max(mres, res[j]);
    info->iterations = iters;
    info->block = BW;
    info->matvecs = matvecs;
    info->spectrum_bound = bound;
    info->max_residual = mres;
    info->converged = converged ? 1 : 0;
}

} // namespace

void check_csr_rows(tk_ctx* ctx, int64_t N, const int64_t* row_ptr, int64_t nnz)
{
    k_check_rows<<<(int)std::max<int64_t>(1, std::min<int64_t>((N + 256) / 256, 4096)), 256, 0, ctx->stream>>>(
        N, row_ptr, nnz, ctx->dev_err);
    TK_CHECK_LAUNCH();
}

int eigen_block_width(int td, int skip)
{
    const int want = td + skip;
    // 32 columns: the guard vectors beyond td + skip raise the damped interval's
    // lower end a, and the products needed fall as sqrt(B / a) -- on the lifted roll
    // (N = 20000, D = 64, k = 16) 6.6k block products of 32 columns against 28k of 16
    return want <= 14 ? 32 : 0;
}

void smallest_eigenvectors(tk_ctx* ctx, int64_t N, int64_t nnz, const int64_t* row_ptr, const int32_t* col_idx,
                           const double* vals, int td, int skip, double tol, int64_t max_matvecs, double* vectors,
                           double* values, tk_eig_info* info)
{
    const int BW = eigen_block_width(td, skip);
    float2* vff = (float2*)ctx->scratch.get("eig.vff", sizeof(float2) * (size_t)std::max<int64_t>(nnz, 1));
    if (nnz > 0)
    {
        k_vals_split<<<(int)std::min<int64_t>((nnz + 255) / 256, 8192), 256, 0, ctx->stream>>>(nnz, vals, vff);
        TK_CHECK_LAUNCH();
    }
    unsigned long long* gb = (unsigned long long*)ctx->scratch.get("eig.gersh", sizeof(unsigned long long));
    TK_CUDA(cudaMemsetAsync(gb, 0, sizeof(unsigned long long), ctx->stream));
    k_gershgorin<<<(int)std::max<int64_t>(1, std::min<int64_t>((N + 7) / 8, (int64_t)ctx->num_sms * 8)), 256, 0,
                   ctx->stream>>>(N, row_ptr, vals, gb);
    TK_CHECK_LAUNCH();
    unsigned long long gbits = 0;
    TK_CUDA(cudaMemcpyAsync(&gbits, gb, sizeof(gbits), cudaMemcpyDeviceToHost, ctx->stream));
    TK_CUDA(cudaStreamSynchronize(ctx->stream));
    double gersh;
    std::memcpy(&gersh, &gbits, sizeof(double));
    const Csr A{N, row_ptr, col_idx, vff};
    const double lz = 1.05 * lanczos_bound(ctx, A, 0x51D3E2F1ull);
    double bound = std::min(gersh, lz);
    if (!(bound > 0.0))
        bound = std::max(gersh, 1e-300);
    std::memset(info, 0, sizeof(*info));
    if (BW == 16)
        run_solver<16>(ctx, A, bound, td, skip, tol, max_matvecs, vectors, values, info);
    else
        run_solver<32>(ctx, A, bound, td, skip, tol, max_matvecs, vectors, values, info);
}

} // namespace tk
