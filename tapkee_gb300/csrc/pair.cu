// pair.cu -- the dense eigenproblem pair (lhs, rhs) of NPE and LLTSA.
//
// construct_neighborhood_preserving_eigenproblem and
// construct_lltsa_eigenproblem (routines/locally_linear.hpp:257-338) turn the
// sparse alignment matrix M (from linear_weight_matrix or
// tangent_weight_matrix) and the feature vectors x_i (the rows of X for the
// linear kernel) into two D x D matrices for a generalized eigensolver:
//   rhs: the upper triangle of sum_i x_i x_i^T (LLTSA: minus s s^T / N with
//        s = sum_i x_i), then (rhs + rhs^T) / 2 -- the lower triangle is zero at
//        that point, so the off-diagonal entries end halved;
//   lhs: the upper triangle of sum over the nonzeros (i, j) of M of
//        M_ij (x_i x_j^T + x_j x_i^T) (LLTSA: minus s s^T / N); lower stays 0.
// Here Y = M X is formed first (one warp per row of the CSR), so that
// lhs = Y^T X + X^T Y on the upper triangle; both sums over the N rows are
// block partials in FP64 over fixed row ranges, added in a fixed order.
#include <cmath>

#include "tk_internal.h"

namespace tk {
namespace {

constexpr int PAIR_RC = 32;       // rows staged per step
constexpr int PAIR_EPT = 8;       // upper-triangle entries per thread
constexpr int PAIR_THREADS = 256;
constexpr int PAIR_EB = PAIR_EPT * PAIR_THREADS;  // entries per CTA column of the grid

__device__ __forceinline__ double x_at(const void* X, int dtype, int64_t off)
{
    return dtype == TK_F64 ? reinterpret_cast<const double*>(X)[off] : (double)reinterpret_cast<const float*>(X)[off];
}

// column-major upper-triangle index e -> (a, b), a <= b, e = b (b + 1) / 2 + a
__device__ __forceinline__ void upper_ab(int e, int& a, int& b)
{
    int bb = (int)((sqrt(8.0 * (double)e + 1.0) - 1.0) * 0.5);
    while (bb * (bb + 1) / 2 > e)
        --bb;
    while ((bb + 1) * (bb + 2) / 2 <= e)
        ++bb;
    b = bb;
    a = e - bb * (bb + 1) / 2;
}

// Y = M X: one warp per row c of the CSR, lanes over the dimensions.
__global__ void k_spmm_rows(int64_t N, int D, const void* X, int dtype, int64_t ldx, const int64_t* __restrict__ rp,
                            const int32_t* __restrict__ col, const double* __restrict__ val, double* Y,
                            unsigned* err)
{
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t c = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < N; c += nw)
    {
        for (int d0 = 0; d0 < D; d0 += 32)
        {
            const int d = d0 + lane;
            double acc = 0.0;
            for (int64_t p = rp[c]; p < rp[c + 1]; ++p)
            {
                const int r = col[p];
                if (r < 0 || r >= N)
                {
                    if (lane == 0)
                        atomicOr(err, DEV_ERR_BOUNDS);
                    continue;
                }
                if (d < D)
                    acc = fma(val[p], x_at(X, dtype, (int64_t)r * ldx + d), acc);
            }
            if (d < D)
                Y[c * D + d] = acc;
        }
    }
}

// Block partials over rows [rb * rows_per, ...): for the upper entries of this
// grid column, P1 = sum_c (y_ca x_cb + x_ca y_cb) and P2 = sum_c x_ca x_cb; the
// first grid column also sums x_c (column sums s).
__global__ void __launch_bounds__(PAIR_THREADS) k_pair_partial(int64_t N, int D, const void* X, int dtype, int64_t ldx,
                                                               const double* __restrict__ Y, int64_t rows_per,
                                                               double* p1, double* p2, double* ps)
{
    extern __shared__ double sm[];
    double* xs = sm;                  // PAIR_RC x D
    double* ys = sm + PAIR_RC * D;    // PAIR_RC x D
    const int t = threadIdx.x;
    const int NE = D * (D + 1) / 2;
    const int rb = blockIdx.x;
    const int64_t r0 = (int64_t)rb * rows_per, r1 = min(N, r0 + rows_per);
    int ea[PAIR_EPT], eb[PAIR_EPT];
    bool on[PAIR_EPT];
#pragma unroll
    for (int m = 0; m < PAIR_EPT; ++m)
    {
        const int e = blockIdx.y * PAIR_EB + t + PAIR_THREADS * m;
        on[m] = e < NE;
        ea[m] = eb[m] = 0;
        if (on[m])
            upper_ab(e, ea[m], eb[m]);
    }
    double a1[PAIR_EPT], a2[PAIR_EPT];
#pragma unroll
    for (int m = 0; m < PAIR_EPT; ++m)
        a1[m] = a2[m] = 0.0;
    double sacc = 0.0;
    for (int64_t c0 = r0; c0 < r1; c0 += PAIR_RC)
    {
        const int nr = (int)min((int64_t)PAIR_RC, r1 - c0);
        __syncthreads();
        for (int q = t; q < nr * D; q += PAIR_THREADS)
        {
            const int rr = q / D, d = q - rr * D;
            xs[rr * D + d] = x_at(X, dtype, (c0 + rr) * ldx + d);
            ys[rr * D + d] = Y[(c0 + rr) * D + d];
        }
        __syncthreads();
        for (int rr = 0; rr < nr; ++rr)
        {
#pragma unroll
            for (int m = 0; m < PAIR_EPT; ++m)
            {
                const double xa = xs[rr * D + ea[m]], xb = xs[rr * D + eb[m]];
                const double ya = ys[rr * D + ea[m]], yb = ys[rr * D + eb[m]];
                a1[m] = fma(ya, xb, fma(xa, yb, a1[m]));
                a2[m] = fma(xa, xb, a2[m]);
            }
            if (blockIdx.y == 0 && t < D)
                sacc += xs[rr * D + t];
        }
    }
#pragma unroll
    for (int m = 0; m < PAIR_EPT; ++m)
        if (on[m])
        {
            const int e = blockIdx.y * PAIR_EB + t + PAIR_THREADS * m;
            p1[(int64_t)rb * NE + e] = a1[m];
            p2[(int64_t)rb * NE + e] = a2[m];
        }
    if (blockIdx.y == 0 && t < D)
        ps[(int64_t)rb * D + t] = sacc;
}

// Sums the partials in row-block order and writes lhs / rhs (column-major).
__global__ void k_pair_final(int kind, int64_t N, int D, int nrb, const double* __restrict__ p1,
                             const double* __restrict__ p2, const double* __restrict__ ps, double* lhs, double* rhs)
{
    const int NE = D * (D + 1) / 2;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < NE; e += gridDim.x * blockDim.x)
    {
        int a, b;
        upper_ab(e, a, b);
        double L = 0.0, R = 0.0;
        for (int rb = 0; rb < nrb; ++rb)
        {
            L += p1[(int64_t)rb * NE + e];
            R += p2[(int64_t)rb * NE + e];
        }
        if (kind == TK_PAIR_LLTSA)
        {
            double sa = 0.0, sb = 0.0;
            for (int rb = 0; rb < nrb; ++rb)
            {
                sa += ps[(int64_t)rb * D + a];
                sb += ps[(int64_t)rb * D + b];
            }
            const double u = -1.0 / (double)N * sa * sb;
            L += u;
            R += u;
        }
        lhs[(int64_t)b * D + a] = L;
        if (a != b)
        {
            lhs[(int64_t)a * D + b] = 0.0;
            rhs[(int64_t)b * D + a] = R / 2.0;
            rhs[(int64_t)a * D + b] = R / 2.0;
        }
        else
            rhs[(int64_t)b * D + a] = R;
    }
}

} // namespace

void eigenproblem_pair(tk_ctx* ctx, int kind, const void* X, int dtype, int64_t N, int D, int64_t ldx,
                       const int64_t* row_ptr, const int32_t* col_idx, const double* vals, double* lhs, double* rhs)
{
    cudaStream_t st = ctx->stream;
    const int NE = D * (D + 1) / 2;
    double* Y = (double*)ctx->scratch.get("pair.y", sizeof(double) * (size_t)N * D);
    const int64_t warps = std::min<int64_t>(N, (int64_t)ctx->num_sms * 64);
    k_spmm_rows<<<(int)((warps + 7) / 8), 256, 0, st>>>(N, D, X, dtype, ldx, row_ptr, col_idx, vals, Y,
                                                        ctx->dev_err);
    TK_CHECK_LAUNCH();
    const int nrb = (int)std::max<int64_t>(1, std::min<int64_t>((N + 1023) / 1024, (int64_t)ctx->num_sms * 2));
    const int64_t rows_per = (N + nrb - 1) / nrb;
    const int neb = (NE + PAIR_EB - 1) / PAIR_EB;
    double* p1 = (double*)ctx->scratch.get("pair.p1", sizeof(double) * (size_t)nrb * NE);
    double* p2 = (double*)ctx->scratch.get("pair.p2", sizeof(double) * (size_t)nrb * NE);
    double* ps = (double*)ctx->scratch.get("pair.ps", sizeof(double) * (size_t)nrb * D);
    const size_t smem = sizeof(double) * 2 * PAIR_RC * (size_t)D;
    TK_CUDA(cudaFuncSetAttribute(k_pair_partial, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_pair_partial<<<dim3(nrb, neb), PAIR_THREADS, smem, st>>>(N, D, X, dtype, ldx, Y, rows_per, p1, p2, ps);
    TK_CHECK_LAUNCH();
    k_pair_final<<<(NE + 255) / 256, 256, 0, st>>>(kind, N, D, nrb, p1, p2, ps, lhs, rhs);
    TK_CHECK_LAUNCH();
}

} // namespace tk
