// lle_grad.cu -- adjoint of the LLE weight solve (reverse-mode derivative of
// W(X) with the neighbour sets held fixed).
//
// Per point i with neighbours n_a, Z_a = n_a - x_i, C = Z Z^T,
// C_r = C + s tr(C) I (s = klle_shift), u = C_r^{-1} 1, w = u / (1^T u).
// Given g = dL/dw:
//   dL/du        = (g - (g.w) 1) / (1^T u)
//   dL/dC_r      = -C_r^{-1} (dL/du) u^T  = -mu w^T,   mu = C_r^{-1} (g - (g.w) 1)
//   dL/dC        = H = dL/dC_r + s tr(dL/dC_r) I = -mu w^T - s (mu.w) I
//   dL/dZ_a      = sum_b (H + H^T)_ab Z_b = -mu_a p - w_a q - 2 s (mu.w) Z_a,
//                  p = sum_b w_b Z_b,  q = sum_b mu_b Z_b
//   dL/dn_a     += dL/dZ_a,   dL/dx_i -= sum_a dL/dZ_a.
// mu comes from the same solve kernel as the weights (FP32 Cholesky refined
// against float-float residuals), with the right-hand side g - (g.w) 1 and no
// normalisation. dL/dX is then a pull, so it is bit-reproducible: k_grad_pq
// stores p_i, q_i and 2 s (mu.w)_i per point, and every output row j sums, in a
// fixed order, its own term -sum_a dL/dZ_{j,a} and then the dL/dZ_{i,a} of every
// edge (i, a) with n_a = j, in ascending i (the reverse lists of assembly).
// The reference has no derivative of this stage; the operator it differentiates
// is linear_weight_matrix's solve (routines/locally_linear.hpp:117-131).
#include "tk_internal.h"

namespace tk {
namespace {

constexpr int G_WARPS = 8;

__device__ __forceinline__ double x_elem(const void* X, int dtype, int64_t off)
{
    return dtype == TK_F64 ? reinterpret_cast<const double*>(X)[off] : (double)reinterpret_cast<const float*>(X)[off];
}

// b = g - (g.w) 1, one warp per point.
__global__ void __launch_bounds__(G_WARPS * 32) k_adjoint_rhs(int64_t N, int k, const double* __restrict__ W,
                                                               const double* __restrict__ G, double* __restrict__ B)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = warp; i < N; i += nwarps)
    {
        double gw = 0.0;
        for (int a = lane; a < k; a += 32)
            gw = fma(G[i * k + a], W[i * k + a], gw);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            gw += __shfl_xor_sync(0xffffffffu, gw, o);
        for (int a = lane; a < k; a += 32)
            B[i * k + a] = G[i * k + a] - gw;
    }
}

// p_i = sum_b w_b Z_b, q_i = sum_b mu_b Z_b (N x D each) and c2_i = 2 s (mu.w)_i;
// one warp per point, lanes over dimensions. A point with a neighbour index
// outside [0, N) raises DEV_ERR_BOUNDS and gets c2 = NaN, p = q = 0.
__global__ void __launch_bounds__(G_WARPS * 32)
    k_grad_pq(const void* X, int dtype, int64_t N, int D, int64_t ldx, const int32_t* __restrict__ idx, int k,
              double klle_shift, const double* __restrict__ W, const double* __restrict__ MU, double* __restrict__ P,
              double* __restrict__ Q, double* __restrict__ C2, unsigned* err)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = warp; i < N; i += nwarps)
    {
        double mw = 0.0;
        bool bad = false;
        for (int a = lane; a < k; a += 32)
        {
            mw = fma(MU[i * k + a], W[i * k + a], mw);
            const int j = idx[i * k + a];
            bad |= (j < 0 || j >= N);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            mw += __shfl_xor_sync(0xffffffffu, mw, o);
        if (__any_sync(0xffffffffu, bad))
        {
            if (lane == 0)
            {
                atomicOr(err, DEV_ERR_BOUNDS);
                C2[i] = __longlong_as_double(0x7ff8000000000000ll);
            }
            for (int d = lane; d < D; d += 32)
                P[i * D + d] = Q[i * D + d] = 0.0;
            continue;
        }
        if (lane == 0)
            C2[i] = 2.0 * klle_shift * mw;
        for (int d = lane; d < D; d += 32)
        {
            const double xi = x_elem(X, dtype, i * ldx + d);
            double p = 0.0, q = 0.0;
            for (int a = 0; a < k; ++a)
            {
                const int64_t j = idx[i * k + a];
                const double z = x_elem(X, dtype, j * ldx + d) - xi;
                p = fma(W[i * k + a], z, p);
                q = fma(MU[i * k + a], z, q);
            }
            P[i * D + d] = p;
            Q[i * D + d] = q;
        }
    }
}

// dL/dx_j (FP64, row stride D): one warp per output point, lanes over
// dimensions; dL/dZ_{i,a} = -mu_ia p_i - w_ia q_i - c2_i Z_{i,a}.
__global__ void __launch_bounds__(G_WARPS * 32)
    k_grad_pull(const void* X, int dtype, int64_t N, int D, int64_t ldx, const int32_t* __restrict__ idx, int k,
                const double* __restrict__ W, const double* __restrict__ MU, const double* __restrict__ P,
                const double* __restrict__ Q, const double* __restrict__ C2, const int64_t* __restrict__ rptr,
                const int32_t* __restrict__ rev, double* __restrict__ gX)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t j = warp; j < N; j += nwarps)
    {
        const double c2j = C2[j];
        const int64_t r0 = rptr[j], r1 = rptr[j + 1];
        for (int d = lane; d < D; d += 32)
        {
            const double xj = x_elem(X, dtype, j * ldx + d);
            double acc = 0.0;
            if (c2j == c2j)  // the point's own edges (its neighbour indices were valid)
                for (int a = 0; a < k; ++a)
                {
                    const int64_t n = idx[j * k + a];
                    const double z = x_elem(X, dtype, n * ldx + d) - xj;
                    acc += MU[j * k + a] * P[j * D + d] + W[j * k + a] * Q[j * D + d] + c2j * z;
                }
            for (int64_t e = r0; e < r1; ++e)
            {
                const int64_t ed = rev[e];
                const int64_t i = ed / k;
                const double c2i = C2[i];
                if (c2i != c2i)
                    continue;
                const double z = xj - x_elem(X, dtype, i * ldx + d);
                acc -= MU[ed] * P[i * D + d] + W[ed] * Q[i * D + d] + c2i * z;
            }
            gX[j * D + d] = acc;
        }
    }
}

} // namespace

void lle_weights_grad(tk_ctx* ctx, const void* X, int dtype, int64_t N, int D, int64_t ldx, const int32_t* idx, int k,
                      double klle_shift, const double* W, const double* G, double* gX)
{
    cudaStream_t st = ctx->stream;
    double* B = (double*)ctx->scratch.get("lleg.rhs", sizeof(double) * (size_t)N * k);
    double* MU = (double*)ctx->scratch.get("lleg.mu", sizeof(double) * (size_t)N * k);
    const int grid = (int)std::min<int64_t>((N + G_WARPS - 1) / G_WARPS, (int64_t)ctx->num_sms * 16);
    k_adjoint_rhs<<<grid, G_WARPS * 32, 0, st>>>(N, k, W, G, B);
    TK_CHECK_LAUNCH();
    lle_solve(ctx, X, dtype, N, D, ldx, idx, k, klle_shift, B, false, MU);
    double* P = (double*)ctx->scratch.get("lleg.p", sizeof(double) * (size_t)N * D);
    double* Q = (double*)ctx->scratch.get("lleg.q", sizeof(double) * (size_t)N * D);
    double* C2 = (double*)ctx->scratch.get("lleg.c2", sizeof(double) * (size_t)N);
    int64_t* rptr = (int64_t*)ctx->scratch.get("lleg.rptr", sizeof(int64_t) * (size_t)(N + 1));
    int32_t* rev = (int32_t*)ctx->scratch.get("lleg.rev", sizeof(int32_t) * (size_t)N * k);
    k_grad_pq<<<grid, G_WARPS * 32, 0, st>>>(X, dtype, N, D, ldx, idx, k, klle_shift, W, MU, P, Q, C2, ctx->dev_err);
    TK_CHECK_LAUNCH();
    reverse_lists(ctx, N, k, idx, rptr, rev);
    k_grad_pull<<<grid, G_WARPS * 32, 0, st>>>(X, dtype, N, D, ldx, idx, k, W, MU, P, Q, C2, rptr, rev, gX);
    TK_CHECK_LAUNCH();
}

} // namespace tk
