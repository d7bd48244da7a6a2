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
// normalisation. The scatter accumulates into dL/dX with FP64 atomics.
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

// dL/dX from mu, w and the neighbour differences; one warp per point, lanes
// over dimensions.
__global__ void __launch_bounds__(G_WARPS * 32)
    k_lle_scatter(const void* X, int dtype, int64_t N, int D, int64_t ldx, const int32_t* __restrict__ idx, int k,
                  double klle_shift, const double* __restrict__ W, const double* __restrict__ MU,
                  double* __restrict__ gX, unsigned* err)
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
                atomicOr(err, DEV_ERR_BOUNDS);
            continue;
        }
        const double c2 = 2.0 * klle_shift * mw;
        for (int d0 = 0; d0 < D; d0 += 32)
        {
            const int d = d0 + lane;
            if (d >= D)
                continue;
            const double xi = x_elem(X, dtype, i * ldx + d);
            double p = 0.0, q = 0.0;
            for (int a = 0; a < k; ++a)
            {
                const int64_t j = idx[i * k + a];
                const double z = x_elem(X, dtype, j * ldx + d) - xi;
                p = fma(W[i * k + a], z, p);
                q = fma(MU[i * k + a], z, q);
            }
            double sdz = 0.0;
            for (int a = 0; a < k; ++a)
            {
                const int64_t j = idx[i * k + a];
                const double z = x_elem(X, dtype, j * ldx + d) - xi;
                const double dz = -MU[i * k + a] * p - W[i * k + a] * q - c2 * z;
                atomicAdd(&gX[j * D + d], dz);
                sdz += dz;
            }
            atomicAdd(&gX[i * D + d], -sdz);
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
    TK_CUDA(cudaMemsetAsync(gX, 0, sizeof(double) * (size_t)N * D, st));
    k_lle_scatter<<<grid, G_WARPS * 32, 0, st>>>(X, dtype, N, D, ldx, idx, k, klle_shift, W, MU, gX, ctx->dev_err);
    TK_CHECK_LAUNCH();
}

} // namespace tk
