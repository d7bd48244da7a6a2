// hessian.cu -- Hessian LLE weights: the per-point part of hessian_weight_matrix
// (routines/locally_linear.hpp:161-255), one warp per point.
//
// Per point the reference
//   1. builds the centred Gram of the neighbours and takes the eigenvectors V of
//      its td largest eigenvalues (:188-204) -- the LTSA basis, computed here by
//      ltsa_basis (FP32 Jacobi plus a float-float subspace refinement);
//   2. forms Yi = [1, V, v_j v_l for j <= l] (:203-214; dp = td (td + 1) / 2
//      product columns);
//   3. orthonormalises the columns of Yi in order, each column projected against
//      the earlier ones one at a time and then scaled to unit norm (:216-225);
//   4. divides a product column by its sum when that sum exceeds 1e-4 (:226-231);
//   5. emits B = Yr Yr^T, Yr the dp product columns, as triplets (n_a, n_b, B_ab)
//      (:234-243).
// Steps 2-4 run here in FP64 (a few hundred FP64 operations per point): lane l
// owns rows l and l + 32 of Yi. The output is Yr (N x k x dp); assembly forms B
// from it, as it forms LTSA's P from V.
//
// B is the projector onto the quadratic part of span[1, V, products]: a rotation
// or sign change of V changes the product columns only within their span, so the
// GPU basis (with its own signs) gives the reference's B. The reference's column
// placement `ct += ct + td - j` (:213) is right for td <= 2 only (for td = 3 it
// writes past the dp columns), so td is limited to 1 or 2.
#include <cmath>

#include "tk_internal.h"

namespace tk {
namespace {

constexpr int H_WARPS = 4;

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <int TD>
__global__ void __launch_bounds__(H_WARPS * 32)
    k_hessian(int64_t N, int k, const double* __restrict__ V, double* __restrict__ Y)
{
    constexpr int DP = TD * (TD + 1) / 2;
    constexpr int NC = 1 + TD + DP;
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = warp; i < N; i += nwarps)
    {
        double y[NC][2];
#pragma unroll
        for (int r = 0; r < 2; ++r)
        {
            const int a = lane + 32 * r;
            const bool in = a < k;
            y[0][r] = in ? 1.0 : 0.0;
#pragma unroll
            for (int t = 0; t < TD; ++t)
                y[1 + t][r] = in ? V[(i * k + a) * TD + t] : 0.0;
            // product columns in the reference's placement (td <= 2): column
            // ct + p + 1 + td holds y_{j+1} * y_{j+p+1}, ct advancing by ct + td - j
            int ct = 0;
#pragma unroll
            for (int j = 0; j < TD; ++j)
            {
#pragma unroll
                for (int p = 0; p < TD - j; ++p)
                    y[ct + p + 1 + TD][r] = y[j + 1][r] * y[j + p + 1][r];
                ct += ct + TD - j;
            }
        }
        // orthonormalise in column order (each projection uses the updated column)
#pragma unroll
        for (int c = 0; c < NC; ++c)
        {
#pragma unroll
            for (int j = 0; j < c; ++j)
            {
                const double rr = warp_sum(fma(y[c][0], y[j][0], y[c][1] * y[j][1]));
                y[c][0] = fma(-rr, y[j][0], y[c][0]);
                y[c][1] = fma(-rr, y[j][1], y[c][1]);
            }
            const double nrm = sqrt(warp_sum(fma(y[c][0], y[c][0], y[c][1] * y[c][1])));
            const double inv = 1.0 / nrm;
            y[c][0] *= inv;
            y[c][1] *= inv;
        }
        // column-sum normalisation of the product columns
#pragma unroll
        for (int q = 0; q < DP; ++q)
        {
            const double s = warp_sum(y[1 + TD + q][0] + y[1 + TD + q][1]);
            if (s > 1e-4)
            {
                y[1 + TD + q][0] /= s;
                y[1 + TD + q][1] /= s;
            }
        }
#pragma unroll
        for (int r = 0; r < 2; ++r)
        {
            const int a = lane + 32 * r;
            if (a < k)
#pragma unroll
                for (int q = 0; q < DP; ++q)
                    Y[(i * k + a) * DP + q] = y[1 + TD + q][r];
        }
    }
}

} // namespace

void hessian_basis(tk_ctx* ctx, const void* X, int dtype, int64_t N, int D, int64_t ldx, const int32_t* idx, int k,
                   int td, double* Y)
{
    if (td < 1 || td > 2)
        throw Error(TK_ERR_UNSUPPORTED, "Hessian LLE supports target_dimension 1 or 2 (the reference places the "
                                        "product columns correctly only for those)");
    if (k > 64)
        throw Error(TK_ERR_UNSUPPORTED, "Hessian LLE supports up to 64 neighbours");
    if (k <= td + td * (td + 1) / 2)
        throw Error(TK_ERR_INVALID_ARG, "Hessian LLE needs more neighbours than 1 + td + td (td + 1) / 2");
    double* V = (double*)ctx->scratch.get("hess.V", sizeof(double) * (size_t)N * k * td);
    ltsa_basis(ctx, X, dtype, N, D, ldx, idx, k, td, V);
    const int grid = (int)std::min<int64_t>((N + H_WARPS - 1) / H_WARPS, (int64_t)ctx->num_sms * 32);
    if (td == 1)
        k_hessian<1><<<grid, H_WARPS * 32, 0, ctx->stream>>>(N, k, V, Y);
    else
        k_hessian<2><<<grid, H_WARPS * 32, 0, ctx->stream>>>(N, k, V, Y);
    TK_CHECK_LAUNCH();
}

} // namespace tk
