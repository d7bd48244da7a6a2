// ltsa.cu -- LTSA local tangent bases, one warp per point.
//
// Per point with neighbours n_0..n_{k-1} (routines/locally_linear.hpp:45-63):
//   K_ab = k(n_a, n_b), double-centred (centerMatrix, utils/matrix.hpp:12-19),
//   V    = eigenvectors of the td largest eigenvalues,
// and the alignment block is P = (1/k) 1 1^T + V V^T (G = [1/sqrt(k) 1, V]).
// The double-centred Gram equals Zc Zc^T with Zc the neighbours minus their
// mean, which is what is accumulated here (in FP32, from FP64-centred
// coordinates, avoiding the cancellation of the raw kernel form). The
// eigen-decomposition is a cyclic Jacobi in shared memory with the round-robin
// (tournament) ordering: each round applies k/2 disjoint rotations in parallel.
// Points whose gap lambda_td - lambda_{td+1} is below 1e-6 of lambda_max have an
// ill-conditioned tangent space; they are redone with an FP64 Jacobi.
#include <cfloat>
#include <cmath>
#include <type_traits>

#include "ff.cuh"
#include "tk_internal.h"

namespace tk {
namespace {

// TD bounds the basis width td (the refinement's arrays): 2, 4 or 8. The float
// kernel takes the smallest that fits td, which keeps its shared memory, and so
// its warps per SM, in step with the basis actually asked for.
// One rotation of a Jacobi round: rows/columns (p, q), cosine and sine.
template <typename T>
struct alignas(2 * sizeof(T)) JacobiRot
{
    int p, q;
    T c, s;
};

template <int M, typename T, int TD = 8>
struct JacobiSmem
{
    T A[M][M + 1];
    T VT[M][M + 2];  // eigenvectors as rows (VT[j][a] = V[a][j]); even stride: 8-byte pairs
    JacobiRot<T> rot[M / 2];
    float Z[M][33];
    float Zl[M][33];     // low parts of the centred coordinates
    float th[32][TD], tl[32][TD];  // t = Zc^T V for one chunk, float-float
    float Vf[M][TD];      // FP32 top eigenvectors
    float GVh[M][TD], GVl[M][TD];  // G V, float-float
    float Rf[M][TD];      // residual G V - V Lam
    float UR[M][TD];      // (u_j . R_t) / (Lam_t - lambda_j)
    float Oh[M][TD], Ol[M][TD];    // refined basis, float-float
    float Lh[TD][TD], Ll[TD][TD];    // Rayleigh quotient V^T G V, float-float
};

// x as a float pair (exact for float32 input, hi + lo split for float64)
__device__ __forceinline__ ff x_ff(const void* X, int dtype, int64_t off)
{
    if (dtype == TK_F64)
    {
        const double v = reinterpret_cast<const double*>(X)[off];
        const float h = (float)v;
        return ff{h, (float)(v - (double)h)};
    }
    return ff{reinterpret_cast<const float*>(X)[off], 0.f};
}

// Coordinates of the neighbours of one point in dimensions [d0, d0 + 32),
// centred on their mean, in float-float: Z[a][lane] + Zl[a][lane] = x_{n_a} -
// mean for d = d0 + lane (zero for a >= k or d >= D).
template <int M, typename T, int TD>
__device__ __forceinline__ void stage_centred(JacobiSmem<M, T, TD>& S, int lane, const void* X, int dtype, int64_t ldx,
                                              int D, const int32_t* nbrs, int k, int d0)
{
    const int d = d0 + lane;
    ff sum = ff_zero();
    if (d < D)
        for (int a = 0; a < k; ++a)
            sum = ff_add(sum, x_ff(X, dtype, (int64_t)nbrs[a] * ldx + d));
    const ff mean = ff_div_f(sum, (float)k);
    for (int a = 0; a < M; ++a)
    {
        ff z = ff_zero();
        if (a < k && d < D)
            z = ff_add(x_ff(X, dtype, (int64_t)nbrs[a] * ldx + d), ff_neg(mean));
        S.Z[a][lane] = z.hi;
        S.Zl[a][lane] = z.lo;
    }
}

// Parallel cyclic Jacobi on the symmetric M x M matrix S.A (one warp). On exit
// diag(A) holds the eigenvalues and the columns of V the eigenvectors.
// A round applies M/2 disjoint rotations G = [[c, -s], [s, c]] at once:
// A <- G A G^T, V <- V G^T. With the indices grouped by rotation, every 2 x 2
// block B of A (rows of rotation i, columns of rotation j) becomes
// G_i B G_j^T, independently of every other block; a lane updates whole blocks
// of the upper triangle (i <= j) and writes both triangles, so one pass over
// the blocks replaces a row pass and a column pass. A diagonal block's
// off-diagonal entry, which its rotation annihilates, is set to zero.
template <int M, typename T, int TD>
__device__ void warp_jacobi(JacobiSmem<M, T, TD>& S, int lane, int max_sweeps)
{
    constexpr int H = M / 2;             // rotations per round
    constexpr int NB = H * (H + 1) / 2;  // blocks (i <= j)
    constexpr int NBR = (NB + 31) / 32;  // blocks per lane
    constexpr int NV = M * H;            // (row of V, rotation) pairs
    constexpr int NVR = (NV + 31) / 32;
    constexpr int NV2 = H * (M / 2);     // (rotation, pair of rows of V) for FP32
    constexpr int NVR2 = (NV2 + 31) / 32;
    // this lane's blocks: e = lane + 32 r in row-major order of the upper triangle
    int bi[NBR], bj[NBR];
#pragma unroll
    for (int r = 0; r < NBR; ++r)
    {
        int e = lane + 32 * r, i = 0;
        bi[r] = -1;
        bj[r] = 0;
        if (e < NB)
        {
            while (e >= H - i)
            {
                e -= H - i;
                ++i;
            }
            bi[r] = i;
            bj[r] = i + e;
        }
    }
    for (int t = lane; t < M * M; t += 32)
        S.VT[t / M][t % M] = (t / M == t % M) ? T(1) : T(0);
    __syncwarp();
    for (int sweep = 0; sweep < max_sweeps; ++sweep)
    {
        // convergence test: off-diagonal vs diagonal mass
        T off = 0, dia = 0;
        for (int t = lane; t < M * M; t += 32)
        {
            const T v = S.A[t / M][t % M];
            if (t / M == t % M)
                dia += v * v;
            else
                off += v * v;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
        {
            off += __shfl_xor_sync(0xffffffffu, off, o);
            dia += __shfl_xor_sync(0xffffffffu, dia, o);
        }
        // stop when the off-diagonal mass reaches the rounding floor of the
        // working precision: rotations leave off-diagonal entries of order
        // eps |A|, so off / dia cannot fall much below (M eps)^2; (8 M eps)^2
        // sits safely above that floor (FP32: ~1e-10 at M = 20, enough for the
        // float-float refinement that follows)
        const T eps = sizeof(T) == 8 ? T(1.1102230246251565e-16) : T(5.9604644775390625e-08);
        const T tol = (T(8 * M) * eps) * (T(8 * M) * eps);
        if (off <= tol * dia || dia == T(0))
            break;
        for (int round = 0; round < M - 1; ++round)
        {
            if (lane < H)
            {
                auto pos = [&](int t) { return t == 0 ? 0 : 1 + ((t - 1 + round) % (M - 1)); };
                int p = pos(lane), q = pos(M - 1 - lane);
                if (p > q)
                {
                    const int tmp = p;
                    p = q;
                    q = tmp;
                }
                const T apq = S.A[p][q], app = S.A[p][p], aqq = S.A[q][q];
                T c = T(1), s = T(0);
                if (apq != T(0))
                {
                    const T theta = (aqq - app) / (T(2) * apq);
                    const T tt = (theta >= T(0) ? T(1) : T(-1)) / (fabs(theta) + sqrt(theta * theta + T(1)));
                    // c^2 + s^2 = 1 to the rounding of c either way; FP32 takes
                    // the hardware reciprocal square root (2 ulp) for 1 / sqrt
                    if constexpr (sizeof(T) == 4)
                        c = rsqrtf(fmaf(tt, tt, 1.f));
                    else
                        c = T(1) / sqrt(tt * tt + T(1));
                    s = tt * c;
                }
                S.rot[lane] = JacobiRot<T>{p, q, c, s};
            }
            __syncwarp();
            // A: the blocks of the upper triangle, both triangles written
#pragma unroll
            for (int r = 0; r < NBR; ++r)
            {
                if (bi[r] < 0)
                    continue;
                const JacobiRot<T> ri = S.rot[bi[r]], rj = S.rot[bj[r]];
                const T b00 = S.A[ri.p][rj.p], b01 = S.A[ri.p][rj.q];
                const T b10 = S.A[ri.q][rj.p], b11 = S.A[ri.q][rj.q];
                // X = B G_j^T, then Y = G_i X
                const T x00 = b00 * rj.c - b01 * rj.s, x01 = b00 * rj.s + b01 * rj.c;
                const T x10 = b10 * rj.c - b11 * rj.s, x11 = b10 * rj.s + b11 * rj.c;
                const T y00 = ri.c * x00 - ri.s * x10, y10 = ri.s * x00 + ri.c * x10;
                T y01 = ri.c * x01 - ri.s * x11;
                T y10w = y10;
                const T y11 = ri.s * x01 + ri.c * x11;
                if (bi[r] == bj[r])
                {
                    y01 = T(0);
                    y10w = T(0);
                }
                S.A[ri.p][rj.p] = y00;
                S.A[ri.p][rj.q] = y01;
                S.A[ri.q][rj.p] = y10w;
                S.A[ri.q][rj.q] = y11;
                if (bi[r] != bj[r])
                {
                    S.A[rj.p][ri.p] = y00;
                    S.A[rj.q][ri.p] = y01;
                    S.A[rj.p][ri.q] = y10w;
                    S.A[rj.q][ri.q] = y11;
                }
            }
            // V <- V G^T, i.e. rows p and q of VT: rotation i, entries (2 a2, 2 a2 + 1)
            if constexpr (sizeof(T) == 4)
            {
#pragma unroll
                for (int r = 0; r < NVR2; ++r)
                {
                    const int e = lane + 32 * r;
                    if (e < NV2)
                    {
                        const int i = e / (M / 2), a = 2 * (e % (M / 2));
                        const JacobiRot<T> ri = S.rot[i];
                        const float2 c2 = make_float2(ri.c, ri.c), s2 = make_float2(ri.s, ri.s);
                        float2* pp = reinterpret_cast<float2*>(&S.VT[ri.p][a]);
                        float2* qq = reinterpret_cast<float2*>(&S.VT[ri.q][a]);
                        const float2 vp = *pp, vq = *qq;
                        *pp = __ffma2_rn(c2, vp, __fmul2_rn(make_float2(-ri.s, -ri.s), vq));
                        *qq = __ffma2_rn(s2, vp, __fmul2_rn(c2, vq));
                    }
                }
            }
            else
            {
#pragma unroll
                for (int r = 0; r < NVR; ++r)
                {
                    const int e = lane + 32 * r;
                    if (e < NV)
                    {
                        const int a = e / H, i = e % H;
                        const JacobiRot<T> ri = S.rot[i];
                        const T vp = S.VT[ri.p][a], vq = S.VT[ri.q][a];
                        S.VT[ri.p][a] = ri.c * vp - ri.s * vq;
                        S.VT[ri.q][a] = ri.s * vp + ri.c * vq;
                    }
                }
            }
            __syncwarp();
        }
    }
}

// Builds the centred neighbour Gram of point i into S.A (type T, M x M, zero
// padded): FP32 products of the high parts for T = float (the refinement
// corrects what this drops), exact pair products in FP64 for T = double.
template <int M, typename T, int TD>
__device__ void centred_gram(JacobiSmem<M, T, TD>& S, int lane, const void* X, int dtype, int64_t ldx, int D,
                             const int32_t* nbrs, int k)
{
    for (int t = lane; t < M * M; t += 32)
        S.A[t / M][t % M] = T(0);
    __syncwarp();
    for (int d0 = 0; d0 < D; d0 += 32)
    {
        stage_centred<M, T>(S, lane, X, dtype, ldx, D, nbrs, k, d0);
        __syncwarp();
        for (int e = lane; e < M * M; e += 32)
        {
            const int a = e / M, b = e % M;
            if (b < a || a >= k || b >= k)
                continue;
            T s = T(0);
            for (int dd = 0; dd < 32; ++dd)
            {
                if (sizeof(T) == 8)
                    s += ((T)S.Z[a][dd] + (T)S.Zl[a][dd]) * ((T)S.Z[b][dd] + (T)S.Zl[b][dd]);
                else
                    s += (T)S.Z[a][dd] * (T)S.Z[b][dd];
            }
            S.A[a][b] += s;
            if (a != b)
                S.A[b][a] += s;
        }
        __syncwarp();
    }
}

// First-order refinement of the top-td invariant subspace. The FP32 Jacobi gives
// eigenpairs (lambda_j, u_j) of the FP32 Gram; the residual R = G V - V (V^T G V)
// of the exact Gram G = Zc Zc^T is formed in float-float from the exactly centred
// coordinates, and each top vector is corrected by
//     v_i += sum_{j not top} u_j (u_j . R_i) / (lambda_i - lambda_j),
// then the basis is re-orthonormalised (modified Gram-Schmidt) in float-float.
// This removes the FP32 Gram and Jacobi errors to first order (error ~ eps^2 /
// gap). Everything runs on the FP32 pipes; the result is S.Oh + S.Ol.
template <int M, int TD>
__device__ void refine_subspace(JacobiSmem<M, float, TD>& S, int lane, const void* X, int dtype, int64_t ldx, int D,
                                const int32_t* nbrs, int k, int td, const int* top)
{
    constexpr int RPL = (M + 31) / 32;  // basis rows per lane: a = lane + 32 r
    for (int e = lane; e < M * td; e += 32)
    {
        const int a = e / td, t = e % td;
        S.Vf[a][t] = (a < k) ? S.VT[top[t]][a] : 0.f;
    }
    __syncwarp();
    ff acc[RPL][TD];
#pragma unroll
    for (int r = 0; r < RPL; ++r)
        for (int t = 0; t < TD; ++t)
            acc[r][t] = ff_zero();
    for (int d0 = 0; d0 < D; d0 += 32)
    {
        stage_centred<M, float>(S, lane, X, dtype, ldx, D, nbrs, k, d0);
        __syncwarp();
        // t_d = sum_a z_ad v_a   (lane = d)
        for (int t = 0; t < td; ++t)
        {
            ff sacc = ff_zero();
            for (int a = 0; a < k; ++a)
                sacc = ff_fma(sacc, S.Z[a][lane], S.Zl[a][lane], S.Vf[a][t], 0.f);
            S.th[lane][t] = sacc.hi;
            S.tl[lane][t] = sacc.lo;
        }
        __syncwarp();
        // (G V)_a += sum_d z_ad t_d   (a = lane + 32 r)
#pragma unroll
        for (int r = 0; r < RPL; ++r)
        {
            const int a = lane + 32 * r;
            if (a < k)
                for (int dd = 0; dd < 32; ++dd)
                {
                    const float zh = S.Z[a][dd], zl = S.Zl[a][dd];
                    for (int t = 0; t < td; ++t)
                        acc[r][t] = ff_fma(acc[r][t], zh, zl, S.th[dd][t], S.tl[dd][t]);
                }
        }
        __syncwarp();
    }
#pragma unroll
    for (int r = 0; r < RPL; ++r)
    {
        const int a = lane + 32 * r;
        if (a < M)
            for (int t = 0; t < td; ++t)
            {
                S.GVh[a][t] = (a < k) ? acc[r][t].hi : 0.f;
                S.GVl[a][t] = (a < k) ? acc[r][t].lo : 0.f;
            }
    }
    __syncwarp();
    // Rayleigh quotient Lam = V^T G V (td x td)
    for (int e = lane; e < td * td; e += 32)
    {
        const int ii = e / td, jj = e % td;
        ff sacc = ff_zero();
        for (int a = 0; a < k; ++a)
            sacc = ff_fma(sacc, S.Vf[a][ii], 0.f, S.GVh[a][jj], S.GVl[a][jj]);
        S.Lh[ii][jj] = sacc.hi;
        S.Ll[ii][jj] = sacc.lo;
    }
    __syncwarp();
    // residual R = G V - V Lam, in float-float, kept in FP32
#pragma unroll
    for (int r = 0; r < RPL; ++r)
    {
        const int a = lane + 32 * r;
        if (a < M)
            for (int t = 0; t < td; ++t)
            {
                ff rr = ff{S.GVh[a][t], S.GVl[a][t]};
                for (int q = 0; q < td; ++q)
                    rr = ff_fma(rr, -S.Vf[a][q], 0.f, S.Lh[q][t], S.Ll[q][t]);
                S.Rf[a][t] = (a < k) ? rr.hi + rr.lo : 0.f;
            }
    }
    __syncwarp();
    // (u_j . R_t) / (Lam_t - lambda_j) for every non-top eigenvector (lanes over j)
    for (int j = lane; j < M; j += 32)
    {
        bool is_top = false;
        for (int t = 0; t < td; ++t)
            is_top |= (top[t] == j);
        const float lj = S.A[j][j];
        for (int t = 0; t < td; ++t)
        {
            float ur = 0.f;
            if (!is_top)
                for (int a = 0; a < k; ++a)
                    ur = fmaf(S.VT[j][a], S.Rf[a][t], ur);
            const float gap = S.Lh[t][t] - lj;
            S.UR[j][t] = (!is_top && gap != 0.f) ? ur / gap : 0.f;
        }
    }
    __syncwarp();
    // corrected basis (rows a = lane + 32 r), float-float
#pragma unroll
    for (int r = 0; r < RPL; ++r)
    {
        const int a = lane + 32 * r;
        if (a < M)
            for (int t = 0; t < td; ++t)
            {
                float c = 0.f;
                if (a < k)
                    for (int j = 0; j < M; ++j)
                        c = fmaf(S.VT[j][a], S.UR[j][t], c);
                const ff o = two_sum(S.Vf[a][t], c);
                S.Oh[a][t] = o.hi;
                S.Ol[a][t] = o.lo;
            }
    }
    __syncwarp();
    // modified Gram-Schmidt in float-float on the td columns
    for (int t = 0; t < td; ++t)
    {
        for (int q = 0; q <= t; ++q)
        {
            ff dot = ff_zero();
            for (int a = lane; a < k; a += 32)
                dot = ff_fma(dot, S.Oh[a][t], S.Ol[a][t], S.Oh[a][q], S.Ol[a][q]);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
                dot = ff_add(dot, ff_shfl_xor(dot, o));
            __syncwarp();
            if (q < t)
            {
                for (int a = lane; a < k; a += 32)
                {
                    const ff v = ff_add(ff{S.Oh[a][t], S.Ol[a][t]}, ff_neg(ff_mul(dot, ff{S.Oh[a][q], S.Ol[a][q]})));
                    S.Oh[a][t] = v.hi;
                    S.Ol[a][t] = v.lo;
                }
            }
            else
            {
                const ff inv = ff_rsqrt(dot);
                for (int a = lane; a < k; a += 32)
                {
                    const ff v = ff_mul(ff{S.Oh[a][t], S.Ol[a][t]}, inv);
                    S.Oh[a][t] = v.hi;
                    S.Ol[a][t] = v.lo;
                }
            }
            __syncwarp();
        }
    }
}

template <int M, int WARPS, int TD>
__global__ void __launch_bounds__(WARPS * 32) k_ltsa(const void* X, int dtype, int64_t N, int D, int64_t ldx,
                                              const int32_t* __restrict__ idx, int k, int td, double* V,
                                              int32_t* refine, unsigned* nrefine, unsigned* err)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    JacobiSmem<M, float, TD>& S = reinterpret_cast<JacobiSmem<M, float, TD>*>(smem_raw)[wib];
    __shared__ int nb_s[WARPS][M];
    const int64_t nw = (int64_t)gridDim.x * WARPS;
    for (int64_t i = (int64_t)blockIdx.x * WARPS + wib; i < N; i += nw)
    {
        for (int a = lane; a < k; a += 32)
        {
            // a neighbour index outside [0, N) is reported and read as the point itself
            int nb = idx[i * k + a];
            if (nb < 0 || (int64_t)nb >= N)
            {
                atomicOr(err, DEV_ERR_BOUNDS);
                nb = (int)i;
            }
            nb_s[wib][a] = nb;
        }
        __syncwarp();
        centred_gram<M, float>(S, lane, X, dtype, ldx, D, nb_s[wib], k);
        warp_jacobi<M, float>(S, lane, 30);
        // top td eigenvalues and the next one: warp arg-max rounds over the
        // diagonal (ties to the lower index)
        __shared__ int top_s[WARPS][8];
        {
            float dv[(M + 31) / 32];
#pragma unroll
            for (int r = 0; r < (M + 31) / 32; ++r)
            {
                const int c = lane + 32 * r;
                dv[r] = (c < M) ? S.A[c][c] : -FLT_MAX;
            }
            float lmax = 0.f, lsel[9];
            for (int t = 0; t <= td && t < M; ++t)
            {
                float bv = -FLT_MAX;
                int bi = 0x7fffffff;
#pragma unroll
                for (int r = 0; r < (M + 31) / 32; ++r)
                    if (dv[r] > bv)
                    {
                        bv = dv[r];
                        bi = lane + 32 * r;
                    }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1)
                {
                    const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
                    const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                    if (ov > bv || (ov == bv && oi < bi))
                    {
                        bv = ov;
                        bi = oi;
                    }
                }
#pragma unroll
                for (int r = 0; r < (M + 31) / 32; ++r)
                    if (lane + 32 * r == bi)
                        dv[r] = -FLT_MAX;
                if (lane == 0 && t < td)
                    top_s[wib][t] = bi;
                if (t == 0)
                    lmax = bv;
                lsel[t] = bv;
            }
            if (lane == 0)
            {
                const float gap = lsel[td - 1] - (td < M ? lsel[td] : 0.f);
                if (!(gap > 1e-6f * fabsf(lmax)))
                    refine[atomicAdd(nrefine, 1u)] = (int32_t)i;
            }
        }
        __syncwarp();
        int top[8];
        for (int t = 0; t < td; ++t)
            top[t] = top_s[wib][td - 1 - t];  // ascending eigenvalue order, like rightCols(td)
        refine_subspace<M>(S, lane, X, dtype, ldx, D, nb_s[wib], k, td, top);
        for (int e = lane; e < k * td; e += 32)
        {
            const int a = e / td, t = e % td;
            V[(i * k + a) * td + t] = (double)S.Oh[a][t] + (double)S.Ol[a][t];
        }
        __syncwarp();
    }
}

// FP64 redo of the points flagged for a small eigen-gap (one warp per block).
template <int M>
__global__ void __launch_bounds__(32) k_ltsa_fp64(const void* X, int dtype, int64_t N, int D, int64_t ldx,
                                                  const int32_t* __restrict__ idx, int k, int td, double* V,
                                                  const int32_t* refine, const unsigned* nrefine, unsigned* err)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    JacobiSmem<M, double>& S = *reinterpret_cast<JacobiSmem<M, double>*>(smem_raw);
    __shared__ int nb_s[M];
    __shared__ int top_s[8];
    const int lane = threadIdx.x;
    const unsigned nr = *nrefine;
    for (unsigned r = blockIdx.x; r < nr; r += gridDim.x)
    {
        const int64_t i = refine[r];
        for (int a = lane; a < k; a += 32)
        {
            int nb = idx[i * k + a];
            if (nb < 0 || (int64_t)nb >= N)
            {
                atomicOr(err, DEV_ERR_BOUNDS);
                nb = (int)i;
            }
            nb_s[a] = nb;
        }
        __syncwarp();
        centred_gram<M, double>(S, lane, X, dtype, ldx, D, nb_s, k);
        warp_jacobi<M, double>(S, lane, 60);
        if (lane == 0)
        {
            int chosen[8];
            for (int t = 0; t < td; ++t)
            {
                int best = -1;
                double bv = -1e300;
                for (int c = 0; c < M; ++c)
                {
                    bool used = false;
                    for (int u = 0; u < t; ++u)
                        used |= (chosen[u] == c);
                    if (!used && S.A[c][c] > bv)
                    {
                        bv = S.A[c][c];
                        best = c;
                    }
                }
                chosen[t] = best;
                top_s[t] = best;
            }
        }
        __syncwarp();
        for (int e = lane; e < k * td; e += 32)
        {
            const int a = e / td, t = e % td;
            V[(i * k + a) * td + t] = S.VT[top_s[td - 1 - t]][a];
        }
        __syncwarp();
    }
}

template <int M>
void launch(tk_ctx* ctx, const void* X, int dtype, int64_t N, int D, int64_t ldx, const int32_t* idx, int k, int td,
            double* V)
{
    constexpr int WARPS = (M <= 32) ? 4 : 2;
    cudaStream_t st = ctx->stream;
    int32_t* refine = (int32_t*)ctx->scratch.get("ltsa.refine", sizeof(int32_t) * (size_t)N);
    unsigned* nrefine = (unsigned*)ctx->scratch.get("ltsa.nrefine", 16);
    TK_CUDA(cudaMemsetAsync(nrefine, 0, 16, st));
    const int grid = (int)std::min<int64_t>((N + WARPS - 1) / WARPS, (int64_t)ctx->num_sms * 16);
    auto run = [&](auto tdc) {
        constexpr int TD = decltype(tdc)::value;
        const size_t smem = sizeof(JacobiSmem<M, float, TD>) * WARPS;
        static_assert(sizeof(JacobiSmem<M, float, TD>) * WARPS <= 200 * 1024, "shared memory budget");
        TK_CUDA(cudaFuncSetAttribute(k_ltsa<M, WARPS, TD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_ltsa<M, WARPS, TD><<<grid, WARPS * 32, smem, st>>>(X, dtype, N, D, ldx, idx, k, td, V, refine, nrefine,
                                                             ctx->dev_err);
        TK_CHECK_LAUNCH();
    };
    if (td <= 2)
        run(std::integral_constant<int, 2>{});
    else if (td <= 4)
        run(std::integral_constant<int, 4>{});
    else
        run(std::integral_constant<int, 8>{});
    const size_t smem64 = sizeof(JacobiSmem<M, double>);
    TK_CUDA(cudaFuncSetAttribute(k_ltsa_fp64<M>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem64));
    k_ltsa_fp64<M><<<ctx->num_sms * 4, 32, smem64, st>>>(X, dtype, N, D, ldx, idx, k, td, V, refine, nrefine,
                                                          ctx->dev_err);
    TK_CHECK_LAUNCH();
}

} // namespace

void ltsa_basis(tk_ctx* ctx, const void* X, int dtype, int64_t N, int D, int64_t ldx, const int32_t* idx, int k,
                int td, double* V)
{
    if (td < 1 || td > 8 || td >= k)
        throw Error(TK_ERR_INVALID_ARG, "LTSA needs 1 <= target_dimension <= 8 and target_dimension < k");
    // the Jacobi works on the zero-padded M x M Gram (M even): pick M close to k,
    // since a sweep costs ~M^3
    if (k <= 12)
        launch<12>(ctx, X, dtype, N, D, ldx, idx, k, td, V);
    else if (k <= 16)
        launch<16>(ctx, X, dtype, N, D, ldx, idx, k, td, V);
    else if (k <= 20)
        launch<20>(ctx, X, dtype, N, D, ldx, idx, k, td, V);
    else if (k <= 24)
        launch<24>(ctx, X, dtype, N, D, ldx, idx, k, td, V);
    else if (k <= 32)
        launch<32>(ctx, X, dtype, N, D, ldx, idx, k, td, V);
    else if (k <= 48)
        launch<48>(ctx, X, dtype, N, D, ldx, idx, k, td, V);
    else if (k <= 64)
        launch<64>(ctx, X, dtype, N, D, ldx, idx, k, td, V);
    else
        throw Error(TK_ERR_UNSUPPORTED, "LTSA bases support up to 64 neighbours");
}

} // namespace tk
