// lle.cu -- LLE reconstruction weights, one warp per point.
//
// Per point x with neighbours n_0..n_{k-1} (routines/locally_linear.hpp:107-131):
//   C_ab = (n_a - x).(n_b - x)          the reference's kernel form
//                                       k(x,x)-k(x,n_a)-k(x,n_b)+k(n_a,n_b)
//   C   += klle_shift * trace(C) * I
//   w    = C^{-1} 1,  w /= sum(w)
// The Gram is accumulated in FP32 from difference vectors staged through shared
// memory in 32-dimension chunks, factorised by an FP32 Cholesky, and the solve
// is refined against a float-float residual r = 1 - (C_true + s_true I) w built
// from the exact differences (two refinement steps when k > D, where C is rank
// deficient and its conditioning is set by klle_shift; one otherwise).
#include <cfloat>

#include "ff.cuh"
#include "tk_internal.h"

namespace tk {
namespace {

// x_a - x_b for element d as an unevaluated float sum hi + lo (exact for float32
// input: two_sum of the two floats; float64 input: the FP64 difference split).
__device__ __forceinline__ ff diff_ff(const void* X, int dtype, int64_t a_off, int64_t b_off)
{
    if (dtype == TK_F64)
    {
        const double z = reinterpret_cast<const double*>(X)[a_off] - reinterpret_cast<const double*>(X)[b_off];
        const float h = (float)z;
        return ff{h, (float)(z - (double)h)};
    }
    return two_sum(reinterpret_cast<const float*>(X)[a_off], -reinterpret_cast<const float*>(X)[b_off]);
}

template <int KP>
struct LleSmem
{
    float Zh[KP][33];
    float Zl[KP][33];
    float C[KP][KP + 1];
    float vh[32], vl[32];
    float r[KP];
    float w[KP];
    float ivd[KP];  // 1 / L_aa of the register factor
};

template <int KP>
__device__ __forceinline__ void chol_solve(LleSmem<KP>& S, int lane)
{
    // forward L y = r
    for (int j = 0; j < KP; ++j)
    {
        __syncwarp();
        const float yj = S.r[j] / S.C[j][j];
        __syncwarp();
        if (lane == 0)
            S.r[j] = yj;
        for (int rr = j + 1 + lane; rr < KP; rr += 32)
            S.r[rr] = fmaf(-S.C[rr][j], yj, S.r[rr]);
    }
    // backward L^T x = y
    for (int j = KP - 1; j >= 0; --j)
    {
        __syncwarp();
        const float xj = S.r[j] / S.C[j][j];
        __syncwarp();
        if (lane == 0)
            S.r[j] = xj;
        for (int rr = lane; rr < j; rr += 32)
            S.r[rr] = fmaf(-S.C[j][rr], xj, S.r[rr]);
    }
    __syncwarp();
}

// Rows of one launch: the points of one problem (row_prob == NULL; row g is
// point g), or the rows of a batch's k-group (row g belongs to problem
// row_prob[g], at point out_row0 + g - probs[.].out_row0 of it). idx, W and rhs
// are indexed by row.
struct LleRows
{
    const void* X;
    int dtype;
    int64_t N;
    int D;
    int64_t ldx;
    int64_t rows;
    const int32_t* row_prob;
    const BatchProb* probs;
    int64_t out_row0;
    unsigned long long* work;  // batch: counter of claimed rows (zero at launch)
};

// Rows a warp of a batch claims at a time. Rows of different problems cost very
// different amounts (a row's cost grows with its problem's D, 3 to 128), so
// warps take chunks from a shared counter instead of fixed runs.
constexpr int LLE_CHUNK = 8;

// Register-resident Cholesky for KP <= 32: lane a holds row a of the matrix
// (L[c] = C_ac for c <= a) and ends with row a of the lower factor and invd =
// 1 / L_aa. Column j's entries travel by shuffles, so no shared-memory round trip
// sits on the factorisation's dependency chain. Reciprocal square roots replace
// the divisions (the float-float refinement absorbs their last-bit errors).
template <int KP>
__device__ __forceinline__ void reg_cholesky(float (&L)[KP], float& invd, int lane)
{
    invd = 1.f;
#pragma unroll
    for (int j = 0; j < KP; ++j)
    {
        const float inv = rsqrtf(fmaxf(__shfl_sync(0xffffffffu, L[j], j), FLT_MIN));
        if (lane == j)
        {
            L[j] = L[j] * inv;
            invd = inv;
        }
        else if (lane > j)
            L[j] = L[j] * inv;
#pragma unroll
        for (int c = 0; c < KP; ++c)  // constant trip count: fully unrolled, c > j folds
        {
            if (c > j)
            {
                const float lcj = __shfl_sync(0xffffffffu, L[j], c);
                if (lane >= c)
                    L[c] = fmaf(-L[j], lcj, L[c]);
            }
        }
    }
}

// Solves L L^T x = r with the register factor; lane a holds r_a and gets x_a.
// Both substitutions are column sweeps: step j broadcasts one solved entry and
// every later (forward) or earlier (backward) lane updates its own entry. The
// backward sweep reads L^T from Ls (row a = row a of L, stride KP + 1), and
// ivd holds 1 / L_jj; both are in shared memory.
template <int KP>
__device__ __forceinline__ float reg_chol_solve(const float (&L)[KP], const float* Ls, const float* ivd, float r,
                                                int lane)
{
    float y = r;
#pragma unroll
    for (int j = 0; j < KP; ++j)
    {
        const float yj = __shfl_sync(0xffffffffu, y, j) * ivd[j];
        if (lane == j)
            y = yj;
        else if (lane > j)
            y = fmaf(-L[j], yj, y);
    }
#pragma unroll
    for (int j = KP - 1; j >= 0; --j)
    {
        const float lji = (lane < j) ? Ls[j * (KP + 1) + lane] : 0.f;
        const float xj = __shfl_sync(0xffffffffu, y, j) * ivd[j];
        if (lane == j)
            y = xj;
        else if (lane < j)
            y = fmaf(-lji, xj, y);
    }
    return y;
}

// The same for KP = 64 with two rows per lane: lane a holds rows a (A0, columns
// 0..31: its entries past column a are zero) and a + 32 (A1), entries c <= row;
// rows of column j travel by shuffles from the lane j & 31. ivd receives 1 / L_jj
// (written by the lane that holds row j). Indices into A0 are taken mod 32 in
// branches that run only for columns below 32.
__device__ __forceinline__ void reg_cholesky64(float (&A0)[32], float (&A1)[64], float* ivd, int lane)
{
#pragma unroll
    for (int j = 0; j < 64; ++j)
    {
        const float djj = __shfl_sync(0xffffffffu, (j < 32) ? A0[j & 31] : A1[j], j & 31);
        const float inv = rsqrtf(fmaxf(djj, FLT_MIN));
        if (lane == (j & 31))
            ivd[j] = inv;
        if (j < 32)
        {
            if (lane >= j)
                A0[j & 31] *= inv;
            A1[j] *= inv;
        }
        else if (lane + 32 >= j)
            A1[j] *= inv;
#pragma unroll
        for (int c = 0; c < 64; ++c)
        {
            if (c > j)
            {
                const float lcj = __shfl_sync(0xffffffffu, (c < 32) ? A0[j & 31] : A1[j], c & 31);
                if (c < 32)
                {
                    if (lane >= c)
                        A0[c & 31] = fmaf(-A0[j & 31], lcj, A0[c & 31]);
                    A1[c] = fmaf(-A1[j], lcj, A1[c]);
                }
                else if (lane + 32 >= c)
                    A1[c] = fmaf(-A1[j], lcj, A1[c]);
            }
        }
    }
}

// Solves L L^T x = r for KP = 64 with the factor of reg_cholesky64 stored in Ls
// (row-major, stride 65) and ivd = 1 / L_jj; lane a holds r_a, r_{a+32} in y0, y1
// and gets x there. The factor's loads do not depend on the sweep, so they are
// issued ahead of the shuffle chain.
__device__ __forceinline__ void reg_chol_solve64(const float* Ls, const float* ivd, float& y0, float& y1, int lane)
{
#pragma unroll
    for (int j = 0; j < 64; ++j)
    {
        const float yj = __shfl_sync(0xffffffffu, (j < 32) ? y0 : y1, j & 31) * ivd[j];
        const float a0 = (lane > j) ? Ls[lane * 65 + j] : 0.f;
        const float a1 = (lane + 32 > j) ? Ls[(lane + 32) * 65 + j] : 0.f;
        if (j < 32)
        {
            if (lane == j)
                y0 = yj;
            else if (lane > j)
                y0 = fmaf(-a0, yj, y0);
            y1 = fmaf(-a1, yj, y1);
        }
        else
        {
            if (lane + 32 == j)
                y1 = yj;
            else if (lane + 32 > j)
                y1 = fmaf(-a1, yj, y1);
        }
    }
#pragma unroll
    for (int j = 63; j >= 0; --j)
    {
        const float xj = __shfl_sync(0xffffffffu, (j < 32) ? y0 : y1, j & 31) * ivd[j];
        const float l0 = (lane < j) ? Ls[j * 65 + lane] : 0.f;
        const float l1 = (lane + 32 < j) ? Ls[j * 65 + lane + 32] : 0.f;
        if (j < 32)
        {
            if (lane == j)
                y0 = xj;
            else if (lane < j)
                y0 = fmaf(-l0, xj, y0);
        }
        else
        {
            if (lane + 32 == j)
                y1 = xj;
            else if (lane + 32 < j)
                y1 = fmaf(-l1, xj, y1);
            y0 = fmaf(-l0, xj, y0);
        }
    }
}

// reg_chol_solve with the factor's rows read from Ls (row a = row a of L, stride
// KP + 1) in both sweeps, so no factor registers stay live: the same values and
// operations, so the same results.
template <int KP>
__device__ __forceinline__ float smem_chol_solve(const float* Ls, const float* ivd, float r, int lane)
{
    float y = r;
#pragma unroll 4
    for (int j = 0; j < KP; ++j)
    {
        const float yj = __shfl_sync(0xffffffffu, y, j) * ivd[j];
        const float lij = (lane > j && lane < KP) ? Ls[lane * (KP + 1) + j] : 0.f;
        if (lane == j)
            y = yj;
        else if (lane > j)
            y = fmaf(-lij, yj, y);
    }
#pragma unroll 4
    for (int j = KP - 1; j >= 0; --j)
    {
        const float lji = (lane < j) ? Ls[j * (KP + 1) + lane] : 0.f;
        const float xj = __shfl_sync(0xffffffffu, y, j) * ivd[j];
        if (lane == j)
            y = xj;
        else if (lane < j)
            y = fmaf(-lji, xj, y);
    }
    return y;
}

// nb[s] holds neighbour lane + 32 s of the lane; a runtime group index picks the
// register by selects (no indexed local-memory access)
template <int NPL>
__device__ __forceinline__ int nb_group(const int (&nb)[NPL], int s)
{
    int v = nb[0];
#pragma unroll
    for (int t = 1; t < NPL; ++t)
        v = (s == t) ? nb[t] : v;
    return v;
}

__device__ __forceinline__ float ld_f(const void* X, int dtype, int64_t off)
{
    return dtype == TK_F64 ? (float)reinterpret_cast<const double*>(X)[off] : reinterpret_cast<const float*>(X)[off];
}

// KP <= 32 holds at most 128 registers (16 warps per SM): its refinement keeps no
// per-lane arrays over the neighbours (see below)
template <int KP, int WARPS, bool BATCH, bool BLOCKED = (KP <= 64)>
__global__ void __launch_bounds__(WARPS * 32, (KP <= 32) ? 16 / WARPS : 1) k_lle(const LleRows RW, const int32_t* __restrict__ idx, int k,
                                                    double klle_shift, const double* __restrict__ rhs,
                                                    int normalize, double* __restrict__ W, unsigned* err)
{
    constexpr int NB4 = KP / 4;
    constexpr int NBLK = BLOCKED ? NB4 * (NB4 + 1) / 2 : 1;
    // (block, dimension group) items: with few blocks the 32-dimension chunk is
    // split into DG ranges so that all lanes accumulate
    constexpr int DG = !BLOCKED ? 1 : ((32 / NBLK) >= 3 ? 3 : ((32 / NBLK) >= 1 ? (32 / NBLK) : 1));
    constexpr int ITEMS = NBLK * DG;
    constexpr int PERL = (ITEMS + 31) / 32;
    constexpr int SPAN = (32 + DG - 1) / DG;
    constexpr int NPL = (KP + 31) / 32;  // neighbours per lane
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    LleSmem<KP>& S = reinterpret_cast<LleSmem<KP>*>(smem_raw)[wib];
    const ff ks = ff{(float)klle_shift, (float)(klle_shift - (double)(float)klle_shift)};
    const int64_t warp = (int64_t)blockIdx.x * WARPS + wib;
    const int64_t nwarps = (int64_t)gridDim.x * WARPS;

    // (I, J) 4x4 blocks of the upper triangle and dimension group of each item of this lane
    int bI[PERL], bJ[PERL], bG[PERL];
#pragma unroll
    for (int m = 0; m < PERL; ++m)
    {
        const int itm = lane + 32 * m;
        int b = (itm < ITEMS) ? itm % NBLK : 0, I = 0;
        while (b >= NB4 - I)
        {
            b -= NB4 - I;
            ++I;
        }
        bI[m] = I;
        bJ[m] = I + b;
        bG[m] = (itm < ITEMS) ? itm / NBLK : 0;
    }

    // batch: each warp claims chunks of consecutive rows, so the problem
    // description is reloaded only where a chunk crosses into the next problem
    const void* X = RW.X;
    int dtype = RW.dtype;
    int64_t N = RW.N;
    int D = RW.D;
    int64_t ldx = RW.ldx;
    int64_t prob_row0 = 0;  // batch: output row of the current problem's point 0
    int cur = -1;
    for (int pass = 0;; ++pass)
    {
    int64_t g_begin, g_end, g_step;
    if constexpr (BATCH)
    {
        unsigned long long c0 = 0;
        if (lane == 0)
            c0 = atomicAdd(RW.work, (unsigned long long)LLE_CHUNK);
        c0 = __shfl_sync(0xffffffffu, c0, 0);
        if ((int64_t)c0 >= RW.rows)
            break;
        g_begin = (int64_t)c0;
        g_end = min(RW.rows, (int64_t)c0 + LLE_CHUNK);
        g_step = 1;
    }
    else
    {
        if (pass > 0)
            break;
        g_begin = warp;
        g_end = RW.rows;
        g_step = nwarps;
    }
    for (int64_t g = g_begin; g < g_end; g += g_step)
    {
        int64_t i = g;
        if constexpr (BATCH)
        {
            const int b = RW.row_prob[g];
            if (b != cur)
            {
                const BatchProb& P = RW.probs[b];
                X = P.X;
                dtype = P.dtype;
                N = P.N;
                D = P.D;
                ldx = P.ldx;
                prob_row0 = P.out_row0;
                cur = b;
            }
            i = RW.out_row0 + g - prob_row0;
        }
        int nb[NPL];
#pragma unroll
        for (int s = 0; s < NPL; ++s)
        {
            const int a = lane + 32 * s;
            nb[s] = (a < k) ? idx[g * k + a] : 0;
            if (a < k && (nb[s] < 0 || nb[s] >= N))
            {
                atomicOr(err, DEV_ERR_BOUNDS);
                nb[s] = 0;
            }
        }

        // ---- FP32 Gram ----
        if (!BLOCKED)
        {
            for (int t = lane; t < KP * KP; t += 32)
                S.C[t / KP][t % KP] = 0.f;
            __syncwarp();
        }
        float acc[PERL][16];
#pragma unroll
        for (int m = 0; m < PERL; ++m)
#pragma unroll
            for (int t = 0; t < 16; ++t)
                acc[m][t] = 0.f;
        for (int d0 = 0; d0 < D; d0 += 32)
        {
            const int d = d0 + lane;
            if (KP <= 64 && dtype == TK_F32)
            {
                // every neighbour value of the chunk in flight at once
                constexpr int KV = (KP <= 64) ? KP : 1;
                const float xi = (d < D) ? ld_f(X, dtype, i * ldx + d) : 0.f;
                float v[KV];
#pragma unroll
                for (int a = 0; a < KV; ++a)
                {
                    const int nba = __shfl_sync(0xffffffffu, nb[(a >> 5) < NPL ? (a >> 5) : 0], a & 31);
                    v[a] = (a < k && d < D) ? ld_f(X, dtype, (int64_t)nba * ldx + d) : xi;
                }
#pragma unroll
                for (int a = 0; a < KV; ++a)
                    S.Zh[a][lane] = v[a] - xi;
            }
            else
            {
#pragma unroll 4
                for (int a = 0; a < KP; ++a)
                {
                    const int nba = __shfl_sync(0xffffffffu, nb_group<NPL>(nb, a >> 5), a & 31);
                    float v = 0.f;
                    if (a < k && d < D)
                        v = diff_ff(X, dtype, (int64_t)nba * ldx + d, i * ldx + d).hi;
                    S.Zh[a][lane] = v;
                }
            }
            __syncwarp();
            if constexpr (!BLOCKED)
            {
                // upper-triangle entries, one lane per entry (large k)
                for (int e = lane; e < KP * KP; e += 32)
                {
                    const int a = e / KP, b = e % KP;
                    if (b < a || b >= k)
                        continue;
                    float sacc = 0.f;
                    for (int dd = 0; dd < 32; ++dd)
                        sacc = fmaf(S.Zh[a][dd], S.Zh[b][dd], sacc);
                    S.C[a][b] += sacc;
                }
                __syncwarp();
                continue;
            }
            else
#pragma unroll
            for (int m = 0; m < PERL; ++m)
            {
                if (lane + 32 * m < ITEMS)
                {
                    const int I4 = 4 * bI[m], J4 = 4 * bJ[m];
                    const int dlo = bG[m] * SPAN, dhi = min(32, dlo + SPAN);
#pragma unroll 4
                    for (int dd = dlo; dd < dhi; ++dd)
                    {
                        float av[4], bv[4];
#pragma unroll
                        for (int t = 0; t < 4; ++t)
                        {
                            av[t] = S.Zh[I4 + t][dd];
                            bv[t] = S.Zh[J4 + t][dd];
                        }
#pragma unroll
                        for (int r = 0; r < 4; ++r)
#pragma unroll
                            for (int c = 0; c < 4; ++c)
                                acc[m][r * 4 + c] = fmaf(av[r], bv[c], acc[m][r * 4 + c]);
                    }
                }
            }
            __syncwarp();
        }
        if (BLOCKED)
        {
            // dimension groups are summed in a fixed order (group 0 writes, then 1, 2 add)
#pragma unroll
            for (int g = 0; g < DG; ++g)
            {
#pragma unroll
                for (int m = 0; m < PERL; ++m)
                    if (lane + 32 * m < ITEMS && bG[m] == g)
                    {
                        const int I4 = 4 * bI[m], J4 = 4 * bJ[m];
#pragma unroll
                        for (int r = 0; r < 4; ++r)
#pragma unroll
                            for (int c = 0; c < 4; ++c)
                                if (I4 + r <= J4 + c)  // upper triangle only
                                    S.C[I4 + r][J4 + c] =
                                        (g == 0) ? acc[m][r * 4 + c] : S.C[I4 + r][J4 + c] + acc[m][r * 4 + c];
                    }
                __syncwarp();
            }
            for (int e = lane; e < KP * KP; e += 32)
            {
                const int a = e / KP, b = e % KP;
                if (a > b)
                    S.C[a][b] = S.C[b][a];
            }
        }
        else
        {
            for (int e = lane; e < KP * KP; e += 32)
            {
                const int a = e / KP, b = e % KP;
                if (b > a)
                    S.C[b][a] = S.C[a][b];
            }
        }
        __syncwarp();
        float trace = 0.f;
        for (int a = lane; a < k; a += 32)
            trace += S.C[a][a];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            trace += __shfl_xor_sync(0xffffffffu, trace, o);
        __syncwarp();
        const float shift = (float)klle_shift * trace;
        for (int a = lane; a < KP; a += 32)
        {
            if (a < k)
                S.C[a][a] += shift;
            else
                S.C[a][a] = 1.f;  // padding rows/columns are zero: identity block
            S.r[a] = (a < k) ? (rhs ? (float)rhs[g * k + a] : 1.f) : 0.f;
        }
        __syncwarp();

        // ---- FP32 Cholesky (lower) ----
        float Lr[KP <= 32 ? KP : 1];
        float invd = 1.f;
        constexpr int K64 = (KP == 64) ? 64 : 1;
        if constexpr (KP == 64)
        {
            float A0[32], A1[64];
#pragma unroll
            for (int c = 0; c < 64; ++c)
            {
                if (c < 32)
                    A0[c & 31] = (c <= lane) ? S.C[lane][c] : 0.f;
                A1[c] = (c <= lane + 32) ? S.C[lane + 32][c] : 0.f;
            }
            reg_cholesky64(A0, A1, S.ivd, lane);
            __syncwarp();
#pragma unroll
            for (int c = 0; c < 64; ++c)
            {
                if (c < 32 && c <= lane)
                    S.C[lane][c] = A0[c & 31];
                if (c <= lane + 32)
                    S.C[lane + 32][c] = A1[c];
            }
            __syncwarp();
            float y0 = S.r[lane], y1 = S.r[lane + 32];
            reg_chol_solve64(&S.C[0][0], S.ivd, y0, y1, lane);
            __syncwarp();
            S.w[lane] = (lane < k) ? y0 : 0.f;
            S.w[lane + 32] = (lane + 32 < k) ? y1 : 0.f;
            __syncwarp();
        }
        else if constexpr (KP <= 32)
        {
#pragma unroll
            for (int c = 0; c < KP; ++c)
                Lr[c] = (lane < KP && c <= lane) ? S.C[lane][c] : 0.f;
            reg_cholesky<KP>(Lr, invd, lane);
            // the factor's rows and reciprocal diagonal, for the backward sweeps
            __syncwarp();
            if (lane < KP)
            {
#pragma unroll
                for (int c = 0; c < KP; ++c)
                    if (c <= lane)
                        S.C[lane][c] = Lr[c];
                S.ivd[lane] = invd;
            }
            __syncwarp();
            const float x = reg_chol_solve<KP>(Lr, &S.C[0][0], S.ivd, lane < KP ? S.r[lane] : 0.f, lane);
            __syncwarp();
            if (lane < KP)
                S.w[lane] = (lane < k) ? x : 0.f;
            __syncwarp();
        }
        else
        {
        for (int j = 0; j < KP; ++j)
        {
            const float ljj = sqrtf(fmaxf(S.C[j][j], FLT_MIN));
            __syncwarp();
            for (int rr = j + 1 + lane; rr < KP; rr += 32)
                S.C[rr][j] /= ljj;
            if (lane == 0)
                S.C[j][j] = ljj;
            __syncwarp();
            for (int rr = j + 1 + lane; rr < KP; rr += 32)
            {
                const float lrj = S.C[rr][j];
                for (int c = j + 1; c <= rr; ++c)
                    S.C[rr][c] = fmaf(-lrj, S.C[c][j], S.C[rr][c]);
            }
            __syncwarp();
        }
        chol_solve<KP>(S, lane);
        for (int a = lane; a < KP; a += 32)
            S.w[a] = (a < k) ? S.r[a] : 0.f;
        __syncwarp();
        }

        // ---- float-float residual refinement ----
        const int iters = (k > D) ? 2 : 1;
        for (int itr = 0; itr < iters; ++itr)
        {
            if (KP <= 32)
            {
                // the chunk's exact differences z_a(d) staged in shared memory (lanes
                // own dimensions for the loads); v(d) = sum_b w_b z_b(d) by the lane
                // owning d; then lane a forms (C w)_a = sum_d z_a(d) v(d) itself. The
                // shift uses the FP32 trace: its relative error (~D 2^-24) enters the
                // residual scaled by klle_shift, far below the solve's own error.
                ff ca = ff_zero();
                for (int d0 = 0; d0 < D; d0 += 32)
                {
                    const int d = d0 + lane;
                    if (dtype == TK_F32)
                    {
                        const float xi = (d < D) ? ld_f(X, dtype, i * ldx + d) : 0.f;
                        constexpr int KV = (KP <= 32) ? KP : 1;
                        float v[KV];
#pragma unroll
                        for (int a = 0; a < KV; ++a)
                        {
                            const int nba = __shfl_sync(0xffffffffu, nb[0], a);
                            v[a] = (a < k && d < D) ? ld_f(X, dtype, (int64_t)nba * ldx + d) : xi;
                        }
#pragma unroll
                        for (int a = 0; a < KV; ++a)
                        {
                            const ff z = two_sum(v[a], -xi);
                            S.Zh[a][lane] = z.hi;
                            S.Zl[a][lane] = z.lo;
                        }
                    }
                    else
                    {
                        for (int a = 0; a < KP && a < 32; ++a)
                        {
                            const int nba = __shfl_sync(0xffffffffu, nb[0], a);
                            ff z = ff_zero();
                            if (a < k && d < D)
                                z = diff_ff(X, dtype, (int64_t)nba * ldx + d, i * ldx + d);
                            S.Zh[a][lane] = z.hi;
                            S.Zl[a][lane] = z.lo;
                        }
                    }
                    __syncwarp();
                    ff vq[4] = {ff_zero(), ff_zero(), ff_zero(), ff_zero()};
                    for (int b = 0; b < k; b += 4)
#pragma unroll
                        for (int t = 0; t < 4; ++t)
                            if (b + t < k)
                                vq[t] = ff_fma(vq[t], S.w[b + t], 0.f, S.Zh[b + t][lane], S.Zl[b + t][lane]);
                    const ff vv = ff_add(ff_add(vq[0], vq[1]), ff_add(vq[2], vq[3]));
                    S.vh[lane] = vv.hi;
                    S.vl[lane] = vv.lo;
                    __syncwarp();
                    if (lane < k)
#pragma unroll 8
                        for (int dd = 0; dd < 32; ++dd)
                            ca = ff_fma(ca, S.Zh[lane][dd], S.Zl[lane][dd], S.vh[dd], S.vl[dd]);
                    __syncwarp();
                }
                float ra = 0.f;
                if (lane < k)
                {
                    const ff sw = ff_mul(ff_mul(ks, ff{trace, 0.f}), ff{S.w[lane], 0.f});
                    ff b = ff{1.f, 0.f};
                    if (rhs)
                    {
                        const double rb = rhs[g * k + lane];
                        b.hi = (float)rb;
                        b.lo = (float)(rb - (double)b.hi);
                    }
                    const ff rr = ff_add(ff_add(b, ff_neg(ca)), ff_neg(sw));
                    ra = rr.hi + rr.lo;
                }
                if (lane < KP)
                    S.r[lane] = ra;
                __syncwarp();
            }
            else
            {
                ff sa[NPL], ta[NPL];
#pragma unroll
                for (int s = 0; s < NPL; ++s)
                {
                    sa[s] = ff_zero();
                    ta[s] = ff_zero();
                }
                for (int d0 = 0; d0 < D; d0 += 32)
                {
                    const int d = d0 + lane;
                    if (KP == 64 && dtype == TK_F32)
                    {
                        // every neighbour value of the chunk in flight at once
                        const float xi = (d < D) ? ld_f(X, dtype, i * ldx + d) : 0.f;
                        float xv[K64];
#pragma unroll
                        for (int a = 0; a < K64; ++a)
                        {
                            const int nba = __shfl_sync(0xffffffffu, nb[(a >> 5) < NPL ? (a >> 5) : 0], a & 31);
                            xv[a] = (a < k && d < D) ? ld_f(X, dtype, (int64_t)nba * ldx + d) : xi;
                        }
#pragma unroll
                        for (int a = 0; a < K64; ++a)
                        {
                            const ff z = two_sum(xv[a], -xi);
                            S.Zh[a][lane] = z.hi;
                            S.Zl[a][lane] = z.lo;
                        }
                    }
                    else
                    {
                        for (int a = 0; a < KP; ++a)
                        {
                            const int nba =
                                __shfl_sync(0xffffffffu, nb_group<NPL>(nb, a >> 5), a & 31);
                            ff z = ff_zero();
                            if (a < k && d < D)
                                z = diff_ff(X, dtype, (int64_t)nba * ldx + d, i * ldx + d);
                            S.Zh[a][lane] = z.hi;
                            S.Zl[a][lane] = z.lo;
                        }
                    }
                    __syncwarp();
                    // v_d = sum_b w_b z_bd for d = d0 + lane, in four independent chains
                    ff vq[4] = {ff_zero(), ff_zero(), ff_zero(), ff_zero()};
                    for (int b = 0; b < k; b += 4)
#pragma unroll
                        for (int t = 0; t < 4; ++t)
                            if (b + t < k)
                                vq[t] = ff_fma(vq[t], S.w[b + t], 0.f, S.Zh[b + t][lane], S.Zl[b + t][lane]);
                    const ff v = ff_add(ff_add(vq[0], vq[1]), ff_add(vq[2], vq[3]));
                    S.vh[lane] = v.hi;
                    S.vl[lane] = v.lo;
                    __syncwarp();
#pragma unroll
                    for (int s = 0; s < NPL; ++s)
                    {
                        const int a = lane + 32 * s;
                        if (a < k)
                            for (int dd = 0; dd < 32; ++dd)
                            {
                                const float zh = S.Zh[a][dd], zl = S.Zl[a][dd];
                                sa[s] = ff_fma(sa[s], zh, zl, S.vh[dd], S.vl[dd]);
                                ta[s] = ff_fma(ta[s], zh, zl, zh, zl);
                            }
                    }
                    __syncwarp();
                }
                // exact trace = sum_a |z_a|^2
                ff tr = ff_zero();
#pragma unroll
                for (int s = 0; s < NPL; ++s)
                    tr = ff_add(tr, ta[s]);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1)
                    tr = ff_add(tr, ff_shfl_xor(tr, o));
                const double shift_true = klle_shift * ff_to_double(tr);
#pragma unroll
                for (int s = 0; s < NPL; ++s)
                {
                    const int a = lane + 32 * s;
                    if (a < KP)
                        S.r[a] = (a < k) ? (float)((rhs ? rhs[g * k + a] : 1.0) - ff_to_double(sa[s]) -
                                                   shift_true * (double)S.w[a])
                                         : 0.f;
                }
                __syncwarp();
            }
            if constexpr (KP == 64)
            {
                float y0 = S.r[lane], y1 = S.r[lane + 32];
                reg_chol_solve64(&S.C[0][0], S.ivd, y0, y1, lane);
                __syncwarp();
                if (lane < k)
                    S.w[lane] += y0;
                if (lane + 32 < k)
                    S.w[lane + 32] += y1;
            }
            else if constexpr (KP <= 32)
            {
                const float x = smem_chol_solve<KP>(&S.C[0][0], S.ivd, lane < KP ? S.r[lane] : 0.f, lane);
                __syncwarp();
                if (lane < k)
                    S.w[lane] += x;
            }
            else
            {
                chol_solve<KP>(S, lane);
                for (int a = lane; a < k; a += 32)
                    S.w[a] += S.r[a];
            }
            __syncwarp();
        }

        // ---- normalise (weights) or store the raw solution (adjoint solve) ----
        if (!normalize)
        {
            for (int a = lane; a < k; a += 32)
                W[g * k + a] = (double)S.w[a];
            __syncwarp();
            continue;
        }
        // w / sum(w) in float-float: the sum, its reciprocal refined by one Newton
        // step (error ~2^-44), and the products, so that the weights sum to one
        // to ~1e-13 without an FP64 division
        ff sum = ff_zero();
        for (int a = lane; a < k; a += 32)
            sum = ff_add(sum, ff{S.w[a], 0.f});
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            sum = ff_add(sum, ff_shfl_xor(sum, o));
        const float y0 = 1.f / sum.hi;
        const ff sy = two_prod(sum.hi, y0);
        const float resid = ((1.f - sy.hi) - sy.lo) - sum.lo * y0;  // 1 - sum * y0
        const float y1 = y0 * resid;                                 // y = y0 + y1
        for (int a = lane; a < k; a += 32)
        {
            const ff q = two_prod(S.w[a], y0);
            W[g * k + a] = (double)q.hi + (double)fmaf(S.w[a], y1, q.lo);
        }
        __syncwarp();
    }
    }
}

// ---------------------------------------------------------------------------
// 33 <= k <= 64, float32 input, one problem: the k_lle solve with 18 KB of shared
// memory per warp instead of 34.5 KB. The factor is kept as a packed lower
// triangle (row r starts at r (r + 1) / 2; the triangular numbers mod 32 are all
// distinct, so the row-per-lane reads of the sweeps hit distinct banks), and one
// 64 x 33 buffer holds the chunk's differences for the Gram, then its raw
// neighbour values for the refinement, which forms the exact differences by
// two-sum as it reads them. Registers then bound the occupancy: 8 warps per SM
// at up to 255 registers (k_lle at k = 64 ran 6). With 12 warps (168 registers)
// the kernel spilled about 0.9 KB per thread and ran no faster than k_lle.
constexpr int L64_WARPS = 8;

struct Lle64Smem
{
    float B[64][33];
    float Lp[64 * 65 / 2];
    float xs[32];
    float vh[32], vl[32];
    float r[64], w[64], ivd[64];
};

__device__ __forceinline__ int tri(int r) { return (r * (r + 1)) >> 1; }

// reg_chol_solve64 on the packed factor
__device__ __forceinline__ void packed_solve64(const float* Lp, const float* ivd, float& y0, float& y1, int lane)
{
    const int t0 = tri(lane), t1 = tri(lane + 32);
#pragma unroll 4
    for (int j = 0; j < 64; ++j)
    {
        const float yj = __shfl_sync(0xffffffffu, (j < 32) ? y0 : y1, j & 31) * ivd[j];
        const float a0 = (lane > j) ? Lp[t0 + j] : 0.f;
        const float a1 = (lane + 32 > j) ? Lp[t1 + j] : 0.f;
        if (j < 32)
        {
            if (lane == j)
                y0 = yj;
            else if (lane > j)
                y0 = fmaf(-a0, yj, y0);
            y1 = fmaf(-a1, yj, y1);
        }
        else
        {
            if (lane + 32 == j)
                y1 = yj;
            else if (lane + 32 > j)
                y1 = fmaf(-a1, yj, y1);
        }
    }
#pragma unroll 4
    for (int j = 63; j >= 0; --j)
    {
        const float xj = __shfl_sync(0xffffffffu, (j < 32) ? y0 : y1, j & 31) * ivd[j];
        const float l0 = (lane < j) ? Lp[tri(j) + lane] : 0.f;
        const float l1 = (lane + 32 < j) ? Lp[tri(j) + lane + 32] : 0.f;
        if (j < 32)
        {
            if (lane == j)
                y0 = xj;
            else if (lane < j)
                y0 = fmaf(-l0, xj, y0);
        }
        else
        {
            if (lane + 32 == j)
                y1 = xj;
            else if (lane + 32 < j)
                y1 = fmaf(-l1, xj, y1);
            y0 = fmaf(-l0, xj, y0);
        }
    }
}

__global__ void __launch_bounds__(L64_WARPS * 32) k_lle64(const float* __restrict__ X, int64_t N, int D, int64_t ldx,
                                                          const int32_t* __restrict__ idx, int k, double klle_shift,
                                                          const double* __restrict__ rhs, int normalize,
                                                          double* __restrict__ W, unsigned* err)
{
    constexpr int NB4 = 16, NBLK = NB4 * (NB4 + 1) / 2, PERL = (NBLK + 31) / 32;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    Lle64Smem& S = reinterpret_cast<Lle64Smem*>(smem_raw)[wib];
    const int64_t nwarps = (int64_t)gridDim.x * L64_WARPS;
    // (I, J) 4 x 4 blocks of the upper triangle owned by this lane
    int bI[PERL], bJ[PERL];
#pragma unroll
    for (int m = 0; m < PERL; ++m)
    {
        int b = (lane + 32 * m < NBLK) ? lane + 32 * m : 0, I = 0;
        while (b >= NB4 - I)
        {
            b -= NB4 - I;
            ++I;
        }
        bI[m] = I;
        bJ[m] = I + b;
    }
    const int t0 = tri(lane), t1 = tri(lane + 32);
    for (int64_t i = (int64_t)blockIdx.x * L64_WARPS + wib; i < N; i += nwarps)
    {
        int nb[2];
#pragma unroll
        for (int s2 = 0; s2 < 2; ++s2)
        {
            const int a = lane + 32 * s2;
            nb[s2] = (a < k) ? idx[i * k + a] : 0;
            if (a < k && (nb[s2] < 0 || nb[s2] >= N))
            {
                atomicOr(err, DEV_ERR_BOUNDS);
                nb[s2] = 0;
            }
        }
        // ---- FP32 Gram of the differences, 4 x 4 blocks in registers ----
        float acc[PERL][16];
#pragma unroll
        for (int m = 0; m < PERL; ++m)
#pragma unroll
            for (int t = 0; t < 16; ++t)
                acc[m][t] = 0.f;
        for (int d0 = 0; d0 < D; d0 += 32)
        {
            const int d = d0 + lane;
            const float xi = (d < D) ? X[i * ldx + d] : 0.f;
            __syncwarp();
            // 32 neighbour values in flight at a time
#pragma unroll
            for (int h = 0; h < 2; ++h)
            {
                float v[32];
#pragma unroll
                for (int a = 0; a < 32; ++a)
                {
                    const int nba = __shfl_sync(0xffffffffu, nb[h], a);
                    v[a] = (32 * h + a < k && d < D) ? X[(int64_t)nba * ldx + d] : xi;
                }
#pragma unroll
                for (int a = 0; a < 32; ++a)
                    S.B[32 * h + a][lane] = v[a] - xi;
            }
            __syncwarp();
#pragma unroll
            for (int m = 0; m < PERL; ++m)
            {
                if (lane + 32 * m < NBLK)
                {
                    const int I4 = 4 * bI[m], J4 = 4 * bJ[m];
#pragma unroll 2
                    for (int dd = 0; dd < 32; ++dd)
                    {
                        float av[4], bv[4];
#pragma unroll
                        for (int t = 0; t < 4; ++t)
                        {
                            av[t] = S.B[I4 + t][dd];
                            bv[t] = S.B[J4 + t][dd];
                        }
#pragma unroll
                        for (int r = 0; r < 4; ++r)
#pragma unroll
                            for (int c = 0; c < 4; ++c)
                                acc[m][r * 4 + c] = fmaf(av[r], bv[c], acc[m][r * 4 + c]);
                    }
                }
            }
        }
        // lower triangle: entry (J4 + c, I4 + r) of the upper block (I4 + r, J4 + c)
#pragma unroll
        for (int m = 0; m < PERL; ++m)
            if (lane + 32 * m < NBLK)
            {
                const int I4 = 4 * bI[m], J4 = 4 * bJ[m];
#pragma unroll
                for (int r = 0; r < 4; ++r)
#pragma unroll
                    for (int c = 0; c < 4; ++c)
                        if (I4 + r <= J4 + c)
                            S.Lp[tri(J4 + c) + I4 + r] = acc[m][r * 4 + c];
            }
        __syncwarp();
        float trace = ((lane < k) ? S.Lp[t0 + lane] : 0.f) + ((lane + 32 < k) ? S.Lp[t1 + lane + 32] : 0.f);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            trace += __shfl_xor_sync(0xffffffffu, trace, o);
        const float shift = (float)klle_shift * trace;
        // regularised diagonal; padding rows and columns (zero) get an identity block
        S.Lp[t0 + lane] = (lane < k) ? S.Lp[t0 + lane] + shift : 1.f;
        S.Lp[t1 + lane + 32] = (lane + 32 < k) ? S.Lp[t1 + lane + 32] + shift : 1.f;
        __syncwarp();

        // ---- FP32 Cholesky in registers, solve with the packed factor ----
        {
            float A0[32], A1[64];
#pragma unroll
            for (int c = 0; c < 64; ++c)
            {
                if (c < 32)
                    A0[c & 31] = (c <= lane) ? S.Lp[t0 + c] : 0.f;
                A1[c] = (c <= lane + 32) ? S.Lp[t1 + c] : 0.f;
            }
            reg_cholesky64(A0, A1, S.ivd, lane);
            __syncwarp();
#pragma unroll
            for (int c = 0; c < 64; ++c)
            {
                if (c < 32 && c <= lane)
                    S.Lp[t0 + c] = A0[c & 31];
                if (c <= lane + 32)
                    S.Lp[t1 + c] = A1[c];
            }
        }
        __syncwarp();
        {
            float y0 = (lane < k) ? (rhs ? (float)rhs[i * k + lane] : 1.f) : 0.f;
            float y1 = (lane + 32 < k) ? (rhs ? (float)rhs[i * k + lane + 32] : 1.f) : 0.f;
            packed_solve64(S.Lp, S.ivd, y0, y1, lane);
            S.w[lane] = (lane < k) ? y0 : 0.f;
            S.w[lane + 32] = (lane + 32 < k) ? y1 : 0.f;
        }
        __syncwarp();

        // ---- float-float residual refinement ----
        const int iters = (k > D) ? 2 : 1;
        for (int itr = 0; itr < iters; ++itr)
        {
            ff sa[2] = {ff_zero(), ff_zero()}, ta[2] = {ff_zero(), ff_zero()};
            for (int d0 = 0; d0 < D; d0 += 32)
            {
                const int d = d0 + lane;
                const float xi = (d < D) ? X[i * ldx + d] : 0.f;
                __syncwarp();
#pragma unroll
                for (int h = 0; h < 2; ++h)
                {
                    float v[32];
#pragma unroll
                    for (int a = 0; a < 32; ++a)
                    {
                        const int nba = __shfl_sync(0xffffffffu, nb[h], a);
                        v[a] = (32 * h + a < k && d < D) ? X[(int64_t)nba * ldx + d] : xi;
                    }
#pragma unroll
                    for (int a = 0; a < 32; ++a)
                        S.B[32 * h + a][lane] = v[a];
                }
                S.xs[lane] = xi;
                __syncwarp();
                // v_d = sum_b w_b z_bd for d = d0 + lane, z exact by two-sum; four chains
                ff vq[4] = {ff_zero(), ff_zero(), ff_zero(), ff_zero()};
                for (int b = 0; b < k; b += 4)
#pragma unroll
                    for (int t = 0; t < 4; ++t)
                        if (b + t < k)
                        {
                            const ff z = two_sum(S.B[b + t][lane], -xi);
                            vq[t] = ff_fma(vq[t], S.w[b + t], 0.f, z.hi, z.lo);
                        }
                const ff vv = ff_add(ff_add(vq[0], vq[1]), ff_add(vq[2], vq[3]));
                S.vh[lane] = vv.hi;
                S.vl[lane] = vv.lo;
                __syncwarp();
#pragma unroll
                for (int s2 = 0; s2 < 2; ++s2)
                {
                    const int a = lane + 32 * s2;
                    if (a < k)
                        for (int dd = 0; dd < 32; ++dd)
                        {
                            const ff z = two_sum(S.B[a][dd], -S.xs[dd]);
                            sa[s2] = ff_fma(sa[s2], z.hi, z.lo, S.vh[dd], S.vl[dd]);
                            ta[s2] = ff_fma(ta[s2], z.hi, z.lo, z.hi, z.lo);
                        }
                }
                __syncwarp();
            }
            // exact trace = sum_a |z_a|^2
            ff tr = ff_add(ta[0], ta[1]);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
                tr = ff_add(tr, ff_shfl_xor(tr, o));
            const double shift_true = klle_shift * ff_to_double(tr);
            float y[2];
#pragma unroll
            for (int s2 = 0; s2 < 2; ++s2)
            {
                const int a = lane + 32 * s2;
                y[s2] = (a < k) ? (float)((rhs ? rhs[i * k + a] : 1.0) - ff_to_double(sa[s2]) -
                                          shift_true * (double)S.w[a])
                                : 0.f;
            }
            packed_solve64(S.Lp, S.ivd, y[0], y[1], lane);
            __syncwarp();
            if (lane < k)
                S.w[lane] += y[0];
            if (lane + 32 < k)
                S.w[lane + 32] += y[1];
            __syncwarp();
        }

        // ---- normalise (weights) or store the raw solution (adjoint solve) ----
        if (!normalize)
        {
            for (int a = lane; a < k; a += 32)
                W[i * k + a] = (double)S.w[a];
            __syncwarp();
            continue;
        }
        ff sum = ff_zero();
        for (int a = lane; a < k; a += 32)
            sum = ff_add(sum, ff{S.w[a], 0.f});
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            sum = ff_add(sum, ff_shfl_xor(sum, o));
        const float y0 = 1.f / sum.hi;
        const ff sy = two_prod(sum.hi, y0);
        const float resid = ((1.f - sy.hi) - sy.lo) - sum.lo * y0;  // 1 - sum * y0
        const float y1 = y0 * resid;
        for (int a = lane; a < k; a += 32)
        {
            const ff q = two_prod(S.w[a], y0);
            W[i * k + a] = (double)q.hi + (double)fmaf(S.w[a], y1, q.lo);
        }
        __syncwarp();
    }
}

template <int KP, int WARPS, bool BATCH>
void launch(tk_ctx* ctx, const LleRows& RW, const int32_t* idx, int k, double klle_shift, const double* rhs,
            int normalize, double* W)
{
    const size_t smem = sizeof(LleSmem<KP>) * WARPS;
    TK_CUDA(cudaFuncSetAttribute(k_lle<KP, WARPS, BATCH>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int64_t want = (RW.rows + WARPS - 1) / WARPS;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)ctx->num_sms * 16));
    k_lle<KP, WARPS, BATCH><<<grid, WARPS * 32, smem, ctx->stream>>>(RW, idx, k, klle_shift, rhs, normalize, W,
                                                               ctx->dev_err);
    TK_CHECK_LAUNCH();
}

template <bool BATCH>
void dispatch(tk_ctx* ctx, const LleRows& RW, const int32_t* idx, int k, double klle_shift, const double* rhs,
              bool normalize, double* W, int warps)
{
    const int nm = normalize ? 1 : 0;
    if (k <= 16 && warps == 4)
        launch<16, 4, BATCH>(ctx, RW, idx, k, klle_shift, rhs, nm, W);
    else if (k <= 16)
        launch<16, 8, BATCH>(ctx, RW, idx, k, klle_shift, rhs, nm, W);
    else if (k <= 32 && warps == 4)
        launch<32, 4, BATCH>(ctx, RW, idx, k, klle_shift, rhs, nm, W);
    else if (k <= 32)
        launch<32, 8, BATCH>(ctx, RW, idx, k, klle_shift, rhs, nm, W);
    else if (k <= 64)
        launch<64, 6, BATCH>(ctx, RW, idx, k, klle_shift, rhs, nm, W);
    else if (!BATCH && k <= 128)
        launch<128, 1, false>(ctx, RW, idx, k, klle_shift, rhs, nm, W);
    else
        throw Error(TK_ERR_UNSUPPORTED, "LLE weights support up to 128 neighbours (64 in a batch)");
}

} // namespace

void lle_solve(tk_ctx* ctx, const void* X, int dtype, int64_t N, int D, int64_t ldx, const int32_t* idx, int k,
               double klle_shift, const double* rhs, bool normalize, double* W)
{
    if (lle_pair_supported(X, dtype, ldx, k))
    {
        lle_pair_solve(ctx, X, N, D, ldx, idx, k, klle_shift, rhs, normalize, W);
        return;
    }
    if (dtype == TK_F32 && k > 32 && k <= 64)
    {
        const size_t smem = sizeof(Lle64Smem) * L64_WARPS;
        TK_CUDA(cudaFuncSetAttribute(k_lle64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        const int64_t want = (N + L64_WARPS - 1) / L64_WARPS;
        const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)ctx->num_sms));
        k_lle64<<<grid, L64_WARPS * 32, smem, ctx->stream>>>(reinterpret_cast<const float*>(X), N, D, ldx, idx, k,
                                                             klle_shift, rhs, normalize ? 1 : 0, W, ctx->dev_err);
        TK_CHECK_LAUNCH();
        return;
    }
    const LleRows RW{X, dtype, N, D, ldx, N, nullptr, nullptr, 0, nullptr};
    dispatch<false>(ctx, RW, idx, k, klle_shift, rhs, normalize, W, 8);
}

void lle_weights_batch(tk_ctx* ctx, const BatchProb* probs, const int32_t* row_prob, int64_t out_row0, int64_t rows,
                       const int32_t* idx, int k, double klle_shift, double* W, int warps)
{
    unsigned long long* work = (unsigned long long*)ctx->scratch.get("lle.work", 256);
    TK_CUDA(cudaMemsetAsync(work, 0, sizeof(unsigned long long), ctx->stream));
    const LleRows RW{nullptr, 0, 0, 0, 0, rows, row_prob, probs, out_row0, work};
    dispatch<true>(ctx, RW, idx, k, klle_shift, nullptr, true, W, warps);
}

void lle_weights(tk_ctx* ctx, const void* X, int dtype, int64_t N, int D, int64_t ldx, const int32_t* idx, int k,
                 double klle_shift, double* W)
{
    lle_solve(ctx, X, dtype, N, D, ldx, idx, k, klle_shift, nullptr, true, W);
}

} // namespace tk
