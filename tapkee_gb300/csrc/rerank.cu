// rerank.cu -- exact FP64 re-rank of screened candidates, certification, and the
// exact fallback for rows the screen cannot certify.
//
// The exact distance is the squared Euclidean distance the reference evaluates
// in kernel form (neighbors/neighbors.hpp:49-52, sqrt(k(i,i) - 2 k(i,j) + k(j,j)),
// squared here: sqrt is monotone and only the ranking is returned), computed as
// sum_d (x_d - y_d)^2 without cancellation:
//   * float32 input: x_d - y_d is split exactly into hi + lo floats and the
//     squares are accumulated in float-float (about 48 significant bits), on the
//     FP32 pipes -- GB300's FP64 rate is a small fraction of its FP32 rate;
//   * float64 input: differences and sums in FP64.
// Either is at least as accurate as the reference's FP64 kernel-trick value,
// whose cancellation error is ~1e-16 |x|^2. The k nearest other points are
// taken in (d2, index) order.
//
// Certification. The screen returns, per query, the KC candidates with the
// smallest approximate values a_j and their largest value T. With the error
// model |a_j - d2_j| <= eps = c1 (|x|^2 + R^2) + c2 |x| R (R = max |x - mean|,
// see screen_error_model), every point outside the list has d2 >= T - eps. If
// the exact k-th smallest d2 among the candidates, e_k, satisfies e_k < T - eps,
// no outside point can enter the top k and the row is exact. Otherwise the row
// goes to the fallback, which scans all N points with an FP32 direct-difference
// filter (relative error <= (D + 4) 2^-23) against e_k, then ranks the few
// survivors in FP64.
//
// Ties at the k-boundary. The reference keeps the first k + 1 records of
// std::nth_element(begin, begin + k + 1, end) over all N (point, distance)
// records in index order, minus the query itself (neighbors/neighbors.hpp:
// 129-146), so exact ties across the boundary are broken by the positions the
// partition leaves them in, not by index. A row whose k-th and (k + 1)-th
// nearest exact distances lie within 1e-12 relative is a tie row: it is counted,
// and k_nth_select recomputes it with a restatement of libstdc++'s introselect
// over the row's N records, taking the first k + 1 records minus the query, in
// partition order. When the query has k + 1 or more exact duplicates it can fall
// outside those k + 1 records; the reference then returns k + 1 neighbours for
// the row. Such rows are counted and listed with their (k + 1)-th neighbour; the
// first k are returned, which is what the reference's weight and connectivity
// routines read (they take k from neighbors[0].size(): routines/
// locally_linear.hpp:96, neighbors/connected.hpp:27).
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>

#include "ff.cuh"
#include "nth_select.h"
#include "tk_internal.h"

namespace tk {
namespace {

constexpr int FB_CAP = 4096;  // fallback survivors per row

__device__ __forceinline__ double ldx_elem(const void* X, int dtype, int64_t off)
{
    return dtype == TK_F64 ? reinterpret_cast<const double*>(X)[off] : (double)reinterpret_cast<const float*>(X)[off];
}

__device__ __forceinline__ bool key_less(double da, int ja, double db, int jb)
{
    return da < db || (da == db && ja < jb);
}

// One warp per query position p (sorted order). Lane l owns candidates
// l, l+32, l+64, ... (KC <= 256).
// Exact squared distance between rows a and b (see the header).
__device__ __forceinline__ double exact_d2(const void* X, int dtype, int64_t ldx, int D, int64_t a, int64_t b)
{
    if (dtype == TK_F64)
    {
        const double* xa = reinterpret_cast<const double*>(X) + a * ldx;
        const double* xb = reinterpret_cast<const double*>(X) + b * ldx;
        double s = 0.0;
        for (int d = 0; d < D; ++d)
        {
            const double z = xa[d] - xb[d];
            s = fma(z, z, s);
        }
        return s;
    }
    const float* xa = reinterpret_cast<const float*>(X) + a * ldx;
    const float* xb = reinterpret_cast<const float*>(X) + b * ldx;
    ff acc = ff_zero();
    float cross = 0.f;  // sum of 2 hi lo (relative size 2^-24 of the total)
    for (int d = 0; d < D; ++d)
    {
        const ff z = two_sum(xa[d], -xb[d]);  // exact difference hi + lo
        acc = ff_add(acc, two_prod(z.hi, z.hi));
        cross = fmaf(2.f * z.hi, z.lo, cross);
    }
    return ff_to_double(acc) + (double)cross;
}

// The exact distance as a normalised float pair (hi, lo): float-float for
// float32 input, the FP64 value split for float64 input. Comparing (hi, lo)
// lexicographically orders the values without FP64 arithmetic.
__device__ __forceinline__ ff exact_key(const void* X, int dtype, int64_t ldx, int D, int64_t a, int64_t b)
{
    if (dtype == TK_F64)
    {
        const double v = exact_d2(X, dtype, ldx, D, a, b);
        const float h = (float)v;
        return ff{h, (float)(v - (double)h)};
    }
    const float* xa = reinterpret_cast<const float*>(X) + a * ldx;
    const float* xb = reinterpret_cast<const float*>(X) + b * ldx;
    ff acc = ff_zero();
    float cross = 0.f;
    for (int d = 0; d < D; ++d)
    {
        const ff z = two_sum(xa[d], -xb[d]);
        acc = ff_add(acc, two_prod(z.hi, z.hi));
        cross = fmaf(2.f * z.hi, z.lo, cross);
    }
    return ff_add(acc, ff{cross, 0.f});
}

__device__ __forceinline__ bool key_less_ff(float ha, float la, int ja, float hb, float lb, int jb)
{
    return ha < hb || (ha == hb && (la < lb || (la == lb && ja < jb)));
}

// The problem a screened row belongs to, and the row's original index in it.
struct RowView
{
    const void* X;
    int dtype;
    int64_t ldx;
    int D;
    int64_t N;
    int k;
    int64_t i;
    float R;
    const int32_t* perm;  // candidate id -> original index (NULL: identity)
    int32_t* idx_out;
    double* d2_out;
};

template <bool BATCH>
__device__ __forceinline__ bool row_view(const RowSpace& S, int64_t p, RowView& v)
{
    if constexpr (!BATCH)
    {
        v = RowView{S.X, S.dtype, S.ldx, S.D, S.N, S.k, (int64_t)S.perm[p], *S.R, S.perm, S.idx_out, S.d2_out};
        return true;
    }
    const int b = S.row_prob[p];
    if (b < 0)
        return false;
    const BatchProb& P = S.probs[b];
    if (p - P.row0 >= P.N)
        return false;
    v = RowView{P.X,      P.dtype,          P.ldx,   P.D, P.N, P.k, (int64_t)S.perm[p], S.prob_R[b], S.perm + P.row0,
                S.idx_all + P.idx_off, nullptr};
    return true;
}

constexpr int RR_WARPS = 8;
constexpr int RR_QMAX = 256;  // largest D whose query row is staged in shared memory

// One warp per query row; lane l owns candidates l, l + 32, ... (KC <= 256).
// float32 input: every candidate gets an FP32 direct-difference distance f (any
// summation order) with
// |f - d2| <= gam f (gam = (D + 8) 2^-23). Since gam f is increasing in f, the
// intervals [(1 - gam) f, (1 + gam) f] of candidates taken in f order are
// ordered too wherever neighbours in that order do not overlap; so only the
// candidates whose interval overlaps a rank neighbour among the first k + 1,
// and the later ones whose interval reaches below the upper end of rank k's,
// need their exact (float-float) distance, and the ranking by (key, index) with
// key = exact value where computed, else f, is the exact ranking. float64 input:
// every candidate's distance in FP64.
template <int KC, bool BATCH>
__global__ void __launch_bounds__(RR_WARPS * 32)
    k_rerank(const RowSpace RS, int64_t rows, const float* nrm, const int32_t* cand_idx, const float* cand_val,
             float c1, float c2, int32_t* failed, double* failed_ub, unsigned* nfailed, int32_t* tie_list,
             unsigned* ntie)
{
    constexpr int PER = (KC + 31) / 32;
    constexpr int NONE = 0x7fffffff - 255;  // slots >= NONE hold no candidate
    __shared__ float f_s[RR_WARPS][KC];
    __shared__ __align__(16) float q_s[RR_WARPS][RR_QMAX];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    float* fr = f_s[wib];
    float* qs = q_s[wib];
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t p = warp; p < rows; p += nwarps)
    {
        RowView V;
        if (!row_view<BATCH>(RS, p, V))
            continue;
        const void* X = V.X;
        const int dtype = V.dtype;
        const int64_t ldx = V.ldx;
        const int D = V.D;
        const int64_t N = V.N;
        const int k = V.k;
        const int64_t i = V.i;
        // relative error bound of the FP32 distances, plus the rounding of the
        // float products that apply it
        const float gam = (float)(D + 8) * 1.1920928955078125e-07f + 4.76837158203125e-07f;
        float kh[PER], kl[PER];  // keys: exact (hi, lo) or the FP32 value (lo = 0)
        int j[PER];
        bool exact[PER];
#pragma unroll
        for (int s = 0; s < PER; ++s)
        {
            const int slot = lane + 32 * s;
            kh[s] = __int_as_float(0x7f800000);  // +inf
            kl[s] = 0.f;
            j[s] = 0x7fffffff - slot;            // distinct, ranks last
            exact[s] = true;
            if (slot < KC)
            {
                const int c = cand_idx[p * KC + slot];
                if (c >= 0 && c < N)
                {
                    const int64_t jj = V.perm ? V.perm[c] : c;
                    if (jj != i)
                        j[s] = (int)jj;
                }
            }
        }
        if (dtype == TK_F64)
        {
#pragma unroll
            for (int s = 0; s < PER; ++s)
                if (j[s] < NONE)
                {
                    const ff e = exact_key(X, dtype, ldx, D, i, j[s]);
                    kh[s] = e.hi;
                    kl[s] = e.lo;
                }
        }
        else if (D <= RR_QMAX && (ldx & 3) == 0 && (reinterpret_cast<uintptr_t>(X) & 15) == 0)
        {
            // FP32 screen of the candidates, lanes owning candidates: each lane
            // reads its candidate's row with 16-byte loads (the rest of each
            // sector stays in L1 for the next load) against the query row
            // staged in shared memory, read as a broadcast
            const float* Xf = reinterpret_cast<const float*>(X);
            __syncwarp();
            for (int d = lane; d < D; d += 32)
                qs[d] = __ldg(Xf + i * ldx + d);
            __syncwarp();
            const int D4 = D >> 2;
            const float4* q4 = reinterpret_cast<const float4*>(qs);
#pragma unroll
            for (int s = 0; s < PER; ++s)
                if (j[s] < NONE)
                {
                    const float* yr = Xf + (int64_t)j[s] * ldx;
                    const float4* y4 = reinterpret_cast<const float4*>(yr);
                    // two dimensions per packed FP32 instruction: z = y - x (one
                    // rounding, as a subtraction), acc += z z
                    const float2 m1 = make_float2(-1.f, -1.f);
                    float2 aa = make_float2(0.f, 0.f), ab = aa;
#pragma unroll 8
                    for (int t = 0; t < D4; ++t)
                    {
                        const float4 y = __ldg(y4 + t);
                        const float4 x = q4[t];
                        const float2 z0 = __ffma2_rn(make_float2(x.x, x.y), m1, make_float2(y.x, y.y));
                        const float2 z1 = __ffma2_rn(make_float2(x.z, x.w), m1, make_float2(y.z, y.w));
                        aa = __ffma2_rn(z0, z0, aa);
                        ab = __ffma2_rn(z1, z1, ab);
                    }
                    float a = (aa.x + aa.y) + (ab.x + ab.y);
                    for (int d = 4 * D4; d < D; ++d)
                    {
                        const float z = __ldg(yr + d) - qs[d];
                        a = fmaf(z, z, a);
                    }
                    kh[s] = a;
                    exact[s] = false;
                }
        }
        else if (D < 32)
        {
            // few dimensions in rows that are not 16-byte aligned: lanes own
            // candidates, scalar loads against the query row staged in shared
            // memory (lanes owning dimensions would leave most lanes idle)
            const float* Xf = reinterpret_cast<const float*>(X);
            __syncwarp();
            if (lane < D)
                qs[lane] = __ldg(Xf + i * ldx + lane);
            __syncwarp();
#pragma unroll
            for (int s = 0; s < PER; ++s)
                if (j[s] < NONE)
                {
                    const float* yr = Xf + (int64_t)j[s] * ldx;
                    float a = 0.f;
                    for (int d = 0; d < D; ++d)
                    {
                        const float z = __ldg(yr + d) - qs[d];
                        a = fmaf(z, z, a);
                    }
                    kh[s] = a;
                    exact[s] = false;
                }
        }
        else
        {
            // FP32 screen of the candidates: lanes own dimensions, so every row
            // load is one coalesced 128-byte segment; a warp reduce-scatter leaves
            // candidate l's sum in lane l
            const float* Xf = reinterpret_cast<const float*>(X);
#pragma unroll
            for (int s = 0; s < PER; ++s)
            {
                float part[32];
#pragma unroll
                for (int r = 0; r < 32; ++r)
                    part[r] = 0.f;
                for (int d0 = 0; d0 < D; d0 += 32)
                {
                    const int d = d0 + lane;
                    const float xq = (d < D) ? __ldg(Xf + i * ldx + d) : 0.f;
#pragma unroll
                    for (int r = 0; r < 32; ++r)
                    {
                        const int row = __shfl_sync(0xffffffffu, j[s], r);
                        if (row < NONE && d < D)
                        {
                            const float z = __ldg(Xf + (int64_t)row * ldx + d) - xq;
                            part[r] = fmaf(z, z, part[r]);
                        }
                    }
                }
#pragma unroll
                for (int lvl = 0; lvl < 5; ++lvl)
                {
                    const int o = 16 >> lvl;
                    const bool upper = (lane & o) != 0;
#pragma unroll
                    for (int q = 0; q < o; ++q)
                    {
                        const float send = upper ? part[q] : part[q + o];
                        const float keep = upper ? part[q + o] : part[q];
                        part[q] = keep + __shfl_xor_sync(0xffffffffu, send, o);
                    }
                }
                if (j[s] < NONE)
                {
                    kh[s] = part[0];
                    exact[s] = false;
                }
            }
        }
        // rank of every element among the KC (key, j) triples
        int rank[PER];
        auto rank_all = [&]() {
#pragma unroll
            for (int s = 0; s < PER; ++s)
                rank[s] = 0;
#pragma unroll
            for (int so = 0; so < PER; ++so)
                for (int m = 0; m < 32; ++m)
                {
                    const float hm = __shfl_sync(0xffffffffu, kh[so], m);
                    const float lm = __shfl_sync(0xffffffffu, kl[so], m);
                    const int jm = __shfl_sync(0xffffffffu, j[so], m);
#pragma unroll
                    for (int s = 0; s < PER; ++s)
                        rank[s] += key_less_ff(hm, lm, jm, kh[s], kl[s], j[s]) ? 1 : 0;
                }
        };
        rank_all();
        if (dtype != TK_F64)
        {
            // overlap test of rank neighbours among ranks 0..k
            __syncwarp();
#pragma unroll
            for (int s = 0; s < PER; ++s)
                if (lane + 32 * s < KC)
                    fr[rank[s]] = kh[s];
            __syncwarp();
            bool need[PER];
            bool any = false;
            // upper end of the interval of rank k (the (k + 1)-th smallest f): a
            // candidate of a later rank whose interval reaches below it may still
            // be among the first k + 1 once exact values replace f, so it is
            // refined too (equal f at the boundary: duplicated points)
            const float U = fr[k] * (1.f + gam);
#pragma unroll
            for (int s = 0; s < PER; ++s)
            {
                need[s] = false;
                const int r = rank[s];
                if (!exact[s] && r <= k)
                {
                    const float lo = kh[s] * (1.f - gam), hi = kh[s] * (1.f + gam);
                    if (r < k && fr[r + 1] * (1.f - gam) <= hi)
                        need[s] = true;
                    if (r > 0 && fr[r - 1] * (1.f + gam) >= lo)
                        need[s] = true;
                    // distances returned to the caller are exact
                    if (V.d2_out && r < k)
                        need[s] = true;
                }
                else if (!exact[s] && kh[s] * (1.f - gam) <= U)
                    need[s] = true;
                any |= need[s];
            }
            if (__any_sync(0xffffffffu, any))
            {
#pragma unroll
                for (int s = 0; s < PER; ++s)
                    if (need[s])
                    {
                        const ff e = exact_key(X, dtype, ldx, D, i, j[s]);
                        kh[s] = e.hi;
                        kl[s] = e.lo;
                        exact[s] = true;
                    }
                rank_all();
            }
        }
        // e_k: an upper bound of the exact k-th distance, from the lane holding
        // rank k-1, rounded up to FP32 (exact pair: hi + lo rounded up; FP32
        // value: f (1 + gam) rounded up)
        unsigned own = 0u;
        float ek_own = 0.f;
#pragma unroll
        for (int s = 0; s < PER; ++s)
            if (rank[s] == k - 1)
            {
                own = 1u;
                ek_own = exact[s] ? __fadd_ru(kh[s], kl[s]) : __fmul_ru(kh[s], __fadd_ru(1.f, gam));
            }
        const unsigned holder = __ballot_sync(0xffffffffu, own != 0u);
        const float ek = __shfl_sync(0xffffffffu, ek_own, holder ? __ffs(holder) - 1 : 0);
        bool certified = true;
        if (lane == 0)
        {
            // the bounds eps are rounded up and T - eps down, so every comparison
            // is at least as strict as in exact arithmetic (FP32 throughout: no
            // FP64 square root per row)
            const float R = V.R;
            const float nx = nrm[p];
            const float base = __fmul_ru(c1, __fadd_ru(nx, __fmul_ru(R, R)));
            const float sr = __fmul_ru(__fsqrt_ru(nx), R);
            const float T = cand_val[p * KC + KC - 1];
            if (T < FLT_MAX)  // a full list: points outside it are bounded below
            {
                const float eps = __fadd_ru(base, __fmul_ru(c2, sr));
                certified = ek < __fsub_rd(T, eps);
            }
            if (RS.far_val)
            {
                // candidates in tiles screened with high parts only: all have
                // screened values >= far_val, with the larger far error bound
                const float A = RS.far_val[p];
                if (A < FLT_MAX)
                {
                    const float eps_far = __fadd_ru(base, __fmul_ru(RS.c2_far, sr));
                    certified = certified && ek < __fsub_rd(A, eps_far);
                }
            }
        }
        certified = __shfl_sync(0xffffffffu, certified, 0);
        if (certified)
        {
#pragma unroll
            for (int s = 0; s < PER; ++s)
                if (rank[s] < k)
                {
                    V.idx_out[i * k + rank[s]] = j[s];
                    if (V.d2_out)
                        V.d2_out[i * k + rank[s]] = (double)kh[s] + (double)kl[s];
                }
            // tie row: ranks k - 1 and k both exact and within 1e-12 relative.
            // Where their FP32 intervals do not overlap (a relative gap of at
            // least ~2^-21) they were not refined, and the row is no tie row.
            unsigned h1 = 0u, h2 = 0u;
            double v1 = 0.0, v2 = 0.0;
#pragma unroll
            for (int s = 0; s < PER; ++s)
            {
                if (rank[s] == k - 1 && exact[s])
                {
                    h1 = 1u;
                    v1 = (double)kh[s] + (double)kl[s];
                }
                if (rank[s] == k && exact[s] && j[s] < NONE)
                {
                    h2 = 1u;
                    v2 = (double)kh[s] + (double)kl[s];
                }
            }
            const unsigned b1 = __ballot_sync(0xffffffffu, h1 != 0u);
            const unsigned b2 = __ballot_sync(0xffffffffu, h2 != 0u);
            if (b1 && b2)
            {
                const double a = __shfl_sync(0xffffffffu, v1, __ffs(b1) - 1);
                const double b = __shfl_sync(0xffffffffu, v2, __ffs(b2) - 1);
                if (lane == 0 && b - a <= 1e-12 * b)
                    tie_list[atomicAdd(ntie, 1u)] = (int32_t)p;
            }
        }
        else if (lane == 0)
        {
            const unsigned fidx = atomicAdd(nfailed, 1u);
            failed[fidx] = (int32_t)p;
            failed_ub[fidx] = (double)ek;
        }
    }
}

// Exact fallback: one CTA per failed row (persistent over the failed list).
template <bool BATCH>
__global__ void __launch_bounds__(256) k_fallback(const RowSpace RS, const int32_t* failed,
                                                  const double* failed_ub, const unsigned* nfailed, unsigned* err,
                                                  int32_t* tie_list, unsigned* ntie)
{
    __shared__ int32_t sj[FB_CAP];
    __shared__ double sd[FB_CAP];
    __shared__ unsigned cnt;
    __shared__ double edge[2];  // exact distances of ranks k - 1 and k
    __shared__ int edge_n;
    const unsigned nf = *nfailed;
    for (unsigned f = blockIdx.x; f < nf; f += gridDim.x)
    {
        const int64_t p = failed[f];
        RowView V;
        if (!row_view<BATCH>(RS, p, V))
            continue;
        const void* X = V.X;
        const int dtype = V.dtype;
        const int64_t ldx = V.ldx;
        const int D = V.D;
        const int64_t N = V.N;
        const int k = V.k;
        const int64_t i = V.i;
        int32_t* idx_out = V.idx_out;
        double* d2_out = V.d2_out;
        double ub = failed_ub[f];
        // FP32 direct-difference filter with a relative slack covering its error
        const double slack = (double)(D + 8) * 1.1920928955078125e-07;
        // More survivors than slots: the k-th smallest exact distance among the
        // FB_CAP kept (real points) bounds e_k too, so the scan is repeated with
        // that tighter bound (a few times at most).
        for (int attempt = 0;; ++attempt)
        {
            const float thr = (float)(ub * (1.0 + slack)) * 1.0000005f + 1e-30f;
            if (threadIdx.x == 0)
            {
                cnt = 0;
                edge_n = 0;
            }
            __syncthreads();
            for (int64_t jj = threadIdx.x; jj < N; jj += blockDim.x)
            {
                if (jj == i)
                    continue;
                float acc = 0.f;
                for (int d0 = 0; d0 < D; d0 += 1024)
                {
                    // D > 1024 is handled in chunks without caching the query
                    for (int d = d0; d < min(D, d0 + 1024); ++d)
                    {
                        const float v = (float)(ldx_elem(X, dtype, jj * ldx + d) - ldx_elem(X, dtype, i * ldx + d));
                        acc = fmaf(v, v, acc);
                    }
                }
                if (acc <= thr)
                {
                    const unsigned s = atomicAdd(&cnt, 1u);
                    if (s < FB_CAP)
                        sj[s] = (int32_t)jj;
                }
            }
            __syncthreads();
            if (cnt <= (unsigned)FB_CAP)
                break;
            if (attempt == 4)
            {
                if (threadIdx.x == 0)
                    atomicOr(err, DEV_ERR_OVERFLOW);
                break;
            }
            for (unsigned t = threadIdx.x; t < (unsigned)FB_CAP; t += blockDim.x)
                sd[t] = exact_d2(X, dtype, ldx, D, i, sj[t]);
            __syncthreads();
            for (unsigned t = threadIdx.x; t < (unsigned)FB_CAP; t += blockDim.x)
            {
                unsigned r = 0;
                for (unsigned m = 0; m < (unsigned)FB_CAP; ++m)
                    r += (sd[m] < sd[t] || (sd[m] == sd[t] && m < t)) ? 1u : 0u;
                if (r == (unsigned)k - 1)
                    edge[0] = sd[t];  // the kept set's k-th smallest
            }
            __syncthreads();
            ub = edge[0];
            __syncthreads();
        }
        const unsigned n = min(cnt, (unsigned)FB_CAP);
        for (unsigned t = threadIdx.x; t < n; t += blockDim.x)
            sd[t] = exact_d2(X, dtype, ldx, D, i, sj[t]);
        __syncthreads();
        if (n < (unsigned)k && threadIdx.x == 0)
            atomicOr(err, DEV_ERR_BOUNDS);
        for (unsigned t = threadIdx.x; t < n; t += blockDim.x)
        {
            unsigned r = 0;
            for (unsigned m = 0; m < n; ++m)
                r += key_less(sd[m], sj[m], sd[t], sj[t]) ? 1u : 0u;
            if (r < (unsigned)k)
            {
                idx_out[i * k + r] = sj[t];
                if (d2_out)
                    d2_out[i * k + r] = sd[t];
            }
            // the (k + 1)-th nearest is a survivor whenever it ties with the k-th:
            // the filter keeps every point up to the k-th distance's upper bound
            if (r + 1 == (unsigned)k || r == (unsigned)k)
            {
                edge[r - (k - 1)] = sd[t];
                atomicAdd(&edge_n, 1);
            }
        }
        __syncthreads();
        if (threadIdx.x == 0 && edge_n == 2 && edge[1] - edge[0] <= 1e-12 * edge[1])
            tie_list[atomicAdd(ntie, 1u)] = (int32_t)p;
        __syncthreads();
    }
}

// One CTA per tie row (persistent over the tie list). The CTA computes the row's
// N exact distances into its slot of the record scratch (N doubles and N ints),
// then thread 0 runs the selection and writes the first k records of the first
// k + 1 minus the query, in partition order. A row where the query is not among
// the first k + 1 records is listed in extra (row, (k + 1)-th neighbour).
template <bool BATCH>
__global__ void __launch_bounds__(256) k_nth_select(const RowSpace RS, const int32_t* tie_list, const unsigned* ntie,
                                                    double* rec_d, int32_t* rec_j, int64_t rec_stride,
                                                    int32_t* extra, unsigned* nextra, unsigned* err)
{
    const unsigned nt = *ntie;
    double* d = rec_d + (int64_t)blockIdx.x * rec_stride;
    int32_t* jv = rec_j + (int64_t)blockIdx.x * rec_stride;
    for (unsigned t = blockIdx.x; t < nt; t += gridDim.x)
    {
        const int64_t p = tie_list[t];
        RowView V;
        if (!row_view<BATCH>(RS, p, V))
            continue;
        const int64_t N = V.N, i = V.i;
        const int k = V.k;
        __syncthreads();  // the previous row's records are no longer read
        for (int64_t m = threadIdx.x; m < N; m += blockDim.x)
        {
            d[m] = exact_d2(V.X, V.dtype, V.ldx, V.D, i, m);
            jv[m] = (int32_t)m;
        }
        __syncthreads();
        if (threadIdx.x == 0)
        {
            NthSelect S{d, jv, false};
            S.nth_element(N, (int64_t)k + 1);
            if (S.bad)
                atomicOr(err, DEV_ERR_NONFINITE);
            else
            {
                const int64_t top = ((int64_t)k + 1 < N) ? (int64_t)k + 1 : N;
                int c = 0;
                int32_t last_other = -1;
                for (int64_t m = 0; m < top; ++m)
                {
                    if (jv[m] == (int32_t)i)
                        continue;
                    if (c < k)
                    {
                        V.idx_out[i * k + c] = jv[m];
                        if (V.d2_out)
                            V.d2_out[i * k + c] = d[m];
                        ++c;
                    }
                    else
                        last_other = jv[m];
                }
                if (last_other >= 0)
                {
                    const unsigned e = atomicAdd(nextra, 1u);
                    if (extra)
                    {
                        extra[2 * e] = (int32_t)i;
                        extra[2 * e + 1] = last_other;
                    }
                }
            }
        }
    }
}

} // namespace

void screen_error_model_far(int Dp, float* c2)
{
    const double u = 5.9604644775390625e-08;  // 2^-24
    // x.y ~ h_x.h_y: the dropped h_x.l_y + l_x.h_y + l_x.l_y is at most
    // (2 2^-11 + 2^-22) |x||y| (|l| <= 2^-11 |x| elementwise, Cauchy-Schwarz),
    // plus FP32 accumulation of Dp / 16 + 1 K-steps (2 ulp each) and the
    // intra-instruction sum (8 ulp); doubled for the 2 x.y term and again for safety
    const double split = 2.0 * 4.8828125e-04 + 2.384185791015625e-07;
    const double accum = (Dp / 16.0 * 2.0 + 10.0) * 2.0 * u;
    *c2 = (float)(2.0 * (split + accum) * 2.0);
}

void screen_error_model(int screen, int Dp, float* c1, float* c2)
{
    const double u = 5.9604644775390625e-08;  // 2^-24
    // c1 covers rounding of the centred coordinates and of the FP32 norms and
    // the final a = |x|^2 + |y|^2 - 2 x.y evaluation.
    *c1 = (float)(16.0 * u);
    if (screen == TK_SCREEN_FP32)
    {
        // sequential FP32 FMA accumulation of Dp products: |err| <= Dp u sum|x_d y_d| <= Dp u |x||y|
        *c2 = (float)(2.0 * (Dp + 4) * u * 2.0);
    }
    else
    {
        // fp16 split x = h + l (|l| <= 2^-11 |x|, l rounded to 2^-22 |x|), dropped l*l
        // term (<= 2^-22 |x||y|), and FP32 tensor-core accumulation of 3 Dp / 16
        // K-steps, each assumed to add at most 2 ulp (truncating adds), plus the
        // intra-instruction sum (8 ulp): all relative to |x||y|.
        const double split = 3.0 * 2.384185791015625e-07;          // 3 * 2^-22
        const double accum = (3.0 * Dp / 16.0 * 2.0 + 8.0) * 2.0 * u;  // ulp = 2^-23
        *c2 = (float)(2.0 * (split + accum) * 2.0);
        // |y|^2 enters through an fp16 hi/lo column (relative 2^-22) and raises the
        // accumulator magnitude by |y|^2 / 2 over the 3 Dp / 16 + 1 K-steps
        *c1 += (float)(2.384185791015625e-07 + (3.0 * Dp / 16.0 + 3.0) * 2.0 * u);
    }
}

namespace {

// Counters of one re-rank pass (device, 16 bytes, cleared by launch_rerank):
// [0] uncertified rows, [1] tie rows, [2] rows with k + 1 reference neighbours.
constexpr int CNT_FAILED = 0, CNT_TIES = 1, CNT_EXTRA = 2;

// CTAs of the tie-row selection: each holds a row's N records (12 B each) in
// the scratch, which is kept to about 64 MB.
int select_grid(tk_ctx* ctx, int64_t max_n)
{
    const int64_t per = std::max<int64_t>(max_n, 1) * 12;
    return (int)std::max<int64_t>(1, std::min<int64_t>(2 * ctx->num_sms, ((int64_t)64 << 20) / per));
}

template <bool BATCH>
void launch_rerank(tk_ctx* ctx, const RowSpace& S, int64_t rows, int kc, const int32_t* cand_idx,
                   const float* cand_val, const float* nrm, float eps_c1, float eps_c2, int32_t* failed,
                   double* failed_ub, int32_t* ties, unsigned* counts)
{
    cudaStream_t st = ctx->stream;
    TK_CUDA(cudaMemsetAsync(counts, 0, 4 * sizeof(unsigned), st));
    const int blocks = 8 * ctx->num_sms;
#define TK_RERANK(KCV)                                                                                         \
    k_rerank<KCV, BATCH><<<blocks, RR_WARPS * 32, 0, st>>>(S, rows, nrm, cand_idx, cand_val, eps_c1, eps_c2, failed,    \
                                                    failed_ub, counts + CNT_FAILED, ties, counts + CNT_TIES)
    if (kc == 32)
        TK_RERANK(32);
    else if (kc == 64)
        TK_RERANK(64);
    else if (kc == 128)
        TK_RERANK(128);
    else if (kc == 256)
        TK_RERANK(256);
    else
        throw Error(TK_ERR_INTERNAL, "rerank: unsupported candidate count");
#undef TK_RERANK
    TK_CHECK_LAUNCH();
    k_fallback<BATCH><<<ctx->num_sms, 256, 0, st>>>(S, failed, failed_ub, counts + CNT_FAILED, ctx->dev_err, ties,
                                                    counts + CNT_TIES);
    TK_CHECK_LAUNCH();
}

} // namespace

int64_t rerank(tk_ctx* ctx, const Prepared& P, const void* X, int dtype, int64_t ldx, int k, int kc,
               const int32_t* cand_idx, const float* cand_val, float eps_c1, float eps_c2, int32_t* idx_out,
               double* d2_out)
{
    cudaStream_t st = ctx->stream;
    const int64_t N = P.N;
    int32_t* failed = (int32_t*)ctx->scratch.get("rerank.failed", sizeof(int32_t) * (size_t)N);
    double* failed_ub = (double*)ctx->scratch.get("rerank.failed_ub", sizeof(double) * (size_t)N);
    int32_t* ties = (int32_t*)ctx->scratch.get("rerank.ties", sizeof(int32_t) * (size_t)N);
    unsigned* counts = (unsigned*)ctx->scratch.get("rerank.nfailed", 16);
    RowSpace S;
    S.X = X;
    S.dtype = dtype;
    S.ldx = ldx;
    S.D = P.D;
    S.N = N;
    S.k = k;
    S.perm = P.perm;
    S.R = P.rmax;
    S.idx_out = idx_out;
    S.d2_out = d2_out;
    S.far_val = P.far_val;
    S.c2_far = P.c2_far;
    launch_rerank<false>(ctx, S, N, kc, cand_idx, cand_val, P.nrm, eps_c1, eps_c2, failed, failed_ub, ties, counts);
    unsigned* hc = reinterpret_cast<unsigned*>(ctx->host_i64);
    TK_CUDA(cudaMemcpyAsync(hc, counts, 4 * sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    TK_CUDA(cudaStreamSynchronize(st));
    const int64_t nfailed = hc[CNT_FAILED];
    const int64_t nties = hc[CNT_TIES];
    ctx->knn_ties = nties;
    ctx->knn_extra = 0;
    if (nties > 0)
    {
        // the reference's selection for the tie rows (rare: exact ties occur in
        // duplicated or lattice data, not in continuous noise)
        const int grid = select_grid(ctx, N);
        double* rec_d = (double*)ctx->scratch.get("rerank.sel_d", sizeof(double) * (size_t)grid * N);
        int32_t* rec_j = (int32_t*)ctx->scratch.get("rerank.sel_j", sizeof(int32_t) * (size_t)grid * N);
        int32_t* extra = (int32_t*)ctx->scratch.get("rerank.extra", sizeof(int32_t) * 2 * (size_t)nties);
        k_nth_select<false><<<grid, 256, 0, st>>>(S, ties, counts + CNT_TIES, rec_d, rec_j, N, extra,
                                                  counts + CNT_EXTRA, ctx->dev_err);
        TK_CHECK_LAUNCH();
        TK_CUDA(cudaMemcpyAsync(hc, counts, 4 * sizeof(unsigned), cudaMemcpyDeviceToHost, st));
        TK_CUDA(cudaStreamSynchronize(st));
        ctx->knn_extra = hc[CNT_EXTRA];
    }
    return nfailed;
}

void rerank_batch(tk_ctx* ctx, const RowSpace& S, int64_t rows, int64_t max_n, int kc, const int32_t* cand_idx,
                  const float* cand_val, const float* nrm, float eps_c1, float eps_c2, unsigned* counts_out)
{
    int32_t* failed = (int32_t*)ctx->scratch.get("rerank.failed", sizeof(int32_t) * (size_t)rows);
    double* failed_ub = (double*)ctx->scratch.get("rerank.failed_ub", sizeof(double) * (size_t)rows);
    int32_t* ties = (int32_t*)ctx->scratch.get("rerank.ties", sizeof(int32_t) * (size_t)rows);
    launch_rerank<true>(ctx, S, rows, kc, cand_idx, cand_val, nrm, eps_c1, eps_c2, failed, failed_ub, ties,
                        counts_out);
    // the selection reads the tie count on the device (no host synchronisation
    // inside a captured batch); extra rows are counted, not listed
    const int grid = select_grid(ctx, max_n);
    double* rec_d = (double*)ctx->scratch.get("rerank.sel_d", sizeof(double) * (size_t)grid * max_n);
    int32_t* rec_j = (int32_t*)ctx->scratch.get("rerank.sel_j", sizeof(int32_t) * (size_t)grid * max_n);
    k_nth_select<true><<<grid, 256, 0, ctx->stream>>>(S, ties, counts_out + CNT_TIES, rec_d, rec_j, max_n, nullptr,
                                                      counts_out + CNT_EXTRA, ctx->dev_err);
    TK_CHECK_LAUNCH();
}

} // namespace tk
