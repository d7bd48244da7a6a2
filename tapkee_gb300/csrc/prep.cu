// prep.cu -- lays the point cloud out for distance screening.
//
// Steps (all on the context stream, no host synchronisation):
//   1. column mean mu (FP64, deterministic two-level reduction);
//   2. a 16-dimensional random sketch s_i = G^T (x_i - mu) of a subsample of the
//      points (FP32) and its 16x16 covariance (deterministic per-block partials);
//   3. the 3 leading principal directions of the sketch (subspace iteration in one
//      block), the 3-D projection of every point and an estimate of
//      max |x_i - mu| that sets the fp16 scale of the tensor screen;
//   4. a Morton-bucket counting sort of the projections (about four points per
//      bucket), giving perm (sorted position -> original index): points close in
//      space get close positions, so a query block finds its neighbours in the
//      first candidate tiles it visits and its top-K threshold tightens at once;
//   5. the screening layout in sorted order: centred FP32 rows xc (Dp-padded),
//      their squared norms (float-float accumulated), fp16 hi/lo splits of
//      2^s * xc and the norm column for the tensor screen, and R = max |xc|.
// The ordering only affects speed: the re-rank and certification make the
// final neighbour sets independent of it.
#include <cuda_fp16.h>

#include <cfloat>
#include <cmath>

#include "ff.cuh"
#include "tk_internal.h"

namespace tk {
namespace {

constexpr int SKETCH = 16;

__device__ __forceinline__ float ldx_f(const void* X, int dtype, int64_t off)
{
    return dtype == TK_F64 ? (float)reinterpret_cast<const double*>(X)[off] : reinterpret_cast<const float*>(X)[off];
}

__device__ __forceinline__ float warp_sum_f(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// order-preserving float <-> uint encoding for atomic min/max
__device__ __forceinline__ unsigned f2ord(float f)
{
    unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(unsigned u)
{
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// 1. column sums: block b sums rows [b*rpb, (b+1)*rpb) for all columns.
__global__ void k_colsum_partial(const void* X, int dtype, int64_t N, int D, int64_t ldx, int64_t rpb,
                                 float* partial)
{
    // FP32 sums in a fixed order: the mean only centres the screening
    // coordinates (the exact distances and the weights use X itself), so its
    // rounding affects no result
    __shared__ float red[4][64];
    const int lane64 = threadIdx.x & 63, grp = threadIdx.x >> 6;  // 4 row groups of 64 columns
    const int64_t r0 = (int64_t)blockIdx.x * rpb;
    const int64_t r1 = min(N, r0 + rpb);
    for (int c0 = 0; c0 < D; c0 += 64)
    {
        const int c = c0 + lane64;
        float s0 = 0.f, s1 = 0.f;
        if (c < D)
        {
            int64_t r = r0 + grp;
            for (; r + 4 < r1; r += 8)
            {
                s0 += ldx_f(X, dtype, r * ldx + c);
                s1 += ldx_f(X, dtype, (r + 4) * ldx + c);
            }
            if (r < r1)
                s0 += ldx_f(X, dtype, r * ldx + c);
        }
        red[grp][lane64] = s0 + s1;
        __syncthreads();
        if (grp == 0 && c < D)
            partial[(int64_t)blockIdx.x * D + c] = ((red[0][lane64] + red[1][lane64]) + red[2][lane64]) + red[3][lane64];
        __syncthreads();
    }
}
// One block per column: a fixed-shape tree over the block partials.
__global__ void k_colsum_final(const float* partial, int nblk, int D, int64_t N, float* meanf)
{
    __shared__ float red[256];
    const int c = blockIdx.x, t = threadIdx.x;
    float acc = 0.f;
    for (int b = t; b < nblk; b += 256)
        acc += partial[(int64_t)b * D + c];
    red[t] = acc;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1)
    {
        if (t < o)
            red[t] += red[t + o];
        __syncthreads();
    }
    if (t == 0)
        meanf[c] = red[0] / (float)N;
}

// deterministic pseudo-random sketch matrix entry in [-1, 1)
__device__ __forceinline__ float sketch_g(int d, int j)
{
    unsigned h = (unsigned)d * 0x9E3779B1u ^ ((unsigned)j * 0x85EBCA77u + 0x27d4eb2fu);
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    h *= 0x297A2D39u;
    h ^= h >> 15;
    return (float)(h >> 8) * (2.0f / 16777216.0f) - 1.0f;
}

__global__ void k_gen_sketch(int D, float* G)
{
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < D * SKETCH; t += gridDim.x * blockDim.x)
        G[t] = sketch_g(t / SKETCH, t % SKETCH);
}

// 2. sketch covariance of a subsample (every stride-th point), per block (FP32;
// only the order of the points depends on it).
__global__ void k_sketch(const void* X, int dtype, int64_t N, int64_t stride, int D, int64_t ldx, const float* meanf,
                         const float* G, float* cov_partial /* blocks x 136 */)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    int pa[5], pb[5];
#pragma unroll
    for (int m = 0; m < 5; ++m)
    {
        int p = lane + 32 * m, a = 0;
        if (p >= 136)
            p = 0;
        while (p >= SKETCH - a)
        {
            p -= SKETCH - a;
            ++a;
        }
        pa[m] = a;
        pb[m] = a + p;
    }
    float acc[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    for (int64_t i = warp * stride; i < N; i += nwarps * stride)
    {
        float s[SKETCH];
#pragma unroll
        for (int j = 0; j < SKETCH; ++j)
            s[j] = 0.f;
        for (int d = lane; d < D; d += 32)
        {
            const float vf = ldx_f(X, dtype, i * ldx + d) - meanf[d];
            const float4* g = reinterpret_cast<const float4*>(G + (size_t)d * SKETCH);
#pragma unroll
            for (int q = 0; q < SKETCH / 4; ++q)
            {
                const float4 gq = g[q];
                s[4 * q + 0] = fmaf(gq.x, vf, s[4 * q + 0]);
                s[4 * q + 1] = fmaf(gq.y, vf, s[4 * q + 1]);
                s[4 * q + 2] = fmaf(gq.z, vf, s[4 * q + 2]);
                s[4 * q + 3] = fmaf(gq.w, vf, s[4 * q + 3]);
            }
        }
#pragma unroll
        for (int j = 0; j < SKETCH; ++j)
            s[j] = warp_sum_f(s[j]);
#pragma unroll
        for (int m = 0; m < 5; ++m)
        {
            float sa = 0.f, sb = 0.f;
#pragma unroll
            for (int j = 0; j < SKETCH; ++j)
            {
                sa = (j == pa[m]) ? s[j] : sa;
                sb = (j == pb[m]) ? s[j] : sb;
            }
            acc[m] = fmaf(sa, sb, acc[m]);
        }
    }
    __shared__ float red[8][160];
    const int wib = threadIdx.x >> 5;
#pragma unroll
    for (int m = 0; m < 5; ++m)
    {
        const int p = lane + 32 * m;
        if (p < 136)
            red[wib][p] = acc[m];
    }
    __syncthreads();
    for (int p = threadIdx.x; p < 136; p += blockDim.x)
    {
        float sacc = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
            sacc += red[w][p];
        cov_partial[(int64_t)blockIdx.x * 136 + p] = sacc;
    }
}

// 3. top-3 principal directions of the sketch covariance by subspace iteration
// (one block, FP32), then H = G V3 (D x 3) for the projection.
__global__ void k_pca3(const float* cov_partial, int nblk, int D, float* H)
{
    __shared__ float C[SKETCH][SKETCH];
    __shared__ float V[SKETCH][3];
    __shared__ float T[SKETCH][3];
    const int t = threadIdx.x;
    for (int p = t; p < 136; p += blockDim.x)
    {
        // eight independent chains keep the loads of the partials in flight
        float s8[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        int w = 0;
        for (; w + 8 <= nblk; w += 8)
        {
#pragma unroll
            for (int u = 0; u < 8; ++u)
                s8[u] += cov_partial[(int64_t)(w + u) * 136 + p];
        }
        for (; w < nblk; ++w)
            s8[0] += cov_partial[(int64_t)w * 136 + p];
        const float s = ((s8[0] + s8[1]) + (s8[2] + s8[3])) + ((s8[4] + s8[5]) + (s8[6] + s8[7]));
        int a = 0, rem = p;
        while (rem >= SKETCH - a)
        {
            rem -= SKETCH - a;
            ++a;
        }
        C[a][a + rem] = s;
        C[a + rem][a] = s;
    }
    if (t < SKETCH * 3)
        V[t / 3][t % 3] = ((t / 3) % 3 == t % 3) ? 1.f : 0.01f * (t / 3 + 1) * (t % 3 + 1);
    __syncthreads();
    for (int it = 0; it < 24; ++it)
    {
        if (t < SKETCH * 3)
        {
            const int i = t / 3, c = t % 3;
            float s = 0.f;
            for (int j = 0; j < SKETCH; ++j)
                s = fmaf(C[i][j], V[j][c], s);
            T[i][c] = s;
        }
        __syncthreads();
        if (t == 0)
        {
            for (int c = 0; c < 3; ++c)
            {
                for (int p = 0; p < c; ++p)
                {
                    float dot = 0.f;
                    for (int j = 0; j < SKETCH; ++j)
                        dot = fmaf(T[j][c], T[j][p], dot);
                    for (int j = 0; j < SKETCH; ++j)
                        T[j][c] = fmaf(-dot, T[j][p], T[j][c]);
                }
                float nrm = 0.f;
                for (int j = 0; j < SKETCH; ++j)
                    nrm = fmaf(T[j][c], T[j][c], nrm);
                const float inv = nrm > 0.f ? rsqrtf(nrm) : 0.f;
                for (int j = 0; j < SKETCH; ++j)
                    T[j][c] = nrm > 0.f ? T[j][c] * inv : (j == c ? 1.f : 0.f);
            }
        }
        __syncthreads();
        if (t < SKETCH * 3)
            V[t / 3][t % 3] = T[t / 3][t % 3];
        __syncthreads();
    }
    for (int d = t; d < D; d += blockDim.x)
        for (int c = 0; c < 3; ++c)
        {
            float s = 0.f;
            for (int j = 0; j < SKETCH; ++j)
                s = fmaf(sketch_g(d, j), V[j][c], s);
            H[d * 3 + c] = s;
        }
}

// projection p_i = H^T (x_i - mu) and its bounding box
__global__ void k_project(const void* X, int dtype, int64_t N, int D, int64_t ldx, const float* meanf,
                          const float* H, float* proj, unsigned* bbox /* 6: min x3, max x3 */, unsigned* rest_ord)
{
    // four rows per iteration: their loads are in flight together
    constexpr int RW = 4;
    float rloc = 0.f;
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int64_t i0 = warp * RW; i0 < N; i0 += nwarps * RW)
    {
        float p[RW][3], r2[RW];
#pragma unroll
        for (int u = 0; u < RW; ++u)
        {
            p[u][0] = p[u][1] = p[u][2] = 0.f;
            r2[u] = 0.f;
        }
        for (int d = lane; d < D; d += 32)
        {
            const float m = meanf[d], h0 = H[d * 3 + 0], h1 = H[d * 3 + 1], h2 = H[d * 3 + 2];
            float v[RW];
#pragma unroll
            for (int u = 0; u < RW; ++u)
                v[u] = (i0 + u < N) ? ldx_f(X, dtype, (i0 + u) * ldx + d) - m : 0.f;
#pragma unroll
            for (int u = 0; u < RW; ++u)
            {
                r2[u] = fmaf(v[u], v[u], r2[u]);
                p[u][0] = fmaf(h0, v[u], p[u][0]);
                p[u][1] = fmaf(h1, v[u], p[u][1]);
                p[u][2] = fmaf(h2, v[u], p[u][2]);
            }
        }
#pragma unroll
        for (int u = 0; u < RW; ++u)
        {
            if (i0 + u >= N)
                break;
#pragma unroll
            for (int c = 0; c < 3; ++c)
            {
                p[u][c] = warp_sum_f(p[u][c]);
                mn[c] = fminf(mn[c], p[u][c]);
                mx[c] = fmaxf(mx[c], p[u][c]);
            }
            if (lane < 3)
                proj[(i0 + u) * 3 + lane] = lane == 0 ? p[u][0] : (lane == 1 ? p[u][1] : p[u][2]);
            rloc = fmaxf(rloc, sqrtf(warp_sum_f(r2[u])));
        }
    }
    if (lane == 0 && rloc > 0.f)
        atomicMax(rest_ord, f2ord(rloc));
    if (lane == 0 && mn[0] <= mx[0])
        for (int c = 0; c < 3; ++c)
        {
            atomicMin(&bbox[c], f2ord(mn[c]));
            atomicMax(&bbox[3 + c], f2ord(mx[c]));
        }
}

__device__ __forceinline__ unsigned spread3(unsigned v)  // 10 bits -> every third bit
{
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__global__ void k_codes(const float* proj, int64_t N, const unsigned* bbox, int shift, unsigned* bucket,
                        unsigned* hist)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x)
    {
        unsigned q[3];
#pragma unroll
        for (int c = 0; c < 3; ++c)
        {
            const float lo = ord2f(bbox[c]), hi = ord2f(bbox[3 + c]);
            const float span = hi - lo;
            float t = span > 0.f ? (proj[i * 3 + c] - lo) / span : 0.f;
            t = fminf(fmaxf(t, 0.f), 1.f);
            q[c] = min(1023u, (unsigned)(t * 1024.f));
        }
        const unsigned code = (spread3(q[0]) << 2) | (spread3(q[1]) << 1) | spread3(q[2]);
        const unsigned b = code >> shift;
        bucket[i] = b;
        atomicAdd(&hist[b], 1u);
    }
}

// position = bucket offset (exclusive scan of the histogram) + arrival order
__global__ void k_scatter(const unsigned* bucket, int64_t N, const int64_t* offs, unsigned* fill, int32_t* perm)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x)
    {
        const unsigned b = bucket[i];
        const int64_t pos = offs[b] + atomicAdd(&fill[b], 1u);
        perm[pos] = (int32_t)i;
    }
}

// 5. screening layout in sorted order (one warp per row).
__global__ void k_layout(const void* X, int dtype, int64_t N, int64_t Npad, int D, int Dp, int64_t ldx,
                         const float* meanf, const int32_t* perm, const unsigned* rest_ord, float* xc, float* nrm,
                         __half* xh, __half* xl, __half* xn, unsigned* rmax_ord, float* scale_out)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    // xh/xl hold xc * 2^s with R * 2^s < 2^14 (fp16 max is 65504); the estimate
    // of R gets a 1% margin
    int e = 0;
    const float Rest = ord2f(*rest_ord) * 1.01f;
    frexpf(Rest > 0.f ? Rest : 1.f, &e);
    const int s = 14 - e;
    const float scale = ldexpf(1.f, s);
    if (warp == 0 && lane == 0 && scale_out)
        *scale_out = (float)s;
    float rloc = 0.f;
    // two rows per iteration: their gathers are in flight together
    constexpr int RW = 2;
    for (int64_t p0 = warp * RW; p0 < Npad; p0 += nwarps * RW)
    {
        int64_t src[RW];
        bool valid[RW];
#pragma unroll
        for (int u = 0; u < RW; ++u)
        {
            valid[u] = p0 + u < N;
            src[u] = valid[u] ? perm[p0 + u] : 0;
        }
        ff n2[RW];
#pragma unroll
        for (int u = 0; u < RW; ++u)
            n2[u] = ff_zero();
        for (int d = lane; d < Dp; d += 32)
        {
            float v[RW];
#pragma unroll
            for (int u = 0; u < RW; ++u)
                v[u] = (valid[u] && d < D) ? ldx_f(X, dtype, src[u] * ldx + d) - meanf[d] : 0.f;
#pragma unroll
            for (int u = 0; u < RW; ++u)
            {
                const int64_t p = p0 + u;
                if (p >= Npad)
                    break;
                n2[u] = ff_add(n2[u], two_prod(v[u], v[u]));
                xc[p * Dp + d] = v[u];
                if (xh)
                {
                    const float vs = v[u] * scale;
                    const __half h = __float2half_rn(vs);
                    const __half l = __float2half_rn(vs - __half2float(h));
                    xh[p * Dp + d] = h;
                    xl[p * Dp + d] = l;
                }
            }
        }
#pragma unroll
        for (int u = 0; u < RW; ++u)
        {
            const int64_t p = p0 + u;
            if (p >= Npad)
                break;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
                n2[u] = ff_add(n2[u], ff_shfl_xor(n2[u], o));
            // n2 is normalised, so hi is |xc|^2 rounded to FP32; sqrtf is within an
            // ulp, which the 1e-6 margin covers
            if (valid[u])
                rloc = fmaxf(rloc, sqrtf(n2[u].hi) * 1.000001f);
            if (lane == 0)
                nrm[p] = valid[u] ? n2[u].hi : __int_as_float(0x7f800000);
            if (xn && lane < 16)
            {
                // -|2^s xc|^2 / 2^14 as fp16 hi + lo: the tensor screen adds 2^13 (h + l)
                // = -|2^s y|^2 / 2 to every dot product through one extra K=16 step.
                // Padding rows stay 0 (the screen skips their indices).
                __half hv = __float2half_rn(0.f);
                if (valid[u] && lane < 2)
                {
                    const float f = ldexpf(1.f, 2 * s - 14);
                    const float t_hi = -n2[u].hi * f, t_lo = -n2[u].lo * f;
                    const __half h = __float2half_rn(t_hi);
                    hv = (lane == 0) ? h : __float2half_rn((t_hi - __half2float(h)) + t_lo);
                }
                xn[p * 16 + lane] = hv;
            }
        }
    }
    if (lane == 0 && rloc > 0.f)
        atomicMax(rmax_ord, f2ord(rloc));
}

__global__ void k_finalize_r(const unsigned* rmax_ord, float* rmax)
{
    rmax[0] = (*rmax_ord == 0u) ? 0.f : ord2f(*rmax_ord);
}

} // namespace

void prepare_points(tk_ctx* ctx, const void* X, int dtype, int64_t N, int D, int64_t ldx, bool tensor,
                    Prepared& P)
{
    cudaStream_t st = ctx->stream;
    P.N = N;
    P.D = D;
    P.Dp = ((D + 63) / 64) * 64;
    P.Npad = ((N + 255) / 256) * 256;
    const int sms = ctx->num_sms;

    // 1. mean
    const int nblk = (int)std::min<int64_t>(4 * sms, std::max<int64_t>(1, (N + 63) / 64));
    const int64_t rpb = (N + nblk - 1) / nblk;
    float* partial = (float*)ctx->scratch.get("prep.partial", sizeof(float) * (size_t)nblk * D);
    float* meanf = (float*)ctx->scratch.get("prep.mean", sizeof(float) * D);
    k_colsum_partial<<<nblk, 256, 0, st>>>(X, dtype, N, D, ldx, rpb, partial);
    TK_CHECK_LAUNCH();
    k_colsum_final<<<D, 256, 0, st>>>(partial, nblk, D, N, meanf);
    TK_CHECK_LAUNCH();

    // 2. sketch covariance (subsample)
    const int sk_blocks = sms;
    float* covp = (float*)ctx->scratch.get("prep.covp", sizeof(float) * sk_blocks * 136);
    // small[0] = R estimate (ordered), small[1] = R (ordered), small[8..13] = bbox
    unsigned* small = (unsigned*)ctx->scratch.get("prep.small", 64 * sizeof(unsigned));
    float* rmax = (float*)ctx->scratch.get("prep.rmax", 2 * sizeof(float));
    unsigned init[16];
    for (int c = 0; c < 16; ++c)
        init[c] = 0u;
    init[8] = init[9] = init[10] = 0xffffffffu;  // bbox min (ordered encoding)
    TK_CUDA(cudaMemcpyAsync(small, init, sizeof(init), cudaMemcpyHostToDevice, st));
    float* G = (float*)ctx->scratch.get("prep.G", sizeof(float) * SKETCH * (size_t)D);
    k_gen_sketch<<<(D * SKETCH + 255) / 256, 256, 0, st>>>(D, G);
    TK_CHECK_LAUNCH();
    const int64_t stride = std::max<int64_t>(1, N / 16384);
    k_sketch<<<sk_blocks, 256, 0, st>>>(X, dtype, N, stride, D, ldx, meanf, G, covp);
    TK_CHECK_LAUNCH();

    // 3. principal directions and projection
    float* H = (float*)ctx->scratch.get("prep.H", sizeof(float) * 3 * (size_t)D);
    k_pca3<<<1, 64, 0, st>>>(covp, sk_blocks, D, H);
    TK_CHECK_LAUNCH();
    float* proj = (float*)ctx->scratch.get("prep.proj", sizeof(float) * 3 * (size_t)N);
    k_project<<<2 * sms, 256, 0, st>>>(X, dtype, N, D, ldx, meanf, H, proj, small + 8, small);
    TK_CHECK_LAUNCH();

    // 4. Morton-bucket counting sort (about four points per bucket)
    int bits = 10;
    while (bits < 24 && ((int64_t)1 << (bits + 2)) < N)
        ++bits;
    const int nb = 1 << bits;
    const int shift = 30 - bits;
    unsigned* bucket = (unsigned*)ctx->scratch.get("prep.bucket", sizeof(unsigned) * (size_t)N);
    unsigned* hist = (unsigned*)ctx->scratch.get("prep.hist", sizeof(unsigned) * (size_t)nb * 2);
    unsigned* fill = hist + nb;
    int64_t* offs = (int64_t*)ctx->scratch.get("prep.offs", sizeof(int64_t) * ((size_t)nb + 1));
    TK_CUDA(cudaMemsetAsync(hist, 0, sizeof(unsigned) * (size_t)nb * 2, st));
    k_codes<<<2 * sms, 256, 0, st>>>(proj, N, small + 8, shift, bucket, hist);
    TK_CHECK_LAUNCH();
    scan_to_offsets(ctx, reinterpret_cast<const int*>(hist), nb, offs);
    P.perm = (int32_t*)ctx->scratch.get("prep.perm", sizeof(int32_t) * (size_t)N);
    k_scatter<<<2 * sms, 256, 0, st>>>(bucket, N, offs, fill, P.perm);
    TK_CHECK_LAUNCH();

    // 5. layout
    P.xc = (float*)ctx->scratch.get("prep.xc", sizeof(float) * (size_t)P.Npad * P.Dp);
    P.nrm = (float*)ctx->scratch.get("prep.nrm", sizeof(float) * (size_t)P.Npad);
    if (tensor)
    {
        P.xh = (uint16_t*)ctx->scratch.get("prep.xh", sizeof(uint16_t) * (size_t)P.Npad * P.Dp);
        P.xl = (uint16_t*)ctx->scratch.get("prep.xl", sizeof(uint16_t) * (size_t)P.Npad * P.Dp);
        P.xn = (uint16_t*)ctx->scratch.get("prep.xn", sizeof(uint16_t) * (size_t)P.Npad * 16);
    }
    else
    {
        P.xh = P.xl = P.xn = nullptr;
    }
    P.rmax = rmax;
    k_layout<<<4 * sms, 256, 0, st>>>(X, dtype, N, P.Npad, D, P.Dp, ldx, meanf, P.perm, small, P.xc, P.nrm,
                                      (__half*)P.xh, (__half*)P.xl, (__half*)P.xn, small + 1, rmax + 1);
    TK_CHECK_LAUNCH();
    k_finalize_r<<<1, 1, 0, st>>>(small + 1, rmax);
    TK_CHECK_LAUNCH();
}

} // namespace tk
