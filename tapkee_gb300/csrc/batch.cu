// batch.cu -- many independent LLE problems of uneven N, D and k as one CUDA
// graph.
//
// The reference runs one embedding per call; a caller with many small problems
// pays per-problem launch sequences, host synchronisations and mostly idle
// GPUs. Here the problems of a batch are planned once:
//   * screen groups (same padded dimension Dp and candidate-list length KC): the
//     problems' points are centred and scaled per problem and stacked, each
//     problem starting at a 256-row boundary, into one fp16 hi/lo layout; one
//     persistent tcgen05 screen kernel per group walks (problem, query blocks)
//     work items sorted by cost; the exact re-rank and the fallback follow in one
//     launch each;
//   * k-groups (same k): the neighbour and weight tables of the group's problems
//     are contiguous and uniform, so one weight-solve launch covers the group and
//     the alignment matrices are assembled as one block-diagonal CSR (capacity
//     sized by the triplet count, so no host read-back is needed).
// The whole sequence is captured once into a CUDA graph and replayed by
// tk_batch_run. Differences from the single-problem path:
// connectivity is not checked (callers that want the reference's 2k retry run
// tk_check_connected per problem), and the spatial order comes from a random
// 16-direction sketch of each problem's covariance.
#include <cuda_fp16.h>

#include <algorithm>
#include <cfloat>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "ff.cuh"
#include "tk_internal.h"

namespace tk {
namespace {

constexpr int B_DMAX = 128;  // largest dimension of the batched tensor screen

__device__ __forceinline__ float xf(const void* X, int dtype, int64_t off)
{
    return dtype == TK_F64 ? (float)reinterpret_cast<const double*>(X)[off] : reinterpret_cast<const float*>(X)[off];
}

// |x_i - mean|^2 in float-float, lanes over dimensions (identical in the
// statistics and the layout kernels, so the radius bounds every stored norm).
__device__ __forceinline__ ff centred_norm2(const BatchProb& P, int64_t i, const float* mean, int lane)
{
    ff n2 = ff_zero();
    for (int d = lane; d < P.D; d += 32)
    {
        const float v = xf(P.X, P.dtype, i * P.ldx + d) - mean[d];
        n2 = ff_add(n2, two_prod(v, v));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        n2 = ff_add(n2, ff_shfl_xor(n2, o));
    return n2;
}

// ---- batched preparation --------------------------------------------------
// Stacked slots of a group come in blocks of 256 that belong to one problem
// (each problem starts on a 256-slot boundary). In input order, slot q of
// problem b holds point q - row0_b (valid while < N_b). The spatial order
// replaces this by the Morton order of each problem's top-3 principal
// coordinates, as the single-problem path does.

// 1. column sums of one 256-slot chunk (FP64, fixed order)
__global__ void __launch_bounds__(256) k_b_colsum(const BatchProb* __restrict__ probs,
                                                  const int32_t* __restrict__ row_prob, double* partial)
{
    __shared__ double part[256];
    const int64_t c0 = (int64_t)blockIdx.x * 256;
    const int b = row_prob[c0];
    const BatchProb P = probs[b];
    const int t = threadIdx.x;
    const int per = 256 / P.D;
    double s = 0.0;
    if (t < per * P.D)
    {
        const int d = t % P.D;
        for (int j = t / P.D; j < 256; j += per)
        {
            const int64_t i = c0 + j - P.row0;
            if (i < P.N)
                s += (double)xf(P.X, P.dtype, i * P.ldx + d);
        }
    }
    part[t] = s;
    __syncthreads();
    if (t < P.D)
    {
        double tot = 0.0;
        for (int q = 0; q < per; ++q)
            tot += part[q * P.D + t];
        partial[(int64_t)blockIdx.x * B_DMAX + t] = tot;
    }
}

constexpr int PCA_SAMPLES = 1024;  // rows of the covariance sketch per problem
constexpr int B_SKETCH = 16;       // random directions of the sketch

// deterministic pseudo-random sketch entry in [-1, 1)
__device__ __forceinline__ float b_sketch_g(int d, int j)
{
    unsigned h = (unsigned)d * 0x9E3779B1u + (unsigned)j * 0x85EBCA77u + 0x165667B1u;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    h *= 0x297A2D39u;
    h ^= h >> 15;
    return (float)(h >> 8) * (2.0f / 16777216.0f) - 1.0f;
}

// 2. per problem (one CTA): the mean, then the top-3 principal directions of a
// randomly sketched covariance (x -> G^T x, G: D x 16) of up to 1024 rows, by
// subspace iteration, mapped back as H = G V (D x 3). FP32: they only order points.
__global__ void __launch_bounds__(256) k_b_mean_pca(const BatchProb* __restrict__ probs, const int32_t* grp_probs,
                                                    const double* partial, float* means, float* H)
{
    __shared__ float mean_s[B_DMAX];
    __shared__ float G[B_DMAX][B_SKETCH];
    __shared__ float red[8][136];
    __shared__ float C[B_SKETCH][B_SKETCH];
    __shared__ float V[B_SKETCH][3], T[B_SKETCH][3];
    const int b = grp_probs[blockIdx.x];
    const BatchProb P = probs[b];
    const int D = P.D, t = threadIdx.x, lane = t & 31, w = t >> 5;
    const int64_t c_first = P.row0 / 256, c_count = (P.N + 255) / 256;
    for (int d = t; d < D; d += 256)
    {
        double tot = 0.0;
        for (int64_t c = 0; c < c_count; ++c)
            tot += partial[(c_first + c) * B_DMAX + d];
        const float m = (float)(tot / (double)P.N);
        mean_s[d] = m;
        means[(int64_t)b * B_DMAX + d] = m;
    }
    for (int e = t; e < D * B_SKETCH; e += 256)
        G[e / B_SKETCH][e % B_SKETCH] = b_sketch_g(e / B_SKETCH, e % B_SKETCH);
    __syncthreads();
    // upper-triangle pair (pa, pb) of the 136 entries owned by each lane
    int pa[5], pb[5];
#pragma unroll
    for (int m = 0; m < 5; ++m)
    {
        int q = lane + 32 * m, a = 0;
        if (q >= 136)
            q = 0;
        while (q >= B_SKETCH - a)
        {
            q -= B_SKETCH - a;
            ++a;
        }
        pa[m] = a;
        pb[m] = a + q;
    }
    float acc[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    const int64_t stride = P.N > PCA_SAMPLES ? P.N / PCA_SAMPLES : 1;
    for (int64_t i = (int64_t)w * stride; i < P.N; i += 8 * stride)
    {
        float sk[B_SKETCH];
#pragma unroll
        for (int j = 0; j < B_SKETCH; ++j)
            sk[j] = 0.f;
        for (int d = lane; d < D; d += 32)
        {
            const float v = xf(P.X, P.dtype, i * P.ldx + d) - mean_s[d];
#pragma unroll
            for (int j = 0; j < B_SKETCH; ++j)
                sk[j] = fmaf(G[d][j], v, sk[j]);
        }
#pragma unroll
        for (int j = 0; j < B_SKETCH; ++j)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
                sk[j] += __shfl_xor_sync(0xffffffffu, sk[j], o);
#pragma unroll
        for (int m = 0; m < 5; ++m)
        {
            float sa = 0.f, sb = 0.f;
#pragma unroll
            for (int j = 0; j < B_SKETCH; ++j)
            {
                sa = (j == pa[m]) ? sk[j] : sa;
                sb = (j == pb[m]) ? sk[j] : sb;
            }
            acc[m] = fmaf(sa, sb, acc[m]);
        }
    }
#pragma unroll
    for (int m = 0; m < 5; ++m)
        if (lane + 32 * m < 136)
            red[w][lane + 32 * m] = acc[m];
    __syncthreads();
    if (t < 136)
    {
        float sacc = 0.f;
        for (int q = 0; q < 8; ++q)
            sacc += red[q][t];
        int a = 0, rem = t;
        while (rem >= B_SKETCH - a)
        {
            rem -= B_SKETCH - a;
            ++a;
        }
        C[a][a + rem] = sacc;
        C[a + rem][a] = sacc;
    }
    if (t < B_SKETCH * 3)
        V[t / 3][t % 3] = ((t / 3) == (t % 3)) ? 1.f : 0.01f * (t / 3 + 1) * (t % 3 + 1);
    __syncthreads();
    for (int it = 0; it < 24; ++it)
    {
        if (t < B_SKETCH * 3)
        {
            const int i = t / 3, c = t % 3;
            float sacc = 0.f;
            for (int j = 0; j < B_SKETCH; ++j)
                sacc = fmaf(C[i][j], V[j][c], sacc);
            T[i][c] = sacc;
        }
        __syncthreads();
        if (t == 0)
        {
            for (int c = 0; c < 3; ++c)
            {
                for (int q = 0; q < c; ++q)
                {
                    float dot = 0.f;
                    for (int j = 0; j < B_SKETCH; ++j)
                        dot = fmaf(T[j][c], T[j][q], dot);
                    for (int j = 0; j < B_SKETCH; ++j)
                        T[j][c] = fmaf(-dot, T[j][q], T[j][c]);
                }
                float nrm = 0.f;
                for (int j = 0; j < B_SKETCH; ++j)
                    nrm = fmaf(T[j][c], T[j][c], nrm);
                const float inv = nrm > 0.f ? rsqrtf(nrm) : 0.f;
                for (int j = 0; j < B_SKETCH; ++j)
                    T[j][c] = nrm > 0.f ? T[j][c] * inv : (j == c ? 1.f : 0.f);
            }
        }
        __syncthreads();
        if (t < B_SKETCH * 3)
            V[t / 3][t % 3] = T[t / 3][t % 3];
        __syncthreads();
    }
    // H = G V, normalised per column so that |projection| <= |x - mean|
    for (int e = t; e < 3 * D; e += 256)
    {
        const int d = e / 3, c = e % 3;
        float sacc = 0.f;
        for (int j = 0; j < B_SKETCH; ++j)
            sacc = fmaf(G[d][j], V[j][c], sacc);
        H[(int64_t)b * 3 * B_DMAX + e] = sacc;
    }
}

// column norms of H (so the projections can be scaled into [-R, R])
__global__ void k_b_hnorm(const int32_t* grp_probs, int count, const BatchProb* __restrict__ probs, float* H)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= count * 3)
        return;
    const int b = grp_probs[q / 3], c = q % 3;
    float* Hb = H + (int64_t)b * 3 * B_DMAX;
    float n = 0.f;
    for (int d = 0; d < probs[b].D; ++d)
        n = fmaf(Hb[d * 3 + c], Hb[d * 3 + c], n);
    const float inv = n > 0.f ? rsqrtf(n) : 0.f;
    for (int d = 0; d < probs[b].D; ++d)
        Hb[d * 3 + c] *= inv;
}

// 3. per slot (input order, one warp per row): radius (the same float-float norm
// as the layout, so R bounds every stored norm) and the 3 principal coordinates
__global__ void __launch_bounds__(256) k_b_project(const BatchProb* __restrict__ probs,
                                                   const int32_t* __restrict__ row_prob, const float* means,
                                                   const float* H, float* proj, unsigned* r_bits)
{
    __shared__ float wmax[8];
    const int64_t c0 = (int64_t)blockIdx.x * 256;
    const int b = row_prob[c0];
    const BatchProb P = probs[b];
    const float* mean = means + (int64_t)b * B_DMAX;
    const float* Hb = H + (int64_t)b * 3 * B_DMAX;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    float rloc = 0.f;
    for (int j = w; j < 256; j += 8)
    {
        const int64_t i = c0 + j - P.row0;
        if (i >= P.N)
            break;
        float p0 = 0.f, p1 = 0.f, p2 = 0.f;
        for (int d = lane; d < P.D; d += 32)
        {
            const float v = xf(P.X, P.dtype, i * P.ldx + d) - mean[d];
            p0 = fmaf(Hb[d * 3 + 0], v, p0);
            p1 = fmaf(Hb[d * 3 + 1], v, p1);
            p2 = fmaf(Hb[d * 3 + 2], v, p2);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
        {
            p0 += __shfl_xor_sync(0xffffffffu, p0, o);
            p1 += __shfl_xor_sync(0xffffffffu, p1, o);
            p2 += __shfl_xor_sync(0xffffffffu, p2, o);
        }
        const ff n2 = centred_norm2(P, i, mean, lane);
        rloc = fmaxf(rloc, (float)sqrt(ff_to_double(n2)) * 1.000001f);
        if (lane < 3)
            proj[(c0 + j) * 3 + lane] = lane == 0 ? p0 : (lane == 1 ? p1 : p2);
    }
    if (lane == 0)
        wmax[w] = rloc;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        float R = 0.f;
        for (int q = 0; q < 8; ++q)
            R = fmaxf(R, wmax[q]);
        atomicMax(&r_bits[b], __float_as_uint(R));  // R >= 0: bits order like values
    }
}

// 4. radius and split exponent s (R 2^s < 2^14) per problem
__global__ void k_b_scale(const int32_t* grp_probs, int count, const unsigned* r_bits, float* prob_R,
                          float* prob_scale)
{
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < count; q += gridDim.x * blockDim.x)
    {
        const int b = grp_probs[q];
        const float R = __uint_as_float(r_bits[b]);
        int e = 0;
        frexpf(R > 0.f ? R * 1.01f : 1.f, &e);
        prob_R[b] = R;
        prob_scale[b] = (float)(14 - e);
    }
}

__device__ __forceinline__ unsigned b_spread3(unsigned v)  // 10 bits -> every third bit
{
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

// 5. Morton bucket (about four points per bucket) of every valid slot
__global__ void k_b_codes(const BatchProb* __restrict__ probs, const int32_t* __restrict__ row_prob, int64_t rows,
                          const float* proj, const float* prob_R, int32_t* bucket, int* hist)
{
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < rows; q += (int64_t)gridDim.x * blockDim.x)
    {
        const int b = row_prob[q];
        const BatchProb& P = probs[b];
        if (q - P.row0 >= P.N)
            continue;
        const float R = prob_R[b];
        unsigned u[3];
#pragma unroll
        for (int c = 0; c < 3; ++c)
        {
            float tt = R > 0.f ? 0.5f * (proj[q * 3 + c] / R + 1.f) : 0.f;
            tt = fminf(fmaxf(tt, 0.f), 1.f);
            u[c] = min(1023u, (unsigned)(tt * 1024.f));
        }
        const unsigned code = (b_spread3(u[0]) << 2) | (b_spread3(u[1]) << 1) | b_spread3(u[2]);
        const int32_t g = (int32_t)(P.hoff + (code >> (30 - P.hbits)));
        bucket[q] = g;
        atomicAdd(&hist[g], 1);
    }
}

// 6. sorted position of every valid slot: perm_st[row0 + position] = point
__global__ void k_b_scatter(const BatchProb* __restrict__ probs, const int32_t* __restrict__ row_prob, int64_t rows,
                            const int32_t* bucket, const int64_t* offs, int* fillc, int32_t* perm_st)
{
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < rows; q += (int64_t)gridDim.x * blockDim.x)
    {
        const int b = row_prob[q];
        const BatchProb& P = probs[b];
        const int64_t i = q - P.row0;
        if (i >= P.N)
            continue;
        const int32_t g = bucket[q];
        const int64_t pos = offs[g] - offs[P.hoff] + atomicAdd(&fillc[g], 1);
        perm_st[P.row0 + pos] = (int32_t)i;
    }
}

// 7. stacked screening layout in sorted order, one warp per stacked row.
__global__ void k_b_layout(const BatchProb* __restrict__ probs, const int32_t* __restrict__ row_prob,
                           const int32_t* __restrict__ perm_st, int64_t rows, int Dp, const float* means,
                           const float* prob_scale, __half* xh, __half* xl, __half* xn, float* nrm)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t p = warp; p < rows; p += nwarps)
    {
        const int b = row_prob[p];
        const BatchProb P = probs[b];
        const bool valid = p - P.row0 < P.N;
        const int64_t i = valid ? perm_st[p] : 0;
        const float* mean = means + (int64_t)b * B_DMAX;
        const int s = valid ? (int)prob_scale[b] : 0;
        const float scale = ldexpf(1.f, s);
        for (int d = lane; d < Dp; d += 32)
        {
            float v = 0.f;
            if (valid && d < P.D)
                v = xf(P.X, P.dtype, i * P.ldx + d) - mean[d];
            const float vs = v * scale;
            const __half h = __float2half_rn(vs);
            xh[p * Dp + d] = h;
            xl[p * Dp + d] = __float2half_rn(vs - __half2float(h));
        }
        ff n2 = ff_zero();
        if (valid)
            n2 = centred_norm2(P, i, mean, lane);
        if (lane == 0)
            nrm[p] = valid ? (float)ff_to_double(n2) : __int_as_float(0x7f800000);
        if (lane < 16)
        {
            // -|2^s xc|^2 / 2^14 as fp16 hi + lo (the norm column of the screen)
            __half v = __float2half_rn(0.f);
            if (valid && lane < 2)
            {
                const float f = ldexpf(1.f, 2 * s - 14);
                const float t_hi = -n2.hi * f, t_lo = -n2.lo * f;
                const __half h = __float2half_rn(t_hi);
                v = (lane == 0) ? h : __float2half_rn((t_hi - __half2float(h)) + t_lo);
            }
            xn[p * 16 + lane] = v;
        }
    }
}

// Neighbour indices of a k-group made group-global (row offset of each problem
// inside the group), as the block-diagonal assembly expects.
__global__ void k_b_globalize(const BatchProb* __restrict__ probs, const int32_t* __restrict__ row_prob,
                              int64_t group_row0, int64_t rows, int k, const int32_t* __restrict__ idx,
                              int32_t* idx_g)
{
    const int64_t n = rows * k;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    {
        const int b = row_prob[e / k];
        idx_g[e] = idx[e] + (int32_t)(probs[b].out_row0 - group_row0);
    }
}

template <typename T>
T* dalloc(std::vector<void*>& owned, size_t count)
{
    void* p = nullptr;
    const size_t bytes = std::max<size_t>(count * sizeof(T), 256);
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess)
    {
        cudaGetLastError();
        throw Error(e == cudaErrorMemoryAllocation ? TK_ERR_OOM : TK_ERR_CUDA,
                    "batch: device allocation of " + std::to_string(bytes) + " bytes failed");
    }
    owned.push_back(p);
    return static_cast<T*>(p);
}

template <typename T>
void upload(T* dst, const std::vector<T>& src, cudaStream_t st)
{
    if (!src.empty())
        TK_CUDA(cudaMemcpyAsync(dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice, st));
}

struct ScreenGroup
{
    int Dp = 0, kc = 0, qt = 1;
    int kmax = 0;            // largest k of the group's problems
    std::vector<int> probs;  // batch (sorted) problem numbers
    int64_t rows = 0;
    __half *xh = nullptr, *xl = nullptr, *xn = nullptr;
    float* nrm = nullptr;
    int32_t* row_prob = nullptr;  // device, per stacked row
    int32_t* grp_probs = nullptr; // device, the group's problems
    int32_t* perm_st = nullptr;   // device, stacked sorted row -> point of its problem
    double* partial = nullptr;    // column sums per 256-row chunk
    float* proj = nullptr;        // 3 principal coordinates per input-order slot
    int32_t* bucket = nullptr;    // Morton bucket per input-order slot
    int* hist = nullptr;          // bucket counts, then fill counters
    int* fillc = nullptr;
    int64_t* offs = nullptr;      // exclusive scan of hist
    int64_t nbuckets = 0;
    int4* items = nullptr;
    int nitems = 0;
    int32_t* cand_idx = nullptr;
    float* cand_val = nullptr;
};

struct KGroup
{
    int k = 0;
    int first = 0, count = 0;  // sorted problem range
    int64_t out_row0 = 0, rows = 0, idx_off = 0;
    int32_t* idx_g = nullptr;
    int64_t* row_ptr = nullptr;
    int32_t* col = nullptr;
    double* val = nullptr;
    int64_t cap = 0;
};

} // namespace
} // namespace tk

using namespace tk;

struct tk_batch
{
    tk_ctx* parent = nullptr;
    tk_ctx* ctx = nullptr;  // private context on the parent's stream: own scratch and error word
    std::vector<void*> owned;
    double klle_shift = 1e-3, nullspace_shift = 1e-9;
    tk_batch_tuning tuning{};
    std::vector<tk_batch_problem> in;  // caller order
    std::vector<int> order;            // sorted position -> caller index
    std::vector<int> pos_of;           // caller index -> sorted position
    std::vector<BatchProb> hp;         // sorted problems
    std::vector<int> kgroup_of;        // sorted position -> k-group
    BatchProb* probs = nullptr;
    int64_t* prob_n = nullptr;
    float *prob_R = nullptr, *prob_scale = nullptr, *means = nullptr, *H = nullptr;
    unsigned* r_bits = nullptr;
    int32_t* row_prob_out = nullptr;
    int32_t* idx_all = nullptr;
    double* w_all = nullptr;
    unsigned* nfailed = nullptr;  // one per screen group
    std::vector<ScreenGroup> sg;
    std::vector<KGroup> kg;
    int64_t total_rows = 0, total_idx = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, evp = nullptr;
    float last_ms = 0.f;
};

namespace tk {
namespace {

template <typename F>
int batch_guard(tk_ctx* ctx, F&& f)
{
    if (!ctx)
        return TK_ERR_INVALID_ARG;
    try
    {
        TK_CUDA(cudaSetDevice(ctx->device));
        f();
        ctx->last_error.clear();
        return TK_OK;
    }
    catch (const Error& e)
    {
        ctx->last_error = e.what();
        log(ctx, TK_LOG_ERROR, e.what());
        return e.status;
    }
    catch (const std::bad_alloc&)
    {
        ctx->last_error = "Not enough memory";
        return TK_ERR_OOM;
    }
    catch (const std::exception& e)
    {
        ctx->last_error = e.what();
        return TK_ERR_INTERNAL;
    }
}

int candidates_for_batch(int k, bool wide) { return (wide || k + 8 > 32) ? 64 : 32; }

// The kernels of one replay, in stream order.
void enqueue(tk_batch* B)
{
    tk_ctx* ctx = B->ctx;
    cudaStream_t st = ctx->stream;
    const int sms = ctx->num_sms;
    for (size_t g = 0; g < B->sg.size(); ++g)
    {
        ScreenGroup& S = B->sg[g];
        const int nprob = (int)S.probs.size();
        const int chunks = (int)(S.rows / 256);
        k_b_colsum<<<chunks, 256, 0, st>>>(B->probs, S.row_prob, S.partial);
        TK_CHECK_LAUNCH();
        k_b_mean_pca<<<nprob, 256, 0, st>>>(B->probs, S.grp_probs, S.partial, B->means, B->H);
        TK_CHECK_LAUNCH();
        k_b_hnorm<<<(3 * nprob + 127) / 128, 128, 0, st>>>(S.grp_probs, nprob, B->probs, B->H);
        TK_CHECK_LAUNCH();
        TK_CUDA(cudaMemsetAsync(B->r_bits, 0, sizeof(unsigned) * B->hp.size(), st));
        k_b_project<<<chunks, 256, 0, st>>>(B->probs, S.row_prob, B->means, B->H, S.proj, B->r_bits);
        TK_CHECK_LAUNCH();
        k_b_scale<<<(nprob + 127) / 128, 128, 0, st>>>(S.grp_probs, nprob, B->r_bits, B->prob_R, B->prob_scale);
        TK_CHECK_LAUNCH();
        TK_CUDA(cudaMemsetAsync(S.hist, 0, sizeof(int) * (size_t)S.nbuckets, st));
        TK_CUDA(cudaMemsetAsync(S.fillc, 0, sizeof(int) * (size_t)S.nbuckets, st));
        k_b_codes<<<2 * sms, 256, 0, st>>>(B->probs, S.row_prob, S.rows, S.proj, B->prob_R, S.bucket, S.hist);
        TK_CHECK_LAUNCH();
        scan_to_offsets(ctx, S.hist, S.nbuckets, S.offs);
        TK_CUDA(cudaMemsetAsync(S.perm_st, 0xff, sizeof(int32_t) * (size_t)S.rows, st));
        k_b_scatter<<<2 * sms, 256, 0, st>>>(B->probs, S.row_prob, S.rows, S.bucket, S.offs, S.fillc, S.perm_st);
        TK_CHECK_LAUNCH();
        k_b_layout<<<4 * sms, 256, 0, st>>>(B->probs, S.row_prob, S.perm_st, S.rows, S.Dp, B->means, B->prob_scale,
                                            S.xh, S.xl, S.xn, S.nrm);
        TK_CHECK_LAUNCH();
        StackedScreen SS;
        SS.Dp = S.Dp;
        SS.kc = S.kc;
        SS.qt = S.qt;
        SS.kmax = S.kmax;
        SS.rows = S.rows;
        SS.xh = reinterpret_cast<const uint16_t*>(S.xh);
        SS.xl = reinterpret_cast<const uint16_t*>(S.xl);
        SS.xn = reinterpret_cast<const uint16_t*>(S.xn);
        SS.nrm = S.nrm;
        SS.items = S.items;
        SS.nitems = S.nitems;
        SS.prob_n = B->prob_n;
        SS.prob_scale = B->prob_scale;
        screen_tensor_batch(ctx, SS, S.cand_idx, S.cand_val);
        float c1, c2;
        screen_error_model(TK_SCREEN_TENSOR, S.Dp, &c1, &c2);
        RowSpace RS;
        RS.perm = S.perm_st;
        RS.row_prob = S.row_prob;
        RS.probs = B->probs;
        RS.prob_R = B->prob_R;
        RS.idx_all = B->idx_all;
        int64_t max_n = 1;
        for (int q : S.probs)
            max_n = std::max<int64_t>(max_n, B->hp[q].N);
        rerank_batch(ctx, RS, S.rows, max_n, S.kc, S.cand_idx, S.cand_val, S.nrm, c1, c2, B->nfailed + 4 * g);
    }
    for (KGroup& K : B->kg)
    {
        lle_weights_batch(ctx, B->probs, B->row_prob_out + K.out_row0, K.out_row0, K.rows, B->idx_all + K.idx_off,
                          K.k, B->klle_shift, B->w_all + K.idx_off, B->tuning.lle_warps);
        k_b_globalize<<<2 * sms, 256, 0, st>>>(B->probs, B->row_prob_out + K.out_row0, K.out_row0, K.rows, K.k,
                                               B->idx_all + K.idx_off, K.idx_g);
        TK_CHECK_LAUNCH();
        assemble_rows_device(ctx, TK_METHOD_KLLE, K.rows, K.k, 0, K.idx_g, B->w_all + K.idx_off,
                             B->nullspace_shift, K.row_ptr);
        assemble_write(ctx, TK_METHOD_KLLE, K.rows, K.k, 0, K.idx_g, B->w_all + K.idx_off, B->nullspace_shift,
                       K.row_ptr, K.col, K.val);
    }
}

void check_errors(tk_batch* B)
{
    unsigned e = 0;
    TK_CUDA(cudaMemcpyAsync(&e, B->ctx->dev_err, sizeof(unsigned), cudaMemcpyDeviceToHost, B->ctx->stream));
    TK_CUDA(cudaStreamSynchronize(B->ctx->stream));
    if (e)
    {
        TK_CUDA(cudaMemsetAsync(B->ctx->dev_err, 0, sizeof(unsigned), B->ctx->stream));
        throw Error((e & DEV_ERR_TIMEOUT) ? TK_ERR_TIMEOUT : ((e & DEV_ERR_BOUNDS) ? TK_ERR_INVALID_ARG : TK_ERR_INTERNAL),
                    "batch: device-side check failed (0x" + std::to_string(e) + ")");
    }
}

void destroy(tk_batch* B)
{
    if (!B)
        return;
    if (B->ctx && B->ctx->stream)
        cudaStreamSynchronize(B->ctx->stream);
    if (B->exec)
        cudaGraphExecDestroy(B->exec);
    if (B->graph)
        cudaGraphDestroy(B->graph);
    if (B->ev0)
        cudaEventDestroy(B->ev0);
    if (B->ev1)
        cudaEventDestroy(B->ev1);
    if (B->evp)
        cudaEventDestroy(B->evp);
    for (void* p : B->owned)
        cudaFree(p);
    if (B->ctx)
        tk_ctx_destroy(B->ctx);
    delete B;
}

void plan(tk_batch* B, const tk_batch_problem* problems, int count)
{
    const int P = count;
    B->in.assign(problems, problems + P);
    for (int p = 0; p < P; ++p)
    {
        const tk_batch_problem& q = problems[p];
        const std::string at = "batch problem " + std::to_string(p) + ": ";
        if (q.dtype != TK_F32 && q.dtype != TK_F64)
            throw Error(TK_ERR_INVALID_ARG, at + "dtype must be TK_F32 or TK_F64");
        if (!q.X)
            throw Error(TK_ERR_INVALID_ARG, at + "X is NULL");
        if (q.N <= 0)
            throw Error(TK_ERR_NO_DATA, at + "no data");
        if (q.D < 1 || q.D > B_DMAX || q.ldx < q.D)
            throw Error(TK_ERR_UNSUPPORTED, at + "batched problems need 1 <= D <= 128 and ldx >= D");
        if (q.k < 1 || q.k > 56 || q.k > q.N - 1)
            throw Error(TK_ERR_INVALID_ARG, at + "need 1 <= k <= min(56, N - 1)");
        if (q.N >= ((int64_t)1 << 31) - 256)
            throw Error(TK_ERR_INVALID_ARG, at + "N must be below 2^31");
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, q.X) != cudaSuccess ||
            !(a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged))
        {
            cudaGetLastError();
            throw Error(TK_ERR_INVALID_ARG, at + "X must be device memory (a batch replays without host copies)");
        }
    }
    // sorted order: by k (k-groups are contiguous), then D, then caller order
    B->order.resize(P);
    std::iota(B->order.begin(), B->order.end(), 0);
    std::stable_sort(B->order.begin(), B->order.end(), [&](int a, int b) {
        if (problems[a].k != problems[b].k)
            return problems[a].k < problems[b].k;
        return problems[a].D < problems[b].D;
    });
    B->pos_of.assign(P, 0);
    for (int s = 0; s < P; ++s)
        B->pos_of[B->order[s]] = s;

    // screen groups by (Dp, KC)
    const bool wide = B->tuning.wide_lists != 0;
    std::vector<std::pair<int, int>> keys;
    B->hp.resize(P);
    int64_t out_row = 0, idx_off = 0;
    for (int s = 0; s < P; ++s)
    {
        const tk_batch_problem& q = problems[B->order[s]];
        BatchProb& h = B->hp[s];
        h.X = q.X;
        h.dtype = q.dtype;
        h.D = q.D;
        h.ldx = q.ldx;
        h.N = q.N;
        h.k = q.k;
        h.out_row0 = out_row;
        h.idx_off = idx_off;
        out_row += q.N;
        idx_off += q.N * (int64_t)q.k;
        const std::pair<int, int> key{q.D <= 64 ? 64 : 128, candidates_for_batch(q.k, wide)};
        auto it = std::find(keys.begin(), keys.end(), key);
        if (it == keys.end())
        {
            keys.push_back(key);
            ScreenGroup g;
            g.Dp = key.first;
            g.kc = key.second;
            g.qt = (g.Dp == 64) ? std::max(1, std::min(2, B->tuning.screen_qt[0])) : 1;
            B->sg.push_back(g);
            it = keys.end() - 1;
        }
        const int gi = (int)(it - keys.begin());
        h.group = gi;
        ScreenGroup& g = B->sg[gi];
        h.row0 = g.rows;
        g.rows += ((q.N + 255) / 256) * 256;
        g.probs.push_back(s);
        g.kmax = std::max(g.kmax, q.k);
        // Morton buckets: about four points each
        int bits = 2;
        while (bits < 24 && ((int64_t)1 << (bits + 2)) < q.N)
            ++bits;
        h.hbits = bits;
        h.hoff = g.nbuckets;
        g.nbuckets += (int64_t)1 << bits;
    }
    B->total_rows = out_row;
    B->total_idx = idx_off;

    // k-groups
    for (int s = 0; s < P;)
    {
        KGroup K;
        K.k = B->hp[s].k;
        K.first = s;
        K.out_row0 = B->hp[s].out_row0;
        K.idx_off = B->hp[s].idx_off;
        while (s < P && B->hp[s].k == K.k)
        {
            K.rows += B->hp[s].N;
            ++s;
        }
        K.count = s - K.first;
        K.cap = K.rows * (int64_t)(K.k + 1) * (K.k + 1);
        B->kg.push_back(K);
    }
    B->kgroup_of.assign(P, 0);
    for (size_t g = 0; g < B->kg.size(); ++g)
        for (int s = B->kg[g].first; s < B->kg[g].first + B->kg[g].count; ++s)
            B->kgroup_of[s] = (int)g;

    // device memory
    cudaStream_t st = B->ctx->stream;
    auto& own = B->owned;
    B->probs = dalloc<BatchProb>(own, P);
    B->prob_n = dalloc<int64_t>(own, P);
    B->prob_R = dalloc<float>(own, P);
    B->prob_scale = dalloc<float>(own, P);
    B->means = dalloc<float>(own, (size_t)P * B_DMAX);
    B->row_prob_out = dalloc<int32_t>(own, (size_t)B->total_rows);
    B->idx_all = dalloc<int32_t>(own, (size_t)B->total_idx);
    B->w_all = dalloc<double>(own, (size_t)B->total_idx);
    B->nfailed = dalloc<unsigned>(own, 4 * B->sg.size());  // re-rank counters, 4 per screen group
    B->H = dalloc<float>(own, (size_t)P * 3 * B_DMAX);
    B->r_bits = dalloc<unsigned>(own, P);
    upload(B->probs, B->hp, st);
    std::vector<int64_t> pn(P);
    std::vector<int32_t> rpo((size_t)B->total_rows);
    for (int s = 0; s < P; ++s)
    {
        pn[s] = B->hp[s].N;
        std::fill(rpo.begin() + B->hp[s].out_row0, rpo.begin() + B->hp[s].out_row0 + B->hp[s].N, s);
    }
    upload(B->prob_n, pn, st);
    upload(B->row_prob_out, rpo, st);
    for (ScreenGroup& g : B->sg)
    {
        g.xh = dalloc<__half>(own, (size_t)g.rows * g.Dp);
        g.xl = dalloc<__half>(own, (size_t)g.rows * g.Dp);
        g.xn = dalloc<__half>(own, (size_t)g.rows * 16);
        g.nrm = dalloc<float>(own, (size_t)g.rows);
        g.cand_idx = dalloc<int32_t>(own, (size_t)g.rows * g.kc);
        g.cand_val = dalloc<float>(own, (size_t)g.rows * g.kc);
        g.row_prob = dalloc<int32_t>(own, (size_t)g.rows);
        g.perm_st = dalloc<int32_t>(own, (size_t)g.rows);
        g.partial = dalloc<double>(own, (size_t)(g.rows / 256) * B_DMAX);
        g.proj = dalloc<float>(own, (size_t)g.rows * 3);
        g.bucket = dalloc<int32_t>(own, (size_t)g.rows);
        g.hist = dalloc<int>(own, (size_t)g.nbuckets);
        g.fillc = dalloc<int>(own, (size_t)g.nbuckets);
        g.offs = dalloc<int64_t>(own, (size_t)g.nbuckets + 1);
        g.grp_probs = dalloc<int32_t>(own, g.probs.size());
        std::vector<int32_t> rp((size_t)g.rows, -1);
        std::vector<int4> items;
        const int qrows = g.qt * 128;
        for (int s : g.probs)
        {
            const BatchProb& h = B->hp[s];
            const int64_t npad = ((h.N + 255) / 256) * 256;
            std::fill(rp.begin() + h.row0, rp.begin() + h.row0 + npad, s);
            for (int64_t q = 0; q < npad; q += qrows)
                items.push_back(make_int4((int)((h.row0 + q) / qrows), (int)(h.row0 / 128), (int)(npad / 128), s));
        }
        // longest items first, spread over the persistent CTAs in that order
        std::stable_sort(items.begin(), items.end(), [](const int4& a, const int4& b) { return a.z > b.z; });
        g.nitems = (int)items.size();
        g.items = dalloc<int4>(own, items.size());
        upload(g.row_prob, rp, st);
        upload(g.grp_probs, std::vector<int32_t>(g.probs.begin(), g.probs.end()), st);
        upload(g.items, items, st);
    }
    for (KGroup& K : B->kg)
    {
        K.idx_g = dalloc<int32_t>(own, (size_t)K.rows * K.k);
        K.row_ptr = dalloc<int64_t>(own, (size_t)K.rows + 1);
        K.col = dalloc<int32_t>(own, (size_t)K.cap);
        K.val = dalloc<double>(own, (size_t)K.cap);
    }
    TK_CUDA(cudaStreamSynchronize(st));
}

} // namespace
} // namespace tk

extern "C" {

void tk_batch_tuning_default(tk_batch_tuning* t)
{
    if (!t)
        return;
    t->screen_qt[0] = 2;
    t->screen_qt[1] = 1;
    t->lle_warps = 8;
    t->wide_lists = 0;
}

int tk_batch_create(tk_ctx* ctx, const tk_batch_problem* problems, int count, double klle_shift,
                    double nullspace_shift, const tk_batch_tuning* tuning, tk_batch** out)
{
    if (!ctx || !out)
        return TK_ERR_INVALID_ARG;
    *out = nullptr;
    tk_batch* B = new (std::nothrow) tk_batch();
    if (!B)
        return TK_ERR_OOM;
    const int rc = batch_guard(ctx, [&] {
        if (!problems || count <= 0)
            throw Error(TK_ERR_NO_DATA, "batch: no problems");
        if (!(klle_shift >= 0.0))
            throw Error(TK_ERR_INVALID_ARG, "batch: klle_shift must be >= 0");
        B->parent = ctx;
        B->klle_shift = klle_shift;
        B->nullspace_shift = nullspace_shift;
        if (tuning)
            B->tuning = *tuning;
        else
            tk_batch_tuning_default(&B->tuning);
        if (B->tuning.lle_warps != 4)
            B->tuning.lle_warps = 8;
        // a private context with its own (capturable, non-legacy) stream, ordered
        // after the parent's stream at every run
        tk_ctx* inner = nullptr;
        const int st = tk_ctx_create(ctx->device, nullptr, &inner);
        if (st != TK_OK)
            throw Error(st, "batch: private context creation failed");
        B->ctx = inner;
        TK_CUDA(cudaEventCreate(&B->ev0));
        TK_CUDA(cudaEventCreate(&B->ev1));
        TK_CUDA(cudaEventCreateWithFlags(&B->evp, cudaEventDisableTiming));
        TK_CUDA(cudaEventRecord(B->evp, ctx->stream));
        TK_CUDA(cudaStreamWaitEvent(B->ctx->stream, B->evp, 0));
        plan(B, problems, count);
        // one eager pass sizes every scratch buffer and checks the plan, so the
        // captured sequence allocates nothing
        enqueue(B);
        check_errors(B);
        TK_CUDA(cudaStreamBeginCapture(B->ctx->stream, cudaStreamCaptureModeThreadLocal));
        try
        {
            enqueue(B);
        }
        catch (...)
        {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(B->ctx->stream, &g);
            if (g)
                cudaGraphDestroy(g);
            cudaGetLastError();
            throw;
        }
        TK_CUDA(cudaStreamEndCapture(B->ctx->stream, &B->graph));
        TK_CUDA(cudaGraphInstantiate(&B->exec, B->graph, 0));
    });
    if (rc != TK_OK)
    {
        destroy(B);
        return rc;
    }
    *out = B;
    return TK_OK;
}

int tk_batch_run(tk_batch* B, float* ms_out)
{
    if (!B)
        return TK_ERR_INVALID_ARG;
    return batch_guard(B->parent, [&] {
        cudaStream_t st = B->ctx->stream;
        TK_CUDA(cudaEventRecord(B->evp, B->parent->stream));
        TK_CUDA(cudaStreamWaitEvent(st, B->evp, 0));
        TK_CUDA(cudaEventRecord(B->ev0, st));
        TK_CUDA(cudaGraphLaunch(B->exec, st));
        TK_CUDA(cudaEventRecord(B->ev1, st));
        check_errors(B);
        TK_CUDA(cudaEventElapsedTime(&B->last_ms, B->ev0, B->ev1));
        if (ms_out)
            *ms_out = B->last_ms;
    });
}

int tk_batch_count(const tk_batch* B) { return B ? (int)B->in.size() : 0; }

int tk_batch_get_info(tk_batch* B, int p, tk_operator_info* info)
{
    if (!B || !info)
        return TK_ERR_INVALID_ARG;
    return batch_guard(B->parent, [&] {
        if (p < 0 || p >= (int)B->in.size())
            throw Error(TK_ERR_INVALID_ARG, "batch: problem index out of range");
        TK_CUDA(cudaStreamSynchronize(B->ctx->stream));
        const int s = B->pos_of[p];
        const BatchProb& h = B->hp[s];
        const KGroup& K = B->kg[B->kgroup_of[s]];
        int64_t ends[2];
        const int64_t r0 = h.out_row0 - K.out_row0;
        TK_CUDA(cudaMemcpy(&ends[0], K.row_ptr + r0, sizeof(int64_t), cudaMemcpyDeviceToHost));
        TK_CUDA(cudaMemcpy(&ends[1], K.row_ptr + r0 + h.N, sizeof(int64_t), cudaMemcpyDeviceToHost));
        unsigned cnt[4] = {};
        TK_CUDA(cudaMemcpy(cnt, B->nfailed + 4 * h.group, sizeof(cnt), cudaMemcpyDeviceToHost));
        std::memset(info, 0, sizeof(*info));
        info->n = h.N;
        info->k = h.k;
        info->method = TK_METHOD_KLLE;
        info->nnz = ends[1] - ends[0];
        info->rows_uncertified = cnt[0];  // of the problem's screen group
        info->tie_rows = cnt[1];
        info->extra_rows = cnt[2];
        info->stage_ms[4] = B->last_ms;
    });
}

int tk_batch_copy(tk_batch* B, int p, int32_t* idx, double* weights, int64_t* row_ptr, int32_t* col_idx, double* vals)
{
    if (!B)
        return TK_ERR_INVALID_ARG;
    return batch_guard(B->parent, [&] {
        if (p < 0 || p >= (int)B->in.size())
            throw Error(TK_ERR_INVALID_ARG, "batch: problem index out of range");
        TK_CUDA(cudaStreamSynchronize(B->ctx->stream));
        const int s = B->pos_of[p];
        const BatchProb& h = B->hp[s];
        const KGroup& K = B->kg[B->kgroup_of[s]];
        const size_t nk = (size_t)h.N * h.k;
        if (idx)
            TK_CUDA(cudaMemcpy(idx, B->idx_all + h.idx_off, sizeof(int32_t) * nk, cudaMemcpyDefault));
        if (weights)
            TK_CUDA(cudaMemcpy(weights, B->w_all + h.idx_off, sizeof(double) * nk, cudaMemcpyDefault));
        if (row_ptr || col_idx || vals)
        {
            const int64_t r0 = h.out_row0 - K.out_row0;
            std::vector<int64_t> rp((size_t)h.N + 1);
            TK_CUDA(cudaMemcpy(rp.data(), K.row_ptr + r0, sizeof(int64_t) * rp.size(), cudaMemcpyDeviceToHost));
            const int64_t base = rp[0], nnz = rp.back() - rp[0];
            if (row_ptr)
            {
                for (auto& v : rp)
                    v -= base;
                TK_CUDA(cudaMemcpy(row_ptr, rp.data(), sizeof(int64_t) * rp.size(), cudaMemcpyDefault));
            }
            if (vals)
                TK_CUDA(cudaMemcpy(vals, K.val + base, sizeof(double) * (size_t)nnz, cudaMemcpyDefault));
            if (col_idx)
            {
                // group-global columns back to the problem's own numbering
                std::vector<int32_t> c((size_t)nnz);
                TK_CUDA(cudaMemcpy(c.data(), K.col + base, sizeof(int32_t) * c.size(), cudaMemcpyDeviceToHost));
                for (auto& v : c)
                    v -= (int32_t)r0;
                TK_CUDA(cudaMemcpy(col_idx, c.data(), sizeof(int32_t) * c.size(), cudaMemcpyDefault));
            }
        }
    });
}

int tk_batch_destroy(tk_batch* B)
{
    destroy(B);
    return TK_OK;
}

} // extern "C"
