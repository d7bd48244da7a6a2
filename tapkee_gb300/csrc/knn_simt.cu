// knn_simt.cu -- plain FP32 CUDA-core distance screen.
//
// For each block of 128 queries (sorted order) the kernel streams every
// candidate tile of 128 points, computes the 128x128 dot products with a
// register-tiled FP32 FMA GEMM (8x8 outputs per thread, 16-deep k chunks
// double-buffered through shared memory), forms the approximate squared
// distance a = |x|^2 + |y|^2 - 2 x.y and keeps, per query row, the KC smallest
// values (sorted list in shared memory). Only entries below the row's current
// KC-th value are recorded (bitmask + value tile), so after the first tiles
// almost no work is spent on the list.
//
// This is the "plain FP32" engine the tensor-core screen is compared with:
// identical data, visit order, candidate lists and certification; only the
// dot-product engine differs.
#include <cfloat>

#include "screen_common.cuh"
#include "tk_internal.h"

namespace tk {
namespace {

constexpr int BN = 128, BK = 16, THREADS = 256;

// BM queries per CTA (128: 8x8 outputs per thread; 64: 4x8, used with the long
// candidate lists of k > 56), KC candidates kept per query.
template <int BM, int KC>
struct SimtSmem
{
    float As[2][BK][BM + 4];
    float Bs[2][BK][BN + 4];
    float dist[BM][BN];
    unsigned mask[BM][BN / 32];
    float lv[BM][KC];
    int32_t li[BM][KC];
    float cmp[BM];   // row threshold minus |x|^2
    float nq[BM];    // query norms
    float nc[BN];    // candidate norms of the current tile
};

template <int BM, int KC>
__global__ void __launch_bounds__(THREADS, 1)
    k_screen_simt(const float* __restrict__ xc, const float* __restrict__ nrm, int64_t Npad, int Dp,
                  int32_t* __restrict__ cand_idx, float* __restrict__ cand_val)
{
    constexpr int TM = BM / 16;  // rows per thread
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SimtSmem<BM, KC>& S = *reinterpret_cast<SimtSmem<BM, KC>*>(smem_raw);
    const int tid = threadIdx.x;
    const int tr = tid >> 4, tc = tid & 15;
    const int64_t q0 = (int64_t)blockIdx.x * BM;
    const int ntiles = (int)(Npad / BN);
    const int nk = Dp / BK;

    for (int t = tid; t < BM * KC; t += THREADS)
    {
        (&S.lv[0][0])[t] = FLT_MAX;
        (&S.li[0][0])[t] = -1;
    }
    if (tid < BM)
    {
        S.nq[tid] = nrm[q0 + tid];
        S.cmp[tid] = FLT_MAX;
    }

    // global -> shared staging (transposed to k-major), float4 per element group
    auto load_chunk = [&](int buf, int64_t c0, int kc) {
        for (int e = tid; e < BM * (BK / 4); e += THREADS)
        {
            const int row = e / (BK / 4), kq = e % (BK / 4);
            const float4 a = *reinterpret_cast<const float4*>(xc + (q0 + row) * Dp + kc * BK + kq * 4);
            S.As[buf][kq * 4 + 0][row] = a.x;
            S.As[buf][kq * 4 + 1][row] = a.y;
            S.As[buf][kq * 4 + 2][row] = a.z;
            S.As[buf][kq * 4 + 3][row] = a.w;
        }
        for (int e = tid; e < BN * (BK / 4); e += THREADS)
        {
            const int row = e / (BK / 4), kq = e % (BK / 4);
            const float4 b = *reinterpret_cast<const float4*>(xc + (c0 + row) * Dp + kc * BK + kq * 4);
            S.Bs[buf][kq * 4 + 0][row] = b.x;
            S.Bs[buf][kq * 4 + 1][row] = b.y;
            S.Bs[buf][kq * 4 + 2][row] = b.z;
            S.Bs[buf][kq * 4 + 3][row] = b.w;
        }
    };

    ZigZag zz((int)((q0 / BN) < ntiles ? (q0 / BN) : 0), ntiles);
    for (int it = 0; it < ntiles; ++it)
    {
        const int tile = zz.next();
        const int64_t c0 = (int64_t)tile * BN;
        float acc[TM][8];
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
            for (int j = 0; j < 8; ++j)
                acc[i][j] = 0.f;

        __syncthreads();  // previous tile's list processing / smem reuse done
        if (tid < BN)
            S.nc[tid] = nrm[c0 + tid];
        load_chunk(0, c0, 0);
        __syncthreads();
        for (int kc = 0; kc < nk; ++kc)
        {
            const int buf = kc & 1;
            if (kc + 1 < nk)
                load_chunk(buf ^ 1, c0, kc + 1);
#pragma unroll
            for (int kk = 0; kk < BK; ++kk)
            {
                float a[TM];
#pragma unroll
                for (int q = 0; q < TM / 4; ++q)
                {
                    const float4 aq = *reinterpret_cast<const float4*>(&S.As[buf][kk][tr * TM + 4 * q]);
                    a[4 * q + 0] = aq.x;
                    a[4 * q + 1] = aq.y;
                    a[4 * q + 2] = aq.z;
                    a[4 * q + 3] = aq.w;
                }
                const float4 b0 = *reinterpret_cast<const float4*>(&S.Bs[buf][kk][tc * 4]);
                const float4 b1 = *reinterpret_cast<const float4*>(&S.Bs[buf][kk][64 + tc * 4]);
                const float b[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
                for (int i = 0; i < TM; ++i)
#pragma unroll
                    for (int j = 0; j < 8; ++j)
                        acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
            }
            __syncthreads();
        }

        // epilogue: record entries below the row threshold
        for (int t = tid; t < BM * (BN / 32); t += THREADS)
            (&S.mask[0][0])[t] = 0u;
        __syncthreads();
#pragma unroll
        for (int i = 0; i < TM; ++i)
        {
            const int r = tr * TM + i;
            const float cmp = S.cmp[r];
#pragma unroll
            for (int j = 0; j < 8; ++j)
            {
                const int c = (j < 4) ? (tc * 4 + j) : (64 + tc * 4 + (j - 4));
                const float v = fmaf(-2.f, acc[i][j], S.nc[c]);
                if (v < cmp)
                {
                    S.dist[r][c] = v;
                    atomicOr(&S.mask[r][c >> 5], 1u << (c & 31));
                }
            }
        }
        __syncthreads();
        if (tid < BM)
        {
            const int r = tid;
            const float nq = S.nq[r];
#pragma unroll 1
            for (int w = 0; w < BN / 32; ++w)
            {
                unsigned bits = S.mask[r][w];
                while (bits)
                {
                    const int b = __ffs(bits) - 1;
                    bits &= bits - 1;
                    const int c = w * 32 + b;
                    list_insert<KC>(S.lv[r], S.li[r], S.dist[r][c] + nq, (int32_t)(c0 + c));
                }
            }
            S.cmp[r] = S.lv[r][KC - 1] - nq;
        }
    }
    __syncthreads();
    for (int t = tid; t < BM * KC; t += THREADS)
    {
        const int r = t / KC, s = t % KC;
        cand_idx[(q0 + r) * KC + s] = S.li[r][s];
        cand_val[(q0 + r) * KC + s] = S.lv[r][s];
    }
}

template <int BM, int KC>
void launch(tk_ctx* ctx, const Prepared& P, int32_t* cand_idx, float* cand_val)
{
    const size_t smem = sizeof(SimtSmem<BM, KC>);
    static_assert(sizeof(SimtSmem<BM, KC>) <= 227 * 1024, "shared memory budget");
    TK_CUDA(cudaFuncSetAttribute(k_screen_simt<BM, KC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int grid = (int)(P.Npad / BM);
    k_screen_simt<BM, KC><<<grid, THREADS, smem, ctx->stream>>>(P.xc, P.nrm, P.Npad, P.Dp, cand_idx, cand_val);
    TK_CHECK_LAUNCH();
}

} // namespace

void screen_fp32(tk_ctx* ctx, const Prepared& P, int kc, int32_t* cand_idx, float* cand_val)
{
    if (kc == 32)
        launch<128, 32>(ctx, P, cand_idx, cand_val);
    else if (kc == 64)
        launch<128, 64>(ctx, P, cand_idx, cand_val);
    else if (kc == 128)
        launch<64, 128>(ctx, P, cand_idx, cand_val);
    else if (kc == 256)
        launch<64, 256>(ctx, P, cand_idx, cand_val);
    else
        throw Error(TK_ERR_INTERNAL, "screen_fp32: unsupported candidate count");
}

} // namespace tk
