// lle_pair.cu -- LLE reconstruction weights for float32 points and k <= 16, two
// points per warp.
//
// The computation of k_lle (lle.cu), for the solve of linear_weight_matrix
// (routines/locally_linear.hpp:107-131):
//   C_ab = (n_a - x).(n_b - x),  C += klle_shift * trace(C) * I,
//   w = C^{-1} rhs (rhs = 1 for the weights),  w /= sum(w)
// with an FP32 Cholesky factor refined against a float-float residual from the
// exact differences. The organisation differs; it is built to issue fewer
// instructions per point:
//   * each half-warp owns one point of a pair, so the register Cholesky and the
//     substitutions (16-lane shuffles) advance two points per instruction;
//   * the neighbour rows and the point's own row are staged once per chunk of 64
//     dimensions into shared memory with 16-byte loads; the refinement reads them
//     there instead of gathering them again (for D <= 64);
//   * the Gram matrix is formed on the tensor cores, warp-wide, one point at a
//     time: mma.sync m16n8k8 with TF32 operands split into a big and a small part
//     (z = big + small + O(2^-22 |z|)), three products per term (big.big,
//     big.small, small.big) accumulated in FP32. This is an FP32-accurate Gram;
//     like the FP32 Gram of k_lle it only seeds the factor, and the float-float
//     refinement against the exact differences sets the accuracy of w;
//   * the refinement's float-float products and sums run on Blackwell's packed
//     FP32 instructions (__fadd2_rn, __fmul2_rn, __ffma2_rn), two neighbours per
//     instruction, each component rounded as its scalar form.
// Requires float32 input with 16-byte aligned rows (X 16-byte aligned, ldx a
// multiple of 4); other inputs take k_lle.
#include <cfloat>
#include <cstdint>

#include "ff.cuh"
#include "tk_internal.h"

namespace tk {
namespace {

constexpr int PW = 8;       // warps per block
constexpr int CH = 64;      // dimensions staged per chunk
constexpr int RS = CH + 4;  // row stride of a staged chunk: conflict-free fragment loads

struct PairSmem
{
    float nr[2][16][RS];  // the chunk of each neighbour row, per point of the pair
    float xr[2][CH];      // the chunk of the points' own rows
    float c[2][16][17];   // Gram, then the rows of the Cholesky factor
    float ivd[2][16];     // reciprocal diagonal of the factor
    float w[2][16];       // the current solution, broadcast to the refinement
};

__device__ __forceinline__ uint32_t to_tf32(float x)
{
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

// d += a * b for one m16n8k8 tile (TF32 operands, FP32 accumulators)
__device__ __forceinline__ void mma_tf32(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1)
{
    asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};\n"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// Packed FP32 (two lanes of arithmetic per instruction) forms of the
// error-free transformations: each component is rounded exactly as the scalar
// __fadd_rn / __fmul_rn / fmaf would round it.
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b)  // a - b, one rounding
{
    return __ffma2_rn(b, make_float2(-1.f, -1.f), a);
}
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }

// (h + l) += (bh + bl) for two independent float-float values, as ff_add
__device__ __forceinline__ void ff_add2(float2& h, float2& l, float2 bh, float2 bl)
{
    const float2 s = add2(h, bh);
    const float2 bb = sub2(s, h);
    const float2 e = add2(sub2(h, sub2(s, bb)), sub2(bh, bb));
    const float2 lo = add2(e, add2(l, bl));
    const float2 s2 = add2(s, lo);  // fast two-sum: |s| >= |lo|
    h = s2;
    l = sub2(lo, sub2(s2, s));
}

// acc += p (ph + pl) without renormalising, for two independent accumulators:
// acc.hi is the running sum, acc.lo collects the exact rounding error of each
// addition (Knuth's two-sum) and the low parts
__device__ __forceinline__ void ff_acc2(float2& ah, float2& al, float2 ph, float2 pl)
{
    const float2 s = add2(ah, ph);
    const float2 bb = sub2(s, ah);
    const float2 e = add2(sub2(ah, sub2(s, bb)), sub2(ph, bb));
    ah = s;
    al = add2(al, add2(e, pl));
}

// Lane l of a 16-lane segment holds row l of a 16 x 16 SPD matrix (L[c], c <= l)
// and ends with row l of its lower Cholesky factor and invd = 1 / L_ll.
__device__ __forceinline__ void chol16(float (&L)[16], float& invd, int l)
{
    invd = 1.f;
#pragma unroll
    for (int j = 0; j < 16; ++j)
    {
        const float inv = rsqrtf(fmaxf(__shfl_sync(0xffffffffu, L[j], j, 16), FLT_MIN));
        if (l >= j)
            L[j] *= inv;
        if (l == j)
            invd = inv;
#pragma unroll
        for (int c = j + 1; c < 16; ++c)
        {
            const float lcj = __shfl_sync(0xffffffffu, L[j], c, 16);
            if (l >= c)
                L[c] = fmaf(-L[j], lcj, L[c]);
        }
    }
}

// Solves L L^T x = r in a 16-lane segment: lane l holds r_l and row l of L
// (Lrow), and gets x_l. The backward sweep reads column l of L from Ls (rows of
// the factor, stride 17); ivd holds the reciprocal diagonal.
__device__ __forceinline__ float solve16(const float (&Lrow)[16], const float* Ls, const float* ivd, float r, int l)
{
    float y = r;
#pragma unroll
    for (int j = 0; j < 16; ++j)
    {
        const float yj = __shfl_sync(0xffffffffu, y, j, 16) * ivd[j];
        if (l == j)
            y = yj;
        else if (l > j)
            y = fmaf(-Lrow[j], yj, y);
    }
#pragma unroll
    for (int j = 15; j >= 0; --j)
    {
        const float lji = (l < j) ? Ls[j * 17 + l] : 0.f;
        const float xj = __shfl_sync(0xffffffffu, y, j, 16) * ivd[j];
        if (l == j)
            y = xj;
        else if (l < j)
            y = fmaf(-lji, xj, y);
    }
    return y;
}

// Stages dimensions [c0, c0 + CH) of the neighbour rows and the point's row of
// this half-warp's point into shared memory (zero beyond D); padding neighbours
// (a >= k) repeat the point itself, so their differences are exactly zero.
__device__ __forceinline__ void stage_chunk(PairSmem& S, int h, int l, const float* __restrict__ X, int64_t ldx, int D,
                                            int64_t p, int nb, int c0)
{
    const int d = c0 + 4 * l;
    auto load4 = [&](int64_t row) {
        const float* src = X + row * ldx + d;
        if (d + 3 < D)
            return __ldg(reinterpret_cast<const float4*>(src));
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (d < D)
            v.x = __ldg(src);
        if (d + 1 < D)
            v.y = __ldg(src + 1);
        if (d + 2 < D)
            v.z = __ldg(src + 2);
        return v;
    };
    float4 v[16];
#pragma unroll
    for (int a = 0; a < 16; ++a)
        v[a] = load4(__shfl_sync(0xffffffffu, nb, (h << 4) + a));
    const float4 xv = load4(p);
#pragma unroll
    for (int a = 0; a < 16; ++a)
        *reinterpret_cast<float4*>(&S.nr[h][a][4 * l]) = v[a];
    *reinterpret_cast<float4*>(&S.xr[h][4 * l]) = xv;
}

__global__ void __launch_bounds__(PW * 32, 2)
    k_lle_pair(const float* __restrict__ X, int64_t N, int D, int64_t ldx, const int32_t* __restrict__ idx, int k,
               double klle_shift, const double* __restrict__ rhs, int normalize, double* __restrict__ W,
               unsigned* err)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    PairSmem& S = reinterpret_cast<PairSmem*>(smem_raw)[wib];
    const int h = lane >> 4, l = lane & 15;  // point of the pair, lane in its half
    const int g = lane >> 2, t = lane & 3;   // mma fragment coordinates
    const ff ks = ff{(float)klle_shift, (float)(klle_shift - (double)(float)klle_shift)};
    const int64_t npairs = (N + 1) / 2;
    const int64_t pw = (int64_t)blockIdx.x * PW + wib;
    const int64_t nw = (int64_t)gridDim.x * PW;
    const int nchunks = (D + CH - 1) / CH;
    for (int64_t pr = pw; pr < npairs; pr += nw)
    {
        const bool valid1 = 2 * pr + 1 < N;  // the second point exists (warp-uniform)
        const int64_t p = valid1 ? 2 * pr + h : 2 * pr;
        const bool active = (h == 0) || valid1;
        int nb = (int)p;
        if (l < k)
        {
            const int j = idx[p * k + l];
            if (j < 0 || j >= N)
            {
                if (active)
                    atomicOr(err, DEV_ERR_BOUNDS);
            }
            else
                nb = j;
        }

        // ---- Gram on the tensor cores: acc[P][n-tile] for P = 0, 1 ----
        float acc[2][2][4];
#pragma unroll
        for (int P = 0; P < 2; ++P)
#pragma unroll
            for (int nt = 0; nt < 2; ++nt)
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    acc[P][nt][e] = 0.f;
        for (int ch = 0; ch < nchunks; ++ch)
        {
            __syncwarp();
            stage_chunk(S, h, l, X, ldx, D, p, nb, ch * CH);
            __syncwarp();
#pragma unroll
            for (int P = 0; P < 2; ++P)
            {
                if (P == 1 && !valid1)
                    break;
#pragma unroll 2
                for (int kk = 0; kk < CH / 8; ++kk)
                {
                    const int d0 = kk * 8 + t, d1 = d0 + 4;
                    const float xa = S.xr[P][d0], xb = S.xr[P][d1];
                    // (rows g, g + 8) per packed instruction
                    const float2 za = sub2(make_float2(S.nr[P][g][d0], S.nr[P][g + 8][d0]), make_float2(xa, xa));
                    const float2 zb = sub2(make_float2(S.nr[P][g][d1], S.nr[P][g + 8][d1]), make_float2(xb, xb));
                    const uint32_t b00 = to_tf32(za.x), b10 = to_tf32(za.y), b01 = to_tf32(zb.x), b11 = to_tf32(zb.y);
                    const float2 sa = sub2(za, make_float2(__uint_as_float(b00), __uint_as_float(b10)));
                    const float2 sb = sub2(zb, make_float2(__uint_as_float(b01), __uint_as_float(b11)));
                    const uint32_t s00 = to_tf32(sa.x), s10 = to_tf32(sa.y);
                    const uint32_t s01 = to_tf32(sb.x), s11 = to_tf32(sb.y);
                    // A = rows g, g + 8 of Z; B (= Z^T) for neighbours 0-7 is row g,
                    // for neighbours 8-15 row g + 8
                    mma_tf32(acc[P][0], b00, b10, b01, b11, b00, b01);
                    mma_tf32(acc[P][0], b00, b10, b01, b11, s00, s01);
                    mma_tf32(acc[P][0], s00, s10, s01, s11, b00, b01);
                    mma_tf32(acc[P][1], b00, b10, b01, b11, b10, b11);
                    mma_tf32(acc[P][1], b00, b10, b01, b11, s10, s11);
                    mma_tf32(acc[P][1], s00, s10, s01, s11, b10, b11);
                }
            }
        }
        __syncwarp();
#pragma unroll
        for (int P = 0; P < 2; ++P)
#pragma unroll
            for (int nt = 0; nt < 2; ++nt)
            {
                S.c[P][g][nt * 8 + 2 * t] = acc[P][nt][0];
                S.c[P][g][nt * 8 + 2 * t + 1] = acc[P][nt][1];
                S.c[P][g + 8][nt * 8 + 2 * t] = acc[P][nt][2];
                S.c[P][g + 8][nt * 8 + 2 * t + 1] = acc[P][nt][3];
            }
        __syncwarp();

        // ---- regularise and factor (each half-warp its own point) ----
        float trace = (l < k) ? S.c[h][l][l] : 0.f;
#pragma unroll
        for (int o = 8; o > 0; o >>= 1)
            trace += __shfl_xor_sync(0xffffffffu, trace, o);
        const float shift = (float)klle_shift * trace;
        float L[16];
#pragma unroll
        for (int c = 0; c < 16; ++c)
            L[c] = (l < k && c <= l && c < k) ? S.c[h][l][c] : 0.f;
        if (l < k)
            L[l] += shift;
        else
            L[l] = 1.f;  // padding: identity block
        float invd;
        chol16(L, invd, l);
        __syncwarp();
#pragma unroll
        for (int c = 0; c < 16; ++c)
            if (c <= l)
                S.c[h][l][c] = L[c];
        S.ivd[h][l] = invd;
        __syncwarp();
        const float b0 = (l < k) ? (rhs ? (float)rhs[p * k + l] : 1.f) : 0.f;
        float w = solve16(L, &S.c[h][0][0], S.ivd[h], b0, l);
        if (l >= k)
            w = 0.f;

        // ---- float-float refinement against the exact differences ----
        const int iters = (k > D) ? 2 : 1;
        for (int itr = 0; itr < iters; ++itr)
        {
            __syncwarp();
            S.w[h][l] = w;
            __syncwarp();
            const float2* wb2 = reinterpret_cast<const float2*>(S.w[h]);
            // neighbours in pairs (2i, 2i + 1): one packed instruction for both
            float2 pth[8], ptl[8];
#pragma unroll
            for (int i = 0; i < 8; ++i)
            {
                pth[i] = make_float2(0.f, 0.f);
                ptl[i] = make_float2(0.f, 0.f);
            }
            for (int ch = 0; ch < nchunks; ++ch)
            {
                if (nchunks > 1)
                {
                    __syncwarp();
                    stage_chunk(S, h, l, X, ldx, D, p, nb, ch * CH);
                    __syncwarp();
                }
#pragma unroll 1
                for (int dd = 0; dd < 4; ++dd)
                {
                    const int d = 4 * l + dd;
                    if (ch * CH + d >= D)
                        break;
                    const float xd = S.xr[h][d];
                    const float2 x2 = make_float2(xd, xd);
                    float2 zh[8], zl[8];
                    float2 vh = make_float2(0.f, 0.f), vl = vh;  // v over even / odd neighbours
#pragma unroll
                    for (int i = 0; i < 8; ++i)
                    {
                        // exact difference n - x = zh + zl (Knuth's two-sum)
                        const float2 n2 = make_float2(S.nr[h][2 * i][d], S.nr[h][2 * i + 1][d]);
                        const float2 zs = sub2(n2, x2);
                        const float2 bb = sub2(zs, n2);
                        zh[i] = zs;
                        zl[i] = sub2(sub2(n2, sub2(zs, bb)), add2(x2, bb));
                        // w z = p + pe exactly for the high part, plus w zl
                        const float2 w2 = wb2[i];
                        const float2 pp = __fmul2_rn(w2, zs);
                        const float2 pe = __ffma2_rn(w2, zs, neg2(pp));
                        ff_acc2(vh, vl, pp, __ffma2_rn(w2, zl[i], pe));
                    }
                    ff v = ff_add(ff{vh.x, vl.x}, ff{vh.y, vl.y});
                    const float2 vh2 = make_float2(v.hi, v.hi), vl2 = make_float2(v.lo, v.lo);
#pragma unroll
                    for (int i = 0; i < 8; ++i)
                    {
                        const float2 pp = __fmul2_rn(zh[i], vh2);
                        const float2 pe = __ffma2_rn(zh[i], vh2, neg2(pp));
                        ff_acc2(pth[i], ptl[i], pp, __ffma2_rn(zh[i], vl2, __ffma2_rn(zl[i], vh2, pe)));
                    }
                }
            }
            // reduce-scatter over the 16 lanes: lane l ends with (C w)_l; the
            // neighbour pairs (2i, 2i + 1) add with packed instructions down to
            // two values, then the last level is scalar
#pragma unroll
            for (int o = 4; o > 0; o >>= 1)  // pair offsets: value offsets 8, 4, 2
            {
                const bool upper = (l & (2 * o)) != 0;
#pragma unroll
                for (int q = 0; q < o; ++q)
                {
                    const float2 sh = upper ? pth[q] : pth[q + o], sl = upper ? ptl[q] : ptl[q + o];
                    float2 kh = upper ? pth[q + o] : pth[q], kl = upper ? ptl[q + o] : ptl[q];
                    const float2 rh = make_float2(__shfl_xor_sync(0xffffffffu, sh.x, 2 * o),
                                                  __shfl_xor_sync(0xffffffffu, sh.y, 2 * o));
                    const float2 rl = make_float2(__shfl_xor_sync(0xffffffffu, sl.x, 2 * o),
                                                  __shfl_xor_sync(0xffffffffu, sl.y, 2 * o));
                    ff_add2(kh, kl, rh, rl);
                    pth[q] = kh;
                    ptl[q] = kl;
                }
            }
            ff part[1];
            {
                const bool upper = (l & 1) != 0;
                const ff send = upper ? ff{pth[0].x, ptl[0].x} : ff{pth[0].y, ptl[0].y};
                const ff keep = upper ? ff{pth[0].y, ptl[0].y} : ff{pth[0].x, ptl[0].x};
                part[0] = ff_add(keep, ff_shfl_xor(send, 1));
            }
            float r = 0.f;
            if (l < k)
            {
                const ff sw = ff_mul(ff_mul(ks, ff{trace, 0.f}), ff{w, 0.f});
                ff bb = ff{1.f, 0.f};
                if (rhs)
                {
                    const double rb = rhs[p * k + l];
                    bb.hi = (float)rb;
                    bb.lo = (float)(rb - (double)bb.hi);
                }
                const ff rr = ff_add(ff_add(bb, ff_neg(part[0])), ff_neg(sw));
                r = rr.hi + rr.lo;
            }
#pragma unroll
            for (int c = 0; c < 16; ++c)
                L[c] = (c <= l) ? S.c[h][l][c] : 0.f;
            const float x = solve16(L, &S.c[h][0][0], S.ivd[h], r, l);
            if (l < k)
                w += x;
        }

        // ---- normalise (weights) or store the raw solution (adjoint solve) ----
        if (!normalize)
        {
            if (active && l < k)
                W[p * k + l] = (double)w;
            continue;
        }
        ff sum = ff{(l < k) ? w : 0.f, 0.f};
#pragma unroll
        for (int o = 8; o > 0; o >>= 1)
            sum = ff_add(sum, ff_shfl_xor(sum, o));
        const float y0 = 1.f / sum.hi;
        const ff sy = two_prod(sum.hi, y0);
        const float resid = ((1.f - sy.hi) - sy.lo) - sum.lo * y0;
        const float y1 = y0 * resid;
        if (active && l < k)
        {
            const ff q = two_prod(w, y0);
            W[p * k + l] = (double)q.hi + (double)fmaf(w, y1, q.lo);
        }
    }
}

} // namespace

bool lle_pair_supported(const void* X, int dtype, int64_t ldx, int k)
{
    return dtype == TK_F32 && k >= 1 && k <= 16 && (ldx % 4) == 0 && (reinterpret_cast<uintptr_t>(X) % 16) == 0;
}

void lle_pair_solve(tk_ctx* ctx, const void* X, int64_t N, int D, int64_t ldx, const int32_t* idx, int k,
                    double klle_shift, const double* rhs, bool normalize, double* W)
{
    const size_t smem = sizeof(PairSmem) * PW;
    TK_CUDA(cudaFuncSetAttribute(k_lle_pair, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int64_t pairs = (N + 1) / 2;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((pairs + PW - 1) / PW, (int64_t)ctx->num_sms * 16));
    k_lle_pair<<<grid, PW * 32, smem, ctx->stream>>>(reinterpret_cast<const float*>(X), N, D, ldx, idx, k, klle_shift,
                                                     rhs, normalize ? 1 : 0, W, ctx->dev_err);
    TK_CHECK_LAUNCH();
}

} // namespace tk
