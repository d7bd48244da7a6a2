// knn_tc.cu -- tensor-core (tcgen05) distance screen for sm_103a.
//
// Each CTA owns QT blocks of 128 queries (sorted order) and streams every
// candidate tile of 128 points through a STAGES-deep TMA pipeline. The dot
// products x.y run on the 5th-generation tensor cores as an fp16 split GEMM
// with FP32 accumulation in tensor memory:
//      x.y ~ 2^-2s (h_x.h_y + h_x.l_y + l_x.h_y),   2^s x = h_x + l_x (fp16 hi/lo)
// (about 22 significant bits; the dropped l_x.l_y term is below 2^-22 |x||y|).
// One more K=16 MMA per tile multiplies a constant A slice (2^13 everywhere) by
// a per-candidate column holding -|2^s y|^2 / 2^14 as fp16 hi + lo, so the
// accumulator is 2^2s (x.y - |y|^2 / 2) and |y|^2 - 2 x.y = -2^(1-2s) acc: the
// epilogue needs no norm loads, only a running max per row.
// Accumulators (128 lanes x 128 columns FP32 per query block) are
// double-buffered in TMEM so the MMA of tile t+1 overlaps the epilogue of tile t.
//
// Warp roles (320 threads):
//   warps 0..7  epilogue: tcgen05.ld the accumulator rows; per 32 columns one
//               max and one compare against the row's KC-th value; only groups
//               that beat it are expanded into the row's sorted register list of
//               the KC smallest a - |x|^2 = |y|^2 - 2 x.y (one thread per row);
//   warp  8     TMA producer (one thread): A tiles once, then B hi/lo tiles;
//   warp  9     TMEM allocator and MMA issuer (one thread).
// Every mbarrier wait is bounded by a wall-clock limit: on expiry the CTA records
// DEV_ERR_TIMEOUT, drains the copies and MMAs it issued (again bounded), frees
// its TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_fp16.h>

#include <cfloat>

#include "screen_common.cuh"
#include "tk_internal.h"

namespace tk {
namespace {

constexpr int TC_N = 128;      // candidates per stage (MMA N)
constexpr int TC_M = 128;      // queries per A tile (MMA M)
constexpr int TC_THREADS = 320;
// Entries per pass of the long-list screen: with 32 columns per TMEM load, a
// 48-entry list (values and ids) fits the 168 registers a thread of a 10-warp CTA
// gets; a 64-entry list spills in the epilogue's loop.
constexpr int TC_PASS = 48;
constexpr uint64_t WAIT_LIMIT_NS = 2000000000ull;  // 2 s per single wait

// QT query blocks of 128 rows share each candidate tile (QT = 2 only for DP = 64:
// two 128-column accumulators double-buffered fill the 512 TMEM columns).
template <int DP, int QT_ = (DP <= 64) ? 2 : 1>
struct TcCfg
{
    static constexpr int QT = QT_;                 // A tiles (query blocks) per work item
    static constexpr int KATOMS = DP / 64;         // 128-byte swizzle atoms along K
    static constexpr int ATOM_BYTES = 128 * 128;   // 128 rows x 128 B (SW128)
    static constexpr int EXTRA_BYTES = 128 * 32;   // 128 rows x 32 B (SW32): the norm column slice
    static constexpr int A_BYTES = QT * 2 * KATOMS * ATOM_BYTES;
    static constexpr int B_OPER_BYTES = 2 * KATOMS * ATOM_BYTES;        // hi + lo
    static constexpr int B_STAGE_BYTES = B_OPER_BYTES + EXTRA_BYTES;    // + norm column
    // as many candidate stages as fit in 227 KB next to the A tiles, the norm
    // slice and the barriers (at most 6)
    static constexpr int FIXED_BYTES = EXTRA_BYTES + 256 + 1024;
    static constexpr int STAGES_FIT = (227 * 1024 - A_BYTES - FIXED_BYTES) / B_STAGE_BYTES;
    static constexpr int STAGES = STAGES_FIT > 6 ? 6 : STAGES_FIT;
    static constexpr int ACC_COLS = QT * TC_N;
    static constexpr int TMEM_COLS = 2 * ACC_COLS;  // 512 or 256, power of two
    static constexpr int EPI_WARPS = 4 * QT;
    static constexpr size_t OFF_AX = (size_t)A_BYTES + (size_t)STAGES * B_STAGE_BYTES;
    static constexpr size_t OFF_BAR = OFF_AX + EXTRA_BYTES;
    static constexpr size_t SMEM = OFF_BAR + 256 + 1024 /*align*/;
    static_assert(STAGES >= 2, "at least two candidate stages");
};

// ---------------------------------------------------------------- PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t gtimer()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// try_wait with a suspend-time hint: the thread sleeps in hardware until the
// phase completes or ~0.5 ms pass, instead of spinning on the issue slots.
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity), "r"(500000u)
        : "memory");
    return ok != 0;
}

// Bounded wait; returns false (and raises the CTA abort flag) on expiry or when
// another role already aborted.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* abort, unsigned* err)
{
    if (mbar_try(bar, parity))
        return true;
    const uint64_t t0 = gtimer();
    for (uint32_t it = 1;; ++it)
    {
        if (mbar_try(bar, parity))
            return true;
        if ((it & 3u) == 0u)
        {
            if (*abort)
                return false;
            if (gtimer() - t0 > WAIT_LIMIT_NS)
            {
                *abort = 1;
                atomicOr(err, DEV_ERR_TIMEOUT);
                return false;
            }
        }
    }
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            dst),
        "l"(map), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

// tcgen05 shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row
// groups 1024 B apart (SBO), version bit 46 set.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr)
{
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// Same for the 32-byte-swizzled K=16 slices (rows of 32 B, 8-row groups 256 B apart).
__device__ __forceinline__ uint64_t umma_desc_sw32(uint32_t saddr)
{
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(256 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)6 << 61);
}

// kind::f16 instruction descriptor: D=F32, A=B=F16, K-major both, N=128, M=128
constexpr uint32_t IDESC = (1u << 4) | ((uint32_t)(TC_N >> 3) << 17) | ((uint32_t)(TC_M >> 4) << 24);

__device__ __forceinline__ void umma_f16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate)
{
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            dtmem),
        "l"(adesc), "l"(bdesc), "r"(IDESC), "r"(accumulate));
}

__device__ __forceinline__ void umma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld32_nowait(uint32_t taddr, float* v)
{
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
#pragma unroll
    for (int t = 0; t < 32; ++t)
        v[t] = __uint_as_float(r[t]);
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// The same for 32 columns.
__device__ __forceinline__ float tmem_ld32_max_nowait(uint32_t taddr, float* v)
{
    float m;
    asm volatile("tcgen05.ld.red.sync.aligned.32x32b.x32.max.f32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, %32, [%33];"
                 : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7]), "=f"(v[8]), "=f"(v[9]), "=f"(v[10]), "=f"(v[11]), "=f"(v[12]), "=f"(v[13]), "=f"(v[14]), "=f"(v[15]), "=f"(v[16]), "=f"(v[17]), "=f"(v[18]), "=f"(v[19]), "=f"(v[20]), "=f"(v[21]), "=f"(v[22]), "=f"(v[23]), "=f"(v[24]), "=f"(v[25]), "=f"(v[26]), "=f"(v[27]), "=f"(v[28]), "=f"(v[29]), "=f"(v[30]), "=f"(v[31]), "=f"(m)
                 : "r"(taddr));
    return m;
}

// 64 accumulator columns of this thread's TMEM lane together with their largest
// value: the .red form of tcgen05.ld reduces over the loaded columns on the way
// out of TMEM, so the filter's common case (nothing in the 64 columns passes)
// needs no max tree. Values and maximum are valid after tmem_wait_ld().
__device__ __forceinline__ float tmem_ld64_max_nowait(uint32_t taddr, float* v)
{
    float m;
    asm volatile("tcgen05.ld.red.sync.aligned.32x32b.x64.max.f32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, %64, [%65];"
                 : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7]), "=f"(v[8]), "=f"(v[9]), "=f"(v[10]), "=f"(v[11]), "=f"(v[12]), "=f"(v[13]), "=f"(v[14]), "=f"(v[15]), "=f"(v[16]), "=f"(v[17]), "=f"(v[18]), "=f"(v[19]), "=f"(v[20]), "=f"(v[21]), "=f"(v[22]), "=f"(v[23]), "=f"(v[24]), "=f"(v[25]), "=f"(v[26]), "=f"(v[27]), "=f"(v[28]), "=f"(v[29]), "=f"(v[30]), "=f"(v[31]), "=f"(v[32]), "=f"(v[33]), "=f"(v[34]), "=f"(v[35]), "=f"(v[36]), "=f"(v[37]), "=f"(v[38]), "=f"(v[39]), "=f"(v[40]), "=f"(v[41]), "=f"(v[42]), "=f"(v[43]), "=f"(v[44]), "=f"(v[45]), "=f"(v[46]), "=f"(v[47]), "=f"(v[48]), "=f"(v[49]), "=f"(v[50]), "=f"(v[51]), "=f"(v[52]), "=f"(v[53]), "=f"(v[54]), "=f"(v[55]), "=f"(v[56]), "=f"(v[57]), "=f"(v[58]), "=f"(v[59]), "=f"(v[60]), "=f"(v[61]), "=f"(v[62]), "=f"(v[63]), "=f"(m)
                 : "r"(taddr));
    return m;
}

__device__ __forceinline__ float fmax3(float a, float b, float c)
{
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// Branchless sorted insertion into a register list (ascending); an entry equal
// to v stays ahead of it. Slot s takes L[s-1] when v < L[s-1], v when
// L[s-1] <= v < L[s], and keeps L[s] otherwise: for the values that is
// min(L[s], max(v, L[s-1])), and each step's lower comparison is the next
// step's upper one.
template <int KC>
__device__ __forceinline__ void reg_insert(float (&L)[KC], int32_t (&I)[KC], float v, int32_t id)
{
    bool up = v < L[KC - 1];
#pragma unroll
    for (int s = KC - 1; s > 0; --s)
    {
        const bool lo = v < L[s - 1];
        I[s] = lo ? I[s - 1] : (up ? id : I[s]);
        L[s] = fminf(L[s], fmaxf(v, L[s - 1]));
        up = lo;
    }
    if (up)
    {
        L[0] = v;
        I[0] = id;
    }
}

struct TcBarriers
{
    uint64_t full[6], empty[6], tfull[2][2], tempty[2][2], afull, aempty, fin;  // t* : [buffer][query block]
    uint32_t tmem_base;
    int abort;
};

// One unit of screening work: QT query blocks starting at stacked row q0, against
// the ntiles candidate tiles of one problem, which start at stacked tile t0.
struct Item
{
    int64_t q0;
    int t0, ntiles;
    int64_t n;  // points of the problem (candidate ids >= n are padding)
    float s;    // scale exponent of the problem's fp16 split
};

// Work of one launch. Single problem: items == nullptr and CTA b owns the query
// rows [b QT 128, (b + 1) QT 128). Batch: a persistent grid walks the items
// (stacked row q0, first tile, tiles, problem) in steps of gridDim.x; every warp
// role walks the same sequence, so the pipeline phases stay in step.
struct ScreenWork
{
    const int4* items;
    int nitems;
    const int64_t* prob_n;
    const float* prob_scale;
};

template <int QROWS, bool BATCH>
__device__ __forceinline__ Item fetch_item(const ScreenWork& W, int j, int64_t N, int ntiles, const float* scale)
{
    Item it;
    if constexpr (!BATCH)
    {
        it.q0 = (int64_t)j * QROWS;
        it.t0 = 0;
        it.ntiles = ntiles;
        it.n = N;
        it.s = scale[0];
    }
    else
    {
        const int4 v = W.items[j];
        it.q0 = (int64_t)v.x * QROWS;
        it.t0 = v.y;
        it.ntiles = v.z;
        it.n = W.prob_n[v.w];
        it.s = W.prob_scale[v.w];
    }
    return it;
}

// Where a launch writes its KC-entry register list per row, for candidate lists
// longer than one such list: pass p of a multi-pass screen writes from entry off
// of rows of ld entries, and keeps only candidates that come after the previous
// passes' lists in the order (screened value, id). `lo` holds each row's last
// screened value of pass p - 1 (before the row norm is added); pass p takes
// t > lo, and t == lo only for ids that entries [0, off) do not hold. Every
// candidate with t < lo is in those entries already (a list that ends at lo
// rejected only values >= its last value at the time, which never rose), so the
// passes together hold the row's smallest screened values in order, and the last
// kept value bounds every candidate outside them. `last` (when set) receives each
// row's last screened value of this pass for the next one.
// Lists may also start full of each row's bound B = 1.01 T_r + 2 eps instead of
// empty (seed_tr = T_r, the row's k-th distance over the other rows of its
// 128-row block; rmax[0] = R; c1, c2 the screen's error model), as in the wide
// kernel: only candidates screened below B are inserted, and a list with fewer
// real entries ends in entries (B, -1). (A later pass runs only where a row needs
// more than one pass's entries, k + 8 > KC, so the k + 1 candidates below B have
// filled the earlier passes' lists.)
struct ListSlice
{
    int ld = 0, off = 0;          // row stride of the output lists and this pass's offset
    // entries written, [off, off + nw): a pass followed by another writes its KC;
    // the last pass writes to the row's end, the first min(KC, nw) of its list
    // (a sorted list cut short still bounds everything outside it by its last
    // kept value) and, past KC, entries (its last value, -1)
    int nw = 0;
    const float* lo = nullptr;    // previous pass's last values (off > 0)
    float* last = nullptr;        // this pass's last values (a later pass follows)
    const float* seed_tr = nullptr;
    const float* rmax = nullptr;
    float c1 = 0.f, c2 = 0.f;
    // near and far tiles (k_classify over 128-row blocks; null: every tile near):
    // far tiles get only the high-part product, and far_val (when set) receives
    // each row's smallest screened value over far tiles
    const uint32_t* near_bits = nullptr;
    int nwords = 0;
    float* far_val = nullptr;
};

__device__ __forceinline__ bool tile_is_near(const ListSlice& sl, int64_t blk, int tile)
{
    return !sl.near_bits || ((__ldg(sl.near_bits + blk * sl.nwords + (tile >> 5)) >> (tile & 31)) & 1u) != 0u;
}

// The row's starting list value in screened units t = |y|^2 - 2 x.y (FLT_MAX:
// no bound). T_r is an FP32 direct-difference sum over centred coordinates: its
// relative rounding (D + 2) 2^-24 is far inside the 1 %, and the centring error
// of a squared distance, at most 2^-22 d R, inside one eps. A neighbour among the
// k nearest screens at most e_k + eps < B, and so does the row itself.
__device__ __forceinline__ float seed_bound(const ListSlice& sl, int64_t q, float nq)
{
    if (!sl.seed_tr)
        return FLT_MAX;
    const float tb = sl.seed_tr[q];
    if (!(nq < FLT_MAX && tb < FLT_MAX))
        return FLT_MAX;
    const float R = sl.rmax[0];
    const float eps = sl.c1 * (nq + R * R) + sl.c2 * sqrtf(nq) * R;
    return fmaf(1.01f, tb, 2.f * eps) - nq;
}

// true when the row's entries [0, off) hold id: only for candidates whose
// screened value equals the previous pass's last value (exact float ties)
__device__ __noinline__ bool listed_before(const int32_t* row_ids, int off, int32_t id)
{
    for (int s = 0; s < off; ++s)
        if (row_ids[s] == id)
            return true;
    return false;
}

template <int DP, int KC, int QT, bool BATCH, bool LATER>
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_screen_tc(const __grid_constant__ CUtensorMap tm_hi, const __grid_constant__ CUtensorMap tm_lo,
                const __grid_constant__ CUtensorMap tm_nrm, const float* __restrict__ scale_log2, int64_t N,
                int64_t Npad, ScreenWork work, int32_t* __restrict__ cand_idx, float* __restrict__ cand_val,
                const float* __restrict__ nrm, ListSlice slice, unsigned* err)
{
    using C = TcCfg<DP, QT>;
    constexpr int QROWS = C::QT * TC_M;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // 1024-byte aligned operand region
    const uint32_t raw = smem_u32(smem_raw);
    const uint32_t base = (raw + 1023u) & ~1023u;
    unsigned char* gbase = smem_raw + (base - raw);
    const uint32_t A_s = base;
    const uint32_t B_s = base + C::A_BYTES;
    const uint32_t AX_s = base + (uint32_t)C::OFF_AX;
    TcBarriers& Bar = *reinterpret_cast<TcBarriers*>(gbase + C::OFF_BAR);
    volatile int* abort = &Bar.abort;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ntiles1 = (int)(Npad / TC_N);
    // single problem: exactly one item, this CTA's; batch: a strided walk
    const int j_first = (int)blockIdx.x;
    const int j_end = BATCH ? work.nitems : j_first + 1;
    const int j_step = BATCH ? (int)gridDim.x : 1;

    if (threadIdx.x == 0)
    {
        for (int s = 0; s < C::STAGES; ++s)
        {
            mbar_init(smem_u32(&Bar.full[s]), 1);
            mbar_init(smem_u32(&Bar.empty[s]), 1);
        }
        for (int b = 0; b < 2; ++b)
        {
            for (int qt = 0; qt < 2; ++qt)
            {
                mbar_init(smem_u32(&Bar.tfull[b][qt]), 1);
                mbar_init(smem_u32(&Bar.tempty[b][qt]), 4);  // the 4 epilogue warps of a query block
            }
        }
        mbar_init(smem_u32(&Bar.afull), 1);
        mbar_init(smem_u32(&Bar.aempty), 1);
        mbar_init(smem_u32(&Bar.fin), 1);
        Bar.abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // constant A slice of the norm step: 2^13 (fp16 0x7000) in every element, so its
    // swizzled layout is irrelevant
    for (int t = threadIdx.x; t < C::EXTRA_BYTES / 4; t += blockDim.x)
        reinterpret_cast<uint32_t*>(gbase + C::OFF_AX)[t] = 0x70007000u;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (warp == 9)
    {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&Bar.tmem_base)),
                     "r"(C::TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = Bar.tmem_base;

    if (warp == 8)
    {
        // ------------------------------------------------------------ producer
        if (lane == 0)
        {
            const uint32_t afull = smem_u32(&Bar.afull);
            int gi = 0;      // candidate tiles issued so far (all items)
            int na = 0;      // A loads issued
            bool ok = true;
            for (int j = j_first; ok && j < j_end; j += j_step)
            {
                const Item I = fetch_item<QROWS, BATCH>(work, j, N, ntiles1, scale_log2);
                // the previous item's MMAs must be done reading the A tiles
                if (na > 0 && !mbar_wait(smem_u32(&Bar.aempty), (uint32_t)(na - 1) & 1u, abort, err))
                    break;
                mbar_expect_tx(afull, C::A_BYTES);
                for (int qt = 0; qt < C::QT; ++qt)
                    for (int part = 0; part < 2; ++part)
                        for (int ka = 0; ka < C::KATOMS; ++ka)
                            tma_load_2d(A_s + ((qt * 2 + part) * C::KATOMS + ka) * C::ATOM_BYTES,
                                        part ? &tm_lo : &tm_hi, ka * 64, (int)(I.q0 + qt * TC_M), afull);
                ++na;
                ZigZag zz((int)(I.q0 / TC_N) - I.t0, I.ntiles);
                for (int it = 0; it < I.ntiles; ++it)
                {
                    const int tile = I.t0 + zz.next();
                    const int slot = gi % C::STAGES;
                    const uint32_t ph = (uint32_t)(gi / C::STAGES) & 1u;
                    if (!mbar_wait(smem_u32(&Bar.empty[slot]), ph ^ 1u, abort, err))
                    {
                        ok = false;
                        break;
                    }
                    const uint32_t fb = smem_u32(&Bar.full[slot]);
                    const uint32_t bst = B_s + slot * C::B_STAGE_BYTES;
                    mbar_expect_tx(fb, C::B_STAGE_BYTES);
                    for (int part = 0; part < 2; ++part)
                        for (int ka = 0; ka < C::KATOMS; ++ka)
                            tma_load_2d(bst + (part * C::KATOMS + ka) * C::ATOM_BYTES, part ? &tm_lo : &tm_hi,
                                        ka * 64, tile * TC_N, fb);
                    tma_load_2d(bst + C::B_OPER_BYTES, &tm_nrm, 0, tile * TC_N, fb);
                    ++gi;
                }
            }
            if (*abort)
            {
                // drain the loads still in flight (bounded)
                volatile int no_abort = 0;
                if (na > 0)
                    mbar_wait(afull, (uint32_t)(na - 1) & 1u, &no_abort, err);
                for (int g = (gi > C::STAGES ? gi - C::STAGES : 0); g < gi; ++g)
                    mbar_wait(smem_u32(&Bar.full[g % C::STAGES]), (uint32_t)(g / C::STAGES) & 1u, &no_abort, err);
            }
        }
    }
    else if (warp == 9)
    {
        // ------------------------------------------------------------ MMA issuer
        if (lane == 0)
        {
            int issued_any = 0;
            const uint64_t axd = umma_desc_sw32(AX_s);
            // descriptors of every A slice (constant) and of stage 0's B slices;
            // later stages add (stage offset >> 4) to the address field
            uint64_t adesc[C::QT][2][DP / 16];
#pragma unroll
            for (int qt = 0; qt < C::QT; ++qt)
#pragma unroll
                for (int part = 0; part < 2; ++part)
#pragma unroll
                    for (int kk = 0; kk < DP / 16; ++kk)
                        adesc[qt][part][kk] = umma_desc(A_s + ((qt * 2 + part) * C::KATOMS + (kk >> 2)) * C::ATOM_BYTES +
                                                        (uint32_t)(kk & 3) * 32u);
            uint64_t bdesc0[2][DP / 16];
#pragma unroll
            for (int part = 0; part < 2; ++part)
#pragma unroll
                for (int kk = 0; kk < DP / 16; ++kk)
                    bdesc0[part][kk] =
                        umma_desc(B_s + (part * C::KATOMS + (kk >> 2)) * C::ATOM_BYTES + (uint32_t)(kk & 3) * 32u);
            const uint64_t bx0 = umma_desc_sw32(B_s + C::B_OPER_BYTES);
            int gi = 0, na = 0;
            bool ok = true;
            for (int j = j_first; ok && j < j_end; j += j_step)
            {
                const Item I = fetch_item<QROWS, BATCH>(work, j, N, ntiles1, scale_log2);
                if (!mbar_wait(smem_u32(&Bar.afull), (uint32_t)na & 1u, abort, err))
                    break;
                ++na;
                tc_fence_after();
                ZigZag zz((int)(I.q0 / TC_N) - I.t0, I.ntiles);
                for (int it = 0; it < I.ntiles; ++it)
                {
                    const int tile = zz.next();  // local to the problem
                    const int slot = gi % C::STAGES;
                    const uint32_t ph = (uint32_t)(gi / C::STAGES) & 1u;
                    const int buf = gi & 1;
                    const uint32_t bph = (uint32_t)(gi >> 1) & 1u;
                    if (!mbar_wait(smem_u32(&Bar.full[slot]), ph, abort, err))
                    {
                        ok = false;
                        break;
                    }
                    const uint64_t soff = (uint64_t)((slot * C::B_STAGE_BYTES) >> 4);
                    // each query block's accumulator half has its own handoff, so its
                    // epilogue warps start as soon as its 13 MMAs are done
#pragma unroll
                    for (int qt = 0; qt < C::QT; ++qt)
                    {
                        if (!mbar_wait(smem_u32(&Bar.tempty[buf][qt]), bph ^ 1u, abort, err))
                        {
                            ok = false;
                            break;
                        }
                        tc_fence_after();
                        const uint32_t d = tmem + (uint32_t)(buf * C::ACC_COLS + qt * TC_N);
                        // norm step first: D = 2^13 (h + l) of -|2^s y|^2 / 2^14
                        umma_f16(d, axd, bx0 + soff, 0u);
                        // far tiles: the high-part product only
                        const int nprod = (BATCH || tile_is_near(slice, I.q0 / TC_M + qt, tile)) ? 3 : 1;
#pragma unroll
                        for (int prod = 0; prod < 3; ++prod)
                        {
                            if (prod >= nprod)
                                break;
                            const int apart = (prod == 2) ? 1 : 0;  // l_x . h_y
                            const int bpart = (prod == 1) ? 1 : 0;  // h_x . l_y
#pragma unroll
                            for (int kk = 0; kk < DP / 16; ++kk)
                                umma_f16(d, adesc[qt][apart][kk], bdesc0[bpart][kk] + soff, 1u);
                        }
                        umma_commit(smem_u32(&Bar.tfull[buf][qt]));
                        issued_any = 1;
                    }
                    if (!ok)
                        break;
                    umma_commit(smem_u32(&Bar.empty[slot]));
                    ++gi;
                }
                // the A tiles are free once this item's MMAs complete
                if (ok)
                    umma_commit(smem_u32(&Bar.aempty));
            }
            if (issued_any)
            {
                // every MMA this thread issued (and its barrier arrivals) completes
                // before TMEM is freed and the CTA's shared memory is released
                volatile int no_abort = 0;
                umma_commit(smem_u32(&Bar.fin));
                mbar_wait(smem_u32(&Bar.fin), 0u, &no_abort, err);
            }
        }
    }
    else if (warp < C::EPI_WARPS)
    {
        // ------------------------------------------------------------ epilogue
        const int quad = warp & 3;
        const int qt = warp >> 2;
        const int row = quad * 32 + lane;
        int gi = 0;
        bool alive = true;
        for (int j = j_first; alive && j < j_end; j += j_step)
        {
            const Item I = fetch_item<QROWS, BATCH>(work, j, N, ntiles1, scale_log2);
            const int64_t q = I.q0 + qt * TC_M + row;
            const float nq = nrm[q];
            // pass p > 0 of a long list: only candidates after the previous passes'
            const float lo = LATER ? slice.lo[q] : 0.f;
            // |y|^2 - 2 x.y = m2 * acc, m2 = -2^(1-2s) (exact power of two)
            const float m2 = -exp2f(1.0f - 2.0f * I.s);
            const float inv_m2 = 1.0f / m2;
            float cmp = BATCH ? FLT_MAX : seed_bound(slice, q, nq);
            float L[KC];
            int32_t Ix[KC];
#pragma unroll
            for (int s = 0; s < KC; ++s)
            {
                L[s] = cmp;
                Ix[s] = -1;
            }
            // without a bound: accept everything until the list fills
            float thr = (cmp < FLT_MAX) ? cmp * inv_m2 : -__int_as_float(0x7f800000);
            const float thr_lo = lo * inv_m2;
            float far_max = -__int_as_float(0x7f800000);  // largest accumulator over far tiles
            const int64_t blk = I.q0 / TC_M + qt;
            ZigZag zz((int)(I.q0 / TC_N) - I.t0, I.ntiles);
            for (int it = 0; it < I.ntiles; ++it)
            {
                const int tile = zz.next();  // local to the problem
                const bool far_tile = !BATCH && !tile_is_near(slice, blk, tile);
                const int buf = gi & 1;
                const uint32_t bph = (uint32_t)(gi >> 1) & 1u;
                ++gi;
                // tcgen05.ld is warp-collective: leave the loop as a whole warp
                const bool ok = mbar_wait(smem_u32(&Bar.tfull[buf][qt]), bph, abort, err);
                if (!__all_sync(0xffffffffu, ok))
                {
                    alive = false;
                    break;
                }
                tc_fence_after();
                const int64_t c0 = (int64_t)tile * TC_N;
                const uint32_t tacc = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(buf * C::ACC_COLS + qt * TC_N);
                // columns per TMEM wait: 64 with 32-entry lists, 32 with 64-entry lists
                constexpr int CPW = (KC <= 32) ? 64 : 32;
#pragma unroll 1
                for (int h = 0; h < TC_N / CPW; ++h)
                {
                    // the round's columns and their largest value from one reducing
                    // TMEM load: one branch per round when nothing passes
                    float v[CPW];
                    float gall;
                    if constexpr (CPW == 64)
                        gall = tmem_ld64_max_nowait(tacc + h * CPW, v);
                    else
                        gall = tmem_ld32_max_nowait(tacc + h * CPW, v);
                    tmem_wait_ld();
                    if (h == TC_N / CPW - 1)
                    {
                        // the last columns are in registers: hand the buffer back now
                        tc_fence_before();
                        __syncwarp();
                        if (lane == 0)
                            mbar_arrive(smem_u32(&Bar.tempty[buf][qt]));
                    }
                    if (far_tile)
                    {
                        // padding columns must not enter far_max
                        const int64_t cf = c0 + h * CPW;
                        if (cf + CPW <= I.n)
                            far_max = fmaxf(far_max, gall);
                        else
                        {
#pragma unroll
                            for (int e = 0; e < CPW; ++e)
                                if (cf + e < I.n)
                                    far_max = fmaxf(far_max, v[e]);
                        }
                    }
                    constexpr int NG = CPW / 8;
                    if (gall > thr)
                    {
#pragma unroll
                        for (int g = 0; g < NG; ++g)
                        {
                            const float* w = v + g * 8;
                            if (fmax3(fmax3(w[0], w[1], w[2]), fmax3(w[3], w[4], w[5]), fmaxf(w[6], w[7])) > thr)
                            {
                                // columns of the group that pass, then one insertion each; a
                                // later pass drops the previous passes' entries (t < lo, i.e.
                                // x > lo / m2, exact as m2 is a power of two) here already
                                unsigned msk = 0u;
#pragma unroll
                                for (int e = 0; e < 8; ++e)
                                    msk |= (w[e] > thr && (!LATER || w[e] <= thr_lo)) ? (1u << e) : 0u;
                                const int64_t cb = c0 + h * CPW + g * 8;
#pragma unroll 1
                                while (msk)
                                {
                                    const int e = __ffs(msk) - 1;
                                    msk &= msk - 1u;
                                    float x = w[0];
#pragma unroll
                                    for (int e2 = 1; e2 < 8; ++e2)
                                        x = (e == e2) ? w[e2] : x;
                                    const float t = m2 * x;
                                    if (t < cmp && cb + e < I.n &&
                                        (!LATER || t > lo ||
                                         (t == lo &&
                                          !listed_before(cand_idx + q * slice.ld, slice.off, (int32_t)(cb + e)))))
                                    {
                                        reg_insert<KC>(L, Ix, t, (int32_t)(cb + e));
                                        cmp = L[KC - 1];
                                        thr = cmp * inv_m2;
                                    }
                                }
                            }
                        }
                    }
                }
            }
            if (!alive)
                break;
            const int64_t o = q * slice.ld + slice.off;
            const int nw = slice.nw;
#pragma unroll
            for (int s = 0; s < KC; ++s)
                if (s < nw)
                {
                    cand_idx[o + s] = Ix[s];
                    cand_val[o + s] = (L[s] < FLT_MAX) ? L[s] + nq : FLT_MAX;
                }
            for (int s = KC; s < nw; ++s)
            {
                cand_idx[o + s] = -1;
                cand_val[o + s] = (L[KC - 1] < FLT_MAX) ? L[KC - 1] + nq : FLT_MAX;
            }
            if (!BATCH && slice.last)
                slice.last[q] = L[KC - 1];
            // smallest screened value over far tiles (high-part products only)
            if (!BATCH && slice.far_val)
                slice.far_val[q] = (far_max > -FLT_MAX) ? m2 * far_max + nq : FLT_MAX;
        }
    }

    tc_fence_before();
    __syncthreads();
    if (warp == 9)
    {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(C::TMEM_COLS));
    }
}

// ---------------------------------------------------------------------------
// Wide screen for padded dimension 64 and 32-entry lists: one CTA per block of
// 128 queries, candidate tiles of 256 rows, tcgen05.mma with N = 256 (half the
// instructions of two N = 128 MMAs and half the shared-memory reads of the A
// operand per output), two 256-column accumulators double-buffered in TMEM.
// The epilogue splits each tile's 256 columns between warps 0-3 (columns
// 0-127) and warps 4-7 (128-255), reading 64 columns per TMEM load with the
// load's own max reduction as the pass filter; each keeps its own top-32 per row, and the
// two lists of a row are merged before they are written. Both half lists hold
// their half's 32 smallest values, so the merged list is the top 32 of the
// union and its last value bounds every candidate outside it, as the
// certification needs.
// Near and far tiles: tiles whose bounding sphere is close to the query block's
// (k_classify) get the full 3-product split; the others only h_x . h_y (5 MMAs
// instead of 13, and no low-part loads). The epilogue records, per row, the
// smallest screened value over far tiles (far_val), which the re-rank certifies
// against with the larger error bound of high-part products.
constexpr int TW_N = 256;
constexpr int TW_KC = 32;
// warps 0-7 epilogue, 8 producer of the high ring, 9 MMA issuer, 10 producer of
// the low ring
constexpr int TW_THREADS = 352;
constexpr uint32_t IDESC_W = (1u << 4) | ((uint32_t)(TW_N >> 3) << 17) | ((uint32_t)(TC_M >> 4) << 24);

struct TwCfg
{
    static constexpr int A_ATOM = 128 * 128;                 // 128 rows x 128 B
    static constexpr int B_ATOM = TW_N * 128;                // 256 rows x 128 B
    static constexpr int A_BYTES = 2 * A_ATOM;               // hi + lo
    static constexpr int AX_BYTES = 128 * 32;                // constant norm slice of A
    static constexpr int BX_BYTES = TW_N * 32;               // norm column slice of B
    // two rings: every tile's high parts and norm column (3 deep), and the low
    // parts that only near tiles load (2 deep)
    static constexpr int B_STAGE = B_ATOM + BX_BYTES;        // 40 KB: high parts + norm column
    static constexpr int STAGES = 3;
    static constexpr int L_STAGE = B_ATOM;                   // 32 KB: low parts
    static constexpr int L_STAGES = 2;
    static constexpr int MERGE_BYTES = 4 * TW_KC * 32 * 8;   // warps 4-7 lists: value + id
    static constexpr int NB_WORDS = 512;                     // near bits staged in shared memory
    static constexpr size_t OFF_B = A_BYTES;
    static constexpr size_t OFF_L = OFF_B + (size_t)STAGES * B_STAGE;
    static constexpr size_t OFF_AX = OFF_L + (size_t)L_STAGES * L_STAGE;
    static constexpr size_t OFF_BAR = OFF_AX + AX_BYTES;
    // the half-list merge runs after the last tile's MMAs: it reuses the high ring
    static constexpr size_t OFF_MERGE = OFF_B;
    static constexpr size_t OFF_FAR = OFF_BAR + 256;
    static constexpr size_t OFF_NB = OFF_FAR + 128 * 4;
    static_assert(MERGE_BYTES <= STAGES * B_STAGE, "merge buffer inside the high ring");
    static constexpr size_t SMEM = OFF_NB + (size_t)NB_WORDS * 4 + 1024;
    static_assert(SMEM <= 227 * 1024, "shared memory budget");
};

struct TwBarriers
{
    uint64_t full[TwCfg::STAGES], empty[TwCfg::STAGES], lfull[TwCfg::L_STAGES], lempty[TwCfg::L_STAGES];
    uint64_t tfull[2], tempty[2], afull, fin;
    uint32_t tmem_base;
    int abort;
};

__device__ __forceinline__ void umma_f16_w(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate)
{
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            dtmem),
        "l"(adesc), "l"(bdesc), "r"(IDESC_W), "r"(accumulate));
}

__global__ void __launch_bounds__(TW_THREADS, 1)
    k_screen_tc_wide(const __grid_constant__ CUtensorMap tmA_hi, const __grid_constant__ CUtensorMap tmA_lo,
                     const __grid_constant__ CUtensorMap tmB_hi, const __grid_constant__ CUtensorMap tmB_lo,
                     const __grid_constant__ CUtensorMap tm_nrm, const float* __restrict__ scale_log2, int64_t N,
                     int64_t Npad, const uint32_t* __restrict__ near_bits, int nwords,
                     int32_t* __restrict__ cand_idx, float* __restrict__ cand_val, float* __restrict__ far_val,
                     const float* __restrict__ nrm, int full_blocks, int parts, int32_t* __restrict__ part_idx,
                     float* __restrict__ part_val, float* __restrict__ part_far, const float* __restrict__ Trow,
                     const float* __restrict__ rmax, float c1, float c2, unsigned* err)
{
    using C = TwCfg;
    constexpr int KC = TW_KC;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    const uint32_t raw = smem_u32(smem_raw);
    const uint32_t base = (raw + 1023u) & ~1023u;
    unsigned char* gbase = smem_raw + (base - raw);
    const uint32_t A_s = base;
    const uint32_t B_s = base + (uint32_t)C::OFF_B;
    const uint32_t L_s = base + (uint32_t)C::OFF_L;
    const uint32_t AX_s = base + (uint32_t)C::OFF_AX;
    TwBarriers& Bar = *reinterpret_cast<TwBarriers*>(gbase + C::OFF_BAR);
    float* merge_v = reinterpret_cast<float*>(gbase + C::OFF_MERGE);
    int32_t* merge_i = reinterpret_cast<int32_t*>(gbase + C::OFF_MERGE + C::MERGE_BYTES / 2);
    float* merge_far = reinterpret_cast<float*>(gbase + C::OFF_FAR);
    volatile int* abort = &Bar.abort;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ntiles = (int)(Npad / TW_N);
    // Work item: CTAs below full_blocks take their whole query block; the blocks
    // after them (the last, partial wave) are split into `parts` items over
    // consecutive stretches of the block's tile order, whose lists k_merge_parts
    // combines.
    int blk = (int)blockIdx.x, part = 0, nparts = 1;
    if (blk >= full_blocks)
    {
        const int e = blk - full_blocks;
        blk = full_blocks + e / parts;
        part = e % parts;
        nparts = parts;
    }
    const int it0 = (int)((int64_t)ntiles * part / nparts);
    const int nit = (int)((int64_t)ntiles * (part + 1) / nparts) - it0;
    const int64_t q0 = (int64_t)blk * TC_M;
    // near (full fp16 split) or far (high parts only) pair of this query block and
    // a tile; the block's bits are staged in shared memory when they fit
    const uint32_t* nb_row = near_bits + (int64_t)blk * nwords;
    uint32_t* nb_s = reinterpret_cast<uint32_t*>(gbase + C::OFF_NB);
    const bool nb_staged = nwords <= C::NB_WORDS;
    if (nb_staged)
        for (int t = threadIdx.x; t < nwords; t += blockDim.x)
            nb_s[t] = __ldg(nb_row + t);
    const uint32_t* nb = nb_staged ? nb_s : nb_row;
    auto is_near = [&](int tile) { return ((nb[tile >> 5] >> (tile & 31)) & 1u) != 0u; };

    if (threadIdx.x == 0)
    {
        for (int st = 0; st < C::STAGES; ++st)
        {
            mbar_init(smem_u32(&Bar.full[st]), 1);
            mbar_init(smem_u32(&Bar.empty[st]), 1);
        }
        for (int st = 0; st < C::L_STAGES; ++st)
        {
            mbar_init(smem_u32(&Bar.lfull[st]), 1);
            mbar_init(smem_u32(&Bar.lempty[st]), 1);
        }
        for (int b = 0; b < 2; ++b)
        {
            mbar_init(smem_u32(&Bar.tfull[b]), 1);
            mbar_init(smem_u32(&Bar.tempty[b]), 8);  // all 8 epilogue warps read each buffer
        }
        mbar_init(smem_u32(&Bar.afull), 1);
        mbar_init(smem_u32(&Bar.fin), 1);
        Bar.abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int t = threadIdx.x; t < C::AX_BYTES / 4; t += blockDim.x)
        reinterpret_cast<uint32_t*>(gbase + C::OFF_AX)[t] = 0x70007000u;  // 2^13 everywhere
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (warp == 9)
    {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&Bar.tmem_base)),
                     "r"(512));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = Bar.tmem_base;

    if (warp == 8)
    {
        // ------------------------------------------------------------ producer
        if (lane == 0)
        {
            const uint32_t afull = smem_u32(&Bar.afull);
            mbar_expect_tx(afull, C::A_BYTES);
            tma_load_2d(A_s, &tmA_hi, 0, (int)q0, afull);
            tma_load_2d(A_s + C::A_ATOM, &tmA_lo, 0, (int)q0, afull);
            ZigZag zz((int)(q0 / TW_N), ntiles);
            for (int s = 0; s < it0; ++s)
                zz.next();
            int issued = 0;  // loads issued into the high ring
            for (int it = 0; it < nit; ++it)
            {
                const int tile = zz.next();
                const int slot = it % C::STAGES;
                const uint32_t ph = (uint32_t)(it / C::STAGES) & 1u;
                if (!mbar_wait(smem_u32(&Bar.empty[slot]), ph ^ 1u, abort, err))
                    break;
                const uint32_t fb = smem_u32(&Bar.full[slot]);
                const uint32_t bst = B_s + slot * C::B_STAGE;
                mbar_expect_tx(fb, (uint32_t)C::B_STAGE);
                tma_load_2d(bst, &tmB_hi, 0, tile * TW_N, fb);
                tma_load_2d(bst + C::B_ATOM, &tm_nrm, 0, tile * TW_N, fb);
                issued = it + 1;
            }
            if (*abort)
            {
                volatile int no_abort = 0;
                mbar_wait(afull, 0u, &no_abort, err);
                for (int g = (issued > C::STAGES ? issued - C::STAGES : 0); g < issued; ++g)
                    mbar_wait(smem_u32(&Bar.full[g % C::STAGES]), (uint32_t)(g / C::STAGES) & 1u, &no_abort, err);
            }
        }
    }
    else if (warp == 10)
    {
        // ------------------------------------------------------------ producer of the low ring
        // (near tiles only), so that runs of near tiles do not hold back the
        // high-part loads of the far tiles behind them
        if (lane == 0)
        {
            ZigZag zz((int)(q0 / TW_N), ntiles);
            for (int s = 0; s < it0; ++s)
                zz.next();
            int lissued = 0;
            for (int it = 0; it < nit; ++it)
            {
                const int tile = zz.next();
                if (!is_near(tile))
                    continue;
                const int ls = lissued % C::L_STAGES;
                const uint32_t lph = (uint32_t)(lissued / C::L_STAGES) & 1u;
                if (!mbar_wait(smem_u32(&Bar.lempty[ls]), lph ^ 1u, abort, err))
                    break;
                const uint32_t lb = smem_u32(&Bar.lfull[ls]);
                mbar_expect_tx(lb, (uint32_t)C::L_STAGE);
                tma_load_2d(L_s + ls * C::L_STAGE, &tmB_lo, 0, tile * TW_N, lb);
                ++lissued;
            }
            if (*abort)
            {
                volatile int no_abort = 0;
                for (int g = (lissued > C::L_STAGES ? lissued - C::L_STAGES : 0); g < lissued; ++g)
                    mbar_wait(smem_u32(&Bar.lfull[g % C::L_STAGES]), (uint32_t)(g / C::L_STAGES) & 1u, &no_abort,
                              err);
            }
        }
    }
    else if (warp == 9)
    {
        // ------------------------------------------------------------ MMA issuer
        if (lane == 0)
        {
            bool ok = mbar_wait(smem_u32(&Bar.afull), 0u, abort, err);
            tc_fence_after();
            int issued_any = 0;
            const uint64_t axd = umma_desc_sw32(AX_s);
            uint64_t adesc[2][4], bdh[4], bdl[4];
#pragma unroll
            for (int part = 0; part < 2; ++part)
#pragma unroll
                for (int kk = 0; kk < 4; ++kk)
                    adesc[part][kk] = umma_desc(A_s + part * C::A_ATOM + (uint32_t)kk * 32u);
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
            {
                bdh[kk] = umma_desc(B_s + (uint32_t)kk * 32u);  // high ring, slot 0
                bdl[kk] = umma_desc(L_s + (uint32_t)kk * 32u);  // low ring, slot 0
            }
            const uint64_t bx0 = umma_desc_sw32(B_s + C::B_ATOM);
            ZigZag zz((int)(q0 / TW_N), ntiles);
            for (int s = 0; s < it0; ++s)
                zz.next();
            int lc = 0;  // near tiles consumed (low-ring position)
            for (int it = 0; ok && it < nit; ++it)
            {
                const bool nr = is_near(zz.next());
                const int slot = it % C::STAGES;
                const uint32_t ph = (uint32_t)(it / C::STAGES) & 1u;
                const int buf = it & 1;
                const uint32_t bph = (uint32_t)(it >> 1) & 1u;
                const int ls = lc % C::L_STAGES;
                if (!mbar_wait(smem_u32(&Bar.full[slot]), ph, abort, err))
                    break;
                if (nr && !mbar_wait(smem_u32(&Bar.lfull[ls]), (uint32_t)(lc / C::L_STAGES) & 1u, abort, err))
                    break;
                if (!mbar_wait(smem_u32(&Bar.tempty[buf]), bph ^ 1u, abort, err))
                    break;
                tc_fence_after();
                const uint64_t soff = (uint64_t)((slot * C::B_STAGE) >> 4);
                const uint64_t loff = (uint64_t)((ls * C::L_STAGE) >> 4);
                const uint32_t d = tmem + (uint32_t)(buf * TW_N);
                umma_f16_w(d, axd, bx0 + soff, 0u);  // -|2^s y|^2 / 2 in every row
#pragma unroll
                for (int kk = 0; kk < 4; ++kk)
                    umma_f16_w(d, adesc[0][kk], bdh[kk] + soff, 1u);  // h_x . h_y
                if (nr)
                {
#pragma unroll
                    for (int kk = 0; kk < 4; ++kk)
                        umma_f16_w(d, adesc[0][kk], bdl[kk] + loff, 1u);  // h_x . l_y
#pragma unroll
                    for (int kk = 0; kk < 4; ++kk)
                        umma_f16_w(d, adesc[1][kk], bdh[kk] + soff, 1u);  // l_x . h_y
                }
                umma_commit(smem_u32(&Bar.tfull[buf]));
                umma_commit(smem_u32(&Bar.empty[slot]));
                if (nr)
                {
                    umma_commit(smem_u32(&Bar.lempty[ls]));
                    ++lc;
                }
                issued_any = 1;
            }
            if (issued_any)
            {
                volatile int no_abort = 0;
                umma_commit(smem_u32(&Bar.fin));
                mbar_wait(smem_u32(&Bar.fin), 0u, &no_abort, err);
            }
        }
    }
    else
    {
        // ------------------------------------------------------------ epilogue
        const int quad = warp & 3;
        const int half = warp >> 2;
        const int row = quad * 32 + lane;
        const int64_t q = q0 + row;
        const float m2 = -exp2f(1.0f - 2.0f * scale_log2[0]);  // a power of two: thr below is exact
        const float inv_m2 = 1.0f / m2;
        // The list starts full of a bound instead of empty: B = 1.01 T_r + 2 eps
        // (T_r bounds this row's k-th neighbour distance, eps is the row's screen
        // error), so only candidates screened below it are inserted. T_r is an
        // FP32 direct-difference sum over centred coordinates: its relative
        // rounding (D + 2) 2^-24 is far inside the 1 %, and the centring error
        // of a squared distance, at most 2^-22 d R, inside one eps (>= c1 R^2 with
        // c1 >= 16 2^-24, and d <= 2 R). A neighbour y of the k nearest so screens
        // at most e_k + eps < B. The k nearest
        // other points and the row itself screen below B, so at least k + 1 real
        // entries survive. A point never inserted has a screened value >= B, and
        // the list's last value is min(B, the 32nd screened value), so the
        // re-rank's certification against the last value covers it as before.
        // B spares every insert of a candidate that cannot be among the k nearest;
        // a list that keeps fewer than 32 real entries ends in entries (B, -1).
        float cmp = FLT_MAX;
        {
            const float nq0 = nrm[q];
            const float tb = Trow[q];
            if (nq0 < FLT_MAX && tb < FLT_MAX)
            {
                const float R = rmax[0];
                const float eps = c1 * (nq0 + R * R) + c2 * sqrtf(nq0) * R;
                cmp = fmaf(1.01f, tb, 2.f * eps) - nq0;
            }
        }
        float L[KC];
        int32_t Ix[KC];
#pragma unroll
        for (int s = 0; s < KC; ++s)
        {
            L[s] = cmp;
            Ix[s] = -1;
        }
        float thr = (cmp < FLT_MAX) ? cmp * inv_m2 : -__int_as_float(0x7f800000);
        float far_max = -__int_as_float(0x7f800000);  // largest accumulator over far tiles
        ZigZag zz((int)(q0 / TW_N), ntiles);
        for (int s = 0; s < it0; ++s)
            zz.next();
        bool alive = true;
        for (int it = 0; it < nit; ++it)
        {
            const int tile = zz.next();
            const int buf = it & 1;
            const uint32_t bph = (uint32_t)(it >> 1) & 1u;
            const bool ok = mbar_wait(smem_u32(&Bar.tfull[buf]), bph, abort, err);
            if (!__all_sync(0xffffffffu, ok))
            {
                alive = false;
                break;
            }
            tc_fence_after();
            const int64_t c0 = (int64_t)tile * TW_N + half * 128;
            const uint32_t tacc = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(buf * TW_N + half * 128);
            const bool far_tile = !is_near(tile);
            const bool ragged = c0 + 128 > N;  // padding columns must not enter far_max
#pragma unroll 1
            for (int h = 0; h < 2; ++h)
            {
                float v[64];
                // the 64 columns and their largest value, from one TMEM load:
                // one branch per 64 columns in the common case (nothing passes)
                const float g64 = tmem_ld64_max_nowait(tacc + h * 64, v);
                tmem_wait_ld();
                if (h == 1)
                {
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0)
                        mbar_arrive(smem_u32(&Bar.tempty[buf]));
                }
                if (far_tile)
                {
                    if (!ragged)
                        far_max = fmaxf(far_max, g64);
                    else
                    {
#pragma unroll
                        for (int e = 0; e < 64; ++e)
                            if (c0 + h * 64 + e < N)
                                far_max = fmaxf(far_max, v[e]);
                    }
                }
                if (g64 > thr)
                {
#pragma unroll
                    for (int g = 0; g < 8; ++g)
                    {
                        const float* w = v + g * 8;
                        if (fmax3(fmax3(w[0], w[1], w[2]), fmax3(w[3], w[4], w[5]), fmaxf(w[6], w[7])) > thr)
                        {
                            // columns of the group that pass, then one insertion each
                            unsigned msk = 0u;
#pragma unroll
                            for (int e = 0; e < 8; ++e)
                                msk |= (w[e] > thr) ? (1u << e) : 0u;
                            const int64_t cb = c0 + h * 64 + g * 8;
#pragma unroll 1
                            while (msk)
                            {
                                const int e = __ffs(msk) - 1;
                                msk &= msk - 1u;
                                float x = w[0];
#pragma unroll
                                for (int e2 = 1; e2 < 8; ++e2)
                                    x = (e == e2) ? w[e2] : x;
                                const float t = m2 * x;
                                if (t < cmp && cb + e < N)
                                {
                                    reg_insert<KC>(L, Ix, t, (int32_t)(cb + e));
                                    cmp = L[KC - 1];
                                    thr = cmp * inv_m2;
                                }
                            }
                        }
                    }
                }
            }
        }
        // merge the two half lists of each row (named barrier of the 8 epilogue warps)
        if (half == 1)
        {
#pragma unroll
            for (int s = 0; s < KC; ++s)
            {
                merge_v[(quad * KC + s) * 32 + lane] = L[s];
                merge_i[(quad * KC + s) * 32 + lane] = Ix[s];
            }
            merge_far[row] = far_max;
        }
        asm volatile("bar.sync 1, 256;" ::: "memory");
        if (half == 0 && __all_sync(0xffffffffu, alive))
        {
#pragma unroll 1
            for (int s = 0; s < KC; ++s)
            {
                const float t = merge_v[(quad * KC + s) * 32 + lane];
                if (t < cmp)  // the other list is sorted: later entries are no smaller
                {
                    reg_insert<KC>(L, Ix, t, merge_i[(quad * KC + s) * 32 + lane]);
                    cmp = L[KC - 1];
                }
            }
            const float nq = nrm[q];
            // a whole block writes its rows' lists; a part writes its own slot
            const int64_t pr = (nparts == 1) ? -1 : ((int64_t)(blk - full_blocks) * TC_M + row) * nparts + part;
            int32_t* oi = (nparts == 1) ? cand_idx + q * KC : part_idx + pr * KC;
            float* ov = (nparts == 1) ? cand_val + q * KC : part_val + pr * KC;
#pragma unroll
            for (int s = 0; s < KC; ++s)
            {
                oi[s] = Ix[s];
                ov[s] = (L[s] < FLT_MAX) ? L[s] + nq : FLT_MAX;
            }
            // smallest screened value over far tiles (high-part products only)
            const float fm = fmaxf(far_max, merge_far[row]);
            const float fv = (fm > -FLT_MAX) ? m2 * fm + nq : FLT_MAX;
            if (nparts == 1)
                far_val[q] = fv;
            else
                part_far[pr] = fv;
        }
    }

    tc_fence_before();
    __syncthreads();
    if (warp == 9)
    {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
    }
}

// Bounding sphere (centre, radius) of every block of ROWS sorted rows of xc
// (valid rows only; radius -1 for a block without valid rows). One CTA per block.
template <int ROWS>
__global__ void __launch_bounds__(256) k_spheres(const float* __restrict__ xc, int64_t N, int Dp, float* ctr,
                                                 float* rad, float* ctrT)
{
    __shared__ float part[256];
    __shared__ float c_s[128];
    __shared__ float wmax[8];
    const int64_t r0 = (int64_t)blockIdx.x * ROWS;
    const int nvalid = (int)max((int64_t)0, min((int64_t)ROWS, N - r0));
    const int t = threadIdx.x;
    // centre: thread t sums dimension t % Dp over rows t / Dp, + 256 / Dp, ...
    const int per = 256 / Dp;
    float sacc = 0.f;
    if (t < per * Dp)
        for (int r = t / Dp; r < nvalid; r += per)
            sacc += xc[(r0 + r) * Dp + t % Dp];
    part[t] = sacc;
    __syncthreads();
    if (t < Dp)
    {
        float tot = 0.f;
        for (int q = 0; q < per; ++q)
            tot += part[q * Dp + t];
        c_s[t] = nvalid > 0 ? tot / (float)nvalid : 0.f;
        ctr[(int64_t)blockIdx.x * Dp + t] = c_s[t];
        if (ctrT)
            ctrT[(int64_t)t * gridDim.x + blockIdx.x] = c_s[t];  // dimension-major copy
    }
    __syncthreads();
    const int lane = t & 31, w = t >> 5;
    float rmax2 = 0.f;
    for (int r = w; r < nvalid; r += 8)
    {
        float d2 = 0.f;
        for (int d = lane; d < Dp; d += 32)
        {
            const float z = xc[(r0 + r) * Dp + d] - c_s[d];
            d2 = fmaf(z, z, d2);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            d2 += __shfl_xor_sync(0xffffffffu, d2, o);
        rmax2 = fmaxf(rmax2, d2);
    }
    if (lane == 0)
        wmax[w] = rmax2;
    __syncthreads();
    if (t == 0)
    {
        float m = 0.f;
        for (int q = 0; q < 8; ++q)
            m = fmaxf(m, wmax[q]);
        // FP32 rounding of the centre and of the squares: widen by a relative 1e-5
        rad[blockIdx.x] = nvalid > 0 ? sqrtf(m) * 1.00001f + 1e-6f : -1.f;
    }
}

// Combines the partial lists of the split blocks: per row, the 32 smallest of
// the parts' sorted lists (ties to the earlier part, so the result does not
// depend on timing) and the smallest far value. One thread per row.
__global__ void k_merge_parts(int64_t row0, int64_t rows, int parts, const int32_t* __restrict__ part_idx,
                              const float* __restrict__ part_val, const float* __restrict__ part_far,
                              int32_t* cand_idx, float* cand_val, float* far_val)
{
    constexpr int KC = TW_KC;
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows)
        return;
    int head[8];
    float hv[8];
    float fv = FLT_MAX;
#pragma unroll
    for (int p = 0; p < 8; ++p)
    {
        head[p] = 0;
        hv[p] = (p < parts) ? part_val[(r * parts + p) * KC] : FLT_MAX;
        if (p < parts)
            fv = fminf(fv, part_far[r * parts + p]);
    }
    const int64_t q = row0 + r;
    for (int s = 0; s < KC; ++s)
    {
        int best = 0;
        float bv = hv[0];
#pragma unroll
        for (int p = 1; p < 8; ++p)
            if (hv[p] < bv)
            {
                bv = hv[p];
                best = p;
            }
        int bh = 0;
#pragma unroll
        for (int p = 0; p < 8; ++p)
            if (p == best)
                bh = head[p];
        cand_idx[q * KC + s] = (bv < FLT_MAX) ? part_idx[(r * parts + best) * KC + bh] : -1;
        cand_val[q * KC + s] = bv;
#pragma unroll
        for (int p = 0; p < 8; ++p)
            if (p == best)
            {
                head[p] = bh + 1;
                hv[p] = (bh + 1 < KC) ? part_val[(r * parts + p) * KC + bh + 1] : FLT_MAX;
            }
    }
    far_val[q] = fv;
}

// Upper bounds of the k-th neighbour distance, from the rows of each 128-row
// block: Tr gets each row's k-th smallest squared distance to the other valid
// rows of its block (direct FP32 differences; +inf for padding rows and when the
// block has at most k valid rows), Tb the largest of them over the block. The
// block's rows are a subset of all points, so each row's true k-th neighbour
// distance e_k is at most its Tr. Tr seeds the row's candidate list in the
// screen, Tb decides near and far tiles. One CTA per block, one thread per row;
// all threads read the same row c at a time (shared-memory broadcast), and
// the KB smallest distances stay sorted in registers (KB >= k), kept by a
// min/max network.
template <int DP, int KB>
__global__ void __launch_bounds__(128, (KB > 32) ? 2 : 4) k_blockmate(const float* __restrict__ xc, int64_t N, int k, float* Tb,
                                                      float* Tr)
{
    __shared__ __align__(16) float xs[128][DP];
    __shared__ float wmax[4];
    const int t = threadIdx.x;
    const int64_t r0 = (int64_t)blockIdx.x * 128;
    const int nvalid = (int)max((int64_t)0, min((int64_t)128, N - r0));
    for (int e = t; e < 128 * DP; e += 128)
    {
        const int r = e / DP, d = e % DP;
        xs[r][d] = (r < nvalid) ? xc[(r0 + r) * DP + d] : 0.f;
    }
    __syncthreads();
    float2 xr[DP / 2];  // this thread's row, in pairs for the packed FP32 instructions
#pragma unroll
    for (int q = 0; q < DP / 4; ++q)
    {
        const float4 v = reinterpret_cast<const float4*>(&xs[t][0])[q];
        xr[2 * q] = make_float2(v.x, v.y);
        xr[2 * q + 1] = make_float2(v.z, v.w);
    }
    float L[KB];  // the KB smallest distances so far, ascending
#pragma unroll
    for (int s = 0; s < KB; ++s)
        L[s] = __int_as_float(0x7f800000);
    const float2 m1 = make_float2(-1.f, -1.f);
    for (int c = 0; c < nvalid; ++c)
    {
        // two dimensions per instruction: z = x - y (one rounding, as a
        // subtraction), acc += z z; four partial sums
        const float4* y4 = reinterpret_cast<const float4*>(&xs[c][0]);
        float2 aa = make_float2(0.f, 0.f), ab = aa;
#pragma unroll
        for (int q = 0; q < DP / 4; ++q)
        {
            const float4 y = y4[q];
            const float2 z0 = __ffma2_rn(make_float2(y.x, y.y), m1, xr[2 * q]);
            const float2 z1 = __ffma2_rn(make_float2(y.z, y.w), m1, xr[2 * q + 1]);
            aa = __ffma2_rn(z0, z0, aa);
            ab = __ffma2_rn(z1, z1, ab);
        }
        const float d2 = (aa.x + aa.y) + (ab.x + ab.y);
        if (c != t && d2 < L[KB - 1])
        {
            // slot s keeps L[s] when d2 >= L[s], takes d2 when L[s-1] <= d2 < L[s],
            // and L[s-1] when d2 < L[s-1]
#pragma unroll
            for (int s = KB - 1; s > 0; --s)
                L[s] = fminf(L[s], fmaxf(d2, L[s - 1]));
            L[0] = fminf(L[0], d2);
        }
    }
    // L is ascending, so its k-th entry is the largest of the first k (a max
    // rather than an indexed read keeps L in registers)
    float mine = 0.f;
#pragma unroll
    for (int s = 0; s < KB; ++s)
        mine = fmaxf(mine, (s < k && t < nvalid) ? L[s] : 0.f);
    Tr[r0 + t] = (t < nvalid) ? mine : __int_as_float(0x7f800000);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        mine = fmaxf(mine, __shfl_xor_sync(0xffffffffu, mine, o));
    if ((t & 31) == 0)
        wmax[t >> 5] = mine;
    __syncthreads();
    if (t == 0)
        Tb[blockIdx.x] = fmaxf(fmaxf(wmax[0], wmax[1]), fmaxf(wmax[2], wmax[3]));
}

// near_bits[b][t] = 1 when candidate tile t may hold one of the k nearest
// neighbours of a query of block b. Every point of a far tile lies at least
// the sphere gap g away, and its screened value is at least g^2 - eps_far(b);
// the re-rank certifies a query x when e_k < far_val - eps_far, which
// g^2 >= T_b + 2 eps_far(b) guarantees, T_b bounding e_k for the block
// (k_blockmate) and eps_far(b) using the largest |x| of the block, so that it
// covers every row's own bound. tau_b carries 1 % for the FP32 rounding of the
// gap and of T_b. Any value of tau is safe: a row that fails certification is
// rescanned exactly; tau only decides how many tiles get the full fp16 split.
// One CTA per query block; thread t takes tiles t, t + 256, ...; the tile
// centres are read dimension-major (tcT[d * nt + tile]), so a warp's loads of
// one dimension are contiguous, and a warp ballot forms each 32-tile word.
__global__ void __launch_bounds__(256) k_classify(const float* __restrict__ qc, const float* __restrict__ qr,
                                                  const float* __restrict__ tcT, const float* __restrict__ tr,
                                                  const float* __restrict__ Tb, int nt, int nwords, int Dp,
                                                  const float* rmax, float c1, float c2f, uint32_t* near_bits)
{
    __shared__ float cb[128];
    const int b = blockIdx.x, t = threadIdx.x, lane = t & 31;
    if (t < Dp)
        cb[t] = qc[(int64_t)b * Dp + t];
    __syncthreads();
    const float R = rmax[0];
    const float rb = qr[b];
    float cn2 = 0.f;
    for (int d = 0; d < Dp; ++d)
        cn2 = fmaf(cb[d], cb[d], cn2);
    const float xm = sqrtf(cn2) + fmaxf(rb, 0.f);  // bound of |x| over the block
    const float eps_far = c1 * (xm * xm + R * R) + c2f * xm * R;
    const float tau = 1.01f * (Tb[b] + 2.f * eps_far);  // +inf for a block of at most k rows
    for (int w0 = 0; w0 < nwords * 32; w0 += 256)
    {
        const int tile = w0 + t;
        bool near = false;
        if (tile < nt && rb >= 0.f && tr[tile] >= 0.f)
        {
            float d2 = 0.f;
            for (int d = 0; d < Dp; ++d)
            {
                const float z = cb[d] - tcT[(int64_t)d * nt + tile];
                d2 = fmaf(z, z, d2);
            }
            const float gap = fmaxf(0.f, sqrtf(d2) - rb - tr[tile]);
            near = gap * gap < tau;
        }
        const unsigned word = __ballot_sync(0xffffffffu, near);
        if (lane == 0 && (tile >> 5) < nwords)
            near_bits[(int64_t)b * nwords + (tile >> 5)] = word;
    }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn)
    {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        TK_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q));
        if (q != cudaDriverEntryPointSuccess || !p)
            throw Error(TK_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
        fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    }
    return fn;
}

void make_map(CUtensorMap* m, const uint16_t* base, int64_t rows, int cols, int box_cols, CUtensorMapSwizzle sw,
              int box_rows = 128)
{
    const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
    const cuuint32_t box[2] = {(cuuint32_t)box_cols, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = encode_fn()(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, (void*)base, dims, strides, box, estr,
                             CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
        throw Error(TK_ERR_CUDA, "cuTensorMapEncodeTiled failed with code " + std::to_string((int)r));
}

template <int DP, int KC, int QT = TcCfg<DP>::QT, bool BATCH = false, bool LATER = false>
void launch(tk_ctx* ctx, const uint16_t* xh, const uint16_t* xl, const uint16_t* xn, const float* nrm,
            int64_t rows, const float* scale, int64_t N, const ScreenWork& work, int grid, int32_t* cand_idx,
            float* cand_val, ListSlice slice = ListSlice{})
{
    if (slice.ld == 0)
        slice.ld = KC;
    if (slice.nw == 0)
        slice.nw = KC;
    if (slice.off + slice.nw > slice.ld)
        throw Error(TK_ERR_INTERNAL, "tensor screen: list slice past the row's end");
    if (LATER != (slice.off > 0) || (LATER && !slice.lo))
        throw Error(TK_ERR_INTERNAL, "tensor screen: list slice does not match the kernel");
    using C = TcCfg<DP, QT>;
    static_assert(C::SMEM <= 227 * 1024, "shared memory budget");
    CUtensorMap mh, ml, mn;
    make_map(&mh, xh, rows, DP, 64, CU_TENSOR_MAP_SWIZZLE_128B);
    make_map(&ml, xl, rows, DP, 64, CU_TENSOR_MAP_SWIZZLE_128B);
    make_map(&mn, xn, rows, 16, 16, CU_TENSOR_MAP_SWIZZLE_32B);
    TK_CUDA(cudaFuncSetAttribute(k_screen_tc<DP, KC, QT, BATCH, LATER>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)C::SMEM));
    k_screen_tc<DP, KC, QT, BATCH, LATER><<<grid, TC_THREADS, C::SMEM, ctx->stream>>>(mh, ml, mn, scale, N, rows, work, cand_idx,
                                                                        cand_val, nrm, slice, ctx->dev_err);
    TK_CHECK_LAUNCH();
}

void launch_wide(tk_ctx* ctx, Prepared& P, int k, int32_t* cand_idx, float* cand_val)
{
    cudaStream_t st = ctx->stream;
    const int nq = (int)(P.Npad / TC_M), nt = (int)(P.Npad / TW_N);
    const int nwords = (nt + 31) / 32;
    float* qc = (float*)ctx->scratch.get("tw.qc", sizeof(float) * (size_t)nq * P.Dp);
    float* qr = (float*)ctx->scratch.get("tw.qr", sizeof(float) * (size_t)nq);
    float* tc = (float*)ctx->scratch.get("tw.tc", sizeof(float) * (size_t)nt * P.Dp);
    float* tcT = (float*)ctx->scratch.get("tw.tcT", sizeof(float) * (size_t)nt * P.Dp);
    float* tr = (float*)ctx->scratch.get("tw.tr", sizeof(float) * (size_t)nt);
    uint32_t* bits = (uint32_t*)ctx->scratch.get("tw.bits", sizeof(uint32_t) * (size_t)nq * nwords);
    float* Tb = (float*)ctx->scratch.get("tw.tb", sizeof(float) * (size_t)nq);
    float* Trow = (float*)ctx->scratch.get("tw.trow", sizeof(float) * (size_t)P.Npad);
    P.far_val = (float*)ctx->scratch.get("tw.far", sizeof(float) * (size_t)P.Npad);
    float c1, c2, c2f;
    screen_error_model(TK_SCREEN_TENSOR, P.Dp, &c1, &c2);
    screen_error_model_far(P.Dp, &c2f);
    P.c2_far = c2f;
    k_spheres<TC_M><<<nq, 256, 0, st>>>(P.xc, P.N, P.Dp, qc, qr, nullptr);
    TK_CHECK_LAUNCH();
    k_spheres<TW_N><<<nt, 256, 0, st>>>(P.xc, P.N, P.Dp, tc, tr, tcT);
    TK_CHECK_LAUNCH();
    if (k <= 16)
        k_blockmate<64, 16><<<nq, 128, 0, st>>>(P.xc, P.N, k, Tb, Trow);
    else
        k_blockmate<64, 32><<<nq, 128, 0, st>>>(P.xc, P.N, k, Tb, Trow);
    TK_CHECK_LAUNCH();
    k_classify<<<nq, 256, 0, st>>>(qc, qr, tcT, tr, Tb, nt, nwords, P.Dp, P.rmax, c1, c2f, bits);
    TK_CHECK_LAUNCH();
    CUtensorMap ah, al, bh, bl, bn;
    make_map(&ah, P.xh, P.Npad, 64, 64, CU_TENSOR_MAP_SWIZZLE_128B, 128);
    make_map(&al, P.xl, P.Npad, 64, 64, CU_TENSOR_MAP_SWIZZLE_128B, 128);
    make_map(&bh, P.xh, P.Npad, 64, 64, CU_TENSOR_MAP_SWIZZLE_128B, TW_N);
    make_map(&bl, P.xl, P.Npad, 64, 64, CU_TENSOR_MAP_SWIZZLE_128B, TW_N);
    make_map(&bn, P.xn, P.Npad, 16, 16, CU_TENSOR_MAP_SWIZZLE_32B, TW_N);
    // One CTA per query block fills whole waves of one CTA per SM; the blocks of
    // the last, partial wave are split into `parts` CTAs each (at most one wave),
    // so the kernel does not wait on a few whole blocks at its end.
    const int sms = std::max(1, ctx->num_sms);
    const int tail = nq % sms;
    int parts = (tail > 0 && nq > sms) ? std::min(8, std::min(sms / tail, nt)) : 1;
    if (parts < 2)
        parts = 1;
    const int full_blocks = (parts == 1) ? nq : nq - tail;
    const int grid = full_blocks + (nq - full_blocks) * parts;
    const int64_t split_rows = (int64_t)(nq - full_blocks) * TC_M;
    int32_t* part_idx = nullptr;
    float *part_val = nullptr, *part_far = nullptr;
    if (parts > 1)
    {
        part_idx = (int32_t*)ctx->scratch.get("tw.pidx", sizeof(int32_t) * (size_t)split_rows * parts * TW_KC);
        part_val = (float*)ctx->scratch.get("tw.pval", sizeof(float) * (size_t)split_rows * parts * TW_KC);
        part_far = (float*)ctx->scratch.get("tw.pfar", sizeof(float) * (size_t)split_rows * parts);
    }
    TK_CUDA(cudaFuncSetAttribute(k_screen_tc_wide, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TwCfg::SMEM));
    k_screen_tc_wide<<<grid, TW_THREADS, TwCfg::SMEM, st>>>(ah, al, bh, bl, bn, P.rmax + 1, P.N, P.Npad, bits, nwords,
                                                           cand_idx, cand_val, P.far_val, P.nrm, full_blocks, parts,
                                                           part_idx, part_val, part_far, Trow, P.rmax, c1, c2,
                                                           ctx->dev_err);
    TK_CHECK_LAUNCH();
    if (parts > 1)
    {
        k_merge_parts<<<(int)((split_rows + 127) / 128), 128, 0, st>>>((int64_t)full_blocks * TC_M, split_rows, parts,
                                                                       part_idx, part_val, part_far, cand_idx,
                                                                       cand_val, P.far_val);
        TK_CHECK_LAUNCH();
    }
}

// The bound that seeds the lists of the long-list passes (padded dimension 64,
// k <= 64): each row's k-th distance over its 128-row block (k_blockmate).
// Without it (other dimensions, larger k) the lists start empty.
// The same bound classifies the candidate tiles (128 rows, the same blocks as the
// query blocks, so one set of spheres serves both) into near and far, as for the
// wide kernel; far_val goes to P for the re-rank's certification.
ListSlice seeded_slice(tk_ctx* ctx, Prepared& P, int k)
{
    ListSlice sl;
    if (P.Dp != 64 || k > 64 || k < 1)
        return sl;
    cudaStream_t st = ctx->stream;
    const int nq = (int)(P.Npad / TC_M);
    const int nwords = (nq + 31) / 32;
    float* Tb = (float*)ctx->scratch.get("tc.tb", sizeof(float) * (size_t)nq);
    float* Trow = (float*)ctx->scratch.get("tc.trow", sizeof(float) * (size_t)P.Npad);
    float* bc = (float*)ctx->scratch.get("tc.bc", sizeof(float) * (size_t)nq * P.Dp);
    float* bcT = (float*)ctx->scratch.get("tc.bcT", sizeof(float) * (size_t)nq * P.Dp);
    float* br = (float*)ctx->scratch.get("tc.br", sizeof(float) * (size_t)nq);
    uint32_t* bits = (uint32_t*)ctx->scratch.get("tc.bits", sizeof(uint32_t) * (size_t)nq * nwords);
    P.far_val = (float*)ctx->scratch.get("tc.far", sizeof(float) * (size_t)P.Npad);
    float c2f;
    screen_error_model(TK_SCREEN_TENSOR, P.Dp, &sl.c1, &sl.c2);
    screen_error_model_far(P.Dp, &c2f);
    P.c2_far = c2f;
    k_blockmate<64, 64><<<nq, 128, 0, st>>>(P.xc, P.N, k, Tb, Trow);
    TK_CHECK_LAUNCH();
    k_spheres<TC_M><<<nq, 256, 0, st>>>(P.xc, P.N, P.Dp, bc, br, bcT);
    TK_CHECK_LAUNCH();
    k_classify<<<nq, 256, 0, st>>>(bc, br, bcT, br, Tb, nq, nwords, P.Dp, P.rmax, sl.c1, c2f, bits);
    TK_CHECK_LAUNCH();
    sl.seed_tr = Trow;
    sl.rmax = P.rmax;
    sl.near_bits = bits;
    sl.nwords = nwords;
    sl.far_val = P.far_val;
    return sl;
}

template <int DP, int KC>
void launch_single(tk_ctx* ctx, Prepared& P, int32_t* cand_idx, float* cand_val)
{
    const ScreenWork single{nullptr, 0, nullptr, nullptr};
    const int grid = (int)(P.Npad / (TcCfg<DP>::QT * TC_M));
    launch<DP, KC>(ctx, P.xh, P.xl, P.xn, P.nrm, P.Npad, P.rmax + 1, P.N, single, grid, cand_idx, cand_val);
}

// Passes of PASS entries that fill rows of kc entries with at least k + 8.
constexpr int pass_count(int k, int kc, int pass)
{
    return ((k + 8 + pass - 1) / pass) < ((kc + pass - 1) / pass) ? (k + 8 + pass - 1) / pass : (kc + pass - 1) / pass;
}

// Lists of kc = 64, 128 or 256 entries per row: passes of the PASS-entry screen
// until the row holds k + 8 entries, pass p writing entries [PASS p, ...) after
// the entries of passes < p; the last pass writes to the row's end.
template <int DP, int PASS>
void launch_passes(tk_ctx* ctx, Prepared& P, int k, int kc, const ListSlice& seed, int32_t* cand_idx,
                   float* cand_val)
{
    const ScreenWork single{nullptr, 0, nullptr, nullptr};
    const int grid = (int)(P.Npad / (TcCfg<DP>::QT * TC_M));
    float* last[2] = {(float*)ctx->scratch.get("tc.last0", sizeof(float) * (size_t)P.Npad),
                      (float*)ctx->scratch.get("tc.last1", sizeof(float) * (size_t)P.Npad)};
    const int passes = pass_count(k, kc, PASS);
    for (int p = 0; p < passes; ++p)
    {
        ListSlice sl = seed;
        sl.ld = kc;
        sl.off = PASS * p;
        sl.nw = (p + 1 < passes) ? PASS : kc - sl.off;
        sl.lo = (p > 0) ? last[(p - 1) & 1] : nullptr;
        sl.last = (p + 1 < passes) ? last[p & 1] : nullptr;
        if (p > 0)
            sl.far_val = nullptr;  // every pass screens the same far values
        if (p == 0)
            launch<DP, PASS>(ctx, P.xh, P.xl, P.xn, P.nrm, P.Npad, P.rmax + 1, P.N, single, grid, cand_idx, cand_val,
                             sl);
        else
            launch<DP, PASS, TcCfg<DP>::QT, false, true>(ctx, P.xh, P.xl, P.xn, P.nrm, P.Npad, P.rmax + 1, P.N,
                                                         single, grid, cand_idx, cand_val, sl);
    }
}

// 48-entry passes do not spill; a 64-entry pass spills registers in the epilogue
// and took about 1.4 times as long (13.0 against 9.0 ms per pass at N = 200000),
// so 64-entry passes are taken only where they need fewer than 3/4 as many.
template <int DP>
void launch_long(tk_ctx* ctx, Prepared& P, int k, int kc, int32_t* cand_idx, float* cand_val)
{
    const ListSlice seed = seeded_slice(ctx, P, k);
    if (4 * pass_count(k, kc, 64) < 3 * pass_count(k, kc, TC_PASS))
        launch_passes<DP, 64>(ctx, P, k, kc, seed, cand_idx, cand_val);
    else
        launch_passes<DP, TC_PASS>(ctx, P, k, kc, seed, cand_idx, cand_val);
}

} // namespace

namespace {

// Self-test of the bounded wait: thread 0 waits, with the screen's own mbar_wait
// and limit, on a shared-memory mbarrier that expects one arrival nobody makes.
// After WAIT_LIMIT_NS the wait gives up, raises DEV_ERR_TIMEOUT and the kernel
// returns; *outcome is 1 for that and 2 if the phase had completed (it cannot).
// No copy, MMA or TMEM allocation is involved, so nothing is left to drain.
__global__ void k_wait_selftest(unsigned* err, int* outcome)
{
    __shared__ __align__(8) uint64_t bar;
    __shared__ int abort_flag;
    if (threadIdx.x != 0)
        return;
    abort_flag = 0;
    const uint32_t b = smem_u32(&bar);
    mbar_init(b, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    const bool done = mbar_wait(b, 0, &abort_flag, err);
    *outcome = done ? 2 : 1;
}

} // namespace

int wait_selftest(tk_ctx* ctx)
{
    int* d = (int*)ctx->scratch.get("selftest.outcome", sizeof(int));
    TK_CUDA(cudaMemsetAsync(d, 0, sizeof(int), ctx->stream));
    k_wait_selftest<<<1, 32, 0, ctx->stream>>>(ctx->dev_err, d);
    TK_CHECK_LAUNCH();
    int h = 0;
    TK_CUDA(cudaMemcpyAsync(&h, d, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    TK_CUDA(cudaStreamSynchronize(ctx->stream));
    return h;
}

bool tensor_screen_supported(int Dp) { return Dp == 64 || Dp == 128; }

void screen_tensor(tk_ctx* ctx, Prepared& P, int kc, int k, int32_t* cand_idx, float* cand_val)
{
    if (!P.xh || !P.xl || !P.xn)
        throw Error(TK_ERR_INTERNAL, "tensor screen needs the fp16 split layout");
    if (kc != 32 && kc != 64 && kc != 128 && kc != 256)
        throw Error(TK_ERR_INTERNAL, "tensor screen: unsupported candidate count " + std::to_string(kc));
    if (P.Dp == 64)
    {
        if (kc == 32)
            launch_wide(ctx, P, k, cand_idx, cand_val);
        else
            launch_long<64>(ctx, P, k, kc, cand_idx, cand_val);
    }
    else if (P.Dp == 128)
    {
        if (kc == 32)
            launch_single<128, 32>(ctx, P, cand_idx, cand_val);
        else
            launch_long<128>(ctx, P, k, kc, cand_idx, cand_val);
    }
    else
        throw Error(TK_ERR_UNSUPPORTED, "the tensor-core screen supports D <= 128 (padded to 64 or 128); use the "
                                        "FP32 screen for D = " +
                                            std::to_string(P.D));
}

void screen_tensor_batch(tk_ctx* ctx, const StackedScreen& S, int32_t* cand_idx, float* cand_val)
{
    const ScreenWork work{S.items, S.nitems, S.prob_n, S.prob_scale};
    const int grid = std::min(S.nitems, ctx->num_sms);
    if (grid <= 0)
        return;
#define TK_SCREEN_BATCH(DPV, KCV, QTV)                                                                            \
    launch<DPV, KCV, QTV, true>(ctx, S.xh, S.xl, S.xn, S.nrm, S.rows, nullptr, 0, work, grid, cand_idx, cand_val, rows)
    // 64-candidate rows of a group whose k are all <= 40 come from the 48-entry
    // list (no spills), padded to 64 with its last value and id -1
    const bool short64 = S.kc == 64 && S.kmax >= 1 && S.kmax + 8 <= TC_PASS;
    ListSlice rows;
    rows.ld = S.kc;
    rows.nw = S.kc;
    if (S.Dp == 64 && S.kc == 32 && S.qt == 2)
        TK_SCREEN_BATCH(64, 32, 2);
    else if (S.Dp == 64 && S.kc == 32 && S.qt == 1)
        TK_SCREEN_BATCH(64, 32, 1);
    else if (S.Dp == 64 && short64 && S.qt == 2)
        TK_SCREEN_BATCH(64, TC_PASS, 2);
    else if (S.Dp == 64 && short64 && S.qt == 1)
        TK_SCREEN_BATCH(64, TC_PASS, 1);
    else if (S.Dp == 64 && S.kc == 64 && S.qt == 2)
        TK_SCREEN_BATCH(64, 64, 2);
    else if (S.Dp == 64 && S.kc == 64 && S.qt == 1)
        TK_SCREEN_BATCH(64, 64, 1);
    else if (S.Dp == 128 && S.kc == 32)
        TK_SCREEN_BATCH(128, 32, 1);
    else if (S.Dp == 128 && short64)
        TK_SCREEN_BATCH(128, TC_PASS, 1);
    else if (S.Dp == 128 && S.kc == 64)
        TK_SCREEN_BATCH(128, 64, 1);
    else
        throw Error(TK_ERR_UNSUPPORTED, "batched tensor screen: unsupported (Dp, KC, QT)");
#undef TK_SCREEN_BATCH
}

} // namespace tk
