// assemble.cu -- CSR assembly of the alignment matrix M (pull formulation).
//
// The reference emits per-point triplets (routines/locally_linear.hpp:133-146
// for LLE, :65-77 for LTSA) and sums duplicates with setFromTriplets
// (utils/sparse.hpp:16-21). Here every output row j gathers its own
// contributions instead, so no atomics touch values and the result is
// bit-reproducible:
//   * reverse adjacency rev(j) = {(r, a) : idx[r][a] == j}, sorted by r;
//   * row j visits its sources in ascending point order -- point j itself and
//     every r in rev(j) -- exactly the order in which a serial run of the
//     reference pushes the triplets that land in row j, and adds each
//     contribution into a per-warp shared-memory hash table keyed by column.
//     Contributions of one source to one row have distinct columns, so one
//     source is one lane-parallel batch and every (row, col) sum is formed in
//     the reference's serial triplet order;
//   * the table is compacted, sorted by column (bitonic, in registers) and
//     written to a per-row scratch (128 or 256 entries) together with its count.
// One pass over the rows (k_rows_fused), then an exclusive scan of the counts
// and a copy of every row into the CSR (k_compact). The contributions of a
// round of sources are loaded into shared memory together before they are
// added, so a row waits for one round of gathers rather than one per source. A
// row whose distinct columns overflow the 256-slot table or the scratch is
// redone by a one-warp kernel with an 8192-slot table, in a count and a fill
// pass.
//
//   LLE  row j: source j  -> (j, 1+shift), (n_a, -w_ja)
//               source r  -> (r, -w_ra), (n_b, w_ra w_rb)       [j = n_a of r]
//   LTSA row j: source j  -> (j, shift)
//               source r  -> (j, +1) then (n_b, -P_r[a][b])      [j = n_a of r]
//               P_r = (1/k) 1 1^T + V_r V_r^T
//   HLLE row j: source r  -> (n_b, B_r[a][b])                    [j = n_a of r]
//               B_r = Y_r Y_r^T, Y_r the dp product columns (routines/
//               locally_linear.hpp:234-243); no diagonal term
// For HLLE the td argument of the kernels is the column count dp of Y.
#include <cstdint>

#include "tk_internal.h"

namespace tk {
namespace {

constexpr int HC = 256;         // hash slots of the big kernel's first attempt
constexpr int HC_BIG = 8192;    // hash slots for rows that overflow the fused pass
constexpr int ROW_WARPS = 8;
constexpr int STAGE = 256;      // staged (column, value) contributions per warp
// fused pass: (hash slots, row scratch entries, staged contributions) -- rows of
// LLE with k <= 24 hold ~3.5 k distinct columns; LTSA and larger k take the
// wider table; k > 40 the widest (LLE at k = 64: 234 distinct columns per row
// on average, many above 256, which the 256-entry scratch sent to the one-warp
// large-table kernel)
constexpr int HC_S = 256, RCAP_S = 128;
constexpr int HC_L = 512, RCAP_L = 256;
constexpr int HC_X = 512, RCAP_X = 512, STAGE_X = 512;

__global__ void k_indeg(const int32_t* __restrict__ idx, int64_t nk, int64_t N, int k, int* cnt, unsigned* repeats,
                        unsigned* err)
{
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nk; e += (int64_t)gridDim.x * blockDim.x)
    {
        const int j = idx[e];
        if (j < 0 || j >= N)
        {
            atomicOr(err, DEV_ERR_BOUNDS);
            continue;
        }
        atomicAdd(&cnt[j], 1);
        // a point listed as its own neighbour, or twice in one list
        const int64_t r = e / k, a = e - r * k;
        bool rep = (j == r);
        for (int b = 0; b < a && !rep; ++b)
            rep = idx[r * k + b] == j;
        if (rep)
            atomicOr(repeats, 1u);
    }
}

// Exclusive scan of n int counters into int64 offsets (out has n+1 entries) in
// three launches: per-segment sums, a one-block scan of the segment sums, and a
// per-segment scan with its offset. Fixed segments, fixed order: deterministic.
constexpr int SCAN_SEG = 2048;  // elements per segment (one 256-thread block)

__global__ void k_seg_sums(const int* in, int64_t n, int64_t* seg)
{
    __shared__ int64_t red[256];
    const int64_t b0 = (int64_t)blockIdx.x * SCAN_SEG;
    int64_t s = 0;
    for (int t = threadIdx.x; t < SCAN_SEG; t += blockDim.x)
        if (b0 + t < n)
            s += in[b0 + t];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1)
    {
        if ((int)threadIdx.x < o)
            red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        seg[blockIdx.x] = red[0];
}

__global__ void k_scan_segs(int64_t* seg, int nseg, int64_t* total)
{
    __shared__ int64_t part[1024];
    const int t = threadIdx.x;
    const int per = (nseg + 1023) / 1024;
    const int b0 = t * per, b1 = min(nseg, b0 + per);
    int64_t s = 0;
    for (int b = b0; b < b1; ++b)
        s += seg[b];
    part[t] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1)
    {
        const int64_t v = (t >= o) ? part[t - o] : 0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    int64_t run = part[t] - s;
    for (int b = b0; b < b1; ++b)
    {
        const int64_t c = seg[b];
        seg[b] = run;
        run += c;
    }
    if (t == 1023)
        *total = part[1023];
}

__global__ void k_seg_scan(const int* in, int64_t n, const int64_t* seg, int64_t* out)
{
    constexpr int PER = SCAN_SEG / 256;
    __shared__ int64_t part[256];
    const int64_t b0 = (int64_t)blockIdx.x * SCAN_SEG + (int64_t)threadIdx.x * PER;
    int64_t v[PER];
    int64_t s = 0;
#pragma unroll
    for (int q = 0; q < PER; ++q)
    {
        v[q] = (b0 + q < n) ? in[b0 + q] : 0;
        s += v[q];
    }
    part[threadIdx.x] = s;
    __syncthreads();
    for (int o = 1; o < 256; o <<= 1)
    {
        const int64_t x = ((int)threadIdx.x >= o) ? part[threadIdx.x - o] : 0;
        __syncthreads();
        part[threadIdx.x] += x;
        __syncthreads();
    }
    int64_t run = seg[blockIdx.x] + part[threadIdx.x] - s;
#pragma unroll
    for (int q = 0; q < PER; ++q)
    {
        if (b0 + q < n)
            out[b0 + q] = run;
        run += v[q];
    }
}

} // namespace

void scan_to_offsets(tk_ctx* ctx, const int* in, int64_t n, int64_t* out)
{
    const int nseg = (int)((n + SCAN_SEG - 1) / SCAN_SEG);
    int64_t* seg = (int64_t*)ctx->scratch.get("asm.scanseg", sizeof(int64_t) * (size_t)std::max(nseg, 1));
    k_seg_sums<<<nseg, 256, 0, ctx->stream>>>(in, n, seg);
    TK_CHECK_LAUNCH();
    k_scan_segs<<<1, 1024, 0, ctx->stream>>>(seg, nseg, out + n);
    TK_CHECK_LAUNCH();
    k_seg_scan<<<nseg, 256, 0, ctx->stream>>>(in, n, seg, out);
    TK_CHECK_LAUNCH();
}

namespace {

// Entries outside [0, N) were flagged by k_indeg (DEV_ERR_BOUNDS, turned into
// TK_ERR_INVALID_ARG by the host after the row phase) and are skipped here too,
// so a caller's bad index is never used as an address.
__global__ void k_fill_rev(const int32_t* __restrict__ idx, int64_t nk, int64_t N, const int64_t* rptr, int* fillc,
                           int32_t* rev)
{
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nk; e += (int64_t)gridDim.x * blockDim.x)
    {
        const int j = idx[e];
        if (j < 0 || j >= N)
            continue;
        const int pos = atomicAdd(&fillc[j], 1);
        rev[rptr[j] + pos] = (int32_t)e;
    }
}

// insertion sort of every reverse list (edge id = r*k + a, ascending = by r)
__global__ void k_sort_rev(int64_t N, const int64_t* rptr, int32_t* rev)
{
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < N; j += (int64_t)gridDim.x * blockDim.x)
    {
        const int64_t b = rptr[j], e = rptr[j + 1];
        for (int64_t p = b + 1; p < e; ++p)
        {
            const int32_t v = rev[p];
            int64_t q = p - 1;
            while (q >= b && rev[q] > v)
            {
                rev[q + 1] = rev[q];
                --q;
            }
            rev[q + 1] = v;
        }
    }
}

__device__ __forceinline__ unsigned hash_col(int c) { return (unsigned)c * 2654435761u; }

template <int CAP>
struct RowTable
{
    int keys[CAP];
    double vals[CAP];
    unsigned long long sortk[CAP];
};

// insert-or-add; returns false if the table is full
template <int CAP, bool VALUES, class Table>
__device__ __forceinline__ bool table_add(Table& T, int col, double v)
{
    unsigned h = hash_col(col) & (CAP - 1);
    for (int probe = 0; probe < CAP; ++probe)
    {
        int key = T.keys[h];
        if (key == -1)
        {
            key = atomicCAS(&T.keys[h], -1, col);
            if (key == -1)
                key = col;  // claimed
        }
        if (key == col)
        {
            if (VALUES)
                T.vals[h] += v;  // distinct columns within a batch: no other lane owns this slot
            return true;
        }
        h = (h + 1) & (CAP - 1);
    }
    return false;
}

// One lane-parallel batch of adds, called by the whole warp (valid marks the
// lanes with a contribution). Lanes whose columns coincide -- possible only for
// a caller's idx that lists a point as its own neighbour or twice -- add in
// lane order, one per step, so no update is lost and the sum is reproducible.
template <int CAP, bool VALUES, class Table>
__device__ __forceinline__ bool warp_add(Table& T, int lane, bool valid, int col, double v)
{
    const unsigned grp = __match_any_sync(0xffffffffu, valid ? col : -2 - lane);
    const int rank = __popc(grp & ((1u << lane) - 1u));
    const int last = (int)__reduce_max_sync(0xffffffffu, valid ? (unsigned)rank : 0u);
    bool ok = true;
    for (int r = 0; r <= last; ++r)
    {
        if (valid && rank == r)
            ok = table_add<CAP, VALUES>(T, col, v);
        __syncwarp();
    }
    return ok;
}

// n / d for 0 <= n < 2^31 and a divisor fixed per launch: one multiply-high by
// m = ceil(2^32 / d) (2^32 - 1 for d = 1) gives floor(n / d) or one more or
// less, and the remainder fixes it.
struct FastDiv
{
    int d;
    unsigned m;
    __host__ __device__ explicit FastDiv(int dd)
        : d(dd), m(dd <= 1 ? 0xffffffffu : (unsigned)((0x100000000ull + (unsigned)dd - 1) / (unsigned)dd)) {}
    __device__ __forceinline__ int div(int n) const
    {
        int q = (int)__umulhi((unsigned)n, m);
        const int r = n - q * d;
        q += (r < 0) ? -1 : ((r >= d) ? 1 : 0);
        return q;
    }
};

// Upper bound of the number of distinct columns in row j.
__device__ __forceinline__ int64_t row_bound(int method, int k, int64_t deg)
{
    return method == TK_METHOD_KLLE ? 1 + k + deg * (k + 1) : 1 + deg * k;
}

// Processes one row with one warp. Returns false on table overflow.
template <int CAP, bool VALUES>
__device__ bool process_row(RowTable<CAP>& T, int lane, int method, int64_t j, int k, int td,
                            const int32_t* __restrict__ idx, const double* __restrict__ wts, double shift,
                            const int64_t* __restrict__ rptr, const int32_t* __restrict__ rev)
{
    for (int h = lane; h < CAP; h += 32)
    {
        T.keys[h] = -1;
        if (VALUES)
            T.vals[h] = 0.0;
    }
    __syncwarp();
    bool ok = true;
    const int64_t b = rptr[j], e = rptr[j + 1];
    bool self_done = false;
    for (int64_t p = b; p <= e; ++p)
    {
        // next source in ascending point order: j itself is merged into rev(j)
        int64_t src;
        int slot = -1;
        if (p < e)
        {
            const int32_t eid = rev[p];
            src = eid / k;
            slot = eid - (int32_t)src * k;
            if (!self_done && j < src)
            {
                src = j;
                slot = -1;
                --p;  // revisit this edge next iteration
            }
        }
        else
        {
            if (self_done)
                break;
            src = j;
        }
        if (src == j && slot < 0)
            self_done = true;

        if (method == TK_METHOD_KLLE)
        {
            if (slot < 0)
            {
                // source j: (j, 1+shift) and (n_a, -w_ja)
                for (int t0 = 0; t0 < k + 1; t0 += 32)
                {
                    const int t = t0 + lane;
                    const bool valid = t < k + 1;
                    const int col = !valid ? 0 : (t == 0) ? (int)j : idx[j * k + t - 1];
                    const double v = (VALUES && valid) ? ((t == 0) ? 1.0 + shift : -wts[j * k + t - 1]) : 0.0;
                    ok &= warp_add<CAP, VALUES>(T, lane, valid, col, v);
                }
            }
            else
            {
                // source r=src, j at slot a: (r, -w_ra), (n_b, w_ra w_rb)
                const double wa = VALUES ? wts[src * k + slot] : 0.0;
                for (int t0 = 0; t0 < k + 1; t0 += 32)
                {
                    const int t = t0 + lane;
                    const bool valid = t < k + 1;
                    const int col = !valid ? 0 : (t == 0) ? (int)src : idx[src * k + t - 1];
                    const double v = (VALUES && valid) ? ((t == 0) ? -wa : wa * wts[src * k + t - 1]) : 0.0;
                    ok &= warp_add<CAP, VALUES>(T, lane, valid, col, v);
                }
            }
        }
        else
        {
            const bool hlle = method == TK_METHOD_HLLE;
            if (slot < 0)
            {
                if (!hlle)
                {
                    if (lane == 0)
                        ok &= table_add<CAP, VALUES>(T, (int)j, shift);
                    __syncwarp();
                }
            }
            else
            {
                if (!hlle)
                {
                    if (lane == 0)
                        ok &= table_add<CAP, VALUES>(T, (int)j, 1.0);
                    __syncwarp();
                }
                const double* Va = wts + (src * k + slot) * (int64_t)td;
                for (int t0 = 0; t0 < k; t0 += 32)
                {
                    const int t = t0 + lane;
                    const bool valid = t < k;
                    double v = 0.0;
                    if (VALUES && valid)
                    {
                        const double* Vb = wts + (src * k + t) * (int64_t)td;
                        double pab = hlle ? 0.0 : 1.0 / k;
                        for (int q = 0; q < td; ++q)
                            pab += Va[q] * Vb[q];
                        v = hlle ? pab : -pab;
                    }
                    ok &= warp_add<CAP, VALUES>(T, lane, valid, valid ? idx[src * k + t] : 0, v);
                }
            }
        }
    }
    return __all_sync(0xffffffffu, ok);
}

// number of occupied slots
template <int CAP>
__device__ int table_count(RowTable<CAP>& T, int lane)
{
    int c = 0;
    for (int h = lane; h < CAP; h += 32)
        c += (T.keys[h] != -1);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        c += __shfl_xor_sync(0xffffffffu, c, o);
    return c;
}

// compact, sort by column and write the row
template <int CAP>
__device__ void table_emit(RowTable<CAP>& T, int lane, int64_t base, int32_t* col_idx, double* vals)
{
    int n = 0;
    for (int h0 = 0; h0 < CAP; h0 += 32)
    {
        const int h = h0 + lane;
        const bool occ = T.keys[h] != -1;
        const unsigned m = __ballot_sync(0xffffffffu, occ);
        if (occ)
        {
            const int pos = n + __popc(m & ((1u << lane) - 1u));
            T.sortk[pos] = ((unsigned long long)(unsigned)T.keys[h] << 20) | (unsigned)h;
        }
        n += __popc(m);
    }
    int P = 1;
    while (P < n)
        P <<= 1;
    for (int t = n + lane; t < P; t += 32)
        T.sortk[t] = ~0ull;
    __syncwarp();
    for (int size = 2; size <= P; size <<= 1)
        for (int stride = size >> 1; stride > 0; stride >>= 1)
        {
            for (int t = lane; t < P / 2; t += 32)
            {
                const int lo = 2 * t - (t & (stride - 1));
                const int hi = lo + stride;
                const bool asc = ((lo & size) == 0);
                const unsigned long long a = T.sortk[lo], bb = T.sortk[hi];
                if ((a > bb) == asc)
                {
                    T.sortk[lo] = bb;
                    T.sortk[hi] = a;
                }
            }
            __syncwarp();
        }
    for (int t = lane; t < n; t += 32)
    {
        const unsigned long long key = T.sortk[t];
        col_idx[base + t] = (int32_t)(key >> 20);
        vals[base + t] = T.vals[key & 0xfffffull];
    }
    __syncwarp();
}

// ---------------------------------------------------------------------------
// Fused row pass: one warp per row, contributions staged per round of sources.

template <int HCT, int ST = STAGE>
struct FusedSmem
{
    int keys[HCT];
    double vals[HCT];
    int scol[ST];
    double sval[ST];  // reused for the 64-bit sort keys of the emission (at most ST)
};

// Bitonic sort of 32 * NK 64-bit keys held NK per lane (element i = e * 32 + lane).
template <int NK>
__device__ __forceinline__ void warp_bitonic(unsigned long long (&key)[NK], int lane)
{
    constexpr int LOGP = 5 + (NK == 16 ? 4 : (NK == 8 ? 3 : (NK == 4 ? 2 : (NK == 2 ? 1 : 0))));
#pragma unroll
    for (int ls = 1; ls <= LOGP; ++ls)
    {
        const int size = 1 << ls;
#pragma unroll
        for (int lt = ls - 1; lt >= 0; --lt)
        {
            const int stride = 1 << lt;
            if (lt >= 5)
            {
                // partner in the same lane: element e pairs with e ^ (stride / 32)
                const int es = stride >> 5;
#pragma unroll
                for (int e = 0; e < NK; ++e)
                {
                    if ((e & es) == 0)
                    {
                        const bool asc = ((e * 32 + lane) & size) == 0;
                        const unsigned long long x = key[e], y = key[e + es];
                        const bool sw = (x > y) == asc;
                        key[e] = sw ? y : x;
                        key[e + es] = sw ? x : y;
                    }
                }
            }
            else
            {
#pragma unroll
                for (int e = 0; e < NK; ++e)
                {
                    const unsigned long long other = __shfl_xor_sync(0xffffffffu, key[e], stride);
                    const bool lower = (lane & stride) == 0;
                    const bool asc = ((e * 32 + lane) & size) == 0;
                    const bool keep_min = (lower == asc);
                    const bool less = key[e] < other;
                    key[e] = (keep_min == less) ? key[e] : other;
                }
            }
        }
    }
}

// Sorts the n occupied slots (keys in F.sval, padded) and writes the row.
template <int NK, class Smem>
__device__ __forceinline__ void emit_sorted(Smem& F, int lane, int n, int32_t* out_col, double* out_val)
{
    const unsigned long long* sk = reinterpret_cast<const unsigned long long*>(F.sval);
    unsigned long long key[NK];
#pragma unroll
    for (int e = 0; e < NK; ++e)
    {
        const int i = e * 32 + lane;
        key[e] = (i < n) ? sk[i] : ~0ull;
    }
    warp_bitonic<NK>(key, lane);
#pragma unroll
    for (int e = 0; e < NK; ++e)
    {
        const int i = e * 32 + lane;
        if (i < n)
        {
            out_col[i] = (int32_t)(key[e] >> 10);
            out_val[i] = F.vals[key[e] & 0x3ffull];
        }
    }
}

// Row j in one pass: table of (column, sum) in the serial triplet order, then
// sorted into the row scratch (scol_out/sval_out, RCAP entries per row). Rows
// that do not fit are listed for the large-table kernel.
template <int HCT, int RCAP, int ST = STAGE>
__global__ void __launch_bounds__(ROW_WARPS * 32, (ST > STAGE ? 2 : (HCT == 256 ? 4 : 3)))
    k_rows_fused(int method, int64_t N, int k, int td, const int32_t* __restrict__ idx,
                 const double* __restrict__ wts, double shift, const int64_t* __restrict__ rptr,
                 const int32_t* __restrict__ rev, int* row_nnz, int32_t* scol_out, double* sval_out,
                 int32_t* big_rows, unsigned* nbig, unsigned char* row_big, const unsigned* repeats)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    FusedSmem<HCT, ST>& F = reinterpret_cast<FusedSmem<HCT, ST>*>(smem_raw)[wib];
    static_assert(RCAP <= ST && HCT <= 1024, "sort keys live in sval; slot ids take 10 bits");
    const int KS = k + 1;          // contributions per source
    const int S = ST / KS;         // sources per round (0 when k >= ST: every row takes the large table)
    const int64_t nw = (int64_t)gridDim.x * ROW_WARPS;
    const bool lle = method == TK_METHOD_KLLE;
    const bool hlle = method == TK_METHOD_HLLE;
    const double inv_k = 1.0 / k;
    const FastDiv div_k(k), div_ks(KS);
    // no point lists itself or a neighbour twice (always so for kNN output):
    // a source's contributions then have distinct columns and add in one step
    const bool distinct = *repeats == 0u;
    for (int64_t j = (int64_t)blockIdx.x * ROW_WARPS + wib; j < N; j += nw)
    {
        __syncwarp();
        const int64_t b = rptr[j], e = rptr[j + 1];
        const int64_t deg = e - b;
        bool ok = S > 0 && row_bound(method, k, deg) <= (int64_t)HC_BIG;
        if (ok)
        {
            for (int h = lane; h < HCT; h += 32)
            {
                F.keys[h] = -1;
                F.vals[h] = 0.0;
            }
            // position of j itself among its sources: after every r <= j (a
            // self-loop r == j, possible in a caller's idx, comes first)
            int pos_j = 0;
            for (int64_t p0 = b; p0 < e; p0 += 32)
            {
                const int64_t p = p0 + lane;
                const bool lt = p < e && (int64_t)div_k.div(rev[p]) <= j;
                pos_j += __popc(__ballot_sync(0xffffffffu, lt));
            }
            const int total = (int)deg + 1;
            for (int r0 = 0; r0 < total && ok; r0 += S)
            {
                const int ns = min(S, total - r0);
                __syncwarp();
                // stage the round's contributions: item it = (source s, entry t)
                for (int it = lane; it < ns * KS; it += 32)
                {
                    const int s = div_ks.div(it), t = it - s * KS;
                    const int p = r0 + s;
                    int64_t src = j;
                    int slot = -1;
                    if (p != pos_j)
                    {
                        const int32_t eid = rev[b + (p < pos_j ? p : p - 1)];
                        src = div_k.div(eid);
                        slot = eid - (int32_t)src * k;
                    }
                    int col = -1;
                    double v = 0.0;
                    if (lle)
                    {
                        if (slot < 0)
                        {
                            // source j: (j, 1 + shift), (n_a, -w_ja)
                            col = (t == 0) ? (int)j : idx[j * k + t - 1];
                            v = (t == 0) ? 1.0 + shift : -wts[j * k + t - 1];
                        }
                        else
                        {
                            // source r, j at slot a: (r, -w_ra), (n_b, w_ra w_rb)
                            const double wa = wts[src * k + slot];
                            col = (t == 0) ? (int)src : idx[src * k + t - 1];
                            v = (t == 0) ? -wa : wa * wts[src * k + t - 1];
                        }
                    }
                    else
                    {
                        if (slot < 0)
                        {
                            // source j: (j, shift); nothing for HLLE
                            col = (t == 0 && !hlle) ? (int)j : -1;
                            v = shift;
                        }
                        else if (t == 0)
                        {
                            col = hlle ? -1 : (int)j;  // LTSA's (j, +1), added before the row of P_r
                            v = 1.0;
                        }
                        else
                        {
                            // LTSA: (n_b, -P_r[a][b]), P_r = (1/k) 1 1^T + V_r V_r^T
                            // HLLE: (n_b, B_r[a][b]),  B_r = Y_r Y_r^T
                            const double* Va = wts + (src * k + slot) * (int64_t)td;
                            const double* Vb = wts + (src * k + t - 1) * (int64_t)td;
                            double pab = hlle ? 0.0 : inv_k;
                            for (int q = 0; q < td; ++q)
                                pab += Va[q] * Vb[q];
                            col = idx[src * k + t - 1];
                            v = hlle ? pab : -pab;
                        }
                    }
                    F.scol[it] = col;
                    F.sval[it] = v;
                }
                __syncwarp();
                // add in source order; one source's entries have distinct columns,
                // except LTSA's (j, +1), which goes first on its own
                for (int s = 0; s < ns; ++s)
                {
                    const int base = s * KS;
                    if (!lle)
                    {
                        if (lane == 0 && F.scol[base] >= 0)
                            ok &= table_add<HCT, true>(F, F.scol[base], F.sval[base]);
                        __syncwarp();
                        for (int t0 = 1; t0 < KS; t0 += 32)
                        {
                            const int t = t0 + lane;
                            const bool valid = t < KS && F.scol[base + t] >= 0;
                            if (distinct)
                            {
                                if (valid)
                                    ok &= table_add<HCT, true>(F, F.scol[base + t], F.sval[base + t]);
                            }
                            else
                                ok &= warp_add<HCT, true>(F, lane, valid, valid ? F.scol[base + t] : 0,
                                                         valid ? F.sval[base + t] : 0.0);
                        }
                    }
                    else
                    {
                        for (int t0 = 0; t0 < KS; t0 += 32)
                        {
                            const int t = t0 + lane;
                            const bool valid = t < KS;
                            if (distinct)
                            {
                                if (valid)
                                    ok &= table_add<HCT, true>(F, F.scol[base + t], F.sval[base + t]);
                            }
                            else
                                ok &= warp_add<HCT, true>(F, lane, valid, valid ? F.scol[base + t] : 0,
                                                         valid ? F.sval[base + t] : 0.0);
                        }
                    }
                    __syncwarp();
                }
                ok = __all_sync(0xffffffffu, ok);
            }
        }
        int n = 0;
        if (ok)
        {
            // compact the occupied slots into 64-bit sort keys (column << 8 | slot)
            __syncwarp();
            unsigned long long* sk = reinterpret_cast<unsigned long long*>(F.sval);
            for (int h0 = 0; h0 < HCT; h0 += 32)
            {
                const int h = h0 + lane;
                const bool occ = F.keys[h] != -1;
                const unsigned m = __ballot_sync(0xffffffffu, occ);
                if (occ && n + __popc(m & ((1u << lane) - 1u)) < RCAP)
                    sk[n + __popc(m & ((1u << lane) - 1u))] =
                        ((unsigned long long)(unsigned)F.keys[h] << 10) | (unsigned)h;
                n += __popc(m);
            }
            __syncwarp();
            ok = n <= RCAP;
        }
        if (!ok)
        {
            if (lane == 0)
            {
                row_big[j] = 1;
                row_nnz[j] = 0;
                big_rows[atomicAdd(nbig, 1u)] = (int32_t)j;
            }
            continue;
        }
        int32_t* oc = scol_out + j * RCAP;
        double* ov = sval_out + j * RCAP;
        if (n <= 64)
            emit_sorted<2>(F, lane, n, oc, ov);
        else if (RCAP <= 128 || n <= 128)
            emit_sorted<4>(F, lane, n, oc, ov);
        else if (RCAP <= 256 || n <= 256)
            emit_sorted<8>(F, lane, n, oc, ov);
        else
            emit_sorted<(RCAP > 256 ? 16 : 8)>(F, lane, n, oc, ov);
        if (lane == 0)
            row_nnz[j] = n;
        __syncwarp();
    }
}

// Copies every row that the fused pass kept from the row scratch (rcap entries
// per row) into the CSR.
__global__ void k_compact(int64_t N, int rcap, const int* __restrict__ row_nnz,
                          const unsigned char* __restrict__ row_big, const int64_t* __restrict__ row_ptr,
                          const int32_t* __restrict__ scol, const double* __restrict__ sval, int32_t* col_idx,
                          double* vals)
{
    const int lane = threadIdx.x & 31;
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t j = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; j < N; j += nw)
    {
        if (row_big[j])
            continue;
        const int n = row_nnz[j];
        const int64_t dst = row_ptr[j];
        for (int i = lane; i < n; i += 32)
        {
            col_idx[dst + i] = scol[j * rcap + i];
            vals[dst + i] = sval[j * rcap + i];
        }
    }
}

// rows with a large in-degree: one warp per block, large table
template <bool VALUES>
__global__ void __launch_bounds__(32)
    k_rows_big(int method, int64_t N, int k, int td, const int32_t* __restrict__ idx,
               const double* __restrict__ wts, double shift, const int64_t* __restrict__ rptr,
               const int32_t* __restrict__ rev, int* row_nnz, const int64_t* __restrict__ row_ptr,
               int32_t* col_idx, double* vals, const int32_t* big_rows, const unsigned* nbig, unsigned* err)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    RowTable<HC_BIG>& T = *reinterpret_cast<RowTable<HC_BIG>*>(smem_raw);
    const int lane = threadIdx.x & 31;
    const unsigned nb = *nbig;
    for (unsigned r = blockIdx.x; r < nb; r += gridDim.x)
    {
        const int64_t j = big_rows[r];
        const bool ok = process_row<HC_BIG, VALUES>(T, lane, method, j, k, td, idx, wts, shift, rptr, rev);
        if (!ok)
        {
            if (lane == 0)
                atomicOr(err, DEV_ERR_OVERFLOW);
            continue;
        }
        if (!VALUES)
        {
            const int c = table_count<HC_BIG>(T, lane);
            if (lane == 0)
                row_nnz[j] = c;
        }
        else
            table_emit<HC_BIG>(T, lane, row_ptr[j], col_idx, vals);
        __syncwarp();
    }
}

} // namespace

namespace {
struct AsmState
{
    int64_t* rptr;
    int32_t* rev;
    int* row_nnz;
    int32_t* big;
    unsigned* nbig;
    unsigned char* row_big;
    int32_t* scol;
    double* sval;
    int rcap;
};

// the wide fused-pass table for LTSA and for LLE with k > 24; the widest for k > 40
bool wide_rows(int method, int k) { return method != TK_METHOD_KLLE || k > 24; }
bool widest_rows(int k) { return k > 40; }

AsmState asm_state(tk_ctx* ctx, int method, int64_t N, int k)
{
    const int64_t nk = N * (int64_t)k;
    AsmState a;
    a.rptr = (int64_t*)ctx->scratch.get("asm.rptr", sizeof(int64_t) * (size_t)(N + 1));
    a.rev = (int32_t*)ctx->scratch.get("asm.rev", sizeof(int32_t) * (size_t)nk);
    a.row_nnz = (int*)ctx->scratch.get("asm.rownnz", sizeof(int) * (size_t)N);
    a.big = (int32_t*)ctx->scratch.get("asm.big", sizeof(int32_t) * (size_t)N);
    a.nbig = (unsigned*)ctx->scratch.get("asm.nbig", 16);
    a.row_big = (unsigned char*)ctx->scratch.get("asm.rowbig", (size_t)N);
    a.rcap = widest_rows(k) ? RCAP_X : (wide_rows(method, k) ? RCAP_L : RCAP_S);
    a.scol = (int32_t*)ctx->scratch.get("asm.scol", sizeof(int32_t) * (size_t)N * a.rcap);
    a.sval = (double*)ctx->scratch.get("asm.sval", sizeof(double) * (size_t)N * a.rcap);
    return a;
}

void set_smem_limits()
{
    const size_t smem_big = sizeof(RowTable<HC_BIG>);
    TK_CUDA(cudaFuncSetAttribute(k_rows_fused<HC_S, RCAP_S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(sizeof(FusedSmem<HC_S>) * ROW_WARPS)));
    TK_CUDA(cudaFuncSetAttribute(k_rows_fused<HC_L, RCAP_L>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(sizeof(FusedSmem<HC_L>) * ROW_WARPS)));
    TK_CUDA(cudaFuncSetAttribute(k_rows_fused<HC_X, RCAP_X, STAGE_X>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(sizeof(FusedSmem<HC_X, STAGE_X>) * ROW_WARPS)));
    TK_CUDA(cudaFuncSetAttribute(k_rows_big<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_big));
    TK_CUDA(cudaFuncSetAttribute(k_rows_big<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_big));
}

int rows_grid(tk_ctx* ctx, int64_t N)
{
    const int64_t want = (N + ROW_WARPS - 1) / ROW_WARPS;
    return (int)std::min<int64_t>(want, (int64_t)ctx->num_sms * 8);
}
} // namespace

void assemble_rows_device(tk_ctx* ctx, int method, int64_t N, int k, int td, const int32_t* idx,
                          const double* weights, double shift, int64_t* row_ptr)
{
    cudaStream_t st = ctx->stream;
    const int64_t nk = N * (int64_t)k;
    if (nk >= (int64_t)1 << 31)
        throw Error(TK_ERR_UNSUPPORTED, "assembly supports N*k < 2^31");
    AsmState a = asm_state(ctx, method, N, k);
    mark(ctx, KM_ASM0);
    int* cnt = (int*)ctx->scratch.get("asm.cnt", sizeof(int) * (size_t)N * 2);
    int* fillc = cnt + N;
    const int g = 4 * ctx->num_sms;
    TK_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int) * (size_t)N * 2, st));
    TK_CUDA(cudaMemsetAsync(a.nbig, 0, 16, st));
    TK_CUDA(cudaMemsetAsync(a.row_big, 0, (size_t)N, st));
    unsigned* repeats = (unsigned*)ctx->scratch.get("asm.repeats", 16);
    TK_CUDA(cudaMemsetAsync(repeats, 0, 16, st));
    k_indeg<<<g, 256, 0, st>>>(idx, nk, N, k, cnt, repeats, ctx->dev_err);
    TK_CHECK_LAUNCH();
    scan_to_offsets(ctx, cnt, N, a.rptr);
    k_fill_rev<<<g, 256, 0, st>>>(idx, nk, N, a.rptr, fillc, a.rev);
    TK_CHECK_LAUNCH();
    k_sort_rev<<<g, 256, 0, st>>>(N, a.rptr, a.rev);
    TK_CHECK_LAUNCH();
    mark(ctx, KM_ASM_REV);
    set_smem_limits();
    if (widest_rows(k))
        k_rows_fused<HC_X, RCAP_X, STAGE_X><<<rows_grid(ctx, N), ROW_WARPS * 32,
                                              sizeof(FusedSmem<HC_X, STAGE_X>) * ROW_WARPS, st>>>(
            method, N, k, td, idx, weights, shift, a.rptr, a.rev, a.row_nnz, a.scol, a.sval, a.big, a.nbig,
            a.row_big, repeats);
    else if (wide_rows(method, k))
        k_rows_fused<HC_L, RCAP_L><<<rows_grid(ctx, N), ROW_WARPS * 32, sizeof(FusedSmem<HC_L>) * ROW_WARPS, st>>>(
            method, N, k, td, idx, weights, shift, a.rptr, a.rev, a.row_nnz, a.scol, a.sval, a.big, a.nbig,
            a.row_big, repeats);
    else
        k_rows_fused<HC_S, RCAP_S><<<rows_grid(ctx, N), ROW_WARPS * 32, sizeof(FusedSmem<HC_S>) * ROW_WARPS, st>>>(
            method, N, k, td, idx, weights, shift, a.rptr, a.rev, a.row_nnz, a.scol, a.sval, a.big, a.nbig,
            a.row_big, repeats);
    TK_CHECK_LAUNCH();
    k_rows_big<false><<<ctx->num_sms, 32, sizeof(RowTable<HC_BIG>), st>>>(method, N, k, td, idx, nullptr, 0.0,
                                                                           a.rptr, a.rev, a.row_nnz, nullptr,
                                                                           nullptr, nullptr, a.big, a.nbig,
                                                                           ctx->dev_err);
    TK_CHECK_LAUNCH();
    mark(ctx, KM_ASM_ROWS);
    scan_to_offsets(ctx, a.row_nnz, N, row_ptr);
}

void reverse_lists(tk_ctx* ctx, int64_t N, int k, const int32_t* idx, int64_t* rptr, int32_t* rev)
{
    cudaStream_t st = ctx->stream;
    const int64_t nk = N * (int64_t)k;
    if (nk >= (int64_t)1 << 31)
        throw Error(TK_ERR_UNSUPPORTED, "reverse lists support N*k < 2^31");
    int* cnt = (int*)ctx->scratch.get("rev.cnt", sizeof(int) * (size_t)N * 2);
    int* fillc = cnt + N;
    unsigned* repeats = (unsigned*)ctx->scratch.get("rev.repeats", 16);
    const int g = 4 * ctx->num_sms;
    TK_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int) * (size_t)N * 2, st));
    k_indeg<<<g, 256, 0, st>>>(idx, nk, N, k, cnt, repeats, ctx->dev_err);
    TK_CHECK_LAUNCH();
    scan_to_offsets(ctx, cnt, N, rptr);
    k_fill_rev<<<g, 256, 0, st>>>(idx, nk, N, rptr, fillc, rev);
    TK_CHECK_LAUNCH();
    k_sort_rev<<<g, 256, 0, st>>>(N, rptr, rev);
    TK_CHECK_LAUNCH();
}

int64_t assemble_rows(tk_ctx* ctx, int method, int64_t N, int k, int td, const int32_t* idx, const double* weights,
                      double shift, int64_t* row_ptr)
{
    assemble_rows_device(ctx, method, N, k, td, idx, weights, shift, row_ptr);
    TK_CUDA(cudaMemcpyAsync(ctx->host_i64, row_ptr + N, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
    TK_CUDA(cudaStreamSynchronize(ctx->stream));
    return ctx->host_i64[0];
}

void assemble_write(tk_ctx* ctx, int method, int64_t N, int k, int td, const int32_t* idx, const double* weights,
                    double shift, const int64_t* row_ptr, int32_t* col_idx, double* vals)
{
    cudaStream_t st = ctx->stream;
    AsmState a = asm_state(ctx, method, N, k);
    set_smem_limits();
    const int64_t warps = std::min<int64_t>(N, (int64_t)ctx->num_sms * 64);
    k_compact<<<(int)((warps + 7) / 8), 256, 0, st>>>(N, a.rcap, a.row_nnz, a.row_big, row_ptr, a.scol, a.sval,
                                                       col_idx, vals);
    TK_CHECK_LAUNCH();
    k_rows_big<true><<<ctx->num_sms, 32, sizeof(RowTable<HC_BIG>), st>>>(method, N, k, td, idx, weights, shift,
                                                                          a.rptr, a.rev, a.row_nnz, row_ptr, col_idx,
                                                                          vals, a.big, a.nbig, ctx->dev_err);
    TK_CHECK_LAUNCH();
    mark(ctx, KM_ASM_END);
}

} // namespace tk
