// connectivity.cu -- is every vertex reachable from vertex 0 along kNN out-edges?
//
// Same predicate as the reference's iterative DFS (neighbors/connected.hpp:19-62).
// check_connected evaluates it in two steps:
//   1. k_in_edges marks every vertex that some list names; a vertex other than 0
//      with no in-edge cannot be reached, so any such vertex answers "not
//      connected" without a traversal (the common case of large kNN graphs, whose
//      anti-hubs are nobody's neighbour);
//   2. otherwise a level-synchronous BFS over the whole GPU: a cooperative launch
//      (every CTA resident), frontiers in global memory, a visited bitmap, and a
//      grid barrier between levels. Every barrier wait is bounded (2 s, the
//      global timer): on expiry the CTA records DEV_ERR_TIMEOUT, raises an abort
//      flag that every waiting CTA polls, and all CTAs return. The level loop is
//      bounded by N (a BFS has at most N levels).
// The allocation-free entry point keeps the one-CTA BFS (bfs_levels): its state
// must fit its fixed static scratch and it takes no cooperative launch.
#include <algorithm>
#include <cstdarg>
#include <cstring>
#include <mutex>

#include "tk_internal.h"

namespace tk {
namespace {

// Level-synchronous BFS from vertex 0 by the whole CTA. visited must be clear
// on entry; index errors are OR-ed into *err. Returns the number of vertices
// reached (valid in thread 0).
__device__ __forceinline__ unsigned long long bfs_levels(int64_t N, int k, const int32_t* __restrict__ idx,
                                                         unsigned* visited, int32_t* qa, int32_t* qb, unsigned* err)
{
    __shared__ unsigned long long cur_n, next_n, total;
    if (threadIdx.x == 0)
    {
        visited[0] = 1u;
        qa[0] = 0;
        cur_n = 1;
        total = 1;
    }
    __syncthreads();
    for (int64_t level = 0; level < N; ++level)
    {
        const unsigned long long n = cur_n;
        if (n == 0)
            break;
        if (threadIdx.x == 0)
            next_n = 0;
        __syncthreads();
        const unsigned long long work = n * (unsigned long long)k;
        for (unsigned long long t = threadIdx.x; t < work; t += blockDim.x)
        {
            const int32_t v = qa[t / k];
            const int32_t nb = idx[(int64_t)v * k + (int)(t % k)];
            if (nb < 0 || nb >= N)
            {
                atomicOr(err, DEV_ERR_BOUNDS);
                continue;
            }
            const unsigned bit = 1u << (nb & 31);
            if ((__ldcg(&visited[nb >> 5]) & bit) == 0u)
            {
                const unsigned old = atomicOr(&visited[nb >> 5], bit);
                if ((old & bit) == 0u)
                {
                    const unsigned long long pos = atomicAdd(&next_n, 1ull);
                    qb[pos] = nb;
                }
            }
        }
        __syncthreads();
        if (threadIdx.x == 0)
        {
            cur_n = next_n;
            total += next_n;
        }
        int32_t* tmp = qa;
        qa = qb;
        qb = tmp;
        __syncthreads();
    }
    return total;
}

// ---- whole-GPU connectivity check --------------------------------------------

// Device state of one check (cleared by the host before the launches).
struct BfsState
{
    unsigned long long reached;  // vertices reached (written by CTA 0)
    unsigned orphans;            // vertices other than 0 without an in-edge
    unsigned front[3];           // frontier sizes, triple-buffered by level
    unsigned bar_count;          // grid barrier: arrivals
    unsigned bar_gen;            // grid barrier: generation
    unsigned abort;              // a CTA gave up waiting
};

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Marks every vertex named by some neighbour list; bad indices are reported.
__global__ void k_in_edges(const int32_t* __restrict__ idx, int64_t nk, int64_t N, unsigned* has_in, unsigned* err)
{
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nk; e += (int64_t)gridDim.x * blockDim.x)
    {
        const int j = idx[e];
        if (j < 0 || j >= N)
        {
            atomicOr(err, DEV_ERR_BOUNDS);
            continue;
        }
        const unsigned bit = 1u << (j & 31);
        if ((__ldcg(&has_in[j >> 5]) & bit) == 0u)
            atomicOr(&has_in[j >> 5], bit);
    }
}

// Counts the vertices 1..N-1 that no list names.
__global__ void k_orphans(const unsigned* __restrict__ has_in, int64_t N, BfsState* st)
{
    const int64_t words = (N + 31) / 32;
    unsigned c = 0;
    for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < words; w += (int64_t)gridDim.x * blockDim.x)
    {
        unsigned valid = (w == words - 1 && (N & 31)) ? ((1u << (N & 31)) - 1u) : 0xffffffffu;
        if (w == 0)
            valid &= ~1u;  // vertex 0 is the start
        c += __popc(~has_in[w] & valid);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c)
        atomicAdd(&st->orphans, c);
}

// Grid barrier for a cooperative launch, with a bounded wait. Returns false when
// this CTA, or another, gave up (the caller returns).
__device__ bool grid_barrier(BfsState* st, unsigned nblocks, unsigned* err)
{
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        ok = 1;
        volatile unsigned* gen = &st->bar_gen;
        volatile unsigned* abort = &st->abort;
        const unsigned g = *gen;
        __threadfence();
        if (atomicAdd(&st->bar_count, 1u) == nblocks - 1)
        {
            atomicExch(&st->bar_count, 0u);
            __threadfence();
            atomicAdd(&st->bar_gen, 1u);
        }
        else
        {
            const uint64_t t0 = global_ns();
            while (*gen == g)
            {
                if (*abort)
                {
                    ok = 0;
                    break;
                }
                if (global_ns() - t0 > 2000000000ull)
                {
                    atomicOr(err, DEV_ERR_TIMEOUT);
                    atomicExch(&st->abort, 1u);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

// Level-synchronous BFS from vertex 0 over the whole grid (cooperative launch).
// The visited bitmap and the counters are cleared by the host. Level L reads the
// frontier size front[L % 3] and its vertices from one array, appends newly
// reached vertices to the other array and to front[(L + 1) % 3], and CTA 0
// clears front[(L + 2) % 3], last read before the previous barrier.
__global__ void __launch_bounds__(512) k_bfs_grid(int64_t N, int k, const int32_t* __restrict__ idx,
                                                  unsigned* visited, int32_t* qa, int32_t* qb, BfsState* st,
                                                  unsigned* err)
{
    if (__ldcg(&st->orphans) != 0u)
        return;  // answered by the in-edge test
    const unsigned nblocks = gridDim.x;
    const int lane = threadIdx.x & 31;
    if (blockIdx.x == 0 && threadIdx.x == 0)
    {
        visited[0] |= 1u;
        qa[0] = 0;
        st->front[0] = 1u;
    }
    if (!grid_barrier(st, nblocks, err))
        return;
    unsigned long long total = 0;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
    for (int64_t level = 0; level < N; ++level)
    {
        const unsigned cur = __ldcg(&st->front[level % 3]);
        if (cur == 0u)
            break;
        total += cur;
        if (blockIdx.x == 0 && threadIdx.x == 0)
            st->front[(level + 2) % 3] = 0u;
        const int32_t* in = (level & 1) ? qb : qa;
        int32_t* out = (level & 1) ? qa : qb;
        unsigned* next = &st->front[(level + 1) % 3];
        const int64_t work = (int64_t)cur * k;
        // the loop runs a whole number of warp passes so that the warp-aggregated
        // append below sees every lane
        for (int64_t t0 = tid - lane; t0 < work; t0 += nthreads)
        {
            const int64_t t = t0 + lane;
            bool fresh = false;
            int32_t nb = 0;
            if (t < work)
            {
                const int32_t v = __ldcg(&in[t / k]);
                nb = idx[(int64_t)v * k + (int)(t % k)];
                if (nb < 0 || nb >= N)
                    atomicOr(err, DEV_ERR_BOUNDS);
                else
                {
                    const unsigned bit = 1u << (nb & 31);
                    if ((__ldcg(&visited[nb >> 5]) & bit) == 0u)
                        fresh = (atomicOr(&visited[nb >> 5], bit) & bit) == 0u;
                }
            }
            const unsigned m = __ballot_sync(0xffffffffu, fresh);
            if (m)
            {
                unsigned base = 0;
                if (lane == __ffs(m) - 1)
                    base = atomicAdd(next, (unsigned)__popc(m));
                base = __shfl_sync(0xffffffffu, base, __ffs(m) - 1);
                if (fresh)
                    out[base + __popc(m & ((1u << lane) - 1u))] = nb;
            }
        }
        if (!grid_barrier(st, nblocks, err))
            return;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0)
        st->reached = total;
}

// Failure-path self-test of grid_barrier: CTA 0 returns without arriving, so the
// other CTAs' waits expire; each records DEV_ERR_TIMEOUT and returns.
__global__ void __launch_bounds__(512) k_barrier_selftest(BfsState* st, unsigned* err)
{
    if (blockIdx.x == 0)
        return;
    if (grid_barrier(st, gridDim.x, err) && threadIdx.x == 0)
        atomicExch(&st->orphans, 2u);  // the barrier completed: not expected
}

} // namespace

int barrier_selftest(tk_ctx* ctx)
{
    cudaStream_t st = ctx->stream;
    BfsState* state = (BfsState*)ctx->scratch.get("bfs.state", sizeof(BfsState));
    TK_CUDA(cudaMemsetAsync(state, 0, sizeof(BfsState), st));
    int per_sm = 0;
    TK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_barrier_selftest, 512, 0));
    const int grid = std::max(2, std::max(1, std::min(per_sm, 2)) * ctx->num_sms);
    void* args[] = {(void*)&state, (void*)&ctx->dev_err};
    TK_CUDA(cudaLaunchCooperativeKernel((const void*)k_barrier_selftest, dim3(grid), dim3(512), args, 0, st));
    TK_CHECK_LAUNCH();
    BfsState h{};
    TK_CUDA(cudaMemcpyAsync(ctx->host_i64, state, sizeof(BfsState), cudaMemcpyDeviceToHost, st));
    TK_CUDA(cudaStreamSynchronize(st));
    std::memcpy(&h, ctx->host_i64, sizeof(BfsState));
    return h.orphans == 2u ? 2 : (h.abort ? 1 : 0);
}

bool check_connected(tk_ctx* ctx, int64_t N, int k, const int32_t* idx)
{
    cudaStream_t st = ctx->stream;
    const size_t words = (size_t)((N + 31) / 32);
    // visited and has_in share one allocation (cleared together)
    unsigned* visited = (unsigned*)ctx->scratch.get("bfs.visited", 2 * sizeof(unsigned) * words);
    unsigned* has_in = visited + words;
    int32_t* qa = (int32_t*)ctx->scratch.get("bfs.qa", sizeof(int32_t) * (size_t)N);
    int32_t* qb = (int32_t*)ctx->scratch.get("bfs.qb", sizeof(int32_t) * (size_t)N);
    BfsState* state = (BfsState*)ctx->scratch.get("bfs.state", sizeof(BfsState));
    TK_CUDA(cudaMemsetAsync(visited, 0, 2 * sizeof(unsigned) * words, st));
    TK_CUDA(cudaMemsetAsync(state, 0, sizeof(BfsState), st));
    const int64_t nk = N * (int64_t)k;
    k_in_edges<<<(int)std::min<int64_t>((nk + 255) / 256, 8 * ctx->num_sms), 256, 0, st>>>(idx, nk, N, has_in,
                                                                                          ctx->dev_err);
    TK_CHECK_LAUNCH();
    k_orphans<<<(int)std::min<int64_t>(((int64_t)words + 255) / 256, 2 * ctx->num_sms), 256, 0, st>>>(has_in, N,
                                                                                                  state);
    TK_CHECK_LAUNCH();
    // every CTA of the BFS must be resident at once (cooperative launch)
    int per_sm = 0;
    TK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bfs_grid, 512, 0));
    const int grid = std::max(1, std::min(per_sm, 2)) * ctx->num_sms;
    void* args[] = {(void*)&N, (void*)&k, (void*)&idx, (void*)&visited, (void*)&qa, (void*)&qb, (void*)&state,
                    (void*)&ctx->dev_err};
    TK_CUDA(cudaLaunchCooperativeKernel((const void*)k_bfs_grid, dim3(grid), dim3(512), args, 0, st));
    TK_CHECK_LAUNCH();
    BfsState h{};
    TK_CUDA(cudaMemcpyAsync(ctx->host_i64, state, sizeof(BfsState), cudaMemcpyDeviceToHost, st));
    TK_CUDA(cudaStreamSynchronize(st));
    std::memcpy(&h, ctx->host_i64, sizeof(BfsState));
    if (h.orphans > 0)
        return false;
    return (int64_t)h.reached == N;
}

} // namespace tk

// ---------------------------------------------------------------------------
// Allocation-free variant: tk_check_connected_noalloc.
//
// tk_check_connected takes its frontier and visited arrays from the context's
// grow-only arena, which calls cudaMalloc on first use and, when a larger graph
// arrives, synchronises the whole device and calls cudaFree. Some callers can
// do neither: a process that has handed the free HBM to a caching allocator
// (PyTorch's keeps freed blocks, so a fresh cudaMalloc can fail while the
// process still has room), or a pipeline that keeps other streams of the same
// GPU busy and cannot accept the device-wide synchronisation of cudaFree. For
// them the BFS scratch lives in one fixed file-scope device array, sized for
// graphs of up to TK_NOALLOC_MAX_POINTS vertices.
// ---------------------------------------------------------------------------

namespace tk {
namespace {

// Layout of the static scratch (byte offsets, each 256-aligned):
//   [0, 256)          head: reached-vertex count (u64) and the error word (u32)
//   visited           one bit per vertex
//   qa, qb            the two frontier arrays, one int32 per vertex
constexpr int64_t NA_MAX = TK_NOALLOC_MAX_POINTS;
constexpr size_t NA_OFF_VISITED = 256;
constexpr size_t NA_OFF_QA = NA_OFF_VISITED + (size_t)(NA_MAX / 32) * sizeof(unsigned);
constexpr size_t NA_OFF_QB = NA_OFF_QA + (size_t)NA_MAX * sizeof(int32_t);
constexpr size_t NA_BYTES = NA_OFF_QB + (size_t)NA_MAX * sizeof(int32_t);
static_assert(NA_MAX % 32 == 0 && NA_OFF_QA % 256 == 0 && NA_OFF_QB % 256 == 0, "scratch layout");
static_assert(NA_BYTES == TK_NOALLOC_SCRATCH_BYTES, "header and layout disagree");

struct NaHead
{
    unsigned long long count;
    unsigned err;
    unsigned pad;
};

// One instance per device; shared by every call on that device.
static __device__ __align__(256) unsigned char g_bfs_scratch[NA_BYTES];

// Same BFS as k_bfs; the kernel itself clears what must start at zero (the
// visited bits of the first N vertices and the error word), so the array needs
// no memset between calls. The frontier arrays and the count are written
// before they are read.
__global__ void __launch_bounds__(1024) k_bfs_noalloc(int64_t N, int k, const int32_t* __restrict__ idx,
                                                      unsigned char* scratch)
{
    NaHead* head = reinterpret_cast<NaHead*>(scratch);
    unsigned* visited = reinterpret_cast<unsigned*>(scratch + NA_OFF_VISITED);
    int32_t* qa = reinterpret_cast<int32_t*>(scratch + NA_OFF_QA);
    int32_t* qb = reinterpret_cast<int32_t*>(scratch + NA_OFF_QB);
    const int64_t words = (N + 31) / 32;
    for (int64_t w = threadIdx.x; w < words; w += blockDim.x)
        visited[w] = 0u;
    if (threadIdx.x == 0)
        head->err = 0u;
    __syncthreads();
    const unsigned long long total = bfs_levels(N, k, idx, visited, qa, qb, &head->err);
    if (threadIdx.x == 0)
        head->count = total;
}

constexpr int NA_MAX_DEVICES = 64;
std::atomic<unsigned char*> g_na_ptr[NA_MAX_DEVICES];
std::mutex g_na_setup;

// Formats into the caller's buffer; never allocates.
int na_fail(char* msg, size_t msg_len, int status, const char* fmt, ...)
{
    if (msg && msg_len)
    {
        va_list ap;
        va_start(ap, fmt);
        std::vsnprintf(msg, msg_len, fmt, ap);
        va_end(ap);
    }
    return status;
}

// Restores the calling thread's current device on every exit path.
struct DeviceGuard
{
    int prev = -1;
    ~DeviceGuard()
    {
        if (prev >= 0)
            cudaSetDevice(prev);
    }
};

} // namespace
} // namespace tk

extern "C" int tk_check_connected_noalloc(int device, void* stream, int64_t N, int k, const int32_t* idx,
                                          int* connected, char* msg, size_t msg_len)
{
    using namespace tk;
    if (msg && msg_len)
        msg[0] = '\0';
    if (N <= 0)
        return na_fail(msg, msg_len, TK_ERR_NO_DATA, "No data");
    if (k < 1 || !idx || !connected)
        return na_fail(msg, msg_len, TK_ERR_INVALID_ARG, "bad arguments (k >= 1, idx and connected non-NULL)");
    if (N > NA_MAX)
        return na_fail(msg, msg_len, TK_ERR_INVALID_ARG,
                       "N = %lld exceeds the limit of tk_check_connected_noalloc (%lld points, %zu bytes of "
                       "static device scratch); use tk_check_connected",
                       (long long)N, (long long)NA_MAX, NA_BYTES);
    if (device < 0 || device >= NA_MAX_DEVICES)
        return na_fail(msg, msg_len, TK_ERR_NO_DEVICE, "device %d out of range", device);

    DeviceGuard guard;
    cudaError_t e = cudaGetDevice(&guard.prev);
    if (e != cudaSuccess)
    {
        guard.prev = -1;
        cudaGetLastError();
        return na_fail(msg, msg_len, TK_ERR_NO_DEVICE, "no CUDA device: %s", cudaGetErrorString(e));
    }
    if ((e = cudaSetDevice(device)) != cudaSuccess)
    {
        cudaGetLastError();
        return na_fail(msg, msg_len, TK_ERR_NO_DEVICE, "cudaSetDevice(%d): %s", device, cudaGetErrorString(e));
    }

    // Set-up, once per device: the device address of this device's instance of
    // the array, and the kernel's module loaded now rather than at first launch.
    unsigned char* scratch = g_na_ptr[device].load(std::memory_order_acquire);
    if (!scratch)
    {
        std::lock_guard<std::mutex> lock(g_na_setup);
        scratch = g_na_ptr[device].load(std::memory_order_relaxed);
        if (!scratch)
        {
            int major = 0, minor = 0;
            cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device);
            cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, device);
            if (!(major == 10 && minor == 3))
                return na_fail(msg, msg_len, TK_ERR_NO_DEVICE, "device %d is sm_%d%d, this library needs sm_103",
                               device, major, minor);
            void* p = nullptr;
            if ((e = cudaGetSymbolAddress(&p, g_bfs_scratch)) != cudaSuccess || !p)
            {
                cudaGetLastError();
                return na_fail(msg, msg_len, TK_ERR_CUDA, "cudaGetSymbolAddress of the BFS scratch: %s",
                               cudaGetErrorString(e));
            }
            cudaFuncAttributes fa;
            if ((e = cudaFuncGetAttributes(&fa, k_bfs_noalloc)) != cudaSuccess)
            {
                cudaGetLastError();
                return na_fail(msg, msg_len, TK_ERR_CUDA, "loading the BFS kernel: %s", cudaGetErrorString(e));
            }
            scratch = static_cast<unsigned char*>(p);
            g_na_ptr[device].store(scratch, std::memory_order_release);
        }
    }

    cudaPointerAttributes pa;
    if (cudaPointerGetAttributes(&pa, idx) != cudaSuccess)
    {
        cudaGetLastError();
        pa.type = cudaMemoryTypeUnregistered;
    }
    const bool on_device = (pa.type == cudaMemoryTypeDevice && pa.device == device) ||
                           pa.type == cudaMemoryTypeManaged;
    if (!on_device)
        return na_fail(msg, msg_len, TK_ERR_INVALID_ARG,
                       "idx must be device (or managed) memory of device %d: this entry point copies nothing",
                       device);

    cudaStream_t st = static_cast<cudaStream_t>(stream);
    k_bfs_noalloc<<<1, 1024, 0, st>>>(N, k, idx, scratch);
    if ((e = cudaGetLastError()) != cudaSuccess)
        return na_fail(msg, msg_len, TK_ERR_CUDA, "BFS launch: %s", cudaGetErrorString(e));
    g_kernel_launches.fetch_add(1, std::memory_order_relaxed);

    NaHead head{};
    if ((e = cudaMemcpyAsync(&head, scratch, sizeof(NaHead), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess)
    {
        cudaGetLastError();
        return na_fail(msg, msg_len, TK_ERR_CUDA, "BFS result: %s", cudaGetErrorString(e));
    }
    if (head.err & DEV_ERR_BOUNDS)
        return na_fail(msg, msg_len, TK_ERR_INVALID_ARG, "device-side check failed: index out of range;");
    if (head.err)
        return na_fail(msg, msg_len, TK_ERR_INTERNAL, "device-side check failed (0x%x)", head.err);
    *connected = (int64_t)head.count == N ? 1 : 0;
    return TK_OK;
}
