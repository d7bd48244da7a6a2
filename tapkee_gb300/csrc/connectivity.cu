// connectivity.cu -- is every vertex reachable from vertex 0 along kNN out-edges?
//
// Same predicate as the reference's iterative DFS (neighbors/connected.hpp:19-62),
// evaluated as a level-synchronous BFS inside one CTA: the visited set is a
// bitmap, frontiers are arrays in global memory. The CTA never waits on another
// CTA, and the level loop is bounded by N (a BFS has at most N levels), so the
// kernel always terminates.
#include <cstdarg>
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

__global__ void __launch_bounds__(1024) k_bfs(int64_t N, int k, const int32_t* __restrict__ idx, unsigned* visited,
                                              int32_t* qa, int32_t* qb, unsigned long long* out_count,
                                              unsigned* err)
{
    const unsigned long long total = bfs_levels(N, k, idx, visited, qa, qb, err);
    if (threadIdx.x == 0)
        *out_count = total;
}

} // namespace

bool check_connected(tk_ctx* ctx, int64_t N, int k, const int32_t* idx)
{
    cudaStream_t st = ctx->stream;
    const size_t words = (size_t)((N + 31) / 32);
    unsigned* visited = (unsigned*)ctx->scratch.get("bfs.visited", sizeof(unsigned) * words);
    int32_t* qa = (int32_t*)ctx->scratch.get("bfs.qa", sizeof(int32_t) * (size_t)N);
    int32_t* qb = (int32_t*)ctx->scratch.get("bfs.qb", sizeof(int32_t) * (size_t)N);
    unsigned long long* cnt = (unsigned long long*)ctx->scratch.get("bfs.count", 16);
    TK_CUDA(cudaMemsetAsync(visited, 0, sizeof(unsigned) * words, st));
    k_bfs<<<1, 1024, 0, st>>>(N, k, idx, visited, qa, qb, cnt, ctx->dev_err);
    TK_CHECK_LAUNCH();
    TK_CUDA(cudaMemcpyAsync(ctx->host_i64, cnt, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    TK_CUDA(cudaStreamSynchronize(st));
    return (int64_t)ctx->host_i64[0] == N;
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
