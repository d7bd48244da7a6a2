// connectivity.cu -- is every vertex reachable from vertex 0 along kNN out-edges?
//
// Same predicate as the reference's iterative DFS (neighbors/connected.hpp:19-62),
// evaluated as a level-synchronous BFS inside one CTA: the visited set is a
// bitmap, frontiers are arrays in global memory. The CTA never waits on another
// CTA, and the level loop is bounded by N (a BFS has at most N levels), so the
// kernel always terminates.
#include "tk_internal.h"

namespace tk {
namespace {

__global__ void __launch_bounds__(1024) k_bfs(int64_t N, int k, const int32_t* __restrict__ idx, unsigned* visited,
                                              int32_t* qa, int32_t* qb, unsigned long long* out_count,
                                              unsigned* err)
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
