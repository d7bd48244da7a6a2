// screen_common.cuh -- pieces shared by the FP32 and tensor-core distance screens.
#pragma once

#include <cstdint>

namespace tk {

// Candidate tiles are visited starting at the query block's own tile and then
// alternately above and below it. After the spatial sort this visits the
// query's spatial neighbourhood first, so per-row thresholds are tight after
// the first tiles and later tiles rarely insert.
struct ZigZag
{
    int up, down, ntiles, step;
    __device__ __forceinline__ ZigZag(int start, int n) : up(start), down(start - 1), ntiles(n), step(0) {}
    __device__ __forceinline__ int next()
    {
        int t;
        const bool take_up = (up < ntiles) && ((step & 1) == 0 || down < 0);
        if (take_up)
            t = up++;
        else
            t = down--;
        ++step;
        return t;
    }
};

// Sorted (ascending) insertion into a per-row list held in shared memory.
// The last entry is dropped. Equal values keep arrival order.
template <int KC>
__device__ __forceinline__ void list_insert(float* vals, int32_t* ids, float v, int32_t id)
{
    if (!(v < vals[KC - 1]))
        return;
    int pos = KC - 1;
    while (pos > 0 && vals[pos - 1] > v)
    {
        vals[pos] = vals[pos - 1];
        ids[pos] = ids[pos - 1];
        --pos;
    }
    vals[pos] = v;
    ids[pos] = id;
}

} // namespace tk
