// nth_select.h -- the reference's neighbour selection: std::nth_element of
// libstdc++ (bits/stl_algo.h, GCC 13), which the reference calls at
// neighbors/neighbors.hpp:135-136 with the strict comparator of :28-34.
//
// Restated over a row's records held as two arrays in index order: the value
// d[m] (the exact squared distance, an order-preserving stand-in for the
// reference's FP64 kernel-trick distance) and the point jv[m]. The steps are
// those of the published libstdc++ source:
//   * __introselect: while the range holds more than 3 records, pick a pivot by
//     __move_median_to_first (first + 1, middle, last - 1) and split with the
//     unguarded Hoare partition; keep the side holding nth; past a depth of
//     2 floor(log2 n) finish with __heap_select and a swap; end with
//     __insertion_sort;
//   * only d[a] < d[b] is compared (the reference's distances_comparator).
// The unguarded scans rely on a strict weak order, which NaN distances would
// break; every scan is therefore bounded to its range, and a scan that would
// leave it sets `bad` instead.
//
// Plain C++ under g++ (the host test compares it with std::nth_element), host
// and device code under nvcc.
#pragma once

#include <cstdint>

#ifdef __CUDACC__
#define TK_HD __host__ __device__
#else
#define TK_HD
#endif

namespace tk {

// floor(log2 n) for n >= 1 (std::__lg)
TK_HD inline int floor_log2(int64_t n)
{
    int r = 0;
    while (n > 1)
    {
        n >>= 1;
        ++r;
    }
    return r;
}

struct NthSelect
{
    double* d;
    int32_t* jv;
    bool bad;

    TK_HD inline bool lt(int64_t a, int64_t b) const { return d[a] < d[b]; }
    TK_HD inline void swp(int64_t a, int64_t b)
    {
        const double td = d[a];
        d[a] = d[b];
        d[b] = td;
        const int32_t tj = jv[a];
        jv[a] = jv[b];
        jv[b] = tj;
    }

    // __move_median_to_first(result, a, b, c)
    TK_HD void median_to_first(int64_t result, int64_t a, int64_t b, int64_t c)
    {
        if (lt(a, b))
        {
            if (lt(b, c))
                swp(result, b);
            else if (lt(a, c))
                swp(result, c);
            else
                swp(result, a);
        }
        else if (lt(a, c))
            swp(result, a);
        else if (lt(b, c))
            swp(result, c);
        else
            swp(result, b);
    }

    // __unguarded_partition(first, last, pivot), scans bounded to [lo, hi): the
    // right-hand scan may stop on the pivot itself (lo = its position)
    TK_HD int64_t partition(int64_t first, int64_t last, int64_t pivot, int64_t lo, int64_t hi)
    {
        for (;;)
        {
            while (lt(first, pivot))
                if (++first >= hi)
                {
                    bad = true;
                    return lo;
                }
            --last;
            while (lt(pivot, last))
                if (--last < lo)
                {
                    bad = true;
                    return lo;
                }
            if (!(first < last))
                return first;
            swp(first, last);
            ++first;
        }
    }

    // __push_heap(first, hole, top, value) with value = (vd, vj)
    TK_HD void push_heap(int64_t first, int64_t hole, int64_t top, double vd, int32_t vj)
    {
        int64_t parent = (hole - 1) / 2;
        while (hole > top && d[first + parent] < vd)
        {
            d[first + hole] = d[first + parent];
            jv[first + hole] = jv[first + parent];
            hole = parent;
            parent = (hole - 1) / 2;
        }
        d[first + hole] = vd;
        jv[first + hole] = vj;
    }

    // __adjust_heap(first, hole, len, value)
    TK_HD void adjust_heap(int64_t first, int64_t hole, int64_t len, double vd, int32_t vj)
    {
        const int64_t top = hole;
        int64_t child = hole;
        while (child < (len - 1) / 2)
        {
            child = 2 * (child + 1);
            if (lt(first + child, first + (child - 1)))
                child--;
            d[first + hole] = d[first + child];
            jv[first + hole] = jv[first + child];
            hole = child;
        }
        if ((len & 1) == 0 && child == (len - 2) / 2)
        {
            child = 2 * (child + 1);
            d[first + hole] = d[first + (child - 1)];
            jv[first + hole] = jv[first + (child - 1)];
            hole = child - 1;
        }
        push_heap(first, hole, top, vd, vj);
    }

    // __heap_select(first, middle, last): __make_heap, then __pop_heap of every
    // later record smaller than the heap's top
    TK_HD void heap_select(int64_t first, int64_t middle, int64_t last)
    {
        const int64_t len = middle - first;
        if (len >= 2)
        {
            int64_t parent = (len - 2) / 2;
            for (;;)
            {
                adjust_heap(first, parent, len, d[first + parent], jv[first + parent]);
                if (parent == 0)
                    break;
                parent--;
            }
        }
        for (int64_t m = middle; m < last; ++m)
            if (lt(m, first))
            {
                const double vd = d[m];
                const int32_t vj = jv[m];
                d[m] = d[first];
                jv[m] = jv[first];
                adjust_heap(first, 0, len, vd, vj);
            }
    }

    // __insertion_sort(first, last) with __unguarded_linear_insert
    TK_HD void insertion_sort(int64_t first, int64_t last)
    {
        if (first == last)
            return;
        for (int64_t m = first + 1; m != last; ++m)
        {
            const double vd = d[m];
            const int32_t vj = jv[m];
            if (vd < d[first])
            {
                for (int64_t q = m; q > first; --q)
                {
                    d[q] = d[q - 1];
                    jv[q] = jv[q - 1];
                }
                d[first] = vd;
                jv[first] = vj;
            }
            else
            {
                int64_t q = m;
                while (vd < d[q - 1])
                {
                    d[q] = d[q - 1];
                    jv[q] = jv[q - 1];
                    if (--q <= first)
                    {
                        bad = true;
                        return;
                    }
                }
                d[q] = vd;
                jv[q] = vj;
            }
        }
    }

    // std::nth_element(0, nth, n)
    TK_HD void nth_element(int64_t n, int64_t nth)
    {
        if (n == 0 || nth == n)
            return;
        int64_t first = 0, last = n;
        int depth = 2 * floor_log2(n);
        while (last - first > 3)
        {
            if (depth == 0)
            {
                heap_select(first, nth + 1, last);
                swp(first, nth);
                return;
            }
            --depth;
            const int64_t mid = first + (last - first) / 2;
            median_to_first(first, first + 1, mid, last - 1);
            const int64_t cut = partition(first + 1, last, first, first, last);
            if (bad)
                return;
            if (cut <= nth)
                first = cut;
            else
                last = cut;
        }
        insertion_sort(first, last);
    }
};

} // namespace tk
