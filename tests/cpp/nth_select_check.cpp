// The device restatement of libstdc++'s std::nth_element (tapkee_gb300/csrc/
// nth_select.h), compiled with g++ and compared with std::nth_element itself on
// the CPU: the whole final arrangement of the records must be identical, not
// only the selected set. Inputs: tie-heavy random values, sorted, reversed and
// constant arrays, and inputs from McIlroy's quicksort adversary ("A Killer
// Adversary for Quicksort", 1999), which drive the introselect past its depth
// limit into the heap-select branch. heap_select is also compared with
// libstdc++'s std::__heap_select directly. Prints "ok".
#include <algorithm>
#include <cstdio>
#include <utility>
#include <vector>

#include "nth_select.h"

namespace {

int failures = 0;
int heap_paths = 0;

unsigned long long state = 0x9E3779B97F4A7C15ull;
unsigned long long next_u64()  // xorshift64*
{
    state ^= state >> 12;
    state ^= state << 25;
    state ^= state >> 27;
    return state * 0x2545F4914F6CDD1Dull;
}

using Rec = std::pair<int32_t, double>;

// Runs both selections on the values v (records in index order) and compares
// the final arrangements.
bool compare(const std::vector<double>& v, int64_t nth, const char* what)
{
    const int64_t n = (int64_t)v.size();
    std::vector<Rec> ref(n);
    for (int64_t m = 0; m < n; ++m)
        ref[m] = {(int32_t)m, v[m]};
    std::nth_element(ref.begin(), ref.begin() + nth, ref.end(),
                     [](const Rec& l, const Rec& r) { return l.second < r.second; });
    std::vector<double> d(v);
    std::vector<int32_t> jv(n);
    for (int64_t m = 0; m < n; ++m)
        jv[m] = (int32_t)m;
    tk::NthSelect S{d.data(), jv.data(), false};
    S.nth_element(n, nth);
    bool ok = !S.bad;
    for (int64_t m = 0; m < n && ok; ++m)
        ok = ref[m].first == jv[m] && ref[m].second == d[m];
    if (!ok)
    {
        std::fprintf(stderr, "FAILED %s: n=%lld nth=%lld bad=%d\n", what, (long long)n, (long long)nth, (int)S.bad);
        ++failures;
    }
    return ok;
}

// McIlroy's adversary: values are assigned lazily ("gas" until frozen) so that
// every partition of a median-of-three quicksort is as unbalanced as possible.
std::vector<double> adversary(int64_t n, int64_t nth)
{
    std::vector<int64_t> val(n), ptr(n);
    const int64_t gas = n;
    int64_t nsolid = 0, candidate = 0;
    for (int64_t m = 0; m < n; ++m)
    {
        val[m] = gas;
        ptr[m] = m;
    }
    std::nth_element(ptr.begin(), ptr.begin() + nth, ptr.end(), [&](int64_t x, int64_t y) {
        if (val[x] == gas && val[y] == gas)
        {
            if (x == candidate)
                val[x] = nsolid++;
            else
                val[y] = nsolid++;
        }
        if (val[x] == gas)
            candidate = x;
        else if (val[y] == gas)
            candidate = y;
        return val[x] < val[y];
    });
    std::vector<double> v(n);
    for (int64_t m = 0; m < n; ++m)
        v[m] = (double)val[m];
    return v;
}

// Whether a selection of v at nth reaches the depth limit (instrumented copy of
// the loop's control flow).
bool reaches_depth_limit(const std::vector<double>& v, int64_t nth)
{
    std::vector<double> d(v);
    std::vector<int32_t> jv(v.size());
    tk::NthSelect S{d.data(), jv.data(), false};
    int64_t first = 0, last = (int64_t)v.size();
    int depth = 2 * tk::floor_log2(last);
    while (last - first > 3)
    {
        if (depth == 0)
            return true;
        --depth;
        const int64_t mid = first + (last - first) / 2;
        S.median_to_first(first, first + 1, mid, last - 1);
        const int64_t cut = S.partition(first + 1, last, first, first, last);
        if (cut <= nth)
            first = cut;
        else
            last = cut;
    }
    return false;
}

void check_heap_select(int64_t n, int64_t middle, int distinct)
{
    std::vector<double> v(n);
    for (auto& x : v)
        x = (double)(next_u64() % (unsigned)distinct);
    std::vector<Rec> ref(n);
    for (int64_t m = 0; m < n; ++m)
        ref[m] = {(int32_t)m, v[m]};
    auto cmp = [](const Rec& l, const Rec& r) { return l.second < r.second; };
    std::__heap_select(ref.begin(), ref.begin() + middle, ref.end(), __gnu_cxx::__ops::__iter_comp_iter(cmp));
    std::vector<double> d(v);
    std::vector<int32_t> jv(n);
    for (int64_t m = 0; m < n; ++m)
        jv[m] = (int32_t)m;
    tk::NthSelect S{d.data(), jv.data(), false};
    S.heap_select(0, middle, n);
    for (int64_t m = 0; m < n; ++m)
        if (ref[m].first != jv[m] || ref[m].second != d[m])
        {
            std::fprintf(stderr, "FAILED heap_select n=%lld middle=%lld\n", (long long)n, (long long)middle);
            ++failures;
            return;
        }
}

} // namespace

int main()
{
    // tie-heavy random values, every nth of small arrays
    for (int64_t n = 1; n <= 40; ++n)
        for (int distinct : {1, 2, 3, 5, 1000})
            for (int64_t nth = 0; nth <= n; ++nth)
            {
                std::vector<double> v(n);
                for (auto& x : v)
                    x = (double)(next_u64() % (unsigned)distinct);
                compare(v, nth, "small random");
            }
    // larger arrays at the reference's nth = k + 1
    for (int rep = 0; rep < 400; ++rep)
    {
        const int64_t n = 2 + (int64_t)(next_u64() % 5000);
        const int distinct = (int)(1 + next_u64() % 50);
        const int64_t k = 1 + (int64_t)(next_u64() % std::min<int64_t>(n - 1, 64));
        std::vector<double> v(n);
        for (auto& x : v)
            x = (double)(next_u64() % (unsigned)distinct);
        v[next_u64() % n] = 0.0;
        compare(v, k + 1 <= n ? k + 1 : n, "random");
    }
    // structured orders
    for (int64_t n : {4, 5, 17, 100, 1001, 4096})
        for (int64_t nth : {(int64_t)0, (int64_t)1, n / 3, n - 1})
        {
            std::vector<double> a(n), b(n), c(n, 7.0), e(n);
            for (int64_t m = 0; m < n; ++m)
            {
                a[m] = (double)m;
                b[m] = (double)(n - m);
                e[m] = (double)std::min(m, n - 1 - m);  // organ pipe
            }
            compare(a, nth, "sorted");
            compare(b, nth, "reversed");
            compare(c, nth, "constant");
            compare(e, nth, "organ pipe");
        }
    // adversarial inputs: the heap-select branch
    for (int64_t n : {64, 500, 2000, 10000})
        for (int64_t nth : {(int64_t)3, (int64_t)13, n / 2})
        {
            const std::vector<double> v = adversary(n, nth);
            if (reaches_depth_limit(v, nth))
                ++heap_paths;
            compare(v, nth, "adversary");
        }
    if (heap_paths == 0)
    {
        std::fprintf(stderr, "FAILED: no adversarial input reached the depth limit\n");
        ++failures;
    }
    for (int rep = 0; rep < 300; ++rep)
    {
        const int64_t n = 1 + (int64_t)(next_u64() % 300);
        const int64_t middle = 1 + (int64_t)(next_u64() % n);
        check_heap_select(n, middle, (int)(1 + next_u64() % 20));
    }
    if (failures)
        return 1;
    std::printf("ok\n");
    return 0;
}
