// facade_check.cpp -- exercises include/tapkee_gb300.hpp the way the reference's
// test/unit/interface.cpp exercises tapkee::with(...).embedUsing(...).
//
//   facade_check host                  keyword handling and errors without a GPU
//   facade_check gpu <X.bin> <N> <D> <out_prefix>
//                                      C1-style LLE run on device 0; writes the
//                                      operator arrays as raw binaries, plus the
//                                      error semantics of the chain on a GPU
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "tapkee_gb300.hpp"

using namespace tapkee_gb300;
using namespace tapkee_gb300::keywords;

namespace {

int failures = 0;

#define CHECK(cond)                                                                                   \
    do                                                                                                \
    {                                                                                                 \
        if (!(cond))                                                                                  \
        {                                                                                             \
            std::fprintf(stderr, "FAILED %s at line %d\n", #cond, __LINE__);                          \
            ++failures;                                                                               \
        }                                                                                             \
    } while (0)

template <class E, class F>
bool throws(F f)
{
    try
    {
        f();
    }
    catch (const E&)
    {
        return true;
    }
    catch (...)
    {
        return false;
    }
    return false;
}

template <class T>
void dump(const std::string& path, const std::vector<T>& v)
{
    std::ofstream f(path, std::ios::binary);
    f.write(reinterpret_cast<const char*>(v.data()), (std::streamsize)(v.size() * sizeof(T)));
}

int host_checks()
{
    // keyword values land in the parameter set; defaults are the reference's
    ParametersSet p = (method = KernelLocallyLinearEmbedding, num_neighbors = 12, klle_shift = 1e-2);
    CHECK(p.values.method == TK_METHOD_KLLE);
    CHECK(p.values.num_neighbors == 12);
    CHECK(p.values.klle_shift == 1e-2);
    CHECK(p.values.target_dimension == 2);
    CHECK(p.values.nullspace_shift == 1e-9);
    CHECK(p.values.check_connectivity == 1);
    // a parameter given twice (embed.hpp:134-136)
    CHECK(throws<multiple_parameter_error>([] { (void)(num_neighbors = 5, num_neighbors = 6); }));
    // no method: the reference's default (PassThru) does not run on this path
    std::vector<double> X(30, 0.0);
    CHECK(throws<unsupported_method_error>([&] { with((num_neighbors = 5)).buildOperatorUsing(X.data(), 3, 10); }));
    // no GPU here: creating the context reports a device error, never crashes
    CHECK(throws<device_error>([&] {
        with((method = KernelLocallyLinearEmbedding, num_neighbors = 5)).buildOperatorUsing(X.data(), 3, 10);
    }));
    return failures;
}

int gpu_run(const char* xpath, long long N, int D, const std::string& prefix)
{
    std::vector<double> X((size_t)N * D);
    {
        std::ifstream f(xpath, std::ios::binary);
        f.read(reinterpret_cast<char*>(X.data()), (std::streamsize)(X.size() * sizeof(double)));
        CHECK(f.good());
    }
    Context ctx(0);
    LocalOperator op = with((method = KernelLocallyLinearEmbedding, neighbors_method = Brute, num_neighbors = 12,
                             klle_shift = 1e-3))
                           .onContext(ctx)
                           .buildOperatorUsing(X.data(), D, N);
    CHECK(op.n == N && op.k == 12);
    CHECK((long long)op.row_ptr.back() == (long long)op.col_idx.size());
    dump(prefix + "idx.bin", op.neighbors);
    dump(prefix + "w.bin", op.weights);
    dump(prefix + "rowptr.bin", op.row_ptr);
    dump(prefix + "col.bin", op.col_idx);
    dump(prefix + "vals.bin", op.values);

    // error semantics of the chain (test/unit/interface.cpp:102-260, methods/base.hpp:85)
    CHECK(throws<wrong_parameter_error>([&] {
        with((method = KernelLocallyLinearEmbedding, num_neighbors = 2)).onContext(ctx).buildOperatorUsing(X.data(), D, N);
    }));
    CHECK(throws<wrong_parameter_error>([&] {
        with((method = KernelLocallyLinearEmbedding, num_neighbors = (int)N)).onContext(ctx).buildOperatorUsing(X.data(), D,
                                                                                                              N);
    }));
    CHECK(throws<no_data_error>([&] {
        with((method = KernelLocallyLinearEmbedding, num_neighbors = 5)).onContext(ctx).buildOperatorUsing(X.data(), D, 0);
    }));
    // embedUsing: the operator and the GPU eigensolver (2 columns after the first)
    TapkeeOutput emb = with((method = KernelLocallyLinearEmbedding, neighbors_method = Brute, num_neighbors = 12,
                             klle_shift = 1e-3))
                           .onContext(ctx)
                           .embedUsing(X.data(), D, N);
    CHECK(emb.n == N && emb.target_dimension == 2 && emb.embedding.size() == (size_t)N * 2);
    CHECK(emb.eigen.converged == 1 && emb.eigenvalues[0] <= emb.eigenvalues[1]);
    dump(prefix + "embedding.bin", emb.embedding);
    // LTSA through the same chain
    LocalOperator lt = with((method = KernelLocalTangentSpaceAlignment, num_neighbors = 12, target_dimension = 2))
                           .onContext(ctx)
                           .buildOperatorUsing(X.data(), D, N);
    CHECK(lt.k == 12 && lt.target_dimension == 2 && lt.weights.size() == (size_t)N * 12 * 2);
    return failures;
}

} // namespace

int main(int argc, char** argv)
{
    try
    {
        if (argc >= 2 && std::strcmp(argv[1], "host") == 0)
            host_checks();
        else if (argc >= 6 && std::strcmp(argv[1], "gpu") == 0)
            gpu_run(argv[2], std::atoll(argv[3]), std::atoi(argv[4]), argv[5]);
        else
        {
            std::fprintf(stderr, "usage: facade_check host | gpu X.bin N D out_prefix\n");
            return 2;
        }
    }
    catch (const std::exception& e)
    {
        std::fprintf(stderr, "unexpected exception: %s\n", e.what());
        return 1;
    }
    if (failures)
        return 1;
    std::printf("ok\n");
    return 0;
}
