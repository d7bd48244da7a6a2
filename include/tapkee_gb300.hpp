/*
 * tapkee_gb300.hpp -- C++ facade over the C ABI in the shape of the reference's
 * chain interface:
 *
 *   using namespace tapkee_gb300;
 *   using namespace tapkee_gb300::keywords;
 *   LocalOperator op = with((method = KernelLocallyLinearEmbedding, neighbors_method = Brute,
 *                            num_neighbors = 12, klle_shift = 1e-3))
 *                          .buildOperatorUsing(X, D, N);
 *
 * It mirrors tapkee::with(ParametersSet) / ParametersInitializedState
 * (chain_interface.hpp:401-480) and the keywords of defines/keywords.hpp for the
 * parameters this stage reads, with the reference's exception types
 * (exceptions.hpp:14-91). embedUsing(X, D, N) runs the whole of the reference's
 * embedUsing(DenseMatrix) for these methods, eigensolver included (the GPU
 * solver of tk_smallest_eigenvectors in place of ARPACK). buildOperatorUsing
 * stops at the sparse alignment matrix M (CSR, symmetric) and hands it back with
 * the neighbours and weights, for a caller with its own eigensolver.
 *
 * Header-only; link against libtapkee_gb300.so.
 */
#ifndef TAPKEE_GB300_HPP
#define TAPKEE_GB300_HPP

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "tapkee_gb300.h"

namespace tapkee_gb300 {

/* ---- exceptions (exceptions.hpp:14-91) ------------------------------------ */

class no_data_error : public std::logic_error
{
public:
    explicit no_data_error(const std::string& m) : std::logic_error(m) {}
};
class unsupported_method_error : public std::logic_error
{
public:
    explicit unsupported_method_error(const std::string& m) : std::logic_error(m) {}
};
class not_enough_memory_error : public std::runtime_error
{
public:
    explicit not_enough_memory_error(const std::string& m) : std::runtime_error(m) {}
};
class cancelled_exception : public std::exception
{
public:
    const char* what() const noexcept override { return "Cancelled"; }
};
class missed_parameter_error : public std::logic_error
{
public:
    explicit missed_parameter_error(const std::string& m) : std::logic_error(m) {}
};
class wrong_parameter_error : public std::logic_error
{
public:
    explicit wrong_parameter_error(const std::string& m) : std::logic_error(m) {}
};
class multiple_parameter_error : public std::runtime_error
{
public:
    explicit multiple_parameter_error(const std::string& m) : std::runtime_error(m) {}
};
class eigendecomposition_error : public std::runtime_error
{
public:
    explicit eigendecomposition_error(const std::string& m) : std::runtime_error(m) {}
};
/* No counterpart in the reference: the GPU, its driver or a bounded device wait failed. */
class device_error : public std::runtime_error
{
public:
    explicit device_error(const std::string& m) : std::runtime_error(m) {}
};

/* Throws the exception type that corresponds to a tk_status. */
inline void throw_status(int status, const std::string& message)
{
    switch (status)
    {
    case TK_OK:
        return;
    case TK_ERR_INVALID_ARG:
    case TK_ERR_BUFFER_TOO_SMALL:
        throw wrong_parameter_error(message);
    case TK_ERR_NO_DATA:
        throw no_data_error(message);
    case TK_ERR_OOM:
        throw not_enough_memory_error(message);
    case TK_ERR_CANCELLED:
        throw cancelled_exception();
    case TK_ERR_UNSUPPORTED:
        throw unsupported_method_error(message);
    case TK_ERR_NOT_CONVERGED:
        throw eigendecomposition_error(message);
    default:
        throw device_error(std::string(tk_status_string(status)) + ": " + message);
    }
}

/* ---- parameter values (defines/methods.hpp) --------------------------------- */

/* The methods this stage serves (defines/methods.hpp:74,82); any other method stays
 * on the reference. */
enum DimensionReductionMethod
{
    KernelLocallyLinearEmbedding = TK_METHOD_KLLE,
    KernelLocalTangentSpaceAlignment = TK_METHOD_KLTSA
};

/* Only the brute-force neighbour search runs here (defines/methods.hpp:161). */
enum NeighborsMethod
{
    Brute = 0
};

enum ScreenEngine
{
    TensorScreen = TK_SCREEN_TENSOR,
    Fp32Screen = TK_SCREEN_FP32
};

/* ---- parameter sets ------------------------------------------------------- */

/* The parameters given to with(): which were set, and their values. */
struct ParametersSet
{
    unsigned given = 0;
    tk_params values;
    int neighbors = Brute;

    ParametersSet() { tk_params_default(&values); }
};

namespace detail {
enum : unsigned
{
    P_METHOD = 1u << 0,
    P_NEIGHBORS_METHOD = 1u << 1,
    P_NUM_NEIGHBORS = 1u << 2,
    P_TARGET_DIMENSION = 1u << 3,
    P_KLLE_SHIFT = 1u << 4,
    P_NULLSPACE_SHIFT = 1u << 5,
    P_CHECK_CONNECTIVITY = 1u << 6,
    P_SCREEN = 1u << 7
};

template <unsigned Bit, class T>
struct Keyword
{
    const char* name;
    ParametersSet operator=(T v) const
    {
        ParametersSet p;
        p.given = Bit;
        set(p, v);
        return p;
    }
    static void set(ParametersSet& p, T v);
};

template <> inline void Keyword<P_METHOD, DimensionReductionMethod>::set(ParametersSet& p, DimensionReductionMethod v)
{
    p.values.method = (int)v;
}
template <> inline void Keyword<P_NEIGHBORS_METHOD, NeighborsMethod>::set(ParametersSet& p, NeighborsMethod v)
{
    p.neighbors = (int)v;
}
template <> inline void Keyword<P_NUM_NEIGHBORS, int>::set(ParametersSet& p, int v) { p.values.num_neighbors = v; }
template <> inline void Keyword<P_TARGET_DIMENSION, int>::set(ParametersSet& p, int v)
{
    p.values.target_dimension = v;
}
template <> inline void Keyword<P_KLLE_SHIFT, double>::set(ParametersSet& p, double v) { p.values.klle_shift = v; }
template <> inline void Keyword<P_NULLSPACE_SHIFT, double>::set(ParametersSet& p, double v)
{
    p.values.nullspace_shift = v;
}
template <> inline void Keyword<P_CHECK_CONNECTIVITY, bool>::set(ParametersSet& p, bool v)
{
    p.values.check_connectivity = v ? 1 : 0;
}
template <> inline void Keyword<P_SCREEN, ScreenEngine>::set(ParametersSet& p, ScreenEngine v)
{
    p.values.screen = (int)v;
}
} // namespace detail

/* Joins two parameter sets; a parameter given twice is an error, as in the
 * reference (embed.hpp:134-136). */
inline ParametersSet operator,(ParametersSet a, const ParametersSet& b)
{
    if (a.given & b.given)
        throw multiple_parameter_error("a parameter is given more than once");
    if (b.given & detail::P_METHOD)
        a.values.method = b.values.method;
    if (b.given & detail::P_NEIGHBORS_METHOD)
        a.neighbors = b.neighbors;
    if (b.given & detail::P_NUM_NEIGHBORS)
        a.values.num_neighbors = b.values.num_neighbors;
    if (b.given & detail::P_TARGET_DIMENSION)
        a.values.target_dimension = b.values.target_dimension;
    if (b.given & detail::P_KLLE_SHIFT)
        a.values.klle_shift = b.values.klle_shift;
    if (b.given & detail::P_NULLSPACE_SHIFT)
        a.values.nullspace_shift = b.values.nullspace_shift;
    if (b.given & detail::P_CHECK_CONNECTIVITY)
        a.values.check_connectivity = b.values.check_connectivity;
    if (b.given & detail::P_SCREEN)
        a.values.screen = b.values.screen;
    a.given |= b.given;
    return a;
}

/* Keywords (defines/keywords.hpp:35,87-88,112,125,235,248,272); screen has no
 * counterpart in the reference and selects the distance-screen engine. */
namespace keywords {
static const detail::Keyword<detail::P_METHOD, DimensionReductionMethod> method{"dimension reduction method"};
static const detail::Keyword<detail::P_NEIGHBORS_METHOD, NeighborsMethod> neighbors_method{"nearest neighbors method"};
static const detail::Keyword<detail::P_NUM_NEIGHBORS, int> num_neighbors{"number of neighbors"};
static const detail::Keyword<detail::P_TARGET_DIMENSION, int> target_dimension{"target dimension"};
static const detail::Keyword<detail::P_KLLE_SHIFT, double> klle_shift{"KLLE regularizer"};
static const detail::Keyword<detail::P_NULLSPACE_SHIFT, double> nullspace_shift{"diagonal shift of nullspace"};
static const detail::Keyword<detail::P_CHECK_CONNECTIVITY, bool> check_connectivity{"check connectivity"};
static const detail::Keyword<detail::P_SCREEN, ScreenEngine> screen{"distance screen engine"};
} // namespace keywords

/* ---- results ---------------------------------------------------------------- */

/* The operator of one call: neighbours (n x k, row-major), weights (n x k for
 * KLLE; the tangent basis n x k x td for KLTSA) and M in CSR (symmetric, so the
 * same arrays are its CSC form; columns ascending within a row). */
struct LocalOperator
{
    int64_t n = 0;
    int k = 0;
    int method = 0;
    int target_dimension = 0;
    std::vector<int32_t> neighbors;
    std::vector<double> weights;
    std::vector<int64_t> row_ptr;
    std::vector<int32_t> col_idx;
    std::vector<double> values;
    tk_operator_info info{};
};

/* embedUsing's result, the embedding part of the reference's TapkeeOutput
 * (defines/types.hpp): N x target_dimension, column-major like its DenseMatrix,
 * with the eigenvalues of M for those columns. */
struct TapkeeOutput
{
    int64_t n = 0;
    int target_dimension = 0;
    std::vector<double> embedding;
    std::vector<double> eigenvalues;
    tk_operator_info info{};
    tk_eig_info eigen{};
};

/* ---- context and chain -------------------------------------------------------- */

/* One GPU context (stream + scratch); reused by every call made through it. */
class Context
{
public:
    explicit Context(int device = 0, void* stream = nullptr)
    {
        tk_ctx* c = nullptr;
        const int st = tk_ctx_create(device, stream, &c);
        if (st != TK_OK)
            throw_status(st, "tk_ctx_create on device " + std::to_string(device) + " failed");
        ctx_.reset(c, [](tk_ctx* p) { tk_ctx_destroy(p); });
    }
    tk_ctx* get() const { return ctx_.get(); }
    void check(int status) const
    {
        if (status != TK_OK)
            throw_status(status, tk_last_error(ctx_.get()));
    }

private:
    std::shared_ptr<tk_ctx> ctx_;
};

/* with(...) result (chain_interface.hpp:401-480). */
class ParametersInitializedState
{
public:
    explicit ParametersInitializedState(const ParametersSet& p) : params_(p) {}

    /* Runs on this context instead of a private one on device 0. */
    ParametersInitializedState& onContext(const Context& c)
    {
        ctx_ = std::make_shared<Context>(c);
        return *this;
    }

    /* X holds N feature vectors of dimension D column-wise (the reference's
     * DenseMatrix, defines/types.hpp:23): X[i*D + d]. Host or device memory. */
    LocalOperator buildOperatorUsing(const double* X, int64_t D, int64_t N) const { return run(X, TK_F64, D, N); }
    LocalOperator buildOperatorUsing(const float* X, int64_t D, int64_t N) const { return run(X, TK_F32, D, N); }

    /* embedUsing(DenseMatrix) (chain_interface.hpp:471-480) for these methods: the
     * operator, then the target_dimension smallest eigenvectors of M after the
     * first (eigendecomposition(SmallestEigenvalues, M, td),
     * methods/kernel_locally_linear_embedding.hpp:27) with the GPU eigensolver,
     * reading M where the operator left it on the device. */
    TapkeeOutput embedUsing(const double* X, int64_t D, int64_t N) const { return embed(X, TK_F64, D, N); }
    TapkeeOutput embedUsing(const float* X, int64_t D, int64_t N) const { return embed(X, TK_F32, D, N); }

private:
    std::shared_ptr<Context> checked_context(int64_t D) const
    {
        if (!(params_.given & detail::P_METHOD))
            throw unsupported_method_error("only KernelLocallyLinearEmbedding and "
                                           "KernelLocalTangentSpaceAlignment run on this path");
        if (params_.neighbors != Brute)
            throw unsupported_method_error("only the Brute neighbours method runs on this path");
        if (D < 1 || D > 0x7fffffff)
            throw wrong_parameter_error("feature dimension out of range");
        return ctx_ ? ctx_ : std::make_shared<Context>(0);
    }

    TapkeeOutput embed(const void* X, int dtype, int64_t D, int64_t N) const
    {
        std::shared_ptr<Context> c = checked_context(D);
        TapkeeOutput out;
        c->check(tk_local_operator(c->get(), &params_.values, X, dtype, N, (int)D, D, &out.info));
        const int64_t* rp = nullptr;
        const int32_t* col = nullptr;
        const double* vals = nullptr;
        c->check(tk_operator_device_views(c->get(), nullptr, nullptr, &rp, &col, &vals));
        out.n = out.info.n;
        out.target_dimension = params_.values.target_dimension;
        out.embedding.resize((size_t)out.n * (size_t)out.target_dimension);
        out.eigenvalues.resize((size_t)out.target_dimension);
        c->check(tk_smallest_eigenvectors(c->get(), out.n, rp, col, vals, out.target_dimension, 1, 0.0, 0,
                                          out.embedding.data(), out.eigenvalues.data(), &out.eigen));
        return out;
    }

    LocalOperator run(const void* X, int dtype, int64_t D, int64_t N) const
    {
        std::shared_ptr<Context> c = checked_context(D);
        LocalOperator op;
        c->check(tk_local_operator(c->get(), &params_.values, X, dtype, N, (int)D, D, &op.info));
        op.n = op.info.n;
        op.k = op.info.k;
        op.method = op.info.method;
        op.target_dimension = op.info.target_dimension;
        const size_t nk = (size_t)op.n * (size_t)op.k;
        op.neighbors.resize(nk);
        op.weights.resize(op.method == TK_METHOD_KLTSA ? nk * (size_t)op.target_dimension : nk);
        op.row_ptr.resize((size_t)op.n + 1);
        op.col_idx.resize((size_t)op.info.nnz);
        op.values.resize((size_t)op.info.nnz);
        c->check(tk_operator_copy(c->get(), op.neighbors.data(), op.weights.data(), op.row_ptr.data(),
                                  op.col_idx.data(), op.values.data()));
        return op;
    }

    ParametersSet params_;
    std::shared_ptr<Context> ctx_;
};

inline ParametersInitializedState with(const ParametersSet& p) { return ParametersInitializedState(p); }

} // namespace tapkee_gb300

#endif /* TAPKEE_GB300_HPP */
