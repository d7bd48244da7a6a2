// capi.cpp -- the extern "C" boundary: contexts, argument checks, host/device
// buffer handling and the stage pipeline of tk_local_operator.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "tk_internal.h"

#define TK_VERSION_STRING "0.1.0"

namespace tk {

std::atomic<long long> g_kernel_launches{0};

void* Scratch::get(const std::string& name, size_t bytes)
{
    Buf& b = bufs[name];
    if (b.bytes < bytes)
    {
        if (b.ptr)
        {
            // the old buffer may still be read by queued work
            TK_CUDA(cudaDeviceSynchronize());
            TK_CUDA(cudaFree(b.ptr));
            b.ptr = nullptr;
            b.bytes = 0;
        }
        size_t nb = std::max(bytes, (size_t)256);
        nb = (nb + 255) & ~(size_t)255;
        void* p = nullptr;
        cudaError_t e = cudaMalloc(&p, nb);
        if (e != cudaSuccess)
        {
            cudaGetLastError();
            throw Error(e == cudaErrorMemoryAllocation ? TK_ERR_OOM : TK_ERR_CUDA,
                        "device allocation of " + std::to_string(nb) + " bytes for '" + name + "' failed: " +
                            cudaGetErrorString(e));
        }
        b.ptr = p;
        b.bytes = nb;
    }
    return b.ptr;
}

void Scratch::release_all()
{
    for (auto& kv : bufs)
        if (kv.second.ptr)
            cudaFree(kv.second.ptr);
    bufs.clear();
}

void log(tk_ctx* ctx, int level, const std::string& msg)
{
    if (ctx && ctx->log_fn)
        ctx->log_fn(level, msg.c_str(), ctx->log_user);
    else if (level == TK_LOG_WARNING || level == TK_LOG_ERROR)
        std::fprintf(stderr, "[tapkee_gb300] %s\n", msg.c_str());
}

namespace {

bool is_device_ptr(const void* p)
{
    if (!p)
        return false;
    cudaPointerAttributes a;
    cudaError_t e = cudaPointerGetAttributes(&a, p);
    if (e != cudaSuccess)
    {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

size_t dtype_size(int dtype) { return dtype == TK_F64 ? 8 : 4; }

void check_dtype(int dtype)
{
    if (dtype != TK_F32 && dtype != TK_F64)
        throw Error(TK_ERR_INVALID_ARG, "dtype must be TK_F32 or TK_F64");
}

// Makes X device-resident (packed if it lives on the host); returns the device
// pointer and its row stride.
const void* device_points(tk_ctx* ctx, const void* X, int dtype, int64_t N, int D, int64_t ldx, int64_t* ldx_dev,
                          const char* name)
{
    if (is_device_ptr(X))
    {
        *ldx_dev = ldx;
        return X;
    }
    const size_t es = dtype_size(dtype);
    void* d = ctx->scratch.get(name, es * (size_t)N * D);
    TK_CUDA(cudaMemcpy2DAsync(d, es * D, X, es * ldx, es * D, (size_t)N, cudaMemcpyHostToDevice, ctx->stream));
    *ldx_dev = D;
    return d;
}

template <typename T>
const T* device_array(tk_ctx* ctx, const T* p, size_t count, const char* name)
{
    if (is_device_ptr(p))
        return p;
    T* d = (T*)ctx->scratch.get(name, sizeof(T) * count);
    TK_CUDA(cudaMemcpyAsync(d, p, sizeof(T) * count, cudaMemcpyHostToDevice, ctx->stream));
    return d;
}

template <typename T>
T* device_out(tk_ctx* ctx, T* p, size_t count, const char* name, bool* is_host)
{
    if (!p)
    {
        *is_host = false;
        return nullptr;
    }
    if (is_device_ptr(p))
    {
        *is_host = false;
        return p;
    }
    *is_host = true;
    return (T*)ctx->scratch.get(name, sizeof(T) * count);
}

template <typename T>
void copy_back(tk_ctx* ctx, T* host, const T* dev, size_t count)
{
    TK_CUDA(cudaMemcpyAsync(host, dev, sizeof(T) * count, cudaMemcpyDeviceToHost, ctx->stream));
}

void check_device_errors(tk_ctx* ctx)
{
    TK_CUDA(cudaMemcpyAsync(ctx->host_err, ctx->dev_err, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
    TK_CUDA(cudaStreamSynchronize(ctx->stream));
    const unsigned e = *ctx->host_err;
    if (e)
    {
        TK_CUDA(cudaMemsetAsync(ctx->dev_err, 0, sizeof(unsigned), ctx->stream));
        std::string m = "device-side check failed:";
        if (e & DEV_ERR_TIMEOUT)
            m += " bounded wait expired;";
        if (e & DEV_ERR_OVERFLOW)
            m += " bounded buffer overflow;";
        if (e & DEV_ERR_BOUNDS)
            m += " index out of range;";
        if (e & DEV_ERR_NONFINITE)
            m += " non-finite value;";
        throw Error((e & DEV_ERR_TIMEOUT) ? TK_ERR_TIMEOUT : ((e & DEV_ERR_BOUNDS) ? TK_ERR_INVALID_ARG : TK_ERR_INTERNAL),
                    m);
    }
}

// Candidates kept per query by the screen: at least k + 8 (the self match and a
// margin for certification).
int candidates_for(int k)
{
    for (int kc : {32, 64, 128, 256})
        if (k + 8 <= kc)
            return kc;
    return -1;
}

// Brute kNN into device buffers; returns uncertified rows.
int64_t knn_device(tk_ctx* ctx, const void* Xd, int dtype, int64_t N, int D, int64_t ldx, int k, int screen,
                   int32_t* idx_d, double* d2_d)
{
    const int kc = candidates_for(k);
    if (kc < 0)
        throw Error(TK_ERR_UNSUPPORTED, "brute kNN supports up to 248 neighbours per point (k = " +
                                            std::to_string(k) + ")");
    // The tensor-core screen keeps its candidate lists in registers (KC <= 64);
    // longer lists (k > 56) are built in kc / 64 passes of 64 entries each.
    const bool tensor = (screen == TK_SCREEN_TENSOR);
    if (tensor && kc > 64)
        log(ctx, TK_LOG_INFO, "k = " + std::to_string(k) + " > 56: tensor screen in " + std::to_string(kc / 64) +
                                  " passes of 64 candidates");
    if (tensor && !tensor_screen_supported(((D + 63) / 64) * 64))
        throw Error(TK_ERR_UNSUPPORTED, "the tensor-core screen supports D <= 128; pass TK_SCREEN_FP32 for D = " +
                                            std::to_string(D));
    Prepared P;
    mark(ctx, KM_PREP);
    prepare_points(ctx, Xd, dtype, N, D, ldx, tensor, P);
    mark(ctx, KM_SCREEN0);
    int32_t* cand_idx = (int32_t*)ctx->scratch.get("knn.cand_idx", sizeof(int32_t) * (size_t)P.Npad * kc);
    float* cand_val = (float*)ctx->scratch.get("knn.cand_val", sizeof(float) * (size_t)P.Npad * kc);
    TK_CUDA(cudaEventRecord(ctx->ev[8], ctx->stream));
    if (tensor)
        screen_tensor(ctx, P, kc, k, cand_idx, cand_val);
    else
        screen_fp32(ctx, P, kc, cand_idx, cand_val);
    TK_CUDA(cudaEventRecord(ctx->ev[9], ctx->stream));
    mark(ctx, KM_SCREEN1);
    float c1, c2;
    screen_error_model(screen, P.Dp, &c1, &c2);
    const int64_t nf = rerank(ctx, P, Xd, dtype, ldx, k, kc, cand_idx, cand_val, c1, c2, idx_d, d2_d);
    mark(ctx, KM_RERANK);
    check_device_errors(ctx);
    ctx->screen_ms = 0.f;
    cudaEventElapsedTime(&ctx->screen_ms, ctx->ev[8], ctx->ev[9]);
    return nf;
}

void validate_points(const void* X, int dtype, int64_t N, int D, int64_t ldx)
{
    check_dtype(dtype);
    if (N <= 0)
        throw Error(TK_ERR_NO_DATA, "No data to embed");
    if (!X)
        throw Error(TK_ERR_INVALID_ARG, "X is NULL");
    if (D <= 0 || ldx < D)
        throw Error(TK_ERR_INVALID_ARG, "need D >= 1 and ldx >= D");
    if (N >= ((int64_t)1 << 31) - 256)
        throw Error(TK_ERR_INVALID_ARG, "N must be below 2^31 (int32 indices)");
}

template <typename F>
int guarded(tk_ctx* ctx, F&& f)
{
    if (!ctx)
        return TK_ERR_INVALID_ARG;
    try
    {
        TK_CUDA(cudaSetDevice(ctx->device));
        f();
        ctx->last_error.clear();
        return TK_OK;
    }
    catch (const Error& e)
    {
        ctx->last_error = e.what();
        log(ctx, TK_LOG_ERROR, e.what());
        return e.status;
    }
    catch (const std::bad_alloc&)
    {
        ctx->last_error = "Not enough memory";
        return TK_ERR_OOM;
    }
    catch (const std::exception& e)
    {
        ctx->last_error = e.what();
        return TK_ERR_INTERNAL;
    }
}

// Device time between two recorded events (0 if either was never recorded; the
// error that leaves is cleared so that the next launch check does not see it).
float elapsed(cudaEvent_t a, cudaEvent_t b)
{
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess)
    {
        cudaGetLastError();
        ms = 0.f;
    }
    return ms;
}

} // namespace
} // namespace tk

using namespace tk;

extern "C" {

const char* tk_version(void) { return TK_VERSION_STRING; }

long long tk_kernel_launch_count(void) { return tk::g_kernel_launches.load(); }

void tk_params_default(tk_params* p)
{
    if (!p)
        return;
    p->method = TK_METHOD_KLLE;
    p->num_neighbors = 5;
    p->target_dimension = 2;
    p->klle_shift = 1e-3;
    p->nullspace_shift = 1e-9;
    p->check_connectivity = 1;
    p->screen = TK_SCREEN_TENSOR;
    p->cancel_function = nullptr;
}

const char* tk_status_string(int s)
{
    switch (s)
    {
    case TK_OK: return "ok";
    case TK_ERR_INVALID_ARG: return "wrong parameter";
    case TK_ERR_NO_DATA: return "no data";
    case TK_ERR_OOM: return "not enough memory";
    case TK_ERR_CUDA: return "CUDA error";
    case TK_ERR_TIMEOUT: return "device wait timed out";
    case TK_ERR_CANCELLED: return "cancelled";
    case TK_ERR_BUFFER_TOO_SMALL: return "buffer too small";
    case TK_ERR_UNSUPPORTED: return "unsupported";
    case TK_ERR_NO_DEVICE: return "no sm_103 device";
    case TK_ERR_INTERNAL: return "internal error";
    default: return "unknown status";
    }
}

int tk_ctx_create(int device, void* stream, tk_ctx** out)
{
    if (!out)
        return TK_ERR_INVALID_ARG;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count)
    {
        cudaGetLastError();
        return TK_ERR_NO_DEVICE;
    }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess)
        return TK_ERR_NO_DEVICE;
    if (!(prop.major == 10 && prop.minor == 3))
        return TK_ERR_NO_DEVICE;
    tk_ctx* ctx = new (std::nothrow) tk_ctx();
    if (!ctx)
        return TK_ERR_OOM;
    ctx->device = device;
    ctx->num_sms = prop.multiProcessorCount;
    int rc = guarded(ctx, [&] {
        if (stream)
        {
            ctx->stream = (cudaStream_t)stream;
            ctx->own_stream = false;
        }
        else
        {
            TK_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
            ctx->own_stream = true;
        }
        TK_CUDA(cudaMalloc(&ctx->dev_err, 256));
        TK_CUDA(cudaMemset(ctx->dev_err, 0, 256));
        TK_CUDA(cudaMallocHost(&ctx->host_err, 256));
        TK_CUDA(cudaMallocHost(&ctx->host_i64, 16 * sizeof(int64_t)));
        for (auto& e : ctx->ev)
            TK_CUDA(cudaEventCreate(&e));
        for (auto& e : ctx->kev)
            TK_CUDA(cudaEventCreate(&e));
    });
    if (rc != TK_OK)
    {
        tk_ctx_destroy(ctx);
        return rc;
    }
    *out = ctx;
    return TK_OK;
}

int tk_ctx_destroy(tk_ctx* ctx)
{
    if (!ctx)
        return TK_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream)
        cudaStreamSynchronize(ctx->stream);
    ctx->scratch.release_all();
    if (ctx->dev_err)
        cudaFree(ctx->dev_err);
    if (ctx->host_err)
        cudaFreeHost(ctx->host_err);
    if (ctx->host_i64)
        cudaFreeHost(ctx->host_i64);
    for (auto& e : ctx->ev)
        if (e)
            cudaEventDestroy(e);
    for (auto& e : ctx->kev)
        if (e)
            cudaEventDestroy(e);
    if (ctx->own_stream && ctx->stream)
        cudaStreamDestroy(ctx->stream);
    delete ctx;
    return TK_OK;
}

const char* tk_last_error(const tk_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

int tk_set_log_callback(tk_ctx* ctx, tk_log_fn fn, void* user)
{
    if (!ctx)
        return TK_ERR_INVALID_ARG;
    ctx->log_fn = fn;
    ctx->log_user = user;
    return TK_OK;
}

int tk_ctx_synchronize(tk_ctx* ctx)
{
    return guarded(ctx, [&] { TK_CUDA(cudaStreamSynchronize(ctx->stream)); });
}

int tk_knn_brute(tk_ctx* ctx, const void* X, int dtype, int64_t N, int D, int64_t ldx, int k, int screen,
                 int32_t* idx_out, double* d2_out, tk_knn_stats* stats)
{
    return guarded(ctx, [&] {
        validate_points(X, dtype, N, D, ldx);
        if (k < 1 || k > N - 1)
            throw Error(TK_ERR_INVALID_ARG, "k must lie in [1, N-1]");
        if (screen != TK_SCREEN_TENSOR && screen != TK_SCREEN_FP32)
            throw Error(TK_ERR_INVALID_ARG, "unknown screen engine");
        if (!idx_out)
            throw Error(TK_ERR_INVALID_ARG, "idx_out is NULL");
        int64_t ldd;
        const void* Xd = device_points(ctx, X, dtype, N, D, ldx, &ldd, "io.X");
        bool ih, dh;
        int32_t* idx_d = device_out(ctx, idx_out, (size_t)N * k, "io.idx", &ih);
        double* d2_d = device_out(ctx, d2_out, (size_t)N * k, "io.d2", &dh);
        const int64_t nf = knn_device(ctx, Xd, dtype, N, D, ldd, k, screen, idx_d, d2_d);
        if (ih)
            copy_back(ctx, idx_out, idx_d, (size_t)N * k);
        if (dh)
            copy_back(ctx, d2_out, d2_d, (size_t)N * k);
        TK_CUDA(cudaStreamSynchronize(ctx->stream));
        if (stats)
        {
            stats->rows_uncertified = nf;
            stats->candidates = candidates_for(k);
            stats->screen = screen;
            stats->tie_rows = ctx->knn_ties;
            stats->extra_rows = ctx->knn_extra;
        }
    });
}

int tk_knn_extra_rows(tk_ctx* ctx, int32_t* rows, int32_t* extra, int64_t capacity, int64_t* count)
{
    return guarded(ctx, [&] {
        if (!count || capacity < 0)
            throw Error(TK_ERR_INVALID_ARG, "bad arguments");
        *count = ctx->knn_extra;
        const int64_t n = std::min<int64_t>(capacity, ctx->knn_extra);
        if (n <= 0 || (!rows && !extra))
            return;
        std::vector<int32_t> pairs((size_t)(2 * n));
        const void* src = ctx->scratch.bufs["rerank.extra"].ptr;
        TK_CUDA(cudaMemcpyAsync(pairs.data(), src, sizeof(int32_t) * (size_t)(2 * n), cudaMemcpyDeviceToHost,
                                ctx->stream));
        TK_CUDA(cudaStreamSynchronize(ctx->stream));
        // rows in ascending order (the device appends them in completion order)
        std::vector<std::pair<int32_t, int32_t>> pr((size_t)n);
        for (int64_t e = 0; e < n; ++e)
            pr[(size_t)e] = {pairs[(size_t)(2 * e)], pairs[(size_t)(2 * e + 1)]};
        std::sort(pr.begin(), pr.end());
        for (int64_t e = 0; e < n; ++e)
        {
            if (rows)
                rows[e] = pr[(size_t)e].first;
            if (extra)
                extra[e] = pr[(size_t)e].second;
        }
    });
}

int tk_check_connected(tk_ctx* ctx, int64_t N, int k, const int32_t* idx, int* connected)
{
    return guarded(ctx, [&] {
        if (N <= 0)
            throw Error(TK_ERR_NO_DATA, "No data");
        if (k < 1 || !idx || !connected)
            throw Error(TK_ERR_INVALID_ARG, "bad arguments");
        const int32_t* idx_d = device_array(ctx, idx, (size_t)N * k, "io.idx_in");
        const bool c = check_connected(ctx, N, k, idx_d);
        check_device_errors(ctx);
        *connected = c ? 1 : 0;
    });
}

int tk_lle_weights(tk_ctx* ctx, const void* X, int dtype, int64_t N, int D, int64_t ldx, const int32_t* idx, int k,
                   double klle_shift, double* W_out)
{
    return guarded(ctx, [&] {
        validate_points(X, dtype, N, D, ldx);
        if (k < 1 || !idx || !W_out)
            throw Error(TK_ERR_INVALID_ARG, "bad arguments");
        int64_t ldd;
        const void* Xd = device_points(ctx, X, dtype, N, D, ldx, &ldd, "io.X");
        const int32_t* idx_d = device_array(ctx, idx, (size_t)N * k, "io.idx_in");
        bool wh;
        double* W_d = device_out(ctx, W_out, (size_t)N * k, "io.W", &wh);
        lle_weights(ctx, Xd, dtype, N, D, ldd, idx_d, k, klle_shift, W_d);
        check_device_errors(ctx);
        if (wh)
            copy_back(ctx, W_out, W_d, (size_t)N * k);
        TK_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

int tk_lle_weights_grad(tk_ctx* ctx, const void* X, int dtype, int64_t N, int D, int64_t ldx, const int32_t* idx,
                        int k, double klle_shift, const double* W, const double* dW, double* dX_out)
{
    return guarded(ctx, [&] {
        validate_points(X, dtype, N, D, ldx);
        if (k < 1 || !idx || !W || !dW || !dX_out)
            throw Error(TK_ERR_INVALID_ARG, "bad arguments");
        if (k > 128)
            throw Error(TK_ERR_UNSUPPORTED, "LLE weights support up to 128 neighbours");
        int64_t ldd;
        const void* Xd = device_points(ctx, X, dtype, N, D, ldx, &ldd, "io.X");
        const int32_t* idx_d = device_array(ctx, idx, (size_t)N * k, "io.idx_in");
        const double* W_d = device_array(ctx, W, (size_t)N * k, "io.W_in");
        const double* G_d = device_array(ctx, dW, (size_t)N * k, "io.dW_in");
        bool gh;
        double* gX_d = device_out(ctx, dX_out, (size_t)N * D, "io.dX", &gh);
        lle_weights_grad(ctx, Xd, dtype, N, D, ldd, idx_d, k, klle_shift, W_d, G_d, gX_d);
        check_device_errors(ctx);
        if (gh)
            copy_back(ctx, dX_out, gX_d, (size_t)N * D);
        TK_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

int tk_hessian_basis(tk_ctx* ctx, const void* X, int dtype, int64_t N, int D, int64_t ldx, const int32_t* idx,
                     int k, int td, double* Y_out)
{
    return guarded(ctx, [&] {
        validate_points(X, dtype, N, D, ldx);
        if (k < 1 || !idx || !Y_out)
            throw Error(TK_ERR_INVALID_ARG, "bad arguments");
        const size_t count = (size_t)N * k * weight_columns(TK_METHOD_HLLE, td);
        int64_t ldd;
        const void* Xd = device_points(ctx, X, dtype, N, D, ldx, &ldd, "io.X");
        const int32_t* idx_d = device_array(ctx, idx, (size_t)N * k, "io.idx_in");
        bool yh;
        double* Y_d = device_out(ctx, Y_out, count, "io.Y", &yh);
        hessian_basis(ctx, Xd, dtype, N, D, ldd, idx_d, k, td, Y_d);
        check_device_errors(ctx);
        if (yh)
            copy_back(ctx, Y_out, Y_d, count);
        TK_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

int tk_ltsa_basis(tk_ctx* ctx, const void* X, int dtype, int64_t N, int D, int64_t ldx, const int32_t* idx, int k,
                  int td, double* V_out)
{
    return guarded(ctx, [&] {
        validate_points(X, dtype, N, D, ldx);
        if (k < 1 || !idx || !V_out)
            throw Error(TK_ERR_INVALID_ARG, "bad arguments");
        int64_t ldd;
        const void* Xd = device_points(ctx, X, dtype, N, D, ldx, &ldd, "io.X");
        const int32_t* idx_d = device_array(ctx, idx, (size_t)N * k, "io.idx_in");
        bool vh;
        double* V_d = device_out(ctx, V_out, (size_t)N * k * td, "io.V", &vh);
        ltsa_basis(ctx, Xd, dtype, N, D, ldd, idx_d, k, td, V_d);
        check_device_errors(ctx);
        if (vh)
            copy_back(ctx, V_out, V_d, (size_t)N * k * td);
        TK_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

int tk_eigenproblem_pair(tk_ctx* ctx, int kind, const void* X, int dtype, int64_t N, int D, int64_t ldx,
                         const int64_t* row_ptr, const int32_t* col_idx, const double* vals, double* lhs,
                         double* rhs)
{
    return guarded(ctx, [&] {
        if (N <= 0)
            throw Error(TK_ERR_NO_DATA, "No data");
        if (kind != TK_PAIR_NPE && kind != TK_PAIR_LLTSA)
            throw Error(TK_ERR_UNSUPPORTED, "unsupported eigenproblem kind");
        if (!X || !row_ptr || !col_idx || !vals || !lhs || !rhs || D < 1 || ldx < D)
            throw Error(TK_ERR_INVALID_ARG, "bad arguments");
        check_dtype(dtype);
        int64_t ldd = 0;
        const void* Xd = device_points(ctx, X, dtype, N, D, ldx, &ldd, "io.X");
        int64_t nnz = 0;
        if (is_device_ptr(row_ptr))
        {
            TK_CUDA(cudaMemcpyAsync(ctx->host_i64, row_ptr + N, sizeof(int64_t), cudaMemcpyDeviceToHost,
                                    ctx->stream));
            TK_CUDA(cudaStreamSynchronize(ctx->stream));
            nnz = ctx->host_i64[0];
        }
        else
            nnz = row_ptr[N];
        if (nnz < 0)
            throw Error(TK_ERR_INVALID_ARG, "row_ptr[N] < 0");
        const int64_t* rp_d = device_array(ctx, row_ptr, (size_t)N + 1, "io.pair_rp");
        const int32_t* c_d = device_array(ctx, col_idx, (size_t)std::max<int64_t>(nnz, 1), "io.pair_col");
        const double* v_d = device_array(ctx, vals, (size_t)std::max<int64_t>(nnz, 1), "io.pair_val");
        check_csr_rows(ctx, N, rp_d, nnz);
        check_device_errors(ctx);
        bool lh = false, rh = false;
        double* l_d = device_out(ctx, lhs, (size_t)D * D, "io.pair_lhs", &lh);
        double* r_d = device_out(ctx, rhs, (size_t)D * D, "io.pair_rhs", &rh);
        eigenproblem_pair(ctx, kind, Xd, dtype, N, D, ldd, rp_d, c_d, v_d, l_d, r_d);
        check_device_errors(ctx);
        if (lh)
            copy_back(ctx, lhs, l_d, (size_t)D * D);
        if (rh)
            copy_back(ctx, rhs, r_d, (size_t)D * D);
        TK_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

int tk_selftest_bounded_wait(tk_ctx* ctx, int* outcome)
{
    return guarded(ctx, [&] {
        const int o = wait_selftest(ctx);
        if (outcome)
            *outcome = o;
        check_device_errors(ctx);
    });
}

int tk_selftest_grid_barrier(tk_ctx* ctx, int* outcome)
{
    return guarded(ctx, [&] {
        const int o = barrier_selftest(ctx);
        if (outcome)
            *outcome = o;
        check_device_errors(ctx);
    });
}

int tk_smallest_eigenvectors(tk_ctx* ctx, int64_t N, const int64_t* row_ptr, const int32_t* col_idx,
                             const double* vals, int target_dimension, int skip, double tol, int64_t max_matvecs,
                             double* vectors, double* values, tk_eig_info* info)
{
    return guarded(ctx, [&] {
        if (N <= 0)
            throw Error(TK_ERR_NO_DATA, "No data");
        if (!row_ptr || !col_idx || !vals || !vectors || !values || target_dimension < 1 || skip < 0)
            throw Error(TK_ERR_INVALID_ARG, "bad arguments");
        const int bw = eigen_block_width(target_dimension, skip);
        if (bw == 0)
            throw Error(TK_ERR_UNSUPPORTED, "the sparse eigensolver takes target_dimension + skip <= 14");
        if (N < 4 * (int64_t)bw)
            throw Error(TK_ERR_INVALID_ARG, "the sparse eigensolver needs N >= " + std::to_string(4 * bw) +
                                                " points; use a dense eigensolver");
        const auto t0 = std::chrono::steady_clock::now();
        int64_t nnz = 0;
        if (is_device_ptr(row_ptr))
        {
            TK_CUDA(cudaMemcpyAsync(ctx->host_i64, row_ptr + N, sizeof(int64_t), cudaMemcpyDeviceToHost,
                                    ctx->stream));
            TK_CUDA(cudaStreamSynchronize(ctx->stream));
            nnz = ctx->host_i64[0];
        }
        else
            nnz = row_ptr[N];
        if (nnz < 0)
            throw Error(TK_ERR_INVALID_ARG, "row_ptr[N] < 0");
        const int64_t* rp_d = device_array(ctx, row_ptr, (size_t)N + 1, "io.eig_rp");
        const int32_t* c_d = device_array(ctx, col_idx, (size_t)std::max<int64_t>(nnz, 1), "io.eig_col");
        const double* v_d = device_array(ctx, vals, (size_t)std::max<int64_t>(nnz, 1), "io.eig_val");
        check_csr_rows(ctx, N, rp_d, nnz);
        check_device_errors(ctx);
        bool vh = false, lh = false;
        double* vec_d = device_out(ctx, vectors, (size_t)N * target_dimension, "io.eig_vec", &vh);
        double* val_d = device_out(ctx, values, (size_t)target_dimension, "io.eig_lam", &lh);
        tk_eig_info inf{};
        smallest_eigenvectors(ctx, N, nnz, rp_d, c_d, v_d, target_dimension, skip, tol > 0 ? tol : 1e-12,
                              max_matvecs > 0 ? max_matvecs : 200000, vec_d, val_d, &inf);
        check_device_errors(ctx);
        if (vh)
            copy_back(ctx, vectors, vec_d, (size_t)N * target_dimension);
        if (lh)
            copy_back(ctx, values, val_d, (size_t)target_dimension);
        TK_CUDA(cudaStreamSynchronize(ctx->stream));
        inf.ms = (float)std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (info)
            *info = inf;
        log(ctx, TK_LOG_INFO,
            "eigensolver: " + std::to_string(inf.iterations) + " rounds, " + std::to_string(inf.matvecs) +
                " block products, residual " + std::to_string(inf.max_residual));
        if (!inf.converged)
            throw Error(TK_ERR_NOT_CONVERGED, "eigendecomposition failed: the residual stayed above tol * B");
    });
}

int tk_assemble(tk_ctx* ctx, int method, int64_t N, int k, int td, const int32_t* idx, const double* weights,
                double shift, int64_t* row_ptr, int32_t* col_idx, double* vals, int64_t* nnz_io)
{
    return guarded(ctx, [&] {
        if (N <= 0)
            throw Error(TK_ERR_NO_DATA, "No data");
        if (method != TK_METHOD_KLLE && method != TK_METHOD_KLTSA && method != TK_METHOD_HLLE)
            throw Error(TK_ERR_UNSUPPORTED, "unsupported method");
        if (k < 1 || !idx || !weights || !nnz_io || (method != TK_METHOD_KLLE && td < 1))
            throw Error(TK_ERR_INVALID_ARG, "bad arguments");
        const size_t wcount = (size_t)N * k * weight_columns(method, td);
        td = method == TK_METHOD_KLLE ? td : weight_columns(method, td);
        const int32_t* idx_d = device_array(ctx, idx, (size_t)N * k, "io.idx_in");
        const double* w_d = device_array(ctx, weights, wcount, "io.w_in");
        bool rh = false;
        int64_t* rp_d = row_ptr ? device_out(ctx, row_ptr, (size_t)N + 1, "io.rowptr", &rh)
                                : (int64_t*)ctx->scratch.get("io.rowptr", sizeof(int64_t) * ((size_t)N + 1));
        const int64_t cap = *nnz_io;
        const int64_t nnz = assemble_rows(ctx, method, N, k, td, idx_d, w_d, shift, rp_d);
        check_device_errors(ctx);
        if (rh)
            copy_back(ctx, row_ptr, rp_d, (size_t)N + 1);
        *nnz_io = nnz;
        if (!col_idx || !vals)
        {
            TK_CUDA(cudaStreamSynchronize(ctx->stream));
            return;
        }
        if (cap < nnz)
            throw Error(TK_ERR_BUFFER_TOO_SMALL, "CSR capacity " + std::to_string(cap) + " < nnz " +
                                                     std::to_string(nnz));
        bool ch, vh;
        int32_t* c_d = device_out(ctx, col_idx, (size_t)nnz, "io.col", &ch);
        double* v_d = device_out(ctx, vals, (size_t)nnz, "io.vals", &vh);
        assemble_write(ctx, method, N, k, td, idx_d, w_d, shift, rp_d, c_d, v_d);
        check_device_errors(ctx);
        if (ch)
            copy_back(ctx, col_idx, c_d, (size_t)nnz);
        if (vh)
            copy_back(ctx, vals, v_d, (size_t)nnz);
        TK_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

int tk_local_operator(tk_ctx* ctx, const tk_params* params, const void* X, int dtype, int64_t N, int D,
                      int64_t ldx, tk_operator_info* info)
{
    return guarded(ctx, [&] {
        ctx->op_valid = false;
        if (!params)
            throw Error(TK_ERR_INVALID_ARG, "params is NULL");
        const tk_params& p = *params;
        if (p.method != TK_METHOD_KLLE && p.method != TK_METHOD_KLTSA && p.method != TK_METHOD_HLLE)
            throw Error(TK_ERR_UNSUPPORTED, "unsupported method");
        check_dtype(dtype);
        // ImplementationBase (methods/base.hpp:38-44): no data, target dimension in [1, N)
        if (N <= 0)
            throw Error(TK_ERR_NO_DATA, "No data to embed");
        validate_points(X, dtype, N, D, ldx);
        if (!(p.target_dimension >= 1 && p.target_dimension < N))
            throw Error(TK_ERR_INVALID_ARG, "[1, " + std::to_string(N) +
                                                ") range check failed for target dimension, its value is " +
                                                std::to_string(p.target_dimension));
        // DynamicImplementation::embedUsing (methods.hpp:30-31): one cancel poll
        if (p.cancel_function && p.cancel_function())
            throw Error(TK_ERR_CANCELLED, "cancelled");
        // find_neighbors_with (methods/base.hpp:85): num_neighbors in [3, N)
        if (!(p.num_neighbors >= 3 && p.num_neighbors < N))
            throw Error(TK_ERR_INVALID_ARG, "[3, " + std::to_string(N) +
                                                ") range check failed for number of neighbors, its value is " +
                                                std::to_string(p.num_neighbors));
        if (p.screen != TK_SCREEN_TENSOR && p.screen != TK_SCREEN_FP32)
            throw Error(TK_ERR_INVALID_ARG, "unknown screen engine");
        const int td = p.target_dimension;

        cudaStream_t st = ctx->stream;
        TK_CUDA(cudaEventRecord(ctx->ev[0], st));
        struct MarksOn
        {
            tk_ctx* c;
            ~MarksOn() { c->marks_on = false; }
        } marks_guard{ctx};
        ctx->marks_on = true;
        int64_t ldd;
        const void* Xd = device_points(ctx, X, dtype, N, D, ldx, &ldd, "op.X");

        // find_neighbors (neighbors/neighbors.hpp:173-213): clamp, brute, connectivity retry
        int k = p.num_neighbors;
        int retries = 0;
        int64_t uncert = 0;
        int32_t* idx_d = nullptr;
        float ms_knn = 0.f, ms_conn = 0.f;
        for (;;)
        {
            if (k > N - 1)
            {
                log(ctx, TK_LOG_WARNING,
                    "Number of neighbors is greater than number of objects to embed. Using greatest possible "
                    "number of neighbors.");
                k = (int)(N - 1);
            }
            idx_d = (int32_t*)ctx->scratch.get("op.idx", sizeof(int32_t) * (size_t)N * k);
            TK_CUDA(cudaEventRecord(ctx->ev[1], st));
            uncert = knn_device(ctx, Xd, dtype, N, D, ldd, k, p.screen, idx_d, nullptr);
            TK_CUDA(cudaEventRecord(ctx->ev[2], st));
            bool connected = true;
            if (p.check_connectivity)
            {
                connected = check_connected(ctx, N, k, idx_d);
                check_device_errors(ctx);
            }
            TK_CUDA(cudaEventRecord(ctx->ev[3], st));
            TK_CUDA(cudaEventSynchronize(ctx->ev[3]));
            ms_knn += elapsed(ctx->ev[1], ctx->ev[2]);
            ms_conn += elapsed(ctx->ev[2], ctx->ev[3]);
            if (connected)
            {
                log(ctx, TK_LOG_INFO, "The neighborhood graph with " + std::to_string(k) + " neighbors is connected.");
                break;
            }
            log(ctx, TK_LOG_WARNING, "The neighborhood graph with " + std::to_string(k) +
                                         " neighbors is not connected. Recomputing with a larger number of "
                                         "neighbors " + std::to_string(2 * k) + ".");
            k *= 2;
            ++retries;
        }

        // weights
        TK_CUDA(cudaEventRecord(ctx->ev[4], st));
        const int wcols = weight_columns(p.method, td);
        const size_t wcount = (size_t)N * k * wcols;
        double* w_d = (double*)ctx->scratch.get("op.w", sizeof(double) * wcount);
        if (p.method == TK_METHOD_KLLE)
            lle_weights(ctx, Xd, dtype, N, D, ldd, idx_d, k, p.klle_shift, w_d);
        else if (p.method == TK_METHOD_KLTSA)
            ltsa_basis(ctx, Xd, dtype, N, D, ldd, idx_d, k, td, w_d);
        else
            hessian_basis(ctx, Xd, dtype, N, D, ldd, idx_d, k, td, w_d);
        // assembly takes the weight columns (HLLE: the dp product columns); the
        // Hessian matrix has no diagonal shift (routines/locally_linear.hpp:236-243)
        const int atd = p.method == TK_METHOD_KLLE ? td : wcols;
        const double ashift = p.method == TK_METHOD_HLLE ? 0.0 : p.nullspace_shift;
        TK_CUDA(cudaEventRecord(ctx->ev[5], st));

        // M
        int64_t* rp_d = (int64_t*)ctx->scratch.get("op.rowptr", sizeof(int64_t) * ((size_t)N + 1));
        const int64_t nnz = assemble_rows(ctx, p.method, N, k, atd, idx_d, w_d, ashift, rp_d);
        int32_t* col_d = (int32_t*)ctx->scratch.get("op.col", sizeof(int32_t) * (size_t)std::max<int64_t>(nnz, 1));
        double* val_d = (double*)ctx->scratch.get("op.vals", sizeof(double) * (size_t)std::max<int64_t>(nnz, 1));
        assemble_write(ctx, p.method, N, k, atd, idx_d, w_d, ashift, rp_d, col_d, val_d);
        TK_CUDA(cudaEventRecord(ctx->ev[6], st));
        check_device_errors(ctx);

        tk_operator_info& o = ctx->op;
        std::memset(&o, 0, sizeof(o));
        o.n = N;
        o.k = k;
        o.method = p.method;
        o.target_dimension = td;
        o.connectivity_retries = retries;
        o.nnz = nnz;
        o.rows_uncertified = uncert;
        o.tie_rows = ctx->knn_ties;
        o.extra_rows = ctx->knn_extra;
        o.stage_ms[0] = ms_knn;
        o.stage_ms[1] = ms_conn;
        o.stage_ms[2] = elapsed(ctx->ev[4], ctx->ev[5]);
        o.stage_ms[3] = elapsed(ctx->ev[5], ctx->ev[6]);
        o.stage_ms[4] = elapsed(ctx->ev[0], ctx->ev[6]);
        o.stage_ms[5] = ctx->screen_ms;
        o.kernel_ms[0] = elapsed(ctx->kev[KM_PREP], ctx->kev[KM_SCREEN0]);
        o.kernel_ms[1] = elapsed(ctx->kev[KM_SCREEN0], ctx->kev[KM_SCREEN1]);
        o.kernel_ms[2] = elapsed(ctx->kev[KM_SCREEN1], ctx->kev[KM_RERANK]);
        o.kernel_ms[3] = o.stage_ms[2];
        o.kernel_ms[4] = elapsed(ctx->kev[KM_ASM0], ctx->kev[KM_ASM_REV]);
        o.kernel_ms[5] = elapsed(ctx->kev[KM_ASM_REV], ctx->kev[KM_ASM_ROWS]);
        o.kernel_ms[6] = elapsed(ctx->kev[KM_ASM_ROWS], ctx->kev[KM_ASM_END]);
        o.kernel_ms[7] = ms_conn;
        ctx->op_valid = true;
        if (info)
            *info = o;
    });
}

int tk_operator_get_info(const tk_ctx* ctx, tk_operator_info* info)
{
    if (!ctx || !info)
        return TK_ERR_INVALID_ARG;
    if (!ctx->op_valid)
        return TK_ERR_INVALID_ARG;
    *info = ctx->op;
    return TK_OK;
}

int tk_operator_device_views(tk_ctx* ctx, const int32_t** idx, const double** weights, const int64_t** row_ptr,
                             const int32_t** col_idx, const double** vals)
{
    if (!ctx || !ctx->op_valid)
        return TK_ERR_INVALID_ARG;
    auto& bufs = ctx->scratch.bufs;
    if (idx)
        *idx = (const int32_t*)bufs["op.idx"].ptr;
    if (weights)
        *weights = (const double*)bufs["op.w"].ptr;
    if (row_ptr)
        *row_ptr = (const int64_t*)bufs["op.rowptr"].ptr;
    if (col_idx)
        *col_idx = (const int32_t*)bufs["op.col"].ptr;
    if (vals)
        *vals = (const double*)bufs["op.vals"].ptr;
    return TK_OK;
}

int tk_operator_copy(tk_ctx* ctx, int32_t* idx, double* weights, int64_t* row_ptr, int32_t* col_idx, double* vals)
{
    return guarded(ctx, [&] {
        if (!ctx->op_valid)
            throw Error(TK_ERR_INVALID_ARG, "no operator held by this context");
        const tk_operator_info& o = ctx->op;
        auto& bufs = ctx->scratch.bufs;
        const size_t nk = (size_t)o.n * o.k;
        const size_t wc = nk * weight_columns(o.method, o.target_dimension);
        auto cp = [&](void* dst, const char* name, size_t bytes) {
            if (!dst || bytes == 0)
                return;
            TK_CUDA(cudaMemcpyAsync(dst, bufs[name].ptr, bytes, cudaMemcpyDefault, ctx->stream));
        };
        cp(idx, "op.idx", nk * sizeof(int32_t));
        cp(weights, "op.w", wc * sizeof(double));
        cp(row_ptr, "op.rowptr", ((size_t)o.n + 1) * sizeof(int64_t));
        cp(col_idx, "op.col", (size_t)o.nnz * sizeof(int32_t));
        cp(vals, "op.vals", (size_t)o.nnz * sizeof(double));
        TK_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

} // extern "C"
