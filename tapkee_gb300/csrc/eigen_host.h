// eigen_host.h -- the small dense linear algebra of the eigensolver's host loop
// (block width x block width): Cholesky for the Cholesky QR, the inverse of its
// triangular factor, and the cyclic Jacobi eigensolver of the Rayleigh-Ritz step.
// Plain C++ (no CUDA), so that host tests compile it with g++ directly.
#pragma once

#include <algorithm>
#include <cmath>
#include <vector>

namespace tk {
namespace eigen_host {

// G = R^T R with R upper triangular (row-major); false if G is not positive definite.
inline bool chol_upper(int n, const std::vector<double>& G, std::vector<double>& R)
{
    R.assign((size_t)n * n, 0.0);
    for (int j = 0; j < n; ++j)
    {
        double d = G[(size_t)j * n + j];
        for (int k = 0; k < j; ++k)
            d -= R[(size_t)k * n + j] * R[(size_t)k * n + j];
        if (!(d > 0.0))
            return false;
        const double rjj = std::sqrt(d);
        R[(size_t)j * n + j] = rjj;
        for (int i = j + 1; i < n; ++i)
        {
            double s = G[(size_t)j * n + i];
            for (int k = 0; k < j; ++k)
                s -= R[(size_t)k * n + j] * R[(size_t)k * n + i];
            R[(size_t)j * n + i] = s / rjj;
        }
    }
    return true;
}

// Inverse of an upper triangular R (row-major), by back substitution per column.
inline std::vector<double> inv_upper(int n, const std::vector<double>& R)
{
    std::vector<double> X((size_t)n * n, 0.0);
    for (int c = 0; c < n; ++c)
        for (int i = c; i >= 0; --i)
        {
            double s = (i == c) ? 1.0 : 0.0;
            for (int k = i + 1; k <= c; ++k)
                s -= R[(size_t)i * n + k] * X[(size_t)k * n + c];
            X[(size_t)i * n + c] = s / R[(size_t)i * n + i];
        }
    return X;
}

// Symmetric eigendecomposition by the cyclic Jacobi method (Golub & Van Loan,
// Matrix Computations, sec. 8.5): w ascending, V row-major with eigenvector j in
// column j.
inline void jacobi_eig(int n, std::vector<double> A, std::vector<double>& w, std::vector<double>& V)
{
    V.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i)
        V[(size_t)i * n + i] = 1.0;
    auto a = [&](int i, int j) -> double& { return A[(size_t)i * n + j]; };
    for (int sweep = 0; sweep < 100; ++sweep)
    {
        double off = 0.0, diag = 0.0;
        for (int i = 0; i < n; ++i)
        {
            diag += a(i, i) * a(i, i);
            for (int j = i + 1; j < n; ++j)
                off += a(i, j) * a(i, j);
        }
        if (off <= 1e-32 * diag || off == 0.0)
            break;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q)
            {
                const double apq = a(p, q);
                if (apq == 0.0)
                    continue;
                const double theta = (a(q, q) - a(p, p)) / (2.0 * apq);
                const double tt = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(tt * tt + 1.0), s = tt * c;
                for (int k = 0; k < n; ++k)
                {
                    const double akp = a(k, p), akq = a(k, q);
                    a(k, p) = c * akp - s * akq;
                    a(k, q) = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k)
                {
                    const double apk = a(p, k), aqk = a(q, k);
                    a(p, k) = c * apk - s * aqk;
                    a(q, k) = s * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k)
                {
                    const double vkp = V[(size_t)k * n + p], vkq = V[(size_t)k * n + q];
                    V[(size_t)k * n + p] = c * vkp - s * vkq;
                    V[(size_t)k * n + q] = s * vkp + c * vkq;
                }
            }
    }
    std::vector<int> ord(n);
    for (int i = 0; i < n; ++i)
        ord[i] = i;
    std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return a(x, x) < a(y, y); });
    w.resize(n);
    std::vector<double> Vs((size_t)n * n);
    for (int c = 0; c < n; ++c)
    {
        w[c] = a(ord[c], ord[c]);
        for (int r = 0; r < n; ++r)
            Vs[(size_t)r * n + c] = V[(size_t)r * n + ord[c]];
    }
    V.swap(Vs);
}

} // namespace eigen_host
} // namespace tk
