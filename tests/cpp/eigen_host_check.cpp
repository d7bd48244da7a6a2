// Host linear algebra of the eigensolver (tapkee_gb300/csrc/eigen_host.h), run on
// the CPU: Cholesky factor, triangular inverse, cyclic Jacobi. Prints "ok".
#include <cmath>
#include <cstdio>
#include <vector>

#include "eigen_host.h"

using namespace tk::eigen_host;

namespace {

int failures = 0;
#define CHECK(cond)                                                                          \
    do                                                                                       \
    {                                                                                        \
        if (!(cond))                                                                         \
        {                                                                                    \
            std::fprintf(stderr, "FAILED %s at line %d\n", #cond, __LINE__);                \
            ++failures;                                                                      \
        }                                                                                    \
    } while (0)

unsigned long long state = 0x2545F4914F6CDD1Dull;
double uniform()  // xorshift64*, in [-1, 1)
{
    state ^= state >> 12;
    state ^= state << 25;
    state ^= state >> 27;
    return (double)((state * 0x2545F4914F6CDD1Dull) >> 11) * 0x1.0p-52 - 1.0;
}

using Mat = std::vector<double>;  // row-major n x n

Mat mul(int n, const Mat& A, const Mat& B, bool ta = false)
{
    Mat C((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < n; ++k)
        {
            const double a = ta ? A[(size_t)k * n + i] : A[(size_t)i * n + k];
            for (int j = 0; j < n; ++j)
                C[(size_t)i * n + j] += a * B[(size_t)k * n + j];
        }
    return C;
}

double max_abs(const Mat& A)
{
    double m = 0.0;
    for (double v : A)
        m = std::fmax(m, std::fabs(v));
    return m;
}

// a random orthogonal matrix (Gram-Schmidt of a random one)
Mat orthogonal(int n)
{
    Mat Q((size_t)n * n);
    for (double& v : Q)
        v = uniform();
    for (int c = 0; c < n; ++c)
    {
        for (int p = 0; p < c; ++p)
        {
            double d = 0.0;
            for (int r = 0; r < n; ++r)
                d += Q[(size_t)r * n + c] * Q[(size_t)r * n + p];
            for (int r = 0; r < n; ++r)
                Q[(size_t)r * n + c] -= d * Q[(size_t)r * n + p];
        }
        double nn = 0.0;
        for (int r = 0; r < n; ++r)
            nn += Q[(size_t)r * n + c] * Q[(size_t)r * n + c];
        for (int r = 0; r < n; ++r)
            Q[(size_t)r * n + c] /= std::sqrt(nn);
    }
    return Q;
}

// A = Q diag(lam) Q^T, then check the decomposition jacobi_eig returns
void check_eig(int n, const std::vector<double>& lam, double rel_tol)
{
    const Mat Q = orthogonal(n);
    Mat A((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
            for (int k = 0; k < n; ++k)
                A[(size_t)i * n + j] += Q[(size_t)i * n + k] * lam[k] * Q[(size_t)j * n + k];
    for (int i = 0; i < n; ++i)  // exactly symmetric input, as the solver symmetrises H
        for (int j = 0; j < i; ++j)
            A[(size_t)i * n + j] = A[(size_t)j * n + i];
    std::vector<double> w;
    Mat V;
    jacobi_eig(n, A, w, V);
    CHECK((int)w.size() == n);
    std::vector<double> sorted = lam;
    std::sort(sorted.begin(), sorted.end());
    double scale = 0.0;
    for (double l : lam)
        scale = std::fmax(scale, std::fabs(l));
    for (int i = 0; i < n; ++i)
    {
        if (i > 0)
            CHECK(w[i - 1] <= w[i]);
        CHECK(std::fabs(w[i] - sorted[i]) <= rel_tol * std::fabs(sorted[i]) + 1e-14 * scale);
    }
    // V^T V = I and A V = V diag(w)
    Mat VtV = mul(n, V, V, true);
    for (int i = 0; i < n; ++i)
        VtV[(size_t)i * n + i] -= 1.0;
    CHECK(max_abs(VtV) < 1e-13);
    Mat AV = mul(n, A, V);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
            AV[(size_t)i * n + j] -= V[(size_t)i * n + j] * w[j];
    CHECK(max_abs(AV) < 1e-13 * scale + 1e-300);
}

} // namespace

int main()
{
    // eigenvalues spread like the Rayleigh-Ritz matrices of the solver (1e-9 .. 1e-5),
    // with a repeated pair, at the block widths used (1, 16, 32) and a few others
    for (int n : {1, 2, 5, 16, 32})
    {
        std::vector<double> lam(n);
        for (int i = 0; i < n; ++i)
            lam[i] = std::pow(10.0, -9.0 + 4.0 * (n > 1 ? (double)i / (n - 1) : 0.0));
        if (n >= 5)
            lam[2] = lam[3];
        check_eig(n, lam, 1e-6);
    }
    {
        std::vector<double> lam(20);  // indefinite, O(1) spectrum
        for (double& l : lam)
            l = uniform() * 3.0;
        check_eig(20, lam, 1e-10);
    }
    // Cholesky of a Gram matrix, and the inverse of its factor
    for (int n : {1, 3, 16, 32})
    {
        const int rows = 4 * n + 3;
        Mat B((size_t)rows * n);
        for (double& v : B)
            v = uniform();
        Mat G((size_t)n * n, 0.0);
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j)
                for (int r = 0; r < rows; ++r)
                    G[(size_t)i * n + j] += B[(size_t)r * n + i] * B[(size_t)r * n + j];
        Mat R;
        CHECK(chol_upper(n, G, R));
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < i; ++j)
                CHECK(R[(size_t)i * n + j] == 0.0);
        Mat RtR = mul(n, R, R, true);
        for (size_t e = 0; e < RtR.size(); ++e)
            RtR[e] -= G[e];
        CHECK(max_abs(RtR) < 1e-12 * max_abs(G));
        Mat Ri = inv_upper(n, R);
        Mat I = mul(n, R, Ri);
        for (int i = 0; i < n; ++i)
            I[(size_t)i * n + i] -= 1.0;
        CHECK(max_abs(I) < 1e-12);
    }
    // not positive definite: reported, not factored
    {
        Mat G = {1.0, 0.0, 0.0, -1.0};
        Mat R;
        CHECK(!chol_upper(2, G, R));
        Mat Z = {0.0, 0.0, 0.0, 0.0};
        CHECK(!chol_upper(2, Z, R));
    }
    if (failures)
        return 1;
    std::printf("ok\n");
    return 0;
}
