// tapkee_oracle.cpp -- CPU restatement of the reference's local-neighborhood
// operator stage, used ONLY as a test checker and as the timed CPU baseline.
//
// TEST INFRASTRUCTURE. Nothing in the product path (the tapkee_gb300 package,
// its CUDA library or its C ABI) links, loads or calls this file. Only tests/,
// __graft_entry__.smoke() and bench.py (its CPU-baseline / reference arm) use it.
//
// Parity status: the reference (lisitsyn/tapkee 1.3.4) is header-only C++ that
// needs Eigen 3.4 for every routine on this path; Eigen is not available where
// this project is built, so the reference cannot be compiled and this file is a
// restatement of its algorithms in plain C++ (FP64, like the reference's
// ScalarType). It is pinned by
//   * the reference's only known-answer test on the path, the 1-D integer line
//     kNN set check (test/unit/neighbors.cpp:17-52 and :92-127), ported in
//     tests/test_oracle.py;
//   * independent third-party implementations of the same published formulas
//     (scikit-learn's barycenter weights / LTSA alignment, scipy sparse algebra),
//     whose outputs are committed as fixtures under tests/golden/.
// The W, M and LTSA-basis VALUES are therefore not pinned by the reference's own
// tests (it has none for them): parity of those values is "unpinned" with
// respect to the reference itself and cross-checked against scikit-learn.
//
// Every routine cites the reference file:line it restates (paths relative to the
// reference project root).

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <stack>
#include <utility>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {

// Linear kernel k(a,b) = <x_a, x_b>, the column dot of
// callbacks/eigen_callbacks.hpp:34-46 (sequential summation order).
static inline double kernel_dot(const double* X, int64_t D, int64_t a, int64_t b)
{
    const double* xa = X + a * D;
    const double* xb = X + b * D;
    double s = 0.0;
    for (int64_t d = 0; d < D; ++d)
        s += xa[d] * xb[d];
    return s;
}

// Brute-force kNN: neighbors/neighbors.hpp:119-149 with the kernel-trick
// distance KernelDistance::distance (neighbors/neighbors.hpp:49-52):
//   dist(i,j) = sqrt(k(i,i) - 2 k(i,j) + k(j,j)).
// For each query all N (index, distance) records are built, std::nth_element
// partitions at k+1 with the strict comparator of neighbors.hpp:28-34, and the
// first k+1 records minus the query itself (by identity) are kept in partition
// order. Rows where the query is not among the first k+1 records (k+1 exact
// duplicates) yield k+1 neighbors in the reference; here the first k are kept,
// row_count[i] records k+1 and extra_out[i] (optional; -1 elsewhere) the
// (k+1)-th, so callers can detect and compare them.
//
// The reference's brute loop is serial; queries are independent, so the loop is
// split across OpenMP threads (same per-query arithmetic, same results).
int oracle_knn_brute(const double* X, int64_t N, int64_t D, int k, int32_t* idx_out, double* dist_out,
                     int32_t* row_count, int32_t* extra_out, int nthreads)
{
    if (N <= 0 || k <= 0 || k > N - 1)
        return -1;
    std::vector<double> kdiag(N);
    for (int64_t i = 0; i < N; ++i)
        kdiag[i] = kernel_dot(X, D, i, i);
#pragma omp parallel num_threads(nthreads > 0 ? nthreads : 1)
    {
        std::vector<std::pair<int64_t, double>> distances;
        distances.reserve(N);
#pragma omp for schedule(dynamic, 16)
        for (int64_t i = 0; i < N; ++i)
        {
            distances.clear();
            for (int64_t j = 0; j < N; ++j)
                distances.emplace_back(j, std::sqrt(kdiag[i] - 2 * kernel_dot(X, D, i, j) + kdiag[j]));
            std::nth_element(distances.begin(), distances.begin() + k + 1, distances.end(),
                             [](const std::pair<int64_t, double>& l, const std::pair<int64_t, double>& r) {
                                 return l.second < r.second;
                             });
            int c = 0, total = 0;
            if (extra_out)
                extra_out[i] = -1;
            for (int m = 0; m < k + 1 && m < N; ++m)
            {
                if (distances[m].first != i)
                {
                    if (c < k)
                    {
                        idx_out[i * k + c] = (int32_t)distances[m].first;
                        if (dist_out)
                            dist_out[i * k + c] = distances[m].second;
                        ++c;
                    }
                    else if (extra_out)
                        extra_out[i] = (int32_t)distances[m].first;
                    ++total;
                }
            }
            if (row_count)
                row_count[i] = total;
        }
    }
    return 0;
}

// Same as oracle_knn_brute for a subset of query rows (used to time a bounded
// sample of the serial reference loop on large N).
int oracle_knn_brute_rows(const double* X, int64_t N, int64_t D, int k, const int64_t* rows, int64_t nrows,
                          int32_t* idx_out, int nthreads)
{
    if (N <= 0 || k <= 0 || k > N - 1)
        return -1;
    std::vector<double> kdiag(N);
    for (int64_t i = 0; i < N; ++i)
        kdiag[i] = kernel_dot(X, D, i, i);
#pragma omp parallel num_threads(nthreads > 0 ? nthreads : 1)
    {
        std::vector<std::pair<int64_t, double>> distances;
        distances.reserve(N);
#pragma omp for schedule(dynamic, 4)
        for (int64_t r = 0; r < nrows; ++r)
        {
            int64_t i = rows[r];
            distances.clear();
            for (int64_t j = 0; j < N; ++j)
                distances.emplace_back(j, std::sqrt(kdiag[i] - 2 * kernel_dot(X, D, i, j) + kdiag[j]));
            std::nth_element(distances.begin(), distances.begin() + k + 1, distances.end(),
                             [](const std::pair<int64_t, double>& l, const std::pair<int64_t, double>& r) {
                                 return l.second < r.second;
                             });
            int c = 0;
            for (int m = 0; m < k + 1 && c < k; ++m)
                if (distances[m].first != i)
                    idx_out[r * k + c++] = (int32_t)distances[m].first;
        }
    }
    return 0;
}

// Iterative DFS from vertex 0 over kNN out-edges: neighbors/connected.hpp:19-62.
// Returns 1 when all N vertices are reached.
int oracle_is_connected(int64_t N, int k, const int32_t* idx)
{
    if (N <= 0)
        return 0;
    std::vector<bool> visited(N, false);
    std::stack<int64_t> stack;
    int64_t nvisited = 0;
    stack.push(0);
    while (!stack.empty())
    {
        int64_t current = stack.top();
        stack.pop();
        if (visited[current])
            continue;
        visited[current] = true;
        ++nvisited;
        if (nvisited == N)
            break;
        for (int j = 0; j < k; ++j)
        {
            int64_t nb = idx[current * k + j];
            if (!visited[nb])
                stack.push(nb);
        }
    }
    return nvisited == N ? 1 : 0;
}

// LDLT with symmetric (diagonal) pivoting and solve C w = rhs, restating the
// algorithm of the dense LDLT the reference calls at
// routines/locally_linear.hpp:130 (pivot = largest remaining |diagonal|).
// C is n x n, row-major, full symmetric; it is overwritten.
static void ldlt_solve(double* C, int n, const double* rhs, double* w)
{
    // Storage during step j: C[j:, j:] is the current (symmetric, full) Schur
    // complement and C[j:, :j] holds the computed unit-lower factor L.
    std::vector<int> perm(n);
    std::iota(perm.begin(), perm.end(), 0);
    std::vector<double> dvals(n);
    for (int j = 0; j < n; ++j)
    {
        int p = j;
        double best = std::fabs(C[j * n + j]);
        for (int t = j + 1; t < n; ++t)
            if (std::fabs(C[t * n + t]) > best)
            {
                best = std::fabs(C[t * n + t]);
                p = t;
            }
        if (p != j)
        {
            std::swap(perm[j], perm[p]);
            for (int t = 0; t < n; ++t)
                std::swap(C[j * n + t], C[p * n + t]);
            for (int t = 0; t < n; ++t)
                std::swap(C[t * n + j], C[t * n + p]);
        }
        const double djj = C[j * n + j];
        dvals[j] = djj;
        for (int i = j + 1; i < n; ++i)
            C[i * n + j] = (djj != 0.0) ? C[i * n + j] / djj : 0.0;
        for (int i = j + 1; i < n; ++i)
            for (int t = j + 1; t < n; ++t)
                C[i * n + t] -= C[i * n + j] * djj * C[t * n + j];
    }
    // P C P^T = L D L^T  ->  w = P^T L^-T D^-1 L^-1 P rhs (zero pivots -> 0,
    // the pseudo-inverse convention of the dense LDLT solve)
    std::vector<double> y(n);
    for (int i = 0; i < n; ++i)
        y[i] = rhs[perm[i]];
    for (int i = 0; i < n; ++i)
        for (int t = 0; t < i; ++t)
            y[i] -= C[i * n + t] * y[t];
    for (int i = 0; i < n; ++i)
        y[i] = (dvals[i] != 0.0) ? y[i] / dvals[i] : 0.0;
    for (int i = n - 1; i >= 0; --i)
        for (int t = i + 1; t < n; ++t)
            y[i] -= C[t * n + i] * y[t];
    for (int i = 0; i < n; ++i)
        w[perm[i]] = y[i];
}

// LLE reconstruction weights: routines/locally_linear.hpp:90-159 (per point,
// :107-131). Gram in kernel form (:118-126)
//   C_ab = k(x,x) - k(x,n_a) - k(x,n_b) + k(n_a,n_b),
// regularised C += klle_shift * trace(C) * I (:128-129), w = C^{-1} 1 (:130),
// w /= sum(w) (:131). W_out is N x k, aligned with idx.
int oracle_lle_weights(const double* X, int64_t N, int64_t D, const int32_t* idx, int k, double klle_shift,
                       double* W_out, int nthreads)
{
#pragma omp parallel num_threads(nthreads > 0 ? nthreads : 1)
    {
        std::vector<double> C(k * k), dots(k), rhs(k, 1.0), w(k);
#pragma omp for schedule(static)
        for (int64_t i = 0; i < N; ++i)
        {
            const int32_t* nb = idx + i * k;
            double kv = kernel_dot(X, D, i, i);
            for (int a = 0; a < k; ++a)
                dots[a] = kernel_dot(X, D, i, nb[a]);
            for (int a = 0; a < k; ++a)
                for (int b = a; b < k; ++b)
                {
                    double v = kv - dots[a] - dots[b] + kernel_dot(X, D, nb[a], nb[b]);
                    C[a * k + b] = v;
                    C[b * k + a] = v;
                }
            double trace = 0.0;
            for (int a = 0; a < k; ++a)
                trace += C[a * k + a];
            for (int a = 0; a < k; ++a)
                C[a * k + a] += klle_shift * trace;
            ldlt_solve(C.data(), k, rhs.data(), w.data());
            double s = 0.0;
            for (int a = 0; a < k; ++a)
                s += w[a];
            for (int a = 0; a < k; ++a)
                W_out[i * k + a] = w[a] / s;
        }
    }
    return 0;
}

// LLE weights of a subset of points (rows[r] with neighbours idx_rows[r]); same
// per-point arithmetic as oracle_lle_weights. Used to time / check a bounded
// sample of a large problem.
int oracle_lle_weights_rows(const double* X, int64_t N, int64_t D, const int64_t* rows, int64_t nrows,
                            const int32_t* idx_rows, int k, double klle_shift, double* W_out, int nthreads)
{
    (void)N;
#pragma omp parallel num_threads(nthreads > 0 ? nthreads : 1)
    {
        std::vector<double> C(k * k), dots(k), rhs(k, 1.0), w(k);
#pragma omp for schedule(static)
        for (int64_t r = 0; r < nrows; ++r)
        {
            const int64_t i = rows[r];
            const int32_t* nb = idx_rows + r * k;
            double kv = kernel_dot(X, D, i, i);
            for (int a = 0; a < k; ++a)
                dots[a] = kernel_dot(X, D, i, nb[a]);
            for (int a = 0; a < k; ++a)
                for (int b = a; b < k; ++b)
                {
                    double v = kv - dots[a] - dots[b] + kernel_dot(X, D, nb[a], nb[b]);
                    C[a * k + b] = v;
                    C[b * k + a] = v;
                }
            double trace = 0.0;
            for (int a = 0; a < k; ++a)
                trace += C[a * k + a];
            for (int a = 0; a < k; ++a)
                C[a * k + a] += klle_shift * trace;
            ldlt_solve(C.data(), k, rhs.data(), w.data());
            double s = 0.0;
            for (int a = 0; a < k; ++a)
                s += w[a];
            for (int a = 0; a < k; ++a)
                W_out[r * k + a] = w[a] / s;
        }
    }
    return 0;
}

// Cyclic Jacobi eigen-decomposition of a symmetric n x n matrix (row-major A,
// destroyed). Eigenvalues ascending in evals; eigenvectors as columns of V
// (row-major n x n). Restates the published cyclic Jacobi method; the
// reference uses a dense self-adjoint eigensolver (routines/locally_linear.hpp:60)
// and only the spanned subspace enters the result (G G^T at :63).
static void jacobi_eigen(double* A, int n, double* evals, double* V)
{
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
            V[i * n + j] = (i == j) ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 100; ++sweep)
    {
        double off = 0.0, diag = 0.0;
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j)
                (i == j ? diag : off) += A[i * n + j] * A[i * n + j];
        if (off <= 1e-30 * (diag + 1e-300))
            break;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q)
            {
                double apq = A[p * n + q];
                if (apq == 0.0)
                    continue;
                double app = A[p * n + p], aqq = A[q * n + q];
                double theta = (aqq - app) / (2.0 * apq);
                double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int r = 0; r < n; ++r)
                {
                    double arp = A[r * n + p], arq = A[r * n + q];
                    A[r * n + p] = c * arp - s * arq;
                    A[r * n + q] = s * arp + c * arq;
                }
                for (int r = 0; r < n; ++r)
                {
                    double apr = A[p * n + r], aqr = A[q * n + r];
                    A[p * n + r] = c * apr - s * aqr;
                    A[q * n + r] = s * apr + c * aqr;
                }
                for (int r = 0; r < n; ++r)
                {
                    double vrp = V[r * n + p], vrq = V[r * n + q];
                    V[r * n + p] = c * vrp - s * vrq;
                    V[r * n + q] = s * vrp + c * vrq;
                }
            }
    }
    // sort ascending
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::vector<double> d(n);
    for (int i = 0; i < n; ++i)
        d[i] = A[i * n + i];
    std::sort(order.begin(), order.end(), [&](int a, int b) { return d[a] < d[b]; });
    std::vector<double> Vs(n * n);
    for (int c = 0; c < n; ++c)
    {
        evals[c] = d[order[c]];
        for (int r = 0; r < n; ++r)
            Vs[r * n + c] = V[r * n + order[c]];
    }
    std::memcpy(V, Vs.data(), sizeof(double) * n * n);
}

// Centred neighbour Gram and its top eigenvectors, shared by the LTSA basis
// (routines/locally_linear.hpp:45-63) and the Hessian weights (:188-204): the
// Gram of the neighbours only, K_ab = k(n_a,n_b) (:47-55 / :188-196), double
// centring centerMatrix (utils/matrix.hpp:12-19), and the eigenvectors of the td
// largest eigenvalues in ascending order, rightCols(td) (:60-61 / :200-204).
// top is k x td row-major; ev receives the k ascending eigenvalues. G, V and cm
// are caller scratch of k*k, k*k and k doubles.
static void local_top_basis(const double* X, int64_t D, const int32_t* nb, int k, int td, double* G, double* V,
                            double* cm, double* ev, double* top)
{
    for (int a = 0; a < k; ++a)
        for (int b = a; b < k; ++b)
        {
            double v = kernel_dot(X, D, nb[a], nb[b]);
            G[a * k + b] = v;
            G[b * k + a] = v;
        }
    // centerMatrix: K + mean(K) - colmean (row-wise) - colmean (col-wise)
    double grand = 0.0;
    for (int b = 0; b < k; ++b)
    {
        double s = 0.0;
        for (int a = 0; a < k; ++a)
            s += G[a * k + b];
        cm[b] = s / k;
    }
    for (int t = 0; t < k * k; ++t)
        grand += G[t];
    grand /= (double)k * k;
    for (int a = 0; a < k; ++a)
        for (int b = 0; b < k; ++b)
            G[a * k + b] = G[a * k + b] + grand - cm[b] - cm[a];
    jacobi_eigen(G, k, ev, V);
    for (int a = 0; a < k; ++a)
        for (int t = 0; t < td; ++t)
            top[a * td + t] = V[a * k + (k - td + t)];
}

// LTSA local tangent basis: routines/locally_linear.hpp:20-88 (per point,
// :45-63), the basis of local_top_basis. V_out is N x k x td (row-major); the
// alignment block is P = (1/k) 1 1^T + V V^T (G = [1/sqrt(k) 1, V], :36-37,63).
// evals_out (optional) receives the k ascending eigenvalues per point.
int oracle_ltsa_basis(const double* X, int64_t N, int64_t D, const int32_t* idx, int k, int td, double* V_out,
                      double* evals_out, int nthreads)
{
#pragma omp parallel num_threads(nthreads > 0 ? nthreads : 1)
    {
        std::vector<double> G(k * k), V(k * k), ev(k), cm(k);
#pragma omp for schedule(static)
        for (int64_t i = 0; i < N; ++i)
        {
            local_top_basis(X, D, idx + i * k, k, td, G.data(), V.data(), cm.data(), ev.data(),
                            V_out + i * (int64_t)k * td);
            if (evals_out)
                for (int a = 0; a < k; ++a)
                    evals_out[i * k + a] = ev[a];
        }
    }
    return 0;
}

// Hessian LLE weights: routines/locally_linear.hpp:161-255 (per point,
// :184-243). With the tangent basis V (k x td) of local_top_basis:
//   Yi = [1, V, products V_j * V_{j+p}]                          (:203-214)
//   Gram-Schmidt over the columns of Yi in order, each column normalised (:216-225)
//   a product column is divided by its sum when the sum exceeds 1e-4 (:226-231)
//   B = Yr Yr^T with Yr the dp = td (td + 1) / 2 product columns    (:234)
// B_out is N x k x k (row-major); the point's triplets are (n_a, n_b, B_ab) for
// all a, b (:236-243). The reference places the product columns with
// ct += ct + td - j (:213), which matches the ordered pairs j <= j + p only for
// td <= 2; for td >= 3 it writes past the dp columns of Yi. This restatement
// therefore accepts td <= 2 and returns -1 otherwise.
int oracle_hessian_blocks(const double* X, int64_t N, int64_t D, const int32_t* idx, int k, int td, double* B_out,
                          int nthreads)
{
    if (td < 1 || td > 2)
        return -1;
    const int dp = td * (td + 1) / 2;
    const int ncol = 1 + td + dp;
#pragma omp parallel num_threads(nthreads > 0 ? nthreads : 1)
    {
        std::vector<double> G(k * k), V(k * k), ev(k), cm(k), top(k * td), Y((size_t)k * ncol);
        auto col = [&](int c) { return Y.data() + (size_t)c * k; };  // column-major Yi
#pragma omp for schedule(static)
        for (int64_t i = 0; i < N; ++i)
        {
            local_top_basis(X, D, idx + i * k, k, td, G.data(), V.data(), cm.data(), ev.data(), top.data());
            for (int a = 0; a < k; ++a)
            {
                col(0)[a] = 1.0;
                for (int t = 0; t < td; ++t)
                    col(1 + t)[a] = top[a * td + t];
            }
            int ct = 0;
            for (int j = 0; j < td; ++j)
            {
                for (int p = 0; p < td - j; ++p)
                    for (int a = 0; a < k; ++a)
                        col(ct + p + 1 + td)[a] = col(j + 1)[a] * col(j + p + 1)[a];
                ct += ct + td - j;
            }
            for (int c = 0; c < ncol; ++c)
            {
                double* yc = col(c);
                for (int j = 0; j < c; ++j)
                {
                    const double* yj = col(j);
                    double r = 0.0;
                    for (int a = 0; a < k; ++a)
                        r += yc[a] * yj[a];
                    for (int a = 0; a < k; ++a)
                        yc[a] -= r * yj[a];
                }
                double nrm = 0.0;
                for (int a = 0; a < k; ++a)
                    nrm += yc[a] * yc[a];
                // (1.f / norm) in the reference: the float 1 promotes to double
                const double inv = 1.0f / std::sqrt(nrm);
                for (int a = 0; a < k; ++a)
                    yc[a] *= inv;
            }
            for (int q = 0; q < dp; ++q)
            {
                double* yc = col(1 + td + q);
                double s = 0.0;
                for (int a = 0; a < k; ++a)
                    s += yc[a];
                if (s > 1e-4)
                    for (int a = 0; a < k; ++a)
                        yc[a] /= s;
            }
            double* B = B_out + i * (int64_t)k * k;
            for (int a = 0; a < k; ++a)
                for (int b = 0; b < k; ++b)
                {
                    double s = 0.0;
                    for (int q = 0; q < dp; ++q)
                        s += col(1 + td + q)[a] * col(1 + td + q)[b];
                    B[a * k + b] = s;
                }
        }
    }
    return 0;
}

// Triplet generation + Eigen-style setFromTriplets (utils/sparse.hpp:16-21):
// duplicates are summed in triplet order; the result is written as CSR with
// ascending column indices per row. Triplets are generated serially, point by
// point, in the push order of
//   LLE  (routines/locally_linear.hpp:133-146):
//        (i,i,1+shift), then per a: (n_a,i,-w_a), (i,n_a,-w_a), (n_a,n_b,w_a w_b) for b
//   LTSA (routines/locally_linear.hpp:65-77):
//        (i,i,shift), then per a: (n_a,n_a,1), (n_a,n_b,-P_ab) for b, P = (1/k)11^T + V V^T
//   HLLE (routines/locally_linear.hpp:236-243):
//        per a: (n_a,n_b,B_ab) for b; no diagonal shift
// method: 0 = LLE (weights = W, N x k), 1 = LTSA (weights = V, N x k x td),
// 2 = Hessian (weights = B, N x k x k; td and shift unused).
// Returns nnz, or -1 if cap is too small (row_ptr is filled in any case).
int64_t oracle_assemble(int method, int64_t N, int k, int td, const int32_t* idx, const double* weights,
                        double shift, int64_t* row_ptr, int32_t* col_idx, double* vals, int64_t cap)
{
    struct Trip
    {
        int32_t r, c;
        double v;
    };
    std::vector<Trip> trips;
    trips.reserve((size_t)N * (k * k + 2 * k + 1));
    std::vector<double> P(k * k);
    for (int64_t i = 0; i < N; ++i)
    {
        const int32_t* nb = idx + i * k;
        if (method == 0)
        {
            const double* w = weights + i * k;
            trips.push_back({(int32_t)i, (int32_t)i, 1.0 + shift});
            for (int a = 0; a < k; ++a)
            {
                trips.push_back({nb[a], (int32_t)i, -w[a]});
                trips.push_back({(int32_t)i, nb[a], -w[a]});
                for (int b = 0; b < k; ++b)
                    trips.push_back({nb[a], nb[b], w[a] * w[b]});
            }
        }
        else if (method == 2)
        {
            const double* B = weights + i * (int64_t)k * k;
            for (int a = 0; a < k; ++a)
                for (int b = 0; b < k; ++b)
                    trips.push_back({nb[a], nb[b], B[a * k + b]});
        }
        else
        {
            const double* V = weights + i * (int64_t)k * td;
            for (int a = 0; a < k; ++a)
                for (int b = 0; b < k; ++b)
                {
                    double s = 1.0 / k;
                    for (int t = 0; t < td; ++t)
                        s += V[a * td + t] * V[b * td + t];
                    P[a * k + b] = s;
                }
            trips.push_back({(int32_t)i, (int32_t)i, shift});
            for (int a = 0; a < k; ++a)
            {
                trips.push_back({nb[a], nb[a], 1.0});
                for (int b = 0; b < k; ++b)
                    trips.push_back({nb[a], nb[b], -P[a * k + b]});
            }
        }
    }
    // stable sort by (row, col): equal entries keep triplet order -> summed in
    // triplet order like setFromTriplets
    std::stable_sort(trips.begin(), trips.end(),
                     [](const Trip& x, const Trip& y) { return x.r != y.r ? x.r < y.r : x.c < y.c; });
    int64_t nnz = 0;
    std::vector<int64_t> counts(N, 0);
    for (size_t t = 0; t < trips.size(); ++t)
        if (t == 0 || trips[t].r != trips[t - 1].r || trips[t].c != trips[t - 1].c)
        {
            ++counts[trips[t].r];
            ++nnz;
        }
    row_ptr[0] = 0;
    for (int64_t r = 0; r < N; ++r)
        row_ptr[r + 1] = row_ptr[r] + counts[r];
    if (col_idx == nullptr || vals == nullptr || cap < nnz)
        return cap < nnz ? -1 : nnz;
    int64_t pos = -1;
    for (size_t t = 0; t < trips.size(); ++t)
    {
        if (t == 0 || trips[t].r != trips[t - 1].r || trips[t].c != trips[t - 1].c)
        {
            ++pos;
            col_idx[pos] = trips[t].c;
            vals[pos] = trips[t].v;
        }
        else
            vals[pos] += trips[t].v;
    }
    return nnz;
}


// construct_neighborhood_preserving_eigenproblem (kind 0) and
// construct_lltsa_eigenproblem (kind 1), routines/locally_linear.hpp:257-338,
// for the linear kernel's feature vectors (the rows of X, points-major). The
// sparse matrix is given in CSR; it is symmetric, so its CSR arrays are also the
// CSC arrays the reference's InnerIterator walks, and the loops below visit
// the nonzeros in that order. lhs and rhs are D x D column-major:
//   rhs: upper triangle of sum_i x_i x_i^T (LLTSA: minus s s^T / N, s = sum_i
//        x_i), then rhs = (rhs + rhs^T) / 2 -- the lower triangle enters as
//        zero, so off-diagonal entries end halved, as in the reference;
//   lhs: upper triangle of sum over nonzeros (i, j) of v (x_i x_j^T + x_j x_i^T)
//        (LLTSA: minus s s^T / N); the lower triangle stays zero.
void oracle_eigenproblem_pair(int kind, int64_t N, int D, const double* X, const int64_t* row_ptr,
                              const int32_t* col_idx, const double* vals, double* lhs, double* rhs)
{
    std::vector<double> L((size_t)D * D, 0.0), R((size_t)D * D, 0.0), s(D, 0.0);
    auto at = [D](std::vector<double>& M, int a, int b) -> double& { return M[(size_t)b * D + a]; };
    for (int64_t i = 0; i < N; ++i)
    {
        const double* x = X + i * D;
        for (int a = 0; a < D; ++a)
            s[a] += x[a];
        for (int b = 0; b < D; ++b)
            for (int a = 0; a <= b; ++a)
                at(R, a, b) += x[a] * x[b];
    }
    if (kind == 1)
        for (int b = 0; b < D; ++b)
            for (int a = 0; a <= b; ++a)
                at(R, a, b) += -1.0 / (double)N * s[a] * s[b];
    for (int64_t c = 0; c < N; ++c)  // outer index (column of the CSC view)
        for (int64_t p = row_ptr[c]; p < row_ptr[c + 1]; ++p)
        {
            const int64_t r = col_idx[p];  // it.row()
            const double v = vals[p];
            const double* xi = X + r * D;
            const double* xj = X + c * D;
            for (int b = 0; b < D; ++b)
                for (int a = 0; a <= b; ++a)
                    at(L, a, b) += v * xi[a] * xj[b] + v * xj[a] * xi[b];
        }
    if (kind == 1)
        for (int b = 0; b < D; ++b)
            for (int a = 0; a <= b; ++a)
                at(L, a, b) += -1.0 / (double)N * s[a] * s[b];
    for (int b = 0; b < D; ++b)
        for (int a = 0; a < D; ++a)
        {
            lhs[(size_t)b * D + a] = L[(size_t)b * D + a];
            rhs[(size_t)b * D + a] = (R[(size_t)b * D + a] + R[(size_t)a * D + b]) / 2.0;
        }
}

} // extern "C"
