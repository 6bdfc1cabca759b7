// Dense symmetric eigensolver for the eigensolvers' projected matrices (n <= ~64),
// host code: Householder reduction to tridiagonal form, then implicit symmetric QR
// steps with Wilkinson shifts (Golub & Van Loan, "Matrix Computations", sections
// 8.3.1 and 8.3.3), accumulating the orthogonal factors into the eigenvectors.
// O(n^3) with a small constant, about 10x fewer operations than cyclic Jacobi at
// n = 40, which matters because the mixed solver's next direction waits on it.
#pragma once

#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

namespace cigpu {

// a: n x n symmetric, row-major (destroyed). On return w holds the eigenvalues in
// ascending order and z (n x n, row-major) the eigenvectors as columns:
// eigenvector j is z[i * n + j], i = 0..n-1.
inline void symmetric_eigh(int n, std::vector<double> &a, std::vector<double> &w, std::vector<double> &z) {
    const size_t N = (size_t)n;
    z.assign(N * N, 0.0);
    for (size_t i = 0; i < N; ++i) z[i * N + i] = 1.0;
    w.assign(N, 0.0);
    if (n == 0) return;
    std::vector<double> v(N), p(N), q(N);
    // ---- Householder: A = Q T Q^T, Q accumulated in z ----
    for (int k = 0; k + 2 < n; ++k) {
        const int len = n - k - 1;
        double nx = 0;
        for (int i = 0; i < len; ++i) nx += a[(size_t)(k + 1 + i) * N + k] * a[(size_t)(k + 1 + i) * N + k];
        nx = std::sqrt(nx);
        if (nx == 0) continue;
        const double x0 = a[(size_t)(k + 1) * N + k];
        const double alpha = x0 >= 0 ? -nx : nx;
        for (int i = 0; i < len; ++i) v[i] = a[(size_t)(k + 1 + i) * N + k];
        v[0] -= alpha;
        double nv = 0;
        for (int i = 0; i < len; ++i) nv += v[i] * v[i];
        nv = std::sqrt(nv);
        if (nv == 0) continue;
        for (int i = 0; i < len; ++i) v[i] /= nv;
        // trailing block B <- H B H = B - 2 v q^T - 2 q v^T, q = B v - (v.Bv) v
        double K = 0;
        for (int i = 0; i < len; ++i) {
            double s = 0;
            const double *row = &a[(size_t)(k + 1 + i) * N + k + 1];
            for (int j = 0; j < len; ++j) s += row[j] * v[j];
            p[i] = s;
            K += v[i] * s;
        }
        for (int i = 0; i < len; ++i) q[i] = p[i] - K * v[i];
        for (int i = 0; i < len; ++i) {
            double *row = &a[(size_t)(k + 1 + i) * N + k + 1];
            for (int j = 0; j < len; ++j) row[j] -= 2.0 * (v[i] * q[j] + q[i] * v[j]);
        }
        a[(size_t)(k + 1) * N + k] = a[(size_t)k * N + k + 1] = alpha;
        for (int i = 1; i < len; ++i) a[(size_t)(k + 1 + i) * N + k] = a[(size_t)k * N + k + 1 + i] = 0.0;
        // Q <- Q H
        for (int r = 0; r < n; ++r) {
            double *row = &z[(size_t)r * N + k + 1];
            double t = 0;
            for (int j = 0; j < len; ++j) t += row[j] * v[j];
            t *= 2.0;
            for (int j = 0; j < len; ++j) row[j] -= t * v[j];
        }
    }
    std::vector<double> d(N), e(N, 0.0);
    for (int i = 0; i < n; ++i) d[i] = a[(size_t)i * N + i];
    for (int i = 0; i + 1 < n; ++i) e[i] = a[(size_t)(i + 1) * N + i];
    // ---- implicit symmetric QR on tridiag(d, e), deflating from the bottom ----
    const double eps = 2.220446049250313e-16;
    int m = n - 1, iters = 0;
    while (m > 0 && iters < 60 * n) {
        if (std::fabs(e[m - 1]) <= eps * (std::fabs(d[m - 1]) + std::fabs(d[m]))) {
            e[m - 1] = 0;
            --m;
            continue;
        }
        int l = m - 1;
        while (l > 0 && std::fabs(e[l - 1]) > eps * (std::fabs(d[l - 1]) + std::fabs(d[l]))) --l;
        ++iters;
        // Wilkinson shift from the trailing 2 x 2 block
        const double dd = 0.5 * (d[m - 1] - d[m]);
        const double em = e[m - 1];
        const double den = dd + (dd >= 0 ? 1.0 : -1.0) * std::hypot(dd, em);
        const double mu = den != 0 ? d[m] - em * em / den : d[m] - std::fabs(em);
        double x = d[l] - mu, zz = e[l];
        double bulge = 0;
        for (int k = l; k < m; ++k) {
            // rotation G = [[c, s], [-s, c]] on rows/cols k, k+1 with G^T (x, zz) = (r, 0)
            const double r = std::hypot(x, zz);
            double c = 1.0, s = 0.0;
            if (r != 0) {
                c = x / r;
                s = -zz / r;
            }
            if (k > l) e[k - 1] = c * e[k - 1] - s * bulge;  // = r; the bulge is gone
            const double pk = d[k], qk = d[k + 1], fk = e[k];
            d[k] = c * c * pk - 2.0 * c * s * fk + s * s * qk;
            d[k + 1] = s * s * pk + 2.0 * c * s * fk + c * c * qk;
            e[k] = c * s * (pk - qk) + (c * c - s * s) * fk;
            if (k + 1 < m) {
                bulge = -s * e[k + 1];
                e[k + 1] = c * e[k + 1];
                x = e[k];
                zz = bulge;
            }
            for (int i = 0; i < n; ++i) {
                double *zi = &z[(size_t)i * N];
                const double zk = zi[k], zk1 = zi[k + 1];
                zi[k] = c * zk - s * zk1;
                zi[k + 1] = s * zk + c * zk1;
            }
        }
    }
    // ascending order
    std::vector<int> idx(N);
    std::iota(idx.begin(), idx.end(), 0);
    std::sort(idx.begin(), idx.end(), [&](int x1, int x2) { return d[x1] < d[x2]; });
    std::vector<double> zs(N * N);
    for (int k = 0; k < n; ++k) {
        w[k] = d[idx[k]];
        for (int i = 0; i < n; ++i) zs[(size_t)i * N + k] = z[(size_t)i * N + idx[k]];
    }
    z.swap(zs);
}

}  // namespace cigpu
