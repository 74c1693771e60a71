// Eigenvalues and eigenvectors of a dense symmetric matrix by the cyclic
// Jacobi method (plane rotations that zero one off-diagonal element at a time,
// sweeping all pairs until the off-diagonal mass is negligible; Golub & Van
// Loan, Matrix Computations, section 8.5).  O(n^3) per sweep, a handful of
// sweeps: meant for the set-up of small polymer Hessians (n up to a few
// thousand), not for a hot path.
#pragma once
#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

namespace pgh {

// a: n x n row-major symmetric (destroyed).  On return w holds the eigenvalues
// in ascending order and column j of v (row-major n x n) the unit eigenvector
// of w[j].  Returns the number of sweeps, or -1 if max_sweeps did not suffice.
inline int eigsym_jacobi(int n, std::vector<double> &a, std::vector<double> &w, std::vector<double> &v,
                         int max_sweeps = 100) {
    v.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; i++) v[(size_t)i * n + i] = 1.0;
    auto A = [&](int i, int j) -> double & { return a[(size_t)i * n + j]; };
    double diag = 0.0;
    for (int i = 0; i < n; i++) diag += A(i, i) * A(i, i);
    int sweep = 0;
    for (; sweep < max_sweeps; sweep++) {
        double off = 0.0;
        for (int p = 0; p < n; p++)
            for (int q = p + 1; q < n; q++) off += A(p, q) * A(p, q);
        if (off <= 1e-30 * std::max(diag, 1e-300)) break;
        for (int p = 0; p < n - 1; p++)
            for (int q = p + 1; q < n; q++) {
                const double apq = A(p, q);
                if (apq == 0.0) continue;
                // rotation angle: tan(2 theta) = 2 a_pq / (a_qq - a_pp), the smaller root for t
                const double theta = (A(q, q) - A(p, p)) / (2.0 * apq);
                const double t = (theta >= 0.0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; k++) {  // columns p, q
                    const double akp = A(k, p), akq = A(k, q);
                    A(k, p) = c * akp - s * akq;
                    A(k, q) = s * akp + c * akq;
                }
                for (int k = 0; k < n; k++) {  // rows p, q
                    const double apk = A(p, k), aqk = A(q, k);
                    A(p, k) = c * apk - s * aqk;
                    A(q, k) = s * apk + c * aqk;
                }
                for (int k = 0; k < n; k++) {  // accumulate V <- V J
                    const double vkp = v[(size_t)k * n + p], vkq = v[(size_t)k * n + q];
                    v[(size_t)k * n + p] = c * vkp - s * vkq;
                    v[(size_t)k * n + q] = s * vkp + c * vkq;
                }
            }
    }
    // ascending order
    std::vector<int> idx(n);
    std::iota(idx.begin(), idx.end(), 0);
    std::sort(idx.begin(), idx.end(), [&](int i, int j) { return A(i, i) < A(j, j); });
    w.resize(n);
    std::vector<double> vs((size_t)n * n);
    for (int j = 0; j < n; j++) {
        w[j] = A(idx[j], idx[j]);
        for (int k = 0; k < n; k++) vs[(size_t)k * n + j] = v[(size_t)k * n + idx[j]];
    }
    v.swap(vs);
    return sweep < max_sweeps ? sweep : -1;
}

}  // namespace pgh
