// Eigenvalues of a small real nonsymmetric matrix, one source for the device and the host.
//
// Householder reduction to upper Hessenberg form, then implicit double-shift QR steps with
// deflation (J. G. F. Francis, "The QR transformation", Comput. J. 4 (1961); Golub & Van Loan,
// Matrix Computations, 4th ed., Algorithms 7.4.2, 7.5.1 and 7.5.2).  Only eigenvalues are
// wanted, so a QR step updates just the active diagonal window: the blocks outside it do not
// change the window's eigenvalues.  Every loop has a fixed bound; a window that needs more
// than the iteration budget makes the call return 1 (no trap, no spin).
//
// Layout: column-major, a[i + j n] = A(i, j), overwritten.  work: n doubles.
#pragma once

#include <math.h>

#if defined(__CUDACC__)
#define TNR_HD __host__ __device__
#else
#define TNR_HD
#endif

namespace tnr {

// Householder vector of a 2- or 3-vector x (m = 2 or 3): v = [1, v1, v2] and beta with
// (I - beta v v^T) x = +-|x| e1; beta = 0 when x is already along e1.
TNR_HD inline void house_small(double x0, double x1, double x2, int m, double* v1, double* v2, double* beta) {
    const double sigma = x1 * x1 + (m == 3 ? x2 * x2 : 0.0);
    if (sigma == 0.0) {
        *v1 = 0.0;
        *v2 = 0.0;
        *beta = 0.0;
        return;
    }
    const double mu = sqrt(x0 * x0 + sigma);
    const double v0 = x0 <= 0.0 ? x0 - mu : -sigma / (x0 + mu);   // x0 - mu without cancellation
    *beta = 2.0 * v0 * v0 / (sigma + v0 * v0);
    *v1 = x1 / v0;
    *v2 = m == 3 ? x2 / v0 : 0.0;
}

// A <- Q^T A Q upper Hessenberg (entries below the subdiagonal set to 0)
TNR_HD inline void hessenberg_reduce(double* a, int n, double* v) {
#define TNR_A(i, j) a[(i) + (long long)(j) * n]
    for (int k = 0; k + 2 < n; ++k) {
        double sigma = 0.0;
        for (int i = k + 2; i < n; ++i) sigma += TNR_A(i, k) * TNR_A(i, k);
        if (sigma == 0.0) continue;
        const double x0 = TNR_A(k + 1, k);
        const double mu = sqrt(x0 * x0 + sigma);
        const double v0 = x0 <= 0.0 ? x0 - mu : -sigma / (x0 + mu);
        const double beta = 2.0 * v0 * v0 / (sigma + v0 * v0);
        v[k + 1] = 1.0;
        for (int i = k + 2; i < n; ++i) v[i] = TNR_A(i, k) / v0;
        for (int j = k; j < n; ++j) {            // rows k+1.. from the left
            double s = 0.0;
            for (int i = k + 1; i < n; ++i) s += v[i] * TNR_A(i, j);
            s *= beta;
            for (int i = k + 1; i < n; ++i) TNR_A(i, j) -= s * v[i];
        }
        for (int i = k + 2; i < n; ++i) TNR_A(i, k) = 0.0;
        for (int i = 0; i < n; ++i) {            // columns k+1.. from the right
            double s = 0.0;
            for (int j = k + 1; j < n; ++j) s += TNR_A(i, j) * v[j];
            s *= beta;
            for (int j = k + 1; j < n; ++j) TNR_A(i, j) -= s * v[j];
        }
    }
#undef TNR_A
}

// Eigenvalues (wr[i] + i wi[i]; complex pairs adjacent, positive imaginary part first) of the
// n x n matrix a.  Returns 0, or 1 when the QR iteration ran out of its budget.
TNR_HD inline int real_eigvals(double* a, int n, double* wr, double* wi, double* work) {
#define TNR_H(i, j) a[(i) + (long long)(j) * n]
    if (n <= 0) return 0;
    hessenberg_reduce(a, n, work);
    const double eps = 2.220446049250313e-16;
    double anorm = 0.0;
    for (int j = 0; j < n; ++j)
        for (int i = 0; i <= (j + 1 < n ? j + 1 : n - 1); ++i) anorm += fabs(TNR_H(i, j));
    int hi = n - 1, iter = 0, total = 0;
    const int budget = 60 * n + 60;
    while (hi >= 0) {
        int l = hi;
        for (; l > 0; --l) {                     // the lowest negligible subdiagonal entry splits
            double s = fabs(TNR_H(l - 1, l - 1)) + fabs(TNR_H(l, l));
            if (s == 0.0) s = anorm;
            if (fabs(TNR_H(l, l - 1)) <= eps * s) {
                TNR_H(l, l - 1) = 0.0;
                break;
            }
        }
        if (l == hi) {                           // a 1 x 1 block
            wr[hi] = TNR_H(hi, hi);
            wi[hi] = 0.0;
            --hi;
            iter = 0;
            continue;
        }
        if (l == hi - 1) {                       // a 2 x 2 block
            const double p = 0.5 * (TNR_H(hi - 1, hi - 1) - TNR_H(hi, hi));
            const double bc = TNR_H(hi - 1, hi) * TNR_H(hi, hi - 1), d = TNR_H(hi, hi);
            const double disc = p * p + bc;
            if (disc >= 0.0) {
                const double z = p + copysign(sqrt(disc), p);
                wr[hi - 1] = d + z;
                wr[hi] = z != 0.0 ? d - bc / z : d;
                wi[hi - 1] = wi[hi] = 0.0;
            } else {
                wr[hi - 1] = wr[hi] = d + p;
                wi[hi - 1] = sqrt(-disc);
                wi[hi] = -wi[hi - 1];
            }
            hi -= 2;
            iter = 0;
            continue;
        }
        if (++total > budget) return 1;
        ++iter;
        // shifts: the trailing 2 x 2 block's trace and determinant; every tenth step of a
        // window an exceptional pair from the last subdiagonal entries breaks cycles
        double s, t;
        if (iter % 10 == 0) {
            const double w = fabs(TNR_H(hi, hi - 1)) + fabs(TNR_H(hi - 1, hi - 2));
            s = 1.5 * w;
            t = w * w;
        } else {
            s = TNR_H(hi - 1, hi - 1) + TNR_H(hi, hi);
            t = TNR_H(hi - 1, hi - 1) * TNR_H(hi, hi) - TNR_H(hi - 1, hi) * TNR_H(hi, hi - 1);
        }
        // first column of (H - s1 I)(H - s2 I), then chase the bulge down the window [l, hi]
        double x = TNR_H(l, l) * TNR_H(l, l) + TNR_H(l, l + 1) * TNR_H(l + 1, l) - s * TNR_H(l, l) + t;
        double y = TNR_H(l + 1, l) * (TNR_H(l, l) + TNR_H(l + 1, l + 1) - s);
        double z = TNR_H(l + 1, l) * TNR_H(l + 2, l + 1);
        for (int k = l; k <= hi - 2; ++k) {
            double v1, v2, beta;
            house_small(x, y, z, 3, &v1, &v2, &beta);
            if (beta != 0.0) {
                const int q = k > l ? k - 1 : l;
                for (int j = q; j <= hi; ++j) {
                    const double p = beta * (TNR_H(k, j) + v1 * TNR_H(k + 1, j) + v2 * TNR_H(k + 2, j));
                    TNR_H(k, j) -= p;
                    TNR_H(k + 1, j) -= p * v1;
                    TNR_H(k + 2, j) -= p * v2;
                }
                const int r = k + 3 < hi ? k + 3 : hi;
                for (int i = l; i <= r; ++i) {
                    const double p = beta * (TNR_H(i, k) + v1 * TNR_H(i, k + 1) + v2 * TNR_H(i, k + 2));
                    TNR_H(i, k) -= p;
                    TNR_H(i, k + 1) -= p * v1;
                    TNR_H(i, k + 2) -= p * v2;
                }
            }
            x = TNR_H(k + 1, k);
            y = TNR_H(k + 2, k);
            if (k < hi - 2) z = TNR_H(k + 3, k);
        }
        {
            const int k = hi - 1;
            double v1, v2, beta;
            house_small(x, y, 0.0, 2, &v1, &v2, &beta);
            if (beta != 0.0) {
                for (int j = k - 1; j <= hi; ++j) {
                    const double p = beta * (TNR_H(k, j) + v1 * TNR_H(k + 1, j));
                    TNR_H(k, j) -= p;
                    TNR_H(k + 1, j) -= p * v1;
                }
                for (int i = l; i <= hi; ++i) {
                    const double p = beta * (TNR_H(i, k) + v1 * TNR_H(i, k + 1));
                    TNR_H(i, k) -= p;
                    TNR_H(i, k + 1) -= p * v1;
                }
            }
        }
    }
    return 0;
#undef TNR_H
}

}  // namespace tnr
