// Oracle test infrastructure (C++ restatement of the reference's collision path).
//
// Symmetric 3x3 eigendecomposition restated from the published EISPACK/JAMA
// procedures that the reference vendors as eig3 (eig3/eig3.cpp:21-134 tred2,
// :138-254 tql2, :256-265 entry): Householder reduction to tridiagonal form,
// then the implicit-shift QL iteration, then an ascending selection sort of the
// eigenvalues with their eigenvector columns. The arithmetic is carried out in
// the same order as those procedures, so that with IEEE double and no
// contraction the results are bit-identical; that sameness is required for the
// OBB axes (and hence the tree) to match the reference builder.
//
// Storage: a[r][c] row-major. On return the eigenvectors are the columns of v,
// eigenvalues ascending in d.
#pragma once

#include <cmath>

namespace port {

namespace eig_detail {

inline double hyp(double x, double y) { return std::sqrt(x * x + y * y); }

// Householder tridiagonalisation (eig3.cpp:21-134). On entry v holds the
// matrix; on exit v holds the accumulated orthogonal transform, d the
// diagonal and off[1..2] the sub-diagonal.
inline void householder(double v[3][3], double d[3], double off[3]) {
    const int N = 3;
    for (int c = 0; c < N; ++c) d[c] = v[N - 1][c];

    for (int i = N - 1; i >= 1; --i) {
        double sc = 0.0;
        double h = 0.0;
        for (int k = 0; k < i; ++k) sc = sc + std::fabs(d[k]);

        if (sc == 0.0) {
            off[i] = d[i - 1];
            for (int c = 0; c < i; ++c) {
                d[c] = v[i - 1][c];
                v[i][c] = 0.0;
                v[c][i] = 0.0;
            }
        } else {
            for (int k = 0; k < i; ++k) {
                d[k] = d[k] / sc;
                h = h + d[k] * d[k];
            }
            double f = d[i - 1];
            double g = std::sqrt(h);
            if (f > 0) g = -g;
            off[i] = sc * g;
            h = h - f * g;
            d[i - 1] = f - g;
            for (int c = 0; c < i; ++c) off[c] = 0.0;

            for (int c = 0; c < i; ++c) {
                f = d[c];
                v[c][i] = f;
                g = off[c] + v[c][c] * f;
                for (int k = c + 1; k <= i - 1; ++k) {
                    g = g + v[k][c] * d[k];
                    off[k] = off[k] + v[k][c] * f;
                }
                off[c] = g;
            }
            f = 0.0;
            for (int c = 0; c < i; ++c) {
                off[c] = off[c] / h;
                f = f + off[c] * d[c];
            }
            const double hh = f / (h + h);
            for (int c = 0; c < i; ++c) off[c] = off[c] - hh * d[c];
            for (int c = 0; c < i; ++c) {
                f = d[c];
                g = off[c];
                for (int k = c; k <= i - 1; ++k) v[k][c] = v[k][c] - (f * off[k] + g * d[k]);
                d[c] = v[i - 1][c];
                v[i][c] = 0.0;
            }
        }
        d[i] = h;
    }

    // Accumulate the transformations.
    for (int i = 0; i < N - 1; ++i) {
        v[N - 1][i] = v[i][i];
        v[i][i] = 1.0;
        const double h = d[i + 1];
        if (h != 0.0) {
            for (int k = 0; k <= i; ++k) d[k] = v[k][i + 1] / h;
            for (int c = 0; c <= i; ++c) {
                double g = 0.0;
                for (int k = 0; k <= i; ++k) g = g + v[k][i + 1] * v[k][c];
                for (int k = 0; k <= i; ++k) v[k][c] = v[k][c] - g * d[k];
            }
        }
        for (int k = 0; k <= i; ++k) v[k][i + 1] = 0.0;
    }
    for (int c = 0; c < N; ++c) {
        d[c] = v[N - 1][c];
        v[N - 1][c] = 0.0;
    }
    v[N - 1][N - 1] = 1.0;
    off[0] = 0.0;
}

// Implicit-shift QL on the tridiagonal form, then ascending sort
// (eig3.cpp:138-254). The reference iterates without a cap; this restatement
// stops after 10,000 sweeps of one eigenvalue, which only a non-finite input
// could reach.
inline void ql_implicit(double v[3][3], double d[3], double off[3]) {
    const int N = 3;
    for (int i = 1; i < N; ++i) off[i - 1] = off[i];
    off[N - 1] = 0.0;

    double f = 0.0;
    double tst1 = 0.0;
    const double eps = std::ldexp(1.0, -52);
    for (int l = 0; l < N; ++l) {
        const double t = std::fabs(d[l]) + std::fabs(off[l]);
        tst1 = (tst1 > t) ? tst1 : t;
        int m = l;
        while (m < N) {
            if (std::fabs(off[m]) <= eps * tst1) break;
            ++m;
        }
        if (m > l) {
            int sweeps = 0;
            do {
                ++sweeps;
                double g = d[l];
                double p = (d[l + 1] - g) / (2.0 * off[l]);
                double r = hyp(p, 1.0);
                if (p < 0) r = -r;
                d[l] = off[l] / (p + r);
                d[l + 1] = off[l] * (p + r);
                const double dl1 = d[l + 1];
                double h = g - d[l];
                for (int i = l + 2; i < N; ++i) d[i] = d[i] - h;
                f = f + h;

                p = d[m];
                double c = 1.0, c2 = c, c3 = c;
                const double el1 = off[l + 1];
                double s = 0.0, s2 = 0.0;
                for (int i = m - 1; i >= l; --i) {
                    c3 = c2;
                    c2 = c;
                    s2 = s;
                    g = c * off[i];
                    h = c * p;
                    r = hyp(p, off[i]);
                    off[i + 1] = s * r;
                    s = off[i] / r;
                    c = p / r;
                    p = c * d[i] - s * g;
                    d[i + 1] = h + s * (c * g + s * d[i]);
                    for (int k = 0; k < N; ++k) {
                        h = v[k][i + 1];
                        v[k][i + 1] = s * v[k][i] + c * h;
                        v[k][i] = c * v[k][i] - s * h;
                    }
                }
                p = -s * s2 * c3 * el1 * off[l] / dl1;
                off[l] = s * p;
                d[l] = c * p;
            } while (std::fabs(off[l]) > eps * tst1 && sweeps < 10000);
        }
        d[l] = d[l] + f;
        off[l] = 0.0;
    }

    for (int i = 0; i < N - 1; ++i) {
        int k = i;
        double p = d[i];
        for (int j = i + 1; j < N; ++j)
            if (d[j] < p) {
                k = j;
                p = d[j];
            }
        if (k != i) {
            d[k] = d[i];
            d[i] = p;
            for (int r = 0; r < N; ++r) {
                const double tmp = v[r][i];
                v[r][i] = v[r][k];
                v[r][k] = tmp;
            }
        }
    }
}

}  // namespace eig_detail

// eig3/eig3.cpp:256-265.
inline void eigen_sym3(const double a[3][3], double v[3][3], double d[3]) {
    double off[3];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) v[r][c] = a[r][c];
    eig_detail::householder(v, d, off);
    eig_detail::ql_implicit(v, d, off);
}

}  // namespace port
