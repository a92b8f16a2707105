// The eig3 eigensystem of a symmetric 3x3 (eig3/eig3.cpp:21-265), for any
// floating type: Householder reduction to tridiagonal form, implicit-shift QL,
// then the ascending selection sort of the eigenvalues with their eigenvector
// columns. Every operation is the published procedure's, in its order, so
// that in double without contraction the results are the CPU's bits (the
// tree build), and in float the refit's axes.
#pragma once

#include <cuda_runtime.h>

namespace cg {

template <typename R>
__device__ __forceinline__ R hyp(R x, R y) {
    return sqrt(x * x + y * y);
}

// Householder reduction of the symmetric 3x3 in v to tridiagonal form
// (eig3.cpp:21-134): v becomes the accumulated transform, d the diagonal,
// e[1..2] the sub-diagonal.
template <typename R>
__device__ void tridiagonalize(R v[3][3], R d[3], R e[3]) {
    for (int c = 0; c < 3; ++c) d[c] = v[2][c];
    for (int i = 2; i >= 1; --i) {
        R scale = R(0), h = R(0);
        for (int k = 0; k < i; ++k) scale = scale + fabs(d[k]);
        if (scale == R(0)) {
            e[i] = d[i - 1];
            for (int c = 0; c < i; ++c) {
                d[c] = v[i - 1][c];
                v[i][c] = R(0);
                v[c][i] = R(0);
            }
        } else {
            for (int k = 0; k < i; ++k) {
                d[k] = d[k] / scale;
                h = h + d[k] * d[k];
            }
            R f = d[i - 1];
            R g = sqrt(h);
            if (f > 0) g = -g;
            e[i] = scale * g;
            h = h - f * g;
            d[i - 1] = f - g;
            for (int c = 0; c < i; ++c) e[c] = R(0);
            for (int c = 0; c < i; ++c) {
                f = d[c];
                v[c][i] = f;
                g = e[c] + v[c][c] * f;
                for (int k = c + 1; k <= i - 1; ++k) {
                    g = g + v[k][c] * d[k];
                    e[k] = e[k] + v[k][c] * f;
                }
                e[c] = g;
            }
            f = R(0);
            for (int c = 0; c < i; ++c) {
                e[c] = e[c] / h;
                f = f + e[c] * d[c];
            }
            const R hh = f / (h + h);
            for (int c = 0; c < i; ++c) e[c] = e[c] - hh * d[c];
            for (int c = 0; c < i; ++c) {
                f = d[c];
                g = e[c];
                for (int k = c; k <= i - 1; ++k) v[k][c] = v[k][c] - (f * e[k] + g * d[k]);
                d[c] = v[i - 1][c];
                v[i][c] = R(0);
            }
        }
        d[i] = h;
    }
    for (int i = 0; i < 2; ++i) {
        v[2][i] = v[i][i];
        v[i][i] = R(1);
        const R h = d[i + 1];
        if (h != R(0)) {
            for (int k = 0; k <= i; ++k) d[k] = v[k][i + 1] / h;
            for (int c = 0; c <= i; ++c) {
                R g = R(0);
                for (int k = 0; k <= i; ++k) g = g + v[k][i + 1] * v[k][c];
                for (int k = 0; k <= i; ++k) v[k][c] = v[k][c] - g * d[k];
            }
        }
        for (int k = 0; k <= i; ++k) v[k][i + 1] = R(0);
    }
    for (int c = 0; c < 3; ++c) {
        d[c] = v[2][c];
        v[2][c] = R(0);
    }
    v[2][2] = R(1);
    e[0] = R(0);
}

// Implicit-shift QL on the tridiagonal form, then the ascending sort of the
// eigenvalues with their eigenvector columns (eig3.cpp:138-254). A sweep
// count limit stops what only a non-finite input could run forever.
template <typename R>
__device__ void ql_sort(R v[3][3], R d[3], R e[3], R eps) {
    for (int i = 1; i < 3; ++i) e[i - 1] = e[i];
    e[2] = R(0);
    R f = 0, tst1 = 0;
    for (int l = 0; l < 3; ++l) {
        const R t = fabs(d[l]) + fabs(e[l]);
        tst1 = (tst1 > t) ? tst1 : t;
        int m = l;
        while (m < 3) {
            if (fabs(e[m]) <= eps * tst1) break;
            ++m;
        }
        if (m > l) {
            int sweeps = 0;
            do {
                ++sweeps;
                R g = d[l];
                R p = (d[l + 1] - g) / (R(2) * e[l]);
                R r = hyp(p, R(1));
                if (p < 0) r = -r;
                d[l] = e[l] / (p + r);
                d[l + 1] = e[l] * (p + r);
                const R dl1 = d[l + 1];
                R h = g - d[l];
                for (int i = l + 2; i < 3; ++i) d[i] = d[i] - h;
                f = f + h;
                p = d[m];
                R c = R(1), c2 = c, c3 = c;
                const R el1 = e[l + 1];
                R s = R(0), s2 = R(0);
                for (int i = m - 1; i >= l; --i) {
                    c3 = c2;
                    c2 = c;
                    s2 = s;
                    g = c * e[i];
                    h = c * p;
                    r = hyp(p, e[i]);
                    e[i + 1] = s * r;
                    s = e[i] / r;
                    c = p / r;
                    p = c * d[i] - s * g;
                    d[i + 1] = h + s * (c * g + s * d[i]);
                    for (int k = 0; k < 3; ++k) {
                        h = v[k][i + 1];
                        v[k][i + 1] = s * v[k][i] + c * h;
                        v[k][i] = c * v[k][i] - s * h;
                    }
                }
                p = -s * s2 * c3 * el1 * e[l] / dl1;
                e[l] = s * p;
                d[l] = c * p;
            } while (fabs(e[l]) > eps * tst1 && sweeps < 10000);
        }
        d[l] = d[l] + f;
        e[l] = R(0);
    }
    for (int i = 0; i < 2; ++i) {
        int k = i;
        R p = d[i];
        for (int j = i + 1; j < 3; ++j)
            if (d[j] < p) {
                k = j;
                p = d[j];
            }
        if (k != i) {
            d[k] = d[i];
            d[i] = p;
            for (int r = 0; r < 3; ++r) {
                const R tmp = v[r][i];
                v[r][i] = v[r][k];
                v[r][k] = tmp;
            }
        }
    }
}

}  // namespace cg
