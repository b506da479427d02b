/*
 * tridiag.h -- test infrastructure only (oracle).
 *
 * Tridiagonal solve by Gaussian elimination with partial pivoting, the
 * published LAPACK ?gtsv algorithm (Anderson et al., LAPACK Users' Guide,
 * routine DGTSV): at each column k the larger of |d[k]| and |dl[k]| is taken
 * as pivot, rows k and k+1 are swapped when the sub-diagonal is larger, which
 * creates one second super-diagonal entry, then back substitution.
 *
 * The reference solves its spline systems with cuSPARSE gtsv2
 * (mepgl/src/interpolation.cu:443-454), a closed library; this restatement
 * stands in for it in the oracle.  The same algorithm (factor once, apply to
 * every right-hand side) is used by the CUDA kernels, so both sides agree to
 * rounding.
 *
 * The factorisation is split from the solve so one factorisation can serve
 * many right-hand sides (every lattice site shares the same matrix).
 */
#ifndef MEPGL_ORACLE_TRIDIAG_H
#define MEPGL_ORACLE_TRIDIAG_H

#include <math.h>

/* Factor the n x n tridiagonal matrix (dl: sub, d: diag, du: super; dl[0] and
 * du[n-1] unused) in place.  On return d holds the pivots U(k,k), du holds
 * U(k,k+1), du2 holds U(k,k+2), dl holds the multipliers and ipiv[k] is 1 when
 * rows k and k+1 were swapped.  Returns 0, or k+1 if U(k,k) is exactly zero. */
#define MEPGL_DEFINE_GTTRF(NAME, T)                                              \
static int NAME(int n, T *dl, T *d, T *du, T *du2, int *ipiv)                   \
{                                                                              \
    for (int k = 0; k < n; ++k) { ipiv[k] = 0; du2[k] = 0; }                    \
    for (int k = 0; k < n - 1; ++k) {                                          \
        T sub = dl[k + 1];                                                     \
        if (fabs((double)d[k]) >= fabs((double)sub)) {                         \
            if (d[k] != 0) {                                                   \
                T l = sub / d[k];                                              \
                dl[k + 1] = l;                                                 \
                d[k + 1] = d[k + 1] - l * du[k];                               \
            } else {                                                           \
                dl[k + 1] = 0;                                                 \
            }                                                                  \
        } else {                                                               \
            T l = d[k] / sub;                                                  \
            d[k] = sub;                                                        \
            dl[k + 1] = l;                                                     \
            T t = du[k];                                                       \
            du[k] = d[k + 1];                                                  \
            d[k + 1] = t - l * d[k + 1];                                       \
            if (k < n - 2) {                                                   \
                du2[k] = du[k + 1];                                            \
                du[k + 1] = -l * du[k + 1];                                    \
            }                                                                  \
            ipiv[k] = 1;                                                       \
        }                                                                      \
    }                                                                          \
    for (int k = 0; k < n; ++k) if (d[k] == 0) return k + 1;                   \
    return 0;                                                                  \
}

/* Solve with the factors of NAME_gttrf for one right-hand side b (length n,
 * element k at b[k*stride]); b is overwritten by the solution. */
#define MEPGL_DEFINE_GTTRS(NAME, T)                                              \
static void NAME(int n, const T *dl, const T *d, const T *du, const T *du2,     \
                 const int *ipiv, T *b, long stride)                            \
{                                                                              \
    for (int k = 0; k < n - 1; ++k) {                                          \
        T bk = b[k * stride], bk1 = b[(k + 1) * stride];                       \
        if (ipiv[k]) {                                                         \
            b[k * stride] = bk1;                                               \
            b[(k + 1) * stride] = bk - dl[k + 1] * bk1;                        \
        } else {                                                               \
            b[(k + 1) * stride] = bk1 - dl[k + 1] * bk;                        \
        }                                                                      \
    }                                                                          \
    b[(n - 1) * stride] = b[(n - 1) * stride] / d[n - 1];                      \
    if (n > 1)                                                                 \
        b[(n - 2) * stride] = (b[(n - 2) * stride]                             \
                               - du[n - 2] * b[(n - 1) * stride]) / d[n - 2];  \
    for (int k = n - 3; k >= 0; --k)                                           \
        b[k * stride] = (b[k * stride] - du[k] * b[(k + 1) * stride]           \
                         - du2[k] * b[(k + 2) * stride]) / d[k];               \
}

#endif
