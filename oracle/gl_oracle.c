/*
 * gl_oracle.c -- CPU restatement of the mepgl hot path (TEST INFRASTRUCTURE).
 *
 * Builds libgl_oracle.so (oracle/Makefile), loaded through ctypes by
 * oracle/cref.py.  Never linked into the product library.  Compiled with
 * -ffp-contract=off so results are identical on x86-64 and AArch64.
 *
 * Exported symbols (X = d for double, f for float):
 *   glo_nn_map                      neighbour codes (nlcg.cu:48-103)
 *   glo_energy_X                    per-image free energy (nlcg.cu:105-240)
 *   glo_gradient_X                  dF/dA, dF/dpsi (nlcg.cu:504-888)
 *   glo_polynomial_X                F(x + a d) coefficients (nlcg.cu:997-1370)
 *   glo_line_search_X               step length (nlcg.cu:1398-1445)
 *   glo_jb_X                        B, J observables (nlcg.cu:243-364)
 *   glo_arc_length_X                arc length (interpolation.cu:39-140)
 *   glo_redistribute_linear_X       linear resample (interpolation.cu:190-250)
 *   glo_redistribute_cubic_X        cubic resample (interpolation.cu:252-481)
 *   glo_solver_*_X                  nlcgSteps / loop() state machine
 *                                   (nlcg.cu:1462-1586, mepgl.cu:38-391)
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "gl_oracle.h"
#include "tridiag.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

MEPGL_DEFINE_GTTRF(glo_gttrf_d, double)
MEPGL_DEFINE_GTTRS(glo_gttrs_d, double)

/* A x = b for an n x n tridiagonal matrix (dl[k] = A[k][k-1], dl[0] unused;
 * d diagonal; du[k] = A[k][k+1]) and nrhs right-hand sides stored one after
 * another in b, overwritten by the solutions: the restated LAPACK gtsv
 * algorithm of tridiag.h, exported so that tests can check it against a
 * LAPACK build.  Returns 0, or k + 1 if the pivot U(k,k) is exactly zero. */
int glo_gtsv_d(int n, const double *dl, const double *d, const double *du, double *b, int nrhs)
{
    double *w = (double *)malloc(sizeof(double) * 4 * (size_t)n);
    int *ipiv = (int *)malloc(sizeof(int) * (size_t)n);
    if (!w || !ipiv) { free(w); free(ipiv); return -1; }
    double *l = w, *dd = w + n, *u = w + 2 * n, *u2 = w + 3 * n;
    memcpy(l, dl, sizeof(double) * n);
    memcpy(dd, d, sizeof(double) * n);
    memcpy(u, du, sizeof(double) * n);
    const int info = glo_gttrf_d(n, l, dd, u, u2, ipiv);
    if (info == 0)
        for (int r = 0; r < nrhs; ++r) glo_gttrs_d(n, l, dd, u, u2, ipiv, b + (size_t)r * n, 1);
    free(w);
    free(ipiv);
    return info;
}

/* Images are independent in every per-image loop, so they run in parallel
 * when built with OpenMP; results do not depend on the thread count. */
#ifdef _OPENMP
#include <omp.h>
#define GLO_OMP_FOR _Pragma("omp parallel for schedule(dynamic)")
int glo_max_threads(void) { return omp_get_max_threads(); }
void glo_set_threads(int n) { omp_set_num_threads(n); }
#else
#define GLO_OMP_FOR
int glo_max_threads(void) { return 1; }
void glo_set_threads(int n) { (void)n; }
#endif

/* Neighbour code of every site (bit order 0:+x 1:+x+y 2:+y 3:-x+y 4:-x
 * 5:-x-y 6:-y 7:+x-y), restating buildNearestNeighbourMap
 * (mepgl/src/nlcg.cu:48-103): a bit is set when both the site and that
 * neighbour lie in the domain. */
void glo_nn_map(int nx, int ny, const int32_t *domain, uint8_t *out)
{
    static const int di[8] = {1, 1, 0, -1, -1, -1, 0, 1};
    static const int dj[8] = {0, 1, 1, 1, 0, -1, -1, -1};
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            unsigned code = 0;
            if (domain[i + nx * j] != 0)
                for (int b = 0; b < 8; ++b) {
                    const int ii = i + di[b], jj = j + dj[b];
                    if (ii < 0 || ii >= nx || jj < 0 || jj >= ny) continue;
                    if (domain[ii + nx * jj] != 0) code |= 1u << b;
                }
            out[i + nx * j] = (uint8_t)code;
        }
}

#define REAL double
#define SFX _d
#include "gl_oracle_impl.h"
#undef REAL
#undef SFX

#define REAL float
#define SFX _f
#include "gl_oracle_impl.h"
#undef REAL
#undef SFX
