/*
 * ref_driver.cpp -- test infrastructure only (oracle).
 *
 * Serial CPU driver for the reference's own kernels (mepgl/src/nlcg.cu and
 * mepgl/src/interpolation.cu, host-compiled through ref_shim.h by
 * ref_build.py).  Every "launch" below loops over the grid the reference uses
 * and calls the kernel body per thread.  The host-side call sequences of the
 * reference (nlcgSteps, loop, arcLength, redistributeLinear/Cubic) are
 * restated here; the kernels themselves are the reference's.
 *
 * Deviations, each forced by running on a CPU:
 *  - per-image sums (parallel_sum::sumArrayF / sumArrayF4,
 *    mepgl/src/parallel_sum.cu:49-67) are accumulated in long double and
 *    rounded once to `real`, instead of the reference's two-level tree;
 *  - cuSPARSE gtsv2 (interpolation.cu:443-454) is replaced by the LAPACK
 *    gtsv algorithm of tridiag.h;
 *  - buildHMatrix (interpolation.cu:252-290) has a __syncthreads() phase
 *    split, emulated by running the kernel twice (it is idempotent);
 *  - generateNewFramesCubic may read h[F] when the running sum of h rounds
 *    below 1 (interpolation.cu:380-386); the emulation pads h with +inf
 *    there, i.e. the walk stops at the last segment.
 *
 * All arrays use the reference device layout: site (i, j) of image n at
 * i + N*j + N*N*n, complex / vector fields as interleaved (x, y) pairs.
 */
#include <cstdint>
#include <vector>
#include <utility>

#include "config.cuh"

thread_local dim3 threadIdx;
thread_local dim3 blockIdx;
thread_local dim3 blockDim;
thread_local dim3 gridDim;

namespace rn {
#include "nlcg_kernels.inc"
}
namespace ri {
#include "interp_kernels.inc"
}

#include "tridiag.h"
MEPGL_DEFINE_GTTRF(ref_gttrf, real)
MEPGL_DEFINE_GTTRS(ref_gttrs, real)

namespace {

template <class K>
void launch(dim3 g, dim3 b, K &&k)
{
    gridDim = g;
    blockDim = b;
    for (unsigned bz = 0; bz < g.z; ++bz)
        for (unsigned by = 0; by < g.y; ++by)
            for (unsigned bx = 0; bx < g.x; ++bx)
                for (unsigned tz = 0; tz < b.z; ++tz)
                    for (unsigned ty = 0; ty < b.y; ++ty)
                        for (unsigned tx = 0; tx < b.x; ++tx) {
                            blockIdx = {bx, by, bz};
                            threadIdx = {tx, ty, tz};
                            k();
                        }
}

/* One CUDA thread per site and image: grid (N*N, F), block 1. */
inline dim3 site_grid(int F) { return dim3{(unsigned)(N * N), (unsigned)F, 1}; }
inline dim3 one() { return dim3{1, 1, 1}; }

void sum_images(const real *density, real *out, int F)
{
    for (int n = 0; n < F; ++n) {
        long double acc = 0;
        for (int i = 0; i < N * N; ++i) acc += density[(size_t)n * N * N + i];
        out[n] = (real)acc;
    }
}

void sum_images4(const real4 *density, real4 *out, int F)
{
    for (int n = 0; n < F; ++n) {
        long double x = 0, y = 0, z = 0, w = 0;
        for (int i = 0; i < N * N; ++i) {
            const real4 &v = density[(size_t)n * N * N + i];
            x += v.x; y += v.y; z += v.z; w += v.w;
        }
        out[n] = real4{(real)x, (real)y, (real)z, (real)w};
    }
}

} // namespace

extern "C" {

/* Layout of the parameter block passed from Python (ctypes). */
struct RefParams {
    int *comp_nn, *sc_nn;
    real *a_1, *b_1, *m_xx_1, *m_yy_1, *a_2, *b_2, *m_xx_2, *m_yy_2, *h;
    real *q_1, *q_2, *eta, *gamma, *delta;
};

int ref_N() { return N; }
double ref_dx() { return (double)dx; }
int ref_real_size() { return (int)sizeof(real); }
int ref_components()
{
#ifdef MULTICOMPONENT
    return 2;
#else
    return 1;
#endif
}
int ref_thin_film()
{
#ifdef NO_SELF_FIELD
    return 1;
#else
    return 0;
#endif
}

/* buildNearestNeighbourMap (nlcg.cu:48-103), launched as in mepgl.cu:598-599. */
void ref_nn_map(int *domain, int *nn)
{
    launch(dim3{(unsigned)(N * N), 1, 1}, one(), [&] { rn::buildNearestNeighbourMap(domain, nn); });
}

#define PARAM_ARGS P->comp_nn, P->sc_nn, P->a_1, P->b_1, P->m_xx_1, P->m_yy_1, \
    P->a_2, P->b_2, P->m_xx_2, P->m_yy_2, P->h, P->q_1, P->q_2, P->eta, P->gamma, P->delta

/* computeFreeEnergy (nlcg.cu:217-240), with the density buffer zeroed first
 * (the reference accumulates into an uninitialised cudaMalloc buffer). */
void ref_free_energy(int F, RefParams *P, real2 *a, real2 *psi_1, real2 *psi_2, real *fenergy,
                     real *density_out)
{
    std::vector<real> dens((size_t)F * N * N, (real)0);
    launch(site_grid(F), one(), [&] {
        rn::freeEnergyDensity(PARAM_ARGS, a, psi_1, psi_2, dens.data());
    });
    sum_images(dens.data(), fenergy, F);
    if (density_out)
        for (size_t i = 0; i < dens.size(); ++i) density_out[i] = dens[i];
}

/* The gradient launches of nlcgSteps (nlcg.cu:1521-1537). */
void ref_gradient(int F, RefParams *P, real2 *a, real2 *psi_1, real2 *psi_2, real2 *a_g,
                  real2 *psi_1_g, real2 *psi_2_g, int maxwell)
{
    if (!maxwell)
        launch(site_grid(F), one(), [&] {
            rn::gradientPsi(PARAM_ARGS, a, psi_1, psi_2, a_g, psi_1_g, psi_2_g);
        });
#ifndef NO_SELF_FIELD
    launch(site_grid(F), one(), [&] {
        rn::gradientA(PARAM_ARGS, a, psi_1, psi_2, a_g, psi_1_g, psi_2_g);
    });
#endif
}

/* polynomialExpansion + the two sums (nlcg.cu:1559-1569). */
void ref_polynomial(int F, RefParams *P, real2 *a, real2 *psi_1, real2 *psi_2, real2 *a_d,
                    real2 *psi_1_d, real2 *psi_2_d, real *fenergy, real4 *poly)
{
    std::vector<real> fd((size_t)F * N * N);
    std::vector<real4> pd((size_t)F * N * N);
    launch(site_grid(F), one(), [&] {
        rn::polynomialExpansion(PARAM_ARGS, a, psi_1, psi_2, a_d, psi_1_d, psi_2_d, fd.data(), pd.data());
    });
    sum_images(fd.data(), fenergy, F);
    sum_images4(pd.data(), poly, F);
}

/* gradientDensity + sums (nlcg.cu:1543-1549). */
void ref_gradient_norms(int F, real2 *a_g, real2 *psi_1_g, real2 *psi_2_g, real2 *a_g_old,
                        real2 *psi_1_g_old, real2 *psi_2_g_old, real *g_norm2, real *g_delta_g)
{
    std::vector<real> n2((size_t)F * N * N), dg((size_t)F * N * N);
    launch(site_grid(F), one(), [&] {
        rn::gradientDensity(a_g, psi_1_g, psi_2_g, a_g_old, psi_1_g_old, psi_2_g_old, n2.data(), dg.data());
    });
    sum_images(n2.data(), g_norm2, F);
    sum_images(dg.data(), g_delta_g, F);
}

/* computeStepDirection (nlcg.cu:955-994). */
void ref_step_direction(int F, real2 *a, real2 *psi_1, real2 *psi_2, real2 *a_g, real2 *psi_1_g,
                        real2 *psi_2_g, real2 *a_d, real2 *psi_1_d, real2 *psi_2_d, real *g_norm2,
                        real *g_norm2_old, real *g_delta_g, int nlcg)
{
    launch(site_grid(F), one(), [&] {
        rn::computeStepDirection(a, psi_1, psi_2, a_g, psi_1_g, psi_2_g, a_d, psi_1_d, psi_2_d, g_norm2,
                                 g_norm2_old, g_delta_g, nlcg != 0);
    });
}

/* lineSearch (nlcg.cu:1398-1445), one thread per image. */
void ref_line_search(int F, real *fenergy, real4 *poly, real *alpha)
{
    launch(dim3{1, (unsigned)F, 1}, one(), [&] { rn::lineSearch(fenergy, poly, alpha); });
}

/* updateFields (nlcg.cu:1372-1396). */
void ref_update(int F, real2 *a, real2 *psi_1, real2 *psi_2, real2 *a_d, real2 *psi_1_d, real2 *psi_2_d,
                real *alpha)
{
    launch(site_grid(F), one(), [&] { rn::updateFields(a, psi_1, psi_2, a_d, psi_1_d, psi_2_d, alpha); });
}

/* computeJB (nlcg.cu:366-380). */
void ref_jb(int F, RefParams *P, real2 *a, real2 *psi_1, real2 *psi_2, real *b, real2 *j_1, real2 *j_2)
{
    launch(site_grid(F), one(), [&] {
        rn::computeJBKernel(P->comp_nn, P->sc_nn, P->a_1, P->b_1, P->m_xx_1, P->m_yy_1, P->a_2, P->b_2,
                            P->m_xx_2, P->m_yy_2, P->h, P->q_1, P->q_2, a, psi_1, psi_2, b, j_1, j_2);
    });
}

/* arcLength (interpolation.cu:143-155). */
void ref_arc_length(int F, real2 *a, real2 *psi_1, real2 *psi_2, real *s)
{
    for (int n = 0; n < F; ++n) s[n] = 0;
    launch(dim3{(unsigned)N, (unsigned)F, 1}, dim3{(unsigned)N, 1, 1},
           [&] { ri::arcLengthParametrization(N, F, a, psi_1, psi_2, s); });
    launch(one(), one(), [&] { ri::computeArcLength(F, s); });
}

/* arcLengthJB (interpolation.cu:157-169). */
void ref_arc_length_jb(int F, real *b, real2 *j_1, real2 *j_2, real *s)
{
    for (int n = 0; n < F; ++n) s[n] = 0;
    launch(dim3{(unsigned)N, (unsigned)F, 1}, dim3{(unsigned)N, 1, 1},
           [&] { ri::arcLengthParametrizationJB(N, F, b, j_1, j_2, s); });
    launch(one(), one(), [&] { ri::computeArcLength(F, s); });
}

/* generateNewFramesLinear for one field (interpolation.cu:190-227, 229-250). */
void ref_redistribute_linear(int F, real *s, real2 *f, int F_new, real2 *f_new)
{
    launch(dim3{(unsigned)(N * N), 1, 1}, one(),
           [&] { ri::generateNewFramesLinear(N, F, s, f, (real)F_new, f_new); });
}

/* redistributeCubic for one field (interpolation.cu:404-481). */
void ref_redistribute_cubic(int F, real *s, real2 *f, int F_new, real2 *f_new)
{
    std::vector<real> h(F + 8, (real)INFINITY), dl(F), d(F), du(F);
    for (int pass = 0; pass < 2; ++pass)
        launch(one(), dim3{(unsigned)F, 1, 1}, [&] { ri::buildHMatrix(F, s, h.data(), dl.data(), d.data(), du.data()); });
    std::vector<real> dx_((size_t)F * N * N), dy_((size_t)F * N * N);
    launch(dim3{(unsigned)(N * N), 1, 1}, one(), [&] {
        ri::computeDeltaX(F, N, dx_.data(), h.data(), f);
        ri::computeDeltaY(F, N, dy_.data(), h.data(), f);
    });
    std::vector<real> fl(dl), fd(d), fu(du), fu2(F);
    std::vector<int> piv(F);
    ref_gttrf(F, fl.data(), fd.data(), fu.data(), fu2.data(), piv.data());
    for (size_t site = 0; site < (size_t)N * N; ++site) {
        ref_gttrs(F, fl.data(), fd.data(), fu.data(), fu2.data(), piv.data(), dx_.data() + site * F, 1);
        ref_gttrs(F, fl.data(), fd.data(), fu.data(), fu2.data(), piv.data(), dy_.data() + site * F, 1);
    }
    launch(dim3{(unsigned)(N * N), 1, 1}, one(), [&] {
        ri::generateNewFramesCubic(N, F, h.data(), dx_.data(), dy_.data(), f, (real)F_new, f_new);
    });
}

/*
 * Emulation of one run of the reference binary's loop() (mepgl.cu:38-391)
 * with the nlcgSteps host sequence (nlcg.cu:1462-1586).  The state arrays a,
 * psi_1, psi_2 are updated in place.  fenergy/alpha/g_norm2 receive the
 * values loop() holds at the end (g_norm2 is loop()'s own buffer, i.e. the
 * slot nlcgSteps writes on even substeps).  fenergy_hist, if not null,
 * receives fenergy after every outer iteration ([iterations][F]).
 */
void ref_loop(int F, RefParams *P, real2 *a, real2 *psi_1, real2 *psi_2, char mode, int iterations,
              int relaxation_steps, int nlcg, real *fenergy, real *alpha_out, real *g_norm2_out,
              real *s_out, real *s_jb_out, real *fenergy_hist)
{
    const size_t M = (size_t)F * N * N;
    std::vector<real2> g[2][3], d[3], xn[3];
    for (int k = 0; k < 2; ++k)
        for (int c = 0; c < 3; ++c) g[k][c].assign(M, real2{0, 0});
    for (int c = 0; c < 3; ++c) { d[c].assign(M, real2{0, 0}); xn[c].assign(M, real2{0, 0}); }
    std::vector<real> S[2];
    S[0].assign(F, (real)INFINITY);
    S[1].assign(F, (real)INFINITY);
    std::vector<real> gdg(F), fe(F), alpha(F, 0), s(F, 0), s_jb(F, 0), bb(M);
    std::vector<real4> poly(F);
    std::vector<real2> j1(M), j2(M);
    std::vector<real2> own[3];
    for (int c = 0; c < 3; ++c) own[c].assign(M, real2{0, 0});
    real2 *x[3] = {own[0].data(), own[1].data(), own[2].data()};
    std::copy(a, a + M, own[0].begin());
    std::copy(psi_1, psi_1 + M, own[1].begin());
    std::copy(psi_2, psi_2 + M, own[2].begin());

    auto nlcg_steps = [&](int iters, bool maxwell) {
        /* nlcgSteps receives the gradient buffers and the two norm buffers by
         * value and swaps its local copies once per substep. */
        int gi = 0, go = 1;    /* loop()'s dev_*_g and dev_*_g_old */
        int si = 0, so = 1;    /* loop()'s g_norm2 and g_norm2_old */
        for (int k = 0; k < iters; ++k) {
            std::swap(si, so);
            std::swap(gi, go);
            for (int n = 0; n < F; ++n) { S[si][n] = 0; gdg[n] = 0; fe[n] = 0; poly[n] = real4{0, 0, 0, 0}; }
            ref_gradient(F, P, x[0], x[1], x[2], g[gi][0].data(), g[gi][1].data(), g[gi][2].data(), maxwell);
            ref_gradient_norms(F, g[gi][0].data(), g[gi][1].data(), g[gi][2].data(), g[go][0].data(),
                               g[go][1].data(), g[go][2].data(), S[si].data(), gdg.data());
            ref_step_direction(F, x[0], x[1], x[2], g[gi][0].data(), g[gi][1].data(), g[gi][2].data(),
                               d[0].data(), d[1].data(), d[2].data(), S[si].data(), S[so].data(), gdg.data(),
                               nlcg);
            ref_polynomial(F, P, x[0], x[1], x[2], d[0].data(), d[1].data(), d[2].data(), fe.data(),
                           poly.data());
            ref_line_search(F, fe.data(), poly.data(), alpha.data());
            ref_update(F, x[0], x[1], x[2], d[0].data(), d[1].data(), d[2].data(), alpha.data());
        }
    };

    auto reparametrize = [&](bool cubic) {
        ref_arc_length(F, x[0], x[1], x[2], s.data());
        ref_jb(F, P, x[0], x[1], x[2], bb.data(), j1.data(), j2.data());
        ref_arc_length_jb(F, bb.data(), j1.data(), j2.data(), s_jb.data());
        for (int c = 0; c < ref_components() + 1; ++c) {
            if (cubic)
                ref_redistribute_cubic(F, s_jb.data(), x[c], F, xn[c].data());
            else
                ref_redistribute_linear(F, s_jb.data(), x[c], F, xn[c].data());
        }
        /* pointer swap of mepgl.cu:215-228: the new frames become the state */
        for (int c = 0; c < ref_components() + 1; ++c) {
            own[c].swap(xn[c]);
            x[c] = own[c].data();
        }
        for (int n = 1; n < F - 1; ++n) { S[0][n] = (real)INFINITY; S[1][n] = (real)INFINITY; }
    };

    for (int it = 0; it < iterations; ++it) {
        if (mode == 'S') nlcg_steps(relaxation_steps, false);
        else if (mode == 'M') nlcg_steps(relaxation_steps, true);
        else if (mode == 'L' || mode == 'C') {
            reparametrize(mode == 'C');
            nlcg_steps(relaxation_steps, false);
        }
        if (fenergy_hist)
            for (int n = 0; n < F; ++n) fenergy_hist[(size_t)it * F + n] = fe[n];
    }
    std::copy(x[0], x[0] + M, a);
    std::copy(x[1], x[1] + M, psi_1);
    std::copy(x[2], x[2] + M, psi_2);
    for (int n = 0; n < F; ++n) {
        if (fenergy) fenergy[n] = fe[n];
        if (alpha_out) alpha_out[n] = alpha[n];
        if (g_norm2_out) g_norm2_out[n] = S[0][n];
        if (s_out) s_out[n] = s[n];
        if (s_jb_out) s_jb_out[n] = s_jb[n];
    }
}

} /* extern "C" */
