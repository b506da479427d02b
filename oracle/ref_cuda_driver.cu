// ref_cuda_driver.cu -- times the reference's own CUDA NLCG (a timing baseline only).
//
// Links against the reference's unmodified nlcg.cu and parallel_sum.cu,
// compiled for this GPU by oracle/ref_cuda_build.py with a generated
// config.cuh / real.cuh (the reference fixes N, dx, the component count and
// the precision at compile time).  It replaces the reference's main()
// (mepgl/src/mepgl.cu:394-791), which needs Boost.program_options and the
// .npy loader, by a plain reader of one binary input file:
//
//   int32 F, int32 N, then N*N int32 comp_domain, N*N int32 sc_domain,
//   9 arrays of N*N reals (a_1 b_1 m_xx_1 m_yy_1 a_2 b_2 m_xx_2 m_yy_2 h),
//   5 reals (q_1 q_2 eta gamma delta), then F*N*N real2 each of a, psi_1, psi_2
//
// (reals of the build's precision, the reference's device layout).  It
// allocates and initialises the NLCG state as the reference's loop() does
// (mepgl/src/mepgl.cu:48-146), runs nlcgSteps(warmup, ...) and then, timed
// with CUDA events, nlcgSteps(steps, ...) -- the reference's host loop with
// its own synchronisations, as loop() calls it once per outer iteration
// (mepgl/src/mepgl.cu:156-172) -- and prints one JSON
// line with the time per step and the per-image energies of the last step,
// so that the reference build's results can be compared with this
// library's on the same input.
//
//   ref_nlcg INPUT STEPS WARMUP [maxwell]
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "config.cuh"
#include "nlcg.cuh"
#include "real.cuh"

#define CK(x)                                                                                       \
    do {                                                                                            \
        cudaError_t e_ = (x);                                                                       \
        if (e_ != cudaSuccess) {                                                                    \
            std::fprintf(stderr, "%s: %s\n", #x, cudaGetErrorString(e_));                          \
            std::exit(2);                                                                           \
        }                                                                                           \
    } while (0)

template <class T>
static T *dev_copy(const std::vector<T> &h)
{
    T *d = nullptr;
    CK(cudaMalloc(&d, h.size() * sizeof(T)));
    CK(cudaMemcpy(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
    return d;
}

template <class T>
static T *dev_zero(size_t n)
{
    T *d = nullptr;
    CK(cudaMalloc(&d, n * sizeof(T)));
    CK(cudaMemset(d, 0, n * sizeof(T)));
    return d;
}

template <class T>
static void read_into(FILE *f, std::vector<T> &v, size_t n)
{
    v.resize(n);
    if (std::fread(v.data(), sizeof(T), n, f) != n) {
        std::fprintf(stderr, "short input file\n");
        std::exit(3);
    }
}

int main(int argc, char **argv)
{
    if (argc < 4) {
        std::fprintf(stderr, "usage: %s INPUT STEPS WARMUP [maxwell]\n", argv[0]);
        return 1;
    }
    const int steps = std::atoi(argv[2]), warmup = std::atoi(argv[3]);
    const bool maxwell = argc > 4 && std::atoi(argv[4]) != 0;
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) {
        std::fprintf(stderr, "cannot open %s\n", argv[1]);
        return 3;
    }
    int32_t hdr[2];
    if (std::fread(hdr, sizeof(int32_t), 2, f) != 2) return 3;
    const int F = hdr[0];
    if (hdr[1] != N) {
        std::fprintf(stderr, "input lattice %d does not match the build's N = %d\n", hdr[1], N);
        return 3;
    }
    const size_t M = (size_t)N * N;
    std::vector<int> comp, sc;
    read_into(f, comp, M);
    read_into(f, sc, M);
    std::vector<real> par[9], q;
    for (auto &p : par) read_into(f, p, M);
    read_into(f, q, 5);
    std::vector<real2> a, p1, p2;
    read_into(f, a, F * M);
    read_into(f, p1, F * M);
    read_into(f, p2, F * M);
    std::fclose(f);
    CK(cudaSetDevice(devNumber));

    int *dev_comp = dev_copy(comp), *dev_sc = dev_copy(sc);
    int *dev_comp_nn = dev_zero<int>(M), *dev_sc_nn = dev_zero<int>(M);
    buildNearestNeighbourMap<<<gridSizeX, 1024>>>(dev_comp, dev_comp_nn);
    buildNearestNeighbourMap<<<gridSizeX, 1024>>>(dev_sc, dev_sc_nn);
    CK(cudaDeviceSynchronize());
    real *dp[9];
    for (int k = 0; k < 9; ++k) dp[k] = dev_copy(par[k]);
    real *dq[5];
    for (int k = 0; k < 5; ++k) dq[k] = dev_copy(std::vector<real>{q[k]});
    real2 *x[3] = {dev_copy(a), dev_copy(p1), dev_copy(p2)};
    real2 *g[3], *g_old[3], *d[3];
    for (int k = 0; k < 3; ++k) {
        g[k] = dev_zero<real2>(F * M);
        g_old[k] = dev_zero<real2>(F * M);
        d[k] = dev_zero<real2>(F * M);
    }
    real *g_norm2_density = dev_zero<real>(F * M), *g_delta_g_density = dev_zero<real>(F * M);
    real *fenergy_density = dev_zero<real>(F * M);
    real4 *poly_density = dev_zero<real4>(F * M);
    real *g_norm2, *g_norm2_old, *g_delta_g, *alpha, *fenergy;
    real4 *poly;
    CK(cudaMallocManaged(&g_norm2, F * sizeof(real)));
    CK(cudaMallocManaged(&g_norm2_old, F * sizeof(real)));
    CK(cudaMallocManaged(&g_delta_g, F * sizeof(real)));
    CK(cudaMallocManaged(&alpha, F * sizeof(real)));
    CK(cudaMallocManaged(&fenergy, F * sizeof(real)));
    CK(cudaMallocManaged(&poly, F * sizeof(real4)));
    for (int n = 0; n < F; ++n) {
        g_norm2[n] = INFINITY;
        g_norm2_old[n] = INFINITY;
    }
    auto step = [&](int iters) {
        nlcgSteps(iters, F, dev_comp_nn, dev_sc_nn, dp[0], dp[1], dp[2], dp[3], dp[4], dp[5], dp[6], dp[7], dp[8],
                  dq[0], dq[1], dq[2], dq[3], dq[4], x[0], x[1], x[2], g[0], g[1], g[2], g_old[0], g_old[1],
                  g_old[2], d[0], d[1], d[2], g_norm2_density, g_delta_g_density, g_norm2, g_norm2_old, g_delta_g,
                  alpha, fenergy_density, poly_density, fenergy, poly, true, maxwell);
    };
    if (warmup > 0) step(warmup);
    CK(cudaDeviceSynchronize());
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    CK(cudaEventRecord(e0));
    step(steps);
    CK(cudaEventRecord(e1));
    CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    // the reference checks none of its launches; a kernel that could not
    // launch (e.g. too many registers for its block size) is reported here
    const cudaError_t launch = cudaGetLastError();
    // the per-image energies nlcgSteps reports (the last line polynomial's
    // constant term: F before the last update, mepgl/src/nlcg.cu:1036,1567);
    // computeFreeEnergy is not used: it accumulates into an uninitialised
    // scratch buffer (mepgl/src/nlcg.cu:223-232)
    const real *dev_fe = fenergy;
    std::printf("{\"n\": %d, \"images\": %d, \"real_bytes\": %d, \"block\": %d, \"steps\": %d, \"warmup\": %d, "
                "\"ms_per_step\": %.6f, \"site_images_per_s\": %.6e, \"launch_error\": \"%s\", \"fenergy\": [",
                N, F, (int)sizeof(real), blockSizeX, steps, warmup, ms / steps, (double)F * M * steps / (ms / 1e3),
                launch == cudaSuccess ? "" : cudaGetErrorString(launch));
    for (int n = 0; n < F; ++n) std::printf("%s%.17g", n ? ", " : "", (double)dev_fe[n]);
    std::printf("]}\n");
    return 0;
}
