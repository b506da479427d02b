// refine.cu -- refinement of a string's images to stationary points of the
// free energy: minima, and index-1 saddles (the transition state whose energy
// above the initial minimum is the barrier, mepgl/post.py:188).
//
// The reference has no such step: its barrier is the largest image energy
// of the relaxed string, which depends on the image count and on the
// reparametrization cadence.  Here the string only seeds the refinement.
//
// Method (per image, all images of the context advanced by the same
// launches, each with its own scalars):
//
//  * Gauge step.  The reference's linearised covariant differences and
//    collocated curl views (mepgl/src/nlcg.cu:149-203) are gauge invariant
//    only to O(dx^2), so smooth gauge transformations A -> A + grad chi,
//    psi_a -> psi_a exp(i q_a chi) change the energy very little (curvature
//    ~1e-6 for chi linear in x on the 64x64 string) and move along curved
//    orbits, where a straight Newton step leaves the orbit and is rejected.
//    Each Newton iteration therefore first minimises the energy over
//    chi = sum_m c_m P_a(X) P_b(Y) (Legendre products, 1 <= a + b <= degree)
//    along the exact orbit: the m x m Hessian of E(c) comes from central
//    differences of the orbit gradient dE/dc_m = g . J phi_m, and the step is
//    applied as an exact gauge transformation.
//  * Min mode (saddles).  The lowest Hessian eigenpair (lambda_1, v_1) by
//    Lanczos with full reorthogonalisation, restarted from the previous v_1
//    (first call: the caller's direction, e.g. the string's chord tangent).
//  * Newton step.  Along v_1: p_1 = g.v_1 / |lambda_1| (uphill); in the
//    complement: (H + mu) p = -(g - (g.v_1) v_1) projected, by conjugate
//    gradients.  Minima use plain shifted CG.  Hessian-vector products are
//    central differences of the gradient kernel, H u = (g(x + h u) -
//    g(x - h u)) / 2h, with |h u| = 1e-6 sqrt(dof).
//  * Preconditioner.  The CG runs preconditioned by the inverse of a
//    constant-coefficient model of the Hessian, one per field component and
//    image: M = sigma - c_x d_xx - c_y d_yy (5-point differences, Neumann
//    boundary), with c_x, c_y and the mass sigma averaged from Hessian
//    columns probed at a comb of bulk sites, applied on the degrees of freedom
//    the energy depends on (mask from one Hessian probe).  M^-1 is exact in
//    the cosine basis: the masked field is mirrored to a 2 nx x 2 ny lattice,
//    transformed by cuFFT (loaded at run time), divided by the model's
//    eigenvalues and transformed back.  It removes the stiff kinetic part of
//    the spectrum (about 3x fewer CG iterations on the 64x64 string, 5x on the
//    256x256 two-component string).  Each solve stops at a relative residual
//    of cg_eta (0.1): linear convergence at about that rate per Newton step
//    costs fewer CG iterations than tighter, superlinear solves.
//  * Globalisation.  The step is kept when it lowers |g|^2 (for an index-1
//    saddle the modified force -g + 2 (g.v_1) v_1 is a descent direction of
//    |g|^2); then mu /= 4, else mu *= 4 (at most 1e8) and the solve is
//    repeated (Levenberg-Marquardt).
//
// Everything runs in IEEE double on the context's FP64 buffers, except the
// preconditioner's transforms (FP32: they only shape the Krylov space; the
// residuals, iterates and steps stay IEEE double).  The CG scalars live on
// the device, so its iterations run as replays of a captured CUDA graph with
// no host round trip inside.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include <dlfcn.h>

#include "context.h"

namespace mepgl {

constexpr int RF_MAX_LZ = 32;       // Lanczos vectors
constexpr int RF_MAX_DEG = 16;      // gauge polynomial degree
constexpr int RF_MAX_GB = (RF_MAX_DEG + 1) * (RF_MAX_DEG + 2) / 2 - 1;   // 152 basis functions
constexpr int RF_DOTS = 40;         // per-image dot results kept per launch
constexpr int RF_NB = 256;          // blocks per image of the vector kernels (upper bound)
constexpr double RF_MU_MAX = 1e8;   // Levenberg-Marquardt shift bound

// per-image device scalars (sc[n * NSC + k])
enum { S_ACTIVE, S_RR, S_R0, S_ETA, S_ALPHA, S_BETA, S_H, S_INV2H, S_MU, S_V1Y, S_G1, S_P1, S_DELTA, S_IT, S_NEG,
       S_ACCEPT, S_INVB, S_ONE, NSC };
enum { OP_NONE, OP_FDSTEP, OP_STORE_V1Y, OP_ALPHA, OP_BETA, OP_CGINIT, OP_STORE_G1, OP_UNIT, OP_PCGINIT, OP_PBETA };

// cuFFT, resolved at run time (the preconditioner is optional: without the
// library the CG runs unpreconditioned).  Handles are ints; the two
// transform types and the success code are cuFFT's public enum values.
using fft_handle = int;
constexpr int FFT_R2C = 0x2a, FFT_C2R = 0x2c, FFT_SUCCESS = 0;

struct FftApi {
    bool ok = false;
    int (*plan_many)(fft_handle *, int, int *, int *, int, int, int *, int, int, int, int) = nullptr;
    int (*exec_r2c)(fft_handle, float *, float2 *) = nullptr;
    int (*exec_c2r)(fft_handle, float2 *, float *) = nullptr;
    int (*set_stream)(fft_handle, cudaStream_t) = nullptr;
    int (*destroy)(fft_handle) = nullptr;
};

FftApi fft_load()
{
    FftApi api;
    std::vector<std::string> names = {"libcufft.so.12", "libcufft.so"};
    for (const char *env : {"CUDA_HOME", "CUDA_PATH"})
        if (const char *h = std::getenv(env)) names.push_back(std::string(h) + "/lib64/libcufft.so.12");
    names.push_back("/usr/local/cuda/lib64/libcufft.so.12");
    void *lib = nullptr;
    for (const auto &n : names)
        if ((lib = dlopen(n.c_str(), RTLD_NOW | RTLD_LOCAL))) break;
    if (!lib) return api;
    api.plan_many = (decltype(api.plan_many))dlsym(lib, "cufftPlanMany");
    api.exec_r2c = (decltype(api.exec_r2c))dlsym(lib, "cufftExecR2C");
    api.exec_c2r = (decltype(api.exec_c2r))dlsym(lib, "cufftExecC2R");
    api.set_stream = (decltype(api.set_stream))dlsym(lib, "cufftSetStream");
    api.destroy = (decltype(api.destroy))dlsym(lib, "cufftDestroy");
    api.ok = api.plan_many && api.exec_r2c && api.exec_c2r && api.set_stream && api.destroy;
    return api;
}

// Loaded once per process (a function-local static: thread-safe initialisation).
FftApi &fft_api()
{
    static FftApi api = fft_load();
    return api;
}

// One vector of the context's shape: nf arrays of F*M (x, y) / (Re, Im) double pairs.
struct Vec {
    double *p[3];
};

struct Term {
    int in;          // input index
    int s1, s2;      // scalar indices multiplying the coefficient (-1: none)
    int cidx;        // coefficient column of `coef` (-1: none)
    double mult;
};

struct LinArgs {
    Vec in[4];
    Term t[4];
    int nt;
    Vec out;
    int gate;            // scalar index: images whose scalar is 0 are not written (-1: all)
    Vec dw;              // partial dot of out with dw (dw.p[0] == null: none)
    int dot_slot;        // K index of that partial
    int dot_k;           // K of the partial buffer layout
    int op;              // with a dot: the per-image scalar step the last block runs (OP_*)
};

struct RefineWork {
    int F = 0, nf = 0, nx = 0, ny = 0;
    long M = 0;
    int nb = 1;                       // blocks per image in the vector kernels
    double *block = nullptr;          // all workspace vectors
    size_t vs = 0;                    // doubles per vector
    Vec g, v1, p, r, y, s, gp, gm, z[2], pmask;   // z: this and the previous preconditioned residual
    Vec lz[RF_MAX_LZ + 1];
    double *part = nullptr;           // partial sums [F][K][nb]
    unsigned *ticket = nullptr;       // per image: blocks that wrote their partials (last one finishes)
    double *dots = nullptr;           // [F][RF_DOTS]
    double *sc = nullptr;             // [F][NSC]
    double *coef = nullptr;           // [F][RF_MAX_LZ + 1] host-given coefficients
    double *gcoef = nullptr;          // [F][RF_MAX_GB] gauge coefficients
    double *gd = nullptr;             // gauge orbit gradients [F][(2 m + 1) m], m <= RF_MAX_GB
    std::vector<double> lam1, mu;
    std::vector<int> has_mode;        // a saddle image has a direction to start its Lanczos from
    std::vector<int> fresh;           // that direction is the caller's (longer first Lanczos)
    // CG iterations, per preconditioning (off / on) and current x buffer
    cudaGraphExec_t cg_graph[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    int64_t graph_launches[2] = {0, 0}, graph_grads[2] = {0, 0};   // kernels and gradients per replay
    bool pc_capture_failed = false;   // the preconditioned iterations then run without a graph
    // preconditioner: planes (n, f, c) mirrored to 2 ny x 2 nx, their spectra
    // (FP32: a preconditioner needs no more, and GB300's FP64 rate would make
    // the transforms cost more than a Hessian product), the model
    // (sigma, c_x, c_y) per plane and the eigenvalue factors 2 - 2 cos(pi k / n)
    // of the two directions
    int planes = 0;
    float *pc_ext = nullptr;
    float2 *pc_spec = nullptr;
    double *pc_coef = nullptr;
    double *pc_eig = nullptr;          // [nx + 1] x-factors, then [2 ny] y-factors
    double *pc_probe = nullptr;        // comb gathers
    size_t pc_probe_cap = 0;
    fft_handle fft_fwd = 0, fft_inv = 0;
    bool fft_plans = false;
    bool pc_failed = false;            // buffers or plans could not be made: no preconditioning
    // gauge-subspace Hessians kept between Newton iterations (and calls on
    // the same state): per image m x m, its age in iterations
    std::vector<std::vector<double>> gauge_h;
    std::vector<int> gauge_age;
    int gauge_m = -1;
    uint64_t state_version = ~0ull;   // the context's state version after the last refinement call
    // gauge Hessians are built from many perturbed copies of the images at
    // once: an internal FP64 context holding `wide_images` of them as one
    // string (chunks of the 2m F perturbations), and their orbit gradients
    mepgl_ctx *wide = nullptr;
    int wide_images = 0;
    // Hessian products: an internal FP64 context of 2F images holding x + h u
    // (images 0..F-1) and x - h u (F..2F-1), so that both gradients of the
    // central difference run as one launch
    mepgl_ctx *hvc = nullptr;
    double *wide_gd = nullptr;
    size_t wide_gd_cap = 0;
    // Legendre tables of the separable orbit gradients and their row sums
    double *gtab = nullptr;
    int gtab_deg = -1;
    double *rows = nullptr;
    size_t rows_cap = 0;
};

void refine_free(RefineWork *w)
{
    if (!w) return;
    for (auto &row : w->cg_graph)
        for (auto &g : row)
            if (g) cudaGraphExecDestroy(g);
    if (w->fft_plans) {
        fft_api().destroy(w->fft_fwd);
        fft_api().destroy(w->fft_inv);
    }
    cudaFree(w->pc_ext);
    cudaFree(w->pc_spec);
    cudaFree(w->pc_coef);
    cudaFree(w->pc_eig);
    cudaFree(w->pc_probe);
    cudaFree(w->block);
    cudaFree(w->part);
    cudaFree(w->ticket);
    cudaFree(w->dots);
    cudaFree(w->sc);
    cudaFree(w->coef);
    cudaFree(w->gcoef);
    cudaFree(w->gd);
    cudaFree(w->wide_gd);
    cudaFree(w->gtab);
    cudaFree(w->rows);
    if (w->wide) mepgl_destroy(w->wide);
    if (w->hvc) mepgl_destroy(w->hvc);
    delete w;
}

namespace {

// ------------------------------------------------------------------ kernels
__device__ __forceinline__ double block_reduce(double v, double *sh)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += sh[k];
    return t;   // valid in thread 0
}

// The vector kernels run on a grid (nb, F): block b of image n covers the
// range [b * per, (b + 1) * per) of each of the image's nf arrays of 2M
// doubles (per even, so that 16-byte pairs stay aligned).
__device__ __forceinline__ void vrange(long M2, int nb, long &r0, long &r1)
{
    long per = (M2 + nb - 1) / nb;
    per += per & 1;
    r0 = blockIdx.x * per;
    r1 = min(M2, r0 + per);
}

// Per-image sums of the partials of image n, then the scalar step `op`
// (thread 0).  Run by a whole block: the last one of a dot kernel's blocks
// for the image (ticket), or a k_dot_sums block.  The partials come through
// L2 (other blocks wrote them).
__device__ void dot_finish(const double *part, int K, int nb, double *dots, double *sc, int op, int n,
                           unsigned *ticket, double *sh)
{
    double s[RF_DOTS];
    for (int k = 0; k < K; ++k) {
        double v = 0.0;
        for (int b = threadIdx.x; b < nb; b += NT) v += __ldcg(part + ((long)n * K + k) * nb + b);
        s[k] = block_reduce(v, sh);
    }
    if (threadIdx.x != 0) return;
    if (ticket) ticket[n] = 0;   // ready for the next launch
    for (int k = 0; k < K; ++k) dots[n * RF_DOTS + k] = s[k];
    double *q = sc + n * NSC;
    const bool act = q[S_ACTIVE] != 0.0;
    switch (op) {
    case OP_FDSTEP:   // s[0] = |u|^2: central-difference step for H u
        if (act && s[0] > 0) {
            q[S_H] = q[S_DELTA] / sqrt(s[0]);
            q[S_INV2H] = 0.5 / q[S_H];
        } else {      // inactive, or u = 0: H u = 0
            q[S_H] = 0.0;
            q[S_INV2H] = 0.0;
        }
        break;
    case OP_STORE_V1Y: q[S_V1Y] = s[0]; break;
    case OP_STORE_G1: q[S_G1] = s[0]; break;
    case OP_ALPHA:    // s[0] = p . (H + mu) p
        if (act) {
            if (s[0] > 0) q[S_ALPHA] = q[S_RR] / s[0];
            else { q[S_ALPHA] = 0.0; q[S_ACTIVE] = 0.0; q[S_NEG] = 1.0; }
        } else {
            q[S_ALPHA] = 0.0;
        }
        break;
    case OP_BETA:     // s[0] = |r_new|^2
        if (act) {
            q[S_BETA] = q[S_RR] > 0 ? s[0] / q[S_RR] : 0.0;
            q[S_RR] = s[0];
            q[S_IT] += 1.0;
            if (!(sqrt(s[0]) > q[S_ETA] * q[S_R0])) q[S_ACTIVE] = 0.0;
        } else {
            q[S_BETA] = 0.0;
        }
        break;
    case OP_CGINIT:   // s[0] = |r_0|^2
        q[S_RR] = s[0];
        q[S_R0] = sqrt(s[0]);
        q[S_IT] = 0.0;
        q[S_NEG] = 0.0;
        if (!(s[0] > 0)) q[S_ACTIVE] = 0.0;
        break;
    case OP_UNIT:     // s[0] = |w|^2: 1/|w| for normalisation
        q[S_INVB] = s[0] > 0 ? 1.0 / sqrt(s[0]) : 0.0;
        break;
    case OP_PCGINIT:  // s[0] = r_0 . z_0, s[1] = |r_0|^2 (z = M^-1 r)
        q[S_RR] = s[0];
        q[S_R0] = sqrt(s[1]);
        q[S_IT] = 0.0;
        q[S_NEG] = 0.0;
        if (!(s[1] > 0) || !(s[0] > 0)) q[S_ACTIVE] = 0.0;
        break;
    case OP_PBETA:    // s[0] = r_new . z_new, s[1] = |r_new|^2, s[2] = r_new . z_old
        if (act) {
            q[S_BETA] = q[S_RR] > 0 ? (s[0] - s[2]) / q[S_RR] : 0.0;
            q[S_RR] = s[0];
            q[S_IT] += 1.0;
            if (!(sqrt(s[1]) > q[S_ETA] * q[S_R0]) || !(s[0] > 0)) q[S_ACTIVE] = 0.0;
        } else {
            q[S_BETA] = 0.0;
        }
        break;
    default: break;
    }
}

// True in every thread of the last block of image n to have written its
// partials (the partial writes are fenced before the ticket is taken).
__device__ __forceinline__ bool last_block(unsigned *ticket, int n, int nb)
{
    __shared__ int is_last;
    if (threadIdx.x == 0) {
        __threadfence();
        is_last = atomicAdd(ticket + n, 1u) == (unsigned)(nb - 1);
    }
    __syncthreads();
    const bool last = is_last != 0;
    if (last) __threadfence();
    return last;
}

// Per-image sums of the partials, then the scalar step `op` (a separate launch,
// for partials written by kernels without a ticket).
__global__ void __launch_bounds__(NT) k_dot_sums(const double *part, int K, int nb, double *dots, double *sc, int op)
{
    __shared__ double sh[NT / 32];
    dot_finish(part, K, nb, dots, sc, op, blockIdx.x, nullptr, sh);
}

// out = sum_t c_t in_t, per image; optional partial dot of out with dw.
template <int NTT>
__global__ void __launch_bounds__(NT) k_lincomb(LinArgs a, long M2, int nf, double *sc, const double *coef,
                                                int ccols, double *part, int nb, unsigned *ticket, double *dots)
{
    __shared__ double sh[NT / 32];
    const int n = blockIdx.y;
    const bool on = a.gate < 0 || sc[n * NSC + a.gate] != 0.0;
    double c[NTT];
#pragma unroll
    for (int k = 0; k < NTT; ++k) {
        double v = a.t[k].mult;
        if (a.t[k].s1 >= 0) v *= sc[n * NSC + a.t[k].s1];
        if (a.t[k].s2 >= 0) v *= sc[n * NSC + a.t[k].s2];
        if (a.t[k].cidx >= 0) v *= coef[n * ccols + a.t[k].cidx];
        c[k] = v;
    }
    long r0, r1;
    vrange(M2, nb, r0, r1);
    const long off = (long)n * M2;
    const bool dot = a.dw.p[0] != nullptr;
    double acc = 0.0;
    if (on)
#pragma unroll
        for (int f = 0; f < 3; ++f) {
            if (f >= nf) break;
            double2 *o = reinterpret_cast<double2 *>(a.out.p[f] + off);
            const double2 *dw = dot ? reinterpret_cast<const double2 *>(a.dw.p[f] + off) : nullptr;
            for (long r = r0 / 2 + threadIdx.x; r < r1 / 2; r += NT) {
                double2 v = make_double2(0.0, 0.0);
#pragma unroll
                for (int k = 0; k < NTT; ++k) {
                    const double2 x = reinterpret_cast<const double2 *>(a.in[k].p[f] + off)[r];
                    v.x += c[k] * x.x;
                    v.y += c[k] * x.y;
                }
                o[r] = v;
                if (dot) {
                    const double2 d = dw[r];
                    acc += v.x * d.x + v.y * d.y;
                }
            }
        }
    if (dot) {
        const double t = block_reduce(acc, sh);
        if (threadIdx.x == 0) part[((long)n * a.dot_k + a.dot_slot) * nb + blockIdx.x] = t;
        if (last_block(ticket, n, nb)) dot_finish(part, a.dot_k, nb, dots, sc, a.op, n, ticket, sh);
    }
}

// Partial dots of up to 4 pairs (u_k, w_k) per image.
struct DotArgs {
    Vec u[4], w[4];
    int k;
};

template <int K>
__global__ void __launch_bounds__(NT) k_dots(DotArgs a, long M2, int nf, double *part, int nb, int op,
                                             unsigned *ticket, double *dots, double *sc)
{
    __shared__ double sh[NT / 32];
    const int n = blockIdx.y;
    long r0, r1;
    vrange(M2, nb, r0, r1);
    const long off = (long)n * M2;
    double acc[K];
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] = 0.0;
#pragma unroll
    for (int f = 0; f < 3; ++f) {
        if (f >= nf) break;
        for (long r = r0 / 2 + threadIdx.x; r < r1 / 2; r += NT) {
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const double2 u = reinterpret_cast<const double2 *>(a.u[k].p[f] + off)[r];
                const double2 w = reinterpret_cast<const double2 *>(a.w[k].p[f] + off)[r];
                acc[k] += u.x * w.x + u.y * w.y;
            }
        }
    }
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const double t = block_reduce(acc[k], sh);
        if (threadIdx.x == 0) part[((long)n * K + k) * nb + blockIdx.x] = t;
    }
    if (last_block(ticket, n, nb)) dot_finish(part, K, nb, dots, sc, op, n, ticket, sh);
}

// Partial dots of w with Lanczos vectors lz_0 .. lz_{K-1} (contiguous, stride vs;
// array f of a vector at offset f * FM2).
__global__ void __launch_bounds__(NT) k_dots_lz(Vec w, const double *lz0, size_t vs, int K, long M2, int nf,
                                                long FM2, double *part, int nb)
{
    __shared__ double sh[NT / 32];
    const int n = blockIdx.y;
    long r0, r1;
    vrange(M2, nb, r0, r1);
    const long off = (long)n * M2;
    for (int k = 0; k < K; ++k) {
        double acc = 0.0;
        for (int f = 0; f < nf; ++f) {
            const double2 *b = reinterpret_cast<const double2 *>(lz0 + k * vs + f * FM2 + off);
            const double2 *x = reinterpret_cast<const double2 *>(w.p[f] + off);
            for (long r = r0 / 2 + threadIdx.x; r < r1 / 2; r += NT) {
                const double2 u = b[r], v = x[r];
                acc += u.x * v.x + u.y * v.y;
            }
        }
        const double t = block_reduce(acc, sh);
        if (threadIdx.x == 0) part[((long)n * K + k) * nb + blockIdx.x] = t;
    }
}

// w = c0 w - sum_k d_k lz_k, d_k = d[n * dstride + k].
__global__ void __launch_bounds__(NT) k_sub_lz(Vec w, double c0, const double *lz0, size_t vs, int K, long M2, int nf,
                                               long FM2, const double *d, int dstride, const double *sc, int gate,
                                               int nb)
{
    const int n = blockIdx.y;
    if (gate >= 0 && sc[n * NSC + gate] == 0.0) return;
    double dk[RF_MAX_LZ + 1];
    for (int k = 0; k < K; ++k) dk[k] = d[n * dstride + k];
    long r0, r1;
    vrange(M2, nb, r0, r1);
    const long off = (long)n * M2;
    for (int f = 0; f < nf; ++f) {
        double2 *x = reinterpret_cast<double2 *>(w.p[f] + off);
        for (long r = r0 / 2 + threadIdx.x; r < r1 / 2; r += NT) {
            double2 v = x[r];
            v.x *= c0;
            v.y *= c0;
            for (int k = 0; k < K; ++k) {
                const double2 b = reinterpret_cast<const double2 *>(lz0 + k * vs + f * FM2 + off)[r];
                v.x -= dk[k] * b.x;
                v.y -= dk[k] * b.y;
            }
            x[r] = v;
        }
    }
}

// ---------------------------------------------------------- gauge kernels
// Legendre polynomials P_0..P_deg at t.
__device__ __forceinline__ void legendre(double t, int deg, double *P)
{
    P[0] = 1.0;
    if (deg >= 1) P[1] = t;
    for (int k = 1; k < deg; ++k) P[k + 1] = ((2 * k + 1) * t * P[k] - k * P[k - 1]) / (k + 1);
}

struct GaugeBasis {
    int deg, m;
    unsigned char a[RF_MAX_GB], b[RF_MAX_GB];
};

__device__ __forceinline__ double coord(int i, int n) { return n > 1 ? (2.0 * i - (n - 1)) / (n - 1) : 0.0; }

// chi at lattice column i, row j: sum_m c_m P_a(X_i) P_b(Y_j) (only >= 0: that basis function alone)
__device__ double chi_at(const GaugeBasis &B, const double *c, int only, int i, int j, int nx, int ny)
{
    double Px[RF_MAX_DEG + 1], Py[RF_MAX_DEG + 1];
    legendre(coord(i, nx), B.deg, Px);
    legendre(coord(j, ny), B.deg, Py);
    if (only >= 0) return Px[B.a[only]] * Py[B.b[only]];
    double v = 0.0;
    for (int m = 0; m < B.m; ++m) v += c[m] * Px[B.a[m]] * Py[B.b[m]];
    return v;
}

struct GaugeField {
    double chi, gx, gy;   // chi and its lattice gradient (central, one-sided at the edges)
};

__device__ GaugeField gauge_field(const GaugeBasis &B, const double *c, int only, int i, int j, int nx, int ny,
                                  double idx)
{
    GaugeField G;
    G.chi = chi_at(B, c, only, i, j, nx, ny);
    const int il = i > 0 ? i - 1 : i, ir = i < nx - 1 ? i + 1 : i;
    const int jd = j > 0 ? j - 1 : j, ju = j < ny - 1 ? j + 1 : j;
    G.gx = (chi_at(B, c, only, ir, j, nx, ny) - chi_at(B, c, only, il, j, nx, ny)) * idx / (ir - il);
    G.gy = (chi_at(B, c, only, i, ju, nx, ny) - chi_at(B, c, only, i, jd, nx, ny)) * idx / (ju - jd);
    return G;
}

// out = U(mult * chi_n) in: A + grad chi, psi_a exp(i q_a chi); chi_n from coef[n][:] (or basis `only`).
__global__ void __launch_bounds__(NT) k_gauge_apply(Vec in, Vec out, GaugeBasis B, const double *coef, int ccols,
                                                    int only, double mult, int nx, int ny, int ncomp, double q1,
                                                    double q2, double idx, const double *sc, int gate)
{
    const int n = blockIdx.y;
    if (gate >= 0 && sc[n * NSC + gate] == 0.0) return;
    const long M = (long)nx * ny;
    for (long s = blockIdx.x * (long)NT + threadIdx.x; s < M; s += (long)gridDim.x * NT) {
        const int i = (int)(s % nx), j = (int)(s / nx);
        const GaugeField G = gauge_field(B, coef + n * ccols, only, i, j, nx, ny, idx);
        const long o = 2 * ((long)n * M + s);
        out.p[0][o] = in.p[0][o] + mult * G.gx;
        out.p[0][o + 1] = in.p[0][o + 1] + mult * G.gy;
        for (int a = 0; a < ncomp; ++a) {
            double sn, cs;
            sincos((a ? q2 : q1) * mult * G.chi, &sn, &cs);
            const double re = in.p[1 + a][o], im = in.p[1 + a][o + 1];
            out.p[1 + a][o] = re * cs - im * sn;
            out.p[1 + a][o + 1] = re * sn + im * cs;
        }
    }
}

// Separable orbit gradients.  With phi_m = P_a(X_i) P_b(Y_j),
//   dE/dc_m = sum_j [ Py_j,b Sx_j,a + DPy_j,b Sy_j,a + Py_j,b Sw_j,a ],
//   Sx_j,a = sum_i gAx DPx_i,a,  Sy_j,a = sum_i gAy Px_i,a,  Sw_j,a = sum_i w Px_i,a,
// w = sum_c q_c (Re psi_c g_Im,c - Im psi_c g_Re,c); P / DP are the Legendre
// values and their lattice differences (central, one-sided at the edge, times
// 1/dx) per column / row, tabulated once.  Per site this is 3 (deg + 1)
// multiply-adds instead of the polynomial recurrences for every function.
struct GaugeTables {
    const double *px, *dpx, *py, *dpy;   // [nx][deg+1], [ny][deg+1]
};

// Wide copies for the gauge Hessian: image b of `out` is perturbation
// w = w0 + b of the 2 m F perturbations, U(+-h phi_k) applied to image n of
// `in`, w = (n m + k) 2 + sign, with phi_k = P_a(X_i) P_b(Y_j) and its lattice
// gradient read from the Legendre tables.  Grid (row blocks, n_out).
__global__ void __launch_bounds__(NT) k_gauge_perturb(Vec in, Vec out, GaugeBasis B, GaugeTables T, int F, int w0,
                                                      int n_out, double h, int nx, int ny, int ncomp, double q1,
                                                      double q2)
{
    const int b = blockIdx.y, w = w0 + b;
    if (b >= n_out || w >= 2 * B.m * F) return;
    const int n = w / (2 * B.m), r = w % (2 * B.m), k = r >> 1;
    const double mult = (r & 1) ? -h : h;
    const int D1 = B.deg + 1, ea = B.a[k], eb = B.b[k];
    const long M = (long)nx * ny;
    for (int j = blockIdx.x; j < ny; j += gridDim.x) {
        const double py = T.py[(long)j * D1 + eb], dpy = T.dpy[(long)j * D1 + eb];
        for (int i = threadIdx.x; i < nx; i += NT) {
            const double px = T.px[(long)i * D1 + ea], dpx = T.dpx[(long)i * D1 + ea];
            const double chi = px * py;
            const long s = (long)j * nx + i;
            const long o = 2 * ((long)n * M + s), ob = 2 * ((long)b * M + s);
            out.p[0][ob] = in.p[0][o] + mult * (dpx * py);
            out.p[0][ob + 1] = in.p[0][o + 1] + mult * (px * dpy);
            for (int a = 0; a < ncomp; ++a) {
                double sn, cs;
                sincos((a ? q2 : q1) * mult * chi, &sn, &cs);
                const double re = in.p[1 + a][o], im = in.p[1 + a][o + 1];
                out.p[1 + a][ob] = re * cs - im * sn;
                out.p[1 + a][ob + 1] = re * sn + im * cs;
            }
        }
    }
}

constexpr int RS_THREADS = 128;

// Row sums: block (j, n) -> rows[(n ny + j) 3 (deg+1) + {x, y, w} (deg+1) + a].
template <int D1>
__global__ void __launch_bounds__(RS_THREADS) k_gauge_rows(Vec x, Vec g, GaugeTables T, int nx, int ny, int ncomp,
                                                           double q1, double q2, double *rows)
{
    __shared__ double sh[RS_THREADS / 32][3 * D1];
    const int j = blockIdx.x, n = blockIdx.y;
    const long M = (long)nx * ny;
    double sx[D1], sy[D1], sw[D1];
#pragma unroll
    for (int a = 0; a < D1; ++a) sx[a] = sy[a] = sw[a] = 0.0;
    for (int i = threadIdx.x; i < nx; i += RS_THREADS) {
        const long o = 2 * ((long)n * M + (long)j * nx + i);
        const double gax = g.p[0][o], gay = g.p[0][o + 1];
        double w = 0.0;
        for (int c = 0; c < ncomp; ++c)
            w += (c ? q2 : q1) * (x.p[1 + c][o] * g.p[1 + c][o + 1] - x.p[1 + c][o + 1] * g.p[1 + c][o]);
        const double *px = T.px + (long)i * D1, *dpx = T.dpx + (long)i * D1;
#pragma unroll
        for (int a = 0; a < D1; ++a) {
            const double p = px[a];
            sx[a] += gax * dpx[a];
            sy[a] += gay * p;
            sw[a] += w * p;
        }
    }
    const int wi = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
    for (int a = 0; a < D1; ++a) {
        double v[3] = {sx[a], sy[a], sw[a]};
#pragma unroll
        for (int t = 0; t < 3; ++t) {
            for (int o = 16; o > 0; o >>= 1) v[t] += __shfl_down_sync(0xffffffffu, v[t], o);
            if (l == 0) sh[wi][t * D1 + a] = v[t];
        }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < 3 * D1; t += RS_THREADS) {
        double v = 0.0;
        for (int k = 0; k < RS_THREADS / 32; ++k) v += sh[k][t];
        rows[((long)n * ny + j) * 3 * D1 + t] = v;
    }
}

// Combination over rows: block n, thread m -> gd[n gstride + slot m_total + m].
__global__ void __launch_bounds__(NT) k_gauge_combine(const double *rows, GaugeBasis B, GaugeTables T, int ny,
                                                      double *gd, int gstride, int slot)
{
    const int n = blockIdx.x, D1 = B.deg + 1;
    for (int m = threadIdx.x; m < B.m; m += NT) {
        const int a = B.a[m], b = B.b[m];
        double v = 0.0;
        for (int j = 0; j < ny; ++j) {
            const double *r = rows + ((long)n * ny + j) * 3 * D1;
            v += T.py[(long)j * D1 + b] * (r[a] + r[2 * D1 + a]) + T.dpy[(long)j * D1 + b] * r[D1 + a];
        }
        gd[(long)n * gstride + slot * B.m + m] = v;
    }
}

// ------------------------------------------------------ preconditioner kernels
__device__ __forceinline__ const double *field_ptr(const Vec &v, int f)
{
    return f == 0 ? v.p[0] : (f == 1 ? v.p[1] : v.p[2]);
}

__device__ __forceinline__ double *field_ptr_w(const Vec &v, int f)
{
    return f == 0 ? v.p[0] : (f == 1 ? v.p[1] : v.p[2]);
}

// Mirror the masked field (n, f) = blockIdx.z to its two planes (Re / x, Im / y)
// of 2 ny x 2 nx: plane row J < ny is lattice row J, row J >= ny is row
// 2 ny - 1 - J (columns alike).  Grid (ceil(2 nx / NT), 2 ny, F nf).
__global__ void __launch_bounds__(NT) k_pc_extend(Vec r, Vec mask, float *ext, int nx, int ny, int nf)
{
    const int I = blockIdx.x * NT + threadIdx.x, J = blockIdx.y, nfz = blockIdx.z;
    const int W = 2 * nx;
    if (I >= W) return;
    const int n = nfz / nf, f = nfz % nf;
    const int i = I < nx ? I : W - 1 - I, j = J < ny ? J : 2 * ny - 1 - J;
    const long o = 2 * ((long)n * nx * ny + (long)j * nx + i);
    const double2 v = *reinterpret_cast<const double2 *>(field_ptr(r, f) + o);
    const double2 m = *reinterpret_cast<const double2 *>(field_ptr(mask, f) + o);
    const long E = 4L * nx * ny, e = (long)J * W + I;
    ext[(2L * nfz) * E + e] = (float)(v.x * m.x);
    ext[(2L * nfz + 1) * E + e] = (float)(v.y * m.y);
}

// Spectrum of plane q = blockIdx.z (2 ny rows of nx + 1 frequencies) divided by
// the model's eigenvalue sigma + c_x ex[kx] + c_y ey[ky], and by the 4 nx ny of
// the unnormalised transform pair.  FP32 like the spectrum (an FP64 division
// per element made this kernel cost more than both transforms).
__global__ void __launch_bounds__(NT) k_pc_scale(float2 *spec, const double *coef, const double *eig, int nx, int ny)
{
    const int kx = blockIdx.x * NT + threadIdx.x, ky = blockIdx.y, q = blockIdx.z;
    if (kx > nx) return;
    const float norm = 4.0f * (float)nx * (float)ny;
    const float sg = (float)coef[3 * q] * norm, cx = (float)coef[3 * q + 1] * norm, cy = (float)coef[3 * q + 2] * norm;
    const float lam = sg + cx * (float)eig[kx] + cy * (float)eig[nx + 1 + ky];
    const long o = (long)q * 2 * ny * (nx + 1) + (long)ky * (nx + 1) + kx;
    const float il = 1.0f / lam;
    float2 v = spec[o];
    v.x *= il;
    v.y *= il;
    spec[o] = v;
}

// z = mask * (top-left ny x nx block of the two planes).  Grid (ceil(nx / NT), ny, F nf).
__global__ void __launch_bounds__(NT) k_pc_extract(const float *ext, Vec z, Vec mask, int nx, int ny, int nf)
{
    const int i = blockIdx.x * NT + threadIdx.x, j = blockIdx.y, nfz = blockIdx.z;
    if (i >= nx) return;
    const int n = nfz / nf, f = nfz % nf;
    const long o = 2 * ((long)n * nx * ny + (long)j * nx + i);
    const long E = 4L * nx * ny, e = (long)j * 2 * nx + i;
    const double2 m = *reinterpret_cast<const double2 *>(field_ptr(mask, f) + o);
    *reinterpret_cast<double2 *>(field_ptr_w(z, f) + o) =
        make_double2((double)ext[(2L * nfz) * E + e] * m.x, (double)ext[(2L * nfz + 1) * E + e] * m.y);
}

// A probe vector with entries in [0.5, 1.5) from a hash of the index.
__global__ void __launch_bounds__(NT) k_pc_hash(Vec u, long n_per_field, int nf)
{
    for (long k = blockIdx.x * (long)NT + threadIdx.x; k < n_per_field; k += (long)gridDim.x * NT) {
        for (int f = 0; f < nf; ++f) {
            uint64_t h = (uint64_t)k * 0x9E3779B97F4A7C15ull + (uint64_t)(f + 1) * 0xD1B54A32D192ED03ull;
            h ^= h >> 31;
            h *= 0xBF58476D1CE4E5B9ull;
            h ^= h >> 29;
            field_ptr_w(u, f)[k] = 0.5 + (double)(h >> 11) * (1.0 / 9007199254740992.0);
        }
    }
}

// mask = 1 where (H u) != 0 (the energy depends on that degree of freedom), else 0.
__global__ void __launch_bounds__(NT) k_pc_mask(Vec y, Vec mask, long n_per_field, int nf)
{
    for (long k = blockIdx.x * (long)NT + threadIdx.x; k < n_per_field; k += (long)gridDim.x * NT)
        for (int f = 0; f < nf; ++f) field_ptr_w(mask, f)[k] = field_ptr(y, f)[k] != 0.0 ? 1.0 : 0.0;
}

// Comb of probe sites: site k = (2 + (k % kx) sp, 2 + (k / kx) sp).
struct Comb {
    int kx, ky, sp;
};

// u: 1 at the comb sites of component c of field f in every image (u zero elsewhere).
__global__ void __launch_bounds__(NT) k_pc_comb(Vec u, Comb cb, int f, int c, int nx, int ny)
{
    const int k = blockIdx.x * NT + threadIdx.x, n = blockIdx.y;
    if (k >= cb.kx * cb.ky) return;
    const int i = 2 + (k % cb.kx) * cb.sp, j = 2 + (k / cb.kx) * cb.sp;
    field_ptr_w(u, f)[2 * ((long)n * nx * ny + (long)j * nx + i) + c] = 1.0;
}

// Column of H at each comb site: out[(n K + k) 6 + t] = diagonal, +x, -x, +y,
// -y neighbours (same component), and 1 when all five are live dofs.
__global__ void __launch_bounds__(NT) k_pc_gather(Vec y, Vec mask, Comb cb, int f, int c, int nx, int ny, double *out)
{
    const int k = blockIdx.x * NT + threadIdx.x, n = blockIdx.y;
    const int K = cb.kx * cb.ky;
    if (k >= K) return;
    const int i = 2 + (k % cb.kx) * cb.sp, j = 2 + (k / cb.kx) * cb.sp;
    const double *yp = field_ptr(y, f), *mp = field_ptr(mask, f);
    const long base = (long)n * nx * ny;
    const long s[5] = {(long)j * nx + i, (long)j * nx + i + 1, (long)j * nx + i - 1, (long)(j + 1) * nx + i,
                       (long)(j - 1) * nx + i};
    double live = 1.0;
    double *o = out + ((long)n * K + k) * 6;
    for (int t = 0; t < 5; ++t) {
        o[t] = yp[2 * (base + s[t]) + c];
        live *= mp[2 * (base + s[t]) + c];
    }
    o[5] = live;
}

// ------------------------------------------------------------ host helpers
// Symmetric eigen-decomposition by cyclic Jacobi rotations: eigenvalues
// ascending in w, eigenvectors in the columns of V (row-major n x n).
void jacobi_eig(int n, std::vector<double> A, std::vector<double> &w, std::vector<double> &V)
{
    V.assign(n * n, 0.0);
    for (int i = 0; i < n; ++i) V[i * n + i] = 1.0;
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0, tot = 0.0;
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                tot += A[i * n + j] * A[i * n + j];
                if (i != j) off += A[i * n + j] * A[i * n + j];
            }
        if (off <= 1e-30 * tot || off == 0.0) break;
        for (int p = 0; p < n; ++p)
            for (int q = p + 1; q < n; ++q) {
                const double apq = A[p * n + q];
                if (apq == 0.0) continue;
                const double th = (A[q * n + q] - A[p * n + p]) / (2 * apq);
                const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1));
                const double c = 1 / std::sqrt(t * t + 1), s = t * c;
                for (int k = 0; k < n; ++k) {
                    const double akp = A[k * n + p], akq = A[k * n + q];
                    A[k * n + p] = c * akp - s * akq;
                    A[k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {
                    const double apk = A[p * n + k], aqk = A[q * n + k];
                    A[p * n + k] = c * apk - s * aqk;
                    A[q * n + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    const double vkp = V[k * n + p], vkq = V[k * n + q];
                    V[k * n + p] = c * vkp - s * vkq;
                    V[k * n + q] = s * vkp + c * vkq;
                }
            }
    }
    std::vector<int> ord(n);
    for (int i = 0; i < n; ++i) ord[i] = i;
    std::sort(ord.begin(), ord.end(), [&](int a, int b) { return A[a * n + a] < A[b * n + b]; });
    w.resize(n);
    std::vector<double> V2(n * n);
    for (int k = 0; k < n; ++k) {
        w[k] = A[ord[k] * n + ord[k]];
        for (int i = 0; i < n; ++i) V2[i * n + k] = V[i * n + ord[k]];
    }
    V.swap(V2);
}

// Cholesky solve of the SPD system H c = -g (m x m, row-major); false if H is not positive definite.
bool cholesky_solve(int m, std::vector<double> H, const double *g, double *c)
{
    for (int j = 0; j < m; ++j) {
        double d = H[j * m + j];
        for (int k = 0; k < j; ++k) d -= H[j * m + k] * H[j * m + k];
        if (!(d > 0)) return false;
        d = std::sqrt(d);
        H[j * m + j] = d;
        for (int i = j + 1; i < m; ++i) {
            double v = H[i * m + j];
            for (int k = 0; k < j; ++k) v -= H[i * m + k] * H[j * m + k];
            H[i * m + j] = v / d;
        }
    }
    std::vector<double> y(m);
    for (int i = 0; i < m; ++i) {
        double v = -g[i];
        for (int k = 0; k < i; ++k) v -= H[i * m + k] * y[k];
        y[i] = v / H[i * m + i];
    }
    for (int i = m - 1; i >= 0; --i) {
        double v = y[i];
        for (int k = i + 1; k < m; ++k) v -= H[k * m + i] * c[k];
        c[i] = v / H[i * m + i];
    }
    return true;
}

struct Ctx {
    mepgl_ctx *c;
    RefineWork *w;
    Launch L;
    int F;
    long M2;
    cudaStream_t st;
    int64_t grads = 0;
    std::vector<double> hsc;   // host copy of the scalars

    Vec x() const
    {
        const StringHost &s = c->strings[0];
        return Vec{{(double *)s.x[c->xi][0], (double *)s.x[c->xi][1], (double *)s.x[c->xi][2]}};
    }
    Vec xt() const
    {
        const StringHost &s = c->strings[0];
        return Vec{{(double *)s.x[c->xi ^ 1][0], (double *)s.x[c->xi ^ 1][1], (double *)s.x[c->xi ^ 1][2]}};
    }
    dim3 vgrid() const { return dim3(w->nb, F); }

    cudaError_t grad(int xbuf, const Vec &out)
    {
        FieldPtrs fp;
        for (int f = 0; f < 3; ++f) fp.p[f] = f < w->nf ? out.p[f] : nullptr;
        ++grads;
        c->launches += 1;
        return launch_gradient_only(L, xbuf, fp, 0);
    }
    cudaError_t lin(const LinArgs &a)
    {
        const double *cf = w->coef;
        const int cc = RF_MAX_LZ + 1;
        unsigned *tk = w->ticket;
        double *ds = w->dots;
        switch (a.nt) {
        case 1: k_lincomb<1><<<vgrid(), NT, 0, st>>>(a, M2, w->nf, w->sc, cf, cc, w->part, w->nb, tk, ds); break;
        case 2: k_lincomb<2><<<vgrid(), NT, 0, st>>>(a, M2, w->nf, w->sc, cf, cc, w->part, w->nb, tk, ds); break;
        case 3: k_lincomb<3><<<vgrid(), NT, 0, st>>>(a, M2, w->nf, w->sc, cf, cc, w->part, w->nb, tk, ds); break;
        default: k_lincomb<4><<<vgrid(), NT, 0, st>>>(a, M2, w->nf, w->sc, cf, cc, w->part, w->nb, tk, ds); break;
        }
        c->launches += 1;
        return cudaGetLastError();
    }
    cudaError_t sums(int K, int op)
    {
        k_dot_sums<<<F, NT, 0, st>>>(w->part, K, w->nb, w->dots, w->sc, op);
        c->launches += 1;
        return cudaGetLastError();
    }
    cudaError_t dots(std::initializer_list<std::pair<Vec, Vec>> pairs, int op)
    {
        DotArgs a;
        memset(&a, 0, sizeof(a));
        for (auto &pr : pairs) {
            a.u[a.k] = pr.first;
            a.w[a.k] = pr.second;
            ++a.k;
        }
        unsigned *tk = w->ticket;
        double *ds = w->dots, *scw = w->sc;
        switch (a.k) {
        case 1: k_dots<1><<<vgrid(), NT, 0, st>>>(a, M2, w->nf, w->part, w->nb, op, tk, ds, scw); break;
        case 2: k_dots<2><<<vgrid(), NT, 0, st>>>(a, M2, w->nf, w->part, w->nb, op, tk, ds, scw); break;
        case 3: k_dots<3><<<vgrid(), NT, 0, st>>>(a, M2, w->nf, w->part, w->nb, op, tk, ds, scw); break;
        default: k_dots<4><<<vgrid(), NT, 0, st>>>(a, M2, w->nf, w->part, w->nb, op, tk, ds, scw); break;
        }
        c->launches += 1;
        return cudaGetLastError();   // the last block of each image sums and runs `op`
    }
    cudaError_t read_scalars()
    {
        hsc.resize((size_t)F * NSC);
        cudaError_t e = cudaMemcpyAsync(hsc.data(), w->sc, hsc.size() * 8, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        return e;
    }
    cudaError_t write_scalars()
    {
        return cudaMemcpyAsync(w->sc, hsc.data(), hsc.size() * 8, cudaMemcpyHostToDevice, st);
    }
    double &S(int n, int k) { return hsc[(size_t)n * NSC + k]; }
};

LinArgs lin_args(Vec out, int gate = -1)
{
    LinArgs a;
    memset(&a, 0, sizeof(a));
    a.out = out;
    a.gate = gate;
    return a;
}

void add_term(LinArgs &a, Vec v, double mult, int s1 = -1, int s2 = -1, int cidx = -1)
{
    a.in[a.nt] = v;
    a.t[a.nt] = Term{a.nt, s1, s2, cidx, mult};
    ++a.nt;
}

#define RK(call)                                                                                    \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess)                                                                      \
            return ctx_fail(R.c, MEPGL_ERR_CUDA, std::string("refine: ") + #call + ": " + cudaGetErrorString(e_)); \
    } while (0)

// An internal FP64 context with the refined context's problem and options
// and `images` images (IEEE double arithmetic), on the same stream.
mepgl_status twin_ctx(Ctx &R, int images, mepgl_ctx **out)
{
    mepgl_ctx *c = R.c;
    const StringHost &s = c->strings[0];
    mepgl_problem p;
    memset(&p, 0, sizeof(p));
    p.nx = s.nx;
    p.ny = s.ny;
    p.n_images = images;
    p.multicomponent = c->ncomp == 2;
    p.thin_film = c->thin_film;
    p.precision = MEPGL_FP64;
    p.dx = s.dx;
    p.q_1 = s.q[0];
    p.q_2 = s.q[1];
    p.eta = s.eta;
    p.gamma = s.gamma;
    p.delta = s.delta;
    const double **pp[9] = {&p.a_1, &p.b_1, &p.m_xx_1, &p.m_yy_1, &p.a_2, &p.b_2, &p.m_xx_2, &p.m_yy_2, &p.h};
    for (int k = 0; k < 9; ++k) *pp[k] = s.params[k].empty() ? nullptr : s.params[k].data();
    if (c->ncomp == 1)
        for (int k = 4; k < 8; ++k) *pp[k] = nullptr;
    p.comp_domain = s.comp.data();
    p.sc_domain = s.sc.data();
    mepgl_options o = c->opt;
    o.fp64_arith = MEPGL_FP64_NATIVE;
    if (mepgl_create(&p, &o, c->stream, out) != MEPGL_OK)
        return ctx_fail(c, MEPGL_ERR_CUDA, std::string("refine: internal context: ") + mepgl_last_error(nullptr));
    return MEPGL_OK;
}

// y = (H + mu) u by central differences (u's step from S_DELTA / |u|); images gated by S_ACTIVE.
// x + h u and x - h u go to the two halves of the Hessian-product context,
// whose gradient then runs as one launch over its 2F images.
mepgl_status hess_vec(Ctx &R, const Vec &u, const Vec &y, bool with_mu)
{
    RefineWork *w = R.w;
    if (!w->hvc) return ctx_fail(R.c, MEPGL_ERR_CUDA, "refine: Hessian-product context missing");
    const StringHost &hs = w->hvc->strings[0];
    const size_t half = (size_t)R.F * R.M2;   // doubles of F images in one field array
    Vec xp, xm, gp, gm;
    for (int f = 0; f < 3; ++f) {
        double *xb = f < w->nf ? (double *)hs.x[0][f] : nullptr;
        double *gb = f < w->nf ? (double *)hs.g[0][f] : nullptr;
        xp.p[f] = xb;
        xm.p[f] = xb ? xb + half : nullptr;
        gp.p[f] = gb;
        gm.p[f] = gb ? gb + half : nullptr;
    }
    RK(R.dots({{u, u}}, OP_FDSTEP));
    LinArgs a = lin_args(xp);
    add_term(a, R.x(), 1.0);
    add_term(a, u, 1.0, S_H);
    RK(R.lin(a));
    a = lin_args(xm);
    add_term(a, R.x(), 1.0);
    add_term(a, u, -1.0, S_H);
    RK(R.lin(a));
    FieldPtrs fp;
    for (int f = 0; f < 3; ++f) fp.p[f] = gp.p[f];
    Launch Lh = ctx_string_launch(w->hvc, 0);
    Lh.paired = 0;
    Lh.stream = R.st;
    R.grads += 2;
    R.c->launches += 1;
    RK(launch_gradient_only(Lh, 0, fp, 0));
    a = lin_args(y);
    add_term(a, gp, 1.0, S_INV2H);
    add_term(a, gm, -1.0, S_INV2H);
    if (with_mu) add_term(a, u, 1.0, S_MU);
    RK(R.lin(a));
    return MEPGL_OK;
}

// ------------------------------------------------------------ preconditioner
// Buffers and cuFFT plans (kept with the workspace); false when cuFFT is
// unavailable or the plans cannot be made.
bool pc_alloc(Ctx &R)
{
    RefineWork *w = R.w;
    if (w->fft_plans) return true;
    FftApi &api = fft_api();
    if (!api.ok || w->pc_failed) return false;
    w->pc_failed = true;   // until the plans exist
    const int nx = w->nx, ny = w->ny;
    w->planes = R.F * w->nf * 2;
    const size_t E = 4ull * nx * ny, S = 2ull * ny * (nx + 1);
    cudaError_t e = cudaMalloc(&w->pc_ext, w->planes * E * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&w->pc_spec, w->planes * S * sizeof(float2));
    if (e == cudaSuccess) e = cudaMalloc(&w->pc_coef, w->planes * 3 * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&w->pc_eig, (nx + 1 + 2 * ny) * sizeof(double));
    if (e != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    std::vector<double> eig(nx + 1 + 2 * ny);
    const double pi = 3.14159265358979323846;
    for (int k = 0; k <= nx; ++k) eig[k] = 2.0 - 2.0 * std::cos(pi * k / nx);
    for (int k = 0; k < 2 * ny; ++k) eig[nx + 1 + k] = 2.0 - 2.0 * std::cos(pi * k / ny);
    if (cudaMemcpy(w->pc_eig, eig.data(), eig.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
        return false;
    int dims[2] = {2 * ny, 2 * nx};
    if (api.plan_many(&w->fft_fwd, 2, dims, nullptr, 1, 0, nullptr, 1, 0, FFT_R2C, w->planes) != FFT_SUCCESS)
        return false;
    if (api.plan_many(&w->fft_inv, 2, dims, nullptr, 1, 0, nullptr, 1, 0, FFT_C2R, w->planes) != FFT_SUCCESS) {
        api.destroy(w->fft_fwd);
        return false;
    }
    w->fft_plans = true;
    w->pc_failed = false;
    return true;
}

// z = P M^-1 r (P: projection off v1; the images' planes all transformed).
mepgl_status pc_apply(Ctx &R, const Vec &r, const Vec &z)
{
    RefineWork *w = R.w;
    FftApi &api = fft_api();
    const int nx = w->nx, ny = w->ny;
    k_pc_extend<<<dim3((2 * nx + NT - 1) / NT, 2 * ny, R.F * w->nf), NT, 0, R.st>>>(r, w->pmask, w->pc_ext, nx, ny,
                                                                                 w->nf);
    RK(cudaGetLastError());
    if (api.set_stream(w->fft_fwd, R.st) != FFT_SUCCESS || api.exec_r2c(w->fft_fwd, w->pc_ext, w->pc_spec) != FFT_SUCCESS)
        return ctx_fail(R.c, MEPGL_ERR_CUDA, "refine: preconditioner forward transform failed");
    k_pc_scale<<<dim3((nx + 1 + NT - 1) / NT, 2 * ny, w->planes), NT, 0, R.st>>>(w->pc_spec, w->pc_coef, w->pc_eig,
                                                                              nx, ny);
    RK(cudaGetLastError());
    if (api.set_stream(w->fft_inv, R.st) != FFT_SUCCESS || api.exec_c2r(w->fft_inv, w->pc_spec, w->pc_ext) != FFT_SUCCESS)
        return ctx_fail(R.c, MEPGL_ERR_CUDA, "refine: preconditioner inverse transform failed");
    k_pc_extract<<<dim3((nx + NT - 1) / NT, ny, R.F * w->nf), NT, 0, R.st>>>(w->pc_ext, z, w->pmask, nx, ny, w->nf);
    R.c->launches += 3;
    RK(cudaGetLastError());
    RK(R.dots({{w->v1, z}}, OP_STORE_V1Y));
    LinArgs a = lin_args(z, S_ACTIVE);
    add_term(a, z, 1.0);
    add_term(a, w->v1, -1.0, S_V1Y);
    RK(R.lin(a));
    return MEPGL_OK;
}

// The model of each image's planes at the current x: the live-dof mask from
// one probe H u (u positive, hashed), then per field component a comb probe
// whose Hessian columns give c_x, c_y and the mass averaged over live bulk
// sites.  Images with S_ACTIVE == 0 keep M = I.  `usable` is false (no
// preconditioning) when the lattice has no comb site, is taller than the
// transform kernels' grid allows, or cuFFT or its buffers are unavailable.
mepgl_status pc_setup(Ctx &R, bool &usable)
{
    RefineWork *w = R.w;
    usable = false;
    const int nx = w->nx, ny = w->ny, F = R.F, nf = w->nf;
    // (the transform kernels put the 2 ny mirrored rows on the grid's y dimension)
    if (nx < 5 || ny < 5 || 2L * ny > 65535) return MEPGL_OK;
    if (!pc_alloc(R)) return MEPGL_OK;
    const long nper = (long)F * 2 * w->M;
    const int grid = (int)std::min<long>((nper + NT - 1) / NT, 4096);
    // 1. mask
    k_pc_hash<<<grid, NT, 0, R.st>>>(w->p, nper, nf);
    R.c->launches += 1;
    RK(cudaGetLastError());
    mepgl_status st = hess_vec(R, w->p, w->y, false);
    if (st != MEPGL_OK) return st;
    k_pc_mask<<<grid, NT, 0, R.st>>>(w->y, w->pmask, nper, nf);
    R.c->launches += 1;
    RK(cudaGetLastError());
    // 2. comb probes: about 1024 sites, spacing >= 4 (the Hessian couples sites
    // at most 2 apart, so the probed columns do not overlap where they are read)
    Comb cb;
    cb.sp = std::max(4, (int)std::ceil(std::sqrt((double)(nx - 4) * (ny - 4) / 1024.0)));
    cb.kx = (nx - 5) / cb.sp + 1;
    cb.ky = (ny - 5) / cb.sp + 1;
    const int K = cb.kx * cb.ky;
    const size_t need = (size_t)2 * nf * F * K * 6;
    if (w->pc_probe_cap < need) {
        cudaFree(w->pc_probe);
        w->pc_probe = nullptr;
        w->pc_probe_cap = 0;
        RK(cudaMalloc(&w->pc_probe, need * sizeof(double)));
        w->pc_probe_cap = need;
    }
    for (int f = 0; f < nf; ++f)
        for (int c = 0; c < 2; ++c) {
            for (int ff = 0; ff < nf; ++ff) RK(cudaMemsetAsync(w->p.p[ff], 0, nper * sizeof(double), R.st));
            k_pc_comb<<<dim3((K + NT - 1) / NT, F), NT, 0, R.st>>>(w->p, cb, f, c, nx, ny);
            R.c->launches += 1;
            RK(cudaGetLastError());
            st = hess_vec(R, w->p, w->y, false);
            if (st != MEPGL_OK) return st;
            k_pc_gather<<<dim3((K + NT - 1) / NT, F), NT, 0, R.st>>>(w->y, w->pmask, cb, f, c, nx, ny,
                                                                  w->pc_probe + (size_t)(f * 2 + c) * F * K * 6);
            R.c->launches += 1;
            RK(cudaGetLastError());
        }
    std::vector<double> h(need);
    RK(cudaMemcpyAsync(h.data(), w->pc_probe, need * sizeof(double), cudaMemcpyDeviceToHost, R.st));
    RK(R.read_scalars());
    // 3. per image and field: c_x, c_y per component, one mass for both
    std::vector<double> coef((size_t)w->planes * 3);
    bool any = false;
    for (int n = 0; n < F; ++n)
        for (int f = 0; f < nf; ++f) {
            double cx[2] = {0, 0}, cy[2] = {0, 0}, mass = 0.0;
            long cnt[2] = {0, 0};
            for (int c = 0; c < 2; ++c) {
                const double *o = h.data() + ((size_t)(f * 2 + c) * F + n) * K * 6;
                for (int k = 0; k < K; ++k, o += 6) {
                    if (o[5] == 0.0) continue;
                    const double sx = -0.5 * (o[1] + o[2]), sy = -0.5 * (o[3] + o[4]);
                    cx[c] += sx;
                    cy[c] += sy;
                    mass += o[0] - 2.0 * sx - 2.0 * sy;
                    ++cnt[c];
                }
            }
            const bool ok = R.S(n, S_ACTIVE) != 0.0 && cnt[0] > 0 && cnt[1] > 0;
            mass = ok ? mass / (double)(cnt[0] + cnt[1]) : 0.0;
            double top = 0.0;
            for (int c = 0; c < 2; ++c) {
                cx[c] = ok ? std::max(0.0, cx[c] / cnt[c]) : 0.0;
                cy[c] = ok ? std::max(0.0, cy[c] / cnt[c]) : 0.0;
                top = std::max(top, cx[c] + cy[c]);
            }
            const double sigma = ok ? std::max(mass, 1e-3 * top) : 1.0;
            for (int c = 0; c < 2; ++c) {
                double *q = coef.data() + 3 * ((size_t)(n * nf + f) * 2 + c);
                q[0] = sigma > 0 ? sigma : 1.0;
                q[1] = sigma > 0 ? cx[c] : 0.0;
                q[2] = sigma > 0 ? cy[c] : 0.0;
            }
            any |= ok;
        }
    RK(cudaMemcpyAsync(w->pc_coef, coef.data(), coef.size() * sizeof(double), cudaMemcpyHostToDevice, R.st));
    RK(cudaStreamSynchronize(R.st));
    if (std::getenv("MEPGL_REFINE_LOG") && std::getenv("MEPGL_REFINE_LOG")[0] == '1')
        for (int n = 0; n < F; ++n)
            for (int f = 0; f < nf; ++f) {
                const double *q = coef.data() + 3 * ((size_t)(n * nf + f) * 2);
                std::fprintf(stderr, "precondition image %d field %d: sigma %.4g  c_x %.4g %.4g  c_y %.4g %.4g\n", n, f,
                             q[0], q[1], q[4], q[2], q[5]);
            }
    usable = any;
    return MEPGL_OK;
}

// Legendre tables of the lattice (see k_gauge_rows), uploaded once per degree.
mepgl_status gauge_tables(Ctx &R, const GaugeBasis &B, GaugeTables &T)
{
    RefineWork *w = R.w;
    const StringHost &s = R.c->strings[0];
    const int D1 = B.deg + 1, nx = s.nx, ny = s.ny;
    if (w->gtab_deg != B.deg) {
        std::vector<double> t((size_t)2 * (nx + ny) * D1);
        auto fill = [&](int n, double *p, double *dp) {
            auto leg = [&](int i, double *P) {
                const double x = n > 1 ? (2.0 * i - (n - 1)) / (n - 1) : 0.0;
                P[0] = 1.0;
                if (B.deg >= 1) P[1] = x;
                for (int k = 1; k < B.deg; ++k) P[k + 1] = ((2 * k + 1) * x * P[k] - k * P[k - 1]) / (k + 1);
            };
            std::vector<double> Pl(D1), Pr(D1);
            for (int i = 0; i < n; ++i) {
                leg(i, p + (size_t)i * D1);
                const int il = i > 0 ? i - 1 : i, ir = i < n - 1 ? i + 1 : i;
                leg(il, Pl.data());
                leg(ir, Pr.data());
                for (int a = 0; a < D1; ++a) dp[(size_t)i * D1 + a] = (Pr[a] - Pl[a]) / (s.dx * (ir - il));
            }
        };
        double *px = t.data(), *dpx = px + (size_t)nx * D1, *py = dpx + (size_t)nx * D1, *dpy = py + (size_t)ny * D1;
        fill(nx, px, dpx);
        fill(ny, py, dpy);
        cudaFree(w->gtab);
        w->gtab = nullptr;
        RK(cudaMalloc(&w->gtab, t.size() * sizeof(double)));
        RK(cudaMemcpy(w->gtab, t.data(), t.size() * sizeof(double), cudaMemcpyHostToDevice));
        w->gtab_deg = B.deg;
    }
    T.px = w->gtab;
    T.dpx = T.px + (size_t)nx * D1;
    T.py = T.dpx + (size_t)nx * D1;
    T.dpy = T.py + (size_t)ny * D1;
    return MEPGL_OK;
}

// Orbit gradients g . J phi_m of n_img images of (x, g) into
// gd[n gstride + slot m_total + m].
mepgl_status orbit_gradients(Ctx &R, const GaugeBasis &B, Vec x, Vec g, int n_img, double *gd, int gstride, int slot)
{
    RefineWork *w = R.w;
    const StringHost &s = R.c->strings[0];
    const int D1 = B.deg + 1;
    GaugeTables T;
    mepgl_status st = gauge_tables(R, B, T);
    if (st != MEPGL_OK) return st;
    const size_t need = (size_t)n_img * s.ny * 3 * D1;
    if (w->rows_cap < need) {
        cudaFree(w->rows);
        w->rows = nullptr;
        RK(cudaMalloc(&w->rows, need * sizeof(double)));
        w->rows_cap = need;
    }
    const dim3 grid(s.ny, n_img);
    const int nc = R.c->ncomp;
    const double q1 = s.q[0], q2 = s.q[1];
    switch (D1) {
#define ROWS_CASE(d)                                                                                \
    case d: k_gauge_rows<d><<<grid, RS_THREADS, 0, R.st>>>(x, g, T, s.nx, s.ny, nc, q1, q2, w->rows); break;
        ROWS_CASE(2) ROWS_CASE(3) ROWS_CASE(4) ROWS_CASE(5) ROWS_CASE(6) ROWS_CASE(7) ROWS_CASE(8) ROWS_CASE(9)
        ROWS_CASE(10) ROWS_CASE(11) ROWS_CASE(12) ROWS_CASE(13) ROWS_CASE(14) ROWS_CASE(15) ROWS_CASE(16)
        ROWS_CASE(17)
#undef ROWS_CASE
    default: return ctx_fail(R.c, MEPGL_ERR_INVALID_ARG, "refine: gauge degree out of range");
    }
    k_gauge_combine<<<n_img, NT, 0, R.st>>>(w->rows, B, T, s.ny, gd, gstride, slot);
    R.c->launches += 2;
    RK(cudaGetLastError());
    return MEPGL_OK;
}

// Orbit gradients g . J phi_k at the 2 m F perturbed states U(+-h phi_i) x_n,
// into out[((n m + i) 2 + sign) m + k].  The perturbed states are images of
// an internal context (chunks of at most 2^25 sites in all), so each
// gradient launch covers hundreds of images instead of the F of the
// refinement.
mepgl_status wide_gauge_gradients(Ctx &R, const GaugeBasis &B, double h, std::vector<double> &out)
{
    RefineWork *w = R.w;
    mepgl_ctx *c = R.c;
    const StringHost &s = c->strings[0];
    const int m = B.m, F = R.F, total = 2 * m * F;
    const long M = s.M();
    const int cap = (int)std::max<long>(1, std::min<long>(total, (1L << 25) / M));
    if (!w->wide || w->wide_images != cap) {
        if (w->wide) mepgl_destroy(w->wide);
        w->wide = nullptr;
        mepgl_status st = twin_ctx(R, cap, &w->wide);
        if (st != MEPGL_OK) return st;
        w->wide_images = cap;
    }
    if (w->wide_gd_cap < (size_t)total * m) {
        cudaFree(w->wide_gd);
        w->wide_gd = nullptr;
        RK(cudaMalloc(&w->wide_gd, (size_t)total * m * sizeof(double)));
        w->wide_gd_cap = (size_t)total * m;
    }
    mepgl_ctx *wc = w->wide;
    const StringHost &ws = wc->strings[0];
    Vec xw{{(double *)ws.x[0][0], (double *)ws.x[0][1], (double *)ws.x[0][2]}};
    Vec gw{{(double *)ws.g[0][0], (double *)ws.g[0][1], (double *)ws.g[0][2]}};
    Launch Lw = ctx_string_launch(wc, 0);
    // float-float gradients: the gauge Hessian is a Newton model of an
    // energy-checked step, and at h = 1e-4 their ~1e-14 relative error
    // enters its central differences as ~1e-10; they run about 4x faster
    // than IEEE double on this GPU
    Lw.paired = 1;
    Lw.stream = R.st;
    const double q1 = s.q[0], q2 = s.q[1];
    const int nc = c->ncomp;
    GaugeTables T;
    mepgl_status tst = gauge_tables(R, B, T);
    if (tst != MEPGL_OK) return tst;
    for (int w0 = 0; w0 < total; w0 += cap) {
        const int nW = std::min(cap, total - w0);
        const dim3 gp((unsigned)std::min(s.ny, 1024), nW);
        k_gauge_perturb<<<gp, NT, 0, R.st>>>(R.x(), xw, B, T, F, w0, nW, h, s.nx, s.ny, nc, q1, q2);
        RK(cudaGetLastError());
        FieldPtrs fp;
        for (int f = 0; f < 3; ++f) fp.p[f] = f < w->nf ? gw.p[f] : nullptr;
        RK(launch_gradient_only(Lw, 0, fp, 0));
        mepgl_status st = orbit_gradients(R, B, xw, gw, nW, w->wide_gd + (size_t)w0 * m, m, 0);
        if (st != MEPGL_OK) return st;
        c->launches += 2;
        R.grads += (nW + F - 1) / F;      // in units of the refinement's own gradient launches
    }
    out.resize((size_t)total * m);
    RK(cudaMemcpyAsync(out.data(), w->wide_gd, out.size() * 8, cudaMemcpyDeviceToHost, R.st));
    RK(cudaStreamSynchronize(R.st));
    return MEPGL_OK;
}

// Gauge-subspace Newton step on every image with S_ACTIVE != 0.  The m x m
// Hessian (2m gradient evaluations) is rebuilt when older than `refresh`
// iterations; in between only the orbit gradient is evaluated.  The step is
// a trial: it is kept only where the energy does not rise; where it does,
// a reused Hessian is rebuilt and the step recomputed once, and a step from
// a fresh Hessian that still raises the energy is dropped.
mepgl_status gauge_step(Ctx &R, const GaugeBasis &B, double h, int refresh)
{
    RefineWork *w = R.w;
    const StringHost &s = R.c->strings[0];
    const int m = B.m, gstride = (2 * m + 1) * m, F = R.F;
    const double q1 = s.q[0], q2 = s.q[1], idx = 1.0 / s.dx;
    const int nc = R.c->ncomp, xb = R.c->xi ^ 1;
    const dim3 gg((unsigned)std::min<long>((s.M() + NT - 1) / NT, 1024), F);
    auto gdots = [&](Vec xx, Vec gv, int slot) -> mepgl_status {
        return orbit_gradients(R, B, xx, gv, F, w->gd, gstride, slot);
    };
    auto energies = [&](int xbuf, std::vector<double> &e) -> mepgl_status {
        RK(launch_energy(R.L, R.c->sc, xbuf, R.c->dscratch));
        R.c->launches += 1;
        e.resize(F);
        RK(cudaMemcpyAsync(e.data(), R.c->dscratch, F * 8, cudaMemcpyDeviceToHost, R.st));
        RK(cudaStreamSynchronize(R.st));
        return MEPGL_OK;
    };
    RK(R.grad(R.c->xi, w->g));
    mepgl_status st = gdots(R.x(), w->g, 0);
    if (st != MEPGL_OK) return st;
    std::vector<double> e0, e1;
    st = energies(R.c->xi, e0);
    if (st != MEPGL_OK) return st;
    RK(R.read_scalars());
    if (w->gauge_m != m) {
        w->gauge_h.assign(F, std::vector<double>());
        w->gauge_age.assign(F, 1 << 30);
        w->gauge_m = m;
    }
    std::vector<int> todo(F, 0);
    for (int n = 0; n < F; ++n) todo[n] = R.S(n, S_ACTIVE) != 0.0;
    std::vector<double> gd((size_t)F * gstride);
    for (int attempt = 0; attempt < 2; ++attempt) {
        bool rebuild = false, any = false;
        for (int n = 0; n < F; ++n) {
            any |= todo[n] != 0;
            if (todo[n] && (attempt > 0 || w->gauge_age[n] >= refresh)) rebuild = true;
        }
        if (!any) break;
        std::vector<double> gw;
        if (rebuild) {
            st = wide_gauge_gradients(R, B, h, gw);
            if (st != MEPGL_OK) return st;
        }
        RK(cudaMemcpyAsync(gd.data(), w->gd, gd.size() * 8, cudaMemcpyDeviceToHost, R.st));
        RK(cudaStreamSynchronize(R.st));
        std::vector<double> coef((size_t)F * RF_MAX_GB, 0.0);
        for (int n = 0; n < F; ++n) {
            if (!todo[n]) continue;
            const double *G = gd.data() + (size_t)n * gstride;
            std::vector<double> &H = w->gauge_h[n];
            if (rebuild) {
                H.assign(m * m, 0.0);
                const double *Gw = gw.data() + (size_t)n * 2 * m * m;   // [(i, sign)][k]
                for (int i = 0; i < m; ++i)
                    for (int k = 0; k < m; ++k)
                        H[k * m + i] = (Gw[(2 * i) * m + k] - Gw[(2 * i + 1) * m + k]) / (2 * h);
                for (int i = 0; i < m; ++i)
                    for (int k = 0; k < i; ++k) H[i * m + k] = H[k * m + i] = 0.5 * (H[i * m + k] + H[k * m + i]);
                w->gauge_age[n] = 0;
            }
            double *c = coef.data() + (size_t)n * RF_MAX_GB;
            if (!cholesky_solve(m, H, G, c)) {
                // not positive definite: c = -H^+ g over the positive part of the spectrum
                std::vector<double> ev, V;
                jacobi_eig(m, H, ev, V);
                std::fill(c, c + m, 0.0);
                for (int e = 0; e < m; ++e) {
                    if (!(ev[e] > 1e-12 * std::fabs(ev[m - 1]))) continue;
                    double proj = 0.0;
                    for (int i = 0; i < m; ++i) proj += V[i * m + e] * G[i];
                    for (int i = 0; i < m; ++i) c[i] -= V[i * m + e] * proj / ev[e];
                }
            }
        }
        RK(cudaMemcpyAsync(w->gcoef, coef.data(), coef.size() * 8, cudaMemcpyHostToDevice, R.st));
        k_gauge_apply<<<gg, NT, 0, R.st>>>(R.x(), R.xt(), B, w->gcoef, RF_MAX_GB, -1, 1.0, s.nx, s.ny, nc, q1, q2, idx,
                                          w->sc, -1);
        R.c->launches += 1;
        RK(cudaGetLastError());
        st = energies(xb, e1);
        if (st != MEPGL_OK) return st;
        RK(R.read_scalars());
        for (int n = 0; n < F; ++n) {
            const bool ok = todo[n] && std::isfinite(e1[n]) && e1[n] <= e0[n] + 1e-13 * std::fabs(e0[n]);
            R.S(n, S_ACCEPT) = ok ? 1.0 : 0.0;
            if (ok) {
                todo[n] = 0;
                ++w->gauge_age[n];
            } else if (todo[n] && rebuild) {
                todo[n] = 0;           // a fresh Hessian's step that raises the energy: no gauge step
            }
        }
        RK(R.write_scalars());
        LinArgs a = lin_args(R.x(), S_ACCEPT);
        add_term(a, R.xt(), 1.0);
        RK(R.lin(a));
    }
    return MEPGL_OK;
}

// Lanczos on the saddle images (S_ACTIVE gates them): `steps` steps from
// w->v1 with full reorthogonalisation (twice); v1 <- the lowest Ritz vector,
// normalised; lam <- its Ritz value.
mepgl_status lanczos(Ctx &R, int steps, std::vector<double> &lam)
{
    RefineWork *w = R.w;
    const long FM2 = (long)R.F * R.M2;
    const int F = R.F;
    RK(R.dots({{w->v1, w->v1}}, OP_UNIT));
    LinArgs a = lin_args(w->lz[0], S_ACTIVE);
    add_term(a, w->v1, 1.0, S_INVB);
    RK(R.lin(a));
    std::vector<double> alpha((size_t)F * steps, 0.0), beta((size_t)F * steps, 0.0);
    std::vector<double> hd((size_t)F * RF_DOTS);
    int done = 0;
    for (int j = 0; j < steps; ++j) {
        mepgl_status st = hess_vec(R, w->lz[j], w->lz[j + 1], false);
        if (st != MEPGL_OK) return st;
        for (int pass = 0; pass < 2; ++pass) {
            k_dots_lz<<<R.vgrid(), NT, 0, R.st>>>(w->lz[j + 1], w->lz[0].p[0], w->vs, j + 1, R.M2, w->nf, FM2,
                                                 w->part, w->nb);
            RK(cudaGetLastError());
            RK(R.sums(j + 1, OP_NONE));
            if (pass == 0) {
                RK(cudaMemcpyAsync(hd.data(), w->dots, hd.size() * 8, cudaMemcpyDeviceToHost, R.st));
                RK(cudaStreamSynchronize(R.st));
                for (int n = 0; n < F; ++n) alpha[(size_t)n * steps + j] = hd[(size_t)n * RF_DOTS + j];
            }
            k_sub_lz<<<R.vgrid(), NT, 0, R.st>>>(w->lz[j + 1], 1.0, w->lz[0].p[0], w->vs, j + 1, R.M2, w->nf, FM2,
                                                w->dots, RF_DOTS, w->sc, S_ACTIVE, w->nb);
            R.c->launches += 2;
            RK(cudaGetLastError());
        }
        RK(R.dots({{w->lz[j + 1], w->lz[j + 1]}}, OP_UNIT));
        RK(R.read_scalars());
        for (int n = 0; n < F; ++n) {
            const double ib = R.S(n, S_INVB);
            beta[(size_t)n * steps + j] = ib > 0 ? 1.0 / ib : 0.0;
        }
        LinArgs b = lin_args(w->lz[j + 1], S_ACTIVE);
        add_term(b, w->lz[j + 1], 1.0, S_INVB);
        RK(R.lin(b));
        done = j + 1;
    }
    // Ritz pair of the lowest eigenvalue of T per image
    std::vector<double> coef((size_t)F * (RF_MAX_LZ + 1), 0.0);
    RK(R.read_scalars());
    lam.assign(F, 0.0);
    for (int n = 0; n < F; ++n) {
        if (R.S(n, S_ACTIVE) == 0.0) continue;
        std::vector<double> T(done * done, 0.0), ev, V;
        for (int j = 0; j < done; ++j) {
            T[j * done + j] = alpha[(size_t)n * steps + j];
            if (j + 1 < done) T[j * done + j + 1] = T[(j + 1) * done + j] = beta[(size_t)n * steps + j];
        }
        jacobi_eig(done, T, ev, V);
        lam[n] = ev[0];
        for (int j = 0; j < done; ++j) coef[(size_t)n * (RF_MAX_LZ + 1) + j] = -V[j * done + 0];
    }
    RK(cudaMemcpyAsync(w->coef, coef.data(), coef.size() * 8, cudaMemcpyHostToDevice, R.st));
    // v1 = 0 * v1 - sum_j (-y_j) lz_j
    k_sub_lz<<<R.vgrid(), NT, 0, R.st>>>(w->v1, 0.0, w->lz[0].p[0], w->vs, done, R.M2, w->nf, FM2, w->coef,
                                        RF_MAX_LZ + 1, w->sc, S_ACTIVE, w->nb);
    R.c->launches += 1;
    RK(cudaGetLastError());
    RK(R.dots({{w->v1, w->v1}}, OP_UNIT));
    LinArgs b = lin_args(w->v1, S_ACTIVE);
    add_term(b, w->v1, 1.0, S_INVB);
    RK(R.lin(b));
    return MEPGL_OK;
}

// One CG iteration on the images with S_ACTIVE != 0 (device scalars only,
// so that a run of iterations can be captured as one CUDA graph).  With
// `pc` the iteration is preconditioned (z = P M^-1 r; S_RR holds r . z) and
// beta is the flexible form r_new . (z_new - z_old) / (r_old . z_old), which
// tolerates the FP32 rounding of M^-1; iteration k writes z[k & 1].
mepgl_status cg_iteration(Ctx &R, bool pc, int k)
{
    RefineWork *w = R.w;
    mepgl_status st = hess_vec(R, w->p, w->y, true);
    if (st != MEPGL_OK) return st;
    // y -= (v1 . y) v1, then p . y
    RK(R.dots({{w->v1, w->y}}, OP_STORE_V1Y));
    LinArgs a = lin_args(w->y, S_ACTIVE);
    add_term(a, w->y, 1.0);
    add_term(a, w->v1, -1.0, S_V1Y);
    a.dw = w->p;
    a.dot_k = 1;
    a.dot_slot = 0;
    a.op = OP_ALPHA;
    RK(R.lin(a));
    a = lin_args(w->s, S_ACTIVE);
    add_term(a, w->s, 1.0);
    add_term(a, w->p, 1.0, S_ALPHA);
    RK(R.lin(a));
    a = lin_args(w->r, S_ACTIVE);
    add_term(a, w->r, 1.0);
    add_term(a, w->y, -1.0, S_ALPHA);
    if (pc) {
        RK(R.lin(a));
        st = pc_apply(R, w->r, w->z[k & 1]);
        if (st != MEPGL_OK) return st;
        RK(R.dots({{w->r, w->z[k & 1]}, {w->r, w->r}, {w->r, w->z[(k & 1) ^ 1]}}, OP_PBETA));
    } else {
        a.dw = w->r;
        a.dot_k = 1;
        a.dot_slot = 0;
        a.op = OP_BETA;
        RK(R.lin(a));
    }
    a = lin_args(w->p, S_ACTIVE);
    add_term(a, pc ? w->z[k & 1] : w->r, 1.0);
    add_term(a, w->p, 1.0, S_BETA);
    RK(R.lin(a));
    return MEPGL_OK;
}

constexpr int CG_GRAPH_ITERS = 8;     // CG iterations per graph replay
static_assert(CG_GRAPH_ITERS % 2 == 0, "the preconditioned iterations alternate two z buffers");

// Projected shifted CG for the images with S_ACTIVE != 0 at entry:
// (H + mu) s = -(g - g1 v1), s orthogonal to v1 (v1 = 0 for minima),
// preconditioned when `pc`.  The iterations run as replays of a captured
// graph of CG_GRAPH_ITERS iterations (images that converge inside a replay
// stop updating); if the preconditioned iterations cannot be captured they
// are launched directly, the same kernels in the same order.
mepgl_status cg_solve(Ctx &R, int max_it, bool pc)
{
    RefineWork *w = R.w;
    LinArgs a = lin_args(w->r, S_ACTIVE);
    add_term(a, w->g, -1.0);
    add_term(a, w->v1, 1.0, S_G1);
    if (pc) {
        RK(R.lin(a));
        mepgl_status st = pc_apply(R, w->r, w->z[1]);   // the "previous" z of iteration 0
        if (st != MEPGL_OK) return st;
        RK(R.dots({{w->r, w->z[1]}, {w->r, w->r}}, OP_PCGINIT));
    } else {
        a.dw = w->r;   // |r|^2
        a.dot_k = 1;
        a.dot_slot = 0;
        a.op = OP_CGINIT;
        RK(R.lin(a));
    }
    a = lin_args(w->p, S_ACTIVE);
    add_term(a, pc ? w->z[1] : w->r, 1.0);
    RK(R.lin(a));
    a = lin_args(w->s, S_ACTIVE);
    add_term(a, w->s, 0.0);
    RK(R.lin(a));
    const int gi = pc ? 1 : 0;
    cudaGraphExec_t &ex = w->cg_graph[gi][R.c->xi & 1];
    const bool direct = pc && w->pc_capture_failed;
    if (!ex && !direct) {
        const int64_t l0 = R.c->launches, g0 = R.grads;
        RK(cudaStreamBeginCapture(R.st, cudaStreamCaptureModeThreadLocal));
        mepgl_status st = MEPGL_OK;
        for (int k = 0; k < CG_GRAPH_ITERS && st == MEPGL_OK; ++k) st = cg_iteration(R, pc, k);
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(R.st, &g);
        cudaGraphExec_t made = nullptr;
        cudaError_t ei = e;
        if (st == MEPGL_OK && e == cudaSuccess) ei = cudaGraphInstantiate(&made, g, 0);
        if (g) cudaGraphDestroy(g);
        R.c->launches = l0;
        R.grads = g0;
        if (st != MEPGL_OK || e != cudaSuccess || ei != cudaSuccess) {
            if (!pc) {
                if (st != MEPGL_OK) return st;
                RK(e);
                RK(ei);
            }
            // the transforms did not capture: clear the error state, launch directly
            cudaGetLastError();
            R.c->err.clear();
            w->pc_capture_failed = true;
        } else {
            ex = made;
            w->graph_launches[gi] = R.c->launches - l0;
            w->graph_grads[gi] = R.grads - g0;
        }
    }
    if (!ex && !w->pc_capture_failed) return ctx_fail(R.c, MEPGL_ERR_CUDA, "refine: CG graph missing");
    for (int it = 0; it < max_it; it += CG_GRAPH_ITERS) {
        if (ex) {
            RK(cudaGraphLaunch(ex, R.st));
            R.c->launches += w->graph_launches[gi];
            R.grads += w->graph_grads[gi];
        } else {
            for (int k = 0; k < CG_GRAPH_ITERS; ++k) {
                mepgl_status st = cg_iteration(R, pc, k);
                if (st != MEPGL_OK) return st;
            }
        }
        if ((it / CG_GRAPH_ITERS) % 2 == 1 || it + CG_GRAPH_ITERS >= max_it) {
            RK(R.read_scalars());
            bool any = false;
            for (int n = 0; n < R.F; ++n) any |= R.S(n, S_ACTIVE) != 0.0;
            if (!any) break;
        }
    }
    return MEPGL_OK;
}

mepgl_status alloc_work(mepgl_ctx *c)
{
    const StringHost &s = c->strings[0];
    RefineWork *w = c->refine;
    if (w && w->F == s.F && w->M == s.M() && w->nf == 1 + c->ncomp) return MEPGL_OK;
    refine_free(w);
    w = c->refine = new RefineWork();
    w->F = s.F;
    w->M = s.M();
    w->nx = s.nx;
    w->ny = s.ny;
    w->nf = 1 + c->ncomp;
    // about four 16-byte pairs per thread and array
    w->nb = (int)std::max<long>(1, std::min<long>(RF_NB, (2 * w->M + 8L * NT - 1) / (8L * NT)));
    w->vs = (size_t)w->nf * w->F * 2 * w->M;
    const int nvec = 11 + RF_MAX_LZ + 1;
    cudaError_t e = cudaMalloc(&w->block, nvec * w->vs * sizeof(double));
    if (e == cudaSuccess) e = cudaMemsetAsync(w->block, 0, nvec * w->vs * sizeof(double), c->stream);
    if (e != cudaSuccess) return ctx_fail(c, MEPGL_ERR_CUDA, std::string("refine workspace: ") + cudaGetErrorString(e));
    auto vec = [&](int k) {
        Vec v;
        for (int f = 0; f < 3; ++f)
            v.p[f] = f < w->nf ? w->block + k * w->vs + (size_t)f * w->F * 2 * w->M : nullptr;
        return v;
    };
    // lz vectors first and contiguous (the multi-dot kernels index them by stride)
    for (int k = 0; k <= RF_MAX_LZ; ++k) w->lz[k] = vec(k);
    int k = RF_MAX_LZ + 1;
    for (Vec *v : {&w->g, &w->v1, &w->p, &w->r, &w->y, &w->s, &w->gp, &w->gm, &w->z[0], &w->z[1], &w->pmask})
        *v = vec(k++);
    const size_t parts = (size_t)w->F * std::max(RF_DOTS, RF_MAX_GB) * w->nb;
    e = cudaMalloc(&w->part, parts * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&w->ticket, (size_t)w->F * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemsetAsync(w->ticket, 0, (size_t)w->F * sizeof(unsigned), c->stream);
    if (e == cudaSuccess) e = cudaMalloc(&w->dots, (size_t)w->F * RF_DOTS * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&w->sc, (size_t)w->F * NSC * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&w->coef, (size_t)w->F * (RF_MAX_LZ + 1) * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&w->gcoef, (size_t)w->F * RF_MAX_GB * sizeof(double));
    if (e == cudaSuccess)
        e = cudaMalloc(&w->gd, (size_t)w->F * (2 * RF_MAX_GB + 1) * RF_MAX_GB * sizeof(double));
    if (e == cudaSuccess) e = cudaMemsetAsync(w->sc, 0, (size_t)w->F * NSC * sizeof(double), c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(w->coef, 0, (size_t)w->F * (RF_MAX_LZ + 1) * sizeof(double), c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(w->gcoef, 0, (size_t)w->F * RF_MAX_GB * sizeof(double), c->stream);
    if (e != cudaSuccess) return ctx_fail(c, MEPGL_ERR_CUDA, std::string("refine workspace: ") + cudaGetErrorString(e));
    w->lam1.assign(w->F, 0.0);
    w->mu.assign(w->F, 0.0);
    w->has_mode.assign(w->F, 0);
    w->fresh.assign(w->F, 0);
    return MEPGL_OK;
}

}  // namespace
}  // namespace mepgl

using namespace mepgl;

extern "C" {

void mepgl_default_refine_options(mepgl_refine_options *o)
{
    if (!o) return;
    memset(o, 0, sizeof(*o));
    o->g_tol = 1e-8;
    o->max_newton = 40;
    o->max_cg = 3000;
    o->lanczos_steps = 12;
    o->gauge_degree = -1;
    o->mu0 = 1e-3;
    o->cg_eta = 0.1;
    o->max_retries = 8;
    o->gauge_refresh = 0;
    o->precondition = 1;
    o->forcing = 0;
}

mepgl_status mepgl_refine_stationary(mepgl_ctx *c, const int32_t *kind, const void *mode_a, const void *mode_psi_1,
                                     const void *mode_psi_2, int memory, const mepgl_refine_options *opt_in,
                                     mepgl_refine_report *report)
{
    if (!c || !kind) return MEPGL_ERR_INVALID_ARG;
    if (c->strings.size() != 1)
        return ctx_fail(c, MEPGL_ERR_UNSUPPORTED, "mepgl_refine_stationary: single-string contexts only");
    if (c->precision != MEPGL_FP64)
        return ctx_fail(c, MEPGL_ERR_UNSUPPORTED, "mepgl_refine_stationary: the refinement runs on FP64 contexts");
    if (c->opt.discretization != MEPGL_DISC_REFERENCE)
        return ctx_fail(c, MEPGL_ERR_UNSUPPORTED, "mepgl_refine_stationary: reference discretisation only");
    mepgl_refine_options opt;
    mepgl_default_refine_options(&opt);
    if (opt_in) opt = *opt_in;
    if (opt.lanczos_steps < 2 || opt.lanczos_steps > RF_MAX_LZ || opt.gauge_degree < -1 ||
        opt.gauge_degree > RF_MAX_DEG || opt.max_newton < 0 || opt.max_cg < 1 || !(opt.g_tol >= 0) ||
        !(opt.mu0 > 0) || !(opt.cg_eta > 0 && opt.cg_eta < 1) || opt.max_retries < 0 || opt.gauge_refresh < 0 ||
        opt.precondition < 0 || opt.precondition > 1 || opt.forcing < 0 || opt.forcing > 1)
        return ctx_fail(c, MEPGL_ERR_INVALID_ARG, "mepgl_refine_stationary: option out of range");
    const int F = c->strings[0].F;
    for (int n = 0; n < F; ++n)
        if (kind[n] != MEPGL_STATIONARY_MINIMUM && kind[n] != MEPGL_STATIONARY_SADDLE && kind[n] != MEPGL_STATIONARY_SKIP)
            return ctx_fail(c, MEPGL_ERR_INVALID_ARG, "mepgl_refine_stationary: bad image kind");
    mepgl_status st = ctx_flush(c);
    if (st != MEPGL_OK) return st;
    st = alloc_work(c);
    if (st != MEPGL_OK) return st;
    RefineWork *w = c->refine;
    const bool new_modes = mode_a || mode_psi_1 || mode_psi_2;
    for (int n = 0; n < F; ++n)
        if (kind[n] == MEPGL_STATIONARY_SADDLE && !new_modes && !w->has_mode[n])
            return ctx_fail(c, MEPGL_ERR_INVALID_ARG,
                            "mepgl_refine_stationary: a saddle image needs an initial direction on its first call");
    if (new_modes || w->state_version != c->state_version)
        for (auto &a : w->gauge_age) a = 1 << 30;
    Ctx R{c, w, ctx_string_launch(c, 0), F, 2 * w->M, c->stream};
    R.L.paired = 0;     // IEEE double gradients
    if (!w->hvc) {      // before any capture: creating it allocates
        st = twin_ctx(R, 2 * F, &w->hvc);
        if (st != MEPGL_OK) return st;
    }
    const StringHost &s = c->strings[0];
    // initial min modes: the caller's directions (then the history restarts)
    if (new_modes) {
        const void *src[3] = {mode_a, mode_psi_1, mode_psi_2};
        const size_t bytes = (size_t)F * s.M() * 2 * sizeof(double);
        for (int f = 0; f < w->nf; ++f) {
            if (src[f])
                RK(cudaMemcpyAsync(w->v1.p[f], src[f], bytes,
                                   memory == MEPGL_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, R.st));
            else
                RK(cudaMemsetAsync(w->v1.p[f], 0, bytes, R.st));
        }
        for (int n = 0; n < F; ++n) {
            w->has_mode[n] = kind[n] == MEPGL_STATIONARY_SADDLE;
            w->fresh[n] = 1;
            w->mu[n] = opt.mu0;
        }
    }
    for (int n = 0; n < F; ++n)
        if (w->mu[n] <= 0) w->mu[n] = opt.mu0;
    // minima and skipped images carry a zero mode (the projections vanish)
    {
        RK(R.read_scalars());
        for (int n = 0; n < F; ++n) R.S(n, S_ACTIVE) = kind[n] == MEPGL_STATIONARY_SADDLE ? 0.0 : 1.0;
        RK(R.write_scalars());
        LinArgs a = lin_args(w->v1, S_ACTIVE);
        add_term(a, w->v1, 0.0);
        RK(R.lin(a));
    }
    GaugeBasis B;
    memset(&B, 0, sizeof(B));
    // auto: one degree per 8 lattice sites of the longer side, 4 to 16
    const int nmax = std::max(s.nx, s.ny);
    // (and at most half the shorter side, where a higher degree has too few
    // rows or columns to be a well-posed basis)
    const int nmin = std::min(s.nx, s.ny);
    B.deg = opt.gauge_degree >= 0 ? opt.gauge_degree
                                  : std::min(std::min(RF_MAX_DEG, std::max(4, nmax / 8)), std::max(1, nmin / 2));
    if (c->thin_film) B.deg = 0;
    for (int d = 1; d <= B.deg; ++d)
        for (int k = 0; k <= d; ++k) {
            B.a[B.m] = (unsigned char)(d - k);
            B.b[B.m] = (unsigned char)k;
            ++B.m;
        }
    const double dof = (double)w->nf * 2 * s.M();
    std::vector<int> done(F, 0), newton_it(F, 0), cg_it(F, 0);
    std::vector<double> gnorm(F, 0.0), energy(F, 0.0);
    for (int n = 0; n < F; ++n) done[n] = kind[n] == MEPGL_STATIONARY_SKIP;
    auto set_active = [&](const std::vector<int> &on) -> mepgl_status {
        RK(R.read_scalars());
        for (int n = 0; n < F; ++n) {
            R.S(n, S_ACTIVE) = on[n] ? 1.0 : 0.0;
            R.S(n, S_DELTA) = 1e-6 * std::sqrt(dof);
            R.S(n, S_MU) = w->mu[n];
            R.S(n, S_ONE) = 1.0;
        }
        RK(R.write_scalars());
        return MEPGL_OK;
    };
    auto measure = [&]() -> mepgl_status {    // energies and |g| of x
        RK(R.grad(c->xi, w->g));
        RK(R.dots({{w->g, w->g}}, OP_NONE));
        std::vector<double> hd((size_t)F * RF_DOTS);
        RK(cudaMemcpyAsync(hd.data(), w->dots, hd.size() * 8, cudaMemcpyDeviceToHost, R.st));
        RK(launch_energy(R.L, c->sc, c->xi, c->dscratch));
        c->launches += 1;
        RK(cudaMemcpyAsync(energy.data(), c->dscratch, F * 8, cudaMemcpyDeviceToHost, R.st));
        RK(cudaStreamSynchronize(R.st));
        for (int n = 0; n < F; ++n) gnorm[n] = std::sqrt(hd[(size_t)n * RF_DOTS]);
        return MEPGL_OK;
    };
    st = measure();
    if (st != MEPGL_OK) return st;
    // preconditioner model at the starting point (images still to refine)
    bool pc = false;
    if (opt.precondition) {
        std::vector<int> todo(F);
        bool any = false;
        for (int n = 0; n < F; ++n) {
            todo[n] = !done[n] && gnorm[n] > opt.g_tol;
            any |= todo[n] != 0;
        }
        if (any && opt.max_newton > 0) {
            st = set_active(todo);
            if (st == MEPGL_OK) st = pc_setup(R, pc);
            if (st != MEPGL_OK) return st;
        }
    }
    // MEPGL_REFINE_LOG=1: one line per image and Newton iteration on stderr
    const char *env = std::getenv("MEPGL_REFINE_LOG");
    const bool log = env && env[0] == '1';
    for (int it = 0; it < opt.max_newton; ++it) {
        double t_gauge = 0.0;
        std::vector<int> act(F);
        bool any = false;
        for (int n = 0; n < F; ++n) {
            if (!done[n] && gnorm[n] <= opt.g_tol) done[n] = 1;
            act[n] = !done[n];
            any |= act[n] != 0;
        }
        if (!any) break;
        // 1. gauge-subspace step
        if (B.m > 0) {
            st = set_active(act);
            const auto tg0 = std::chrono::steady_clock::now();
            // auto: small bases are cheap to rebuild and a fresh Hessian saves
            // iterations; large ones (2m gradients each) are reused
            const int refresh = opt.gauge_refresh > 0 ? opt.gauge_refresh : (B.m <= 64 ? 1 : 4);
            if (st == MEPGL_OK) st = gauge_step(R, B, 1e-4, refresh);
            if (st != MEPGL_OK) return st;
            t_gauge = std::chrono::duration<double>(std::chrono::steady_clock::now() - tg0).count();
        }
        // 2. min modes of the saddle images
        const auto tl0 = std::chrono::steady_clock::now();
        std::vector<int> sad(F);
        bool any_sad = false;
        for (int n = 0; n < F; ++n) {
            sad[n] = act[n] && kind[n] == MEPGL_STATIONARY_SADDLE;
            any_sad |= sad[n] != 0;
        }
        if (any_sad) {
            st = set_active(sad);
            if (st != MEPGL_OK) return st;
            std::vector<double> lam;
            int steps = opt.lanczos_steps;
            for (int n = 0; n < F; ++n)
                if (sad[n] && w->fresh[n]) steps = std::max(steps, std::min(RF_MAX_LZ, 30));
            st = lanczos(R, steps, lam);
            if (st != MEPGL_OK) return st;
            for (int n = 0; n < F; ++n)
                if (sad[n]) {
                    w->lam1[n] = lam[n];
                    w->fresh[n] = 0;
                }
        }
        const double t_lanczos = std::chrono::duration<double>(std::chrono::steady_clock::now() - tl0).count();
        // 3. gradient, g1 = v1 . g, uphill step along v1, shifted CG in the complement
        st = set_active(act);
        if (st != MEPGL_OK) return st;
        RK(R.grad(c->xi, w->g));
        RK(R.dots({{w->v1, w->g}, {w->g, w->g}}, OP_STORE_G1));
        std::vector<double> hd((size_t)F * RF_DOTS);
        RK(cudaMemcpyAsync(hd.data(), w->dots, hd.size() * 8, cudaMemcpyDeviceToHost, R.st));
        RK(R.read_scalars());
        std::vector<double> g2(F);
        for (int n = 0; n < F; ++n) {
            g2[n] = hd[(size_t)n * RF_DOTS + 1];
            const double g1 = R.S(n, S_G1);
            double p1 = 0.0;
            if (kind[n] == MEPGL_STATIONARY_SADDLE && act[n]) {
                p1 = g1 / std::max(std::fabs(w->lam1[n]), 1e-8);
                const double cap = 1.0;
                if (std::fabs(p1) > cap) p1 = p1 > 0 ? cap : -cap;
            }
            R.S(n, S_P1) = p1;
        }
        RK(R.write_scalars());
        std::vector<int> pending = act, cg_before = cg_it, tries_used(F, 0);
        double cg_seconds = 0.0;
        std::vector<int> neg_hits(F, 0);
        const auto tn0 = std::chrono::steady_clock::now();
        for (int tries = 0; tries <= opt.max_retries; ++tries) {
            for (int n = 0; n < F; ++n) tries_used[n] += pending[n];
            st = set_active(pending);
            if (st != MEPGL_OK) return st;
            RK(R.read_scalars());
            // forcing term: cg_eta (linear convergence at about that rate per
            // Newton step), or sqrt|g| capped at cg_eta (superlinear, tighter
            // solves); never tighter than reaching g_tol needs
            for (int n = 0; n < F; ++n) {
                const double gn = std::sqrt(g2[n]);
                const double need = gn > 0 ? 0.5 * opt.g_tol / gn : 0.0;
                R.S(n, S_ETA) = opt.forcing == 1 ? std::min(opt.cg_eta, std::max(std::sqrt(gn), need))
                                                 : std::min(0.5, std::max(opt.cg_eta, need));
            }
            RK(R.write_scalars());
            const auto tc0 = std::chrono::steady_clock::now();
            st = cg_solve(R, opt.max_cg, pc);
            if (st != MEPGL_OK) return st;
            RK(R.read_scalars());
            cg_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - tc0).count();
            for (int n = 0; n < F; ++n)
                if (pending[n]) {
                    cg_it[n] += (int)R.S(n, S_IT);
                    neg_hits[n] += R.S(n, S_NEG) != 0.0;
                }
            // trial x + s + p1 v1 (pending images), merit |g(trial)|^2
            for (int n = 0; n < F; ++n) R.S(n, S_ACTIVE) = pending[n] ? 1.0 : 0.0;
            RK(R.write_scalars());
            LinArgs a = lin_args(R.xt());
            add_term(a, R.x(), 1.0);
            add_term(a, w->s, 1.0, S_ACTIVE);
            add_term(a, w->v1, 1.0, S_P1, S_ACTIVE);
            RK(R.lin(a));
            RK(R.grad(c->xi ^ 1, w->gp));
            RK(R.dots({{w->gp, w->gp}}, OP_NONE));
            RK(cudaMemcpyAsync(hd.data(), w->dots, hd.size() * 8, cudaMemcpyDeviceToHost, R.st));
            RK(cudaStreamSynchronize(R.st));
            bool again = false;
            for (int n = 0; n < F; ++n) {
                R.S(n, S_ACCEPT) = 0.0;
                if (!pending[n]) continue;
                const double gt2 = hd[(size_t)n * RF_DOTS];
                if (std::isfinite(gt2) && gt2 < g2[n] * (1 - 1e-4)) {
                    R.S(n, S_ACCEPT) = 1.0;
                    w->mu[n] = std::max(w->mu[n] / 4, 1e-12);
                    pending[n] = 0;
                } else {
                    // bounded: from a seed where no step lowers |g|^2 (far from any
                    // stationary point) the shift would otherwise grow without end
                    w->mu[n] = std::min(w->mu[n] * 4, RF_MU_MAX);
                    again = true;
                }
            }
            RK(R.write_scalars());
            a = lin_args(R.x(), S_ACCEPT);
            add_term(a, R.xt(), 1.0);
            RK(R.lin(a));
            if (!again) break;
        }
        for (int n = 0; n < F; ++n)
            if (act[n]) ++newton_it[n];
        st = measure();
        if (st != MEPGL_OK) return st;
        if (log)
            for (int n = 0; n < F; ++n)
                if (act[n])
                    std::fprintf(stderr,
                                 "refine image %d (%s): |g| %.3e -> %.3e  E %.13f  mu %.2e  tries %d  cg %d  "
                                 "lambda1 %.5f  grads %lld  newton-step %.3f s of which CG %.3f s  gauge %.3f s  "
                                 "lanczos %.3f s  cg-negative %d  pc %d%s\n",
                                 n, kind[n] == MEPGL_STATIONARY_SADDLE ? "saddle" : "minimum", std::sqrt(g2[n]),
                                 gnorm[n], energy[n], w->mu[n], tries_used[n], cg_it[n] - cg_before[n], w->lam1[n],
                                 (long long)R.grads,
                                 std::chrono::duration<double>(std::chrono::steady_clock::now() - tn0).count(),
                                 cg_seconds, t_gauge, t_lanczos, neg_hits[n], pc ? 1 : 0,
                                 pc && w->pc_capture_failed ? " (direct launches)" : "");
    }
    w->state_version = c->state_version;
    if (report)
        for (int n = 0; n < F; ++n) {
            mepgl_refine_report &r = report[n];
            r.energy = energy[n];
            r.g_norm = gnorm[n];
            r.min_curvature = kind[n] == MEPGL_STATIONARY_SADDLE ? w->lam1[n] : 0.0;
            r.mu = w->mu[n];
            r.newton_iterations = newton_it[n];
            r.cg_iterations = cg_it[n];
            r.gradient_evaluations = (int32_t)std::min<int64_t>(R.grads, INT32_MAX);
            r.converged = kind[n] == MEPGL_STATIONARY_SKIP || gnorm[n] <= opt.g_tol;
            r.preconditioned = pc ? 1 : 0;
        }
    return ctx_check_device_status(c);
}

}  // extern "C"
