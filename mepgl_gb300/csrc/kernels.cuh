// kernels.cuh -- host-side launch interface of the lattice kernels.
#pragma once

#include "common.cuh"

namespace mepgl {

constexpr int LS_GRID = 2001;         // line-search grid points x_0 .. x_2000

// Rows per lattice tile for a precision (0 float, 1 double); tiles are TX wide.
int tile_rows(int precision);
// Kernel launches per NLCG step and launch group (2, or 3 with the split direction pass).
int nlcg_step_launches();
// Kernel names of the two NLCG passes for a precision (0 float, 1 double) and arithmetic.
void nlcg_pass_kernels(int precision, int paired, const char **grad, const char **dir_poly);
// Copy the neighbour-code weight tables to constant memory (idempotent).
cudaError_t upload_mask_tables();

struct Launch {
    const Batch *batch;          // host copy; passed by value to the kernels
    const TileRef *tiles;        // device
    int tile0;                   // global index of tiles[0] (tiles are in (string, image, row, column) order)
    int n_tiles;
    int grid;                    // blocks launched (grid-stride over tiles)
    int precision;               // 0 float, 1 double
    int paired;                  // 1: NLCG passes in float-float arithmetic on double fields
    int ncomp;                   // 1 or 2 (uniform over the strings of a context)
    cudaStream_t stream;
};

struct StepFlags {
    int xin, xout;     // x buffers read / written by the gradient pass
    int gcur, gprev;   // gradient slots
    int din, dout;     // direction buffers read / written by the direction pass
    int use_cg, maxwell, thin_film_any;
    int poly_compat, ls_exact;
};

// True when this build has fused FP32 NLCG steps (one persistent launch per call).
bool nlcg_fused(int precision);
// Fused steps are used for batches of at most fuse_waves() x strip_pass_slots()
// tiles: resident blocks of the FP32 pass kernels on the current device.
int fuse_waves();
int strip_pass_slots(int ncomp);
// `steps` NLCG steps (iterations it0, it0 + 1, ...; step 0 with the buffers
// of f0) of the launch's tiles in one persistent launch; queue (one counter)
// and stage (one per global image, n_stage) are reset on the stream first.
// first_item > 0 starts the queue there (the wait self-test); each per-image
// wait polls at most max_polls times.
constexpr unsigned STAGE_WAIT_POLLS = 1u << 22;   // about 100 ns to 1 us per poll
cudaError_t launch_nlcg_fused(const Launch &L, const Scalars &sc, const StepFlags &f0, int it0, int steps,
                              unsigned long long *queue, unsigned *stage, int n_stage,
                              unsigned long long first_item = 0, unsigned max_polls = STAGE_WAIT_POLLS);
// Pass 1: x <- x + alpha_pend d (into x[xout]); g = dF/dx; |g|^2, g.(g - g_prev);
// the last tile of each image sets beta.
cudaError_t launch_grad(const Launch &L, const Scalars &sc, const StepFlags &f);
// Pass 2: d <- -g + beta d (into d[dout]); quartic of F(x + a d); the last
// tile of each image runs the line search and sets alpha, alpha_pend.
cudaError_t launch_dir_poly(const Launch &L, const Scalars &sc, const StepFlags &f);
// x[xbuf] += alpha_pend d[dbuf]; alpha_pend = 0.
// Paired FP64: whether the NLCG passes keep x as float-float pairs, and the
// in-place conversion of `pairs` complex values of x to (1) or from (0) them.
bool x_pairs();
cudaError_t launch_x_format(void *x, long pairs, int to_pairs, cudaStream_t st);
cudaError_t launch_apply_update(const Launch &L, const Scalars &sc, const StringDesc *host_strings, int n_strings,
                                int xbuf, int dbuf);
// Energy of x[xbuf] into sc.fenergy_out (per image).
cudaError_t launch_energy(const Launch &L, const Scalars &sc, int xbuf, double *out);
cudaError_t launch_param_adjoint(const Launch &L, const Scalars &sc, int xbuf, double *out);
// Gradient of x[xbuf] into the three arrays of `out` (single string).
struct FieldPtrs { void *p[3]; };
// Gradient of every image into `out` (FP64 launches with L.paired: float-float arithmetic).
cudaError_t launch_gradient_only(const Launch &L, int xbuf, FieldPtrs out, int maxwell);
// B, J of x[xbuf] written to per-string arrays (b: F*M reals, j: F*M pairs).
cudaError_t launch_jb(const Launch &L, const Scalars &sc, int xbuf, void *const *b, void *const (*j)[2]);

// Arc length of one string over nf per-image arrays of `width` reals per site
// (reals of the context precision).  Result: s[0..F) (device doubles), using
// part (>= tiles_per_image * F doubles) as scratch.  A string of zero or
// non-finite length sets *bad (device int) and gets the uniform s = n/(F-1).
cudaError_t launch_arc_length(int precision, const void *const *fields, const int *width, int nf, long sites, int F,
                              double *part, double *s, int *bad, cudaStream_t st);
// Device status flags (Scalars::status): [0] a stage wait of the fused NLCG
// launch ran out; [1] count of non-finite per-image scalars after NLCG steps,
// [2] the first such image + 1; [3] a string of zero or non-finite arc length.
constexpr int STATUS_WAIT = 0, STATUS_NONFINITE = 1, STATUS_NONFINITE_IMAGE = 2, STATUS_ARC = 3;
// Checks energy and |g|^2 (slot 0 or 1) of n_images images (see STATUS_NONFINITE).
cudaError_t launch_check_scalars(const Scalars &sc, int n_images, int slot, cudaStream_t st);
// Initial-guess parameters of launch_generate (see mepgl_guess).
struct GuessParams {
    double x0, y0, dx, psi_abs_1, psi_abs_2, noise, b_z;
    int gauge, profile;
    unsigned long long seed;
};
// Fill a, psi_1[, psi_2] (F images of nx*ny pairs) with the builder's initial
// guess; comp / sc: int32 domains on the device; tracks: n_tracks*F*4 doubles
// (x, y, winding, component) on the device.
cudaError_t launch_generate(int precision, void *a, void *p1, void *p2, int nx, int ny, int F, int ncomp,
                            const int32_t *comp, const int32_t *sc, const double *tracks, int n_tracks,
                            const GuessParams &g, cudaStream_t st);
// out[n] = dx2 * sum of b over image n (M reals per image, context precision).
cudaError_t launch_flux(int precision, const void *b, long M, int F, double dx2, double *out, cudaStream_t st);
// out[n] = winding sum of psi (pairs) of image n around the rectangle `inset`
// sites inside the lattice edge (requires nx, ny > 2 inset + 1).
cudaError_t launch_winding(int precision, const void *psi, int nx, int ny, int F, int inset, double *out,
                           cudaStream_t st);
// Plan of a redistribution from F to F_new images on the arc length s:
// segment k and weight w per output image; for cubic also h and the
// factorised spline matrix (dl, d, du, du2, ipiv) -- all in `plan`.
struct RedistPlan {
    int *k;          // [F_new]
    double *w;       // [F_new]
    double *h;       // [F + 1]
    double *dl, *d, *du, *du2;   // [F]
    int *ipiv;       // [F]
    int *status;
    // cubic: 1 / h [F], 1 / d [F], per output image {w, 1 - w, h_k^2 (w^3 - w),
    // h_k^2 (wm^3 - wm)} [4 F_new], the end conditions' factors [8]
    double *aux;
};
// doubles of RedistPlan::aux for a plan of capacity `cap` images
inline size_t redist_aux_size(int cap) { return (size_t)6 * cap + 8; }
cudaError_t launch_redist_plan(const double *s, int F, int F_new, int cubic, int spline, const RedistPlan &p,
                               cudaStream_t st);
// Linear resample of `pairs` interleaved pairs per image (precision real).
cudaError_t launch_redist_linear(int precision, const void *f, void *fnew, long pairs, int F_new, const RedistPlan &p,
                                 cudaStream_t st);
// Cubic resample; `sigma` is scratch of 2 * pairs * F reals of the precision.
// Bytes of global scratch a cubic resample needs (0 when its columns fit in
// shared memory, which holds for strings of up to several hundred images).
size_t redist_cubic_scratch_bytes(int precision, long pairs, int F, int F_new);
cudaError_t launch_redist_cubic(int precision, const void *f, void *fnew, void *sigma, long pairs, int F, int F_new,
                                int spline, const RedistPlan &p, cudaStream_t st);
// Precision conversion of n reals.
cudaError_t launch_convert(const void *src, int src_prec, void *dst, int dst_prec, long n, cudaStream_t st);

}  // namespace mepgl
