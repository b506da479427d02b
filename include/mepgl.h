/*
 * mepgl.h -- C ABI of the GB300 implementation of mepgl's string-method hot
 * path (libmepgl_gb300.so).
 *
 * The reference (maiani/mepgl) has no library boundary: its host operators
 * are C++ functions taking ~40 raw device pointers each, with the lattice
 * size, spacing, component count and precision fixed at compile time
 * (mepgl/src/nlcg.cuh:18-54, mepgl/src/interpolation.cuh:6-24,
 * mepgl/src/config.cuh).  This header is the boundary that replaces them: an
 * opaque context owns every device buffer, the compile-time constants are
 * runtime fields of mepgl_problem, and every call returns a status instead
 * of exiting the process (mepgl/src/cuda_errors.cuh:561-571).  Each entry
 * point names the reference function it stands in for.
 *
 * Data layout (identical to the reference's device layout,
 * mepgl/src/io.cu:69-123): site (i, j) of image n at index
 * i + nx*j + nx*ny*n, x fastest; A, psi_1 and psi_2 are arrays of (x, y) /
 * (Re, Im) pairs of the context's precision (float or double).  Lattice
 * parameter arrays are nx*ny doubles in the same site order.  Per-image
 * scalars (energies, norms, steps, arc lengths) are always double.
 *
 * Threading: a context is bound to the CUDA stream given at creation and is
 * not re-entrant; use one context per stream.  Calls that return host data
 * synchronise that stream; the others are asynchronous.
 *
 * Failure detection (the reference has none: NaN fields give NaN energies,
 * a zero-length string divides 0 by 0, mepgl/src/interpolation.cu:126-140).
 * Each mepgl_nlcg_steps / mepgl_iteration call ends with a device check of
 * every image's energy and |g|^2; a NaN or infinity there, a string of zero
 * or non-finite arc length, or a fused-launch wait that ran out sets a
 * device flag.  Asynchronous calls cannot report it; the next call that
 * synchronises the stream (mepgl_image_scalars, mepgl_free_energy,
 * mepgl_get_state, mepgl_arc_length, mepgl_redistribute, mepgl_iteration in
 * modes L and C, mepgl_set_precision, mepgl_synchronize) returns
 * MEPGL_ERR_NAN (MEPGL_ERR_CUDA for the wait) with the string and image in
 * mepgl_last_error, and clears the flag.  The context stays usable.
 */
#ifndef MEPGL_H
#define MEPGL_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum mepgl_status {
    MEPGL_OK = 0,
    MEPGL_ERR_INVALID_ARG = 1,   /* bad size, pointer or option                    */
    MEPGL_ERR_CUDA = 2,          /* a CUDA runtime call or kernel launch failed    */
    MEPGL_ERR_NAN = 3,           /* a per-image scalar became NaN or infinite, or
                                    the string has no arc length (see below)       */
    MEPGL_ERR_IO = 4,            /* file reading / writing (npy helpers)           */
    MEPGL_ERR_UNSUPPORTED = 5,   /* option not available for this problem         */
    MEPGL_ERR_STATE = 6          /* call not valid in the context's current state  */
} mepgl_status;

enum { MEPGL_FP32 = 0, MEPGL_FP64 = 1 };          /* working precision of the fields  */
enum { MEPGL_HOST = 0, MEPGL_DEVICE = 1,          /* where a caller buffer lives      */
       MEPGL_STAGED = 2 };                         /* mepgl_set_state: the staged copy */
enum { MEPGL_LS_COMPAT = 0, MEPGL_LS_EXACT = 1 }; /* step: geometric scan | its exact
                                                     first local minimum     */
enum { MEPGL_POLY_COMPAT = 0, MEPGL_POLY_EXACT = 1 };       /* line polynomial        */
enum { MEPGL_SPLINE_COMPAT = 0, MEPGL_SPLINE_FMM = 1 };     /* cubic evaluation       */
enum { MEPGL_METRIC_FIELDS = 0, MEPGL_METRIC_JB = 1 };      /* arc-length metric      */
enum { MEPGL_REDIST_LINEAR = 0, MEPGL_REDIST_CUBIC = 1 };
/* Kinetic and magnetic terms: the reference's linearised covariant differences
 * with four collocated curl views (mepgl/src/nlcg.cu:149-203), or gauge links
 * U = exp(i q A dx) with one curl per plaquette (exactly gauge invariant; no
 * reference counterpart; energy, gradient and adjoints only, no NLCG). */
enum { MEPGL_DISC_REFERENCE = 0, MEPGL_DISC_LINK = 1 };
/* Arithmetic of the two NLCG passes for FP64 fields: IEEE double, or
 * float-float pairs on the FP32 pipes (about 48 significant bits, several
 * times faster on GPUs whose FP64 rate is a small fraction of FP32).  Fields,
 * reductions, line search and every other kernel stay double.  No
 * reference counterpart. */
enum { MEPGL_FP64_NATIVE = 0, MEPGL_FP64_PAIRED = 1 };
/* How the FP32 NLCG steps of a mepgl_nlcg_steps call are launched: two pass
 * kernels per step, or every step of the call in one persistent launch whose
 * tiles wait on per-image stage counters instead of kernel boundaries.  AUTO
 * fuses the batches of at most a few waves of tiles, where the boundaries
 * idle much of the GPU.  Both give the same results bit for bit.  No
 * reference counterpart. */
enum { MEPGL_FP32_STEPS_AUTO = 0, MEPGL_FP32_STEPS_PASSES = 1, MEPGL_FP32_STEPS_FUSED = 2 };

/* The physical problem.  Replaces the generated headers config.cuh/real.cuh
 * (N, dx, MULTICOMPONENT, NO_SELF_FIELD, DOUBLE_PRECISION) and the lattice
 * inputs read by loadInput (mepgl/src/io.cu:10-126).  All pointers are host
 * pointers, read during mepgl_create only.  The *_2 arrays may be NULL when
 * multicomponent == 0.  Domains are int32, nonzero = inside. */
typedef struct mepgl_problem {
    int32_t nx, ny;            /* lattice (the reference has nx == ny == N)    */
    int32_t n_images;          /* F                                            */
    int32_t multicomponent;    /* 0: psi_1 only, 1: psi_1 and psi_2            */
    int32_t thin_film;         /* 1: no magnetic self-field, A is frozen       */
    int32_t precision;         /* MEPGL_FP32 or MEPGL_FP64                     */
    double dx;
    double q_1, q_2, eta, gamma, delta;
    const double *a_1, *b_1, *m_xx_1, *m_yy_1;
    const double *a_2, *b_2, *m_xx_2, *m_yy_2;
    const double *h;
    const int32_t *comp_domain, *sc_domain;
} mepgl_problem;

/* Method options.  The defaults (mepgl_default_options) reproduce the
 * reference: compat line search and polynomial, compat spline, (B, J)
 * metric (mepgl/src/mepgl.cu:32). */
typedef struct mepgl_options {
    int32_t line_search;       /* MEPGL_LS_*                                    */
    int32_t line_polynomial;   /* MEPGL_POLY_*                                  */
    int32_t spline;            /* MEPGL_SPLINE_*                                */
    int32_t metric;            /* MEPGL_METRIC_*                                */
    int32_t use_graphs;        /* capture NLCG steps as CUDA graphs (default 1) */
    int32_t tile_rows;         /* rows per stencil tile: 0 = auto, 4, 8 or 16   */
    int32_t discretization;    /* MEPGL_DISC_*                                  */
    int32_t fp64_arith;        /* MEPGL_FP64_*                                  */
    int32_t fp32_steps;        /* MEPGL_FP32_STEPS_*                            */
} mepgl_options;

typedef struct mepgl_ctx mepgl_ctx;

/* Defaults described above. */
void mepgl_default_options(mepgl_options *opt);

/* Version string of the library. */
const char *mepgl_version(void);

/* Create a context: uploads parameters and masks, allocates all device
 * buffers (fields, gradients, directions, scratch) once.  `stream` is a
 * cudaStream_t (NULL = default stream).  Replaces the allocation and setup
 * part of main() (mepgl/src/mepgl.cu:453-616). */
mepgl_status mepgl_create(const mepgl_problem *prob, const mepgl_options *opt, void *stream, mepgl_ctx **out);

/* Free every device buffer of the context. */
mepgl_status mepgl_destroy(mepgl_ctx *ctx);

/* Message of the last failed call on this context (or of the last failed
 * mepgl_create on this thread when ctx is NULL). */
const char *mepgl_last_error(const mepgl_ctx *ctx);

/* Copy the string in / out.  a, psi_1, psi_2: F*nx*ny pairs of the context's
 * precision, in host or device memory.  psi_2 is ignored for one component.
 * mepgl_set_state resets the NLCG history (the reference starts every run
 * from zero gradients and infinite norms, mepgl/src/mepgl.cu:127-146). */
mepgl_status mepgl_set_state(mepgl_ctx *ctx, const void *a, const void *psi_1, const void *psi_2, int memory);

/* Staged upload of the next state (single-string contexts).  No counterpart
 * in the reference, which loads its state once per run.  For callers that
 * feed a new state every few steps from host memory: the copy of a, psi_1,
 * psi_2 (host or device memory, the context's precision and shape) into a
 * staging buffer of the context runs on a second stream and this call
 * returns at once, so the copy overlaps whatever the context computes
 * meanwhile.  mepgl_set_state(ctx, NULL, NULL, NULL, MEPGL_STAGED) then
 * waits for that copy on the context's stream and installs it (a device
 * copy, then the history reset of mepgl_set_state).  Host arrays should be
 * pinned for the copy to be asynchronous, and must stay unchanged until that
 * mepgl_set_state returns.  A later stage replaces an earlier one that was
 * not installed.  The staging buffer (one state) is kept until destroy. */
mepgl_status mepgl_stage_state(mepgl_ctx *ctx, const void *a, const void *psi_1, const void *psi_2, int memory);
mepgl_status mepgl_get_state(mepgl_ctx *ctx, void *a, void *psi_1, void *psi_2, int memory);

/* Initial string built on the device, for lattices too large to build on the
 * host.  Replaces StringBuilder.generate_matter_fields /
 * generate_vector_potential (mepgl/mepgl_lib/builder.py:107-223): for each
 * image and component |psi| = psi_abs * prod over that component's vortices
 * with a nonzero winding in the image of f(r), theta = sum winding *
 * atan2(y - y_v, x - x_v), plus Gaussian noise of deviation `noise` on Re and
 * Im (Philox4x32-10 keyed by `seed`: reproducible, independent of the launch),
 * times the superconducting domain; A from the gauge of b_z (0: A = 0,
 * 1: Landau_x, 2: Landau_y, 3: symmetric) times the computational domain.
 * Site (i, j) sits at (x0 + i dx, y0 + j dx).  profile 0: f = tanh(-r^2), the
 * builder's envelope; 1: f = tanh(r / sqrt 2).  The builder's component-2
 * phase function is not available (phase 0).  Sets the state and resets the
 * NLCG history like mepgl_set_state. */
typedef struct mepgl_vortex {
    int32_t component;         /* 1 or 2                                         */
    int32_t pad;
    const double *x, *y;       /* host arrays of F positions                     */
    const int32_t *winding;    /* host array of F windings (0: absent)           */
} mepgl_vortex;

typedef struct mepgl_guess {
    double x0, y0;
    double psi_abs_1, psi_abs_2;
    double noise;
    double b_z;
    int32_t gauge;
    int32_t profile;
    uint64_t seed;
    const mepgl_vortex *vortices;
    int32_t n_vortices;
    int32_t pad;
} mepgl_guess;

mepgl_status mepgl_generate_string(mepgl_ctx *ctx, const mepgl_guess *guess);
mepgl_status mepgl_batch_generate_string(mepgl_ctx *ctx, int string, const mepgl_guess *guess);

/* Per-image free energy of the current state (host array of F doubles).
 * Replaces computeFreeEnergy (mepgl/src/nlcg.cu:217-240). */
mepgl_status mepgl_free_energy(mepgl_ctx *ctx, double *fenergy);

/* Free energy and gradient dF/d(A, psi) of the current state.  Gradients
 * have the layout of the fields; NULL outputs are skipped.  Replaces the
 * gradientPsi / gradientA launches (mepgl/src/nlcg.cu:1521-1537). */
mepgl_status mepgl_energy_grad(mepgl_ctx *ctx, double *fenergy, void *g_a, void *g_psi_1, void *g_psi_2,
                               int memory);

/* `iterations` nonlinear-conjugate-gradient steps on every image.
 * use_cg = 0 gives steepest descent; maxwell_only = 1 freezes psi (mode M).
 * Replaces nlcgSteps (mepgl/src/nlcg.cu:1462-1586), with its gradient
 * buffer convention: each call starts from the same "previous" slot. */
mepgl_status mepgl_nlcg_steps(mepgl_ctx *ctx, int iterations, int use_cg, int maxwell_only);

/* Restart conjugate gradients (norm history = infinity) for images
 * [first, last).  The reference does this for the interior images after
 * every reparametrization (mepgl/src/mepgl.cu:231-234). */
mepgl_status mepgl_reset_cg(mepgl_ctx *ctx, int first_image, int last_image);

/* Per-image scalars after the last NLCG step (host arrays of F doubles;
 * NULL skips): energy before the step's update, |g|^2 of the slot the
 * reference's loop() reads, and the step length alpha. */
mepgl_status mepgl_image_scalars(mepgl_ctx *ctx, double *fenergy, double *g_norm2, double *alpha);

/* Observables of the current state, per image (host arrays of F doubles,
 * NULL skips), computed on the device: the magnetic flux dx^2 * sum B
 * (mepgl/post.py:131-133) and, for each component, the winding sum of
 * compute_winding (mepgl/mepgl_lib/gl_utils.py:10-41): the linearised phase
 * steps (u dv - v du) / (u^2 + v^2) around a rectangle, about 2 pi per
 * enclosed vortex.  inset = 0 walks the lattice edge as the reference does
 * (NaN where |psi| = 0 there, e.g. outside the superconductor); inset > 0
 * walks the rectangle that many sites inside.  winding_2 is ignored for
 * one component. */
mepgl_status mepgl_observables(mepgl_ctx *ctx, int inset, double *flux, double *winding_1, double *winding_2);
mepgl_status mepgl_batch_observables(mepgl_ctx *ctx, int string, int inset, double *flux, double *winding_1,
                                     double *winding_2);

/* Parameter adjoints (no reference counterpart): per image (host arrays of
 * F doubles, NULL skips) the partial derivatives of the free energy at the
 * current, fixed fields with respect to a uniform shift of the applied field
 * h (dF/dH), to eta and to gamma.  At a stationary image (a converged end
 * state) they are the total derivatives of its energy (envelope theorem). */
mepgl_status mepgl_param_adjoint(mepgl_ctx *ctx, double *dF_dH, double *dF_deta, double *dF_dgamma);
mepgl_status mepgl_batch_param_adjoint(mepgl_ctx *ctx, int string, double *dF_dH, double *dF_deta,
                                       double *dF_dgamma);

/* B (F*nx*ny reals) and J_1, J_2 (pairs) of the current state; NULL skips.
 * Replaces computeJB (mepgl/src/nlcg.cu:366-380). */
mepgl_status mepgl_compute_jb(mepgl_ctx *ctx, void *b, void *j_1, void *j_2, int memory);

/* Normalised arc length (host array of F doubles) in the field metric or
 * the (B, J) metric.  Replaces arcLength / arcLengthJB
 * (mepgl/src/interpolation.cu:143-169).  A string of zero or non-finite
 * length (all images equal, non-finite fields) returns MEPGL_ERR_NAN and
 * s = n / (F - 1), on which a linear resample keeps every image. */
mepgl_status mepgl_arc_length(mepgl_ctx *ctx, int metric, double *s);

/* Reparametrize the string to F_new equidistant images in the context's
 * metric, linear or cubic.  F_new == F (or F_new < 0) keeps the buffers;
 * otherwise the context is resized (the reference's final F_out resample,
 * mepgl/src/mepgl.cu:699-766; single-string contexts only).  With several
 * strings and F_new < 0 every string is reparametrized.  Does NOT restart CG
 * (see mepgl_reset_cg).  Replaces redistributeLinear / redistributeCubic
 * (mepgl/src/interpolation.cu:229-481).  Needs F >= 2 (linear) or F >= 4
 * (cubic), else MEPGL_ERR_INVALID_ARG.  Two equal adjacent images (a
 * segment of zero length, 0/0 in the reference) resample to their state;
 * a string of zero arc length returns MEPGL_ERR_NAN, and a singular cubic
 * spline matrix too. */
mepgl_status mepgl_redistribute(mepgl_ctx *ctx, int kind, int F_new);

/* Batched strings.  No counterpart in the reference, which runs parameter
 * sweeps as separate processes (mepgl/batch_run.py:9-21).  One context holds
 * n_strings strings of possibly different lattice size and image count (same
 * component count, thin-film switch and precision); mepgl_nlcg_steps and
 * mepgl_iteration advance all of them with the same launches (groups of 16
 * strings per launch).  The single-string calls above act on string 0; the
 * calls below address a string by index.  Setting any string's state
 * restarts the NLCG history of the whole context. */
mepgl_status mepgl_create_batch(const mepgl_problem *probs, int n_strings, const mepgl_options *opt, void *stream,
                                mepgl_ctx **out);
int mepgl_string_count(const mepgl_ctx *ctx);
mepgl_status mepgl_batch_info(const mepgl_ctx *ctx, int string, int *nx, int *ny, int *n_images);
mepgl_status mepgl_batch_set_state(mepgl_ctx *ctx, int string, const void *a, const void *psi_1, const void *psi_2,
                                   int memory);
mepgl_status mepgl_batch_get_state(mepgl_ctx *ctx, int string, void *a, void *psi_1, void *psi_2, int memory);
mepgl_status mepgl_batch_free_energy(mepgl_ctx *ctx, int string, double *fenergy);
mepgl_status mepgl_batch_image_scalars(mepgl_ctx *ctx, int string, double *fenergy, double *g_norm2,
                                       double *alpha);
mepgl_status mepgl_batch_arc_length(mepgl_ctx *ctx, int string, int metric, double *s);

/* One outer iteration of the reference's loop() in mode 'S', 'M', 'L' or
 * 'C' (mepgl/src/mepgl.cu:148-303): optional reparametrization + CG restart
 * of the interior images, then relaxation_steps NLCG steps. */
mepgl_status mepgl_iteration(mepgl_ctx *ctx, char mode, int relaxation_steps, int use_cg);

/* Change the working precision in place (FP32 <-> FP64): the fields are
 * converted, the NLCG history is reset.  Used for FP32 bulk relaxation
 * followed by FP64 polish. */
mepgl_status mepgl_set_precision(mepgl_ctx *ctx, int precision);

/* Number of images, working precision, and the number of kernel launches
 * issued by this context so far (graph replays count their kernels). */
mepgl_status mepgl_info(const mepgl_ctx *ctx, int *n_images, int *precision, int64_t *kernel_launches);

/* Run `steps` NLCG steps launched one pass at a time with CUDA events
 * between the passes on the context's stream, and return the mean duration
 * (milliseconds) of the gradient pass and of the direction/line pass.  The
 * steps are real steps: the state advances.  No reference counterpart (the
 * reference has no timing facility); used by the benchmark's roofline. */
mepgl_status mepgl_profile_passes(mepgl_ctx *ctx, int steps, int use_cg, double *ms_grad, double *ms_dir_poly);

/* Names of the kernels that run the two NLCG passes of this context in its
 * current precision and FP64 arithmetic (FP32 passes are warp-strip or
 * shared-memory-tile kernels, chosen when the library is built), and of the
 * kernel that runs whole mepgl_nlcg_steps calls as one persistent launch
 * ("" when the passes are launched separately; mepgl_profile_passes always
 * times the separate pass kernels).  The strings are static.  No reference
 * counterpart; labels timings and profiler captures. */
mepgl_status mepgl_pass_kernels(const mepgl_ctx *ctx, const char **grad, const char **dir_poly, const char **fused);

/* Self-test of the fused launch's bounded waits: one fused launch whose work
 * queue starts after the gradient items of its step, so every direction item
 * waits for an image stage that nothing sets, gives up after a short poll
 * limit and sets the device status flag.  *timed_out = 1 when the flag was
 * set (then cleared).  The launch writes no field or scalar, so the context
 * continues as before.  FP32 contexts of a build with fused steps; no
 * reference counterpart. */
mepgl_status mepgl_fused_wait_selftest(mepgl_ctx *ctx, int *timed_out);

/* Allocation-free free energy.  No counterpart in the reference.  For callers
 * that cannot allocate device memory -- an embedding that owns a fixed
 * device arena and hands out only pre-allocated buffers, a host framework
 * whose memory pool owns the whole device, or a plugin whose host process
 * forbids cudaMalloc after start-up -- this evaluates the per-image FP64
 * free energy of caller-owned device arrays without a context and without
 * any allocation.
 * Inputs (all device pointers): comp_code / sc_code are int32 neighbour
 * codes per site (the layout of the reference's buildNearestNeighbourMap),
 * the nine parameter arrays are per-site doubles, a / psi_1 / psi_2 are the
 * F images as double pairs; fenergy receives F doubles.  Scratch for the
 * reduction lives in fixed device arrays of the library (4 MiB + 16 KiB per
 * GPU that loads it, kept until the process exits): the string must satisfy
 * n_images <= 4096 and n_images * ceil(nx/32) * ceil(ny/8) <= 65536 (and the
 * lattice nx <= 32767*32, ny <= 32767*8), else MEPGL_ERR_INVALID_ARG.  The
 * first call on a device resolves the scratch addresses and uploads
 * constant tables; make that first call before any stream capture.  They
 * are kept until exit, so a device reset afterwards is not supported.  All
 * calls share the scratch, so calls that overlap on the GPU (different
 * streams, no ordering) race.  A CUDA error already pending when the call
 * starts is reported (MEPGL_ERR_CUDA) and left pending for its owner.
 * Asynchronous on `stream` (a cudaStream_t, NULL = default stream).
 * Errors: mepgl_noalloc_last_error. */
mepgl_status mepgl_free_energy_noalloc(int nx, int ny, int n_images, int multicomponent, int thin_film, double dx,
                                       const int32_t *comp_code, const int32_t *sc_code, const double *a_1,
                                       const double *b_1, const double *m_xx_1, const double *m_yy_1,
                                       const double *a_2, const double *b_2, const double *m_xx_2,
                                       const double *m_yy_2, const double *h, double q_1, double q_2, double eta,
                                       double gamma, double delta, const void *a, const void *psi_1,
                                       const void *psi_2, double *fenergy, void *stream);

/* Message of the last failed mepgl_free_energy_noalloc on this thread. */
const char *mepgl_noalloc_last_error(void);

/* Refinement of images to stationary points of the free energy (no
 * reference counterpart: the reference's barrier is the largest image
 * energy of the relaxed string, mepgl/post.py:188, which depends on the
 * image count and the reparametrization cadence).  Each image of the
 * context's string (FP64 single-string contexts, reference discretisation)
 * is refined in place, per kind[n]:
 *   MEPGL_STATIONARY_MINIMUM  to a local minimum (a string end state);
 *   MEPGL_STATIONARY_SADDLE   to an index-1 saddle (the transition state),
 *                             by min-mode Newton: the lowest Hessian mode by
 *                             Lanczos, an uphill Newton step along it and a
 *                             shifted Newton step (Levenberg-Marquardt, by
 *                             conjugate gradients) in its complement;
 *   MEPGL_STATIONARY_SKIP     left unchanged.
 * Each iteration first minimises over smooth gauge transformations of the
 * image (Legendre products of total degree <= gauge_degree), along which
 * the reference's discretisation is gauge invariant only to O(dx^2): the
 * energy there is nearly flat and the orbits curved, which stalls Newton
 * steps taken in straight lines.  Hessian-vector products are central
 * differences of the gradient, in IEEE double.  mode_a / mode_psi_1 /
 * mode_psi_2 (layout of the fields, `memory` host or device; NULL for all
 * three continues from the modes of the previous call) give the initial
 * direction of each saddle image, e.g. the string's chord tangent
 * x_{k+1} - x_{k-1}; other images' entries are ignored.  Stops per image
 * when |g| (Euclidean norm over the image's fields) <= g_tol or after
 * max_newton iterations; the report (host array of F, may be NULL) gives
 * energy, |g|, the lowest curvature and counts.  Workspace (about 41
 * copies of the fields) is allocated on the first call and kept. */
enum { MEPGL_STATIONARY_MINIMUM = 0, MEPGL_STATIONARY_SADDLE = 1, MEPGL_STATIONARY_SKIP = 2 };

typedef struct mepgl_refine_options {
    double g_tol;              /* |g| target (default 1e-8)                       */
    int32_t max_newton;        /* Newton iterations (default 40)                  */
    int32_t max_cg;            /* CG iterations per linear solve (default 3000)   */
    int32_t lanczos_steps;     /* per min-mode update (default 12, 30 at start)   */
    int32_t gauge_degree;      /* gauge polynomial degree <= 16, 0 = off,
                                  -1 = auto: max(nx, ny) / 8 within 4..16, at most
                                  min(nx, ny) / 2 (default)                        */
    double mu0;                /* initial Levenberg-Marquardt shift (1e-3)        */
    double cg_eta;             /* CG relative tolerance (0.1), see `forcing`      */
    int32_t max_retries;       /* rejected steps retried per iteration (8)        */
    int32_t gauge_refresh;     /* iterations a gauge-subspace Hessian is reused; 0 =
                                  auto: 1 up to 64 gauge functions, else 4 (default);
                                  kept between calls while the state is unchanged */
    int32_t precondition;      /* 1: CG preconditioned by the cosine-basis inverse of a
                                  constant-coefficient model of the Hessian (needs
                                  cuFFT at run time; without it the CG runs
                                  unpreconditioned), 0: plain CG (default 1) */
    int32_t forcing;           /* CG tolerance per Newton step: 0 = cg_eta (default;
                                  linear convergence at about that rate), 1 =
                                  sqrt|g| capped at cg_eta (superlinear, tighter
                                  solves); never tighter than g_tol needs      */
} mepgl_refine_options;

typedef struct mepgl_refine_report {
    double energy;             /* free energy after the refinement                */
    double g_norm;             /* |g| after the refinement                        */
    double min_curvature;      /* saddles: the lowest Hessian eigenvalue          */
    double mu;                 /* Levenberg-Marquardt shift reached               */
    int32_t newton_iterations, cg_iterations, gradient_evaluations, converged;
    int32_t preconditioned;    /* the CG of this call was preconditioned          */
} mepgl_refine_report;

void mepgl_default_refine_options(mepgl_refine_options *opt);
mepgl_status mepgl_refine_stationary(mepgl_ctx *ctx, const int32_t *kind, const void *mode_a,
                                     const void *mode_psi_1, const void *mode_psi_2, int memory,
                                     const mepgl_refine_options *opt, mepgl_refine_report *report);

/* Wait for the context's stream. */
mepgl_status mepgl_synchronize(mepgl_ctx *ctx);

#ifdef __cplusplus
}
#endif
#endif
