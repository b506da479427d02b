// kernels.cu -- CUDA kernels of libmepgl_gb300 (sm_103a).
//
// The NLCG iteration of the reference (nlcgSteps, mepgl/src/nlcg.cu:1462-1586:
// ~12 kernels, 4 two-level reductions, ~10 device-wide syncs per step) is two
// passes over the string here:
//
//   k_grad      x <- x + alpha_pend d   (the previous step's update, fused)
//               g  = dF/dx              (gradientPsi + gradientA)
//               |g|^2, g.(g - g_prev)   (gradientDensity + 2 sums)
//               last tile of an image:  beta (computeStepDirection's scalar)
//   k_dir_poly  d <- -g + beta d        (computeStepDirection)
//               quartic F(x + a d)      (polynomialExpansion + 2 sums)
//               last tile of an image:  line search -> alpha (lineSearch)
//
// so one step reads x, d, g_prev, g (twice with halo, served mostly by L2)
// and writes x, g, d: 9 state-sized streams instead of the reference's ~20.
// x and d are ping-ponged because neighbouring tiles read them as halo while
// they are being rewritten.
//
// Tiles are 32 x TileRows<T> sites (16 rows in FP32, 8 in FP64) staged with
// a one-site halo in shared memory; each thread computes TileRows/8 sites of
// one column.  Addresses inside an image are 32-bit offsets from per-tile
// base pointers.
#include <type_traits>

#include "kernels.cuh"
#include "site_ops.cuh"
#include "site_pair.cuh"

namespace mepgl {

// Tuning knobs (compile time): tile rows per precision and the minimum
// resident blocks per SM requested from ptxas for the two NLCG passes.
#ifndef MEPGL_ROWS_F32
#define MEPGL_ROWS_F32 16
#endif
#ifndef MEPGL_ROWS_F64
#define MEPGL_ROWS_F64 8
#endif
#ifndef MEPGL_MINB_GRAD
#define MEPGL_MINB_GRAD 4
#endif
#ifndef MEPGL_MINB_DIR
#define MEPGL_MINB_DIR 4
#endif

// 1: the direction d = -g + beta d is formed by a pointwise pass and the
// polynomial pass copies the x and d halo tiles with cp.async; 0: one fused
// pass forms d over the halo tile in registers
#ifndef MEPGL_SPLIT_DIR
#define MEPGL_SPLIT_DIR 0
#endif
// 1: the direction pass of FP32 strings copies the raw x, g and d halo tiles
// with cp.async and forms -g + beta d in shared memory; 0: x by cp.async,
// g and d through registers
#ifndef MEPGL_DIR_ASYNC
#define MEPGL_DIR_ASYNC 0
#endif
// 1: the gradient pass copies the raw x and d halo tiles with cp.async and
// forms x + alpha d in shared memory; 0: through registers (stage mode 1)
#ifndef MEPGL_GRAD_ASYNC
#define MEPGL_GRAD_ASYNC 0
#endif

// the float-float passes hold twice the registers of FP32 ones
// FP32 NLCG passes as warp strips (strip.cuh) instead of shared-memory tiles
#ifndef MEPGL_STRIP
#define MEPGL_STRIP 1
#endif
#ifndef MEPGL_MINB_STRIP
#define MEPGL_MINB_STRIP 16   // single-warp blocks per SM: 128 registers
#endif
#ifndef MEPGL_MINB_STRIP_GRAD
#define MEPGL_MINB_STRIP_GRAD MEPGL_MINB_STRIP
#endif
#ifndef MEPGL_MINB_STRIP_DIR
#define MEPGL_MINB_STRIP_DIR MEPGL_MINB_STRIP
#endif
// strip row loop unrolled by the window period; interior sites with unit weights
#ifndef MEPGL_STRIP_UNROLL
#define MEPGL_STRIP_UNROLL 0
#endif
#ifndef MEPGL_STRIP_INTERIOR
#define MEPGL_STRIP_INTERIOR 0
#endif
// two-component FP32 strips in packed FP32x2 arithmetic (site_pair.cuh)
#ifndef MEPGL_STRIP_PAIR
#define MEPGL_STRIP_PAIR 1
#endif
// FP32 NLCG steps as one persistent launch with per-image stage counters (strip.cuh)
#ifndef MEPGL_STRIP_FUSED
#define MEPGL_STRIP_FUSED 0
#endif
// FP32 strip launches of a single string use kernels specialised for it
#ifndef MEPGL_STRIP_ONE
#define MEPGL_STRIP_ONE 1
#endif
#ifndef MEPGL_MINB_STRIP_FUSED
#define MEPGL_MINB_STRIP_FUSED MEPGL_MINB_STRIP
#endif
// explicit register cap of the fused kernel (0: from MEPGL_MINB_STRIP_FUSED)
#ifndef MEPGL_MAXREG_FUSED
#define MEPGL_MAXREG_FUSED 0
#endif
// fused steps only for batches of at most this many waves of the pass kernels
// (beyond that the boundaries cost little and the pass kernels hold more warps)
#ifndef MEPGL_FUSE_WAVES
#define MEPGL_FUSE_WAVES 4
#endif
#if MEPGL_STRIP && MEPGL_SPLIT_DIR
#error "MEPGL_SPLIT_DIR applies to the tile kernels; build it with MEPGL_STRIP=0"
#endif
// paired FP64 passes of two-component strings in packed float-float arithmetic
#ifndef MEPGL_FF_PAIR
#define MEPGL_FF_PAIR 1
#endif
#ifndef MEPGL_MINB_GRAD_FF
#define MEPGL_MINB_GRAD_FF 3
#endif
#ifndef MEPGL_MINB_DIR_FF
#define MEPGL_MINB_DIR_FF 2
#endif
template <class T> struct MinBlocks { static constexpr int grad = MEPGL_MINB_GRAD, dir = MEPGL_MINB_DIR; };
template <> struct MinBlocks<ff> { static constexpr int grad = MEPGL_MINB_GRAD_FF, dir = MEPGL_MINB_DIR_FF; };
// Gradient tile kernels whose stencil spills at their register budget stage
// one halo element at a time and read the previous gradient after the
// stencil.  MEPGL_GRAD_LEAN: 0 none, 1 the float-float kernels (default),
// 2 every precision.
#ifndef MEPGL_GRAD_LEAN
#define MEPGL_GRAD_LEAN 1
#endif
template <class T> struct GradLean {
    static constexpr bool v = MEPGL_GRAD_LEAN == 2 || (MEPGL_GRAD_LEAN == 1 && std::is_same<T, ff>::value);
};

// Paired FP64: while the NLCG passes run, the fields x hold float-float
// pairs too (launch_x_format converts them in place before and after), so
// the passes read and write them without double conversions.
#ifndef MEPGL_FF_XPAIRS
#define MEPGL_FF_XPAIRS 1
#endif
template <class T> struct XPairs { static constexpr bool v = MEPGL_FF_XPAIRS != 0 && std::is_same<T, ff>::value; };

template <class T> struct TileRows { static constexpr int v = sizeof(T) == 4 ? MEPGL_ROWS_F32 : MEPGL_ROWS_F64; };
// Two-component float-float NLCG passes run the packed stencils (site_pair.cuh).
template <class T, int NC> struct FFPacked {
    static constexpr bool v = MEPGL_FF_PAIR && NC == 2 && std::is_same<T, ff>::value;
};
template <> struct TileRows<ff> { static constexpr int v = MEPGL_ROWS_F64; };

int nlcg_step_launches() { return 2 + MEPGL_SPLIT_DIR; }

bool nlcg_fused(int precision) { return MEPGL_STRIP && MEPGL_STRIP_FUSED && precision == 0; }

int fuse_waves() { return MEPGL_FUSE_WAVES; }

void nlcg_pass_kernels(int precision, int paired, const char **grad, const char **dir_poly)
{
    (void)paired;
    const bool strip = MEPGL_STRIP && precision == 0;
    *grad = strip ? "k_grad_s" : "k_grad";
    *dir_poly = strip ? "k_dir_poly_s" : "k_dir_poly";
}

int tile_rows(int precision) { return precision == 1 ? TileRows<double>::v : TileRows<float>::v; }

cudaError_t upload_mask_tables()
{
    static MaskTable<float> f;
    static MaskTable<double> d;
    build_mask_table(f);
    build_mask_table(d);
    cudaError_t e = cudaMemcpyToSymbol(c_mask_f, &f, sizeof(f));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_mask_d, &d, sizeof(d));
    return e;
}

namespace {

// Base pointers of one image's fields for one tile.
template <class T, int NC>
struct ImagePtrs {                  // storage type (double for float-float)
    const vec2_t<store_t<T>> *in[1 + NC];
    const vec2_t<store_t<T>> *aux[1 + NC];
    vec2_t<store_t<T>> *out[1 + NC];
};

// ------------------------------------------------------------------ staging
// The (TYT+2) x (TX+2) halo tile is split into flat element indices spread
// over the block; each thread first issues every global load of all its
// elements (independent, so they are in flight together), then combines and
// stores them.  Out-of-lattice elements are zero.
// mode 0: x = in;  mode 1: x = in + alpha * aux (and interior x -> out);
// mode 2: x = -aux + beta * in, i.e. the new direction (interior -> out).
// IN_WORK / AUX_WORK: in (and out) / aux are NLCG work arrays (g, d) rather
// than fields.
// CHUNK: one element's loads in flight at a time instead of all of them
// (fewer registers live, for the kernels whose stencil is near its budget).
template <class T, int NC, int TYT, int MODE, bool IN_WORK = false, bool AUX_WORK = false, bool CHUNK = false>
__device__ __forceinline__ void stage(Tile<T, NC, TYT> &t, const StringDesc &S, const ImagePtrs<T, NC> &ip, int i0,
                                      int j0, T coef, bool write_out, bool masks)
{
    using V = vec2_t<T>;
    constexpr int HW = TX + 2, HE = (TYT + 2) * HW, NI = (HE + NT - 1) / NT, KB = CHUNK ? 1 : NI;
    const bool aux = MODE == 2 || (MODE == 1 && coef != (T)0);
    V f[NI][1 + NC], a[NI][1 + NC];
    uint16_t m[NI];
    int sidx[NI];
    bool ok[NI];
#pragma unroll
    for (int k0 = 0; k0 < NI; k0 += KB) {
#pragma unroll
    for (int k = k0; k < k0 + KB; ++k) {
        const int e = threadIdx.x + k * NT;
        const int hy = e / HW, hx = e - hy * HW;
        const int gi = i0 + hx - 1, gj = j0 + hy - 1;
        ok[k] = e < HE && gi >= 0 && gi < S.nx && gj >= 0 && gj < S.ny;
        sidx[k] = ok[k] ? gi + S.nx * gj : 0;
        m[k] = 0;
#pragma unroll
        for (int c = 0; c < 1 + NC; ++c) {
            f[k][c].x = f[k][c].y = (T)0;
            a[k][c].x = a[k][c].y = (T)0;
        }
        if (ok[k]) {
            const int s = sidx[k];
#pragma unroll
            for (int c = 0; c < 1 + NC; ++c) f[k][c] = IN_WORK ? loadw<T>(ip.in[c] + s) : load2<T>(ip.in[c] + s);
            if (aux)
#pragma unroll
                for (int c = 0; c < 1 + NC; ++c)
                    a[k][c] = AUX_WORK ? loadw<T>(ip.aux[c] + s) : load2<T>(ip.aux[c] + s);
            if (masks)
                m[k] = S.mask ? S.mask[s]
                              : (uint16_t)((S.code_comp[s] & 0xff) | ((S.code_sc[s] & 0xff) << 8));
        }
    }
#pragma unroll
    for (int k = k0; k < k0 + KB; ++k) {
        const int e = threadIdx.x + k * NT;
        if (e >= HE) continue;
        const int hy = e / HW, hx = e - hy * HW;
        V v[1 + NC];
#pragma unroll
        for (int c = 0; c < 1 + NC; ++c) {
            if (MODE == 2) {
                v[c].x = -a[k][c].x + coef * f[k][c].x;
                v[c].y = -a[k][c].y + coef * f[k][c].y;
            } else if (MODE == 1 && aux) {
                v[c].x = f[k][c].x + coef * a[k][c].x;
                v[c].y = f[k][c].y + coef * a[k][c].y;
            } else {
                v[c] = f[k][c];
            }
        }
        if (write_out && ok[k] && hx >= 1 && hx <= TX && hy >= 1 && hy <= TYT)
#pragma unroll
            for (int c = 0; c < 1 + NC; ++c) {
                if (IN_WORK) storew<T>(ip.out[c] + sidx[k], v[c]);
                else store2<T>(ip.out[c] + sidx[k], v[c]);
            }
        t.A[hy][hx] = v[0];
#pragma unroll
        for (int c = 0; c < NC; ++c) t.P[c][hy][hx] = v[1 + c];
        if (masks) t.m[hy][hx] = m[k];
    }
    }
}

// Asynchronous copy of a plain halo tile (no arithmetic on the values):
// cp.async per element, zero-filled outside the lattice, so its latency
// overlaps the register-staged arrays that follow.  The neighbour codes
// (2 bytes, below the 4-byte copy size) are loaded into m[] for the caller
// to store; cp_async_wait_all() + a barrier complete the tile.
__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

template <int BYTES>
__device__ __forceinline__ void cp_async(void *dst, const void *src, bool valid)
{
    const int n = valid ? BYTES : 0;
    if (BYTES == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(smem_u32(dst)), "l"(src), "r"(n)
                     : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;\n" ::"r"(smem_u32(dst)), "l"(src), "n"(BYTES),
                     "r"(n)
                     : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

template <class T, int NC, int TYT>
__device__ __forceinline__ void stage_async(TileF<T, NC, TYT> &t, const StringDesc &S,
                                            const vec2_t<T> *const *src, int i0, int j0, uint16_t *m)
{
    using V = vec2_t<T>;
    constexpr int HW = TX + 2, HE = (TYT + 2) * HW, NI = (HE + NT - 1) / NT;
#pragma unroll
    for (int k = 0; k < NI; ++k) {
        const int e = threadIdx.x + k * NT;
        if (m) m[k] = 0;
        if (e >= HE) continue;
        const int hy = e / HW, hx = e - hy * HW;
        const int gi = i0 + hx - 1, gj = j0 + hy - 1;
        const bool ok = gi >= 0 && gi < S.nx && gj >= 0 && gj < S.ny;
        const int s = ok ? gi + S.nx * gj : 0;
        cp_async<sizeof(V)>(&t.A[hy][hx], src[0] + s, ok);
#pragma unroll
        for (int c = 0; c < NC; ++c) cp_async<sizeof(V)>(&t.P[c][hy][hx], src[1 + c] + s, ok);
        if (m && ok) m[k] = S.mask[s];
    }
}

template <class T, int NC, int TYT>
__device__ __forceinline__ void store_codes(Tile<T, NC, TYT> &t,
                                            const uint16_t (&m)[(((TYT + 2) * (TX + 2)) + NT - 1) / NT])
{
    constexpr int HW = TX + 2, HE = (TYT + 2) * HW, NI = (HE + NT - 1) / NT;
#pragma unroll
    for (int k = 0; k < NI; ++k) {
        const int e = threadIdx.x + k * NT;
        if (e < HE) t.m[e / HW][e % HW] = m[k];
    }
}

template <class T, int NC>
__device__ __forceinline__ void image_ptrs(ImagePtrs<T, NC> &ip, void *const *in, void *const *aux, void *const *out,
                                           size_t off)
{
#pragma unroll
    for (int c = 0; c < 1 + NC; ++c) {
        using W = vec2_t<store_t<T>>;
        ip.in[c] = in ? static_cast<const W *>(in[c]) + off : nullptr;
        ip.aux[c] = aux ? static_cast<const W *>(aux[c]) + off : nullptr;
        ip.out[c] = out ? static_cast<W *>(out[c]) + off : nullptr;
    }
}

// Slot of a tile's partial sums: the global tile index of (string, image, row,
// column), independent of which launch (whole batch or one string) covers it.
__device__ __forceinline__ int part_slot(const StringDesc &S, const TileRef &tr)
{
    return S.tile_base + (tr.n * S.tiles_y + tr.ty) * S.tiles_x + tr.tx;
}

__device__ __forceinline__ TileRef flat_tile(const StringDesc &S, int tt)
{
    const int tpi = S.tiles_x * S.tiles_y, n = tt / tpi, r = tt - n * tpi, ty = r / S.tiles_x;
    TileRef t;
    t.s = 0;
    t.ty = (int16_t)ty;
    t.tx = (int16_t)(r - ty * S.tiles_x);
    t.pad = 0;
    t.n = n;
    return t;
}

// Field h at a neighbour (per-site strings only).
template <class T>
__device__ __forceinline__ T h_site(const StringDesc &S, const SiteParams<T> &p, int s)
{
    return S.per_site ? from_store<T>(static_cast<const store_t<T> *>(S.ph)[s]) : p.h;
}

// --------------------------------------------------------------- line search
// Quartic A + B x + C x^2 + D x^3 + E x^4 evaluated in round-to-nearest
// double without contraction, in the oracle's order.
__device__ __forceinline__ double quartic_rn(const double *c, double x)
{
    const double x2 = __dmul_rn(x, x);
    double f = __dmul_rn(c[4], __dmul_rn(x2, x2));
    f = __dadd_rn(f, __dmul_rn(__dmul_rn(__dmul_rn(c[3], x), x), x));
    f = __dadd_rn(f, __dmul_rn(__dmul_rn(c[2], x), x));
    f = __dadd_rn(f, __dmul_rn(c[1], x));
    return __dadd_rn(f, c[0]);
}

// lineSearch (nlcg.cu:1398-1445) by one warp: first p in 1..2000 with
// f(x_p) > f(x_{p-1}) (else 2000); alpha = x_p / m in the working precision.
template <class T>
__device__ double line_search_scan(const double *c, const double *xt)
{
    const int lane = threadIdx.x & 31;
    double f_prev = quartic_rn(c, xt[0]);
    int found = 0;
    for (int base = 1; base <= 2000; base += 32) {
        const int p = base + lane;
        const double fp = p <= 2000 ? quartic_rn(c, xt[p]) : 0.0;
        double fl = __shfl_up_sync(0xffffffffu, fp, 1);
        if (lane == 0) fl = f_prev;
        const unsigned bal = __ballot_sync(0xffffffffu, p <= 2000 && fp > fl);
        if (bal) { found = base + __ffs(bal) - 1; break; }
        f_prev = __shfl_sync(0xffffffffu, fp, 31);
    }
    const int j = found ? found : 2000;
    const T m = (T)1.025f;
    return (double)((T)xt[j] / m);
}

// Exact version of the reference's scan: the first local minimum of the
// quartic downhill from alpha = 0, i.e. the smallest positive root of the
// cubic derivative with positive curvature (closed-form roots, two Newton
// steps each); `fallback` (the scan's answer) when p'(0) >= 0 or none exists.
__device__ double line_search_exact(const double *c, double fallback)
{
    const double a3 = 4 * c[4], a2 = 3 * c[3], a1 = 2 * c[2], a0 = c[1];
    double roots[3];
    int nr = 0;
    if (fabs(a0) + fabs(a1) + fabs(a2) + fabs(a3) == 0) return fallback;
    if (fabs(a3) > 1e-300) {
        const double A2 = a2 / a3, A1 = a1 / a3, A0 = a0 / a3;
        const double Q = (3 * A1 - A2 * A2) / 9, R = (9 * A2 * A1 - 27 * A0 - 2 * A2 * A2 * A2) / 54;
        const double disc = Q * Q * Q + R * R;
        if (disc >= 0) {
            const double sd = sqrt(disc);
            roots[nr++] = -A2 / 3 + cbrt(R + sd) + cbrt(R - sd);
        } else {
            const double th = acos(R / sqrt(-Q * Q * Q)), r = 2 * sqrt(-Q);
            roots[nr++] = r * cos(th / 3) - A2 / 3;
            roots[nr++] = r * cos((th + 2 * M_PI) / 3) - A2 / 3;
            roots[nr++] = r * cos((th + 4 * M_PI) / 3) - A2 / 3;
        }
    } else if (fabs(a2) > 1e-300) {
        const double disc = a1 * a1 - 4 * a2 * a0;
        if (disc >= 0) {
            const double sq = sqrt(disc), qq = -0.5 * (a1 + (a1 >= 0 ? sq : -sq));
            if (qq != 0) { roots[nr++] = qq / a2; roots[nr++] = a0 / qq; }
        }
    } else if (a1 != 0) {
        roots[nr++] = -a0 / a1;
    }
    // the scan stops at the first increase: not a descent direction -> its answer
    if (!(a0 < 0)) return fallback;
    double best = -1;
    for (int t = 0; t < nr; ++t) {
        double r = roots[t];
        for (int it = 0; it < 2; ++it) {
            const double dp = a0 + r * (a1 + r * (a2 + r * a3)), ddp = a1 + r * (2 * a2 + r * 3 * a3);
            if (ddp != 0) r -= dp / ddp;
        }
        const double ddp = a1 + r * (2 * a2 + r * 3 * a3);
        if (!(r > 0) || !(ddp > 0)) continue;
        if (best < 0 || r < best) best = r;   // first local minimum downhill from 0
    }
    return best < 0 ? fallback : best;
}

// ------------------------------------------------------------------ kernels
template <class T, int NC>
__global__ void __launch_bounds__(NT, MinBlocks<T>::grad) k_grad(const __grid_constant__ Batch bt, const TileRef *__restrict__ tiles,
                                             int n_tiles, Scalars sc, StepFlags f)
{
    constexpr int TYT = TileRows<T>::v;
    using V = vec2_t<T>;
    __shared__ Tile<T, NC, TYT> t;
#if MEPGL_GRAD_ASYNC
    __shared__ TileF<T, NC, TYT> dt;
#endif
    __shared__ double red[NT / 32 * 2];
    for (int tt = blockIdx.x; tt < n_tiles; tt += gridDim.x) {
        const TileRef tr = tiles[tt];
        const StringDesc &S = bt.s[tr.s];
        const int img = S.img_base + tr.n;
        const int i0 = tr.tx * TX, j0 = tr.ty * TYT;
        const size_t off = (size_t)tr.n * S.nx * S.ny;
        ImagePtrs<T, NC> ip;
        image_ptrs<T, NC>(ip, S.x[f.xin], S.d[f.din], S.x[f.xout], off);
#if MEPGL_GRAD_ASYNC
        if constexpr (std::is_same<T, ff>::value) {
            stage<T, NC, TYT, 1, XPairs<T>::v, true, GradLean<T>::v>(t, S, ip, i0, j0, (T)sc.alpha_pend[img], true, true);
        } else {
            constexpr int HW = TX + 2, HE = (TYT + 2) * HW, NI = (HE + NT - 1) / NT;
            const T alpha = (T)sc.alpha_pend[img];
            uint16_t codes[NI];
            stage_async<T, NC, TYT>(t, S, ip.in, i0, j0, codes);
            if (alpha != (T)0) stage_async<T, NC, TYT>(dt, S, ip.aux, i0, j0, nullptr);
            store_codes<T, NC, TYT>(t, codes);
            cp_async_wait_all();
            __syncthreads();
            // x <- x + alpha d over the halo tile; interior x -> x[xout]
#pragma unroll
            for (int k = 0; k < NI; ++k) {
                const int e = threadIdx.x + k * NT;
                if (e >= HE) continue;
                const int hy = e / HW, hx = e - hy * HW;
                V v[1 + NC];
                v[0] = t.A[hy][hx];
#pragma unroll
                for (int c = 0; c < NC; ++c) v[1 + c] = t.P[c][hy][hx];
                if (alpha != (T)0) {
                    V dv = dt.A[hy][hx];
                    v[0].x = v[0].x + alpha * dv.x;
                    v[0].y = v[0].y + alpha * dv.y;
                    t.A[hy][hx] = v[0];
#pragma unroll
                    for (int c = 0; c < NC; ++c) {
                        dv = dt.P[c][hy][hx];
                        v[1 + c].x = v[1 + c].x + alpha * dv.x;
                        v[1 + c].y = v[1 + c].y + alpha * dv.y;
                        t.P[c][hy][hx] = v[1 + c];
                    }
                }
                const int gi = i0 + hx - 1, gj = j0 + hy - 1;
                if (hx >= 1 && hx <= TX && hy >= 1 && hy <= TYT && gi < S.nx && gj < S.ny)
#pragma unroll
                    for (int c = 0; c < 1 + NC; ++c) ip.out[c][gi + S.nx * gj] = v[c];
            }
        }
#else
        stage<T, NC, TYT, 1, XPairs<T>::v, true, GradLean<T>::v>(t, S, ip, i0, j0, (T)sc.alpha_pend[img], true, true);
#endif
        using W = vec2_t<store_t<T>>;
        W *gcur[1 + NC];
        const W *gprev[1 + NC];
#pragma unroll
        for (int c = 0; c < 1 + NC; ++c) {
            gcur[c] = static_cast<W *>(S.g[f.gcur][c]) + off;
            gprev[c] = static_cast<const W *>(S.g[f.gprev][c]) + off;
        }
        SiteParams<T> p;
        p.load_uniform(S);
        __syncthreads();
        T v[2] = {(T)0, (T)0};
        const int lx = threadIdx.x & 31, gi = i0 + lx;
        // previous gradient of this thread's sites, loaded before the stencil
        // (lean kernels: after it, so that it holds no registers meanwhile)
        V gold[TYT / 8][1 + NC];
        if (!GradLean<T>::v)
#pragma unroll
        for (int r = 0; r < TYT / 8; ++r) {
            const int gj = j0 + (threadIdx.x >> 5) + 8 * r;
#pragma unroll
            for (int c = 0; c < 1 + NC; ++c) {
                gold[r][c].x = gold[r][c].y = (T)0;
                if (gi < S.nx && gj < S.ny) gold[r][c] = loadw<T>(gprev[c] + gi + S.nx * gj);
            }
        }
#pragma unroll
        for (int r = 0; r < TYT / 8; ++r) {
            const int ly = (threadIdx.x >> 5) + 8 * r, gj = j0 + ly;
            if (gi < S.nx && gj < S.ny) {
                const int s = gi + S.nx * gj;
                Wts<T> w;
                w.load(t.m[ly + 1][lx + 1]);
                T hr = p.h, hl = p.h, hu = p.h, hd = p.h;
                if (S.per_site) {
                    p.load_site(S, s, NC);
                    hr = h_site(S, p, s + 1 < S.nx * S.ny ? s + 1 : s);
                    hl = h_site(S, p, s > 0 ? s - 1 : s);
                    hu = h_site(S, p, gj + 1 < S.ny ? s + S.nx : s);
                    hd = h_site(S, p, gj > 0 ? s - S.nx : s);
                }
                T g[2 + 2 * NC];
                if constexpr (FFPacked<T, NC>::v) {
                    PairParams<T> pp;
                    pp.set(p);
                    site_gradient_pair<T>(pair_view_tile(t, lx + 1, ly + 1), p, pp, w, hr, hl, hu, hd, f.maxwell,
                                          S.thin_film, g);
                } else {
                    site_gradient<T, NC, TYT>(t, lx + 1, ly + 1, p, w, hr, hl, hu, hd, f.maxwell, S.thin_film, g);
                }
                if (GradLean<T>::v)
#pragma unroll
                    for (int c = 0; c < 1 + NC; ++c) gold[r][c] = loadw<T>(gprev[c] + s);
#pragma unroll
                for (int c = 0; c < 1 + NC; ++c) {
                    V gv;
                    gv.x = g[2 * c];
                    gv.y = g[2 * c + 1];
                    storew<T>(gcur[c] + s, gv);
                    const V go = gold[r][c];
                    v[0] += gv.x * gv.x + gv.y * gv.y;
                    v[1] += gv.x * (gv.x - go.x) + gv.y * (gv.y - go.y);
                }
            }
        }
        const int tpi = S.tiles_x * S.tiles_y;
        double tot[2];
        if (finish_image<2>(v, red, sc, part_slot(S, tr), S.tile_base + tr.n * tpi, tpi, img, tot) && threadIdx.x == 0) {
            (f.gcur ? sc.gn1 : sc.gn0)[img] = tot[0];
            sc.gdg[img] = tot[1];
            double beta = 0.0;
            if (f.use_cg) {
                beta = tot[1] / (f.gprev ? sc.gn1 : sc.gn0)[img];
                beta = beta > 0.0 ? beta : 0.0;   // Polak-Ribiere clipped at 0; NaN -> 0
            }
            sc.beta[img] = beta;
        }
        __syncthreads();
    }
}

template <class T, int NC>
__global__ void __launch_bounds__(NT, MinBlocks<T>::dir) k_dir_poly(const __grid_constant__ Batch bt,
                                                 const TileRef *__restrict__ tiles, int n_tiles, Scalars sc,
                                                 StepFlags f)
{
    constexpr int TYT = TileRows<T>::v;
    __shared__ Tile<T, NC, TYT> tx;
    __shared__ Tile<T, NC, TYT> td;
    // raw gradient tile of the all-asynchronous FP32 variant (16 bytes otherwise)
    constexpr bool DIR_ASYNC = MEPGL_DIR_ASYNC && !MEPGL_SPLIT_DIR && std::is_same<T, float>::value;
    __shared__ __align__(16) unsigned char g_raw[DIR_ASYNC ? sizeof(TileF<T, NC, TYT>) : 16];
    __shared__ double red[NT / 32 * 5];
    __shared__ double coef[5];
    for (int tt = blockIdx.x; tt < n_tiles; tt += gridDim.x) {
        const TileRef tr = tiles[tt];
        const StringDesc &S = bt.s[tr.s];
        const int img = S.img_base + tr.n;
        const int i0 = tr.tx * TX, j0 = tr.ty * TYT;
        const size_t off = (size_t)tr.n * S.nx * S.ny;
        ImagePtrs<T, NC> ipx, ipd;
        image_ptrs<T, NC>(ipx, S.x[f.xout], nullptr, nullptr, off);
        image_ptrs<T, NC>(ipd, S.d[f.din], S.g[f.gcur], S.d[f.dout], off);
        if constexpr (std::is_same<T, ff>::value) {
            // float-float tiles are staged through registers
            stage<T, NC, TYT, 0, XPairs<T>::v>(tx, S, ipx, i0, j0, (T)0, false, true);
#if MEPGL_SPLIT_DIR
            ImagePtrs<T, NC> ipn;
            image_ptrs<T, NC>(ipn, S.d[f.dout], nullptr, nullptr, off);
            stage<T, NC, TYT, 0, true>(td, S, ipn, i0, j0, (T)0, false, false);
#else
            stage<T, NC, TYT, 2, true, true>(td, S, ipd, i0, j0, (T)sc.beta[img], true, false);
#endif
        } else {
            uint16_t codes[((TYT + 2) * (TX + 2) + NT - 1) / NT];
            stage_async<T, NC, TYT>(tx, S, ipx.in, i0, j0, codes);
            if constexpr (DIR_ASYNC) {
                TileF<T, NC, TYT> &tg = *reinterpret_cast<TileF<T, NC, TYT> *>(g_raw);
                stage_async<T, NC, TYT>(tg, S, ipd.aux, i0, j0, nullptr);
                stage_async<T, NC, TYT>(td, S, ipd.in, i0, j0, nullptr);
                store_codes<T, NC, TYT>(tx, codes);
                cp_async_wait_all();
                __syncthreads();
                // d <- -g + beta d over the halo tile; interior d -> d[dout]
                using V = vec2_t<T>;
                constexpr int HW = TX + 2, HE = (TYT + 2) * HW, NI = (HE + NT - 1) / NT;
                const T beta = (T)sc.beta[img];
#pragma unroll
                for (int k = 0; k < NI; ++k) {
                    const int e = threadIdx.x + k * NT;
                    if (e >= HE) continue;
                    const int hy = e / HW, hx = e - hy * HW;
                    V v[1 + NC];
                    {
                        const V gv = tg.A[hy][hx], dv = td.A[hy][hx];
                        v[0].x = -gv.x + beta * dv.x;
                        v[0].y = -gv.y + beta * dv.y;
                        td.A[hy][hx] = v[0];
                    }
#pragma unroll
                    for (int c = 0; c < NC; ++c) {
                        const V gv = tg.P[c][hy][hx], dv = td.P[c][hy][hx];
                        v[1 + c].x = -gv.x + beta * dv.x;
                        v[1 + c].y = -gv.y + beta * dv.y;
                        td.P[c][hy][hx] = v[1 + c];
                    }
                    const int gi = i0 + hx - 1, gj = j0 + hy - 1;
                    if (hx >= 1 && hx <= TX && hy >= 1 && hy <= TYT && gi < S.nx && gj < S.ny)
#pragma unroll
                        for (int c = 0; c < 1 + NC; ++c) ipd.out[c][gi + S.nx * gj] = v[c];
                }
            } else {
#if MEPGL_SPLIT_DIR
            const vec2_t<T> *dsrc[1 + NC];
#pragma unroll
            for (int c = 0; c < 1 + NC; ++c) dsrc[c] = ipd.out[c];
            stage_async<T, NC, TYT>(td, S, dsrc, i0, j0, nullptr);
#else
            stage<T, NC, TYT, 2, true, true>(td, S, ipd, i0, j0, (T)sc.beta[img], true, false);
#endif
            store_codes<T, NC, TYT>(tx, codes);
            cp_async_wait_all();
            }
        }
        SiteParams<T> p;
        p.load_uniform(S);
        __syncthreads();
        T v[5] = {(T)0, (T)0, (T)0, (T)0, (T)0};
        const int lx = threadIdx.x & 31, gi = i0 + lx;
#pragma unroll
        for (int r = 0; r < TYT / 8; ++r) {
            const int ly = (threadIdx.x >> 5) + 8 * r, gj = j0 + ly;
            if (gi < S.nx && gj < S.ny) {
                Wts<T> w;
                w.load(tx.m[ly + 1][lx + 1]);
                if (S.per_site) p.load_site(S, gi + S.nx * gj, NC);
                T o[5];
                if constexpr (FFPacked<T, NC>::v) {
                    PairParams<T> pp;
                    pp.set(p);
                    site_poly_pair<T>(pair_view_tile(tx, lx + 1, ly + 1), pair_view_tile(td, lx + 1, ly + 1), p, pp,
                                      w, f.poly_compat, S.thin_film, o);
                } else {
                    site_poly<T, NC, TYT>(tx, td, lx + 1, ly + 1, p, w, f.poly_compat, S.thin_film, o);
                }
#pragma unroll
                for (int k = 0; k < 5; ++k) v[k] += o[k];
            }
        }
        const int tpi = S.tiles_x * S.tiles_y;
        double tot[5];
        if (finish_image<5>(v, red, sc, part_slot(S, tr), S.tile_base + tr.n * tpi, tpi, img, tot)) {
            if (threadIdx.x == 0) {
#pragma unroll
                for (int k = 0; k < 5; ++k) coef[k] = tot[k];
                sc.fenergy[img] = tot[0];
#pragma unroll
                for (int k = 0; k < 4; ++k) sc.poly[4 * img + k] = tot[1 + k];
            }
            __syncthreads();
            if (threadIdx.x < 32) {
                // the scan's grid and rounding follow the stored precision
                const double *xt = sizeof(store_t<T>) == 8 ? sc.xtab_d : sc.xtab_f;
                double alpha = line_search_scan<store_t<T>>(coef, xt);
                if (f.ls_exact) alpha = line_search_exact(coef, alpha);
                if (threadIdx.x == 0) {
                    sc.alpha[img] = alpha;
                    sc.alpha_pend[img] = alpha;
                }
            }
        }
        __syncthreads();
    }
}

#include "strip.cuh"

// d[dout] = -g + beta d[din] at every site of the launch's tiles (the
// pointwise half of computeStepDirection, nlcg.cu:955-994, when the
// direction and polynomial passes are split).
template <class T, int NC>
__global__ void __launch_bounds__(NT) k_dir_update(const __grid_constant__ Batch bt,
                                                   const TileRef *__restrict__ tiles, int n_tiles, Scalars sc,
                                                   StepFlags f)
{
    constexpr int TYT = TileRows<T>::v;
    using V = vec2_t<T>;
    for (int tt = blockIdx.x; tt < n_tiles; tt += gridDim.x) {
        const TileRef tr = tiles[tt];
        const StringDesc &S = bt.s[tr.s];
        const T beta = (T)sc.beta[S.img_base + tr.n];
        const size_t off = (size_t)tr.n * S.nx * S.ny;
        const int gi = tr.tx * TX + (threadIdx.x & 31);
        V gv[TYT / 8][1 + NC], dv[TYT / 8][1 + NC];
#pragma unroll
        for (int r = 0; r < TYT / 8; ++r) {
            const int gj = tr.ty * TYT + (threadIdx.x >> 5) + 8 * r;
            if (gi < S.nx && gj < S.ny)
#pragma unroll
                for (int c = 0; c < 1 + NC; ++c) {
                    const int s = gi + S.nx * gj;
                    using W = vec2_t<store_t<T>>;
                    gv[r][c] = loadw<T>(static_cast<const W *>(S.g[f.gcur][c]) + off + s);
                    dv[r][c] = loadw<T>(static_cast<const W *>(S.d[f.din][c]) + off + s);
                }
        }
#pragma unroll
        for (int r = 0; r < TYT / 8; ++r) {
            const int gj = tr.ty * TYT + (threadIdx.x >> 5) + 8 * r;
            if (gi < S.nx && gj < S.ny)
#pragma unroll
                for (int c = 0; c < 1 + NC; ++c) {
                    V v;
                    v.x = -gv[r][c].x + beta * dv[r][c].x;
                    v.y = -gv[r][c].y + beta * dv[r][c].y;
                    storew<T>(static_cast<vec2_t<store_t<T>> *>(S.d[f.dout][c]) + off + gi + S.nx * gj, v);
                }
        }
    }
}

template <class T, int NC>
__global__ void __launch_bounds__(NT) k_energy(const __grid_constant__ Batch bt, const TileRef *__restrict__ tiles,
                                               int n_tiles, Scalars sc, int xbuf, double *out)
{
    constexpr int TYT = TileRows<T>::v;
    __shared__ Tile<T, NC, TYT> t;
    __shared__ double red[NT / 32];
    for (int tt = blockIdx.x; tt < n_tiles; tt += gridDim.x) {
        // without a tile table: one string, tiles in (image, row, column) order
        const TileRef tr = tiles ? tiles[tt] : flat_tile(bt.s[0], tt);
        const StringDesc &S = bt.s[tr.s];
        const int img = S.img_base + tr.n;
        const int i0 = tr.tx * TX, j0 = tr.ty * TYT;
        ImagePtrs<T, NC> ip;
        image_ptrs<T, NC>(ip, S.x[xbuf], nullptr, nullptr, (size_t)tr.n * S.nx * S.ny);
        stage<T, NC, TYT, 0>(t, S, ip, i0, j0, (T)0, false, true);
        SiteParams<T> p;
        p.load_uniform(S);
        __syncthreads();
        T v[1] = {(T)0};
        const int lx = threadIdx.x & 31, gi = i0 + lx;
#pragma unroll
        for (int r = 0; r < TYT / 8; ++r) {
            const int ly = (threadIdx.x >> 5) + 8 * r, gj = j0 + ly;
            if (gi < S.nx && gj < S.ny) {
                Wts<T> w;
                w.load(t.m[ly + 1][lx + 1]);
                if (S.per_site) p.load_site(S, gi + S.nx * gj, NC);
                v[0] += S.disc ? site_energy_link<T, NC, TYT>(t, lx + 1, ly + 1, p, w, S.thin_film)
                               : site_energy<T, NC, TYT>(t, lx + 1, ly + 1, p, w, S.thin_film);
            }
        }
        const int tpi = S.tiles_x * S.tiles_y;
        double tot[1];
        if (finish_image<1>(v, red, sc, part_slot(S, tr), S.tile_base + tr.n * tpi, tpi, img, tot) && threadIdx.x == 0)
            out[img] = tot[0];
        __syncthreads();
    }
}

// Per-image dF/dH, dF/deta, dF/dgamma at fixed fields (out[3 img + k]).
template <class T, int NC>
__global__ void __launch_bounds__(NT) k_param_adjoint(const __grid_constant__ Batch bt,
                                                      const TileRef *__restrict__ tiles, int n_tiles, Scalars sc,
                                                      int xbuf, double *out)
{
    constexpr int TYT = TileRows<T>::v;
    __shared__ Tile<T, NC, TYT> t;
    __shared__ double red[NT / 32 * 3];
    for (int tt = blockIdx.x; tt < n_tiles; tt += gridDim.x) {
        const TileRef tr = tiles[tt];
        const StringDesc &S = bt.s[tr.s];
        const int img = S.img_base + tr.n;
        const int i0 = tr.tx * TX, j0 = tr.ty * TYT;
        ImagePtrs<T, NC> ip;
        image_ptrs<T, NC>(ip, S.x[xbuf], nullptr, nullptr, (size_t)tr.n * S.nx * S.ny);
        stage<T, NC, TYT, 0>(t, S, ip, i0, j0, (T)0, false, true);
        SiteParams<T> p;
        p.load_uniform(S);
        __syncthreads();
        T v[3] = {(T)0, (T)0, (T)0};
        const int lx = threadIdx.x & 31, gi = i0 + lx;
#pragma unroll
        for (int r = 0; r < TYT / 8; ++r) {
            const int ly = (threadIdx.x >> 5) + 8 * r, gj = j0 + ly;
            if (gi < S.nx && gj < S.ny) {
                Wts<T> w;
                w.load(t.m[ly + 1][lx + 1]);
                if (S.per_site) p.load_site(S, gi + S.nx * gj, NC);
                if (S.disc) {
                    T u[3] = {(T)0, v[1], v[2]};
                    site_param_adjoint<T, NC, TYT>(t, lx + 1, ly + 1, p, w, 1, u);
                    v[1] = u[1];
                    v[2] = u[2];
                    if (!S.thin_film) v[0] += site_dh_link<T, NC, TYT>(t, lx + 1, ly + 1, p, w);
                } else {
                    site_param_adjoint<T, NC, TYT>(t, lx + 1, ly + 1, p, w, S.thin_film, v);
                }
            }
        }
        const int tpi = S.tiles_x * S.tiles_y;
        double tot[3];
        if (finish_image<3>(v, red, sc, part_slot(S, tr), S.tile_base + tr.n * tpi, tpi, img, tot) &&
            threadIdx.x == 0) {
            out[3 * img] = tot[0];
            out[3 * img + 1] = tot[1];
            out[3 * img + 2] = tot[2];
        }
        __syncthreads();
    }
}

template <class T, int NC>
__global__ void __launch_bounds__(NT) k_gradient_only(const __grid_constant__ Batch bt,
                                                      const TileRef *__restrict__ tiles, int n_tiles, int xbuf,
                                                      FieldPtrs out, int maxwell)
{
    constexpr int TYT = TileRows<T>::v;
    using V = vec2_t<T>;
    __shared__ Tile<T, NC, TYT> t;
    for (int tt = blockIdx.x; tt < n_tiles; tt += gridDim.x) {
        const TileRef tr = tiles[tt];
        const StringDesc &S = bt.s[tr.s];
        const int i0 = tr.tx * TX, j0 = tr.ty * TYT;
        const size_t off = (size_t)tr.n * S.nx * S.ny;
        ImagePtrs<T, NC> ip;
        image_ptrs<T, NC>(ip, S.x[xbuf], nullptr, nullptr, off);
        stage<T, NC, TYT, 0>(t, S, ip, i0, j0, (T)0, false, true);
        SiteParams<T> p;
        p.load_uniform(S);
        __syncthreads();
        const int lx = threadIdx.x & 31, gi = i0 + lx;
#pragma unroll
        for (int r = 0; r < TYT / 8; ++r) {
            const int ly = (threadIdx.x >> 5) + 8 * r, gj = j0 + ly;
            if (gi < S.nx && gj < S.ny) {
                const int s = gi + S.nx * gj;
                Wts<T> w;
                w.load(t.m[ly + 1][lx + 1]);
                T hr = p.h, hl = p.h, hu = p.h, hd = p.h;
                if (S.per_site) {
                    p.load_site(S, s, NC);
                    hr = h_site(S, p, s + 1 < S.nx * S.ny ? s + 1 : s);
                    hl = h_site(S, p, s > 0 ? s - 1 : s);
                    hu = h_site(S, p, gj + 1 < S.ny ? s + S.nx : s);
                    hd = h_site(S, p, gj > 0 ? s - S.nx : s);
                }
                T g[2 + 2 * NC];
                if constexpr (std::is_same<T, ff>::value) {   // float-float: the reference form only
                    site_gradient<T, NC, TYT>(t, lx + 1, ly + 1, p, w, hr, hl, hu, hd, maxwell, S.thin_film, g);
                } else if (S.disc) {
                    T hmx_l[2] = {p.hmx[0], p.hmx[1]}, hmy_d[2] = {p.hmy[0], p.hmy[1]};
                    if (S.per_site)
                        for (int c = 0; c < NC; ++c) {
                            if (gi > 0) hmx_l[c] = (T)0.5 / static_cast<const T *>(S.pmxx[c])[s - 1];
                            if (gj > 0) hmy_d[c] = (T)0.5 / static_cast<const T *>(S.pmyy[c])[s - S.nx];
                        }
                    site_gradient_link<T, NC, TYT>(t, lx + 1, ly + 1, p, w, hl, hd, hmx_l, hmy_d, maxwell,
                                                   S.thin_film, g);
                } else {
                    site_gradient<T, NC, TYT>(t, lx + 1, ly + 1, p, w, hr, hl, hu, hd, maxwell, S.thin_film, g);
                }
#pragma unroll
                for (int c = 0; c < 1 + NC; ++c) {
                    V gv;
                    gv.x = g[2 * c];
                    gv.y = g[2 * c + 1];
                    store2<T>(static_cast<vec2_t<store_t<T>> *>(out.p[c]) + off + s, gv);
                }
            }
        }
        __syncthreads();
    }
}

template <class T, int NC>
__global__ void __launch_bounds__(NT) k_jb(const __grid_constant__ Batch bt, const TileRef *__restrict__ tiles,
                                           int n_tiles, int xbuf, T *b, vec2_t<T> *j1, vec2_t<T> *j2)
{
    constexpr int TYT = TileRows<T>::v;
    using V = vec2_t<T>;
    __shared__ Tile<T, NC, TYT> t;
    for (int tt = blockIdx.x; tt < n_tiles; tt += gridDim.x) {
        const TileRef tr = tiles[tt];
        const StringDesc &S = bt.s[tr.s];
        const int i0 = tr.tx * TX, j0 = tr.ty * TYT;
        const size_t off = (size_t)tr.n * S.nx * S.ny;
        ImagePtrs<T, NC> ip;
        image_ptrs<T, NC>(ip, S.x[xbuf], nullptr, nullptr, off);
        stage<T, NC, TYT, 0>(t, S, ip, i0, j0, (T)0, false, true);
        SiteParams<T> p;
        p.load_uniform(S);
        __syncthreads();
        const int lx = threadIdx.x & 31, gi = i0 + lx;
#pragma unroll
        for (int r = 0; r < TYT / 8; ++r) {
            const int ly = (threadIdx.x >> 5) + 8 * r, gj = j0 + ly;
            if (gi < S.nx && gj < S.ny) {
                const size_t k = off + gi + (size_t)S.nx * gj;
                Wts<T> w;
                w.load(t.m[ly + 1][lx + 1]);
                if (S.per_site) p.load_site(S, gi + S.nx * gj, NC);
                T o[1 + 2 * NC];
                site_jb<T, NC, TYT>(t, lx + 1, ly + 1, p, w, o);
                b[k] = o[0];
                V v;
                v.x = o[1];
                v.y = o[2];
                j1[k] = v;
                if (NC == 2) {
                    v.x = o[3];
                    v.y = o[4];
                    j2[k] = v;
                }
            }
        }
        __syncthreads();
    }
}

// x += alpha_pend[image] d over one image per blockIdx.y.  W: the compute
// type of the NLCG passes that wrote d (ff: d holds float-float pairs, the
// update runs in double on their values).
template <class T, class W = T>
__global__ void __launch_bounds__(NT) k_apply_update(vec2_t<T> *x, const vec2_t<T> *d, const double *alpha_pend,
                                                     long M)
{
    const T a = (T)alpha_pend[blockIdx.y];
    if (a == (T)0) return;
    const long off = (long)blockIdx.y * M;
    for (long p = blockIdx.x * (long)NT + threadIdx.x; p < M; p += (long)gridDim.x * NT) {
        vec2_t<T> v = x[off + p];
        vec2_t<T> dd;
        if constexpr (std::is_same<W, ff>::value) {
            const ff2 w = loadw<ff>(d + off + p);
            dd.x = to_double(w.x);
            dd.y = to_double(w.y);
        } else {
            dd = d[off + p];
        }
        v.x = v.x + a * dd.x;
        v.y = v.y + a * dd.y;
        x[off + p] = v;
    }
}

// Fields x between double pairs and float-float pairs, in place (an ff2
// fills the 16 bytes of a double2).  A double holds a float-float pair that
// the passes wrote exactly, so a round trip returns the same doubles.
template <bool TO_PAIRS>
__global__ void __launch_bounds__(NT) k_x_format(double2 *x, long n)
{
    for (long i = blockIdx.x * (long)NT + threadIdx.x; i < n; i += (long)gridDim.x * NT) {
        if (TO_PAIRS) {
            const double2 v = x[i];
            ff2 w;
            w.x = to_ff(v.x);
            w.y = to_ff(v.y);
            storew<ff>(x + i, w);
        } else {
            const ff2 w = loadw<ff>(x + i);
            x[i] = make_double2(to_double(w.x), to_double(w.y));
        }
    }
}

// Arc length: squared image-to-image distance over every site (no mask, no
// dx^2; interpolation.cu:39-92).  Block (bx, n) covers sites
// [bx * NT * ARC_SPT, ...) of image n against image n - 1: each thread issues
// all its loads of both images, then adds them in the fixed order (site,
// field, component), so each (image, site block) partial is the same sum
// one walk through the images would give.
constexpr int ARC_SPT = 4;

template <class T>
__global__ void __launch_bounds__(NT) k_arc_partial(const T *__restrict__ f0, const T *__restrict__ f1,
                                                    const T *__restrict__ f2, int w0, int w1, int w2, long sites,
                                                    double *part)
{
    __shared__ double red[NT / 32];
    const T *fs[3] = {f0, f1, f2};
    const int ws[3] = {w0, w1, w2};
    const int n = blockIdx.y;
    const long base = (long)blockIdx.x * NT * ARC_SPT + threadIdx.x;
    T acc = 0;
    if (n > 0) {
        T cur[3][ARC_SPT][2], prv[3][ARC_SPT][2];
#pragma unroll
        for (int f = 0; f < 3; ++f)
#pragma unroll
            for (int q = 0; q < ARC_SPT; ++q) {
                const long s = base + (long)q * NT;
                cur[f][q][0] = cur[f][q][1] = prv[f][q][0] = prv[f][q][1] = 0;
                if (!fs[f] || s >= sites) continue;
                if (ws[f] == 2) {   // one vector load per site and image
                    const vec2_t<T> *v = reinterpret_cast<const vec2_t<T> *>(fs[f]);
                    const vec2_t<T> c = v[(long)n * sites + s], p = v[(long)(n - 1) * sites + s];
                    cur[f][q][0] = c.x;
                    cur[f][q][1] = c.y;
                    prv[f][q][0] = p.x;
                    prv[f][q][1] = p.y;
                } else {
                    cur[f][q][0] = fs[f][(long)n * sites + s];
                    prv[f][q][0] = fs[f][(long)(n - 1) * sites + s];
                }
            }
#pragma unroll
        for (int q = 0; q < ARC_SPT; ++q) {
            if (base + (long)q * NT >= sites) continue;
            T d2 = 0;
#pragma unroll
            for (int f = 0; f < 3; ++f) {
                if (!fs[f]) continue;
#pragma unroll
                for (int w = 0; w < 2; ++w) {
                    if (w >= ws[f]) continue;
                    d2 += (cur[f][q][w] - prv[f][q][w]) * (cur[f][q][w] - prv[f][q][w]);
                }
            }
            acc += d2;
        }
    }
    const T vv[1] = {acc};
    double tot[1];
    block_sum<1>(vv, tot, red);
    if (threadIdx.x == 0) part[(size_t)n * gridDim.x + blockIdx.x] = tot[0];
}

// ------------------------------------------------------- initial strings
// Counter-based Gaussian noise: Philox4x32-10 (Salmon, Moraes, Dror and
// Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC 2011) keyed by the
// seed and counted by (image, site, component), then Box-Muller.  Each site
// draws the same numbers whatever the launch shape.
__device__ __forceinline__ void philox_round(uint32_t (&c)[4], uint32_t (&k)[2])
{
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0], p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t h0 = (uint32_t)(p0 >> 32), l0 = (uint32_t)p0, h1 = (uint32_t)(p1 >> 32), l1 = (uint32_t)p1;
    c[0] = h1 ^ c[1] ^ k[0];
    c[1] = l1;
    c[2] = h0 ^ c[3] ^ k[1];
    c[3] = l0;
    k[0] += 0x9E3779B9u;
    k[1] += 0xBB67AE85u;
}

__device__ __forceinline__ void philox4x32_10(uint32_t (&c)[4], uint64_t seed)
{
    uint32_t k[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
#pragma unroll
    for (int r = 0; r < 10; ++r) philox_round(c, k);
}

// two standard normals from the counter (n, s, component)
__device__ __forceinline__ void normal_pair(uint64_t seed, int n, long s, int comp, double &z0, double &z1)
{
    uint32_t c[4] = {(uint32_t)s, (uint32_t)((unsigned long long)s >> 32), (uint32_t)n, (uint32_t)comp};
    philox4x32_10(c, seed);
    // 53-bit uniforms in (0, 1]
    const double u1 = ((double)(((uint64_t)c[0] << 21) ^ (c[1] >> 11)) + 1.0) * 0x1.0p-53;
    const double u2 = (double)(((uint64_t)c[2] << 21) ^ (c[3] >> 11)) * 0x1.0p-53;
    const double r = sqrt(-2.0 * log(u1));
    double sn, cs;
    sincospi(2.0 * u2, &sn, &cs);
    z0 = r * cs;
    z1 = r * sn;
}

// The initial guess of the reference's StringBuilder (builder.py:107-189)
// for every image at once: per component |psi| = psi_abs * prod_v f(r_v),
// theta = sum_v w_v atan2(y - y_v, x - x_v) over the vortex tracks with a
// nonzero winding in that image, plus N(0, noise^2) on Re and Im, times the
// superconducting domain; A from the gauge of B_z times the computational
// domain.  f = tanh(-r^2) (the builder's profile) or tanh(r / sqrt 2).
// tracks: n_tracks x F x {x, y, winding, component} doubles.
template <class T>
__global__ void k_generate(vec2_t<T> *a, vec2_t<T> *p1, vec2_t<T> *p2, int nx, int ny, int F, int ncomp,
                           const int32_t *comp, const int32_t *sc, const double *tracks, int n_tracks, GuessParams g)
{
    const long M = (long)nx * ny;
    for (long e = blockIdx.x * (long)NT + threadIdx.x; e < M * F; e += (long)gridDim.x * NT) {
        const int n = (int)(e / M);
        const long s = e - (long)n * M;
        const int i = (int)(s % nx), j = (int)(s / nx);
        const double x = g.x0 + i * g.dx, y = g.y0 + j * g.dx;
        const double cm = comp[s] ? 1.0 : 0.0, scm = sc[s] ? 1.0 : 0.0;
        vec2_t<T> av;
        double ax = 0.0, ay = 0.0;
        if (g.gauge == 1) ax = -g.b_z * y;
        else if (g.gauge == 2) ay = g.b_z * x;
        else if (g.gauge == 3) { ax = -0.5 * g.b_z * y; ay = 0.5 * g.b_z * x; }
        av.x = (T)(ax * cm);
        av.y = (T)(ay * cm);
        a[e] = av;
        for (int c = 0; c < ncomp; ++c) {
            double mag = c == 0 ? g.psi_abs_1 : g.psi_abs_2, th = 0.0;
            for (int v = 0; v < n_tracks; ++v) {
                const double *t = tracks + ((size_t)v * F + n) * 4;
                if ((int)t[3] != c + 1 || t[2] == 0.0) continue;
                const double dxv = x - t[0], dyv = y - t[1], r2 = dxv * dxv + dyv * dyv;
                mag *= g.profile == 0 ? tanh(-r2) : tanh(sqrt(r2) * 0.70710678118654752440);
                th += t[2] * atan2(dyv, dxv);
            }
            double z0 = 0.0, z1 = 0.0;
            if (g.noise != 0.0) normal_pair(g.seed, n, s, c, z0, z1);
            double sn, cs;
            sincos(th, &sn, &cs);
            vec2_t<T> pv;
            pv.x = (T)((mag * cs + g.noise * z0) * scm);
            pv.y = (T)((mag * sn + g.noise * z1) * scm);
            (c == 0 ? p1 : p2)[e] = pv;
        }
    }
}

// Magnetic flux of every image: Phi_n = dx^2 sum_sites B (post.py:131-133);
// one block per image, double sums in a fixed order.
template <class T>
__global__ void k_flux(const T *__restrict__ b, long M, int F, double dx2, double *out)
{
    __shared__ double red[NT / 32];
    for (int n = blockIdx.x; n < F; n += gridDim.x) {
        const T *bn = b + (size_t)n * M;
        double v[1] = {0.0};
        for (long s = threadIdx.x; s < M; s += NT) v[0] += (double)bn[s];
        double tot[1];
        block_sum<1>(v, tot, red);
        if (threadIdx.x == 0) out[n] = tot[0] * dx2;
    }
}

// Winding sum of one field per image (compute_winding, gl_utils.py:10-41):
// around the rectangle `inset` sites inside the lattice edge, counter-
// clockwise from the lower-left corner, sum of the linearised phase steps
// (u dv - v du) / (u^2 + v^2) taken at the start of each step (2 pi per
// vortex enclosed, approximately).  The loop visits (W - 1) steps along
// each horizontal side and (H - 1) along each vertical side.
template <class T>
__global__ void k_winding(const vec2_t<T> *__restrict__ psi, int nx, int ny, int F, int inset, double *out)
{
    __shared__ double red[NT / 32];
    const int W = nx - 2 * inset, H = ny - 2 * inset, i0 = inset, j0 = inset, i1 = nx - 1 - inset,
              j1 = ny - 1 - inset;
    const int L = 2 * (W - 1) + 2 * (H - 1);
    for (int n = blockIdx.x; n < F; n += gridDim.x) {
        const vec2_t<T> *pn = psi + (size_t)n * nx * ny;
        double v[1] = {0.0};
        for (int t = threadIdx.x; t < L; t += NT) {
            int ia, ja, ib, jb;
            if (t < W - 1) {
                ia = i0 + t; ja = j0; ib = ia + 1; jb = ja;
            } else if (t < (W - 1) + (H - 1)) {
                const int k = t - (W - 1);
                ia = i1; ja = j0 + k; ib = ia; jb = ja + 1;
            } else if (t < 2 * (W - 1) + (H - 1)) {
                const int k = t - (W - 1) - (H - 1);
                ia = i1 - k; ja = j1; ib = ia - 1; jb = ja;
            } else {
                const int k = t - 2 * (W - 1) - (H - 1);
                ia = i0; ja = j1 - k; ib = ia; jb = ja - 1;
            }
            const vec2_t<T> a = pn[ia + (size_t)nx * ja], b = pn[ib + (size_t)nx * jb];
            const double u = a.x, w = a.y, du = (double)b.x - u, dv = (double)b.y - w;
            v[0] += (u * dv - w * du) / (u * u + w * w);
        }
        double tot[1];
        block_sum<1>(v, tot, red);
        if (threadIdx.x == 0) out[n] = tot[0];
    }
}

// computeArcLength (interpolation.cu:126-140), first half: block n adds
// image n's partials.
__global__ void k_arc_sum(const double *part, int nblocks, double *s)
{
    __shared__ double red[NT / 32];
    const int n = blockIdx.x;
    double v[1] = {0.0};
    for (int b = threadIdx.x; b < nblocks; b += NT) v[0] += part[(size_t)n * nblocks + b];
    double tot[1];
    block_sum<1>(v, tot, red);
    if (threadIdx.x == 0) s[n] = tot[0];
}

// Second half: cumulative sqrt, normalised so that s[F-1] = 1.  The square
// roots and the divisions (slow in FP64 here) run across the block; one
// thread adds in image order.  Strings of more than ARC_CUM_MAX images run
// it all in one thread.
//
// A string of zero or non-finite length (all images equal, or a non-finite
// field) has no arc length: the reference divides 0 by 0 there
// (interpolation.cu:126-140).  Here *bad is set and s becomes the uniform
// n / (F - 1), computed as the resample plan computes its output positions,
// so that a linear resample onto as many images copies every image exactly;
// the host reports the flag as an error.
constexpr int ARC_CUM_MAX = 4096;

__device__ __forceinline__ bool arc_total_ok(double t) { return t > 0.0 && t <= 1.7976931348623157e308; }

__global__ void k_arc_cumulate(int F, double *s, int *bad)
{
    __shared__ double r[ARC_CUM_MAX];
    __shared__ double total;
    if (F == 1) {     // a single image has no length to normalise
        if (threadIdx.x == 0) s[0] = 0.0;
        return;
    }
    if (F > ARC_CUM_MAX) {
        if (threadIdx.x == 0) {
            double acc = 0.0;
            s[0] = 0.0;
            for (int n = 1; n < F; ++n) {
                acc += sqrt(s[n]);
                s[n] = acc;
            }
            const bool ok = arc_total_ok(acc);
            if (!ok) atomicExch(bad, 1);
            for (int n = 0; n < F; ++n) s[n] = ok ? s[n] / acc : (double)n / (double)(F - 1);
        }
        return;
    }
    for (int n = threadIdx.x; n < F; n += blockDim.x) r[n] = n == 0 ? 0.0 : sqrt(s[n]);
    __syncthreads();
    if (threadIdx.x == 0) {
        double acc = 0.0;
        for (int n = 1; n < F; ++n) {
            acc += r[n];
            r[n] = acc;
        }
        total = acc;
        if (!arc_total_ok(acc)) atomicExch(bad, 1);
    }
    __syncthreads();
    const bool ok = arc_total_ok(total);
    for (int n = threadIdx.x; n < F; n += blockDim.x) s[n] = ok ? r[n] / total : (double)n / (double)(F - 1);
}

// Finiteness of the per-image scalars after a call's NLCG steps: the energy
// (constant term of the last line polynomial) and |g|^2 of the slot the
// last step wrote.  A NaN or infinite value (from non-finite fields, or a
// step that overflowed) counts into status[1]; status[2] keeps the first
// such image + 1.  The host reports them at its next synchronising call.
__global__ void k_check_scalars(const double *fenergy, const double *gn, int n_images, int *status)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= n_images) return;
    const double e = fenergy[n], g = gn[n];
    const double big = 1.7976931348623157e308;
    if (!(fabs(e) <= big) || !(g <= big)) {
        atomicAdd(status + 1, 1);
        atomicCAS(status + 2, 0, n + 1);
    }
}

// Redistribution plan: segment and weight per output image, and for the
// cubic spline the Forsythe-Malcolm-Moler matrix (buildHMatrix,
// interpolation.cu:252-290) factorised once by Gaussian elimination with
// partial pivoting (the LAPACK gtsv algorithm) for every site's system.
// One block of 32 threads.  The segment walk and the elimination are
// sequential (thread 0); everything that is not (differences h, output
// positions, weights, and the reciprocals and per-image coefficients that
// spare the cubic resample its divisions) is spread over the block, because
// every FP64 division and square root is slow on this GPU.  The arrays live
// in shared memory when they fit, else in the plan's global arrays.

// Shared-memory bytes of the plan kernel: s, h, dl, d, du, du2 [F or F+1],
// output positions and segment starts [F_new] as doubles; ipiv [F] and the
// segments [F_new] as ints.
__host__ __device__ inline size_t redist_plan_smem(int F, int F_new)
{
    return (size_t)(6 * F + 1 + 2 * F_new) * sizeof(double) + (size_t)(F + F_new) * sizeof(int);
}

// Weight of the segment's end image.  A segment of zero length (two equal
// adjacent images, where the reference divides 0 by 0) takes its end image:
// both ends are the same state.
__device__ __forceinline__ double redist_weight(double num, double len) { return len != 0.0 ? num / len : 1.0; }

__global__ void k_redist_plan(const double *s_in, int F, int F_new, int cubic, int spline, RedistPlan p, int use_smem)
{
    if (blockIdx.x != 0) return;
    extern __shared__ double plan_sm[];
    const int t = threadIdx.x, nt = blockDim.x;
    const double *s = s_in;
    double *h = p.h, *dl = p.dl, *d = p.d, *du = p.du, *du2 = p.du2, *snew = nullptr, *sst = nullptr;
    int *ipiv = p.ipiv, *kk = p.k;
    if (use_smem) {
        double *ss = plan_sm;
        h = ss + F;
        dl = h + F + 1;
        d = dl + F;
        du = d + F;
        du2 = du + F;
        snew = du2 + F;
        sst = snew + F_new;
        ipiv = reinterpret_cast<int *>(sst + F_new);
        kk = ipiv + F;
        for (int n = t; n < F; n += nt) ss[n] = s_in[n];
        s = ss;
        __syncthreads();
    }
    // h[n] = s[n] - s[n-1]; output positions n / (F_new - 1)
    for (int n = t; n <= F; n += nt) h[n] = n == 0 ? 0.0 : (n == F ? INFINITY : s[n] - s[n - 1]);
    if (use_smem)
        for (int n = t; n < F_new; n += nt) snew[n] = (double)n / (double)(F_new - 1);
    __syncthreads();
    const bool walk_sum = cubic && spline == 0;
    if (t == 0) {
        // segment walk (comparisons and additions only when the positions are staged)
        int k = 1;
        double seg_start = 0.0, seg_end = walk_sum ? h[1] : s[1];
        for (int n = 0; n < F_new; ++n) {
            const double s_new = use_smem ? snew[n] : (double)n / (double)(F_new - 1);
            if (walk_sum) {
                while (seg_end < s_new) { k++; seg_start += h[k - 1]; seg_end += h[k]; }
            } else {
                while (seg_end < s_new && k < F - 1) { k++; seg_start = s[k - 1]; seg_end = s[k]; }
            }
            if (k >= F) k = F - 1;
            kk[n] = k;
            if (use_smem) sst[n] = seg_start;
            else p.w[n] = redist_weight(s_new - seg_start, cubic ? h[k] : (s[k] - s[k - 1]));
        }
    }
    __syncthreads();
    if (use_smem)
        for (int n = t; n < F_new; n += nt) {
            const int k = kk[n];
            p.k[n] = k;
            p.w[n] = redist_weight(snew[n] - sst[n], cubic ? h[k] : (s[k] - s[k - 1]));
        }
    if (!cubic) {
        if (use_smem)
            for (int n = t; n <= F; n += nt) p.h[n] = h[n];
        return;
    }
    if (t == 0) {
        for (int n = 0; n < F; ++n) { dl[n] = d[n] = du[n] = du2[n] = 0.0; ipiv[n] = 0; }
        d[0] = -h[1];
        du[0] = h[1];
        for (int n = 1; n < F - 1; ++n) { dl[n] = h[n]; d[n] = 2 * (h[n] + h[n + 1]); du[n] = h[n + 1]; }
        dl[F - 1] = h[F - 1];
        d[F - 1] = -h[F - 1];
        for (int q = 0; q < F - 1; ++q) {
            const double sub = dl[q + 1];
            if (fabs(d[q]) >= fabs(sub)) {
                if (d[q] != 0) {
                    const double l = sub / d[q];
                    dl[q + 1] = l;
                    d[q + 1] = d[q + 1] - l * du[q];
                } else {
                    dl[q + 1] = 0;
                }
            } else {
                const double l = d[q] / sub;
                d[q] = sub;
                dl[q + 1] = l;
                const double tmp = du[q];
                du[q] = d[q + 1];
                d[q + 1] = tmp - l * d[q + 1];
                if (q < F - 2) {
                    du2[q] = du[q + 1];
                    du[q + 1] = -l * du[q + 1];
                }
                ipiv[q] = 1;
            }
        }
        for (int q = 0; q < F; ++q)
            if (d[q] == 0 && p.status) *p.status = 1;
    }
    __syncthreads();
    // factors out (from shared memory), and the cubic resample's uniform coefficients
    double *rh = p.aux, *rd = rh + F, *ev = rd + F, *ends = ev + 4 * F_new;
    for (int n = t; n <= F; n += nt) {
        if (use_smem) p.h[n] = h[n];
        if (n == F) continue;
        if (use_smem) {
            p.dl[n] = dl[n];
            p.d[n] = d[n];
            p.du[n] = du[n];
            p.du2[n] = du2[n];
            p.ipiv[n] = ipiv[n];
        }
        rh[n] = n > 0 ? 1.0 / h[n] : 0.0;
        rd[n] = 1.0 / d[n];
    }
    for (int n = t; n < F_new; n += nt) {
        const int k = kk[n];
        const double w = p.w[n], wm = spline == 0 ? (w - 1) : (1 - w), hk2 = h[k] * h[k];
        ev[4 * n] = w;
        ev[4 * n + 1] = 1 - w;
        ev[4 * n + 2] = hk2 * (w * w * w - w);
        ev[4 * n + 3] = hk2 * (wm * wm * wm - wm);
    }
    if (t == 0) {   // end conditions: third divided differences at both ends
        ends[0] = 1.0 / (h[3] + h[2]);
        ends[1] = 1.0 / (h[2] + h[1]);
        ends[2] = 1.0 / (h[3] + h[2] + h[1]);
        ends[3] = h[1] * h[1];
        ends[4] = 1.0 / (h[F - 1] + h[F - 2]);
        ends[5] = 1.0 / (h[F - 2] + h[F - 3]);
        ends[6] = 1.0 / (h[F - 1] + h[F - 2] + h[F - 3]);
        ends[7] = -(h[F - 1] * h[F - 1]);
    }
}

// Linear resample: block row blockIdx.y is output image n, the blocks of the
// row stride over its reals, V of them per access (V = 4 for float fields
// whose image size allows 16-byte vectors, 2 for double, else 1).
template <class T, int V>
__global__ void __launch_bounds__(NT) k_redist_linear(const T *f, T *fnew, long reals, const int *kk, const double *ww)
{
    using Vec = typename std::conditional<V == 4, float4, typename std::conditional<V == 2, double2, T>::type>::type;
    const int n = blockIdx.y;
    const int k = kk[n];
    const T w = (T)ww[n];
    const Vec *a = reinterpret_cast<const Vec *>(f + (long)k * reals);
    const Vec *b = reinterpret_cast<const Vec *>(f + (long)(k - 1) * reals);
    Vec *o = reinterpret_cast<Vec *>(fnew + (long)n * reals);
    const long nv = reals / V;
    for (long i = blockIdx.x * (long)NT + threadIdx.x; i < nv; i += (long)gridDim.x * NT) {
        const Vec va = a[i], vb = b[i];
        const T *pa = reinterpret_cast<const T *>(&va), *pb = reinterpret_cast<const T *>(&vb);
        Vec vo;
        T *po = reinterpret_cast<T *>(&vo);
#pragma unroll
        for (int c = 0; c < V; ++c) po[c] = w * pa[c] + (1 - w) * pb[c];
        o[i] = vo;
    }
}

// Cubic resample (computeDeltaX/Y + gtsv + generateNewFramesCubic,
// interpolation.cu:292-402), one thread per real of a site: builds the
// right-hand side, solves with the shared factors, evaluates the new
// images.  The arithmetic type C is that of the fields: float for FP32
// fields, as the reference's FP32 build computes its spline, and double for
// FP64 ones.  Every division is a product with a reciprocal the plan made
// once, and the per-image evaluation weights come from the plan too, so a
// real costs about ten multiply-adds per image.  SG(n), the thread's column
// of the solution, lives in shared memory ([n][thread]) or, for strings too
// long for that, in the strided global scratch.

// Uniform data of one resample in type C, staged in shared memory per block.
template <class C>
struct CubicUniform {
    C *rh, *rd, *dl, *du, *du2, *ev, *ends;
    int *ipiv, *kk;
};

template <class C>
__host__ __device__ inline size_t cubic_uniform_bytes(int F, int F_new)
{
    return ((size_t)(5 * F + 4 * F_new + 8) * sizeof(C) + (size_t)(F + F_new) * sizeof(int) + 15) & ~(size_t)15;
}

template <class C>
__device__ __forceinline__ CubicUniform<C> stage_cubic_uniform(const RedistPlan &p, int F, int F_new, char *sm)
{
    CubicUniform<C> u;
    u.rh = reinterpret_cast<C *>(sm);
    u.rd = u.rh + F;
    u.dl = u.rd + F;
    u.du = u.dl + F;
    u.du2 = u.du + F;
    u.ev = u.du2 + F;
    u.ends = u.ev + 4 * F_new;
    u.ipiv = reinterpret_cast<int *>(u.ends + 8);
    u.kk = u.ipiv + F;
    const double *rh = p.aux, *rd = rh + F, *ev = rd + F, *ends = ev + 4 * F_new;
    for (int n = threadIdx.x; n < F; n += blockDim.x) {
        u.rh[n] = (C)rh[n];
        u.rd[n] = (C)rd[n];
        u.dl[n] = (C)p.dl[n];
        u.du[n] = (C)p.du[n];
        u.du2[n] = (C)p.du2[n];
        u.ipiv[n] = p.ipiv[n];
    }
    for (int n = threadIdx.x; n < 4 * F_new; n += blockDim.x) u.ev[n] = (C)ev[n];
    for (int n = threadIdx.x; n < F_new; n += blockDim.x) u.kk[n] = p.k[n];
    if (threadIdx.x < 8) u.ends[threadIdx.x] = (C)ends[threadIdx.x];
    __syncthreads();
    return u;
}

template <class T, class C, bool SMEM>
__device__ __forceinline__ void redist_cubic_real(const T *__restrict__ f, T *__restrict__ fnew, C *sig, long reals,
                                                  long e, int F, int F_new, const CubicUniform<C> &u)
{
#define FV(n) ((C)f[(long)(n) * reals + e])
#define SG(n) (SMEM ? sig[(n) * (int)blockDim.x + (int)threadIdx.x] : sig[(long)(n) * reals + e])
    // the column of f into the solution's storage, eight loads in flight at a time
    {
        int n = 0;
        for (; n + 8 <= F; n += 8) {
            C v[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) v[i] = FV(n + i);
#pragma unroll
            for (int i = 0; i < 8; ++i) SG(n + i) = v[i];
        }
        for (; n < F; ++n) SG(n) = FV(n);
    }
    // first divided differences D[n] = (f_n - f_{n-1}) / h_n, n >= 1; the
    // right-hand side overwrites f in place (f_n is carried in fp)
    const C D1 = (SG(1) - SG(0)) * u.rh[1], D2 = (SG(2) - SG(1)) * u.rh[2], D3 = (SG(3) - SG(2)) * u.rh[3];
    const C Dm1 = (SG(F - 1) - SG(F - 2)) * u.rh[F - 1], Dm2 = (SG(F - 2) - SG(F - 3)) * u.rh[F - 2];
    const C Dm3 = (SG(F - 3) - SG(F - 4)) * u.rh[F - 3];
    const C d3s = ((D3 - D2) * u.ends[0] - (D2 - D1) * u.ends[1]) * u.ends[2];
    const C d3e = ((Dm1 - Dm2) * u.ends[4] - (Dm2 - Dm3) * u.ends[5]) * u.ends[6];
    C Dn = D1, fp = SG(1);
    for (int n = 1; n < F - 1; ++n) {
        const C fn1 = SG(n + 1);
        const C Dn1 = (fn1 - fp) * u.rh[n + 1];
        SG(n) = Dn1 - Dn;
        Dn = Dn1;
        fp = fn1;
    }
    SG(0) = u.ends[3] * d3s;
    SG(F - 1) = u.ends[7] * d3e;
    // forward elimination with the recorded pivots
    for (int q = 0; q < F - 1; ++q) {
        const C bk = SG(q), bk1 = SG(q + 1);
        if (u.ipiv[q]) {
            SG(q) = bk1;
            SG(q + 1) = bk - u.dl[q + 1] * bk1;
        } else {
            SG(q + 1) = bk1 - u.dl[q + 1] * bk;
        }
    }
    SG(F - 1) = SG(F - 1) * u.rd[F - 1];
    SG(F - 2) = (SG(F - 2) - u.du[F - 2] * SG(F - 1)) * u.rd[F - 2];
    for (int q = F - 3; q >= 0; --q) SG(q) = (SG(q) - u.du[q] * SG(q + 1) - u.du2[q] * SG(q + 2)) * u.rd[q];
    // new images: f re-read (from L2), four outputs' loads in flight at a time
    int n = 0;
    for (; n + 4 <= F_new; n += 4) {
        C a[4], b[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int k = u.kk[n + i];
            a[i] = FV(k);
            b[i] = FV(k - 1);
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int k = u.kk[n + i];
            const C *c = u.ev + 4 * (n + i);
            fnew[(long)(n + i) * reals + e] = (T)(c[0] * a[i] + c[1] * b[i] + c[2] * SG(k) + c[3] * SG(k - 1));
        }
    }
    for (; n < F_new; ++n) {
        const int k = u.kk[n];
        const C *c = u.ev + 4 * n;
        fnew[(long)n * reals + e] = (T)(c[0] * FV(k) + c[1] * FV(k - 1) + c[2] * SG(k) + c[3] * SG(k - 1));
    }
#undef FV
#undef SG
}

// Arithmetic type of the cubic resample for fields of type T.
template <class T> using cubic_t = T;

template <class T>
__global__ void __launch_bounds__(NT) k_redist_cubic(const T *f, T *fnew, cubic_t<T> *sig, long reals, int F,
                                                     int F_new, RedistPlan p)
{
    extern __shared__ __align__(16) char cubic_sm[];
    const CubicUniform<cubic_t<T>> u = stage_cubic_uniform<cubic_t<T>>(p, F, F_new, cubic_sm);
    for (long e = blockIdx.x * (long)NT + threadIdx.x; e < reals; e += (long)gridDim.x * NT)
        redist_cubic_real<T, cubic_t<T>, false>(f, fnew, sig, reals, e, F, F_new, u);
}

// Shared-memory columns: after the uniform data, F * blockDim.x values;
// each thread owns one column, so no barrier is needed after the staging.
template <class T>
__global__ void __launch_bounds__(128) k_redist_cubic_s(const T *f, T *fnew, long reals, int F, int F_new,
                                                        RedistPlan p)
{
    extern __shared__ __align__(16) char cubic_sm[];
    const CubicUniform<cubic_t<T>> u = stage_cubic_uniform<cubic_t<T>>(p, F, F_new, cubic_sm);
    cubic_t<T> *cols = reinterpret_cast<cubic_t<T> *>(cubic_sm + cubic_uniform_bytes<cubic_t<T>>(F, F_new));
    for (long e0 = blockIdx.x * (long)blockDim.x; e0 < reals; e0 += (long)gridDim.x * blockDim.x) {
        const long e = e0 + threadIdx.x;
        if (e < reals) redist_cubic_real<T, cubic_t<T>, true>(f, fnew, cols, reals, e, F, F_new, u);
    }
}

template <class S, class D>
__global__ void k_convert(const S *src, D *dst, long n)
{
    for (long e = blockIdx.x * (long)NT + threadIdx.x; e < n; e += (long)gridDim.x * NT) dst[e] = (D)src[e];
}

inline int grid_for(long n, int cap = 152 * 16)
{
    long b = (n + NT - 1) / NT;
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

}  // namespace

// ----------------------------------------------------------------- launchers
#define DISPATCH(L, KERNEL, ...)                                                                    \
    do {                                                                                            \
        if ((L).precision == 1) {                                                                   \
            if ((L).ncomp == 2) KERNEL<double, 2><<<(L).grid, NT, 0, (L).stream>>>(__VA_ARGS__);   \
            else KERNEL<double, 1><<<(L).grid, NT, 0, (L).stream>>>(__VA_ARGS__);                  \
        } else {                                                                                    \
            if ((L).ncomp == 2) KERNEL<float, 2><<<(L).grid, NT, 0, (L).stream>>>(__VA_ARGS__);    \
            else KERNEL<float, 1><<<(L).grid, NT, 0, (L).stream>>>(__VA_ARGS__);                   \
        }                                                                                           \
    } while (0)

// The NLCG passes also exist in float-float arithmetic (paired FP64 mode).
#define DISPATCH_NLCG(L, KERNEL, ...)                                                               \
    do {                                                                                            \
        if ((L).paired && (L).precision == 1) {                                                     \
            if ((L).ncomp == 2) KERNEL<ff, 2><<<(L).grid, NT, 0, (L).stream>>>(__VA_ARGS__);        \
            else KERNEL<ff, 1><<<(L).grid, NT, 0, (L).stream>>>(__VA_ARGS__);                       \
        } else {                                                                                    \
            DISPATCH(L, KERNEL, __VA_ARGS__);                                                       \
        }                                                                                           \
    } while (0)

// FP64 and float-float NLCG passes (tile kernels).
#define DISPATCH_WIDE(L, KERNEL, ...)                                                               \
    do {                                                                                            \
        if ((L).paired) {                                                                           \
            if ((L).ncomp == 2) KERNEL<ff, 2><<<(L).grid, NT, 0, (L).stream>>>(__VA_ARGS__);        \
            else KERNEL<ff, 1><<<(L).grid, NT, 0, (L).stream>>>(__VA_ARGS__);                       \
        } else {                                                                                    \
            if ((L).ncomp == 2) KERNEL<double, 2><<<(L).grid, NT, 0, (L).stream>>>(__VA_ARGS__);    \
            else KERNEL<double, 1><<<(L).grid, NT, 0, (L).stream>>>(__VA_ARGS__);                   \
        }                                                                                           \
    } while (0)

// FP32 NLCG passes: one single-warp block per tile; launches of one string
// take the kernels that read its descriptor at fixed offsets.
#define DISPATCH_STRIP(L, KERNEL, ...)                                                              \
    do {                                                                                            \
        if (strip_one(L)) {                                                                         \
            if ((L).ncomp == 2) KERNEL<float, 2, true><<<(L).n_tiles, NTS, 0, (L).stream>>>(__VA_ARGS__); \
            else KERNEL<float, 1, true><<<(L).n_tiles, NTS, 0, (L).stream>>>(__VA_ARGS__);          \
        } else {                                                                                    \
            if ((L).ncomp == 2) KERNEL<float, 2, false><<<(L).n_tiles, NTS, 0, (L).stream>>>(__VA_ARGS__); \
            else KERNEL<float, 1, false><<<(L).n_tiles, NTS, 0, (L).stream>>>(__VA_ARGS__);         \
        }                                                                                           \
    } while (0)

// Single-string FP32 launch (MEPGL_STRIP_ONE = 0 sends every launch through
// the indexed-descriptor kernels).
static inline bool strip_one(const Launch &L) { return MEPGL_STRIP_ONE && L.batch->n == 1; }

cudaError_t launch_grad(const Launch &L, const Scalars &sc, const StepFlags &f)
{
#if MEPGL_STRIP
    if (L.precision == 0) DISPATCH_STRIP(L, k_grad_s, *L.batch, L.tile0, sc, f);
    else DISPATCH_WIDE(L, k_grad, *L.batch, L.tiles, L.n_tiles, sc, f);
#else
    DISPATCH_NLCG(L, k_grad, *L.batch, L.tiles, L.n_tiles, sc, f);
#endif
    return cudaGetLastError();
}

cudaError_t launch_dir_poly(const Launch &L, const Scalars &sc, const StepFlags &f)
{
#if MEPGL_SPLIT_DIR
    {
        Launch U = L;
        U.grid = L.n_tiles < 152 * 16 ? L.n_tiles : 152 * 16;
        DISPATCH_NLCG(U, k_dir_update, *U.batch, U.tiles, U.n_tiles, sc, f);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
#endif
#if MEPGL_STRIP
    if (L.precision == 0) DISPATCH_STRIP(L, k_dir_poly_s, *L.batch, L.tile0, sc, f);
    else DISPATCH_WIDE(L, k_dir_poly, *L.batch, L.tiles, L.n_tiles, sc, f);
#else
    DISPATCH_NLCG(L, k_dir_poly, *L.batch, L.tiles, L.n_tiles, sc, f);
#endif
    return cudaGetLastError();
}

int strip_pass_slots(int ncomp)
{
#if MEPGL_STRIP
    static int slots[2] = {0, 0};
    const int ci = ncomp == 2 ? 1 : 0;
    if (slots[ci] == 0) {
        int dev = 0, sms = 0, nb = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            return 0;
        const cudaError_t e = ci ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_dir_poly_s<float, 2, false>, NTS, 0)
                                 : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_dir_poly_s<float, 1, false>, NTS, 0);
        if (e != cudaSuccess) return 0;
        slots[ci] = nb * sms;
    }
    return slots[ci];
#else
    (void)ncomp;
    return 0;
#endif
}

cudaError_t launch_nlcg_fused(const Launch &L, const Scalars &sc, const StepFlags &f0, int it0, int steps,
                              unsigned long long *queue, unsigned *stage, int n_stage, unsigned long long first_item,
                              unsigned max_polls)
{
#if MEPGL_STRIP
    static int slots[4] = {0, 0, 0, 0};
    const bool one = strip_one(L);
    const int ci = (L.ncomp == 2 ? 1 : 0) + (one ? 2 : 0);
    if (slots[ci] == 0) {
        int dev = 0, sms = 0, nb = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess) {
            switch (ci) {
            case 0: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_nlcg_s<float, 1, false>, NTS, 0); break;
            case 1: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_nlcg_s<float, 2, false>, NTS, 0); break;
            case 2: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_nlcg_s<float, 1, true>, NTS, 0); break;
            default: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_nlcg_s<float, 2, true>, NTS, 0); break;
            }
        }
        if (e != cudaSuccess) return e;
        slots[ci] = nb * sms > 0 ? nb * sms : 1;
    }
    StepPlan plan;
    plan.xi0 = f0.xin;
    plan.di0 = f0.din;
    plan.it0 = it0;
    plan.base = f0;
    cudaError_t e = first_item ? cudaMemcpyAsync(queue, &first_item, sizeof(first_item), cudaMemcpyHostToDevice, L.stream)
                               : cudaMemsetAsync(queue, 0, sizeof(unsigned long long), L.stream);
    if (e == cudaSuccess && first_item) e = cudaStreamSynchronize(L.stream);   // first_item is a host local
    if (e == cudaSuccess) e = cudaMemsetAsync(stage, 0, sizeof(unsigned) * (size_t)n_stage, L.stream);
    if (e != cudaSuccess) return e;
    const long long items = 2LL * L.n_tiles * steps;
    const int grid = items < slots[ci] ? (int)items : slots[ci];
#define FUSED_ARGS *L.batch, L.tile0, L.n_tiles, steps, plan, sc, queue, stage, max_polls
    switch (ci) {
    case 0: k_nlcg_s<float, 1, false><<<grid, NTS, 0, L.stream>>>(FUSED_ARGS); break;
    case 1: k_nlcg_s<float, 2, false><<<grid, NTS, 0, L.stream>>>(FUSED_ARGS); break;
    case 2: k_nlcg_s<float, 1, true><<<grid, NTS, 0, L.stream>>>(FUSED_ARGS); break;
    default: k_nlcg_s<float, 2, true><<<grid, NTS, 0, L.stream>>>(FUSED_ARGS); break;
    }
#undef FUSED_ARGS
    return cudaGetLastError();
#else
    (void)L; (void)sc; (void)f0; (void)it0; (void)steps; (void)queue; (void)stage; (void)n_stage;
    (void)first_item; (void)max_polls;
    return cudaErrorNotSupported;
#endif
}

cudaError_t launch_energy(const Launch &L, const Scalars &sc, int xbuf, double *out)
{
    DISPATCH(L, k_energy, *L.batch, L.tiles, L.n_tiles, sc, xbuf, out);
    return cudaGetLastError();
}

// FP64 launches with L.paired compute in float-float on the double fields
// (about 48 bits) and store double gradients; the link discretisation has
// no float-float form and stays IEEE double.
cudaError_t launch_gradient_only(const Launch &L, int xbuf, FieldPtrs out, int maxwell)
{
    if (L.paired && L.precision == 1 && !L.batch->s[0].disc) {
        if (L.ncomp == 2) k_gradient_only<ff, 2><<<L.grid, NT, 0, L.stream>>>(*L.batch, L.tiles, L.n_tiles, xbuf, out, maxwell);
        else k_gradient_only<ff, 1><<<L.grid, NT, 0, L.stream>>>(*L.batch, L.tiles, L.n_tiles, xbuf, out, maxwell);
    } else {
        DISPATCH(L, k_gradient_only, *L.batch, L.tiles, L.n_tiles, xbuf, out, maxwell);
    }
    return cudaGetLastError();
}

cudaError_t launch_param_adjoint(const Launch &L, const Scalars &sc, int xbuf, double *out)
{
    DISPATCH(L, k_param_adjoint, *L.batch, L.tiles, L.n_tiles, sc, xbuf, out);
    return cudaGetLastError();
}

cudaError_t launch_jb(const Launch &L, const Scalars &sc, int xbuf, void *const *b, void *const (*j)[2])
{
    (void)sc;
    if (L.precision == 1) {
        if (L.ncomp == 2)
            k_jb<double, 2><<<L.grid, NT, 0, L.stream>>>(*L.batch, L.tiles, L.n_tiles, xbuf, (double *)b[0],
                                                         (double2 *)j[0][0], (double2 *)j[0][1]);
        else
            k_jb<double, 1><<<L.grid, NT, 0, L.stream>>>(*L.batch, L.tiles, L.n_tiles, xbuf, (double *)b[0],
                                                         (double2 *)j[0][0], (double2 *)j[0][1]);
    } else {
        if (L.ncomp == 2)
            k_jb<float, 2><<<L.grid, NT, 0, L.stream>>>(*L.batch, L.tiles, L.n_tiles, xbuf, (float *)b[0],
                                                        (float2 *)j[0][0], (float2 *)j[0][1]);
        else
            k_jb<float, 1><<<L.grid, NT, 0, L.stream>>>(*L.batch, L.tiles, L.n_tiles, xbuf, (float *)b[0],
                                                        (float2 *)j[0][0], (float2 *)j[0][1]);
    }
    return cudaGetLastError();
}

cudaError_t launch_apply_update(const Launch &L, const Scalars &sc, const StringDesc *hs, int n_strings, int xbuf,
                                int dbuf)
{
    for (int si = 0; si < n_strings; ++si) {
        const StringDesc &S = hs[si];
        const long M = (long)S.nx * S.ny;
        for (int c = 0; c < 1 + S.ncomp; ++c) {
            const dim3 grid((unsigned)((M + NT - 1) / NT < 64 ? (M + NT - 1) / NT : 64), (unsigned)S.F);
            if (L.precision == 1 && L.paired)   // d holds float-float pairs (paired passes)
                k_apply_update<double, ff><<<grid, NT, 0, L.stream>>>(
                    (double2 *)S.x[xbuf][c], (const double2 *)S.d[dbuf][c], sc.alpha_pend + S.img_base, M);
            else if (L.precision == 1)
                k_apply_update<double><<<grid, NT, 0, L.stream>>>(
                    (double2 *)S.x[xbuf][c], (const double2 *)S.d[dbuf][c], sc.alpha_pend + S.img_base, M);
            else
                k_apply_update<float><<<grid, NT, 0, L.stream>>>(
                    (float2 *)S.x[xbuf][c], (const float2 *)S.d[dbuf][c], sc.alpha_pend + S.img_base, M);
        }
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    int total_images = 0;
    for (int si = 0; si < n_strings; ++si) total_images += hs[si].F;
    return cudaMemsetAsync(sc.alpha_pend, 0, sizeof(double) * total_images, L.stream);
}

cudaError_t launch_check_scalars(const Scalars &sc, int n_images, int slot, cudaStream_t st)
{
    k_check_scalars<<<(n_images + NT - 1) / NT, NT, 0, st>>>(sc.fenergy, slot ? sc.gn1 : sc.gn0, n_images, sc.status);
    return cudaGetLastError();
}

cudaError_t launch_arc_length(int precision, const void *const *fields, const int *width, int nf, long sites, int F,
                              double *part, double *s, int *bad, cudaStream_t st)
{
    const int nb = (int)((sites + (long)NT * ARC_SPT - 1) / ((long)NT * ARC_SPT));
    const dim3 grid(nb, F);
    const void *f[3] = {nf > 0 ? fields[0] : nullptr, nf > 1 ? fields[1] : nullptr, nf > 2 ? fields[2] : nullptr};
    const int w[3] = {nf > 0 ? width[0] : 0, nf > 1 ? width[1] : 0, nf > 2 ? width[2] : 0};
    if (precision == 1)
        k_arc_partial<double><<<grid, NT, 0, st>>>((const double *)f[0], (const double *)f[1], (const double *)f[2],
                                                   w[0], w[1], w[2], sites, part);
    else
        k_arc_partial<float><<<grid, NT, 0, st>>>((const float *)f[0], (const float *)f[1], (const float *)f[2],
                                                  w[0], w[1], w[2], sites, part);
    k_arc_sum<<<F, NT, 0, st>>>(part, nb, s);
    k_arc_cumulate<<<1, NT, 0, st>>>(F, s, bad);
    return cudaGetLastError();
}

cudaError_t launch_generate(int precision, void *a, void *p1, void *p2, int nx, int ny, int F, int ncomp,
                            const int32_t *comp, const int32_t *sc, const double *tracks, int n_tracks,
                            const GuessParams &g, cudaStream_t st)
{
    const long n = (long)nx * ny * F;
    long b = (n + NT - 1) / NT;
    const int grid = (int)(b < 1 ? 1 : (b > 152 * 32 ? 152 * 32 : b));
    if (precision == 1)
        k_generate<double><<<grid, NT, 0, st>>>((double2 *)a, (double2 *)p1, (double2 *)p2, nx, ny, F, ncomp, comp, sc,
                                                tracks, n_tracks, g);
    else
        k_generate<float><<<grid, NT, 0, st>>>((float2 *)a, (float2 *)p1, (float2 *)p2, nx, ny, F, ncomp, comp, sc,
                                               tracks, n_tracks, g);
    return cudaGetLastError();
}

cudaError_t launch_flux(int precision, const void *b, long M, int F, double dx2, double *out, cudaStream_t st)
{
    const int grid = F < 152 * 4 ? F : 152 * 4;
    if (precision == 1) k_flux<double><<<grid, NT, 0, st>>>((const double *)b, M, F, dx2, out);
    else k_flux<float><<<grid, NT, 0, st>>>((const float *)b, M, F, dx2, out);
    return cudaGetLastError();
}

cudaError_t launch_winding(int precision, const void *psi, int nx, int ny, int F, int inset, double *out,
                           cudaStream_t st)
{
    const int grid = F < 152 * 4 ? F : 152 * 4;
    if (precision == 1) k_winding<double><<<grid, NT, 0, st>>>((const double2 *)psi, nx, ny, F, inset, out);
    else k_winding<float><<<grid, NT, 0, st>>>((const float2 *)psi, nx, ny, F, inset, out);
    return cudaGetLastError();
}

cudaError_t launch_redist_plan(const double *s, int F, int F_new, int cubic, int spline, const RedistPlan &p,
                               cudaStream_t st)
{
    const size_t sm = redist_plan_smem(F, F_new);
    const int use_smem = sm <= 48 * 1024;
    k_redist_plan<<<1, 32, use_smem ? sm : 0, st>>>(s, F, F_new, cubic, spline, p, use_smem);
    return cudaGetLastError();
}

cudaError_t launch_redist_linear(int precision, const void *f, void *fnew, long pairs, int F_new, const RedistPlan &p,
                                 cudaStream_t st)
{
    const long reals = 2 * pairs;
    // blocks per output image: about four waves of the GPU in all
    auto grid = [&](long nv) {
        long bx = (nv + NT - 1) / NT, cap = (152L * 8 * 4 + F_new - 1) / F_new;
        bx = bx < cap ? bx : cap;
        return dim3((unsigned)(bx < 1 ? 1 : bx), (unsigned)F_new);
    };
    if (precision == 1) {
        k_redist_linear<double, 2><<<grid(reals / 2), NT, 0, st>>>((const double *)f, (double *)fnew, reals, p.k, p.w);
    } else if (reals % 4 == 0) {
        k_redist_linear<float, 4><<<grid(reals / 4), NT, 0, st>>>((const float *)f, (float *)fnew, reals, p.k, p.w);
    } else {
        k_redist_linear<float, 1><<<grid(reals), NT, 0, st>>>((const float *)f, (float *)fnew, reals, p.k, p.w);
    }
    return cudaGetLastError();
}

// Shape of a cubic resample launch: threads per block and dynamic shared
// memory of the shared-memory form (32 KB of columns per block where F
// allows: 128 threads, 64 or 32; up to 200 KB in all at 32 threads), or
// sm = 0 when the string is too long for it and the global scratch is used.
static void cubic_shape(int precision, int F, int F_new, int *tpb_out, size_t *sm_out)
{
    const size_t cs = precision == 1 ? sizeof(double) : sizeof(float);
    const size_t ub = precision == 1 ? cubic_uniform_bytes<double>(F, F_new) : cubic_uniform_bytes<float>(F, F_new);
    int tpb = 128;
    while (tpb > 32 && (size_t)tpb * F * cs > 32 * 1024) tpb >>= 1;
    const size_t sm = ub + (size_t)tpb * F * cs;
    *tpb_out = tpb;
    *sm_out = sm <= 200 * 1024 ? sm : 0;
}

size_t redist_cubic_scratch_bytes(int precision, long pairs, int F, int F_new)
{
    int tpb;
    size_t sm;
    cubic_shape(precision, F, F_new, &tpb, &sm);
    return sm ? 0 : (size_t)2 * pairs * F * (precision == 1 ? sizeof(double) : sizeof(float));
}

cudaError_t launch_redist_cubic(int precision, const void *f, void *fnew, void *sigma, long pairs, int F, int F_new,
                                int spline, const RedistPlan &p, cudaStream_t st)
{
    (void)spline;   // folded into the plan's evaluation weights
    const long reals = 2 * pairs;
    const size_t ub = precision == 1 ? cubic_uniform_bytes<double>(F, F_new) : cubic_uniform_bytes<float>(F, F_new);
    int tpb;
    size_t sm;
    cubic_shape(precision, F, F_new, &tpb, &sm);
    cudaError_t e = cudaSuccess;
    if (sm) {
        const long blocks = (reals + tpb - 1) / tpb;
        const int grid = (int)(blocks < 152 * 32 ? blocks : 152 * 32);
        if (precision == 1) {
            if (sm > 48 * 1024)
                e = cudaFuncSetAttribute(k_redist_cubic_s<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
            if (e != cudaSuccess) return e;
            k_redist_cubic_s<double><<<grid, tpb, sm, st>>>((const double *)f, (double *)fnew, reals, F, F_new, p);
        } else {
            if (sm > 48 * 1024)
                e = cudaFuncSetAttribute(k_redist_cubic_s<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
            if (e != cudaSuccess) return e;
            k_redist_cubic_s<float><<<grid, tpb, sm, st>>>((const float *)f, (float *)fnew, reals, F, F_new, p);
        }
        return cudaGetLastError();
    }
    if (ub > 200 * 1024 || !sigma) return cudaErrorInvalidValue;   // more than about 2,800 images
    if (ub > 48 * 1024)
        e = precision == 1
                ? cudaFuncSetAttribute(k_redist_cubic<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ub)
                : cudaFuncSetAttribute(k_redist_cubic<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ub);
    if (e != cudaSuccess) return e;
    if (precision == 1)
        k_redist_cubic<double><<<grid_for(reals), NT, ub, st>>>((const double *)f, (double *)fnew, (double *)sigma,
                                                                reals, F, F_new, p);
    else
        k_redist_cubic<float><<<grid_for(reals), NT, ub, st>>>((const float *)f, (float *)fnew, (float *)sigma, reals,
                                                               F, F_new, p);
    return cudaGetLastError();
}

bool x_pairs() { return MEPGL_FF_XPAIRS != 0; }

cudaError_t launch_x_format(void *x, long pairs, int to_pairs, cudaStream_t st)
{
    if (to_pairs) k_x_format<true><<<grid_for(pairs), NT, 0, st>>>((double2 *)x, pairs);
    else k_x_format<false><<<grid_for(pairs), NT, 0, st>>>((double2 *)x, pairs);
    return cudaGetLastError();
}

cudaError_t launch_convert(const void *src, int src_prec, void *dst, int dst_prec, long n, cudaStream_t st)
{
    if (src_prec == 0 && dst_prec == 1)
        k_convert<float, double><<<grid_for(n), NT, 0, st>>>((const float *)src, (double *)dst, n);
    else if (src_prec == 1 && dst_prec == 0)
        k_convert<double, float><<<grid_for(n), NT, 0, st>>>((const double *)src, (float *)dst, n);
    else
        return cudaMemcpyAsync(dst, src, n * (src_prec ? 8 : 4), cudaMemcpyDeviceToDevice, st);
    return cudaGetLastError();
}

}  // namespace mepgl

// ===================================================== allocation-free energy
//
// Some callers cannot allocate device memory: embedded solvers that own a
// fixed device arena and hand out only pre-allocated buffers, host
// frameworks whose memory pool owns the whole device, or plugins whose host
// process forbids cudaMalloc after start-up (an allocation there can
// synchronise the device in the middle of its pipelined work).  mepgl_free_energy_noalloc serves them: it
// evaluates the per-image free energy of caller-owned device arrays without
// creating a context and without any allocation.  The per-tile partial sums
// and per-image tickets of the deterministic reduction live in the fixed
// arrays below, which every GPU that loads this library holds until the
// process exits (4 MiB + 16 KiB per device).
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/mepgl.h"

namespace {

constexpr int NOALLOC_MAX_TILES = 65536;     // images x ceil(nx/32) x ceil(ny/8)
constexpr int NOALLOC_MAX_IMAGES = 4096;
constexpr int NOALLOC_MAX_DEVICES = 64;

static __device__ __align__(256) double g_noalloc_part[NOALLOC_MAX_TILES * 8];
static __device__ __align__(256) unsigned g_noalloc_ticket[NOALLOC_MAX_IMAGES];

struct NoallocScratch {
    bool ready;
    double *part;
    unsigned *ticket;
};
std::mutex g_noalloc_mu;
NoallocScratch g_noalloc[NOALLOC_MAX_DEVICES];
thread_local std::string g_noalloc_err;

// Device addresses of the scratch arrays, resolved once per device with that
// device current (a host-side reference to the array names is not a device
// address).  Also uploads the constant neighbour-code tables.  Both are kept
// for the life of the process: a device reset (cudaDeviceReset, or a reset
// of the primary context by the host framework) is not supported, since the
// cached addresses and the constant tables would then be stale.
cudaError_t noalloc_setup(int dev, NoallocScratch *out)
{
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    NoallocScratch &s = g_noalloc[dev];
    if (!s.ready) {
        cudaError_t e = cudaGetSymbolAddress((void **)&s.part, g_noalloc_part);
        if (e != cudaSuccess) return e;
        e = cudaGetSymbolAddress((void **)&s.ticket, g_noalloc_ticket);
        if (e != cudaSuccess) return e;
        e = mepgl::upload_mask_tables();
        if (e != cudaSuccess) return e;
        s.ready = true;
    }
    *out = s;
    return cudaSuccess;
}

mepgl_status noalloc_fail(mepgl_status st, const std::string &m)
{
    g_noalloc_err = m;
    return st;
}

}  // namespace

extern "C" const char *mepgl_noalloc_last_error(void) { return g_noalloc_err.c_str(); }

extern "C" mepgl_status mepgl_free_energy_noalloc(int nx, int ny, int n_images, int multicomponent, int thin_film,
                                                  double dx, const int32_t *comp_code, const int32_t *sc_code,
                                                  const double *a_1, const double *b_1, const double *m_xx_1,
                                                  const double *m_yy_1, const double *a_2, const double *b_2,
                                                  const double *m_xx_2, const double *m_yy_2, const double *h,
                                                  double q_1, double q_2, double eta, double gamma, double delta,
                                                  const void *a, const void *psi_1, const void *psi_2,
                                                  double *fenergy, void *stream)
{
    using namespace mepgl;
    constexpr int rows = MEPGL_ROWS_F64;
    if (nx < 2 || ny < 2 || n_images < 1 || !(dx > 0))
        return noalloc_fail(MEPGL_ERR_INVALID_ARG, "need nx, ny >= 2, n_images >= 1, dx > 0");
    if (!comp_code || !sc_code || !a_1 || !b_1 || !m_xx_1 || !m_yy_1 || !h || !a || !psi_1 || !fenergy ||
        (multicomponent && (!a_2 || !b_2 || !m_xx_2 || !m_yy_2 || !psi_2)))
        return noalloc_fail(MEPGL_ERR_INVALID_ARG, "null device pointer");
    const long tiles_x = (nx + TX - 1) / TX, tiles_y = (ny + rows - 1) / rows;
    const long n_tiles = tiles_x * tiles_y * n_images;
    // tile coordinates are 16-bit (TileRef), as in mepgl_create
    if (nx > 32767 * TX || ny > 32767 * rows || (long)nx * ny >= (1L << 31))
        return noalloc_fail(MEPGL_ERR_INVALID_ARG, "lattice too large: need nx <= 32767*32, ny <= 32767*8 "
                                                   "and nx * ny < 2^31");
    if (n_images > NOALLOC_MAX_IMAGES || n_tiles > NOALLOC_MAX_TILES)
        return noalloc_fail(MEPGL_ERR_INVALID_ARG,
                            "string too large for the fixed scratch: need n_images <= 4096 and "
                            "n_images * ceil(nx/32) * ceil(ny/8) <= 65536");
    // An error left pending by the caller's own earlier work is reported as
    // such and left in place, not taken for a failure of this call.
    cudaError_t pend = cudaPeekAtLastError();
    if (pend != cudaSuccess)
        return noalloc_fail(MEPGL_ERR_CUDA, std::string("error pending before this call (left for the caller): ") +
                                                cudaGetErrorString(pend));
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NOALLOC_MAX_DEVICES)
        return noalloc_fail(MEPGL_ERR_CUDA, "no usable current device");
    NoallocScratch scr;
    cudaError_t e = noalloc_setup(dev, &scr);
    if (e != cudaSuccess) return noalloc_fail(MEPGL_ERR_CUDA, std::string("scratch setup: ") + cudaGetErrorString(e));

    Batch bt;
    memset(&bt, 0, sizeof(bt));
    bt.n = 1;
    StringDesc &S = bt.s[0];
    S.nx = nx;
    S.ny = ny;
    S.F = n_images;
    S.ncomp = multicomponent ? 2 : 1;
    S.tiles_x = (int)tiles_x;
    S.tiles_y = (int)tiles_y;
    S.thin_film = thin_film ? 1 : 0;
    S.per_site = 1;
    const double *pa[2] = {a_1, multicomponent ? a_2 : a_1}, *pb[2] = {b_1, multicomponent ? b_2 : b_1};
    const double *px[2] = {m_xx_1, multicomponent ? m_xx_2 : m_xx_1}, *py[2] = {m_yy_1, multicomponent ? m_yy_2 : m_yy_1};
    for (int c = 0; c < 2; ++c) {
        S.pa[c] = pa[c];
        S.pb[c] = pb[c];
        S.pmxx[c] = px[c];
        S.pmyy[c] = py[c];
    }
    S.ph = h;
    S.ud.q[0] = q_1;
    S.ud.q[1] = q_2;
    S.ud.eta = eta;
    S.ud.gamma = gamma;
    S.ud.delta = delta;
    S.ud.idx = 1.0 / dx;
    S.ud.dx2 = dx * dx;
    S.ud.dx = dx;
    S.code_comp = comp_code;
    S.code_sc = sc_code;
    S.x[0][0] = const_cast<void *>(a);
    S.x[0][1] = const_cast<void *>(psi_1);
    S.x[0][2] = multicomponent ? const_cast<void *>(psi_2) : nullptr;
    Scalars sc;
    memset(&sc, 0, sizeof(sc));
    sc.part = scr.part;
    sc.ticket = scr.ticket;
    cudaStream_t st = (cudaStream_t)stream;
    // the tickets must start at zero; the array keeps the previous call's contents
    e = cudaMemsetAsync(scr.ticket, 0, sizeof(unsigned) * n_images, st);
    if (e != cudaSuccess) return noalloc_fail(MEPGL_ERR_CUDA, std::string("ticket reset: ") + cudaGetErrorString(e));
    if (multicomponent)
        k_energy<double, 2><<<(unsigned)n_tiles, NT, 0, st>>>(bt, nullptr, (int)n_tiles, sc, 0, fenergy);
    else
        k_energy<double, 1><<<(unsigned)n_tiles, NT, 0, st>>>(bt, nullptr, (int)n_tiles, sc, 0, fenergy);
    e = cudaGetLastError();
    if (e != cudaSuccess) return noalloc_fail(MEPGL_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
    return MEPGL_OK;
}
