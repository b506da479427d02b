// common.cuh -- shared device-side definitions of libmepgl_gb300.
//
// Work decomposition.  Every pass over the string is a list of tiles; a
// tile is TX x TY sites of one image of one string.  Kernels walk the tile
// list with a grid-stride loop, so one launch covers every image of up to
// MAX_STRINGS strings (strings may differ in size and image count).
// Per-image reductions are deterministic: each tile writes one partial per
// quantity, and the last tile of an image to finish (atomic ticket per
// image) sums that image's partials in a fixed order.
//
// Precision.  Fields are float or double (T).  Sums are formed in T inside
// a block (fixed pairwise shuffle trees), then in double across tiles and
// images.  GB300's FP64 pipe is a small fraction of its FP32
// rate, so FP32 kernels avoid any per-site double arithmetic or conversion.
#pragma once

#include <cstdint>
#include <type_traits>
#include <cuda_runtime.h>

#include "pair_float.cuh"

namespace mepgl {

constexpr int TX = 32;        // tile width: one warp per tile row
constexpr int NT = 256;       // threads per block for the lattice kernels
constexpr int MAX_STRINGS = 16;   // strings per launch (descriptors travel as a kernel parameter)

template <class T> struct Vec2;
template <> struct Vec2<float> { using type = float2; };
template <> struct Vec2<double> { using type = double2; };
template <> struct Vec2<ff> { using type = ff2; };
template <class T> using vec2_t = typename Vec2<T>::type;

// Storage type of a compute type: float-float arithmetic works on double
// fields (the paired FP64 mode); float and double are stored as computed.
template <class T> struct Store { using type = T; };
template <> struct Store<ff> { using type = double; };
template <class T> using store_t = typename Store<T>::type;

template <class T> __device__ __forceinline__ T from_store(store_t<T> v) { return v; }
template <> __device__ __forceinline__ ff from_store<ff>(double v) { return to_ff(v); }
template <class T> __device__ __forceinline__ store_t<T> to_store(T v) { return v; }
template <> __device__ __forceinline__ double to_store<ff>(ff v) { return to_double(v); }

template <class T> __device__ __forceinline__ vec2_t<T> load2(const vec2_t<store_t<T>> *p) { return *p; }
template <> __device__ __forceinline__ ff2 load2<ff>(const double2 *p)
{
    const double2 d = *p;
    ff2 r;
    r.x = to_ff(d.x);
    r.y = to_ff(d.y);
    return r;
}
template <class T> __device__ __forceinline__ void store2(vec2_t<store_t<T>> *p, vec2_t<T> v) { *p = v; }
template <> __device__ __forceinline__ void store2<ff>(double2 *p, ff2 v)
{
    *p = make_double2(to_double(v.x), to_double(v.y));
}

// Storage of the NLCG work arrays (gradient g and direction d): the compute
// type itself for float and double; float-float pairs in the paired FP64 mode
// (ff2 fills the same 16 bytes as double2), so the paired passes move them
// without conversions.  The arrays are internal to the NLCG passes and the
// pending-step update, and are zeroed (a valid value in every format)
// whenever the history is reset.
template <class T> __device__ __forceinline__ vec2_t<T> loadw(const vec2_t<store_t<T>> *p) { return load2<T>(p); }
template <> __device__ __forceinline__ ff2 loadw<ff>(const double2 *p)
{
    const float4 q = *reinterpret_cast<const float4 *>(p);
    ff2 r;
    r.x = ff(q.x, q.y);
    r.y = ff(q.z, q.w);
    return r;
}
template <class T> __device__ __forceinline__ void storew(vec2_t<store_t<T>> *p, vec2_t<T> v) { store2<T>(p, v); }
template <> __device__ __forceinline__ void storew<ff>(double2 *p, ff2 v)
{
    *reinterpret_cast<float4 *>(p) = make_float4(v.x.hi, v.x.lo, v.y.hi, v.y.lo);
}

// Uniform GL parameters in one precision (hm* = 0.5 / m, aob = a / b).
template <class T>
struct Uniform {
    T a[2], b[2], hmx[2], hmy[2], aob[2], q[2];
    T eta, gamma, delta, h, idx, dx2, dx;
};

// One string (one lattice, F images) as seen by the kernels.  Field buffers
// hold three arrays each (A, psi_1, psi_2) of F*nx*ny pairs; psi_2 is null
// for one component.  Buffers: x (state, ping-pong), g (gradient, two
// slots), d (direction, ping-pong).
struct StringDesc {
    int nx, ny, F, ncomp;
    int tiles_x, tiles_y;     // tiles per image
    int img_base;             // first global image index of this string
    int tile_base;            // first global tile index of this string
    int thin_film;
    int disc;                 // 0: the reference's linearised differences, 1: gauge links
    int per_site;             // 1: parameters read from the arrays below
    Uniform<float> uf;
    Uniform<double> ud;
    Uniform<ff> uff;          // ud split into float pairs (paired FP64 mode)
    const void *pa[2], *pb[2], *pmxx[2], *pmyy[2], *ph;  // per-site (type T)
    const uint16_t *mask;     // per site: comp code | sc code << 8
    const int32_t *code_comp, *code_sc;   // used when mask is null: int32 codes per site
    void *x[2][3], *g[2][3], *d[2][3];

    template <class T> __host__ __device__ const Uniform<T> &u() const;
};
template <> __host__ __device__ inline const Uniform<float> &StringDesc::u<float>() const { return uf; }
template <> __host__ __device__ inline const Uniform<double> &StringDesc::u<double>() const { return ud; }
template <> __host__ __device__ inline const Uniform<ff> &StringDesc::u<ff>() const { return uff; }

// Descriptors of the strings covered by one launch; passed by value as a
// __grid_constant__ kernel parameter, i.e. read through the constant cache.
struct Batch {
    int n;
    StringDesc s[MAX_STRINGS];
};

struct TileRef {
    int16_t s;        // string within the batch
    int16_t ty;       // tile row
    int16_t tx;       // tile column
    int16_t pad;
    int32_t n;        // image
};

// Per-image scalars of the whole context (index = img_base + n).
struct Scalars {
    double *gn0, *gn1;    // |g|^2, two slots (nlcgSteps' g_norm2 / g_norm2_old)
    double *gdg;          // g . (g - g_prev)
    double *beta;         // Polak-Ribiere coefficient of the last step
    double *alpha;        // step of the last line search (reported)
    double *alpha_pend;   // step not yet applied to x (0 = nothing pending)
    double *fenergy;      // energy (polynomial constant term)
    double *poly;         // [img][4] = B, C, D, E
    double *part;         // per-tile partials, [tile][8]
    unsigned *ticket;     // per-image arrival counters
    double *xtab_f, *xtab_d;   // line-search grid x_p, p = 0..2000, rounded to float / double
    int *status;          // device-side error flags
};

__device__ __forceinline__ unsigned bit(unsigned c, int n) { return (c >> n) & 1u; }

// Block-wide sum of NV values; a pairwise tree in T inside each warp, then
// across the warps in float (FP32 fields) or double (the others).  Result
// (double) valid in thread 0.
template <int NV, class T>
__device__ __forceinline__ void block_sum(const T (&v)[NV], double (&out)[NV], double *smem /* NT/32*NV */)
{
    T w[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        w[k] = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) w[k] += shfl_down(w[k], o);
    }
    const int wi = threadIdx.x >> 5, l = threadIdx.x & 31;
    if constexpr (std::is_same<T, float>::value) {
        // FP32 fields: the eight warp sums are added in float too (the FP64
        // pipe is scarce; one conversion per quantity and block)
        float *fs = reinterpret_cast<float *>(smem);
        if (l == 0)
#pragma unroll
            for (int k = 0; k < NV; ++k) fs[wi * NV + k] = w[k];
        __syncthreads();
        if (threadIdx.x < 32) {
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                float t = (l < NT / 32) ? fs[l * NV + k] : 0.0f;
#pragma unroll
                for (int o = NT / 64; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
                out[k] = (double)t;
            }
        }
    } else {
        if (l == 0)
#pragma unroll
            for (int k = 0; k < NV; ++k) smem[wi * NV + k] = (double)w[k];
        __syncthreads();
        if (threadIdx.x < 32) {
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                double t = (l < NT / 32) ? smem[l * NV + k] : 0.0;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
                out[k] = t;
            }
        }
    }
    __syncthreads();
}

// Write this tile's NV partials; return true (in every thread) if this
// block is the last of its image, in which case `tot` holds the image sums
// (in thread 0) computed over the image's partials in index order.
template <int NV, class T>
__device__ __forceinline__ bool finish_image(const T (&v)[NV], double *smem, const Scalars &sc, int tile,
                                             int first_tile, int tiles_per_image, int img, double (&tot)[NV])
{
    __shared__ bool last;
    double mine[NV];
    block_sum<NV>(v, mine, smem);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) sc.part[(size_t)tile * 8 + k] = mine[k];
        __threadfence();
        const unsigned prev = atomicAdd(&sc.ticket[img], 1u);
        last = (prev == (unsigned)tiles_per_image - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double acc[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[k] = 0;
    for (int t = threadIdx.x; t < tiles_per_image; t += NT) {
        const double *p = sc.part + (size_t)(first_tile + t) * 8;
#pragma unroll
        for (int k = 0; k < NV; ++k) acc[k] += __ldcg(p + k);
    }
    block_sum<NV>(acc, tot, smem);
    if (threadIdx.x == 0) sc.ticket[img] = 0;
    return true;
}

}  // namespace mepgl
