// strip.cuh -- the two NLCG passes as warp strips (FP32 fields), launched
// as two pass kernels per step or as one fused persistent launch per call
// (end of file).  Included by kernels.cu inside its anonymous namespace,
// after the tile kernels, whose helpers (part_slot, h_site, line search) it
// uses.
//
// A block is one warp.  In the pass kernels it owns one tile of the usual
// tiling (TX = 32 columns x TYT rows of one image); in the fused kernel it
// takes tiles from a work queue.  Everything that depends on the tile
// (pointers, parameters, row numbers) is uniform over the block.  Lane l holds column i0 + l and walks down the
// tile's rows with a three-row window of its column in registers; the
// x-neighbours come from the adjacent lanes by shuffles.  Lanes 0 and 31
// copy the halo column next to them (i0 - 1, i0 + 32) into a three-row ring
// in shared memory with cp.async and read it back themselves, so no lane
// waits for another.  Rows j0 - 1 and j0 + TYT are read as halo rows.
// While a row is computed, the loads of the next row are in flight.  Every
// tile leaves one partial per quantity in the slot the tile kernels use,
// and the last tile of an image (atomic ticket) finishes it.
#pragma once

constexpr int NTS = 32;   // threads per block of the strip kernels

// Two-component FP32 strings run the packed stencils (site_pair.cuh): the
// window then holds psi as (Re psi_1, Re psi_2), (Im psi_1, Im psi_2) in the
// two pair slots of the components.
template <class T, int NC>
struct StripPacked {
    static constexpr bool v = MEPGL_STRIP_PAIR && NC == 2 && std::is_same<T, float>::value;
};

// (re, im) of two components <-> (Re 1, Re 2), (Im 1, Im 2): a 2 x 2 transpose.
template <class V>
__device__ __forceinline__ void transpose_pair(V &a, V &b)
{
    const V p = a, q = b;
    a.x = p.x;
    a.y = q.x;
    b.x = p.y;
    b.y = q.y;
}

constexpr unsigned FULL_MASK = 0xffffffffu;

// Register window of one site: A(dx, dy), P(c, dx, dy); the strip kernels
// fill the entries their stencil reads and leave the others zero.
template <class T, int NC>
struct RegView {
    vec2_t<T> a[3][3];
    vec2_t<T> p[NC][3][3];
    __device__ __forceinline__ vec2_t<T> A(int dx, int dy) const { return a[dy + 1][dx + 1]; }
    __device__ __forceinline__ vec2_t<T> P(int c, int dx, int dy) const { return p[c][dy + 1][dx + 1]; }
    __device__ __forceinline__ void clear()
    {
#pragma unroll
        for (int y = 0; y < 3; ++y)
#pragma unroll
            for (int x = 0; x < 3; ++x) {
                a[y][x].x = a[y][x].y = (T)0;
#pragma unroll
                for (int c = 0; c < NC; ++c) p[c][y][x].x = p[c][y][x].y = (T)0;
            }
    }
};

// Packed view of a register window (PairView) from a RegView of the same
// site whose psi slots already hold the packed pairs.
template <class T, int NC>
__device__ __forceinline__ PairView<T> pair_view(const RegView<T, NC> &r)
{
    PairView<T> v;
#pragma unroll
    for (int y = 0; y < 3; ++y)
#pragma unroll
        for (int x = 0; x < 3; ++x) {
            v.a[y][x] = r.a[y][x];
            v.px[y][x] = r.p[0][y][x];
            v.py[y][x] = r.p[NC - 1][y][x];
        }
    return v;
}

template <class T>
__device__ __forceinline__ vec2_t<T> zero2()
{
    vec2_t<T> z;
    z.x = z.y = (T)0;
    return z;
}

// Value of the lane to the right (column + 1); lane 31 takes its halo.
template <class T>
__device__ __forceinline__ vec2_t<T> from_right(vec2_t<T> v, vec2_t<T> halo, int lane)
{
    vec2_t<T> r;
    r.x = __shfl_down_sync(FULL_MASK, v.x, 1);
    r.y = __shfl_down_sync(FULL_MASK, v.y, 1);
    return lane == TX - 1 ? halo : r;
}

// Value of the lane to the left (column - 1); lane 0 takes its halo.
template <class T>
__device__ __forceinline__ T from_left(T v, T halo, int lane)
{
    const T l = __shfl_up_sync(FULL_MASK, v, 1);
    return lane == 0 ? halo : l;
}

template <class T>
__device__ __forceinline__ vec2_t<T> from_left2(vec2_t<T> v, vec2_t<T> halo, int lane)
{
    vec2_t<T> l;
    l.x = from_left<T>(v.x, halo.x, lane);
    l.y = from_left<T>(v.y, halo.y, lane);
    return l;
}

// Column geometry of one lane within its tile.
struct StripLane {
    int lane, gi, hc;   // own column, halo column (lanes 0 and 31)
    bool cok, hok;      // own column / halo column inside the lattice
};

__device__ __forceinline__ StripLane strip_lane(const StringDesc &S, int i0)
{
    StripLane L;
    L.lane = threadIdx.x & 31;
    L.gi = i0 + L.lane;
    L.hc = L.lane == 0 ? i0 - 1 : i0 + TX;
    L.cok = L.gi < S.nx;
    L.hok = (L.lane == 0 || L.lane == TX - 1) && L.hc >= 0 && L.hc < S.nx;
    return L;
}

// Loads of one row j: NA arrays of (1 + NC) pair fields at the lane's
// column (zero outside the lattice); array a is read if bit a of cmask is set.
template <class T, int NC, int NA>
__device__ __forceinline__ void strip_load(vec2_t<T> (&c)[NA][1 + NC], const vec2_t<T> *const (&src)[NA][1 + NC],
                                           const StringDesc &S, const StripLane &L, int j, unsigned cmask)
{
    const bool rok = j >= 0 && j < S.ny;
    const int sc_ = rok && L.cok ? L.gi + S.nx * j : 0;
#pragma unroll
    for (int a = 0; a < NA; ++a)
#pragma unroll
        for (int k = 0; k < 1 + NC; ++k) c[a][k] = zero2<T>();
#pragma unroll
    for (int a = 0; a < NA; ++a)
        if (((cmask >> a) & 1u) && rok && L.cok)
#pragma unroll
            for (int k = 0; k < 1 + NC; ++k) c[a][k] = src[a][k][sc_];
}

// Halo column of row j: lanes 0 and 31 copy arrays a < NR of hmask at their
// halo column into slot[side][a] by cp.async (zero-filled outside the
// lattice).  Every lane commits one group per call (empty for the others,
// or when `issue` is false), so group counts stay uniform.
template <class T, int NC, int NR, int NA>
__device__ __forceinline__ void strip_halo(vec2_t<T> (&slot)[2][NR][1 + NC], const vec2_t<T> *const (&src)[NA][1 + NC],
                                           const StringDesc &S, const StripLane &L, int j, unsigned hmask, bool issue)
{
    if (issue && (L.lane == 0 || L.lane == TX - 1)) {
        const bool hv = j >= 0 && j < S.ny && L.hok;
        const int sh = hv ? L.hc + S.nx * j : 0;
        vec2_t<T>(&dst)[NR][1 + NC] = slot[L.lane == 0 ? 0 : 1];
#pragma unroll
        for (int a = 0; a < NR; ++a)
            if ((hmask >> a) & 1u)
#pragma unroll
                for (int k = 0; k < 1 + NC; ++k) cp_async<sizeof(vec2_t<T>)>(&dst[a][k], src[a][k] + sh, hv);
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}

// Wait until at most N of this thread's newest cp.async groups are pending.
template <int N>
__device__ __forceinline__ void cp_async_wait_groups() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Tile g of the global tile order (strings in order, each from its
// tile_base: image, tile row, tile column), derived from the block index and
// the descriptors alone so that it is uniform over the block.
// ONE: the launch covers a single string (bt.n == 1); its descriptor is
// then read at fixed offsets, i.e. as constant operands, not through
// indexed constant loads.
template <bool ONE>
__device__ __forceinline__ TileRef strip_tile(const Batch &bt, int g)
{
    int s = 0;
    if (!ONE)
        for (int k = 1; k < bt.n; ++k)
            if (g >= bt.s[k].tile_base) s = k;
    TileRef t = flat_tile(bt.s[s], g - bt.s[s].tile_base);
    t.s = (int16_t)s;
    return t;
}

// Packed neighbour codes of the lane's site in row j (0 outside the lattice).
__device__ __forceinline__ uint16_t strip_code(const StringDesc &S, const StripLane &L, int j)
{
    if (!(j >= 0 && j < S.ny && L.cok)) return 0;
    const int s = L.gi + S.nx * j;
    return S.mask ? S.mask[s] : (uint16_t)((S.code_comp[s] & 0xff) | ((S.code_sc[s] & 0xff) << 8));
}

// Warp form of finish_image: the tile's NV partials leave from lane 0; if
// this tile is the last of its image, every lane receives the image sums
// (its partials added in index order) and the function returns true.
template <int NV, class T>
__device__ __forceinline__ bool finish_image_warp(const T (&v)[NV], const Scalars &sc, int tile, int first_tile,
                                                  int tiles_per_image, int img, double (&tot)[NV])
{
    const int lane = threadIdx.x & 31;
    T w[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        w[k] = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) w[k] += shfl_down(w[k], o);
    }
    int last = 0;
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) sc.part[(size_t)tile * 8 + k] = (double)w[k];
        __threadfence();
        last = atomicAdd(&sc.ticket[img], 1u) == (unsigned)tiles_per_image - 1;
    }
    last = __shfl_sync(FULL_MASK, last, 0);
    if (!last) return false;
    __threadfence();
    double acc[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[k] = 0.0;
    for (int t = lane; t < tiles_per_image; t += 32) {
        const double *p = sc.part + (size_t)(first_tile + t) * 8;
#pragma unroll
        for (int k = 0; k < NV; ++k) acc[k] += __ldcg(p + k);
    }
#pragma unroll
    for (int k = 0; k < NV; ++k) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_down_sync(FULL_MASK, acc[k], o);
        tot[k] = __shfl_sync(FULL_MASK, acc[k], 0);
    }
    if (lane == 0) sc.ticket[img] = 0;
    return true;
}

// One row of x + alpha d as the gradient window holds it: fields of the
// lane's column, A of the columns left and right, the row's previous
// gradient and neighbour codes.
template <class T, int NC>
struct GradRow {
    vec2_t<T> x[1 + NC], al, ar, gold[1 + NC];
    uint16_t m;
};

// Halo ring of the gradient pass: [row % 3][side][x, d][field].
template <class T, int NC>
using GradRing = vec2_t<T>[3][2][2][1 + NC];

// Pass A on one tile as a warp strip: x <- x + alpha_pend d over the tile
// (+ halo), the gradient of every site, |g|^2 and g . (g - g_prev); the last
// tile of an image computes beta.  Same semantics as k_grad.  Returns true
// (in every lane) when this tile finished its image.  Before the tile's
// partials are counted every lane fences its field stores, so that a
// consumer that has seen the image finished (same launch) reads them.
template <class T, int NC, bool ONE>
__device__ __forceinline__ bool grad_tile(const Batch &bt, const TileRef tr, const Scalars &sc, const StepFlags &f,
                                          GradRing<T, NC> &ring)
{
    constexpr int TYT = TileRows<T>::v;
    using V = vec2_t<T>;
    const StringDesc &S = bt.s[ONE ? 0 : tr.s];
    const int img = S.img_base + tr.n;
    const int i0 = tr.tx * TX, j0 = tr.ty * TYT;
    const size_t off = (size_t)tr.n * S.nx * S.ny;
    const StripLane L = strip_lane(S, i0);
    const V *src[3][1 + NC];
    V *xout[1 + NC], *gcur[1 + NC];
#pragma unroll
    for (int c = 0; c < 1 + NC; ++c) {
        src[0][c] = static_cast<const V *>(S.x[f.xin][c]) + off;
        src[1][c] = static_cast<const V *>(S.d[f.din][c]) + off;
        src[2][c] = static_cast<const V *>(S.g[f.gprev][c]) + off;
        xout[c] = static_cast<V *>(S.x[f.xout][c]) + off;
        gcur[c] = static_cast<V *>(S.g[f.gcur][c]) + off;
    }
    const T alpha = (T)__ldcg(sc.alpha_pend + img);
    const unsigned fields = alpha != (T)0 ? 3u : 1u;   // d is not read when nothing is pending
    SiteParams<T> p;
    p.load_uniform(S);
    V rc[3][1 + NC];
    uint16_t rm;
    // raw row j -> window row (x + alpha d; left / right A by shuffles)
    auto take = [&](GradRow<T, NC> &R, int j, V (&hp)[NC], const V (&raw)[3][1 + NC], uint16_t m) {
        cp_async_wait_groups<0>();   // row j's halo is in the newest groups
        const V(&h)[2][1 + NC] = ring[(j + 3) % 3][L.lane == 0 ? 0 : 1];
        V hx[1 + NC];
#pragma unroll
        for (int c = 0; c < 1 + NC; ++c) {
            R.x[c].x = raw[0][c].x + alpha * raw[1][c].x;
            R.x[c].y = raw[0][c].y + alpha * raw[1][c].y;
            const V hv = h[0][c], hd = fields & 2u ? h[1][c] : zero2<T>();
            hx[c].x = hv.x + alpha * hd.x;
            hx[c].y = hv.y + alpha * hd.y;
            R.gold[c] = raw[2][c];
        }
        if constexpr (StripPacked<T, NC>::v) {
            transpose_pair(R.x[1], R.x[NC]);
            transpose_pair(hx[1], hx[NC]);
        }
        R.al = from_left2<T>(R.x[0], hx[0], L.lane);
        R.ar = from_right<T>(R.x[0], hx[0], L.lane);
#pragma unroll
        for (int c = 0; c < NC; ++c) hp[c] = hx[1 + c];
        R.m = m;
    };
    auto load = [&](V (&raw)[3][1 + NC], uint16_t &m, int j, bool gold) {
        strip_load<T, NC, 3>(raw, src, S, L, j, gold ? fields | 4u : fields);
        strip_halo<T, NC, 2, 3>(ring[(j + 3) % 3], src, S, L, j, fields, true);
        m = strip_code(S, L, j);
    };
    GradRow<T, NC> Rm, R0, Rp;
    V hp0[NC], hp1[NC];
    {   // the first three rows are loaded together: one memory latency, not three
        V ra[3][1 + NC], rb[3][1 + NC];
        uint16_t ma, mb;
        load(ra, ma, j0 - 1, false);
        load(rb, mb, j0, true);
        load(rc, rm, j0 + 1, true);
        take(Rm, j0 - 1, hp0, ra, ma);
        take(R0, j0, hp0, rb, mb);
    }
    const int rows = S.ny - j0 < TYT ? S.ny - j0 : TYT;
    T v[2] = {(T)0, (T)0};
#if MEPGL_STRIP_UNROLL
#pragma unroll 3   // the window rotates with period 3: unrolled, its copies become renames
#else
#pragma unroll 1
#endif
    for (int r = 0; r < rows; ++r) {
        const int j = j0 + r;
        take(Rp, j + 1, hp1, rc, rm);
        if (r + 1 < rows) load(rc, rm, j + 2, true);
        const int s = L.gi + S.nx * j;
        if (L.cok) {
            V o[1 + NC];
#pragma unroll
            for (int c = 0; c < 1 + NC; ++c) o[c] = R0.x[c];
            if constexpr (StripPacked<T, NC>::v) transpose_pair(o[1], o[NC]);
#pragma unroll
            for (int c = 0; c < 1 + NC; ++c) xout[c][s] = o[c];
        }
        RegView<T, NC> w3;
        w3.clear();
        w3.a[0][0] = Rm.al; w3.a[0][1] = Rm.x[0]; w3.a[0][2] = Rm.ar;
        w3.a[1][0] = R0.al; w3.a[1][1] = R0.x[0]; w3.a[1][2] = R0.ar;
        w3.a[2][0] = Rp.al; w3.a[2][1] = Rp.x[0]; w3.a[2][2] = Rp.ar;
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            w3.p[c][0][1] = Rm.x[1 + c];
            w3.p[c][1][1] = R0.x[1 + c];
            w3.p[c][2][1] = Rp.x[1 + c];
            w3.p[c][1][0] = from_left2<T>(R0.x[1 + c], hp0[c], L.lane);
            w3.p[c][1][2] = from_right<T>(R0.x[1 + c], hp0[c], L.lane);
        }
        if (L.cok) {
            T hr = p.h, hl = p.h, hu = p.h, hd = p.h;
            if (S.per_site) {
                p.load_site(S, s, NC);
                hr = h_site(S, p, s + 1 < S.nx * S.ny ? s + 1 : s);
                hl = h_site(S, p, s > 0 ? s - 1 : s);
                hu = h_site(S, p, j + 1 < S.ny ? s + S.nx : s);
                hd = h_site(S, p, j > 0 ? s - S.nx : s);
            }
            T g[2 + 2 * NC];
            Wts<T> w;
            if constexpr (StripPacked<T, NC>::v) {
                w.load(R0.m);
                PairParams<T> pp;
                pp.set(p);
                site_gradient_pair<T>(pair_view(w3), p, pp, w, hr, hl, hu, hd, f.maxwell, S.thin_film, g);
            } else if (MEPGL_STRIP_INTERIOR && R0.m == 0xffffu) {   // interior site: unit weights, folded in
                w.interior();
                site_gradient_v<T, NC>(w3, p, w, hr, hl, hu, hd, f.maxwell, S.thin_film, g);
            } else {
                w.load(R0.m);
                site_gradient_v<T, NC>(w3, p, w, hr, hl, hu, hd, f.maxwell, S.thin_film, g);
            }
#pragma unroll
            for (int c = 0; c < 1 + NC; ++c) {
                V gv;
                gv.x = g[2 * c];
                gv.y = g[2 * c + 1];
                gcur[c][s] = gv;
                const V go = R0.gold[c];
                v[0] += gv.x * gv.x + gv.y * gv.y;
                v[1] += gv.x * (gv.x - go.x) + gv.y * (gv.y - go.y);
            }
        }
        Rm = R0;
        R0 = Rp;
#pragma unroll
        for (int c = 0; c < NC; ++c) hp0[c] = hp1[c];
    }
    const int tpi = S.tiles_x * S.tiles_y;
    double tot[2];
    __threadfence();
    __syncwarp();
    const bool fin = finish_image_warp<2>(v, sc, part_slot(S, tr), S.tile_base + tr.n * tpi, tpi, img, tot);
    if (fin && L.lane == 0) {
        (f.gcur ? sc.gn1 : sc.gn0)[img] = tot[0];
        sc.gdg[img] = tot[1];
        double beta = 0.0;
        if (f.use_cg) {
            beta = tot[1] / __ldcg((f.gprev ? sc.gn1 : sc.gn0) + img);
            beta = beta > 0.0 ? beta : 0.0;   // Polak-Ribiere clipped at 0; NaN -> 0
        }
        sc.beta[img] = beta;
    }
    return fin;
}

template <class T, int NC, bool ONE>
__global__ void __launch_bounds__(NTS, MEPGL_MINB_STRIP_GRAD) k_grad_s(const __grid_constant__ Batch bt,
                                                                  int tile0, Scalars sc, StepFlags f)
{
    __shared__ __align__(16) GradRing<T, NC> ring;
    grad_tile<T, NC, ONE>(bt, strip_tile<ONE>(bt, tile0 + (int)blockIdx.x), sc, f, ring);
}

// One row of the polynomial window: fields and new direction of the lane's
// column and the row's neighbour codes.
template <class T, int NC>
struct DirRow {
    vec2_t<T> x[1 + NC], d[1 + NC];
    uint16_t m;
};

// Halo ring of the direction pass: [row % 3][side][x, g, d][field].
template <class T, int NC>
using DirRing = vec2_t<T>[3][2][3][1 + NC];

// Pass B on one tile as a warp strip: d <- -g + beta d over the tile
// (+ halo), the quartic coefficients of F(x + a d); the last tile of an
// image runs the line search.  Same semantics as k_dir_poly.  Returns true
// (in every lane) when this tile finished its image; field stores are
// fenced as in grad_tile.
template <class T, int NC, bool ONE>
__device__ __forceinline__ bool dir_tile(const Batch &bt, const TileRef tr, const Scalars &sc, const StepFlags &f,
                                         DirRing<T, NC> &ring, double (&coef)[5])
{
    constexpr int TYT = TileRows<T>::v;
    using V = vec2_t<T>;
    const StringDesc &S = bt.s[ONE ? 0 : tr.s];
    const int img = S.img_base + tr.n;
    const int i0 = tr.tx * TX, j0 = tr.ty * TYT;
    const size_t off = (size_t)tr.n * S.nx * S.ny;
    const StripLane L = strip_lane(S, i0);
    const V *src[3][1 + NC];
    V *dout[1 + NC];
#pragma unroll
    for (int c = 0; c < 1 + NC; ++c) {
        src[0][c] = static_cast<const V *>(S.x[f.xout][c]) + off;
        src[1][c] = static_cast<const V *>(S.g[f.gcur][c]) + off;
        src[2][c] = static_cast<const V *>(S.d[f.din][c]) + off;
        dout[c] = static_cast<V *>(S.d[f.dout][c]) + off;
    }
    const T beta = (T)__ldcg(sc.beta + img);
    SiteParams<T> p;
    p.load_uniform(S);
    V rc[3][1 + NC];
    uint16_t rm;
    auto take = [&](DirRow<T, NC> &R, const V (&raw)[3][1 + NC], uint16_t m) {
#pragma unroll
        for (int c = 0; c < 1 + NC; ++c) {
            R.x[c] = raw[0][c];
            R.d[c].x = -raw[1][c].x + beta * raw[2][c].x;
            R.d[c].y = -raw[1][c].y + beta * raw[2][c].y;
        }
        if constexpr (StripPacked<T, NC>::v) {
            transpose_pair(R.x[1], R.x[NC]);
            transpose_pair(R.d[1], R.d[NC]);
        }
        R.m = m;
    };
    auto load = [&](V (&raw)[3][1 + NC], uint16_t &m, int j, bool issue) {
        strip_load<T, NC, 3>(raw, src, S, L, j, issue ? 7u : 0u);
        strip_halo<T, NC, 3, 3>(ring[(j + 3) % 3], src, S, L, j, 7u, issue);
        m = strip_code(S, L, j);
    };
    DirRow<T, NC> R0, Rp;
    T xm_ax, dm_ax;   // row j - 1: only A_x of x and of d is read
    {   // the first three rows are loaded together: one memory latency, not three
        V ra[3][1 + NC], rb[3][1 + NC];
        uint16_t ma, mb;
        load(ra, ma, j0 - 1, true);
        load(rb, mb, j0, true);
        load(rc, rm, j0 + 1, true);
        take(R0, ra, ma);
        xm_ax = R0.x[0].x;
        dm_ax = R0.d[0].x;
        take(R0, rb, mb);
    }
    const int rows = S.ny - j0 < TYT ? S.ny - j0 : TYT;
    T v[5] = {(T)0, (T)0, (T)0, (T)0, (T)0};
#if MEPGL_STRIP_UNROLL
#pragma unroll 2   // the window rotates with period 2: unrolled, its copies become renames
#else
#pragma unroll 1
#endif
    for (int r = 0; r < rows; ++r) {
        const int j = j0 + r;
        take(Rp, rc, rm);
        if (r + 1 < rows) load(rc, rm, j + 2, true);
        else strip_halo<T, NC, 3, 3>(ring[0], src, S, L, j + 2, 0u, false);
        cp_async_wait_groups<2>();   // groups of rows j + 1 and j + 2 may still be pending
        const int s = L.gi + S.nx * j;
        if (L.cok) {
            V o[1 + NC];
#pragma unroll
            for (int c = 0; c < 1 + NC; ++c) o[c] = R0.d[c];
            if constexpr (StripPacked<T, NC>::v) transpose_pair(o[1], o[NC]);
#pragma unroll
            for (int c = 0; c < 1 + NC; ++c) dout[c][s] = o[c];
        }
        // halo column of row j (this lane's side), new direction formed here
        const V(&h)[3][1 + NC] = ring[j % 3][L.lane == 0 ? 0 : 1];
        V hx[1 + NC], hd[1 + NC];
#pragma unroll
        for (int c = 0; c < 1 + NC; ++c) {
            hx[c] = h[0][c];
            const V hg = h[1][c], hdd = h[2][c];
            hd[c].x = -hg.x + beta * hdd.x;
            hd[c].y = -hg.y + beta * hdd.y;
        }
        if constexpr (StripPacked<T, NC>::v) {
            transpose_pair(hx[1], hx[NC]);
            transpose_pair(hd[1], hd[NC]);
        }
        RegView<T, NC> vx, vd;
        vx.clear();
        vd.clear();
        vx.a[1][1] = R0.x[0];
        vd.a[1][1] = R0.d[0];
        vx.a[1][2] = from_right<T>(R0.x[0], hx[0], L.lane);
        vd.a[1][2] = from_right<T>(R0.d[0], hd[0], L.lane);
        vx.a[1][0].y = from_left<T>(R0.x[0].y, hx[0].y, L.lane);
        vd.a[1][0].y = from_left<T>(R0.d[0].y, hd[0].y, L.lane);
        vx.a[0][1].x = xm_ax;
        vd.a[0][1].x = dm_ax;
        vx.a[2][1] = Rp.x[0];
        vd.a[2][1] = Rp.d[0];
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            vx.p[c][1][1] = R0.x[1 + c];
            vd.p[c][1][1] = R0.d[1 + c];
            vx.p[c][1][2] = from_right<T>(R0.x[1 + c], hx[1 + c], L.lane);
            vd.p[c][1][2] = from_right<T>(R0.d[1 + c], hd[1 + c], L.lane);
            vx.p[c][2][1] = Rp.x[1 + c];
            vd.p[c][2][1] = Rp.d[1 + c];
        }
        if (L.cok) {
            if (S.per_site) p.load_site(S, s, NC);
            T o[5];
            Wts<T> w;
            if constexpr (StripPacked<T, NC>::v) {
                w.load(R0.m);
                PairParams<T> pp;
                pp.set(p);
                site_poly_pair<T>(pair_view(vx), pair_view(vd), p, pp, w, f.poly_compat, S.thin_film, o);
            } else if (MEPGL_STRIP_INTERIOR && R0.m == 0xffffu) {   // interior site: unit weights, folded in
                w.interior();
                site_poly_v<T, NC>(vx, vd, p, w, f.poly_compat, S.thin_film, o);
            } else {
                w.load(R0.m);
                site_poly_v<T, NC>(vx, vd, p, w, f.poly_compat, S.thin_film, o);
            }
#pragma unroll
            for (int k = 0; k < 5; ++k) v[k] += o[k];
        }
        xm_ax = R0.x[0].x;
        dm_ax = R0.d[0].x;
        R0 = Rp;
    }
    // the halo copy of the row below the tile may still be in flight: complete it before the
    // ring can be reused (the fused kernel runs more tiles in the same block)
    cp_async_wait_groups<0>();
    const int tpi = S.tiles_x * S.tiles_y;
    double tot[5];
    __threadfence();
    __syncwarp();
    const bool fin = finish_image_warp<5>(v, sc, part_slot(S, tr), S.tile_base + tr.n * tpi, tpi, img, tot);
    if (fin) {
        if (L.lane == 0) {
#pragma unroll
            for (int k = 0; k < 5; ++k) coef[k] = tot[k];
            sc.fenergy[img] = tot[0];
#pragma unroll
            for (int k = 0; k < 4; ++k) sc.poly[4 * img + k] = tot[1 + k];
        }
        __syncwarp();
        // the scan's grid and rounding follow the stored precision
        const double *xt = sizeof(store_t<T>) == 8 ? sc.xtab_d : sc.xtab_f;
        double alpha = line_search_scan<store_t<T>>(coef, xt);
        if (f.ls_exact) alpha = line_search_exact(coef, alpha);
        if (L.lane == 0) {
            sc.alpha[img] = alpha;
            sc.alpha_pend[img] = alpha;
        }
        __syncwarp();
    }
    return fin;
}

template <class T, int NC, bool ONE>
__global__ void __launch_bounds__(NTS, MEPGL_MINB_STRIP_DIR) k_dir_poly_s(const __grid_constant__ Batch bt,
                                                                      int tile0, Scalars sc, StepFlags f)
{
    __shared__ __align__(16) DirRing<T, NC> ring;
    __shared__ double coef[5];
    dir_tile<T, NC, ONE>(bt, strip_tile<ONE>(bt, tile0 + (int)blockIdx.x), sc, f, ring, coef);
}

// ------------------------------------------------------------ fused steps
// `steps` NLCG steps of one launch's tiles in a single persistent launch.
// Work items are (step, pass, tile) in that order, handed out by a global
// counter.  The direction pass of an image needs only that image's
// gradient pass of the same step, and the next gradient pass of an image
// needs only its direction pass (the step alpha), so an item waits on a
// per-image stage counter instead of a kernel boundary: stage = 2k + 1 once
// the gradient pass of step k finished the image, 2k + 2 once its
// direction pass did.  An item depends only on items handed out before it,
// and an item is only taken by a running block, so the waits always end;
// each is still bounded, and a wait that runs out sets status[0] and
// ends its block.

// Step plan of a fused launch: the buffers and gradient slot of step k
// follow from those of step 0 as the separate launches toggle them.
struct StepPlan {
    int xi0, di0, it0;   // x and d buffers read by step 0; iteration number of step 0
    StepFlags base;      // use_cg, maxwell and the line-search options
    __device__ __forceinline__ StepFlags step(int k) const
    {
        StepFlags f = base;
        f.gcur = (it0 + k) & 1;
        f.gprev = f.gcur ^ 1;
        f.xin = xi0 ^ (k & 1);
        f.xout = f.xin ^ 1;
        f.din = di0 ^ (k & 1);
        f.dout = f.din ^ 1;
        return f;
    }
};

// Lane 0 waits until stage >= need (acquire, then a fence so that the whole
// warp's later loads see what the finishing block wrote), polling at most
// max_polls times; false if the wait ran out.
__device__ __forceinline__ bool wait_stage(const unsigned *stage, unsigned need, unsigned max_polls, int *status)
{
    int ok = 1;
    if ((threadIdx.x & 31) == 0) {
        unsigned polls = 0, v;
        for (;;) {
            asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(stage) : "memory");
            if (v >= need) break;
            if (++polls > max_polls) {
                atomicExch(status, 1);
                ok = 0;
                break;
            }
            __nanosleep(64);
        }
        __threadfence();
    }
    ok = __shfl_sync(FULL_MASK, ok, 0);
    __syncwarp();
    return ok != 0;
}

__device__ __forceinline__ void publish_stage(unsigned *stage, unsigned value)
{
    if ((threadIdx.x & 31) == 0) {
        __threadfence();
        asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(stage), "r"(value) : "memory");
    }
    __syncwarp();
}

// Register budget of the fused kernel: an explicit cap, or the one
// resident-block target implies.
#if MEPGL_MAXREG_FUSED
#define MEPGL_FUSED_BOUNDS __maxnreg__(MEPGL_MAXREG_FUSED)
#else
#define MEPGL_FUSED_BOUNDS __launch_bounds__(NTS, MEPGL_MINB_STRIP_FUSED)
#endif

template <class T, int NC, bool ONE>
__global__ void MEPGL_FUSED_BOUNDS k_nlcg_s(const __grid_constant__ Batch bt, int tile0, int n_tiles, int steps,
                                            StepPlan plan, Scalars sc, unsigned long long *queue, unsigned *stage,
                                            unsigned max_polls)
{
    __shared__ __align__(16) GradRing<T, NC> gring;
    __shared__ __align__(16) DirRing<T, NC> dring;
    __shared__ double coef[5];
    const unsigned long long per_step = 2ull * (unsigned long long)n_tiles;
    const unsigned long long total = per_step * (unsigned long long)steps;
    for (;;) {
        unsigned long long item = 0;
        if ((threadIdx.x & 31) == 0) item = atomicAdd(queue, 1ull);
        item = __shfl_sync(FULL_MASK, item, 0);
        if (item >= total) return;
        const int k = (int)(item / per_step);
        const int r = (int)(item - (unsigned long long)k * per_step);
        const int pass = r >= n_tiles ? 1 : 0, u = r - pass * n_tiles;
        const TileRef tr = strip_tile<ONE>(bt, tile0 + u);
        const int img = bt.s[ONE ? 0 : tr.s].img_base + tr.n;
        const unsigned need = 2u * (unsigned)k + (unsigned)pass;
        if (need > 0 && !wait_stage(stage + img, need, max_polls, sc.status)) return;
        const StepFlags f = plan.step(k);
        if (pass == 0) {
            if (grad_tile<T, NC, ONE>(bt, tr, sc, f, gring)) publish_stage(stage + img, need + 1);
        } else {
            if (dir_tile<T, NC, ONE>(bt, tr, sc, f, dring, coef)) publish_stage(stage + img, need + 1);
        }
    }
}
