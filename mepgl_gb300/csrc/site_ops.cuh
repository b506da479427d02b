// site_ops.cuh -- per-site Ginzburg-Landau stencil terms read from a
// shared-memory tile (tile + one-site halo).
//
// The discretisation is the reference's (mepgl/src/nlcg.cu): psi and A live
// on sites; on a link i -> j along e the kinetic term uses the linearised
// covariant differences
//   u0 = -(Re psi_j - Re psi_i)/dx - q A_i,e Im psi_i   (u1: A_j, psi_j)
//   v0 = +(Im psi_j - Im psi_i)/dx - q A_i,e Re psi_i   (v1: A_j, psi_j)
// with energy (u0^2 + u1^2 + v0^2 + v1^2) / (4 m) times the fraction of the
// two superconducting plaquettes sharing the link; the magnetic term takes,
// at every site, four collocated views of curl A - h (forward/backward
// differences of A_y along x and of A_x along y), each weighted 1/8 when the
// plaquette is inside the computational domain.
//
// Domain handling is branchless: every link / plaquette term is multiplied
// by a weight that is zero when the reference would skip it.  The weights
// of a site come from two constant tables indexed by its 8-bit neighbour
// codes (bit order 0:+x 1:+x+y 2:+y 3:-x+y 4:-x 5:-x-y 6:-y 7:+x-y,
// nlcg.cu:48-103), so no bit arithmetic or int->float conversion runs per
// site.  Outside-lattice halo values are zero, so masked terms are finite.
#pragma once

#include "common.cuh"

namespace mepgl {

// Weights of a superconducting code: area fraction, link weights (forward
// x, backward x, forward y, backward y; zero when the link is absent), and
// the bare link bits (used by J).  Of a computational code: the validity
// (0/1) of the four curl views UR, UL, LL, LR.
template <class T>
struct MaskTable {
    T sc[256][12];    // area, wfx, wbx, wfy, wby, lfx, lbx, lfy, lby, 0, 0, 0
    T cc[256][4];     // vUR, vUL, vLL, vLR
};
// Defined here: kernels.cu is the only translation unit that includes this file.
__constant__ MaskTable<float> c_mask_f;
__constant__ MaskTable<double> c_mask_d;

template <class T> __device__ __forceinline__ const MaskTable<T> &mask_table();
template <> __device__ __forceinline__ const MaskTable<float> &mask_table<float>() { return c_mask_f; }
template <> __device__ __forceinline__ const MaskTable<double> &mask_table<double>() { return c_mask_d; }
// the weights are multiples of 1/4, exact in float: float-float reads the float table
template <class T> struct MaskOf { using type = T; };
template <> struct MaskOf<ff> { using type = float; };

template <class T>
struct Wts {
    T area, wfx, wbx, wfy, wby, lfx, lbx, lfy, lby;
    T vUR, vUL, vLL, vLR;
    __device__ __forceinline__ void load(unsigned mk)
    {
        const auto &M = mask_table<typename MaskOf<T>::type>();
        const unsigned s = mk >> 8, c = mk & 0xffu;
        area = M.sc[s][0]; wfx = M.sc[s][1]; wbx = M.sc[s][2]; wfy = M.sc[s][3]; wby = M.sc[s][4];
        lfx = M.sc[s][5]; lbx = M.sc[s][6]; lfy = M.sc[s][7]; lby = M.sc[s][8];
        vUR = M.cc[c][0]; vUL = M.cc[c][1]; vLL = M.cc[c][2]; vLR = M.cc[c][3];
    }
    // weights of a site whose eight neighbours are all inside both domains
    // (codes 0xff | 0xff << 8): every weight is 1
    __device__ __forceinline__ void interior()
    {
        area = wfx = wbx = wfy = wby = lfx = lbx = lfy = lby = (T)1;
        vUR = vUL = vLL = vLR = (T)1;
    }
};

// Host-side construction of the tables (same arithmetic as nlcg.cu:522-525,
// 186-187, 533-609 etc.: weights are exact multiples of 1/4).
template <class T>
inline void build_mask_table(MaskTable<T> &M)
{
    for (unsigned k = 0; k < 256; ++k) {
        auto b = [&](int n) { return (int)((k >> n) & 1u); };
        M.sc[k][0] = (T)(b(0) * b(1) * b(2) + b(2) * b(3) * b(4) + b(4) * b(5) * b(6) + b(6) * b(7) * b(0)) / (T)4;
        M.sc[k][1] = b(0) ? (T)(b(1) * b(2) + b(6) * b(7)) / (T)2 : (T)0;
        M.sc[k][2] = b(4) ? (T)(b(2) * b(3) + b(5) * b(6)) / (T)2 : (T)0;
        M.sc[k][3] = b(2) ? (T)(b(0) * b(1) + b(3) * b(4)) / (T)2 : (T)0;
        M.sc[k][4] = b(6) ? (T)(b(4) * b(5) + b(7) * b(0)) / (T)2 : (T)0;
        M.sc[k][5] = (T)b(0);
        M.sc[k][6] = (T)b(4);
        M.sc[k][7] = (T)b(2);
        M.sc[k][8] = (T)b(6);
        M.sc[k][9] = M.sc[k][10] = M.sc[k][11] = (T)0;
        M.cc[k][0] = (T)(b(0) & b(1) & b(2));
        M.cc[k][1] = (T)(b(2) & b(3) & b(4));
        M.cc[k][2] = (T)(b(4) & b(5) & b(6));
        M.cc[k][3] = (T)(b(6) & b(7) & b(0));
    }
}

// Fields of a tile of TYT rows (+ halo): A, psi_1[, psi_2].
template <class T, int NC, int TYT>
struct TileF {
    vec2_t<T> A[TYT + 2][TX + 2];
    vec2_t<T> P[NC][TYT + 2][TX + 2];
};

// The same with the packed neighbour codes of each site.
template <class T, int NC, int TYT>
struct Tile : TileF<T, NC, TYT> {
    uint16_t m[TYT + 2][TX + 2];
};

// Neighbourhood of one site read from a shared-memory tile: A(dx, dy) and
// P(c, dx, dy) for |dx|, |dy| <= 1.  The stencil functions below that take a
// view also run on register windows (the strip kernels).
template <class T, int NC, int TYT>
struct TileView {
    const TileF<T, NC, TYT> &t;
    int lx, ly;
    __device__ __forceinline__ vec2_t<T> A(int dx, int dy) const { return t.A[ly + dy][lx + dx]; }
    __device__ __forceinline__ vec2_t<T> P(int c, int dx, int dy) const { return t.P[c][ly + dy][lx + dx]; }
};

// Parameters of one site (uniform strings read the descriptor).
template <class T>
struct SiteParams {
    T a[2], b[2], hmx[2], hmy[2], aob[2];  // hmx = 0.5 / m_xx
    T q[2], eta, gamma, delta, h, idx, dx2, dx;
    __device__ __forceinline__ void load_uniform(const StringDesc &S)
    {
        const Uniform<T> &U = S.template u<T>();
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            a[c] = U.a[c]; b[c] = U.b[c]; hmx[c] = U.hmx[c]; hmy[c] = U.hmy[c]; aob[c] = U.aob[c]; q[c] = U.q[c];
        }
        eta = U.eta; gamma = U.gamma; delta = U.delta; h = U.h; idx = U.idx; dx2 = U.dx2; dx = U.dx;
    }
    // per-site overrides (strings whose parameter arrays are not uniform)
    __device__ __forceinline__ void load_site(const StringDesc &S, int s, int nc)
    {
        using St = store_t<T>;
        for (int c = 0; c < nc; ++c) {
            const St av = static_cast<const St *>(S.pa[c])[s], bv = static_cast<const St *>(S.pb[c])[s];
            a[c] = from_store<T>(av);
            b[c] = from_store<T>(bv);
            hmx[c] = from_store<T>((St)0.5 / static_cast<const St *>(S.pmxx[c])[s]);
            hmy[c] = from_store<T>((St)0.5 / static_cast<const St *>(S.pmyy[c])[s]);
            aob[c] = from_store<T>(av / bv);
        }
        h = from_store<T>(static_cast<const St *>(S.ph)[s]);
    }
};

template <class T>
__device__ __forceinline__ void link4(T Ai, T Aj, vec2_t<T> pi, vec2_t<T> pj, T q, T idx, T t[4])
{
    const T dre = (pj.x - pi.x) * idx, dim = (pj.y - pi.y) * idx;
    const T qi = q * Ai, qj = q * Aj;
    t[0] = -dre - qi * pi.y;
    t[1] = -dre - qj * pj.y;
    t[2] = dim - qi * pi.x;
    t[3] = dim - qj * pj.x;
}

#define TA(dx_, dy_) (t.A[ly + (dy_)][lx + (dx_)])
#define TP(c_, dx_, dy_) (t.P[c_][ly + (dy_)][lx + (dx_)])

// Free-energy density x dx^2 (freeEnergyDensity, nlcg.cu:105-214).
template <class T, int NC, int TYT>
__device__ __forceinline__ T site_energy(const Tile<T, NC, TYT> &t, int lx, int ly, const SiteParams<T> &p,
                                         const Wts<T> &w, int thin_film)
{
    const vec2_t<T> A0 = TA(0, 0);
    T nl = 0;
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        const vec2_t<T> P0 = TP(c, 0, 0);
        const T r = p.aob[c] + P0.x * P0.x + P0.y * P0.y;
        nl += p.b[c] * (T)0.5 * r * r;
    }
    if (NC == 2) {
        const vec2_t<T> P1 = TP(0, 0, 0), P2 = TP(NC - 1, 0, 0);
        const T R = P1.x * P2.x + P1.y * P2.y, I = P1.x * P2.y - P1.y * P2.x;
        nl += p.eta * R;
        nl += p.gamma * (T)0.5 * (P1.x * P1.x + P1.y * P1.y) * (P2.x * P2.x + P2.y * P2.y);
        nl += p.delta * (T)0.5 * (R * R - I * I);
    }
    T kx = 0, ky = 0;
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        T q4[4];
        link4(A0.x, TA(1, 0).x, TP(c, 0, 0), TP(c, 1, 0), p.q[c], p.idx, q4);
        kx += (T)0.5 * p.hmx[c] * (q4[0] * q4[0] + q4[1] * q4[1] + q4[2] * q4[2] + q4[3] * q4[3]);
        link4(A0.y, TA(0, 1).y, TP(c, 0, 0), TP(c, 0, 1), p.q[c], p.idx, q4);
        ky += (T)0.5 * p.hmy[c] * (q4[0] * q4[0] + q4[1] * q4[1] + q4[2] * q4[2] + q4[3] * q4[3]);
    }
    T em = 0;
    if (!thin_film) {
        const T ayp = (TA(1, 0).y - A0.y) * p.idx, aym = (A0.y - TA(-1, 0).y) * p.idx;
        const T axp = (TA(0, 1).x - A0.x) * p.idx, axm = (A0.x - TA(0, -1).x) * p.idx;
        const T r0 = ayp - axp - p.h, r1 = aym - axp - p.h, r2 = aym - axm - p.h, r3 = ayp - axm - p.h;
        em = (T)0.125 * (w.vUR * r0 * r0 + w.vUL * r1 * r1 + w.vLL * r2 * r2 + w.vLR * r3 * r3);
    }
    return (kx * w.wfx + ky * w.wfy + nl * w.area + em) * p.dx2;
}

// Partial derivatives of site_energy at fixed fields with respect to a
// uniform shift of the applied field h, to eta and to gamma (no reference
// counterpart): out[0] = -1/4 sum_views w_v (curl - h), out[1] = area Re(psi1
// psi2*), out[2] = area |psi1|^2 |psi2|^2 / 2, each times dx^2.
template <class T, int NC, int TYT>
__device__ __forceinline__ void site_param_adjoint(const Tile<T, NC, TYT> &t, int lx, int ly,
                                                   const SiteParams<T> &p, const Wts<T> &w, int thin_film, T *out)
{
    if (NC == 2) {
        const vec2_t<T> P1 = TP(0, 0, 0), P2 = TP(NC - 1, 0, 0);
        out[1] += (P1.x * P2.x + P1.y * P2.y) * w.area * p.dx2;
        out[2] += (T)0.5 * (P1.x * P1.x + P1.y * P1.y) * (P2.x * P2.x + P2.y * P2.y) * w.area * p.dx2;
    }
    if (!thin_film) {
        const vec2_t<T> A0 = TA(0, 0);
        const T ayp = (TA(1, 0).y - A0.y) * p.idx, aym = (A0.y - TA(-1, 0).y) * p.idx;
        const T axp = (TA(0, 1).x - A0.x) * p.idx, axm = (A0.x - TA(0, -1).x) * p.idx;
        const T r0 = ayp - axp - p.h, r1 = aym - axp - p.h, r2 = aym - axm - p.h, r3 = ayp - axm - p.h;
        out[0] -= (T)0.25 * (w.vUR * r0 + w.vUL * r1 + w.vLL * r2 + w.vLR * r3) * p.dx2;
    }
}

// ------------------------------------------------------- gauge links
// The link (Peierls) discretisation of the same functional (no reference
// counterpart): A_e at a site is the variable of the link to its +e
// neighbour; per link and component the kinetic energy is
// w_e / (2 m_e) |psi_t - U psi_s|^2 with U = exp(i q A_e dx); per plaquette
// (lower-left corner s) 1/2 v_UR (B - h)^2 dx^2 with
// B = (A_x(s) + A_y(s+x) - A_x(s+y) - A_y(s)) / dx.  Exactly invariant under
// psi -> psi e^{i q chi}, A_e(s) -> A_e(s) + (chi(s+e) - chi(s)) / dx.
template <class T> __device__ __forceinline__ void cis(T a, T &c, T &s);
template <> __device__ __forceinline__ void cis<float>(float a, float &c, float &s) { sincosf(a, &s, &c); }
template <> __device__ __forceinline__ void cis<double>(double a, double &c, double &s) { sincos(a, &s, &c); }

template <class T>
__device__ __forceinline__ T cond_density(const vec2_t<T> *P, int nc, const SiteParams<T> &p)
{
    T nl = 0;
    for (int c = 0; c < nc; ++c) {
        const T r = p.aob[c] + P[c].x * P[c].x + P[c].y * P[c].y;
        nl += p.b[c] * (T)0.5 * r * r;
    }
    if (nc == 2) {
        const T R = P[0].x * P[1].x + P[0].y * P[1].y, I = P[0].x * P[1].y - P[0].y * P[1].x;
        nl += p.eta * R + p.gamma * (T)0.5 * (P[0].x * P[0].x + P[0].y * P[0].y) * (P[1].x * P[1].x + P[1].y * P[1].y)
            + p.delta * (T)0.5 * (R * R - I * I);
    }
    return nl;
}

template <class T, int NC, int TYT>
__device__ __forceinline__ T site_energy_link(const Tile<T, NC, TYT> &t, int lx, int ly, const SiteParams<T> &p,
                                              const Wts<T> &w, int thin_film)
{
    vec2_t<T> P0[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) P0[c] = TP(c, 0, 0);
    const T nl = cond_density<T>(P0, NC, p);
    T kin = 0;
#pragma unroll
    for (int dir = 0; dir < 2; ++dir) {
        const int ox = dir == 0 ? 1 : 0, oy = 1 - ox;
        const T Ae = dir == 0 ? TA(0, 0).x : TA(0, 0).y, wl = dir == 0 ? w.wfx : w.wfy;
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            T cu, su;
            cis<T>(p.q[c] * Ae * p.dx, cu, su);
            const vec2_t<T> ps = P0[c], pt = TP(c, ox, oy);
            const T zr = pt.x - (cu * ps.x - su * ps.y), zi = pt.y - (su * ps.x + cu * ps.y);
            kin += wl * (dir == 0 ? p.hmx[c] : p.hmy[c]) * (zr * zr + zi * zi);
        }
    }
    T em = 0;
    if (!thin_film) {
        const T B = (TA(0, 0).x + TA(1, 0).y - TA(0, 1).x - TA(0, 0).y) * p.idx - p.h;
        em = (T)0.5 * w.vUR * B * B;
    }
    return kin + (nl * w.area + em) * p.dx2;
}

// Gradient of the link functional at one site (gather form): its own
// forward links, the backward links owned by its -x / -y neighbours (whose
// masses are hmx_l / hmy_d = 1 / (2 m) there), and the plaquettes with
// lower-left corners s, s-x, s-y (applied fields h, hl, hd).
template <class T, int NC, int TYT>
__device__ __forceinline__ void site_gradient_link(const Tile<T, NC, TYT> &t, int lx, int ly, const SiteParams<T> &p,
                                                   const Wts<T> &w, T hl, T hd, const T *hmx_l, const T *hmy_d,
                                                   int maxwell, int thin_film, T *out)
{
#pragma unroll
    for (int k = 0; k < 2 + 2 * NC; ++k) out[k] = 0;
    const T ar = w.area * p.dx2;
    vec2_t<T> P0[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) P0[c] = TP(c, 0, 0);
    if (!maxwell) {
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            const T x = P0[c].x, y = P0[c].y, r2 = x * x + y * y;
            out[2 + 2 * c] += (T)2 * x * (p.a[c] + p.b[c] * r2) * ar;
            out[3 + 2 * c] += (T)2 * y * (p.a[c] + p.b[c] * r2) * ar;
        }
        if (NC == 2) {
            const T x1 = P0[0].x, y1 = P0[0].y, x2 = P0[NC - 1].x, y2 = P0[NC - 1].y;
            const T R = x1 * x2 + y1 * y2, I = x1 * y2 - y1 * x2, r1 = x1 * x1 + y1 * y1, r2 = x2 * x2 + y2 * y2;
            out[2] += (p.eta * x2 + p.gamma * x1 * r2 + p.delta * (R * x2 - I * y2)) * ar;
            out[3] += (p.eta * y2 + p.gamma * y1 * r2 + p.delta * (R * y2 + I * x2)) * ar;
            out[2 + 2 * (NC - 1)] += (p.eta * x1 + p.gamma * x2 * r1 + p.delta * (R * x1 + I * y1)) * ar;
            out[3 + 2 * (NC - 1)] += (p.eta * y1 + p.gamma * y2 * r1 + p.delta * (R * y1 - I * x1)) * ar;
        }
    }
#pragma unroll
    for (int dir = 0; dir < 2; ++dir) {
        const int ox = dir == 0 ? 1 : 0, oy = 1 - ox;
        const T Ae = dir == 0 ? TA(0, 0).x : TA(0, 0).y, wf = dir == 0 ? w.wfx : w.wfy;
        const T Ab = dir == 0 ? TA(-1, 0).x : TA(0, -1).y, wb = dir == 0 ? w.wbx : w.wby;
        T ga = 0;
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            const T q = p.q[c];
            // own forward link s -> s + e
            const T kf = wf * (dir == 0 ? p.hmx[c] : p.hmy[c]);
            T cu, su;
            cis<T>(q * Ae * p.dx, cu, su);
            const vec2_t<T> ps = P0[c], pt = TP(c, ox, oy);
            const T ur = cu * ps.x - su * ps.y, ui = su * ps.x + cu * ps.y;
            const T zr = pt.x - ur, zi = pt.y - ui;
            ga += (T)2 * kf * q * p.dx * (zr * ui - zi * ur);
            // backward link s - e -> s, owned by the neighbour
            const T kb = wb * (dir == 0 ? hmx_l[c] : hmy_d[c]);
            T cb, sb;
            cis<T>(q * Ab * p.dx, cb, sb);
            const vec2_t<T> pb = TP(c, -ox, -oy);
            const T br = ps.x - (cb * pb.x - sb * pb.y), bi = ps.y - (sb * pb.x + cb * pb.y);
            if (!maxwell) {
                out[2 + 2 * c] += (T)2 * kb * br - (T)2 * kf * (cu * zr + su * zi);
                out[3 + 2 * c] += (T)2 * kb * bi - (T)2 * kf * (cu * zi - su * zr);
            }
        }
        if (!thin_film) out[dir] += ga;
    }
    if (!thin_film) {
        const T r0 = w.vUR * ((TA(0, 0).x + TA(1, 0).y - TA(0, 1).x - TA(0, 0).y) * p.idx - p.h) * p.dx;
        const T rd = w.vLR * ((TA(0, -1).x + TA(1, -1).y - TA(0, 0).x - TA(0, -1).y) * p.idx - hd) * p.dx;
        const T rl = w.vUL * ((TA(-1, 0).x + TA(0, 0).y - TA(-1, 1).x - TA(-1, 0).y) * p.idx - hl) * p.dx;
        out[0] += r0 - rd;
        out[1] += rl - r0;
    }
}

// dF/dH of the link functional at one site: -v_UR (B - h) dx^2.
template <class T, int NC, int TYT>
__device__ __forceinline__ T site_dh_link(const Tile<T, NC, TYT> &t, int lx, int ly, const SiteParams<T> &p,
                                          const Wts<T> &w)
{
    return -w.vUR * ((TA(0, 0).x + TA(1, 0).y - TA(0, 1).x - TA(0, 0).y) * p.idx - p.h) * p.dx2;
}

// Gradient dF/dA (out[0..1]) and dF/dpsi_c (out[2+2c..]) at one site,
// restating gradientPsi (nlcg.cu:504-744) and gradientA (nlcg.cu:746-888).
// Both link ends use the mass of this site, as the reference does.  hr, hl,
// hu, hd: applied field at the right, left, upper and lower neighbours.
#define VA(dx_, dy_) (v.A((dx_), (dy_)))
#define VP(c_, dx_, dy_) (v.P((c_), (dx_), (dy_)))
template <class T, int NC, class View>
__device__ __forceinline__ void site_gradient_v(const View &v, const SiteParams<T> &p, const Wts<T> &w, T hr, T hl,
                                                T hu, T hd, int maxwell, int thin_film, T *out)
{
    const vec2_t<T> A0 = VA(0, 0);
    const vec2_t<T> Ar = VA(1, 0), Al = VA(-1, 0), Au = VA(0, 1), Ad = VA(0, -1);
    T gax = 0, gay = 0;
    const T idx = p.idx;
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        const vec2_t<T> P0 = VP(c, 0, 0);
        const T x = P0.x, y = P0.y, r2 = x * x + y * y, q = p.q[c];
        T gx = (2 * p.a[c] * x + p.b[c] * 2 * x * r2) * w.area;
        T gy = (2 * p.a[c] * y + p.b[c] * 2 * y * r2) * w.area;
        T u[4];
        {
            link4(A0.x, Ar.x, P0, VP(c, 1, 0), q, idx, u);
            const T f = p.hmx[c] * w.wfx, qa = q * A0.x;
            gx += f * ((u[0] + u[1]) * idx - qa * u[2]);
            gy += f * (-(u[2] + u[3]) * idx - qa * u[0]);
            gax -= f * q * (y * u[0] + x * u[2]);
        }
        {
            link4(Al.x, A0.x, VP(c, -1, 0), P0, q, idx, u);
            const T f = p.hmx[c] * w.wbx, qa = q * A0.x;
            gx += f * (-(u[1] + u[0]) * idx - qa * u[3]);
            gy += f * ((u[3] + u[2]) * idx - qa * u[1]);
            gax -= f * q * (y * u[1] + x * u[3]);
        }
        {
            link4(A0.y, Au.y, P0, VP(c, 0, 1), q, idx, u);
            const T f = p.hmy[c] * w.wfy, qa = q * A0.y;
            gx += f * ((u[0] + u[1]) * idx - qa * u[2]);
            gy += f * (-(u[2] + u[3]) * idx - qa * u[0]);
            gay -= f * q * (y * u[0] + x * u[2]);
        }
        {
            link4(Ad.y, A0.y, VP(c, 0, -1), P0, q, idx, u);
            const T f = p.hmy[c] * w.wby, qa = q * A0.y;
            gx += f * (-(u[1] + u[0]) * idx - qa * u[3]);
            gy += f * ((u[3] + u[2]) * idx - qa * u[1]);
            gay -= f * q * (y * u[1] + x * u[3]);
        }
        out[2 + 2 * c] = gx;
        out[3 + 2 * c] = gy;
    }
    if (NC == 2) {
        const vec2_t<T> P1 = VP(0, 0, 0), P2 = VP(NC - 1, 0, 0);
        const T x1 = P1.x, y1 = P1.y, x2 = P2.x, y2 = P2.y;
        const T r1 = x1 * x1 + y1 * y1, r2 = x2 * x2 + y2 * y2;
        const T R = x1 * x2 + y1 * y2, I = x1 * y2 - y1 * x2;
        out[2] += (p.eta * x2 + p.gamma * x1 * r2 + p.delta * (x2 * R - y2 * I)) * w.area;
        out[3] += (p.eta * y2 + p.gamma * y1 * r2 + p.delta * (y2 * R + x2 * I)) * w.area;
        out[2 + 2 * (NC - 1)] += (p.eta * x1 + p.gamma * x2 * r1 + p.delta * (x1 * R + y1 * I)) * w.area;
        out[3 + 2 * (NC - 1)] += (p.eta * y1 + p.gamma * y2 * r1 + p.delta * (y1 * R - x1 * I)) * w.area;
    }
#pragma unroll
    for (int k = 2; k < 2 + 2 * NC; ++k) out[k] = maxwell ? (T)0 : out[k] * p.dx2;

    if (!thin_film) {
        // link differences ex(i,j) = d_x A_y on the x-link i -> i+1, ey(i,j) = d_y A_x
        const T ex0 = (Ar.y - A0.y) * idx, exm = (A0.y - Al.y) * idx;
        const T ey0 = (Au.x - A0.x) * idx, eym = (A0.x - Ad.x) * idx;
        const T exu = (VA(1, 1).y - Au.y) * idx, exmu = (Au.y - VA(-1, 1).y) * idx;
        const T exd = (VA(1, -1).y - Ad.y) * idx, exmd = (Ad.y - VA(-1, -1).y) * idx;
        const T eyr = (VA(1, 1).x - Ar.x) * idx, eyrm = (Ar.x - VA(1, -1).x) * idx;
        const T eyl = (VA(-1, 1).x - Al.x) * idx, eylm = (Al.x - VA(-1, -1).x) * idx;
        const T h = p.h;
        // residuals of the collocated views of this site and of the
        // neighbours' views of the same plaquettes (nlcg.cu:852-883)
        const T rUR = ex0 - ey0 - h, rUL = exm - ey0 - h, rLL = exm - eym - h, rLR = ex0 - eym - h;
        const T c4 = (T)0.25 * idx;
        gax += c4 * (w.vUR * (rUR + (exu - ey0 - hu)) + w.vUL * (rUL + (exmu - ey0 - hu)) -
                     w.vLL * (rLL + (exmd - eym - hd)) - w.vLR * (rLR + (exd - eym - hd)));
        gay += c4 * (-w.vUR * (rUR + (ex0 - eyr - hr)) + w.vUL * (rUL + (exm - eyl - hl)) +
                     w.vLL * (rLL + (exm - eylm - hl)) - w.vLR * (rLR + (ex0 - eyrm - hr)));
        out[0] = gax * p.dx2;
        out[1] = gay * p.dx2;
    } else {
        out[0] = 0;
        out[1] = 0;
    }
}

template <class T, int NC, int TYT>
__device__ __forceinline__ void site_gradient(const Tile<T, NC, TYT> &t, int lx, int ly, const SiteParams<T> &p,
                                              const Wts<T> &w, T hr, T hl, T hu, T hd, int maxwell, int thin_film,
                                              T *out)
{
    site_gradient_v<T, NC>(TileView<T, NC, TYT>{t, lx, ly}, p, w, hr, hl, hu, hd, maxwell, thin_film, out);
}

// Quartic coefficients of F(x + a d) at one site (polynomialExpansion,
// nlcg.cu:997-1370): out = {A, B, C, D, E}.  compat keeps the reference's
// x-link first-order slip and y-link halved cubic coefficient.
template <class T, int NC, class View, class DView>
__device__ __forceinline__ void site_poly_v(const View &v, const DView &dv, const SiteParams<T> &p, const Wts<T> &w,
                                            int compat, int thin_film, T *out)
{
    T e = 0, b1 = 0, c2 = 0, d3 = 0, e4 = 0;
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        const vec2_t<T> P0 = VP(c, 0, 0), D0 = dv.P(c, 0, 0);
        const T n0 = p.aob[c] + P0.x * P0.x + P0.y * P0.y;
        const T n1 = 2 * (P0.x * D0.x + P0.y * D0.y);
        const T n2 = D0.x * D0.x + D0.y * D0.y;
        const T bb = p.b[c];
        e += bb * ((T)0.5 * n0 * n0);
        b1 += bb * (n0 * n1);
        c2 += bb * ((T)0.5 * n1 * n1 + n0 * n2);
        d3 += bb * (n1 * n2);
        e4 += bb * ((T)0.5 * n2 * n2);
    }
    if (NC == 2) {
        const vec2_t<T> P1 = VP(0, 0, 0), P2 = VP(NC - 1, 0, 0);
        const vec2_t<T> D1 = dv.P(0, 0, 0), D2 = dv.P(NC - 1, 0, 0);
        const T x1 = P1.x, y1 = P1.y, x2 = P2.x, y2 = P2.y;
        const T u1 = D1.x, v1 = D1.y, u2 = D2.x, v2 = D2.y;
        const T R0 = x1 * x2 + y1 * y2, R1 = u1 * x2 + v1 * y2 + x1 * u2 + y1 * v2, R2 = u1 * u2 + v1 * v2;
        const T I0 = x1 * y2 - y1 * x2, I1 = x1 * v2 + u1 * y2 - y1 * u2 - v1 * x2, I2 = u1 * v2 - v1 * u2;
        const T r1 = x1 * x1 + y1 * y1, r2 = x2 * x2 + y2 * y2;
        const T s1 = 2 * (x1 * u1 + y1 * v1), s2 = 2 * (x2 * u2 + y2 * v2);
        const T t1 = u1 * u1 + v1 * v1, t2 = u2 * u2 + v2 * v2;
        const T g = p.gamma * (T)0.5, dd = p.delta * (T)0.5;
        e += p.eta * R0 + g * r1 * r2 + dd * (R0 * R0 - I0 * I0);
        b1 += p.eta * R1 + g * (s1 * r2 + s2 * r1) + dd * (2 * R1 * R0 - 2 * I1 * I0);
        c2 += p.eta * R2 + g * (s1 * s2 + r1 * t2 + r2 * t1) + dd * (R1 * R1 - I1 * I1 + 2 * R0 * R2 - 2 * I0 * I2);
        d3 += g * (s1 * t2 + s2 * t1) + dd * (2 * R1 * R2 - 2 * I1 * I2);
        e4 += g * (t1 * t2) + dd * (R2 * R2 - I2 * I2);
    }
    e *= w.area; b1 *= w.area; c2 *= w.area; d3 *= w.area; e4 *= w.area;
    if (!thin_film) {
        const vec2_t<T> A0 = VA(0, 0), a0 = dv.A(0, 0);
        const T idx = p.idx;
        const T ayp = (VA(1, 0).y - A0.y) * idx, aym = (A0.y - VA(-1, 0).y) * idx;
        const T axp = (VA(0, 1).x - A0.x) * idx, axm = (A0.x - VA(0, -1).x) * idx;
        const T dyp = (dv.A(1, 0).y - a0.y) * idx, dym = (a0.y - dv.A(-1, 0).y) * idx;
        const T dxp = (dv.A(0, 1).x - a0.x) * idx, dxm = (a0.x - dv.A(0, -1).x) * idx;
        T em0 = 0, em1 = 0, em2 = 0, m0, m1;
#define EMV(wv, yy, xx, dyy, dxx)        \
        m0 = yy - xx - p.h;              \
        m1 = dyy - dxx;                  \
        em0 += wv * (m0 * m0);           \
        em1 += wv * (m0 * m1);           \
        em2 += wv * (m1 * m1);
        EMV(w.vUR, ayp, axp, dyp, dxp)
        EMV(w.vUL, aym, axp, dym, dxp)
        EMV(w.vLL, aym, axm, dym, dxm)
        EMV(w.vLR, ayp, axm, dyp, dxm)
#undef EMV
        e += em0 * (T)0.125;
        b1 += em1 * (T)0.25;
        c2 += em2 * (T)0.125;
    }
#pragma unroll
    for (int dir = 0; dir < 2; ++dir) {
        const int ox = dir == 0 ? 1 : 0, oy = dir == 0 ? 0 : 1;
        const T Ai = dir == 0 ? VA(0, 0).x : VA(0, 0).y;
        const T Aj = dir == 0 ? VA(ox, oy).x : VA(ox, oy).y;
        const T ai = dir == 0 ? dv.A(0, 0).x : dv.A(0, 0).y;
        const T aj = dir == 0 ? dv.A(ox, oy).x : dv.A(ox, oy).y;
        const T wl = dir == 0 ? w.wfx : w.wfy;
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            const T q = p.q[c];
            const T qd = (compat && dir == 0) ? (T)-1 : q;
            const vec2_t<T> pi = VP(c, 0, 0), pj = VP(c, ox, oy);
            const vec2_t<T> di = dv.P(c, 0, 0), dj = dv.P(c, ox, oy);
            T t0[4];
            link4(Ai, Aj, pi, pj, q, p.idx, t0);
            const T ddre = (dj.x - di.x) * p.idx, ddim = (dj.y - di.y) * p.idx;
            const T qAi = q * Ai, qAj = q * Aj, qdai = qd * ai, qdaj = qd * aj;
            T t1[4], t2[4];
            t1[0] = -ddre - qAi * di.y - qdai * pi.y;
            t1[1] = -ddre - qAj * dj.y - qdaj * pj.y;
            t1[2] = ddim - qAi * di.x - qdai * pi.x;
            t1[3] = ddim - qAj * dj.x - qdaj * pj.x;
            const T qai = q * ai, qaj = q * aj;
            t2[0] = -qai * di.y;
            t2[1] = -qaj * dj.y;
            t2[2] = -qai * di.x;
            t2[3] = -qaj * dj.x;
            T se = 0, sb = 0, scc = 0, sd = 0, s4 = 0;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                se += t0[k] * t0[k];
                sb += t0[k] * t1[k];
                scc += (T)0.5 * t1[k] * t1[k] + t0[k] * t2[k];
                sd += t1[k] * t2[k];
                s4 += t2[k] * t2[k];
            }
            const T f = (dir == 0 ? p.hmx[c] : p.hmy[c]) * wl;   // = w / (2 m)
            e += (T)0.5 * se * f;
            b1 += sb * f;
            c2 += scc * f;
            d3 += sd * f * ((compat && dir == 1) ? (T)0.5 : (T)1);
            e4 += (T)0.5 * s4 * f;
        }
    }
    out[0] = e * p.dx2;
    out[1] = b1 * p.dx2;
    out[2] = c2 * p.dx2;
    out[3] = d3 * p.dx2;
    out[4] = e4 * p.dx2;
}

template <class T, int NC, int TYT>
__device__ __forceinline__ void site_poly(const Tile<T, NC, TYT> &t, const TileF<T, NC, TYT> &dt, int lx, int ly,
                                          const SiteParams<T> &p, const Wts<T> &w, int compat, int thin_film, T *out)
{
    site_poly_v<T, NC>(TileView<T, NC, TYT>{t, lx, ly}, TileView<T, NC, TYT>{dt, lx, ly}, p, w, compat, thin_film, out);
}
#undef VA
#undef VP

// B and J at one site (computeJBKernel, nlcg.cu:243-364).
template <class T, int NC, int TYT>
__device__ __forceinline__ void site_jb(const Tile<T, NC, TYT> &t, int lx, int ly, const SiteParams<T> &p,
                                        const Wts<T> &w, T *out /* 1+2NC */)
{
    const vec2_t<T> A0 = TA(0, 0);
    const T idx = p.idx;
    const T ayp = (TA(1, 0).y - A0.y) * idx, aym = (A0.y - TA(-1, 0).y) * idx;
    const T axp = (TA(0, 1).x - A0.x) * idx, axm = (A0.x - TA(0, -1).x) * idx;
    T bb = 0;
    bb += w.vUR * ((T)0.25 * (ayp - axp));
    bb += w.vUL * ((T)0.25 * (aym - axp));
    bb += w.vLL * ((T)0.25 * (aym - axm));
    bb += w.vLR * ((T)0.25 * (ayp - axm));
    if (bb != (T)0) bb /= (w.vUR + w.vUL + w.vLL + w.vLR) * (T)0.25;
    out[0] = bb;
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        const vec2_t<T> P0 = TP(c, 0, 0);
        const T q = p.q[c];
        T jx = 0, jy = 0, u[4];
        link4(A0.x, TA(1, 0).x, P0, TP(c, 1, 0), q, idx, u);
        jx += w.lfx * (p.hmx[c] * q * (P0.y * u[0] + P0.x * u[2]));
        link4(TA(-1, 0).x, A0.x, TP(c, -1, 0), P0, q, idx, u);
        jx += w.lbx * (p.hmx[c] * q * (P0.y * u[1] + P0.x * u[3]));
        link4(A0.y, TA(0, 1).y, P0, TP(c, 0, 1), q, idx, u);
        jy += w.lfy * (p.hmy[c] * q * (P0.y * u[0] + P0.x * u[2]));
        link4(TA(0, -1).y, A0.y, TP(c, 0, -1), P0, q, idx, u);
        jy += w.lby * (p.hmy[c] * q * (P0.y * u[1] + P0.x * u[3]));
        out[1 + 2 * c] = jx;
        out[2 + 2 * c] = jy;
    }
}

#undef TA
#undef TP

}  // namespace mepgl
