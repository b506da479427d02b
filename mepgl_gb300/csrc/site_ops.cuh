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
#pragma once

#include "common.cuh"

namespace mepgl {

template <class T, int NC, int TY>
struct Tile {
    vec2_t<T> A[TY + 2][TX + 2];
    vec2_t<T> P[NC][TY + 2][TX + 2];
    uint16_t m[TY + 2][TX + 2];
};

// Parameters of one site (uniform strings read the descriptor).
template <class T>
struct SiteParams {
    T a[2], b[2], hmx[2], hmy[2], aob[2];  // hmx = 0.5 / m_xx
    T q[2], eta, gamma, delta, h, idx, dx2;
    __device__ __forceinline__ void load(const StringDesc &S, long s, int nc)
    {
        for (int c = 0; c < nc; ++c) {
            if (S.per_site) {
                a[c] = static_cast<const T *>(S.pa[c])[s];
                b[c] = static_cast<const T *>(S.pb[c])[s];
                hmx[c] = (T)0.5 / static_cast<const T *>(S.pmxx[c])[s];
                hmy[c] = (T)0.5 / static_cast<const T *>(S.pmyy[c])[s];
                aob[c] = a[c] / b[c];
            } else {
                a[c] = (T)S.a[c];
                b[c] = (T)S.b[c];
                hmx[c] = (T)S.hmx[c];
                hmy[c] = (T)S.hmy[c];
                aob[c] = (T)S.aob[c];
            }
            q[c] = (T)S.q[c];
        }
        eta = (T)S.eta;
        gamma = (T)S.gamma;
        delta = (T)S.delta;
        h = S.per_site ? static_cast<const T *>(S.ph)[s] : (T)S.h;
        idx = (T)S.inv_dx;
        const T dx = (T)S.dx;
        dx2 = dx * dx;
    }
};

template <class T>
__device__ __forceinline__ T h_at(const StringDesc &S, const SiteParams<T> &p, long s)
{
    return S.per_site ? static_cast<const T *>(S.ph)[s] : p.h;
}

template <class T>
__device__ __forceinline__ void link4(T Ai, T Aj, vec2_t<T> pi, vec2_t<T> pj, T q, T idx, T t[4])
{
    const T dre = (pj.x - pi.x) * idx, dim = (pj.y - pi.y) * idx;
    t[0] = -dre - q * Ai * pi.y;
    t[1] = -dre - q * Aj * pj.y;
    t[2] = dim - q * Ai * pi.x;
    t[3] = dim - q * Aj * pj.x;
}

__device__ __forceinline__ int area4(unsigned sc)
{
    return bit(sc, 0) * bit(sc, 1) * bit(sc, 2) + bit(sc, 2) * bit(sc, 3) * bit(sc, 4) +
           bit(sc, 4) * bit(sc, 5) * bit(sc, 6) + bit(sc, 6) * bit(sc, 7) * bit(sc, 0);
}

#define TA(dx_, dy_) (t.A[ly + (dy_)][lx + (dx_)])
#define TP(c_, dx_, dy_) (t.P[c_][ly + (dy_)][lx + (dx_)])

// Free-energy density x dx^2 (freeEnergyDensity, nlcg.cu:105-214).
template <class T, int NC, int TY>
__device__ __forceinline__ T site_energy(const Tile<T, NC, TY> &t, int lx, int ly, const SiteParams<T> &p, int thin_film)
{
    const unsigned mk = t.m[ly][lx], cc = mk & 0xffu, sc = mk >> 8;
    const T area = (T)area4(sc) * (T)0.25;
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
    nl *= area;
    T kx = 0, ky = 0;
    if (bit(sc, 0)) {
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            T q4[4];
            link4(A0.x, TA(1, 0).x, TP(c, 0, 0), TP(c, 1, 0), p.q[c], p.idx, q4);
            kx += (T)0.5 * p.hmx[c] * (q4[0] * q4[0] + q4[1] * q4[1] + q4[2] * q4[2] + q4[3] * q4[3]);
        }
    }
    if (bit(sc, 2)) {
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            T q4[4];
            link4(A0.y, TA(0, 1).y, TP(c, 0, 0), TP(c, 0, 1), p.q[c], p.idx, q4);
            ky += (T)0.5 * p.hmy[c] * (q4[0] * q4[0] + q4[1] * q4[1] + q4[2] * q4[2] + q4[3] * q4[3]);
        }
    }
    kx *= (T)(bit(sc, 1) * bit(sc, 2) + bit(sc, 6) * bit(sc, 7)) * (T)0.5;
    ky *= (T)(bit(sc, 0) * bit(sc, 1) + bit(sc, 3) * bit(sc, 4)) * (T)0.5;
    T em = 0;
    if (!thin_film) {
        const T ayp = bit(cc, 0) ? (TA(1, 0).y - A0.y) * p.idx : (T)0;
        const T aym = bit(cc, 4) ? (A0.y - TA(-1, 0).y) * p.idx : (T)0;
        const T axp = bit(cc, 2) ? (TA(0, 1).x - A0.x) * p.idx : (T)0;
        const T axm = bit(cc, 6) ? (A0.x - TA(0, -1).x) * p.idx : (T)0;
        T r;
        if (bit(cc, 0) & bit(cc, 1) & bit(cc, 2)) { r = ayp - axp - p.h; em += r * r; }
        if (bit(cc, 2) & bit(cc, 3) & bit(cc, 4)) { r = aym - axp - p.h; em += r * r; }
        if (bit(cc, 4) & bit(cc, 5) & bit(cc, 6)) { r = aym - axm - p.h; em += r * r; }
        if (bit(cc, 6) & bit(cc, 7) & bit(cc, 0)) { r = ayp - axm - p.h; em += r * r; }
        em *= (T)0.125;
    }
    return (kx + ky + nl + em) * p.dx2;
}

// Gradient dF/dA (out[0..1]) and dF/dpsi_c (out[2+2c..]) at one site,
// restating gradientPsi (nlcg.cu:504-744) and gradientA (nlcg.cu:746-888).
// Both link ends use the mass of this site, as the reference does.
template <class T, int NC, int TY>
__device__ __forceinline__ void site_gradient(const Tile<T, NC, TY> &t, int lx, int ly, const SiteParams<T> &p,
                              const StringDesc &S, long s, int maxwell, int thin_film, T *out)
{
    const unsigned mk = t.m[ly][lx], cc = mk & 0xffu, sc = mk >> 8;
    const T area = (T)area4(sc) * (T)0.25;
    const T w0 = (T)(bit(sc, 1) * bit(sc, 2) + bit(sc, 6) * bit(sc, 7)) * (T)0.5;   // forward x
    const T w1 = (T)(bit(sc, 2) * bit(sc, 3) + bit(sc, 5) * bit(sc, 6)) * (T)0.5;   // backward x
    const T w2 = (T)(bit(sc, 0) * bit(sc, 1) + bit(sc, 3) * bit(sc, 4)) * (T)0.5;   // forward y
    const T w3 = (T)(bit(sc, 4) * bit(sc, 5) + bit(sc, 7) * bit(sc, 0)) * (T)0.5;   // backward y
    const vec2_t<T> A0 = TA(0, 0);
    T gax = 0, gay = 0;
    const T idx = p.idx;
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        const vec2_t<T> P0 = TP(c, 0, 0);
        const T x = P0.x, y = P0.y, r2 = x * x + y * y, q = p.q[c];
        T gx = (2 * p.a[c] * x + p.b[c] * 2 * x * r2) * area;
        T gy = (2 * p.a[c] * y + p.b[c] * 2 * y * r2) * area;
        T u[4];
        if (bit(sc, 0)) {
            link4(A0.x, TA(1, 0).x, P0, TP(c, 1, 0), q, idx, u);
            const T f = p.hmx[c] * w0;
            gx += f * ((u[0] + u[1]) * idx - q * A0.x * u[2]);
            gy += f * (-(u[2] + u[3]) * idx - q * A0.x * u[0]);
            gax -= f * q * (y * u[0] + x * u[2]);
        }
        if (bit(sc, 4)) {
            link4(TA(-1, 0).x, A0.x, TP(c, -1, 0), P0, q, idx, u);
            const T f = p.hmx[c] * w1;
            gx += f * (-(u[1] + u[0]) * idx - q * A0.x * u[3]);
            gy += f * ((u[3] + u[2]) * idx - q * A0.x * u[1]);
            gax -= f * q * (y * u[1] + x * u[3]);
        }
        if (bit(sc, 2)) {
            link4(A0.y, TA(0, 1).y, P0, TP(c, 0, 1), q, idx, u);
            const T f = p.hmy[c] * w2;
            gx += f * ((u[0] + u[1]) * idx - q * A0.y * u[2]);
            gy += f * (-(u[2] + u[3]) * idx - q * A0.y * u[0]);
            gay -= f * q * (y * u[0] + x * u[2]);
        }
        if (bit(sc, 6)) {
            link4(TA(0, -1).y, A0.y, TP(c, 0, -1), P0, q, idx, u);
            const T f = p.hmy[c] * w3;
            gx += f * (-(u[1] + u[0]) * idx - q * A0.y * u[3]);
            gy += f * ((u[3] + u[2]) * idx - q * A0.y * u[1]);
            gay -= f * q * (y * u[1] + x * u[3]);
        }
        out[2 + 2 * c] = gx;
        out[3 + 2 * c] = gy;
    }
    if (NC == 2) {
        const vec2_t<T> P1 = TP(0, 0, 0), P2 = TP(NC - 1, 0, 0);
        const T x1 = P1.x, y1 = P1.y, x2 = P2.x, y2 = P2.y;
        const T r1 = x1 * x1 + y1 * y1, r2 = x2 * x2 + y2 * y2;
        const T R = x1 * x2 + y1 * y2, I = x1 * y2 - y1 * x2;
        out[2] += (p.eta * x2 + p.gamma * x1 * r2 + p.delta * (x2 * R - y2 * I)) * area;
        out[3] += (p.eta * y2 + p.gamma * y1 * r2 + p.delta * (y2 * R + x2 * I)) * area;
        out[2 + 2 * (NC - 1)] += (p.eta * x1 + p.gamma * x2 * r1 + p.delta * (x1 * R + y1 * I)) * area;
        out[3 + 2 * (NC - 1)] += (p.eta * y1 + p.gamma * y2 * r1 + p.delta * (y1 * R - x1 * I)) * area;
    }
#pragma unroll
    for (int k = 2; k < 2 + 2 * NC; ++k) out[k] = maxwell ? (T)0 : out[k] * p.dx2;

    if (!thin_film) {
        const int nx = S.nx;
        const T c4 = (T)0.25 * idx;
#define AX(a_, b_) TA(a_, b_).x
#define AY(a_, b_) TA(a_, b_).y
        if (bit(cc, 0) & bit(cc, 1) & bit(cc, 2)) {
            const T r = (AY(1, 0) - AY(0, 0)) * idx - (AX(0, 1) - AX(0, 0)) * idx - p.h;
            gax += c4 * r;
            gay -= c4 * r;
            gay -= c4 * ((AY(1, 0) - AY(0, 0)) * idx - (AX(1, 1) - AX(1, 0)) * idx - h_at(S, p, s + 1));
            gax += c4 * ((AY(1, 1) - AY(0, 1)) * idx - (AX(0, 1) - AX(0, 0)) * idx - h_at(S, p, s + nx));
        }
        if (bit(cc, 2) & bit(cc, 3) & bit(cc, 4)) {
            const T r = (AY(0, 0) - AY(-1, 0)) * idx - (AX(0, 1) - AX(0, 0)) * idx - p.h;
            gax += c4 * r;
            gay += c4 * r;
            gax += c4 * ((AY(0, 1) - AY(-1, 1)) * idx - (AX(0, 1) - AX(0, 0)) * idx - h_at(S, p, s + nx));
            gay += c4 * ((AY(0, 0) - AY(-1, 0)) * idx - (AX(-1, 1) - AX(-1, 0)) * idx - h_at(S, p, s - 1));
        }
        if (bit(cc, 4) & bit(cc, 5) & bit(cc, 6)) {
            const T r = (AY(0, 0) - AY(-1, 0)) * idx - (AX(0, 0) - AX(0, -1)) * idx - p.h;
            gax -= c4 * r;
            gay += c4 * r;
            gay += c4 * ((AY(0, 0) - AY(-1, 0)) * idx - (AX(-1, 0) - AX(-1, -1)) * idx - h_at(S, p, s - 1));
            gax -= c4 * ((AY(0, -1) - AY(-1, -1)) * idx - (AX(0, 0) - AX(0, -1)) * idx - h_at(S, p, s - nx));
        }
        if (bit(cc, 6) & bit(cc, 7) & bit(cc, 0)) {
            const T r = (AY(1, 0) - AY(0, 0)) * idx - (AX(0, 0) - AX(0, -1)) * idx - p.h;
            gax -= c4 * r;
            gay -= c4 * r;
            gax -= c4 * ((AY(1, -1) - AY(0, -1)) * idx - (AX(0, 0) - AX(0, -1)) * idx - h_at(S, p, s - nx));
            gay -= c4 * ((AY(1, 0) - AY(0, 0)) * idx - (AX(1, 0) - AX(1, -1)) * idx - h_at(S, p, s + 1));
        }
#undef AX
#undef AY
        out[0] = gax * p.dx2;
        out[1] = gay * p.dx2;
    } else {
        out[0] = 0;
        out[1] = 0;
    }
}

// Quartic coefficients of F(x + a d) at one site (polynomialExpansion,
// nlcg.cu:997-1370): out = {A, B, C, D, E}.  compat keeps the reference's
// x-link first-order slip and y-link halved cubic coefficient.
template <class T, int NC, int TY>
__device__ __forceinline__ void site_poly(const Tile<T, NC, TY> &t, const Tile<T, NC, TY> &dt, int lx, int ly,
                          const SiteParams<T> &p, int compat, int thin_film, T *out)
{
    const unsigned mk = t.m[ly][lx], cc = mk & 0xffu, sc = mk >> 8;
    const T area = (T)area4(sc) * (T)0.25;
    T e = 0, b1 = 0, c2 = 0, d3 = 0, e4 = 0;
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        const vec2_t<T> P0 = TP(c, 0, 0), D0 = dt.P[c][ly][lx];
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
        const vec2_t<T> P1 = TP(0, 0, 0), P2 = TP(NC - 1, 0, 0);
        const vec2_t<T> D1 = dt.P[0][ly][lx], D2 = dt.P[NC - 1][ly][lx];
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
    e *= area; b1 *= area; c2 *= area; d3 *= area; e4 *= area;
    if (!thin_film) {
        const vec2_t<T> A0 = TA(0, 0), a0 = dt.A[ly][lx];
        const T idx = p.idx;
        const T ayp = (TA(1, 0).y - A0.y) * idx, aym = (A0.y - TA(-1, 0).y) * idx;
        const T axp = (TA(0, 1).x - A0.x) * idx, axm = (A0.x - TA(0, -1).x) * idx;
        const T dyp = (dt.A[ly][lx + 1].y - a0.y) * idx, dym = (a0.y - dt.A[ly][lx - 1].y) * idx;
        const T dxp = (dt.A[ly + 1][lx].x - a0.x) * idx, dxm = (a0.x - dt.A[ly - 1][lx].x) * idx;
        T em0 = 0, em1 = 0, em2 = 0;
        T m0, m1;
#define EMV(cond, yy, xx, dyy, dxx)                                   \
        if (cond) {                                                   \
            m0 = yy - xx - p.h;                                       \
            m1 = dyy - dxx;                                           \
            em0 += (T)0.5 * m0 * m0;                                  \
            em1 += m0 * m1;                                           \
            em2 += (T)0.5 * m1 * m1;                                  \
        }
        EMV(bit(cc, 0) & bit(cc, 1) & bit(cc, 2), ayp, axp, dyp, dxp)
        EMV(bit(cc, 2) & bit(cc, 3) & bit(cc, 4), aym, axp, dym, dxp)
        EMV(bit(cc, 4) & bit(cc, 5) & bit(cc, 6), aym, axm, dym, dxm)
        EMV(bit(cc, 6) & bit(cc, 7) & bit(cc, 0), ayp, axm, dyp, dxm)
#undef EMV
        e += em0 * (T)0.25;
        b1 += em1 * (T)0.25;
        c2 += em2 * (T)0.25;
    }
    const T cwx = (T)(bit(sc, 1) * bit(sc, 2) + bit(sc, 6) * bit(sc, 7)) * (T)0.5;
    const T cwy = (T)(bit(sc, 0) * bit(sc, 1) + bit(sc, 3) * bit(sc, 4)) * (T)0.5;
#pragma unroll
    for (int dir = 0; dir < 2; ++dir) {
        if (!bit(sc, dir == 0 ? 0 : 2)) continue;
        const int ox = dir == 0 ? 1 : 0, oy = dir == 0 ? 0 : 1;
        const T Ai = dir == 0 ? TA(0, 0).x : TA(0, 0).y;
        const T Aj = dir == 0 ? TA(ox, oy).x : TA(ox, oy).y;
        const T ai = dir == 0 ? dt.A[ly][lx].x : dt.A[ly][lx].y;
        const T aj = dir == 0 ? dt.A[ly + oy][lx + ox].x : dt.A[ly + oy][lx + ox].y;
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            const T q = p.q[c];
            const T qd = (compat && dir == 0) ? (T)-1 : q;
            const vec2_t<T> pi = TP(c, 0, 0), pj = TP(c, ox, oy);
            const vec2_t<T> di = dt.P[c][ly][lx], dj = dt.P[c][ly + oy][lx + ox];
            T t0[4];
            link4(Ai, Aj, pi, pj, q, p.idx, t0);
            const T ddre = (dj.x - di.x) * p.idx, ddim = (dj.y - di.y) * p.idx;
            T t1[4], t2[4];
            t1[0] = -ddre - q * Ai * di.y - qd * ai * pi.y;
            t1[1] = -ddre - q * Aj * dj.y - qd * aj * pj.y;
            t1[2] = ddim - q * Ai * di.x - qd * ai * pi.x;
            t1[3] = ddim - q * Aj * dj.x - qd * aj * pj.x;
            t2[0] = -q * ai * di.y;
            t2[1] = -q * aj * dj.y;
            t2[2] = -q * ai * di.x;
            t2[3] = -q * aj * dj.x;
            T se = 0, sb = 0, scc = 0, sd = 0, s4 = 0;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                se += t0[k] * t0[k];
                sb += t0[k] * t1[k];
                scc += (T)0.5 * t1[k] * t1[k] + t0[k] * t2[k];
                sd += t1[k] * t2[k];
                s4 += t2[k] * t2[k];
            }
            const T f = (dir == 0 ? p.hmx[c] * cwx : p.hmy[c] * cwy);   // = w / (2 m)
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

// B and J at one site (computeJBKernel, nlcg.cu:243-364).
template <class T, int NC, int TY>
__device__ __forceinline__ void site_jb(const Tile<T, NC, TY> &t, int lx, int ly, const SiteParams<T> &p, T *out /* 1+2NC */)
{
    const unsigned mk = t.m[ly][lx], cc = mk & 0xffu, sc = mk >> 8;
    const vec2_t<T> A0 = TA(0, 0);
    const T idx = p.idx;
    T bb = 0;
    if (bit(cc, 0) & bit(cc, 1) & bit(cc, 2)) bb += (T)0.25 * ((TA(1, 0).y - A0.y) * idx - (TA(0, 1).x - A0.x) * idx);
    if (bit(cc, 2) & bit(cc, 3) & bit(cc, 4)) bb += (T)0.25 * ((A0.y - TA(-1, 0).y) * idx - (TA(0, 1).x - A0.x) * idx);
    if (bit(cc, 4) & bit(cc, 5) & bit(cc, 6)) bb += (T)0.25 * ((A0.y - TA(-1, 0).y) * idx - (A0.x - TA(0, -1).x) * idx);
    if (bit(cc, 6) & bit(cc, 7) & bit(cc, 0)) bb += (T)0.25 * ((TA(1, 0).y - A0.y) * idx - (A0.x - TA(0, -1).x) * idx);
    if (bb != (T)0) bb /= (T)area4(cc) * (T)0.25;
    out[0] = bb;
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        const vec2_t<T> P0 = TP(c, 0, 0);
        const T q = p.q[c];
        T jx = 0, jy = 0, u[4];
        if (bit(sc, 0)) { link4(A0.x, TA(1, 0).x, P0, TP(c, 1, 0), q, idx, u); jx += p.hmx[c] * q * (P0.y * u[0] + P0.x * u[2]); }
        if (bit(sc, 4)) { link4(TA(-1, 0).x, A0.x, TP(c, -1, 0), P0, q, idx, u); jx += p.hmx[c] * q * (P0.y * u[1] + P0.x * u[3]); }
        if (bit(sc, 2)) { link4(A0.y, TA(0, 1).y, P0, TP(c, 0, 1), q, idx, u); jy += p.hmy[c] * q * (P0.y * u[0] + P0.x * u[2]); }
        if (bit(sc, 6)) { link4(TA(0, -1).y, A0.y, TP(c, 0, -1), P0, q, idx, u); jy += p.hmy[c] * q * (P0.y * u[1] + P0.x * u[3]); }
        out[1 + 2 * c] = jx;
        out[2 + 2 * c] = jy;
    }
}

#undef TA
#undef TP

}  // namespace mepgl
