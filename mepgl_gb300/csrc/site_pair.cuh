// site_pair.cuh -- the gradient and quartic stencils of a two-component
// string with both components in packed pairs.
//
// Every per-component quantity is a pair (component 1, component 2), and
// the per-component arithmetic of site_gradient_v / site_poly_v runs as one
// packed FP32x2 operation for both components: for FP32 fields the pair is
// a float2 (fma.rn.f32x2, mul.rn.f32x2, add.rn.f32x2 on sm_100 and later);
// for the paired FP64 mode it is a packed float-float (ffp, each operation
// the float-float algorithm lane by lane).  The terms are those of the
// scalar stencils (same links, views and masks); what carries no component
// (A, the magnetic views, the couplings between the components) stays
// scalar.  Negated factors (-q, -dre) are formed once, so that every link
// term is one multiply-add.  Constants are written S(...): for float-float
// a bare float literal would convert to the int overloads.
#pragma once

#include "site_ops.cuh"

namespace mepgl {

template <class S> struct PairOf;
template <> struct PairOf<float> { using type = float2; };
template <> struct PairOf<ff> { using type = ffp; };

__device__ __forceinline__ float2 bc2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 mk2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float lane0(float2 a) { return a.x; }
__device__ __forceinline__ float lane1(float2 a) { return a.y; }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
// a - b (b * -1 is exact, so this rounds once, as a - b does)
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, bc2(-1.0f), a); }
__device__ __forceinline__ float hsum2(float2 a) { return a.x + a.y; }

__device__ __forceinline__ ffp bc2(ff a) { return ffp{make_float2(a.hi, a.hi), make_float2(a.lo, a.lo)}; }
__device__ __forceinline__ ffp mk2(ff a, ff b) { return ffp{make_float2(a.hi, b.hi), make_float2(a.lo, b.lo)}; }
__device__ __forceinline__ ff lane0(ffp a) { return ff(a.hi.x, a.lo.x); }
__device__ __forceinline__ ff lane1(ffp a) { return ff(a.hi.y, a.lo.y); }
__device__ __forceinline__ ffp add2(ffp a, ffp b) { return a + b; }
__device__ __forceinline__ ffp mul2(ffp a, ffp b) { return a * b; }
__device__ __forceinline__ ffp fma2(ffp a, ffp b, ffp c) { return a * b + c; }
__device__ __forceinline__ ffp sub2(ffp a, ffp b) { return a - b; }
__device__ __forceinline__ ff hsum2(ffp a) { return lane0(a) + lane1(a); }

// Neighbourhood of one site: A (x, y) and Re / Im psi of both components
// at (dx, dy) = [dy + 1][dx + 1].
template <class S>
struct PairView {
    using P = typename PairOf<S>::type;
    vec2_t<S> a[3][3];
    P px[3][3], py[3][3];
};

// Per-component parameters as pairs (uniform over a tile unless the string
// has per-site arrays, then per site).
template <class S>
struct PairParams {
    using P = typename PairOf<S>::type;
    P nq, hmx, hmy, aob, b, bh, a2, b2, idx, nidx;
    __device__ __forceinline__ void set(const SiteParams<S> &p)
    {
        nq = mk2(-p.q[0], -p.q[1]);
        hmx = mk2(p.hmx[0], p.hmx[1]);
        hmy = mk2(p.hmy[0], p.hmy[1]);
        aob = mk2(p.aob[0], p.aob[1]);
        b = mk2(p.b[0], p.b[1]);
        bh = mk2(S(0.5f) * p.b[0], S(0.5f) * p.b[1]);
        a2 = mk2(S(2.0f) * p.a[0], S(2.0f) * p.a[1]);
        b2 = mk2(S(2.0f) * p.b[0], S(2.0f) * p.b[1]);
        idx = bc2(p.idx);
        nidx = bc2(-p.idx);
    }
};

// Packed view of one site of a shared-memory tile of a two-component string.
template <class S, int TYT>
__device__ __forceinline__ PairView<S> pair_view_tile(const TileF<S, 2, TYT> &t, int lx, int ly)
{
    PairView<S> v;
#pragma unroll
    for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
        for (int dx = -1; dx <= 1; ++dx) {
            v.a[dy + 1][dx + 1] = t.A[ly + dy][lx + dx];
            const vec2_t<S> p1 = t.P[0][ly + dy][lx + dx], p2 = t.P[1][ly + dy][lx + dx];
            v.px[dy + 1][dx + 1] = mk2(p1.x, p2.x);
            v.py[dy + 1][dx + 1] = mk2(p1.y, p2.y);
        }
    return v;
}

// The four linearised covariant differences of one link i -> j (link4),
// both components: u0 = -dre - q A_i Im psi_i, u1 = -dre - q A_j Im psi_j,
// u2 = dim - q A_i Re psi_i, u3 = dim - q A_j Re psi_j.
template <class S, class P>
__device__ __forceinline__ void link4_pair(P nqi, P nqj, P xi, P yi, P xj, P yj, const PairParams<S> &pp, P (&u)[4])
{
    const P ndre = mul2(sub2(xi, xj), pp.idx), dim = mul2(sub2(yj, yi), pp.idx);
    u[0] = fma2(nqi, yi, ndre);
    u[1] = fma2(nqj, yj, ndre);
    u[2] = fma2(nqi, xi, dim);
    u[3] = fma2(nqj, xj, dim);
}

// Gradient dF/dA (out[0..1]) and dF/dpsi_c (out[2 + 2c], out[3 + 2c]) at
// one site; the terms of site_gradient_v for NC = 2.
template <class S>
__device__ __forceinline__ void site_gradient_pair(const PairView<S> &v, const SiteParams<S> &p,
                                                   const PairParams<S> &pp, const Wts<S> &w, S hr, S hl, S hu, S hd,
                                                   int maxwell, int thin_film, S *out)
{
    using P = typename PairOf<S>::type;
    using V = vec2_t<S>;
    const V A0 = v.a[1][1], Ar = v.a[1][2], Al = v.a[1][0], Au = v.a[2][1], Ad = v.a[0][1];
    const S idx = p.idx;
    const P X = v.px[1][1], Y = v.py[1][1];
    const P r2 = fma2(Y, Y, mul2(X, X));
    const P area = bc2(w.area);
    // a |psi|^2 + b/2 |psi|^4:  2 psi (a + b |psi|^2)
    const P k = fma2(pp.b2, r2, pp.a2);
    P gx = mul2(mul2(X, k), area), gy = mul2(mul2(Y, k), area);
    P gax = bc2(S(0.0f)), gay = bc2(S(0.0f));
    const P nqA0x = mul2(pp.nq, bc2(A0.x)), nqA0y = mul2(pp.nq, bc2(A0.y));
    P u[4];
    {   // own forward x-link
        link4_pair<S, P>(nqA0x, mul2(pp.nq, bc2(Ar.x)), X, Y, v.px[1][2], v.py[1][2], pp, u);
        const P f = mul2(pp.hmx, bc2(w.wfx));
        gx = fma2(f, fma2(nqA0x, u[2], mul2(add2(u[0], u[1]), pp.idx)), gx);
        gy = fma2(f, fma2(nqA0x, u[0], mul2(add2(u[2], u[3]), pp.nidx)), gy);
        gax = fma2(mul2(f, pp.nq), fma2(Y, u[0], mul2(X, u[2])), gax);
    }
    {   // backward x-link (from the -x neighbour)
        link4_pair<S, P>(mul2(pp.nq, bc2(Al.x)), nqA0x, v.px[1][0], v.py[1][0], X, Y, pp, u);
        const P f = mul2(pp.hmx, bc2(w.wbx));
        gx = fma2(f, fma2(nqA0x, u[3], mul2(add2(u[0], u[1]), pp.nidx)), gx);
        gy = fma2(f, fma2(nqA0x, u[1], mul2(add2(u[2], u[3]), pp.idx)), gy);
        gax = fma2(mul2(f, pp.nq), fma2(Y, u[1], mul2(X, u[3])), gax);
    }
    {   // own forward y-link
        link4_pair<S, P>(nqA0y, mul2(pp.nq, bc2(Au.y)), X, Y, v.px[2][1], v.py[2][1], pp, u);
        const P f = mul2(pp.hmy, bc2(w.wfy));
        gx = fma2(f, fma2(nqA0y, u[2], mul2(add2(u[0], u[1]), pp.idx)), gx);
        gy = fma2(f, fma2(nqA0y, u[0], mul2(add2(u[2], u[3]), pp.nidx)), gy);
        gay = fma2(mul2(f, pp.nq), fma2(Y, u[0], mul2(X, u[2])), gay);
    }
    {   // backward y-link (from the -y neighbour)
        link4_pair<S, P>(mul2(pp.nq, bc2(Ad.y)), nqA0y, v.px[0][1], v.py[0][1], X, Y, pp, u);
        const P f = mul2(pp.hmy, bc2(w.wby));
        gx = fma2(f, fma2(nqA0y, u[3], mul2(add2(u[0], u[1]), pp.nidx)), gx);
        gy = fma2(f, fma2(nqA0y, u[1], mul2(add2(u[2], u[3]), pp.idx)), gy);
        gay = fma2(mul2(f, pp.nq), fma2(Y, u[1], mul2(X, u[3])), gay);
    }
    {   // couplings between the components (scalar)
        const S x1 = lane0(X), y1 = lane0(Y), x2 = lane1(X), y2 = lane1(Y), r1 = lane0(r2), s2 = lane1(r2);
        const S R = x1 * x2 + y1 * y2, I = x1 * y2 - y1 * x2;
        out[2] = lane0(gx) + (p.eta * x2 + p.gamma * x1 * s2 + p.delta * (x2 * R - y2 * I)) * w.area;
        out[3] = lane0(gy) + (p.eta * y2 + p.gamma * y1 * s2 + p.delta * (y2 * R + x2 * I)) * w.area;
        out[4] = lane1(gx) + (p.eta * x1 + p.gamma * x2 * r1 + p.delta * (x1 * R + y1 * I)) * w.area;
        out[5] = lane1(gy) + (p.eta * y1 + p.gamma * y2 * r1 + p.delta * (y1 * R - x1 * I)) * w.area;
    }
#pragma unroll
    for (int c = 2; c < 6; ++c) out[c] = maxwell ? S(0.0f) : out[c] * p.dx2;

    if (!thin_film) {
        // magnetic views, as site_gradient_v
        const S ex0 = (Ar.y - A0.y) * idx, exm = (A0.y - Al.y) * idx;
        const S ey0 = (Au.x - A0.x) * idx, eym = (A0.x - Ad.x) * idx;
        const S exu = (v.a[2][2].y - Au.y) * idx, exmu = (Au.y - v.a[2][0].y) * idx;
        const S exd = (v.a[0][2].y - Ad.y) * idx, exmd = (Ad.y - v.a[0][0].y) * idx;
        const S eyr = (v.a[2][2].x - Ar.x) * idx, eyrm = (Ar.x - v.a[0][2].x) * idx;
        const S eyl = (v.a[2][0].x - Al.x) * idx, eylm = (Al.x - v.a[0][0].x) * idx;
        const S h = p.h;
        const S rUR = ex0 - ey0 - h, rUL = exm - ey0 - h, rLL = exm - eym - h, rLR = ex0 - eym - h;
        const S c4 = S(0.25f) * idx;
        const S mx = c4 * (w.vUR * (rUR + (exu - ey0 - hu)) + w.vUL * (rUL + (exmu - ey0 - hu)) -
                           w.vLL * (rLL + (exmd - eym - hd)) - w.vLR * (rLR + (exd - eym - hd)));
        const S my = c4 * (-w.vUR * (rUR + (ex0 - eyr - hr)) + w.vUL * (rUL + (exm - eyl - hl)) +
                           w.vLL * (rLL + (exm - eylm - hl)) - w.vLR * (rLR + (ex0 - eyrm - hr)));
        out[0] = (hsum2(gax) + mx) * p.dx2;
        out[1] = (hsum2(gay) + my) * p.dx2;
    } else {
        out[0] = S(0.0f);
        out[1] = S(0.0f);
    }
}

// Quartic coefficients {A, B, C, D, E} of F(x + a d) at one site; the terms
// of site_poly_v for NC = 2 (compat: the reference's x-link first-order slip
// and halved y-link cubic coefficient).
template <class S>
__device__ __forceinline__ void site_poly_pair(const PairView<S> &v, const PairView<S> &dv, const SiteParams<S> &p,
                                               const PairParams<S> &pp, const Wts<S> &w, int compat, int thin_film,
                                               S *out)
{
    using P = typename PairOf<S>::type;
    using V = vec2_t<S>;
    const P X = v.px[1][1], Y = v.py[1][1], U = dv.px[1][1], Vd = dv.py[1][1];
    // condensation b/2 (a/b + |psi + a d|^2)^2 per component
    const P n0 = fma2(Y, Y, fma2(X, X, pp.aob));
    const P n1h = fma2(Y, Vd, mul2(X, U));
    const P n1 = add2(n1h, n1h);
    const P n2 = fma2(Vd, Vd, mul2(U, U));
    const P pe = mul2(pp.bh, mul2(n0, n0)), pb = mul2(pp.b, mul2(n0, n1));
    const P pc = fma2(pp.bh, mul2(n1, n1), mul2(pp.b, mul2(n0, n2)));
    const P pd = mul2(pp.b, mul2(n1, n2)), p4 = mul2(pp.bh, mul2(n2, n2));
    S e = hsum2(pe), b1 = hsum2(pb), c2 = hsum2(pc), d3 = hsum2(pd), e4 = hsum2(p4);
    {   // couplings between the components (scalar)
        const S x1 = lane0(X), y1 = lane0(Y), x2 = lane1(X), y2 = lane1(Y);
        const S u1 = lane0(U), v1 = lane0(Vd), u2 = lane1(U), v2 = lane1(Vd);
        const S R0 = x1 * x2 + y1 * y2, R1 = u1 * x2 + v1 * y2 + x1 * u2 + y1 * v2, R2 = u1 * u2 + v1 * v2;
        const S I0 = x1 * y2 - y1 * x2, I1 = x1 * v2 + u1 * y2 - y1 * u2 - v1 * x2, I2 = u1 * v2 - v1 * u2;
        const S r1 = x1 * x1 + y1 * y1, r2 = x2 * x2 + y2 * y2;
        const S s1 = 2 * (x1 * u1 + y1 * v1), s2 = 2 * (x2 * u2 + y2 * v2);
        const S t1 = u1 * u1 + v1 * v1, t2 = u2 * u2 + v2 * v2;
        const S g = p.gamma * S(0.5f), dd = p.delta * S(0.5f);
        e += p.eta * R0 + g * r1 * r2 + dd * (R0 * R0 - I0 * I0);
        b1 += p.eta * R1 + g * (s1 * r2 + s2 * r1) + dd * (2 * R1 * R0 - 2 * I1 * I0);
        c2 += p.eta * R2 + g * (s1 * s2 + r1 * t2 + r2 * t1) + dd * (R1 * R1 - I1 * I1 + 2 * R0 * R2 - 2 * I0 * I2);
        d3 += g * (s1 * t2 + s2 * t1) + dd * (2 * R1 * R2 - 2 * I1 * I2);
        e4 += g * (t1 * t2) + dd * (R2 * R2 - I2 * I2);
    }
    e *= w.area; b1 *= w.area; c2 *= w.area; d3 *= w.area; e4 *= w.area;
    if (!thin_film) {
        const V A0 = v.a[1][1], a0 = dv.a[1][1];
        const S idx = p.idx;
        const S ayp = (v.a[1][2].y - A0.y) * idx, aym = (A0.y - v.a[1][0].y) * idx;
        const S axp = (v.a[2][1].x - A0.x) * idx, axm = (A0.x - v.a[0][1].x) * idx;
        const S dyp = (dv.a[1][2].y - a0.y) * idx, dym = (a0.y - dv.a[1][0].y) * idx;
        const S dxp = (dv.a[2][1].x - a0.x) * idx, dxm = (a0.x - dv.a[0][1].x) * idx;
        S em0 = S(0.0f), em1 = S(0.0f), em2 = S(0.0f), m0, m1;
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
        e += em0 * S(0.125f);
        b1 += em1 * S(0.25f);
        c2 += em2 * S(0.125f);
    }
    P ke = bc2(S(0.0f)), kb = ke, kc = ke, kd = ke, k4 = ke;
#pragma unroll
    for (int dir = 0; dir < 2; ++dir) {
        // link i -> j: i the site, j its +x (dir 0) or +y (dir 1) neighbour
        const S Ai = dir == 0 ? v.a[1][1].x : v.a[1][1].y, Aj = dir == 0 ? v.a[1][2].x : v.a[2][1].y;
        const S ai = dir == 0 ? dv.a[1][1].x : dv.a[1][1].y, aj = dir == 0 ? dv.a[1][2].x : dv.a[2][1].y;
        const P xj = dir == 0 ? v.px[1][2] : v.px[2][1], yj = dir == 0 ? v.py[1][2] : v.py[2][1];
        const P uj = dir == 0 ? dv.px[1][2] : dv.px[2][1], vj = dir == 0 ? dv.py[1][2] : dv.py[2][1];
        const P nqi = mul2(pp.nq, bc2(Ai)), nqj = mul2(pp.nq, bc2(Aj));
        P t0[4];
        link4_pair<S, P>(nqi, nqj, X, Y, xj, yj, pp, t0);
        // first order: -ddre - q A d_psi - qd a psi (qd = -1 on compat x-links), second: -q a d_psi
        const P nddre = mul2(sub2(U, uj), pp.idx), ddim = mul2(sub2(vj, Vd), pp.idx);
        const P nqd = (compat && dir == 0) ? bc2(S(1.0f)) : pp.nq;
        const P nqdai = mul2(nqd, bc2(ai)), nqdaj = mul2(nqd, bc2(aj));
        const P nqai = mul2(pp.nq, bc2(ai)), nqaj = mul2(pp.nq, bc2(aj));
        P t1[4], t2[4];
        t1[0] = fma2(nqdai, Y, fma2(nqi, Vd, nddre));
        t1[1] = fma2(nqdaj, yj, fma2(nqj, vj, nddre));
        t1[2] = fma2(nqdai, X, fma2(nqi, U, ddim));
        t1[3] = fma2(nqdaj, xj, fma2(nqj, uj, ddim));
        t2[0] = mul2(nqai, Vd);
        t2[1] = mul2(nqaj, vj);
        t2[2] = mul2(nqai, U);
        t2[3] = mul2(nqaj, uj);
        P se = mul2(t0[0], t0[0]), sb = mul2(t0[0], t1[0]), sc1 = mul2(t1[0], t1[0]);
        P sc2 = mul2(t0[0], t2[0]), sd = mul2(t1[0], t2[0]), s4 = mul2(t2[0], t2[0]);
#pragma unroll
        for (int q = 1; q < 4; ++q) {
            se = fma2(t0[q], t0[q], se);
            sb = fma2(t0[q], t1[q], sb);
            sc1 = fma2(t1[q], t1[q], sc1);
            sc2 = fma2(t0[q], t2[q], sc2);
            sd = fma2(t1[q], t2[q], sd);
            s4 = fma2(t2[q], t2[q], s4);
        }
        const P f = mul2(dir == 0 ? pp.hmx : pp.hmy, bc2(dir == 0 ? w.wfx : w.wfy));   // = w / (2 m)
        const P fh = mul2(f, bc2(S(0.5f)));
        ke = fma2(se, fh, ke);
        kb = fma2(sb, f, kb);
        kc = fma2(sc2, f, fma2(sc1, fh, kc));
        kd = fma2(sd, (compat && dir == 1) ? fh : f, kd);
        k4 = fma2(s4, fh, k4);
    }
    out[0] = (e + hsum2(ke)) * p.dx2;
    out[1] = (b1 + hsum2(kb)) * p.dx2;
    out[2] = (c2 + hsum2(kc)) * p.dx2;
    out[3] = (d3 + hsum2(kd)) * p.dx2;
    out[4] = (e4 + hsum2(k4)) * p.dx2;
}

}  // namespace mepgl
