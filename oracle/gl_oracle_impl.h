/*
 * gl_oracle_impl.h -- precision-generic body of the C oracle (TEST
 * INFRASTRUCTURE; see gl_oracle.h).  Included by gl_oracle.c once per
 * precision with REAL (float or double) and SFX (suffix token) defined.
 */
#define GLO_CAT2(a, b) a##b
#define GLO_CAT(a, b) GLO_CAT2(a, b)
#define FN(name) GLO_CAT(name, SFX)
#define PROB FN(glo_problem_)

typedef struct PROB {
    int nx, ny, ncomp, thin_film;
    REAL dx;
    const uint8_t *comp_nn, *sc_nn;
    const REAL *a[2], *b[2], *mxx[2], *myy[2], *h;
    REAL q[2], eta, gamma, delta;
} PROB;

static inline REAL FN(sq)(REAL x) { return x * x; }

/* ------------------------------------------------------------------ energy
 * Per-site free-energy density x dx^2, restating freeEnergyDensity
 * (mepgl/src/nlcg.cu:105-214): condensation + couplings weighted by the
 * fraction of valid superconducting plaquettes around the site (121-149),
 * linearised covariant differences on the +x and +y links (151-183) weighted
 * by the two plaquettes sharing the link (186-187), and four collocated
 * "views" of the curl A - h around the site (189-203).
 */
static REAL FN(site_energy)(const PROB *P, const REAL *A, const REAL *const ps[2], long o, int i, int j)
{
    const int nx = P->nx;
    const long s = i + (long)nx * j, k = o + s;
    const unsigned sc = P->sc_nn[s], cc = P->comp_nn[s];
    const REAL dx = P->dx;
#define B_(c, n) (((c) >> (n)) & 1u)
    const int area_n = B_(sc, 0) * B_(sc, 1) * B_(sc, 2) + B_(sc, 2) * B_(sc, 3) * B_(sc, 4)
                     + B_(sc, 4) * B_(sc, 5) * B_(sc, 6) + B_(sc, 6) * B_(sc, 7) * B_(sc, 0);
    REAL nl = 0;
    for (int c = 0; c < P->ncomp; ++c) {
        const REAL x = ps[c][2 * k], y = ps[c][2 * k + 1];
        const REAL a = P->a[c][s], b = P->b[c][s];
        nl += b / (REAL)2 * FN(sq)(a / b + FN(sq)(x) + FN(sq)(y));
    }
    if (P->ncomp == 2) {
        const REAL x1 = ps[0][2 * k], y1 = ps[0][2 * k + 1], x2 = ps[1][2 * k], y2 = ps[1][2 * k + 1];
        nl += P->eta * (x1 * x2 + y1 * y2);
        nl += P->gamma / (REAL)2 * (FN(sq)(x1) + FN(sq)(y1)) * (FN(sq)(x2) + FN(sq)(y2));
        nl += P->delta / (REAL)2 * (FN(sq)(x1 * x2 + y1 * y2) - FN(sq)(x1 * y2 - y1 * x2));
    }
    nl *= (REAL)area_n / (REAL)4;

    REAL kx = 0, ky = 0;
    for (int dir = 0; dir < 2; ++dir) {
        const int bit = dir == 0 ? 0 : 2;
        if (!B_(sc, bit)) continue;
        const long kj = k + (dir == 0 ? 1 : nx);
        const REAL Ai = A[2 * k + dir], Aj = A[2 * kj + dir];
        REAL acc = 0;
        for (int c = 0; c < P->ncomp; ++c) {
            const REAL q = P->q[c];
            const REAL m = dir == 0 ? P->mxx[c][s] : P->myy[c][s];
            const REAL *p = ps[c];
            const REAL dre = (p[2 * kj] - p[2 * k]) / dx, dim = (p[2 * kj + 1] - p[2 * k + 1]) / dx;
            acc += (REAL)0.25 / m * (FN(sq)(-dre - q * Ai * p[2 * k + 1]) + FN(sq)(-dre - q * Aj * p[2 * kj + 1])
                                   + FN(sq)(dim - q * Ai * p[2 * k]) + FN(sq)(dim - q * Aj * p[2 * kj]));
        }
        if (dir == 0) kx = acc; else ky = acc;
    }
    kx *= (REAL)(B_(sc, 1) * B_(sc, 2) + B_(sc, 6) * B_(sc, 7)) / (REAL)2;
    ky *= (REAL)(B_(sc, 0) * B_(sc, 1) + B_(sc, 3) * B_(sc, 4)) / (REAL)2;

    REAL em = 0;
    if (!P->thin_film) {
        const REAL h = P->h[s];
        /* the four views: (curl from the row/column of this site) */
        const REAL ayp = B_(cc, 0) ? (A[2 * (k + 1) + 1] - A[2 * k + 1]) / dx : 0;      /* d_x A_y, forward */
        const REAL aym = B_(cc, 4) ? (A[2 * k + 1] - A[2 * (k - 1) + 1]) / dx : 0;      /* backward */
        const REAL axp = B_(cc, 2) ? (A[2 * (k + nx)] - A[2 * k]) / dx : 0;            /* d_y A_x, forward */
        const REAL axm = B_(cc, 6) ? (A[2 * k] - A[2 * (k - nx)]) / dx : 0;            /* backward */
        if (B_(cc, 0) && B_(cc, 1) && B_(cc, 2)) em += (REAL)0.125 * FN(sq)(ayp - axp - h);
        if (B_(cc, 2) && B_(cc, 3) && B_(cc, 4)) em += (REAL)0.125 * FN(sq)(aym - axp - h);
        if (B_(cc, 4) && B_(cc, 5) && B_(cc, 6)) em += (REAL)0.125 * FN(sq)(aym - axm - h);
        if (B_(cc, 6) && B_(cc, 7) && B_(cc, 0)) em += (REAL)0.125 * FN(sq)(ayp - axm - h);
    }
    REAL d = 0;
    d += (kx + ky) * dx * dx;
    d += nl * dx * dx;
    d += em * dx * dx;
    return d;
}

/* Neumaier-compensated running sum (deterministic, platform independent). */
typedef struct { double s, c; } FN(ksum);
static inline void FN(kadd)(FN(ksum) *a, double v)
{
    double t = a->s + v;
    if (fabs(a->s) >= fabs(v)) a->c += (a->s - t) + v;
    else a->c += (v - t) + a->s;
    a->s = t;
}
static inline double FN(kval)(const FN(ksum) *a) { return a->s + a->c; }

/* computeFreeEnergy (nlcg.cu:217-240): per-image sums of the density. */
void FN(glo_energy)(const PROB *P, int F, const REAL *A, const REAL *p1, const REAL *p2, double *out)
{
    const REAL *ps[2] = {p1, p2};
    const long M = (long)P->nx * P->ny;
    GLO_OMP_FOR
    for (int n = 0; n < F; ++n) {
        FN(ksum) acc = {0, 0};
        for (int j = 0; j < P->ny; ++j)
            for (int i = 0; i < P->nx; ++i) FN(kadd)(&acc, FN(site_energy)(P, A, ps, n * M, i, j));
        out[n] = FN(kval)(&acc);
    }
}

/* Parameter adjoints of the per-image energy (no reference counterpart):
 * partial derivatives of glo_energy at fixed fields with respect to a uniform
 * shift of the applied field h (dF/dH), to eta and to gamma, differentiating
 * the terms of site_energy above: -1/4 sum_views (curl - h), and
 * area/4 * Re(psi1 psi2*) and area/4 * |psi1|^2 |psi2|^2 / 2, each times dx^2.
 * out[3 n + 0..2] = dF_n/dH, dF_n/deta, dF_n/dgamma. */
void FN(glo_param_adjoint)(const PROB *P, int F, const REAL *A, const REAL *p1, const REAL *p2, double *out)
{
    const long M = (long)P->nx * P->ny;
    const int nx = P->nx;
    GLO_OMP_FOR
    for (int n = 0; n < F; ++n) {
        FN(ksum) dh = {0, 0}, de = {0, 0}, dg = {0, 0};
        for (int j = 0; j < P->ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const long s = i + (long)nx * j, k = n * M + s;
                const unsigned sc = P->sc_nn[s], cc = P->comp_nn[s];
                const REAL dx = P->dx, dx2 = dx * dx;
                if (P->ncomp == 2) {
                    const int area_n = B_(sc, 0) * B_(sc, 1) * B_(sc, 2) + B_(sc, 2) * B_(sc, 3) * B_(sc, 4)
                                     + B_(sc, 4) * B_(sc, 5) * B_(sc, 6) + B_(sc, 6) * B_(sc, 7) * B_(sc, 0);
                    const REAL x1 = p1[2 * k], y1 = p1[2 * k + 1], x2 = p2[2 * k], y2 = p2[2 * k + 1];
                    const REAL w = (REAL)area_n / (REAL)4;
                    FN(kadd)(&de, (double)((x1 * x2 + y1 * y2) * w * dx2));
                    FN(kadd)(&dg, (double)((FN(sq)(x1) + FN(sq)(y1)) * (FN(sq)(x2) + FN(sq)(y2)) / (REAL)2 * w * dx2));
                }
                if (!P->thin_film) {
                    const REAL h = P->h[s];
                    const REAL ayp = B_(cc, 0) ? (A[2 * (k + 1) + 1] - A[2 * k + 1]) / dx : 0;
                    const REAL aym = B_(cc, 4) ? (A[2 * k + 1] - A[2 * (k - 1) + 1]) / dx : 0;
                    const REAL axp = B_(cc, 2) ? (A[2 * (k + nx)] - A[2 * k]) / dx : 0;
                    const REAL axm = B_(cc, 6) ? (A[2 * k] - A[2 * (k - nx)]) / dx : 0;
                    REAL em = 0;
                    if (B_(cc, 0) && B_(cc, 1) && B_(cc, 2)) em += ayp - axp - h;
                    if (B_(cc, 2) && B_(cc, 3) && B_(cc, 4)) em += aym - axp - h;
                    if (B_(cc, 4) && B_(cc, 5) && B_(cc, 6)) em += aym - axm - h;
                    if (B_(cc, 6) && B_(cc, 7) && B_(cc, 0)) em += ayp - axm - h;
                    FN(kadd)(&dh, (double)(-(REAL)0.25 * em * dx2));
                }
            }
        out[3 * n] = FN(kval)(&dh);
        out[3 * n + 1] = FN(kval)(&de);
        out[3 * n + 2] = FN(kval)(&dg);
    }
}

/* ------------------------------------------------- link discretisation
 * Gauge-link (Peierls) form of the same functional, no reference
 * counterpart.  A_e at site s is the link variable of the link s -> s + e;
 * per link and component the kinetic energy is w_e / (2 m_e) |psi_t - U psi_s|^2
 * with U = exp(i q A_e dx) (w_e, m_e: the reference's link weight and the mass
 * at s); per plaquette with lower-left corner s, 1/2 v (B - h)^2 dx^2 with
 * B = (A_x(s) + A_y(s+x) - A_x(s+y) - A_y(s)) / dx and v the validity of the
 * reference's upper-right curl view; the condensation terms are unchanged.
 * Under psi_c -> psi_c exp(i q_c chi), A_e(s) -> A_e(s) + (chi(s+e) - chi(s))/dx
 * every term is invariant exactly (the eta and delta terms when q_1 = q_2). */
static void FN(cis)(REAL a, REAL *c, REAL *s)
{
    *c = (REAL)cos((double)a);
    *s = (REAL)sin((double)a);
}

static REAL FN(link_weight)(unsigned sc, int dir)
{
    return dir == 0 ? (REAL)(B_(sc, 0) ? (B_(sc, 1) * B_(sc, 2) + B_(sc, 6) * B_(sc, 7)) : 0) / (REAL)2
                    : (REAL)(B_(sc, 2) ? (B_(sc, 0) * B_(sc, 1) + B_(sc, 3) * B_(sc, 4)) : 0) / (REAL)2;
}

static REAL FN(condensation)(const PROB *P, const REAL *const ps[2], long k, long s)
{
    REAL nl = 0;
    for (int c = 0; c < P->ncomp; ++c) {
        const REAL x = ps[c][2 * k], y = ps[c][2 * k + 1];
        nl += P->b[c][s] / (REAL)2 * FN(sq)(P->a[c][s] / P->b[c][s] + FN(sq)(x) + FN(sq)(y));
    }
    if (P->ncomp == 2) {
        const REAL x1 = ps[0][2 * k], y1 = ps[0][2 * k + 1], x2 = ps[1][2 * k], y2 = ps[1][2 * k + 1];
        nl += P->eta * (x1 * x2 + y1 * y2);
        nl += P->gamma / (REAL)2 * (FN(sq)(x1) + FN(sq)(y1)) * (FN(sq)(x2) + FN(sq)(y2));
        nl += P->delta / (REAL)2 * (FN(sq)(x1 * x2 + y1 * y2) - FN(sq)(x1 * y2 - y1 * x2));
    }
    return nl;
}

static REAL FN(area)(unsigned sc)
{
    return (REAL)(B_(sc, 0) * B_(sc, 1) * B_(sc, 2) + B_(sc, 2) * B_(sc, 3) * B_(sc, 4)
                  + B_(sc, 4) * B_(sc, 5) * B_(sc, 6) + B_(sc, 6) * B_(sc, 7) * B_(sc, 0)) / (REAL)4;
}

void FN(glo_energy_link)(const PROB *P, int F, const REAL *A, const REAL *p1, const REAL *p2, double *out)
{
    const REAL *ps[2] = {p1, p2};
    const int nx = P->nx;
    const long M = (long)nx * P->ny;
    const REAL dx = P->dx;
    GLO_OMP_FOR
    for (int n = 0; n < F; ++n) {
        FN(ksum) acc = {0, 0};
        for (int j = 0; j < P->ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const long s = i + (long)nx * j, k = n * M + s;
                const unsigned sc = P->sc_nn[s], cc = P->comp_nn[s];
                REAL e = FN(condensation)(P, ps, k, s) * FN(area)(sc) * dx * dx;
                for (int dir = 0; dir < 2; ++dir) {
                    const REAL w = FN(link_weight)(sc, dir);
                    if (w == 0) continue;
                    const long t = k + (dir == 0 ? 1 : nx);
                    for (int c = 0; c < P->ncomp; ++c) {
                        const REAL m = dir == 0 ? P->mxx[c][s] : P->myy[c][s];
                        REAL cu, su;
                        FN(cis)(P->q[c] * A[2 * k + dir] * dx, &cu, &su);
                        const REAL *p = ps[c];
                        const REAL zr = p[2 * t] - (cu * p[2 * k] - su * p[2 * k + 1]);
                        const REAL zi = p[2 * t + 1] - (su * p[2 * k] + cu * p[2 * k + 1]);
                        e += w / ((REAL)2 * m) * (zr * zr + zi * zi);
                    }
                }
                if (!P->thin_film && B_(cc, 0) && B_(cc, 1) && B_(cc, 2)) {
                    const REAL B = (A[2 * k] + A[2 * (k + 1) + 1] - A[2 * (k + nx)] - A[2 * k + 1]) / dx;
                    e += (REAL)0.5 * FN(sq)(B - P->h[s]) * dx * dx;
                }
                FN(kadd)(&acc, (double)e);
            }
        out[n] = FN(kval)(&acc);
    }
}

void FN(glo_gradient_link)(const PROB *P, int F, const REAL *A, const REAL *p1, const REAL *p2, REAL *gA,
                           REAL *g1, REAL *g2, int maxwell)
{
    const REAL *ps[2] = {p1, p2};
    REAL *gp[2] = {g1, g2};
    const int nx = P->nx, nc = P->ncomp;
    const long M = (long)nx * P->ny;
    const REAL dx = P->dx;
    GLO_OMP_FOR
    for (int n = 0; n < F; ++n) {
        memset(gA + 2 * n * M, 0, 2 * M * sizeof(REAL));
        for (int c = 0; c < nc; ++c) memset(gp[c] + 2 * n * M, 0, 2 * M * sizeof(REAL));
        for (int j = 0; j < P->ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const long s = i + (long)nx * j, k = n * M + s;
                const unsigned sc = P->sc_nn[s], cc = P->comp_nn[s];
                const REAL ar = FN(area)(sc) * dx * dx;
                if (!maxwell) {
                    for (int c = 0; c < nc; ++c) {
                        const REAL x = ps[c][2 * k], y = ps[c][2 * k + 1], r2 = x * x + y * y;
                        gp[c][2 * k] += (REAL)2 * x * (P->a[c][s] + P->b[c][s] * r2) * ar;
                        gp[c][2 * k + 1] += (REAL)2 * y * (P->a[c][s] + P->b[c][s] * r2) * ar;
                    }
                    if (nc == 2) {
                        const REAL x1 = ps[0][2 * k], y1 = ps[0][2 * k + 1], x2 = ps[1][2 * k], y2 = ps[1][2 * k + 1];
                        const REAL R = x1 * x2 + y1 * y2, I = x1 * y2 - y1 * x2;
                        const REAL r1 = x1 * x1 + y1 * y1, r2 = x2 * x2 + y2 * y2;
                        gp[0][2 * k] += (P->eta * x2 + P->gamma * x1 * r2 + P->delta * (R * x2 - I * y2)) * ar;
                        gp[0][2 * k + 1] += (P->eta * y2 + P->gamma * y1 * r2 + P->delta * (R * y2 + I * x2)) * ar;
                        gp[1][2 * k] += (P->eta * x1 + P->gamma * x2 * r1 + P->delta * (R * x1 + I * y1)) * ar;
                        gp[1][2 * k + 1] += (P->eta * y1 + P->gamma * y2 * r1 + P->delta * (R * y1 - I * x1)) * ar;
                    }
                }
                for (int dir = 0; dir < 2; ++dir) {
                    const REAL w = FN(link_weight)(sc, dir);
                    if (w == 0) continue;
                    const long t = k + (dir == 0 ? 1 : nx);
                    for (int c = 0; c < nc; ++c) {
                        const REAL m = dir == 0 ? P->mxx[c][s] : P->myy[c][s], q = P->q[c];
                        const REAL kk = w / ((REAL)2 * m);
                        REAL cu, su;
                        FN(cis)(q * A[2 * k + dir] * dx, &cu, &su);
                        const REAL *p = ps[c];
                        const REAL ur = cu * p[2 * k] - su * p[2 * k + 1], ui = su * p[2 * k] + cu * p[2 * k + 1];
                        const REAL zr = p[2 * t] - ur, zi = p[2 * t + 1] - ui;
                        if (!maxwell) {
                            gp[c][2 * t] += (REAL)2 * kk * zr;
                            gp[c][2 * t + 1] += (REAL)2 * kk * zi;
                            /* -2k conj(U) z */
                            gp[c][2 * k] += -(REAL)2 * kk * (cu * zr + su * zi);
                            gp[c][2 * k + 1] += -(REAL)2 * kk * (cu * zi - su * zr);
                        }
                        /* 2k q dx Im(conj(z) U psi_s) */
                        if (!P->thin_film) gA[2 * k + dir] += (REAL)2 * kk * q * dx * (zr * ui - zi * ur);
                    }
                }
                if (!P->thin_film && B_(cc, 0) && B_(cc, 1) && B_(cc, 2)) {
                    const REAL B = (A[2 * k] + A[2 * (k + 1) + 1] - A[2 * (k + nx)] - A[2 * k + 1]) / dx;
                    const REAL r = (B - P->h[s]) * dx;
                    gA[2 * k] += r;
                    gA[2 * (k + 1) + 1] += r;
                    gA[2 * (k + nx)] -= r;
                    gA[2 * k + 1] -= r;
                }
            }
    }
}

/* ---------------------------------------------------------------- gradient
 * Restates gradientPsi (nlcg.cu:504-744) and gradientA (nlcg.cu:746-888).
 * On a link i -> j along direction e the reference uses, per component,
 *   u0 = -(Re psi_j - Re psi_i)/dx - q A_i Im psi_i,  u1 = same with A_j, psi_j
 *   v0 = +(Im psi_j - Im psi_i)/dx - q A_i Re psi_i,  v1 = same with A_j, psi_j
 * and the energy (u0^2+u1^2+v0^2+v1^2)/(4m) w.  The gradient at a site sums
 * the derivative of its forward link (start end) and of its backward link
 * (finish end); both use the mass at the site itself (nlcg.cu:555,579,...).
 */
static void FN(link_terms)(const REAL *p, const REAL *A, long ki, long kj, int dir, REAL q, REAL dx, REAL t[4])
{
    const REAL Ai = A[2 * ki + dir], Aj = A[2 * kj + dir];
    const REAL dre = (p[2 * kj] - p[2 * ki]) / dx, dim = (p[2 * kj + 1] - p[2 * ki + 1]) / dx;
    t[0] = -dre - q * Ai * p[2 * ki + 1];
    t[1] = -dre - q * Aj * p[2 * kj + 1];
    t[2] = dim - q * Ai * p[2 * ki];
    t[3] = dim - q * Aj * p[2 * kj];
}

void FN(glo_gradient)(const PROB *P, int F, const REAL *A, const REAL *p1, const REAL *p2, REAL *gA,
                      REAL *g1, REAL *g2, int maxwell)
{
    const REAL *ps[2] = {p1, p2};
    REAL *gs[2] = {g1, g2};
    const int nx = P->nx;
    const long M = (long)nx * P->ny;
    const REAL dx = P->dx;
    GLO_OMP_FOR
    for (int n = 0; n < F; ++n)
        for (int j = 0; j < P->ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const long s = i + (long)nx * j, k = n * M + s;
                const unsigned sc = P->sc_nn[s], cc = P->comp_nn[s];
                const REAL area = (REAL)(B_(sc, 0) * B_(sc, 1) * B_(sc, 2) + B_(sc, 2) * B_(sc, 3) * B_(sc, 4)
                                       + B_(sc, 4) * B_(sc, 5) * B_(sc, 6) + B_(sc, 6) * B_(sc, 7) * B_(sc, 0)) / (REAL)4;
                /* link weights: forward x, backward x, forward y, backward y */
                const REAL w[4] = {
                    (REAL)(B_(sc, 1) * B_(sc, 2) + B_(sc, 6) * B_(sc, 7)) / (REAL)2,
                    (REAL)(B_(sc, 2) * B_(sc, 3) + B_(sc, 5) * B_(sc, 6)) / (REAL)2,
                    (REAL)(B_(sc, 0) * B_(sc, 1) + B_(sc, 3) * B_(sc, 4)) / (REAL)2,
                    (REAL)(B_(sc, 4) * B_(sc, 5) + B_(sc, 7) * B_(sc, 0)) / (REAL)2};
                const int lbit[4] = {0, 4, 2, 6};
                const long lnb[4] = {k + 1, k - 1, k + nx, k - nx};
                REAL gax = 0, gay = 0;
                for (int c = 0; c < P->ncomp; ++c) {
                    const REAL *p = ps[c];
                    const REAL q = P->q[c];
                    const REAL x = p[2 * k], y = p[2 * k + 1], r2 = FN(sq)(x) + FN(sq)(y);
                    REAL gx = (2 * P->a[c][s] * x + P->b[c][s] * 2 * x * r2) * area;
                    REAL gy = (2 * P->a[c][s] * y + P->b[c][s] * 2 * y * r2) * area;
                    for (int l = 0; l < 4; ++l) {
                        if (!B_(sc, lbit[l])) continue;
                        const int dir = l < 2 ? 0 : 1;
                        const REAL m = dir == 0 ? P->mxx[c][s] : P->myy[c][s];
                        const REAL Ak = A[2 * k + dir];
                        REAL t[4];
                        if (l % 2 == 0) { /* forward link: this site is the start */
                            FN(link_terms)(p, A, k, lnb[l], dir, q, dx, t);
                            gx += (REAL)0.5 / m * (t[0] / dx + t[1] / dx - q * Ak * t[2]) * w[l];
                            gy += (REAL)0.5 / m * (-t[2] / dx - t[3] / dx - q * Ak * t[0]) * w[l];
                            gax += dir == 0 ? -(REAL)0.5 * q / m * (y * t[0] + x * t[2]) * w[l] : 0;
                            gay += dir == 1 ? -(REAL)0.5 * q / m * (y * t[0] + x * t[2]) * w[l] : 0;
                        } else {          /* backward link: this site is the finish */
                            FN(link_terms)(p, A, lnb[l], k, dir, q, dx, t);
                            gx += (REAL)0.5 / m * (-t[1] / dx - t[0] / dx - q * Ak * t[3]) * w[l];
                            gy += (REAL)0.5 / m * (t[3] / dx + t[2] / dx - q * Ak * t[1]) * w[l];
                            gax += dir == 0 ? -(REAL)0.5 * q / m * (y * t[1] + x * t[3]) * w[l] : 0;
                            gay += dir == 1 ? -(REAL)0.5 * q / m * (y * t[1] + x * t[3]) * w[l] : 0;
                        }
                    }
                    if (!maxwell) { gs[c][2 * k] = gx; gs[c][2 * k + 1] = gy; }
                }
                if (P->ncomp == 2 && !maxwell) {
                    const REAL x1 = p1[2 * k], y1 = p1[2 * k + 1], x2 = p2[2 * k], y2 = p2[2 * k + 1];
                    const REAL r1 = FN(sq)(x1) + FN(sq)(y1), r2 = FN(sq)(x2) + FN(sq)(y2);
                    const REAL R = x1 * x2 + y1 * y2, I = x1 * y2 - y1 * x2;
                    /* bilinear Josephson (nlcg.cu:622-629) */
                    g1[2 * k] += P->eta * x2 * area; g1[2 * k + 1] += P->eta * y2 * area;
                    g2[2 * k] += P->eta * x1 * area; g2[2 * k + 1] += P->eta * y1 * area;
                    /* density coupling (nlcg.cu:631-637) */
                    g1[2 * k] += P->gamma * x1 * r2 * area; g1[2 * k + 1] += P->gamma * y1 * r2 * area;
                    g2[2 * k] += P->gamma * x2 * r1 * area; g2[2 * k + 1] += P->gamma * y2 * r1 * area;
                    /* biquadratic Josephson (nlcg.cu:639-648) */
                    g1[2 * k] += P->delta * (x2 * R - y2 * I) * area;
                    g1[2 * k + 1] += P->delta * (y2 * R + x2 * I) * area;
                    g2[2 * k] += P->delta * (x1 * R + y1 * I) * area;
                    g2[2 * k + 1] += P->delta * (y1 * R - x1 * I) * area;
                }
                if (!maxwell)
                    for (int c = 0; c < P->ncomp; ++c) { gs[c][2 * k] *= dx * dx; gs[c][2 * k + 1] *= dx * dx; }

                /* curl: every collocated view of a plaquette containing A at this
                 * site, with the applied field h of the viewing site
                 * (nlcg.cu:852-883). */
                if (!P->thin_film) {
                    const REAL *h = P->h;
#define AX(kk) A[2 * (kk)]
#define AY(kk) A[2 * (kk) + 1]
                    const REAL c4 = (REAL)0.25 / dx;
                    if (B_(cc, 0) && B_(cc, 1) && B_(cc, 2)) {
                        const REAL r = (AY(k + 1) - AY(k)) / dx - (AX(k + nx) - AX(k)) / dx - h[s];
                        gax += c4 * r; gay -= c4 * r;
                        gay -= c4 * ((AY(k + 1) - AY(k)) / dx - (AX(k + nx + 1) - AX(k + 1)) / dx - h[s + 1]);
                        gax += c4 * ((AY(k + 1 + nx) - AY(k + nx)) / dx - (AX(k + nx) - AX(k)) / dx - h[s + nx]);
                    }
                    if (B_(cc, 2) && B_(cc, 3) && B_(cc, 4)) {
                        const REAL r = (AY(k) - AY(k - 1)) / dx - (AX(k + nx) - AX(k)) / dx - h[s];
                        gax += c4 * r; gay += c4 * r;
                        gax += c4 * ((AY(k + nx) - AY(k + nx - 1)) / dx - (AX(k + nx) - AX(k)) / dx - h[s + nx]);
                        gay += c4 * ((AY(k) - AY(k - 1)) / dx - (AX(k + nx - 1) - AX(k - 1)) / dx - h[s - 1]);
                    }
                    if (B_(cc, 4) && B_(cc, 5) && B_(cc, 6)) {
                        const REAL r = (AY(k) - AY(k - 1)) / dx - (AX(k) - AX(k - nx)) / dx - h[s];
                        gax -= c4 * r; gay += c4 * r;
                        gay += c4 * ((AY(k) - AY(k - 1)) / dx - (AX(k - 1) - AX(k - 1 - nx)) / dx - h[s - 1]);
                        gax -= c4 * ((AY(k - nx) - AY(k - nx - 1)) / dx - (AX(k) - AX(k - nx)) / dx - h[s - nx]);
                    }
                    if (B_(cc, 6) && B_(cc, 7) && B_(cc, 0)) {
                        const REAL r = (AY(k + 1) - AY(k)) / dx - (AX(k) - AX(k - nx)) / dx - h[s];
                        gax -= c4 * r; gay -= c4 * r;
                        gax -= c4 * ((AY(k - nx + 1) - AY(k - nx)) / dx - (AX(k) - AX(k - nx)) / dx - h[s - nx]);
                        gay -= c4 * ((AY(k + 1) - AY(k)) / dx - (AX(k + 1) - AX(k + 1 - nx)) / dx - h[s + 1]);
                    }
#undef AX
#undef AY
                    gA[2 * k] = gax * dx * dx;
                    gA[2 * k + 1] = gay * dx * dx;
                } else {
                    gA[2 * k] = 0;
                    gA[2 * k + 1] = 0;
                }
            }
    if (maxwell) {
        const long tot = 2 * F * M;
        for (long t = 0; t < tot; ++t) { g1[t] = 0; if (P->ncomp == 2) g2[t] = 0; }
    }
}

/* ------------------------------------------------------------ polynomial
 * Coefficients of F(x + alpha d) = A + B a + C a^2 + D a^3 + E a^4 per image,
 * restating polynomialExpansion (nlcg.cu:997-1370).  With compat != 0 the
 * reference's two slips are kept: the x-link first-order term adds
 * +A_d psi instead of -q A_d psi (nlcg.cu:1162-1165, 1269-1272) and the
 * y-link cubic coefficient carries an extra factor 1/2 (nlcg.cu:1251,1358).
 * With compat == 0 the coefficients are the exact expansion.
 */
static void FN(site_poly)(const PROB *P, const REAL *A, const REAL *const ps[2], const REAL *dA,
                          const REAL *const ds[2], long o, int i, int j, int compat, REAL out[5])
{
    const int nx = P->nx;
    const long s = i + (long)nx * j, k = o + s;
    const unsigned sc = P->sc_nn[s], cc = P->comp_nn[s];
    const REAL dx = P->dx, dx2 = dx * dx;
    REAL e = 0, b1 = 0, c2 = 0, d3 = 0, e4 = 0;
    const REAL area = (REAL)(B_(sc, 0) * B_(sc, 1) * B_(sc, 2) + B_(sc, 2) * B_(sc, 3) * B_(sc, 4)
                           + B_(sc, 4) * B_(sc, 5) * B_(sc, 6) + B_(sc, 6) * B_(sc, 7) * B_(sc, 0)) / (REAL)4;
    for (int c = 0; c < P->ncomp; ++c) {
        const REAL x = ps[c][2 * k], y = ps[c][2 * k + 1], u = ds[c][2 * k], v = ds[c][2 * k + 1];
        const REAL bb = P->b[c][s];
        const REAL n0 = P->a[c][s] / bb + x * x + y * y, n1 = 2 * (x * u + y * v), n2 = u * u + v * v;
        e += bb * ((REAL)0.5 * n0 * n0) * area * dx2;
        b1 += bb * (n0 * n1) * area * dx2;
        c2 += bb * ((REAL)0.5 * n1 * n1 + n0 * n2) * area * dx2;
        d3 += bb * (n1 * n2) * area * dx2;
        e4 += bb * ((REAL)0.5 * n2 * n2) * area * dx2;
    }
    if (P->ncomp == 2) {
        const REAL x1 = ps[0][2 * k], y1 = ps[0][2 * k + 1], x2 = ps[1][2 * k], y2 = ps[1][2 * k + 1];
        const REAL u1 = ds[0][2 * k], v1 = ds[0][2 * k + 1], u2 = ds[1][2 * k], v2 = ds[1][2 * k + 1];
        const REAL w = area * dx2;
        /* eta Re(psi1 psi2*) */
        const REAL R0 = x1 * x2 + y1 * y2, R1 = u1 * x2 + v1 * y2 + x1 * u2 + y1 * v2, R2 = u1 * u2 + v1 * v2;
        e += P->eta * R0 * w; b1 += P->eta * R1 * w; c2 += P->eta * R2 * w;
        /* gamma/2 |psi1|^2 |psi2|^2 */
        const REAL r1 = x1 * x1 + y1 * y1, r2 = x2 * x2 + y2 * y2;
        const REAL s1 = 2 * (x1 * u1 + y1 * v1), s2 = 2 * (x2 * u2 + y2 * v2);
        const REAL t1 = u1 * u1 + v1 * v1, t2 = u2 * u2 + v2 * v2;
        const REAL g = P->gamma / (REAL)2;
        e += g * r1 * r2 * w;
        b1 += g * (s1 * r2 + s2 * r1) * w;
        c2 += g * (s1 * s2 + r1 * t2 + r2 * t1) * w;
        d3 += g * (s1 * t2 + s2 * t1) * w;
        e4 += g * (t1 * t2) * w;
        /* delta/2 (Re^2 - Im^2) of psi1 psi2* */
        const REAL I0 = x1 * y2 - y1 * x2, I1 = x1 * v2 + u1 * y2 - y1 * u2 - v1 * x2, I2 = u1 * v2 - v1 * u2;
        const REAL dd = P->delta / (REAL)2;
        e += dd * (R0 * R0 - I0 * I0) * w;
        b1 += dd * (2 * R1 * R0 - 2 * I1 * I0) * w;
        c2 += dd * (R1 * R1 - I1 * I1 + 2 * R0 * R2 - 2 * I0 * I2) * w;
        d3 += dd * (2 * R1 * R2 - 2 * I1 * I2) * w;
        e4 += dd * (R2 * R2 - I2 * I2) * w;
    }
    if (!P->thin_film) {
        const REAL h = P->h[s];
#define AX(X, kk) (X)[2 * (kk)]
#define AY(X, kk) (X)[2 * (kk) + 1]
        const int views[4][3] = {{0, 1, 2}, {2, 3, 4}, {4, 5, 6}, {6, 7, 0}};
        for (int vw = 0; vw < 4; ++vw) {
            if (!(B_(cc, views[vw][0]) && B_(cc, views[vw][1]) && B_(cc, views[vw][2]))) continue;
            const int fwdx = (vw == 0 || vw == 3), fwdy = (vw == 0 || vw == 1);
            const long kx0 = fwdx ? k : k - 1, kx1 = fwdx ? k + 1 : k;
            const long ky0 = fwdy ? k : k - nx, ky1 = fwdy ? k + nx : k;
            const REAL m0 = (AY(A, kx1) - AY(A, kx0)) / dx - (AX(A, ky1) - AX(A, ky0)) / dx - h;
            const REAL m1 = (AY(dA, kx1) - AY(dA, kx0)) / dx - (AX(dA, ky1) - AX(dA, ky0)) / dx;
            e += ((REAL)0.5 * m0 * m0) * (REAL)0.25 * dx2;
            b1 += (m0 * m1) * (REAL)0.25 * dx2;
            c2 += ((REAL)0.5 * m1 * m1) * (REAL)0.25 * dx2;
        }
#undef AX
#undef AY
    }
    const REAL cw[2] = {(REAL)(B_(sc, 1) * B_(sc, 2) + B_(sc, 6) * B_(sc, 7)) / (REAL)2,
                        (REAL)(B_(sc, 0) * B_(sc, 1) + B_(sc, 3) * B_(sc, 4)) / (REAL)2};
    for (int dir = 0; dir < 2; ++dir) {
        if (!B_(sc, dir == 0 ? 0 : 2)) continue;
        const long kj = k + (dir == 0 ? 1 : nx);
        const REAL Ai = A[2 * k + dir], Aj = A[2 * kj + dir];
        const REAL ai = dA[2 * k + dir], aj = dA[2 * kj + dir];
        for (int c = 0; c < P->ncomp; ++c) {
            const REAL *p = ps[c], *d = ds[c];
            const REAL q = P->q[c];
            const REAL m = dir == 0 ? P->mxx[c][s] : P->myy[c][s];
            /* coefficient of A_d psi in the first-order term */
            const REAL qd = (compat && dir == 0) ? (REAL)-1 : q;
            REAL t0[4], t1[4], t2[4];
            FN(link_terms)(p, A, k, kj, dir, q, dx, t0);
            const REAL ddre = (d[2 * kj] - d[2 * k]) / dx, ddim = (d[2 * kj + 1] - d[2 * k + 1]) / dx;
            t1[0] = -ddre - q * Ai * d[2 * k + 1] - qd * ai * p[2 * k + 1];
            t1[1] = -ddre - q * Aj * d[2 * kj + 1] - qd * aj * p[2 * kj + 1];
            t1[2] = ddim - q * Ai * d[2 * k] - qd * ai * p[2 * k];
            t1[3] = ddim - q * Aj * d[2 * kj] - qd * aj * p[2 * kj];
            t2[0] = -q * ai * d[2 * k + 1];
            t2[1] = -q * aj * d[2 * kj + 1];
            t2[2] = -q * ai * d[2 * k];
            t2[3] = -q * aj * d[2 * kj];
            REAL se = 0, sb = 0, scc = 0, sd = 0, s4 = 0;
            for (int t = 0; t < 4; ++t) {
                se += (REAL)0.5 * t0[t] * t0[t];
                sb += t0[t] * t1[t];
                scc += (REAL)0.5 * t1[t] * t1[t] + t0[t] * t2[t];
                sd += t1[t] * t2[t];
                s4 += (REAL)0.5 * t2[t] * t2[t];
            }
            const REAL f = cw[dir] / (2 * m) * dx2;
            e += se * f;
            b1 += sb * f;
            c2 += scc * f;
            d3 += sd * f * ((compat && dir == 1) ? (REAL)0.5 : (REAL)1);
            e4 += s4 * f;
        }
    }
    out[0] = e; out[1] = b1; out[2] = c2; out[3] = d3; out[4] = e4;
}

void FN(glo_polynomial)(const PROB *P, int F, const REAL *A, const REAL *p1, const REAL *p2, const REAL *dA,
                        const REAL *d1, const REAL *d2, int compat, double *energy, double *poly4)
{
    const REAL *ps[2] = {p1, p2}, *ds[2] = {d1, d2};
    const long M = (long)P->nx * P->ny;
    GLO_OMP_FOR
    for (int n = 0; n < F; ++n) {
        FN(ksum) acc[5] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}, {0, 0}};
        for (int j = 0; j < P->ny; ++j)
            for (int i = 0; i < P->nx; ++i) {
                REAL o[5];
                FN(site_poly)(P, A, ps, dA, ds, n * M, i, j, compat, o);
                for (int t = 0; t < 5; ++t) FN(kadd)(&acc[t], o[t]);
            }
        energy[n] = FN(kval)(&acc[0]);
        for (int t = 0; t < 4; ++t) poly4[4 * n + t] = FN(kval)(&acc[t + 1]);
    }
}

/* ------------------------------------------------------------ line search
 * lineSearch (nlcg.cu:1398-1445): scan x_p = x_0 m^p (x_0 = 1e-10, m = 1.025f,
 * both rounded to REAL, the product rounded to REAL each step), stop at the
 * first p <= 2000 where the quartic increases, alpha = x_p / m.  The quartic
 * is evaluated in double as E (x^2)^2 + D x x x + C x x + B x + A (no
 * fused multiply-add; the CUDA kernel evaluates it the same way).
 */
static double FN(quartic)(const double c[5], double x)
{
    const double x2 = x * x;
    double f = c[4] * (x2 * x2);
    f = f + c[3] * x * x * x;
    f = f + c[2] * x * x;
    f = f + c[1] * x;
    f = f + c[0];
    return f;
}

static double FN(line_search_compat)(const double c[5])
{
    const REAL m = (REAL)1.025f;
    REAL x = (REAL)1e-10;
    double f_old = FN(quartic)(c, (double)x);
    for (int p = 0; p < 2000; ++p) {
        x = x * m;
        const double f_new = FN(quartic)(c, (double)x);
        if (f_new > f_old) break;
        f_old = f_new;
    }
    return (double)(REAL)(x / m);
}

/* Exact version of the compat scan: the first local minimum of the quartic
 * reached from alpha = 0 downhill, i.e. the smallest positive root of
 * p'(a) = B + 2C a + 3D a^2 + 4E a^3 (closed form, then two Newton steps)
 * with p'' > 0.  The scan stops at the first increase, so when p'(0) >= 0 or
 * no such root exists this falls back to the scan itself. */
static double FN(line_search_exact)(const double c[5])
{
    const double a3 = 4 * c[4], a2 = 3 * c[3], a1 = 2 * c[2], a0 = c[1];
    double roots[3];
    int nr = 0;
    const double scale = fabs(a0) + fabs(a1) + fabs(a2) + fabs(a3);
    if (scale == 0) return FN(line_search_compat)(c);
    if (fabs(a3) > 1e-300) {
        const double A2 = a2 / a3, A1 = a1 / a3, A0 = a0 / a3;
        const double Q = (3 * A1 - A2 * A2) / 9, R = (9 * A2 * A1 - 27 * A0 - 2 * A2 * A2 * A2) / 54;
        const double disc = Q * Q * Q + R * R;
        if (disc >= 0) {
            const double sd = sqrt(disc);
            const double S = cbrt(R + sd), T = cbrt(R - sd);
            roots[nr++] = -A2 / 3 + S + T;
        } else {
            const double th = acos(R / sqrt(-Q * Q * Q));
            const double r = 2 * sqrt(-Q);
            roots[nr++] = r * cos(th / 3) - A2 / 3;
            roots[nr++] = r * cos((th + 2 * M_PI) / 3) - A2 / 3;
            roots[nr++] = r * cos((th + 4 * M_PI) / 3) - A2 / 3;
        }
    } else if (fabs(a2) > 1e-300) {
        const double disc = a1 * a1 - 4 * a2 * a0;
        if (disc >= 0) {
            const double sq = sqrt(disc);
            const double qq = -0.5 * (a1 + (a1 >= 0 ? sq : -sq));
            if (qq != 0) { roots[nr++] = qq / a2; roots[nr++] = a0 / qq; }
        }
    } else if (a1 != 0) {
        roots[nr++] = -a0 / a1;
    }
    if (!(a0 < 0)) return FN(line_search_compat)(c);
    double best = -1;
    for (int t = 0; t < nr; ++t) {
        double r = roots[t];
        for (int it = 0; it < 2; ++it) {
            const double dp = a0 + r * (a1 + r * (a2 + r * a3));
            const double ddp = a1 + r * (2 * a2 + r * 3 * a3);
            if (ddp != 0) r -= dp / ddp;
        }
        const double ddp = a1 + r * (2 * a2 + r * 3 * a3);
        if (!(r > 0) || !(ddp > 0)) continue;
        if (best < 0 || r < best) best = r;
    }
    if (best < 0) return FN(line_search_compat)(c);
    return best;
}

void FN(glo_line_search)(int F, const double *energy, const double *poly4, int mode, double *alpha)
{
    for (int n = 0; n < F; ++n) {
        const double c[5] = {energy[n], poly4[4 * n], poly4[4 * n + 1], poly4[4 * n + 2], poly4[4 * n + 3]};
        alpha[n] = mode == GLO_LS_EXACT ? FN(line_search_exact)(c) : FN(line_search_compat)(c);
    }
}

/* --------------------------------------------------------------------- B, J
 * computeJBKernel (nlcg.cu:243-364): B at a site = mean of the collocated
 * curl views of its valid computational plaquettes; J_alpha from the
 * forward and backward links (no link weights, no dx^2).
 */
void FN(glo_jb)(const PROB *P, int F, const REAL *A, const REAL *p1, const REAL *p2, REAL *b, REAL *j1, REAL *j2)
{
    const REAL *ps[2] = {p1, p2};
    REAL *js[2] = {j1, j2};
    const int nx = P->nx;
    const long M = (long)nx * P->ny;
    const REAL dx = P->dx;
    GLO_OMP_FOR
    for (int n = 0; n < F; ++n)
        for (int j = 0; j < P->ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const long s = i + (long)nx * j, k = n * M + s;
                const unsigned sc = P->sc_nn[s], cc = P->comp_nn[s];
#define AX(kk) A[2 * (kk)]
#define AY(kk) A[2 * (kk) + 1]
                REAL bb = 0;
                if (B_(cc, 0) && B_(cc, 1) && B_(cc, 2)) bb += (REAL)0.25 * ((AY(k + 1) - AY(k)) / dx - (AX(k + nx) - AX(k)) / dx);
                if (B_(cc, 2) && B_(cc, 3) && B_(cc, 4)) bb += (REAL)0.25 * ((AY(k) - AY(k - 1)) / dx - (AX(k + nx) - AX(k)) / dx);
                if (B_(cc, 4) && B_(cc, 5) && B_(cc, 6)) bb += (REAL)0.25 * ((AY(k) - AY(k - 1)) / dx - (AX(k) - AX(k - nx)) / dx);
                if (B_(cc, 6) && B_(cc, 7) && B_(cc, 0)) bb += (REAL)0.25 * ((AY(k + 1) - AY(k)) / dx - (AX(k) - AX(k - nx)) / dx);
#undef AX
#undef AY
                if (bb != 0) {
                    const int cnt = B_(cc, 0) * B_(cc, 1) * B_(cc, 2) + B_(cc, 2) * B_(cc, 3) * B_(cc, 4)
                                  + B_(cc, 4) * B_(cc, 5) * B_(cc, 6) + B_(cc, 6) * B_(cc, 7) * B_(cc, 0);
                    bb /= (REAL)cnt / (REAL)4;
                }
                b[k] = bb;
                for (int c = 0; c < P->ncomp; ++c) {
                    const REAL *p = ps[c];
                    const REAL q = P->q[c];
                    const REAL x = p[2 * k], y = p[2 * k + 1];
                    REAL jx = 0, jy = 0;
                    REAL t[4];
                    if (B_(sc, 0)) { FN(link_terms)(p, A, k, k + 1, 0, q, dx, t); jx += (REAL)0.5 * q / P->mxx[c][s] * (y * t[0] + x * t[2]); }
                    if (B_(sc, 4)) { FN(link_terms)(p, A, k - 1, k, 0, q, dx, t); jx += (REAL)0.5 * q / P->mxx[c][s] * (y * t[1] + x * t[3]); }
                    if (B_(sc, 2)) { FN(link_terms)(p, A, k, k + nx, 1, q, dx, t); jy += (REAL)0.5 * q / P->myy[c][s] * (y * t[0] + x * t[2]); }
                    if (B_(sc, 6)) { FN(link_terms)(p, A, k - nx, k, 1, q, dx, t); jy += (REAL)0.5 * q / P->myy[c][s] * (y * t[1] + x * t[3]); }
                    js[c][2 * k] = jx;
                    js[c][2 * k + 1] = jy;
                }
            }
}

/* -------------------------------------------------------------- arc length
 * arcLengthParametrization{,JB} + computeArcLength (interpolation.cu:39-140):
 * squared distance between consecutive images over all sites (no mask, no
 * dx^2), cumulative square root, normalised so that s[F-1] = 1.
 * `fields` lists nf pointers to per-image arrays of `width` reals per site.
 */
static void FN(arc_finish)(int F, double *s)
{
    s[0] = 0;
    for (int n = 1; n < F; ++n) s[n] = s[n - 1] + sqrt(s[n]);
    for (int n = 0; n < F; ++n) s[n] /= s[F - 1];
}

void FN(glo_arc_length)(int F, long M, int nf, const REAL *const *fields, const int *width, double *s)
{
    s[0] = 0;
    GLO_OMP_FOR
    for (int n = 1; n < F; ++n) {
        FN(ksum) acc = {0, 0};
        for (long t = 0; t < M; ++t) {
            REAL d2 = 0;
            for (int f = 0; f < nf; ++f)
                for (int w = 0; w < width[f]; ++w) {
                    const long kk = width[f] * (n * M + t) + w, kp = width[f] * ((n - 1) * M + t) + w;
                    d2 += FN(sq)(fields[f][kk] - fields[f][kp]);
                }
            FN(kadd)(&acc, d2);
        }
        s[n] = FN(kval)(&acc);
    }
    FN(arc_finish)(F, s);
}

/* ---------------------------------------------------------- redistribution
 * Linear: generateNewFramesLinear (interpolation.cu:190-227).  Cubic:
 * buildHMatrix / computeDelta / gtsv / generateNewFramesCubic
 * (interpolation.cu:252-402) with the Forsythe-Malcolm-Moler end
 * conditions; spline == GLO_SPLINE_COMPAT keeps the reference's sign of the
 * sigma_{k-1} term (392-400) and its running-sum segment walk (376-386);
 * GLO_SPLINE_FMM uses the textbook sign and the node values s[k].
 * f is F images of M sites x 2 reals, f_new receives F_new images.
 */
void FN(glo_redistribute_linear)(int F, long M, const double *s, const REAL *f, int F_new, REAL *f_new)
{
    int k = 1;
    double seg_start = 0, seg_end = s[1];
    for (int n = 0; n < F_new; ++n) {
        const double s_new = (double)n / (double)(F_new - 1);
        while (seg_end < s_new && k < F - 1) { k++; seg_start = s[k - 1]; seg_end = s[k]; }
        if (k >= F) k = F - 1;
        const REAL w = (REAL)((s_new - seg_start) / (s[k] - s[k - 1]));
        for (long t = 0; t < 2 * M; ++t)
            f_new[2 * M * n + t] = w * f[2 * M * k + t] + (1 - w) * f[2 * M * (k - 1) + t];
    }
}

void FN(glo_redistribute_cubic)(int F, long M, const double *s, const REAL *f, int F_new, REAL *f_new, int spline)
{
    double *h = (double *)calloc(F + 1, sizeof(double));
    double *dl = (double *)calloc(F, sizeof(double)), *d = (double *)calloc(F, sizeof(double));
    double *du = (double *)calloc(F, sizeof(double)), *du2 = (double *)calloc(F, sizeof(double));
    int *ipiv = (int *)calloc(F, sizeof(int));
    double *rhs = (double *)calloc(F, sizeof(double)), *D = (double *)calloc(F, sizeof(double));
    double *sig = (double *)calloc((size_t)F * 2 * M, sizeof(double));
    h[0] = 0;
    for (int n = 1; n < F; ++n) h[n] = s[n] - s[n - 1];
    h[F] = INFINITY;
    d[0] = -h[1]; du[0] = h[1];
    for (int n = 1; n < F - 1; ++n) { dl[n] = h[n]; d[n] = 2 * (h[n] + h[n + 1]); du[n] = h[n + 1]; }
    dl[F - 1] = h[F - 1]; d[F - 1] = -h[F - 1];
    glo_gttrf_d(F, dl, d, du, du2, ipiv);
    for (long t = 0; t < 2 * M; ++t) {
        for (int n = 1; n < F; ++n) D[n] = ((double)f[2 * M * n + t] - (double)f[2 * M * (n - 1) + t]) / h[n];
        const double d3s = ((D[3] - D[2]) / (h[3] + h[2]) - (D[2] - D[1]) / (h[2] + h[1])) / (h[3] + h[2] + h[1]);
        const double d3e = ((D[F - 1] - D[F - 2]) / (h[F - 1] + h[F - 2]) - (D[F - 2] - D[F - 3]) / (h[F - 2] + h[F - 3]))
                         / (h[F - 1] + h[F - 2] + h[F - 3]);
        for (int n = 1; n < F - 1; ++n) rhs[n] = D[n + 1] - D[n];
        rhs[0] = h[1] * h[1] * d3s;
        rhs[F - 1] = -(h[F - 1] * h[F - 1]) * d3e;
        glo_gttrs_d(F, dl, d, du, du2, ipiv, rhs, 1);
        for (int n = 0; n < F; ++n) sig[(size_t)F * t + n] = rhs[n];
    }
    int k = 1;
    double seg_start = 0, seg_end = spline == GLO_SPLINE_COMPAT ? h[1] : s[1];
    for (int n = 0; n < F_new; ++n) {
        const double s_new = (double)n / (double)(F_new - 1);
        if (spline == GLO_SPLINE_COMPAT) {
            while (seg_end < s_new) { k++; seg_start += h[k - 1]; seg_end += h[k]; }
        } else {
            while (seg_end < s_new && k < F - 1) { k++; seg_start = s[k - 1]; seg_end = s[k]; }
        }
        if (k >= F) k = F - 1;
        const double w = (s_new - seg_start) / h[k];
        const double wm = spline == GLO_SPLINE_COMPAT ? (w - 1) : (1 - w);
        const double hk2 = h[k] * h[k];
        for (long t = 0; t < 2 * M; ++t) {
            const double sk = sig[(size_t)F * t + k], sk1 = sig[(size_t)F * t + k - 1];
            f_new[2 * M * n + t] = (REAL)(w * f[2 * M * k + t] + (1 - w) * f[2 * M * (k - 1) + t]
                                          + hk2 * ((w * w * w - w) * sk + (wm * wm * wm - wm) * sk1));
        }
    }
    free(h); free(dl); free(d); free(du); free(du2); free(ipiv); free(rhs); free(D); free(sig);
}

/* ------------------------------------------------------------------ solver
 * The NLCG state machine of nlcgSteps (nlcg.cu:1462-1586) and loop()
 * (mepgl.cu:38-391), with the same buffers and slot semantics as the CUDA
 * library: nlcgSteps receives its gradient and norm buffers by value, so each
 * call starts by treating slot 0 as "previous" and writes slot 1 on odd
 * substeps, slot 0 on even ones.
 */
typedef struct FN(glo_solver) {
    PROB P;
    int F;
    long M;
    REAL *x[3], *g[2][3], *d[3], *xn[3];
    double *S[2], *gdg, *fe, *poly, *alpha, *s, *s_jb;
    int ls_mode, poly_compat;
} FN(glo_solver);

FN(glo_solver) *FN(glo_solver_create)(const PROB *P, int F, const REAL *A, const REAL *p1, const REAL *p2,
                                      int ls_mode, int poly_compat)
{
    FN(glo_solver) *S = (FN(glo_solver) *)calloc(1, sizeof(FN(glo_solver)));
    S->P = *P;
    S->F = F;
    S->M = (long)P->nx * P->ny;
    const size_t n2 = (size_t)2 * F * S->M;
    for (int c = 0; c < 3; ++c) {
        S->x[c] = (REAL *)calloc(n2, sizeof(REAL));
        S->xn[c] = (REAL *)calloc(n2, sizeof(REAL));
        S->d[c] = (REAL *)calloc(n2, sizeof(REAL));
        S->g[0][c] = (REAL *)calloc(n2, sizeof(REAL));
        S->g[1][c] = (REAL *)calloc(n2, sizeof(REAL));
    }
    memcpy(S->x[0], A, n2 * sizeof(REAL));
    memcpy(S->x[1], p1, n2 * sizeof(REAL));
    if (P->ncomp == 2) memcpy(S->x[2], p2, n2 * sizeof(REAL));
    for (int t = 0; t < 2; ++t) {
        S->S[t] = (double *)malloc(F * sizeof(double));
        for (int n = 0; n < F; ++n) S->S[t][n] = INFINITY;
    }
    S->gdg = (double *)calloc(F, sizeof(double));
    S->fe = (double *)calloc(F, sizeof(double));
    S->poly = (double *)calloc(4 * F, sizeof(double));
    S->alpha = (double *)calloc(F, sizeof(double));
    S->s = (double *)calloc(F, sizeof(double));
    S->s_jb = (double *)calloc(F, sizeof(double));
    S->ls_mode = ls_mode;
    S->poly_compat = poly_compat;
    return S;
}

void FN(glo_solver_destroy)(FN(glo_solver) *S)
{
    for (int c = 0; c < 3; ++c) { free(S->x[c]); free(S->xn[c]); free(S->d[c]); free(S->g[0][c]); free(S->g[1][c]); }
    free(S->S[0]); free(S->S[1]); free(S->gdg); free(S->fe); free(S->poly); free(S->alpha); free(S->s); free(S->s_jb);
    free(S);
}

void FN(glo_solver_nlcg_steps)(FN(glo_solver) *S, int iters, int use_cg, int maxwell)
{
    const int F = S->F;
    const long M = S->M, n2 = 2 * M;
    const int nc = S->P.ncomp;
    for (int it = 1; it <= iters; ++it) {
        const int cur = it & 1, prev = cur ^ 1;
        REAL **g = S->g[cur], **go = S->g[prev];
        FN(glo_gradient)(&S->P, F, S->x[0], S->x[1], S->x[2], g[0], g[1], g[2], maxwell);
        /* gradientDensity (nlcg.cu:919-949); absent components are zero */
    GLO_OMP_FOR
        for (int n = 0; n < F; ++n) {
            FN(ksum) a = {0, 0}, b = {0, 0};
            for (int c = 0; c < 1 + nc; ++c)
                for (long t = n * n2; t < (n + 1) * n2; ++t) {
                    FN(kadd)(&a, (double)(g[c][t] * g[c][t]));
                    FN(kadd)(&b, (double)(g[c][t] * (g[c][t] - go[c][t])));
                }
            S->S[cur][n] = FN(kval)(&a);
            S->gdg[n] = FN(kval)(&b);
        }
        /* computeStepDirection (nlcg.cu:955-994), Polak-Ribiere clipped at 0 */
    GLO_OMP_FOR
        for (int n = 0; n < F; ++n) {
            double beta = 0;
            if (use_cg) {
                beta = S->gdg[n] / S->S[prev][n];
                beta = beta > 0 ? beta : 0;
            }
            const REAL bt = (REAL)beta;
            for (int c = 0; c < 1 + nc; ++c)
                for (long t = n * n2; t < (n + 1) * n2; ++t) S->d[c][t] = -g[c][t] + bt * S->d[c][t];
        }
        FN(glo_polynomial)(&S->P, F, S->x[0], S->x[1], S->x[2], S->d[0], S->d[1], S->d[2], S->poly_compat, S->fe,
                           S->poly);
        FN(glo_line_search)(F, S->fe, S->poly, S->ls_mode, S->alpha);
        /* updateFields (nlcg.cu:1372-1396) */
    GLO_OMP_FOR
        for (int n = 0; n < F; ++n) {
            const REAL al = (REAL)S->alpha[n];
            for (int c = 0; c < 1 + nc; ++c)
                for (long t = n * n2; t < (n + 1) * n2; ++t) S->x[c][t] = S->x[c][t] + al * S->d[c][t];
        }
    }
}

/* CG restart of the interior images after a reparametrization (mepgl.cu:231-234). */
void FN(glo_solver_reset_interior)(FN(glo_solver) *S)
{
    for (int n = 1; n < S->F - 1; ++n) { S->S[0][n] = INFINITY; S->S[1][n] = INFINITY; }
}

void FN(glo_solver_arc_lengths)(FN(glo_solver) *S, double *s_fields, double *s_jb)
{
    const int F = S->F, nc = S->P.ncomp;
    const long M = S->M;
    const REAL *fl[3] = {S->x[0], S->x[1], S->x[2]};
    const int wd[3] = {2, 2, 2};
    FN(glo_arc_length)(F, M, 1 + nc, fl, wd, s_fields);
    REAL *b = (REAL *)calloc((size_t)F * M, sizeof(REAL));
    REAL *j1 = (REAL *)calloc((size_t)2 * F * M, sizeof(REAL)), *j2 = (REAL *)calloc((size_t)2 * F * M, sizeof(REAL));
    FN(glo_jb)(&S->P, F, S->x[0], S->x[1], S->x[2], b, j1, j2);
    const REAL *jl[3] = {b, j1, j2};
    const int jw[3] = {1, 2, 2};
    FN(glo_arc_length)(F, M, 1 + nc, jl, jw, s_jb);
    free(b); free(j1); free(j2);
}

/* One outer iteration of loop() in mode S, M, L or C (mepgl.cu:148-303);
 * kind of spline as in glo_redistribute_cubic. */
void FN(glo_solver_iteration)(FN(glo_solver) *S, char mode, int relaxation_steps, int use_cg, int spline)
{
    const int F = S->F, nc = S->P.ncomp;
    const long M = S->M;
    if (mode == 'S' || mode == 'M') {
        FN(glo_solver_nlcg_steps)(S, relaxation_steps, use_cg, mode == 'M');
        return;
    }
    if (mode != 'L' && mode != 'C') return;
    FN(glo_solver_arc_lengths)(S, S->s, S->s_jb);
    for (int c = 0; c < 1 + nc; ++c) {
        if (mode == 'L') FN(glo_redistribute_linear)(F, M, S->s_jb, S->x[c], F, S->xn[c]);
        else FN(glo_redistribute_cubic)(F, M, S->s_jb, S->x[c], F, S->xn[c], spline);
        REAL *t = S->x[c]; S->x[c] = S->xn[c]; S->xn[c] = t;
    }
    FN(glo_solver_reset_interior)(S);
    FN(glo_solver_nlcg_steps)(S, relaxation_steps, use_cg, 0);
}

void FN(glo_solver_get)(const FN(glo_solver) *S, REAL *A, REAL *p1, REAL *p2, double *fenergy, double *g_norm2,
                        double *alpha, double *s, double *s_jb)
{
    const size_t n2 = (size_t)2 * S->F * S->M;
    if (A) memcpy(A, S->x[0], n2 * sizeof(REAL));
    if (p1) memcpy(p1, S->x[1], n2 * sizeof(REAL));
    if (p2) memcpy(p2, S->x[2], n2 * sizeof(REAL));
    for (int n = 0; n < S->F; ++n) {
        if (fenergy) fenergy[n] = S->fe[n];
        if (g_norm2) g_norm2[n] = S->S[0][n];
        if (alpha) alpha[n] = S->alpha[n];
        if (s) s[n] = S->s[n];
        if (s_jb) s_jb[n] = S->s_jb[n];
    }
}

#undef B_
#undef PROB
#undef FN
#undef GLO_CAT
#undef GLO_CAT2
