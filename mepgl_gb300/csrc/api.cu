// api.cu -- the C ABI of libmepgl_gb300 (include/mepgl.h): context,
// buffers, NLCG orchestration with CUDA-graph replay, reparametrization.
//
// A context owns one or more strings (all of one precision and component
// count) and every device buffer they need, allocated at creation: fields
// x (ping-pong), gradients g (two slots), directions d (ping-pong),
// packed neighbour masks, per-site parameters when not uniform, per-image
// scalars and per-tile partials.  The reference instead allocated and freed
// scratch inside every call (mepgl/src/nlcg.cu:225-239,
// mepgl/src/parallel_sum.cu:49-67, mepgl/src/interpolation.cu:410-480).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "context.h"

using namespace mepgl;

namespace {

thread_local std::string g_create_error;

}  // namespace

namespace {

const double INF = INFINITY;

mepgl_status fail(mepgl_ctx *c, mepgl_status st, const std::string &msg)
{
    if (c) c->err = msg;
    else g_create_error = msg;
    return st;
}

#define CK(ctx, call)                                                                               \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess)                                                                      \
            return fail(ctx, MEPGL_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));  \
    } while (0)

size_t real_size(int prec) { return prec == 1 ? 8 : 4; }

template <class T>
void *upload_as(mepgl_ctx *c, const std::vector<double> &v, cudaError_t *e)
{
    std::vector<T> tmp(v.begin(), v.end());
    void *p = nullptr;
    *e = cudaMalloc(&p, tmp.size() * sizeof(T));
    if (*e == cudaSuccess) *e = cudaMemcpy(p, tmp.data(), tmp.size() * sizeof(T), cudaMemcpyHostToDevice);
    (void)c;
    return p;
}

std::vector<uint16_t> masks_of(const StringHost &s)
{
    static const int di[8] = {1, 1, 0, -1, -1, -1, 0, 1};
    static const int dj[8] = {0, 1, 1, 1, 0, -1, -1, -1};
    std::vector<uint16_t> m(s.M());
    for (int j = 0; j < s.ny; ++j)
        for (int i = 0; i < s.nx; ++i) {
            unsigned code[2] = {0, 0};
            const std::vector<int32_t> *dom[2] = {&s.comp, &s.sc};
            for (int w = 0; w < 2; ++w) {
                if ((*dom[w])[i + (long)s.nx * j] == 0) continue;
                for (int b = 0; b < 8; ++b) {
                    const int ii = i + di[b], jj = j + dj[b];
                    if (ii < 0 || ii >= s.nx || jj < 0 || jj >= s.ny) continue;
                    if ((*dom[w])[ii + (long)s.nx * jj] != 0) code[w] |= 1u << b;
                }
            }
            m[i + (long)s.nx * j] = (uint16_t)(code[0] | (code[1] << 8));
        }
    return m;
}

void free_string_buffers(StringHost &s)
{
    for (int b = 0; b < 2; ++b)
        for (int f = 0; f < 3; ++f) {
            cudaFree(s.x[b][f]);
            cudaFree(s.g[b][f]);
            cudaFree(s.d[b][f]);
            s.x[b][f] = s.g[b][f] = s.d[b][f] = nullptr;
        }
}

void free_string_params(StringHost &s)
{
    for (auto &p : s.dparams) { cudaFree(p); p = nullptr; }
    cudaFree(s.dmask);
    s.dmask = nullptr;
}

mepgl_status alloc_string_buffers(mepgl_ctx *c, StringHost &s)
{
    const size_t bytes = (size_t)s.F * s.M() * 2 * real_size(c->precision);
    for (int b = 0; b < 2; ++b)
        for (int f = 0; f < 1 + c->ncomp; ++f) {
            CK(c, cudaMalloc(&s.x[b][f], bytes));
            CK(c, cudaMalloc(&s.g[b][f], bytes));
            CK(c, cudaMalloc(&s.d[b][f], bytes));
            CK(c, cudaMemsetAsync(s.x[b][f], 0, bytes, c->stream));
            CK(c, cudaMemsetAsync(s.g[b][f], 0, bytes, c->stream));
            CK(c, cudaMemsetAsync(s.d[b][f], 0, bytes, c->stream));
        }
    return MEPGL_OK;
}

mepgl_status upload_string_params(mepgl_ctx *c, StringHost &s)
{
    free_string_params(s);
    const std::vector<uint16_t> m = masks_of(s);
    CK(c, cudaMalloc(&s.dmask, m.size() * sizeof(uint16_t)));
    CK(c, cudaMemcpy(s.dmask, m.data(), m.size() * sizeof(uint16_t), cudaMemcpyHostToDevice));
    if (!s.uniform) {
        for (int k = 0; k < 9; ++k) {
            if (k >= 4 && k < 8 && c->ncomp == 1) continue;
            cudaError_t e;
            s.dparams[k] = c->precision == 1 ? upload_as<double>(c, s.params[k], &e) : upload_as<float>(c, s.params[k], &e);
            CK(c, e);
        }
    }
    return MEPGL_OK;
}

void fill_desc(mepgl_ctx *c, int si, int img_base, int tile_base)
{
    StringHost &s = c->strings[si];
    StringDesc &D = c->hdesc[si];
    memset(&D, 0, sizeof(D));
    D.nx = s.nx;
    D.ny = s.ny;
    D.F = s.F;
    D.ncomp = c->ncomp;
    D.tiles_x = (s.nx + TX - 1) / TX;
    D.tiles_y = (s.ny + tile_rows(c->precision) - 1) / tile_rows(c->precision);
    D.img_base = img_base;
    D.tile_base = tile_base;
    D.thin_film = c->thin_film;
    D.per_site = s.uniform ? 0 : 1;
    // uniform parameters, formed in double and rounded once per precision
    Uniform<double> &U = D.ud;
    for (int k = 0; k < 2; ++k) {
        const int o = 4 * k;
        U.a[k] = s.params[o][0];
        U.b[k] = s.params[o + 1][0];
        U.hmx[k] = 0.5 / s.params[o + 2][0];
        U.hmy[k] = 0.5 / s.params[o + 3][0];
        U.aob[k] = U.a[k] / U.b[k];
        U.q[k] = s.q[k];
        D.pa[k] = s.dparams[o];
        D.pb[k] = s.dparams[o + 1];
        D.pmxx[k] = s.dparams[o + 2];
        D.pmyy[k] = s.dparams[o + 3];
    }
    U.eta = s.eta;
    U.gamma = s.gamma;
    U.delta = s.delta;
    U.h = s.params[8][0];
    U.idx = 1.0 / s.dx;
    U.dx2 = s.dx * s.dx;
    U.dx = s.dx;
    Uniform<float> &Uf = D.uf;
    for (int k = 0; k < 2; ++k) {
        Uf.a[k] = (float)U.a[k];
        Uf.b[k] = (float)U.b[k];
        Uf.hmx[k] = (float)U.hmx[k];
        Uf.hmy[k] = (float)U.hmy[k];
        Uf.aob[k] = (float)U.aob[k];
        Uf.q[k] = (float)U.q[k];
    }
    Uf.eta = (float)U.eta;
    Uf.gamma = (float)U.gamma;
    Uf.delta = (float)U.delta;
    Uf.h = (float)U.h;
    Uf.idx = (float)U.idx;
    Uf.dx2 = (float)s.dx * (float)s.dx;
    Uf.dx = (float)s.dx;
    Uniform<ff> &Up = D.uff;      // the double values split into float pairs
    for (int k = 0; k < 2; ++k) {
        Up.a[k] = ff(U.a[k]);
        Up.b[k] = ff(U.b[k]);
        Up.hmx[k] = ff(U.hmx[k]);
        Up.hmy[k] = ff(U.hmy[k]);
        Up.aob[k] = ff(U.aob[k]);
        Up.q[k] = ff(U.q[k]);
    }
    Up.eta = ff(U.eta);
    Up.gamma = ff(U.gamma);
    Up.delta = ff(U.delta);
    Up.h = ff(U.h);
    Up.idx = ff(U.idx);
    Up.dx2 = ff(U.dx2);
    Up.dx = ff(U.dx);
    D.disc = c->opt.discretization;
    D.ph = s.dparams[8];
    D.mask = s.dmask;
    for (int b = 0; b < 2; ++b)
        for (int f = 0; f < 3; ++f) {
            D.x[b][f] = s.x[b][f];
            D.g[b][f] = s.g[b][f];
            D.d[b][f] = s.d[b][f];
        }
}

void free_scalars(mepgl_ctx *c)
{
    Scalars &S = c->sc;
    cudaFree(S.gn0); cudaFree(S.gn1); cudaFree(S.gdg); cudaFree(S.beta); cudaFree(S.alpha);
    cudaFree(S.alpha_pend); cudaFree(S.fenergy); cudaFree(S.poly); cudaFree(S.part); cudaFree(S.ticket);
    cudaFree(S.xtab_f); cudaFree(S.xtab_d); cudaFree(S.status);
    memset(&S, 0, sizeof(S));
    cudaFree(c->fqueue); c->fqueue = nullptr;
    cudaFree(c->fstage); c->fstage = nullptr;
    cudaFree(c->dscratch); c->dscratch = nullptr;
    cudaFree(c->ds); cudaFree(c->ds_jb); c->ds = c->ds_jb = nullptr;
    cudaFree(c->dtiles); c->dtiles = nullptr;
}

void drop_graphs(mepgl_ctx *c)
{
    for (auto &kv : c->graphs) cudaGraphExecDestroy(kv.second);
    c->graphs.clear();
}

// (Re)build tile table, descriptors and per-image arrays for the current strings.
mepgl_status build_layout(mepgl_ctx *c)
{
    drop_graphs(c);
    free_scalars(c);
    c->hdesc.assign(c->strings.size(), StringDesc{});
    std::vector<TileRef> tiles;
    int img = 0;
    c->string_tile0.clear();
    c->string_ntiles.clear();
    c->batches.clear();
    c->batch_tile0.clear();
    c->batch_ntiles.clear();
    c->string_batch.clear();
    for (size_t si = 0; si < c->strings.size(); ++si) {
        const int in_batch = (int)(si % MAX_STRINGS);
        if (in_batch == 0) {
            c->batches.emplace_back();
            memset(&c->batches.back(), 0, sizeof(Batch));
            c->batch_tile0.push_back((int)tiles.size());
        }
        fill_desc(c, (int)si, img, (int)tiles.size());
        const StringDesc &D = c->hdesc[si];
        Batch &B = c->batches.back();
        B.s[in_batch] = D;
        B.n = in_batch + 1;
        c->string_batch.push_back((int)c->batches.size() - 1);
        c->string_tile0.push_back((int)tiles.size());
        for (int n = 0; n < D.F; ++n)
            for (int ty = 0; ty < D.tiles_y; ++ty)
                for (int tx = 0; tx < D.tiles_x; ++tx)
                    tiles.push_back(TileRef{(int16_t)in_batch, (int16_t)ty, (int16_t)tx, 0, n});
        c->string_ntiles.push_back((int)tiles.size() - c->string_tile0.back());
        img += D.F;
    }
    for (size_t b = 0; b < c->batches.size(); ++b)
        c->batch_ntiles.push_back((b + 1 < c->batches.size() ? c->batch_tile0[b + 1] : (int)tiles.size()) -
                                  c->batch_tile0[b]);
    c->n_tiles = (int)tiles.size();
    c->total_images = img;
    CK(c, cudaMalloc(&c->dtiles, sizeof(TileRef) * tiles.size()));
    CK(c, cudaMemcpy(c->dtiles, tiles.data(), sizeof(TileRef) * tiles.size(), cudaMemcpyHostToDevice));
    Scalars &S = c->sc;
    const size_t I = (size_t)img;
    for (double **p : {&S.gn0, &S.gn1, &S.gdg, &S.beta, &S.alpha, &S.alpha_pend, &S.fenergy})
        CK(c, cudaMalloc(p, I * sizeof(double)));
    CK(c, cudaMalloc(&S.poly, 4 * I * sizeof(double)));
    CK(c, cudaMalloc(&S.part, (size_t)c->n_tiles * 8 * sizeof(double) + 4096 * sizeof(double)));
    CK(c, cudaMalloc(&S.ticket, I * sizeof(unsigned)));
    CK(c, cudaMemset(S.ticket, 0, I * sizeof(unsigned)));
    CK(c, cudaMalloc(&S.status, 16 * sizeof(int)));
    CK(c, cudaMemset(S.status, 0, 16 * sizeof(int)));
    CK(c, cudaMalloc(&c->fqueue, sizeof(unsigned long long)));
    CK(c, cudaMalloc(&c->fstage, I * sizeof(unsigned)));
    // line-search grid x_p = x_0 * m^p rounded to float / double at every step
    std::vector<double> xf(LS_GRID), xd(LS_GRID);
    float fx = 1e-10f;
    const float fm = 1.025f;
    double dxx = 1e-10;
    const double dm = (double)1.025f;
    for (int p = 0; p < LS_GRID; ++p) {
        xf[p] = fx;
        xd[p] = dxx;
        fx = fx * fm;
        dxx = dxx * dm;
    }
    CK(c, cudaMalloc(&S.xtab_f, LS_GRID * sizeof(double)));
    CK(c, cudaMalloc(&S.xtab_d, LS_GRID * sizeof(double)));
    CK(c, cudaMemcpy(S.xtab_f, xf.data(), LS_GRID * sizeof(double), cudaMemcpyHostToDevice));
    CK(c, cudaMemcpy(S.xtab_d, xd.data(), LS_GRID * sizeof(double), cudaMemcpyHostToDevice));
    CK(c, cudaMalloc(&c->dscratch, (3 * I + 64) * sizeof(double)));
    int fmax = 0;
    for (auto &s : c->strings) fmax = fmax > s.F ? fmax : s.F;
    CK(c, cudaMalloc(&c->ds, (fmax + 1) * sizeof(double)));
    CK(c, cudaMalloc(&c->ds_jb, (fmax + 1) * sizeof(double)));
    CK(c, cudaMemset(c->ds, 0, (fmax + 1) * sizeof(double)));
    CK(c, cudaMemset(c->ds_jb, 0, (fmax + 1) * sizeof(double)));
    c->host_s.assign(fmax, 0.0);
    c->host_sjb.assign(fmax, 0.0);
    return MEPGL_OK;
}

// Restart NLCG history: zero g and d, |g|^2 = inf, nothing pending.
mepgl_status reset_history(mepgl_ctx *c)
{
    for (auto &s : c->strings) {
        const size_t bytes = (size_t)s.F * s.M() * 2 * real_size(c->precision);
        for (int b = 0; b < 2; ++b)
            for (int f = 0; f < 1 + c->ncomp; ++f) {
                CK(c, cudaMemsetAsync(s.g[b][f], 0, bytes, c->stream));
                CK(c, cudaMemsetAsync(s.d[b][f], 0, bytes, c->stream));
            }
    }
    std::vector<double> inf(c->total_images, INF);
    CK(c, cudaMemcpyAsync(c->sc.gn0, inf.data(), inf.size() * 8, cudaMemcpyHostToDevice, c->stream));
    CK(c, cudaMemcpyAsync(c->sc.gn1, inf.data(), inf.size() * 8, cudaMemcpyHostToDevice, c->stream));
    for (double *p : {c->sc.alpha, c->sc.alpha_pend, c->sc.fenergy, c->sc.beta, c->sc.gdg})
        CK(c, cudaMemsetAsync(p, 0, c->total_images * 8, c->stream));
    CK(c, cudaMemsetAsync(c->sc.poly, 0, c->total_images * 32, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    c->pending = false;
    return MEPGL_OK;
}

// Launch covering a whole batch of strings, or (si >= 0) the tiles of one string.
Launch make_launch(mepgl_ctx *c, int batch, int si = -1)
{
    Launch L;
    L.batch = &c->batches[batch];
    const int t0 = si >= 0 ? c->string_tile0[si] : c->batch_tile0[batch];
    L.tiles = c->dtiles + t0;
    L.tile0 = t0;
    L.n_tiles = si >= 0 ? c->string_ntiles[si] : c->batch_ntiles[batch];
    L.grid = L.n_tiles;
    L.precision = c->precision;
    L.paired = c->opt.fp64_arith == MEPGL_FP64_PAIRED ? 1 : 0;
    L.ncomp = c->ncomp;
    L.stream = c->stream;
    return L;
}

Launch string_launch(mepgl_ctx *c, int si) { return make_launch(c, c->string_batch[si], si); }

mepgl_status flush(mepgl_ctx *c)
{
    if (!c->pending) return MEPGL_OK;
    CK(c, launch_apply_update(make_launch(c, 0), c->sc, c->hdesc.data(), (int)c->hdesc.size(), c->xi, c->di));
    c->launches += (int64_t)c->strings.size() * (1 + c->ncomp);
    c->pending = false;
    return MEPGL_OK;
}

StepFlags step_flags(mepgl_ctx *c, int it, int use_cg, int maxwell)
{
    StepFlags f;
    f.gcur = it & 1;
    f.gprev = f.gcur ^ 1;
    f.xin = c->xi;
    f.xout = c->xi ^ 1;
    f.din = c->di;
    f.dout = c->di ^ 1;
    f.use_cg = use_cg;
    f.maxwell = maxwell;
    f.thin_film_any = c->thin_film;
    f.poly_compat = c->opt.line_polynomial == MEPGL_POLY_COMPAT;
    f.ls_exact = c->opt.line_search == MEPGL_LS_EXACT;
    return f;
}

mepgl_status one_step(mepgl_ctx *c, int it, int use_cg, int maxwell)
{
    const StepFlags f = step_flags(c, it, use_cg, maxwell);
    const int nb = (int)c->batches.size();
    for (int b = 0; b < nb; ++b) CK(c, launch_grad(make_launch(c, b), c->sc, f));
    for (int b = 0; b < nb; ++b) CK(c, launch_dir_poly(make_launch(c, b), c->sc, f));
    c->xi ^= 1;
    c->di ^= 1;
    c->launches += (int64_t)nlcg_step_launches() * nb;
    c->pending = true;
    return MEPGL_OK;
}

mepgl_status two_step_graph(mepgl_ctx *c, int use_cg, int maxwell, cudaGraphExec_t *out)
{
    auto key = std::make_tuple(c->xi, c->di, use_cg, maxwell);
    auto it = c->graphs.find(key);
    if (it != c->graphs.end()) {
        *out = it->second;
        return MEPGL_OK;
    }
    const int xi0 = c->xi, di0 = c->di;
    const int64_t l0 = c->launches;
    CK(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    mepgl_status st = one_step(c, 1, use_cg, maxwell);
    if (st == MEPGL_OK) st = one_step(c, 2, use_cg, maxwell);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    c->xi = xi0;
    c->di = di0;
    c->launches = l0;
    if (st != MEPGL_OK) return st;
    CK(c, e);
    cudaGraphExec_t ex = nullptr;
    CK(c, cudaGraphInstantiate(&ex, g, 0));
    cudaGraphDestroy(g);
    c->graphs[key] = ex;
    *out = ex;
    return MEPGL_OK;
}

// Fused FP32 steps pay where a batch is a few waves of the pass kernels
// (the kernel boundaries then idle much of the GPU); on larger batches the
// pass kernels, which hold more warps per SM, are faster.
bool use_fused(const mepgl_ctx *c)
{
    if (!nlcg_fused(c->precision) || c->opt.fp32_steps == MEPGL_FP32_STEPS_PASSES) return false;
    if (c->opt.fp32_steps == MEPGL_FP32_STEPS_FUSED) return true;
    const long long cap = (long long)fuse_waves() * strip_pass_slots(c->ncomp);
    for (int n : c->batch_ntiles)
        if (n > cap) return false;
    return true;
}

// Paired FP64 passes keep the fields x as float-float pairs (x_pairs()):
// the current x of every string changes format before the passes and back
// after them, so that every other kernel and copy sees double.
bool paired_x(const mepgl_ctx *c)
{
    return c->precision == 1 && c->opt.fp64_arith == MEPGL_FP64_PAIRED && x_pairs();
}

mepgl_status x_format(mepgl_ctx *c, int to_pairs)
{
    for (auto &s : c->strings)
        for (int f = 0; f < 1 + c->ncomp; ++f)
            CK(c, launch_x_format(s.x[c->xi][f], (long)s.F * s.M(), to_pairs, c->stream));
    c->launches += (int64_t)c->strings.size() * (1 + c->ncomp);
    return MEPGL_OK;
}

mepgl_status nlcg_steps_body(mepgl_ctx *c, int iters, int use_cg, int maxwell);

// After the steps of a call, one small launch checks every image's energy
// and |g|^2 (the slot the last step wrote) for NaN / infinity; the flags are
// reported by the next synchronising call (check_device_status).
mepgl_status check_scalars(mepgl_ctx *c, int iters)
{
    if (iters <= 0) return MEPGL_OK;
    CK(c, launch_check_scalars(c->sc, c->total_images, iters & 1, c->stream));
    c->launches += 1;
    return MEPGL_OK;
}

mepgl_status nlcg_steps(mepgl_ctx *c, int iters, int use_cg, int maxwell)
{
    if (iters <= 0 || !paired_x(c)) {
        mepgl_status st = nlcg_steps_body(c, iters, use_cg, maxwell);
        return st != MEPGL_OK ? st : check_scalars(c, iters);
    }
    mepgl_status st = x_format(c, 1);
    if (st != MEPGL_OK) return st;
    st = nlcg_steps_body(c, iters, use_cg, maxwell);
    const mepgl_status back = x_format(c, 0);
    if (st == MEPGL_OK) st = back;
    return st != MEPGL_OK ? st : check_scalars(c, iters);
}

mepgl_status nlcg_steps_body(mepgl_ctx *c, int iters, int use_cg, int maxwell)
{
    if (iters > 0 && use_fused(c)) {
        // all steps of a batch in one persistent launch (per-image stages instead of kernel boundaries)
        const StepFlags f0 = step_flags(c, 1, use_cg, maxwell);
        for (size_t b = 0; b < c->batches.size(); ++b)
            CK(c, launch_nlcg_fused(make_launch(c, (int)b), c->sc, f0, 1, iters, c->fqueue, c->fstage,
                                    c->total_images));
        c->xi ^= iters & 1;
        c->di ^= iters & 1;
        c->launches += (int64_t)c->batches.size();
        c->pending = true;
        return MEPGL_OK;
    }
    int it = 1;
    if (c->opt.use_graphs && iters >= 2) {
        cudaGraphExec_t ex;
        mepgl_status st = two_step_graph(c, use_cg, maxwell, &ex);
        if (st != MEPGL_OK) return st;
        for (; it + 1 <= iters; it += 2) {
            CK(c, cudaGraphLaunch(ex, c->stream));
            c->launches += 2 * (int64_t)nlcg_step_launches() * c->batches.size();
        }
        c->pending = true;
    }
    for (; it <= iters; ++it) {
        mepgl_status st = one_step(c, it, use_cg, maxwell);
        if (st != MEPGL_OK) return st;
    }
    return MEPGL_OK;
}

// Device-side error flags (STATUS_* in kernels.cuh): a stage wait of the
// fused NLCG launch that ran out (the launch then stopped early), non-finite
// per-image scalars after NLCG steps, a string of zero or non-finite arc
// length.  Read on the stream after the work before it, then cleared; the
// first raised flag is reported.
mepgl_status check_device_status(mepgl_ctx *c)
{
    int st[4] = {0, 0, 0, 0};
    CK(c, cudaMemcpyAsync(st, c->sc.status, sizeof(st), cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    if (!(st[STATUS_WAIT] | st[STATUS_NONFINITE] | st[STATUS_ARC])) return MEPGL_OK;
    CK(c, cudaMemsetAsync(c->sc.status, 0, sizeof(st), c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    if (st[STATUS_WAIT])
        return fail(c, MEPGL_ERR_CUDA, "fused NLCG launch: a per-image stage wait ran out; the steps are incomplete");
    if (st[STATUS_NONFINITE]) {
        int g = st[STATUS_NONFINITE_IMAGE] - 1, si = 0;
        while (si + 1 < (int)c->hdesc.size() && g >= c->hdesc[si + 1].img_base) ++si;
        return fail(c, MEPGL_ERR_NAN,
                    "non-finite energy or gradient norm after NLCG steps in " + std::to_string(st[STATUS_NONFINITE]) +
                        " image(s), first: string " + std::to_string(si) + " image " +
                        std::to_string(g - c->hdesc[si].img_base));
    }
    return fail(c, MEPGL_ERR_NAN,
                "arc length of the string is zero or not finite (all images equal, or non-finite fields); "
                "it was taken as uniform, so a linear resample kept the images");
}

mepgl_status copy_fields(mepgl_ctx *c, StringHost &s, void *const *dst, const void *const *src, int memory, bool in)
{
    const size_t bytes = (size_t)s.F * s.M() * 2 * real_size(c->precision);
    const cudaMemcpyKind k = memory == MEPGL_DEVICE ? cudaMemcpyDeviceToDevice
                             : in                    ? cudaMemcpyHostToDevice
                                                     : cudaMemcpyDeviceToHost;
    for (int f = 0; f < 1 + c->ncomp; ++f) {
        if (!(in ? src[f] : dst[f])) continue;
        CK(c, cudaMemcpyAsync(dst[f], src[f], bytes, k, c->stream));
    }
    CK(c, cudaStreamSynchronize(c->stream));
    return MEPGL_OK;
}

// Arc length of string si into c->ds (fields) or c->ds_jb (B, J).
mepgl_status arc_length(mepgl_ctx *c, int si, int metric, double **where)
{
    StringHost &s = c->strings[si];
    mepgl_status st = flush(c);
    if (st != MEPGL_OK) return st;
    const void *fl[3];
    int w[3];
    int nf = 1 + c->ncomp;
    if (metric == MEPGL_METRIC_FIELDS) {
        for (int f = 0; f < nf; ++f) { fl[f] = s.x[c->xi][f]; w[f] = 2; }
        *where = c->ds;
    } else {
        // B, J into the spare direction buffer (its contents are not needed)
        void *b[1] = {s.d[c->di ^ 1][0]};
        void *j[1][2] = {{s.d[c->di ^ 1][1], c->ncomp == 2 ? s.d[c->di ^ 1][2] : s.d[c->di ^ 1][1]}};
        CK(c, launch_jb(string_launch(c, si), c->sc, c->xi, b, j));
        c->launches += 1;
        fl[0] = b[0]; w[0] = 1;
        fl[1] = j[0][0]; w[1] = 2;
        fl[2] = j[0][1]; w[2] = 2;
        *where = c->ds_jb;
    }
    CK(c, launch_arc_length(c->precision, fl, w, nf, s.M(), s.F, c->sc.part, *where, c->sc.status + STATUS_ARC,
                            c->stream));
    c->launches += 2;
    return MEPGL_OK;
}

mepgl_status ensure_plan(mepgl_ctx *c, int F, int F_new)
{
    const int need = (F > F_new ? F : F_new) + 2;
    if (need <= c->plan_cap) return MEPGL_OK;
    RedistPlan &p = c->plan;
    cudaFree(p.k); cudaFree(p.w); cudaFree(p.h); cudaFree(p.dl); cudaFree(p.d); cudaFree(p.du); cudaFree(p.du2);
    cudaFree(p.ipiv); cudaFree(p.status); cudaFree(p.aux);
    CK(c, cudaMalloc(&p.aux, redist_aux_size(need) * sizeof(double)));
    CK(c, cudaMalloc(&p.k, need * sizeof(int)));
    CK(c, cudaMalloc(&p.ipiv, need * sizeof(int)));
    CK(c, cudaMalloc(&p.status, 4 * sizeof(int)));
    CK(c, cudaMemset(p.status, 0, 4 * sizeof(int)));
    for (double **q : {&p.w, &p.h, &p.dl, &p.d, &p.du, &p.du2}) CK(c, cudaMalloc(q, need * sizeof(double)));
    c->plan_cap = need;
    return MEPGL_OK;
}

// Reparametrize string si into the spare x buffer.  The caller flips c->xi
// once every string has been written (all strings share the buffer index).
mepgl_status redistribute_into_spare(mepgl_ctx *c, int si, int kind);
mepgl_status ensure_cubic_scratch(mepgl_ctx *c, size_t need);

mepgl_status redistribute(mepgl_ctx *c, int kind, int F_new)
{
    if (c->strings.size() != 1) {
        if (F_new >= 0) return fail(c, MEPGL_ERR_UNSUPPORTED, "resizing a string is for single-string contexts");
        for (size_t si = 0; si < c->strings.size(); ++si) {
            mepgl_status st = redistribute_into_spare(c, (int)si, kind);
            if (st != MEPGL_OK) return st;
        }
        c->xi ^= 1;
        return MEPGL_OK;
    }
    StringHost &s = c->strings[0];
    const int F = s.F;
    if (F_new < 0 || F_new == F) {
        mepgl_status st = redistribute_into_spare(c, 0, kind);
        if (st != MEPGL_OK) return st;
        c->xi ^= 1;
        return MEPGL_OK;
    }
    if (F < 2 || F_new < 2) return fail(c, MEPGL_ERR_INVALID_ARG, "redistribute: need at least 2 images");
    if (kind == MEPGL_REDIST_CUBIC && F < 4)
        return fail(c, MEPGL_ERR_INVALID_ARG, "cubic reparametrization needs at least 4 images");
    double *sp = nullptr;
    mepgl_status st = arc_length(c, 0, MEPGL_METRIC_FIELDS, &sp);
    if (st != MEPGL_OK) return st;
    st = arc_length(c, 0, MEPGL_METRIC_JB, &sp);
    if (st != MEPGL_OK) return st;
    double *s_use = c->opt.metric == MEPGL_METRIC_FIELDS ? c->ds : c->ds_jb;
    st = ensure_plan(c, F, F_new);
    if (st != MEPGL_OK) return st;
    const int cubic = kind == MEPGL_REDIST_CUBIC;
    CK(c, launch_redist_plan(s_use, F, F_new, cubic, c->opt.spline, c->plan, c->stream));
    c->launches += 1;
    void *target[3] = {};
    const size_t rs = real_size(c->precision);
    for (int f = 0; f < 1 + c->ncomp; ++f) CK(c, cudaMalloc(&target[f], (size_t)F_new * s.M() * 2 * rs));
    if (cubic) {
        st = ensure_cubic_scratch(c, redist_cubic_scratch_bytes(c->precision, s.M(), F, F_new));
        if (st != MEPGL_OK) return st;
    }
    for (int f = 0; f < 1 + c->ncomp; ++f) {
        if (cubic)
            CK(c, launch_redist_cubic(c->precision, s.x[c->xi][f], target[f], c->cubic_scratch, s.M(), F, F_new,
                                      c->opt.spline, c->plan, c->stream));
        else
            CK(c, launch_redist_linear(c->precision, s.x[c->xi][f], target[f], s.M(), F_new, c->plan, c->stream));
        c->launches += 1;
    }
    // resize: new buffers for F_new images, state moved in, history reset
    CK(c, cudaStreamSynchronize(c->stream));
    st = check_device_status(c);    // before build_layout renews the flags
    if (st != MEPGL_OK) {
        for (int f = 0; f < 1 + c->ncomp; ++f) cudaFree(target[f]);
        return st;
    }
    free_string_buffers(s);
    s.F = F_new;
    st = alloc_string_buffers(c, s);
    if (st != MEPGL_OK) return st;
    for (int f = 0; f < 1 + c->ncomp; ++f) {
        CK(c, cudaMemcpyAsync(s.x[0][f], target[f], (size_t)F_new * s.M() * 2 * rs, cudaMemcpyDeviceToDevice, c->stream));
        cudaFree(target[f]);
    }
    c->xi = 0;
    c->di = 0;
    st = build_layout(c);
    if (st != MEPGL_OK) return st;
    return reset_history(c);
}

mepgl_status ensure_cubic_scratch(mepgl_ctx *c, size_t need)
{
    if (need <= c->cubic_cap) return MEPGL_OK;
    cudaFree(c->cubic_scratch);
    c->cubic_scratch = nullptr;
    c->cubic_cap = 0;
    CK(c, cudaMalloc(&c->cubic_scratch, need));
    c->cubic_cap = need;
    return MEPGL_OK;
}

mepgl_status redistribute_into_spare(mepgl_ctx *c, int si, int kind)
{
    StringHost &s = c->strings[si];
    const int F = s.F;
    if (F < 2) return fail(c, MEPGL_ERR_INVALID_ARG, "redistribute: need at least 2 images");
    const int cubic = kind == MEPGL_REDIST_CUBIC;
    if (cubic && F < 4) return fail(c, MEPGL_ERR_INVALID_ARG, "cubic reparametrization needs at least 4 images");
    double *sp = nullptr;
    mepgl_status st = arc_length(c, si, MEPGL_METRIC_FIELDS, &sp);
    if (st == MEPGL_OK) st = arc_length(c, si, MEPGL_METRIC_JB, &sp);
    if (st == MEPGL_OK) st = ensure_plan(c, F, F);
    if (st == MEPGL_OK && cubic) st = ensure_cubic_scratch(c, redist_cubic_scratch_bytes(c->precision, s.M(), F, F));
    if (st != MEPGL_OK) return st;
    double *s_use = c->opt.metric == MEPGL_METRIC_FIELDS ? c->ds : c->ds_jb;
    CK(c, launch_redist_plan(s_use, F, F, cubic, c->opt.spline, c->plan, c->stream));
    c->launches += 1;
    for (int f = 0; f < 1 + c->ncomp; ++f) {
        if (cubic)
            CK(c, launch_redist_cubic(c->precision, s.x[c->xi][f], s.x[c->xi ^ 1][f], c->cubic_scratch, s.M(), F, F,
                                      c->opt.spline, c->plan, c->stream));
        else
            CK(c, launch_redist_linear(c->precision, s.x[c->xi][f], s.x[c->xi ^ 1][f], s.M(), F, c->plan,
                                       c->stream));
        c->launches += 1;
    }
    return MEPGL_OK;
}

mepgl_status reset_cg(mepgl_ctx *c, int first, int last)
{
    if (first < 0 || last > c->total_images || first > last)
        return fail(c, MEPGL_ERR_INVALID_ARG, "reset_cg: image range out of bounds");
    if (first == last) return MEPGL_OK;
    std::vector<double> inf(last - first, INF);
    CK(c, cudaMemcpyAsync(c->sc.gn0 + first, inf.data(), inf.size() * 8, cudaMemcpyHostToDevice, c->stream));
    CK(c, cudaMemcpyAsync(c->sc.gn1 + first, inf.data(), inf.size() * 8, cudaMemcpyHostToDevice, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    return MEPGL_OK;
}

}  // namespace

namespace mepgl {
mepgl_status ctx_fail(mepgl_ctx *c, mepgl_status st, const std::string &msg) { return fail(c, st, msg); }
Launch ctx_string_launch(mepgl_ctx *c, int si) { return string_launch(c, si); }
mepgl_status ctx_flush(mepgl_ctx *c) { return flush(c); }
mepgl_status ctx_check_device_status(mepgl_ctx *c) { return check_device_status(c); }
}  // namespace mepgl

// ======================================================================= ABI
extern "C" {

void mepgl_default_options(mepgl_options *o)
{
    if (!o) return;
    o->line_search = MEPGL_LS_COMPAT;
    o->line_polynomial = MEPGL_POLY_COMPAT;
    o->spline = MEPGL_SPLINE_COMPAT;
    o->metric = MEPGL_METRIC_JB;
    o->use_graphs = 1;
    o->tile_rows = 0;
    o->discretization = MEPGL_DISC_REFERENCE;
    o->fp64_arith = MEPGL_FP64_NATIVE;
    o->fp32_steps = MEPGL_FP32_STEPS_AUTO;
}

const char *mepgl_version(void) { return "mepgl_gb300 0.1 (sm_103a)"; }

const char *mepgl_last_error(const mepgl_ctx *c) { return c ? c->err.c_str() : g_create_error.c_str(); }

mepgl_status mepgl_create(const mepgl_problem *p, const mepgl_options *opt, void *stream, mepgl_ctx **out)
{
    return mepgl_create_batch(p, 1, opt, stream, out);
}

mepgl_status mepgl_create_batch(const mepgl_problem *probs, int n_strings, const mepgl_options *opt, void *stream,
                                mepgl_ctx **out)
{
    if (!probs || !out || n_strings < 1) return fail(nullptr, MEPGL_ERR_INVALID_ARG, "mepgl_create: null argument");
    *out = nullptr;
    for (int si = 0; si < n_strings; ++si) {
        const mepgl_problem *p = &probs[si];
        if (p->nx < 2 || p->ny < 2 || p->n_images < 1 || !(p->dx > 0))
            return fail(nullptr, MEPGL_ERR_INVALID_ARG, "mepgl_create: need nx, ny >= 2, n_images >= 1, dx > 0");
        if (p->nx > 32767 * TX || p->ny > 32767 * 8 || (long)p->nx * p->ny >= (1L << 31))
            return fail(nullptr, MEPGL_ERR_INVALID_ARG, "mepgl_create: lattice too large");
        if (p->precision != MEPGL_FP32 && p->precision != MEPGL_FP64)
            return fail(nullptr, MEPGL_ERR_INVALID_ARG, "mepgl_create: precision must be MEPGL_FP32 or MEPGL_FP64");
        const double *arr[9] = {p->a_1, p->b_1, p->m_xx_1, p->m_yy_1, p->a_2, p->b_2, p->m_xx_2, p->m_yy_2, p->h};
        for (int k = 0; k < 9; ++k)
            if (!arr[k] && !(k >= 4 && k < 8 && !p->multicomponent))
                return fail(nullptr, MEPGL_ERR_INVALID_ARG, "mepgl_create: missing parameter array");
        if (!p->comp_domain || !p->sc_domain)
            return fail(nullptr, MEPGL_ERR_INVALID_ARG, "mepgl_create: missing domain");
        if (p->multicomponent != probs[0].multicomponent || p->thin_film != probs[0].thin_film ||
            p->precision != probs[0].precision)
            return fail(nullptr, MEPGL_ERR_UNSUPPORTED,
                        "mepgl_create_batch: all strings need the same component count, thin-film switch and precision");
    }
    if (upload_mask_tables() != cudaSuccess)
        return fail(nullptr, MEPGL_ERR_CUDA, "mepgl_create: cannot upload the neighbour-code tables");
    const mepgl_problem *p = &probs[0];
    mepgl_ctx *c = new mepgl_ctx();
    if (opt) c->opt = *opt;
    else mepgl_default_options(&c->opt);
    if ((c->opt.discretization != MEPGL_DISC_REFERENCE && c->opt.discretization != MEPGL_DISC_LINK) ||
        (c->opt.fp64_arith != MEPGL_FP64_NATIVE && c->opt.fp64_arith != MEPGL_FP64_PAIRED) ||
        c->opt.fp32_steps < MEPGL_FP32_STEPS_AUTO || c->opt.fp32_steps > MEPGL_FP32_STEPS_FUSED) {
        delete c;
        return fail(nullptr, MEPGL_ERR_INVALID_ARG, "mepgl_create: unknown discretization, fp64_arith or fp32_steps");
    }
    c->ncomp = p->multicomponent ? 2 : 1;
    c->thin_film = p->thin_film ? 1 : 0;
    c->precision = p->precision;
    c->stream = (cudaStream_t)stream;
    if (!c->stream) {
        // graph capture is not allowed on the legacy default stream
        if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
            delete c;
            return fail(nullptr, MEPGL_ERR_CUDA, "mepgl_create: cannot create a stream");
        }
        c->own_stream = true;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, dev);
    mepgl_status st = MEPGL_OK;
    for (int si = 0; si < n_strings && st == MEPGL_OK; ++si) {
        const mepgl_problem *q = &probs[si];
        const double *arr[9] = {q->a_1, q->b_1, q->m_xx_1, q->m_yy_1, q->a_2, q->b_2, q->m_xx_2, q->m_yy_2, q->h};
        StringHost s;
        s.nx = q->nx;
        s.ny = q->ny;
        s.F = q->n_images;
        s.dx = q->dx;
        s.q[0] = q->q_1;
        s.q[1] = q->q_2;
        s.eta = q->eta;
        s.gamma = q->gamma;
        s.delta = q->delta;
        const long M = s.M();
        s.uniform = true;
        for (int k = 0; k < 9; ++k) {
            if (arr[k]) s.params[k].assign(arr[k], arr[k] + M);
            else s.params[k].assign(M, 1.0);
            for (long i = 1; i < M && s.uniform; ++i)
                if (s.params[k][i] != s.params[k][0]) s.uniform = false;
        }
        s.comp.assign(q->comp_domain, q->comp_domain + M);
        s.sc.assign(q->sc_domain, q->sc_domain + M);
        c->strings.push_back(std::move(s));
        st = upload_string_params(c, c->strings.back());
        if (st == MEPGL_OK) st = alloc_string_buffers(c, c->strings.back());
    }
    if (st == MEPGL_OK) st = build_layout(c);
    if (st == MEPGL_OK) st = reset_history(c);
    if (st != MEPGL_OK) {
        g_create_error = c->err;
        mepgl_destroy(c);
        return st;
    }
    *out = c;
    return MEPGL_OK;
}

mepgl_status mepgl_destroy(mepgl_ctx *c)
{
    if (!c) return MEPGL_OK;
    cudaStreamSynchronize(c->stream);
    drop_graphs(c);
    for (auto &s : c->strings) {
        free_string_buffers(s);
        free_string_params(s);
    }
    free_scalars(c);
    refine_free(c->refine);
    c->refine = nullptr;
    RedistPlan &p = c->plan;
    cudaFree(p.k); cudaFree(p.w); cudaFree(p.h); cudaFree(p.dl); cudaFree(p.d); cudaFree(p.du); cudaFree(p.du2);
    cudaFree(p.ipiv); cudaFree(p.status); cudaFree(p.aux);
    cudaFree(c->cubic_scratch);
    if (c->copy_stream) {
        cudaStreamSynchronize(c->copy_stream);
        cudaStreamDestroy(c->copy_stream);
    }
    if (c->stage_done) cudaEventDestroy(c->stage_done);
    for (void *b : c->stage) cudaFree(b);
    if (c->own_stream) cudaStreamDestroy(c->stream);
    delete c;
    return MEPGL_OK;
}

mepgl_status mepgl_set_state(mepgl_ctx *c, const void *a, const void *psi_1, const void *psi_2, int memory)
{
    if (c) ++c->state_version;
    if (!c) return MEPGL_ERR_INVALID_ARG;
    if (memory == MEPGL_STAGED) {
        // the staged copy: the context's stream waits for it, then takes it over
        if (!c->staged) return fail(c, MEPGL_ERR_INVALID_ARG, "mepgl_set_state: nothing staged");
        if (c->strings.size() != 1) return fail(c, MEPGL_ERR_UNSUPPORTED, "staged state is for single-string contexts");
        mepgl_status st = flush(c);
        if (st != MEPGL_OK) return st;
        StringHost &s = c->strings[0];
        CK(c, cudaStreamWaitEvent(c->stream, c->stage_done, 0));
        for (int f = 0; f < 1 + c->ncomp; ++f)
            CK(c, cudaMemcpyAsync(s.x[c->xi][f], c->stage[f], c->stage_bytes, cudaMemcpyDeviceToDevice, c->stream));
        c->staged = false;
        return reset_history(c);
    }
    if (!a || !psi_1 || (c->ncomp == 2 && !psi_2))
        return fail(c, MEPGL_ERR_INVALID_ARG, "mepgl_set_state: null field");
    return mepgl_batch_set_state(c, 0, a, psi_1, psi_2, memory);
}

mepgl_status mepgl_stage_state(mepgl_ctx *c, const void *a, const void *psi_1, const void *psi_2, int memory)
{
    if (!c) return MEPGL_ERR_INVALID_ARG;
    if (!a || !psi_1 || (c->ncomp == 2 && !psi_2))
        return fail(c, MEPGL_ERR_INVALID_ARG, "mepgl_stage_state: null field");
    if (memory != MEPGL_HOST && memory != MEPGL_DEVICE)
        return fail(c, MEPGL_ERR_INVALID_ARG, "mepgl_stage_state: memory must be MEPGL_HOST or MEPGL_DEVICE");
    if (c->strings.size() != 1) return fail(c, MEPGL_ERR_UNSUPPORTED, "staged state is for single-string contexts");
    StringHost &s = c->strings[0];
    const size_t bytes = (size_t)s.F * s.M() * 2 * real_size(c->precision);
    if (!c->copy_stream) {
        CK(c, cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
        CK(c, cudaEventCreateWithFlags(&c->stage_done, cudaEventDisableTiming));
    }
    if (c->stage_bytes != bytes) {
        // (re)allocation: nothing of an earlier stage may still be in flight
        CK(c, cudaStreamSynchronize(c->copy_stream));
        for (void *&b : c->stage) {
            cudaFree(b);
            b = nullptr;
        }
        c->stage_bytes = 0;
        for (int f = 0; f < 1 + c->ncomp; ++f) CK(c, cudaMalloc(&c->stage[f], bytes));
        c->stage_bytes = bytes;
    }
    const void *src[3] = {a, psi_1, psi_2};
    const cudaMemcpyKind k = memory == MEPGL_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    for (int f = 0; f < 1 + c->ncomp; ++f) CK(c, cudaMemcpyAsync(c->stage[f], src[f], bytes, k, c->copy_stream));
    CK(c, cudaEventRecord(c->stage_done, c->copy_stream));
    c->staged = true;
    return MEPGL_OK;
}

mepgl_status mepgl_batch_set_state(mepgl_ctx *c, int string, const void *a, const void *psi_1, const void *psi_2,
                                   int memory)
{
    if (c) ++c->state_version;
    if (!c || string < 0 || string >= (int)c->strings.size() || !a || !psi_1 || (c->ncomp == 2 && !psi_2))
        return fail(c, MEPGL_ERR_INVALID_ARG, "mepgl_batch_set_state: bad string index or null field");
    mepgl_status st = flush(c);
    if (st != MEPGL_OK) return st;
    StringHost &s = c->strings[string];
    void *dst[3] = {s.x[c->xi][0], s.x[c->xi][1], s.x[c->xi][2]};
    const void *src[3] = {a, psi_1, psi_2};
    st = copy_fields(c, s, dst, src, memory, true);
    if (st != MEPGL_OK) return st;
    return reset_history(c);
}

mepgl_status mepgl_generate_string(mepgl_ctx *c, const mepgl_guess *g)
{
    if (c) ++c->state_version;
    return mepgl_batch_generate_string(c, 0, g);
}

mepgl_status mepgl_batch_generate_string(mepgl_ctx *c, int string, const mepgl_guess *g)
{
    if (c) ++c->state_version;
    if (!c || !g || string < 0 || string >= (int)c->strings.size() || (g->n_vortices > 0 && !g->vortices) ||
        g->n_vortices < 0 || g->gauge < 0 || g->gauge > 3 || g->profile < 0 || g->profile > 1)
        return fail(c, MEPGL_ERR_INVALID_ARG, "mepgl_generate_string: bad string index or guess");
    mepgl_status st = flush(c);
    if (st != MEPGL_OK) return st;
    StringHost &s = c->strings[string];
    const int F = s.F;
    std::vector<double> tr((size_t)g->n_vortices * F * 4);
    for (int v = 0; v < g->n_vortices; ++v) {
        const mepgl_vortex &V = g->vortices[v];
        if (!V.x || !V.y || !V.winding || V.component < 1 || V.component > c->ncomp)
            return fail(c, MEPGL_ERR_INVALID_ARG, "mepgl_generate_string: incomplete vortex track");
        for (int n = 0; n < F; ++n) {
            double *t = &tr[((size_t)v * F + n) * 4];
            t[0] = V.x[n];
            t[1] = V.y[n];
            t[2] = (double)V.winding[n];
            t[3] = (double)V.component;
        }
    }
    // domains and tracks travel in one temporary device buffer
    const size_t M = (size_t)s.M(), bytes = 2 * M * sizeof(int32_t) + tr.size() * sizeof(double) + 64;
    char *buf = nullptr;
    CK(c, cudaMalloc(&buf, bytes));
    int32_t *dcomp = (int32_t *)buf, *dsc = dcomp + M;
    double *dtr = (double *)(buf + ((2 * M * sizeof(int32_t) + 15) & ~(size_t)15));
    cudaError_t e = cudaMemcpyAsync(dcomp, s.comp.data(), M * sizeof(int32_t), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dsc, s.sc.data(), M * sizeof(int32_t), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess && !tr.empty())
        e = cudaMemcpyAsync(dtr, tr.data(), tr.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream);
    GuessParams p;
    p.x0 = g->x0;
    p.y0 = g->y0;
    p.dx = s.dx;
    p.psi_abs_1 = g->psi_abs_1;
    p.psi_abs_2 = g->psi_abs_2;
    p.noise = g->noise;
    p.b_z = g->b_z;
    p.gauge = g->gauge;
    p.profile = g->profile;
    p.seed = g->seed;
    if (e == cudaSuccess)
        e = launch_generate(c->precision, s.x[c->xi][0], s.x[c->xi][1], s.x[c->xi][2], s.nx, s.ny, F, c->ncomp, dcomp,
                            dsc, dtr, g->n_vortices, p, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(buf);
    CK(c, e);
    c->launches += 1;
    return reset_history(c);
}

mepgl_status mepgl_get_state(mepgl_ctx *c, void *a, void *psi_1, void *psi_2, int memory)
{
    return mepgl_batch_get_state(c, 0, a, psi_1, psi_2, memory);
}

mepgl_status mepgl_batch_get_state(mepgl_ctx *c, int string, void *a, void *psi_1, void *psi_2, int memory)
{
    if (!c || string < 0 || string >= (int)c->strings.size())
        return fail(c, MEPGL_ERR_INVALID_ARG, "mepgl_batch_get_state: bad string index");
    mepgl_status st = flush(c);
    if (st != MEPGL_OK) return st;
    StringHost &s = c->strings[string];
    void *dst[3] = {a, psi_1, psi_2};
    const void *src[3] = {s.x[c->xi][0], s.x[c->xi][1], s.x[c->xi][2]};
    st = copy_fields(c, s, dst, src, memory, false);
    if (st == MEPGL_OK) st = check_device_status(c);
    return st;
}

mepgl_status mepgl_free_energy(mepgl_ctx *c, double *fenergy) { return mepgl_batch_free_energy(c, 0, fenergy); }

mepgl_status mepgl_batch_free_energy(mepgl_ctx *c, int string, double *fenergy)
{
    if (!c || !fenergy || string < 0 || string >= (int)c->strings.size())
        return fail(c, MEPGL_ERR_INVALID_ARG, "mepgl_free_energy: null argument or bad string index");
    mepgl_status st = flush(c);
    if (st != MEPGL_OK) return st;
    CK(c, launch_energy(string_launch(c, string), c->sc, c->xi, c->dscratch));
    c->launches += 1;
    CK(c, cudaMemcpyAsync(fenergy, c->dscratch + c->hdesc[string].img_base, c->strings[string].F * sizeof(double),
                          cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    st = check_device_status(c);
    if (st != MEPGL_OK) return st;
    for (int n = 0; n < c->strings[string].F; ++n)
        if (!std::isfinite(fenergy[n]))
            return fail(c, MEPGL_ERR_NAN, "mepgl_free_energy: non-finite energy of image " + std::to_string(n) +
                                              " (non-finite fields)");
    return MEPGL_OK;
}

mepgl_status mepgl_param_adjoint(mepgl_ctx *c, double *dF_dH, double *dF_deta, double *dF_dgamma)
{
    return mepgl_batch_param_adjoint(c, 0, dF_dH, dF_deta, dF_dgamma);
}

mepgl_status mepgl_batch_param_adjoint(mepgl_ctx *c, int string, double *dF_dH, double *dF_deta, double *dF_dgamma)
{
    if (!c || string < 0 || string >= (int)c->strings.size())
        return fail(c, MEPGL_ERR_INVALID_ARG, "mepgl_param_adjoint: bad string index");
    mepgl_status st = flush(c);
    if (st != MEPGL_OK) return st;
    CK(c, launch_param_adjoint(string_launch(c, string), c->sc, c->xi, c->dscratch));
    c->launches += 1;
    const int F = c->strings[string].F;
    std::vector<double> h(3 * (size_t)F);
    CK(c, cudaMemcpyAsync(h.data(), c->dscratch + 3 * (size_t)c->hdesc[string].img_base, h.size() * sizeof(double),
                          cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    for (int n = 0; n < F; ++n) {
        if (dF_dH) dF_dH[n] = h[3 * n];
        if (dF_deta) dF_deta[n] = h[3 * n + 1];
        if (dF_dgamma) dF_dgamma[n] = h[3 * n + 2];
    }
    return MEPGL_OK;
}

mepgl_status mepgl_batch_info(const mepgl_ctx *c, int string, int *nx, int *ny, int *n_images)
{
    if (!c || string < 0 || string >= (int)c->strings.size()) return MEPGL_ERR_INVALID_ARG;
    if (nx) *nx = c->strings[string].nx;
    if (ny) *ny = c->strings[string].ny;
    if (n_images) *n_images = c->strings[string].F;
    return MEPGL_OK;
}

int mepgl_string_count(const mepgl_ctx *c) { return c ? (int)c->strings.size() : 0; }

mepgl_status mepgl_energy_grad(mepgl_ctx *c, double *fenergy, void *g_a, void *g_psi_1, void *g_psi_2, int memory)
{
    if (!c) return MEPGL_ERR_INVALID_ARG;
    mepgl_status st = flush(c);
    if (st != MEPGL_OK) return st;
    StringHost &s = c->strings[0];
    if (fenergy) {
        st = mepgl_free_energy(c, fenergy);
        if (st != MEPGL_OK) return st;
    }
    if (!g_a && !g_psi_1 && !g_psi_2) return MEPGL_OK;
    const bool direct = memory == MEPGL_DEVICE && g_a && g_psi_1 && (c->ncomp == 1 || g_psi_2);
    FieldPtrs out;
    for (int f = 0; f < 3; ++f) out.p[f] = s.d[c->di ^ 1][f];   // spare direction buffer
    if (direct) {
        out.p[0] = g_a;
        out.p[1] = g_psi_1;
        out.p[2] = c->ncomp == 2 ? g_psi_2 : nullptr;
    }
    Launch L = string_launch(c, 0);
    L.paired = 0;   // the gradient a caller asks for is IEEE double in every FP64 mode
    CK(c, launch_gradient_only(L, c->xi, out, 0));
    c->launches += 1;
    if (direct) {
        CK(c, cudaStreamSynchronize(c->stream));
        return MEPGL_OK;
    }
    void *dst[3] = {g_a, g_psi_1, g_psi_2};
    const void *src[3] = {out.p[0], out.p[1], out.p[2]};
    return copy_fields(c, s, dst, src, memory, false);
}

mepgl_status mepgl_nlcg_steps(mepgl_ctx *c, int iterations, int use_cg, int maxwell_only)
{
    if (c) ++c->state_version;
    if (!c || iterations < 0) return fail(c, MEPGL_ERR_INVALID_ARG, "mepgl_nlcg_steps: bad argument");
    if (c->opt.discretization == MEPGL_DISC_LINK)
        return fail(c, MEPGL_ERR_UNSUPPORTED,
                    "mepgl_nlcg_steps: the link discretisation has no quartic line polynomial; use mepgl_energy_grad");
    return nlcg_steps(c, iterations, use_cg ? 1 : 0, maxwell_only ? 1 : 0);
}

mepgl_status mepgl_reset_cg(mepgl_ctx *c, int first_image, int last_image)
{
    if (!c) return MEPGL_ERR_INVALID_ARG;
    return reset_cg(c, first_image, last_image);
}

mepgl_status mepgl_image_scalars(mepgl_ctx *c, double *fenergy, double *g_norm2, double *alpha)
{
    return mepgl_batch_image_scalars(c, 0, fenergy, g_norm2, alpha);
}

mepgl_status mepgl_batch_image_scalars(mepgl_ctx *c, int string, double *fenergy, double *g_norm2, double *alpha)
{
    if (!c || string < 0 || string >= (int)c->strings.size()) return fail(c, MEPGL_ERR_INVALID_ARG, "bad string");
    const int F = c->strings[string].F, o = c->hdesc[string].img_base;
    if (fenergy) CK(c, cudaMemcpyAsync(fenergy, c->sc.fenergy + o, F * 8, cudaMemcpyDeviceToHost, c->stream));
    // loop()'s g_norm2 is the slot nlcgSteps writes on even substeps
    if (g_norm2) CK(c, cudaMemcpyAsync(g_norm2, c->sc.gn0 + o, F * 8, cudaMemcpyDeviceToHost, c->stream));
    if (alpha) CK(c, cudaMemcpyAsync(alpha, c->sc.alpha + o, F * 8, cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    return check_device_status(c);
}

mepgl_status mepgl_compute_jb(mepgl_ctx *c, void *b, void *j_1, void *j_2, int memory)
{
    if (!c) return MEPGL_ERR_INVALID_ARG;
    mepgl_status st = flush(c);
    if (st != MEPGL_OK) return st;
    StringHost &s = c->strings[0];
    void *bb[1] = {s.d[c->di ^ 1][0]};
    void *jj[1][2] = {{s.d[c->di ^ 1][1], c->ncomp == 2 ? s.d[c->di ^ 1][2] : s.d[c->di ^ 1][1]}};
    CK(c, launch_jb(string_launch(c, 0), c->sc, c->xi, bb, jj));
    c->launches += 1;
    const size_t rs = real_size(c->precision), n = (size_t)s.F * s.M();
    const cudaMemcpyKind k = memory == MEPGL_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (b) CK(c, cudaMemcpyAsync(b, bb[0], n * rs, k, c->stream));
    if (j_1) CK(c, cudaMemcpyAsync(j_1, jj[0][0], 2 * n * rs, k, c->stream));
    if (j_2 && c->ncomp == 2) CK(c, cudaMemcpyAsync(j_2, jj[0][1], 2 * n * rs, k, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    return MEPGL_OK;
}

mepgl_status mepgl_observables(mepgl_ctx *c, int inset, double *flux, double *winding_1, double *winding_2)
{
    return mepgl_batch_observables(c, 0, inset, flux, winding_1, winding_2);
}

mepgl_status mepgl_batch_observables(mepgl_ctx *c, int string, int inset, double *flux, double *winding_1,
                                     double *winding_2)
{
    if (!c || string < 0 || string >= (int)c->strings.size())
        return fail(c, MEPGL_ERR_INVALID_ARG, "mepgl_observables: bad string index");
    StringHost &s = c->strings[string];
    if (inset < 0 || s.nx - 2 * inset < 2 || s.ny - 2 * inset < 2)
        return fail(c, MEPGL_ERR_INVALID_ARG, "mepgl_observables: the winding loop needs nx, ny > 2 inset + 1");
    mepgl_status st = flush(c);
    if (st != MEPGL_OK) return st;
    const int F = s.F;
    double *out = c->dscratch;      // flux, winding 1, winding 2: 3F doubles
    if (flux) {
        void *bb[1] = {s.d[c->di ^ 1][0]};
        void *jj[1][2] = {{s.d[c->di ^ 1][1], c->ncomp == 2 ? s.d[c->di ^ 1][2] : s.d[c->di ^ 1][1]}};
        CK(c, launch_jb(string_launch(c, string), c->sc, c->xi, bb, jj));
        CK(c, launch_flux(c->precision, bb[0], s.M(), F, s.dx * s.dx, out, c->stream));
        c->launches += 2;
    }
    for (int k = 0; k < c->ncomp; ++k) {
        if (!(k == 0 ? winding_1 : winding_2)) continue;
        CK(c, launch_winding(c->precision, s.x[c->xi][1 + k], s.nx, s.ny, F, inset, out + (size_t)(1 + k) * F,
                             c->stream));
        c->launches += 1;
    }
    if (flux) CK(c, cudaMemcpyAsync(flux, out, F * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    if (winding_1) CK(c, cudaMemcpyAsync(winding_1, out + F, F * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    if (winding_2 && c->ncomp == 2)
        CK(c, cudaMemcpyAsync(winding_2, out + 2 * (size_t)F, F * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    return MEPGL_OK;
}

mepgl_status mepgl_arc_length(mepgl_ctx *c, int metric, double *s)
{
    return mepgl_batch_arc_length(c, 0, metric, s);
}

mepgl_status mepgl_batch_arc_length(mepgl_ctx *c, int string, int metric, double *s)
{
    if (!c || !s || string < 0 || string >= (int)c->strings.size())
        return fail(c, MEPGL_ERR_INVALID_ARG, "mepgl_arc_length: null argument or bad string index");
    double *where = nullptr;
    mepgl_status st = arc_length(c, string, metric, &where);
    if (st != MEPGL_OK) return st;
    CK(c, cudaMemcpyAsync(s, where, c->strings[string].F * 8, cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    return check_device_status(c);
}

mepgl_status mepgl_redistribute(mepgl_ctx *c, int kind, int F_new)
{
    if (c) ++c->state_version;
    if (!c) return MEPGL_ERR_INVALID_ARG;
    if (kind != MEPGL_REDIST_LINEAR && kind != MEPGL_REDIST_CUBIC)
        return fail(c, MEPGL_ERR_INVALID_ARG, "mepgl_redistribute: unknown kind");
    mepgl_status st = redistribute(c, kind, F_new);
    if (st != MEPGL_OK) return st;
    CK(c, cudaStreamSynchronize(c->stream));
    st = check_device_status(c);
    if (st != MEPGL_OK) return st;
    int bad = 0;
    CK(c, cudaMemcpy(&bad, c->plan.status, sizeof(int), cudaMemcpyDeviceToHost));
    if (bad) {
        CK(c, cudaMemset(c->plan.status, 0, sizeof(int)));
        return fail(c, MEPGL_ERR_NAN, "spline matrix is singular (coincident images)");
    }
    return MEPGL_OK;
}

mepgl_status mepgl_iteration(mepgl_ctx *c, char mode, int relaxation_steps, int use_cg)
{
    if (!c || relaxation_steps < 0) return fail(c, MEPGL_ERR_INVALID_ARG, "mepgl_iteration: bad argument");
    if (c->opt.discretization == MEPGL_DISC_LINK)
        return fail(c, MEPGL_ERR_UNSUPPORTED, "mepgl_iteration: not available with the link discretisation");
    mepgl_status st = MEPGL_OK;
    switch (mode) {
    case 'S': return mepgl_nlcg_steps(c, relaxation_steps, use_cg, 0);
    case 'M': return mepgl_nlcg_steps(c, relaxation_steps, use_cg, 1);
    case 'L':
    case 'C': {
        // every string is reparametrized, then its interior images restart CG
        st = mepgl_redistribute(c, mode == 'L' ? MEPGL_REDIST_LINEAR : MEPGL_REDIST_CUBIC, -1);
        if (st != MEPGL_OK) return st;
        for (size_t si = 0; si < c->strings.size() && st == MEPGL_OK; ++si) {
            const int F = c->strings[si].F, o = c->hdesc[si].img_base;
            st = reset_cg(c, o + 1, F - 1 > 1 ? o + F - 1 : o + 1);
        }
        if (st != MEPGL_OK) return st;
        return mepgl_nlcg_steps(c, relaxation_steps, use_cg, 0);
    }
    default: return fail(c, MEPGL_ERR_INVALID_ARG, "mepgl_iteration: mode must be S, M, L or C");
    }
}

mepgl_status mepgl_set_precision(mepgl_ctx *c, int precision)
{
    if (c) ++c->state_version;
    if (!c || (precision != MEPGL_FP32 && precision != MEPGL_FP64))
        return fail(c, MEPGL_ERR_INVALID_ARG, "mepgl_set_precision: bad precision");
    if (precision == c->precision) return MEPGL_OK;
    mepgl_status st = flush(c);
    if (st == MEPGL_OK) st = check_device_status(c);   // before build_layout renews the flags
    if (st != MEPGL_OK) return st;
    const int old = c->precision;
    for (auto &s : c->strings) {
        const long n = (long)s.F * s.M() * 2;
        void *tmp[3] = {};
        for (int f = 0; f < 1 + c->ncomp; ++f) {
            CK(c, cudaMalloc(&tmp[f], n * real_size(precision)));
            CK(c, launch_convert(s.x[c->xi][f], old, tmp[f], precision, n, c->stream));
        }
        CK(c, cudaStreamSynchronize(c->stream));
        free_string_buffers(s);
        c->precision = precision;
        st = alloc_string_buffers(c, s);
        c->precision = old;
        if (st != MEPGL_OK) return st;
        for (int f = 0; f < 1 + c->ncomp; ++f) {
            CK(c, cudaMemcpyAsync(s.x[0][f], tmp[f], n * real_size(precision), cudaMemcpyDeviceToDevice, c->stream));
        }
        CK(c, cudaStreamSynchronize(c->stream));
        for (int f = 0; f < 1 + c->ncomp; ++f) cudaFree(tmp[f]);
    }
    c->precision = precision;
    for (auto &s : c->strings) {
        st = upload_string_params(c, s);
        if (st != MEPGL_OK) return st;
    }
    c->xi = 0;
    c->di = 0;
    st = build_layout(c);
    if (st != MEPGL_OK) return st;
    return reset_history(c);
}

mepgl_status mepgl_info(const mepgl_ctx *c, int *n_images, int *precision, int64_t *kernel_launches)
{
    if (!c) return MEPGL_ERR_INVALID_ARG;
    if (n_images) *n_images = c->strings[0].F;
    if (precision) *precision = c->precision;
    if (kernel_launches) *kernel_launches = c->launches;
    return MEPGL_OK;
}

mepgl_status mepgl_pass_kernels(const mepgl_ctx *c, const char **grad, const char **dir_poly, const char **fused)
{
    if (!c || !grad || !dir_poly || !fused) return MEPGL_ERR_INVALID_ARG;
    nlcg_pass_kernels(c->precision, c->opt.fp64_arith == MEPGL_FP64_PAIRED, grad, dir_poly);
    *fused = use_fused(c) ? "k_nlcg_s" : "";
    return MEPGL_OK;
}

mepgl_status mepgl_fused_wait_selftest(mepgl_ctx *c, int *timed_out)
{
    if (!c || !timed_out) return MEPGL_ERR_INVALID_ARG;
    if (!nlcg_fused(c->precision))
        return fail(c, MEPGL_ERR_UNSUPPORTED, "mepgl_fused_wait_selftest: needs an FP32 context and fused steps");
    mepgl_status st = flush(c);
    if (st != MEPGL_OK) return st;
    const Launch L = make_launch(c, 0);
    CK(c, launch_nlcg_fused(L, c->sc, step_flags(c, 1, 1, 0), 1, 1, c->fqueue, c->fstage, c->total_images,
                            (unsigned long long)L.n_tiles, 4096u));
    c->launches += 1;
    int flag = 0;
    CK(c, cudaMemcpyAsync(&flag, c->sc.status, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    if (flag) CK(c, cudaMemsetAsync(c->sc.status, 0, sizeof(int), c->stream));
    *timed_out = flag ? 1 : 0;
    return MEPGL_OK;
}

mepgl_status mepgl_profile_passes(mepgl_ctx *c, int steps, int use_cg, double *ms_grad, double *ms_dir_poly)
{
    if (c && c->opt.discretization == MEPGL_DISC_LINK)
        return fail(c, MEPGL_ERR_UNSUPPORTED, "mepgl_profile_passes: not available with the link discretisation");
    if (!c || steps < 1) return fail(c, MEPGL_ERR_INVALID_ARG, "mepgl_profile_passes: steps must be >= 1");
    std::vector<cudaEvent_t> ev(2 * steps + 1);
    for (auto &e : ev) CK(c, cudaEventCreate(&e));
    const int nb = (int)c->batches.size();
    const bool px = paired_x(c);
    if (px) {
        mepgl_status st = x_format(c, 1);
        if (st != MEPGL_OK) return st;
    }
    CK(c, cudaEventRecord(ev[0], c->stream));
    for (int it = 1; it <= steps; ++it) {
        const StepFlags f = step_flags(c, it, use_cg ? 1 : 0, 0);
        for (int b = 0; b < nb; ++b) CK(c, launch_grad(make_launch(c, b), c->sc, f));
        CK(c, cudaEventRecord(ev[2 * it - 1], c->stream));
        for (int b = 0; b < nb; ++b) CK(c, launch_dir_poly(make_launch(c, b), c->sc, f));
        CK(c, cudaEventRecord(ev[2 * it], c->stream));
        c->xi ^= 1;
        c->di ^= 1;
        c->launches += (int64_t)nlcg_step_launches() * nb;
        c->pending = true;
    }
    if (px) {
        mepgl_status st = x_format(c, 0);
        if (st != MEPGL_OK) return st;
    }
    CK(c, cudaEventSynchronize(ev[2 * steps]));
    double tg = 0, td = 0;
    for (int it = 1; it <= steps; ++it) {
        float a = 0, b = 0;
        CK(c, cudaEventElapsedTime(&a, ev[2 * it - 2], ev[2 * it - 1]));
        CK(c, cudaEventElapsedTime(&b, ev[2 * it - 1], ev[2 * it]));
        tg += a;
        td += b;
    }
    for (auto &e : ev) cudaEventDestroy(e);
    if (ms_grad) *ms_grad = tg / steps;
    if (ms_dir_poly) *ms_dir_poly = td / steps;
    return MEPGL_OK;
}

mepgl_status mepgl_synchronize(mepgl_ctx *c)
{
    if (!c) return MEPGL_ERR_INVALID_ARG;
    CK(c, cudaStreamSynchronize(c->stream));
    return check_device_status(c);
}

}  // extern "C"
