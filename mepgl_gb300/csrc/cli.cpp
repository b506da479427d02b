// cli.cpp -- the `mepgl` executable: drop-in for the reference binary
// (mepgl/src/mepgl.cu:421-881) on top of libmepgl_gb300.
//
//   mepgl --simname S --mode {S,M,L,C} --Fin F --Fout F_out --iterations K
//         [--precision fp32|fp64|mixed] [--relaxation-steps n]
//         [--line-polynomial compat|exact] [--line-search compat|exact]
//         [--spline compat|fmm] [--polish-iterations P]
//
// Reads ./simulations/S/input_data/ and writes ./simulations/S/output_data/
// with the reference's file names and .npy layout (io.cu:10-291), prints the
// same per-iteration table and rewrites ./energy.csv after every iteration
// (mepgl.cu:311-355).  Keys on stdin while running (mepgl.cu:635-673):
// q = stop and save, + / - = relaxation steps, C = toggle conjugate gradients.
//
// Compile-time settings of the reference (N, dx, MULTICOMPONENT,
// NO_SELF_FIELD, DOUBLE_PRECISION, default relaxation steps) are read at run
// time from input_data/mepgl.cfg (written by the launcher; `key = value`
// lines), falling back to the inputs themselves: N from the arrays, dx from
// x.npy, two components when 0/u_2.npy exists.
#include <poll.h>
#include <sys/stat.h>
#include <unistd.h>

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "mepgl.h"
#include "npy.h"

namespace {

struct Args {
    std::string simname;
    char mode = 'S';
    int F = -1, F_out = -1, iterations = 1;
    std::map<std::string, std::string> opt;
};

void usage()
{
    std::printf("Options:\n"
                "  --simname arg     Simulation name\n"
                "  --mode arg        Mode selected (M, S, L, C)\n"
                "  --Fin arg         Number of frames of the input guess\n"
                "  --Fout arg        Number of frames of the output\n"
                "  --iterations arg  Number of iterations\n"
                "  --precision arg   fp32 | fp64 | mixed (FP32, then FP64 for the last iterations)\n"
                "  --relaxation-steps n, --polish-iterations n\n"
                "  --line-polynomial compat|exact, --line-search compat|exact, --spline compat|fmm\n"
                "  --fp64-arith native|paired (FP64 NLCG passes in float-float pairs)\n");
}

Args parse(int argc, char **argv)
{
    Args a;
    for (int i = 1; i < argc; ++i) {
        std::string k = argv[i], v;
        if (k == "--help" || k == "-h") { usage(); std::exit(0); }
        if (k.rfind("--", 0) != 0) throw std::runtime_error("unexpected argument " + k);
        const size_t eq = k.find('=');
        if (eq != std::string::npos) { v = k.substr(eq + 1); k = k.substr(0, eq); }
        else if (i + 1 < argc) v = argv[++i];
        else throw std::runtime_error("missing value for " + k);
        k = k.substr(2);
        if (k != "Fin" && k != "Fout")
            for (char &ch : k)
                if (ch == '-') ch = '_';   // --relaxation-steps == relaxation_steps in mepgl.cfg
        if (k == "simname") a.simname = v;
        else if (k == "mode") a.mode = v.empty() ? 'S' : v[0];
        else if (k == "Fin") a.F = std::stoi(v);
        else if (k == "Fout") a.F_out = std::stoi(v);
        else if (k == "iterations") a.iterations = std::stoi(v);
        else a.opt[k] = v;
    }
    if (a.simname.empty()) throw std::runtime_error("--simname is required");
    return a;
}

std::map<std::string, std::string> read_cfg(const std::string &path)
{
    std::map<std::string, std::string> m;
    std::ifstream f(path);
    std::string line;
    while (std::getline(f, line)) {
        const size_t h = line.find('#');
        if (h != std::string::npos) line = line.substr(0, h);
        const size_t eq = line.find('=');
        if (eq == std::string::npos) continue;
        auto trim = [](std::string s) {
            const size_t b = s.find_first_not_of(" \t"), e = s.find_last_not_of(" \t\r");
            return b == std::string::npos ? std::string() : s.substr(b, e - b + 1);
        };
        m[trim(line.substr(0, eq))] = trim(line.substr(eq + 1));
    }
    return m;
}

bool exists(const std::string &p)
{
    struct stat st;
    return stat(p.c_str(), &st) == 0;
}

void mkdirs(const std::string &p)
{
    std::string cur;
    for (size_t i = 0; i < p.size(); ++i) {
        cur.push_back(p[i]);
        if (p[i] == '/' || i + 1 == p.size()) mkdir(cur.c_str(), 0755);
    }
}

// numpy [i][j] (axis 0 = x) <-> library i + nx*j
std::vector<double> to_lib(const std::vector<double> &a, size_t nx, size_t ny)
{
    std::vector<double> o(nx * ny);
    for (size_t i = 0; i < nx; ++i)
        for (size_t j = 0; j < ny; ++j) o[i + nx * j] = a[j + ny * i];
    return o;
}

template <class T>
std::vector<T> to_npy(const T *a, size_t nx, size_t ny, size_t stride = 1, size_t off = 0)
{
    std::vector<T> o(nx * ny);
    for (size_t i = 0; i < nx; ++i)
        for (size_t j = 0; j < ny; ++j) o[j + ny * i] = a[(i + nx * j) * stride + off];
    return o;
}

// A failure with the library status it maps to; the process exits with
// that status (3 = MEPGL_ERR_NAN for non-finite data, 1 for anything that
// is not a library status).
struct StatusError : std::runtime_error {
    int status;
    StatusError(int st, const std::string &m) : std::runtime_error(m), status(st) {}
};

std::vector<double> load2d(const std::string &p, size_t &nx, size_t &ny)
{
    npy::Array a = npy::read(p);
    if (a.shape.size() != 2) throw std::runtime_error(p + ": expected a 2-D array");
    if (nx == 0) { nx = a.shape[0]; ny = a.shape[1]; }
    if (a.shape[0] != nx || a.shape[1] != ny) throw std::runtime_error(p + ": shape mismatch");
    std::vector<double> v = npy::as_double(a);
    // the reference reads inputs unchecked (mepgl/src/io.cu:18-125); a NaN or
    // infinity in any input would only show as non-finite energies later
    for (size_t k = 0; k < v.size(); ++k)
        if (!std::isfinite(v[k]))
            throw StatusError(MEPGL_ERR_NAN, p + ": non-finite value at flat index " + std::to_string(k));
    return to_lib(v, nx, ny);
}

void check(mepgl_status st, mepgl_ctx *ctx, const char *what)
{
    if (st != MEPGL_OK) throw StatusError(st, std::string(what) + ": " + mepgl_last_error(ctx));
}

template <class T>
void save_fields(const std::string &out, mepgl_ctx *ctx, int F, size_t nx, size_t ny, int nc)
{
    const size_t M = nx * ny, n2 = 2 * M * F;
    std::vector<T> a(n2), p1(n2), p2(nc == 2 ? n2 : 2), b(M * F), j1(n2), j2(nc == 2 ? n2 : 2);
    check(mepgl_get_state(ctx, a.data(), p1.data(), nc == 2 ? p2.data() : nullptr, MEPGL_HOST), ctx, "get_state");
    check(mepgl_compute_jb(ctx, b.data(), j1.data(), nc == 2 ? j2.data() : nullptr, MEPGL_HOST), ctx, "compute_jb");
    const std::vector<size_t> sh = {nx, ny};
    for (int n = 0; n < F; ++n) {
        const std::string d = out + std::to_string(n) + "/";
        mkdirs(d);
        const size_t o2 = 2 * M * n, o1 = M * n;
        npy::write(d + "u_1.npy", to_npy(p1.data() + o2, nx, ny, 2, 0).data(), sh);
        npy::write(d + "v_1.npy", to_npy(p1.data() + o2, nx, ny, 2, 1).data(), sh);
        npy::write(d + "ax.npy", to_npy(a.data() + o2, nx, ny, 2, 0).data(), sh);
        npy::write(d + "ay.npy", to_npy(a.data() + o2, nx, ny, 2, 1).data(), sh);
        if (nc == 2) {
            npy::write(d + "u_2.npy", to_npy(p2.data() + o2, nx, ny, 2, 0).data(), sh);
            npy::write(d + "v_2.npy", to_npy(p2.data() + o2, nx, ny, 2, 1).data(), sh);
        }
        npy::write(d + "jx_1.npy", to_npy(j1.data() + o2, nx, ny, 2, 0).data(), sh);
        npy::write(d + "jy_1.npy", to_npy(j1.data() + o2, nx, ny, 2, 1).data(), sh);
        npy::write(d + "b.npy", to_npy(b.data() + o1, nx, ny).data(), sh);
        if (nc == 2) {
            npy::write(d + "jx_2.npy", to_npy(j2.data() + o2, nx, ny, 2, 0).data(), sh);
            npy::write(d + "jy_2.npy", to_npy(j2.data() + o2, nx, ny, 2, 1).data(), sh);
        }
    }
}

template <class T>
void save_scalar_arrays(const std::string &out, const std::vector<double> &v, const char *name)
{
    std::vector<T> t(v.begin(), v.end());
    npy::write(out + name, t.data(), {t.size()});
}

int run(const Args &A)
{
    std::setvbuf(stdout, nullptr, _IONBF, 0);
    const std::string in = "./simulations/" + A.simname + "/input_data/";
    const std::string out = "./simulations/" + A.simname + "/output_data/";
    std::map<std::string, std::string> cfg = read_cfg("./mepgl.cfg");
    for (auto &kv : read_cfg(in + "mepgl.cfg")) cfg[kv.first] = kv.second;
    for (auto &kv : A.opt) cfg[kv.first] = kv.second;
    auto opt = [&](const std::string &k, const std::string &d) { return cfg.count(k) ? cfg[k] : d; };

    size_t nx = 0, ny = 0;
    std::vector<double> x = load2d(in + "x.npy", nx, ny), y = load2d(in + "y.npy", nx, ny);
    double dx = cfg.count("dx") ? std::stod(cfg["dx"]) : 0.0;
    if (!(dx > 0)) dx = x[1] - x[0];   // x varies along the lattice's first axis
    const std::string pnames[9] = {"a_1", "b_1", "m_xx_1", "m_yy_1", "a_2", "b_2", "m_xx_2", "m_yy_2", "h"};
    std::vector<double> par[9];
    for (int k = 0; k < 9; ++k) par[k] = load2d(in + pnames[k] + ".npy", nx, ny);
    std::vector<double> cdom = load2d(in + "comp_domain.npy", nx, ny), sdom = load2d(in + "sc_domain.npy", nx, ny);
    std::vector<int32_t> comp(cdom.begin(), cdom.end()), sc(sdom.begin(), sdom.end());
    const std::vector<double> q = npy::as_double(npy::read(in + "q.npy"));
    if (q.size() < 5) throw std::runtime_error("q.npy must hold q_1, q_2, eta, gamma, delta");
    for (size_t k = 0; k < 5; ++k)
        if (!std::isfinite(q[k])) throw StatusError(MEPGL_ERR_NAN, in + "q.npy: non-finite coupling");
    const bool mc = cfg.count("multicomponent") ? std::stoi(cfg["multicomponent"]) != 0 : exists(in + "0/u_2.npy");
    const int nc = mc ? 2 : 1;
    int F = A.F;
    if (F < 1) {
        F = 0;
        while (exists(in + std::to_string(F) + "/u_1.npy")) ++F;
    }
    if (F < 1) throw StatusError(MEPGL_ERR_INVALID_ARG, in + ": no images (0/u_1.npy missing)");
    // the arc-length resample needs two images, the cubic spline four
    // (mepgl/src/interpolation.cu:252-322); the reference would index past its arrays
    if ((A.mode == 'L' && F < 2) || (A.mode == 'C' && F < 4))
        throw StatusError(MEPGL_ERR_INVALID_ARG, std::string("mode ") + A.mode + " needs at least " +
                                                     (A.mode == 'C' ? "4" : "2") + " images, got " + std::to_string(F));
    const int F_out = A.F_out < 1 ? F : A.F_out;
    const std::string prec = opt("precision", opt("double_precision", "0") == "1" ? "fp64" : "fp32");
    const bool mixed = prec == "mixed";
    const int precision = prec == "fp64" ? MEPGL_FP64 : MEPGL_FP32;
    std::atomic<int> relax(std::stoi(opt("relaxation_steps", "10")));
    const int polish = std::stoi(opt("polish_iterations", std::to_string(std::max(1, A.iterations / 10))));

    // fields: numpy [i][j] per image -> library pairs
    const size_t M = nx * ny;
    std::vector<double> fa(2 * M * F), f1(2 * M * F), f2(2 * M * F, 0.0);
    for (int n = 0; n < F; ++n) {
        const std::string d = in + std::to_string(n) + "/";
        const char *names[6] = {"ax.npy", "ay.npy", "u_1.npy", "v_1.npy", "u_2.npy", "v_2.npy"};
        std::vector<double> *dst[3] = {&fa, &f1, &f2};
        for (int k = 0; k < 2 + 2 * nc; ++k) {
            std::vector<double> v = load2d(d + names[k], nx, ny);
            std::vector<double> &t = *dst[k / 2];
            for (size_t s = 0; s < M; ++s) t[2 * (M * n + s) + (k % 2)] = v[s];
        }
    }

    mepgl_problem P{};
    P.nx = (int)nx;
    P.ny = (int)ny;
    P.n_images = F;
    P.multicomponent = mc ? 1 : 0;
    P.thin_film = std::stoi(opt("thin_film", "0"));
    P.precision = precision;
    P.dx = dx;
    P.q_1 = q[0]; P.q_2 = q[1]; P.eta = q[2]; P.gamma = q[3]; P.delta = q[4];
    P.a_1 = par[0].data(); P.b_1 = par[1].data(); P.m_xx_1 = par[2].data(); P.m_yy_1 = par[3].data();
    P.a_2 = par[4].data(); P.b_2 = par[5].data(); P.m_xx_2 = par[6].data(); P.m_yy_2 = par[7].data();
    P.h = par[8].data();
    P.comp_domain = comp.data();
    P.sc_domain = sc.data();
    mepgl_options O;
    mepgl_default_options(&O);
    O.line_polynomial = opt("line_polynomial", "compat") == "exact" ? MEPGL_POLY_EXACT : MEPGL_POLY_COMPAT;
    O.line_search = opt("line_search", "compat") == "exact" ? MEPGL_LS_EXACT : MEPGL_LS_COMPAT;
    O.spline = opt("spline", "compat") == "fmm" ? MEPGL_SPLINE_FMM : MEPGL_SPLINE_COMPAT;
    O.fp64_arith = opt("fp64_arith", "native") == "paired" ? MEPGL_FP64_PAIRED : MEPGL_FP64_NATIVE;

    std::printf("%s\n\nSimulation name: %s\n", mepgl_version(), A.simname.c_str());
    std::printf("Lattice %zu x %zu, dx = %g, %d images, %d component(s), precision %s\n", nx, ny, dx, F, nc,
                prec.c_str());
    if (O.line_polynomial == MEPGL_POLY_COMPAT && (q[0] != -1.0 || (mc && q[1] != -1.0)))
        std::printf("note: the reference's line polynomial is exact only for charges -1; "
                    "consider --line-polynomial exact\n");
    mepgl_ctx *ctx = nullptr;
    if (mepgl_create(&P, &O, nullptr, &ctx) != MEPGL_OK) throw std::runtime_error(mepgl_last_error(nullptr));
    // the context precision decides the host type of the state
    auto set_state = [&](int p) {
        if (p == MEPGL_FP64) {
            check(mepgl_set_state(ctx, fa.data(), f1.data(), mc ? f2.data() : nullptr, MEPGL_HOST), ctx, "set_state");
        } else {
            std::vector<float> a(fa.begin(), fa.end()), b(f1.begin(), f1.end()), c(f2.begin(), f2.end());
            check(mepgl_set_state(ctx, a.data(), b.data(), mc ? c.data() : nullptr, MEPGL_HOST), ctx, "set_state");
        }
    };
    set_state(precision);

    std::vector<double> fe(F), fe_old(F, INFINITY), gn(F), al(F), s(F), sjb(F);
    check(mepgl_free_energy(ctx, fe.data()), ctx, "free_energy");
    const int stride = std::max((F - 1) / 10, 1);
    std::printf("┌──────┬────────────────┐ \n| Sys# |  Free Energy   | \n├──────┼────────────────┤ \n");
    for (int n = 0; n < F; n += stride) std::printf("|  %3.3d | %.8e | \n", n, fe[n]);
    std::printf("└──────┴────────────────┘ \nStarting MEP-MGL.\n\n");

    std::atomic<bool> stop(false), nlcg(true), done(false);
    std::thread keys([&] {
        char buf[8];
        while (!done.load()) {
            pollfd p{0, POLLIN, 0};
            if (poll(&p, 1, 200) <= 0) continue;
            const ssize_t r = read(0, buf, sizeof(buf));
            if (r <= 0) break;    // EOF: no controller attached
            for (ssize_t i = 0; i < r; ++i) {
                if (buf[i] == 'q') { std::printf("I am quitting! Please wait.\n"); stop = true; }
                else if (buf[i] == '+') std::printf("relaxation_steps = %d\n", ++relax);
                else if (buf[i] == '-') { if (relax > 1) --relax; std::printf("relaxation_steps = %d\n", relax.load()); }
                else if (buf[i] == 'C') { nlcg = !nlcg; std::printf("NLCG set %s\n", nlcg ? "ON" : "OFF"); }
            }
        }
    });

    int status = 0;
    int cur_prec = precision;
    for (int it = 0; it < A.iterations && !stop; ++it) {
        if (mixed && cur_prec == MEPGL_FP32 && it >= A.iterations - polish) {
            check(mepgl_set_precision(ctx, MEPGL_FP64), ctx, "set_precision");
            cur_prec = MEPGL_FP64;
            std::printf("=> switching to FP64 for the last %d iterations\n", A.iterations - it);
        }
        std::printf("\nIteration:   %d\n", it + 1);
        check(mepgl_iteration(ctx, A.mode, relax.load(), nlcg.load() ? 1 : 0), ctx, "iteration");
        check(mepgl_image_scalars(ctx, fe.data(), gn.data(), al.data()), ctx, "image_scalars");
        if (A.mode == 'L' || A.mode == 'C') check(mepgl_arc_length(ctx, MEPGL_METRIC_JB, sjb.data()), ctx, "arc");
        double gmean = 0;
        for (int n = 0; n < F; ++n) gmean += std::sqrt(gn[n]);
        gmean /= (double)F * M;
        std::printf("┌──────┬──────┬─────────────────┬─────────────────┬────────────────┬────────────────┐\n"
                    "│ Sys# │   s  │  Free Energy    │  Delta Energy   │      ||g||     │      alpha     │\n"
                    "├──────┼──────┼─────────────────┼─────────────────┼────────────────┼────────────────┤\n");
        for (int n = 0; n < F; n += stride)
            std::printf("│  %3.3d │ %4.2f │ %+.8e │ %+.8e │ %.8e │ %.8e │\n", n, sjb[n], fe[n], fe[n] - fe_old[n],
                        std::sqrt(gn[n]) / M, al[n]);
        std::printf("└──────┴──────┴─────────────────┴─────────────────┴────────────────┴────────────────┘\n\n"
                    "||g||_mean      %e       \n\n", gmean);
        fe_old = fe;
        std::ofstream csv("energy.csv");
        csv << std::scientific;
        for (int n = 0; n < F; ++n) csv << fe[n] << (n + 1 < F ? "," : "");
        bool bad = false;
        for (int n = 0; n < F; ++n) bad |= !std::isfinite(fe[n]);
        if (bad) {
            std::printf("error: non-finite energy, stopping\n");
            status = 3;
            break;
        }
    }
    done = true;
    keys.join();

    int Fo = F;
    if (F_out != F) {
        check(mepgl_redistribute(ctx, MEPGL_REDIST_LINEAR, F_out), ctx, "redistribute");
        Fo = F_out;
    }
    std::vector<double> fo(Fo), so(Fo), sjbo(Fo);
    check(mepgl_free_energy(ctx, fo.data()), ctx, "free_energy");
    check(mepgl_arc_length(ctx, MEPGL_METRIC_FIELDS, so.data()), ctx, "arc_length");
    check(mepgl_arc_length(ctx, MEPGL_METRIC_JB, sjbo.data()), ctx, "arc_length_jb");
    const int stride_o = std::max((Fo - 1) / 10, 1);
    std::printf("┌──────┬────────────────┐ \n| Sys# |  Free Energy   | \n├──────┼────────────────┤ \n");
    for (int n = 0; n < Fo; n += stride_o) std::printf("|  %3.3d | %.8e | \n", n, fo[n]);
    std::printf("└──────┴────────────────┘ \n");

    std::printf("Saving results...  ");
    mkdirs(out);
    int final_prec = MEPGL_FP64;
    mepgl_info(ctx, nullptr, &final_prec, nullptr);
    const std::vector<size_t> sh = {nx, ny};
    auto save_lattice = [&](auto tag) {
        using T = decltype(tag);
        save_scalar_arrays<T>(out, fo, "fenergy.npy");
        save_scalar_arrays<T>(out, so, "s.npy");
        save_scalar_arrays<T>(out, sjbo, "s_jb.npy");
        save_scalar_arrays<T>(out, q, "q.npy");
        npy::write(out + "x.npy", to_npy<T>(std::vector<T>(x.begin(), x.end()).data(), nx, ny).data(), sh);
        npy::write(out + "y.npy", to_npy<T>(std::vector<T>(y.begin(), y.end()).data(), nx, ny).data(), sh);
        for (int k = 0; k < 9; ++k)
            npy::write(out + pnames[k] + ".npy",
                       to_npy<T>(std::vector<T>(par[k].begin(), par[k].end()).data(), nx, ny).data(), sh);
        save_fields<T>(out, ctx, Fo, nx, ny, nc);
    };
    npy::write(out + "comp_domain.npy", to_npy(comp.data(), nx, ny).data(), sh);
    npy::write(out + "sc_domain.npy", to_npy(sc.data(), nx, ny).data(), sh);
    if (final_prec == MEPGL_FP64) save_lattice(double());
    else save_lattice(float());
    {
        // settings travel with the data, so a reload (output -> input) keeps them
        std::map<std::string, std::string> eff = cfg;
        char buf[64];
        std::snprintf(buf, sizeof(buf), "%.17g", dx);
        eff["dx"] = buf;
        eff["multicomponent"] = mc ? "1" : "0";
        eff["thin_film"] = std::to_string(P.thin_film);
        eff["relaxation_steps"] = std::to_string(relax.load());
        std::ofstream f(out + "mepgl.cfg");
        f << "# runtime settings of the mepgl executable\n";
        for (auto &kv : eff) f << kv.first << " = " << kv.second << "\n";
    }
    std::printf("done.\nFinished\n");
    mepgl_destroy(ctx);
    return status;
}

}  // namespace

int main(int argc, char **argv)
{
    try {
        return run(parse(argc, argv));
    } catch (const StatusError &e) {
        std::fprintf(stderr, "mepgl: %s\n", e.what());
        return e.status;
    } catch (const std::exception &e) {
        std::fprintf(stderr, "mepgl: %s\n", e.what());
        return 1;
    }
}
