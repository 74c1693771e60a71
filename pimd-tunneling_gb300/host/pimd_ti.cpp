// pimd_ti.cpp -- C++ front end of the TI-PIMD path: the pimd_par.f90 flow
// (namelist &MCDATA on standard input, masses.dat / well1.dat / well2.dat /
// path.xyz in the working directory) on one GPU through the C-ABI.  The MPI
// distribution of (lambda point x replica) tasks (pimd_par.f90:243-308, 389)
// becomes one batch of rings on the device and a device-side reduction.
//
// Keys beyond the reference's namelist: pes ('1d', '2dtest', 'synth9',
// 'synth18', 'harmonic'), pes_params (file with one number per line),
// precision ('mixed' | 'fp64'), form ('auto' | 'plain' | 'fused' | 'tensor'),
// seed (RNG key base; replica j uses seed + j, lambda point i uses stream i),
// init ('path': beads on the path as init_path does, verletmodule.f90:40-48;
// 'well': every bead at well 1), init_sigma (Gaussian noise on the start
// positions), chunk (steps per device launch sequence).
// restart = 1 writes restart.ckpt after the run, restart = 2 continues from it
// (a bitwise checkpoint of the device state; replaces restart_proc*.xyz).
#include <chrono>
#include <cmath>
#include <cstdio>
#include <iostream>
#include <string>
#include <vector>

#include "../../include/pimdgpu.h"
#include "namelist.hpp"

using namespace pgdrv;

static int pes_id_of(const std::string &s) {
    std::string p = lower(s);
    if (p == "1d") return PG_PES_1D;
    if (p == "2dtest") return PG_PES_2DTEST;
    if (p == "synth9") return PG_PES_SYNTH9;
    if (p == "synth18") return PG_PES_SYNTH18;
    if (p == "harmonic") return PG_PES_HARMONIC;
    throw std::runtime_error("unknown pes '" + s + "'");
}

static std::vector<double> read_numbers(const std::string &path) {
    std::vector<double> v;
    if (path.empty()) return v;
    std::ifstream f(path);
    if (!f) throw std::runtime_error("cannot open " + path);
    double x;
    while (f >> x) v.push_back(x);
    return v;
}

#define CHECK(call)                                                                    \
    do {                                                                               \
        int _rc = (call);                                                              \
        if (_rc != PG_OK) {                                                            \
            std::fprintf(stderr, "pimdgpu error %d in %s: %s\n", _rc, #call, pg_last_error()); \
            return 2;                                                                  \
        }                                                                              \
    } while (0)

int main(int argc, char **argv) {
    bool parse_only = argc > 1 && std::string(argv[1]) == "--parse-only";
    Namelist nl;
    try {
        nl = Namelist::parse(read_all(std::cin), "MCDATA");
    } catch (std::exception &e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    // defaults: pimd_par.f90:60-88
    const int64_t n = nl.integer("n", 100);
    const double beta = nl.real("beta", 100.0);
    const int64_t NMC = nl.integer("NMC", 5000000);
    const int64_t Noutput = nl.integer("Noutput", 100000);
    const double dt = nl.real("dt", 1.0e-3);
    const int64_t nintegral = nl.integer("nintegral", 5);
    const int64_t nrep = nl.integer("nrep", 1);
    const int thermostat = (int)nl.integer("thermostat", 1);
    const int ndim = (int)nl.integer("ndim", 3);
    const int natom = (int)nl.integer("natom", 1);
    const int xunit = (int)nl.integer("xunit", 1);
    const int64_t imin = nl.integer("imin", 0);
    const double tau = nl.real("tau", 1.0);
    const double gamma = nl.real("gamma", 1.0);
    const double dHdrlimit = nl.real("dHdrlimit", -1.0);
    const bool readpath = nl.logical("readpath", true);
    const bool cayley = nl.logical("cayley", false);
    const bool iprint = nl.logical("iprint", false);
    const int64_t npath = nl.integer("npath", 0);
    const int restart = (int)nl.integer("restart", 0);
    const std::string pes = nl.str("pes", "1d");
    const std::string prec = lower(nl.str("precision", "mixed"));
    const std::string form = lower(nl.str("form", "auto"));
    const uint64_t seed = (uint64_t)nl.integer("seed", 0);
    const std::string init = lower(nl.str("init", "path"));
    const double init_sigma = nl.real("init_sigma", 0.0);
    const int64_t chunk = nl.integer("chunk", 5000);
    const std::string pesfile = nl.str("pes_params", "");
    if (parse_only) {
        std::printf("{\"n\": %lld, \"beta\": %.17g, \"NMC\": %lld, \"Noutput\": %lld, \"dt\": %.17g, "
                    "\"nintegral\": %lld, \"nrep\": %lld, \"thermostat\": %d, \"ndim\": %d, \"natom\": %d, "
                    "\"xunit\": %d, \"imin\": %lld, \"tau\": %.17g, \"gamma\": %.17g, \"dHdrlimit\": %.17g, "
                    "\"readpath\": %s, \"cayley\": %s, \"npath\": %lld, \"restart\": %d, \"pes\": \"%s\", "
                    "\"precision\": \"%s\", \"form\": \"%s\", \"seed\": %llu, \"init\": \"%s\", "
                    "\"init_sigma\": %.17g}\n",
                    (long long)n, beta, (long long)NMC, (long long)Noutput, dt, (long long)nintegral,
                    (long long)nrep, thermostat, ndim, natom, xunit, (long long)imin, tau, gamma, dHdrlimit,
                    readpath ? "true" : "false", cayley ? "true" : "false", (long long)npath, restart,
                    pes.c_str(), prec.c_str(), form.c_str(), (unsigned long long)seed, init.c_str(), init_sigma);
        return 0;
    }
    auto t0 = std::chrono::steady_clock::now();
    const int nd = ndim * natom;
    const double betan = beta / (double)(n + 1);  // pimd_par.f90:94
    std::vector<std::string> label;
    std::vector<double> mass;
    std::vector<double> w1, w2, params;
    int pid;
    try {
        read_masses("masses.dat", natom, label, mass);
        w1 = read_well("well1.dat", ndim, natom, xunit);
        w2 = read_well("well2.dat", ndim, natom, xunit);
        params = read_numbers(pesfile);
        pid = pes_id_of(pes);
    } catch (std::exception &e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    std::printf(" Running with parameters (in a.u.):\n beta, betan, n= %.10g %.10g %lld\n", beta, betan, (long long)n);
    std::printf(" NMC, Noutput, dt= %lld %lld %.10g\n with integration points %lld\n and %lld repetitions\n",
                (long long)NMC, (long long)Noutput, dt, (long long)nintegral, (long long)nrep);
    std::printf(" %s\n", thermostat == 1 ? "Running with Andersen thermostat" : "Running with Langevin thermostat");

    pg_ctx *ctx = nullptr;
    CHECK(pg_create(&ctx, 0));
    // V0 = V(well1) (pimd_par.f90:166)
    CHECK(pg_set_system(ctx, ndim, natom, mass.data(), pid, params.data(), (int64_t)params.size(), 0.0));
    double v0 = 0.0;
    CHECK(pg_pes_eval(ctx, 1, w1.data(), &v0, nullptr, PG_FP64));
    CHECK(pg_set_system(ctx, ndim, natom, mass.data(), pid, params.data(), (int64_t)params.size(), v0));
    double vw[2];
    std::vector<double> ww(w1);
    ww.insert(ww.end(), w2.begin(), w2.end());
    CHECK(pg_pes_eval(ctx, 2, ww.data(), vw, nullptr, PG_FP64));
    std::printf(" Potential at wells: %.12g %.12g\n", vw[0], vw[1]);

    // path: spline of path.xyz against normalised arc length, or the straight line
    std::vector<std::vector<double>> frames;
    if (readpath && npath >= 2) {
        try {
            frames = read_path_xyz("path.xyz", (int)npath, ndim, natom, xunit);
        } catch (std::exception &e) {
            std::fprintf(stderr, "%s\n", e.what());
            return 1;
        }
    } else {
        frames = {w1, w2};
    }
    const int64_t np = (int64_t)frames.size();
    std::vector<double> lam(np, 0.0);
    for (int64_t i = 1; i < np; i++) {
        double d = 0.0;
        for (int k = 0; k < nd; k++) d += (frames[i][k] - frames[i - 1][k]) * (frames[i][k] - frames[i - 1][k]);
        lam[i] = lam[i - 1] + std::sqrt(d);
    }
    for (auto &l : lam) l /= lam[np - 1];
    std::vector<std::vector<double>> ycol(nd, std::vector<double>(np)), y2(nd, std::vector<double>(np));
    for (int k = 0; k < nd; k++) {
        for (int64_t i = 0; i < np; i++) ycol[k][i] = frames[i][k];
        CHECK(pg_spline(lam.data(), ycol[k].data(), np, 1.0e31, 1.0e31, y2[k].data()));
    }
    auto path_at = [&](double xi, int k, double *y, double *g) {
        return pg_splint(lam.data(), ycol[k].data(), y2[k].data(), np, xi, y, g);
    };
    // Gauss-Legendre points and end points (pimd_par.f90:212-221)
    std::vector<double> xi(nintegral), wq(nintegral);
    CHECK(pg_gauleg(0.0, 1.0, xi.data(), wq.data(), nintegral));
    std::vector<double> a(nd), b((size_t)nintegral * nd), dbdl((size_t)nintegral * nd);
    for (int k = 0; k < nd; k++) CHECK(path_at(0.0, k, &a[k], nullptr));
    for (int64_t i = 0; i < nintegral; i++)
        for (int k = 0; k < nd; k++) CHECK(path_at(xi[i], k, &b[i * nd + k], &dbdl[i * nd + k]));
    // start positions per lambda point
    std::vector<double> xref((size_t)nintegral * nd * n);
    for (int64_t i = 0; i < nintegral; i++)
        for (int k = 0; k < nd; k++)
            for (int64_t bead = 0; bead < n; bead++) {
                double v = w1[k];
                if (init == "path") {
                    double xe = (double)bead * xi[i] / (double)(n - 1);  // verletmodule.f90:43
                    CHECK(path_at(xe, k, &v, nullptr));
                }
                xref[(i * nd + k) * n + bead] = v;
            }
    const int64_t nrings = nintegral * nrep;
    std::vector<int32_t> rlam(nrings);
    std::vector<uint64_t> rseed(nrings);
    std::vector<uint32_t> rstream(nrings);
    for (int64_t i = 0; i < nintegral; i++)
        for (int64_t j = 0; j < nrep; j++) {
            rlam[i * nrep + j] = (int32_t)i;
            rseed[i * nrep + j] = seed + (uint64_t)j;
            rstream[i * nrep + j] = (uint32_t)i;
        }
    pg_ti_config cfg;
    cfg.nbeads = n;
    cfg.beta = beta;
    cfg.dt = dt;
    cfg.tau = tau;
    cfg.gamma = gamma;
    cfg.thermostat = thermostat;
    cfg.precision = prec == "fp64" ? PG_FP64 : PG_MIXED;
    cfg.form = form == "plain" ? PG_FORM_PLAIN : form == "fused" ? PG_FORM_FUSED : form == "tensor" ? PG_FORM_TENSOR
                                                                                                     : PG_FORM_AUTO;
    cfg.cayley = cayley ? 1 : 0;
    cfg.imin = imin;
    cfg.noutput = Noutput;
    cfg.dhdr_limit = dHdrlimit;
    cfg.init_sigma = init_sigma;
    CHECK(pg_ti_setup(ctx, &cfg, nrings, nintegral, rlam.data(), rseed.data(), rstream.data(), a.data(), b.data(),
                      dbdl.data(), xref.data(), nullptr, nullptr));
    if (restart == 2) CHECK(pg_ti_checkpoint_load(ctx, "restart.ckpt"));
    int64_t done = 0;
    CHECK(pg_ti_get_step(ctx, &done));
    while (done < NMC) {
        int64_t k = std::min(chunk, NMC - done);
        CHECK(pg_ti_advance(ctx, k));
        done += k;
        if (iprint) std::printf(" %.2f %% of the steps done\n", 100.0 * (double)done / (double)NMC);
    }
    if (restart >= 1) CHECK(pg_ti_checkpoint_save(ctx, "restart.ckpt"));
    std::vector<double> mean(nintegral), var(nintegral);
    std::vector<int64_t> cnt(nintegral);
    CHECK(pg_ti_lambda_reduce(ctx, mean.data(), var.data(), cnt.data()));
    std::vector<int32_t> status(nrings);
    CHECK(pg_ti_get_results(ctx, nullptr, nullptr, nullptr, status.data()));
    int64_t bad = 0;
    for (auto s : status) bad += s != 0;
    std::printf(" final answers per integration point:\n");
    for (int64_t i = 0; i < nintegral; i++) std::printf(" %lld %.15g %.15g\n", (long long)(i + 1), xi[i], mean[i]);
    double dA, sA, q;
    CHECK(pg_ti_assemble(nintegral, wq.data(), mean.data(), var.data(), betan, &dA, &sA, &q));
    // pimd_par.f90:420-424
    std::printf(" beta, betan, n= %.10g %.10g %lld\n", beta, betan, (long long)n);
    std::printf(" final Delta A= %.15g +/- %.15g %.15g\n", dA, std::sqrt(sA), std::sqrt(sA / (double)nrep));
    std::printf(" q/q0= %.15g %.15g %.15g\n", q, betan * std::sqrt(sA) * q, betan * std::sqrt(sA / (double)nrep) * q);
    std::printf(" q0/q= %.15g %.15g %.15g\n", 1.0 / q, betan * std::sqrt(sA) / q,
                betan * std::sqrt(sA / (double)nrep) / q);
    double delta = 0.0;
    if (pg_splitting_from_ratio(beta, q, &delta) == PG_OK)
        std::printf(" splitting Delta= %.15g (%.10g cm-1)\n", delta, delta * 219474.63);
    if (bad) std::printf(" rings with a NaN: %lld\n", (long long)bad);
    double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::printf(" Ran in %.3f s\n", secs);
    pg_destroy(ctx);
    return 0;
}
