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
// positions), chunk (steps per device launch sequence), tune (JSON-lines cache
// of the autotuner: with form 'auto' the launch parameters are tuned on the
// first run of each batch shape and read back afterwards).
// Three-dimensional wells and path frames are aligned as the reference does
// (keys alignwell, atom1, atom2, atom3; aligned_wells.xyz with alignwell);
// --prepare-only prints the aligned start configurations and stops.
// restart >= 1 writes, after the run, the reference's restart files
// restart_proc<iproc>_<ii>.xyz (verletmodule.f90:162-185; the task -> (rank,
// local index) split of pimd_par.f90:109-110, 332-353 for nproc ranks, key
// nproc, default 1) and restart.ckpt, a bitwise checkpoint of the device state.
// restart = 2 continues from restart.ckpt when present, else from the restart
// files (positions, momenta, dHdr sums, step count), and runs NMC further
// steps as the reference does.  Deviation: the estimator is divided by the
// number of accumulated samples (the reference divides by NMC + restartnmc -
// imin although it skips imin steps again after a restart).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <random>
#include <string>
#include <vector>

#include "../../include/pimdgpu.h"
#include "align.hpp"
#include "eigsym.hpp"
#include "namelist.hpp"
#include "pes_names.hpp"

using namespace pgdrv;

// readhess diagonalises the polymer Hessian with the host Jacobi solver: at most
// this many dofs (n * ndim * natom) per lambda point.
constexpr int kReadhessMaxDof = 1024;

// restart_proc<iproc>_<ii>.xyz of task r: nproc contiguous blocks of
// ncalcs = ceil(ntask / nproc) tasks (pimd_par.f90:109-110, 352).
static std::string restart_name(int64_t r, int64_t ntask, int64_t nproc) {
    const int64_t ncalcs = (ntask + nproc - 1) / nproc;
    return "restart_proc" + std::to_string(r / ncalcs) + "_" + std::to_string(r % ncalcs + 1) + ".xyz";
}

// write_restart (verletmodule.f90:162-185): per bead natom, dHdr, label x y z;
// then per bead natom, step, label px py pz.  Coordinates beyond ndim are 0.
// x, p: [dof][bead] of one ring, dof = atom * ndim + dim.
static bool write_restart_xyz(const std::string &path, int64_t n, int ndim, int natom,
                              const std::vector<std::string> &label, const double *x, const double *p,
                              double dhdr, int64_t step) {
    FILE *f = std::fopen(path.c_str(), "w");
    if (!f) return false;
    for (int pass = 0; pass < 2; pass++)
        for (int64_t i = 0; i < n; i++) {
            std::fprintf(f, " %d\n", natom);
            if (pass == 0)
                std::fprintf(f, " %.17g\n", dhdr);
            else
                std::fprintf(f, " %lld\n", (long long)step);
            const double *v = pass == 0 ? x : p;
            for (int j = 0; j < natom; j++) {
                std::fprintf(f, " %s", label[j].c_str());
                for (int d = 0; d < 3; d++) std::fprintf(f, " %.17g", d < ndim ? v[((int64_t)j * ndim + d) * n + i] : 0.0);
                std::fprintf(f, "\n");
            }
        }
    return std::fclose(f) == 0;
}

static bool read_restart_xyz(const std::string &path, int64_t n, int ndim, int natom, double *x, double *p,
                             double *dhdr, int64_t *step) {
    std::ifstream f(path);
    if (!f) return false;
    for (int pass = 0; pass < 2; pass++)
        for (int64_t i = 0; i < n; i++) {
            int na = 0;
            if (!(f >> na) || na != natom) return false;
            if (pass == 0) {
                if (!(f >> *dhdr)) return false;
            } else {
                long long st = 0;
                if (!(f >> st)) return false;
                if (i > 0 && st != *step) return false;  // one step count per file
                *step = st;
            }
            double *v = pass == 0 ? x : p;
            for (int j = 0; j < natom; j++) {
                std::string lab;
                double c[3];
                if (!(f >> lab >> c[0] >> c[1] >> c[2])) return false;
                for (int d = 0; d < ndim && d < 3; d++) v[((int64_t)j * ndim + d) * n + i] = c[d];
            }
        }
    return true;
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
    bool prepare_only = argc > 1 && std::string(argv[1]) == "--prepare-only";
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
    const bool readhess = nl.logical("readhess", false);  // pimd_par.f90:83
    const bool alignwell = nl.logical("alignwell", false);  // pimd_par.f90:80
    const int atom1 = (int)nl.integer("atom1", 1), atom2 = (int)nl.integer("atom2", 2),
              atom3 = (int)nl.integer("atom3", 3);  // pimd_par.f90:84-86
    const bool iprint = nl.logical("iprint", false);
    const int64_t npath = nl.integer("npath", 0);
    const int restart = (int)nl.integer("restart", 0);
    const int64_t nproc = std::max<int64_t>(1, nl.integer("nproc", 1));
    const bool instapath = nl.logical("instapath", false);  // pimd_par.f90:76
    const bool centre = nl.logical("centre", false);        // pimd_par.f90:77
    const bool fixedends = nl.logical("fixedends", true);   // pimd_par.f90:81
    const std::string pes = nl.str("pes", "1d");
    const std::string prec = lower(nl.str("precision", "mixed"));
    const std::string form = lower(nl.str("form", "auto"));
    const uint64_t seed = (uint64_t)nl.integer("seed", 0);
    const std::string init = lower(nl.str("init", "path"));
    const double init_sigma = nl.real("init_sigma", 0.0);
    const int64_t chunk = nl.integer("chunk", 5000);
    const std::string pesfile = nl.str("pes_params", "");
    const std::string tune = nl.str("tune", "");
    nl.accept({"use_mkl", "basename"});  // pimd_par.f90:43-44: no effect here
    if (!nl.check(std::cerr)) return 1;
    {
        RangeCheck rc{std::cerr};
        rc.need(n >= 2, "n (beads) must be at least 2");
        rc.need(beta > 0.0, "beta must be positive");
        rc.need(dt > 0.0, "dt must be positive");
        rc.need(tau > 0.0, "tau must be positive");
        rc.need(gamma >= 0.0, "gamma must not be negative");
        rc.need(NMC >= 0 && imin >= 0, "NMC and imin must not be negative");
        rc.need(nintegral >= 1 && nrep >= 1, "nintegral and nrep must be at least 1");
        rc.need(ndim >= 1 && natom >= 1, "ndim and natom must be at least 1");
        rc.need(thermostat == 1 || thermostat == 2, "thermostat must be 1 (Andersen) or 2 (Langevin)");
        rc.need(chunk >= 1, "chunk must be at least 1");
        rc.need(!readpath || npath == 0 || npath >= 2, "npath must be at least 2 with readpath");
        if (!rc.ok) return 1;
    }
    if (parse_only) {
        std::printf("{\"n\": %lld, \"beta\": %.17g, \"NMC\": %lld, \"Noutput\": %lld, \"dt\": %.17g, "
                    "\"nintegral\": %lld, \"nrep\": %lld, \"thermostat\": %d, \"ndim\": %d, \"natom\": %d, "
                    "\"xunit\": %d, \"imin\": %lld, \"tau\": %.17g, \"gamma\": %.17g, \"dHdrlimit\": %.17g, "
                    "\"readpath\": %s, \"cayley\": %s, \"npath\": %lld, \"restart\": %d, \"pes\": \"%s\", "
                    "\"precision\": \"%s\", \"form\": \"%s\", \"seed\": %llu, \"init\": \"%s\", "
                    "\"init_sigma\": %.17g, \"nproc\": %lld, \"instapath\": %s, \"centre\": %s, "
                    "\"fixedends\": %s, \"tune\": \"%s\", \"readhess\": %s, \"alignwell\": %s, "
                    "\"atom1\": %d, \"atom2\": %d, \"atom3\": %d}\n",
                    (long long)n, beta, (long long)NMC, (long long)Noutput, dt, (long long)nintegral,
                    (long long)nrep, thermostat, ndim, natom, xunit, (long long)imin, tau, gamma, dHdrlimit,
                    readpath ? "true" : "false", cayley ? "true" : "false", (long long)npath, restart,
                    pes.c_str(), prec.c_str(), form.c_str(), (unsigned long long)seed, init.c_str(), init_sigma,
                    (long long)nproc, instapath ? "true" : "false", centre ? "true" : "false",
                    fixedends ? "true" : "false", tune.c_str(), readhess ? "true" : "false",
                    alignwell ? "true" : "false", atom1, atom2, atom3);
        return 0;
    }
    if (readhess && !prepare_only && n * ndim * natom > kReadhessMaxDof) {  // Jacobi eigensolver: O(n^3) per sweep
        std::fprintf(stderr, "readhess = .true. with %lld polymer dofs: this driver diagonalises at most %d; "
                             "run the Python driver (drivers.run_ti(..., readhess=True))\n",
                     (long long)(n * ndim * natom), kReadhessMaxDof);
        return 1;
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
    // wells aligned as pimd_par.f90:159-183 does (three-dimensional systems;
    // others are left as read, where the reference stops,
    // instantonmod.f90:234-237)
    const bool can_align = pgh::align_supported(ndim, natom, atom1, atom2, atom3);
    if (can_align) {
        const pgh::AlignAngles ang = pgh::align_wells_ti(w1, w2, natom, atom1, atom2, atom3, alignwell);
        if (alignwell) {
            char c[160];
            std::snprintf(c, sizeof c, "rotation angles: %.17g %.17g %.17g", ang.theta1, ang.theta2, ang.theta3);
            if (!write_xyz("aligned_wells.xyz", {w1, w2}, {c, c}, ndim, natom, label)) {
                std::fprintf(stderr, "cannot write aligned_wells.xyz\n");
                return 1;
            }
        }
    }
    // path: spline of path.xyz against normalised arc length, or the straight
    // line; the frames of path.xyz aligned by the angles of the first
    // (instantonmod.f90:916-932)
    std::vector<std::vector<double>> frames;
    pgh::AlignAngles path_ang;  // of the path's first frame (aligned.xyz)
    const bool from_path = readpath && npath >= 2;
    if (from_path) {
        try {
            frames = read_path_xyz("path.xyz", (int)npath, ndim, natom, xunit);
        } catch (std::exception &e) {
            std::fprintf(stderr, "%s\n", e.what());
            return 1;
        }
        if (can_align) {
            path_ang = pgh::get_align(frames[0], natom, atom1, atom2, atom3);
            pgh::align_frames(frames, natom, atom1, atom2, atom3);
        }
    } else {
        frames = {w1, w2};
    }
    if (prepare_only) {  // the inputs as the run would use them, no device
        print_frames_json(w1, w2, frames);
        return 0;
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

    // normalised arc length of the path frames (instantonmod.f90:928-937)
    auto arc_length = [&](const std::vector<std::vector<double>> &fr) {
        std::vector<double> l(fr.size(), 0.0);
        for (size_t i = 1; i < fr.size(); i++) {
            double d = 0.0;
            for (int k = 0; k < nd; k++) d += (fr[i][k] - fr[i - 1][k]) * (fr[i][k] - fr[i - 1][k]);
            l[i] = l[i - 1] + std::sqrt(d);
        }
        for (auto &v : l) v /= l.back();
        return l;
    };
    std::vector<double> lam = arc_length(frames);
    // start beads xtilde at (k-1)/(n-1) on the path's spline (instantonmod.f90:940-950),
    // replaced by the instanton with instapath; written to aligned.xyz
    std::vector<double> xtilde;
    if (from_path) {
        const int64_t npf = (int64_t)frames.size();
        std::vector<double> yk(npf), y2k(npf);
        xtilde.resize((size_t)nd * n);
        for (int k = 0; k < nd; k++) {
            for (int64_t i = 0; i < npf; i++) yk[i] = frames[i][k];
            CHECK(pg_spline(lam.data(), yk.data(), npf, 1.0e31, 1.0e31, y2k.data()));
            for (int64_t bead = 0; bead < n; bead++)
                CHECK(pg_splint(lam.data(), yk.data(), y2k.data(), npf, (double)bead / (double)(n - 1),
                                &xtilde[(size_t)k * n + bead], nullptr));
        }
    }
    if (instapath) {
        // instanton from the path guess (instantonmod.f90:945-983): beads at
        // xi = (k-1)/(n-1) on the spline, optimised with fixed ends at the wells
        // or, with fixedends = F, free-ended (instanton(xtilde)); the action's
        // betan is that of the driver (pimd_par.f90:94)
        const int64_t npf = (int64_t)frames.size();
        std::vector<double> xt((size_t)nd * n), yk(npf), y2k(npf);
        for (int k = 0; k < nd; k++) {
            for (int64_t i = 0; i < npf; i++) yk[i] = frames[i][k];
            CHECK(pg_spline(lam.data(), yk.data(), npf, 1.0e31, 1.0e31, y2k.data()));
            for (int64_t bead = 0; bead < n; bead++)
                CHECK(pg_splint(lam.data(), yk.data(), y2k.data(), npf, (double)bead / (double)(n - 1),
                                &xt[(size_t)k * n + bead], nullptr));
        }
        std::printf(" Finding instanton\n");
        pg_lbfgs_opts o{};
        o.m = 8;  // instantonmod.f90:716
        o.max_backtracks = 40;
        o.maxiter = 200000;
        o.factr = 1.0e6;
        o.pgtol = 1.0e-5;
        double um = 0.0;
        int64_t it = 0;
        int32_t ist = 0;
        CHECK(pg_set_fixedends(ctx, fixedends ? 1 : 0));
        CHECK(pg_instanton_optimize(ctx, 1, n, xt.data(), fixedends ? w1.data() : nullptr,
                                    fixedends ? w2.data() : nullptr, &betan, &o, &um, &it, &ist));
        CHECK(pg_set_fixedends(ctx, 1));
        std::printf(" Found instanton after %lld iterations (status %d).\n", (long long)it, ist);
        if (from_path) xtilde = xt;
        // the new path: [well 1, beads, well 2] with fixed ends, the n beads
        // alone with free ends (instantonmod.f90:959-970)
        frames.clear();
        if (fixedends) frames.push_back(w1);
        for (int64_t bead = 0; bead < n; bead++) {
            std::vector<double> f(nd);
            for (int k = 0; k < nd; k++) f[k] = xt[(size_t)k * n + bead];
            frames.push_back(f);
        }
        if (fixedends) frames.push_back(w2);
        FILE *fi = std::fopen("instanton.xyz", "w");
        if (fi) {
            for (int64_t bead = 0; bead < n; bead++) {
                std::fprintf(fi, " %d\n Energy of minimum %lld\n", natom, (long long)(bead + 1));
                for (int j = 0; j < natom; j++) {
                    std::fprintf(fi, " %s", label[j].c_str());
                    for (int d = 0; d < ndim; d++) std::fprintf(fi, " %.17g", xt[(size_t)(j * ndim + d) * n + bead] * 0.529177);
                    std::fprintf(fi, "\n");
                }
            }
            std::fclose(fi);
        }
        lam = arc_length(frames);
    }
    if (centre) {
        // barrier top xm = the zero of dV/dlambda on (0.3, 0.7) by bisection
        // (instantonmod.f90:832-871), then lambda = a l^2 + b l with
        // a = 2 - 4 xm, b = 4 xm - 1 (instantonmod.f90:993-1004), solved as
        // l = 2 lambda / (b + sqrt(b^2 + 4 a lambda)): the reference's root for
        // either sign of a, finite for a -> 0 (a symmetric barrier).
        const int64_t npf = (int64_t)frames.size();
        std::vector<double> vpath(npf), vy2(npf);
        std::vector<double> flat((size_t)npf * nd);
        for (int64_t i = 0; i < npf; i++)
            for (int k = 0; k < nd; k++) flat[(size_t)i * nd + k] = frames[i][k];
        CHECK(pg_pes_eval(ctx, npf, flat.data(), vpath.data(), nullptr, PG_FP64));
        CHECK(pg_spline(lam.data(), vpath.data(), npf, 1.0e31, 1.0e31, vy2.data()));
        auto dv = [&](double l) {
            double y = 0.0, g = 0.0;
            pg_splint(lam.data(), vpath.data(), vy2.data(), npf, l, &y, &g);
            return g;
        };
        double x1 = 0.3, x2 = 0.7, f1 = dv(x1), f2 = dv(x2);
        if (f1 * f2 >= 0.0) {
            std::fprintf(stderr, "centre: the barrier top is not bracketed in (0.3, 0.7)\n");
            return 1;
        }
        double xm = f1 < 0.0 ? x1 : x2, dx = f1 < 0.0 ? x2 - x1 : x1 - x2;
        for (int j = 0; j < 40; j++) {
            dx *= 0.5;
            const double xmid = xm + dx, fm = dv(xmid);
            if (fm <= 0.0) xm = xmid;
            if (std::fabs(dx) < 1.0e-6 || fm == 0.0) break;
        }
        const double ca = 2.0 - 4.0 * xm, cb = 4.0 * xm - 1.0;
        for (auto &l : lam) l = 2.0 * l / (cb + std::sqrt(cb * cb + 4.0 * ca * l));
        std::printf(" Centred, %.15g %.15g %.15g\n", ca, cb, xm);
    }
    const int64_t np = (int64_t)frames.size();
    std::vector<std::vector<double>> ycol(nd, std::vector<double>(np)), y2(nd, std::vector<double>(np));
    for (int k = 0; k < nd; k++) {
        for (int64_t i = 0; i < np; i++) ycol[k][i] = frames[i][k];
        CHECK(pg_spline(lam.data(), ycol[k].data(), np, 1.0e31, 1.0e31, y2[k].data()));
    }
    if (from_path) {
        const double ang[3] = {path_ang.theta1, path_ang.theta2, path_ang.theta3};
        if (!write_read_path_files(y2, xtilde, n, ndim, natom, label, ang)) {
            std::fprintf(stderr, "cannot write testspline.csv / aligned.xyz\n");
            return 1;
        }
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
    {  // xi, V(path(xi)) and |db/dxi| per point (pimd_par.f90:223-225)
        std::vector<double> vb(nintegral);
        CHECK(pg_pes_eval(ctx, nintegral, b.data(), vb.data(), nullptr, PG_FP64));
        for (int64_t i = 0; i < nintegral; i++) {
            double g2 = 0.0;
            for (int k = 0; k < nd; k++) g2 += dbdl[i * nd + k] * dbdl[i * nd + k];
            std::printf(" %.15g %.15g %.15g\n", xi[i], vb[i], std::sqrt(g2));
        }
    }
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
    const int64_t nstate = nrings * nd * n;
    bool from_files = false;
    std::vector<double> x0, p0, dsum(nrings);
    int64_t step0 = 0;
    if (restart == 2 && !std::ifstream("restart.ckpt")) {
        x0.resize(nstate);
        p0.resize(nstate);
        for (int64_t r = 0; r < nrings; r++) {
            int64_t st = 0;
            const std::string name = restart_name(r, nrings, nproc);
            if (!read_restart_xyz(name, n, ndim, natom, &x0[r * nd * n], &p0[r * nd * n], &dsum[r], &st)) {
                std::fprintf(stderr, "cannot read restart file %s\n", name.c_str());
                return 1;
            }
            if (r == 0) step0 = st;
            if (st != step0) {
                std::fprintf(stderr, "restart files disagree on the step count (%s)\n", name.c_str());
                return 1;
            }
        }
        from_files = true;
    }
    if (!tune.empty()) CHECK(pg_set_tuning(ctx, tune.c_str(), PG_TUNE_ON));
    // readhess (verletmodule.f90:49-88): the beads on the path plus displacements
    // along the eigenvectors of the polymer Hessian at the path beads, which is
    // what detJ diagonalises (instantonmod.f90:782-827; the interpolated Hessian
    // it is passed is not used).  Every mode but the lowest with eta^2 > 0 moves
    // bead i, dimension j, atom k by sqrt(1 / (eta^2 m_k)) tempx(mode) times the
    // eigenvector component natom (j + ndim i) + k, the reference's indexing.
    // tempx ~ N(0, 1 / beta) from a generator seeded with the ring's seed and
    // stream (the reference uses MKL VSL).
    std::vector<double> xh;
    if (readhess && !from_files) {
        const int tot = (int)(n * nd);
        xh.resize(nstate);
        std::vector<double> band((size_t)(nd + 1) * tot), H, ev, vec;
        for (int64_t i = 0; i < nintegral; i++) {
            const double *xp = &xref[(size_t)i * nd * n];
            CHECK(pg_um_hessian(ctx, n, betan, xp, 0, 0, band.data()));
            H.assign((size_t)tot * tot, 0.0);
            for (int r = 0; r <= nd; r++)
                for (int c = 0; c + r < tot; c++) {
                    const double h = band[(size_t)r + (size_t)(nd + 1) * c];
                    H[(size_t)(c + r) * tot + c] = h;
                    H[(size_t)c * tot + c + r] = h;
                }
            if (pgh::eigsym_jacobi(tot, H, ev, vec) < 0) {
                std::fprintf(stderr, "readhess: the Jacobi eigensolver did not converge\n");
                return 1;
            }
            for (int64_t j = 0; j < nrep; j++) {
                const int64_t r = i * nrep + j;
                std::mt19937_64 gen(rseed[r] * 0x9E3779B97F4A7C15ull ^ ((uint64_t)rstream[r] << 32) ^ 0x52454144ull);
                std::normal_distribution<double> gauss(0.0, std::sqrt(1.0 / beta));
                std::vector<double> tempx(tot);
                for (auto &t : tempx) t = gauss(gen);
                double *xr = &xh[(size_t)r * nd * n];
                std::copy(xp, xp + (size_t)nd * n, xr);
                for (int m = 1; m < tot; m++) {
                    if (!(ev[m] > 0.0)) continue;  // the reference skips eta^2 < 0 (and divides by eta^2 = 0)
                    for (int64_t i2 = 0; i2 < n; i2++)
                        for (int j2 = 0; j2 < ndim; j2++)
                            for (int k2 = 0; k2 < natom; k2++) {
                                const int64_t idof2 = (int64_t)natom * (j2 + (int64_t)ndim * i2) + k2;
                                xr[((int64_t)k2 * ndim + j2) * n + i2] +=
                                    std::sqrt(1.0 / (ev[m] * mass[k2])) * tempx[m] * vec[(size_t)idof2 * tot + m];
                            }
                }
            }
        }
    }
    const double *xstart = from_files ? x0.data() : (readhess ? xh.data() : nullptr);
    CHECK(pg_ti_setup(ctx, &cfg, nrings, nintegral, rlam.data(), rseed.data(), rstream.data(), a.data(), b.data(),
                      dbdl.data(), xref.data(), xstart, from_files ? p0.data() : nullptr));
    if (restart == 2) {
        if (from_files) {
            std::vector<int64_t> ns(nrings, std::max<int64_t>(0, step0 - imin));
            CHECK(pg_ti_set_accumulators(ctx, dsum.data(), ns.data(), step0));
        } else {
            CHECK(pg_ti_checkpoint_load(ctx, "restart.ckpt"));
        }
    }
    int64_t done = 0;
    CHECK(pg_ti_get_step(ctx, &done));
    const int64_t start = done, target = restart == 2 ? done + NMC : NMC;
    // restart files (and restart.ckpt) every Noutput steps past imin and at the
    // end, as propagate_pimd_pile does (verletmodule.f90:389-395, 412): the
    // reference writes before its step ii when ii >= Noutput steps have passed
    // since the last write and ii > imin (ii counted from 1 in this run), and
    // labels that state with ii; here the label is the number of steps the state
    // has taken, so that a continuation resumes the Philox streams exactly
    auto write_files = [&](int64_t step_count) -> int {
        CHECK(pg_ti_checkpoint_save(ctx, "restart.ckpt"));
        std::vector<double> xs(nstate), ps(nstate), ds(nrings);
        CHECK(pg_ti_get_state(ctx, xs.data(), ps.data()));
        CHECK(pg_ti_get_results(ctx, ds.data(), nullptr, nullptr, nullptr));
        for (int64_t r = 0; r < nrings; r++)
            if (!write_restart_xyz(restart_name(r, nrings, nproc), n, ndim, natom, label, &xs[r * nd * n],
                                   &ps[r * nd * n], ds[r], step_count)) {
                std::fprintf(stderr, "cannot write restart file for task %lld\n", (long long)r);
                return 1;
            }
        return 0;
    };
    const int64_t never = INT64_MAX / 4;
    int64_t next_ii = restart >= 1 && Noutput > 0 ? std::max<int64_t>(Noutput, imin + 1) : never;
    while (done < target) {
        const int64_t at = next_ii < never ? start + next_ii - 1 : never;  // state before step next_ii
        const int64_t k = std::min(chunk, std::min(target, at) - done);
        if (k > 0) {
            CHECK(pg_ti_advance(ctx, k));
            done += k;
            if (iprint) std::printf(" %.2f %% of the steps done\n", 100.0 * (double)(done - start) / (double)NMC);
        }
        if (done == at && done < target) {
            if (int rc = write_files(done)) return rc;
            next_ii += Noutput;
        }
    }
    if (restart >= 1)
        if (int rc = write_files(done)) return rc;
    std::vector<double> mean(nintegral), var(nintegral);
    std::vector<int64_t> cnt(nintegral);
    CHECK(pg_ti_lambda_reduce(ctx, mean.data(), var.data(), cnt.data()));
    std::vector<int32_t> status(nrings);
    CHECK(pg_ti_get_results(ctx, nullptr, nullptr, nullptr, status.data()));
    int64_t bad = 0;
    for (auto s : status) bad += s != 0;
    std::printf(" final answers per integration point:\n");
    for (int64_t i = 0; i < nintegral; i++) std::printf(" %lld %.15g %.15g\n", (long long)(i + 1), xi[i], mean[i]);
    // a lambda point whose rings were all left out (NaN-flagged, or no sample
    // yet) has no estimate: stop rather than integrate a zero
    for (int64_t i = 0; i < nintegral; i++)
        if (cnt[i] <= 0) {
            std::fprintf(stderr, "integration point %lld has no valid ring (all NaN-flagged or without samples)\n",
                         (long long)(i + 1));
            return 3;
        }
    double dA, sA, q;
    CHECK(pg_ti_assemble(nintegral, wq.data(), mean.data(), var.data(), betan, &dA, &sA, &q));
    // standard error of dA: sum w_i^2 var_i / n_i over the rings each point kept
    // (the reference's sigmaA / nrep when every ring counts, pimd_par.f90:422)
    double sA_n = 0.0;
    for (int64_t i = 0; i < nintegral; i++) sA_n += wq[i] * wq[i] * var[i] / (double)cnt[i];
    // pimd_par.f90:420-424
    std::printf(" beta, betan, n= %.10g %.10g %lld\n", beta, betan, (long long)n);
    std::printf(" final Delta A= %.15g +/- %.15g %.15g\n", dA, std::sqrt(sA), std::sqrt(sA_n));
    std::printf(" q/q0= %.15g %.15g %.15g\n", q, betan * std::sqrt(sA) * q, betan * std::sqrt(sA_n) * q);
    std::printf(" q0/q= %.15g %.15g %.15g\n", 1.0 / q, betan * std::sqrt(sA) / q, betan * std::sqrt(sA_n) / q);
    double delta = 0.0;
    if (pg_splitting_from_ratio(beta, q, &delta) == PG_OK)
        std::printf(" splitting Delta= %.15g (%.10g cm-1)\n", delta, delta * 219474.63);
    if (bad) std::printf(" rings with a NaN: %lld\n", (long long)bad);
    double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::printf(" Ran in %.3f s\n", secs);
    pg_destroy(ctx);
    return 0;
}
