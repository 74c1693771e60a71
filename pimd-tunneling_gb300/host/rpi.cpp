// rpi.cpp -- C++ front end of the ring-polymer-instanton path: the rpi_ser.f90
// flow (namelist &RPIDATA on standard input, masses.dat / well1.dat /
// well2.dat / path.xyz) on one GPU through the C-ABI:
//   betan = beta/n (rpi_ser.f90:45); V0 = V(well1); start path by linear
//   interpolation or from path.xyz (rpi_ser.f90:133-174); instanton by the
//   on-device L-BFGS; lndetJ0 at all beads in well 1 (single well, every
//   eigenvalue); lndetJ at the instanton (eigenvalue 1 dropped); S, Omega, Delta
//   (rpi_ser.f90:222-237, 354-381).
// Keys beyond the reference's namelist: pes, pes_params (as pimd_ti), m (L-BFGS
// history, reference 8), pgtol (reference eps2 = 1e-5), factr (1e6), maxiter,
// quirks (1: the reference's Hessian band and mcmod_2dtest Hessian).
// Three-dimensional wells are aligned with alignwell (aligned_ends.xyz) and
// path frames always, as the reference does; --prepare-only prints the aligned
// start configurations and stops.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <iostream>
#include <string>
#include <vector>

#include "../../include/pimdgpu.h"
#include "align.hpp"
#include "eigsym.hpp"
#include "namelist.hpp"
#include "pes_names.hpp"

using namespace pgdrv;

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
        nl = Namelist::parse(read_all(std::cin), "RPIDATA");
    } catch (std::exception &e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    // defaults: rpi_ser.f90:28-42
    const int64_t n = nl.integer("n", 100);
    const double beta = nl.real("beta", 30.0);
    const int ndim = (int)nl.integer("ndim", 3);
    const int natom = (int)nl.integer("natom", 1);
    const int xunit = (int)nl.integer("xunit", 1);
    const int64_t npath = nl.integer("npath", 0);
    const bool readpath = nl.logical("readpath", true);
    const std::string pes = nl.str("pes", "1d");
    const std::string pesfile = nl.str("pes_params", "");
    const int m = (int)nl.integer("m", 8);
    const double pgtol = nl.real("pgtol", 1.0e-5);
    const double factr = nl.real("factr", 1.0e6);
    const int64_t maxiter = nl.integer("maxiter", 200000);
    const int quirks = (int)nl.integer("quirks", 0);
    const bool angular = nl.logical("angular", false);                  // rpi_ser.f90:35
    const int64_t npoints = nl.integer("npoints", 10);                  // rpi_ser.f90:34
    const double cutofftheta = nl.real("cutofftheta", 2.0 * 3.14159265358979);  // no reference default
    const double cutoffphi = nl.real("cutoffphi", 3.14159265358979);            // no reference default
    const bool alignwell = nl.logical("alignwell", false);              // rpi_ser.f90:38
    const bool checkhess = nl.logical("checkhess", false);              // rpi_ser.f90:42
    const bool output_instanton = nl.logical("output_instanton", false);  // rpi_ser.f90:36
    // the action with or without the end-point springs (rpi_ser.f90:39, 370-374);
    // the angular grid always has them (rpi_ser.f90:53)
    const bool fixedends = nl.logical("fixedends", true) || angular;
    nl.accept({"alignpath", "basename"});  // rpi_ser.f90:23: no effect in the reference's flow
    if (!nl.check(std::cerr)) return 1;
    {
        RangeCheck rc{std::cerr};
        rc.need(n >= 2, "n (beads) must be at least 2");
        rc.need(beta > 0.0, "beta must be positive");
        rc.need(ndim >= 1 && natom >= 1, "ndim and natom must be at least 1");
        rc.need(m >= 1 && maxiter >= 1, "m and maxiter must be at least 1");
        rc.need(!angular || npoints >= 1, "npoints must be at least 1");
        if (!rc.ok) return 1;
    }
    const int atom1 = (int)nl.integer("atom1", 1), atom2 = (int)nl.integer("atom2", 2),
              atom3 = (int)nl.integer("atom3", 3);  // rpi_par.f90:53-55
    if (parse_only) {
        std::printf("{\"n\": %lld, \"beta\": %.17g, \"ndim\": %d, \"natom\": %d, \"xunit\": %d, \"npath\": %lld, "
                    "\"readpath\": %s, \"pes\": \"%s\", \"m\": %d, \"pgtol\": %.17g, \"factr\": %.17g, "
                    "\"maxiter\": %lld, \"quirks\": %d, \"angular\": %s, \"npoints\": %lld, \"alignwell\": %s, "
                    "\"atom1\": %d, \"atom2\": %d, \"atom3\": %d, \"checkhess\": %s, \"output_instanton\": %s, "
                    "\"fixedends\": %s}\n",
                    (long long)n, beta, ndim, natom, xunit, (long long)npath, readpath ? "true" : "false",
                    pes.c_str(), m, pgtol, factr, (long long)maxiter, quirks, angular ? "true" : "false",
                    (long long)npoints, alignwell ? "true" : "false", atom1, atom2, atom3,
                    checkhess ? "true" : "false", output_instanton ? "true" : "false", fixedends ? "true" : "false");
        return 0;
    }
    auto t0 = std::chrono::steady_clock::now();
    const int nd = ndim * natom;
    const double betan = beta / (double)n;  // rpi_ser.f90:45
    std::vector<std::string> label;
    std::vector<double> mass, w1, w2, params;
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
    // with alignwell each well aligned by its own angles (rpi_ser.f90:74-92);
    // the frames of path.xyz always, by the angles of the first
    // (instantonmod.f90:926-932); three-dimensional systems only (the
    // reference stops otherwise, instantonmod.f90:234-237)
    const bool can_align = pgh::align_supported(ndim, natom, atom1, atom2, atom3);
    if (can_align && alignwell) {
        w1 = pgh::align_atoms(w1, natom, atom1, pgh::get_align(w1, natom, atom1, atom2, atom3));
        w2 = pgh::align_atoms(w2, natom, atom1, pgh::get_align(w2, natom, atom1, atom2, atom3));
        if (!write_xyz("aligned_ends.xyz", {w1, w2}, {"Well1", "Well2"}, ndim, natom, label)) {
            std::fprintf(stderr, "cannot write aligned_ends.xyz\n");
            return 1;
        }
    }
    std::vector<std::vector<double>> fr;
    pgh::AlignAngles path_ang;  // of the path's first frame (aligned.xyz)
    if (readpath && npath >= 2) {
        try {
            fr = read_path_xyz("path.xyz", (int)npath, ndim, natom, xunit);
        } catch (std::exception &e) {
            std::fprintf(stderr, "%s\n", e.what());
            return 1;
        }
        if (can_align) {
            path_ang = pgh::get_align(fr[0], natom, atom1, atom2, atom3);
            pgh::align_frames(fr, natom, atom1, atom2, atom3);
        }
    }
    if (prepare_only) {  // the inputs as the run would use them, no device
        print_frames_json(w1, w2, fr.empty() ? std::vector<std::vector<double>>{w1, w2} : fr);
        return 0;
    }
    pg_ctx *ctx = nullptr;
    CHECK(pg_create(&ctx, 0));
    CHECK(pg_set_system(ctx, ndim, natom, mass.data(), pid, params.data(), (int64_t)params.size(), 0.0));
    double v0 = 0.0;
    CHECK(pg_pes_eval(ctx, 1, w1.data(), &v0, nullptr, PG_FP64));
    CHECK(pg_set_system(ctx, ndim, natom, mass.data(), pid, params.data(), (int64_t)params.size(), v0));
    std::printf(" beta= %.10g n= %lld\n beta_n= %.10g\n", beta, (long long)n, betan);
    // start path (x[dof*n + bead])
    std::vector<double> x((size_t)nd * n);
    if (!fr.empty()) {
        std::vector<double> lam(fr.size(), 0.0);
        for (size_t i = 1; i < fr.size(); i++) {
            double d = 0.0;
            for (int k = 0; k < nd; k++) d += (fr[i][k] - fr[i - 1][k]) * (fr[i][k] - fr[i - 1][k]);
            lam[i] = lam[i - 1] + std::sqrt(d);
        }
        for (auto &l : lam) l /= lam.back();
        std::vector<std::vector<double>> y2all(nd);
        for (int k = 0; k < nd; k++) {
            std::vector<double> y(fr.size());
            std::vector<double> &y2 = y2all[k];
            y2.resize(fr.size());
            for (size_t i = 0; i < fr.size(); i++) y[i] = fr[i][k];
            CHECK(pg_spline(lam.data(), y.data(), (int64_t)fr.size(), 1.0e31, 1.0e31, y2.data()));
            for (int64_t bead = 0; bead < n; bead++)
                CHECK(pg_splint(lam.data(), y.data(), y2.data(), (int64_t)fr.size(), (double)bead / (double)(n - 1),
                                &x[(size_t)k * n + bead], nullptr));
        }
        const double ang[3] = {path_ang.theta1, path_ang.theta2, path_ang.theta3};
        if (!write_read_path_files(y2all, x, n, ndim, natom, label, ang)) {  // instantonmod.f90:1013-1031
            std::fprintf(stderr, "cannot write testspline.csv / aligned.xyz\n");
            return 1;
        }
    } else {
        for (int k = 0; k < nd; k++)
            for (int64_t bead = 1; bead <= n; bead++)  // rpi_ser.f90:157-163
                x[(size_t)k * n + bead - 1] = ((double)(n - bead) * w1[k] + (double)(bead - 1) * w2[k]) / (double)(n - 1);
        std::vector<std::string> notes;
        for (int64_t bead = 1; bead <= n; bead++) notes.push_back("Energy of minimum " + std::to_string(bead));
        std::vector<std::vector<double>> beads(n, std::vector<double>(nd));
        for (int k = 0; k < nd; k++)
            for (int64_t bead = 0; bead < n; bead++) beads[bead][k] = x[(size_t)k * n + bead];
        if (!write_xyz("aligned.xyz", beads, notes, ndim, natom, label)) {  // rpi_ser.f90:164-172
            std::fprintf(stderr, "cannot write aligned.xyz\n");
            return 1;
        }
    }
    if (checkhess) {
        // Hessian at well 1 written row by row (hessian_well1.dat) and the
        // eigenvalues of its mass-weighted form times 219475 (rpi_ser.f90:105-129)
        std::printf(" Calculating Hessian as test\n");
        std::vector<double> h((size_t)nd * nd), a((size_t)nd * nd), eta2, vec;
        CHECK(pg_pes_hessian(ctx, 1, w1.data(), h.data(), quirks));
        FILE *fh = std::fopen("hessian_well1.dat", "w");
        if (!fh) {
            std::fprintf(stderr, "cannot write hessian_well1.dat\n");
            return 1;
        }
        for (int r = 0; r < nd; r++) {  // row (atom j, dim i) = dof r; columns dof c, atom-major
            for (int c = 0; c < nd; c++) std::fprintf(fh, " %.17g", h[(size_t)r + (size_t)nd * c]);
            std::fprintf(fh, "\n");
        }
        std::fclose(fh);
        for (int r = 0; r < nd; r++)
            for (int c = 0; c < nd; c++)
                a[(size_t)r * nd + c] = h[(size_t)r + (size_t)nd * c] / std::sqrt(mass[r / ndim] * mass[c / ndim]);
        if (pgh::eigsym_jacobi(nd, a, eta2, vec) < 0) {
            std::fprintf(stderr, "checkhess: the eigensolver did not converge\n");
            return 1;
        }
        std::printf(" normal modes:\n");
        for (int j = 0; j < nd; j++) std::printf(" %d %.15g\n", j + 1, eta2[j] * 219475.0);
    }
    std::printf(" Locating instanton\n");
    pg_lbfgs_opts o{};
    o.m = m;
    o.max_backtracks = 40;
    o.maxiter = maxiter;
    o.factr = factr;
    o.pgtol = pgtol;
    double UM = 0.0;
    int64_t it = 0;
    int32_t st = 0;
    // fixedends = F: the free-ended action, optimised without the end points
    // (instanton(xtilde), instantonmod.f90:724-762)
    CHECK(pg_set_fixedends(ctx, fixedends ? 1 : 0));
    CHECK(pg_instanton_optimize(ctx, 1, n, x.data(), fixedends ? w1.data() : nullptr,
                                fixedends ? w2.data() : nullptr, &betan, &o, &UM, &it, &st));
    std::printf(" Found instanton after %lld iterations (status %d).\n", (long long)it, st);
    // V along the instanton (rpi_ser.f90:180-190): when a bead lies below
    // well 1 the reference moves V0 to that bead's energy, which lowers every
    // action that follows by n * min V; instanton.xyz and
    // instantonpathenergy.csv carry the energies before that shift
    // (rpi_ser.f90:192-218)
    std::vector<double> vpath(n);
    {
        std::vector<double> xc((size_t)n * nd);
        for (int64_t bead = 0; bead < n; bead++)
            for (int k = 0; k < nd; k++) xc[(size_t)bead * nd + k] = x[(size_t)k * n + bead];
        CHECK(pg_pes_eval(ctx, n, xc.data(), vpath.data(), nullptr, PG_FP64));
    }
    const double vmin = *std::min_element(vpath.begin(), vpath.end());
    const double vshift = vmin < 0.0 ? vmin : 0.0;
    if (vmin < 0.0) {
        double vw2 = 0.0;
        CHECK(pg_pes_eval(ctx, 1, w2.data(), &vw2, nullptr, PG_FP64));
        std::printf(" New V0= %.15g\n New wells= %.15g %.15g\n", v0 + vmin, -vmin, vw2 - vmin);
    }
    {
        FILE *fi = std::fopen("instanton.xyz", "w");
        FILE *fe = std::fopen("instantonpathenergy.csv", "w");
        if (!fi || !fe) {
            std::fprintf(stderr, "cannot write instanton.xyz / instantonpathenergy.csv\n");
            return 1;
        }
        std::vector<double> lam(n, 0.0);
        for (int64_t bead = 0; bead < n; bead++) {
            std::fprintf(fi, " %d\n Energy of minimum %.17g\n", natom, vpath[bead]);
            for (int j = 0; j < natom; j++) {
                std::fprintf(fi, " %s", label[j].c_str());
                for (int d = 0; d < 3; d++)
                    std::fprintf(fi, " %.17g", d < ndim ? x[(size_t)(j * ndim + d) * n + bead] * 0.529177 : 0.0);
                std::fprintf(fi, "\n");
            }
            if (bead > 0) {
                double dd = 0.0;
                for (int k = 0; k < nd; k++) {
                    const double e = x[(size_t)k * n + bead] - x[(size_t)k * n + bead - 1];
                    dd += e * e;
                }
                lam[bead] = lam[bead - 1] + std::sqrt(dd);
            }
        }
        for (int64_t bead = 0; bead < n; bead++)
            std::fprintf(fe, " %.17g %.17g\n", n > 1 && lam[n - 1] > 0.0 ? lam[bead] / lam[n - 1] : 0.0, vpath[bead]);
        std::fclose(fi);
        std::fclose(fe);
    }
    // S = betan UM(xtilde[, well1, well2]) (rpi_ser.f90:370-374): the optimiser's
    // action, with or without the end springs as it was optimised
    UM -= (double)n * vshift;
    std::vector<double> xharm((size_t)nd * n);
    for (int k = 0; k < nd; k++)
        for (int64_t bead = 0; bead < n; bead++) xharm[(size_t)k * n + bead] = w1[k];
    double ld0 = 0.0, ld = 0.0, emin = 0.0;
    int64_t nsk0 = 0, nsk = 0;
    CHECK(pg_instanton_logdet(ctx, 1, n, xharm.data(), &betan, 1, 0, quirks, &ld0, nullptr, &nsk0));
    std::printf(" Skipped %lld states\n", (long long)nsk0);
    CHECK(pg_instanton_logdet(ctx, 1, n, x.data(), &betan, 0, 1, quirks, &ld, &emin, &nsk));
    std::printf(" 1 %.15g\n Skipped %lld states\n lndetJ %.15g %.15g\n", emin, (long long)(nsk > 0 ? nsk - 1 : 0), ld, ld0);
    double S, omega, delta;
    CHECK(pg_rpi_assemble(betan, UM, ld, ld0, &S, &omega, &delta));
    const double gam = std::exp(0.5 * (ld - ld0));
    std::printf(" phi= %.15g\n s_kink= %.15g\n theta, N*theta= %.15g %.15g\n", gam, S, omega, omega * (double)n);
    std::printf(" h_ij= %.15g %.15g\n RPI delta= %.15g %.15g\n", omega / betan, 219475.0 * omega / betan, delta,
                delta * 219475.0);
    if (angular) {
        // Solid-angle grid (rpi_ser.f90:241-348): well 2 rotated by Gauss-Legendre
        // angles, the instanton re-optimised from the one above for every
        // orientation -- all orientations in one batched optimisation and one
        // batched log-det -- and I(beta) = tanh(Omega N) per point (3-D: 1 when
        // Omega N > 1).  3-D: R_x(theta) R_z(phi) R_x(eta) on every atom
        // (rotate_atoms, instantonmod.f90:346-376); 2-D: rotation by eta in the
        // plane (the reference applies its 3 x 3 x-axis matrix to 2-vectors there).
        const double twopi = 2.0 * 3.14159265358979, pi = 3.14159265358979;
        std::vector<double> th(npoints), wth(npoints), ph(npoints), wph(npoints), et(npoints), wet(npoints);
        CHECK(pg_gauleg(0.0, std::min(twopi, cutofftheta), et.data(), wet.data(), npoints));
        const bool three = ndim == 3;
        if (three) {
            CHECK(pg_gauleg(0.0, std::min(twopi, cutofftheta), th.data(), wth.data(), npoints));
            CHECK(pg_gauleg(0.0, std::min(pi, cutoffphi), ph.data(), wph.data(), npoints));
        } else if (ndim != 2) {
            std::fprintf(stderr, "angular needs ndim = 2 or 3\n");
            return 1;
        }
        auto rot = [&](std::vector<double> &w, int axis, double ang) {  // rotate_atoms
            if (std::fabs(ang) <= 1e-10) return;
            const double c = std::cos(ang), s = std::sin(ang);
            const int j = axis == 1 ? 1 : 0, k = axis == 1 ? 2 : 1;
            for (int at = 0; at < natom; at++) {
                double *v = &w[(size_t)at * ndim];
                const double vj = v[j], vk = v[k];
                v[j] = c * vj + s * vk;
                v[k] = -s * vj + c * vk;
            }
        };
        const int64_t nb = three ? npoints * npoints * npoints : npoints;
        std::vector<double> bb((size_t)nb * nd), wts(nb), xs((size_t)nb * nd * n), bn(nb, betan), ang((size_t)nb * 3);
        for (int64_t q = 0; q < nb; q++) {
            std::vector<double> w(w2);
            const int64_t ii = three ? q / (npoints * npoints) : 0, jj = three ? (q / npoints) % npoints : 0,
                          kk = q % npoints;
            if (three) {
                rot(w, 1, et[kk]);
                rot(w, 3, ph[jj]);
                rot(w, 1, th[ii]);
                wts[q] = wth[ii] * wph[jj] * wet[kk];
                ang[3 * q] = th[ii];
                ang[3 * q + 1] = ph[jj];
            } else {
                rot(w, 3, et[kk]);
                wts[q] = wet[kk];
            }
            ang[3 * q + 2] = et[kk];
            std::copy(w.begin(), w.end(), bb.begin() + q * nd);
            std::copy(x.begin(), x.end(), xs.begin() + q * nd * n);
        }
        std::vector<double> um(nb), lda(nb);
        std::vector<int64_t> its(nb), nska(nb);
        std::vector<int32_t> sts(nb);
        CHECK(pg_instanton_optimize(ctx, nb, n, xs.data(), w1.data(), bb.data(), bn.data(), &o, um.data(), its.data(),
                                    sts.data()));
        CHECK(pg_instanton_logdet(ctx, nb, n, xs.data(), bn.data(), 0, 1, quirks, lda.data(), nullptr, nska.data()));
        FILE *fa = std::fopen("angularI.dat", "w");
        if (!fa) {
            std::fprintf(stderr, "cannot write angularI.dat\n");
            return 1;
        }
        if (output_instanton) {
            // the last orientation's instanton, as the reference's per-orientation
            // overwrites leave it (rpi_ser.f90:261-270, 311-320: Angstrom in 3-D,
            // bohr in 2-D)
            const double *xl = xs.data() + (size_t)(nb - 1) * nd * n;
            FILE *fi = std::fopen("instanton.xyz", "w");
            if (!fi) {
                std::fprintf(stderr, "cannot write instanton.xyz\n");
                return 1;
            }
            for (int64_t bead = 0; bead < n; bead++) {
                std::fprintf(fi, " %d\n Energy of minimum %lld\n", natom, (long long)(bead + 1));
                for (int j = 0; j < natom; j++) {
                    std::fprintf(fi, " %s", label[j].c_str());
                    for (int d = 0; d < ndim; d++)
                        std::fprintf(fi, " %.17g", xl[(size_t)(j * ndim + d) * n + bead] * (three ? 0.529177 : 1.0));
                    std::fprintf(fi, "\n");
                }
            }
            std::fclose(fi);
        }
        for (int64_t q = 0; q < nb; q++) {
            double Sq, om, dq;
            CHECK(pg_rpi_assemble(betan, um[q] - (double)n * vshift, lda[q], ld0, &Sq, &om, &dq));
            double ib = std::tanh(om * (double)n);
            if (three && om * (double)n > 1.0) ib = 1.0;
            if (three) {
                std::fprintf(fa, " %.17g %.17g %.17g %.17g %.17g\n", ang[3 * q], ang[3 * q + 1], ang[3 * q + 2], wts[q], ib);
                std::printf(" %.10g %.10g %.10g %.10g %.10g %.15g\n", ang[3 * q], ang[3 * q + 1], ang[3 * q + 2], wts[q],
                            ib, lda[q]);
            } else {
                std::fprintf(fa, " %.17g %.17g %.17g\n", ang[3 * q + 2], wts[q], ib);
                std::printf(" %.10g %.10g %.10g %.15g %.15g\n", ang[3 * q + 2], wts[q], ib, lda[q], Sq);
            }
        }
        std::fclose(fa);
    }
    double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::printf(" Ran in %.3f s\n", secs);
    pg_destroy(ctx);
    return 0;
}
