// crossover.cpp -- C++ front end of crossover.f90: the crossover inverse
// temperature beta_c = 2 pi / sqrt(-eta^2_min) of a transition state.
// &CROSSDATA on standard input (ndim = 3, natom = 1, xunit = 2 by default,
// crossover.f90:16-20), masses.dat and transition.xyz ("natom / comment /
// label x y z", Angstrom for xunit = 2) in the working directory; the Hessian
// from pg_pes_hessian on the GPU, its mass-weighted eigenvalues on the host
// (cyclic Jacobi, where the reference calls dsyevd).  Prints the eigenvalues
// and "Crossover beta=" as the reference does.
// Keys beyond the reference's namelist: pes, pes_params (as pimd_ti), quirks
// (1: the reference's mcmod_2dtest Hessian).  --parse-only prints the parsed
// namelist as JSON.
#include <cmath>
#include <cstdio>
#include <iostream>
#include <string>
#include <vector>

#include "../../include/pimdgpu.h"
#include "crossover.hpp"
#include "namelist.hpp"
#include "pes_names.hpp"

using namespace pgdrv;

int main(int argc, char **argv) {
    const bool parse_only = argc > 1 && std::string(argv[1]) == "--parse-only";
    Namelist nl;
    try {
        nl = Namelist::parse(read_all(std::cin), "CROSSDATA");
    } catch (std::exception &e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    const int ndim = (int)nl.integer("ndim", 3);  // crossover.f90:16-18
    const int natom = (int)nl.integer("natom", 1);
    const int xunit = (int)nl.integer("xunit", 2);
    const std::string pes = nl.str("pes", "1d");
    const std::string pesfile = nl.str("pes_params", "");
    const int quirks = (int)nl.integer("quirks", 0);
    if (!nl.check(std::cerr)) return 1;
    if (parse_only) {
        std::printf("{\"ndim\": %d, \"natom\": %d, \"xunit\": %d, \"pes\": \"%s\", \"quirks\": %d}\n", ndim, natom,
                    xunit, pes.c_str(), quirks);
        return 0;
    }
    if (ndim < 1 || natom < 1) {
        std::fprintf(stderr, "ndim and natom must be positive\n");
        return 1;
    }
    std::vector<std::string> label;
    std::vector<double> mass, params, ts;
    int pid;
    try {
        read_masses("masses.dat", natom, label, mass);
        ts = read_path_xyz("transition.xyz", 1, ndim, natom, xunit)[0];
        params = read_numbers(pesfile);
        pid = pes_id_of(pes);
    } catch (std::exception &e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    const int nd = ndim * natom;
    pg_ctx *ctx = nullptr;
    std::vector<double> hess((size_t)nd * nd);
    int rc = pg_create(&ctx, 0);
    if (rc == PG_OK)
        rc = pg_set_system(ctx, ndim, natom, mass.data(), pid, params.data(), (int64_t)params.size(), 0.0);
    if (rc == PG_OK) rc = pg_pes_hessian(ctx, 1, ts.data(), hess.data(), quirks);
    if (rc != PG_OK) {
        std::fprintf(stderr, "pimdgpu error %d: %s\n", rc, pg_last_error());
        if (ctx) pg_destroy(ctx);
        return 2;
    }
    pg_destroy(ctx);
    std::vector<double> eta2;
    const double beta_c = pgh::crossover_beta(ndim, natom, hess, mass, eta2);
    for (double e : eta2) std::printf(" %.15g", e);
    std::printf("\n Crossover beta= %.15g\n", beta_c);
    if (std::isnan(beta_c)) {
        std::fprintf(stderr, "no negative eigenvalue: transition.xyz is not a saddle point\n");
        return 1;
    }
    return 0;
}
