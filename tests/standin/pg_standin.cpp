// Stand-in for the C-ABI calls the namelist drivers make, computed by the
// oracle on the CPU, so that the drivers' host logic (input files, alignment,
// the order of the calls, the arithmetic between them, the files they write)
// can be run end to end without a GPU.  TEST INFRASTRUCTURE ONLY: it is
// compiled into a scratch directory by the tests and linked into test copies of
// the drivers; the shipped drivers link libpimdgpu.
//
// pg_instanton_optimize does not optimise: it returns the path it is given and
// its action, which is enough to check what the drivers do with the result.
// pg_instanton_logdet diagonalises the oracle's band Hessian densely.
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <vector>

#include "eigsym.hpp"
#include "oracle.h"
#include "pimdgpu.h"

struct pg_ctx {
    or_pes pes;
    std::vector<double> params, mass;
};

extern "C" {

const char *pg_last_error(void) { return "stand-in"; }
int pg_create(pg_ctx **c, int32_t) {
    *c = new pg_ctx();
    return PG_OK;
}
int pg_destroy(pg_ctx *c) {
    delete c;
    return PG_OK;
}
int pg_set_system(pg_ctx *c, int64_t ndim, int64_t natom, const double *mass, int32_t pes_id, const double *params,
                  int64_t nparams, double V0) {
    c->params.assign(params, params + nparams);
    c->mass.assign(mass, mass + natom);
    c->pes = or_pes{pes_id, (int32_t)ndim, (int32_t)natom, (int32_t)nparams, V0, c->params.data()};
    return PG_OK;
}
static int64_t ndof(const pg_ctx *c) { return (int64_t)c->pes.ndim * c->pes.natom; }
int pg_pes_eval(pg_ctx *c, int64_t nconf, const double *x, double *V, double *grad, int32_t) {
    const int64_t nd = ndof(c);
    for (int64_t k = 0; k < nconf; k++) {
        if (V) V[k] = or_V(&c->pes, x + k * nd);
        if (grad) or_Vprime(&c->pes, x + k * nd, grad + k * nd);
    }
    return PG_OK;
}
int pg_pes_hessian(pg_ctx *c, int64_t nconf, const double *x, double *hess, int32_t quirks) {
    const int64_t nd = ndof(c);
    for (int64_t k = 0; k < nconf; k++) or_Vdoubleprime(&c->pes, x + k * nd, hess + k * nd * nd, quirks);
    return PG_OK;
}
int pg_gauleg(double x1, double x2, double *x, double *w, int64_t n) {
    or_gauleg(x1, x2, x, w, n);
    return PG_OK;
}
int pg_spline(const double *x, const double *y, int64_t n, double yp1, double ypn, double *y2) {
    or_spline(x, y, n, yp1, ypn, y2);
    return PG_OK;
}
int pg_splint(const double *xa, const double *ya, const double *y2a, int64_t n, double x, double *y, double *dydx) {
    if (y) *y = or_splint(xa, ya, y2a, n, x);
    if (dydx) *dydx = or_splin_grad(xa, ya, y2a, n, x);
    return PG_OK;
}
int pg_instanton_optimize(pg_ctx *c, int64_t nbeta, int64_t N, double *x, const double *a, const double *b,
                          const double *betan, const pg_lbfgs_opts *, double *UM, int64_t *niter, int32_t *status) {
    const int64_t nd = ndof(c);
    for (int64_t k = 0; k < nbeta; k++) {
        if (UM) UM[k] = or_UM(&c->pes, c->mass.data(), N, betan[k], x + k * nd * N, a, b + k * nd, 1);
        if (niter) niter[k] = 0;
        if (status) status[k] = 0;
    }
    return PG_OK;
}
int pg_instanton_logdet(pg_ctx *c, int64_t nbeta, int64_t N, const double *x, const double *betan,
                        int32_t singlewell, int32_t skip_lowest, int32_t quirks, double *lndet, double *eta2_min,
                        int64_t *nskipped) {
    const int64_t nd = ndof(c), n = nd * N;
    for (int64_t k = 0; k < nbeta; k++) {
        std::vector<double> band((size_t)(nd + 1) * n), a((size_t)n * n, 0.0), w, v;
        or_UMhessian(&c->pes, c->mass.data(), N, betan[k], x + k * nd * N, singlewell, quirks, band.data());
        for (int64_t j = 0; j < n; j++)
            for (int64_t r = 0; r <= nd && j + r < n; r++)
                a[(size_t)(j + r) * n + j] = a[(size_t)j * n + j + r] = band[(size_t)r + (size_t)(nd + 1) * j];
        if (pgh::eigsym_jacobi((int)n, a, w, v) < 0) return PG_ERR_NUMERIC;
        double s = 0.0;
        int64_t skipped = 0;
        for (int64_t i = 0; i < n; i++) {
            if ((skip_lowest && i == 0) || !(w[i] > 0.0)) {
                skipped++;
                continue;
            }
            s += std::log(w[i]);
        }
        lndet[k] = s;
        if (eta2_min) eta2_min[k] = w[0];
        if (nskipped) nskipped[k] = skipped;
    }
    return PG_OK;
}
int pg_rpi_assemble(double betan, double UM, double lndetJ, double lndetJ0, double *S, double *omega,
                    double *delta) {
    const double s = betan * UM, gam = std::exp(0.5 * (lndetJ - lndetJ0));
    const double om = betan * std::exp(-s) * std::sqrt(s / (2.0 * OR_PI_REF)) / gam;
    if (S) *S = s;
    if (omega) *omega = om;
    if (delta) *delta = 2.0 * om / betan;
    return PG_OK;
}

}  // extern "C"
