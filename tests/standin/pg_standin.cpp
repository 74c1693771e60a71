// Stand-in for the C-ABI calls the namelist drivers make, computed by the
// oracle on the CPU, so that the drivers' host logic (input files, alignment,
// the order of the calls, the arithmetic between them, the files they write)
// can be run end to end without a GPU.  TEST INFRASTRUCTURE ONLY: it is
// compiled into a scratch directory by the tests and linked into test copies of
// the drivers; the shipped drivers link libpimdgpu.
//
// pg_instanton_optimize does not optimise: it returns the path it is given and
// its action, which is enough to check what the drivers do with the result;
// PG_STANDIN_ENDS names a file that receives the end points of a batched call.
// pg_instanton_logdet diagonalises the oracle's band Hessian densely.  The TI
// batch runs the oracle's ring propagation (the reference step order for
// PG_FORM_PLAIN, the normal-mode-resident order otherwise); no checkpoint
// file is written, so restarts read the restart_proc files.
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "eigsym.hpp"
#include "oracle.h"
#include "pimdgpu.h"

struct TiBatch {
    or_ti_params prm{};
    int64_t nrings = 0, nlam = 0, step = 0;
    std::vector<int32_t> lam;
    std::vector<uint64_t> seed;
    std::vector<uint32_t> stream;
    std::vector<double> a, b, dbdl, xref, x, p;
    std::vector<or_ring_result> res;
};

struct pg_ctx {
    or_pes pes;
    std::vector<double> params, mass;
    TiBatch ti;
    int fixedends = 1;
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
int pg_set_wait_limit(pg_ctx *, int64_t ns) { return ns < 0 ? PG_ERR_ARG : PG_OK; }
int pg_fp32_peak(pg_ctx *, double *) { return PG_ERR_UNSUPPORTED; }
int pg_set_fixedends(pg_ctx *c, int32_t fixedends) {
    c->fixedends = fixedends;
    return PG_OK;
}
int pg_instanton_optimize(pg_ctx *c, int64_t nbeta, int64_t N, double *x, const double *a, const double *b,
                          const double *betan, const pg_lbfgs_opts *, double *UM, int64_t *niter, int32_t *status) {
    const int64_t nd = ndof(c);
    if (nbeta > 1 && b && std::getenv("PG_STANDIN_ENDS")) {  // the end points of a batch, one number per line
        FILE *f = std::fopen(std::getenv("PG_STANDIN_ENDS"), "w");
        if (!f) return PG_ERR_ARG;
        for (int64_t i = 0; i < nbeta * nd; i++) std::fprintf(f, "%.17g\n", b[i]);
        std::fclose(f);
    }
    for (int64_t k = 0; k < nbeta; k++) {
        if (UM) UM[k] = or_UM(&c->pes, c->mass.data(), N, betan[k], x + k * nd * N, a, b ? b + k * nd : nullptr,
                              c->fixedends);
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

int pg_splitting_from_ratio(double beta, double qratio, double *delta) {
    if (!(qratio > -1.0 && qratio < 1.0)) return PG_ERR_NUMERIC;
    *delta = 2.0 * std::atanh(qratio) / beta;
    return PG_OK;
}
int pg_um_hessian(pg_ctx *c, int64_t N, double betan, const double *x, int32_t singlewell, int32_t quirks,
                  double *band) {
    or_UMhessian(&c->pes, c->mass.data(), N, betan, x, singlewell, quirks, band);
    return PG_OK;
}
int pg_set_tuning(pg_ctx *, const char *, int32_t) { return PG_OK; }
// no checkpoint file: a restart then goes through the restart_proc files
int pg_ti_checkpoint_save(pg_ctx *, const char *) { return PG_OK; }
int pg_ti_checkpoint_load(pg_ctx *, const char *) { return PG_ERR_ARG; }

// TI batch: every ring advanced by the oracle's ring propagation with the
// same Philox streams (purposes 2 / 1 for the start positions / momenta).
// PG_STANDIN_X0 names a file that receives the start positions x0 the driver
// passes (text, one number per line).
int pg_ti_setup(pg_ctx *c, const pg_ti_config *cfg, int64_t nrings, int64_t nlambda, const int32_t *ring_lambda,
                const uint64_t *ring_seed, const uint32_t *ring_stream, const double *a, const double *b,
                const double *dbdl, const double *xref, const double *x0, const double *p0) {
    TiBatch &t = c->ti;
    const int64_t nd = ndof(c), P = cfg->nbeads, ns = nd * P;
    t.prm = or_ti_params{P, cfg->beta, cfg->beta / (double)(P + 1), cfg->dt, cfg->tau, cfg->gamma, cfg->thermostat,
                         cfg->cayley, cfg->form == PG_FORM_PLAIN ? 0 : 1, 0, cfg->imin, cfg->noutput,
                         cfg->dhdr_limit, cfg->init_sigma};
    t.nrings = nrings;
    t.nlam = nlambda;
    t.step = 0;
    t.lam.assign(ring_lambda, ring_lambda + nrings);
    t.seed.assign(ring_seed, ring_seed + nrings);
    t.stream.assign(ring_stream, ring_stream + nrings);
    t.a.assign(a, a + nd);
    t.b.assign(b, b + nlambda * nd);
    t.dbdl.assign(dbdl, dbdl + nlambda * nd);
    t.xref.assign(xref, xref + nlambda * ns);
    t.x.assign((size_t)nrings * ns, 0.0);
    t.p.assign((size_t)nrings * ns, 0.0);
    t.res.assign(nrings, or_ring_result{});
    std::vector<double> T((size_t)P * P), lam(P), bm((size_t)c->pes.natom * P), bv((size_t)P * nd);
    or_init_nm(P, c->pes.ndim, c->pes.natom, c->mass.data(), t.prm.betan, t.prm.tau, a, b, T.data(), lam.data(),
               bm.data(), bv.data());
    for (int64_t r = 0; r < nrings; r++) {
        or_ring_init(&c->pes, c->mass.data(), &t.prm, T.data(), bm.data(), &t.xref[(size_t)t.lam[r] * ns], t.seed[r],
                     t.stream[r], 0, 2, 1, &t.x[(size_t)r * ns], &t.p[(size_t)r * ns]);
        if (x0) std::copy(x0 + r * ns, x0 + (r + 1) * ns, t.x.begin() + r * ns);
        if (p0) std::copy(p0 + r * ns, p0 + (r + 1) * ns, t.p.begin() + r * ns);
        t.res[r].and_rkick = -1;
    }
    if (const char *k = std::getenv("PG_STANDIN_NAN_RING")) {  // a NaN in the start of the listed rings
        for (const char *q = k; *q;) {                           // (fault injection; comma-separated)
            char *e = nullptr;
            const int64_t r = std::strtoll(q, &e, 10);
            if (e == q) break;
            if (r >= 0 && r < nrings) t.x[(size_t)r * ns] = std::nan("");
            q = *e == ',' ? e + 1 : e;
        }
    }
    if (x0 && std::getenv("PG_STANDIN_X0")) {
        FILE *f = std::fopen(std::getenv("PG_STANDIN_X0"), "w");
        if (!f) return PG_ERR_ARG;
        for (int64_t i = 0; i < nrings * ns; i++) std::fprintf(f, "%.17g\n", x0[i]);
        std::fclose(f);
    }
    return PG_OK;
}
// PG_STANDIN_FAIL_AT = k: a call that would take the batch past step k fails
// without advancing (a run that dies there, for the restart tests).
int pg_ti_advance(pg_ctx *c, int64_t nsteps) {
    TiBatch &t = c->ti;
    if (const char *f = std::getenv("PG_STANDIN_FAIL_AT"))
        if (t.step + nsteps > std::atoll(f)) return PG_ERR_CUDA;
    const int64_t nd = ndof(c), ns = nd * t.prm.P;
    for (int64_t r = 0; r < t.nrings; r++) {
        const int64_t l = t.lam[r];
        or_ring_propagate(&c->pes, c->mass.data(), &t.prm, t.a.data(), &t.b[(size_t)l * nd], &t.dbdl[(size_t)l * nd],
                          &t.xref[(size_t)l * ns], t.seed[r], t.stream[r], t.step, nsteps, &t.x[(size_t)r * ns],
                          &t.p[(size_t)r * ns], &t.res[r]);
    }
    t.step += nsteps;
    return PG_OK;
}
int pg_ti_get_step(pg_ctx *c, int64_t *step) {
    *step = c->ti.step;
    return PG_OK;
}
int pg_ti_get_state(pg_ctx *c, double *x, double *p) {
    if (x) std::copy(c->ti.x.begin(), c->ti.x.end(), x);
    if (p) std::copy(c->ti.p.begin(), c->ti.p.end(), p);
    return PG_OK;
}
int pg_ti_get_results(pg_ctx *c, double *dhdr_sum, int64_t *nsamples, int64_t *nreinit, int32_t *status) {
    for (int64_t r = 0; r < c->ti.nrings; r++) {
        const or_ring_result &q = c->ti.res[r];
        if (dhdr_sum) dhdr_sum[r] = q.dhdr_sum;
        if (nsamples) nsamples[r] = q.nsamples;
        if (nreinit) nreinit[r] = q.nreinit;
        if (status) status[r] = q.status ? PG_RING_NAN : 0;
    }
    return PG_OK;
}
int pg_ti_set_accumulators(pg_ctx *c, const double *dhdr_sum, const int64_t *nsamples, int64_t step) {
    for (int64_t r = 0; r < c->ti.nrings; r++) {
        c->ti.res[r].dhdr_sum = dhdr_sum[r];
        c->ti.res[r].nsamples = nsamples[r];
    }
    c->ti.step = step;
    return PG_OK;
}
int pg_ti_lambda_reduce(pg_ctx *c, double *mean, double *var, int64_t *count) {
    const TiBatch &t = c->ti;
    const double bn2 = t.prm.betan * t.prm.betan;
    for (int64_t l = 0; l < t.nlam; l++) {
        double s = 0.0, s2 = 0.0, n = 0.0;
        for (int64_t r = 0; r < t.nrings; r++) {
            if (t.lam[r] != l || t.res[r].status || t.res[r].nsamples <= 0) continue;  // as the library
            const double ns = (double)t.res[r].nsamples;
            const double v = t.res[r].dhdr_sum / ns / bn2;
            s += v;
            s2 += v * v;
            n += 1.0;
        }
        const double m = n > 0 ? s / n : 0.0;
        if (mean) mean[l] = m;
        if (var) var[l] = n > 0 ? s2 / n - m * m : 0.0;
        if (count) count[l] = (int64_t)n;
    }
    return PG_OK;
}
int pg_ti_assemble(int64_t nintegral, const double *weights, const double *mean, const double *var, double betan,
                   double *dA, double *sigmaA, double *qratio) {
    double d = 0.0, s = 0.0;
    for (int64_t i = 0; i < nintegral; i++) {
        if (mean[i] == mean[i]) d += weights[i] * mean[i];  // as the library
        s += weights[i] * weights[i] * var[i];
    }
    *dA = d;
    *sigmaA = s;
    *qratio = std::exp(-d * betan);
    return PG_OK;
}

int pg_ti_advance_timed(pg_ctx *c, int64_t nsteps, double *ms) {  // host wall time
    const auto t0 = std::chrono::steady_clock::now();
    const int rc = pg_ti_advance(c, nsteps);
    if (ms) *ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return rc;
}
int pg_ti_get_form(pg_ctx *c, int64_t, int32_t *form, int64_t *launches) {
    if (form) *form = c->ti.prm.nm_resident ? PG_FORM_FUSED : PG_FORM_PLAIN;
    if (launches) *launches = 1;
    return PG_OK;
}
int pg_ti_release(pg_ctx *c) {
    c->ti = TiBatch();
    return PG_OK;
}
int32_t pg_version(void) { return 0; }
int pg_instanton_fg(pg_ctx *c, int64_t nbeta, int64_t N, const double *x, const double *a, const double *b,
                    const double *betan, double *UM, double *grad) {
    const int64_t nd = ndof(c);
    std::vector<double> g((size_t)nd * N);
    for (int64_t k = 0; k < nbeta; k++) {
        const double u = or_UMforceenergy(&c->pes, c->mass.data(), N, betan[k], x + k * nd * N, a,
                                          b ? b + k * nd : nullptr, c->fixedends, g.data());
        if (UM) UM[k] = u;
        if (grad) std::copy(g.begin(), g.end(), grad + k * nd * N);
    }
    return PG_OK;
}
int pg_splitting_two_beta(double beta1, double ratio1, double beta2, double ratio2, double *delta,
                          double *betabar) {
    const double y1 = std::atanh(ratio1), y2 = std::atanh(ratio2);
    *delta = 2.0 * (y2 - y1) / (beta2 - beta1);
    if (betabar) *betabar = y2 != y1 ? (beta1 * y2 - beta2 * y1) / (y2 - y1) : std::nan("");
    return PG_OK;
}
int pg_irrep_ratios(int64_t nirrep, int64_t nop, const double *chars, const double *rho, double *ratio) {
    for (int64_t i = 0; i < nirrep; i++) {
        double em = 0.0, ep = 0.0;
        for (int64_t g = 0; g < nop; g++) {
            em += (1.0 - chars[i * nop + g]) * rho[g];
            ep += (1.0 + chars[i * nop + g]) * rho[g];
        }
        ratio[i] = em / ep;
    }
    return PG_OK;
}
// not in the stand-in
int pg_nm_transform(pg_ctx *, int64_t, int64_t, const double *, double *, int32_t) { return PG_ERR_ARG; }
int pg_nm_transform_noalloc(int64_t, int64_t, const double *, double *, void *) { return PG_ERR_ARG; }
int pg_propagate_pimd(pg_ctx *, const pg_ti_config *, int64_t, int64_t, const double *, const double *,
                      const double *, const uint64_t *, const uint32_t *, double *, double *, double *, int32_t *) {
    return PG_ERR_ARG;
}
int pg_ti_advance_group(pg_ctx *const *ctxs, int64_t nctx, int64_t nsteps, double *ms) {  // one after another
    const auto t0 = std::chrono::steady_clock::now();
    for (int64_t i = 0; i < nctx; i++)
        if (int rc = pg_ti_advance(ctxs[i], nsteps)) return rc;
    if (ms) *ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return PG_OK;
}
int pg_ti_kernel_times(pg_ctx *, int64_t, int32_t *, double *, int64_t *, double *, const char **) {
    return PG_ERR_ARG;
}
int pg_ti_get_tuning(pg_ctx *, int32_t *, int32_t *, int32_t *) { return PG_ERR_ARG; }

}  // extern "C"
