// pg_instanton.cu -- ring-polymer instanton: action, adjoint gradient, L-BFGS, Hessian, log-det.
#include "pg_internal.h"

using namespace pg;

extern "C" int pg_instanton_fg(pg_ctx *ctx, int64_t, int64_t, const double *, const double *,
                               const double *, const double *, double *, double *) {
    (void)ctx;
    return fail(PG_ERR_UNSUPPORTED, "not built yet");
}
extern "C" int pg_instanton_optimize(pg_ctx *, int64_t, int64_t, double *, const double *,
                                     const double *, const double *, const pg_lbfgs_opts *,
                                     double *, int64_t *, int32_t *) {
    return fail(PG_ERR_UNSUPPORTED, "not built yet");
}
extern "C" int pg_um_hessian(pg_ctx *, int64_t, double, const double *, int32_t, int32_t, double *) {
    return fail(PG_ERR_UNSUPPORTED, "not built yet");
}
extern "C" int pg_instanton_logdet(pg_ctx *, int64_t, int64_t, const double *, const double *,
                                   int32_t, int32_t, int32_t, double *, double *, int64_t *) {
    return fail(PG_ERR_UNSUPPORTED, "not built yet");
}
