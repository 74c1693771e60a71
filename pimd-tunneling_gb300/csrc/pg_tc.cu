// pg_tc.cu -- tcgen05 (5th-generation tensor core) kernels for sm_103a.
#include "pg_internal.h"

namespace pg {

int tc_built() { return 0; }
int tc_supported(const TiState &, const pg_ctx &) { return 0; }
int tc_prepare(pg_ctx *, TiState &) { return fail(PG_ERR_UNSUPPORTED, "tensor-core form not built"); }
int tc_launch(pg_ctx *, TiState &, int64_t, int64_t nsteps, cudaStream_t) {
    if (nsteps < 0) return PG_OK;
    return fail(PG_ERR_UNSUPPORTED, "tensor-core form not built");
}
int tc_nm_transform(pg_ctx *, int64_t, int64_t, const double *, double *) {
    return fail(PG_ERR_UNSUPPORTED, "tensor-core transform not built");
}

}  // namespace pg
