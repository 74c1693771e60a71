// pg_internal.h -- context layout and helpers shared by the library's translation units.
#pragma once
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include "../../include/pimdgpu.h"
#include "pg_device.cuh"

namespace pg {

// NVTX range over an API call (header-only NVTX3: a no-op unless a profiler
// attaches), so that ncu --nvtx filters and timeline tools name the calls.
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

void set_error(const std::string &msg);
int fail(int code, const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);

#define PG_CUDA(call)                                     \
    do {                                                  \
        cudaError_t _e = (call);                          \
        if (_e != cudaSuccess) return cuda_fail(_e, #call); \
    } while (0)

// Device buffer owned by a context.
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    ~DevBuf() { release(); }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
    cudaError_t ensure(size_t nbytes) {
        if (nbytes <= bytes && ptr) return cudaSuccess;
        release();
        cudaError_t e = cudaMalloc(&ptr, nbytes > 0 ? nbytes : 16);
        if (e == cudaSuccess) bytes = nbytes;
        return e;
    }
    template <typename T> T *as() const { return reinterpret_cast<T *>(ptr); }
};

// Per-ring accumulator and scalar state (FP64 estimator accumulation).
struct RingAcc {
    double dhdr_sum;
    int64_t nsamples;
    int64_t nreinit;
    int64_t and_count;
    int64_t and_rkick;
    int32_t status;
    int32_t pad;  // step at which a NaN was first seen
};

// Per (atom, mode) constants of the normal-mode propagator.
struct ModeCoef {
    double rA, rB, rC, rD;  // half-step rotation [pi'; q'] = [rA rB; rC rD] [pi; q]
    double ou_a;            // c1^2
    double ou_s;            // sqrt(beadmass/betan) c2 sqrt(1 + c1^2)
    double pscale;          // sqrt(beadmass/betan): NM Maxwell momentum scale
    double bm;              // beadmass
};

struct TiState {
    pg_ti_config cfg{};
    int64_t nrings = 0, nlambda = 0;
    int P = 0, nd = 0;
    double betan = 0.0;
    int64_t step = 0;
    int form = 0;            // resolved PG_FORM_*
    int tc_blocked = 0;      // tensor form: 0 = fused 64-column tiles (P = 128), 1 = blocked GEMMs (any P)
    int tc_mb = 1;           // blocked tensor form: 128-row blocks of the zero-padded T
    int tf_fused = 0;        // blocked batch run by the persistent folded step (P = 256, k_tf_step)
    bool fp32 = false;       // state held in FP32
    DevBuf q, pi, x, f;      // ring state (fused: NM q/pi + Cartesian x; plain: x/p in x/pi)
    DevBuf T;                // P*P FP64 transform (reference values)
    DevBuf Tbf;              // split-BF16 transform for the tensor-core kernel
    DevBuf sintab;           // 2P+2 scaled sine table, FP64
    DevBuf coef;             // natom*P ModeCoef
    DevBuf bv;               // nlambda*nd*P endpoint shifts (beadvec)
    DevBuf bvtab;            // 3P: the sine and scale tables beadvec is formed from
    DevBuf x0, p0;           // FP64 staging of caller-given start positions / momenta
    DevBuf kickflag;         // per-ring Andersen kick flag (blocked tensor form)
    DevBuf tccol;            // per-column table of the tcgen05 step kernel (spring line, Philox key, weight)
    DevBuf tfimg;            // folded split-BF16 image of T (P = 256) of the persistent folded step
    const void *tf_img_ptr = nullptr;  // the buffer tfimg's image was written to
    // host-side caches across batches: T of the last P, the mode coefficients,
    // and what the tensor-core tables on the device were built from
    std::vector<double> hostT;
    int hostT_P = 0;
    std::vector<ModeCoef> hcoef;
    std::vector<float> tc_tabs;    // FP32 coefficient + folded-map tables last uploaded
    int tc_img_P = 0;              // P of the split image in Tbf (0: none)
    const void *tc_img_ptr = nullptr;
    bool tc_attr = false;          // kernel attributes set
    // launch parameters chosen by the autotuner (0: the built-in choice)
    int simt_threads = 0;          // threads per ring CTA of the fused SIMT kernel (32, 64 or 128)
    int tc_steps = 0;              // MD steps per k_tc_step launch
    DevBuf dbdl;             // nlambda*nd
    DevBuf avec, bvec;       // nd start point, nlambda*nd end points
    DevBuf xref;             // nlambda*nd*P
    DevBuf ringlam, ringseed, ringstream;
    DevBuf acc;              // nrings RingAcc
    DevBuf red;              // reduction output
    std::map<int64_t, cudaGraphExec_t> graphs;
    std::string graph_sig;   // signature of the batch the graphs were captured for
    // pg_ti_advance_group with this context first: one graph over every context
    // of the group, keyed by the step count and all the batches' signatures
    std::map<std::string, cudaGraphExec_t> group_graphs;
    ~TiState();
};

}  // namespace pg

struct pg_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    int sm_count = 0;
    // system (mcmod_mass module state)
    bool have_system = false;
    int ndim = 0, natom = 0, nd = 0, pes_id = 0;
    int canon9 = 0;  // the 9-atom surface's table lists all 36 pairs i < j in order
    double V0 = 0.0;
    std::vector<double> mass, params;
    std::vector<float> fparams;  // host copy of the FP32 surface parameters (PesArgs::fparams)
    pg::DevBuf d_params, d_fparams, d_mass;
    pg::DevBuf scratch_a, scratch_b, scratch_c, scratch_d;
    pg::TiState *ti = nullptr;
    // autotuning of AUTO batches (pg_set_tuning): JSON-lines cache file and mode
    std::string tune_path;
    int tune_mode = 0;
    // instantonmod's module variable fixedends (instantonmod.f90:7): with 0 the
    // polymer action drops the springs to the end points a, b (pg_set_fixedends)
    int fixedends = 1;
    // wall-time bound of the tensor-core transform's device waits (pg_set_wait_limit)
    int64_t wait_ns = 2000000000;
    pg::PesArgs pes_args() const {
        pg::PesArgs pa;
        pa.id = pes_id;
        pa.ndim = ndim;
        pa.natom = natom;
        pa.nd = nd;
        pa.nparams = (int)params.size();
        pa.canon9 = canon9;
        pa.V0 = V0;
        pa.params = d_params.as<double>();
        pa.fparams = d_fparams.as<float>();
        return pa;
    }
};

namespace pg {
int check_ctx(pg_ctx *ctx, bool need_system);
// Launchers implemented in pg_ti.cu / pg_tc.cu / pg_instanton.cu.
int ti_release(pg_ctx *ctx);
int tc_built();
int tc_supported(const TiState &st, const pg_ctx &ctx);
int tf_supported(const TiState &st, const pg_ctx &ctx);  // blocked batch for the persistent folded step
int tc_prepare(pg_ctx *ctx, TiState &st);
int tc_launch(pg_ctx *ctx, TiState &st, int64_t step0, int64_t nsteps, cudaStream_t s);
int tc_nm_transform(pg_ctx *ctx, int64_t P, int64_t ncol, const double *in, double *out);
int32_t tc_error(pg_ctx *ctx, TiState &st);
int tc_kernel_times(pg_ctx *ctx, TiState &st, int64_t nsteps, double *ms, int64_t *count, int *nsub);
int tc_steps_per_launch(const TiState &st);  // MD steps per k_tc_step launch
// dHdrlimit re-initialisation of the flagged rings of a blocked tensor-form
// batch after the estimator computed at step offset sofs (pg_ti.cu)
int ti_launch_reinit(pg_ctx *ctx, TiState &st, int64_t sofs, cudaStream_t s);
}  // namespace pg
