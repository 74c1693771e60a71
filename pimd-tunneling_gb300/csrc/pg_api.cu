// pg_api.cu -- context management, PES evaluation, the batched NM transform
// and the host-side assembly helpers of the C-ABI (include/pimdgpu.h).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "pg_hessian.cuh"
#include "pg_internal.h"

namespace pg {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }

int fail(int code, const std::string &msg) {
    set_error(msg);
    return code;
}

int cuda_fail(cudaError_t e, const char *what) {
    std::string m = std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e);
    set_error(m);
    return PG_ERR_CUDA;
}

int check_ctx(pg_ctx *ctx, bool need_system) {
    if (!ctx) return fail(PG_ERR_ARG, "null context");
    if (need_system && !ctx->have_system) return fail(PG_ERR_STATE, "pg_set_system has not been called");
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    return PG_OK;
}

// ---------------------------------------------------------------- kernels
__global__ void k_pes_eval_d(PesArgs pa, int64_t nconf, const double *__restrict__ x,
                             double *__restrict__ V, double *__restrict__ grad) {
    int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= nconf) return;
    double xb[kMaxDof], gb[kMaxDof];
    for (int i = 0; i < pa.nd; i++) xb[i] = x[c * pa.nd + i];
    double v = pes_vgrad<double>(pa, xb, gb);
    if (V) V[c] = v;
    if (grad)
        for (int i = 0; i < pa.nd; i++) grad[c * pa.nd + i] = gb[i];
}

__global__ void k_pes_eval_f(PesArgs pa, int64_t nconf, const double *__restrict__ x,
                             double *__restrict__ V, double *__restrict__ grad) {
    int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= nconf) return;
    float xb[kMaxDof], gb[kMaxDof];
    for (int i = 0; i < pa.nd; i++) xb[i] = (float)x[c * pa.nd + i];
    float v = pes_vgrad<float>(pa, xb, gb);
    if (V) V[c] = (double)v;
    if (grad)
        for (int i = 0; i < pa.nd; i++) grad[c * pa.nd + i] = (double)gb[i];
}

// One thread per (configuration, column) for finite-difference surfaces, one
// thread per configuration for analytic ones.
__global__ void k_pes_hessian(PesArgs pa, int64_t nconf, const double *__restrict__ x,
                              double *__restrict__ hess, int quirks, int fd) {
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int64_t nd2 = (int64_t)pa.nd * pa.nd;
    if (fd) {
        int64_t c = t / pa.nd;
        int a = (int)(t % pa.nd);
        if (c >= nconf) return;
        double xb[kMaxDof];
        for (int i = 0; i < pa.nd; i++) xb[i] = x[c * pa.nd + i];
        hess_fd_column(pa, xb, a, hess + c * nd2);
    } else {
        if (t >= nconf) return;
        double xb[kMaxDof];
        for (int i = 0; i < pa.nd; i++) xb[i] = x[t * pa.nd + i];
        pes_hessian(pa, xb, hess + t * nd2, quirks);
    }
}

// out[:, c] = T in[:, c], T read from the FP64 reference table (coalesced in i).
__global__ void k_nm_transform_d(int P, int64_t ncol, const double *__restrict__ T,
                                 const double *__restrict__ in, double *__restrict__ out) {
    extern __shared__ double sv[];
    int64_t c = blockIdx.x;
    for (int k = threadIdx.x; k < P; k += blockDim.x) sv[k] = in[c * P + k];
    __syncthreads();
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        double s = 0.0;
        for (int k = 0; k < P; k++) s += T[(int64_t)k * P + i] * sv[k];
        out[c * P + i] = s;
    }
}

__global__ void k_nm_transform_f(int P, int64_t ncol, const double *__restrict__ T,
                                 const double *__restrict__ in, double *__restrict__ out) {
    extern __shared__ float sf[];
    int64_t c = blockIdx.x;
    for (int k = threadIdx.x; k < P; k += blockDim.x) sf[k] = (float)in[c * P + k];
    __syncthreads();
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        float s = 0.f;
        for (int k = 0; k < P; k++) s = fmaf((float)T[(int64_t)k * P + i], sf[k], s);
        out[c * P + i] = (double)s;
    }
}

// Host: T_il = sin(i l pi/(P+1)) sqrt(2/(P+1)) with the reference's pi (verletmodule.f90:318-320).
void build_transmatrix(int P, std::vector<double> &T) {
    T.assign((size_t)P * P, 0.0);
    for (int i = 1; i <= P; i++)
        for (int l = i; l <= P; l++) {
            double t = std::sin((double)((int64_t)i * l) * kPiRef / (double)(P + 1)) *
                       std::sqrt(2.0 / (double)(P + 1));
            T[(size_t)(i - 1) + (size_t)P * (l - 1)] = t;
            T[(size_t)(l - 1) + (size_t)P * (i - 1)] = t;
        }
}

}  // namespace pg

using namespace pg;

// ---------------------------------------------------------------- context
extern "C" int32_t pg_version(void) { return 10000; }

extern "C" const char *pg_last_error(void) { return g_last_error.c_str(); }

extern "C" int pg_create(pg_ctx **out, int32_t device) {
    if (!out) return fail(PG_ERR_ARG, "null output pointer");
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0)
        return fail(PG_ERR_CUDA, "no CUDA device available (this library has no CPU fallback)");
    if (device < 0 || device >= n) return fail(PG_ERR_ARG, "device index out of range");
    e = cudaSetDevice(device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    pg_ctx *c = new pg_ctx();
    c->device = device;
    e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete c;
        return cuda_fail(e, "cudaStreamCreate");
    }
    cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
    *out = c;
    return PG_OK;
}

extern "C" int pg_destroy(pg_ctx *ctx) {
    if (!ctx) return PG_OK;
    cudaSetDevice(ctx->device);
    ti_release(ctx);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return PG_OK;
}

extern "C" int pg_set_system(pg_ctx *ctx, int64_t ndim, int64_t natom, const double *mass,
                             int32_t pes_id, const double *params, int64_t nparams, double V0) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if (ndim < 1 || natom < 1 || ndim * natom > kMaxDof)
        return fail(PG_ERR_ARG, "ndim*natom must be in [1, 64]");
    if (!mass) return fail(PG_ERR_ARG, "mass is NULL");
    if (pes_id < PG_PES_1D || pes_id > PG_PES_DISTGAUSS) return fail(PG_ERR_ARG, "unknown pes_id");
    if (nparams < 0 || (nparams > 0 && !params)) return fail(PG_ERR_ARG, "bad params");
    if (pes_id == PG_PES_2DTEST && (ndim * natom != 2)) return fail(PG_ERR_ARG, "2dtest needs ndof = 2");
    if (pes_id == PG_PES_2DTEST && nparams >= 1 && (params[0] < 1 || params[0] > 6))
        return fail(PG_ERR_ARG, "2dtest supports 1..6 wells");
    if (pes_id == PG_PES_SYNTH9 || pes_id == PG_PES_SYNTH18) {
        if (ndim != 3) return fail(PG_ERR_ARG, "synthetic molecular surfaces need ndim = 3");
        if (nparams < 1) return fail(PG_ERR_ARG, "synthetic surfaces need parameters");
    }
    if (pes_id == PG_PES_SYNTH9) {
        int64_t np = (int64_t)params[0];
        if (np < 0 || nparams < 1 + 5 * np + 5) return fail(PG_ERR_ARG, "synth9 parameter vector too short");
        for (int64_t q = 0; q < np; q++) {
            int64_t i = (int64_t)params[1 + 5 * q], j = (int64_t)params[2 + 5 * q];
            if (i < 0 || j < 0 || i >= natom || j >= natom || i == j)
                return fail(PG_ERR_ARG, "synth9 pair index out of range");
        }
        for (int k = 0; k < 3; k++) {
            int64_t a = (int64_t)params[1 + 5 * np + k];
            if (a < 0 || a >= natom) return fail(PG_ERR_ARG, "synth9 atom index out of range");
        }
    }
    if (pes_id == PG_PES_SYNTH18) {
        if (nparams < 9 || (int64_t)params[0] * 3 != natom)
            return fail(PG_ERR_ARG, "synth18 needs 9 parameters and natom = 3*nmol");
    }
    if (pes_id == PG_PES_DISTGAUSS) {
        if (ndim != 3 || natom < 2) return fail(PG_ERR_ARG, "distgauss needs ndim = 3 and natom >= 2");
        if (nparams < 6 || (int64_t)params[0] != natom) return fail(PG_ERR_ARG, "distgauss header: natom mismatch");
        const int64_t nm = (int64_t)params[2], n1 = (int64_t)params[3], n2 = (int64_t)params[4],
                      n3 = (int64_t)params[5];
        if (nm < 0 || n1 < 0 || n2 < 0 || n3 < 0 || nparams != 6 + 4 * nm + 5 * n1 + 8 * n2 + 11 * n3)
            return fail(PG_ERR_ARG, "distgauss: parameter count does not match the term counts");
        const int64_t npair = natom * (natom - 1) / 2;
        const double *q = params + 6;
        const int64_t width[4] = {4, 5, 8, 11}, nidx[4] = {1, 1, 2, 3}, count[4] = {nm, n1, n2, n3};
        for (int t = 0; t < 4; t++)
            for (int64_t i = 0; i < count[t]; i++, q += width[t])
                for (int64_t c = 0; c < nidx[t]; c++)
                    if (!(q[c] >= 0.0 && q[c] < (double)npair && q[c] == std::floor(q[c])))
                        return fail(PG_ERR_ARG, "distgauss: distance index out of range");
    }
    for (int64_t i = 0; i < natom; i++)
        if (!(mass[i] > 0.0)) return fail(PG_ERR_ARG, "masses must be positive");
    ti_release(ctx);
    ctx->ndim = (int)ndim;
    ctx->natom = (int)natom;
    ctx->nd = (int)(ndim * natom);
    ctx->pes_id = pes_id;
    ctx->V0 = V0;
    ctx->mass.assign(mass, mass + natom);
    ctx->params.assign(params, params + nparams);
    ctx->canon9 = 0;
    if (pes_id == PG_PES_SYNTH9 && natom == 9 && ndim == 3 && nparams >= 1 + 5 * 36 + 5 && params[0] == 36.0) {
        int q = 0, ok = 1;
        for (int i = 0; i < 9; i++)
            for (int j = i + 1; j < 9; j++, q++)
                if (params[1 + 5 * q] != (double)i || params[2 + 5 * q] != (double)j) ok = 0;
        for (int k = 0; k < 3; k++) {  // the quartic's atoms lie in 0..8
            const double a = params[1 + 5 * 36 + k];
            if (!(a >= 0.0 && a <= 8.0 && a == (double)(int)a)) ok = 0;
        }
        ctx->canon9 = ok;
    }
    PG_CUDA(ctx->d_params.ensure(sizeof(double) * (nparams > 0 ? nparams : 1)));
    if (nparams > 0)
        PG_CUDA(cudaMemcpyAsync(ctx->d_params.ptr, ctx->params.data(), sizeof(double) * nparams,
                                cudaMemcpyHostToDevice, ctx->stream));
    {
        // FP32 copy for the FP32 surfaces; the 2-D surface's well centres follow
        // (FP64 cos / sin as in mcmod_2dtest.f90:16-24, rounded once)
        std::vector<float> fp(params, params + nparams);
        if (pes_id == PG_PES_2DTEST) {
            int m = nparams >= 4 ? (int)params[0] : 6;
            double rho0 = nparams >= 4 ? params[3] : 3.0;
            for (int k = 0; k < 6; k++) {
                bool in = k < m;
                fp.push_back(in ? (float)(rho0 * std::cos((double)(k + 1) * 2.0 * kPiRef / (double)m)) : 0.f);
                fp.push_back(in ? (float)(rho0 * std::sin((double)(k + 1) * 2.0 * kPiRef / (double)m)) : 0.f);
            }
        }
        ctx->fparams = fp;
        PG_CUDA(ctx->d_fparams.ensure(sizeof(float) * (fp.size() > 0 ? fp.size() : 1)));
        if (!fp.empty())
            PG_CUDA(cudaMemcpyAsync(ctx->d_fparams.ptr, ctx->fparams.data(), sizeof(float) * fp.size(),
                                    cudaMemcpyHostToDevice, ctx->stream));
    }
    PG_CUDA(ctx->d_mass.ensure(sizeof(double) * natom));
    PG_CUDA(cudaMemcpyAsync(ctx->d_mass.ptr, ctx->mass.data(), sizeof(double) * natom, cudaMemcpyHostToDevice,
                            ctx->stream));
    PG_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->have_system = true;
    return PG_OK;
}

// ---------------------------------------------------------------- PES
extern "C" int pg_pes_eval(pg_ctx *ctx, int64_t nconf, const double *x, double *V, double *grad,
                           int32_t precision) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (nconf < 0 || (nconf > 0 && !x)) return fail(PG_ERR_ARG, "bad x / nconf");
    if (nconf == 0) return PG_OK;
    if (precision != PG_FP64 && precision != PG_MIXED) return fail(PG_ERR_ARG, "bad precision");
    size_t nx = (size_t)nconf * ctx->nd;
    PG_CUDA(ctx->scratch_a.ensure(nx * sizeof(double)));
    PG_CUDA(ctx->scratch_b.ensure(nx * sizeof(double)));
    PG_CUDA(ctx->scratch_c.ensure((size_t)nconf * sizeof(double)));
    PG_CUDA(cudaMemcpyAsync(ctx->scratch_a.ptr, x, nx * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    int bs = 128;
    int64_t nb = (nconf + bs - 1) / bs;
    double *dV = V ? ctx->scratch_c.as<double>() : nullptr;
    double *dg = grad ? ctx->scratch_b.as<double>() : nullptr;
    if (precision == PG_FP64)
        k_pes_eval_d<<<(unsigned)nb, bs, 0, ctx->stream>>>(ctx->pes_args(), nconf, ctx->scratch_a.as<double>(), dV, dg);
    else
        k_pes_eval_f<<<(unsigned)nb, bs, 0, ctx->stream>>>(ctx->pes_args(), nconf, ctx->scratch_a.as<double>(), dV, dg);
    PG_CUDA(cudaGetLastError());
    if (V) PG_CUDA(cudaMemcpyAsync(V, dV, nconf * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    if (grad) PG_CUDA(cudaMemcpyAsync(grad, dg, nx * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    PG_CUDA(cudaStreamSynchronize(ctx->stream));
    return PG_OK;
}

extern "C" int pg_pes_hessian(pg_ctx *ctx, int64_t nconf, const double *x, double *hess,
                              int32_t quirks) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (nconf < 0 || (nconf > 0 && (!x || !hess))) return fail(PG_ERR_ARG, "bad x / hess / nconf");
    if (nconf == 0) return PG_OK;
    size_t nx = (size_t)nconf * ctx->nd, nh = nx * ctx->nd;
    PG_CUDA(ctx->scratch_a.ensure(nx * sizeof(double)));
    PG_CUDA(ctx->scratch_b.ensure(nh * sizeof(double)));
    PG_CUDA(cudaMemcpyAsync(ctx->scratch_a.ptr, x, nx * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    int fd = (ctx->pes_id == PG_PES_1D || ctx->pes_id == PG_PES_SYNTH18 || ctx->pes_id == PG_PES_DISTGAUSS) ? 1 : 0;
    int64_t nthreads = fd ? nconf * ctx->nd : nconf;
    int bs = 128;
    k_pes_hessian<<<(unsigned)((nthreads + bs - 1) / bs), bs, 0, ctx->stream>>>(
        ctx->pes_args(), nconf, ctx->scratch_a.as<double>(), ctx->scratch_b.as<double>(), quirks, fd);
    PG_CUDA(cudaGetLastError());
    PG_CUDA(cudaMemcpyAsync(hess, ctx->scratch_b.ptr, nh * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    PG_CUDA(cudaStreamSynchronize(ctx->stream));
    return PG_OK;
}

// ---------------------------------------------------------------- FP32 peak
// Measurement helper for the roofline of the SIMT work: FP32 FMA throughput of
// this GPU, 8 independent chains per thread, as scalar FMAs or as packed f32x2
// FMAs (one instruction, two lanes of work).
template <bool PAIRED>
__global__ void __launch_bounds__(256) k_fp32_fma(float *__restrict__ out, int iters, float mul, float add) {
    const float s = 1e-3f * (float)(threadIdx.x + 1);
    if (PAIRED) {
        uint64_t acc[8], m2, a2;
        asm("mov.b64 %0, {%1, %1};" : "=l"(m2) : "f"(mul));
        asm("mov.b64 %0, {%1, %1};" : "=l"(a2) : "f"(add));
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const float v = s + (float)j;
            asm("mov.b64 %0, {%1, %2};" : "=l"(acc[j]) : "f"(v), "f"(-v));
        }
        for (int it = 0; it < iters; it++)
#pragma unroll
            for (int j = 0; j < 8; j++) asm volatile("fma.rn.f32x2 %0, %0, %1, %2;" : "+l"(acc[j]) : "l"(m2), "l"(a2));
        float t = 0.f;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            float lo, hi;
            asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(acc[j]));
            t += lo + hi;
        }
        if (t == 12345.678f) out[0] = t;  // keeps the chains live; never true in practice
    } else {
        float acc[8];
#pragma unroll
        for (int j = 0; j < 8; j++) acc[j] = s + (float)j;
        for (int it = 0; it < iters; it++)
#pragma unroll
            for (int j = 0; j < 8; j++) asm volatile("fma.rn.f32 %0, %0, %1, %2;" : "+f"(acc[j]) : "f"(mul), "f"(add));
        float t = 0.f;
#pragma unroll
        for (int j = 0; j < 8; j++) t += acc[j];
        if (t == 12345.678f) out[0] = t;
    }
}

extern "C" int pg_fp32_peak(pg_ctx *ctx, double *tflops) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if (!tflops) return fail(PG_ERR_ARG, "NULL tflops");
    PG_CUDA(ctx->scratch_a.ensure(64));
    float *out = ctx->scratch_a.as<float>();
    const unsigned grid = (unsigned)ctx->sm_count * 4;
    const int iters = 16384;
    cudaEvent_t e0, e1;
    PG_CUDA(cudaEventCreate(&e0));
    PG_CUDA(cudaEventCreate(&e1));
    double best = 0.0;
    for (int paired = 0; paired < 2; paired++) {
        for (int rep = 0; rep < 4; rep++) {
            PG_CUDA(cudaEventRecord(e0, ctx->stream));
            if (paired)
                k_fp32_fma<true><<<grid, 256, 0, ctx->stream>>>(out, iters, 0.999f, 1e-4f);
            else
                k_fp32_fma<false><<<grid, 256, 0, ctx->stream>>>(out, iters, 0.999f, 1e-4f);
            PG_CUDA(cudaGetLastError());
            PG_CUDA(cudaEventRecord(e1, ctx->stream));
            PG_CUDA(cudaEventSynchronize(e1));
            float ms = 0.f;
            PG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            const double flops = 2.0 * 8.0 * (paired ? 2.0 : 1.0) * iters * (double)grid * 256.0;
            if (rep > 0 && ms > 0.f) best = std::max(best, flops / (ms * 1e-3) / 1e12);  // rep 0: warm-up
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *tflops = best;
    return PG_OK;
}

extern "C" int pg_set_wait_limit(pg_ctx *ctx, int64_t ns) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if (ns < 0 || ns > (int64_t)60000000000LL) return fail(PG_ERR_ARG, "wait limit must lie in [0, 60 s]");
    ctx->wait_ns = ns;
    return PG_OK;
}

// ---------------------------------------------------------------- NM transform
extern "C" int pg_nm_transform(pg_ctx *ctx, int64_t P, int64_t ncol, const double *in, double *out,
                               int32_t precision) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if (P < 1 || P > 4096 || ncol < 0 || (ncol > 0 && (!in || !out)))
        return fail(PG_ERR_ARG, "bad P / ncol / buffers");
    if (ncol == 0) return PG_OK;
    if (precision == PG_MIXED && P == 128 && tc_built()) return tc_nm_transform(ctx, P, ncol, in, out);
    std::vector<double> T;
    build_transmatrix((int)P, T);
    size_t n = (size_t)P * ncol;
    PG_CUDA(ctx->scratch_a.ensure(n * sizeof(double)));
    PG_CUDA(ctx->scratch_b.ensure(n * sizeof(double)));
    PG_CUDA(ctx->scratch_c.ensure((size_t)P * P * sizeof(double)));
    PG_CUDA(cudaMemcpyAsync(ctx->scratch_c.ptr, T.data(), (size_t)P * P * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    PG_CUDA(cudaMemcpyAsync(ctx->scratch_a.ptr, in, n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    if (precision == PG_FP64)
        k_nm_transform_d<<<(unsigned)ncol, 128, P * sizeof(double), ctx->stream>>>(
            (int)P, ncol, ctx->scratch_c.as<double>(), ctx->scratch_a.as<double>(), ctx->scratch_b.as<double>());
    else
        k_nm_transform_f<<<(unsigned)ncol, 128, P * sizeof(float), ctx->stream>>>(
            (int)P, ncol, ctx->scratch_c.as<double>(), ctx->scratch_a.as<double>(), ctx->scratch_b.as<double>());
    PG_CUDA(cudaGetLastError());
    PG_CUDA(cudaMemcpyAsync(out, ctx->scratch_b.ptr, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    PG_CUDA(cudaStreamSynchronize(ctx->stream));
    return PG_OK;
}

// ---------------------------------------------------------------- host assembly
extern "C" int pg_gauleg(double x1, double x2, double *x, double *w, int64_t n) {
    if (n < 1 || !x || !w) return fail(PG_ERR_ARG, "bad gauleg arguments");
    const double EPS = 3.0e-14;  // verletmodule.f90:128-129
    int64_t m = (n + 1) / 2;
    double xm = 0.5 * (x2 + x1), xl = 0.5 * (x2 - x1);
    for (int64_t i = 1; i <= m; i++) {
        double z = std::cos(kPiRef * ((double)i - 0.25) / ((double)n + 0.5));
        double z1, pp, p1, p2, p3;
        int guard = 0;
        do {
            p1 = 1.0;
            p2 = 0.0;
            for (int64_t j = 1; j <= n; j++) {
                p3 = p2;
                p2 = p1;
                p1 = ((2.0 * (double)j - 1.0) * z * p2 - ((double)j - 1.0) * p3) / (double)j;
            }
            pp = (double)n * (z * p1 - p2) / (z * z - 1.0);
            z1 = z;
            z = z1 - p1 / pp;
        } while (std::fabs(z - z1) > EPS && ++guard < 100);
        x[i - 1] = xm - xl * z;
        x[n - i] = xm + xl * z;
        w[i - 1] = 2.0 * xl / ((1.0 - z * z) * pp * pp);
        w[n - i] = w[i - 1];
    }
    return PG_OK;
}

extern "C" int pg_spline(const double *x, const double *y, int64_t n, double yp1, double ypn, double *y2) {
    if (n < 2 || !x || !y || !y2) return fail(PG_ERR_ARG, "spline needs n >= 2 points");
    std::vector<double> a(n, 0.0), b(n, 0.0), c(n, 0.0), r(n, 0.0), ro;
    for (int64_t i = 0; i < n - 1; i++) {
        c[i] = x[i + 1] - x[i];
        if (c[i] == 0.0) return fail(PG_ERR_ARG, "spline abscissae must be distinct");
    }
    for (int64_t i = 0; i < n - 1; i++) r[i] = 6.0 * ((y[i + 1] - y[i]) / c[i]);
    ro = r;
    for (int64_t i = 1; i < n - 1; i++) r[i] = ro[i] - ro[i - 1];
    for (int64_t i = 1; i < n - 1; i++) a[i] = c[i - 1];
    for (int64_t i = 1; i < n - 1; i++) b[i] = 2.0 * (c[i] + a[i]);
    b[0] = 1.0;
    b[n - 1] = 1.0;
    if (yp1 > 0.99e30) {
        r[0] = 0.0;
        c[0] = 0.0;
    } else {
        r[0] = (3.0 / (x[1] - x[0])) * ((y[1] - y[0]) / (x[1] - x[0]) - yp1);
        c[0] = 0.5;
    }
    if (ypn > 0.99e30) {
        r[n - 1] = 0.0;
        a[n - 1] = 0.0;
    } else {
        r[n - 1] = (-3.0 / (x[n - 1] - x[n - 2])) * ((y[n - 1] - y[n - 2]) / (x[n - 1] - x[n - 2]) - ypn);
        a[n - 1] = 0.5;
    }
    // tridag (instantonmod.f90:446-480)
    std::vector<double> gam(n, 0.0);
    double bet = b[0];
    if (bet == 0.0) return fail(PG_ERR_NUMERIC, "tridag: zero pivot");
    y2[0] = r[0] / bet;
    for (int64_t j = 1; j < n; j++) {
        gam[j] = c[j - 1] / bet;
        bet = b[j] - a[j] * gam[j];
        if (bet == 0.0) return fail(PG_ERR_NUMERIC, "tridag: zero pivot");
        y2[j] = (r[j] - a[j] * y2[j - 1]) / bet;
    }
    for (int64_t j = n - 2; j >= 0; j--) y2[j] = y2[j] - gam[j + 1] * y2[j + 1];
    return PG_OK;
}

static int64_t nr_locate(const double *xx, int64_t n, double x) {
    bool ascnd = xx[n - 1] >= xx[0];
    int64_t jl = 0, ju = n + 1;
    while (ju - jl > 1) {
        int64_t jm = (ju + jl) / 2;
        if (ascnd == (x >= xx[jm - 1]))
            jl = jm;
        else
            ju = jm;
    }
    if (x == xx[0]) return 1;
    if (x == xx[n - 1]) return n - 1;
    return jl;
}

extern "C" int pg_splint(const double *xa, const double *ya, const double *y2a, int64_t n, double x,
                         double *y, double *dydx) {
    if (n < 2 || !xa || !ya || !y2a) return fail(PG_ERR_ARG, "splint needs n >= 2 points");
    int64_t klo = nr_locate(xa, n, x);
    if (klo > n - 1) klo = n - 1;
    if (klo < 1) klo = 1;
    int64_t khi = klo + 1;
    double h = xa[khi - 1] - xa[klo - 1];
    if (h == 0.0) return fail(PG_ERR_ARG, "bad xa input in splint");
    double a = (xa[khi - 1] - x) / h, b = (x - xa[klo - 1]) / h;
    if (y)
        *y = a * ya[klo - 1] + b * ya[khi - 1] +
             ((a * a * a - a) * y2a[klo - 1] + (b * b * b - b) * y2a[khi - 1]) * (h * h) / 6.0;
    if (dydx)
        *dydx = ((ya[khi - 1] - ya[klo - 1]) / h) +
                ((1.0 - 3.0 * a * a) * y2a[klo - 1] + (3.0 * b * b - 1.0) * y2a[khi - 1]) * h / 6.0;
    return PG_OK;
}

extern "C" int pg_ti_assemble(int64_t nintegral, const double *weights, const double *mean,
                              const double *var, double betan, double *dA, double *sigmaA,
                              double *qratio) {
    if (nintegral < 1 || !weights || !mean || !var) return fail(PG_ERR_ARG, "bad assemble arguments");
    double answer = 0.0, sA = 0.0;
    for (int64_t i = 0; i < nintegral; i++) {
        if (mean[i] == mean[i]) answer += weights[i] * mean[i];
        sA += var[i] * weights[i] * weights[i];
    }
    if (dA) *dA = answer;
    if (sigmaA) *sigmaA = sA;
    if (qratio) *qratio = std::exp(-answer * betan);
    return PG_OK;
}

extern "C" int pg_splitting_from_ratio(double beta, double qratio, double *delta) {
    if (!delta || !(beta > 0.0)) return fail(PG_ERR_ARG, "bad splitting arguments");
    if (!(qratio > -1.0 && qratio < 1.0)) return fail(PG_ERR_NUMERIC, "q/q0 outside (-1, 1)");
    *delta = 2.0 * std::atanh(qratio) / beta;
    return PG_OK;
}

extern "C" int pg_splitting_two_beta(double beta1, double ratio1, double beta2, double ratio2, double *delta,
                                     double *betabar) {
    if (!delta || !(beta1 > 0.0) || !(beta2 > 0.0) || beta1 == beta2)
        return fail(PG_ERR_ARG, "bad two-beta splitting arguments");
    if (!(ratio1 > -1.0 && ratio1 < 1.0) || !(ratio2 > -1.0 && ratio2 < 1.0))
        return fail(PG_ERR_NUMERIC, "ratio outside (-1, 1)");
    const double y1 = std::atanh(ratio1), y2 = std::atanh(ratio2);
    *delta = 2.0 * (y2 - y1) / (beta2 - beta1);
    if (betabar) *betabar = y2 != y1 ? (beta1 * y2 - beta2 * y1) / (y2 - y1) : std::nan("");
    return PG_OK;
}

extern "C" int pg_irrep_ratios(int64_t nirrep, int64_t nop, const double *chars, const double *rho,
                               double *ratio) {
    if (nirrep < 0 || nop < 1 || (nirrep > 0 && (!chars || !rho || !ratio)))
        return fail(PG_ERR_ARG, "bad irrep-ratio arguments");
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

extern "C" int pg_rpi_assemble(double betan, double UM, double lndetJ, double lndetJ0, double *S,
                               double *omega, double *delta) {
    double s = betan * UM;
    double gam = std::exp(0.5 * (lndetJ - lndetJ0));
    double om = betan * std::exp(-s) * std::sqrt(s / (2.0 * kPiRef)) / gam;
    if (S) *S = s;
    if (omega) *omega = om;
    if (delta) *delta = 2.0 * om / betan;
    return PG_OK;
}
