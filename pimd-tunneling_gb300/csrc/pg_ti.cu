// pg_ti.cu -- TI-PIMD propagation on the GPU.
//
//  * Fused persistent SIMT kernel (FP64 or FP32 state): one CTA per ring runs
//    many MD steps in one launch.  The state is held in normal-mode space
//    (q = T x - beadvec, pi = T p), so a Langevin step needs two transforms
//    (T F for the kick, T (q + beadvec) for the positions) instead of the
//    reference's ten (verletmodule.f90:423-435, 494-561, 634-667); T is
//    symmetric and its own inverse, so both orders give the same dynamics in
//    exact arithmetic.
//  * Plain form (FP64): per-step kernel launches in the reference step order
//    with ten transforms per Langevin step -- the "plain FP64" denominator.
//  * Device-side per-lambda reduction of the TI integrand (pimd_par.f90:379,
//    401-409) and bitwise checkpoint / restart.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "pg_internal.h"
#include "pg_tune.h"

namespace pg {

void build_transmatrix(int P, std::vector<double> &T);

TiState::~TiState() {
    for (auto &kv : graphs) cudaGraphExecDestroy(kv.second);
    graphs.clear();
    for (auto &kv : group_graphs) cudaGraphExecDestroy(kv.second);
    group_graphs.clear();
}

// ---------------------------------------------------------------- device params
struct TiArgs {
    PesArgs pes;
    int P, nd, ndim, natom;
    int64_t nrings;
    double dt, betan;
    int64_t imin;
    double noutput;
    double dhdr_limit, init_sigma;
    const double *mass;       // natom
    const ModeCoef *coef;     // natom*P
    const double *T;          // P*P FP64
    const float *Tf;          // P*P FP32 copy
    const double *bv;         // nlambda*nd*P
    const double *avec;       // nd: fixed start point a
    const double *bvec;       // nlambda*nd: end points b
    const double *dbdl;       // nlambda*nd
    const double *xref;       // nlambda*nd*P
    const int32_t *ringlam;
    const uint64_t *ringseed;
    const uint32_t *ringstream;
    RingAcc *acc;
    const int64_t *step_dev;  // global step counter (device)
};

template <typename R> __device__ __forceinline__ const R *tmat(const TiArgs &a);
template <> __device__ __forceinline__ const double *tmat<double>(const TiArgs &a) { return a.T; }
template <> __device__ __forceinline__ const float *tmat<float>(const TiArgs &a) { return a.Tf; }

template <typename R> __device__ __forceinline__ bool is_nan(R v) { return v != v; }

// ---------------------------------------------------------------- fused kernel helpers
// Up to kMvDofs dofs of a ring share every read of T in the ring transforms.
constexpr int kMvDofs = 8;

// Shared memory of the kernels that run ring transforms: kMvDofs P-vectors.
inline size_t ring_smem_bytes(int P, bool fp32) {
    return (size_t)kMvDofs * (size_t)P * (fp32 ? sizeof(float) : sizeof(double));
}

// One pass of ring_tmv over NB dofs d0..d0+NB-1 (NB a compile-time width).
template <int NB, typename R, typename Load, typename Store>
__device__ __forceinline__ void ring_tmv_pass(const R *__restrict__ T, int P, int d0, R *__restrict__ sbuf, Load &load,
                                              Store &store) {
    for (int e = threadIdx.x; e < NB * P; e += blockDim.x) {
        const int dd = e / P, k = e - dd * P;
        sbuf[k * NB + dd] = load(d0 + dd, k);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        R acc[NB];
#pragma unroll
        for (int dd = 0; dd < NB; dd++) acc[dd] = (R)0;
        for (int k = 0; k < P; k++) {
            const R t = T[(size_t)k * P + i];
            const R *v = sbuf + k * NB;
#pragma unroll
            for (int dd = 0; dd < NB; dd++) acc[dd] += t * v[dd];
        }
#pragma unroll
        for (int dd = 0; dd < NB; dd++) store(d0 + dd, i, acc[dd]);
    }
    __syncthreads();
}

// store(dof, i, sum_k T[k][i] v[dof][k]) for every (dof, i) of one ring, where
// v[dof][k] = load(dof, k).  Passes of 8, 4, 2 or 1 dofs: v is staged in
// shared memory as sbuf[k][dd], each thread owns outputs i and reads T[k][i]
// once per pass for all dofs of the pass.  Every output sums k = 0..P-1 in
// order (the dsymv-order sum of the CPU restatement).
template <typename R, typename Load, typename Store>
__device__ __forceinline__ void ring_tmv(const TiArgs &a, R *__restrict__ sbuf, Load load, Store store) {
    const R *T = tmat<R>(a);
    const int P = a.P, nd = a.nd;
    int d0 = 0;
    while (d0 < nd) {
        const int left = nd - d0;
        if (left >= 8) {
            ring_tmv_pass<8>(T, P, d0, sbuf, load, store);
            d0 += 8;
        } else if (left >= 4) {
            ring_tmv_pass<4>(T, P, d0, sbuf, load, store);
            d0 += 4;
        } else if (left >= 2) {
            ring_tmv_pass<2>(T, P, d0, sbuf, load, store);
            d0 += 2;
        } else {
            ring_tmv_pass<1>(T, P, d0, sbuf, load, store);
            d0 += 1;
        }
    }
}

// out[dof][i] = sum_k T[k][i] * (in[dof][k] + sh[dof][k])  for all (dof, i) of one ring
// (in == out allowed: a pass stages its dofs before writing them).
template <typename R>
__device__ __forceinline__ void ring_matvec(const TiArgs &a, const R *in, const double *__restrict__ sh, R *out,
                                            R *__restrict__ sbuf) {
    const int P = a.P;
    if (sh)
        ring_tmv<R>(
            a, sbuf, [&](int dof, int k) { return (R)((double)in[dof * P + k] + sh[dof * P + k]); },
            [&](int dof, int i, R v) { out[dof * P + i] = v; });
    else
        ring_tmv<R>(
            a, sbuf, [&](int dof, int k) { return in[dof * P + k]; }, [&](int dof, int i, R v) { out[dof * P + i] = v; });
}

template <typename R>
__device__ __forceinline__ void ring_forces(const TiArgs &a, const R *__restrict__ x,
                                            R *__restrict__ f) {
    const int P = a.P;
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        R xb[kMaxDof], gb[kMaxDof];
        for (int d = 0; d < a.nd; d++) xb[d] = x[d * P + i];
        pes_vgrad<R>(a.pes, xb, gb);
        for (int d = 0; d < a.nd; d++) f[d * P + i] = gb[d];
    }
}

// Half-step free-polymer rotation of every normal mode of one ring.
template <typename R>
__device__ __forceinline__ void ring_rotate(const TiArgs &a, R *__restrict__ q, R *__restrict__ pi) {
    const int P = a.P;
    for (int e = threadIdx.x; e < a.nd * P; e += blockDim.x) {
        int dof = e / P, k = e - dof * P;
        const ModeCoef &c = a.coef[(dof / a.ndim) + a.natom * k];
        R pv = pi[e], qv = q[e];
        pi[e] = (R)c.rA * pv + (R)c.rB * qv;
        q[e] = (R)c.rC * pv + (R)c.rD * qv;
    }
}

__device__ __forceinline__ double ring_contr(const TiArgs &a, const double *dbdl, double xlast,
                                             int dof) {
    return a.mass[dof / a.ndim] * (-xlast) * dbdl[dof];
}

// Spring line of the fixed-end polymer: x*_i = a + (b - a) i/(P+1), i = 1..P.
// T x* = beadvec (verletmodule.f90:326-335), so x = T (q + beadvec) = T q + x*.
__device__ __forceinline__ double xstar(const TiArgs &a, int lam, int dof, int bead) {
    double av = a.avec[dof], bv = a.bvec[(size_t)lam * a.nd + dof];
    return av + (bv - av) * (double)(bead + 1) / (double)(a.P + 1);
}

// Positions x = T (q + beadvec).  FP64: the reference arithmetic.  FP32: T q + x*,
// so the large end-point shift never passes through FP32 rounding.
template <typename R>
__device__ __forceinline__ void ring_positions(const TiArgs &a, int lam, const R *__restrict__ q,
                                               R *__restrict__ x, R *__restrict__ sbuf) {
    if constexpr (sizeof(R) == sizeof(double)) {
        ring_matvec<R>(a, q, a.bv + (size_t)lam * a.nd * a.P, x, sbuf);
    } else {
        ring_matvec<R>(a, q, nullptr, x, sbuf);
        for (int e = threadIdx.x; e < a.nd * a.P; e += blockDim.x) {
            int dof = e / a.P, i = e - dof * a.P;
            x[e] = (R)((double)x[e] + xstar(a, lam, dof, i));
        }
        __syncthreads();
    }
}

// NM coordinates q = T x - beadvec (FP64) or T (x - x*) (FP32).
template <typename R>
__device__ __forceinline__ void ring_nm_coords(const TiArgs &a, int lam, const R *__restrict__ x,
                                               R *__restrict__ q, R *__restrict__ sbuf) {
    const int P = a.P;
    if constexpr (sizeof(R) == sizeof(double)) {
        ring_matvec<R>(a, x, nullptr, q, sbuf);
        const double *bv = a.bv + (size_t)lam * a.nd * P;
        for (int e = threadIdx.x; e < a.nd * P; e += blockDim.x) q[e] = q[e] - bv[e];
        __syncthreads();
    } else {
        ring_tmv<R>(
            a, sbuf, [&](int dof, int k) { return (R)((double)x[dof * P + k] - xstar(a, lam, dof, k)); },
            [&](int dof, int i, R v) { q[dof * P + i] = v; });
    }
}

// Ring (re)initialisation: x = xref + sigma N, pi = pscale N, q = T x - beadvec.
template <typename R>
__device__ void ring_init_state(const TiArgs &a, int64_t r, uint32_t step, uint32_t px,
                                uint32_t pp, R *x, R *q, R *pi, R *sbuf, bool use_x,
                                bool use_p) {
    const int P = a.P;
    const int lam = a.ringlam[r];
    const uint64_t seed = a.ringseed[r];
    const uint32_t stream = a.ringstream[r];
    if (use_x) {
        for (int e = threadIdx.x; e < a.nd * P; e += blockDim.x) {
            double z = a.init_sigma != 0.0 ? normal_d(seed, stream, step, px, (uint32_t)e) : 0.0;
            x[e] = (R)(a.xref[(size_t)lam * a.nd * P + e] + a.init_sigma * z);
        }
    }
    if (use_p) {
        for (int e = threadIdx.x; e < a.nd * P; e += blockDim.x) {
            int dof = e / P, k = e - dof * P;
            double z = normal_d(seed, stream, step, pp, (uint32_t)e);
            pi[e] = (R)(z * sqrt(1.0 / a.betan) * sqrt(a.coef[(dof / a.ndim) + a.natom * k].bm));
        }
    }
    __syncthreads();
    ring_nm_coords<R>(a, lam, x, q, sbuf);
}

// ---------------------------------------------------------------- fused kernel
// One CTA per ring; nsteps MD steps per launch.  THERMO: 1 Andersen, 2 Langevin.
template <typename R, int THERMO>
__global__ void __launch_bounds__(128) k_ti_fused(TiArgs a, R *__restrict__ gq, R *__restrict__ gpi,
                                                  R *__restrict__ gx, R *__restrict__ gf,
                                                  int64_t nsteps) {
    extern __shared__ unsigned char smem_raw[];
    R *sbuf = reinterpret_cast<R *>(smem_raw);
    __shared__ int s_flag;
    __shared__ int s_kick;
    const int64_t r = blockIdx.x;
    if (r >= a.nrings) return;
    const int P = a.P, nd = a.nd;
    const size_t off = (size_t)r * nd * P;
    R *q = gq + off, *pi = gpi + off, *x = gx + off, *f = gf + off;
    const int lam = a.ringlam[r];
    const double *dbdl = a.dbdl + (size_t)lam * nd;
    const uint64_t seed = a.ringseed[r];
    const uint32_t stream = a.ringstream[r];
    RingAcc acc = a.acc[r];
    const int64_t step0 = *a.step_dev;
    const R dt = (R)a.dt;
    if (acc.status) return;  // a ring that saw a NaN stays frozen
    for (int64_t s = step0; s < step0 + nsteps; s++) {
        const uint32_t st = (uint32_t)s;
        if (THERMO == 2) {
            // kick: pi -= dt T grad V(x)
            ring_forces<R>(a, x, f);
            __syncthreads();
            ring_matvec<R>(a, f, nullptr, f, sbuf);  // f <- T f (in place through sbuf per dof)
            if (threadIdx.x == 0) s_flag = 0;
            __syncthreads();
            for (int e = threadIdx.x; e < nd * P; e += blockDim.x) {
                int dof = e / P, k = e - dof * P;
                const ModeCoef &c = a.coef[(dof / a.ndim) + a.natom * k];
                R pv = pi[e] - dt * f[e];
                R qv = q[e];
                // rotate dt/2
                R p1 = (R)c.rA * pv + (R)c.rB * qv;
                R q1 = (R)c.rC * pv + (R)c.rD * qv;
                // OU (verletmodule.f90:651-652)
                R z = normal_r<R>(seed, stream, st, kRngLangevin, (uint32_t)e);
                p1 = (R)c.ou_a * p1 + (R)c.ou_s * z;
                // rotate dt/2
                pi[e] = (R)c.rA * p1 + (R)c.rB * q1;
                q[e] = (R)c.rC * p1 + (R)c.rD * q1;
                if (is_nan(pi[e])) s_flag = 1;
            }
            __syncthreads();
        } else {
            // Andersen schedule (verletmodule.f90:204-234)
            if (threadIdx.x == 0) {
                acc.and_count += 1;
                s_kick = acc.and_count >= acc.and_rkick;
                if (s_kick) {
                    acc.and_count = 0;
                    acc.and_rkick = poisson_d(seed, stream, st, kRngPoisson, a.noutput);
                }
                s_flag = 0;
            }
            __syncthreads();
            if (s_kick) {
                for (int e = threadIdx.x; e < nd * P; e += blockDim.x) {
                    int dof = e / P, k = e - dof * P;
                    double z = normal_d(seed, stream, st, kRngAndersen, (uint32_t)e);
                    pi[e] = (R)(z * sqrt(1.0 / a.betan) * sqrt(a.coef[(dof / a.ndim) + a.natom * k].bm));
                }
                __syncthreads();
            }
            ring_rotate<R>(a, q, pi);
            __syncthreads();
            ring_positions<R>(a, lam, q, x, sbuf);
            ring_forces<R>(a, x, f);
            __syncthreads();
            ring_matvec<R>(a, f, nullptr, f, sbuf);
            for (int e = threadIdx.x; e < nd * P; e += blockDim.x) {
                pi[e] = pi[e] - dt * f[e];
                if (is_nan(pi[e])) s_flag = 1;
            }
            __syncthreads();
            ring_rotate<R>(a, q, pi);
            __syncthreads();
        }
        // positions x = T (q + beadvec)
        ring_positions<R>(a, lam, q, x, sbuf);
        if (s_flag) {
            if (threadIdx.x == 0) {
                acc.status |= PG_RING_NAN;
                acc.pad = (int32_t)s;  // step at which the NaN was seen
            }
            break;
        }
        // estimator (verletmodule.f90:397-409), FP64 accumulation
        if (s >= a.imin) {
            if (threadIdx.x == 0) {
                double contr = 0.0;  // same summation order as verletmodule.f90:399-403
                for (int j = 0; j < a.ndim; j++)
                    for (int k = 0; k < a.natom; k++) {
                        int dof = k * a.ndim + j;
                        contr = contr + ring_contr(a, dbdl, (double)x[dof * P + (P - 1)], dof);
                    }
                acc.nsamples += 1;
                if (THERMO != 2 || fabs(contr) < a.dhdr_limit || a.dhdr_limit < 0.0) {
                    acc.dhdr_sum += contr;
                    s_flag = 0;
                } else {
                    acc.nreinit += 1;
                    s_flag = 2;
                }
            }
            __syncthreads();
            if (s_flag == 2) {
                ring_init_state<R>(a, r, st, kRngReinitX, kRngReinitP, x, q, pi, sbuf, true, true);
                if (threadIdx.x == 0) s_flag = 0;
                __syncthreads();
            }
        }
    }
    if (threadIdx.x == 0) a.acc[r] = acc;
}

// dHdrlimit re-initialisation for the blocked tensor form
// (verletmodule.f90:404-409): a ring whose estimate of step s - 1 went over the
// limit (flagged by the force kernel of step s) starts again from init_path's
// state with the streams the SIMT form uses after step s - 1, and gets the
// forces at its new positions, so that the kick of step s, which follows, runs
// from the re-initialised state.  One CTA per ring; unflagged rings return.
template <typename R>
__global__ void __launch_bounds__(128) k_ti_reinit(TiArgs a, uint8_t *__restrict__ flag, int64_t sofs,
                                                   R *__restrict__ gq, R *__restrict__ gpi, R *__restrict__ gx,
                                                   R *__restrict__ gf) {
    extern __shared__ unsigned char smem_raw[];
    R *sbuf = reinterpret_cast<R *>(smem_raw);
    const int64_t r = blockIdx.x;
    if (r >= a.nrings || !flag[r]) return;  // uniform over the CTA
    const size_t off = (size_t)r * a.nd * a.P;
    const uint32_t st = (uint32_t)(*a.step_dev + sofs - 1);
    ring_init_state<R>(a, r, st, kRngReinitX, kRngReinitP, gx + off, gq + off, gpi + off, sbuf, true, true);
    __syncthreads();
    ring_forces<R>(a, gx + off, gf + off);
    __syncthreads();
    if (threadIdx.x == 0) flag[r] = 0;
}

// Initial state: x from x0 or xref + noise, momenta from p0 or NM Maxwell.
template <typename R>
__global__ void k_ti_init(TiArgs a, R *__restrict__ gq, R *__restrict__ gpi, R *__restrict__ gx,
                          const double *__restrict__ x0, const double *__restrict__ p0) {
    extern __shared__ unsigned char smem_raw[];
    R *sbuf = reinterpret_cast<R *>(smem_raw);
    const int64_t r = blockIdx.x;
    if (r >= a.nrings) return;
    const int P = a.P, nd = a.nd;
    const size_t off = (size_t)r * nd * P;
    R *q = gq + off, *pi = gpi + off, *x = gx + off;
    if (x0)
        for (int e = threadIdx.x; e < nd * P; e += blockDim.x) x[e] = (R)x0[off + e];
    if (p0)
        for (int e = threadIdx.x; e < nd * P; e += blockDim.x) pi[e] = (R)p0[off + e];
    __syncthreads();
    ring_init_state<R>(a, r, 0u, kRngInitX, kRngInitP, x, q, pi, sbuf, x0 == nullptr, p0 == nullptr);
    if (p0) {
        // pi = T p0 (the momenta were given in Cartesian form)
        ring_matvec<R>(a, pi, nullptr, pi, sbuf);
    }
    if (threadIdx.x == 0) {
        RingAcc z;
        z.dhdr_sum = 0.0;
        z.nsamples = 0;
        z.nreinit = 0;
        z.and_count = 0;
        z.and_rkick = poisson_d(a.ringseed[r], a.ringstream[r], 0u, kRngPoisson0, a.noutput);
        z.status = 0;
        z.pad = 0;
        a.acc[r] = z;
    }
}

// Cartesian momenta p = T pi (state read-out).
template <typename R>
__global__ void k_ti_momenta(TiArgs a, const R *__restrict__ gpi, double *__restrict__ pout) {
    extern __shared__ unsigned char smem_raw[];
    R *sbuf = reinterpret_cast<R *>(smem_raw);
    const int64_t r = blockIdx.x;
    if (r >= a.nrings) return;
    const int P = a.P, nd = a.nd;
    const size_t off = (size_t)r * nd * P;
    ring_tmv<R>(
        a, sbuf, [&](int dof, int k) { return gpi[off + dof * P + k]; },
        [&](int dof, int i, R v) { pout[off + dof * P + i] = (double)v; });
}

template <typename R>
__global__ void k_to_double(const R *__restrict__ in, double *__restrict__ out, size_t n) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = (double)in[i];
}

__global__ void k_step_add(int64_t *step_dev, int64_t n) { *step_dev += n; }

// beadvec(i, dof) of every lambda point (verletmodule.f90:326-335) from the
// host's tables: tab[i] = sin(i pi/(P+1)), tab[P + i] = sin(P i pi/(P+1)),
// tab[2P + i] = (lam_i betan)^2, sq = sqrt(2/(P+1)).
__global__ void k_beadvec(const double *__restrict__ a, const double *__restrict__ b,
                          const double *__restrict__ tab, double sq, int64_t nlambda, int nd, int P,
                          double *__restrict__ bv) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nlambda * nd * P) return;
    const int i = (int)(e % P);
    const int64_t ld = e / P;
    const int dof = (int)(ld % nd);
    const int64_t l = ld / nd;
    double v = a[dof] * tab[i] + b[l * nd + dof] * tab[P + i];
    v = v * sq;
    bv[e] = v / tab[2 * P + i];
}

// ---------------------------------------------------------------- plain form (FP64)
// State: x (Cartesian positions), p (Cartesian momenta); scratch wq, wp.
// step_v: p -= dt grad V(x) (verletmodule.f90:565-585); one thread per (ring, bead).
__global__ void k_plain_kick(TiArgs a, const double *__restrict__ x, double *__restrict__ p,
                             double t) {
    int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int64_t r = idx / a.P;
    int i = (int)(idx - r * a.P);
    if (r >= a.nrings) return;
    if (a.acc[r].status) return;
    const size_t off = (size_t)r * a.nd * a.P;
    double xb[kMaxDof], gb[kMaxDof];
    for (int d = 0; d < a.nd; d++) xb[d] = x[off + d * a.P + i];
    pes_vgrad<double>(a.pes, xb, gb);
    bool bad = false;
    for (int d = 0; d < a.nd; d++) {
        double v = p[off + d * a.P + i] - gb[d] * t;
        p[off + d * a.P + i] = v;
        bad |= (v != v);
    }
    if (bad) atomicOr(&a.acc[r].status, PG_RING_NAN);
}

// One dense symmetric matvec per dof, as dsymv (verletmodule.f90:254-286).
__device__ __forceinline__ void plain_mv(const TiArgs &a, const double *__restrict__ in,
                                         const double *__restrict__ sh, double sgn,
                                         double *__restrict__ out, double *sbuf) {
    const int P = a.P;
    for (int dof = 0; dof < a.nd; dof++) {
        for (int k = threadIdx.x; k < P; k += blockDim.x) sbuf[k] = in[dof * P + k];
        __syncthreads();
        for (int i = threadIdx.x; i < P; i += blockDim.x) {
            double s = 0.0;
            for (int k = 0; k < P; k++) s += a.T[(size_t)k * P + i] * sbuf[k];
            out[dof * P + i] = sh ? s + sgn * sh[dof * P + i] : s;
        }
        __syncthreads();
    }
}

// step_nm (verletmodule.f90:494-561): forward transforms, rotation, backward transforms.
__global__ void k_plain_nm(TiArgs a, double *__restrict__ gx, double *__restrict__ gp,
                           double *__restrict__ gq, double *__restrict__ gw) {
    extern __shared__ double sb[];
    const int64_t r = blockIdx.x;
    if (r >= a.nrings || a.acc[r].status) return;
    const int P = a.P, nd = a.nd;
    const size_t off = (size_t)r * nd * P;
    double *x = gx + off, *p = gp + off, *q = gq + off, *w = gw + off;
    const double *bv = a.bv + (size_t)a.ringlam[r] * nd * P;
    plain_mv(a, p, nullptr, 0.0, w, sb);   // pip = T p
    plain_mv(a, x, bv, -1.0, q, sb);       // q = T x - beadvec
    bool bad = false;
    for (int e = threadIdx.x; e < nd * P; e += blockDim.x) {
        int dof = e / P, k = e - dof * P;
        const ModeCoef &c = a.coef[(dof / a.ndim) + a.natom * k];
        double pv = w[e], qv = q[e];
        double np = c.rA * pv + c.rB * qv;
        double nq = c.rC * pv + c.rD * qv;
        w[e] = np;
        q[e] = nq;
        bad |= (np != np);
    }
    if (bad) atomicOr(&a.acc[r].status, PG_RING_NAN);
    __syncthreads();
    plain_mv(a, w, nullptr, 0.0, p, sb);   // p = T pip
    // x = T (q + beadvec)
    for (int e = threadIdx.x; e < nd * P; e += blockDim.x) q[e] = q[e] + bv[e];
    __syncthreads();
    plain_mv(a, q, nullptr, 0.0, x, sb);
}

// step_langevin (verletmodule.f90:634-667).
__global__ void k_plain_langevin(TiArgs a, double *__restrict__ gp, double *__restrict__ gw) {
    extern __shared__ double sb[];
    const int64_t r = blockIdx.x;
    if (r >= a.nrings || a.acc[r].status) return;
    const int P = a.P, nd = a.nd;
    const size_t off = (size_t)r * nd * P;
    double *p = gp + off, *w = gw + off;
    const uint32_t st = (uint32_t)(*a.step_dev);
    plain_mv(a, p, nullptr, 0.0, w, sb);
    for (int e = threadIdx.x; e < nd * P; e += blockDim.x) {
        int dof = e / P, k = e - dof * P;
        const ModeCoef &c = a.coef[(dof / a.ndim) + a.natom * k];
        double z = normal_d(a.ringseed[r], a.ringstream[r], st, kRngLangevin, (uint32_t)e);
        w[e] = c.ou_a * w[e] + c.ou_s * z;
    }
    __syncthreads();
    plain_mv(a, w, nullptr, 0.0, p, sb);
}

// Andersen resampling check (verletmodule.f90:204-234) for the plain form.
__global__ void k_plain_andersen(TiArgs a, double *__restrict__ gp, double *__restrict__ gw) {
    extern __shared__ double sb[];
    __shared__ int s_kick;
    const int64_t r = blockIdx.x;
    if (r >= a.nrings || a.acc[r].status) return;
    const int P = a.P, nd = a.nd;
    const size_t off = (size_t)r * nd * P;
    const uint32_t st = (uint32_t)(*a.step_dev);
    if (threadIdx.x == 0) {
        RingAcc &acc = a.acc[r];
        acc.and_count += 1;
        s_kick = acc.and_count >= acc.and_rkick;
        if (s_kick) {
            acc.and_count = 0;
            acc.and_rkick = poisson_d(a.ringseed[r], a.ringstream[r], st, kRngPoisson, a.noutput);
        }
    }
    __syncthreads();
    if (!s_kick) return;
    double *w = gw + off;
    for (int e = threadIdx.x; e < nd * P; e += blockDim.x) {
        int dof = e / P, k = e - dof * P;
        double z = normal_d(a.ringseed[r], a.ringstream[r], st, kRngAndersen, (uint32_t)e);
        w[e] = z * sqrt(1.0 / a.betan) * sqrt(a.coef[(dof / a.ndim) + a.natom * k].bm);
    }
    __syncthreads();
    plain_mv(a, w, nullptr, 0.0, gp + off, sb);
}

// Estimator + dHdrlimit re-initialisation (verletmodule.f90:397-409) for the plain form.
__global__ void k_plain_estimator(TiArgs a, int thermo, double *__restrict__ gx,
                                  double *__restrict__ gp, double *__restrict__ gw) {
    extern __shared__ double sb[];
    __shared__ int s_re;
    const int64_t r = blockIdx.x;
    if (r >= a.nrings || a.acc[r].status) return;
    const int P = a.P, nd = a.nd;
    const size_t off = (size_t)r * nd * P;
    const int64_t s = *a.step_dev;
    if (s < a.imin) return;
    const int lam = a.ringlam[r];
    const double *dbdl = a.dbdl + (size_t)lam * nd;
    if (threadIdx.x == 0) {
        RingAcc &acc = a.acc[r];
        double contr = 0.0;
        for (int j = 0; j < a.ndim; j++)
            for (int k = 0; k < a.natom; k++) {
                int dof = k * a.ndim + j;
                contr = contr + ring_contr(a, dbdl, gx[off + dof * P + P - 1], dof);
            }
        acc.nsamples += 1;
        s_re = 0;
        if (thermo != 2 || fabs(contr) < a.dhdr_limit || a.dhdr_limit < 0.0) {
            acc.dhdr_sum += contr;
        } else {
            acc.nreinit += 1;
            s_re = 1;
        }
    }
    __syncthreads();
    if (!s_re) return;
    const uint32_t st = (uint32_t)s;
    const uint64_t seed = a.ringseed[r];
    const uint32_t stream = a.ringstream[r];
    double *w = gw + off;
    for (int e = threadIdx.x; e < nd * P; e += blockDim.x) {
        int dof = e / P, k = e - dof * P;
        double zx = a.init_sigma != 0.0 ? normal_d(seed, stream, st, kRngReinitX, (uint32_t)e) : 0.0;
        gx[off + e] = a.xref[(size_t)lam * nd * P + e] + a.init_sigma * zx;
        double z = normal_d(seed, stream, st, kRngReinitP, (uint32_t)e);
        w[e] = z * sqrt(1.0 / a.betan) * sqrt(a.coef[(dof / a.ndim) + a.natom * k].bm);
    }
    __syncthreads();
    plain_mv(a, w, nullptr, 0.0, gp + off, sb);
}

// Plain-form initial state: x, p Cartesian.
__global__ void k_plain_init(TiArgs a, double *__restrict__ gx, double *__restrict__ gp,
                             double *__restrict__ gw, const double *__restrict__ x0,
                             const double *__restrict__ p0) {
    extern __shared__ double sb[];
    const int64_t r = blockIdx.x;
    if (r >= a.nrings) return;
    const int P = a.P, nd = a.nd;
    const size_t off = (size_t)r * nd * P;
    const int lam = a.ringlam[r];
    const uint64_t seed = a.ringseed[r];
    const uint32_t stream = a.ringstream[r];
    for (int e = threadIdx.x; e < nd * P; e += blockDim.x) {
        if (x0) {
            gx[off + e] = x0[off + e];
        } else {
            double z = a.init_sigma != 0.0 ? normal_d(seed, stream, 0u, kRngInitX, (uint32_t)e) : 0.0;
            gx[off + e] = a.xref[(size_t)lam * nd * P + e] + a.init_sigma * z;
        }
        if (p0) {
            gp[off + e] = p0[off + e];
        } else {
            int dof = e / P, k = e - dof * P;
            double z = normal_d(seed, stream, 0u, kRngInitP, (uint32_t)e);
            gw[off + e] = z * sqrt(1.0 / a.betan) * sqrt(a.coef[(dof / a.ndim) + a.natom * k].bm);
        }
    }
    __syncthreads();
    if (!p0) plain_mv(a, gw + off, nullptr, 0.0, gp + off, sb);
    if (threadIdx.x == 0) {
        RingAcc z;
        z.dhdr_sum = 0.0;
        z.nsamples = 0;
        z.nreinit = 0;
        z.and_count = 0;
        z.and_rkick = poisson_d(seed, stream, 0u, kRngPoisson0, a.noutput);
        z.status = 0;
        z.pad = 0;
        a.acc[r] = z;
    }
}

// ---------------------------------------------------------------- K4 reduction
// Per lambda: mean / variance of integrand = dhdr_sum/nsamples/betan^2 over its
// rings (pimd_par.f90:379, 401-409).  One CTA per lambda, warp shuffles.
__global__ void k_lambda_reduce(const RingAcc *__restrict__ acc, const int32_t *__restrict__ ringlam,
                                int64_t nrings, double betan, double *__restrict__ out) {
    const int lam = blockIdx.x;
    double s = 0.0, s2 = 0.0, n = 0.0;
    for (int64_t r = threadIdx.x; r < nrings; r += blockDim.x) {
        // rings that met a NaN (their trajectory stopped there) or hold no
        // sample yet carry no estimate: left out of the mean and the count
        if (ringlam[r] != lam || (acc[r].status & PG_RING_NAN) || acc[r].nsamples <= 0) continue;
        double ns = (double)acc[r].nsamples;
        double v = acc[r].dhdr_sum / ns / (betan * betan);
        s += v;
        s2 += v * v;
        n += 1.0;
    }
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
        n += __shfl_xor_sync(0xffffffffu, n, o);
    }
    __shared__ double sh[3][32];
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) {
        sh[0][w] = s;
        sh[1][w] = s2;
        sh[2][w] = n;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double S = 0, S2 = 0, N = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) {
            S += sh[0][i];
            S2 += sh[1][i];
            N += sh[2][i];
        }
        double mean = N > 0 ? S / N : 0.0;
        double var = N > 0 ? S2 / N - mean * mean : 0.0;
        out[3 * lam + 0] = mean;
        out[3 * lam + 1] = var;
        out[3 * lam + 2] = N;
    }
}

// ---------------------------------------------------------------- host side
static TiArgs make_args(pg_ctx *ctx, TiState &st, int64_t *step_dev) {
    TiArgs a;
    a.pes = ctx->pes_args();
    a.P = st.P;
    a.nd = st.nd;
    a.ndim = ctx->ndim;
    a.natom = ctx->natom;
    a.nrings = st.nrings;
    a.dt = st.cfg.dt;
    a.betan = st.betan;
    a.imin = st.cfg.imin;
    a.noutput = (double)st.cfg.noutput;
    a.dhdr_limit = st.cfg.dhdr_limit;
    a.init_sigma = st.cfg.init_sigma;
    a.mass = ctx->d_mass.as<double>();
    a.coef = st.coef.as<ModeCoef>();
    a.T = st.T.as<double>();
    a.Tf = reinterpret_cast<const float *>(st.T.as<double>() + (size_t)st.P * st.P);
    a.bv = st.bv.as<double>();
    a.avec = st.avec.as<double>();
    a.bvec = st.bvec.as<double>();
    a.dbdl = st.dbdl.as<double>();
    a.xref = st.xref.as<double>();
    a.ringlam = st.ringlam.as<int32_t>();
    a.ringseed = st.ringseed.as<uint64_t>();
    a.ringstream = st.ringstream.as<uint32_t>();
    a.acc = st.acc.as<RingAcc>();
    a.step_dev = step_dev;
    return a;
}

static int64_t *step_ptr(TiState &st) {
    // the global step counter lives in the tail of the reduction buffer
    return reinterpret_cast<int64_t *>(st.red.as<double>() + 3 * st.nlambda);
}

static int threads_for(int P, int nd) {
    int n = P * nd;
    if (n >= 128 || P >= 128) return 128;
    if (n >= 64) return 64;
    return 32;
}

static int launch_steps(pg_ctx *ctx, TiState &st, int64_t nsteps, cudaStream_t s) {
    TiArgs a = make_args(ctx, st, step_ptr(st));
    const int P = st.P, nd = st.nd;
    int th = st.simt_threads > 0 ? st.simt_threads : threads_for(P, nd);
    unsigned grid = (unsigned)st.nrings;
    if (st.form == PG_FORM_TENSOR) return tc_launch(ctx, st, 0, nsteps, s);
    if (st.form == PG_FORM_FUSED) {
        size_t sm = ring_smem_bytes(P, st.fp32);
        int thermo = st.cfg.thermostat;
        if (st.fp32) {
            if (thermo == PG_LANGEVIN)
                k_ti_fused<float, 2><<<grid, th, sm, s>>>(a, st.q.as<float>(), st.pi.as<float>(), st.x.as<float>(), st.f.as<float>(), nsteps);
            else
                k_ti_fused<float, 1><<<grid, th, sm, s>>>(a, st.q.as<float>(), st.pi.as<float>(), st.x.as<float>(), st.f.as<float>(), nsteps);
        } else {
            if (thermo == PG_LANGEVIN)
                k_ti_fused<double, 2><<<grid, th, sm, s>>>(a, st.q.as<double>(), st.pi.as<double>(), st.x.as<double>(), st.f.as<double>(), nsteps);
            else
                k_ti_fused<double, 1><<<grid, th, sm, s>>>(a, st.q.as<double>(), st.pi.as<double>(), st.x.as<double>(), st.f.as<double>(), nsteps);
        }
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return cuda_fail(e, "k_ti_fused launch");
        k_step_add<<<1, 1, 0, s>>>(step_ptr(st), nsteps);
        return PG_OK;
    }
    // plain form: per-step launches in the reference order
    size_t sm = (size_t)P * sizeof(double);
    int64_t nthr = st.nrings * P;
    unsigned kgrid = (unsigned)((nthr + 127) / 128);
    double *x = st.x.as<double>(), *p = st.pi.as<double>(), *q = st.q.as<double>(), *w = st.f.as<double>();
    for (int64_t i = 0; i < nsteps; i++) {
        if (st.cfg.thermostat == PG_LANGEVIN) {
            k_plain_kick<<<kgrid, 128, 0, s>>>(a, x, p, st.cfg.dt);
            k_plain_nm<<<grid, th, sm, s>>>(a, x, p, q, w);
            k_plain_langevin<<<grid, th, sm, s>>>(a, p, w);
            k_plain_nm<<<grid, th, sm, s>>>(a, x, p, q, w);
        } else {
            k_plain_andersen<<<grid, th, sm, s>>>(a, p, w);
            k_plain_nm<<<grid, th, sm, s>>>(a, x, p, q, w);
            k_plain_kick<<<kgrid, 128, 0, s>>>(a, x, p, st.cfg.dt);
            k_plain_nm<<<grid, th, sm, s>>>(a, x, p, q, w);
        }
        k_plain_estimator<<<grid, th, sm, s>>>(a, st.cfg.thermostat, x, p, w);
        k_step_add<<<1, 1, 0, s>>>(step_ptr(st), 1);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "plain-form launch");
    return PG_OK;
}

int ti_launch_reinit(pg_ctx *ctx, TiState &st, int64_t sofs, cudaStream_t s) {
    TiArgs a = make_args(ctx, st, step_ptr(st));
    k_ti_reinit<float><<<(unsigned)st.nrings, threads_for(st.P, st.nd), ring_smem_bytes(st.P, true), s>>>(
        a, st.kickflag.as<uint8_t>(), sofs, st.q.as<float>(), st.pi.as<float>(), st.x.as<float>(), st.f.as<float>());
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? PG_OK : cuda_fail(e, "k_ti_reinit launch");
}

int ti_release(pg_ctx *ctx) {
    if (ctx && ctx->ti) {
        delete ctx->ti;
        ctx->ti = nullptr;
    }
    return PG_OK;
}

// Everything a captured advance graph bakes into its launches: the batch
// shape and configuration, the surface and masses (the tensor kernels take
// surface constants by value), and every device buffer address.
static std::string graph_signature(const pg_ctx *ctx, const TiState &st) {
    std::string sig;
    auto add = [&](const void *p, size_t n) { sig.append(reinterpret_cast<const char *>(p), n); };
    add(&st.cfg, sizeof(st.cfg));
    add(&st.nrings, sizeof(st.nrings));
    add(&st.nlambda, sizeof(st.nlambda));
    int ints[7] = {st.P, st.nd, st.form, st.tc_blocked, st.fp32 ? 1 : 0, ctx->sm_count, st.tf_fused};
    add(ints, sizeof(ints));
    int sys[6] = {ctx->pes_id, ctx->ndim, ctx->natom, ctx->nd, st.simt_threads, st.tc_steps};
    add(sys, sizeof(sys));
    add(&ctx->V0, sizeof(double));
    add(ctx->params.data(), ctx->params.size() * sizeof(double));
    add(ctx->mass.data(), ctx->mass.size() * sizeof(double));
    const void *ptrs[] = {st.q.ptr, st.pi.ptr, st.x.ptr, st.f.ptr, st.T.ptr, st.Tbf.ptr, st.coef.ptr, st.bv.ptr, st.kickflag.ptr, st.tccol.ptr,
                          st.dbdl.ptr, st.avec.ptr, st.bvec.ptr, st.xref.ptr, st.ringlam.ptr, st.ringseed.ptr,
                          st.ringstream.ptr, st.acc.ptr, st.red.ptr, ctx->d_params.ptr, ctx->d_fparams.ptr,
                          ctx->d_mass.ptr};
    add(ptrs, sizeof(ptrs));
    return sig;
}

static int resolve_form(pg_ctx *ctx, TiState &st) {
    int form = st.cfg.form;
    if (st.cfg.precision == PG_FP64) {
        if (form == PG_FORM_TENSOR) return fail(PG_ERR_UNSUPPORTED, "the tensor-core form needs PG_MIXED");
        st.form = (form == PG_FORM_PLAIN) ? PG_FORM_PLAIN : PG_FORM_FUSED;
        st.fp32 = false;
        return PG_OK;
    }
    if (form == PG_FORM_PLAIN) return fail(PG_ERR_UNSUPPORTED, "the plain form is FP64 only");
    st.fp32 = true;
    if (form == PG_FORM_FUSED) {
        st.form = PG_FORM_FUSED;
        return PG_OK;
    }
    const int tcv = tc_supported(st, *ctx);
    if (form == PG_FORM_TENSOR && !tcv)
        return fail(PG_ERR_UNSUPPORTED,
                    "the tensor-core form supports the Langevin (with or without dHdrlimit) and Andersen "
                    "thermostats with P <= 512 and P % 4 == 0");
    // AUTO: the fused tiles whenever they apply; the blocked GEMMs for batches of at
    // least 2^20 bead-dofs (smaller batches leave most of the GPU idle in them).
    bool use = tcv == 1 || (tcv == 2 && (form == PG_FORM_TENSOR || st.nrings * st.nd * st.P >= (1 << 20)));
    st.form = use ? PG_FORM_TENSOR : PG_FORM_FUSED;
    st.tc_blocked = (use && tcv == 2) ? 1 : 0;
    st.tf_fused = (st.tc_blocked && tf_supported(st, *ctx)) ? 1 : 0;
    return PG_OK;
}

}  // namespace pg

using namespace pg;

static int ti_setup_impl(pg_ctx *ctx, const pg_ti_config *cfg, int64_t nrings, int64_t nlambda,
                         const int32_t *ring_lambda, const uint64_t *ring_seed, const uint32_t *ring_stream,
                         const double *a, const double *b, const double *dbdl, const double *xref, const double *x0,
                         const double *p0, int simt_threads, int tc_steps) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (!cfg) return fail(PG_ERR_ARG, "cfg is NULL");
    if (cfg->nbeads < 2 || cfg->nbeads > 1024) return fail(PG_ERR_ARG, "nbeads must be in [2, 1024]");
    if (nrings < 1 || nrings > (int64_t)1 << 30) return fail(PG_ERR_ARG, "nrings out of range");
    if (nlambda < 1 || nlambda > ((int64_t)1 << 26)) return fail(PG_ERR_ARG, "nlambda out of range");
    if (!ring_lambda || !ring_seed || !ring_stream || !a || !b || !dbdl)
        return fail(PG_ERR_ARG, "NULL ring / endpoint array");
    if (!x0 && !xref) return fail(PG_ERR_ARG, "need x0 or xref");
    if (!(cfg->beta > 0.0) || !(cfg->dt > 0.0) || !(cfg->tau > 0.0) || cfg->gamma < 0.0)
        return fail(PG_ERR_ARG, "beta, dt, tau must be > 0 and gamma >= 0");
    if (cfg->thermostat != PG_LANGEVIN && cfg->thermostat != PG_ANDERSEN)
        return fail(PG_ERR_ARG, "thermostat must be 1 (Andersen) or 2 (Langevin)");
    if (cfg->precision != PG_FP64 && cfg->precision != PG_MIXED) return fail(PG_ERR_ARG, "bad precision");
    if (cfg->form < PG_FORM_AUTO || cfg->form > PG_FORM_TENSOR) return fail(PG_ERR_ARG, "bad form");
    if (cfg->imin < 0) return fail(PG_ERR_ARG, "imin must be >= 0");
    for (int64_t r = 0; r < nrings; r++)
        if (ring_lambda[r] < 0 || ring_lambda[r] >= nlambda) return fail(PG_ERR_ARG, "ring_lambda out of range");

    // Reuse the device buffers of a previous batch (ensure() only grows them).
    // Captured graphs bake in launch arguments: they are kept only when the
    // new batch has the same signature (see graph_signature), else dropped.
    if (!ctx->ti) ctx->ti = new TiState();
    TiState &st = *ctx->ti;
    st.cfg = *cfg;
    st.nrings = nrings;
    st.nlambda = nlambda;
    st.P = (int)cfg->nbeads;
    st.nd = ctx->nd;
    st.betan = cfg->beta / (double)(cfg->nbeads + 1);  // pimd_par.f90:94
    st.step = 0;
    st.simt_threads = simt_threads;
    st.tc_steps = tc_steps;
    rc = resolve_form(ctx, st);
    if (rc) {
        ti_release(ctx);
        return rc;
    }
    const int P = st.P, nd = st.nd, natom = ctx->natom;
    const double betan = st.betan;

    // init_nm (verletmodule.f90:306-338): lam, beadmass, beadvec; transmatrix
    if (st.hostT_P != P) {  // T depends on P only
        build_transmatrix(P, st.hostT);
        st.hostT_P = P;
    }
    const std::vector<double> &T = st.hostT;
    std::vector<double> lam(P);
    for (int i = 1; i <= P; i++) lam[i - 1] = 2.0 * std::sin((double)i * kPiRef / (double)(2 * P + 2)) / betan;
    std::vector<ModeCoef> coef((size_t)natom * P);
    const double t = 0.5 * cfg->dt;
    for (int i = 0; i < P; i++)
        for (int k = 0; k < natom; k++) {
            double bm = ctx->mass[k] * (lam[i] * cfg->tau) * (lam[i] * cfg->tau);
            double om = std::sqrt(ctx->mass[k] / bm) * lam[i];  // verletmodule.f90:519
            ModeCoef c;
            if (cfg->cayley) {  // verletmodule.f90:520-526
                double den = 4.0 + om * om * t * t;
                c.rA = (4.0 - om * om * t * t) / den;
                c.rB = -4.0 * bm * om * om * t / den;
                c.rC = 4.0 * t / (bm * den);
                c.rD = c.rA;
            } else {  // verletmodule.f90:528-531
                c.rA = std::cos(t * om);
                c.rB = -om * bm * std::sin(om * t);
                c.rC = std::sin(om * t) / (om * bm);
                c.rD = std::cos(t * om);
            }
            double c1 = std::exp(-cfg->gamma * cfg->dt * lam[i] * std::sqrt(ctx->mass[k] / bm));  // :383
            double c2 = std::sqrt(1.0 - c1 * c1);
            c.ou_a = c1 * c1;
            c.ou_s = std::sqrt(bm / betan) * c2 * std::sqrt(1.0 + c1 * c1);
            c.pscale = std::sqrt(bm / betan);
            c.bm = bm;
            coef[(size_t)k + (size_t)natom * i] = c;
        }
    st.hcoef = coef;
    // beadvec tables (verletmodule.f90:326-335); the nlambda x nd x P values are
    // formed on the device by k_beadvec
    std::vector<double> bvtab(3 * (size_t)P);
    for (int i = 1; i <= P; i++) {
        bvtab[i - 1] = std::sin((double)i * kPiRef / (double)(P + 1));
        bvtab[P + i - 1] = std::sin((double)(P * i) * kPiRef / (double)(P + 1));
        bvtab[2 * P + i - 1] = (lam[i - 1] * betan) * (lam[i - 1] * betan);
    }
    const double bvsq = std::sqrt(2.0 / (double)(P + 1));
    // the reference positions are read only to initialise rings without x0 and
    // by dHdrlimit re-initialisation
    const bool need_xref = !x0 || cfg->dhdr_limit >= 0.0;

    size_t nstate = (size_t)nrings * nd * P;
    size_t esz = st.fp32 ? sizeof(float) : sizeof(double);
    cudaError_t e;
#define ENS(buf, n)                                                   \
    if ((e = (buf).ensure(n)) != cudaSuccess) {                       \
        ti_release(ctx);                                              \
        return cuda_fail(e, "device allocation for the ring batch");  \
    }
    ENS(st.q, nstate * esz);
    ENS(st.pi, nstate * esz);
    ENS(st.x, nstate * esz);
    ENS(st.f, nstate * esz);
    ENS(st.T, (size_t)P * P * (sizeof(double) + sizeof(float)));
    ENS(st.coef, coef.size() * sizeof(ModeCoef));
    ENS(st.bv, (size_t)nlambda * nd * P * sizeof(double));
    ENS(st.bvtab, bvtab.size() * sizeof(double));
    ENS(st.dbdl, (size_t)nlambda * nd * sizeof(double));
    ENS(st.avec, (size_t)nd * sizeof(double));
    ENS(st.bvec, (size_t)nlambda * nd * sizeof(double));
    ENS(st.xref, (size_t)nlambda * nd * P * sizeof(double));
    ENS(st.ringlam, (size_t)nrings * sizeof(int32_t));
    ENS(st.ringseed, (size_t)nrings * sizeof(uint64_t));
    ENS(st.ringstream, (size_t)nrings * sizeof(uint32_t));
    ENS(st.acc, (size_t)nrings * sizeof(RingAcc));
    ENS(st.red, (size_t)(3 * nlambda + 1) * sizeof(double));
    ENS(st.kickflag, (size_t)nrings);  // per-ring flags of the blocked tensor form (Andersen kick / re-init)
    if (x0) ENS(st.x0, nstate * sizeof(double));
    if (p0) ENS(st.p0, nstate * sizeof(double));
    DevBuf &dx0 = st.x0, &dp0 = st.p0;
#undef ENS
    {
        const std::string sig = graph_signature(ctx, st);
        if (sig != st.graph_sig) {
            for (auto &kv : st.graphs) cudaGraphExecDestroy(kv.second);
            st.graphs.clear();
            for (auto &kv : st.group_graphs) cudaGraphExecDestroy(kv.second);
            st.group_graphs.clear();
            st.graph_sig = sig;
        }
    }
    std::vector<float> Tf(T.begin(), T.end());
    cudaStream_t s = ctx->stream;
    PG_CUDA(cudaMemsetAsync(st.kickflag.ptr, 0, (size_t)nrings, s));  // no ring flagged
    PG_CUDA(cudaMemcpyAsync(st.T.ptr, T.data(), T.size() * sizeof(double), cudaMemcpyHostToDevice, s));
    PG_CUDA(cudaMemcpyAsync(st.T.as<double>() + (size_t)P * P, Tf.data(), Tf.size() * sizeof(float), cudaMemcpyHostToDevice, s));
    PG_CUDA(cudaMemcpyAsync(st.coef.ptr, coef.data(), coef.size() * sizeof(ModeCoef), cudaMemcpyHostToDevice, s));
    PG_CUDA(cudaMemcpyAsync(st.bvtab.ptr, bvtab.data(), bvtab.size() * sizeof(double), cudaMemcpyHostToDevice, s));
    PG_CUDA(cudaMemcpyAsync(st.dbdl.ptr, dbdl, (size_t)nlambda * nd * sizeof(double), cudaMemcpyHostToDevice, s));
    PG_CUDA(cudaMemcpyAsync(st.avec.ptr, a, (size_t)nd * sizeof(double), cudaMemcpyHostToDevice, s));
    PG_CUDA(cudaMemcpyAsync(st.bvec.ptr, b, (size_t)nlambda * nd * sizeof(double), cudaMemcpyHostToDevice, s));
    {
        const int64_t nbv = nlambda * nd * P;
        k_beadvec<<<(unsigned)((nbv + 255) / 256), 256, 0, s>>>(st.avec.as<double>(), st.bvec.as<double>(),
                                                               st.bvtab.as<double>(), bvsq, nlambda, nd, P,
                                                               st.bv.as<double>());
        PG_CUDA(cudaGetLastError());
    }
    if (need_xref) {
        if (xref)
            PG_CUDA(cudaMemcpyAsync(st.xref.ptr, xref, (size_t)nlambda * nd * P * sizeof(double),
                                    cudaMemcpyHostToDevice, s));
        else
            PG_CUDA(cudaMemsetAsync(st.xref.ptr, 0, (size_t)nlambda * nd * P * sizeof(double), s));
    }
    PG_CUDA(cudaMemcpyAsync(st.ringlam.ptr, ring_lambda, nrings * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    PG_CUDA(cudaMemcpyAsync(st.ringseed.ptr, ring_seed, nrings * sizeof(uint64_t), cudaMemcpyHostToDevice, s));
    PG_CUDA(cudaMemcpyAsync(st.ringstream.ptr, ring_stream, nrings * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
    PG_CUDA(cudaMemsetAsync(st.red.ptr, 0, (size_t)(3 * nlambda + 1) * sizeof(double), s));
    if (x0) PG_CUDA(cudaMemcpyAsync(dx0.ptr, x0, nstate * sizeof(double), cudaMemcpyHostToDevice, s));
    if (p0) PG_CUDA(cudaMemcpyAsync(dp0.ptr, p0, nstate * sizeof(double), cudaMemcpyHostToDevice, s));

    TiArgs ta = make_args(ctx, st, step_ptr(st));
    int th = threads_for(P, nd);
    size_t sm = ring_smem_bytes(P, st.fp32);
    if (sm > 48 * 1024) {  // FP64 with P > 768: opt in to more than 48 KB
        PG_CUDA(cudaFuncSetAttribute(k_ti_fused<double, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        PG_CUDA(cudaFuncSetAttribute(k_ti_fused<double, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        PG_CUDA(cudaFuncSetAttribute(k_ti_init<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        PG_CUDA(cudaFuncSetAttribute(k_ti_momenta<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    }
    if (st.form == PG_FORM_PLAIN) {
        k_plain_init<<<(unsigned)nrings, th, (size_t)P * sizeof(double), s>>>(
            ta, st.x.as<double>(), st.pi.as<double>(), st.f.as<double>(), dx0.as<double>(), dp0.as<double>());
    } else if (st.fp32) {
        k_ti_init<float><<<(unsigned)nrings, th, sm, s>>>(ta, st.q.as<float>(), st.pi.as<float>(), st.x.as<float>(),
                                                          dx0.as<double>(), dp0.as<double>());
    } else {
        k_ti_init<double><<<(unsigned)nrings, th, sm, s>>>(ta, st.q.as<double>(), st.pi.as<double>(), st.x.as<double>(),
                                                           dx0.as<double>(), dp0.as<double>());
    }
    PG_CUDA(cudaGetLastError());
    PG_CUDA(cudaStreamSynchronize(s));
    if (st.form == PG_FORM_TENSOR) {
        rc = tc_prepare(ctx, st);
        if (rc) {
            ti_release(ctx);
            return rc;
        }
        const std::string sig = graph_signature(ctx, st);  // tc_prepare may have moved the tensor tables
        if (sig != st.graph_sig) {
            for (auto &kv : st.graphs) cudaGraphExecDestroy(kv.second);
            st.graphs.clear();
            for (auto &kv : st.group_graphs) cudaGraphExecDestroy(kv.second);
            st.group_graphs.clear();
            st.graph_sig = sig;
        }
    }
    return PG_OK;
}

static int ti_advance_impl(pg_ctx *ctx, int64_t nsteps, double *device_ms);

// ---------------------------------------------------------------- autotuning of AUTO batches
// pg_set_tuning(path, mode): with mode PG_TUNE_CACHE a setup with form AUTO takes
// the form and SIMT block size recorded in the JSON-lines file `path` for its
// key; with PG_TUNE_ON a key that is not there is tuned on the batch itself:
// every candidate (tensor form where it applies, fused SIMT form with 32, 64 or
// 128 threads per ring) is set up and advanced for a short timed probe, the
// fastest is appended to the file, and the batch is set up again with it (so
// its initial state is that of a plain setup with the chosen parameters).
static std::string tune_key(pg_ctx *ctx, const pg_ti_config *cfg, int64_t nrings) {
    cudaDeviceProp prop;
    std::string dev = cudaGetDeviceProperties(&prop, ctx->device) == cudaSuccess ? prop.name : "unknown";
    for (char &ch : dev)
        if (ch == '"' || ch == '\\') ch = '_';
    int64_t nb = 1;
    while (nb < nrings) nb <<= 1;  // batch size bucket
    char buf[512];
    snprintf(buf, sizeof(buf), "%s|sm%d|P%lld|nd%d|natom%d|pes%d|prec%d|th%d|cay%d|lim%d|rings%lld", dev.c_str(),
             ctx->sm_count, (long long)cfg->nbeads, ctx->nd, ctx->natom, ctx->pes_id, (int)cfg->precision,
             (int)cfg->thermostat, (int)cfg->cayley, cfg->dhdr_limit >= 0.0 ? 1 : 0, (long long)nb);
    return buf;
}

extern "C" int pg_set_tuning(pg_ctx *ctx, const char *cache_path, int32_t mode) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if (mode < PG_TUNE_OFF || mode > PG_TUNE_ON) return fail(PG_ERR_ARG, "bad tuning mode");
    if (mode != PG_TUNE_OFF && (!cache_path || !*cache_path)) return fail(PG_ERR_ARG, "tuning needs a cache path");
    ctx->tune_mode = mode;
    ctx->tune_path = mode != PG_TUNE_OFF ? cache_path : "";
    return PG_OK;
}

extern "C" int pg_ti_get_tuning(pg_ctx *ctx, int32_t *form, int32_t *simt_threads, int32_t *tc_steps) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (!ctx->ti) return fail(PG_ERR_STATE, "pg_ti_setup has not been called");
    if (form) *form = ctx->ti->form;
    if (simt_threads) *simt_threads = ctx->ti->simt_threads;
    if (tc_steps) *tc_steps = ctx->ti->tc_steps;
    return PG_OK;
}

extern "C" int pg_ti_setup(pg_ctx *ctx, const pg_ti_config *cfg, int64_t nrings, int64_t nlambda,
                           const int32_t *ring_lambda, const uint64_t *ring_seed,
                           const uint32_t *ring_stream, const double *a, const double *b,
                           const double *dbdl, const double *xref, const double *x0,
                           const double *p0) {
    NvtxRange nvtx_range("pg_ti_setup");
    auto setup = [&](const pg_ti_config *c, int th, int steps) {
        return ti_setup_impl(ctx, c, nrings, nlambda, ring_lambda, ring_seed, ring_stream, a, b, dbdl, xref, x0,
                             p0, th, steps);
    };
    if (!ctx || !cfg || cfg->form != PG_FORM_AUTO || ctx->tune_mode == PG_TUNE_OFF || !ctx->have_system ||
        nrings < 1)
        return setup(cfg, 0, 0);
    const std::string key = tune_key(ctx, cfg, nrings);
    TuneChoice c;
    pg_ti_config cc = *cfg;
    if (tune_lookup(ctx->tune_path, key, c)) {
        cc.form = c.form;
        if (setup(&cc, c.simt_threads, c.tc_steps) == PG_OK) return PG_OK;
        return setup(cfg, 0, 0);  // a record that no longer applies
    }
    if (ctx->tune_mode != PG_TUNE_ON) return setup(cfg, 0, 0);
    std::vector<TuneChoice> cand;
    {
        TuneChoice t;
        t.form = PG_FORM_TENSOR;
        cand.push_back(t);
        for (int th : {32, 64, 128}) {
            t.form = PG_FORM_FUSED;
            t.simt_threads = th;
            cand.push_back(t);
        }
    }
    int best = -1;
    for (size_t i = 0; i < cand.size(); i++) {
        cc.form = cand[i].form;
        if (setup(&cc, cand[i].simt_threads, cand[i].tc_steps) != PG_OK) continue;  // does not apply
        // probe: a two-step estimate, then about 20 ms (4 .. 200 steps) after a warm-up advance
        double ms = 0.0;
        if (ti_advance_impl(ctx, 2, &ms) != PG_OK) continue;
        const int64_t k = std::max<int64_t>(4, std::min<int64_t>(200, (int64_t)(20.0 / std::max(ms / 2.0, 1e-4))));
        if (ti_advance_impl(ctx, k, nullptr) != PG_OK || ti_advance_impl(ctx, k, &ms) != PG_OK) continue;
        cand[i].ms_per_step = ms / (double)k;
        if (best < 0 || cand[i].ms_per_step < cand[best].ms_per_step) best = (int)i;
    }
    if (best < 0) return setup(cfg, 0, 0);  // report the plain setup's outcome
    tune_record(ctx->tune_path, key, cand[best]);
    cc.form = cand[best].form;
    return setup(&cc, cand[best].simt_threads, cand[best].tc_steps);
}

static int ti_advance_group(pg_ctx *const *ctxs, int64_t nctx, int64_t nsteps, double *device_ms);

extern "C" int pg_ti_advance(pg_ctx *ctx, int64_t nsteps) { return ti_advance_impl(ctx, nsteps, nullptr); }

extern "C" int pg_ti_advance_timed(pg_ctx *ctx, int64_t nsteps, double *device_ms) {
    if (!device_ms) return fail(PG_ERR_ARG, "device_ms is NULL");
    return ti_advance_impl(ctx, nsteps, device_ms);
}

// The executable graph of an n-step advance (captured on first use).
static int ti_graph(pg_ctx *ctx, int64_t n, cudaGraphExec_t *out) {
    TiState &st = *ctx->ti;
    auto it = st.graphs.find(n);
    if (it != st.graphs.end()) {
        *out = it->second;
        return PG_OK;
    }
    cudaGraph_t g = nullptr;
    cudaGraphExec_t exec = nullptr;
    PG_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    int lrc = launch_steps(ctx, st, n, ctx->stream);
    cudaError_t ee = cudaStreamEndCapture(ctx->stream, &g);
    if (lrc || ee != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        (void)cudaGetLastError();  // the failed capture's error stays with this call
        if (lrc) return lrc;
        return cuda_fail(ee, "cudaStreamEndCapture");
    }
    ee = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    if (ee != cudaSuccess) return cuda_fail(ee, "cudaGraphInstantiate");
    st.graphs[n] = exec;
    *out = exec;
    return PG_OK;
}

// One executable graph for an nsteps advance of every context of a group (one
// batch per bead number): the first context's stream forks to the others by an
// event, each context's step kernels are captured on its own stream, and the
// branches join back, so the whole uneven-P advance is a single graph launch
// whose branches run concurrently.  Cached on the first context, keyed by the
// step count and every batch's graph signature (which holds each buffer
// address the launches bake in).
static int group_graph(pg_ctx *const *ctxs, int64_t nctx, int64_t n, cudaGraphExec_t *out) {
    TiState &st0 = *ctxs[0]->ti;
    std::string key(reinterpret_cast<const char *>(&n), sizeof(n));
    for (int64_t i = 0; i < nctx; i++) {
        const std::string &g = ctxs[i]->ti->graph_sig;
        const uint64_t len = g.size();
        key.append(reinterpret_cast<const char *>(&len), sizeof(len));
        key += g;
    }
    auto it = st0.group_graphs.find(key);
    if (it != st0.group_graphs.end()) {
        *out = it->second;
        return PG_OK;
    }
    cudaStream_t s0 = ctxs[0]->stream;
    std::vector<cudaEvent_t> ev((size_t)nctx, nullptr);
    for (auto &e : ev) PG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    cudaGraph_t g = nullptr;
    int lrc = PG_OK;
    cudaError_t ce = cudaStreamBeginCapture(s0, cudaStreamCaptureModeThreadLocal);
    if (ce == cudaSuccess) {
        cudaEventRecord(ev[0], s0);
        for (int64_t i = 1; i < nctx; i++) cudaStreamWaitEvent(ctxs[i]->stream, ev[0], 0);
        for (int64_t i = 0; i < nctx && !lrc; i++) lrc = launch_steps(ctxs[i], *ctxs[i]->ti, n, ctxs[i]->stream);
        for (int64_t i = 1; i < nctx; i++) {  // every branch joins stream 0, also after a failed launch
            cudaEventRecord(ev[i], ctxs[i]->stream);
            cudaStreamWaitEvent(s0, ev[i], 0);
        }
        ce = cudaStreamEndCapture(s0, &g);
    }
    for (auto e : ev) cudaEventDestroy(e);
    if (lrc || ce != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        (void)cudaGetLastError();  // the failed capture's error stays with this call
        if (lrc) return lrc;
        return cuda_fail(ce, "capture of the group graph");
    }
    cudaGraphExec_t exec = nullptr;
    ce = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaGraphInstantiate (group)");
    st0.group_graphs[key] = exec;
    *out = exec;
    return PG_OK;
}

// Checks an advance of nsteps and captures the graphs it needs.  launch = true
// also replays them on the context's stream (without waiting).  Plain form:
// graphs of up to 64 steps; fused forms: one graph per nsteps.
static int ti_enqueue(pg_ctx *ctx, int64_t nsteps, bool launch) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (!ctx->ti) return fail(PG_ERR_STATE, "pg_ti_setup has not been called");
    if (nsteps < 0) return fail(PG_ERR_ARG, "nsteps must be >= 0");
    TiState &st = *ctx->ti;
    if (st.step + nsteps > (int64_t)0xFFFFFFFFLL) return fail(PG_ERR_ARG, "step counter would exceed 2^32");
    int64_t chunk = (st.form == PG_FORM_PLAIN) ? (nsteps < 64 ? nsteps : 64) : nsteps;
    int64_t done = 0;
    while (done < nsteps) {
        int64_t n = (nsteps - done) < chunk ? (nsteps - done) : chunk;
        cudaGraphExec_t exec = nullptr;
        rc = ti_graph(ctx, n, &exec);
        if (rc) return rc;
        if (launch) PG_CUDA(cudaGraphLaunch(exec, ctx->stream));
        done += n;
    }
    return PG_OK;
}

// Completes an enqueued advance: waits for the stream, moves the host step
// counter, reads the tensor-core kernels' error word.
static int ti_finish(pg_ctx *ctx, int64_t nsteps) {
    TiState &st = *ctx->ti;
    PG_CUDA(cudaStreamSynchronize(ctx->stream));
    st.step += nsteps;
    if (st.form == PG_FORM_TENSOR) {
        int32_t kerr = tc_error(ctx, st);
        if (kerr) return fail(PG_ERR_NUMERIC, "tensor-core kernel: a barrier wait timed out (error word " +
                                                  std::to_string(kerr) + ")");
    }
    return PG_OK;
}

static int ti_advance_impl(pg_ctx *ctx, int64_t nsteps, double *device_ms) {
    NvtxRange nvtx_range("pg_ti_advance");
    pg_ctx *one[1] = {ctx};
    return ti_advance_group(one, 1, nsteps, device_ms);
}

// Advances several contexts on one device together: every context's graph is
// launched on its own stream before any is waited for, so batches of different
// bead numbers run concurrently.  device_ms (optional) spans all of them.
static int ti_advance_group(pg_ctx *const *ctxs, int64_t nctx, int64_t nsteps, double *device_ms) {
    if (!ctxs || nctx <= 0) return fail(PG_ERR_ARG, "no contexts");
    for (int64_t i = 0; i < nctx; i++) {
        int rc = check_ctx(ctxs[i], true);
        if (rc) return rc;
        if (!ctxs[i]->ti) return fail(PG_ERR_STATE, "pg_ti_setup has not been called");
        if (ctxs[i]->device != ctxs[0]->device) return fail(PG_ERR_ARG, "contexts on different devices");
        for (int64_t k = 0; k < i; k++)
            if (ctxs[k] == ctxs[i]) return fail(PG_ERR_ARG, "a context appears twice");
    }
    if (nsteps < 0) return fail(PG_ERR_ARG, "nsteps must be >= 0");
    if (nsteps == 0) {
        if (device_ms) *device_ms = 0.0;
        return PG_OK;
    }
    PG_CUDA(cudaSetDevice(ctxs[0]->device));
    for (int64_t i = 0; i < nctx; i++) {
        int rc = ti_enqueue(ctxs[i], nsteps, false);  // checks; captures outside the timed span
        if (rc) return rc;
    }
    cudaStream_t s0 = ctxs[0]->stream;
    bool combined = nctx > 1;  // the plain form replays graphs of up to 64 steps: per-stream path
    for (int64_t i = 0; i < nctx; i++)
        if (ctxs[i]->ti->form == PG_FORM_PLAIN) combined = false;
    if (combined) {
        cudaGraphExec_t exec = nullptr;
        int rc = group_graph(ctxs, nctx, nsteps, &exec);
        if (rc) return rc;
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        PG_CUDA(cudaEventCreate(&e0));
        cudaError_t ce = cudaEventCreate(&e1);
        if (ce == cudaSuccess) ce = cudaEventRecord(e0, s0);
        if (ce == cudaSuccess) ce = cudaGraphLaunch(exec, s0);
        if (ce == cudaSuccess) ce = cudaEventRecord(e1, s0);
        // the group's work ran on stream 0: wait for it there first
        for (int64_t i = 0; i < nctx; i++) {
            int r = ti_finish(ctxs[i], nsteps);
            if (r && !rc) rc = r;
        }
        if (ce != cudaSuccess && !rc) rc = cuda_fail(ce, "group graph launch");
        if (!rc && device_ms) {
            float ms = 0.f;
            ce = cudaEventElapsedTime(&ms, e0, e1);
            if (ce != cudaSuccess) rc = cuda_fail(ce, "cudaEventElapsedTime");
            *device_ms = (double)ms;
        }
        cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        return rc;
    }
    std::vector<cudaEvent_t> ev;
    auto cleanup = [&]() {
        for (auto e : ev) cudaEventDestroy(e);
    };
    if (device_ms || nctx > 1) {
        ev.resize((size_t)nctx + 2, nullptr);
        for (auto &e : ev) {
            cudaError_t ce = cudaEventCreate(&e);
            if (ce != cudaSuccess) {
                cleanup();
                return cuda_fail(ce, "cudaEventCreate");
            }
        }
        // start: the other streams wait for the start event on stream 0
        cudaEventRecord(ev[0], s0);
        for (int64_t i = 1; i < nctx; i++) cudaStreamWaitEvent(ctxs[i]->stream, ev[0], 0);
    }
    for (int64_t i = 0; i < nctx; i++) {
        int rc = ti_enqueue(ctxs[i], nsteps, true);
        if (rc) {
            for (int64_t k = 0; k < nctx; k++) cudaStreamSynchronize(ctxs[k]->stream);
            cleanup();
            return rc;
        }
    }
    if (!ev.empty()) {
        // join: stream 0 waits for every other stream, then records the end
        for (int64_t i = 1; i < nctx; i++) {
            cudaEventRecord(ev[1 + i], ctxs[i]->stream);
            cudaStreamWaitEvent(s0, ev[1 + i], 0);
        }
        cudaEventRecord(ev[1], s0);
    }
    int rc = PG_OK;
    for (int64_t i = nctx - 1; i >= 0; i--) {
        int r = ti_finish(ctxs[i], nsteps);
        if (r && !rc) rc = r;
    }
    if (!rc && device_ms) {
        float ms = 0.f;
        cudaError_t ce = cudaEventElapsedTime(&ms, ev[0], ev[1]);
        if (ce != cudaSuccess) rc = cuda_fail(ce, "cudaEventElapsedTime");
        *device_ms = (double)ms;
    }
    cleanup();
    return rc;
}

extern "C" int pg_ti_advance_group(pg_ctx *const *ctxs, int64_t nctx, int64_t nsteps, double *device_ms) {
    NvtxRange nvtx_range("pg_ti_advance_group");
    return ti_advance_group(ctxs, nctx, nsteps, device_ms);
}

extern "C" int pg_ti_get_step(pg_ctx *ctx, int64_t *step) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (!ctx->ti) return fail(PG_ERR_STATE, "pg_ti_setup has not been called");
    if (step) *step = ctx->ti->step;
    return PG_OK;
}

extern "C" int pg_ti_kernel_times(pg_ctx *ctx, int64_t nsteps, int32_t *nkinds, double *ms_per_launch,
                                  int64_t *count, double *bytes_per_launch, const char **names) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (!ctx->ti) return fail(PG_ERR_STATE, "pg_ti_setup has not been called");
    if (nsteps < 1 || !nkinds || !ms_per_launch || !count || !bytes_per_launch)
        return fail(PG_ERR_ARG, "bad kernel-time arguments");
    TiState &st = *ctx->ti;
    const double arr = (double)st.nrings * st.nd * st.P * (st.fp32 ? 4.0 : 8.0);  // one state array
    if (st.form == PG_FORM_TENSOR) {
        double ms[2];
        int64_t n[2];
        if (st.tf_fused) {
            int nsub = 1;
            rc = tc_kernel_times(ctx, st, nsteps, ms, n, &nsub);
            if (rc) return rc;
            *nkinds = 2;
            ms_per_launch[0] = ms[0];
            ms_per_launch[1] = ms[1];
            count[0] = n[0];
            count[1] = n[1];
            bytes_per_launch[0] = 4.0 * arr * nsub;  // k_tf_step: read q, pi; write q, pi; per MD step
            bytes_per_launch[1] = 2.0 * arr;         // read-out pass: read q, write x
            if (names) {
                static thread_local std::string tf_name;
                tf_name = "k_tf_step (" + std::to_string(nsub) +
                          " MD steps per launch, P = 256: folded T resident, two warp groups on alternate chunks)";
                names[0] = tf_name.c_str();
                names[1] = "k_tf_out (read-out: positions and last estimator; two half GEMMs)";
            }
        } else if (st.tc_blocked && st.cfg.thermostat == PG_ANDERSEN) {
            double ms3[3];
            int64_t n3[3];
            int nsub = 1;
            rc = tc_kernel_times(ctx, st, nsteps, ms3, n3, &nsub);
            if (rc) return rc;
            *nkinds = 1;
            ms_per_launch[0] = ms3[0];
            count[0] = n3[0];
            bytes_per_launch[0] = 14.0 * arr;  // q, pi twice; x, F, the GEMM operands
            if (names) names[0] = "blocked Andersen step (schedule, resample + rotation, k_tb_pos, k_tb_force, k_tb_kick_nm, estimator)";
        } else if (st.tc_blocked) {
            double ms3[3];
            int64_t n3[3];
            int nsub = 1;
            rc = tc_kernel_times(ctx, st, nsteps, ms3, n3, &nsub);
            if (rc) return rc;
            *nkinds = 3;
            for (int k = 0; k < 3; k++) {
                ms_per_launch[k] = ms3[k];
                count[k] = n3[k];
            }
            bytes_per_launch[0] = 2.0 * arr;  // k_tb_pos: read q, write x
            bytes_per_launch[1] = 2.0 * arr;  // k_tb_force: read x, write F
            bytes_per_launch[2] = 5.0 * arr;  // k_tb_kick: read F, q, pi; write q, pi
            if (names) {
                names[0] = "k_tb_pos (positions: blocked split-BF16 tcgen05 GEMM)";
                names[1] = "k_tb_force (FP32 surface forces and estimator, SIMT)";
                names[2] = "k_tb_kick (T F: blocked split-BF16 tcgen05 GEMM; kick, rotation, OU)";
            }
        } else {
            int nsub = 1;
            rc = tc_kernel_times(ctx, st, nsteps, ms, n, &nsub);
            if (rc) return rc;
            *nkinds = 2;
            ms_per_launch[0] = ms[0];
            ms_per_launch[1] = ms[1];
            count[0] = n[0];
            count[1] = n[1];
            bytes_per_launch[0] = 4.0 * arr * nsub;  // k_tc_step: read q, pi; write q, pi; per MD step
            bytes_per_launch[1] = 2.0 * arr;         // k_tc_final: read q, write x
            if (names) {
                static thread_local std::string step_name;
                step_name = "k_tc_step (" + std::to_string(nsub) +
                            " MD steps per launch, each two split-BF16 tcgen05 GEMMs, forces, OU)";
                names[0] = step_name.c_str();
                names[1] = "k_tc_final (positions and last estimator; one split-BF16 tcgen05 GEMM)";
            }
        }
        st.step += nsteps;
        int32_t kerr = tc_error(ctx, st);
        if (kerr) return fail(PG_ERR_NUMERIC, "tensor-core kernel error word " + std::to_string(kerr));
        return PG_OK;
    }
    // fused / plain: one timed advance (graph) = one launch of the dominant kernel
    double ms = 0.0;
    rc = pg_ti_advance_timed(ctx, nsteps, &ms);
    if (rc) return rc;
    *nkinds = 1;
    ms_per_launch[0] = ms;
    count[0] = 1;
    bytes_per_launch[0] = 4.0 * arr;  // state in and out once per launch (q, pi, x, acc)
    if (names) names[0] = st.form == PG_FORM_FUSED ? "k_ti_fused (SIMT)" : "plain-form step sequence";
    return PG_OK;
}

extern "C" int pg_ti_get_form(pg_ctx *ctx, int64_t nsteps, int32_t *form, int64_t *launches) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (!ctx->ti) return fail(PG_ERR_STATE, "pg_ti_setup has not been called");
    TiState &st = *ctx->ti;
    if (form) *form = st.form;
    if (launches) {
        if (st.form == PG_FORM_TENSOR && st.tc_blocked && st.cfg.thermostat == PG_ANDERSEN)
            *launches = nsteps > 0 ? 6 * nsteps + 2 : 0;  // six per step; positions, counter
        else if (st.form == PG_FORM_TENSOR && st.tf_fused)  // step launches of up to tc_steps_per_launch(); read-out, counter
            *launches = nsteps > 0 ? (nsteps + tc_steps_per_launch(st) - 1) / tc_steps_per_launch(st) + 2 : 0;
        else if (st.form == PG_FORM_TENSOR && st.tc_blocked && st.cfg.dhdr_limit >= 0.0)
            *launches = nsteps > 0 ? 4 * nsteps + 3 : 0;  // pos, force, re-init, kick (the first step: no re-init); pos, estimator, re-init, counter
        else if (st.form == PG_FORM_TENSOR && st.tc_blocked)
            *launches = nsteps > 0 ? 3 * nsteps + 3 : 0;  // pos, force, kick per step; pos, estimator, counter
        else if (st.form == PG_FORM_TENSOR)  // step kernels of up to tc_steps_per_launch() steps; final pass, counter
            *launches = nsteps > 0 ? (nsteps + tc_steps_per_launch(st) - 1) / tc_steps_per_launch(st) + 2 : 0;
        else if (st.form == PG_FORM_FUSED)
            *launches = nsteps > 0 ? 2 : 0;  // fused kernel + step counter
        else
            *launches = 6 * nsteps;  // kick, nm, langevin (or Andersen), nm, estimator, step counter
    }
    return PG_OK;
}

extern "C" int pg_ti_get_state(pg_ctx *ctx, double *x, double *p) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (!ctx->ti) return fail(PG_ERR_STATE, "pg_ti_setup has not been called");
    TiState &st = *ctx->ti;
    size_t n = (size_t)st.nrings * st.nd * st.P;
    cudaStream_t s = ctx->stream;
    PG_CUDA(ctx->scratch_a.ensure(n * sizeof(double)));
    PG_CUDA(ctx->scratch_b.ensure(n * sizeof(double)));
    TiArgs ta = make_args(ctx, st, step_ptr(st));
    int th = threads_for(st.P, st.nd);
    if (st.form == PG_FORM_TENSOR) {
        rc = tc_launch(ctx, st, 0, -1, s);  // read-out: writes x, pi back to the SIMT layout
        if (rc) return rc;
    }
    // both conversions first, then both copies, one wait
    const double *xs = st.x.as<double>(), *ps = st.pi.as<double>();
    if (x && st.fp32) {
        k_to_double<float><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(st.x.as<float>(), ctx->scratch_a.as<double>(), n);
        xs = ctx->scratch_a.as<double>();
    }
    if (p && st.form != PG_FORM_PLAIN) {
        size_t sm = ring_smem_bytes(st.P, st.fp32);
        if (st.fp32)
            k_ti_momenta<float><<<(unsigned)st.nrings, th, sm, s>>>(ta, st.pi.as<float>(), ctx->scratch_b.as<double>());
        else
            k_ti_momenta<double><<<(unsigned)st.nrings, th, sm, s>>>(ta, st.pi.as<double>(), ctx->scratch_b.as<double>());
        ps = ctx->scratch_b.as<double>();
    }
    PG_CUDA(cudaGetLastError());
    if (x) PG_CUDA(cudaMemcpyAsync(x, xs, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (p) PG_CUDA(cudaMemcpyAsync(p, ps, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    PG_CUDA(cudaStreamSynchronize(s));
    return PG_OK;
}

extern "C" int pg_ti_get_results(pg_ctx *ctx, double *dhdr_sum, int64_t *nsamples, int64_t *nreinit,
                                 int32_t *status) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (!ctx->ti) return fail(PG_ERR_STATE, "pg_ti_setup has not been called");
    TiState &st = *ctx->ti;
    std::vector<RingAcc> acc(st.nrings);
    PG_CUDA(cudaMemcpyAsync(acc.data(), st.acc.ptr, st.nrings * sizeof(RingAcc), cudaMemcpyDeviceToHost, ctx->stream));
    PG_CUDA(cudaStreamSynchronize(ctx->stream));
    for (int64_t r = 0; r < st.nrings; r++) {
        if (dhdr_sum) dhdr_sum[r] = acc[r].dhdr_sum;
        if (nsamples) nsamples[r] = acc[r].nsamples;
        if (nreinit) nreinit[r] = acc[r].nreinit;
        if (status) status[r] = acc[r].status;
    }
    return PG_OK;
}

extern "C" int pg_ti_set_accumulators(pg_ctx *ctx, const double *dhdr_sum, const int64_t *nsamples, int64_t step) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (!ctx->ti) return fail(PG_ERR_STATE, "pg_ti_setup has not been called");
    if (!dhdr_sum || !nsamples) return fail(PG_ERR_ARG, "dhdr_sum and nsamples are required");
    if (step < 0 || step > (int64_t)0xFFFFFFFFLL) return fail(PG_ERR_ARG, "step out of range");
    TiState &st = *ctx->ti;
    for (int64_t r = 0; r < st.nrings; r++)
        if (nsamples[r] < 0) return fail(PG_ERR_ARG, "negative sample count");
    std::vector<RingAcc> acc(st.nrings);
    PG_CUDA(cudaMemcpyAsync(acc.data(), st.acc.ptr, st.nrings * sizeof(RingAcc), cudaMemcpyDeviceToHost, ctx->stream));
    PG_CUDA(cudaStreamSynchronize(ctx->stream));
    for (int64_t r = 0; r < st.nrings; r++) {
        acc[r].dhdr_sum = dhdr_sum[r];
        acc[r].nsamples = nsamples[r];
    }
    PG_CUDA(cudaMemcpyAsync(st.acc.ptr, acc.data(), st.nrings * sizeof(RingAcc), cudaMemcpyHostToDevice, ctx->stream));
    PG_CUDA(cudaMemcpyAsync(step_ptr(st), &step, sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
    PG_CUDA(cudaStreamSynchronize(ctx->stream));
    st.step = step;
    return PG_OK;
}

extern "C" int pg_ti_lambda_reduce(pg_ctx *ctx, double *mean, double *var, int64_t *count) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (!ctx->ti) return fail(PG_ERR_STATE, "pg_ti_setup has not been called");
    TiState &st = *ctx->ti;
    k_lambda_reduce<<<(unsigned)st.nlambda, 256, 0, ctx->stream>>>(st.acc.as<RingAcc>(), st.ringlam.as<int32_t>(),
                                                                     st.nrings, st.betan, st.red.as<double>());
    PG_CUDA(cudaGetLastError());
    std::vector<double> out(3 * st.nlambda);
    PG_CUDA(cudaMemcpyAsync(out.data(), st.red.ptr, out.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    PG_CUDA(cudaStreamSynchronize(ctx->stream));
    for (int64_t l = 0; l < st.nlambda; l++) {
        if (mean) mean[l] = out[3 * l];
        if (var) var[l] = out[3 * l + 1];
        if (count) count[l] = (int64_t)out[3 * l + 2];
    }
    return PG_OK;
}

// Checkpoint layout: header, then q, pi, x (state precision), then RingAcc[nrings].
struct CkptHeader {
    char magic[8];
    int32_t version, form, fp32, P;
    int64_t nrings, nd, step;
    pg_ti_config cfg;
};

extern "C" int pg_ti_checkpoint_save(pg_ctx *ctx, const char *path) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (!ctx->ti) return fail(PG_ERR_STATE, "pg_ti_setup has not been called");
    if (!path) return fail(PG_ERR_ARG, "path is NULL");
    TiState &st = *ctx->ti;
    if (st.form == PG_FORM_TENSOR) {
        rc = tc_launch(ctx, st, 0, -1, ctx->stream);
        if (rc) return rc;
    }
    size_t n = (size_t)st.nrings * st.nd * st.P * (st.fp32 ? sizeof(float) : sizeof(double));
    std::vector<unsigned char> buf(3 * n + st.nrings * sizeof(RingAcc));
    PG_CUDA(cudaMemcpyAsync(buf.data(), st.q.ptr, n, cudaMemcpyDeviceToHost, ctx->stream));
    PG_CUDA(cudaMemcpyAsync(buf.data() + n, st.pi.ptr, n, cudaMemcpyDeviceToHost, ctx->stream));
    PG_CUDA(cudaMemcpyAsync(buf.data() + 2 * n, st.x.ptr, n, cudaMemcpyDeviceToHost, ctx->stream));
    PG_CUDA(cudaMemcpyAsync(buf.data() + 3 * n, st.acc.ptr, st.nrings * sizeof(RingAcc), cudaMemcpyDeviceToHost, ctx->stream));
    PG_CUDA(cudaStreamSynchronize(ctx->stream));
    CkptHeader h;
    memset(&h, 0, sizeof(h));
    memcpy(h.magic, "PGCKPT01", 8);
    h.version = 1;
    h.form = st.form;
    h.fp32 = st.fp32;
    h.P = st.P;
    h.nrings = st.nrings;
    h.nd = st.nd;
    h.step = st.step;
    h.cfg = st.cfg;
    FILE *fp = fopen(path, "wb");
    if (!fp) return fail(PG_ERR_IO, std::string("cannot open ") + path);
    bool ok = fwrite(&h, sizeof(h), 1, fp) == 1 && fwrite(buf.data(), 1, buf.size(), fp) == buf.size();
    ok = (fclose(fp) == 0) && ok;
    if (!ok) return fail(PG_ERR_IO, "checkpoint write failed");
    return PG_OK;
}

extern "C" int pg_ti_checkpoint_load(pg_ctx *ctx, const char *path) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (!ctx->ti) return fail(PG_ERR_STATE, "set up the same batch with pg_ti_setup before loading");
    if (!path) return fail(PG_ERR_ARG, "path is NULL");
    TiState &st = *ctx->ti;
    FILE *fp = fopen(path, "rb");
    if (!fp) return fail(PG_ERR_IO, std::string("cannot open ") + path);
    CkptHeader h;
    if (fread(&h, sizeof(h), 1, fp) != 1 || memcmp(h.magic, "PGCKPT01", 8) != 0) {
        fclose(fp);
        return fail(PG_ERR_IO, "not a pimdgpu checkpoint");
    }
    if (h.form != st.form || h.fp32 != (int)st.fp32 || h.P != st.P || h.nrings != st.nrings || h.nd != st.nd) {
        fclose(fp);
        return fail(PG_ERR_ARG, "checkpoint does not match the current batch (form/precision/P/nrings/ndof)");
    }
    size_t n = (size_t)st.nrings * st.nd * st.P * (st.fp32 ? sizeof(float) : sizeof(double));
    std::vector<unsigned char> buf(3 * n + st.nrings * sizeof(RingAcc));
    size_t got = fread(buf.data(), 1, buf.size(), fp);
    fclose(fp);
    if (got != buf.size()) return fail(PG_ERR_IO, "truncated checkpoint");
    PG_CUDA(cudaMemcpyAsync(st.q.ptr, buf.data(), n, cudaMemcpyHostToDevice, ctx->stream));
    PG_CUDA(cudaMemcpyAsync(st.pi.ptr, buf.data() + n, n, cudaMemcpyHostToDevice, ctx->stream));
    PG_CUDA(cudaMemcpyAsync(st.x.ptr, buf.data() + 2 * n, n, cudaMemcpyHostToDevice, ctx->stream));
    PG_CUDA(cudaMemcpyAsync(st.acc.ptr, buf.data() + 3 * n, st.nrings * sizeof(RingAcc), cudaMemcpyHostToDevice, ctx->stream));
    int64_t stepv = h.step;
    PG_CUDA(cudaMemcpyAsync(step_ptr(st), &stepv, sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
    PG_CUDA(cudaStreamSynchronize(ctx->stream));
    st.step = h.step;
    if (st.form == PG_FORM_TENSOR) {
        rc = tc_prepare(ctx, st);
        if (rc) return rc;
    }
    return PG_OK;
}

extern "C" int pg_ti_release(pg_ctx *ctx) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    return ti_release(ctx);
}

extern "C" int pg_propagate_pimd(pg_ctx *ctx, const pg_ti_config *cfg, int64_t ntask, int64_t nmc,
                                 const double *a, const double *b, const double *dbdl,
                                 const uint64_t *seed, const uint32_t *stream, double *x, double *p,
                                 double *dHdr, int32_t *status) {
    NvtxRange nvtx_range("pg_propagate_pimd");
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (!x || !p || !dHdr || ntask < 1 || nmc < 0) return fail(PG_ERR_ARG, "bad propagate arguments");
    std::vector<int32_t> lam(ntask);
    for (int64_t i = 0; i < ntask; i++) lam[i] = (int32_t)i;
    rc = pg_ti_setup(ctx, cfg, ntask, ntask, lam.data(), seed, stream, a, b, dbdl, x, x, p);
    if (rc) return rc;
    rc = pg_ti_advance(ctx, nmc);
    if (rc) return rc;
    rc = pg_ti_get_state(ctx, x, p);
    if (rc) return rc;
    std::vector<double> sum(ntask);
    std::vector<int64_t> ns(ntask);
    rc = pg_ti_get_results(ctx, sum.data(), ns.data(), nullptr, status);
    if (rc) return rc;
    for (int64_t i = 0; i < ntask; i++) dHdr[i] = ns[i] > 0 ? sum[i] / (double)ns[i] : 0.0;
    return PG_OK;
}
