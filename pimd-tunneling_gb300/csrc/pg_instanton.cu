// pg_instanton.cu -- ring-polymer instanton on the GPU, FP64 throughout:
//   * batched fixed-end polymer action UM and its gradient (instantonmod.f90:17-151);
//     the PES gradient is the hand-written reverse mode of each surface, which
//     recomputes every pair distance instead of storing forward intermediates;
//   * batched L-BFGS driven by that gradient, one thread-block cluster of up to
//     8 CTAs per beta (replaces the setulb loop of instantonmod.f90:679-777);
//   * mass-weighted polymer Hessian in LAPACK lower band storage (UMhessian,
//     instantonmod.f90:155-217) and its log-determinant by a banded LDL^T with
//     Sylvester inertia, eigenvalues below zero / the lowest one by bisection
//     (replaces DSBEVD + the log sums of rpi_ser.f90:222-237, 354-366).
#include <cmath>
#include <cstring>
#include <vector>

#include "pg_hessian.cuh"
#include "pg_internal.h"

namespace pg {

bool hess_is_fd_host(int id) { return id == PG_PES_1D || id == PG_PES_SYNTH18 || id == PG_PES_DISTGAUSS; }

namespace {

struct InstArgs {
    PesArgs pes;
    int N, nd, ndim, natom;
    int fixedends;        // 0: no springs to a and b (instantonmod.f90:35-44, 63-72, 115-124, 138)
    const double *mass;   // natom
    const double *a;      // nd, fixed start
    const double *b;      // nbeta*nd, fixed ends
    const double *betan;  // nbeta
};

__device__ __forceinline__ double block_sum(double v, double *sred) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    if (l == 0) sred[w] = v;
    __syncthreads();
    double t = 0.0;
    for (int i = 0; i < nw; i++) t += sred[i];
    return t;
}

__device__ __forceinline__ double block_max(double v, double *sred) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    if (l == 0) sred[w] = v;
    __syncthreads();
    double t = sred[0];
    for (int i = 1; i < nw; i++) t = fmax(t, sred[i]);
    return t;
}

// UM and dUM/dx of polymer k (x, g: [dof][N]); every thread returns UM.
__device__ double polymer_fg(const InstArgs &A, int k, const double *__restrict__ x, double *__restrict__ g,
                             double *sred) {
    const int N = A.N, nd = A.nd;
    const double bn = A.betan[k];
    const double *b = A.b + (size_t)k * nd;
    double part = 0.0;
    // bead potentials and their adjoint gradients (mcmod V / Vprime)
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        double xb[kMaxDof], gb[kMaxDof];
        for (int d = 0; d < nd; d++) xb[d] = x[d * N + i];
        part += pes_vgrad<double>(A.pes, xb, gb);
        for (int d = 0; d < nd; d++) g[d * N + i] = gb[d];
    }
    __syncthreads();
    // springs between neighbours and, with fixed ends, to a and b
    // (instantonmod.f90:25-43, 59-78); free ends: an end bead has one neighbour,
    // m (x_1 - x_2) / betan^2 and m (x_N - x_N-1) / betan^2 (instantonmod.f90:66, 72)
    const bool fixed = A.fixedends != 0;
    for (int e = threadIdx.x; e < nd * N; e += blockDim.x) {
        const int dof = e / N, i = e - dof * N;
        const double m = A.mass[dof / A.ndim];
        const double xl = i > 0 ? x[e - 1] : (fixed ? A.a[dof] : x[e]);
        const double xr = i < N - 1 ? x[e + 1] : (fixed ? b[dof] : x[e]);
        g[e] = m * (2.0 * x[e] - xl - xr) / (bn * bn) + g[e];
        const double c = 0.5 * m / (bn * bn);
        if (i < N - 1) part += c * (x[e + 1] - x[e]) * (x[e + 1] - x[e]);
        if (fixed && i == 0) part += c * (x[e] - A.a[dof]) * (x[e] - A.a[dof]);
        if (fixed && i == N - 1) part += c * (b[dof] - x[e]) * (b[dof] - x[e]);
    }
    double um = block_sum(part, sred);
    __syncthreads();
    return um;
}

__global__ void k_inst_fg(InstArgs A, const double *__restrict__ x, double *__restrict__ um,
                          double *__restrict__ g) {
    __shared__ double sred[32];
    const int k = blockIdx.x;
    const size_t off = (size_t)k * A.nd * A.N;
    double v = polymer_fg(A, k, x + off, g + off, sred);
    if (threadIdx.x == 0) um[k] = v;
}

struct LbfgsArgs {
    int m, max_bt;
    int64_t maxiter;
    double factr, pgtol;
};

// Scratch per polymer: x, g, d, xt, gt (5n) + S, Y (2 m n) + 2 m (unused: rho and alpha live in
// each CTA's shared memory).

// ---------------------------------------------------------------- L-BFGS over a thread-block cluster
// The same optimiser with each polymer spread over a cluster of CS CTAs (CS =
// 1, 2, 4, 8): CTA r of the cluster owns beads [r N / CS, (r + 1) N / CS) of
// every dof, evaluates their surface terms and springs and keeps its slice of
// x, g, d, S, Y.  On GB300 the FP64 pipe of one SM bounds a polymer's
// evaluation and two-loop recursion, so CS SMs per polymer divide that time.
// Every dot product, norm and maximum is a CTA reduction followed by a
// cluster reduction: each CTA writes its partial to its own shared memory,
// the cluster synchronises (release / acquire), and every CTA reads the CS
// partials through distributed shared memory and combines them in rank order.
// All CTAs therefore hold bit-identical scalars and take every branch alike,
// so they reach the same cluster barriers.  Two partial slots alternate, so one
// cluster barrier per reduction suffices: a slot is written again only after
// the next reduction's barrier, which every CTA reaches after reading it.
// Neighbour beads across a slice boundary are read from global memory after a
// cluster barrier at the start of each evaluation.
__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ double ld_dsmem(const double *p, uint32_t rank) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    uint32_t ra;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(a), "r"(rank));
    double v;
    asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(ra) : "memory");
    return v;
}

struct ClRed {
    double *sred;   // CTA reduction scratch (32 doubles)
    double *cslot;  // this CTA's two partial slots
    int ph;         // slot of the next reduction
};

template <int CS, bool MAX>
__device__ __forceinline__ double cl_reduce(double v, ClRed &R) {
    v = MAX ? block_max(v, R.sred) : block_sum(v, R.sred);
    if (CS == 1) return v;
    if (threadIdx.x == 0) R.cslot[R.ph] = v;
    cluster_sync_all();
    double t = ld_dsmem(&R.cslot[R.ph], 0);
#pragma unroll
    for (uint32_t r = 1; r < (uint32_t)CS; r++) {
        const double u = ld_dsmem(&R.cslot[R.ph], r);
        t = MAX ? fmax(t, u) : t + u;
    }
    R.ph ^= 1;
    return t;
}

// The slice of one CTA: elements e = dof N + i, i in [i0, i1), walked as
// t = dof ns + (i - i0) so that consecutive threads take consecutive beads.
struct Slice {
    int N, nd, i0, ns;
    __device__ __forceinline__ int count() const { return nd * ns; }
    __device__ __forceinline__ int elem(int t) const {
        const int dof = t / ns;
        return dof * N + i0 + (t - dof * ns);
    }
};

template <int CS>
__device__ __forceinline__ double cl_dot(const double *a, const double *b, const Slice &sl, ClRed &R) {
    double s = 0.0;
    for (int t = threadIdx.x; t < sl.count(); t += blockDim.x) {
        const int e = sl.elem(t);
        s += a[e] * b[e];
    }
    return cl_reduce<CS, false>(s, R);
}

// UM and dUM/dx on this CTA's slice (x and g: [dof][N]; every thread gets UM).
template <int CS>
__device__ double polymer_fg_cl(const InstArgs &A, int k, const double *__restrict__ x, double *__restrict__ g,
                                const Slice &sl, ClRed &R) {
    if (CS > 1)
        cluster_sync_all();  // every slice of the point x is written (neighbour beads cross slices)
    else
        __syncthreads();
    const int N = A.N, nd = A.nd;
    const double bn = A.betan[k];
    const double *b = A.b + (size_t)k * nd;
    double part = 0.0;
    for (int i = sl.i0 + threadIdx.x; i < sl.i0 + sl.ns; i += blockDim.x) {
        double xb[kMaxDof], gb[kMaxDof];
        for (int d = 0; d < nd; d++) xb[d] = x[d * N + i];
        part += pes_vgrad<double>(A.pes, xb, gb);
        for (int d = 0; d < nd; d++) g[d * N + i] = gb[d];
    }
    __syncthreads();
    const bool fixed = A.fixedends != 0;
    for (int t = threadIdx.x; t < sl.count(); t += blockDim.x) {
        const int e = sl.elem(t);
        const int dof = e / N, i = e - dof * N;
        const double m = A.mass[dof / A.ndim];
        const double xe = x[e];
        // neighbours may lie in another CTA's slice: read them from L2 (__ldcg)
        const double xn = i < N - 1 ? __ldcg(x + e + 1) : 0.0;
        const double xl = i > 0 ? __ldcg(x + e - 1) : (fixed ? A.a[dof] : xe);
        const double xr = i < N - 1 ? xn : (fixed ? b[dof] : xe);
        g[e] = m * (2.0 * xe - xl - xr) / (bn * bn) + g[e];
        const double c = 0.5 * m / (bn * bn);
        if (i < N - 1) part += c * (xn - xe) * (xn - xe);
        if (fixed && i == 0) part += c * (xe - A.a[dof]) * (xe - A.a[dof]);
        if (fixed && i == N - 1) part += c * (b[dof] - xe) * (b[dof] - xe);
    }
    return cl_reduce<CS, false>(part, R);
}

template <int CS>
__global__ void __launch_bounds__(512) k_inst_lbfgs_cl(InstArgs A, LbfgsArgs L, double *__restrict__ xio,
                                                       double *__restrict__ scratch, double *__restrict__ um_out,
                                                       int64_t *__restrict__ iters, int32_t *__restrict__ status) {
    __shared__ double sred[32];
    __shared__ double cslot[2];
    __shared__ double s_rho[64], s_alpha[64];
    const uint32_t rank = CS > 1 ? cluster_rank() : 0u;
    const int k = (int)(blockIdx.x / CS);
    const int n = A.nd * A.N, m = L.m;
    Slice sl;
    sl.N = A.N;
    sl.nd = A.nd;
    sl.i0 = (int)((int64_t)rank * A.N / CS);
    sl.ns = (int)((int64_t)(rank + 1) * A.N / CS) - sl.i0;
    ClRed R{sred, cslot, 0};
    double *ws = scratch + (size_t)k * ((size_t)(5 + 2 * m) * n + 2 * m);
    double *x = ws, *g = ws + n, *d = ws + 2 * (size_t)n, *xt = ws + 3 * (size_t)n, *gt = ws + 4 * (size_t)n;
    double *S = ws + 5 * (size_t)n, *Y = S + (size_t)m * n;
    double *xk = xio + (size_t)k * n;
    const int cnt = sl.count();
    for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
        const int e = sl.elem(t);
        x[e] = xk[e];
    }
    double f = polymer_fg_cl<CS>(A, k, x, g, sl, R);
    const double eps = 2.220446049250313e-16;
    int npair = 0, head = 0;  // circular history
    int st = 1;
    int64_t it = 0;
    for (; it < L.maxiter; it++) {
        double gmax = 0.0;
        for (int t = threadIdx.x; t < cnt; t += blockDim.x) gmax = fmax(gmax, fabs(g[sl.elem(t)]));
        gmax = cl_reduce<CS, true>(gmax, R);
        if (gmax <= L.pgtol) {
            st = 0;
            break;
        }
        // two-loop recursion: d = -H g
        for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
            const int e = sl.elem(t);
            d[e] = -g[e];
        }
        __syncthreads();
        for (int c = 0; c < npair; c++) {
            const int j = (head - 1 - c + m) % m;
            const double a_ = s_rho[j] * cl_dot<CS>(S + (size_t)j * n, d, sl, R);
            if (threadIdx.x == 0) s_alpha[j] = a_;
            for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
                const int e = sl.elem(t);
                d[e] -= a_ * Y[(size_t)j * n + e];
            }
            __syncthreads();
        }
        if (npair > 0) {
            const int j = (head - 1 + m) % m;
            const double yy = cl_dot<CS>(Y + (size_t)j * n, Y + (size_t)j * n, sl, R);
            const double gam = 1.0 / (s_rho[j] * yy);
            for (int t = threadIdx.x; t < cnt; t += blockDim.x) d[sl.elem(t)] *= gam;
            __syncthreads();
        }
        for (int c = npair - 1; c >= 0; c--) {
            const int j = (head - 1 - c + m) % m;
            const double bt = s_rho[j] * cl_dot<CS>(Y + (size_t)j * n, d, sl, R);
            const double a_ = s_alpha[j];
            for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
                const int e = sl.elem(t);
                d[e] += (a_ - bt) * S[(size_t)j * n + e];
            }
            __syncthreads();
        }
        double gd = cl_dot<CS>(g, d, sl, R);
        if (!(gd < 0.0)) {  // not a descent direction: restart from steepest descent
            npair = 0;
            for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
                const int e = sl.elem(t);
                d[e] = -g[e];
            }
            __syncthreads();
            gd = cl_dot<CS>(g, d, sl, R);
        }
        // initial step: 1, or 1/|d| before any curvature pair (as L-BFGS-B's first iteration)
        double t = 1.0;
        if (npair == 0) {
            const double dn = sqrt(cl_dot<CS>(d, d, sl, R));
            t = dn > 0.0 ? fmin(1.0, 1.0 / dn) : 1.0;
        }
        bool accepted = false;
        double ft = 0.0;
        for (int bt = 0; bt <= L.max_bt; bt++) {
            for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
                const int e = sl.elem(q);
                xt[e] = x[e] + t * d[e];
            }
            ft = polymer_fg_cl<CS>(A, k, xt, gt, sl, R);
            if (ft <= f + 1.0e-4 * t * gd) {
                accepted = true;
                break;
            }
            // safeguarded quadratic interpolation of f(t)
            const double tq = -gd * t * t / (2.0 * (ft - f - gd * t));
            t = (tq > 0.1 * t && tq < 0.5 * t) ? tq : 0.5 * t;
        }
        if (!accepted) {
            st = 2;
            break;
        }
        // new curvature pair s = xt - x, y = gt - g
        double *Sj = S + (size_t)head * n, *Yj = Y + (size_t)head * n;
        for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
            const int e = sl.elem(q);
            Sj[e] = xt[e] - x[e];
            Yj[e] = gt[e] - g[e];
        }
        __syncthreads();
        const double sy = cl_dot<CS>(Sj, Yj, sl, R);
        const double yy = cl_dot<CS>(Yj, Yj, sl, R);
        if (sy > eps * yy) {
            if (threadIdx.x == 0) s_rho[head] = 1.0 / sy;
            head = (head + 1) % m;
            npair = npair < m ? npair + 1 : m;
        }
        const double fold = f;
        for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
            const int e = sl.elem(q);
            x[e] = xt[e];
            g[e] = gt[e];
        }
        f = ft;
        __syncthreads();
        // relative reduction test of L-BFGS-B: (f_k - f_k+1)/max(|f_k|, |f_k+1|, 1) <= factr * eps
        if ((fold - f) <= L.factr * eps * fmax(fmax(fabs(fold), fabs(f)), 1.0)) {
            st = 0;
            it++;
            break;
        }
    }
    for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
        const int e = sl.elem(q);
        xk[e] = x[e];
    }
    if (threadIdx.x == 0 && rank == 0) {
        um_out[k] = f;
        iters[k] = it;
        status[k] = st;
    }
    if (CS > 1) cluster_sync_all();  // no CTA leaves while another may still read its partial slots
}

// Per-bead PES Hessians of polymer k (FD surfaces: one thread per (bead, column)).
__global__ void k_bead_hessians(PesArgs pa, int N, int nbeta, const double *__restrict__ x,
                                double *__restrict__ hb, int quirks, int singlewell) {
    const int nd = pa.nd;
    const bool fd = hess_is_fd(pa.id);
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t per = fd ? (int64_t)N * nd : (int64_t)N;
    const int64_t k = t / per;
    if (k >= nbeta) return;
    const int64_t r = t - k * per;
    const int i = fd ? (int)(r / nd) : (int)r;
    if (singlewell && i > 0) return;  // instantonmod.f90:183: only bead 1 when singlewell
    double xb[kMaxDof];
    const double *xk = x + (size_t)k * nd * N;
    for (int d = 0; d < nd; d++) xb[d] = xk[d * N + i];
    double *h = hb + ((size_t)k * N + i) * nd * nd;
    if (fd)
        hess_fd_column(pa, xb, (int)(r % nd), h);
    else
        pes_hessian(pa, xb, h, quirks);
}

// Band assembly of UMhessian: one thread per (polymer, bead, idof1).
__global__ void k_band_assemble(InstArgs A, int nbeta, const double *__restrict__ hb, int singlewell,
                                int quirks, double *__restrict__ band) {
    const int N = A.N, nd = A.nd, ld = nd + 1;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t k = t / ((int64_t)N * nd);
    if (k >= nbeta) return;
    const int64_t r = t - k * (int64_t)N * nd;
    const int i = (int)(r / nd), id1 = (int)(r % nd);
    const int64_t tot = (int64_t)N * nd;
    const double bn = A.betan[k];
    const double *h = hb + ((size_t)k * N + (singlewell ? 0 : i)) * nd * nd;
    double *bk = band + (size_t)k * ld * tot;
    const int64_t f1 = (int64_t)nd * i + id1;
    const int k1 = id1 / A.ndim;
    for (int id2 = id1; id2 < nd; id2++) {
        const int k2 = id2 / A.ndim;
        const double hv = h[id2 + nd * id1] / sqrt(A.mass[k1] * A.mass[k2]);
        if (id2 == id1) {
            bk[0 + ld * f1] = 2.0 / (bn * bn) + hv;
        } else {
            bk[(id2 - id1) + ld * f1] = hv;
        }
    }
    // rows below the intra-bead block in this column: zero, then the spring coupling
    for (int rr = nd - id1; rr <= nd; rr++)
        if (rr >= 1) bk[rr + ld * f1] = 0.0;
    const bool coupled = quirks ? (i > 0) : (i < N - 1);
    if (coupled && f1 + nd < tot) bk[nd + ld * f1] = -1.0 / (bn * bn);
}

// Banded LDL^T (no pivoting) of (A - sigma I) for polymer k, sliding (kd+1)^2
// window in shared memory.  Returns log|det| and the number of negative pivots
// (Sylvester inertia = number of eigenvalues below sigma).
__global__ void k_band_ldl(int64_t n, int kd, const double *__restrict__ band, const double *__restrict__ sigma,
                           double *__restrict__ logabs, int64_t *__restrict__ nneg) {
    extern __shared__ double W[];  // (kd+1) slots x (kd+1) rows
    __shared__ double s_d;
    const int k = blockIdx.x;
    const int ld = kd + 1;
    const double *bk = band + (size_t)k * ld * n;
    const double sg = sigma[k];
    // load columns 0..kd
    for (int e = threadIdx.x; e < ld * ld; e += blockDim.x) {
        const int c = e / ld, r = e - c * ld;
        double v = (c < n && c + r < n) ? bk[r + (size_t)ld * c] : 0.0;
        if (r == 0) v -= sg;
        W[(c % ld) * ld + r] = v;
    }
    // triangle (ii, kk) with 1 <= kk <= ii <= kd assigned to threads (<= 4 each)
    const int ntri = kd * (kd + 1) / 2;
    int tri_i[4], tri_k[4], ntq = 0;
    for (int q = threadIdx.x; q < ntri && ntq < 4; q += blockDim.x) {
        int ii = 1;
        while ((ii + 1) * ii / 2 <= q) ii++;
        tri_i[ntq] = ii;
        tri_k[ntq] = q - ii * (ii - 1) / 2 + 1;
        ntq++;
    }
    __syncthreads();
    double la = 0.0;
    int64_t nn = 0;
    for (int64_t j = 0; j < n; j++) {
        const int s = (int)(j % ld);
        if (threadIdx.x == 0) {
            double dj = W[s * ld + 0];
            if (dj == 0.0) dj = 1e-300;
            s_d = dj;
            la += log(fabs(dj));
            nn += dj < 0.0 ? 1 : 0;
        }
        __syncthreads();
        const double dj = s_d;
        for (int t = 0; t < ntq; t++) {
            const int ii = tri_i[t], kk = tri_k[t];
            if (j + ii >= n) continue;
            const double lij = W[s * ld + ii], lkj = W[s * ld + kk];
            const int sk = (int)((j + kk) % ld);
            W[sk * ld + (ii - kk)] -= lij * lkj / dj;
        }
        __syncthreads();
        // retire column j, load column j + kd + 1 into its slot
        const int64_t c = j + ld;
        for (int r = threadIdx.x; r < ld; r += blockDim.x) {
            double v = (c < n && c + r < n) ? bk[r + (size_t)ld * c] : 0.0;
            if (r == 0) v -= sg;
            W[s * ld + r] = v;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        logabs[k] = la;
        nneg[k] = nn;
    }
}

// One warp per factorisation f (polymer fpoly[f] at the shift fsig[f]): the
// banded LDL^T of k_band_ldl with warp synchronisation only.  The (kd+1)^2
// window lives in shared memory (one per warp); the columns entering the window
// are loaded kLdlAhead steps early into a register ring (lane r holds rows r
// and r + 32); |det| is carried as a mantissa in [0.5, 1) and a binary exponent
// (one log at the end); the Sylvester inertia counts the negative pivots.
// Requires kd + 1 <= 64.  One warp per CTA, so that the factorisations of a
// round spread over the SMs (their FP64 pipes bound the kernel).
constexpr int kLdlWarps = 1;
constexpr int kLdlAhead = 8;
__global__ void __launch_bounds__(32 * kLdlWarps) k_band_ldl_w(int64_t n, int kd, const double *__restrict__ band,
                                                               int nfac, const int32_t *__restrict__ fpoly,
                                                               const double *__restrict__ fsig,
                                                               double *__restrict__ logabs,
                                                               int64_t *__restrict__ nneg) {
    extern __shared__ double smw[];
    const int ld = kd + 1;
    const int ntri = kd * (kd + 1) / 2;
    double *Ls = smw + (size_t)kLdlWarps * ld * ld;  // per warp: the pivot column scaled by 1/d
    uint16_t *tri = reinterpret_cast<uint16_t *>(Ls + (size_t)kLdlWarps * ld);
    for (int q = threadIdx.x; q < ntri; q += blockDim.x) {  // (ii, kk), 1 <= kk <= ii <= kd
        int ii = 1;
        while ((ii + 1) * ii / 2 <= q) ii++;
        tri[q] = (uint16_t)((ii << 8) | (q - ii * (ii - 1) / 2 + 1));
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int f = blockIdx.x * kLdlWarps + warp;
    if (f >= nfac) return;  // whole warps
    double *W = smw + (size_t)warp * ld * ld;
    double *L = Ls + (size_t)warp * ld;
    const double *bk = band + (size_t)fpoly[f] * ld * n;
    const double sg = fsig[f];
    auto colv = [&](int64_t c, int r) -> double {  // row r of column c of (A - sigma I), 0 outside
        if (r >= ld || c >= n || c + r >= n) return 0.0;
        const double v = bk[r + (size_t)ld * c];
        return r == 0 ? v - sg : v;
    };
    for (int e = lane; e < ld * ld; e += 32) {
        const int c = e / ld, r = e - c * ld;
        W[c * ld + r] = colv(c, r);  // column c < ld in slot c
    }
    double pre[kLdlAhead][2];
#pragma unroll
    for (int u = 0; u < kLdlAhead; u++) {
        pre[u][0] = colv(ld + u, lane);
        pre[u][1] = colv(ld + u, lane + 32);
    }
    __syncwarp();
    double mant = 1.0;
    int64_t ex = 0, nn = 0;
    int sl = 0;  // window slot of column j
    for (int64_t j0 = 0; j0 < n; j0 += kLdlAhead) {
#pragma unroll
        for (int u = 0; u < kLdlAhead; u++) {
            const int64_t j = j0 + u;
            if (j >= n) break;  // warp-uniform
            double dj = W[sl * ld];
            if (dj == 0.0) dj = 1e-300;
            nn += dj < 0.0 ? 1 : 0;
            {  // mant <- mant |d_j| scaled back into [0.5, 1) through its IEEE exponent field
                const long long bits = __double_as_longlong(mant * fabs(dj));
                ex += ((bits >> 52) & 0x7ff) - 1022;
                mant = __longlong_as_double((bits & ~(0x7ffLL << 52)) | (1022LL << 52));
            }
            const double rinv = 1.0 / dj;
            if (lane < ld) L[lane] = W[sl * ld + lane] * rinv;
            if (lane + 32 < ld) L[lane + 32] = W[sl * ld + lane + 32] * rinv;
            __syncwarp();
            for (int q = lane; q < ntri; q += 32) {  // W(j+kk, j+ii) -= l_ii d l_kk = L[ii] W(j, j+kk)
                const int tv = tri[q], ii = tv >> 8, kk = tv & 255;
                if (j + ii >= n) continue;
                int sk = sl + kk;
                if (sk >= ld) sk -= ld;
                W[sk * ld + (ii - kk)] -= L[ii] * W[sl * ld + kk];
            }
            __syncwarp();
            // slot sl takes column j + ld; its ring entry is refilled kLdlAhead columns on
            if (lane < ld) W[sl * ld + lane] = pre[u][0];
            if (lane + 32 < ld) W[sl * ld + lane + 32] = pre[u][1];
            pre[u][0] = colv(j + ld + kLdlAhead, lane);
            pre[u][1] = colv(j + ld + kLdlAhead, lane + 32);
            __syncwarp();
            sl = sl + 1 == ld ? 0 : sl + 1;
        }
    }
    if (lane == 0) {
        logabs[f] = log(mant) + (double)ex * 0.6931471805599453;
        nneg[f] = nn;
    }
}

// Gershgorin lower bound of every band and its smallest diagonal element, one
// CTA per polymer.
__global__ void k_band_bounds(int64_t n, int kd, const double *__restrict__ band, double *__restrict__ glo,
                              double *__restrict__ dmin) {
    __shared__ double s_lo[32], s_mn[32];
    const int ld = kd + 1;
    const double *bk = band + (size_t)blockIdx.x * ld * n;
    double lo = 1e300, mn = 1e300;
    for (int64_t c = threadIdx.x; c < n; c += blockDim.x) {
        double rad = 0.0;
        for (int r = 1; r <= kd; r++) {
            if (c + r < n) rad += fabs(bk[r + (size_t)ld * c]);
            if (c - r >= 0) rad += fabs(bk[r + (size_t)ld * (c - r)]);
        }
        const double dg = bk[(size_t)ld * c];
        lo = fmin(lo, dg - rad);
        mn = fmin(mn, dg);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    }
    if ((threadIdx.x & 31) == 0) {
        s_lo[threadIdx.x >> 5] = lo;
        s_mn[threadIdx.x >> 5] = mn;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) {
            lo = fmin(lo, s_lo[w]);
            mn = fmin(mn, s_mn[w]);
        }
        glo[blockIdx.x] = lo;
        dmin[blockIdx.x] = mn;
    }
}

InstArgs make_inst_args(pg_ctx *ctx, int N, const double *da, const double *db, const double *dbn) {
    InstArgs A;
    A.pes = ctx->pes_args();
    A.N = N;
    A.fixedends = ctx->fixedends;
    A.nd = ctx->nd;
    A.ndim = ctx->ndim;
    A.natom = ctx->natom;
    A.mass = ctx->d_mass.as<double>();
    A.a = da;
    A.b = db;
    A.betan = dbn;
    return A;
}

// Device band of nbeta polymers (ld x tot each) into ctx->scratch_d.
int build_bands(pg_ctx *ctx, int64_t nbeta, int64_t N, const double *dx, const double *dbn, int singlewell,
                int quirks) {
    const int nd = ctx->nd;
    const int64_t tot = N * nd, ld = nd + 1;
    PG_CUDA(ctx->scratch_c.ensure((size_t)nbeta * N * nd * nd * sizeof(double)));
    PG_CUDA(ctx->scratch_d.ensure((size_t)nbeta * ld * tot * sizeof(double)));
    PG_CUDA(cudaMemsetAsync(ctx->scratch_d.ptr, 0, (size_t)nbeta * ld * tot * sizeof(double), ctx->stream));
    const bool fd = hess_is_fd_host(ctx->pes_id);
    int64_t nth = fd ? nbeta * N * nd : nbeta * N;
    k_bead_hessians<<<(unsigned)((nth + 127) / 128), 128, 0, ctx->stream>>>(
        ctx->pes_args(), (int)N, (int)nbeta, dx, ctx->scratch_c.as<double>(), quirks, singlewell);
    PG_CUDA(cudaGetLastError());
    InstArgs A = make_inst_args(ctx, (int)N, nullptr, nullptr, dbn);
    int64_t nb = nbeta * N * nd;
    k_band_assemble<<<(unsigned)((nb + 127) / 128), 128, 0, ctx->stream>>>(A, (int)nbeta, ctx->scratch_c.as<double>(),
                                                                           singlewell, quirks, ctx->scratch_d.as<double>());
    PG_CUDA(cudaGetLastError());
    return PG_OK;
}

}  // namespace
}  // namespace pg

using namespace pg;

static int upload(pg_ctx *ctx, DevBuf &buf, const double *h, size_t n) {
    PG_CUDA(buf.ensure(n * sizeof(double)));
    PG_CUDA(cudaMemcpyAsync(buf.ptr, h, n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    return PG_OK;
}

// [a (nd) | b (nbeta nd) | betan (nbeta)] on the device.  With free ends
// (pg_set_fixedends(ctx, 0)) a and b may be NULL: the action never reads them,
// and zeros stand in (the reference passes neither, instantonmod.f90:756-762).
static int upload_ends(pg_ctx *ctx, DevBuf &dab, int64_t nbeta, const double *a, const double *b,
                       const double *betan) {
    const int nd = ctx->nd;
    if (ctx->fixedends && (!a || !b)) return fail(PG_ERR_ARG, "fixed ends need the end points a and b");
    PG_CUDA(dab.ensure((size_t)(nd + nbeta * nd + nbeta) * sizeof(double)));
    if (a)
        PG_CUDA(cudaMemcpyAsync(dab.ptr, a, nd * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    else
        PG_CUDA(cudaMemsetAsync(dab.ptr, 0, nd * sizeof(double), ctx->stream));
    if (b)
        PG_CUDA(cudaMemcpyAsync(dab.as<double>() + nd, b, nbeta * nd * sizeof(double), cudaMemcpyHostToDevice,
                                ctx->stream));
    else
        PG_CUDA(cudaMemsetAsync(dab.as<double>() + nd, 0, nbeta * nd * sizeof(double), ctx->stream));
    PG_CUDA(cudaMemcpyAsync(dab.as<double>() + nd + nbeta * nd, betan, nbeta * sizeof(double), cudaMemcpyHostToDevice,
                            ctx->stream));
    return PG_OK;
}

extern "C" int pg_set_fixedends(pg_ctx *ctx, int32_t fixedends) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if (fixedends != 0 && fixedends != 1) return fail(PG_ERR_ARG, "fixedends must be 0 or 1");
    ctx->fixedends = fixedends;
    return PG_OK;
}

extern "C" int pg_instanton_fg(pg_ctx *ctx, int64_t nbeta, int64_t N, const double *x, const double *a,
                               const double *b, const double *betan, double *UM, double *grad) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (nbeta < 1 || N < 2 || !x || !betan) return fail(PG_ERR_ARG, "bad instanton_fg arguments");
    const int nd = ctx->nd;
    const size_t n = (size_t)nbeta * nd * N;
    DevBuf dx, dg, dab, dum;
    if ((rc = upload(ctx, dx, x, n))) return rc;
    if ((rc = upload_ends(ctx, dab, nbeta, a, b, betan))) return rc;
    PG_CUDA(dg.ensure(n * sizeof(double)));
    PG_CUDA(dum.ensure(nbeta * sizeof(double)));
    InstArgs A = make_inst_args(ctx, (int)N, dab.as<double>(), dab.as<double>() + nd, dab.as<double>() + nd + nbeta * nd);
    k_inst_fg<<<(unsigned)nbeta, 256, 0, ctx->stream>>>(A, dx.as<double>(), dum.as<double>(), dg.as<double>());
    PG_CUDA(cudaGetLastError());
    if (UM) PG_CUDA(cudaMemcpyAsync(UM, dum.ptr, nbeta * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    if (grad) PG_CUDA(cudaMemcpyAsync(grad, dg.ptr, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    PG_CUDA(cudaStreamSynchronize(ctx->stream));
    return PG_OK;
}

extern "C" int pg_instanton_optimize(pg_ctx *ctx, int64_t nbeta, int64_t N, double *x, const double *a,
                                     const double *b, const double *betan, const pg_lbfgs_opts *opts, double *UM,
                                     int64_t *niter, int32_t *status) {
    NvtxRange nvtx_range("pg_instanton_optimize");
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (nbeta < 1 || N < 2 || !x || !betan || !opts) return fail(PG_ERR_ARG, "bad optimize arguments");
    if (opts->m < 1 || opts->m > 64 || opts->maxiter < 1 || opts->max_backtracks < 0)
        return fail(PG_ERR_ARG, "bad L-BFGS options");
    const int cs_req = opts->cluster_ctas;
    if (cs_req != 0 && cs_req != 1 && cs_req != 2 && cs_req != 4 && cs_req != 8)
        return fail(PG_ERR_ARG, "cluster_ctas must be 0, 1, 2, 4 or 8");
    if (cs_req > N) return fail(PG_ERR_ARG, "cluster_ctas exceeds the number of beads");
    const int nd = ctx->nd;
    const size_t n1 = (size_t)nd * N, n = (size_t)nbeta * n1;
    DevBuf dx, dab, dum, dit, dst;
    if ((rc = upload(ctx, dx, x, n))) return rc;
    if ((rc = upload_ends(ctx, dab, nbeta, a, b, betan))) return rc;
    const size_t per = (size_t)(5 + 2 * opts->m) * n1 + 2 * opts->m;
    PG_CUDA(ctx->scratch_b.ensure((size_t)nbeta * per * sizeof(double)));
    PG_CUDA(dum.ensure(nbeta * sizeof(double)));
    PG_CUDA(dit.ensure(nbeta * sizeof(int64_t)));
    PG_CUDA(dst.ensure(nbeta * sizeof(int32_t)));
    InstArgs A = make_inst_args(ctx, (int)N, dab.as<double>(), dab.as<double>() + nd, dab.as<double>() + nd + nbeta * nd);
    LbfgsArgs L;
    L.m = opts->m;
    L.max_bt = opts->max_backtracks;
    L.maxiter = opts->maxiter;
    L.factr = opts->factr;
    L.pgtol = opts->pgtol;
    // CTAs per polymer: as many as the GPU holds for the whole batch in one
    // wave (at most 8, a portable cluster), keeping at least 16 beads per CTA
    int cs = cs_req;
    if (cs == 0) {
        cs = 1;
        while (cs < 8 && nbeta * (cs * 2) <= (int64_t)ctx->sm_count && N >= 16 * (int64_t)(cs * 2)) cs *= 2;
    }
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3((unsigned)(nbeta * cs));
    lc.blockDim = dim3(512);
    lc.stream = ctx->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)cs;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    lc.attrs = attr;
    lc.numAttrs = 1;
    double *xdev = dx.as<double>(), *sdev = ctx->scratch_b.as<double>(), *udev = dum.as<double>();
    int64_t *idev = dit.as<int64_t>();
    int32_t *stdev = dst.as<int32_t>();
    cudaError_t e = cudaSuccess;
    switch (cs) {
        case 1: e = cudaLaunchKernelEx(&lc, k_inst_lbfgs_cl<1>, A, L, xdev, sdev, udev, idev, stdev); break;
        case 2: e = cudaLaunchKernelEx(&lc, k_inst_lbfgs_cl<2>, A, L, xdev, sdev, udev, idev, stdev); break;
        case 4: e = cudaLaunchKernelEx(&lc, k_inst_lbfgs_cl<4>, A, L, xdev, sdev, udev, idev, stdev); break;
        default: e = cudaLaunchKernelEx(&lc, k_inst_lbfgs_cl<8>, A, L, xdev, sdev, udev, idev, stdev); break;
    }
    PG_CUDA(e);
    PG_CUDA(cudaGetLastError());
    PG_CUDA(cudaMemcpyAsync(x, dx.ptr, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    if (UM) PG_CUDA(cudaMemcpyAsync(UM, dum.ptr, nbeta * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    if (niter) PG_CUDA(cudaMemcpyAsync(niter, dit.ptr, nbeta * sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
    if (status) PG_CUDA(cudaMemcpyAsync(status, dst.ptr, nbeta * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    PG_CUDA(cudaStreamSynchronize(ctx->stream));
    return PG_OK;
}

extern "C" int pg_um_hessian(pg_ctx *ctx, int64_t N, double betan, const double *x, int32_t singlewell,
                             int32_t quirks, double *band) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (N < 2 || !x || !band) return fail(PG_ERR_ARG, "bad um_hessian arguments");
    const int nd = ctx->nd;
    DevBuf dx, dbn;
    if ((rc = upload(ctx, dx, x, (size_t)nd * N))) return rc;
    if ((rc = upload(ctx, dbn, &betan, 1))) return rc;
    rc = build_bands(ctx, 1, N, dx.as<double>(), dbn.as<double>(), singlewell, quirks);
    if (rc) return rc;
    PG_CUDA(cudaMemcpyAsync(band, ctx->scratch_d.ptr, (size_t)(nd + 1) * N * nd * sizeof(double),
                            cudaMemcpyDeviceToHost, ctx->stream));
    PG_CUDA(cudaStreamSynchronize(ctx->stream));
    return PG_OK;
}

// log|det(H_p - sigma I)| and inertia of factorisations f = (fpoly[f], fsig[f]).
struct LdlBufs {
    DevBuf poly, sig, logv, neg;
};
static int band_factor(pg_ctx *ctx, int64_t nbeta, int64_t n, int kd, const std::vector<int32_t> &fpoly,
                       const std::vector<double> &fsig, std::vector<double> &hlog, std::vector<int64_t> &hneg,
                       LdlBufs &b) {
    const int nfac = (int)fpoly.size();
    hlog.assign(nfac, 0.0);
    hneg.assign(nfac, 0);
    if (nfac == 0) return PG_OK;
    PG_CUDA(b.poly.ensure((size_t)nfac * sizeof(int32_t)));
    PG_CUDA(b.sig.ensure((size_t)nfac * sizeof(double)));
    PG_CUDA(b.logv.ensure((size_t)nfac * sizeof(double)));
    PG_CUDA(b.neg.ensure((size_t)nfac * sizeof(int64_t)));
    PG_CUDA(cudaMemcpyAsync(b.poly.ptr, fpoly.data(), nfac * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream));
    PG_CUDA(cudaMemcpyAsync(b.sig.ptr, fsig.data(), nfac * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    const int ld = kd + 1;
    if (ld <= 64) {
        const size_t sm = (size_t)kLdlWarps * (ld + 1) * ld * sizeof(double) +
                          (size_t)kd * (kd + 1) / 2 * sizeof(uint16_t);
        if (sm > 48 * 1024)
            PG_CUDA(cudaFuncSetAttribute(k_band_ldl_w, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        k_band_ldl_w<<<(unsigned)((nfac + kLdlWarps - 1) / kLdlWarps), 32 * kLdlWarps, sm, ctx->stream>>>(
            n, kd, ctx->scratch_d.as<double>(), nfac, b.poly.as<int32_t>(), b.sig.as<double>(), b.logv.as<double>(),
            b.neg.as<int64_t>());
        PG_CUDA(cudaGetLastError());
    } else {  // wide bands: one CTA per polymer and shift, per polymer in turn
        int th = kd * (kd + 1) / 2;
        th = th < 32 ? 32 : (th > 512 ? 512 : ((th + 31) / 32) * 32);
        if (kd * (kd + 1) / 2 > 4 * th) return fail(PG_ERR_UNSUPPORTED, "band width too large for the LDL kernel");
        std::vector<double> sig1(nbeta, 0.0);
        for (int f = 0; f < nfac; f++) {
            // the polymer-indexed kernel: polymer fpoly[f] only, at its shift
            PG_CUDA(cudaMemcpyAsync(b.sig.as<double>() + nfac - 1, &fsig[f], sizeof(double), cudaMemcpyHostToDevice,
                                    ctx->stream));
            (void)sig1;
            k_band_ldl<<<1, th, (size_t)ld * ld * sizeof(double), ctx->stream>>>(
                n, kd, ctx->scratch_d.as<double>() + (size_t)fpoly[f] * ld * n, b.sig.as<double>() + nfac - 1,
                b.logv.as<double>() + f, b.neg.as<int64_t>() + f);
            PG_CUDA(cudaGetLastError());
            PG_CUDA(cudaStreamSynchronize(ctx->stream));  // the shift slot is reused
        }
    }
    PG_CUDA(cudaMemcpyAsync(hlog.data(), b.logv.ptr, nfac * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    PG_CUDA(cudaMemcpyAsync(hneg.data(), b.neg.ptr, nfac * sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
    PG_CUDA(cudaStreamSynchronize(ctx->stream));
    return PG_OK;
}

extern "C" int pg_instanton_logdet(pg_ctx *ctx, int64_t nbeta, int64_t N, const double *x, const double *betan,
                                   int32_t singlewell, int32_t skip_lowest, int32_t quirks, double *lndet,
                                   double *eta2_min, int64_t *nskipped) {
    NvtxRange nvtx_range("pg_instanton_logdet");
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (nbeta < 1 || N < 2 || !x || !betan || !lndet) return fail(PG_ERR_ARG, "bad logdet arguments");
    const int nd = ctx->nd, kd = nd, ld = nd + 1;
    const int64_t n = N * nd;
    DevBuf dx, dbn, dglo, ddmin;
    LdlBufs lb;
    if ((rc = upload(ctx, dx, x, (size_t)nbeta * n))) return rc;
    if ((rc = upload(ctx, dbn, betan, nbeta))) return rc;
    PG_CUDA(dglo.ensure(nbeta * sizeof(double)));
    PG_CUDA(ddmin.ensure(nbeta * sizeof(double)));
    rc = build_bands(ctx, nbeta, N, dx.as<double>(), dbn.as<double>(), singlewell, quirks);
    if (rc) return rc;
    // Gershgorin lower bound and smallest diagonal element of every band
    std::vector<double> glo(nbeta), dmin(nbeta);
    k_band_bounds<<<(unsigned)nbeta, 256, 0, ctx->stream>>>(n, kd, ctx->scratch_d.as<double>(), dglo.as<double>(),
                                                              ddmin.as<double>());
    PG_CUDA(cudaGetLastError());
    PG_CUDA(cudaMemcpyAsync(glo.data(), dglo.ptr, nbeta * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    PG_CUDA(cudaMemcpyAsync(dmin.data(), ddmin.ptr, nbeta * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    PG_CUDA(cudaStreamSynchronize(ctx->stream));
    std::vector<int32_t> fpoly(nbeta);
    std::vector<double> fsig(nbeta, 0.0), la0, lac;
    std::vector<int64_t> nn0, nnc;
    for (int64_t k = 0; k < nbeta; k++) fpoly[k] = (int32_t)k;
    rc = band_factor(ctx, nbeta, n, kd, fpoly, fsig, la0, nn0, lb);  // sigma = 0: log|det| and inertia
    if (rc) return rc;
    // eigenvalues below zero (and the lowest one) by multisection on the inertia
    // count: S shifts per polymer and round split its interval into S + 1 parts.
    // A factorisation is a chain of n dependent pivots (its time hardly depends
    // on how many run at once), so a round uses about ten warps per SM.
    const int S = ld <= 64 ? (int)std::max<int64_t>(3, std::min<int64_t>(63, 10 * (int64_t)std::max(ctx->sm_count, 1) / nbeta))
                           : 1;
    const int kMaxNeg = 8;
    std::vector<std::vector<double>> negs(nbeta);
    std::vector<double> lmin(nbeta, 0.0);
    int64_t maxneg = 0;
    for (int64_t k = 0; k < nbeta; k++) maxneg = std::max<int64_t>(maxneg, nn0[k]);
    if (maxneg > kMaxNeg) return fail(PG_ERR_NUMERIC, "more than 8 negative Hessian eigenvalues");
    // index list per polymer: eigenvalues 1..nn0 (all negative), or eigenvalue 1 if skip_lowest
    for (int idx = 1; idx <= std::max<int64_t>(maxneg, 1); idx++) {
        std::vector<double> lo(nbeta), hi(nbeta);
        std::vector<char> act(nbeta, 0);
        bool any = false;
        for (int64_t k = 0; k < nbeta; k++) {
            if (idx <= nn0[k]) {
                lo[k] = glo[k];
                hi[k] = 0.0;
                act[k] = 1;
            } else if (idx == 1 && (skip_lowest || eta2_min)) {
                lo[k] = std::fmax(0.0, glo[k]);
                hi[k] = dmin[k];
                act[k] = 1;
            }
            any = any || act[k];
        }
        if (!any) break;
        for (int itb = 0; itb < 200; itb++) {
            fpoly.clear();
            fsig.clear();
            for (int64_t k = 0; k < nbeta; k++) {
                if (!act[k]) continue;
                if (!((hi[k] - lo[k]) > 1e-13 * std::fmax(std::fabs(lo[k]), std::fabs(hi[k])) &&
                      (hi[k] - lo[k]) > 1e-300))
                    continue;  // converged
                for (int t = 0; t < S; t++) {
                    fpoly.push_back((int32_t)k);
                    fsig.push_back(lo[k] + (hi[k] - lo[k]) * (double)(t + 1) / (double)(S + 1));
                }
            }
            if (fpoly.empty()) break;
            rc = band_factor(ctx, nbeta, n, kd, fpoly, fsig, lac, nnc, lb);
            if (rc) return rc;
            for (size_t f0 = 0; f0 < fpoly.size(); f0 += S) {  // the S shifts of one polymer, ascending
                const int64_t k = fpoly[f0];
                int t = 0;
                while (t < S && nnc[f0 + t] < idx) t++;  // first shift with >= idx eigenvalues below
                const double nlo = t > 0 ? fsig[f0 + t - 1] : lo[k];
                const double nhi = t < S ? fsig[f0 + t] : hi[k];
                lo[k] = nlo;
                hi[k] = nhi;
            }
        }
        for (int64_t k = 0; k < nbeta; k++) {
            if (!act[k]) continue;
            double ev = 0.5 * (lo[k] + hi[k]);
            if (idx <= nn0[k]) negs[k].push_back(ev);
            if (idx == 1) lmin[k] = ev;
        }
    }
    for (int64_t k = 0; k < nbeta; k++) {
        // sum of log eta^2 over eta^2 > 0 = log|det| - sum over the negative ones
        double s = la0[k];
        for (double v : negs[k]) s -= std::log(std::fabs(v));
        int64_t skipped = (int64_t)negs[k].size();
        if (skip_lowest && nn0[k] == 0) {  // eigenvalue 1 is positive: drop it too
            s -= std::log(lmin[k]);
            skipped += 1;
        }
        lndet[k] = s;
        if (eta2_min) eta2_min[k] = lmin[k];
        if (nskipped) nskipped[k] = skipped;
    }
    return PG_OK;
}
