// pg_device.cuh -- device building blocks shared by the ring-polymer kernels:
// counter-based RNG (Philox4x32-10), normal deviates, and the PES functors
// (device twins of the mcmod_* V / Vprime routines).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace pg {

constexpr double kPiRef = 3.14159265358979;  // instantonmod.f90:4 (truncated)
constexpr double kTwoPi = 6.283185307179586;

// ---------------------------------------------------------------- Philox4x32-10
// Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3",
// SC'11.  Counter = {block, step, stream, purpose}, key = 64-bit seed.
struct U4 {
    uint32_t x, y, z, w;
};

__host__ __device__ __forceinline__ U4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2,
                                                     uint32_t c3, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; r++) {
        // 32 x 32 -> 64-bit products (one wide multiply each on the device)
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t lo0 = (uint32_t)p0, hi0 = (uint32_t)(p0 >> 32);
        const uint32_t lo1 = (uint32_t)p1, hi1 = (uint32_t)(p1 >> 32);
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return U4{c0, c1, c2, c3};
}

// RNG purposes (counter word 3).
enum : uint32_t {
    kRngLangevin = 0,   // OU noise, one normal per (dof, mode) per step
    kRngInitP = 1,      // initial NM momenta
    kRngInitX = 2,      // initial position noise
    kRngAndersen = 3,   // Andersen momentum resampling
    kRngPoisson0 = 4,   // first Andersen interval
    kRngReinitX = 5,    // dHdrlimit re-initialisation, positions
    kRngReinitP = 6,    // dHdrlimit re-initialisation, momenta
    kRngPoisson = 7,    // later Andersen intervals
};

__host__ __device__ __forceinline__ U4 philox_block(uint64_t seed, uint32_t stream, uint32_t step,
                                                    uint32_t purpose, uint32_t blk) {
    return philox4x32_10(blk, step, stream, purpose, (uint32_t)seed, (uint32_t)(seed >> 32));
}

__host__ __device__ __forceinline__ double u32_unit_d(uint32_t w) {
    return ((double)w + 0.5) * 2.3283064365386963e-10;
}

// FP64 Box-Muller pair from two words: (r cos th, r sin th).
__device__ __forceinline__ void box_muller_d(uint32_t wa, uint32_t wb, double &z0, double &z1) {
    double ua = u32_unit_d(wa), ub = u32_unit_d(wb);
    double r = sqrt(-2.0 * log(ua));
    double s, c;
    sincos(kTwoPi * ub, &s, &c);
    z0 = r * c;
    z1 = r * s;
}

// n-th normal of the stream in FP64 (bit-compatible with the CPU restatement up
// to libm rounding).
__device__ __forceinline__ double normal_d(uint64_t seed, uint32_t stream, uint32_t step,
                                           uint32_t purpose, uint32_t n) {
    U4 o = philox_block(seed, stream, step, purpose, n >> 2);
    uint32_t wa, wb;
    if ((n >> 1) & 1) {
        wa = o.z;
        wb = o.w;
    } else {
        wa = o.x;
        wb = o.y;
    }
    double z0, z1;
    box_muller_d(wa, wb, z0, z1);
    return (n & 1) ? z1 : z0;
}

// FP32 Box-Muller from the top 24 bits of the same words: radius from one
// MUFU lg2 and one rsqrt, angle 2 pi u from the hardware sine / cosine on
// [-pi, pi) (2 pi u = theta + pi, so sin and cos change sign); absolute error
// of a normal below 1e-5, far inside the thermostat's statistical noise.
__device__ __forceinline__ void box_muller_f(uint32_t wa, uint32_t wb, float &z0, float &z1) {
    float ua = ((float)(wa >> 8) + 0.5f) * 5.9604644775390625e-08f;
    // lg2.approx has an absolute error near u = 1 and can return 0 (or a tiny
    // positive value) there; clamp so that r stays finite (r -> ~0 for u -> 1).
    float t = fmaxf(-2.0f * 0.69314718055994531f * __log2f(ua), 1.0e-30f);
    float r = t * rsqrtf(t);
    const float ub = ((float)(wb >> 8) + 0.5f) * 5.9604644775390625e-08f;  // (0, 1)
    float s, c;
    __sincosf(6.2831853071795865f * (ub - 0.5f), &s, &c);
    z0 = -r * c;
    z1 = -r * s;
}

__device__ __forceinline__ float normal_f(uint64_t seed, uint32_t stream, uint32_t step,
                                          uint32_t purpose, uint32_t n) {
    U4 o = philox_block(seed, stream, step, purpose, n >> 2);
    uint32_t wa, wb;
    if ((n >> 1) & 1) {
        wa = o.z;
        wb = o.w;
    } else {
        wa = o.x;
        wb = o.y;
    }
    float z0, z1;
    box_muller_f(wa, wb, z0, z1);
    return (n & 1) ? z1 : z0;
}

template <typename R>
__device__ __forceinline__ R normal_r(uint64_t seed, uint32_t stream, uint32_t step,
                                      uint32_t purpose, uint32_t n);
template <>
__device__ __forceinline__ double normal_r<double>(uint64_t seed, uint32_t stream, uint32_t step,
                                                   uint32_t purpose, uint32_t n) {
    return normal_d(seed, stream, step, purpose, n);
}
template <>
__device__ __forceinline__ float normal_r<float>(uint64_t seed, uint32_t stream, uint32_t step,
                                                 uint32_t purpose, uint32_t n) {
    return normal_f(seed, stream, step, purpose, n);
}

__device__ __forceinline__ double uniform_d(uint64_t seed, uint32_t stream, uint32_t step,
                                            uint32_t purpose, uint32_t n) {
    U4 o = philox_block(seed, stream, step, purpose, n >> 2);
    uint32_t w = (n & 3) == 0 ? o.x : (n & 3) == 1 ? o.y : (n & 3) == 2 ? o.z : o.w;
    return u32_unit_d(w);
}

// Andersen kick interval (mean < 30: inversion; else rounded normal approximation).
__device__ __forceinline__ int64_t poisson_d(uint64_t seed, uint32_t stream, uint32_t step,
                                             uint32_t purpose, double mean) {
    if (mean < 30.0) {
        double u = uniform_d(seed, stream, step, purpose, 0u);
        double pk = exp(-mean), cdf = pk;
        int64_t k = 0;
        while (u > cdf && k < 1000) {
            k++;
            pk *= mean / (double)k;
            cdf += pk;
        }
        return k;
    }
    double z = normal_d(seed, stream, step, purpose, 0u);
    double v = floor(mean + sqrt(mean) * z + 0.5);
    return v < 0.0 ? 0 : (int64_t)v;
}

// ---------------------------------------------------------------- PES functors
// Parameter layouts match include/pimdgpu.h:
//   1D:       [Vheight, x0]
//   2DTEST:   [m, a0, b0, rho0]
//   SYNTH9:   [npair, (i, j, D, a, r0) x npair, iH, iO1, iO2, B, s0]
//   SYNTH18:  [nmol, kr, re, ktheta, theta_e, eps, sigma, qO, qH]
//   HARMONIC: [k]
//   DISTGAUSS: [natom, shift, nmorse, ng1, ng2, ng3, terms...] (pes_distgauss)
enum : int { kPes1D = 1, kPes2D = 2, kPesSynth9 = 3, kPesSynth18 = 4, kPesHarm = 5, kPesDistGauss = 6 };
constexpr int kMaxDofPes = 64;  // = kMaxDof (the largest surface: 18 atoms x 3 = 54 dofs)

struct PesArgs {
    int id, ndim, natom, nd, nparams;
    int canon9;  // 9-atom surface whose table lists all 36 pairs i < j in order (unrolled FP32 path)
    double V0;
    const double *params;  // device (or shared) pointer
    // FP32 copy of params (device or shared), read by the FP32 surfaces so that
    // no FP64 conversion runs per evaluation; for the 2-D surface it is followed
    // by the 12 well-centre coordinates (x1, y1, ..., x6, y6), rounded from FP64.
    const float *fparams;
};

// Number of extra FP32 values that follow the parameters in fparams.
__host__ __device__ __forceinline__ int pes_fparams_extra(int id) { return id == 2 ? 12 : 0; }

// Parameter vector of the surface in the arithmetic type R.
template <typename R> __device__ __forceinline__ const R *pes_params(const PesArgs &pa);
template <> __device__ __forceinline__ const double *pes_params<double>(const PesArgs &pa) { return pa.params; }
template <> __device__ __forceinline__ const float *pes_params<float>(const PesArgs &pa) { return pa.fparams; }

// mcmod_1d.f90:14-35.  No V0 (the reference module does not subtract it).
template <typename R>
__device__ __forceinline__ R pes_1d(const PesArgs &pa, const R *x, R *g) {
    R H = (R)1.0, x0 = (R)1.0;
    if (pa.nparams >= 2) {
        H = pes_params<R>(pa)[0];
        x0 = pes_params<R>(pa)[1];
    }
    R v = 0;
    for (int i = 0; i < pa.nd; i++) {
        R t = (x[i] / x0) * (x[i] / x0) - (R)1.0;
        v += H * t * t;
        if (g) g[i] = t * (R)4.0 * H * x[i] / (x0 * x0);
    }
    return v;
}

// mcmod_2dtest.f90:29-61, FP64: same operation order as the reference.
__device__ __forceinline__ double pes_2d_d(const PesArgs &pa, const double *x, double *g) {
    int m = 6;
    double a0 = 2.0, b0 = 0.2, rho0 = 3.0;
    if (pa.nparams >= 4) {
        m = (int)pa.params[0];
        a0 = pa.params[1];
        b0 = pa.params[2];
        rho0 = pa.params[3];
    }
    double v = 0.0, gx = 0.0, gy = 0.0;
    for (int k = 1; k <= m; k++) {
        double xk = rho0 * cos((double)k * 2.0 * kPiRef / (double)m);
        double yk = rho0 * sin((double)k * 2.0 * kPiRef / (double)m);
        double dx = x[0] - xk, dy = x[1] - yk;
        double u = dx * dx + dy * dy;
        double ea = exp(-a0 * u), eb = exp(-b0 * u);
        v = v - 0.5 * ea;
        v = v - 0.5 * eb;
        gx = gx + a0 * dx * ea;
        gx = gx + b0 * dx * eb;
        gy = gy + a0 * dy * ea;
        gy = gy + b0 * dy * eb;
    }
    if (g) {
        g[0] = gx;
        g[1] = gy;
    }
    return v - pa.V0;
}

// FP32 twin of mcmod_2dtest with well centres from a table wc[2m] and the
// repo parameters a0 = 10 b0 exploited as exp(-a0 u) = exp(-b0 u)^10 when the
// parameters have that ratio (one MUFU exp per well).
__device__ __forceinline__ float pes_2d_f(const PesArgs &pa, const float *wc, int m, float a0,
                                          float b0, bool pow10, const float *x, float *g) {
    float v = 0.f, gx = 0.f, gy = 0.f;
    for (int k = 0; k < m; k++) {
        float dx = x[0] - wc[2 * k], dy = x[1] - wc[2 * k + 1];
        float u = dx * dx + dy * dy;
        float eb = __expf(-b0 * u);
        float ea;
        if (pow10) {
            float e2 = eb * eb, e4 = e2 * e2, e8 = e4 * e4;
            ea = e8 * e2;
        } else {
            ea = __expf(-a0 * u);
        }
        v -= 0.5f * (ea + eb);
        float c = a0 * ea + b0 * eb;
        gx += c * dx;
        gy += c * dy;
    }
    if (g) {
        g[0] = gx;
        g[1] = gy;
    }
    return v - (float)pa.V0;
}

template <typename R>
__device__ __forceinline__ R pes_harm(const PesArgs &pa, const R *x, R *g) {
    R k = pa.nparams >= 1 ? pes_params<R>(pa)[0] : (R)1.0;
    R v = 0;
    for (int i = 0; i < pa.nd; i++) {
        v += (R)0.5 * k * x[i] * x[i];
        if (g) g[i] = k * x[i];
    }
    return v - (R)pa.V0;
}

// Square root and division in the surfaces: IEEE in both precisions.  (An
// rsqrt-based square root and the fast divide in FP32 let one ring of the
// 18-atom surface at P = 512 run away within 100 steps where the IEEE
// operations, and FP64, keep it bounded.)
template <typename R> __device__ __forceinline__ R my_sqrt(R v);
template <> __device__ __forceinline__ double my_sqrt<double>(double v) { return sqrt(v); }
template <> __device__ __forceinline__ float my_sqrt<float>(float v) { return sqrtf(v); }
template <typename R> __device__ __forceinline__ R pdiv(R a, R b) { return a / b; }
template <typename R> __device__ __forceinline__ R my_exp(R v);
template <> __device__ __forceinline__ double my_exp<double>(double v) { return exp(v); }
template <> __device__ __forceinline__ float my_exp<float>(float v) { return __expf(v); }
template <typename R> __device__ __forceinline__ R my_acos(R v);
template <> __device__ __forceinline__ double my_acos<double>(double v) { return acos(v); }
template <> __device__ __forceinline__ float my_acos<float>(float v) { return acosf(v); }

// Pair (I, J) of the 9-atom surface's canonical table (all 36 pairs i < j in
// order, pair q at q = 8 I - I (I - 1) / 2 + J - I - 1), then its successors.
// Template recursion makes every coordinate index a compile-time constant
// whatever the caller's loops (a nest of unrolled loops inside a caller's loop
// can be left rolled, which puts the coordinate arrays in local memory).
template <typename R, int I, int J>
__device__ __forceinline__ void s9_pairs(const R *pp, const R (&xr)[27], R (&gr)[27], R &v, bool grad) {
    if constexpr (I < 8) {
        constexpr int q = I * 8 - I * (I - 1) / 2 + (J - I - 1);
        const R *r = pp + 1 + 5 * q;
        const R D = (R)r[2], a = (R)r[3], r0 = (R)r[4];
        const R d0 = xr[3 * I] - xr[3 * J], d1 = xr[3 * I + 1] - xr[3 * J + 1], d2 = xr[3 * I + 2] - xr[3 * J + 2];
        const R rr = my_sqrt<R>(d0 * d0 + d1 * d1 + d2 * d2);
        const R e = my_exp<R>(-a * (rr - r0));
        const R om = (R)1.0 - e;
        v += D * om * om;
        if (grad) {
            const R dvdr = pdiv<R>((R)2.0 * D * a * om * e, rr);
            gr[3 * I] += dvdr * d0;
            gr[3 * I + 1] += dvdr * d1;
            gr[3 * I + 2] += dvdr * d2;
            gr[3 * J] -= dvdr * d0;
            gr[3 * J + 1] -= dvdr * d1;
            gr[3 * J + 2] -= dvdr * d2;
        }
        if constexpr (J < 8)
            s9_pairs<R, I, J + 1>(pp, xr, gr, v, grad);
        else
            s9_pairs<R, I + 1, I + 2>(pp, xr, gr, v, grad);
    }
}

// The 9-atom surface when its table lists all 36 pairs i < j in order: the
// pairs are expanded at compile time (s9_pairs), so every atom index is a
// constant and the 27 coordinates and gradient components stay in registers
// (the table's indices need local or shared arrays).  The arithmetic and its
// order are those of pes_synth9; the quartic's three atoms are picked by
// comparisons.
template <typename R>
__device__ __forceinline__ R pes_synth9_canon(const PesArgs &pa, const R *x, R *g) {
    const R *pp = pes_params<R>(pa);
    R xr[27], gr[27];
#pragma unroll
    for (int k = 0; k < 27; k++) {
        xr[k] = x[k];
        gr[k] = 0;
    }
    R v = 0;
    s9_pairs<R, 0, 1>(pp, xr, gr, v, g != nullptr);
    const R *w = pp + 1 + 5 * 36;
    const int iH = (int)w[0], iO1 = (int)w[1], iO2 = (int)w[2];
    const R B = (R)w[3], s0 = (R)w[4];
    R xH[3] = {0, 0, 0}, xO1[3] = {0, 0, 0}, xO2[3] = {0, 0, 0};
#pragma unroll
    for (int at = 0; at < 9; at++)
#pragma unroll
        for (int c = 0; c < 3; c++) {
            if (at == iH) xH[c] = xr[3 * at + c];
            if (at == iO1) xO1[c] = xr[3 * at + c];
            if (at == iO2) xO2[c] = xr[3 * at + c];
        }
    R e1[3], e2[3], r1 = 0, r2 = 0;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        e1[c] = xH[c] - xO1[c];
        e2[c] = xH[c] - xO2[c];
        r1 += e1[c] * e1[c];
        r2 += e2[c] * e2[c];
    }
    r1 = my_sqrt<R>(r1);
    r2 = my_sqrt<R>(r2);
    const R s = r1 - r2;
    const R t = (s / s0) * (s / s0) - (R)1.0;
    v += B * t * t;
    if (g) {
        const R dvds = (R)4.0 * B * t * s / (s0 * s0);
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const R a1 = dvds * e1[c] / r1, a2 = dvds * e2[c] / r2;
#pragma unroll
            for (int at = 0; at < 9; at++) {
                if (at == iH) gr[3 * at + c] += a1 - a2;
                if (at == iO1) gr[3 * at + c] -= a1;
                if (at == iO2) gr[3 * at + c] += a2;
            }
        }
#pragma unroll
        for (int k = 0; k < 27; k++) g[k] = gr[k];
    }
    return v - (R)pa.V0;
}

// Synthetic 9-atom surface: Morse pair network + quartic double well in
// s = |r_H - r_O1| - |r_H - r_O2|.  Reverse-mode gradient: each pair's
// distance is recomputed, dV/dr is scattered through dr/dx (Wilson B row).
template <typename R>
__device__ __forceinline__ R pes_synth9(const PesArgs &pa, const R *x, R *g) {
    if constexpr (sizeof(R) == 4)  // FP32 only: the FP64 callers run 512-thread CTAs whose registers it would exceed
        if (pa.canon9) return pes_synth9_canon<R>(pa, x, g);
    const R *pp = pes_params<R>(pa);
    int npair = (int)pp[0];
    if (g)
        for (int i = 0; i < pa.nd; i++) g[i] = 0;
    R v = 0;
    for (int q = 0; q < npair; q++) {
        const R *r = pp + 1 + 5 * q;
        int i = (int)r[0], j = (int)r[1];
        R D = (R)r[2], a = (R)r[3], r0 = (R)r[4];
        R d0 = x[3 * i] - x[3 * j], d1 = x[3 * i + 1] - x[3 * j + 1], d2 = x[3 * i + 2] - x[3 * j + 2];
        R rr = my_sqrt<R>(d0 * d0 + d1 * d1 + d2 * d2);
        R e = my_exp<R>(-a * (rr - r0));
        R om = (R)1.0 - e;
        v += D * om * om;
        if (g) {
            R dvdr = pdiv<R>((R)2.0 * D * a * om * e, rr);
            g[3 * i] += dvdr * d0;
            g[3 * i + 1] += dvdr * d1;
            g[3 * i + 2] += dvdr * d2;
            g[3 * j] -= dvdr * d0;
            g[3 * j + 1] -= dvdr * d1;
            g[3 * j + 2] -= dvdr * d2;
        }
    }
    const R *w = pp + 1 + 5 * npair;
    int iH = (int)w[0], iO1 = (int)w[1], iO2 = (int)w[2];
    R B = (R)w[3], s0 = (R)w[4];
    R e1[3], e2[3], r1 = 0, r2 = 0;
    for (int c = 0; c < 3; c++) {
        e1[c] = x[3 * iH + c] - x[3 * iO1 + c];
        e2[c] = x[3 * iH + c] - x[3 * iO2 + c];
        r1 += e1[c] * e1[c];
        r2 += e2[c] * e2[c];
    }
    r1 = my_sqrt<R>(r1);
    r2 = my_sqrt<R>(r2);
    R s = r1 - r2;
    R t = (s / s0) * (s / s0) - (R)1.0;
    v += B * t * t;
    if (g) {
        R dvds = (R)4.0 * B * t * s / (s0 * s0);
        for (int c = 0; c < 3; c++) {
            R a1 = dvds * e1[c] / r1, a2 = dvds * e2[c] / r2;
            g[3 * iH + c] += a1 - a2;
            g[3 * iO1 + c] -= a1;
            g[3 * iO2 + c] += a2;
        }
    }
    return v - (R)pa.V0;
}

// Synthetic 18-atom flexible water cluster (harmonic bonds / angles, O-O
// Lennard-Jones, intermolecular point charges).
template <typename R>
__device__ __forceinline__ R pes_synth18(const PesArgs &pa, const R *x, R *g) {
    const R *pp = pes_params<R>(pa);
    int nmol = (int)pp[0];
    R kr = (R)pp[1], re = (R)pp[2], kth = (R)pp[3], the = (R)pp[4], eps = (R)pp[5], sig = (R)pp[6];
    R qO = (R)pp[7], qH = (R)pp[8];
    if (g)
        for (int i = 0; i < 9 * nmol; i++) g[i] = 0;
    R v = 0;
    for (int m = 0; m < nmol; m++) {
        const R *O = x + 9 * m, *H1 = O + 3, *H2 = O + 6;
        R u1[3], u2[3], r1 = 0, r2 = 0;
        for (int c = 0; c < 3; c++) {
            u1[c] = H1[c] - O[c];
            u2[c] = H2[c] - O[c];
            r1 += u1[c] * u1[c];
            r2 += u2[c] * u2[c];
        }
        r1 = my_sqrt<R>(r1);
        r2 = my_sqrt<R>(r2);
        R ct = pdiv<R>(u1[0] * u2[0] + u1[1] * u2[1] + u1[2] * u2[2], r1 * r2);
        ct = ct > (R)1.0 ? (R)1.0 : (ct < (R)-1.0 ? (R)-1.0 : ct);
        R th = my_acos<R>(ct);
        v += (R)0.5 * kr * ((r1 - re) * (r1 - re) + (r2 - re) * (r2 - re));
        v += (R)0.5 * kth * (th - the) * (th - the);
        if (g) {
            R st = my_sqrt<R>((R)1.0 - ct * ct);
            if (st < (R)1e-12) st = (R)1e-12;
            R dth = kth * (th - the);
            for (int c = 0; c < 3; c++) {
                R n1 = pdiv<R>(u1[c], r1), n2 = pdiv<R>(u2[c], r2);
                R gb1 = kr * (r1 - re) * n1, gb2 = kr * (r2 - re) * n2;
                R ga1 = pdiv<R>(-dth * (n2 - ct * n1), r1 * st);
                R ga2 = pdiv<R>(-dth * (n1 - ct * n2), r2 * st);
                g[9 * m + 3 + c] += gb1 + ga1;
                g[9 * m + 6 + c] += gb2 + ga2;
                g[9 * m + c] -= gb1 + ga1 + gb2 + ga2;
            }
        }
    }
    // site pairs of molecules m < n.  FP32: the two molecules' coordinates and
    // gradient in registers for their nine site pairs (ia, ib unrolled), read
    // from and written back to x / g once per molecule pair; every gradient
    // component receives its terms in the same order as pair by pair (FP64 keeps
    // the pair-by-pair loop: its 36 doubles would lower the occupancy of the FP64
    // kernels for every surface).
    if constexpr (sizeof(R) == 8) {
        for (int m = 0; m < nmol; m++)
            for (int n = m + 1; n < nmol; n++)
                for (int ia = 0; ia < 3; ia++)
                    for (int ib = 0; ib < 3; ib++) {
                        const R *A = x + 9 * m + 3 * ia, *Bp = x + 9 * n + 3 * ib;
                        R d0 = A[0] - Bp[0], d1 = A[1] - Bp[1], d2 = A[2] - Bp[2];
                        R r2 = d0 * d0 + d1 * d1 + d2 * d2;
                        R r = my_sqrt<R>(r2);
                        R qa = ia == 0 ? qO : qH, qb = ib == 0 ? qO : qH;
                        R e = pdiv<R>(qa * qb, r);
                        R dvr = pdiv<R>(-e, r2);
                        if (ia == 0 && ib == 0) {
                            R sr2 = pdiv<R>(sig * sig, r2);
                            R sr6 = sr2 * sr2 * sr2;
                            R sr12 = sr6 * sr6;
                            e += (R)4.0 * eps * (sr12 - sr6);
                            dvr += pdiv<R>((R)4.0 * eps * ((R)-12.0 * sr12 + (R)6.0 * sr6), r2);
                        }
                        v += e;
                        if (g) {
                            int ai = 9 * m + 3 * ia, bi = 9 * n + 3 * ib;
                            g[ai] += dvr * d0;
                            g[ai + 1] += dvr * d1;
                            g[ai + 2] += dvr * d2;
                            g[bi] -= dvr * d0;
                            g[bi + 1] -= dvr * d1;
                            g[bi + 2] -= dvr * d2;
                        }
                    }
        return v - (R)pa.V0;
    }
    for (int m = 0; m < nmol; m++) {
        R xm[9], gm[9];
#pragma unroll
        for (int k = 0; k < 9; k++) {
            xm[k] = x[9 * m + k];
            gm[k] = g ? g[9 * m + k] : (R)0;
        }
        for (int n = m + 1; n < nmol; n++) {
            R xn[9], gn[9];
#pragma unroll
            for (int k = 0; k < 9; k++) {
                xn[k] = x[9 * n + k];
                gn[k] = g ? g[9 * n + k] : (R)0;
            }
#pragma unroll
            for (int ia = 0; ia < 3; ia++)
#pragma unroll
                for (int ib = 0; ib < 3; ib++) {
                    const R d0 = xm[3 * ia] - xn[3 * ib], d1 = xm[3 * ia + 1] - xn[3 * ib + 1],
                            d2 = xm[3 * ia + 2] - xn[3 * ib + 2];
                    R r2 = d0 * d0 + d1 * d1 + d2 * d2;
                    R r = my_sqrt<R>(r2);
                    R qa = ia == 0 ? qO : qH, qb = ib == 0 ? qO : qH;
                    R e = pdiv<R>(qa * qb, r);
                    R dvr = pdiv<R>(-e, r2);
                    if (ia == 0 && ib == 0) {
                        R sr2 = pdiv<R>(sig * sig, r2);
                        R sr6 = sr2 * sr2 * sr2;
                        R sr12 = sr6 * sr6;
                        e += (R)4.0 * eps * (sr12 - sr6);
                        dvr += pdiv<R>((R)4.0 * eps * ((R)-12.0 * sr12 + (R)6.0 * sr6), r2);
                    }
                    v += e;
                    gm[3 * ia] += dvr * d0;
                    gm[3 * ia + 1] += dvr * d1;
                    gm[3 * ia + 2] += dvr * d2;
                    gn[3 * ib] -= dvr * d0;
                    gn[3 * ib + 1] -= dvr * d1;
                    gn[3 * ib + 2] -= dvr * d2;
                }
            if (g) {
#pragma unroll
                for (int k = 0; k < 9; k++) g[9 * n + k] = gn[k];
            }
        }
        if (g) {
#pragma unroll
            for (int k = 0; k < 9; k++) g[9 * m + k] = gm[k];
        }
    }
    return v - (R)pa.V0;
}

// Generic dispatch (FP64 and the generic FP32 path).
// Morse terms and 1-, 2- and 3-D Gaussians in the interatomic distances: the
// functional form of pes_malonaldehyde.f90 (distances :9357-9365, v_morse
// :9598-9610, v_gauss :9650-9670, the energy sums :9406-9440), with the term
// tables as parameters:
//   [natom, shift, nmorse, ng1, ng2, ng3,
//    nmorse x (k, re, al, de)                          (de (e^{al (re - r_k)} - 1))^2
//    ng1 x (k, x, a, d, s)                             d (e^{-a (r_k - x)^2 / 2} - s)
//    ng2 x (k1, k2, x1, x2, a1, a2, d, s)              d (e^{-(a1 u1^2 + a2 u2^2) / 2} - s)
//    ng3 x (k1, k2, k3, x1, x2, x3, a1, a2, a3, d, s)]
// where r_k is the distance of atom pair k: i > j, k = i (i - 1) / 2 + j
// (0-based), the reference's ordering.  V = shift + sum of terms - V0.
constexpr int kMaxPairs = (kMaxDofPes / 3) * (kMaxDofPes / 3 - 1) / 2;
template <typename R>
__device__ R pes_distgauss(const PesArgs &pa, const R *x, R *g) {
    const R *pp = pes_params<R>(pa);
    const int na = pa.natom;
    R r[kMaxPairs], dv[kMaxPairs];
    int k = 0;
    for (int i = 1; i < na; i++)
        for (int j = 0; j < i; j++) {
            const R d0 = x[3 * i] - x[3 * j], d1 = x[3 * i + 1] - x[3 * j + 1], d2 = x[3 * i + 2] - x[3 * j + 2];
            r[k] = my_sqrt<R>(d0 * d0 + d1 * d1 + d2 * d2);
            dv[k] = (R)0;
            k++;
        }
    R v = pp[1];
    const int nm = (int)pp[2], n1 = (int)pp[3], n2 = (int)pp[4], n3 = (int)pp[5];
    const R *q = pp + 6;
    for (int t = 0; t < nm; t++, q += 4) {
        const int kk = (int)q[0];
        const R e = my_exp<R>(q[2] * (q[1] - r[kk]));
        const R w = e - (R)1.0;
        v += (q[3] * w) * (q[3] * w);
        dv[kk] -= (R)2.0 * q[3] * q[3] * w * e * q[2];
    }
    for (int t = 0; t < n1; t++, q += 5) {
        const int kk = (int)q[0];
        const R u = r[kk] - q[1];
        const R e = my_exp<R>((R)-0.5 * q[2] * u * u);
        v += q[3] * (e - q[4]);
        dv[kk] -= q[3] * e * q[2] * u;
    }
    for (int t = 0; t < n2; t++, q += 8) {
        const int k1 = (int)q[0], k2 = (int)q[1];
        const R u1 = r[k1] - q[2], u2 = r[k2] - q[3];
        const R e = my_exp<R>((R)-0.5 * (q[4] * u1 * u1 + q[5] * u2 * u2));
        v += q[6] * (e - q[7]);
        const R de = q[6] * e;
        dv[k1] -= de * q[4] * u1;
        dv[k2] -= de * q[5] * u2;
    }
    for (int t = 0; t < n3; t++, q += 11) {
        const int k1 = (int)q[0], k2 = (int)q[1], k3 = (int)q[2];
        const R u1 = r[k1] - q[3], u2 = r[k2] - q[4], u3 = r[k3] - q[5];
        const R e = my_exp<R>((R)-0.5 * (q[6] * u1 * u1 + q[7] * u2 * u2 + q[8] * u3 * u3));
        v += q[9] * (e - q[10]);
        const R de = q[9] * e;
        dv[k1] -= de * q[6] * u1;
        dv[k2] -= de * q[7] * u2;
        dv[k3] -= de * q[8] * u3;
    }
    if (g) {
        for (int i = 0; i < 3 * na; i++) g[i] = (R)0;
        k = 0;
        for (int i = 1; i < na; i++)
            for (int j = 0; j < i; j++) {
                const R f = pdiv<R>(dv[k], r[k]);
                for (int c = 0; c < 3; c++) {
                    const R d = x[3 * i + c] - x[3 * j + c];
                    g[3 * i + c] += f * d;
                    g[3 * j + c] -= f * d;
                }
                k++;
            }
    }
    return v - (R)pa.V0;
}

template <typename R>
__device__ __forceinline__ R pes_vgrad(const PesArgs &pa, const R *x, R *g);

template <>
__device__ __forceinline__ double pes_vgrad<double>(const PesArgs &pa, const double *x, double *g) {
    switch (pa.id) {
    case kPes1D: return pes_1d<double>(pa, x, g);
    case kPes2D: return pes_2d_d(pa, x, g);
    case kPesSynth9: return pes_synth9<double>(pa, x, g);
    case kPesSynth18: return pes_synth18<double>(pa, x, g);
    case kPesHarm: return pes_harm<double>(pa, x, g);
    case kPesDistGauss: return pes_distgauss<double>(pa, x, g);
    default: return 0.0;
    }
}

template <>
__device__ __forceinline__ float pes_vgrad<float>(const PesArgs &pa, const float *x, float *g) {
    switch (pa.id) {
    case kPes1D: return pes_1d<float>(pa, x, g);
    case kPes2D: {
        int m = 6;
        float a0 = 2.f, b0 = 0.2f;
        if (pa.nparams >= 4) {
            m = (int)pa.fparams[0];
            a0 = pa.fparams[1];
            b0 = pa.fparams[2];
        }
        if (m > 6) m = 6;
        return pes_2d_f(pa, pa.fparams + pa.nparams, m, a0, b0, a0 == 10.f * b0, x, g);
    }
    case kPesSynth9: return pes_synth9<float>(pa, x, g);
    case kPesSynth18: return pes_synth18<float>(pa, x, g);
    case kPesHarm: return pes_harm<float>(pa, x, g);
    case kPesDistGauss: return pes_distgauss<float>(pa, x, g);
    default: return 0.f;
    }
}

constexpr int kMaxDof = 64;  // 18 atoms x 3 = 54 is the largest configured surface

}  // namespace pg
