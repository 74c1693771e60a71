// pg_hessian.cuh -- device Hessians of the PES functors (Vdoubleprime twins).
#pragma once
#include "pg_device.cuh"

namespace pg {

// Central finite difference of the gradient, eps = 1e-4, for perturbed dof a
// (mcmod_1d.f90:38-58): writes hess[a + nd*b] for every b.
__device__ inline void hess_fd_column(const PesArgs &pa, const double *x, int a, double *hess) {
    double xw[kMaxDof], gp[kMaxDof], gm[kMaxDof];
    for (int i = 0; i < pa.nd; i++) xw[i] = x[i];
    const double eps = 1e-4;
    double x0 = xw[a];
    xw[a] = x0 + eps;
    pes_vgrad<double>(pa, xw, gp);
    xw[a] = xw[a] - 2.0 * eps;
    pes_vgrad<double>(pa, xw, gm);
    for (int b = 0; b < pa.nd; b++) hess[a + pa.nd * b] = (gp[b] - gm[b]) / (2.0 * eps);
}

// mcmod_2dtest.f90:64-102 (quirks) or the exact Hessian.
__device__ inline void hess_2d(const PesArgs &pa, const double *x, double *hess, int quirks) {
    int m = 6;
    double a0 = 2.0, b0 = 0.2, rho0 = 3.0;
    if (pa.nparams >= 4) {
        m = (int)pa.params[0];
        a0 = pa.params[1];
        b0 = pa.params[2];
        rho0 = pa.params[3];
    }
    double hxx = 0.0, hxy = 0.0, hyy = 0.0;
    for (int k = 1; k <= m; k++) {
        double xk = rho0 * cos((double)k * 2.0 * kPiRef / (double)m);
        double yk = rho0 * sin((double)k * 2.0 * kPiRef / (double)m);
        double dx = x[0] - xk, dy = x[1] - yk;
        double u = dx * dx + dy * dy;
        double ea = exp(-a0 * u), eb = exp(-b0 * u);
        double dvdu = a0 * ea + b0 * eb;
        double d2 = -a0 * a0 * ea - b0 * b0 * eb;
        if (quirks) {
            hxx = (d2 * dx + dvdu) * dx;
            hxy = (d2 * dy + dvdu) * dx;
            hyy = (d2 * dy + dvdu) * dy;
        } else {
            hxx += 2.0 * d2 * dx * dx + dvdu;
            hxy += 2.0 * d2 * dx * dy;
            hyy += 2.0 * d2 * dy * dy + dvdu;
        }
    }
    hess[0] = hxx;
    hess[1] = hxy;
    hess[2] = hxy;
    hess[3] = hyy;
}

// w1 * Hess(r_ij) + w2 * grad r_ij grad r_ij^T added into hess.
__device__ inline void add_dist_hess(double *hess, int nd, int i, int j, const double *x,
                                     double w1, double w2) {
    double d[3], r = 0.0;
    for (int c = 0; c < 3; c++) {
        d[c] = x[3 * i + c] - x[3 * j + c];
        r += d[c] * d[c];
    }
    r = sqrt(r);
    for (int c1 = 0; c1 < 3; c1++)
        for (int c2 = 0; c2 < 3; c2++) {
            double u1 = d[c1] / r, u2 = d[c2] / r;
            double blk = w1 * (((c1 == c2) ? 1.0 : 0.0) - u1 * u2) / r + w2 * u1 * u2;
            hess[(3 * i + c1) + nd * (3 * i + c2)] += blk;
            hess[(3 * j + c1) + nd * (3 * j + c2)] += blk;
            hess[(3 * i + c1) + nd * (3 * j + c2)] -= blk;
            hess[(3 * j + c1) + nd * (3 * i + c2)] -= blk;
        }
}

// Analytic Hessian of the synthetic 9-atom surface.
__device__ inline void hess_synth9(const PesArgs &pa, const double *x, double *hess) {
    const double *pp = pa.params;
    int npair = (int)pp[0];
    int nd = pa.nd;
    for (int i = 0; i < nd * nd; i++) hess[i] = 0.0;
    for (int q = 0; q < npair; q++) {
        const double *r = pp + 1 + 5 * q;
        int i = (int)r[0], j = (int)r[1];
        double D = r[2], a = r[3], r0 = r[4];
        double d0 = x[3 * i] - x[3 * j], d1 = x[3 * i + 1] - x[3 * j + 1], d2 = x[3 * i + 2] - x[3 * j + 2];
        double rr = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
        double e = exp(-a * (rr - r0));
        double dv = 2.0 * D * a * (1.0 - e) * e;
        double d2v = 2.0 * D * a * a * e * (2.0 * e - 1.0);
        add_dist_hess(hess, nd, i, j, x, dv, d2v);
    }
    const double *w = pp + 1 + 5 * npair;
    int iH = (int)w[0], iO1 = (int)w[1], iO2 = (int)w[2];
    double B = w[3], s0 = w[4];
    double e1[3], e2[3], r1 = 0.0, r2 = 0.0;
    for (int c = 0; c < 3; c++) {
        e1[c] = x[3 * iH + c] - x[3 * iO1 + c];
        e2[c] = x[3 * iH + c] - x[3 * iO2 + c];
        r1 += e1[c] * e1[c];
        r2 += e2[c] * e2[c];
    }
    r1 = sqrt(r1);
    r2 = sqrt(r2);
    double s = r1 - r2;
    double t = (s / s0) * (s / s0) - 1.0;
    double dvds = 4.0 * B * t * s / (s0 * s0);
    double d2vds2 = 4.0 * B * (3.0 * s * s / (s0 * s0) - 1.0) / (s0 * s0);
    add_dist_hess(hess, nd, iH, iO1, x, dvds, 0.0);
    add_dist_hess(hess, nd, iH, iO2, x, -dvds, 0.0);
    double gs[kMaxDof];
    for (int i = 0; i < nd; i++) gs[i] = 0.0;
    for (int c = 0; c < 3; c++) {
        gs[3 * iH + c] += e1[c] / r1 - e2[c] / r2;
        gs[3 * iO1 + c] -= e1[c] / r1;
        gs[3 * iO2 + c] += e2[c] / r2;
    }
    for (int aa = 0; aa < nd; aa++)
        for (int bb = 0; bb < nd; bb++) hess[aa + nd * bb] += d2vds2 * gs[aa] * gs[bb];
}

__device__ inline bool hess_is_fd(int id) { return id == kPes1D || id == kPesSynth18 || id == kPesDistGauss; }

// Full Hessian of one configuration by one thread (analytic surfaces) or the
// FD column a (FD surfaces; a < 0 computes every column).
__device__ inline void pes_hessian(const PesArgs &pa, const double *x, double *hess, int quirks) {
    switch (pa.id) {
    case kPes2D: hess_2d(pa, x, hess, quirks); return;
    case kPesSynth9: hess_synth9(pa, x, hess); return;
    case kPesHarm: {
        double k = pa.nparams >= 1 ? pa.params[0] : 1.0;
        for (int i = 0; i < pa.nd * pa.nd; i++) hess[i] = 0.0;
        for (int i = 0; i < pa.nd; i++) hess[i + pa.nd * i] = k;
        return;
    }
    default:
        for (int a = 0; a < pa.nd; a++) hess_fd_column(pa, x, a, hess);
        return;
    }
}

}  // namespace pg
