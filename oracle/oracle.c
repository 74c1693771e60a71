/*
 * oracle.c -- CPU FP64 restatement of the reference ring-polymer algorithms.
 *
 * TEST INFRASTRUCTURE ONLY (the parity reference of the tests and the timed
 * CPU baseline).  The product library never links or calls this file.
 * Parity with the reference is UNPINNED: the Fortran/MKL/MPI reference cannot
 * be built here, and it ships no golden vectors; the pins are analytic known
 * answers (see oracle.h).
 *
 * Each function names the reference routine (file:line) whose arithmetic it
 * restates.  Deliberate deviations from the reference:
 *   (i)   Philox4x32-10 + Box-Muller replaces MKL VSL MT19937/ICDF (closed,
 *         clock-seeded: verletmodule.f90:350-368); seeds are explicit.
 *   (ii)  The Andersen Poisson interval uses inversion (mean < 30) or the
 *         rounded normal approximation (mean >= 30) instead of VSL POISNORM.
 *   (iii) Alignment is not applied (ndim != 3 stops the reference,
 *         instantonmod.f90:234-237).
 *   (iv)  quirks=0 corrects the mcmod_2dtest Hessian (mcmod_2dtest.f90:73-86)
 *         and the missing bead-1/bead-2 spring coupling of UMhessian
 *         (instantonmod.f90:203); quirks=1 reproduces both.
 */
#include "oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------- */
/* PES                                                                       */
/* ------------------------------------------------------------------------- */

/* mcmod_1d.f90:8-35.  params = [Vheight, x0] (defaults 1, 1).  V0 is not
 * subtracted: the reference V for this module ignores V0 (mcmod_1d.f90:20). */
static void p1d(const or_pes *pes, double *H, double *x0) {
    *H = 1.0;
    *x0 = 1.0;
    if (pes->nparams >= 2) {
        *H = pes->params[0];
        *x0 = pes->params[1];
    }
}

static double v_1d(const or_pes *pes, const double *x, double *g) {
    double H, x0;
    p1d(pes, &H, &x0);
    int nd = pes->ndim * pes->natom;
    double v = 0.0;
    for (int i = 0; i < nd; i++) {
        double t = (x[i] / x0) * (x[i] / x0) - 1.0;
        v += H * t * t;
        if (g) g[i] = t * 4.0 * H * x[i] / (x0 * x0);
    }
    return v;
}

/* mcmod_2dtest.f90:11-61.  params = [m, a0, b0, rho0] (defaults 6, 2, 0.2, 3).
 * Well centres use the reference's truncated pi. */
typedef struct { int m; double a0, b0, rho0; } p2d_t;
static p2d_t p2d(const or_pes *pes) {
    p2d_t p = {6, 2.0, 0.2, 3.0};
    if (pes->nparams >= 4) {
        p.m = (int)pes->params[0];
        p.a0 = pes->params[1];
        p.b0 = pes->params[2];
        p.rho0 = pes->params[3];
    }
    return p;
}

static double v_2d(const or_pes *pes, const double *x, double *g) {
    p2d_t p = p2d(pes);
    double v = 0.0, gx = 0.0, gy = 0.0;
    for (int k = 1; k <= p.m; k++) {
        double xk = p.rho0 * cos((double)k * 2.0 * OR_PI_REF / (double)p.m);
        double yk = p.rho0 * sin((double)k * 2.0 * OR_PI_REF / (double)p.m);
        double dx = x[0] - xk, dy = x[1] - yk;
        double u = dx * dx + dy * dy;
        double ea = exp(-p.a0 * u), eb = exp(-p.b0 * u);
        v = v - 0.5 * ea;
        v = v - 0.5 * eb;
        gx = gx + p.a0 * dx * ea;
        gx = gx + p.b0 * dx * eb;
        gy = gy + p.a0 * dy * ea;
        gy = gy + p.b0 * dy * eb;
    }
    if (g) {
        g[0] = gx;
        g[1] = gy;
    }
    return v - pes->V0;
}

/* Harmonic test surface V = k/2 sum x^2 (no reference counterpart; used for
 * analytic known answers).  params = [k]. */
static double v_harm(const or_pes *pes, const double *x, double *g) {
    double k = pes->nparams >= 1 ? pes->params[0] : 1.0;
    int nd = pes->ndim * pes->natom;
    double v = 0.0;
    for (int i = 0; i < nd; i++) {
        v += 0.5 * k * x[i] * x[i];
        if (g) g[i] = k * x[i];
    }
    return v - pes->V0;
}

/* Synthetic 9-atom surface: pair Morse network plus a quartic double well in
 * the proton-transfer coordinate s = |r_H - r_O1| - |r_H - r_O2|.
 * params = [npair, (i, j, D, a, r0) x npair, iH, iO1, iO2, B, s0]
 * V = sum_p D (1 - exp(-a (r - r0)))^2 + B ((s/s0)^2 - 1)^2 - V0.
 * (No reference counterpart: the structural template is the pair-distance /
 * B-matrix form of pes_malonaldehyde.f90:9362-9490.) */
static double v_synth9(const or_pes *pes, const double *x, double *g) {
    const double *pp = pes->params;
    int npair = (int)pp[0];
    int nd = 3 * pes->natom;
    if (g) memset(g, 0, sizeof(double) * nd);
    double v = 0.0;
    for (int q = 0; q < npair; q++) {
        const double *r = pp + 1 + 5 * q;
        int i = (int)r[0], j = (int)r[1];
        double D = r[2], a = r[3], r0 = r[4];
        double d0 = x[3 * i] - x[3 * j], d1 = x[3 * i + 1] - x[3 * j + 1],
               d2 = x[3 * i + 2] - x[3 * j + 2];
        double rr = sqrt(d0 * d0 + d1 * d1 + d2 * d2);
        double e = exp(-a * (rr - r0));
        double om = 1.0 - e;
        v += D * om * om;
        if (g) {
            double dvdr = 2.0 * D * a * om * e / rr;
            g[3 * i] += dvdr * d0;
            g[3 * i + 1] += dvdr * d1;
            g[3 * i + 2] += dvdr * d2;
            g[3 * j] -= dvdr * d0;
            g[3 * j + 1] -= dvdr * d1;
            g[3 * j + 2] -= dvdr * d2;
        }
    }
    const double *w = pp + 1 + 5 * npair;
    int iH = (int)w[0], iO1 = (int)w[1], iO2 = (int)w[2];
    double B = w[3], s0 = w[4];
    double e1[3], e2[3];
    double r1 = 0.0, r2 = 0.0;
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
    v += B * t * t;
    if (g) {
        double dvds = 4.0 * B * t * s / (s0 * s0);
        for (int c = 0; c < 3; c++) {
            double a1 = dvds * e1[c] / r1, a2 = dvds * e2[c] / r2;
            g[3 * iH + c] += a1 - a2;
            g[3 * iO1 + c] -= a1;
            g[3 * iO2 + c] += a2;
        }
    }
    return v - pes->V0;
}

/* Synthetic 18-atom water-cluster surface.  Atoms are ordered (O, H, H) per
 * molecule.  params = [nmol, kr, re, ktheta, theta_e, eps, sigma, qO, qH]
 * V = sum_m [kr/2 ((r1-re)^2 + (r2-re)^2) + ktheta/2 (theta-theta_e)^2]
 *   + sum_{m<n} [4 eps ((sigma/r_OO)^12 - (sigma/r_OO)^6) + sum_{i in m, j in n} q_i q_j / r_ij]
 *   - V0.  (No reference counterpart.) */
static double v_synth18(const or_pes *pes, const double *x, double *g) {
    const double *pp = pes->params;
    int nmol = (int)pp[0];
    double kr = pp[1], re = pp[2], kth = pp[3], the = pp[4], eps = pp[5], sig = pp[6];
    double qO = pp[7], qH = pp[8];
    int nd = 9 * nmol;
    if (g) memset(g, 0, sizeof(double) * nd);
    double v = 0.0;
    for (int m = 0; m < nmol; m++) {
        const double *O = x + 9 * m, *H1 = O + 3, *H2 = O + 6;
        double u1[3], u2[3], r1 = 0.0, r2 = 0.0;
        for (int c = 0; c < 3; c++) {
            u1[c] = H1[c] - O[c];
            u2[c] = H2[c] - O[c];
            r1 += u1[c] * u1[c];
            r2 += u2[c] * u2[c];
        }
        r1 = sqrt(r1);
        r2 = sqrt(r2);
        double ct = (u1[0] * u2[0] + u1[1] * u2[1] + u1[2] * u2[2]) / (r1 * r2);
        if (ct > 1.0) ct = 1.0;
        if (ct < -1.0) ct = -1.0;
        double th = acos(ct);
        v += 0.5 * kr * ((r1 - re) * (r1 - re) + (r2 - re) * (r2 - re));
        v += 0.5 * kth * (th - the) * (th - the);
        if (g) {
            double st = sqrt(1.0 - ct * ct);
            if (st < 1e-12) st = 1e-12;
            double dth = kth * (th - the);
            for (int c = 0; c < 3; c++) {
                double n1 = u1[c] / r1, n2 = u2[c] / r2;
                double gb1 = kr * (r1 - re) * n1, gb2 = kr * (r2 - re) * n2;
                /* d theta / d H1 = -(n2 - ct n1) / (r1 sin theta) */
                double ga1 = -dth * (n2 - ct * n1) / (r1 * st);
                double ga2 = -dth * (n1 - ct * n2) / (r2 * st);
                g[9 * m + 3 + c] += gb1 + ga1;
                g[9 * m + 6 + c] += gb2 + ga2;
                g[9 * m + c] -= gb1 + ga1 + gb2 + ga2;
            }
        }
    }
    for (int m = 0; m < nmol; m++) {
        for (int n = m + 1; n < nmol; n++) {
            for (int ia = 0; ia < 3; ia++) {
                for (int ib = 0; ib < 3; ib++) {
                    const double *A = x + 9 * m + 3 * ia, *Bp = x + 9 * n + 3 * ib;
                    double d0 = A[0] - Bp[0], d1 = A[1] - Bp[1], d2 = A[2] - Bp[2];
                    double r2 = d0 * d0 + d1 * d1 + d2 * d2;
                    double r = sqrt(r2);
                    double qa = ia == 0 ? qO : qH, qb = ib == 0 ? qO : qH;
                    double e = qa * qb / r;
                    double dvdr_over_r = -e / r2;
                    if (ia == 0 && ib == 0) {
                        double sr2 = sig * sig / r2;
                        double sr6 = sr2 * sr2 * sr2;
                        double sr12 = sr6 * sr6;
                        e += 4.0 * eps * (sr12 - sr6);
                        dvdr_over_r += 4.0 * eps * (-12.0 * sr12 + 6.0 * sr6) / r2;
                    }
                    v += e;
                    if (g) {
                        int ai = 9 * m + 3 * ia, bi = 9 * n + 3 * ib;
                        g[ai] += dvdr_over_r * d0;
                        g[ai + 1] += dvdr_over_r * d1;
                        g[ai + 2] += dvdr_over_r * d2;
                        g[bi] -= dvdr_over_r * d0;
                        g[bi + 1] -= dvdr_over_r * d1;
                        g[bi + 2] -= dvdr_over_r * d2;
                    }
                }
            }
        }
    }
    return v - pes->V0;
}

/* Morse terms and 1-, 2-, 3-D Gaussians in the interatomic distances, the
 * functional form of pes_malonaldehyde.f90 (distances :9357-9365, v_morse
 * :9598-9610, v_gauss :9650-9670, energy sums :9406-9440); the gradient by
 * the chain rule through the distances (the B matrix of :9368-9384).
 * params = [natom, shift, nmorse, ng1, ng2, ng3, nmorse x (k, re, al, de),
 *           ng1 x (k, x, a, d, s), ng2 x (k1, k2, x1, x2, a1, a2, d, s),
 *           ng3 x (k1, k2, k3, x1, x2, x3, a1, a2, a3, d, s)],
 * k = i (i - 1) / 2 + j for atoms i > j (0-based). */
static double v_distgauss(const or_pes *pes, const double *x, double *g) {
    const double *pp = pes->params;
    const int na = pes->natom, npair = na * (na - 1) / 2;
    double *r = (double *)calloc((size_t)npair, sizeof(double));
    double *dv = (double *)calloc((size_t)npair, sizeof(double));
    int k = 0;
    for (int i = 1; i < na; i++)
        for (int j = 0; j < i; j++) {
            double s2 = 0.0;
            for (int c = 0; c < 3; c++) s2 += (x[3 * i + c] - x[3 * j + c]) * (x[3 * i + c] - x[3 * j + c]);
            r[k++] = sqrt(s2);
        }
    double v = pp[1];
    const int nm = (int)pp[2], n1 = (int)pp[3], n2 = (int)pp[4], n3 = (int)pp[5];
    const double *q = pp + 6;
    for (int t = 0; t < nm; t++, q += 4) {
        int kk = (int)q[0];
        double e = exp(q[2] * (q[1] - r[kk])), w = e - 1.0;
        v += (q[3] * w) * (q[3] * w);
        dv[kk] -= 2.0 * q[3] * q[3] * w * e * q[2];
    }
    for (int t = 0; t < n1; t++, q += 5) {
        int kk = (int)q[0];
        double u = r[kk] - q[1], e = exp(-0.5 * q[2] * u * u);
        v += q[3] * (e - q[4]);
        dv[kk] -= q[3] * e * q[2] * u;
    }
    for (int t = 0; t < n2; t++, q += 8) {
        int k1 = (int)q[0], k2 = (int)q[1];
        double u1 = r[k1] - q[2], u2 = r[k2] - q[3];
        double e = exp(-0.5 * (q[4] * u1 * u1 + q[5] * u2 * u2));
        v += q[6] * (e - q[7]);
        dv[k1] -= q[6] * e * q[4] * u1;
        dv[k2] -= q[6] * e * q[5] * u2;
    }
    for (int t = 0; t < n3; t++, q += 11) {
        int k1 = (int)q[0], k2 = (int)q[1], k3 = (int)q[2];
        double u1 = r[k1] - q[3], u2 = r[k2] - q[4], u3 = r[k3] - q[5];
        double e = exp(-0.5 * (q[6] * u1 * u1 + q[7] * u2 * u2 + q[8] * u3 * u3));
        v += q[9] * (e - q[10]);
        dv[k1] -= q[9] * e * q[6] * u1;
        dv[k2] -= q[9] * e * q[7] * u2;
        dv[k3] -= q[9] * e * q[8] * u3;
    }
    if (g) {
        memset(g, 0, sizeof(double) * 3 * na);
        k = 0;
        for (int i = 1; i < na; i++)
            for (int j = 0; j < i; j++, k++)
                for (int c = 0; c < 3; c++) {
                    double d = (x[3 * i + c] - x[3 * j + c]) / r[k];
                    g[3 * i + c] += dv[k] * d;
                    g[3 * j + c] -= dv[k] * d;
                }
    }
    free(r);
    free(dv);
    return v - pes->V0;
}

static double pes_eval(const or_pes *pes, const double *x, double *g) {
    switch (pes->id) {
    case OR_PES_1D: return v_1d(pes, x, g);
    case OR_PES_2DTEST: return v_2d(pes, x, g);
    case OR_PES_SYNTH9: return v_synth9(pes, x, g);
    case OR_PES_SYNTH18: return v_synth18(pes, x, g);
    case OR_PES_HARMONIC: return v_harm(pes, x, g);
    case OR_PES_DISTGAUSS: return v_distgauss(pes, x, g);
    default: return NAN;
    }
}

double or_V(const or_pes *pes, const double *x) { return pes_eval(pes, x, NULL); }
void or_Vprime(const or_pes *pes, const double *x, double *grad) { pes_eval(pes, x, grad); }
double or_potforce(const or_pes *pes, const double *x, double *grad) {
    return pes_eval(pes, x, grad);
}

/* Central finite-difference Hessian of Vprime with eps = 1e-4, restating
 * mcmod_1d.f90:38-58 (same perturbation arithmetic: x+eps, then x+eps-2eps). */
static void hess_fd(const or_pes *pes, const double *x, double *hess) {
    int nd = pes->ndim * pes->natom;
    double eps = 1e-4;
    double *xw = (double *)malloc(sizeof(double) * nd);
    double *gp = (double *)malloc(sizeof(double) * nd);
    double *gm = (double *)malloc(sizeof(double) * nd);
    memcpy(xw, x, sizeof(double) * nd);
    for (int a = 0; a < nd; a++) {
        double x0 = xw[a];
        xw[a] = x0 + eps;
        pes_eval(pes, xw, gp);
        xw[a] = xw[a] - 2.0 * eps;
        pes_eval(pes, xw, gm);
        xw[a] = x0;
        for (int b = 0; b < nd; b++) hess[a + nd * b] = (gp[b] - gm[b]) / (2.0 * eps);
    }
    free(xw);
    free(gp);
    free(gm);
}

/* mcmod_2dtest.f90:64-102.  quirks=1: the reference (overwrite per well, so only
 * the last well survives, and its chain rule); quirks=0: the exact Hessian. */
static void hess_2d(const or_pes *pes, const double *x, double *hess, int quirks) {
    p2d_t p = p2d(pes);
    double hxx = 0.0, hxy = 0.0, hyy = 0.0;
    for (int k = 1; k <= p.m; k++) {
        double xk = p.rho0 * cos((double)k * 2.0 * OR_PI_REF / (double)p.m);
        double yk = p.rho0 * sin((double)k * 2.0 * OR_PI_REF / (double)p.m);
        double dx = x[0] - xk, dy = x[1] - yk;
        double u = dx * dx + dy * dy;
        double ea = exp(-p.a0 * u), eb = exp(-p.b0 * u);
        double dvdu = p.a0 * ea + p.b0 * eb;
        double d2 = -p.a0 * p.a0 * ea - p.b0 * p.b0 * eb;
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

/* Add the Hessian of a distance r_ij to hess with weight w (hess[a+nd*b]). */
static void add_dist_hess(double *hess, int nd, int i, int j, const double *x, double w1,
                          double w2) {
    /* w1 * d2r/dxdx + w2 * dr/dx dr/dx^T */
    double d[3], r = 0.0;
    for (int c = 0; c < 3; c++) {
        d[c] = x[3 * i + c] - x[3 * j + c];
        r += d[c] * d[c];
    }
    r = sqrt(r);
    for (int c1 = 0; c1 < 3; c1++) {
        for (int c2 = 0; c2 < 3; c2++) {
            double u1 = d[c1] / r, u2 = d[c2] / r;
            double blk = w1 * (((c1 == c2) ? 1.0 : 0.0) - u1 * u2) / r + w2 * u1 * u2;
            hess[(3 * i + c1) + nd * (3 * i + c2)] += blk;
            hess[(3 * j + c1) + nd * (3 * j + c2)] += blk;
            hess[(3 * i + c1) + nd * (3 * j + c2)] -= blk;
            hess[(3 * j + c1) + nd * (3 * i + c2)] -= blk;
        }
    }
}

/* Analytic Hessian of the synthetic 9-atom surface. */
static void hess_synth9(const or_pes *pes, const double *x, double *hess) {
    const double *pp = pes->params;
    int npair = (int)pp[0];
    int nd = 3 * pes->natom;
    memset(hess, 0, sizeof(double) * nd * nd);
    for (int q = 0; q < npair; q++) {
        const double *r = pp + 1 + 5 * q;
        int i = (int)r[0], j = (int)r[1];
        double D = r[2], a = r[3], r0 = r[4];
        double d0 = x[3 * i] - x[3 * j], d1 = x[3 * i + 1] - x[3 * j + 1],
               d2 = x[3 * i + 2] - x[3 * j + 2];
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
    /* dV'(s) * Hess(s) + V''(s) grad s grad s^T */
    add_dist_hess(hess, nd, iH, iO1, x, dvds, 0.0);
    add_dist_hess(hess, nd, iH, iO2, x, -dvds, 0.0);
    double gs[27 * 3];
    memset(gs, 0, sizeof(double) * nd);
    for (int c = 0; c < 3; c++) {
        gs[3 * iH + c] += e1[c] / r1 - e2[c] / r2;
        gs[3 * iO1 + c] -= e1[c] / r1;
        gs[3 * iO2 + c] += e2[c] / r2;
    }
    for (int aa = 0; aa < nd; aa++)
        for (int bb = 0; bb < nd; bb++) hess[aa + nd * bb] += d2vds2 * gs[aa] * gs[bb];
}

void or_Vdoubleprime(const or_pes *pes, const double *x, double *hess, int quirks) {
    int nd = pes->ndim * pes->natom;
    switch (pes->id) {
    case OR_PES_2DTEST: hess_2d(pes, x, hess, quirks); return;
    case OR_PES_SYNTH9: hess_synth9(pes, x, hess); return;
    case OR_PES_HARMONIC: {
        double k = pes->nparams >= 1 ? pes->params[0] : 1.0;
        memset(hess, 0, sizeof(double) * nd * nd);
        for (int i = 0; i < nd; i++) hess[i + nd * i] = k;
        return;
    }
    default: hess_fd(pes, x, hess); return;
    }
}

/* ------------------------------------------------------------------------- */
/* RNG                                                                       */
/* ------------------------------------------------------------------------- */

/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11). */
void or_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; r++) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n1 = lo1;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        uint32_t n3 = lo0;
        c0 = n0;
        c1 = n1;
        c2 = n2;
        c3 = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

/* Stream layout: key = seed (lo, hi); counter = {n/4, step, stream, purpose}.
 * Uniform u = (w + 0.5) * 2^-32.  Normals come in Box-Muller pairs from
 * (w0, w1) and (w2, w3): z = sqrt(-2 ln u_a) * (cos, sin)(2 pi u_b). */
static void philox_block(uint64_t seed, uint32_t stream, uint32_t step, uint32_t purpose,
                         uint32_t blk, uint32_t out[4]) {
    uint32_t ctr[4] = {blk, step, stream, purpose};
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    or_philox4x32_10(ctr, key, out);
}

static double u32_to_unit(uint32_t w) { return ((double)w + 0.5) * 2.3283064365386963e-10; }

double or_uniform(uint64_t seed, uint32_t stream, uint32_t step, uint32_t purpose, uint32_t n) {
    uint32_t o[4];
    philox_block(seed, stream, step, purpose, n >> 2, o);
    return u32_to_unit(o[n & 3]);
}

#define OR_TWO_PI 6.283185307179586

double or_normal(uint64_t seed, uint32_t stream, uint32_t step, uint32_t purpose, uint32_t n) {
    uint32_t o[4];
    philox_block(seed, stream, step, purpose, n >> 2, o);
    int pair = (n >> 1) & 1;
    double ua = u32_to_unit(o[2 * pair]);
    double ub = u32_to_unit(o[2 * pair + 1]);
    double r = sqrt(-2.0 * log(ua));
    double th = OR_TWO_PI * ub;
    return (n & 1) ? r * sin(th) : r * cos(th);
}

/* Andersen kick interval (replaces virngpoisson POISNORM, verletmodule.f90:202,230).
 * mean < 30: inversion with one uniform; else floor(mean + sqrt(mean) z + 0.5). */
int64_t or_poisson(uint64_t seed, uint32_t stream, uint32_t step, uint32_t purpose, double mean) {
    if (mean < 30.0) {
        double u = or_uniform(seed, stream, step, purpose, 0u);
        double pk = exp(-mean), cdf = pk;
        int64_t k = 0;
        while (u > cdf && k < 1000) {
            k++;
            pk *= mean / (double)k;
            cdf += pk;
        }
        return k;
    }
    double z = or_normal(seed, stream, step, purpose, 0u);
    double v = floor(mean + sqrt(mean) * z + 0.5);
    return v < 0.0 ? 0 : (int64_t)v;
}

/* ------------------------------------------------------------------------- */
/* Normal modes                                                              */
/* ------------------------------------------------------------------------- */

/* verletmodule.f90:306-338 (init_nm). */
void or_init_nm(int64_t P, int64_t ndim, int64_t natom, const double *mass, double betan,
                double tau, const double *a, const double *b, double *T, double *lam,
                double *beadmass, double *beadvec) {
    int64_t nd = ndim * natom;
    for (int64_t i = 1; i <= P; i++) {
        lam[i - 1] = 2.0 * sin((double)i * OR_PI_REF / (double)(2 * P + 2)) / betan;
        for (int64_t j = 0; j < natom; j++)
            beadmass[j + natom * (i - 1)] = mass[j] * (lam[i - 1] * tau) * (lam[i - 1] * tau);
        for (int64_t l = i; l <= P; l++) {
            double t = sin((double)(i * l) * OR_PI_REF / (double)(P + 1)) * sqrt(2.0 / (double)(P + 1));
            T[(i - 1) + P * (l - 1)] = t;
            T[(l - 1) + P * (i - 1)] = t;
        }
        for (int64_t j = 0; j < ndim; j++) {
            for (int64_t k = 0; k < natom; k++) {
                int64_t dof = k * ndim + j;
                double bv = a[dof] * sin((double)i * OR_PI_REF / (double)(P + 1)) +
                            b[dof] * sin((double)(P * i) * OR_PI_REF / (double)(P + 1));
                bv = bv * sqrt(2.0 / (double)(P + 1));
                bv = bv / ((lam[i - 1] * betan) * (lam[i - 1] * betan));
                beadvec[(i - 1) + P * dof] = bv;
            }
        }
    }
    (void)nd;
}

/* verletmodule.f90:254-266 (dsymv with the full symmetric matrix). */
void or_nm_forward(int64_t P, const double *T, const double *x, double *q, const double *shift) {
    for (int64_t i = 0; i < P; i++) {
        double s = 0.0;
        for (int64_t l = 0; l < P; l++) s += T[i + P * l] * x[l];
        q[i] = s;
    }
    if (shift)
        for (int64_t i = 0; i < P; i++) q[i] = q[i] - shift[i];
}

/* verletmodule.f90:270-286 (nmtransform_backward). */
void or_nm_backward(int64_t P, const double *T, const double *q, double *x, const double *shift) {
    double *qs = (double *)malloc(sizeof(double) * P);
    for (int64_t i = 0; i < P; i++) qs[i] = shift ? q[i] + shift[i] : q[i];
    for (int64_t i = 0; i < P; i++) {
        double s = 0.0;
        for (int64_t l = 0; l < P; l++) s += T[i + P * l] * qs[l];
        x[i] = s;
    }
    free(qs);
}

/* ------------------------------------------------------------------------- */
/* TI propagation                                                            */
/* ------------------------------------------------------------------------- */

typedef struct ring_ws {
    int64_t P, nd, natom, ndim;
    double *T, *lam, *beadmass, *beadvec;
    double *c1, *c2;          /* [natom*P] */
    double *q, *pip, *tmp, *g, *force, *xb;
} ring_ws;

static void ws_alloc(ring_ws *w, int64_t P, int64_t ndim, int64_t natom) {
    w->P = P;
    w->ndim = ndim;
    w->natom = natom;
    w->nd = ndim * natom;
    w->T = (double *)malloc(sizeof(double) * P * P);
    w->lam = (double *)malloc(sizeof(double) * P);
    w->beadmass = (double *)malloc(sizeof(double) * natom * P);
    w->beadvec = (double *)malloc(sizeof(double) * P * w->nd);
    w->c1 = (double *)malloc(sizeof(double) * natom * P);
    w->c2 = (double *)malloc(sizeof(double) * natom * P);
    w->q = (double *)malloc(sizeof(double) * P * w->nd);
    w->pip = (double *)malloc(sizeof(double) * P * w->nd);
    w->tmp = (double *)malloc(sizeof(double) * P * w->nd);
    w->g = (double *)malloc(sizeof(double) * w->nd);
    w->force = (double *)malloc(sizeof(double) * P * w->nd);
    w->xb = (double *)malloc(sizeof(double) * w->nd);
}

static void ws_free(ring_ws *w) {
    free(w->T); free(w->lam); free(w->beadmass); free(w->beadvec); free(w->c1); free(w->c2);
    free(w->q); free(w->pip); free(w->tmp); free(w->g); free(w->force); free(w->xb);
}

static void ws_setup(ring_ws *w, const double *mass, const or_ti_params *prm, const double *a,
                     const double *b) {
    or_init_nm(w->P, w->ndim, w->natom, mass, prm->betan, prm->tau, a, b, w->T, w->lam,
               w->beadmass, w->beadvec);
    /* verletmodule.f90:380-386 */
    for (int64_t i = 0; i < w->P; i++) {
        for (int64_t j = 0; j < w->natom; j++) {
            double bm = w->beadmass[j + w->natom * i];
            double c = exp(-prm->gamma * prm->dt * w->lam[i] * sqrt(mass[j] / bm));
            w->c1[j + w->natom * i] = c;
            w->c2[j + w->natom * i] = sqrt(1.0 - c * c);
        }
    }
}

/* verletmodule.f90:565-585 (step_v): p -= grad V(x_bead) * t. */
static int step_v(const or_pes *pes, ring_ws *w, const double *x, double *p, double t) {
    int64_t P = w->P;
    for (int64_t i = 0; i < P; i++) {
        for (int64_t d = 0; d < w->nd; d++) w->xb[d] = x[d * P + i];
        or_Vprime(pes, w->xb, w->g);
        for (int64_t d = 0; d < w->nd; d++) {
            p[d * P + i] = p[d * P + i] - w->g[d] * t;
            if (p[d * P + i] != p[d * P + i]) return 1;
        }
    }
    return 0;
}

/* Free-polymer rotation of one normal mode (verletmodule.f90:515-532). */
static void nm_rotate(double *q, double *pi, double t, double omegak, double bm, int cayley) {
    double np, nq;
    if (cayley) {
        np = *pi * (4.0 - omegak * omegak * t * t) - 4.0 * (*q) * bm * omegak * omegak * t;
        np = np / (4.0 + omegak * omegak * t * t);
        nq = *q * (4.0 - omegak * omegak * t * t) + 4.0 * (*pi) * t / bm;
        nq = nq / (4.0 + omegak * omegak * t * t);
    } else {
        np = *pi * cos(t * omegak) - *q * omegak * bm * sin(omegak * t);
        nq = *q * cos(t * omegak) + *pi * sin(omegak * t) / (omegak * bm);
    }
    *pi = np;
    *q = nq;
}

/* verletmodule.f90:494-561 (step_nm with transform=.true.). */
static int step_nm_ref(ring_ws *w, const double *mass, double *x, double *p, double t,
                       int cayley) {
    int64_t P = w->P;
    for (int64_t d = 0; d < w->nd; d++) {
        or_nm_forward(P, w->T, p + d * P, w->pip + d * P, NULL);
        or_nm_forward(P, w->T, x + d * P, w->q + d * P, w->beadvec + d * P);
    }
    for (int64_t i = 0; i < P; i++) {
        for (int64_t j = 0; j < w->ndim; j++) {
            for (int64_t k = 0; k < w->natom; k++) {
                int64_t d = k * w->ndim + j;
                double bm = w->beadmass[k + w->natom * i];
                double omegak = sqrt(mass[k] / bm) * w->lam[i];
                nm_rotate(&w->q[d * P + i], &w->pip[d * P + i], t, omegak, bm, cayley);
                if (w->pip[d * P + i] != w->pip[d * P + i]) return 1;
            }
        }
    }
    for (int64_t d = 0; d < w->nd; d++) {
        or_nm_backward(P, w->T, w->pip + d * P, p + d * P, NULL);
        or_nm_backward(P, w->T, w->q + d * P, x + d * P, w->beadvec + d * P);
    }
    return 0;
}

/* verletmodule.f90:634-667 (step_langevin). */
static void step_langevin_ref(ring_ws *w, const double *mass, double betan, double *p,
                              uint64_t seed, uint32_t stream, uint32_t step) {
    int64_t P = w->P;
    for (int64_t j = 0; j < w->ndim; j++) {
        for (int64_t k = 0; k < w->natom; k++) {
            int64_t d = k * w->ndim + j;
            or_nm_forward(P, w->T, p + d * P, w->pip + d * P, NULL);
            for (int64_t i = 0; i < P; i++) {
                double c1 = w->c1[k + w->natom * i], c2 = w->c2[k + w->natom * i];
                double bm = w->beadmass[k + w->natom * i];
                double z = or_normal(seed, stream, step, 0u, (uint32_t)(d * P + i));
                w->pip[d * P + i] = (c1 * c1) * w->pip[d * P + i] +
                                    sqrt(bm / betan) * c2 * sqrt(1.0 + c1 * c1) * z;
            }
            or_nm_backward(P, w->T, w->pip + d * P, p + d * P, NULL);
        }
    }
    (void)mass;
}

/* NM-resident step state: q (shifted NM positions), pip (NM momenta), x. */
static void nmres_from_cart(ring_ws *w, const double *x, const double *p) {
    for (int64_t d = 0; d < w->nd; d++) {
        or_nm_forward(w->P, w->T, x + d * w->P, w->q + d * w->P, w->beadvec + d * w->P);
        or_nm_forward(w->P, w->T, p + d * w->P, w->pip + d * w->P, NULL);
    }
}

static void nmres_positions(ring_ws *w, double *x) {
    for (int64_t d = 0; d < w->nd; d++)
        or_nm_backward(w->P, w->T, w->q + d * w->P, x + d * w->P, w->beadvec + d * w->P);
}

static void nmres_momenta(ring_ws *w, double *p) {
    for (int64_t d = 0; d < w->nd; d++)
        or_nm_backward(w->P, w->T, w->pip + d * w->P, p + d * w->P, NULL);
}

/* Normal-mode kick: pip -= t * T grad V(x). */
static int nmres_kick(const or_pes *pes, ring_ws *w, const double *x, double t) {
    int64_t P = w->P;
    for (int64_t i = 0; i < P; i++) {
        for (int64_t d = 0; d < w->nd; d++) w->xb[d] = x[d * P + i];
        or_Vprime(pes, w->xb, w->g);
        for (int64_t d = 0; d < w->nd; d++) w->force[d * P + i] = w->g[d];
    }
    for (int64_t d = 0; d < w->nd; d++) {
        or_nm_forward(P, w->T, w->force + d * P, w->tmp + d * P, NULL);
        for (int64_t i = 0; i < P; i++) {
            w->pip[d * P + i] = w->pip[d * P + i] - t * w->tmp[d * P + i];
            if (w->pip[d * P + i] != w->pip[d * P + i]) return 1;
        }
    }
    return 0;
}

static void nmres_rotate(ring_ws *w, const double *mass, double t, int cayley) {
    int64_t P = w->P;
    for (int64_t i = 0; i < P; i++)
        for (int64_t k = 0; k < w->natom; k++) {
            double bm = w->beadmass[k + w->natom * i];
            double omegak = sqrt(mass[k] / bm) * w->lam[i];
            for (int64_t j = 0; j < w->ndim; j++) {
                int64_t d = k * w->ndim + j;
                nm_rotate(&w->q[d * P + i], &w->pip[d * P + i], t, omegak, bm, cayley);
            }
        }
}

static void nmres_ou(ring_ws *w, double betan, uint64_t seed, uint32_t stream, uint32_t step) {
    int64_t P = w->P;
    for (int64_t d = 0; d < w->nd; d++) {
        int64_t k = d / w->ndim;
        for (int64_t i = 0; i < P; i++) {
            double c1 = w->c1[k + w->natom * i], c2 = w->c2[k + w->natom * i];
            double bm = w->beadmass[k + w->natom * i];
            double z = or_normal(seed, stream, step, 0u, (uint32_t)(d * P + i));
            w->pip[d * P + i] = (c1 * c1) * w->pip[d * P + i] +
                                sqrt(bm / betan) * c2 * sqrt(1.0 + c1 * c1) * z;
        }
    }
}

/* p = T * (sqrt(beadmass/betan) * z) (verletmodule.f90:102-115, 211-229). */
static void sample_nm_momenta(ring_ws *w, double betan, uint64_t seed, uint32_t stream,
                              uint32_t step, uint32_t purpose, double *pnm) {
    int64_t P = w->P;
    for (int64_t d = 0; d < w->nd; d++) {
        int64_t k = d / w->ndim;
        for (int64_t i = 0; i < P; i++) {
            double z = or_normal(seed, stream, step, purpose, (uint32_t)(d * P + i));
            pnm[d * P + i] = z * sqrt(1.0 / betan) * sqrt(w->beadmass[k + w->natom * i]);
        }
    }
}

void or_ring_init(const or_pes *pes, const double *mass, const or_ti_params *prm,
                  const double *T, const double *beadmass, const double *xref,
                  uint64_t seed, uint32_t stream, uint32_t step, uint32_t purpose_x,
                  uint32_t purpose_p, double *x, double *p) {
    int64_t P = prm->P, nd = (int64_t)pes->ndim * pes->natom, natom = pes->natom;
    for (int64_t d = 0; d < nd; d++)
        for (int64_t i = 0; i < P; i++) {
            double z = prm->init_sigma != 0.0
                           ? or_normal(seed, stream, step, purpose_x, (uint32_t)(d * P + i))
                           : 0.0;
            x[d * P + i] = xref[d * P + i] + prm->init_sigma * z;
        }
    double *vel = (double *)malloc(sizeof(double) * P);
    for (int64_t d = 0; d < nd; d++) {
        int64_t k = d / pes->ndim;
        for (int64_t i = 0; i < P; i++) {
            double z = or_normal(seed, stream, step, purpose_p, (uint32_t)(d * P + i));
            vel[i] = z * sqrt(1.0 / prm->betan) * sqrt(beadmass[k + natom * i]);
        }
        or_nm_backward(P, T, vel, p + d * P, NULL);
    }
    free(vel);
    (void)mass;
}

static double estimator(const ring_ws *w, const double *mass, const double *x,
                        const double *dbdl) {
    /* verletmodule.f90:397-403 */
    double contr = 0.0;
    for (int64_t j = 0; j < w->ndim; j++)
        for (int64_t k = 0; k < w->natom; k++) {
            int64_t d = k * w->ndim + j;
            contr = contr + mass[k] * (-x[d * w->P + (w->P - 1)]) * dbdl[d];
        }
    return contr;
}

/* verletmodule.f90:372-416 (Langevin) and 190-250 (Andersen).  Step s is the
 * 0-based global step (the reference's ii = s + 1), so chunked calls with the
 * same res reproduce one long call.  Andersen kick state lives in res. */
void or_ring_propagate(const or_pes *pes, const double *mass, const or_ti_params *prm,
                       const double *a, const double *b, const double *dbdl,
                       const double *xref, uint64_t seed, uint32_t stream,
                       int64_t step0, int64_t nsteps, double *x, double *p,
                       or_ring_result *res) {
    ring_ws w;
    ws_alloc(&w, prm->P, pes->ndim, pes->natom);
    ws_setup(&w, mass, prm, a, b);
    double dt = prm->dt;
    int status = 0;
    if (prm->nm_resident) nmres_from_cart(&w, x, p);
    if (prm->thermostat == 1 && res->and_rkick < 0) {
        res->and_count = 0;
        res->and_rkick = or_poisson(seed, stream, 0u, 4u, (double)prm->noutput);
    }
    for (int64_t s = step0; s < step0 + nsteps && !status; s++) {
        uint32_t st = (uint32_t)s;
        if (prm->thermostat == 2) {
            if (!prm->nm_resident) {
                status |= step_v(pes, &w, x, p, dt);
                status |= step_nm_ref(&w, mass, x, p, 0.5 * dt, prm->cayley);
                step_langevin_ref(&w, mass, prm->betan, p, seed, stream, st);
                status |= step_nm_ref(&w, mass, x, p, 0.5 * dt, prm->cayley);
            } else {
                status |= nmres_kick(pes, &w, x, dt);
                nmres_rotate(&w, mass, 0.5 * dt, prm->cayley);
                nmres_ou(&w, prm->betan, seed, stream, st);
                nmres_rotate(&w, mass, 0.5 * dt, prm->cayley);
                nmres_positions(&w, x);
            }
        } else {
            /* verletmodule.f90:204-234: resample all NM momenta when the interval ends */
            res->and_count += 1;
            if (res->and_count >= res->and_rkick) {
                res->and_count = 0;
                if (!prm->nm_resident) {
                    sample_nm_momenta(&w, prm->betan, seed, stream, st, 3u, w.pip);
                    nmres_momenta(&w, p);
                } else {
                    sample_nm_momenta(&w, prm->betan, seed, stream, st, 3u, w.pip);
                }
                res->and_rkick = or_poisson(seed, stream, st, 7u, (double)prm->noutput);
            }
            /* verletmodule.f90:291-302 (time_step_nm) */
            if (!prm->nm_resident) {
                status |= step_nm_ref(&w, mass, x, p, 0.5 * dt, prm->cayley);
                status |= step_v(pes, &w, x, p, dt);
                status |= step_nm_ref(&w, mass, x, p, 0.5 * dt, prm->cayley);
            } else {
                nmres_rotate(&w, mass, 0.5 * dt, prm->cayley);
                nmres_positions(&w, x);
                status |= nmres_kick(pes, &w, x, dt);
                nmres_rotate(&w, mass, 0.5 * dt, prm->cayley);
                nmres_positions(&w, x);
            }
        }
        if (s >= prm->imin) {
            double contr = estimator(&w, mass, x, dbdl);
            if (prm->thermostat != 2 || fabs(contr) < prm->dhdr_limit || prm->dhdr_limit < 0.0) {
                res->dhdr_sum += contr;
            } else {
                /* verletmodule.f90:404-409: re-initialise the ring in place */
                or_ring_init(pes, mass, prm, w.T, w.beadmass, xref, seed, stream, st, 5u, 6u, x,
                             p);
                if (prm->nm_resident) nmres_from_cart(&w, x, p);
                res->nreinit += 1;
            }
            res->nsamples += 1;
        }
    }
    if (prm->nm_resident) nmres_momenta(&w, p);
    res->status = status;
    ws_free(&w);
}

/* ------------------------------------------------------------------------- */
/* Batched CPU baseline                                                      */
/* ------------------------------------------------------------------------- */

typedef struct batch_job {
    const or_pes *pes;
    const double *mass;
    const or_ti_params *prm;
    const int32_t *lam_index;
    const uint64_t *seeds;
    const uint32_t *streams;
    const double *a, *b, *dbdl, *xref;
    int64_t nsteps, nrings, nd;
    double *x, *p;
    or_ring_result *res;
    int64_t next;
    pthread_mutex_t lock;
} batch_job;

static void *batch_worker(void *arg) {
    batch_job *J = (batch_job *)arg;
    int64_t P = J->prm->P;
    for (;;) {
        pthread_mutex_lock(&J->lock);
        int64_t r = J->next++;
        pthread_mutex_unlock(&J->lock);
        if (r >= J->nrings) break;
        int32_t li = J->lam_index[r];
        J->res[r].dhdr_sum = 0.0;
        J->res[r].nsamples = 0;
        J->res[r].nreinit = 0;
        J->res[r].status = 0;
        J->res[r].pad = 0;
        J->res[r].and_count = 0;
        J->res[r].and_rkick = -1;
        or_ring_propagate(J->pes, J->mass, J->prm, J->a, J->b + li * J->nd, J->dbdl + li * J->nd,
                          J->xref + li * J->nd * P, J->seeds[r], J->streams[r], 0, J->nsteps,
                          J->x + r * J->nd * P, J->p + r * J->nd * P, &J->res[r]);
    }
    return NULL;
}

int or_ti_run_batch(const or_pes *pes, const double *mass, const or_ti_params *prm,
                    int64_t nrings, const int32_t *lam_index, const uint64_t *seeds,
                    const uint32_t *streams, const double *a, const double *b,
                    const double *dbdl, const double *xref, int64_t nsteps,
                    int32_t nthreads, double *x, double *p, or_ring_result *res) {
    batch_job J;
    J.pes = pes;
    J.mass = mass;
    J.prm = prm;
    J.lam_index = lam_index;
    J.seeds = seeds;
    J.streams = streams;
    J.a = a;
    J.b = b;
    J.dbdl = dbdl;
    J.xref = xref;
    J.nsteps = nsteps;
    J.nrings = nrings;
    J.nd = (int64_t)pes->ndim * pes->natom;
    J.x = x;
    J.p = p;
    J.res = res;
    J.next = 0;
    pthread_mutex_init(&J.lock, NULL);
    if (nthreads < 1) nthreads = 1;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
    for (int i = 0; i < nthreads; i++) pthread_create(&th[i], NULL, batch_worker, &J);
    for (int i = 0; i < nthreads; i++) pthread_join(th[i], NULL);
    free(th);
    pthread_mutex_destroy(&J.lock);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Instanton                                                                 */
/* ------------------------------------------------------------------------- */

/* instantonmod.f90:17-46 (UM).  x[dof*N + bead]. */
double or_UM(const or_pes *pes, const double *mass, int64_t N, double betan, const double *x,
             const double *a, const double *b, int fixedends) {
    int64_t nd = (int64_t)pes->ndim * pes->natom;
    double *xb = (double *)malloc(sizeof(double) * nd);
    double um = 0.0;
    for (int64_t i = 0; i < N - 1; i++) {
        for (int64_t d = 0; d < nd; d++) xb[d] = x[d * N + i];
        um = um + or_V(pes, xb);
        for (int64_t j = 0; j < pes->ndim; j++)
            for (int64_t k = 0; k < pes->natom; k++) {
                int64_t d = k * pes->ndim + j;
                double dx = x[d * N + i + 1] - x[d * N + i];
                um = um + (0.5 * mass[k] / (betan * betan)) * dx * dx;
            }
    }
    for (int64_t d = 0; d < nd; d++) xb[d] = x[d * N + N - 1];
    um = um + or_V(pes, xb);
    if (fixedends) {
        for (int64_t j = 0; j < pes->ndim; j++)
            for (int64_t k = 0; k < pes->natom; k++) {
                int64_t d = k * pes->ndim + j;
                double d1 = x[d * N] - a[d], d2 = b[d] - x[d * N + N - 1];
                um = um + (0.5 * mass[k] / (betan * betan)) * d1 * d1;
                um = um + (0.5 * mass[k] / (betan * betan)) * d2 * d2;
            }
    }
    free(xb);
    return um;
}

/* instantonmod.f90:50-89 (UMprime). */
void or_UMprime(const or_pes *pes, const double *mass, int64_t N, double betan,
                const double *x, const double *a, const double *b, int fixedends,
                double *grad) {
    int64_t nd = (int64_t)pes->ndim * pes->natom;
    double *xb = (double *)malloc(sizeof(double) * nd);
    double *g = (double *)malloc(sizeof(double) * nd);
    double bb = betan * betan;
    for (int64_t i = 0; i < N; i++) {
        for (int64_t j = 0; j < pes->ndim; j++)
            for (int64_t k = 0; k < pes->natom; k++) {
                int64_t d = k * pes->ndim + j;
                const double *xd = x + d * N;
                double v;
                if (i == 0) {
                    v = fixedends ? mass[k] * (2.0 * xd[0] - a[d] - xd[1]) / bb
                                  : mass[k] * (xd[0] - xd[1]) / bb;
                } else if (i == N - 1) {
                    v = fixedends ? mass[k] * (2.0 * xd[N - 1] - xd[N - 2] - b[d]) / bb
                                  : mass[k] * (xd[N - 1] - xd[N - 2]) / bb;
                } else {
                    v = mass[k] * (2.0 * xd[i] - xd[i - 1] - xd[i + 1]) / bb;
                }
                grad[d * N + i] = v;
            }
        for (int64_t d = 0; d < nd; d++) xb[d] = x[d * N + i];
        or_Vprime(pes, xb, g);
        for (int64_t d = 0; d < nd; d++) grad[d * N + i] = grad[d * N + i] + g[d];
    }
    free(xb);
    free(g);
}

/* instantonmod.f90:93-151 (UMforceenergy). */
double or_UMforceenergy(const or_pes *pes, const double *mass, int64_t N, double betan,
                        const double *x, const double *a, const double *b, int fixedends,
                        double *grad) {
    or_UMprime(pes, mass, N, betan, x, a, b, fixedends, grad);
    return or_UM(pes, mass, N, betan, x, a, b, fixedends);
}

/* instantonmod.f90:155-217 (UMhessian), LAPACK lower band storage:
 * band[(1 + r - c) - 1 + (nd+1)*c] = A(r, c) for c <= r <= c + nd (0-based r, c). */
void or_UMhessian(const or_pes *pes, const double *mass, int64_t N, double betan,
                  const double *x, int singlewell, int quirks, double *band) {
    int64_t nd = (int64_t)pes->ndim * pes->natom;
    int64_t ld = nd + 1;
    int64_t tot = N * nd;
    memset(band, 0, sizeof(double) * ld * tot);
    double *hess = (double *)calloc(nd * nd, sizeof(double));
    double *xb = (double *)malloc(sizeof(double) * nd);
    double bb = betan * betan;
    for (int64_t i = 0; i < N; i++) {
        if ((i == 0 && singlewell) || !singlewell) {
            for (int64_t d = 0; d < nd; d++) xb[d] = x[d * N + i];
            or_Vdoubleprime(pes, xb, hess, quirks);
        }
        for (int64_t j1 = 0; j1 < pes->ndim; j1++)
            for (int64_t k1 = 0; k1 < pes->natom; k1++)
                for (int64_t j2 = 0; j2 < pes->ndim; j2++)
                    for (int64_t k2 = 0; k2 < pes->natom; k2++) {
                        int64_t id1 = k1 * pes->ndim + j1, id2 = k2 * pes->ndim + j2;
                        int64_t f1 = nd * i + id1, f2 = nd * i + id2;
                        if (f2 < f1) continue;
                        /* hess(j2,k2,j1,k1) = hess[id2 + nd*id1] */
                        double h = hess[id2 + nd * id1] / sqrt(mass[k1] * mass[k2]);
                        if (id1 == id2) {
                            band[0 + ld * f1] = 2.0 / bb + h;
                            int coupled = quirks ? (i > 0) : (i < N - 1);
                            if (coupled && f1 + nd < tot) band[nd + ld * f1] = -1.0 / bb;
                        } else {
                            band[(f2 - f1) + ld * f1] = h;
                        }
                    }
    }
    free(hess);
    free(xb);
}

/* ------------------------------------------------------------------------- */
/* Quadrature and splines                                                    */
/* ------------------------------------------------------------------------- */

/* verletmodule.f90:124-160 (gauleg). */
void or_gauleg(double x1, double x2, double *x, double *w, int64_t n) {
    const double EPS = 3.0e-14;
    int64_t m = (n + 1) / 2;
    double xm = 0.5 * (x2 + x1), xl = 0.5 * (x2 - x1);
    for (int64_t i = 1; i <= m; i++) {
        double z = cos(OR_PI_REF * ((double)i - 0.25) / ((double)n + 0.5));
        double z1, pp, p1, p2, p3;
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
        } while (fabs(z - z1) > EPS);
        x[i - 1] = xm - xl * z;
        x[n - i] = xm + xl * z;
        w[i - 1] = 2.0 * xl / ((1.0 - z * z) * pp * pp);
        w[n - i] = w[i - 1];
    }
}

/* instantonmod.f90:446-480 (tridag), 0-based: a[1..n-1], b[0..n-1], c[0..n-2]. */
static void tridag(const double *a, const double *b, const double *c, const double *r,
                   double *u, int64_t n) {
    double *gam = (double *)malloc(sizeof(double) * n);
    double bet = b[0];
    u[0] = r[0] / bet;
    for (int64_t j = 1; j < n; j++) {
        gam[j] = c[j - 1] / bet;
        bet = b[j] - a[j] * gam[j];
        u[j] = (r[j] - a[j] * u[j - 1]) / bet;
    }
    for (int64_t j = n - 2; j >= 0; j--) u[j] = u[j] - gam[j + 1] * u[j + 1];
    free(gam);
}

/* instantonmod.f90:397-442 (spline). */
void or_spline(const double *x, const double *y, int64_t n, double yp1, double ypn, double *y2) {
    double *a = (double *)calloc(n, sizeof(double));
    double *b = (double *)calloc(n, sizeof(double));
    double *c = (double *)calloc(n, sizeof(double));
    double *r = (double *)calloc(n, sizeof(double));
    for (int64_t i = 0; i < n - 1; i++) c[i] = x[i + 1] - x[i];
    for (int64_t i = 0; i < n - 1; i++) r[i] = 6.0 * ((y[i + 1] - y[i]) / c[i]);
    /* r(2:n-1) = r(2:n-1) - r(1:n-2): array semantics, right side read first */
    double *rold = (double *)malloc(sizeof(double) * n);
    memcpy(rold, r, sizeof(double) * n);
    for (int64_t i = 1; i < n - 1; i++) r[i] = rold[i] - rold[i - 1];
    free(rold);
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
    tridag(a, b, c, r, y2, n);
    free(a);
    free(b);
    free(c);
    free(r);
}

/* instantonmod.f90:565-603 (locate), returns the 1-based NR index. */
int64_t or_locate(const double *xx, int64_t n, double x) {
    int ascnd = xx[n - 1] >= xx[0];
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

/* instantonmod.f90:499-528 (splint). */
double or_splint(const double *xa, const double *ya, const double *y2a, int64_t n, double x) {
    int64_t klo = or_locate(xa, n, x);
    if (klo > n - 1) klo = n - 1;
    if (klo < 1) klo = 1;
    int64_t khi = klo + 1;
    double h = xa[khi - 1] - xa[klo - 1];
    double a = (xa[khi - 1] - x) / h;
    double b = (x - xa[klo - 1]) / h;
    return a * ya[klo - 1] + b * ya[khi - 1] +
           ((a * a * a - a) * y2a[klo - 1] + (b * b * b - b) * y2a[khi - 1]) * (h * h) / 6.0;
}

/* instantonmod.f90:532-561 (splin_grad). */
double or_splin_grad(const double *xa, const double *ya, const double *y2a, int64_t n, double x) {
    int64_t klo = or_locate(xa, n, x);
    if (klo > n - 1) klo = n - 1;
    if (klo < 1) klo = 1;
    int64_t khi = klo + 1;
    double h = xa[khi - 1] - xa[klo - 1];
    double a = (xa[khi - 1] - x) / h;
    double b = (x - xa[klo - 1]) / h;
    return ((ya[khi - 1] - ya[klo - 1]) / h) +
           ((1.0 - 3.0 * a * a) * y2a[klo - 1] + (3.0 * b * b - 1.0) * y2a[khi - 1]) * h / 6.0;
}

/* pimd_par.f90:399-424. */
void or_ti_assemble(int64_t nintegral, int64_t nrep, const double *weights,
                    const double *integrands, double betan, double *dA, double *sigmaA,
                    double *qratio) {
    double answer = 0.0, sA = 0.0;
    for (int64_t i = 0; i < nintegral; i++) {
        double f = 0.0, s = 0.0;
        for (int64_t j = 0; j < nrep; j++) {
            double v = integrands[nrep * i + j];
            f += v;
            s += v * v;
        }
        f = f / (double)nrep;
        s = s / (double)nrep;
        s = s - f * f;
        if (f == f) answer = answer + weights[i] * f;
        sA = sA + s * weights[i] * weights[i];
    }
    *dA = answer;
    *sigmaA = sA;
    *qratio = exp(-answer * betan);
}
