/*
 * oracle.h -- CPU FP64 restatement of the reference ring-polymer algorithms.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (the pimdgpu library, its
 * host drivers) links, loads or calls this code.  Only tests/, the smoke()
 * entry point and the cpu_baseline / reference legs of bench.py use it, and
 * only as the parity reference or as the timed CPU baseline.
 *
 * PARITY UNPINNED: the reference (Fortran + MKL + MPI) cannot be compiled on
 * this machine or on the GPU host (no Fortran compiler, no MKL, no MPI), and
 * the reference ships no golden vectors, fixtures or tests.  The restatement
 * is pinned instead to analytic known answers (harmonic fixed-end polymer,
 * DST-I orthogonality, Gauss-Legendre exactness, equipartition, NVE energy
 * conservation, finite-difference derivatives) and to Philox known-answer
 * vectors; see tests/test_oracle_*.py.
 *
 * Conventions (follow the reference, verletmodule.f90 / instantonmod.f90):
 *   - one configuration x(ndim,natom) is stored as x[dof], dof = atom*ndim+dim
 *     (Fortran column-major order of x(ndim,natom));
 *   - one ring polymer x(P,ndim,natom) is stored as x[dof*P + bead]
 *     (Fortran column-major order of x(n,ndim,natom): bead index fastest);
 *   - all arithmetic is double precision (the reference builds with -r8);
 *   - pi is the reference's truncated constant 3.14159265358979
 *     (instantonmod.f90:4, mcmod_2dtest.f90:14).
 */
#ifndef PIMD_ORACLE_H
#define PIMD_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OR_PI_REF 3.14159265358979

/* PES identifiers (same numbering as the product library). */
enum { OR_PES_1D = 1, OR_PES_2DTEST = 2, OR_PES_SYNTH9 = 3, OR_PES_SYNTH18 = 4,
       OR_PES_HARMONIC = 5, OR_PES_DISTGAUSS = 6 };

typedef struct or_pes {
    int32_t id;
    int32_t ndim, natom;
    int32_t nparams;
    double V0;
    const double *params; /* layout per PES, documented in oracle.c */
} or_pes;

/* ---- PES (mcmod_*: V, Vprime, Vdoubleprime) ---- */
double or_V(const or_pes *pes, const double *x);
void or_Vprime(const or_pes *pes, const double *x, double *grad);
double or_potforce(const or_pes *pes, const double *x, double *grad);
/* hess[a + ndof*b] = d grad_b / d x_a (reference hess(i,j,k,l) memory order).
 * quirks != 0 reproduces the reference Hessian of mcmod_2dtest exactly. */
void or_Vdoubleprime(const or_pes *pes, const double *x, double *hess, int quirks);

/* ---- RNG: Philox4x32-10 and the normal / uniform streams ---- */
void or_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* n-th standard normal of stream (seed, stream, step, purpose) */
double or_normal(uint64_t seed, uint32_t stream, uint32_t step, uint32_t purpose, uint32_t n);
double or_uniform(uint64_t seed, uint32_t stream, uint32_t step, uint32_t purpose, uint32_t n);
int64_t or_poisson(uint64_t seed, uint32_t stream, uint32_t step, uint32_t purpose, double mean);

/* ---- normal modes: init_nm, nmtransform_* ---- */
void or_init_nm(int64_t P, int64_t ndim, int64_t natom, const double *mass, double betan,
                double tau, const double *a, const double *b, double *T, double *lam,
                double *beadmass, double *beadvec);
void or_nm_forward(int64_t P, const double *T, const double *x, double *q,
                   const double *shift /* nullable, length P */);
void or_nm_backward(int64_t P, const double *T, const double *q, double *x,
                    const double *shift /* nullable */);

/* ---- TI propagation ---- */
typedef struct or_ti_params {
    int64_t P;
    double beta, betan, dt, tau, gamma;
    int32_t thermostat;  /* 1 Andersen, 2 Langevin */
    int32_t cayley;
    int32_t nm_resident; /* 0: reference 10-transform step; 1: NM-resident 2-transform step */
    int32_t pad;
    int64_t imin, noutput;
    double dhdr_limit;
    double init_sigma;   /* noise added to xref at (re)initialisation */
} or_ti_params;

typedef struct or_ring_result {
    double dhdr_sum;     /* sum of accepted estimator contributions */
    int64_t nsamples;    /* steps past imin (the reference's averaging count) */
    int64_t nreinit;     /* dHdrlimit re-initialisations */
    int64_t and_count;   /* Andersen: steps since the last momentum resampling */
    int64_t and_rkick;   /* Andersen: current Poisson interval, < 0 = not drawn yet */
    int32_t status;      /* 0 ok, 1 NaN seen */
    int32_t pad;
} or_ring_result;

/* Build the starting state of one ring: x = xref + sigma*N(0,1) (purpose 2),
 * p = T * (sqrt(beadmass/betan) * N(0,1)) (purpose 1), verletmodule.f90:102-115. */
void or_ring_init(const or_pes *pes, const double *mass, const or_ti_params *prm,
                  const double *T, const double *beadmass, const double *xref,
                  uint64_t seed, uint32_t stream, uint32_t step, uint32_t purpose_x,
                  uint32_t purpose_p, double *x, double *p);

/* Advance one ring by nsteps starting at global step step0 (0-based).
 * x, p (Cartesian, [dof*P+bead]) are in/out. */
void or_ring_propagate(const or_pes *pes, const double *mass, const or_ti_params *prm,
                       const double *a, const double *b, const double *dbdl,
                       const double *xref, uint64_t seed, uint32_t stream,
                       int64_t step0, int64_t nsteps, double *x, double *p,
                       or_ring_result *res);

/* Batched CPU run over many rings with nthreads worker threads (the timed CPU
 * baseline).  Ring r uses lam_index[r] to pick b/dbdl/xref rows. */
int or_ti_run_batch(const or_pes *pes, const double *mass, const or_ti_params *prm,
                    int64_t nrings, const int32_t *lam_index, const uint64_t *seeds,
                    const uint32_t *streams, const double *a, const double *b,
                    const double *dbdl, const double *xref, int64_t nsteps,
                    int32_t nthreads, double *x, double *p, or_ring_result *res);

/* ---- instanton: UM / UMprime / UMforceenergy / UMhessian ---- */
double or_UM(const or_pes *pes, const double *mass, int64_t N, double betan, const double *x,
             const double *a, const double *b, int fixedends);
void or_UMprime(const or_pes *pes, const double *mass, int64_t N, double betan,
                const double *x, const double *a, const double *b, int fixedends,
                double *grad);
double or_UMforceenergy(const or_pes *pes, const double *mass, int64_t N, double betan,
                        const double *x, const double *a, const double *b, int fixedends,
                        double *grad);
/* Lower band storage (ndof+1) x (N*ndof), column-major: band[r + (ndof+1)*c]. */
void or_UMhessian(const or_pes *pes, const double *mass, int64_t N, double betan,
                  const double *x, int singlewell, int quirks, double *band);

/* ---- TI quadrature and path utilities ---- */
void or_gauleg(double x1, double x2, double *x, double *w, int64_t n);
void or_spline(const double *x, const double *y, int64_t n, double yp1, double ypn, double *y2);
double or_splint(const double *xa, const double *ya, const double *y2a, int64_t n, double x);
double or_splin_grad(const double *xa, const double *ya, const double *y2a, int64_t n, double x);
int64_t or_locate(const double *xx, int64_t n, double x);

/* pimd_par.f90:399-424 assembly. integrands[nintegral*nrep] ordered (point, rep). */
void or_ti_assemble(int64_t nintegral, int64_t nrep, const double *weights,
                    const double *integrands, double betan, double *dA, double *sigmaA,
                    double *qratio);

#ifdef __cplusplus
}
#endif
#endif
