/*
 * pimdgpu.h -- C-ABI of the GB300 (sm_103a) ring-polymer library.
 *
 * Drop-in boundary for the ring-polymer hot path of pimd-tunneling: the PES
 * module interface (mcmod_*.f90), the TI-PIMD propagation (verletmodule.f90),
 * the ring-polymer-instanton action / gradient / Hessian and optimiser
 * (instantonmod.f90) and the driver-level assembly (pimd_par.f90, rpi_ser.f90).
 * Each entry point cites the reference routine it replaces.
 *
 * Conventions
 *   - Every function returns PG_OK (0) or a PG_ERR_* code; pg_last_error()
 *     returns the message of the last failure on the calling thread.
 *   - Integers that the reference declares as default INTEGER are int64_t
 *     (the reference builds with -i8); reals are double (-r8).
 *   - One configuration x(ndim,natom) is x[dof], dof = atom*ndim + dim.
 *     One ring x(P,ndim,natom) is x[dof*P + bead] (Fortran column-major, bead
 *     fastest).  Batches of rings are ring-major: x[(ring*ndof + dof)*P + bead].
 *   - Caller owns all host arrays.  The context owns its device memory and its
 *     CUDA stream; calls are synchronous at return.  One host thread per context.
 *   - There is no CPU fallback: a context cannot be created without a GPU.
 */
#ifndef PIMDGPU_H
#define PIMDGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PG_OK 0
#define PG_ERR_ARG 1        /* invalid argument or size */
#define PG_ERR_CUDA 2       /* CUDA runtime failure */
#define PG_ERR_STATE 3      /* call out of order (e.g. advance before setup) */
#define PG_ERR_UNSUPPORTED 4
#define PG_ERR_IO 5
#define PG_ERR_NUMERIC 6    /* NaN / non-convergence reported by a kernel */

/* PES identifiers (the mcmod_* module selected at build time in the reference). */
#define PG_PES_1D 1        /* mcmod_1d.f90: quartic double well per coordinate */
#define PG_PES_2DTEST 2    /* mcmod_2dtest.f90: 2-D ring of six Gaussian wells */
#define PG_PES_SYNTH9 3    /* 9-atom Morse network + quartic proton-transfer well */
#define PG_PES_SYNTH18 4   /* 18-atom flexible water hexamer (harmonic + LJ + charges) */
#define PG_PES_HARMONIC 5  /* V = k/2 |x|^2, analytic test surface */
#define PG_PES_DISTGAUSS 6 /* Morse + 1/2/3-D Gaussians in interatomic distances, tables as parameters:
                              the form of pes_malonaldehyde.f90 (layout in pg_device.cuh) */

/* Precision of the TI propagation. */
#define PG_FP64 0          /* FP64 everywhere */
#define PG_MIXED 1         /* FP32 forces/state, split-BF16 tensor-core NM transform
                              where available, FP64 estimator accumulation */

/* Execution form of the TI propagation. */
#define PG_FORM_AUTO 0     /* fused persistent kernel; tensor-core variant when supported */
#define PG_FORM_PLAIN 1    /* per-step kernel launches in the reference step order
                              (10 NM transforms per Langevin step), FP64 only */
#define PG_FORM_FUSED 2    /* fused persistent SIMT kernel (FP64 or FP32) */
#define PG_FORM_TENSOR 3   /* tcgen05 forms (PG_MIXED only): the persistent step kernel for
                              P = 128 on the 1-D and 2-D surfaces, the persistent folded
                              step for P = 256 on the 9-atom surface (Langevin without
                              dHdrlimit), otherwise three blocked-GEMM kernels per step */

#define PG_ANDERSEN 1
#define PG_LANGEVIN 2

/* Ring status bits (pg_ti_get_results). */
#define PG_RING_NAN 1
#define PG_RING_TIMEOUT 2

typedef struct pg_ctx pg_ctx;

/* ---------------------------------------------------------------- context */
int pg_create(pg_ctx **ctx, int32_t device);
int pg_destroy(pg_ctx *ctx);
const char *pg_last_error(void);
int32_t pg_version(void);

/* Module state of mcmod_mass: V_init + n/ndim/natom/mass/V0
 * (mcmod_waterdimer.f90:1-17, pimd_par.f90:113-117,152-166). */
int pg_set_system(pg_ctx *ctx, int64_t ndim, int64_t natom, const double *mass,
                  int32_t pes_id, const double *params, int64_t nparams, double V0);

/* ---------------------------------------------------------------- PES */
/* Batched V / Vprime / potforce (mcmod_1d.f90:14-35, mcmod_2dtest.f90:29-61,
 * mcmod_waterdimer.f90:60-81).  x[nconf*ndof]; V[nconf] and grad[nconf*ndof]
 * may each be NULL.  precision: PG_FP64 or PG_MIXED (FP32 evaluation). */
int pg_pes_eval(pg_ctx *ctx, int64_t nconf, const double *x, double *V, double *grad,
                int32_t precision);
/* Batched Vdoubleprime (mcmod_1d.f90:38-58, mcmod_2dtest.f90:64-102):
 * hess[c*ndof*ndof + a + ndof*b] = d grad_b / d x_a.  quirks=1 reproduces the
 * reference's mcmod_2dtest Hessian exactly (only the last well, its chain rule). */
int pg_pes_hessian(pg_ctx *ctx, int64_t nconf, const double *x, double *hess, int32_t quirks);

/* ---------------------------------------------------------------- normal modes */
/* Batched fixed-end normal-mode transform out = T in, T_il = sqrt(2/(P+1))
 * sin(pi i l/(P+1)) (init_nm / nmtransform_forward, verletmodule.f90:254-266,
 * 306-338); T is symmetric and its own inverse, so this is also the backward
 * transform.  in/out[ncol*P], column-major.  precision PG_MIXED runs the
 * split-BF16 tcgen05 transform (P = 128) or FP32. */
int pg_nm_transform(pg_ctx *ctx, int64_t P, int64_t ncol, const double *in, double *out,
                    int32_t precision);

/* Measurement helper (no counterpart in the reference): the FP32 FMA
 * throughput of the context's GPU in TFLOP/s (best of three timed launches of
 * scalar and packed f32x2 FMA chains), the peak of the SIMT term of the
 * roofline. */
int pg_fp32_peak(pg_ctx *ctx, double *tflops);
/* Failure detection: deadline, in ns from the kernel's start, of the
 * device-side waits (for the bulk copy of T and for the GEMM) of the
 * tensor-core transform of pg_nm_transform (PG_MIXED, P = 128); default 2e9
 * (2 s); 0 makes the first wait give up.  A wait that runs out makes the call
 * return PG_ERR_NUMERIC; the kernel first lets the copy or GEMM it waited for
 * finish (bounded by 2 s), so the context stays usable.  No counterpart in
 * the reference, which has no device waits (it stops on a NaN,
 * verletmodule.f90:533-536). */
int pg_set_wait_limit(pg_ctx *ctx, int64_t ns);
/* Allocation-free variant of the split-BF16 tcgen05 transform (pg_nm_transform
 * with PG_MIXED, P = 128).  No counterpart in the reference.  It is for callers
 * that cannot call cudaMalloc: a Fortran / MPI host program that gives all of
 * the GPU's memory to its own pool allocator at start-up, or code in a section
 * where cudaMalloc's implicit device synchronisation is not allowed.  d_in /
 * d_out are caller-owned device buffers of ncol*128 doubles; stream is a
 * cudaStream_t (NULL = default stream); synchronous at return.  The only
 * scratch is a static 64 KB device array (the split image of T plus an error
 * word) that every GPU loading the library holds until exit; P must be 128
 * (anything else is PG_ERR_ARG).  The first call on a device builds the image
 * there; make that first call before any stream capture.  All calls share the
 * array: calls that overlap on the GPU race.  Allocates no device or pinned
 * memory. */
int pg_nm_transform_noalloc(int64_t P, int64_t ncol, const double *d_in, double *d_out, void *stream);

/* ---------------------------------------------------------------- TI-PIMD */
typedef struct pg_ti_config {
    int64_t nbeads;      /* P (namelist n) */
    double beta;         /* namelist beta; the ring uses betan = beta/(P+1) (pimd_par.f90:94) */
    double dt;           /* namelist dt */
    double tau;          /* namelist tau: NM mass scaling, all mode periods = 2 pi tau */
    double gamma;        /* namelist gamma: c1 = exp(-gamma dt / tau) (verletmodule.f90:383) */
    int32_t thermostat;  /* PG_ANDERSEN or PG_LANGEVIN (namelist thermostat) */
    int32_t precision;   /* PG_FP64 or PG_MIXED */
    int32_t form;        /* PG_FORM_* */
    int32_t cayley;      /* namelist cayley */
    int64_t imin;        /* namelist imin: estimator starts after imin steps */
    int64_t noutput;     /* namelist Noutput: Andersen Poisson mean */
    double dhdr_limit;   /* namelist dHdrlimit; < 0 disables */
    double init_sigma;   /* Gaussian noise added to xref at (re)initialisation */
} pg_ti_config;

/* Set up a batch of rings (the task loop of pimd_par.f90:321-381, batched).
 * Ring r uses endpoint row ring_lambda[r] of b/dbdl/xref, RNG key ring_seed[r]
 * and stream id ring_stream[r].  a[ndof] is the fixed start point, b[nlambda*ndof]
 * the ξ-dependent end points, dbdl[nlambda*ndof] their ξ-derivatives.
 * Initial positions: x0 (nrings*ndof*P) if given, else xref[lambda] (nlambda*ndof*P)
 * plus init_sigma N(0,1).  Initial momenta: p0 if given, else normal-mode Maxwell
 * momenta (verletmodule.f90:102-115). */
int pg_ti_setup(pg_ctx *ctx, const pg_ti_config *cfg, int64_t nrings, int64_t nlambda,
                const int32_t *ring_lambda, const uint64_t *ring_seed,
                const uint32_t *ring_stream, const double *a, const double *b,
                const double *dbdl, const double *xref, const double *x0, const double *p0);
/* Advance every ring by nsteps MD steps (the hot loop of propagate_pimd_pile /
 * propagate_pimd_nm, verletmodule.f90:389-411 / 203-245).  Replays a captured
 * CUDA graph when the same nsteps is requested again. */
int pg_ti_advance(pg_ctx *ctx, int64_t nsteps);
/* pg_ti_advance that also returns the device time of the launched work in
 * milliseconds, measured with CUDA events recorded on the context's stream. */
int pg_ti_advance_timed(pg_ctx *ctx, int64_t nsteps, double *device_ms);

/* Advances the TI batches of nctx contexts on one device by nsteps each: the
 * mixed-P task list of pimd_par.f90:245-381 (one context per bead number P) as
 * one call.  The step kernels of every context are captured into one CUDA
 * graph (a concurrent branch per context, forked from and joined to the first
 * context's stream) and the whole advance is a single graph launch; batches in
 * the plain form run on their own streams instead.  device_ms (may be NULL) is
 * the device time from the launch to the last completion.  No counterpart in
 * the reference (its ranks run one task at a time). */
int pg_ti_advance_group(pg_ctx *const *ctxs, int64_t nctx, int64_t nsteps, double *device_ms);
/* Advance nsteps with one CUDA-event pair around every kernel launch (no graph)
 * and report, for up to 4 kernel kinds of the chosen form, the mean device time
 * per launch (ms_per_launch[k]), the launches (count[k]), and the algorithmic
 * HBM bytes one launch moves (bytes_per_launch[k]); names[k] points to the
 * kernel's name (valid until the next call on the same thread).  Returns the
 * number of kinds in *nkinds. */
int pg_ti_kernel_times(pg_ctx *ctx, int64_t nsteps, int32_t *nkinds, double *ms_per_launch,
                       int64_t *count, double *bytes_per_launch, const char **names);
/* Cartesian positions and momenta of every ring (nrings*ndof*P each; either may be NULL). */
int pg_ti_get_state(pg_ctx *ctx, double *x, double *p);
/* Per-ring estimator sums: dhdr_sum[r] = sum of accepted contributions,
 * nsamples[r] = steps past imin (the divisor of verletmodule.f90:413),
 * nreinit[r] = dHdrlimit re-initialisations, status[r] = PG_RING_* bits.
 * Any pointer may be NULL. */
int pg_ti_get_results(pg_ctx *ctx, double *dhdr_sum, int64_t *nsamples, int64_t *nreinit,
                      int32_t *status);
/* Restores the per-ring estimator sums and sample counts and the batch step
 * counter (the Philox streams continue from it): the continuation of
 * propagate_pimd_pile after its restart file is read (verletmodule.f90:388, 413;
 * pimd_par.f90:356-369), for state set by pg_ti_setup(x0, p0) from that file.
 * The status, re-initialisation and Andersen counters are left as they are. */
int pg_ti_set_accumulators(pg_ctx *ctx, const double *dhdr_sum, const int64_t *nsamples, int64_t step);
/* Per-lambda reduction of integrand = dHdr/betan^2 over the rings of each lambda
 * (pimd_par.f90:379, 401-409), on the device: mean[nlambda], var[nlambda]
 * (E[I^2]-E[I]^2), count[nlambda].  Rings flagged PG_RING_NAN and rings with
 * no sample yet are left out; count is the number of rings used. */
int pg_ti_lambda_reduce(pg_ctx *ctx, double *mean, double *var, int64_t *count);
/* Global step counter of the batch (steps already taken). */
int pg_ti_get_step(pg_ctx *ctx, int64_t *step);
/* Execution form chosen for the batch (PG_FORM_PLAIN / _FUSED / _TENSOR) and the
 * number of kernel launches one pg_ti_advance(nsteps) issues. */
int pg_ti_get_form(pg_ctx *ctx, int64_t nsteps, int32_t *form, int64_t *launches);

/* Autotuning of batches set up with form PG_FORM_AUTO (a project addition; the
 * reference has no launch parameters).  mode PG_TUNE_CACHE: pg_ti_setup takes the
 * form and the SIMT threads per ring recorded for the batch's key (device, P,
 * dofs, surface, precision, thermostat, batch-size bucket) in the JSON-lines file
 * cache_path, else its built-in choice; PG_TUNE_ON: a key not in the file is
 * tuned on the batch (each candidate set up and advanced for a short timed
 * probe), the fastest is appended to the file, and the batch is set up again
 * with it.  PG_TUNE_OFF (the default) disables both. */
#define PG_TUNE_OFF 0
#define PG_TUNE_CACHE 1
#define PG_TUNE_ON 2
int pg_set_tuning(pg_ctx *ctx, const char *cache_path, int32_t mode);
/* Launch parameters of the current batch: form, SIMT threads per ring and MD
 * steps per tensor-step launch (0: built-in choice).  Any pointer may be NULL. */
int pg_ti_get_tuning(pg_ctx *ctx, int32_t *form, int32_t *simt_threads, int32_t *tc_steps);
/* Bitwise checkpoint of the whole batch state (positions, momenta, estimator
 * accumulators, RNG step counters); replaces write_restart / restart=2
 * (verletmodule.f90:162-185, pimd_par.f90:331-370). */
int pg_ti_checkpoint_save(pg_ctx *ctx, const char *path);
int pg_ti_checkpoint_load(pg_ctx *ctx, const char *path);
int pg_ti_release(pg_ctx *ctx);

/* Drop-in for a batch of propagate_pimd_pile / propagate_pimd_nm calls
 * (verletmodule.f90:372-416 / 190-250): ntask rings with end points b[task],
 * dbdl[task]; x, p (ntask*ndof*P) in/out; dHdr[task] = averaged estimator
 * (divided by nmc - imin, verletmodule.f90:413). */
int pg_propagate_pimd(pg_ctx *ctx, const pg_ti_config *cfg, int64_t ntask, int64_t nmc,
                      const double *a, const double *b, const double *dbdl,
                      const uint64_t *seed, const uint32_t *stream, double *x, double *p,
                      double *dHdr, int32_t *status);

/* ---------------------------------------------------------------- TI host assembly */
/* gauleg (verletmodule.f90:124-160). */
int pg_gauleg(double x1, double x2, double *x, double *w, int64_t n);
/* Natural cubic spline second derivatives (instantonmod.f90:397-442). */
int pg_spline(const double *x, const double *y, int64_t n, double yp1, double ypn, double *y2);
/* splint / splin_grad (instantonmod.f90:499-561). */
int pg_splint(const double *xa, const double *ya, const double *y2a, int64_t n, double x,
              double *y, double *dydx);
/* Final TI assembly (pimd_par.f90:411-424): dA = sum w_i mean_i,
 * sigmaA = sum w_i^2 var_i, qratio = exp(-dA*betan). */
int pg_ti_assemble(int64_t nintegral, const double *weights, const double *mean,
                   const double *var, double betan, double *dA, double *sigmaA,
                   double *qratio);
/* Tunnelling splitting from the fixed-end ratio q/q0 = tanh(beta Delta/2)
 * (python_utils/multiwell_waterdimer.py:6-10). */
int pg_splitting_from_ratio(double beta, double qratio, double *delta);
/* Splitting from ratios at two inverse temperatures, which removes an offset
 * beta_bar in artanh(ratio) = Delta (beta - beta_bar) / 2
 * (python_utils/multiwell_waterdimer.py:6-16): with y_k = artanh(ratio_k),
 * Delta = 2 (y2 - y1) / (beta2 - beta1) and
 * beta_bar = (beta1 y2 - beta2 y1) / (y2 - y1).  betabar may be NULL; it is
 * NaN when y1 = y2. */
int pg_splitting_two_beta(double beta1, double ratio1, double beta2, double ratio2, double *delta,
                          double *betabar);
/* Ratio of one tunnelling level pair per irreducible representation of a
 * multi-well system (python_utils/multiwell_waterdimer.py:67-75): with
 * rho[g] the path ratio of operation g (rho of the identity = 1) and
 * chars[i*nop + g] the character of representation i,
 * ratio[i] = sum_g (1 - chars[i*nop+g]) rho[g] / sum_g (1 + chars[i*nop+g]) rho[g]. */
int pg_irrep_ratios(int64_t nirrep, int64_t nop, const double *chars, const double *rho, double *ratio);

/* ---------------------------------------------------------------- instanton */
typedef struct pg_lbfgs_opts {
    int32_t m;               /* history length (reference m = 8, instantonmod.f90:716) */
    int32_t max_backtracks;  /* line-search backtrack cap (reference maxiter = 40) */
    int64_t maxiter;         /* iteration cap */
    double factr;            /* relative decrease tolerance factr*eps (reference 1e6) */
    double pgtol;            /* gradient infinity-norm tolerance (reference eps2) */
    int32_t cluster_ctas;    /* CTAs (one thread-block cluster) per polymer: 1, 2, 4 or 8; 0 = as
                                many as the GPU holds for the batch (the sums then run in a
                                different order, so results differ at round-off) */
    int32_t reserved;        /* 0 */
} pg_lbfgs_opts;

/* Fixed or free end points of the polymer action (instantonmod's module
 * variable fixedends, instantonmod.f90:7; namelist key fixedends of
 * rpi_ser.f90:23 and pimd_par.f90:44).  1 (default): springs of m/(2 betan^2)
 * tie bead 1 to a and bead N to b.  0: no end springs, so an end bead feels only
 * its one neighbour (instantonmod.f90:35-44, 63-72, 115-124, 138-151); a and b
 * may then be NULL in pg_instanton_fg / pg_instanton_optimize.  Applies to those
 * two calls; the Hessian of pg_um_hessian / pg_instanton_logdet is the same
 * either way, as UMhessian is. */
int pg_set_fixedends(pg_ctx *ctx, int32_t fixedends);
/* Batched UMforceenergy over nbeta independent polymers (instantonmod.f90:17-151):
 * x[nbeta*ndof*N], UM[nbeta], grad[nbeta*ndof*N] (either may be NULL);
 * end points a[ndof], b[nbeta*ndof] (NULL allowed with free ends); betan[nbeta]. */
int pg_instanton_fg(pg_ctx *ctx, int64_t nbeta, int64_t N, const double *x, const double *a,
                    const double *b, const double *betan, double *UM, double *grad);
/* Batched instanton optimisation (instantonmod.f90:679-777) by an on-device FP64
 * L-BFGS driven by the adjoint gradient, each polymer on a thread-block cluster
 * of opts->cluster_ctas CTAs; x in/out; UM[nbeta], niter[nbeta], status[nbeta]
 * (0 converged, 1 iteration cap, 2 line-search failure). */
int pg_instanton_optimize(pg_ctx *ctx, int64_t nbeta, int64_t N, double *x, const double *a,
                          const double *b, const double *betan, const pg_lbfgs_opts *opts,
                          double *UM, int64_t *niter, int32_t *status);
/* UMhessian in LAPACK lower band storage (instantonmod.f90:155-217):
 * band[(ndof+1) * N*ndof], column-major.  quirks=1 reproduces the reference's
 * spring-coupling placement (no bead 1-2 coupling) and mcmod_2dtest Hessian. */
int pg_um_hessian(pg_ctx *ctx, int64_t N, double betan, const double *x, int32_t singlewell,
                  int32_t quirks, double *band);
/* detJ + the log-sum of rpi_ser.f90:222-237, 354-366 over nbeta polymers:
 * lndet[k] = sum over eigenvalues eta^2 > 0 of log eta^2 of the mass-weighted
 * Hessian, skipping the lowest eigenvalue when skip_lowest.  eta2_min[k] = lowest
 * eigenvalue, nskipped[k] = number of eigenvalues left out. */
int pg_instanton_logdet(pg_ctx *ctx, int64_t nbeta, int64_t N, const double *x,
                        const double *betan, int32_t singlewell, int32_t skip_lowest,
                        int32_t quirks, double *lndet, double *eta2_min, int64_t *nskipped);
/* RPI assembly (rpi_ser.f90:368-381): S = betan*UM, Gamma = exp((lndetJ-lndetJ0)/2),
 * omega = betan exp(-S) sqrt(S/2pi)/Gamma, delta = 2 omega/betan. */
int pg_rpi_assemble(double betan, double UM, double lndetJ, double lndetJ0, double *S,
                    double *omega, double *delta);

#ifdef __cplusplus
}
#endif
#endif
