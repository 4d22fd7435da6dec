/*
 * macaw_gb300.h -- C-ABI of the GB300-native G-MCTDH propagation core.
 *
 * The entry points replace the equation-of-motion and integrator calls of the
 * reference's time loop (Macaw, source/propagator.f90).  A Fortran driver binds
 * them with ISO_C_BINDING (interface blocks with bind(C)); every integer that crosses the
 * boundary is int64_t because the reference is built with -fdefault-integer-8
 * (Makefile:18), every complex is interleaved FP64 (double complex), every
 * array is column-major, and every index is 0-based (the Fortran shim subtracts 1).
 *
 * Calls are synchronous at return, one context owns one CUDA stream on the
 * current device, and a context is not thread-safe.  All functions return 0 on
 * success or a negative status:
 *   -1 unsupported feature   -2 eigensolver did not converge   -3 Krylov cap
 *   -4 step underflow        -5 non-finite state                -6 CUDA error
 *   -7 bad argument
 * There is no CPU fallback: without a usable GPU mctdh_create returns -6.
 */
#ifndef MACAW_GB300_H
#define MACAW_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mctdh_ctx mctdh_ctx_t;

/* Contents of the reference's global modules after set-up (psidef.f90,
 * hamilton.f90:17-62, dvr.f90:11-29, storage.f90, globals.f90:26-44).
 * Array element (i, j) of a Fortran array X(n1, n2) is X[i + n1*j]. */
typedef struct mctdh_setup {
  int64_t nstates, nmodes, ndof, nham, maxdof;
  const int64_t *nspf;          /* nSPF(nmodes, nstates)                         */
  const int64_t *nmodedof;      /* nmodeDOF(nmodes)                              */
  const int64_t *idof;          /* iDOF(maxdof, nmodes), 0-based dofs            */
  const int64_t *multiset;      /* MultiSet(nmodes), 0/1                         */
  const int64_t *is_gwp;        /* 1 if the mode uses Gaussian SPFs              */
  const int64_t *ngp;           /* ngp(ndof)                                     */
  const double *dvr_grid;       /* grid(:, dof) packed; offsets in dvr_grid_off  */
  const int64_t *dvr_grid_off;  /* (ndof), -1 for gwp dofs                       */
  const double *dvr_mats;       /* d1DVR, d2DVR, xd1DVR per dof, each ngp x ngp  */
  const int64_t *dvr_mat_off;   /* (ndof) offset of d1DVR; d2 at +ngp^2, xd1 at +2 ngp^2 */
  const double *ae;             /* ae(nham), interleaved complex                 */
  const int64_t *lhs_el;        /* lhs_el(nham), 0-based                         */
  const int64_t *rhs_el;        /* rhs_el(nham), 0-based                         */
  int64_t nopermax;
  const int64_t *noper;         /* nOper(nmodes)                                 */
  const int64_t *oper;          /* Oper(-1:maxdof, nopermax, nmodes) as [(2+maxdof) x nopermax x nmodes] */
  const int64_t *ioper;         /* iOper(nmodes, nham), 0-based                  */
  const int64_t *is_identity;   /* IsIdentity(nmodes, nopermax)                  */
  const int64_t *skip_term;     /* SkipTerm(nmodes, nham)                        */
  const int64_t *ipsispf;       /* ipsiSPF(nmodes, nstates), 0-based offsets     */
  int64_t dimpsi;
  const double *gwpa;           /* GWPa(maxdof, ns00max, nmodgwp)                */
  int64_t ns00max;
  double eps_rho, eps_ovl, eps_C, eps_int, eps_A, eps_psi;
  double min_stepsize, writetime;
  double der_factor_re, der_factor_im;  /* -i for propagation, -1 for relaxation */
  int64_t int_type_psi;                 /* 1 = Cash-Karp for the CMF2 SPF sweeps  */
  int64_t precision;                    /* 0 FP64; 1 FP32 products, compensated contractions;
                                           2 compensated products and contractions; 3 FP32 products
                                           and contractions; 4 as 1 with compensated H_B products of the
                                           Lanczos steps; 5 as 2 with FP32 H_B products; 6 as 1 with
                                           FP32-summed mean-field contractions (densities compensated) */
  int64_t int_order, int_par1;          /* Adams PECE order and extra EC iterations (abm<order><par1>) */
  /* Operators whose expectation values are written (the 'expect' keyword,
   * input.f90:196-216, terms read by Read_Operators, input.f90:516-748).  Their
   * mode operators are entries of oper after the Hamiltonian's (hamilton.f90:139-161). */
  int64_t nexpect;
  const int64_t *expect_nterms;  /* nOpTerms(nexpect)                                    */
  const double *expect_ae;       /* aeExtra, the terms of all operators concatenated, complex */
  const int64_t *expect_lhs;     /* lhs_elExtra, 0-based, concatenated                   */
  const int64_t *expect_rhs;     /* rhs_elExtra                                          */
  const int64_t *expect_ioper;   /* iOperExtra(nmodes, total terms), 0-based             */
  /* Statistical mixtures and dissipation (input.f90:156, 216-229, 262, 596-616;
   * gmctdh_objects.f90:481-1141; derivatives.f90:70-83, 238-242).  Every coefficient
   * array that crosses the boundary holds the npackets packets one after the other
   * (APacketOffset(W) = W * nAConftot, init_calc.f90:50-53).  Dissipative terms
   * follow the Hamiltonian's terms in ae/lhs_el/rhs_el/ioper/skip_term (nham counts
   * them) with term_kind 1 for a term of a type-1 operator alpha V rho V^+ (ae =
   * aeExtra, term_diss1 = its operator, diss1_ae = aeD1 = alpha / 2) and 2 for a term
   * of a type-2 operator beta (W rho + rho W^+) (ae = i aeD2 aeExtra, aeD2 = beta).
   * term_kind NULL: every term is Hamiltonian.  Mixtures (up to 16 packets) and
   * dissipation (up to 4 type-1 operators; a type-1 term between two states needs
   * equal SPF counts in both) run with the derivative-based integrators; CMF2
   * returns -1 for them. */
  int64_t npackets;              /* npackets, 0 or 1 for a single wave packet            */
  double eps_pop;                /* eps_pop (0: the reference's default 1e-6)            */
  const int64_t *term_kind;      /* (nham) 0 Hamiltonian, 1 type-1, 2 type-2, or NULL    */
  const int64_t *term_diss1;     /* (nham) type-1 operator of a kind-1 term (0-based)    */
  int64_t ndiss1;                /* number of type-1 operators                           */
  const double *diss1_ae;        /* aeD1(ndiss1)                                         */
  /* Parametrised DOF operators (input.f90:950-1072; values built by alloc_h1mode,
   * hamilton.f90:210-290): an operator code 200 + j multiplies the grid by
   * gridOper(:, j, dof); a code -200 - j applies the projector v v^T with
   * v = gridOper(:, j, dof) (MultTensProj, hamilton.f90:632-661).  grid_oper
   * holds gridOper(ngpmax, nopparam, ndof) column-major (j 1-based in the codes,
   * 0-based in the array); NULL when nopparam is 0. */
  int64_t nopparam;
  int64_t ngpmax;
  const double *grid_oper;
  /* operDVR (the sin^-2 matrix of Legendre DVRs, dvr.f90:361-530) for code -4:
   * ngp x ngp column-major per dof at oper_dvr_off[dof] (-1 where absent);
   * both NULL when no dof uses it. */
  const double *oper_dvr;
  const int64_t *oper_dvr_off;
  /* 1: every regularised inverse of rho starts its Jacobi eigen-decomposition
   * from the identity.  0 (default): from the previous call's eigenvectors, the
   * same decomposition up to rounding in fewer sweeps; rounding then depends on
   * the call history (ensembles always start cold, so that each member repeats
   * the arithmetic of a context created with 1). */
  int64_t reginv_cold;
} mctdh_setup_t;

/* Build the device context: uploads the operators, plans the batched kernels
 * and allocates device mirrors of A and psi.  Replaces the allocation part of
 * init_calc.f90:1-226 (alloc_h1mode, alloc_MeanField, alloc_rho, alloc_AVec). */
int64_t mctdh_create(const mctdh_setup_t *setup, mctdh_ctx_t **ctx);
int64_t mctdh_destroy(mctdh_ctx_t *ctx);

/* Integrator codes of mctdh_step / mctdh_propagate: 1 Cash-Karp RK, 2 Dormand-Prince
 * RK, 3 Adams PECE of order int_order with int_par1 extra EC iterations (the first
 * int_order steps of a propagation with Cash-Karp, propagator.f90:156-181;
 * integrator.f90:244-380), 4 Bulirsch-Stoer (bsstep, integrator.f90:418-608), 10 CMF2. */

/* Equation of motion (A, psi, t) -> (dA, dpsi) on host buffers.
 * Replaces Calc_Derivs(A0, psi0, dA, dpsi, tt) -- derivatives.f90:39. */
int64_t mctdh_calc_derivs(mctdh_ctx_t *ctx, const double *A, const double *psi,
                          double *dA, double *dpsi, double t);

/* One adaptive Runge-Kutta step on host buffers (A, psi updated in place; dA,
 * dpsi are the derivatives at t on entry and, for Dormand-Prince, at t+hdid on
 * return).  method: 1 Cash-Karp, 2 Dormand-Prince.
 * Replaces rkqs(A0, psi0, dA, dpsi, tt, htry, hdid, hnext, int_method) --
 * integrator.f90:36. */
int64_t mctdh_rkqs(mctdh_ctx_t *ctx, double *A, double *psi, double *dA, double *dpsi,
                   double t, double htry, double *hdid, double *hnext, int64_t method);

/* One CMF2 step on host buffers (grid and Gaussian-mode models; Gaussian modes
 * propagate B = D^H S A with D = S^-1/2 recomputed at the step start, so DD0 is
 * not an argument; mixtures and dissipative models return -1).
 * Replaces cmf2(A0, psi0, DD0, tt, htry, hdid, hnext) -- cmf2_base.f90:47. */
int64_t mctdh_cmf2(mctdh_ctx_t *ctx, double *A, double *psi, double t, double htry,
                   double *hdid, double *hnext);

/* Step replay.  One rkck/rkdp attempt of fixed length dt (integrator.f90:95-221
 * plus the DeltaPsi error of :60-61): A, psi <- the 5th-order state, errmax <-
 * DeltaPsi / eps_int, no step control.  And one CMF2 attempt of length h that is
 * always completed as if accepted (cmf2_base.f90:76-176 and :186-190), error <-
 * max(err_A, err_psi) / eps_int.  They let a caller replay a recorded step
 * sequence: the reference's error norm sqrt|2(1 - Re<1|2>/sqrt(<1|1><2|2>))|
 * (gmctdh_objects.f90:222) sits at its rounding floor for accepted steps, so
 * free-running step sequences of two FP64 implementations differ by noise. */
int64_t mctdh_rk_attempt(mctdh_ctx_t *ctx, double *A, double *psi, double *dA, double *dpsi,
                         double t, double dt, int64_t method, double *errmax);
int64_t mctdh_cmf2_attempt(mctdh_ctx_t *ctx, double *A, double *psi, double t, double h, double *error);

/* Device-resident state: upload (also records the start state used by C(t)),
 * download.  Download replaces the host copies WriteOutput needs for the
 * restart and psi files (output.f90:231-252). */
int64_t mctdh_set_state(mctdh_ctx_t *ctx, const double *A, const double *psi, int64_t as_start);
int64_t mctdh_get_state(mctdh_ctx_t *ctx, double *A, double *psi);

/* The inner loop of propagate_wf (propagator.f90:115-134 RK, :276-296 CMF2) on
 * the resident state, from *t up to the next output time tnext.  *step carries
 * the proposed step size between calls exactly like `stepsize` in the
 * reference.  int_type: 1 rk45, 2 dopri, 10 cmf2.  Returns steps/attempts/EOMs. */
int64_t mctdh_propagate(mctdh_ctx_t *ctx, int64_t int_type, double tnext, double *t, double *step,
                        int64_t *nsteps, int64_t *nattempts, int64_t *neom);

/* One accepted step on the resident state: the body of the inner loop of
 * propagate_wf (propagator.f90:116-117 for rk45/dopri, :276 for cmf2), with the
 * reference's retry logic inside.  int_type: 1 rk45, 2 dopri, 10 cmf2. */
int64_t mctdh_step(mctdh_ctx_t *ctx, int64_t int_type, double t, double htry, double *hdid, double *hnext,
                   int64_t *nattempts);

/* Work counters: kernel launches, EOM evaluations (Calc_Derivs equivalents,
 * including the mean-field evaluations of CMF2) and H_B * B products. */
int64_t mctdh_counters(mctdh_ctx_t *ctx, int64_t *launches, int64_t *eom, int64_t *hb);

/* Measured FP64 FMA throughput of the current device (TFLOP/s), the roofline
 * denominator of the FP64 kernels. */
int64_t mctdh_fp64_peak(double *tflops);

/* CUDA events on the context's stream (slots 0..15) for device-side timing. */
int64_t mctdh_event_record(mctdh_ctx_t *ctx, int64_t slot);
int64_t mctdh_event_elapsed(mctdh_ctx_t *ctx, int64_t slot0, int64_t slot1, double *ms);

/* The reference's routine timers (timingmod.f90:16-103) on CUDA events: timer
 * 1 CalcDerivs, 2 normWF/wf_ovl, 3 Calc_MeanField, 4 Calc_CY, 5 Calc_h1mode,
 * 6 Calc_Der_SPF_DVR, 7 Calc_Der_SPF_GWP, 8 Lanczos (the reference's numbering),
 * device time between the routine's first and last launch on the context's
 * streams.  mode: 0 off, 1 on, 2 on and reset; while on, the CUDA graphs of the
 * CMF2 sweeps are not used.  mctdh_write_timings writes the `timing` file
 * (write_timings, timingmod.f90:72-103) with the caller's wall time. */
int64_t mctdh_timing(mctdh_ctx_t *ctx, int64_t mode);
int64_t mctdh_timing_read(mctdh_ctx_t *ctx, int64_t timer, int64_t *calls, double *ms);
int64_t mctdh_write_timings(mctdh_ctx_t *ctx, const char *path, double walltime_s);

/* Per-kernel-class timing with CUDA events.  enable: 0 off, 1 on, 2 on and reset.  kid: 0 mode products,
 * 1 single-hole contractions, 2 reductions, 3 h1mode/SPF operators, 4 regularised
 * inverses, 5 term sums, 6 SPF derivatives, 7 elementwise.  flops/bytes are the
 * algorithmic work of the timed launches. */
int64_t mctdh_profile(mctdh_ctx_t *ctx, int64_t enable);
int64_t mctdh_profile_read(mctdh_ctx_t *ctx, int64_t kid, double *ms, int64_t *launches, double *flops,
                           double *bytes);

/* Observables written by WriteOutput (output.f90:35-87, :144-150) for the
 * resident state: energyMF / sum(pop), state populations from rho of mode 1,
 * norm = sum(pop), and C(t) = <Psi(0)|Psi(t)>. */
int64_t mctdh_observables(mctdh_ctx_t *ctx, double t, double *energy, double *pop, double *norm,
                          double *auto_re, double *auto_im);

/* The rest of WriteOutput for the resident state, computed on the device (only
 * the results are copied back):
 * - mctdh_expect: Expectation (output.f90:449-500), values[i] = sum_t ae_t <A_l| prod_m h_m |A_r>
 *   of expectation operator i (nexpect interleaved complex values);
 * - mctdh_natpop: natural populations natpop(nspfmax, nmodes, nstates), decreasing, with
 *   nspfmax = max nSPF; for Gaussian modes the gross Gaussian populations and the population
 *   errors ggp, poperr(ns00max, nmodgwp, nstates) (output.f90:88-140); ggp/poperr may be NULL;
 * - mctdh_densmat: the reduced density matrix rho(mode, state) as written to the densmat
 *   file (output.f90:276-300), n x n interleaved complex, both triangles filled. */
/* Device memory the context holds (state vectors, stage and Krylov vectors, every
 * planned intermediate, descriptors), in bytes.  The batched plan keeps all chain
 * intermediates of one EOM alive, so this grows with terms x modes x configurations. */
int64_t mctdh_device_bytes(mctdh_ctx_t *ctx, int64_t *bytes);

/* Packet populations of the resident mixture as written by WriteOutput
 * (output.f90:44-60): WPpop normalised to unit sum and sorted decreasing
 * (npackets values), and the entropy -sum p ln p / ln npackets over p >= 1e-8
 * (0 for a single packet). */
int64_t mctdh_packets(mctdh_ctx_t *ctx, double *wppop, double *entropy);

int64_t mctdh_expect(mctdh_ctx_t *ctx, double *values);
int64_t mctdh_natpop(mctdh_ctx_t *ctx, double *natpop, double *ggp, double *poperr);
int64_t mctdh_densmat(mctdh_ctx_t *ctx, int64_t mode, int64_t state, double *rho);
/* Calc_Density (output.f90:332-445) along DOF `dof` (0-based) for every state:
 * density(ngp, nstates).  Grid DOFs: the diagonal of the DOF's density matrix in
 * the DVR, and with trafo = trafoDVR of the DOF (basis x grid, leading dimension
 * ldt) density_pop(ngp, nstates), the populations of the basis functions
 * underlying the DVR (trafo or density_pop NULL skips them).  Gaussian DOFs: the
 * density on ngp equidistant points of [xmin, xmax] = dvrpar(1:2, dof). */
int64_t mctdh_density(mctdh_ctx_t *ctx, int64_t dof, const double *trafo, int64_t ldt, double xmin,
                      double xmax, double *density, double *density_pop);

/* norm_wf (gmctdh_objects.f90:21) and WF_Ovl (gmctdh_objects.f90:101) on host buffers. */
int64_t mctdh_norm_wf(mctdh_ctx_t *ctx, const double *A, const double *psi, double *norm);
int64_t mctdh_wf_ovl(mctdh_ctx_t *ctx, const double *A1, const double *psi1, const double *A2,
                     const double *psi2, double *ovl_re, double *ovl_im);

/* Kernel launches issued by this context since creation (for accounting). */
int64_t mctdh_launch_count(mctdh_ctx_t *ctx);

/* Density matrix of one mode without any device allocation.  This entry point
 * has no counterpart in the reference (which always allocates on the host).  It
 * serves callers that cannot call cudaMalloc where they need the result: code
 * running while a stream is captured into a CUDA graph, programs that give the
 * GPU a fixed memory budget, or a driver that already keeps A in device memory
 * it manages itself.
 *   A      device pointer: one state's coefficient tensor, sizes nspf[0..nmodes-1],
 *          mode 1 fastest (init_calc.f90:531-536)
 *   rho    device pointer, column-major with leading dimension ld:
 *          rho(j1, j2) = sum over all other modes of conj(A(.., j1, ..)) A(.., j2, ..),
 *          the contraction of Calc_rho1mode (gmctdh_objects.f90:452-457) for a grid mode
 *   stream cudaStream_t to launch on (NULL: the legacy default stream); the call
 *          returns after launching, rho is ready once the stream has run.
 * Limit: nspf[mode] <= 32.  Larger sizes, host pointers, buffers of another
 * GPU or a bad mode return -7 (message in mctdh_last_error(NULL)) without
 * launching anything; a CUDA error left pending by an earlier call returns -6
 * and is not cleared.
 * Scratch: a 2 MiB file-scope __device__ array that every GPU loading this
 * library holds until exit.  The first call on a device looks up its address
 * with cudaGetSymbolAddress (make that first call before any stream capture);
 * the address is cached per device, so the device must not be reset
 * (cudaDeviceReset) while the library is loaded.
 * All calls share the array: calls that overlap on the GPU (different streams
 * without ordering) race and return wrong results.  Each call writes every
 * scratch entry it later reads, so nothing carries over between calls. */
int64_t mctdh_density_matrix_noalloc(const double *A, const int64_t *nspf, int64_t nmodes, int64_t mode,
                                     double *rho, int64_t ld, void *stream);

/* Learned mean-field extrapolator: a multilayer perceptron with BF16 weights and
 * activations and FP32 accumulation (tanh hidden layers, linear output), trained
 * with hand-written forward, backward and Adam kernels.  No reference
 * counterpart: it plugs into CMF2 between the mean-field evaluations of
 * cmf2_base.f90:78-87 and :122-130.  widths[0..nlayers]: layer sizes.
 * Parameters are flat FP32: per layer W (N x K, row-major) then b (N). */
typedef struct mctdh_mlp mctdh_mlp_t;
int64_t mctdh_mlp_create(const int64_t *widths, int64_t nlayers, uint64_t seed, mctdh_mlp_t **mlp);
int64_t mctdh_mlp_destroy(mctdh_mlp_t *mlp);
int64_t mctdh_mlp_nparams(mctdh_mlp_t *mlp, int64_t *n);
int64_t mctdh_mlp_set_params(mctdh_mlp_t *mlp, const float *params);
int64_t mctdh_mlp_get_params(mctdh_mlp_t *mlp, float *params);
int64_t mctdh_mlp_predict(mctdh_mlp_t *mlp, const float *X, float *Y, int64_t M);
int64_t mctdh_mlp_grad(mctdh_mlp_t *mlp, const float *X, const float *T, int64_t M, float *grad, double *loss);
int64_t mctdh_mlp_train(mctdh_mlp_t *mlp, const float *X, const float *T, int64_t M, int64_t batch, int64_t epochs,
                        double lr, double *loss);

/* Mean-field extrapolation inside CMF2 (no reference counterpart).  A snapshot is
 * every density matrix and mean field of the grid modes (E complex entries).
 * record: 1 start, 0 stop and clear, 2 clear and start; every accepted CMF2 step
 * computed with the plain scheme stores (t0, h, snapshot at t0, snapshot at
 * t0 + h/2).  attach: with a trained network (NULL detaches) and the half-step
 * snapshots of the last five accepted steps in the context's history, the mean
 * fields at a step start (the evaluation of cmf2_base.f90:78-87) come from the
 * quartic extrapolation of that history plus the network's residual, and only
 * h1mode is computed there; the half-step mean fields (:122-130) are computed as
 * always, and a step whose computed half-step snapshot differs from the
 * extrapolation's prediction for it by more than tol (relative 2-norm) is redone
 * with the plain scheme.  Grid-mode models only (Gaussian-mode models keep the
 * plain scheme).  The network maps MCTDH_MFX_NFEAT inputs per entry (Newton
 * increments of orders 1-4 through the five half-step snapshots at the step
 * start and at its half step, Re/Im, divided by the RMS of the first-order
 * increment at the half step, then four spacing ratios; each column divided by
 * fscale[j]) to MCTDH_MFX_NOUT outputs (Re/Im residual at the step start and at
 * the half step, in units of that RMS times tscale[j]). */
#define MCTDH_MFX_NFEAT 20
#define MCTDH_MFX_NOUT 4
int64_t mctdh_mfx_size(mctdh_ctx_t *ctx, int64_t *E);
int64_t mctdh_mfx_record(mctdh_ctx_t *ctx, int64_t enable);
int64_t mctdh_mfx_fetch(mctdh_ctx_t *ctx, int64_t maxrec, double *t0, double *h, double *snap0, double *snaphalf,
                        int64_t *n);
int64_t mctdh_mfx_attach(mctdh_ctx_t *ctx, mctdh_mlp_t *mlp, const double *fscale, const double *tscale,
                         double tol);
/* orders: the polynomial orders (1-4, default 4) through the last order + 1
 * history snapshots that the network's residual is added to, at the step start
 * and at the half step (chosen at training on held-out steps). */
int64_t mctdh_mfx_orders(mctdh_ctx_t *ctx, int64_t order_start, int64_t order_half);
/* gate: extrapolate a step start only when the first attempt of the previous
 * step had a CMF2 error (in units of the tolerance) below `gate` (default: no
 * limit), i.e. while the step control has room for the extrapolation's error. */
int64_t mctdh_mfx_gate(mctdh_ctx_t *ctx, double gate);
/* predict: run the attached extrapolator on a given history (5 x E complex
 * snapshots, oldest first, at times ts[5]) for the times tau0 (a step start) and
 * tau1 (its half step); writes the two predicted snapshots (E complex each) and
 * clears the history. */
int64_t mctdh_mfx_predict(mctdh_ctx_t *ctx, const double *hist, const double *ts, double tau0, double tau1,
                          double *out0, double *out1);
/* log: one row per CMF2 attempt of a context with extrapolation state
 * (t, h, error estimate / eps_int, predicted step start 0/1, half-step mismatch or -1). */
int64_t mctdh_mfx_log(mctdh_ctx_t *ctx, int64_t maxrows, double *rows, int64_t *n);
/* stats: steps taken with predicted step-start mean fields, steps redone because
 * the half-step check failed, attempts with predicted mean fields rejected by the
 * CMF2 error estimate (the retry computes them), and the last half-step mismatch
 * (-1 before any). */
int64_t mctdh_mfx_stats(mctdh_ctx_t *ctx, int64_t *mlp_steps, int64_t *fallbacks, int64_t *rejected,
                        double *last_rel);

/* Ensembles of independent wavepackets of uneven shape (no reference counterpart:
 * the reference runs one wavepacket per process).  Each member is described by
 * its own set-up record; every stage of the EOM is one launch over all members,
 * and adaptive RK (int_type 1 Cash-Karp, 2 Dormand-Prince; rkqs,
 * integrator.f90:36-91, per member) runs the members in lockstep.  Members are
 * DVR models in one precision mode; CMF2 is not offered for ensembles.
 * propagate: t[i] and step[i] (in/out) as propagate_wf keeps them
 * (propagator.f90:110-134), every member advanced to tnext; nrounds counts the
 * lockstep attempt rounds.  calc_derivs: the EOM of every member at its state
 * (read with get_derivs).  stream: the CUDA stream the ensemble runs on. */
typedef struct mctdh_ens mctdh_ens_t;
int64_t mctdh_ens_create(const mctdh_setup_t *setups, int64_t n, mctdh_ens_t **ens);
int64_t mctdh_ens_destroy(mctdh_ens_t *ens);
int64_t mctdh_ens_set_state(mctdh_ens_t *ens, int64_t i, const double *A, const double *psi, int64_t as_start);
int64_t mctdh_ens_get_state(mctdh_ens_t *ens, int64_t i, double *A, double *psi);
int64_t mctdh_ens_calc_derivs(mctdh_ens_t *ens);
int64_t mctdh_ens_get_derivs(mctdh_ens_t *ens, int64_t i, double *dA, double *dpsi);
int64_t mctdh_ens_propagate(mctdh_ens_t *ens, int64_t int_type, double tnext, double *t, double *step,
                            int64_t *nrounds, int64_t *neom);
int64_t mctdh_ens_observables(mctdh_ens_t *ens, int64_t i, double *energy, double *pop, double *norm,
                              double *auto_re, double *auto_im);
int64_t mctdh_ens_counters(mctdh_ens_t *ens, int64_t *launches, int64_t *eom, int64_t *rounds);
int64_t mctdh_ens_stream(mctdh_ens_t *ens, void **stream);
/* Launch-shape autotuner of an ensemble (no reference counterpart).  Unless
 * switched off, the first mctdh_ens_propagate times one merged EOM evaluation
 * for each candidate shape -- fibre tiles per contraction block (2, 4, 8, 16),
 * blocks per contraction (32, 64, 128) and, for split-precision members,
 * tensor-core or CUDA-core mode products -- and keeps the fastest; then, on that
 * shape, persistent CTAs (2 or 4 contraction CTAs and twice as many mode-product
 * CTAs per SM, each walking the batch's blocks) against one CTA per block.  mode 1 runs
 * it now on the current states, mode 0 keeps the planned shapes (an ensemble
 * whose members must repeat the arithmetic of single contexts bit for bit),
 * mode 2 keeps them with the persistent kernels on a minimal grid (every CTA
 * walks many blocks; the same arithmetic);
 * -7 once a propagation has fixed the shapes.  mctdh_ens_tuning reports the
 * chosen shape, its EOM time (ms) against the planned shape's, and the number of
 * candidates timed (0: not tuned).  Each attempt round of mctdh_ens_propagate
 * runs as one CUDA graph. */
int64_t mctdh_ens_autotune(mctdh_ens_t *ens, int64_t mode);
int64_t mctdh_ens_tuning(mctdh_ens_t *ens, int64_t *tiles_per_block, int64_t *block_cap, int64_t *tensor_cores,
                         double *eom_ms, double *default_eom_ms, int64_t *candidates);
/* Algorithmic cost of one merged EOM evaluation of all members: the FLOPs and
 * bytes (operands read once, results written once) of its mode products and
 * single-hole contractions, the roofline numerator of the EOM time. */
int64_t mctdh_ens_eom_cost(mctdh_ens_t *ens, double *flops, double *bytes);
/* Persistent CTAs chosen by the autotuner for the merged mode products and
 * contractions (0: one CTA per block of the batch). */
int64_t mctdh_ens_persistent(mctdh_ens_t *ens, int64_t *prod_ctas, int64_t *hole_ctas);
const char *mctdh_ens_last_error(mctdh_ens_t *ens);

/* Tensor-core kernels (no reference counterpart).  The FP32 mode products of the
 * split-precision paths can run as tcgen05 MMAs (TF32 parts, FP32 accumulation)
 * for batches whose largest SPF count is at least min_n and at most 16, with a
 * one- or two-stage pipeline (default 1).  Single contexts default to min_n = 17
 * (the CUDA-core kernel, faster on the measured models); ensembles let their
 * autotuner choose.  status: *enabled is 1 unless the environment variable
 * MACAW_GB300_TC=0 selected the CUDA-core kernels for this process; *timeouts is
 * 1 when a tensor-core kernel gave up waiting for its MMAs since the previous
 * call (the flag is cleared).  config: 0 keeps a setting; it applies to launches
 * issued afterwards (CUDA graphs captured earlier keep their kernels). */
int64_t mctdh_tensor_core_status(int64_t *enabled, int64_t *timeouts);
int64_t mctdh_tensor_core_config(int64_t min_n, int64_t stages);

/* Last error message of the context (or of the last failed create when ctx is NULL). */
const char *mctdh_last_error(mctdh_ctx_t *ctx);

#ifdef __cplusplus
}
#endif
#endif /* MACAW_GB300_H */
