/* melvin_gb300.h -- C ABI of the GB300 (sm_103a) kernels behind the Melvin.py
 * per-timestep hot path.
 *
 * Every entry point takes plain pointers and sizes.  Unless stated
 * otherwise, array arguments are DEVICE pointers:
 *   - spectral arrays are interleaved complex128 (re, im pairs of double),
 *     row-major with the reference's spectral shape: (2nn+1, nm) when fully
 *     spectral, (nn, nz) for Fourier-x / finite-difference-z
 *     (melvin/Parameters.py:72-79, melvin/ArrayFactory.py:28-45);
 *   - physical arrays are float64, row-major (nx, nz), z contiguous
 *     (melvin/ArrayFactory.py:47-62);
 *   - derivative histories are the reference's TimeDerivative buffer,
 *     complex128 of shape (order, *spectral_shape) (melvin/TimeDerivative.py:13-20);
 *   - `stream` is a cudaStream_t (NULL = legacy default stream);
 *   - `work` is caller-owned device scratch of at least the size returned
 *     by mgb_workspace_bytes for the same call family.
 * Work is enqueued asynchronously on `stream`.  Every function returns an
 * mgb_status; mgb_last_error() gives a one-line description of the most
 * recent failure on the calling thread.  Citations are to Melvin.py source
 * files relative to that project's root.
 */
#ifndef MELVIN_GB300_H
#define MELVIN_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum mgb_status {
  MGB_OK = 0,
  MGB_ERR_INVALID = 1,     /* bad argument (null pointer, shape, option) */
  MGB_ERR_UNSUPPORTED = 2, /* valid for the reference, not built here (e.g. non power-of-two FFT length) */
  MGB_ERR_CUDA = 3,        /* a CUDA runtime call failed */
  MGB_ERR_NONFINITE = 4,   /* NaN / Inf met by a checked reduction */
  MGB_ERR_CFL = 5,         /* CFL condition breached (melvin/Integrator.py:35-44) */
  MGB_ERR_NOMEM = 6        /* admission / allocation refused */
} mgb_status;

typedef enum mgb_precision {
  MGB_PREC_DOUBLE = 0, /* FP64 transforms, derivatives and products */
  MGB_PREC_SPLIT = 1,  /* FP32 transforms/derivatives/products, FP64 state, history and solves */
  MGB_PREC_DFLOAT = 2  /* double-float (FP32 pair, 48-bit significand) transforms, derivatives and
                          products on the FP32 pipes; FP64 state, history and solves */
} mgb_precision;

/* Grid and discretisation, the subset of Parameters the path depends on
 * (melvin/Parameters.py:9-30, 63-92). */
typedef struct mgb_grid {
  int32_t nx, nz;   /* physical points */
  double lx, lz;    /* box lengths; dx = lx/nx, dz = lz/nz */
  int32_t fdm_z;    /* 0: discretisation ["spectral","spectral"]; 1: ["spectral","fdm"] */
  int32_t sdo;      /* spatial_derivative_order: 2 or 4 */
  int32_t precision;/* mgb_precision */
} mgb_grid;

typedef struct mgb_plan mgb_plan;

/* Spectral derivative kinds for mgb_spectral_derivative. */
typedef enum mgb_deriv {
  MGB_DDX = 0,   /* Variable.sddx   melvin/SpatialDifferentiator.py:50-53 */
  MGB_DDZ = 1,   /* Variable.sddz   :55-58 (FDM-z: pddz on the spectral array, :36-40) */
  MGB_D2DX2 = 2, /* Variable.sd2dx2 :60-63 */
  MGB_D2DZ2 = 3, /* Variable.sd2dz2 :65-68 (FDM-z: pd2dz2, :106-128) */
  MGB_NABLA2 = 4 /* Variable.snabla2 melvin/Variable.py:111-113 */
} mgb_deriv;

/* ---- plans ------------------------------------------------------------- */

/* Validate the grid, upload twiddle tables and (FDM-z) the tridiagonal
 * factors.  Replaces the set-up done by Simulation.__init__ and
 * Simulation.init_laplacian_solver (melvin/Simulation.py:19-50, 67-74,
 * melvin/LaplacianSolver.py:7-56).  Fully spectral: 9 <= nx, nz <= 4096;
 * the fused kernels (mgb_vec_dot_nabla, mgb_velocity_from_vorticity,
 * mgb_step and the batched step) need powers of two in [16, 4096], the
 * transforms and pointwise verbs take any such length (transform lengths
 * that are not powers of two run as Bluestein convolutions).  Fourier-x /
 * FDM-z: a power-of-two nx in [16, 4096] and 5 <= nz <= 1800. */
int mgb_plan_create(const mgb_grid* grid, mgb_plan** out);
int mgb_plan_destroy(mgb_plan* plan);
/* Spectral (rows, cols) and physical (nx, nz) shapes of the plan. */
int mgb_plan_shapes(const mgb_plan* plan, int32_t* spec_rows, int32_t* spec_cols,
                    int32_t* phys_rows, int32_t* phys_cols);
/* Scratch bytes: family 0 = per-verb transforms, family 1 = fused step with
 * `nfields` advected fields. */
int mgb_workspace_bytes(const mgb_plan* plan, int32_t family, int32_t nfields, size_t* bytes);
const char* mgb_status_string(int32_t status);
const char* mgb_last_error(void);

/* ---- transforms (melvin/SpectralTransformer.py) ------------------------- */

/* Spectral -> physical: SpectralTransformer.to_physical, fully spectral
 * (:90-150) or x-only (:33-61). */
int mgb_to_physical(const mgb_plan* plan, const void* spec, double* phys, void* work, void* stream);
/* Physical -> spectral: SpectralTransformer.to_spectral (:152-199, :63-88). */
int mgb_to_spectral(const mgb_plan* plan, const double* phys, void* spec, void* work, void* stream);

/* ---- cosine and sine bases ---------------------------------------------
 * Basis functions per axis (melvin/BasisFunctions.py:5-9).  The reference
 * transforms a cosine or sine axis of n points as a mirrored periodic signal
 * of 2(n-1) points (melvin/SpectralTransformer.py:90-199); here that length,
 * like n on a complex-exponential axis, must lie in [16, 4096] (a power of
 * two runs as a block FFT, any other length as a Bluestein convolution of
 * power-of-two FFTs).
 * Unlike the reference, to_physical leaves its input unchanged (the
 * reference doubles the zeroth cosine mode of its input in place,
 * melvin/SpectralTransformer.py:122-125; the result equals the reference's
 * first call).  Fully spectral plans only. */
typedef enum mgb_basis {
  MGB_BASIS_COMPLEX_EXP = 0,
  MGB_BASIS_COSINE = 1,
  MGB_BASIS_SINE = 2
} mgb_basis;

/* SpectralTransformer.to_physical / to_spectral with basis (bx, bz). */
int mgb_to_physical_basis(const mgb_plan* plan, int32_t bx, int32_t bz, const void* spec, double* phys, void* work,
                          void* stream);
int mgb_to_spectral_basis(const mgb_plan* plan, int32_t bx, int32_t bz, const double* phys, void* spec, void* work,
                          void* stream);
/* Spectral derivative verbs with the basis factors of gen_diff_factors /
 * gen_diff2_factors (melvin/BasisFunctions.py:44-59,
 * melvin/SpatialDifferentiator.py:50-74): cosine and sine axes multiply by
 * the real -pi n/L or pi n/L, and by -(pi n/L)^2 for second derivatives. */
int mgb_spectral_derivative_basis(const mgb_plan* plan, int32_t kind, int32_t bx, int32_t bz, const void* in,
                                  void* out, void* stream);
/* calc_lap(basis_fns) (melvin/SpatialDifferentiator.py:70-74). */
int mgb_laplacian_basis(const mgb_plan* plan, int32_t bx, int32_t bz, double* lap, void* stream);
/* The fully spectral Poisson divide with that Laplacian (melvin/LaplacianSolver.py:58-68). */
int mgb_poisson_solve_basis(const mgb_plan* plan, int32_t bx, int32_t bz, const void* rhs, void* out, void* stream);

/* ---- derivatives (melvin/SpatialDifferentiator.py) ---------------------- */

/* Central finite-difference d/dx of a physical field, x periodic
 * (pddx, :76-89 order 2, :130-155 order 4). */
int mgb_pddx(const mgb_plan* plan, const double* in, double* out, void* stream);
/* Central finite-difference d/dz of a physical field, periodic when z is
 * spectral, Dirichlet (outer points left 0) when z is FDM (pddz, :91-104,
 * :157-185). */
int mgb_pddz(const mgb_plan* plan, const double* in, double* out, void* stream);
/* Spectral derivative verbs; `in` and `out` are spectral arrays. */
int mgb_spectral_derivative(const mgb_plan* plan, int32_t kind, const void* in, void* out, void* stream);
/* calc_lap (:70-74): real (rows, cols) array d2x*n^2 + d2z*m^2 (fully spectral). */
int mgb_laplacian(const mgb_plan* plan, double* lap, void* stream);

/* ---- streamfunction inversion (melvin/LaplacianSolver.py) -------------- */

/* Solve lap(out) = rhs: spectral divide with lap(0,0) := 1 (:58-68) or the
 * per-mode Dirichlet tridiagonal systems (:21-56, 70-79). */
int mgb_poisson_solve(const mgb_plan* plan, const void* rhs, void* out, void* stream);

/* ---- nonlinear term and velocity --------------------------------------- */

/* Variable.vec_dot_nabla (melvin/Variable.py:119-128): writes q_phys =
 * to_physical(q_spec) and out_spec = to_spectral(pddx(ux*q) + pddz(uz*q)). */
int mgb_vec_dot_nabla(const mgb_plan* plan, const void* q_spec, double* q_phys,
                      const double* ux, const double* uz, void* out_spec, void* work,
                      void* stream);
/* calc_velocity_from_vorticity (melvin/utility.py:62-79): psi = solve(-w);
 * uz_spec = sddx(psi) and uz_phys = to_physical(uz_spec); fully spectral:
 * ux_spec = -sddz(psi), ux_phys = to_physical(ux_spec); FDM-z: psi_phys =
 * to_physical(psi), ux_phys = -pddz(psi_phys) (ux_spec untouched and may be
 * NULL; psi_phys may be NULL, then scratch holds it). */
int mgb_velocity_from_vorticity(const mgb_plan* plan, const void* w_spec, void* psi_spec,
                                void* ux_spec, void* uz_spec, double* psi_phys,
                                double* ux_phys, double* uz_phys, void* work, void* stream);

/* Size of the built-in scratch array used by mgb_vec_dot_nabla_noalloc. */
#define MGB_NOALLOC_SCRATCH_BYTES (4u << 20)

/* mgb_vec_dot_nabla for callers that cannot allocate device memory: code
 * running under a framework that owns every device allocation and passes a
 * kernel only its operands and results, or a real-time loop where
 * allocation is not allowed.  Same inputs, outputs
 * and results as mgb_vec_dot_nabla, but the transform scratch comes from a
 * fixed MGB_NOALLOC_SCRATCH_BYTES array in the library's device memory
 * (held by every GPU that loads the library until the process exits), so
 * the call allocates nothing.  Grids whose scratch would exceed it (2*nx*nm
 * complex128 fully spectral, nx*nz doubles for FDM-z; e.g. 512x512 fits)
 * are rejected with MGB_ERR_UNSUPPORTED.  The first call on a device looks
 * up the array's device address (cudaGetSymbolAddress) with that device
 * current; make that first call before any stream capture.  The plan's
 * device must be current (MGB_ERR_INVALID otherwise).  All calls on a
 * device share the array: calls that overlap on the GPU race and must be
 * serialised by the caller.  No counterpart in the reference. */
int mgb_vec_dot_nabla_noalloc(const mgb_plan* plan, const void* q_spec, double* q_phys, const double* ux,
                              const double* uz, void* out_spec, void* stream);

/* ---- time integration (melvin/Integrator.py) --------------------------- */

/* _semi_implicit_spectral (:58-63): var = ((1+(1-a)dt L) var + AB(hist)) /
 * (1 - a dt L), L = lin_op (real, spectral shape); the caller advances
 * curr.  `order` 2 or 4, `curr` = TimeDerivative._curr_idx. */
int mgb_integrate_semi_implicit(const mgb_plan* plan, void* var, void* hist, int32_t order,
                                int32_t curr, double dt, double alpha, const double* lin_op,
                                void* stream);
/* _explicit (:53-56): hist[curr] += diffusion; var += AB(hist). */
int mgb_integrate_explicit(const mgb_plan* plan, void* var, void* hist, int32_t order,
                           int32_t curr, double dt, const void* diffusion, void* stream);
/* Predictor (corrector=0: AB2/AB4, :5-18) or corrector (corrector=1:
 * AM2/AM4, :20-33) value written to `out`. */
int mgb_adams(const mgb_plan* plan, int32_t corrector, const void* hist, int32_t order,
              int32_t curr, double dt, void* out, void* stream);

/* ---- diagnostics ------------------------------------------------------- */

/* Device reductions over physical ux, uz (deterministic order):
 * out[0] = calc_kinetic_energy (melvin/utility.py:42-59),
 * out[1] = max(ux), out[2] = max(uz) (signed maxima used by
 * Integrator.set_dt, melvin/Integrator.py:35-44).  `out` is device memory
 * of 3 doubles; `work` needs mgb_workspace_bytes(family 0). */
int mgb_diagnostics(const mgb_plan* plan, const double* ux, const double* uz, double* out,
                    void* work, void* stream);

/* ---- fused timestep ---------------------------------------------------- */

/* One linear term of an advected field's right-hand side:
 * rhs += coef * op(src), op 0 = value, 1 = d/dx (i kx), 2 = d/dz (i kz);
 * src = field index, or -1 for the streamfunction psi = solve(-field 0).
 * E.g. `- params.Pr * params.Ra * tmp.sddx()`
 * (examples/rayleigh_benard_convection.py:102-105) is {src=T, op=1,
 * coef=-Pr*Ra}; `- uz[:]` (examples/double_diffusive_convection.py:115) is
 * {src=-1, op=1, coef=-1}. */
typedef struct mgb_term {
  int32_t src;
  int32_t op;
  double coef;
} mgb_term;

/* Boundary/mean rules applied after the update (bit flags). */
enum {
  MGB_BC_ZERO_M0 = 1,      /* field[:, 0] = 0  (examples/double_diffusive_convection.py:122-124) */
  MGB_BC_DIRICHLET_W = 2,  /* FDM-z vorticity rows: w[1:, edges] = 0, w[0, :] = 0
                              (examples/rayleigh_benard_convection.py:112-142) */
  MGB_BC_DIRICHLET_T = 4   /* FDM-z scalar: t[0, lower edge] = 1, t[0, upper edge] = 0,
                              t[1:, edges] = 0 (same lines) */
};

typedef struct mgb_field_eq {
  double kappa;        /* diffusion coefficient: lin_op = kappa * lap */
  int32_t nterms;      /* <= 4 */
  mgb_term terms[4];
  int32_t bc;          /* MGB_BC_* flags */
} mgb_field_eq;

enum {
  MGB_INT_SEMI_IMPLICIT = 0, /* Integrator._semi_implicit_spectral (fully spectral only) */
  MGB_INT_EXPLICIT = 1,      /* Integrator._explicit */
  MGB_INT_PECE = 2           /* AB predictor, re-evaluation, AM corrector (defined here;
                                the reference defines the AM formulae but never calls them) */
};

/* The equation set of one user loop body: field 0 is the vorticity, the
 * others are scalars advected by the same velocity. */
typedef struct mgb_equation {
  int32_t nfields;     /* 1..3 */
  int32_t integrator;  /* MGB_INT_* */
  int32_t order;       /* integrator_order: 2 or 4 */
  double alpha;        /* semi-implicit alpha (Parameters.alpha = 0.51) */
  mgb_field_eq f[3];
  int32_t diag_flux;   /* 0: three diagnostics; k in 1..nfields: a fourth, the convective flux
                          mean(uz * q) of field k-1 in physical space (the Nusselt number of
                          examples/double_diffusive_convection.py:20-23 is 1 minus it) */
} mgb_equation;

/* Compute into `work` the per-mode update coefficients of `eq` at `dt`
 * (for the fully spectral semi-implicit update: (1 + (1-alpha) dt L) /
 * (1 - alpha dt L) and the Adams-Bashforth weight over (1 - alpha dt L),
 * L = kappa * lap; melvin/Integrator.py:58-63).  Call it before mgb_step
 * and again whenever eq, dt or the workspace change; mgb_step returns
 * MGB_ERR_INVALID when the last preparation on the plan does not match.
 * A no-op for FDM-z plans. */
int mgb_step_prepare(const mgb_plan* plan, const mgb_equation* eq, double dt, void* work, void* stream);

/* One timestep of the whole loop body (velocity from vorticity, nonlinear
 * terms, linear terms, update, boundary rules) for `eq`, fused into a few
 * kernels.  q[f]: spectral states (updated in place); hist[f]: histories;
 * `curr` is the history slot that receives this step's derivative (the
 * caller advances it afterwards, as TimeDerivative.advance does).  `diag`
 * (device, 3 doubles, or 4 when eq->diag_flux is set; may be NULL)
 * receives kinetic energy, max ux, max uz of the velocity at the start of
 * the step, and the convective flux eq->diag_flux asks for. */
int mgb_step(const mgb_plan* plan, const mgb_equation* eq, void* const* q, void* const* hist,
             int32_t curr, double dt, void* work, double* diag, void* stream);

/* A batch of independent simulations on one grid, advanced together by
 * mgb_batch_step: every kernel of the step covers all members (the last grid
 * dimension indexes the member).  Slot k's fields sit at
 *   states     q    + (k*nfields + f) * rows*cols            (complex128)
 *   histories  hist + ((k*nfields + f) * order) * rows*cols  (complex128)
 * so a pool of slots can hold simulations that start and finish at
 * different times: `members` lists the slots to advance in this call.
 * Extends the per-simulation loop of the examples (e.g.
 * examples/kelvin_helmholtz_instability.py:115-131) to an ensemble. */
typedef struct mgb_batch {
  int32_t count;            /* members advanced by this call, 1..65535 */
  const int32_t* members;   /* device array of `count` slot indices, or NULL for slots 0..count-1 */
  void* q;                  /* states, complex128 [slots][nfields][rows][cols] */
  void* hist;               /* histories, complex128 [slots][nfields][order][rows][cols] */
  const double* term_coef;  /* optional device [slots][3][4]: per-slot coefficients of the
                               equation's linear terms (replacing mgb_term.coef), e.g. a
                               per-run density ratio */
} mgb_batch;

/* Scratch bytes of mgb_batch_step for `count` members. */
int mgb_batch_workspace_bytes(const mgb_plan* plan, int32_t nfields, int32_t count, size_t* bytes);
/* mgb_step for a batch: one call advances every listed member by one step
 * (same equation, dt and curr for all; mgb_step_prepare on the same
 * workspace first).  `diag` (device, count x 3 doubles, or count x 4
 * with eq->diag_flux; may be NULL) receives each member's diagnostics as
 * mgb_step does. */
int mgb_batch_step(const mgb_plan* plan, const mgb_equation* eq, const mgb_batch* batch, int32_t curr,
                   double dt, void* work, double* diag, void* stream);

/* Number of kernels one mgb_step launches for `eq` on this plan (not
 * counting the diagnostics fold): 3 fully spectral, 4 FDM-z explicit, 8
 * FDM-z predictor-corrector.  No reference counterpart (instrumentation). */
int mgb_step_kernel_count(const mgb_plan* plan, const mgb_equation* eq, int32_t* count);
/* mgb_step that also records caller-created CUDA events on `stream`:
 * events[0] before the first kernel and events[k] after kernel k, for
 * k < nevents (count+1 events time every kernel).  No reference
 * counterpart (instrumentation for per-kernel rooflines). */
int mgb_step_events(const mgb_plan* plan, const mgb_equation* eq, void* const* q, void* const* hist,
                    int32_t curr, double dt, void* work, double* diag, void* stream,
                    void* const* events, int32_t nevents);
/* mgb_step whose kernel k first makes `stream` wait for the caller-created
 * CUDA event waits[k] (k < nwaits; NULL entries: no wait).  Data that only
 * a later kernel reads can then arrive on another stream while the earlier
 * kernels run: the history slots are read only by the update, kernel 2 of
 * every step (the forward x pass; on FDM-z plans the forward x pass of the
 * first stage).  No reference counterpart (the reference's arrays are
 * host-resident). */
int mgb_step_waits(const mgb_plan* plan, const mgb_equation* eq, void* const* q, void* const* hist,
                   int32_t curr, double dt, void* work, double* diag, void* stream,
                   void* const* waits, int32_t nwaits);

/* Throughput probe of the FP64 FMA pipe (the denominator of the FP64-ALU
 * roofline of the FP64 step): launches `blocks` CTAs whose threads run
 * independent chains of `iters` FP64 FMAs each and writes to *flops
 * (host) the FP64 flops the launch retires (an FMA counts two); the caller
 * times the launch on `stream`.  `sink` (device, `blocks` doubles) is never
 * written in practice.  No reference counterpart (instrumentation). */
int mgb_fp64_fma_probe(double* sink, int32_t blocks, int32_t iters, double* flops, void* stream);

/* ---- device-driven run: the Simulation loop without host synchronisation --
 * The reference keeps t, dt and the loop counter on the host and, in
 * Simulation.end_loop, fires loop-counted tickers (melvin/Ticker.py:1-35):
 * the CFL check Integrator.set_dt every cfl_cadence loops
 * (melvin/Integrator.py:35-44, melvin/Simulation.py:79-84,99-100) and the
 * scalar trackers every tracker_cadence loops (melvin/Simulation.py:86-97),
 * and stops when t reaches final_time (melvin/Simulation.py:134-135).  A
 * driven run keeps all of that in a device-resident mgb_run_state: the
 * step's kernels read dt from it and return at once for iterations past
 * the stop point, and a one-thread tick kernel does end_loop, the CFL
 * shrink / breach test and the tracker samples.  The caller launches
 * iterations without waiting and reads the state when it wants to.
 * Loop-counted tickers fire on iterations known in advance, so the caller
 * passes per iteration which of them fire (MGB_RUN_* flags). */
typedef enum mgb_run_status {
  MGB_RUN_RUNNING = 0,
  MGB_RUN_FINISHED = 1,   /* t reached final_time */
  MGB_RUN_CFL_BREACH = 2, /* dt > CFL limit or NaN velocity: "CFL condition breached" */
  MGB_RUN_PAUSED = 3      /* t passed cfg->pause_time: the caller fires its time-based tickers */
} mgb_run_status;

typedef struct mgb_run_state {   /* device memory, filled by the caller before mgb_run_begin */
  double t;                /* Simulation._t */
  double dt;               /* Integrator._dt */
  int64_t loop;            /* Simulation._loop_counter: completed iterations */
  int64_t stop_loop;       /* iterations with index >= stop_loop do not run (set on the device) */
  int64_t cfl_counter;     /* CFL ticker counter: fires after iteration L when counter < L+1 */
  int64_t tracker_counter; /* tracker ticker counter */
  int64_t cfl_fired;       /* times the CFL ticker fired */
  int64_t tracker_fired;   /* times the tracker ticker fired */
  int32_t status;          /* mgb_run_status */
  int32_t dt_changed;      /* the last tick shrank dt (coefficients are refreshed) */
  int32_t ntracked;        /* tracker samples written */
  int32_t dropped;         /* tracker samples that found the buffer full */
  double diag[4];          /* kinetic energy, max ux, max uz of the last diagnosed step, and the
                              convective flux when eq->diag_flux is set */
} mgb_run_state;

typedef struct mgb_run_config {  /* host memory */
  double final_time;       /* Parameters.final_time */
  double cfl_cutoff;       /* Parameters.cfl_cutoff */
  int32_t cfl_cadence;     /* loops between CFL checks */
  int32_t tracker_cadence; /* loops between tracker samples */
  int32_t capacity;        /* tracker buffer length */
  int32_t horizon;         /* the caller ticks at least every `horizon` iterations */
  double pause_time;       /* pause after the first end_loop with t > pause_time (the next dump or
                              save time of the time-based tickers; +inf for none) */
  double* tracker_t;       /* device [capacity]: t of each sample */
  double* tracker_ke;      /* device [capacity]: kinetic energy (calc_kinetic_energy, melvin/utility.py:42-59) */
  double* tracker_flux;    /* device [capacity] or NULL: the convective flux of eq->diag_flux at
                              each sample (1 minus the Nusselt number of
                              examples/double_diffusive_convection.py:20-23) */
} mgb_run_config;

#define MGB_RUN_TICK 1   /* tick after this iteration (end_loop, stop point) */
#define MGB_RUN_CFL 2    /* the CFL ticker fires after this iteration (implies a tick) */
#define MGB_RUN_TRACK 4  /* the tracker ticker fires after this iteration (implies a tick) */

/* Compute the stop point of `state` (device) from its t, dt, loop and
 * cfg->final_time.  Call after filling the state and after mgb_step_prepare
 * with the state's dt. */
int mgb_run_begin(const mgb_plan* plan, mgb_run_state* state, const mgb_run_config* cfg, void* stream);
/* Iteration `loop` of a driven run: mgb_step with dt read from the state,
 * skipped on the device when the run stopped before it, then the tick when
 * `flags` ask for one (after a CFL shrink, the fully spectral update
 * coefficients are recomputed on the device).  `curr` is the history slot
 * of this iteration, as for mgb_step. */
int mgb_run_step(const mgb_plan* plan, const mgb_equation* eq, void* const* q, void* const* hist, int32_t curr,
                 int64_t loop, int32_t flags, void* work, mgb_run_state* state, const mgb_run_config* cfg,
                 void* stream);

/* ---- tile variants of the fused step (fully spectral plans) -------------
 * Each of the three fused-step kernels comes in up to MGB_TILE_VARIANTS
 * variants that differ in the work given to one CTA, the largest FFT radix
 * and the kind of transform:
 *   MGB_FAMILY_XINV, MGB_FAMILY_XFWD (x passes): columns per CTA;
 *   MGB_FAMILY_ZSTEP (z pass): pairs of grid rows per CTA.
 * Variants 0-3 keep the transform in shared memory (kind 0); z-pass variant
 * 4 (FP32, lengths 128..4096) keeps every thread's points in registers and
 * exchanges them through shared memory between passes (kind 1).  A fresh
 * plan selects its fastest default per precision (mgb_plan_get_tiles).  An autotuner times the variants on the
 * caller's workload and sets the fastest per plan and field count.  The
 * reference leaves the equivalent choice to numpy.fft's internal plan
 * (melvin/SpectralTransformer.py:58,85,132,191). */
#define MGB_TILE_VARIANTS 5
typedef enum mgb_family {
  MGB_FAMILY_XINV = 0,   /* inverse x pass (velocity and fields to z-mode columns) */
  MGB_FAMILY_ZSTEP = 1,  /* z pass: to physical rows, products, z stencil, back */
  MGB_FAMILY_XFWD = 2    /* forward x pass, x stencil, linear terms, update */
} mgb_family;

typedef struct mgb_tile_info {
  int32_t available;    /* 1 when the variant exists for this plan (its shared memory fits) */
  int32_t shape;        /* columns per CTA (x passes) or row pairs per CTA (z pass) */
  int32_t radix;        /* largest FFT radix (8 or 16) */
  int32_t kind;         /* 0: shared-memory passes; 1: register-resident points */
  uint64_t smem_bytes;  /* dynamic shared memory per CTA */
} mgb_tile_info;

/* Describe variant `variant` of `family` for `nfields` advected fields (1..3). */
int mgb_tile_info_get(const mgb_plan* plan, int32_t family, int32_t nfields, int32_t variant,
                      mgb_tile_info* info);
/* Select the variants (tiles[family]) that mgb_step / mgb_batch_step use
 * for `nfields` advected fields; MGB_ERR_INVALID for an unavailable one. */
int mgb_plan_set_tiles(mgb_plan* plan, int32_t nfields, const int32_t* tiles);
/* Read the current selection into tiles[3]. */
int mgb_plan_get_tiles(const mgb_plan* plan, int32_t nfields, int32_t* tiles);

#ifdef __cplusplus
}
#endif

#endif /* MELVIN_GB300_H */
