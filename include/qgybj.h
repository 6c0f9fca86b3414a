/*
 * qgybj.h — C-ABI of the GB300 (sm_103a) QG-YBJ+ time step.
 *
 * The Fortran host of the reference (main_waqg.f90, init.f90, IO_ncf.f90 and
 * a parameters file) binds these entry points through ISO_C_BINDING in place
 * of the fft.f90 / derivatives.f90 / elliptic.f90 / mpi.f90 routines.  Every
 * function returns an int status (QG_OK == 0); qg_last_error() gives the text.
 *
 * Array conventions (identical in memory to the reference's Fortran arrays):
 *   spectral "kvar": interleaved complex double [nz][ikty][iktx]
 *                    == double complex kvar(iktx, ikty, nz), iktx = n1/2+1, ikty = n2
 *                    ky in FFT order (kya = 0..n2/2-1, 0*, -n2/2+1..-1, init.f90:35-41)
 *   physical "rvar": double [nz][n2][n1+2] == double precision rvar(n1+2, n2, nz)
 * Only interior z levels are exchanged (the reference's halo levels are
 * dropped).  Pointers may be host or device memory; nothing is retained past
 * a call.  One host thread per handle; calls on a handle are stream-ordered
 * on the handle's own CUDA stream and synchronous unless stated otherwise.
 */
#ifndef QGYBJ_H
#define QGYBJ_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
enum qg_status {
  QG_OK = 0,
  QG_ERR_ARG = 1,          /* bad dimensions, null pointer, unknown field id       */
  QG_ERR_CUDA = 2,         /* a CUDA runtime call or kernel launch failed          */
  QG_ERR_NONFINITE = 3,    /* NaN/Inf in an input array (configuration, or a       *
                            * retained mode given to qg_set_state), or a step     *
                            * that produced a non-finite q*                       */
  QG_ERR_PIVOT = 4,        /* zero or non-dominant pivot in a tridiagonal factor   */
                           /*   (the DGTSV INFO>0 case, elliptic.f90:192,209)      */
  QG_ERR_TIMEOUT = 5,      /* a bounded device-side wait expired                   */
  QG_ERR_UNSUPPORTED = 6,  /* configuration outside what the build implements      */
  QG_ERR_NOMEM = 7         /* device allocation failed                             */
};

enum qg_precision {
  QG_PREC_FP64 = 0,        /* every operation in FP64                               */
  QG_PREC_MIXED = 1        /* FP32 FFTs/Jacobians/leapfrog; FP64 tridiagonal solves */
};                         /*   and FP64 diagnostics                                */

/* Field ids for qg_set_state / qg_get_state (main_waqg.f90:15-60). */
enum qg_field {
  QG_Q = 0,      /* qk   : QG potential vorticity at n                 */
  QG_QOLD = 1,   /* qok  : q at n-1 (filtered)                          */
  QG_BR = 2,     /* BRk  : real part of B = L+A at n                    */
  QG_BI = 3,     /* BIk                                                 */
  QG_BROLD = 4,  /* BRok                                                */
  QG_BIOLD = 5,  /* BIok                                                */
  QG_PSI = 6,    /* psik : streamfunction                               */
  QG_AR = 7,     /* ARk  : real part of A                               */
  QG_AI = 8,     /* AIk                                                 */
  QG_CR = 9,     /* CRk  : A_z (get only, elliptic.f90:437-450)         */
  QG_CI = 10,    /* CIk  : (get only)                                   */
  QG_QSTAR = 11, /* q* = q - q^w of the last step (get only)            */
  QG_NFIELDS = 12
};

/* Run configuration: the values of the reference's parameters module that
 * the step reads (parameters_test1.f90) plus the base state of
 * init_base_state (init.f90:177-264).  Arrays are copied by qg_create. */
typedef struct qg_config {
  int n1, n2, n3;          /* resolution; n1 == n2, a power of two in [16,1024]; 2 <= n3 <= 1024 */
  int precision;           /* enum qg_precision                                        */
  int device;              /* CUDA device ordinal                                      */
  /* physics switches (parameters_test1.f90:22-29) */
  int ybj_plus, fixed_flow, no_feedback, passive_scalar, linear, no_dispersion, inviscid;
  double dz;               /* vertical grid spacing (L3/n3)                            */
  double Bu, Ro, W2F;      /* Burger, Rossby, wave-to-flow velocity ratio squared      */
  double delt, gamma;      /* time step, Robert-Asselin coefficient                    */
  double nuh1, nuh2, nuh1w, nuh2w;   /* horizontal hyperdiffusion coefficients        */
  int ilap1, ilap2, ilap1w, ilap2w;  /* their Laplacian powers                        */
  double nuz;              /* vertical q diffusion (dissipation_q_nv)                  */
  const double* a_ell_ut;  /* [n3] Bu/N^2 at za(iz) = iz*dz                            */
  const double* rho_ut;    /* [n3] or NULL (= 1)                                       */
  const double* rho_st;    /* [n3] or NULL (= 1)                                       */
  const double* r_2ut;     /* [n3] N^2 at za(iz), or NULL (= Bu/a_ell_ut); diagnostics */
  int levels_per_batch;    /* z levels per phase-A batch; 0 = choose automatically     */
  int use_graphs;          /* 1 = replay the step as a CUDA graph (default), 0 = launch */
  int solve_columns;       /* columns per CTA of the column solves: 16, 32 or 64; 0 = 32 */
} qg_config;

typedef struct qg_handle qg_handle;

/* FP64 domain integrals (diagnostics.f90:647-743, 16-211, 1262-1363), each a
 * vertical sum divided by n3, without the dimensional Uw_scale^2 factors. */
typedef struct qg_energy {
  double wke;      /* wave kinetic energy  sum_L |B|^2 - 1/2 |B(0,0)|^2          */
  double wpe;      /* wave potential energy  (0.5/(N^2 Bu)) kh^2 |A_z|^2          */
  double wce;      /* 1/8 Bu^-2 kh^4 |A|^2                                         */
  double ke;       /* flow kinetic energy  kh^2 |psi|^2                            */
  double pe;       /* flow potential energy  (Bu/N^2) |psi_z|^2                    */
  double zeta2;    /* <zeta_z^2> = 2 sum kh^4 |psi|^2                              */
  double omegah2;  /* <omega_H^2> = 2 sum kh^2 |psi_z|^2                           */
} qg_energy;

/* Fills *cfg with the switches of the YBJ+ step (ybj_plus=1, everything else
 * 0 except inviscid=1), precision MIXED, device 0, graphs on. */
int qg_config_defaults(qg_config* cfg);

/* Replaces initialize_fftw (fft.f90:32-52) and the tables of init_arrays /
 * init_base_state (init.f90:17-264): builds the dealiasing mask, integrating
 * factors, tridiagonal factor tables and device buffers.  QG_ERR_PIVOT when a
 * tridiagonal factorisation would need a row interchange or hits a zero pivot. */
int qg_create(const qg_config* cfg, qg_handle** out);

/* Replaces kill_fftw (fft.f90:112-119). */
int qg_destroy(qg_handle* h);

/* Text of the last error on h, or, when h is NULL, of the last failed call
 * made without a handle on this thread (qg_create, qg_fft_c2r_noalloc). */
const char* qg_last_error(const qg_handle* h);

/* Host <-> device copies of the resident state, levels [level0, level0+nlev).
 * kvar is [nlev][ikty][iktx] interleaved complex.  Values on modes with L=0
 * are discarded by qg_set_state (every step of the reference zeroes them);
 * a NaN or infinity on a retained mode makes qg_set_state return
 * QG_ERR_NONFINITE (the values are stored all the same). */
int qg_set_state(qg_handle* h, int field, const double* kvar, int level0, int nlev);
int qg_get_state(qg_handle* h, int field, double* kvar, int level0, int nlev);

/* Initialisation sequence of main_waqg.f90:129-147 on the resident state:
 * optional sumB (derivatives.f90:1073-1118), q = init_q(psi) (init.f90:591),
 * old levels = current levels, and A = A_solver_ybj_plus(B) (YBJ+; with
 * ybj_plus = 0 the A the host set is kept, as the reference keeps the A of
 * its initial-condition fields). */
int qg_init_state(qg_handle* h, int apply_sumB, int q_from_psi);
/* With fixed_flow = 1, q is set to 0 instead (main_waqg.f90:141-146). */

/* One full time step on the device: main_waqg.f90:202-317 (euler_first=1,
 * forward Euler) or 331-467 (leapfrog + Robert-Asselin filter).  Returns
 * QG_ERR_NONFINITE when the step's q* (= q - q^w, which depends on q and B)
 * holds a NaN or infinity on a retained mode: the run has blown up (the
 * reference would carry on and write NaN to its dumps). */
int qg_step(qg_handle* h, int euler_first);

/* nsteps steps; the first is forward Euler when euler_first=1.  Asynchronous:
 * returns once the work is queued on the handle's stream. */
int qg_steps_async(qg_handle* h, int nsteps, int euler_first);
/* Waits for h's stream; reports what its kernels raised since the last
 * check: QG_ERR_TIMEOUT (a bounded wait expired) or QG_ERR_NONFINITE (a
 * queued step produced a non-finite q*). */
int qg_synchronize(qg_handle* h);

/* Failure-path check of the bounded device-side waits: runs on h's stream a
 * kernel whose wait (the mbarrier wait the row kernels use for their bulk
 * copies) nothing completes; it gives up after ~0.5 s of SM clocks and the
 * call returns QG_ERR_TIMEOUT, with h still usable. */
int qg_selftest_wait(qg_handle* h);

/* The handle's cudaStream_t (as void*) for event timing by the host. */
int qg_get_stream(qg_handle* h, void** stream);

/* FP64 energy / enstrophy integrals of the resident state.  FP64 handles sum
 * in FP64.  Mixed handles (FP32 state) form the sums of squares in FP32-pair
 * arithmetic (exact products, TwoSum accumulation; a thread whose FP32 pairs
 * overflow recomputes in FP64): within ~2^-40 of the FP64 sums of the same
 * FP32 values, plus 2^-100 absolute per mode where squares underflow FP32. */
int qg_diagnostics_fp64(qg_handle* h, qg_energy* out);
/* The same in two halves, for a host that reads them every step without
 * stalling the run: _async queues the integrals of the state as it stands
 * after the work queued so far (a step may follow at once: its first
 * kernels, which only read the state, run beside the integrals, and its
 * update waits for them); _wait blocks until they are done and returns them.
 * One _async at a time per handle (QG_ERR_ARG while one is uncollected).
 * Not for members of an ensemble stack. */
int qg_diagnostics_fp64_async(qg_handle* h);
int qg_diagnostics_fp64_wait(qg_handle* h, qg_energy* out);

/* Kernel classes of one step, for qg_profile_step. */
enum qg_kernel_class {
  QG_K_DISSIPATION = 0,  /* dissipation_q_nv (only when inviscid == 0 and nuz != 0) */
  QG_K_COL_INV = 1,      /* y-inverse transforms of u, v, zeta, q, BR, BI           */
  QG_K_ROW_MAIN = 2,     /* x-transforms and products of convol/refraction          */
  QG_K_COL_UPDATE = 3,   /* y-forward transforms, leapfrog/filter, q^w y-inverse    */
  QG_K_ROW_QW = 4,       /* x-transforms and products of compute_qw                 */
  QG_K_COL_QW = 5,       /* y-forward transforms of q^w, q* = q - q^w               */
  QG_K_SOLVE = 6,        /* FP64 tridiagonal solves q*->psi (and B->A when not split) */
  QG_K_SOLVE_A = 7,      /* FP64 tridiagonal solves B->A on their own: they run beside *
                          * the q^w kernels in a step, one after another when profiled */
  QG_K_NCLASSES = 8
};

/* Profiling aid (no counterpart in the reference): runs one step without the
 * CUDA graph, with CUDA events around every kernel launch, and returns per
 * kernel class the summed device time (ms) and the number of launches.  The
 * state advances exactly as with qg_step. */
int qg_profile_step(qg_handle* h, int euler_first, double* ms, int* launches, int nclasses);

/* ---- routine-level drop-ins (same argument sets as the Fortran routines,
 *      interior levels only, no scratch arrays) ---------------------------- */

/* fft.f90:55-66: per-level 2D r2c of rvar, divided by n1*n2. */
int qg_fft_r2c(qg_handle* h, const double* rvar, double* kvar, int nz);
/* fft.f90:71-83: realit then unnormalised per-level 2D c2r.  kvar is read
 * only (the reference's in-place transform destroys it). */
int qg_fft_c2r(qg_handle* h, const double* kvar, double* rvar, int nz);
/* derivatives.f90:607-803 */
int qg_convol_waqg(qg_handle* h, const double* uk, const double* vk, const double* qk,
                   const double* BRk, const double* BIk,
                   double* nqk, double* nBRk, double* nBIk, int nz);
/* derivatives.f90:810-900 */
int qg_refraction_waqg(qg_handle* h, const double* BRk, const double* BIk, const double* psik,
                       double* rBRk, double* rBIk, int nz);
/* derivatives.f90:906-1032 */
int qg_compute_qw(qg_handle* h, const double* BRk, const double* BIk, double* qwk, int nz);
/* Output path: the real-space FP32 fields of the netCDF dumps, interior
 * levels level0 .. level0+nlev-1, layout out[z][y][x] (x fastest, the
 * Fortran psi_clean(n1,n2,n3h0) / BR_clean order).
 * qg_dump_psi replaces IO_ncf.f90:35-58 (ncdump_psi): out = real(psi * U_scale * L_scale),
 * the product taken left to right in FP64 and rounded to FP32.
 * qg_dump_la replaces IO_ncf.f90:137-146 (ncdump_la): out = real(B * Uw_scale) for the
 * real and imaginary parts of B; with la != 0 the YBJ+ conversion
 * LA = B + 0.25*kh2*A/Bu on the retained modes is applied first
 * (diagnostics.f90:1698-1727).  Pass the scales as the host holds them
 * (the reference's Uw_scale = 2.5e-5 is a single-precision literal). */
int qg_dump_psi(qg_handle* h, float* out, int level0, int nlev, double U_scale, double L_scale);
int qg_dump_la(qg_handle* h, float* outR, float* outI, int level0, int nlev, double Uw_scale, int la);
/* Omega equation (the vertical-velocity diagnostic, main_waqg.f90:164-167),
 * all n3 interior levels, dense spectral layout.
 * qg_omega_eqn_rhs replaces derivatives.f90:1469-1586: rhs = r2c(2 J(psi_z, lap psi)),
 * psi_z and the interpolated psi on the unstaggered level between z and z+1
 * (0 and psi(top) at the top level).
 * qg_omega_equation replaces elliptic.f90:463-567: per column with kh2 != 0 and
 * L = 1 the tridiagonal system of the n3-1 unstaggered levels (DGTSV order,
 * FP64); w at the top level and in every other column is 0.
 * qg_omega: both, from the handle's resident psi. */
int qg_omega_eqn_rhs(qg_handle* h, const double* psik, double* rhs);
int qg_omega_equation(qg_handle* h, const double* rhs, double* wk);
int qg_omega(qg_handle* h, double* wk);
/* elliptic.f90:145-247: all n3 levels, z-major layout (no transpose). */
int qg_psi_solver(qg_handle* h, const double* qstar, double* psik);
/* elliptic.f90:346-460: all n3 levels; ck may be NULL. */
int qg_A_solver_ybj_plus(qg_handle* h, const double* bk, double* ak, double* ck);

/* ---- adjoint (no counterpart in the reference) ---------------------------- */

/* Objective of qg_adjoint_run: J = sum over the subvolume of 1/2 |LA|^2 at the
 * final step, LA = B + kh^2 A / (4 Bu) (diagnostics.f90:1698-1706) in physical
 * space; subvolume = the central quarter of the horizontal domain
 * (x, y in [n/4, 3n/4) grid points) and the levels with zs >= 0.8 (top 20 %). */
enum { QG_OBJ_LA_SUBVOLUME = 0 };

/* Reverse-mode gradient of J after nsteps (first step forward Euler) with
 * respect to the initial q, BR and BI (all n3 levels, kvar layout, host or
 * device pointers).  The forward model is the step with psi and A derived
 * from (q, B) at every step, including t = 0 (psi0 = psi_solver(q0 - q^w(B0))).
 * Checkpoints every ckpt_every steps; the forward steps inside a segment are
 * recomputed with the step kernels, the reverse steps use hand-written
 * adjoint kernels.  Gradients are with respect to the real and imaginary
 * parts of the retained (L=1) modes; pass NULL gradients for J alone.
 * FP64 handles only (QG_ERR_UNSUPPORTED otherwise); requires rho = 1. */
int qg_adjoint_run(qg_handle* h, const double* q0, const double* BR0, const double* BI0, int nsteps,
                   int ckpt_every, int objective, double* J, double* grad_q0, double* grad_BR0, double* grad_BI0);

/* One step and its adjoint at the carried state X = (q, q_old, BR, BI,
 * BR_old, BI_old) (six kvar arrays, all n3 levels): Xn = step(X) and
 * lX_out = (d step/d X)^T lX.  For tangent-linear/adjoint (dot-product)
 * checks.  Any of Xn / lX_out may be NULL. */
int qg_adjoint_step(qg_handle* h, int euler_first, const double* const* X, const double* const* lX,
                    double* const* Xn, double* const* lX_out);

/* ---- ensembles and tuning (no counterpart in the reference) -------------- */

/* An ensemble of independent runs, possibly of different sizes and
 * parameters, advanced together.  Members that share the resolution,
 * precision, physics switches, Bu, dz, gamma, nuz, the Laplacian powers, the
 * solve block shape and the vertical profiles (a_ell_ut, rho, N^2) - and so
 * differ only in delt, Ro, W2F and the hyperdiffusion coefficients - are
 * stacked in z into one run of members*n3 levels: each kernel of the step
 * then runs once for the whole stack, every member a vertical segment with
 * its own top and bottom, its own time step, Rossby number, W2F and
 * integrating factors (YBJ+ only; regular-YBJ members run unstacked).  One
 * CUDA graph per step kind forks every run (stack or unstacked member) onto
 * its own stream and joins them, so one graph launch advances all members.
 * Results are bitwise those of the members run alone.
 * qg_ensemble_member returns a handle per member: for a stacked member a
 * view of its levels of the stack, valid for qg_set_state, qg_get_state,
 * qg_init_state, qg_diagnostics_fp64, qg_dump_psi / qg_dump_la and the
 * transform drop-ins; calls that act on a whole run (steps, solves, omega,
 * adjoint, profiling) return QG_ERR_UNSUPPORTED on a view.  Member handles
 * belong to the ensemble.  All members must use the same device. */
typedef struct qg_ensemble qg_ensemble;
int qg_ensemble_create(const qg_config* cfgs, int nmembers, qg_ensemble** out);
int qg_ensemble_member(qg_ensemble* e, int member, qg_handle** h);
/* nsteps steps of every member (the first forward Euler when euler_first=1);
 * asynchronous, like qg_steps_async. */
int qg_ensemble_step(qg_ensemble* e, int nsteps, int euler_first);
/* Number of chains of runs the step graph runs concurrently (default 8; 1
 * runs them one after another).  Runs (stacks and unstacked members) are
 * dealt to the chains largest first, each to the chain with the fewest cells
 * so far.  Drops the captured graphs; results do not depend on it. */
int qg_ensemble_set_lanes(qg_ensemble* e, int lanes);
/* Waits for the ensemble's stream; QG_ERR_TIMEOUT / QG_ERR_NONFINITE as
 * qg_synchronize for the first run that raised one (named in the error
 * text; a stack reports for all its members); every status is cleared. */
int qg_ensemble_synchronize(qg_ensemble* e);
int qg_ensemble_get_stream(qg_ensemble* e, void** stream);
int qg_ensemble_destroy(qg_ensemble* e);
const char* qg_ensemble_last_error(const qg_ensemble* e);
/* One step of every run of the ensemble (stacks and unstacked members), one
 * run after another, with CUDA events around each launch, as
 * qg_profile_step: per kernel class the summed device time and the launch
 * count.  It advances the state like qg_ensemble_step. */
int qg_ensemble_profile_step(qg_ensemble* e, int euler_first, double* ms, int* launches, int nclasses);

/* Autotuner: times candidate phase-A batch depths (levels per batch: the L2
 * footprint of the (kx,y) scratch planes and the wave count of the column
 * kernels) on a handle built from cfg and reports the fastest.  The state
 * content does not change the cost, so the candidates run on a zero state. */
typedef struct qg_tuning {
  int levels_per_batch;      /* fastest candidate                          */
  double ms_per_step;        /* its time per step                          */
  int ncandidates;           /* candidates timed (<= 16)                   */
  int candidates[16];        /* their batch depths ...                     */
  double candidate_ms[16];   /* ... and times per step                     */
  int solve_columns;         /* fastest columns per CTA of the column solves */
  int nsolve;                /* solve shapes timed (<= 4)                  */
  int solve_candidates[4];   /* their columns per CTA ...                  */
  double solve_candidate_ms[4]; /* ... and times per step                  */
} qg_tuning;
/* Times nsteps steps of a throw-away handle built from cfg for every
 * candidate batch depth, then, at the fastest depth, for every block shape
 * of the column solves (16, 32, 64 columns per CTA); returns the fastest
 * pair (set them in qg_config.levels_per_batch / solve_columns). */
int qg_autotune(const qg_config* cfg, int nsteps, qg_tuning* out);

/* Allocation-free variant of qg_fft_c2r.  No counterpart in the reference.
 * For callers that cannot allocate device memory: a host whose device memory
 * is fixed at start-up under a hard cap shared with other processes on the
 * GPU, or a host loop that cannot pay for cudaMalloc/cudaFree (cudaFree
 * synchronises the whole device and would stall work on other streams).
 * The caller owns both buffers; the call allocates nothing (no cudaMalloc,
 * cudaFree or allocating library routine).  FP64.
 *   kvar: device pointer, interleaved complex [nz][n][n/2+1] (read only),
 *         16-byte aligned (read as complex pairs)
 *   rvar: device pointer, double [nz][n][n+2], 8-byte aligned; the two
 *         padding values per row are 0
 * Both must be memory of the current device (or managed memory); anything
 * else, and a misaligned pointer, is QG_ERR_ARG before any launch.  A CUDA
 * error already pending from the caller's earlier work is left in place and
 * the call returns QG_ERR_CUDA without launching.
 * The (kx,y) intermediate lives in a file-scope 8 MiB static device array,
 * held by every GPU that loads the library until the process exits: n must
 * be a power of two in [16, 512] so that one level's plane fits, otherwise
 * QG_ERR_UNSUPPORTED; levels are transformed in chunks, so any nz works.
 * The work is queued on `stream` (a cudaStream_t; NULL = the legacy default
 * stream) and the call returns without synchronising.  The first call on a
 * device does a one-time set-up with that device current (device addresses
 * of the static arrays, twiddle upload, kernel attributes); make that first
 * call before any stream capture.  All calls share the one static scratch:
 * calls that overlap on the GPU (unordered streams) race, so order them on
 * one stream.  Each call writes every scratch element before reading it, so
 * nothing needs clearing between calls.  Errors: qg_last_error(NULL). */
int qg_fft_c2r_noalloc(const double* kvar, double* rvar, int n, int nz, void* stream);

/* Self-check of the mixed path's FP32 <-> FP64 conversions, which the FP64
 * column solves (elliptic.f90:145-460) and diagnostics do with integer
 * operations to keep the FP64 pipe free: every FP32 bit pattern and 2^32
 * FP64 patterns (all sign/exponent fields, rounding-boundary mantissas)
 * converted both ways on `device` and compared bit for bit with the
 * hardware conversions.  Returns the mismatch counts (0 and 0 expected).
 * Errors: qg_last_error(NULL). */
int qg_selftest_conversions(int device, long long* mismatches32, long long* mismatches64);

#ifdef __cplusplus
}
#endif
#endif /* QGYBJ_H */
