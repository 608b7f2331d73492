/*
 * fluidsim_gpu.h -- C ABI of the GB300 (sm_103a) implementation of the
 * fluidsim per-step hot path: Scharfetter-Gummel particle fluxes and RHS,
 * local-mean-energy coefficients, RK-Merson stages with the embedded error
 * estimate and adaptive dt, and the semi-implicit electrostatic Poisson solve.
 *
 * Every entry point replaces one Fortran subroutine (or one block of the main
 * loop) of the reference.  The Fortran caller binds them through
 * ISO_C_BINDING; plain pointers, sizes and POD structs only.
 *
 *   reference (file:line)                          entry point here
 *   ---------------------------------------------  -----------------------
 *   lapl_init  lapl_lib.F90:22-55                 \
 *   ptcl_init  ptcl_lib.F90:15-30                  > fs_create
 *   circ_init  circ_lib.F90:213-223               /
 *   ptcl_step  ptcl_lib.F90:32-97                  fs_ptcl_step
 *     (ptclEqn ptcl_lib.F90:99-550, rk_step ptcl_props.F90:30-140,
 *      circ_step circ_lib.F90:19-210, get_Flux ptcl_props.F90:142-165)
 *   lapl_solve lapl_lib.F90:57-121                 fs_lapl_solve
 *     (laplEqn :123-379, laplJ :381-609, dFdPh :611-636, KSPSolve :103)
 *   accept branch  main.F90:83-101                 fs_accept
 *   reject branch  main.F90:103-121                fs_reject
 *   main loop body main.F90:68-121                 fs_run (device-resident loop)
 *   module arrays ni/ne/nt/nm (ptcl_lib.F90:7-10),
 *     ph (lapl_lib.F90:14)                         fs_upload_state / fs_download_state
 *   maxval(ne)  main.F90:131                       fs_max_ne
 *   module arrays sig_pl/sig_mi/sig_or
 *     (sfc_lib.F90:7)                              fs_get_surface_charge / fs_set_surface_charge
 *   KSPDestroy/VecDestroy/MatDestroy main.F90:159  fs_destroy
 *
 * Array layout at the boundary is the reference's: Fortran column-major
 * (bx+2, by+2[, level]) with a one-cell ghost ring, x fastest, leading
 * dimension ld >= nx+2.  All field state lives in device memory owned by the
 * context between calls; host arrays are only borrowed during upload/download.
 *
 * Return values: FS_OK (0) or a negative FS_ERR_* code; fs_last_error() gives
 * the message.  No entry point calls exit/abort.  One host thread per context.
 */
#ifndef FLUIDSIM_GPU_H
#define FLUIDSIM_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FS_ABI_VERSION 1

/* error codes */
#define FS_OK                  0
#define FS_ERR_INVALID        -1   /* bad argument or configuration            */
#define FS_ERR_CUDA           -2   /* CUDA runtime error                        */
#define FS_ERR_NAN            -3   /* NaN in a RHS (ptcl_lib.F90:530-549) or in
                                      the Poisson RHS (lapl_lib.F90:376-378)    */
#define FS_ERR_NEG_DENSITY    -4   /* get_Te negative density stop
                                      (ptcl_props.F90:171-177)                  */
#define FS_ERR_MIN_DT         -5   /* minimum timestep stop (ptcl_lib.F90:68-72) */
#define FS_ERR_NOT_CONVERGED  -6   /* Krylov solve did not converge              */
#define FS_ERR_UNSUPPORTED    -7   /* option outside the implemented scope       */
#define FS_ERR_NOMEM          -8   /* device allocation failed                   */
#define FS_ERR_NO_DEVICE      -9   /* no CUDA device / extension not usable      */

/* fs_config.coef_mode */
#define FS_COEF_FITS   0   /* reference polynomial fits (ptcl_props.F90:182-429)   */
#define FS_COEF_TABLE  1   /* log-spaced table over mean energy, Arrhenius k_ir     */

/* fs_config.precision */
#define FS_PREC_FP64   0   /* plain FP64 path (the drop-in)                          */
#define FS_PREC_MIXED  1   /* FP32 flux/RHS and multigrid, FP64 accumulation         */

/* Run configuration.  Lengths in units of x0, voltage in units of ph0, time in
 * units of t0 (props.F90:33-37), i.e. the reference's nondimensional units. */
typedef struct fs_config {
    int32_t abi_version;    /* must be FS_ABI_VERSION                               */
    int32_t nx, ny;         /* interior nodes (g%nx, g%ny); one block: bx=nx, by=ny  */
    int32_t nspecies;       /* 3: ni, ne, nt ; 4: + metastables nm                   */
    int32_t coef_mode;      /* FS_COEF_*                                              */
    int32_t cyl;            /* 1: cylindrical r-weighting in y (props.F90:47)          */
    int32_t rf;             /* source (circ_lib.F90:26-50): 0 DC, 1 AC sin(pi t) through
                               the RC circuit, 2 and 3 the pulse shapes              */
    int32_t adaptive;       /* 1: PI dt controller + reject (reference)               */
                            /* 0: dt held fixed, attempts never rejected              */
    int32_t precision;      /* FS_PREC_*                                              */
    int32_t lapl_maxit;     /* Krylov iteration cap                                   */
    int32_t table_n;        /* table points (FS_COEF_TABLE)                           */
    int32_t mg_smooth;      /* red-black GS sweep pairs per V-cycle leg (default 2;   */
                            /* the FP64 solver's finest level pre-smooths with one */
                            /* pair fewer, at least one)                           */
    double  table_emin_ev;  /* table range in mean energy [eV]                        */
    double  table_emax_ev;
    double  kir_arrh_a;     /* Arrhenius ionisation prefactor [m^3/s] (table mode)    */
    double  kir_arrh_e;     /* Arrhenius activation energy [eV]                       */
    double  p_torr;         /* gas pressure (props.F90:41)                            */
    double  tg_k;           /* gas temperature (props.F90:40)                         */
    double  gam;            /* secondary emission coefficient (ptcl_props.F90:25)     */
    double  n_init;         /* uniform initial density of ptcl_init (props.F90:44)    */
    double  l, w, ew, gap;  /* g%l, g%w, g%ew, g%gap                                  */
    double  vl;             /* applied voltage Vmax (circ_init)                       */
    double  res;            /* circuit resistance (main.F90:43,286), nondim           */
    double  abs_tol;        /* RK-Merson error tolerances (ptcl_props.F90:35)         */
    double  rel_tol;
    double  dt_min;         /* minimum-dt stop (ptcl_lib.F90:68), reference 1.1e-12   */
    double  lapl_rtol;      /* Poisson relative residual ||A d + b|| / ||b||          */
} fs_config;

/* Mesh produced by the caller's g_init (props.F90:52-235). */
typedef struct fs_mesh {
    const double  *dx;      /* nx+1 : dx(i) = x(i+1) - x(i)                           */
    const double  *dlx;     /* nx   : dlx(i) = (dx(i+1) + dx(i)) / 2                  */
    const double  *dy;      /* ny+1                                                   */
    const double  *dly;     /* ny                                                     */
    const double  *r;       /* ny+2 : y node coordinates, g%r                          */
    const int32_t *type_x;  /* nx*ny column-major g%type_x(i,j) at (i-1)+(j-1)*nx     */
    const int32_t *type_y;  /* nx*ny column-major g%type_y                            */
} fs_mesh;

/* Derived physical constants (props.F90:24-47, ptcl_props.F90:5-25). */
typedef struct fs_constants {
    double pi, eps0, e, kb, me, x0, ph0, t0, wp02, w2;
    double tg, p, ninf, n_zero;
    double mi, mui, vi, Di, Dm, k_r, k_mp, k_2q, k_3q;
    double h_ir, h_ex, h_si, h_sc, gam;
    double nmin_nt;         /* energy-density floor n_zero/ph0/1e2 (ptcl_lib.F90:56)   */
    double cap;             /* circuit capacitance (circ_lib.F90:221)                 */
} fs_constants;

/* Per-step statistics filled by fs_run / fs_get_stats. */
typedef struct fs_stats {
    double  t;              /* g%t                                                    */
    double  dt;             /* g%dt                                                   */
    double  t_m;            /* min dielectric relaxation time of the last step        */
    double  ida, idc;       /* electrode currents of the last circ_step               */
    double  err_cur;        /* last RK-Merson error norm                              */
    double  lapl_relres;    /* last Poisson relative residual                         */
    int64_t steps;          /* accepted main-loop iterations (ts)                     */
    int64_t attempts;       /* RK attempts run (including rejected ones)              */
    int64_t rk_rejects;     /* attempts rejected by the error norm                    */
    int64_t lapl_rejects;   /* steps rejected because the Poisson solve failed        */
    int64_t lapl_iters;     /* total Krylov iterations                                */
    int32_t last_lapl_iters;
    int32_t lerr;           /* lerr of the last Poisson solve                         */
    double  dt_step;        /* dt of the last accepted RK attempt (before the
                               controller's update of g%dt, ptcl_lib.F90:59-95)       */
} fs_stats;

typedef struct fs_ctx fs_ctx;

/* Library identification: ABI version, and the device it runs on. */
int32_t fs_abi_version(void);

/* Derived constants for a configuration (host only, no device needed). */
int fs_get_constants(const fs_config *cfg, fs_constants *out);

/* Coefficient table (FS_COEF_TABLE) as the device uses it: ncoef rows of
 * table_n values, rows in the order mue, De, k_ir, k_ex, nu, beta, k_sc, k_si.
 * Host only.  out must hold 8*table_n doubles. */
int fs_build_table(const fs_config *cfg, double *out);

/* lapl_init + ptcl_init + circ_init: allocate all device state, set the
 * reference's uniform initial state (ni=ne=nm=n_init, nt=ne*Tg*kb/e/ph0,
 * ph=ph_mi=0, t=0), Vmax=Vd=vl.  dt is set with fs_set_time. */
int fs_create(const fs_config *cfg, const fs_mesh *mesh, fs_ctx **out);
void fs_destroy(fs_ctx *ctx);

/* Message of the last error on ctx (or of the last failed fs_create when
 * ctx is NULL). */
const char *fs_last_error(const fs_ctx *ctx);

/* g%t and g%dt. */
int fs_set_time(fs_ctx *ctx, double t, double dt);

/* The rest of the step state a restart needs (with the three-level densities,
 * phi, g%t, g%dt, the circuit and the wall charge): ptcl_step's err_prev
 * (ptcl_lib.F90:11), the PI controller's memory, and main's step counter ts
 * (main.F90:12; ptcl_step runs once ts > 1).  A context restored from these
 * continues bit for bit as the one they were read from. */
int fs_get_controller(fs_ctx *ctx, double *err_prev, int64_t *ts);
int fs_set_controller(fs_ctx *ctx, double err_prev, int64_t ts);

/* Module arrays <-> device.  Species arrays are (ld, ny+2, nlev) column-major
 * like ni(bx+2,by+2,3); nlev = 3 (all RK levels) or 1 (the one array is used
 * for every level).  nm may be NULL when nspecies == 3.  ph is (ld, ny+2).
 * ph_mi (lapl_lib.F90:14) is set equal to ph on upload. */
int fs_upload_state(fs_ctx *ctx, const double *ni, const double *ne,
                    const double *nt, const double *nm, const double *ph,
                    int32_t ld, int32_t nlev);
int fs_download_state(fs_ctx *ctx, double *ni, double *ne, double *nt,
                      double *nm, double *ph, int32_t ld, int32_t nlev);

/* ptcl_step(g, ph, Em) with Em = 0: five RK-Merson stages, restarting on
 * rejection, then the PI controller.  dt_inout is g%dt (in: the dt to use; out:
 * the controller's next dt).  t_m_out: min over stage-5 cells of
 * 1/(mue*ne + mui*ni), starting from 1e9 (main.F90:74).  attempts_out: RK
 * attempts including rejected ones.  Any output pointer may be NULL. */
int fs_ptcl_step(fs_ctx *ctx, double *dt_inout, double *t_m_out,
                 double *ida_out, double *idc_out, int32_t *attempts_out);

/* lapl_solve(g, ne(:,:,1), ni(:,:,1), nt(:,:,1), sig, lerr): assemble the
 * semi-implicit correction system with g%dt = dt, solve it to cfg->lapl_rtol
 * (relative to the right-hand side's norm, as the reference's KSP; the
 * multigrid-preconditioned CG starts from the previous solve's correction
 * scaled to minimise the initial residual, see fs_get_lapl_guess), and on
 * success ph += delta, ph_mi = ph.  lerr_out = 0 converged, 1 not (the caller
 * then rejects the step, main.F90:102-121). */
int fs_lapl_solve(fs_ctx *ctx, double dt, int32_t *lerr_out,
                  int32_t *iters_out, double *relres_out);

/* Level rotation of main.F90:83-101 (accept: t += dt, n3 <- n2, n2 <- n1,
 * sig_or <- sig_mi, sig_mi <- sig_pl) and main.F90:103-121 (reject: dt /= 2,
 * n1 <- n3, n2 <- n3, sig_pl = sig_mi = sig_or). */
int fs_accept(fs_ctx *ctx);
int fs_reject(fs_ctx *ctx);

/* sfc_lib's module arrays sig_pl, sig_mi, sig_or (sfc_lib.F90:7): the
 * surface charge of the dielectric wall, nx+2 entries each with Fortran index
 * i at [i-1]; a NULL pointer skips that array.  A mesh whose last row has
 * type_y == 3 nodes (the reference's rwall, props.F90:191-195) turns the
 * wall on: fs_ptcl_step advances the charge with sfc_step's Merson stages
 * (sfc_lib.F90:19-80) and fs_lapl_solve reads sig_pl as lapl_solve's sig.
 * The charge starts at zero (sfc_init, sfc_lib.F90:84-90).  FP64 contexts. */
/* circ_lib's module scalars (circ_lib.F90:8): get writes Vd_pl, Vd_mi, Vd_or
 * and the source voltage Vsrc of the last particle step into v4[0..3]; set
 * takes Vd_pl, Vd_mi, Vd_or from v3[0..2] (a restart).  Vd_pl is what the
 * reference writes to vd.dat. */
int fs_get_circuit(fs_ctx *ctx, double *v4);
int fs_set_circuit(fs_ctx *ctx, const double *v3);

int fs_get_surface_charge(fs_ctx *ctx, double *sig_pl, double *sig_mi, double *sig_or);
int fs_set_surface_charge(fs_ctx *ctx, const double *sig_pl, const double *sig_mi,
                          const double *sig_or);

/* The Poisson solver's warm-start vector: the previous solve's correction of
 * phi, which (scaled by the factor that minimises the initial residual) is
 * the next solve's initial guess.  Part of the restart state, so that a
 * restored FP64 context continues bit for bit.  ld >= bx+2 doubles per row,
 * (by+2) rows, the reference's layout; the ghost ring is zero.  In a mixed-
 * precision context the vector is its float-float iterate (xh + xl).  No
 * reference counterpart (the reference's KSP starts from zero,
 * lapl_lib.F90:52). */
int fs_get_lapl_guess(fs_ctx *ctx, double *d, int32_t ld);
int fs_set_lapl_guess(fs_ctx *ctx, const double *d, int32_t ld);

/* nsteps iterations of the main.F90:68-121 loop body on the device:
 * ptcl_step (when ts > 1), lapl_solve, accept or reject.  Host work per
 * iteration is limited to reading back the control scalars. */
int fs_run(fs_ctx *ctx, int32_t nsteps, fs_stats *stats_out);

int fs_get_stats(fs_ctx *ctx, fs_stats *out);

/* maxval(ne) over the whole module array -- every level, ghosts included
 * (main.F90:131).  NaN entries are skipped (the maximum of the other values
 * is returned; an all-NaN array gives -inf): the ptcl_step and lapl_solve
 * entry points report NaN densities themselves (FS_ERR_NAN). */
int fs_max_ne(fs_ctx *ctx, double *out);

/* ---- diagnostics with no counterpart in the reference ------------------- */

/* The cudaStream_t all of ctx's work is issued on (for CUDA-event timing). */
void *fs_stream(fs_ctx *ctx);

/* Per-launch CUDA-event timing of kernel classes: 0 RK stage, 1 Poisson
 * assembly, 2 multigrid smoothing, 3 multigrid transfer, 4 bottom solve,
 * 5 CG vector kernels, 6 coarse operators, 7 control kernels.
 * fs_profile(ctx, mask) resets the totals and times the classes whose bit
 * (1 << class) is set in mask (0 turns it off).  Timing any of classes 2-5
 * runs the Krylov loop from the host instead of as one CUDA graph.
 * fs_profile_read returns total milliseconds and launch counts of the first
 * n classes. */
#define FS_PROF_NCLASS 8   /* class 7: small control kernels */
int fs_profile(fs_ctx *ctx, int32_t enable);
int fs_profile_read(fs_ctx *ctx, double *ms_out, int64_t *launches_out, int32_t n);

/* Number of kernels ctx has launched since fs_create. */
int64_t fs_launch_count(fs_ctx *ctx);

/* Tile shape of the FP64 RK stage kernel (nodes per CTA): 32 x 8 (the
 * default), 32 x 4 or 64 x 4.  Results do not depend on it (fixed-order
 * sums per tile, then over tiles in index order: the sums differ in their
 * last bits between shapes, not between runs); an autotuner may pick the
 * fastest per grid size.  A fused batch (fs_batch_run_fused) launches each
 * stage once per tile shape present.  64 x 4 takes 3 species. */
int fs_set_stage_tile(fs_ctx *ctx, int32_t bx, int32_t by);

/* Smoother of the Poisson solvers' V-cycles: -1 (the default) chosen from the
 * mesh, 0 point red-black Gauss-Seidel, 1 zebra x-line Gauss-Seidel (each row
 * of one parity solved exactly along x: tridiagonal, chunked Thomas plus
 * cyclic reduction, one CTA per row) on the finest level.  The default takes
 * x-line smoothing where the middle column's x faces conduct more than twice
 * as well as its y faces (a mesh anisotropic in the bulk, e.g. a square
 * domain on a grid with nx > ny), point smoothing with the electrode-strip
 * sweeps otherwise.  Rows of up to 4715 nodes on the FP64 path,
 * 9680 on the mixed one (else mode 1 gives FS_ERR_UNSUPPORTED and mode -1
 * stays with point smoothing).  Replaces the
 * solvers' CUDA graphs at their next use.  No reference counterpart: PETSc's
 * KSPSetFromOptions run-time solver choice (lapl_lib.F90:50-54). */
int fs_set_line_smoother(fs_ctx *ctx, int32_t mode);
/* 1 while the V-cycles use x-line smoothing, 0 point; -1 for a null context. */
int fs_line_smoother(fs_ctx *ctx);

/* FP64 issue rate of device `device`: fused multiply-adds per second of a
 * DFMA microbenchmark (4 to 16 CTAs per SM, 8 or 16 independent chains per
 * thread, the best of all shapes and of 5 timed launches each, CUDA
 * events).  The roof of the FP64-issue-bound kernels (RK stage, Poisson
 * assembly); FP64 FLOP/s = 2 x this.  Needs no context; changes no device
 * setting. */
int fs_fp64_rate(int32_t device, double *dfma_per_s);

/* The FP64 kernels' elementary functions on n host values, for accuracy
 * tests: fn 0 the table-driven logarithm and 1 the table-driven exponential
 * the FP64 kernels use, 2 and 3 CUDA's log and exp.  Runs on the current
 * device; allocates and frees its own device buffers. */
int fs_math_eval(int32_t fn, const double *x, double *y, int64_t n);

/* One 3x3 convolution (zero padding) of the learned preconditioner's network
 * through its tcgen05 tensor-core path, on host arrays, for tests: in1
 * [B][H][W][c1] and in2 [B][H][W][c2] (the decoder's concatenation; NULL
 * when c2 = 0) as BF16 bit patterns, w [9][cout][c1 + c2] (tap = 3 (dy+1) +
 * (dx+1)) and bias [cout] in FP32.  mode 0: out is FP32 [B][H][W][cout],
 * bias added; mode 1: out is BF16 bit patterns, bias and ReLU applied.
 * Channels: c1, c2 multiples of 16 (of 64 above 64), cout a multiple of 16
 * up to 128.
 * Returns 0, or a negative code (-1 bad arguments, -2 no device memory or
 * shared memory over the limit, -3 TMA descriptor, -6 a bounded wait ran
 * out, -100 - e for the CUDA error e). */
int fs_conv3x3_tc(int32_t B, int32_t H, int32_t W, int32_t c1, int32_t c2, int32_t cout,
                  const uint16_t *in1, const uint16_t *in2, const float *w, const float *bias,
                  int32_t mode, void *out);

/* Measurement of the bound of those convolutions (no counterpart in the
 * reference): SM cycles per tcgen05.mma instruction (M = 128, N = n, K = 16,
 * BF16 -> FP32, operands in shared memory) issued back to back by one
 * thread, on the current device, clock64-timed, no clocks or settings
 * touched.  n a multiple of 16 in 16..256.  Returns 0, -1 bad arguments, -2
 * set-up failed, -3 launch failed, -6 the bounded wait ran out. */
int fs_mma_rate(int32_t n, double *cycles_per_mma);

/* fs_max_ne for callers that may not allocate device memory after set-up
 * (this entry point has no counterpart in the reference): same result as
 * fs_max_ne, with its scratch in a fixed device array of the library instead
 * of per-call memory from the stream-ordered allocator.  The array holds the
 * partial maxima of at most 33,554,432 values -- the three RK levels of n_e
 * with ghost rings, i.e. grids up to 3342 x 3342; larger contexts get
 * FS_ERR_INVALID.  The first call on a device looks the array up and must
 * come before any stream capture.  Every call shares the array: calls whose
 * GPU work overlaps race on it.  ctx's device must be current. */
int fs_max_ne_noalloc(fs_ctx *ctx, double *out);

/* The reference's output files (props.F90:239-320 set-up, writeOut
 * main.F90:297-333), written into directory dir: init = 1 creates
 * meshx.dat / meshy.dat and empties f1..f5.dat, time.dat, vd.dat, ida.dat,
 * idc.dat, dt.dat, flx.dat; init = 0 appends the current state -- raw native
 * FP64, same units and layout as the reference, so its save.py reads them.
 * With three species f5.dat gets zeros; flx.dat (the EM flux) gets 0.
 * init = 0 returns once the record is queued: a kernel on the context's
 * stream converts the fields (the state as of the call), a stream of the
 * writer's own copies the result to pinned host memory, and a writer thread
 * appends it to the files while the caller keeps stepping.  The first
 * init = 0 call allocates 5 nx ny doubles on the device and as much pinned
 * host memory.  One record is in flight at a time; the next
 * fs_write_output, fs_output_wait and fs_destroy wait for it, and a write
 * error surfaces from whichever of the first two comes next. */
int fs_write_output(fs_ctx *ctx, const char *dir, int32_t init);
/* Wait until the record in flight is on disk; its status. */
int fs_output_wait(fs_ctx *ctx);

/* ---- Many independent discharges (voltage / pressure sweeps).  No single
 * counterpart in the reference, which runs one discharge per invocation
 * (main.F90) and builds I-V curves from many runs.  Advances the n contexts
 * concurrently with nthreads host threads (one discharge per thread at a
 * time, largest grids first): each runs `steps` main-loop iterations as
 * fs_run does, stopping early once its time reaches t_end (t_end <= 0: no
 * limit).  Contexts keep their own adaptive dt and convergence.  out[i]
 * (may be NULL) gets instance i's statistics -- its electrode currents are
 * the last step's -- and rc_out[i] (may be NULL) its return code; the call
 * returns the first nonzero code, or FS_OK.  No context may be used by
 * another thread during the call. */
int fs_batch_run(fs_ctx **ctx, int32_t n, int32_t steps, double t_end, int32_t nthreads, fs_stats *out,
                 int32_t *rc_out);

/* fs_batch_run with the RK stages of the discharges fused: every round runs
 * one RK-Merson attempt of each unfinished discharge (those past the two
 * Poisson-only start-up iterations) as ONE launch per stage (per stage tile
 * shape present, see fs_set_stage_tile) over the tiles of all of them and one
 * launch of all their step-size controllers, each
 * discharge with its own dt and its own accept/reject; then, nthreads host
 * threads in parallel, the Poisson solve (its CUDA graph) and the level
 * rotation of every discharge whose attempt was accepted; a rejected attempt
 * is retried in the next round.  The discharges are split into groups of about
 * equal node count (8 by default, FS_FUSED_GROUPS=1..16 in the environment),
 * each with its own rounds on its own host thread and stream, so that one
 * group's Poisson solves overlap another's stages.  Each discharge takes
 * exactly the steps it takes alone.  FP64 contexts with 3 species, DC source,
 * no dielectric wall, all on one device (else FS_ERR_UNSUPPORTED). */
int fs_batch_run_fused(fs_ctx **ctx, int32_t n, int32_t steps, double t_end, int32_t nthreads, fs_stats *out,
                       int32_t *rc_out);

/* ---- Learned Poisson preconditioner (FS_PREC_MIXED contexts only).  No
 * counterpart in the reference, which hands the system to PETSc
 * (lapl_lib.F90:83-104).  A BF16 convolutional network (a four-level U-Net,
 * 16 to 64 channels, 258,528 parameters, on the tcgen05 tensor cores with
 * FP32 accumulation) on the fine grid.  In a CG iteration that runs it, the
 * preconditioner is z = V(r) + N(s): V the multigrid V-cycle, s = r - M V(r)
 * the residual it leaves, N the network's estimate of the correction a second
 * V-cycle would add for s (inputs: s, the two face-coupling shares of the
 * diagonal -- the grid-spacing map -- and the net charge density).  The
 * flexible CG tolerates the nonlinear preconditioner; the refinement of the
 * mixed solver (the true residual, to FP64 accuracy) judges convergence, so
 * every solve reaches lapl_rtol exactly as without the network, and after 3
 * stalled iterations (inner residual falling by less than 4x) the network is
 * switched off for the rest of that solve.  One black-red Gauss-Seidel pass
 * follows the correction.  In mode 1 the library times
 * every solve and runs each next one with whichever of the two -- with or
 * without the network -- has been faster on average (a stalled solve counts
 * double), trying the other one every 25 solves at first (the interval
 * doubling to 400 while the other keeps losing, and 400 at once while the
 * network is more than twice as slow).
 *
 * fs_lpc_init      allocate the network (seeded He init), its training state
 *                  and up to max_samples stored training pairs (full grids);
 *                  training batches of up to max_batch crops of crop x crop
 *                  cells (a multiple of 8; 0: 128; at most the grid).
 * fs_lpc_harvest   after fs_lapl_solve: re-solve the step's assembled system
 *                  with the plain multigrid-PCG, take up to per_solve of its
 *                  residuals r, and store for each the pair (features of
 *                  s = r - M V(r), the second V-cycle's correction V(s)).
 *                  phi is not changed.
 * fs_lpc_train     iters Adam steps (lr) on batches of random crops of the
 *                  stored pairs (seeded); loss_hist (may be NULL) gets each
 *                  step's training loss.
 * fs_lpc_use       0: plain multigrid-PCG; 1: the network where it pays off
 *                  (see above); 2: the network in every solve.
 * fs_lpc_weights   copy the FP32 parameters out (to_device = 0) or in
 *                  (to_device = 1, Adam state reset); n must equal nparam.
 * fs_lpc_grad      loss and parameter gradient for given inputs on batch
 *                  full grids: feat [batch][h][w][4], tgt [batch][h][w], mask
 *                  [h][w]; pred (may be NULL) gets the predictions
 *                  [batch][h][w].
 * fs_lpc_info      NN grid size (h, w: the grid padded to multiples of 8),
 *                  stored pairs, parameter count; off = 1 if the last solve
 *                  switched the network off; solves since fs_lpc_use turned
 *                  the network on and how many of them ran it (any output
 *                  pointer may be NULL). */
int fs_lpc_init(fs_ctx *ctx, int32_t crop, int32_t max_batch, int32_t max_samples, uint64_t seed);
int fs_lpc_harvest(fs_ctx *ctx, int32_t per_solve, int32_t *added);
int fs_lpc_train(fs_ctx *ctx, int32_t iters, int32_t batch, float lr, uint64_t seed, float *loss_hist);
int fs_lpc_use(fs_ctx *ctx, int32_t on);
int fs_lpc_weights(fs_ctx *ctx, float *w, int64_t n, int32_t to_device);
int fs_lpc_grad(fs_ctx *ctx, const float *feat, const float *tgt, const float *mask, int32_t batch, float *grad,
                float *loss, float *pred);
int fs_lpc_info(fs_ctx *ctx, int32_t *h, int32_t *w, int32_t *nsamples, int64_t *nparam, int32_t *off,
                int64_t *solves, int64_t *nn_solves);

#ifdef __cplusplus
}
#endif
#endif /* FLUIDSIM_GPU_H */
