/*
 * fs_oracle.h -- CPU oracle for the fluidsim hot path.  TEST INFRASTRUCTURE:
 * only tests/, __graft_entry__.smoke() and bench.py (cpu_baseline and the
 * reference arm) may load it, and only as the checker / the timed CPU
 * baseline.  The product never links or calls it.
 *
 * It is a line-by-line C++ restatement of the reference Fortran routines, in
 * their operation order, on the reference's 1-based column-major arrays:
 *   ptcl_props.F90:5-25,30-429 ; ptcl_lib.F90:15-550 ; circ_lib.F90:19-223 ;
 *   lapl_lib.F90:57-636 ; props.F90:24-47 ; main.F90:68-121.
 * PETSc's KSPSolve (lapl_lib.F90:103) is replaced by the oracle's own FP64
 * solvers: a banded LU (exact to rounding) or BiCGStab with block-Jacobi
 * ILU(0), the PETSc default preconditioner with one block per thread.
 *
 * Parity status: UNPINNED apart from the coefficient fits get_mue, get_De,
 * get_Dt and get_nu, which tests/test_golden_coef.py checks against the
 * reference's own Python copies of them (coeftest.py, wvgAC.py).  The
 * reference has no tests, golden vectors or fixtures, and it cannot be built
 * here or on the GPU host (no Fortran compiler, MPI or PETSc), so the rest of
 * this restatement is checked against analytic known-answer tests
 * (tests/test_oracle_kat.py and the wall and circuit tests).
 *
 * The interface mirrors include/fluidsim_gpu.h entry for entry, prefixed or_.
 */
#ifndef FS_ORACLE_H
#define FS_ORACLE_H
#include "../include/fluidsim_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct or_ctx or_ctx;

#define OR_SOLVER_DIRECT   0   /* banded LU, no pivoting                          */
#define OR_SOLVER_BICGSTAB 1   /* BiCGStab + block-Jacobi ILU(0), to cfg->lapl_rtol */

int or_get_constants(const fs_config *cfg, fs_constants *out);
int or_build_table(const fs_config *cfg, double *out);
int or_create(const fs_config *cfg, const fs_mesh *mesh, int32_t solver, or_ctx **out);
void or_destroy(or_ctx *ctx);
const char *or_last_error(const or_ctx *ctx);
int or_set_threads(int32_t nthreads);
int or_set_time(or_ctx *ctx, double t, double dt);
int or_get_controller(or_ctx *ctx, double *err_prev, int64_t *ts);
int or_set_controller(or_ctx *ctx, double err_prev, int64_t ts);
int or_upload_state(or_ctx *ctx, const double *ni, const double *ne,
                    const double *nt, const double *nm, const double *ph,
                    int32_t ld, int32_t nlev);
int or_download_state(or_ctx *ctx, double *ni, double *ne, double *nt,
                      double *nm, double *ph, int32_t ld, int32_t nlev);
/* k?(:,:,stage) of the last ptcl_step, (ld, ny+2, 5) per species. */
int or_download_k(or_ctx *ctx, double *ki, double *ke, double *kt, double *km, int32_t ld);
int or_ptcl_step(or_ctx *ctx, double *dt_inout, double *t_m_out,
                 double *ida_out, double *idc_out, int32_t *attempts_out);
int or_lapl_solve(or_ctx *ctx, double dt, int32_t *lerr_out,
                  int32_t *iters_out, double *relres_out);
/* Assemble only: b (nx*ny, the laplEqn value per row) and the 5 row entries of
 * A per interior node in the order west, east, south, north, centre
 * (0 where the reference sets no column). */
int or_lapl_assemble(or_ctx *ctx, double dt, double *b, double *a5);
/* sfc_lib's sig_pl, sig_mi, sig_or (bx+2 entries each; NULL skips one). */
int or_get_surface_charge(or_ctx *ctx, double *sig_pl, double *sig_mi, double *sig_or);
int or_set_surface_charge(or_ctx *ctx, const double *sig_pl, const double *sig_mi,
                          const double *sig_or);
/* circ_lib's Vd_pl, Vd_mi, Vd_or and the last source voltage Vsrc (get: 4
 * values; set: the first 3). */
int or_get_circuit(or_ctx *ctx, double *v4);
int or_set_circuit(or_ctx *ctx, const double *v3);
int or_accept(or_ctx *ctx);
int or_reject(or_ctx *ctx);
int or_run(or_ctx *ctx, int32_t nsteps, fs_stats *stats_out);
int or_get_stats(or_ctx *ctx, fs_stats *out);

/* Single-routine entry points for known-answer tests. */
double or_get_flux(double E, double dh, int32_t q, double mu, double D,
                   double nl, double nr);
double or_dfdph(double E_pl, double E_mi, int32_t q, double mu, double D,
                double dx, double n1, double n2);
/* coefficient by index (0 mue,1 De,2 k_ir,3 k_ex,4 nu,5 beta,6 k_sc,7 k_si)
 * at nondimensional mean energy T, through the configured mode; 8 get_mut and
 * 9 get_Dt, always from the fits. */
double or_coef(const or_ctx *ctx, int32_t which, double T);

#ifdef __cplusplus
}
#endif
#endif
