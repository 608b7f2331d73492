// fs_internal.h -- device layout, kernel parameters and context of the CUDA
// implementation behind include/fluidsim_gpu.h.
//
// Device field layout: every 2D field is an FP64 (or FP32) array of
// (ny+2) rows of `pitch` elements; element (gi, gj) -- 0-based, ghost ring
// included, gi = Fortran i-1 -- lives at gj*pitch + gi.  pitch is nx+2
// rounded up to 32 elements so rows start on 256-byte boundaries.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/fluidsim_gpu.h"
#include "fs_fits.h"

#define FS_MAX_SPECIES 4
#define FS_NBUF 5            // level/stage buffers per species
#define FS_TAB_STRIDE 16     // doubles per table node: 8 values + 8 slopes
#define FS_MG_MAX_LEVELS 16

// status bits raised by kernels (Ctrl::status)
#define FS_ST_NEG_DENSITY 1u
#define FS_ST_NAN 2u
#define FS_ST_DFDPH_NAN 4u
#define FS_ST_BNAN 8u

// Physics and mesh constants passed by value to the particle and assembly kernels.
struct PhysParams {
    int nx, ny, pitch, nspecies, cyl;
    int ntab;
    double ph0, e, pi, me, t0, x0;
    double mui, Di, vi, Dm, gam, ninf, tg, kb, mi, inv_mi;
    double h_ir, h_ex, h_si, k_mp, k_r, k_2q, k_3q;
    double nmin[FS_MAX_SPECIES];   // floors: n_zero, n_zero, n_zero/ph0/1e2, n_zero
    double abs_tol, rel_tol;
    double lemin, inv_h;           // table abscissa: ln(emin), (n-1)/ln(emax/emin)
    double ve_coef;                // (16 e ph0)/(3 pi me): ve = sqrt(ve_coef*Te)*t0/x0
    double tg_term;                // Tg*kb/e/ph0 (ptcl_lib.F90:508)
    double e100;                   // exp(-100): the SG exponent clamp
    int fits;                      // coefficients from the fits per node (FS_COEF_FITS) instead of the table
    FitEval fit;
};

// FP32 copies of the constants the mixed-precision kernels use, formed once on
// the host so that no kernel converts or divides FP64 parameters per thread.
struct PhysF {
    float ph0, ln_ph0, mui, vi, gam, Di, mui_Di, ve_c, t0_x0, Dm, ninf, me_mi, tg_term;
    float h_ir, h_ex, h_si, k_mp, k_r, k_2q, k_3q_ninf2;
    float lemin, inv_h, ntab_m1;
    float abs_tol, rel_tol;
    float nmin[FS_MAX_SPECIES];
};

// FP32 copy of the mesh arrays (same layout as MeshDev's blob).
struct MeshF {
    const float *dx, *dy, *inv_dx, *inv_dy, *dlx, *dly, *inv_dlx, *inv_dly, *r;
};

// Mesh arrays on the device (all FP64, 0-based).
struct MeshDev {
    const double *dx, *dy;         // nx+1, ny+1: face spacings (Fortran dx(1..nx+1))
    const double *inv_dx, *inv_dy;
    const double *dlx, *dly;       // nx, ny: control-volume widths of interior nodes 1..n
    const double *inv_dlx, *inv_dly;
    const double *r;               // ny+2
    const int8_t *tx, *ty;         // (nx, ny) row-major by gj: tx[(gj-1)*nx + gi-1]
    const double *dr_a, *dr_c;     // per row gj (ny+2): current weights of circ_step
};

// Device-resident control block (one per context).
struct Ctrl {
    double dt;            // g%dt
    double err_prev;      // ptcl_lib.F90:11
    double err_cur;
    double t_m;           // running min over stage-5 cells
    double ida, idc;
    double scfac;
    double dt_step;       // dt of the last attempt, before the controller's update
    unsigned int status;  // FS_ST_* bits
    int rejected;         // last attempt rejected by the error norm
    int min_dt;           // dt fell to dt_min
    int lpc_stalls;       // mixed solver: stalled iterations with the learned correction
    // Krylov scalars
    double rz, rz_old, pq, alpha, beta, rnorm2, bnorm2, relres;
    int cg_done, cg_iters, cg_fail, pad2;
    double r0in2;              // mixed solver: inner residual norm^2 at the last refinement
    int inner_it, refine;      // mixed solver: inner iterations since it, refinement due
    double rr_prev;            // mixed solver: previous inner residual norm^2
    double spare[2];           // [0]: step length of the learned correction; [1]: FP64 solver's warm-start scale
    int lpc_off;               // learned correction switched off for this solve (stall)
    int cgm_restarted;         // mixed solver: the last refinement restarted the search direction
    double vd_pl, vd_mi;       // electrode voltage of the RC circuit (AC source, circ_lib.F90:158-174)
    double kv[6];              // its Merson slopes kv(1..5)
    unsigned int counter[8];   // last-block-done counters of grid reductions
    double host_result;        // host-side landing slot of single-value results
};

// One species' buffers.
struct SpeciesBufs {
    double *buf[FS_NBUF];
    double *k[3];           // k1, k3, k4
};

// Multigrid level (FP32 mirror, mixed precision).
struct MGLevelF {
    int nx, ny, pitch;
    float *mc, *ce, *cn, *extra, *inv_mc;
    float *rhs, *x, *res;
    float *xd;              // iterate after the fused down-smoothing (read by the fused up kernel)
};

// Multigrid level (FP64 plain path).
struct MGLevel {
    int nx, ny, pitch;      // interior size; fields are (ny+2) x pitch with ghost ring
    double *mc, *ce, *cn, *extra, *inv_mc;
    double *rhs, *x, *res;
    double *xd;             // iterate after the fused down-smoothing (read by the fused up kernel)
};

// Kernel classes timed by the optional per-launch event profiler.
enum ProfClass { PROF_STAGE = 0, PROF_ASSEMBLE, PROF_SMOOTH, PROF_TRANSFER, PROF_BOTTOM, PROF_CG,
                 PROF_COARSEN, PROF_OTHER, PROF_NCLASS };

struct ProfPair {
    cudaEvent_t a, b;
    int cls;
    int closed;
};

struct fs_ctx {
    fs_config cfg;
    fs_constants k;
    PhysParams pp;
    int nx, ny, pitch;
    size_t field_elems;          // (ny+2)*pitch
    int device;
    int nsm;                     // multiprocessors of the device
    cudaStream_t stream;
    std::string err;

    // mesh
    double *d_mesh_blob;
    int8_t *d_types;
    MeshDev mesh;
    std::vector<double> h_dr_a, h_dr_c;
    std::vector<int32_t> h_tx, h_ty;
    std::vector<double> h_r;
    std::vector<double> h_x, h_y;   // node coordinates, ghost ring included (x(1) = y(1) = 0)
    struct fs_output *out;          // asynchronous output writer (fs_output.cpp), on first use

    // table
    double *d_tab;

    // fields
    SpeciesBufs sp[FS_MAX_SPECIES];
    int lev[3];                  // buffer index holding Fortran level 1,2,3 (same for all species)
    double *ph, *ph_mi;
    double *d_part;              // per-block partial sums (4 species)
    int nblk_stage;              // blocks of one stage launch
    int stage_bx, stage_by;      // its tile shape (FP64 path)
    double *d_rows;              // per-row current contributions (2*(ny+2))
    // sfc_lib state (dielectric wall, type_y == 3 on the last row): three
    // slots of nx+2 charges (Fortran sig(i) at [i-1]) holding sig_pl, sig_mi,
    // sig_or by sig_slot[0..2], then the five Merson slopes ks(:, stage)
    double *d_sig;
    int sig_slot[3];
    int rwall;
    // per-step face data (phi is frozen during ptcl_step): field E and the
    // ion SG flux coefficients, flux = cl*n_left - cr*n_right, for the x face
    // east of node (gi,gj) and the y face north of it
    // and of dFdPh, dF/dv = dl*n_left + dr*n_right (lapl_lib.F90:611-636)
    double *fx_e, *fx_cl, *fx_cr, *fy_e, *fy_cl, *fy_cr;
    double *fx_dl, *fx_dr, *fy_dl, *fy_dr;
    int faces_valid;             // face data matches the current phi
    Ctrl *d_ctrl;
    Ctrl *h_ctrl;                // pinned mirror

    // Poisson
    MGLevel mg[FS_MG_MAX_LEVELS];
    int mg_nlev;
    int mg_fused;                // coarse launched levels use the fused kernels
    int mg_lb, mg_dl;            // first level of the one-CTA bottom solver; its dense level
    int strip_kl, strip_kr;      // electrode strips of the finest level: columns 1..kl and kr..nx
    int strip_w;                 // their snapshot's row width (StripSnap)
    int mg_xline;                // V-cycles smooth with zebra x-line sweeps (k_xline)
    int mg_aniso;                // the mesh is anisotropic beyond the electrode strips
    int mg_xline_mode;           // 0: chosen from the mesh (fs_mg_strips), 1: point, 2: x-line
    double *strip_snap64;        // the snapshot, FP64 solver
    float *strip_snap32;         // the snapshot, FP32 finest level (mixed solver, FP64 solver with mg_lf = 0)
    // FP64 solver: levels mg_lf.. of its preconditioner run in FP32 (mg_lf =
    // mg_nlev: none; 0: all), on these arrays, with the FP32 dense inverse d_ainvc
    int mg_lf;
    MGLevelF mgc[FS_MG_MAX_LEVELS];
    float *d_ainvc;
    double *d_ainv64;            // dense inverse of level mg_dl (FP64 solver)
    float *d_ainv32;             // dense inverse of level mg_dl (mixed solver)
    double *p, *q, *z, *r, *xs, *bs, *dinv;  // CG vectors: solution xs, rhs D*b, 1/D
    int dinv_done;               // 1/D (a property of the mesh) has been written
    double *d_cg_part;
    int cg_nblk;
    // CG loop as a CUDA graph with a conditional WHILE node (built on first use)
    cudaGraph_t cg_graph;
    cudaGraphExec_t cg_exec;
    int cg_graph_built;
    int cg_body_kernels;         // kernels per loop iteration (launch accounting)

    // per-launch event profiler: bitmask of the timed kernel classes (0 = off)
    int prof_on;
    int64_t launches;            // kernels launched by this context
    std::vector<ProfPair> prof_pending, prof_free;
    double prof_ms[PROF_NCLASS];
    int64_t prof_n[PROF_NCLASS];

    // mixed precision (FS_PREC_MIXED): FP32 log-density companions of the
    // state buffers, FP32 stage derivatives, FP32 face data and table, FP32
    // multigrid hierarchy
    int mixed;
    PhysF pf;
    MeshF meshf;
    float *d_meshf;
    float *lbuf[FS_MAX_SPECIES][FS_NBUF];
    float *k32[FS_MAX_SPECIES][3];
    float *f32[10];              // fx_e, fx_cl, fx_cr, fx_dl, fx_dr, fy_e, fy_cl, fy_cr, fy_dl, fy_dr
    float *d_tab32;
    MGLevelF mgf[FS_MG_MAX_LEVELS];
    float *p32, *q32, *w32;      // FP32 inner CG vectors (w = M z)
    float *xh32, *xl32, *dinv32; // the mixed CG's iterate as a float-float pair; 1/D in FP32
    // learned preconditioner (fs_lpc.cu): network on the fine grid
    struct LpcState *lpc;
    int lpc_on, pad_lpc;
    // choice between the two solvers, judged on measured solve time
    double lpc_t_nn, lpc_t_plain;   // moving averages of the solve time (ms), < 0: none yet
    int lpc_use_next, lpc_since_probe;
    int64_t lpc_solves, lpc_nn_solves;   // solves since fs_lpc_use turned it on, and those that ran the network
    int lpc_probe_every, lpc_probe_pending;   // probe interval of the other choice, last solve was a probe
    float *lpc_snap;             // harvested residual snapshots (fine FP32 fields)
    float *lpc_s32, *lpc_d32;    // the residual the V-cycle leaves and the network's correction
    int lpc_snap_max;
    cudaGraph_t cgm_graph[2];    // [0] plain MG-PCG, [1] with the learned correction
    cudaGraphExec_t cgm_exec[2];
    int cgm_graph_built[2];
    int cgm_body_kernels[2];

    // host mirrors of scalar state
    double t, dt;
    double Vmax, Vsrc, Vd_pl, Vd_mi, Vd_or;
    int64_t ts;
    fs_stats st;
};

// ---------------------------------------------------------------- host helpers
int fs_set_error(fs_ctx *c, int code, const char *fmt, ...);
void fs_host_constants(const fs_config &cfg, fs_constants &k);
void fs_host_table(const fs_config &cfg, const fs_constants &k, std::vector<double> &rows);
double fs_circ_source(const fs_config &cfg, const fs_constants &k, double t);   // Vsrc(t), circ_lib.F90:26-50

// particle kernels (fs_ptcl.cu; the mixed-precision step in fs_mixed.cu)
void fs_circuit_launch(fs_ctx *c, int stg, float *fx_e32);
int fs_ptcl_step_impl(fs_ctx *c, int *attempts);
int fs_ptcl_step_mixed(fs_ctx *c, int *attempts);
int fs_mixed_alloc(fs_ctx *c, const std::vector<double> &tab_rows);
void fs_mixed_free(fs_ctx *c);
int fs_mixed_sync_logs(fs_ctx *c);   // FP32 log companions of every state buffer
void fs_faces_update_mixed(fs_ctx *c);
int fs_lapl_solve_mixed(fs_ctx *c, int *lerr, int *iters, double *relres);
int fs_ptcl_alloc(fs_ctx *c);
void fs_ptcl_reset(fs_ctx *c);     // t_m, status and current rows of a new step
int fs_ptcl_control(fs_ctx *c);   // controller + status check after five stages
// surface charge slot `which` (0 sig_pl, 1 sig_mi, 2 sig_or) and the slopes
inline double *fs_sig(fs_ctx *c, int which) { return c->d_sig + (size_t)c->sig_slot[which] * (c->nx + 2); }
inline double *fs_sig_ks(fs_ctx *c) { return c->d_sig + (size_t)3 * (c->nx + 2); }
int fs_sig_copy(fs_ctx *c, int dst, int src);   // slot dst <- slot src, on the stream
void fs_faces_update(fs_ctx *c);   // recompute the face data if phi changed
// many discharges, one launch per RK stage (fs_ptcl.cu; DC, FP64, no wall)
struct FsBatchWork;
int fs_set_stage_tile_impl(fs_ctx *c, int bx, int by);
int fs_batch_work_alloc(fs_ctx **cs, int n, FsBatchWork **out);
void fs_batch_work_free(FsBatchWork *w);
int fs_ptcl_batch_attempt(fs_ctx **cs, int n, FsBatchWork *w, const int *act, const int *fresh, int *rej, int *rc);
// Poisson (fs_lapl.cu)
int fs_lapl_alloc(fs_ctx *c);
int fs_set_line_smoother_impl(fs_ctx *c, int mode);
int fs_lapl_mixed_reconfigure(fs_ctx *c);
int fs_mg_strips(fs_ctx *c);    // electrode strips of the finest level (strip_kl, strip_kr) and their snapshot
void fs_lapl_free(fs_ctx *c);
int fs_lapl_solve_impl(fs_ctx *c, int *lerr, int *iters, double *relres);
// mixed-precision Poisson (fs_lapl_mixed.cu)
int fs_lapl_alloc_mixed(fs_ctx *c);
void fs_lapl_free_mixed(fs_ctx *c);
// learned preconditioner (fs_lapl_mixed.cu, network in fs_lpc.cu)
int fs_lpc_init_impl(fs_ctx *c, int crop, int max_batch, int max_samples, uint64_t seed);
void fs_lpc_free_impl(fs_ctx *c);
int fs_lpc_harvest_impl(fs_ctx *c, int per_solve, int *added);
int fs_lpc_train_impl(fs_ctx *c, int iters, int batch, float lr, uint64_t seed, float *loss_hist);
int fs_lpc_grad_impl(fs_ctx *c, const float *feat, const float *tgt, const float *mask, int batch, float *grad,
                     float *loss, float *pred);
// output writer (fs_output.cpp): waits for the record in flight, stops the thread
void fs_output_free(fs_ctx *c);
// one output record converted on the device into dev, on the context's
// stream (fs_api.cu)
cudaError_t fs_output_stage(fs_ctx *c, double *dev, double x03);
// misc device helpers (fs_api.cu)
int fs_run(fs_ctx *c, int32_t nsteps, fs_stats *out);
int fs_cuda_check(fs_ctx *c, cudaError_t e, const char *what);
int fs_sync_ctrl(fs_ctx *c);
// Held while a context captures and instantiates its CUDA graphs: captures
// of several contexts from several host threads at once (the batch drivers'
// first solves) have failed and left an invalid graph behind.
std::mutex &fs_graph_mutex();
// Raise a kernel's dynamic shared-memory limit to at least `bytes` on the
// current device.  The limit belongs to the kernel, not to a context: every
// context asks for what its grid needs and the largest request stays in
// force (setting it per context let a later, smaller grid lower it below
// what an earlier context's launches take).
cudaError_t fs_smem_limit(const void *kernel, size_t bytes);
// profiler: bracket one launch; drained at every fs_sync_ctrl
void fs_prof_begin(fs_ctx *c, int cls);
void fs_prof_end(fs_ctx *c);
void fs_prof_drain(fs_ctx *c);
void fs_prof_free(fs_ctx *c);
