// fs_api.cu -- C ABI of the CUDA implementation (include/fluidsim_gpu.h):
// context creation (lapl_init + ptcl_init + circ_init), state transfer, the
// per-step entry points and the main-loop rotation of main.F90:83-121.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <cmath>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "fs_internal.h"

static thread_local std::string g_err;

// NVTX range over one reference routine (ptcl_step, lapl_solve, the main-loop
// body), visible to profilers that attach; a no-op without one
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
};

int fs_set_error(fs_ctx *c, int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    else g_err = buf;
    return code;
}

int fs_cuda_check(fs_ctx *c, cudaError_t e, const char *what) {
    if (e == cudaSuccess) return FS_OK;
    int code = (e == cudaErrorMemoryAllocation) ? FS_ERR_NOMEM : FS_ERR_CUDA;
    return fs_set_error(c, code, "%s: %s", what, cudaGetErrorString(e));
}

cudaError_t fs_smem_limit(const void *kernel, size_t bytes) {
    static std::mutex m;
    static std::map<std::pair<const void *, int>, size_t> cur;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(m);
    size_t &v = cur[{kernel, dev}];
    if (bytes <= v) return cudaSuccess;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) v = bytes;
    return e;
}

std::mutex &fs_graph_mutex() {
    static std::mutex m;
    return m;
}

int fs_sync_ctrl(fs_ctx *c) {
    cudaError_t e = cudaMemcpyAsync(c->h_ctrl, c->d_ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess && c->prof_on) fs_prof_drain(c);
    return fs_cuda_check(c, e, "stream");
}

void fs_prof_begin(fs_ctx *c, int cls) {
    c->launches++;
    if (!(c->prof_on & (1 << cls))) return;
    ProfPair p;
    if (!c->prof_free.empty()) {
        p = c->prof_free.back();
        c->prof_free.pop_back();
    } else {
        cudaEventCreate(&p.a);
        cudaEventCreate(&p.b);
    }
    p.cls = cls;
    p.closed = 0;
    cudaEventRecord(p.a, c->stream);
    c->prof_pending.push_back(p);
}

void fs_prof_end(fs_ctx *c) {
    if (!c->prof_on || c->prof_pending.empty() || c->prof_pending.back().closed) return;
    cudaEventRecord(c->prof_pending.back().b, c->stream);
    c->prof_pending.back().closed = 1;
}

void fs_prof_drain(fs_ctx *c) {
    for (ProfPair &p : c->prof_pending) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
            c->prof_ms[p.cls] += ms;
            c->prof_n[p.cls] += 1;
        }
        c->prof_free.push_back(p);
    }
    c->prof_pending.clear();
}

void fs_prof_free(fs_ctx *c) {
    for (ProfPair &p : c->prof_pending) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
    for (ProfPair &p : c->prof_free) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
    c->prof_pending.clear();
    c->prof_free.clear();
}

namespace {

__global__ void k_fill(double *p, size_t n, double v) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        p[i] = v;
}

__global__ void k_set_dt(Ctrl *c, double dt) { c->dt = dt; }

// One writeOut record in the reference's units (main.F90:297-333), the
// interior block of each field x fastest, as the files hold it: f1 = phi ph0,
// f2 = n_e / x0^3, f3 = n_i / x0^3, f4 = n_eps / x0^3 ph0 / 1.5 (the same
// operations in the same order as the host conversion, IEEE-rounded), f5 =
// n_m / x0^3 or zeros with three species.
__global__ void k_output_record(const double *ph, const double *ni, const double *ne, const double *nt,
                                const double *nm, int nx, int ny, int P, double x03, double ph0, double *dst) {
    const size_t n = (size_t)nx * ny;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(q % nx), j = (int)(q / nx);
        const size_t o = (size_t)(j + 1) * P + i + 1;
        dst[q] = ph[o] * ph0;
        dst[n + q] = ne[o] / x03;
        dst[2 * n + q] = ni[o] / x03;
        dst[3 * n + q] = nt[o] / x03 * ph0 / 1.5;
        dst[4 * n + q] = nm ? nm[o] / x03 : 0.0;
    }
}

// maxval over the three RK levels of one species, ghost ring included:
// pass 1, CTA b takes elements [b*FS_MAX_PER_CTA, (b+1)*FS_MAX_PER_CTA) of
// the flattened (level, row, column) index space and writes its maximum to
// part[b]; pass 2, one CTA reduces the partial maxima into *out.
#define FS_MAX_PER_CTA 16384
__global__ void __launch_bounds__(256) k_max_part(const double *a, const double *b, const double *d, int nx,
                                                  int ny, int P, double *part) {
    __shared__ double s[256];
    const long n1 = (long)(nx + 2) * (ny + 2), n = 3 * n1;
    const long lo = (long)blockIdx.x * FS_MAX_PER_CTA, hi = lo + FS_MAX_PER_CTA < n ? lo + FS_MAX_PER_CTA : n;
    const double *arr[3] = {a, b, d};
    double m = -INFINITY;
    for (long q = lo + threadIdx.x; q < hi; q += blockDim.x) {
        const int l = (int)(q / n1);
        const long r = q - (long)l * n1;
        const int gi = (int)(r % (nx + 2)), gj = (int)(r / (nx + 2));
        m = fmax(m, arr[l][(size_t)gj * P + gi]);
    }
    s[threadIdx.x] = m;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) s[threadIdx.x] = fmax(s[threadIdx.x], s[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}

__global__ void __launch_bounds__(256) k_max_final(const double *part, int nblk, double *out) {
    __shared__ double s[256];
    double m = -INFINITY;
    for (int q = threadIdx.x; q < nblk; q += blockDim.x) m = fmax(m, part[q]);
    s[threadIdx.x] = m;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) s[threadIdx.x] = fmax(s[threadIdx.x], s[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = s[0];
}

int max_parts(const fs_ctx *c) {
    const long n = 3L * (c->nx + 2) * (c->ny + 2);
    return (int)((n + FS_MAX_PER_CTA - 1) / FS_MAX_PER_CTA);
}

// Launch both passes of the ne maximum with scratch = nblk partials + 1 result.
void launch_max_ne(fs_ctx *c, double *scratch, int nblk) {
    const SpeciesBufs &b = c->sp[1];
    c->launches += 2;
    k_max_part<<<nblk, 256, 0, c->stream>>>(b.buf[c->lev[0]], b.buf[c->lev[1]], b.buf[c->lev[2]], c->nx, c->ny,
                                            c->pitch, scratch);
    k_max_final<<<1, 256, 0, c->stream>>>(scratch, nblk, scratch + nblk);
}

int validate(const fs_config *cfg, const fs_mesh *m) {
    if (!cfg || !m) return fs_set_error(nullptr, FS_ERR_INVALID, "null config or mesh");
    if (cfg->abi_version != FS_ABI_VERSION)
        return fs_set_error(nullptr, FS_ERR_INVALID, "ABI version %d, library %d", cfg->abi_version, FS_ABI_VERSION);
    if (cfg->nx < 3 || cfg->ny < 2)
        return fs_set_error(nullptr, FS_ERR_UNSUPPORTED, "grid must have nx >= 3 and ny >= 2 (got %d x %d)", cfg->nx, cfg->ny);
    if ((long)cfg->nx * cfg->ny > (1L << 28))
        return fs_set_error(nullptr, FS_ERR_INVALID, "grid too large");
    if (cfg->nspecies != 3 && cfg->nspecies != 4) return fs_set_error(nullptr, FS_ERR_INVALID, "nspecies must be 3 or 4");
    if (cfg->coef_mode != FS_COEF_TABLE && cfg->coef_mode != FS_COEF_FITS)
        return fs_set_error(nullptr, FS_ERR_INVALID, "unknown coefficient mode %d", cfg->coef_mode);
    if (cfg->coef_mode == FS_COEF_FITS && cfg->precision != FS_PREC_FP64)
        return fs_set_error(nullptr, FS_ERR_UNSUPPORTED, "the fit coefficient mode runs on the FP64 path only");
    if (cfg->table_n < 2 || !(cfg->table_emax_ev > cfg->table_emin_ev) || !(cfg->table_emin_ev > 0))
        return fs_set_error(nullptr, FS_ERR_INVALID, "bad coefficient table range");
    if (cfg->rf < 0 || cfg->rf > 3)
        return fs_set_error(nullptr, FS_ERR_UNSUPPORTED, "rf must be 0 (DC), 1 (AC) or 2, 3 (pulses), got %d", cfg->rf);
    if (cfg->rf == 1 && !(cfg->res > 0))
        return fs_set_error(nullptr, FS_ERR_INVALID, "the AC source's RC circuit needs res > 0");
    if (cfg->precision != FS_PREC_FP64 && cfg->precision != FS_PREC_MIXED)
        return fs_set_error(nullptr, FS_ERR_INVALID, "unknown precision mode %d", cfg->precision);
    if (cfg->mg_smooth < 1 || cfg->mg_smooth > 8) return fs_set_error(nullptr, FS_ERR_INVALID, "mg_smooth must be 1..8");
    if (cfg->lapl_maxit < 1) return fs_set_error(nullptr, FS_ERR_INVALID, "lapl_maxit must be positive");
    for (long q = 0; q < (long)cfg->nx * cfg->ny; q++) {
        int tx = m->type_x[q], ty = m->type_y[q];
        if (tx < -2 || tx > 2 || ty < -2 || ty > 3)
            return fs_set_error(nullptr, FS_ERR_UNSUPPORTED, "node type (%d,%d) at %ld not supported", tx, ty, q);
        if (ty == 3 && q / cfg->nx != cfg->ny - 1)   // g_init puts the wall on the last row only
            return fs_set_error(nullptr, FS_ERR_UNSUPPORTED, "dielectric wall node off the last row at %ld", q);
    }
    return FS_OK;
}

void free_ctx(fs_ctx *c) {
    if (!c) return;
    fs_output_free(c);
    fs_lpc_free_impl(c);
    fs_lapl_free(c);
    if (c->mixed) {
        fs_lapl_free_mixed(c);
        fs_mixed_free(c);
    }
    for (int s = 0; s < FS_MAX_SPECIES; s++) {
        for (int b = 0; b < FS_NBUF; b++) cudaFree(c->sp[s].buf[b]);
        for (int k = 0; k < 3; k++) cudaFree(c->sp[s].k[k]);
    }
    cudaFree(c->ph);
    cudaFree(c->ph_mi);
    cudaFree(c->d_part);
    cudaFree(c->d_rows);
    cudaFree(c->d_sig);
    double *faces[] = {c->fx_e, c->fx_cl, c->fx_cr, c->fy_e, c->fy_cl, c->fy_cr,
                       c->fx_dl, c->fx_dr, c->fy_dl, c->fy_dr};
    for (double *f : faces) cudaFree(f);
    cudaFree(c->d_ctrl);
    cudaFree(c->d_mesh_blob);
    cudaFree(c->d_types);
    cudaFree(c->d_tab);
    if (c->h_ctrl) cudaFreeHost(c->h_ctrl);
    fs_prof_free(c);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

int set_dt_dev(fs_ctx *c, double dt) {
    c->dt = dt;
    fs_prof_begin(c, PROF_OTHER);
    k_set_dt<<<1, 1, 0, c->stream>>>(c->d_ctrl, dt);
    fs_prof_end(c);
    return fs_cuda_check(c, cudaGetLastError(), "set dt");
}

}  // namespace

extern "C" {

int32_t fs_abi_version(void) { return FS_ABI_VERSION; }

int fs_get_constants(const fs_config *cfg, fs_constants *out) {
    if (!cfg || !out) return FS_ERR_INVALID;
    fs_host_constants(*cfg, *out);
    return FS_OK;
}

int fs_build_table(const fs_config *cfg, double *out) {
    if (!cfg || !out || cfg->table_n < 2) return FS_ERR_INVALID;
    fs_constants k;
    fs_host_constants(*cfg, k);
    std::vector<double> rows;
    fs_host_table(*cfg, k, rows);
    memcpy(out, rows.data(), rows.size() * sizeof(double));
    return FS_OK;
}

const char *fs_last_error(const fs_ctx *c) { return c ? c->err.c_str() : g_err.c_str(); }

int fs_create(const fs_config *cfg, const fs_mesh *m, fs_ctx **out) {
    if (!out) return fs_set_error(nullptr, FS_ERR_INVALID, "null output handle");
    *out = nullptr;
    int rc = validate(cfg, m);
    if (rc) return rc;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fs_set_error(nullptr, FS_ERR_NO_DEVICE, "no CUDA device");
    fs_ctx *c = new fs_ctx();
    memset(&c->st, 0, sizeof(c->st));
    c->cfg = *cfg;
    c->nx = cfg->nx;
    c->ny = cfg->ny;
    c->pitch = ((cfg->nx + 2 + 31) / 32) * 32;
    c->field_elems = (size_t)(cfg->ny + 2) * c->pitch;
    cudaGetDevice(&c->device);
    cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, c->device);
    if (c->nsm < 1) c->nsm = 1;
    fs_host_constants(*cfg, c->k);
    const fs_constants &k = c->k;
    const int nx = c->nx, ny = c->ny;
#define CK(call, what)                                      \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) {                            \
            rc = fs_cuda_check(nullptr, e_, what);          \
            free_ctx(c);                                    \
            return rc;                                      \
        }                                                   \
    } while (0)
    CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "stream");

    // physics parameters
    PhysParams &pp = c->pp;
    memset(&pp, 0, sizeof(pp));
    pp.nx = nx; pp.ny = ny; pp.pitch = c->pitch; pp.nspecies = cfg->nspecies; pp.cyl = cfg->cyl;
    pp.ntab = cfg->table_n;
    pp.ph0 = k.ph0; pp.e = k.e; pp.pi = k.pi; pp.me = k.me; pp.t0 = k.t0; pp.x0 = k.x0;
    pp.mui = k.mui; pp.Di = k.Di; pp.vi = k.vi; pp.Dm = k.Dm; pp.gam = k.gam; pp.ninf = k.ninf;
    pp.tg = k.tg; pp.kb = k.kb; pp.mi = k.mi; pp.inv_mi = 1.0 / k.mi;
    pp.h_ir = k.h_ir; pp.h_ex = k.h_ex; pp.h_si = k.h_si;
    pp.k_mp = k.k_mp; pp.k_r = k.k_r; pp.k_2q = k.k_2q; pp.k_3q = k.k_3q;
    pp.nmin[0] = k.n_zero; pp.nmin[1] = k.n_zero; pp.nmin[2] = k.nmin_nt; pp.nmin[3] = k.n_zero;
    pp.abs_tol = cfg->abs_tol; pp.rel_tol = cfg->rel_tol;
    pp.lemin = std::log(cfg->table_emin_ev);
    pp.inv_h = (double)(cfg->table_n - 1) / (std::log(cfg->table_emax_ev) - pp.lemin);
    pp.ve_coef = (16.0 * k.e * k.ph0) / (3.0 * k.pi * k.me);
    pp.tg_term = k.tg * k.kb / k.e / k.ph0;
    pp.e100 = std::exp(-100.0);
    pp.fits = cfg->coef_mode == FS_COEF_FITS;
    pp.fit = fs_fit_eval(k);

    // mesh blob: dx, inv_dx (nx+1), dy, inv_dy (ny+1), dlx, inv_dlx (nx), dly, inv_dly (ny),
    // r (ny+2), dr_a, dr_c (ny+2)
    std::vector<double> blob;
    auto push = [&](const double *p, int n) { size_t o = blob.size(); blob.insert(blob.end(), p, p + n); return o; };
    std::vector<double> inv_dx(nx + 1), inv_dy(ny + 1), inv_dlx(nx), inv_dly(ny);
    for (int i = 0; i <= nx; i++) inv_dx[i] = 1.0 / m->dx[i];
    for (int j = 0; j <= ny; j++) inv_dy[j] = 1.0 / m->dy[j];
    for (int i = 0; i < nx; i++) inv_dlx[i] = 1.0 / m->dlx[i];
    for (int j = 0; j < ny; j++) inv_dly[j] = 1.0 / m->dly[j];
    // node coordinates for the output writer: x(1) = 0, x(i+1) = x(i) + dx(i)
    c->h_x.assign(nx + 2, 0.0);
    c->h_y.assign(ny + 2, 0.0);
    for (int i = 0; i <= nx; i++) c->h_x[i + 1] = c->h_x[i] + m->dx[i];
    for (int j = 0; j <= ny; j++) c->h_y[j + 1] = c->h_y[j] + m->dy[j];
    // circ_step current weights per row (circ_lib.F90:87-151)
    c->h_dr_a.assign(ny + 2, 0.0);
    c->h_dr_c.assign(ny + 2, 0.0);
    for (int gj = 1; gj <= ny; gj++) {
        double dr = cfg->cyl ? m->dy[gj - 1] * m->r[gj - 1] * 2.0 * k.pi : m->dy[gj - 1] * cfg->w;
        if (m->r[gj] < cfg->ew) dr = 0.0;
        if (m->type_x[(size_t)(gj - 1) * nx + 0] == -2) c->h_dr_a[gj] = dr;
        if (m->type_x[(size_t)(gj - 1) * nx + nx - 1] == 2) c->h_dr_c[gj] = dr;
    }
    size_t o_dx = push(m->dx, nx + 1), o_idx = push(inv_dx.data(), nx + 1);
    size_t o_dy = push(m->dy, ny + 1), o_idy = push(inv_dy.data(), ny + 1);
    size_t o_dlx = push(m->dlx, nx), o_idlx = push(inv_dlx.data(), nx);
    size_t o_dly = push(m->dly, ny), o_idly = push(inv_dly.data(), ny);
    size_t o_r = push(m->r, ny + 2), o_dra = push(c->h_dr_a.data(), ny + 2), o_drc = push(c->h_dr_c.data(), ny + 2);
    CK(cudaMalloc(&c->d_mesh_blob, blob.size() * sizeof(double)), "cudaMalloc mesh");
    CK(cudaMemcpy(c->d_mesh_blob, blob.data(), blob.size() * sizeof(double), cudaMemcpyHostToDevice), "mesh upload");
    std::vector<int8_t> types((size_t)2 * nx * ny);
    for (size_t q = 0; q < (size_t)nx * ny; q++) {
        types[q] = (int8_t)m->type_x[q];
        types[(size_t)nx * ny + q] = (int8_t)m->type_y[q];
        if (m->type_y[q] == 3) c->rwall = 1;
    }
    CK(cudaMalloc(&c->d_types, types.size()), "cudaMalloc types");
    CK(cudaMemcpy(c->d_types, types.data(), types.size(), cudaMemcpyHostToDevice), "types upload");
    MeshDev &md = c->mesh;
    double *B = c->d_mesh_blob;
    md.dx = B + o_dx; md.inv_dx = B + o_idx; md.dy = B + o_dy; md.inv_dy = B + o_idy;
    md.dlx = B + o_dlx; md.inv_dlx = B + o_idlx; md.dly = B + o_dly; md.inv_dly = B + o_idly;
    md.r = B + o_r; md.dr_a = B + o_dra; md.dr_c = B + o_drc;
    md.tx = c->d_types;
    md.ty = c->d_types + (size_t)nx * ny;

    // coefficient table, node-major: 8 values then 8 slopes f(k+1)-f(k)
    std::vector<double> rows;
    {
        fs_host_table(*cfg, k, rows);
        const int n = cfg->table_n;
        std::vector<double> t((size_t)n * FS_TAB_STRIDE, 0.0);
        for (int i = 0; i < n; i++)
            for (int r = 0; r < 8; r++) {
                t[(size_t)i * FS_TAB_STRIDE + r] = rows[(size_t)r * n + i];
                t[(size_t)i * FS_TAB_STRIDE + 8 + r] = i + 1 < n ? rows[(size_t)r * n + i + 1] - rows[(size_t)r * n + i] : 0.0;
            }
        CK(cudaMalloc(&c->d_tab, t.size() * sizeof(double)), "cudaMalloc table");
        CK(cudaMemcpy(c->d_tab, t.data(), t.size() * sizeof(double), cudaMemcpyHostToDevice), "table upload");
    }

    // fields, ptcl_init (ptcl_lib.F90:22-29) and lapl_init (lapl_lib.F90:27-28)
    const size_t n = c->field_elems;
    const double nt0 = cfg->n_init * k.tg * k.kb / k.e / k.ph0;
    for (int s = 0; s < cfg->nspecies; s++) {
        double v0 = s == 2 ? nt0 : cfg->n_init;
        for (int b = 0; b < FS_NBUF; b++) {
            CK(cudaMalloc(&c->sp[s].buf[b], n * sizeof(double)), "cudaMalloc species");
            k_fill<<<256, 256, 0, c->stream>>>(c->sp[s].buf[b], n, v0);
        }
        for (int q = 0; q < 3; q++) {
            CK(cudaMalloc(&c->sp[s].k[q], n * sizeof(double)), "cudaMalloc k");
            CK(cudaMemsetAsync(c->sp[s].k[q], 0, n * sizeof(double), c->stream), "memset k");
        }
    }
    c->lev[0] = c->lev[1] = c->lev[2] = 0;
    CK(cudaMalloc(&c->ph, n * sizeof(double)), "cudaMalloc ph");
    CK(cudaMalloc(&c->ph_mi, n * sizeof(double)), "cudaMalloc ph_mi");
    CK(cudaMemsetAsync(c->ph, 0, n * sizeof(double), c->stream), "memset ph");
    CK(cudaMemsetAsync(c->ph_mi, 0, n * sizeof(double), c->stream), "memset ph_mi");
    CK(cudaMalloc(&c->d_ctrl, sizeof(Ctrl)), "cudaMalloc ctrl");
    CK(cudaMallocHost(&c->h_ctrl, sizeof(Ctrl)), "cudaMallocHost ctrl");
    memset(c->h_ctrl, 0, sizeof(Ctrl));
    c->h_ctrl->err_prev = 1.0;
    c->h_ctrl->t_m = 1e9;
    CK(cudaMemcpyAsync(c->d_ctrl, c->h_ctrl, sizeof(Ctrl), cudaMemcpyHostToDevice, c->stream), "ctrl init");
    c->mixed = cfg->precision == FS_PREC_MIXED;
    if ((rc = fs_ptcl_alloc(c)) || (rc = fs_lapl_alloc(c)) ||
        (c->mixed && ((rc = fs_mixed_alloc(c, rows)) || (rc = fs_lapl_alloc_mixed(c)) ||
                      (rc = fs_mixed_sync_logs(c))))) {
        g_err = c->err;
        free_ctx(c);
        return rc;
    }
    // circ_init (circ_lib.F90:213-223)
    c->Vmax = c->Vsrc = c->Vd_pl = c->Vd_mi = c->Vd_or = cfg->vl;
    c->t = 0.0;
    c->dt = 0.0;
    c->ts = 0;
    CK(cudaStreamSynchronize(c->stream), "create");
#undef CK
    *out = c;
    return FS_OK;
}

void fs_destroy(fs_ctx *c) {
    if (!c) return;
    cudaStreamSynchronize(c->stream);
    free_ctx(c);
}

int fs_set_time(fs_ctx *c, double t, double dt) {
    if (!c) return FS_ERR_INVALID;
    c->t = t;
    return set_dt_dev(c, dt);
}

int fs_get_controller(fs_ctx *c, double *err_prev, int64_t *ts) {
    if (!c) return FS_ERR_INVALID;
    int rc = fs_sync_ctrl(c);
    if (rc) return rc;
    if (err_prev) *err_prev = c->h_ctrl->err_prev;
    if (ts) *ts = c->ts;
    return FS_OK;
}

int fs_set_controller(fs_ctx *c, double err_prev, int64_t ts) {
    if (!c) return FS_ERR_INVALID;
    if (!(err_prev > 0.0)) return fs_set_error(c, FS_ERR_INVALID, "err_prev must be positive");
    c->ts = ts;
    cudaError_t e = cudaMemcpyAsync(&c->d_ctrl->err_prev, &err_prev, sizeof(double), cudaMemcpyHostToDevice,
                                    c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return fs_cuda_check(c, e, "set controller");
}

int fs_upload_state(fs_ctx *c, const double *ni, const double *ne, const double *nt, const double *nm,
                    const double *ph, int32_t ld, int32_t nlev) {
    if (!c) return FS_ERR_INVALID;
    if (ld < c->nx + 2 || (nlev != 1 && nlev != 3))
        return fs_set_error(c, FS_ERR_INVALID, "upload: ld %d < nx+2 or nlev %d not 1/3", ld, nlev);
    const double *src[FS_MAX_SPECIES] = {ni, ne, nt, nm};
    const size_t w = (size_t)(c->nx + 2) * sizeof(double), hp = (size_t)ld * sizeof(double),
                 dp = (size_t)c->pitch * sizeof(double);
    const int rows = c->ny + 2;
    cudaError_t e = cudaSuccess;
    for (int s = 0; s < c->cfg.nspecies && e == cudaSuccess; s++) {
        if (!src[s]) continue;
        for (int l = 0; l < nlev && e == cudaSuccess; l++)
            e = cudaMemcpy2DAsync(c->sp[s].buf[l], dp, src[s] + (size_t)l * ld * rows, hp, w, rows,
                                  cudaMemcpyHostToDevice, c->stream);
        // the remaining buffers start as copies of level 1, ghost ring included
        for (int b = nlev; b < FS_NBUF && e == cudaSuccess; b++)
            e = cudaMemcpyAsync(c->sp[s].buf[b], c->sp[s].buf[0], c->field_elems * sizeof(double),
                                cudaMemcpyDeviceToDevice, c->stream);
    }
    if (e == cudaSuccess) {
        if (nlev == 1) { c->lev[0] = c->lev[1] = c->lev[2] = 0; }
        else { c->lev[0] = 0; c->lev[1] = 1; c->lev[2] = 2; }
    }
    if (e == cudaSuccess && c->mixed && fs_mixed_sync_logs(c)) return FS_ERR_CUDA;
    if (ph && e == cudaSuccess) {
        c->faces_valid = 0;
        e = cudaMemcpy2DAsync(c->ph, dp, ph, hp, w, rows, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(c->ph_mi, c->ph, c->field_elems * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return fs_cuda_check(c, e, "upload_state");
}

int fs_download_state(fs_ctx *c, double *ni, double *ne, double *nt, double *nm, double *ph,
                      int32_t ld, int32_t nlev) {
    if (!c) return FS_ERR_INVALID;
    if (ld < c->nx + 2 || (nlev != 1 && nlev != 3))
        return fs_set_error(c, FS_ERR_INVALID, "download: ld %d < nx+2 or nlev %d not 1/3", ld, nlev);
    double *dst[FS_MAX_SPECIES] = {ni, ne, nt, nm};
    const size_t w = (size_t)(c->nx + 2) * sizeof(double), hp = (size_t)ld * sizeof(double),
                 dp = (size_t)c->pitch * sizeof(double);
    const int rows = c->ny + 2;
    cudaError_t e = cudaSuccess;
    for (int s = 0; s < c->cfg.nspecies && e == cudaSuccess; s++) {
        if (!dst[s]) continue;
        for (int l = 0; l < nlev && e == cudaSuccess; l++)
            e = cudaMemcpy2DAsync(dst[s] + (size_t)l * ld * rows, hp, c->sp[s].buf[c->lev[l]], dp, w, rows,
                                  cudaMemcpyDeviceToHost, c->stream);
    }
    if (ph && e == cudaSuccess)
        e = cudaMemcpy2DAsync(ph, hp, c->ph, dp, w, rows, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return fs_cuda_check(c, e, "download_state");
}

int fs_get_lapl_guess(fs_ctx *c, double *d, int32_t ld) {
    if (!c || !d) return FS_ERR_INVALID;
    if (ld < c->nx + 2) return fs_set_error(c, FS_ERR_INVALID, "lapl guess: ld %d < nx+2", ld);
    const int rows = c->ny + 2, w = c->nx + 2;
    cudaError_t e;
    if (c->mixed) {   // the mixed solver's iterate is the float-float pair xh + xl
        std::vector<float> h((size_t)rows * w), l((size_t)rows * w);
        e = cudaMemcpy2DAsync(h.data(), w * sizeof(float), c->xh32, (size_t)c->pitch * sizeof(float),
                              w * sizeof(float), rows, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess)
            e = cudaMemcpy2DAsync(l.data(), w * sizeof(float), c->xl32, (size_t)c->pitch * sizeof(float),
                                  w * sizeof(float), rows, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e == cudaSuccess)
            for (int j = 0; j < rows; j++)
                for (int i = 0; i < w; i++)
                    d[(size_t)j * ld + i] = (double)h[(size_t)j * w + i] + (double)l[(size_t)j * w + i];
        return fs_cuda_check(c, e, "get_lapl_guess");
    }
    e = cudaMemcpy2DAsync(d, (size_t)ld * sizeof(double), c->xs, (size_t)c->pitch * sizeof(double),
                          w * sizeof(double), rows, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return fs_cuda_check(c, e, "get_lapl_guess");
}

int fs_set_lapl_guess(fs_ctx *c, const double *d, int32_t ld) {
    if (!c || !d) return FS_ERR_INVALID;
    if (ld < c->nx + 2) return fs_set_error(c, FS_ERR_INVALID, "lapl guess: ld %d < nx+2", ld);
    cudaError_t e;
    if (c->mixed) {   // split into the float-float pair, interior only
        const int nx = c->nx, ny = c->ny;
        std::vector<float> h((size_t)ny * nx), l((size_t)ny * nx);
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                const double v = d[(size_t)(j + 1) * ld + i + 1];
                const float hv = (float)v;
                h[(size_t)j * nx + i] = hv;
                l[(size_t)j * nx + i] = (float)(v - (double)hv);
            }
        e = cudaMemcpy2DAsync(c->xh32 + c->pitch + 1, (size_t)c->pitch * sizeof(float), h.data(), nx * sizeof(float),
                              nx * sizeof(float), ny, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess)
            e = cudaMemcpy2DAsync(c->xl32 + c->pitch + 1, (size_t)c->pitch * sizeof(float), l.data(),
                                  nx * sizeof(float), nx * sizeof(float), ny, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        return fs_cuda_check(c, e, "set_lapl_guess");
    }
    // interior only: the ghost ring of the iterate stays zero
    e = cudaMemcpy2DAsync(c->xs + c->pitch + 1, (size_t)c->pitch * sizeof(double), d + ld + 1,
                          (size_t)ld * sizeof(double), (size_t)c->nx * sizeof(double), c->ny,
                          cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return fs_cuda_check(c, e, "set_lapl_guess");
}

int fs_ptcl_step(fs_ctx *c, double *dt_inout, double *t_m_out, double *ida_out, double *idc_out,
                 int32_t *attempts_out) {
    if (!c) return FS_ERR_INVALID;
    NvtxRange range("ptcl_step");
    int rc;
    if (dt_inout && (rc = set_dt_dev(c, *dt_inout))) return rc;
    int attempts = 0;
    rc = c->mixed ? fs_ptcl_step_mixed(c, &attempts) : fs_ptcl_step_impl(c, &attempts);
    if (dt_inout) *dt_inout = c->h_ctrl->dt;
    if (t_m_out) *t_m_out = c->h_ctrl->t_m;
    if (ida_out) *ida_out = c->h_ctrl->ida;
    if (idc_out) *idc_out = c->h_ctrl->idc;
    if (attempts_out) *attempts_out = attempts;
    return rc;
}

int fs_lapl_solve(fs_ctx *c, double dt, int32_t *lerr_out, int32_t *iters_out, double *relres_out) {
    if (!c) return FS_ERR_INVALID;
    NvtxRange range("lapl_solve");
    int rc = set_dt_dev(c, dt);
    if (rc) return rc;
    int lerr = 1, iters = 0;
    double relres = 0;
    rc = c->mixed ? fs_lapl_solve_mixed(c, &lerr, &iters, &relres) : fs_lapl_solve_impl(c, &lerr, &iters, &relres);
    c->st.lapl_iters += iters;
    c->st.last_lapl_iters = iters;
    c->st.lapl_relres = relres;
    c->st.lerr = lerr;
    if (lerr_out) *lerr_out = lerr;
    if (iters_out) *iters_out = iters;
    if (relres_out) *relres_out = relres;
    return rc;
}

int fs_accept(fs_ctx *c) {
    if (!c) return FS_ERR_INVALID;
    c->ts++;
    c->t = c->t + c->dt;
    c->lev[2] = c->lev[1];   // n3 <- n2
    c->lev[1] = c->lev[0];   // n2 <- n1
    c->Vd_or = c->Vd_mi;
    c->Vd_mi = c->Vd_pl;
    if (c->rwall) {   // sig_or <- sig_mi, sig_mi <- sig_pl: rotate the slots, sig_pl keeps its values
        const int pl = c->sig_slot[0], mi = c->sig_slot[1], orr = c->sig_slot[2];
        c->sig_slot[2] = mi;
        c->sig_slot[1] = pl;
        c->sig_slot[0] = orr;
        return fs_sig_copy(c, 0, 1);
    }
    return FS_OK;
}

int fs_reject(fs_ctx *c) {
    if (!c) return FS_ERR_INVALID;
    c->lev[0] = c->lev[2];   // n1 <- n3
    c->lev[1] = c->lev[2];   // n2 <- n3
    c->Vd_pl = c->Vd_or;
    c->Vd_mi = c->Vd_or;
    int rc;
    if (c->rwall && ((rc = fs_sig_copy(c, 0, 2)) || (rc = fs_sig_copy(c, 1, 2)))) return rc;
    return set_dt_dev(c, c->dt / 2.0);
}

int fs_run(fs_ctx *c, int32_t nsteps, fs_stats *out) {
    if (!c) return FS_ERR_INVALID;
    for (int s = 0; s < nsteps; s++) {
        NvtxRange step("main loop step");
        int rc;
        if (c->ts > 1) {
            NvtxRange range("ptcl_step");
            int att = 0;
            if ((rc = c->mixed ? fs_ptcl_step_mixed(c, &att) : fs_ptcl_step_impl(c, &att))) return rc;
        }
        int lerr = 1, iters = 0;
        double relres = 0;
        {
            NvtxRange range("lapl_solve");
            if ((rc = c->mixed ? fs_lapl_solve_mixed(c, &lerr, &iters, &relres)
                               : fs_lapl_solve_impl(c, &lerr, &iters, &relres)))
                return rc;
        }
        c->st.lapl_iters += iters;
        c->st.last_lapl_iters = iters;
        c->st.lapl_relres = relres;
        c->st.lerr = lerr;
        if (lerr == 0) {
            if ((rc = fs_accept(c))) return rc;
        } else {
            c->st.lapl_rejects++;
            if ((rc = fs_reject(c))) return rc;
        }
    }
    return fs_get_stats(c, out);
}

int fs_get_circuit(fs_ctx *c, double *v) {
    if (!c || !v) return FS_ERR_INVALID;
    v[0] = c->Vd_pl; v[1] = c->Vd_mi; v[2] = c->Vd_or; v[3] = c->Vsrc;
    return FS_OK;
}

int fs_set_circuit(fs_ctx *c, const double *v) {
    if (!c || !v) return FS_ERR_INVALID;
    c->Vd_pl = v[0]; c->Vd_mi = v[1]; c->Vd_or = v[2];
    return FS_OK;
}

int fs_get_surface_charge(fs_ctx *c, double *sig_pl, double *sig_mi, double *sig_or) {
    if (!c) return FS_ERR_INVALID;
    double *dst[3] = {sig_pl, sig_mi, sig_or};
    for (int q = 0; q < 3; q++) {
        if (!dst[q]) continue;
        cudaError_t e = cudaMemcpyAsync(dst[q], fs_sig(c, q), sizeof(double) * (c->nx + 2), cudaMemcpyDeviceToHost,
                                        c->stream);
        if (e != cudaSuccess) return fs_cuda_check(c, e, "surface charge download");
    }
    cudaError_t e = cudaStreamSynchronize(c->stream);
    return e == cudaSuccess ? FS_OK : fs_cuda_check(c, e, "surface charge download");
}

int fs_set_surface_charge(fs_ctx *c, const double *sig_pl, const double *sig_mi, const double *sig_or) {
    if (!c) return FS_ERR_INVALID;
    const double *src[3] = {sig_pl, sig_mi, sig_or};
    for (int q = 0; q < 3; q++) {
        if (!src[q]) continue;
        cudaError_t e = cudaMemcpyAsync(fs_sig(c, q), src[q], sizeof(double) * (c->nx + 2), cudaMemcpyHostToDevice,
                                        c->stream);
        if (e != cudaSuccess) return fs_cuda_check(c, e, "surface charge upload");
    }
    cudaError_t e = cudaStreamSynchronize(c->stream);
    return e == cudaSuccess ? FS_OK : fs_cuda_check(c, e, "surface charge upload");
}

int fs_get_stats(fs_ctx *c, fs_stats *out) {
    if (!c) return FS_ERR_INVALID;
    if (!out) return FS_OK;
    c->st.t = c->t;
    c->st.dt = c->dt;
    c->st.t_m = c->h_ctrl->t_m;
    c->st.ida = c->h_ctrl->ida;
    c->st.idc = c->h_ctrl->idc;
    c->st.err_cur = c->h_ctrl->err_cur;
    c->st.dt_step = c->h_ctrl->dt_step;
    c->st.steps = c->ts;
    *out = c->st;
    return FS_OK;
}

void *fs_stream(fs_ctx *c) { return c ? (void *)c->stream : nullptr; }

int64_t fs_launch_count(fs_ctx *c) { return c ? c->launches : -1; }

int fs_set_stage_tile(fs_ctx *c, int32_t bx, int32_t by) {
    if (!c) return FS_ERR_INVALID;
    return fs_set_stage_tile_impl(c, bx, by);
}

int fs_set_line_smoother(fs_ctx *c, int32_t mode) {
    if (!c) return FS_ERR_INVALID;
    std::lock_guard<std::mutex> lock(fs_graph_mutex());
    return fs_set_line_smoother_impl(c, mode);
}

int fs_line_smoother(fs_ctx *c) { return c ? c->mg_xline : -1; }

int fs_profile(fs_ctx *c, int32_t enable) {
    if (!c) return FS_ERR_INVALID;
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e == cudaSuccess) fs_prof_drain(c);
    c->prof_on = enable & ((1 << PROF_NCLASS) - 1);
    for (int i = 0; i < PROF_NCLASS; i++) { c->prof_ms[i] = 0.0; c->prof_n[i] = 0; }
    return fs_cuda_check(c, e, "profile");
}

int fs_profile_read(fs_ctx *c, double *ms_out, int64_t *launches_out, int32_t n) {
    if (!c || n < 0) return FS_ERR_INVALID;
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e == cudaSuccess) fs_prof_drain(c);
    for (int i = 0; i < n && i < PROF_NCLASS; i++) {
        if (ms_out) ms_out[i] = c->prof_ms[i];
        if (launches_out) launches_out[i] = c->prof_n[i];
    }
    return fs_cuda_check(c, e, "profile_read");
}

// maxval(ne) over the whole module array, every level and the ghost ring
// included (main.F90:131).  The partial maxima live in scratch memory taken
// from the stream-ordered allocator for the duration of the call.
int fs_max_ne(fs_ctx *c, double *out) {
    if (!c || !out) return FS_ERR_INVALID;
    const int nblk = max_parts(c);
    double *d;
    cudaError_t e = cudaMallocAsync((void **)&d, sizeof(double) * (nblk + 1), c->stream);
    if (e != cudaSuccess) return fs_cuda_check(c, e, "max_ne");
    launch_max_ne(c, d, nblk);
    e = cudaMemcpyAsync(out, d + nblk, sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    cudaFreeAsync(d, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return fs_cuda_check(c, e, "max_ne");
}

// ---------------------------------------------------------------------------
// fs_max_ne_noalloc: fs_max_ne for callers that may not allocate device
// memory once their run is set up -- for example a stepping loop that runs
// with the stream-ordered allocator or cudaMalloc forbidden after
// initialisation, where fs_max_ne's per-call scratch is not allowed.  The
// partial maxima go to a file-scope device array instead: at most
// FS_NOALLOC_MAX_PARTS partials of FS_MAX_PER_CTA values each, i.e. the three
// RK levels of n_e with their ghost rings may hold up to 33,554,432 values
// (a 3342 x 3342 grid); larger contexts are rejected with FS_ERR_INVALID.
// Every GPU that loads this library holds the array (16 KB) until the
// process exits.  The first call on a device looks up the array's device
// address (cudaGetSymbolAddress) with that device current; make that first
// call before any stream capture.  All calls share the one array and it keeps
// the last call's contents: calls whose work overlaps on the GPU (two
// contexts or streams at once) race on it.  Nothing in it has to start at
// zero -- each call writes every partial it reads.
#define FS_NOALLOC_MAX_PARTS 2048
#define FS_NOALLOC_MAX_DEVICES 64
static __device__ __align__(256) double fs_noalloc_scratch[FS_NOALLOC_MAX_PARTS + 1];
static std::mutex g_noalloc_mu;
static double *g_noalloc_ptr[FS_NOALLOC_MAX_DEVICES];

extern "C" int fs_max_ne_noalloc(fs_ctx *c, double *out) {
    if (!c || !out) return FS_ERR_INVALID;
    const int nblk = max_parts(c);
    if (nblk > FS_NOALLOC_MAX_PARTS)
        return fs_set_error(c, FS_ERR_INVALID,
                            "fs_max_ne_noalloc: %ld values exceed its scratch limit of %ld "
                            "(%d partial maxima of %d values); use fs_max_ne",
                            3L * (c->nx + 2) * (c->ny + 2), (long)FS_NOALLOC_MAX_PARTS * FS_MAX_PER_CTA,
                            FS_NOALLOC_MAX_PARTS, FS_MAX_PER_CTA);
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fs_cuda_check(c, e, "fs_max_ne_noalloc");
    if (dev != c->device || dev < 0 || dev >= FS_NOALLOC_MAX_DEVICES)
        return fs_set_error(c, FS_ERR_INVALID, "fs_max_ne_noalloc: the context's device %d must be current (is %d)",
                            c->device, dev);
    double *scratch;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        if (!g_noalloc_ptr[dev]) {
            double *p = nullptr;
            e = cudaGetSymbolAddress((void **)&p, fs_noalloc_scratch);
            if (e != cudaSuccess) return fs_cuda_check(c, e, "fs_max_ne_noalloc: cudaGetSymbolAddress");
            g_noalloc_ptr[dev] = p;
        }
        scratch = g_noalloc_ptr[dev];
    }
    launch_max_ne(c, scratch, nblk);
    // the result lands in the context's pinned control block, so no staging
    e = cudaMemcpyAsync(&c->h_ctrl->host_result, scratch + nblk, sizeof(double), cudaMemcpyDeviceToHost,
                        c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return fs_cuda_check(c, e, "fs_max_ne_noalloc");
    *out = c->h_ctrl->host_result;
    return FS_OK;
}

}  // extern "C"

// ------------------------------------------------ learned Poisson preconditioner
#include "fs_lpc.cuh"

int fs_lpc_init(fs_ctx *c, int32_t crop, int32_t max_batch, int32_t max_samples, uint64_t seed) {
    if (!c) return FS_ERR_INVALID;
    return fs_lpc_init_impl(c, crop, max_batch, max_samples, seed);
}

int fs_lpc_harvest(fs_ctx *c, int32_t per_solve, int32_t *added) {
    if (!c) return FS_ERR_INVALID;
    int a = 0;
    int rc = fs_lpc_harvest_impl(c, per_solve, &a);
    if (added) *added = a;
    return rc;
}

int fs_lpc_train(fs_ctx *c, int32_t iters, int32_t batch, float lr, uint64_t seed, float *loss_hist) {
    if (!c) return FS_ERR_INVALID;
    if (iters < 0) return fs_set_error(c, FS_ERR_INVALID, "iters must be >= 0");
    return fs_lpc_train_impl(c, iters, batch, lr, seed, loss_hist);
}

int fs_lpc_use(fs_ctx *c, int32_t on) {
    if (!c) return FS_ERR_INVALID;
    if (on && !c->lpc) return fs_set_error(c, FS_ERR_INVALID, "learned preconditioner not initialised");
    if (on < 0 || on > 2) return fs_set_error(c, FS_ERR_INVALID, "fs_lpc_use mode %d not 0, 1 or 2", on);
    c->lpc_on = on;   // the solver keeps one CG graph with and one without the network
    c->lpc_t_nn = -1.0;
    c->lpc_t_plain = -1.0;
    c->lpc_use_next = 1;
    c->lpc_since_probe = 0;
    c->lpc_probe_every = 25;
    c->lpc_probe_pending = 0;
    c->lpc_solves = c->lpc_nn_solves = 0;
    return FS_OK;
}

int fs_lpc_weights(fs_ctx *c, float *w, int64_t n, int32_t to_device) {
    if (!c || !w) return FS_ERR_INVALID;
    if (!c->lpc) return fs_set_error(c, FS_ERR_INVALID, "learned preconditioner not initialised");
    LpcState *L = c->lpc;
    if ((size_t)n != L->net.nparam) return fs_set_error(c, FS_ERR_INVALID, "expected %zu parameters", L->net.nparam);
    cudaError_t e;
    if (to_device) {
        e = cudaMemcpyAsync(L->w, w, n * sizeof(float), cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(L->m, 0, n * sizeof(float), c->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(L->v, 0, n * sizeof(float), c->stream);
        L->adam_t = 0;
        if (e == cudaSuccess) lpc_refresh(L, c->stream);
    } else {
        e = cudaMemcpyAsync(w, L->w, n * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return fs_cuda_check(c, e, "learned preconditioner weights");
}

int fs_lpc_grad(fs_ctx *c, const float *feat, const float *tgt, const float *mask, int32_t batch, float *grad,
                float *loss, float *pred) {
    if (!c || !feat || !tgt || !mask) return FS_ERR_INVALID;
    return fs_lpc_grad_impl(c, feat, tgt, mask, batch, grad, loss, pred);
}

int fs_lpc_info(fs_ctx *c, int32_t *h, int32_t *w, int32_t *nsamples, int64_t *nparam, int32_t *off,
                int64_t *solves, int64_t *nn_solves) {
    if (!c) return FS_ERR_INVALID;
    if (!c->lpc) return fs_set_error(c, FS_ERR_INVALID, "learned preconditioner not initialised");
    if (h) *h = c->lpc->Hn;
    if (w) *w = c->lpc->Wn;
    if (nsamples) *nsamples = c->lpc->nsamp < c->lpc->Nmax ? c->lpc->nsamp : c->lpc->Nmax;
    if (nparam) *nparam = (int64_t)c->lpc->net.nparam;
    if (off) *off = c->h_ctrl->lpc_off;
    if (solves) *solves = c->lpc_solves;
    if (nn_solves) *nn_solves = c->lpc_nn_solves;
    return FS_OK;
}

// The converted record of the level-1 fields into dev (5 nx ny doubles),
// queued on the context's stream.
cudaError_t fs_output_stage(fs_ctx *c, double *dev, double x03) {
    const int ns = c->cfg.nspecies, lv = c->lev[0];
    const size_t n = (size_t)c->nx * c->ny;
    const int nb = (int)std::min<size_t>((n + 255) / 256, 4096);
    k_output_record<<<nb, 256, 0, c->stream>>>(c->ph, c->sp[0].buf[lv], c->sp[1].buf[lv], c->sp[2].buf[lv],
                                               ns == 4 ? c->sp[3].buf[lv] : nullptr, c->nx, c->ny, c->pitch, x03,
                                               c->k.ph0, dev);
    return cudaGetLastError();
}
