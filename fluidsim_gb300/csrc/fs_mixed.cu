// fs_mixed.cu -- the particle step in mixed precision (FS_PREC_MIXED).
//
// Same algorithm as fs_ptcl.cu (ptclEqn ptcl_lib.F90:99-550, rk_step
// ptcl_props.F90:71-139, circ_step circ_lib.F90:19-210), with the flux/RHS
// evaluation in FP32 on densities stored as FP32 log-densities, and FP64 kept
// for the accepted-state accumulation (n = n3 + dt * sum c_i k_i is formed in
// FP64 from the FP32 increment) and for the RK-Merson error norm.
//
// Log form of the Scharfetter-Gummel flux.  With B(x) = x/(e^x - 1) and the
// cell Peclet number a = q mu E h / D,
//   F = (D/h) (B(-a) n_L - B(a) n_R)
//     = (D/h) B(-a) n_L (1 - exp(l_R - l_L - a))    for a >= 0
//     = -(D/h) B(a) n_R (1 - exp(l_L - l_R + a))    for a <  0,
// which is get_Flux (ptcl_props.F90:142-165) rearranged: the difference that
// cancels near Boltzmann equilibrium is carried by expm1 to full FP32 relative
// accuracy, and B uses its series 1 - x/2 + x^2/12 near x = 0.
//
// Stored FP32 fields: ln n_i, ln n_e and, for the energy density, the log of
// the mean energy in eV, ln(n_eps ph0 / n_e), with ln n_eps recovered as
// ln n_e + that - ln ph0.  The mean energy indexes the rate table, whose
// Arrhenius-like rates amplify an error in ln(eps) by ~15.8/eps; stored this
// way it has the rounding of a number of magnitude |ln eps_eV| < 4 instead
// of that of ln n_eps (up to ~13).
#include <cmath>
#include <cstdio>
#include <cuda_runtime.h>

#include "fs_internal.h"
#include "fs_wall.cuh"

#define BX 32
#define BY 8
#define NT (BX * BY)
#define HX (BX + 2)
#define HY (BY + 2)

namespace {

// B(x) = x/(e^x - 1)
__device__ __forceinline__ float bern(float x) {
    if (fabsf(x) < 1e-3f) return 1.0f - 0.5f * x + x * x * (1.0f / 12.0f);
    return x / expm1f(x);
}

// The three Scharfetter-Gummel fluxes of one face from log densities, branch
// free.  With s = sign(a) and the upwind node u (left for a >= 0):
//   F = s C_u n_u (1 - exp(s (l_R - l_L) - |a|)),
// C_u = (D/h) B(-|a|) -- for the ions the precomputed cl (a >= 0) or cr.
// The electron and energy fluxes share a = -mue E h / De and B(-|a|)
// (mut/Dt = mue/De, ptcl_lib.F90:142-143).
__device__ __forceinline__ void sg3(float ai, float cl, float cr, float ae, float g, float niL, float niR, float liL,
                                    float liR, float neL, float neR, float leL, float leR, float ntL, float ntR,
                                    float ltL, float ltR, float &fi, float &fe, float &ft) {
    const bool ui = ai >= 0.0f;
    const float si = ui ? 1.0f : -1.0f;
    fi = si * (ui ? cl * niL : cr * niR) * (-expm1f(si * (liR - liL) - fabsf(ai)));
    const float x = fabsf(ae);
    const float b = x < 1e-3f ? 1.0f + 0.5f * x + x * x * (1.0f / 12.0f) : x / (-expm1f(-x));
    const bool ue = ae >= 0.0f;
    const float gb = (ue ? g : -g) * b;
    const float se = ue ? 1.0f : -1.0f;
    fe = gb * (ue ? neL : neR) * (-expm1f(se * (leR - leL) - x));
    ft = (5.0f / 3.0f) * gb * (ue ? ntL : ntR) * (-expm1f(se * (ltR - ltL) - x));
}

// -B'(x), the coefficient of dFdPh: dF/dv = -B'(-a) n_L - B'(a) n_R
__device__ __forceinline__ float mbprime(float x) {
    if (fabsf(x) < 0.5f) {
        float x2 = x * x;
        return 0.5f - x * (1.0f / 6.0f - x2 * (1.0f / 180.0f - x2 * (1.0f / 5040.0f - x2 * (1.0f / 151200.0f))));
    }
    if (x > 0.0f) {
        float em = expf(-x), d = 1.0f - em;
        return -(em / d - x * em / (d * d));
    }
    float ex = expf(x), d = expm1f(x);
    return -((d - x * ex) / (d * d));
}

struct FaceMixArgs {
    PhysParams pp;
    PhysF f;
    MeshDev m;
    MeshF mf;
    const double *ph;
    double *fx_e, *fy_e;     // FP64 face fields (the assembly's Laplacian needs them)
    float *f32[10];          // fx_e, fx_cl, fx_cr, fx_dl, fx_dr, fy_e, fy_cl, fy_cr, fy_dl, fy_dr
};

// Face data while phi is frozen: E (FP64 and FP32), the ion flux
// coefficients cl = (Di/h) B(-a), cr = (Di/h) B(a) and the ion dFdPh
// coefficients -B'(-a), -B'(a) (0 where |mui E| < 1e-12, as dFdPh).
__device__ __forceinline__ void ion_face32(const PhysF &pf, float E, float h, float ih, float *out) {
    const float a = pf.mui_Di * E * h;
    const float d = pf.Di * ih;
    out[0] = E;
    out[1] = d * bern(-a);
    out[2] = d * bern(a);
    if (fabsf(pf.mui * E) < 1e-12f) {
        out[3] = out[4] = 0.0f;
    } else {
        out[3] = mbprime(-a);
        out[4] = mbprime(a);
    }
}

__global__ void k_faces_mix(const FaceMixArgs a) {
    const int gi = blockIdx.x * blockDim.x + threadIdx.x, gj = blockIdx.y * blockDim.y + threadIdx.y;
    const int nx = a.pp.nx, ny = a.pp.ny, P = a.pp.pitch;
    if (gi > nx || gj > ny) return;
    const size_t o = (size_t)gj * P + gi;
    float v[5];
    if (gj >= 1) {
        double E = -(a.ph[o + 1] - a.ph[o]) * a.m.inv_dx[gi];
        a.fx_e[o] = E;
        ion_face32(a.f, (float)E, a.mf.dx[gi], a.mf.inv_dx[gi], v);
        for (int k = 0; k < 5; k++) a.f32[k][o] = v[k];
    }
    if (gi >= 1) {
        double E = -(a.ph[o + P] - a.ph[o]) * a.m.inv_dy[gj];
        a.fy_e[o] = E;
        ion_face32(a.f, (float)E, a.mf.dy[gj], a.mf.inv_dy[gj], v);
        for (int k = 0; k < 5; k++) a.f32[5 + k][o] = v[k];
    }
}

// FP32 log companion of a whole field (ghost ring included): ln n, or with a
// denominator field ln(scale * n / den) -- the energy density is kept as the
// log of the mean energy in eV, ln(n_eps ph0 / n_e)
__global__ void k_log32(const double *n, const double *den, double scale, float *l, size_t cnt) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < cnt; i += (size_t)gridDim.x * blockDim.x) {
        double v = den ? scale * n[i] / den[i] : n[i];
        l[i] = logf(fmaxf((float)v, 1e-30f));
    }
}

__global__ void k_d2f(const double *in, float *out, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = (float)in[i];
}

// circ_step ghosts in mixed mode: phi ghost and both face fields of the row
__global__ void k_circ_ghost_mix(double *ph, const int8_t *tx, const double *r, const double *dx,
                                 double *fx_e64, float *fx_e32, int nx, int ny, int P, double ew, double vd) {
    int gj = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (gj > ny) return;
    const size_t o = (size_t)gj * P;
    if (r[gj] <= ew) {
        if (tx[(gj - 1) * nx + 0] == -2) {
            ph[o + 0] = vd / 2.0;
            double E = -(ph[o + 1] - ph[o + 0]) / dx[0];
            fx_e64[o + 0] = E;
            fx_e32[o + 0] = (float)E;
        }
        if (tx[(gj - 1) * nx + nx - 1] == 2) {
            ph[o + nx + 1] = vd / (-2.0);
            double E = -(ph[o + nx + 1] - ph[o + nx]) / dx[nx];
            fx_e64[o + nx] = E;
            fx_e32[o + nx] = (float)E;
        }
    }
}

struct StageMixArgs {
    PhysParams pp;
    PhysF f;
    MeshDev m;
    MeshF mf;
    const float *tab;               // FP32 table, FS_TAB_STRIDE floats per node
    const float *lin[FS_MAX_SPECIES];
    const float *lbase[FS_MAX_SPECIES];     // FP32 log companions of the base state
    const double *nbase[FS_MAX_SPECIES];
    double *nout[FS_MAX_SPECIES];   // FP64 output (stages 4 and 5), else null
    float *lout[FS_MAX_SPECIES];
    const float *k1[FS_MAX_SPECIES];
    const float *k3[FS_MAX_SPECIES];
    const float *k4[FS_MAX_SPECIES];
    float *kout[FS_MAX_SPECIES];
    const double *ph;
    const float *fx_e, *fx_cl, *fx_cr, *fy_e, *fy_cl, *fy_cr;
    Ctrl *ctrl;
    double *part;
    double *rows;
    WallArgs wall;                  // dielectric wall (FP64): charge, slopes, FP64 table
    int rows_every_stage;           // the RC circuit needs the electrode current after every stage
    int stage;
    int nblk;
};

__device__ __forceinline__ void tab32(const StageMixArgs &a, float lneps, int &k, float &w) {
    float u = (lneps - a.f.lemin) * a.f.inv_h;
    if (!(u >= 0.0f)) u = 0.0f;
    if (u > a.f.ntab_m1) u = a.f.ntab_m1;
    int i = (int)u;
    if (i > a.pp.ntab - 2) i = a.pp.ntab - 2;
    k = i;
    w = u - (float)i;
}
__device__ __forceinline__ float tv32(const float *tab, int k, float w, int row) {
    const float *t = tab + (size_t)k * FS_TAB_STRIDE;
    return __ldg(t + row) + w * __ldg(t + 8 + row);
}

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

template <int NS>
__global__ void __launch_bounds__(NT, 4) k_stage_mix(const StageMixArgs a) {
    __shared__ float s_l[NS][HY][HX];
    __shared__ float s_n[NS][HY][HX];
    __shared__ float s_te[HY][HX], s_mue[HY][HX], s_de[HY][HX];
    __shared__ float s_w[BY][BX];
    __shared__ int s_k[BY][BX];
    __shared__ float s_fx[NS][BY][BX + 1];
    __shared__ float s_fy[NS][BY + 1][BX];
    __shared__ float s_ex[BY][BX + 1];
    __shared__ float s_ey[BY + 1][BX];
    __shared__ double s_red[NS][NT / 32];
    __shared__ double s_tm[NT / 32];

    const PhysParams &pp = a.pp;
    const int nx = pp.nx, ny = pp.ny, P = pp.pitch;
    const int tid = threadIdx.x;
    const int gx0 = blockIdx.x * BX + 1, gy0 = blockIdx.y * BY + 1;
    const PhysF &pf = a.f;
    const float ln_ph0 = pf.ln_ph0;
    const float mui = pf.mui, vi = pf.vi, gam = pf.gam;
    const float mui_Di = pf.mui_Di;
    const float ve_c = pf.ve_c, t0_x0 = pf.t0_x0;
    unsigned int st = 0;

    // tile + halo: log densities, densities, mean energy and its table coefficients
    for (int q = tid; q < HX * HY; q += NT) {
        int lx = q % HX, ly = q / HX;
        int gi = gx0 - 1 + lx, gj = gy0 - 1 + ly;
        bool in = gi <= nx + 1 && gj <= ny + 1;
        size_t o = (size_t)gj * P + gi;
        float lw = 0.0f;
#pragma unroll
        for (int s = 0; s < NS; s++) {
            float l = in ? a.lin[s][o] : 0.0f;
            if (s == 2) {                   // stored: ln(mean energy in eV)
                lw = l;
                l = s_l[1][ly][lx] + lw - ln_ph0;
            }
            s_l[s][ly][lx] = l;
            s_n[s][ly][lx] = expf(l);
        }
        float te = 0, mu = 0, de = 0;
        if (gi >= 1 && gi <= nx && gj >= 1 && gj <= ny) {
            te = expf(lw - ln_ph0);
            int k; float w;
            tab32(a, lw, k, w);
            mu = tv32(a.tab, k, w, 0);
            de = tv32(a.tab, k, w, 1);
            if (lx >= 1 && lx <= BX && ly >= 1 && ly <= BY) { s_k[ly - 1][lx - 1] = k; s_w[ly - 1][lx - 1] = w; }
        }
        s_te[ly][lx] = te; s_mue[ly][lx] = mu; s_de[ly][lx] = de;
    }
    __syncthreads();

    // x faces between gi = gx0-1+c and gi+1
    for (int q = tid; q < BY * (BX + 1); q += NT) {
        int c = q % (BX + 1), r = q / (BX + 1);
        int gi = gx0 - 1 + c, gj = gy0 + r;
        if (gj > ny || gi > nx) continue;
        int lx = c, ly = r + 1;
        const size_t of = (size_t)gj * P + gi;
        float E = a.fx_e[of];
        float fi = 0, fe = 0, ft = 0, fm = 0, eu = E;
        int tl = gi >= 1 ? a.m.tx[(gj - 1) * nx + gi - 1] : 0;
        int tr = gi + 1 <= nx ? a.m.tx[(gj - 1) * nx + gi] : 0;
        if (gi == 0 && tr == -1) {
            eu = 0.0f;
        } else if (gi == nx && tl == 1) {
            eu = 0.0f;
        } else if ((gi == 0 && tr == -2) || (gi == nx && tl == 2)) {
            const bool left = gi == 0;
            const int lc = left ? lx + 1 : lx;
            const size_t og = (size_t)gj * P + (left ? 0 : nx + 1), oc = (size_t)gj * P + (left ? 1 : nx);
            float te = s_te[ly][lc], ni = s_n[0][ly][lc], ne = s_n[1][ly][lc], nt = s_n[2][ly][lc];
            float aa = (a.ph[og] > a.ph[oc]) ? 1.0f : 0.0f;
            float mue = s_mue[ly][lc], mut = (5.0f / 3.0f) * mue;
            float ve = sqrtf(ve_c * te) * t0_x0;
            float sgn = left ? -1.0f : 1.0f;
            fi = (1.0f - aa) * mui * E * ni + sgn * (0.25f * vi * ni);
            fe = -(aa * mue * E * ne) + sgn * (0.25f * ve * ne) - gam * fi;
            ft = -(aa * mut * E * nt) + sgn * ((1.0f / 3.0f) * ve * nt) - gam * te * fi;
            if (NS == 4) fm = sgn * (0.5f * vi * s_n[3][ly][lc]);
        } else {
            float dh = a.mf.dx[gi], idh = a.mf.inv_dx[gi];
            float mue = 0.5f * (s_mue[ly][lx] + s_mue[ly][lx + 1]);
            float De = 0.5f * (s_de[ly][lx] + s_de[ly][lx + 1]);
            float ai = E * dh * mui_Di;
            float ae = -mue * E * dh / De, g = De * idh;
            sg3(ai, a.fx_cl[of], a.fx_cr[of], ae, g, s_n[0][ly][lx], s_n[0][ly][lx + 1], s_l[0][ly][lx],
                s_l[0][ly][lx + 1], s_n[1][ly][lx], s_n[1][ly][lx + 1], s_l[1][ly][lx], s_l[1][ly][lx + 1],
                s_n[2][ly][lx], s_n[2][ly][lx + 1], s_l[2][ly][lx], s_l[2][ly][lx + 1], fi, fe, ft);
            if (NS == 4) fm = -pf.Dm * (s_n[3][ly][lx + 1] - s_n[3][ly][lx]) * idh;
            if (a.stage == 5 || a.rows_every_stage) {
                if (gi == 1 && a.m.dr_a[gj] != 0.0) a.rows[gj] = a.m.dr_a[gj] * (double)(fi - fe);
                if (gi == nx - 1 && a.m.dr_c[gj] != 0.0) a.rows[(ny + 2) + gj] = a.m.dr_c[gj] * (double)(fi - fe);
            }
        }
        s_fx[0][r][c] = fi; s_fx[1][r][c] = fe; s_fx[2][r][c] = ft;
        if (NS == 4) s_fx[3][r][c] = fm;
        s_ex[r][c] = eu;
    }
    __syncthreads();
    // y faces between gj = gy0-1+r and gj+1
    for (int q = tid; q < (BY + 1) * BX; q += NT) {
        int c = q % BX, r = q / BX;
        int gi = gx0 + c, gj = gy0 - 1 + r;
        if (gi > nx || gj > ny) continue;
        int lx = c + 1, ly = r;
        const size_t of = (size_t)gj * P + gi;
        float E = a.fy_e[of];
        float fi = 0, fe = 0, ft = 0, fm = 0, eu = E;
        int tb = gj >= 1 ? a.m.ty[(gj - 1) * nx + gi - 1] : 0;
        int tt = gj + 1 <= ny ? a.m.ty[gj * nx + gi - 1] : 0;
        if (gj == 0 && tt == -1) {
            eu = 0.0f;
        } else if (gj == 0 && tt == -2) {
            // no lower y electrode flux in ptclEqn: zero flux, face field kept
        } else if (gj == ny && tb == 1) {
            eu = 0.0f;
        } else if (gj == ny && tb == 3) {
            const int lc = ly;
            double wfi, wfe, wft, wfm;
            eu = (float)fs_wall_face<NS>(pp, a.wall, a.m.dy[ny], a.ctrl->dt, a.stage, gi, s_te[lc][lx],
                                         s_n[0][lc][lx], s_n[1][lc][lx], s_n[2][lc][lx],
                                         NS == 4 ? s_n[3][lc][lx] : 0.0f, s_mue[lc][lx], s_de[lc][lx], wfi, wfe,
                                         wft, wfm, st);
            fi = (float)wfi; fe = (float)wfe; ft = (float)wft; fm = (float)wfm;
        } else if (gj == ny && tb == 2) {
            const int lc = ly;
            const size_t og = (size_t)(ny + 1) * P + gi, oc = (size_t)ny * P + gi;
            float te = s_te[lc][lx], ni = s_n[0][lc][lx], ne = s_n[1][lc][lx], nt = s_n[2][lc][lx];
            float aa = (a.ph[og] > a.ph[oc]) ? 1.0f : 0.0f;
            float mue = s_mue[lc][lx], mut = (5.0f / 3.0f) * mue;
            float ve = sqrtf(ve_c * te) * t0_x0;
            fi = (1.0f - aa) * mui * E * ni + 0.25f * vi * ni;
            float fix = s_fx[0][lc - 1][lx];   // x-direction ion flux (ptcl_lib.F90:427-433)
            fe = -(aa * mue * E * ne) + 0.25f * ve * ne - gam * fix;
            ft = -(aa * mut * E * nt) + (1.0f / 3.0f) * ve * nt - gam * te * fix;
            if (NS == 4) fm = 0.5f * vi * s_n[3][lc][lx];
        } else {
            float dh = a.mf.dy[gj], idh = a.mf.inv_dy[gj];
            float mue = 0.5f * (s_mue[ly][lx] + s_mue[ly + 1][lx]);
            float De = 0.5f * (s_de[ly][lx] + s_de[ly + 1][lx]);
            float ai = E * dh * mui_Di;
            float ae = -mue * E * dh / De, g = De * idh;
            sg3(ai, a.fy_cl[of], a.fy_cr[of], ae, g, s_n[0][ly][lx], s_n[0][ly + 1][lx], s_l[0][ly][lx],
                s_l[0][ly + 1][lx], s_n[1][ly][lx], s_n[1][ly + 1][lx], s_l[1][ly][lx], s_l[1][ly + 1][lx],
                s_n[2][ly][lx], s_n[2][ly + 1][lx], s_l[2][ly][lx], s_l[2][ly + 1][lx], fi, fe, ft);
            if (NS == 4) fm = -pf.Dm * (s_n[3][ly + 1][lx] - s_n[3][ly][lx]) * idh;
        }
        s_fy[0][r][c] = fi; s_fy[1][r][c] = fe; s_fy[2][r][c] = ft;
        if (NS == 4) s_fy[3][r][c] = fm;
        s_ey[r][c] = eu;
    }
    __syncthreads();

    const int lx = tid % BX, ly = tid / BX;
    const int gi = gx0 + lx, gj = gy0 + ly;
    double qerr[NS];
#pragma unroll
    for (int s = 0; s < NS; s++) qerr[s] = 0.0;
    double tm = 1e300;
    if (gi <= nx && gj <= ny) {
        const size_t o = (size_t)gj * P + gi;
        const int hx = lx + 1, hy = ly + 1;
        const float te = s_te[hy][hx];
        const float ni = s_n[0][hy][hx], ne = s_n[1][hy][hx];
        const float nm = NS == 4 ? s_n[3][hy][hx] : 0.0f;
        const int kk = s_k[ly][lx];
        const float w = s_w[ly][lx];
        const float k_ir = tv32(a.tab, kk, w, 2), k_ex = tv32(a.tab, kk, w, 3);
        const float nu = tv32(a.tab, kk, w, 4), beta = tv32(a.tab, kk, w, 5);
        const float idlx = a.mf.inv_dlx[gi - 1], idly = a.mf.inv_dly[gj - 1];
        float dfdx[NS], dfdy[NS];
        if (pp.cyl) {
            const float r0 = a.mf.r[gj], rp = a.mf.r[gj + 1] + r0, rm = r0 + a.mf.r[gj - 1];
#pragma unroll
            for (int s = 0; s < NS; s++) {
                dfdx[s] = (s_fx[s][ly][lx + 1] - s_fx[s][ly][lx]) * idlx;
                dfdy[s] = (s_fy[s][ly + 1][lx] * rp * 0.5f - s_fy[s][ly][lx] * rm * 0.5f) * idly / r0;
            }
        } else {
#pragma unroll
            for (int s = 0; s < NS; s++) {
                dfdx[s] = (s_fx[s][ly][lx + 1] - s_fx[s][ly][lx]) * idlx;
                dfdy[s] = (s_fy[s][ly + 1][lx] - s_fy[s][ly][lx]) * idly;
            }
        }
        const float fex = (s_fx[1][ly][lx + 1] + s_fx[1][ly][lx]) * 0.5f;
        const float exa = (s_ex[ly][lx] + s_ex[ly][lx + 1]) * 0.5f;
        const float fey = (s_fy[1][ly + 1][lx] + s_fy[1][ly][lx]) * 0.5f;
        const float eya = (s_ey[ly][lx] + s_ey[ly + 1][lx]) * 0.5f;
        const float ninf = pf.ninf;
        float term_sie = k_ir * ninf * ne - beta * ni * ne;
        float k_si = 0.0f, k_sc = 0.0f;
        if (NS == 4) {
            k_sc = tv32(a.tab, kk, w, 6);
            k_si = tv32(a.tab, kk, w, 7);
            term_sie = term_sie + k_si * nm * ne + pf.k_mp * (nm * nm);
        }
        const float term_st1 = -(fex * exa + fey * eya);
        const float term_st2 = -(ne * nu * pf.me_mi * (te / 1.5f - pf.tg_term));
        const float term_st3 = -(pf.h_ir * k_ir * ninf * ne) - pf.h_si * k_si * nm * ne
                             - pf.h_ex * k_ex * ninf * ne;
        float kv[NS];
        kv[0] = -dfdx[0] - dfdy[0] + term_sie;
        kv[1] = -dfdx[1] - dfdy[1] + term_sie;
        kv[2] = -dfdx[2] - dfdy[2] + term_st1 + term_st2 + term_st3;
        if (NS == 4) {
            float term_sm = k_ex * ninf * ne - k_si * nm * ne - k_sc * nm * ne - pf.k_r * nm * ne
                          - 2.0f * pf.k_mp * (nm * nm) - pf.k_2q * ninf * nm
                          - pf.k_3q_ninf2 * nm;
            kv[3] = -dfdx[3] - dfdy[3] + term_sm;
        }
        const double dt = a.ctrl->dt;
        const float dtf = (float)dt;
        const int stg = a.stage;
        float vf[NS];
        float lb[NS];
        if (stg <= 3) {   // intermediate stage states: FP32 from the FP32 log base
#pragma unroll
            for (int s = 0; s < NS; s++) lb[s] = a.lbase[s][o];
        }
#pragma unroll
        for (int s = 0; s < NS; s++) {
            if (isnan(kv[s])) st |= FS_ST_NAN;
            if (a.kout[s]) a.kout[s][o] = kv[s];
            float comb;
            if (stg == 1) comb = kv[s] * (1.0f / 3.0f);
            else if (stg == 2) comb = (a.k1[s][o] + kv[s]) * (1.0f / 6.0f);
            else if (stg == 3) comb = (a.k1[s][o] + kv[s] * 3.0f) * 0.125f;
            else if (stg == 4) comb = (a.k1[s][o] - a.k3[s][o] * 3.0f + kv[s] * 4.0f) * 0.5f;
            else comb = (a.k1[s][o] + a.k4[s][o] * 4.0f + kv[s]) * (1.0f / 6.0f);
            if (stg <= 3) {
                const float n3 = expf(s == 2 ? lb[1] + lb[2] - ln_ph0 : lb[s]);
                vf[s] = fmaxf(n3 + dtf * comb, pf.nmin[s]);
                continue;
            }
            // stages 4 and 5 produce the states the step keeps: FP64 accumulation
            const double n3 = a.nbase[s][o];
            const double v = fmax(n3 + dt * (double)comb, pp.nmin[s]);
            vf[s] = (float)v;
            a.nout[s][o] = v;
            if (stg == 5) {
                const double k1 = a.k1[s][o], k3 = a.k3[s][o], k4 = a.k4[s][o];
                // the Merson combination cancels to O(dt^4): formed in FP64
                const float err = (float)fabs(dt * (k1 * (2.0 / 30.0) - k3 * (3.0 / 10.0) + k4 * (4.0 / 15.0)
                                                    - (double)kv[s] * (1.0 / 30.0)));
                const float qq = err / (pf.abs_tol + pf.rel_tol * fabsf((float)n3));
                qerr[s] = (double)(qq * qq);
            }
        }
#pragma unroll
        for (int s = 0; s < NS; s++)
            a.lout[s][o] = s == 2 ? logf(vf[2] * pf.ph0 / vf[1]) : logf(vf[s]);
        if (stg == 5) {
            const int ty = a.m.ty[(gj - 1) * nx + gi - 1], tx = a.m.tx[(gj - 1) * nx + gi - 1];
            float mue2;
            if (ty == 0 || ty < 0) mue2 = 0.5f * (s_mue[hy][hx] + s_mue[hy + 1][hx]);
            else if (ty == 1 && (tx == 0 || tx < 0)) mue2 = 0.5f * (s_mue[hy][hx] + s_mue[hy][hx + 1]);
            else mue2 = s_mue[hy][hx];
            tm = (double)(1.0f / (mue2 * ne + mui * ni));
        }
    }
    if (st) atomicOr(&a.ctrl->status, st);
    if (a.stage == 5) {
        const int wid = tid >> 5, lane = tid & 31;
#pragma unroll
        for (int s = 0; s < NS; s++) {
            double v = warp_sum(qerr[s]);
            if (lane == 0) s_red[s][wid] = v;
        }
        for (int o = 16; o > 0; o >>= 1) tm = fmin(tm, __shfl_down_sync(0xffffffffu, tm, o));
        if (lane == 0) s_tm[wid] = tm;
        __syncthreads();
        if (tid < NS) {
            double v = 0.0;
            for (int wv = 0; wv < NT / 32; wv++) v += s_red[tid][wv];
            a.part[(size_t)tid * a.nblk + blockIdx.y * gridDim.x + blockIdx.x] = v;
        }
        if (tid == 0) {
            double m = s_tm[0];
            for (int wv = 1; wv < NT / 32; wv++) m = fmin(m, s_tm[wv]);
            if (m > 0.0 && m < 1e300)
                atomicMin((unsigned long long *)&a.ctrl->t_m, (unsigned long long)__double_as_longlong(m));
        }
    }
}

}  // namespace

// ---------------------------------------------------------------- host side
int fs_mixed_alloc(fs_ctx *c, const std::vector<double> &rows) {
    const size_t n = c->field_elems;
    cudaError_t e = cudaSuccess;
    for (int s = 0; s < c->cfg.nspecies && e == cudaSuccess; s++) {
        for (int b = 0; b < FS_NBUF && e == cudaSuccess; b++) e = cudaMalloc(&c->lbuf[s][b], n * sizeof(float));
        for (int k = 0; k < 3 && e == cudaSuccess; k++) {
            e = cudaMalloc(&c->k32[s][k], n * sizeof(float));
            if (e == cudaSuccess) e = cudaMemset(c->k32[s][k], 0, n * sizeof(float));
        }
    }
    for (int f = 0; f < 10 && e == cudaSuccess; f++) {
        e = cudaMalloc(&c->f32[f], n * sizeof(float));
        if (e == cudaSuccess) e = cudaMemset(c->f32[f], 0, n * sizeof(float));
    }
    if (e != cudaSuccess) return fs_cuda_check(c, e, "cudaMalloc (mixed)");
    const int nt = c->cfg.table_n;
    std::vector<float> t((size_t)nt * FS_TAB_STRIDE, 0.0f);
    for (int i = 0; i < nt; i++)
        for (int r = 0; r < 8; r++) {
            t[(size_t)i * FS_TAB_STRIDE + r] = (float)rows[(size_t)r * nt + i];
            t[(size_t)i * FS_TAB_STRIDE + 8 + r] =
                i + 1 < nt ? (float)(rows[(size_t)r * nt + i + 1] - rows[(size_t)r * nt + i]) : 0.0f;
        }
    e = cudaMalloc(&c->d_tab32, t.size() * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpy(c->d_tab32, t.data(), t.size() * sizeof(float), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fs_cuda_check(c, e, "mixed table");

    // FP32 constants
    const PhysParams &p = c->pp;
    PhysF &f = c->pf;
    f.ph0 = (float)p.ph0; f.ln_ph0 = (float)std::log(p.ph0);
    f.mui = (float)p.mui; f.vi = (float)p.vi; f.gam = (float)p.gam; f.Di = (float)p.Di;
    f.mui_Di = (float)(p.mui / p.Di);
    f.ve_c = (float)p.ve_coef; f.t0_x0 = (float)(p.t0 / p.x0);
    f.Dm = (float)p.Dm; f.ninf = (float)p.ninf; f.me_mi = (float)(p.me / p.mi);
    f.tg_term = (float)(p.tg * p.kb / p.e / p.ph0);
    f.h_ir = (float)p.h_ir; f.h_ex = (float)p.h_ex; f.h_si = (float)p.h_si;
    f.k_mp = (float)p.k_mp; f.k_r = (float)p.k_r; f.k_2q = (float)p.k_2q;
    f.k_3q_ninf2 = (float)(p.k_3q * p.ninf * p.ninf);
    f.lemin = (float)p.lemin; f.inv_h = (float)p.inv_h; f.ntab_m1 = (float)(p.ntab - 1);
    f.abs_tol = (float)p.abs_tol; f.rel_tol = (float)p.rel_tol;
    for (int q = 0; q < FS_MAX_SPECIES; q++) f.nmin[q] = (float)p.nmin[q];
    // FP32 mesh: the FP64 blob converted element by element, same offsets
    const size_t nblob = (size_t)(c->mesh.dr_c - c->d_mesh_blob) + c->ny + 2;
    e = cudaMalloc(&c->d_meshf, nblob * sizeof(float));
    if (e != cudaSuccess) return fs_cuda_check(c, e, "cudaMalloc (FP32 mesh)");
    c->launches++;
    k_d2f<<<64, 256, 0, c->stream>>>(c->d_mesh_blob, c->d_meshf, nblob);
    auto fp = [&](const double *d) { return (const float *)(c->d_meshf + (d - c->d_mesh_blob)); };
    MeshF &m = c->meshf;
    m.dx = fp(c->mesh.dx); m.dy = fp(c->mesh.dy); m.inv_dx = fp(c->mesh.inv_dx); m.inv_dy = fp(c->mesh.inv_dy);
    m.dlx = fp(c->mesh.dlx); m.dly = fp(c->mesh.dly); m.inv_dlx = fp(c->mesh.inv_dlx);
    m.inv_dly = fp(c->mesh.inv_dly); m.r = fp(c->mesh.r);
    return fs_cuda_check(c, cudaGetLastError(), "FP32 mesh");
}

void fs_mixed_free(fs_ctx *c) {
    for (int s = 0; s < FS_MAX_SPECIES; s++) {
        for (int b = 0; b < FS_NBUF; b++) cudaFree(c->lbuf[s][b]);
        for (int k = 0; k < 3; k++) cudaFree(c->k32[s][k]);
    }
    for (int f = 0; f < 10; f++) cudaFree(c->f32[f]);
    cudaFree(c->d_tab32);
    cudaFree(c->d_meshf);
}

int fs_mixed_sync_logs(fs_ctx *c) {
    for (int s = 0; s < c->cfg.nspecies; s++)
        for (int b = 0; b < FS_NBUF; b++) {
            c->launches++;
            k_log32<<<2 * c->nsm, 256, 0, c->stream>>>(c->sp[s].buf[b], s == 2 ? c->sp[1].buf[b] : nullptr,
                                                        c->pp.ph0, c->lbuf[s][b], c->field_elems);
        }
    return fs_cuda_check(c, cudaGetLastError(), "log densities");
}

void fs_faces_update_mixed(fs_ctx *c) {
    if (c->faces_valid) return;
    FaceMixArgs f;
    f.pp = c->pp;
    f.f = c->pf;
    f.m = c->mesh;
    f.mf = c->meshf;
    f.ph = c->ph;
    f.fx_e = c->fx_e;
    f.fy_e = c->fy_e;
    for (int k = 0; k < 10; k++) f.f32[k] = c->f32[k];
    dim3 b(32, 8), g((c->nx + 1 + 31) / 32, (c->ny + 1 + 7) / 8);
    fs_prof_begin(c, PROF_OTHER);
    k_faces_mix<<<g, b, 0, c->stream>>>(f);
    fs_prof_end(c);
    c->faces_valid = 1;
}

// ptcl_step in mixed precision: buffer handling as fs_ptcl_step_impl; stages
// 1-3 only produce the FP32 log state, stages 4 and 5 also the FP64 one.
int fs_ptcl_step_mixed(fs_ctx *c, int *attempts_out) {
    const int ns = c->cfg.nspecies;
    const int L2 = c->lev[1], L3 = c->lev[2];
    int freeb[FS_NBUF], nf = 0;
    for (int b = 0; b < FS_NBUF; b++)
        if (b != L2 && b != L3) freeb[nf++] = b;
    const int SA = freeb[0], SB = freeb[1], OUT = freeb[2];
    int in1 = L2;
    int attempts = 0;
    const bool rc_circuit = c->cfg.rf == 1;
    // source voltage at the step's time (circ_lib.F90:26-50); without the RC
    // circuit the electrode voltage is the source's (:176-177)
    c->Vsrc = fs_circ_source(c->cfg, c->k, c->t);
    fs_ptcl_reset(c);
    fs_faces_update_mixed(c);
    dim3 grid((c->nx + BX - 1) / BX, (c->ny + BY - 1) / BY);
    for (;;) {
        attempts++;
        StageMixArgs a;
        memset(&a, 0, sizeof(a));
        a.pp = c->pp;
        a.f = c->pf;
        a.m = c->mesh;
        a.mf = c->meshf;
        a.tab = c->d_tab32;
        a.ph = c->ph;
        a.fx_e = c->f32[0]; a.fx_cl = c->f32[1]; a.fx_cr = c->f32[2];
        a.fy_e = c->f32[5]; a.fy_cl = c->f32[6]; a.fy_cr = c->f32[7];
        a.ctrl = c->d_ctrl;
        a.part = c->d_part;
        a.rows = c->d_rows;
        a.wall = {c->d_tab, fs_sig(c, 2), fs_sig(c, 1), fs_sig(c, 0), fs_sig_ks(c)};
        a.rows_every_stage = rc_circuit;
        a.nblk = c->nblk_stage;
        const int ins[5] = {in1, SA, SB, SA, SB};
        const int outs[5] = {SA, SB, SA, SB, OUT};
        for (int stg = 1; stg <= 5; stg++) {
            a.stage = stg;
            for (int s = 0; s < ns; s++) {
                a.lin[s] = c->lbuf[s][ins[stg - 1]];
                a.nbase[s] = c->sp[s].buf[L3];
                a.lbase[s] = c->lbuf[s][L3];
                a.lout[s] = c->lbuf[s][outs[stg - 1]];
                a.nout[s] = stg >= 4 ? c->sp[s].buf[outs[stg - 1]] : nullptr;
                a.k1[s] = c->k32[s][0];
                a.k3[s] = c->k32[s][1];
                a.k4[s] = c->k32[s][2];
                a.kout[s] = stg == 1 ? c->k32[s][0] : stg == 3 ? c->k32[s][1] : stg == 4 ? c->k32[s][2] : nullptr;
            }
            fs_prof_begin(c, PROF_STAGE);
            if (ns == 4) k_stage_mix<4><<<grid, NT, 0, c->stream>>>(a);
            else k_stage_mix<3><<<grid, NT, 0, c->stream>>>(a);
            fs_prof_end(c);
            if (rc_circuit) {
                fs_circuit_launch(c, stg, c->f32[0]);
            } else if (stg == 1) {
                c->launches++;
                k_circ_ghost_mix<<<(c->ny + 127) / 128, 128, 0, c->stream>>>(
                    c->ph, c->mesh.tx, c->mesh.r, c->mesh.dx, c->fx_e, c->f32[0], c->nx, c->ny, c->pitch,
                    c->cfg.ew, c->Vsrc);
            }
        }
        int rc = fs_ptcl_control(c);
        if (rc) return rc;
        const Ctrl &h = *c->h_ctrl;
        if (rc_circuit) {
            c->Vd_pl = h.vd_pl;
            c->Vd_mi = h.vd_mi;
        } else {
            c->Vd_pl = c->Vd_mi = c->Vsrc;
        }
        if (!h.rejected) break;
        c->st.rk_rejects++;
        c->Vd_pl = c->Vd_or;
        c->Vd_mi = c->Vd_or;
        if (c->rwall && ((rc = fs_sig_copy(c, 0, 2)) || (rc = fs_sig_copy(c, 1, 2)))) return rc;
        in1 = L3;
        if (attempts > 100000) return fs_set_error(c, FS_ERR_MIN_DT, "RK restart limit");
    }
    c->lev[0] = OUT;
    c->lev[1] = SB;
    c->dt = c->h_ctrl->dt;
    c->st.attempts += attempts;
    if (attempts_out) *attempts_out = attempts;
    return FS_OK;
}
