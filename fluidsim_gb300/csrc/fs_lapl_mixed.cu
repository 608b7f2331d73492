// fs_lapl_mixed.cu -- the semi-implicit Poisson solve in mixed precision
// (FS_PREC_MIXED).
//
// Same system as fs_lapl.cu (laplEqn lapl_lib.F90:123-379, laplJ :381-609,
// dFdPh :611-636), split by precision:
//   * assembly: the flux and flux-derivative terms (every exponential) and
//     the matrix coefficients in FP32; the Gauss-law part of the right-hand
//     side, div E + n_i - n_e, and the assembled right-hand side in FP64;
//   * the multigrid hierarchy and every V-cycle in FP32;
//   * CG in FP64: the iterate, the residual, the search directions, the
//     operator product (FP64 arithmetic on the FP32 coefficients) and every
//     dot product.  Each V-cycle solves the correction equation for the FP64
//     residual in FP32 -- the iterative-refinement step -- and the outer
//     iteration is flexible CG (beta = z_new.(r_new - r_old) / z_old.r_old),
//     which tolerates the rounding of the FP32 preconditioner, so the
//     residual reaches lapl_rtol exactly as in the FP64 solver.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <chrono>
#include <cstring>
#include <vector>
#include <cuda_runtime.h>

#include "fs_internal.h"
#include "fs_lpc.cuh"
#include "fs_mg.cuh"
#include "fs_wall.cuh"

#define ABX 32
#define ABY 8
#define ANT (ABX * ABY)

namespace {

// B(x) = x/(e^x - 1) at +-a and -B'(+-a), from one expm1f.
//   bm = B(-a), bp = B(a), dm = -B'(-a), dp = -B'(a);  dm + dp = 1.
__device__ __forceinline__ void bern4(float a, float &bm, float &bp, float &dm, float &dp) {
    const float x = fabsf(a);
    const float d = -expm1f(-x);          // 1 - e^-x
    const float em = 1.0f - d;
    float b_neg, b_pos, d_pos;            // B(-x), B(x), -B'(x) for x >= 0
    if (x < 1e-3f) {
        b_neg = 1.0f + 0.5f * x + x * x * (1.0f / 12.0f);
        b_pos = 1.0f - 0.5f * x + x * x * (1.0f / 12.0f);
    } else {
        b_neg = x / d;
        b_pos = b_neg * em;
    }
    if (x < 0.5f) {
        const float x2 = x * x;
        d_pos = 0.5f - x * (1.0f / 6.0f - x2 * (1.0f / 180.0f - x2 * (1.0f / 5040.0f - x2 * (1.0f / 151200.0f))));
    } else {
        d_pos = em * (x - d) / (d * d);
    }
    const bool pos = a >= 0.0f;
    bm = pos ? b_neg : b_pos;
    bp = pos ? b_pos : b_neg;
    dp = pos ? d_pos : 1.0f - d_pos;
    dm = pos ? 1.0f - d_pos : d_pos;
}

struct AsmMixArgs {
    PhysParams pp;
    PhysF f;
    MeshDev m;
    MeshF mf;
    const float *tab;
    const double *ni, *ne, *nt, *ph, *phm;
    const double *fx_e, *fy_e;
    const float *f32[10];
    const Ctrl *ctrl;
    Ctrl *ctrl_w;
    const double *tab64;      // FP64 table (the dielectric wall's row)
    const double *sig;        // sig_pl of the dielectric wall, nx+2
    float *mc, *ce, *cn, *extra, *inv_mc;
    double *rhs;
};

__device__ __forceinline__ void tab32(const PhysParams &pp, const PhysF &pf, float lneps, int &k, float &w) {
    float u = (lneps - pf.lemin) * pf.inv_h;
    if (!(u >= 0.0f)) u = 0.0f;
    if (u > pf.ntab_m1) u = pf.ntab_m1;
    int i = (int)u;
    if (i > pp.ntab - 2) i = pp.ntab - 2;
    k = i;
    w = u - (float)i;
}
__device__ __forceinline__ float tv32(const float *tab, int k, float w, int row) {
    const float *t = tab + (size_t)k * FS_TAB_STRIDE;
    return __ldg(t + row) + w * __ldg(t + 8 + row);
}

// Interior face: ion and electron fluxes and the face conductance
// 1/h + dt (mui/h dFi + mue/h dFe).
__device__ __forceinline__ void sg_face_mix(const PhysF &pf, const float *fc, size_t of, float E,
                                            float Emi, bool same, float dh, float idh, float mue, float De,
                                            float nil, float nir, float nel, float ner, float dt,
                                            float &fi, float &fe, float &cf) {
    const float mui = pf.mui;
    fi = fc[1] * nil - fc[2] * nir;
    float dFi;
    if (same) {
        dFi = fc[3] * nil + fc[4] * nir;
    } else {
        float bm, bp, dm, dp;
        bern4(pf.mui_Di * Emi * dh, bm, bp, dm, dp);
        dFi = fabsf(mui * Emi) < 1e-12f ? 0.0f : dm * nil + dp * nir;
    }
    float bm, bp, dm, dp;
    const float ae = -mue * E * dh / De;
    bern4(ae, bm, bp, dm, dp);
    fe = De * idh * (bm * nel - bp * ner);
    float dFe;
    if (same) {
        dFe = fabsf(mue * E) < 1e-12f ? 0.0f : dm * nel + dp * ner;
    } else {
        bern4(-mue * Emi * dh / De, bm, bp, dm, dp);
        dFe = fabsf(mue * Emi) < 1e-12f ? 0.0f : dm * nel + dp * ner;
    }
    cf = idh + dt * (mui * idh * dFi + mue * idh * dFe);
}

__global__ void __launch_bounds__(ANT, 3) k_assemble_mix(const AsmMixArgs a) {
    __shared__ float s_ni[ABY + 2][ABX + 2], s_ne[ABY + 2][ABX + 2];
    __shared__ float s_te[ABY + 2][ABX + 2], s_mu[ABY + 2][ABX + 2], s_de[ABY + 2][ABX + 2];
    __shared__ float s_xfi[ABY][ABX + 1], s_xfe[ABY][ABX + 1], s_xc[ABY][ABX + 1];
    __shared__ float s_yfi[ABY + 1][ABX], s_yfe[ABY + 1][ABX], s_yc[ABY + 1][ABX];
    __shared__ double s_xe[ABY][ABX + 1], s_ye[ABY + 1][ABX];
    const PhysParams &pp = a.pp;
    const int nx = pp.nx, ny = pp.ny, P = pp.pitch;
    const int tid = threadIdx.x;
    const int gx0 = blockIdx.x * ABX + 1, gy0 = blockIdx.y * ABY + 1;
    const double dt = a.ctrl->dt;
    const float dtf = (float)dt;
    const PhysF &pf = a.f;
    const float ln_ph0 = pf.ln_ph0;
    const float mui = pf.mui, vi = pf.vi, gam = pf.gam;
    const float ve_c = pf.ve_c, t0_x0 = pf.t0_x0;
    unsigned int st = 0;
    for (int q = tid; q < (ABX + 2) * (ABY + 2); q += ANT) {
        int lx = q % (ABX + 2), ly = q / (ABX + 2);
        int gi = gx0 - 1 + lx, gj = gy0 - 1 + ly;
        bool in = gi <= nx + 1 && gj <= ny + 1;
        size_t o = (size_t)gj * P + gi;
        float ni = in ? (float)a.ni[o] : 0.0f, ne = in ? (float)a.ne[o] : 0.0f;
        s_ni[ly][lx] = ni;
        s_ne[ly][lx] = ne;
        float te = 0, mu = 0, de = 0;
        if (gi >= 1 && gi <= nx && gj >= 1 && gj <= ny) {
            const float nt32 = (float)a.nt[o];
            float lneps;
            if ((nt32 >= 0.0f) && (ne >= 0.0f)) {
                te = nt32 / ne;
                lneps = logf(nt32 * pf.ph0 / ne);   // ln(mean energy in eV)
            } else {
                st |= FS_ST_NEG_DENSITY;
                te = 1e-8f;
                lneps = logf(1e-8f) + ln_ph0;
            }
            int k; float w;
            tab32(pp, pf, lneps, k, w);
            mu = tv32(a.tab, k, w, 0);
            de = tv32(a.tab, k, w, 1);
        }
        s_te[ly][lx] = te; s_mu[ly][lx] = mu; s_de[ly][lx] = de;
    }
    __syncthreads();
    // x faces between gi and gi+1
    for (int q = tid; q < ABY * (ABX + 1); q += ANT) {
        int c = q % (ABX + 1), r = q / (ABX + 1);
        int gi = gx0 - 1 + c, gj = gy0 + r;
        if (gj > ny || gi > nx) continue;
        int lx = c, ly = r + 1;
        const size_t of = (size_t)gj * P + gi;
        const float dh = a.mf.dx[gi], idh = a.mf.inv_dx[gi];
        const double E64 = a.fx_e[of];
        const float E = a.f32[0][of];
        int tl = gi >= 1 ? a.m.tx[(gj - 1) * nx + gi - 1] : 0;
        int tr = gi + 1 <= nx ? a.m.tx[(gj - 1) * nx + gi] : 0;
        float fi = 0, fe = 0, cf = 0;
        double eu = E64;
        if (gi == 0 && tr == -1) {
            eu = 0.0;
        } else if (gi == nx && tl == 1) {
            eu = 0.0;
        } else if ((gi == 0 && tr == -2) || (gi == nx && tl == 2)) {   // electrode rows
            const bool left = gi == 0;
            const int lc = left ? lx + 1 : lx;
            const size_t og = (size_t)gj * P + (left ? 0 : nx + 1), oc = (size_t)gj * P + (left ? 1 : nx);
            const float te = s_te[ly][lc], ni = s_ni[ly][lc], ne = s_ne[ly][lc], mue = s_mu[ly][lc];
            const int ac = (a.ph[og] > a.ph[oc]) ? 1 : 0;
            const float aa = (float)ac;
            const float ve = sqrtf(ve_c * te) * t0_x0;
            const float sgn = left ? -1.0f : 1.0f;
            fi = (1.0f - aa) * mui * E * ni + sgn * (0.25f * vi * ni);
            fe = -(aa * mue * E * ne) + sgn * (0.25f * ve * ne) - gam * fi;
            float dfi, dfe;
            if (left) {
                dfi = (float)(1 - ac) * mui * ni * idh;
                dfe = -((float)ac * mue * ne * idh) - gam * dfi;
                cf = idh + dtf * (dfi - dfe);
            } else {
                dfi = (float)(ac - 1) * mui * ni * idh;
                dfe = (float)ac * mue * ne * idh - gam * dfi;
                cf = idh - dtf * (dfi - dfe);
            }
        } else {
            const float mue = 0.5f * (s_mu[ly][lx] + s_mu[ly][lx + 1]);
            const float De = 0.5f * (s_de[ly][lx] + s_de[ly][lx + 1]);
            const size_t ol = (size_t)gj * P + gi;
            const bool same = a.phm[ol] == a.ph[ol] && a.phm[ol + 1] == a.ph[ol + 1];
            const float Emi = same ? E : (float)(-(a.phm[ol + 1] - a.phm[ol]) * a.m.inv_dx[gi]);
            const float fc[5] = {E, a.f32[1][of], a.f32[2][of], a.f32[3][of], a.f32[4][of]};
            sg_face_mix(pf, fc, of, E, Emi, same, dh, idh, mue, De, s_ni[ly][lx], s_ni[ly][lx + 1],
                        s_ne[ly][lx], s_ne[ly][lx + 1], dtf, fi, fe, cf);
            if (isnan(cf)) st |= FS_ST_DFDPH_NAN;
        }
        s_xfi[r][c] = fi; s_xfe[r][c] = fe; s_xe[r][c] = eu; s_xc[r][c] = cf;
    }
    // y faces between gj and gj+1
    for (int q = tid; q < (ABY + 1) * ABX; q += ANT) {
        int c = q % ABX, r = q / ABX;
        int gi = gx0 + c, gj = gy0 - 1 + r;
        if (gi > nx || gj > ny) continue;
        int lx = c + 1, ly = r;
        const size_t of = (size_t)gj * P + gi;
        const float dh = a.mf.dy[gj], idh = a.mf.inv_dy[gj];
        const double E64 = a.fy_e[of];
        const float E = a.f32[5][of];
        int tb = gj >= 1 ? a.m.ty[(gj - 1) * nx + gi - 1] : 0;
        int tt = gj + 1 <= ny ? a.m.ty[gj * nx + gi - 1] : 0;
        float fi = 0, fe = 0, cf = 0;
        double eu = E64;
        if (gj == 0 && tt == -1) {
            eu = 0.0;
        } else if (gj == 0 && tt == -2) {
            // laplEqn has no lower y electrode flux (zero); laplJ has its derivative
            const int lc = ly + 1;
            const float ni = s_ni[lc][lx], ne = s_ne[lc][lx], mue = s_mu[lc][lx];
            const int ac = (a.ph[(size_t)0 * P + gi] > a.ph[(size_t)1 * P + gi]) ? 1 : 0;
            const float dfi = (float)(1 - ac) * mui * ni / dh;
            const float dfe = -((float)ac * mue * ne / dh) - gam * dfi;
            cf = 1.0f / dh + dtf * (dfi - dfe);
        } else if (gj == ny && tb == 1) {
            eu = 0.0;
        } else if (gj == ny && tb == 3) {
            // dielectric wall, one row, in FP64 as on the FP64 path: field
            // -sig (lapl_lib.F90:72-76,263-265), fluxes into an empty wall node
            // with the node's own coefficients (:322-331), a boundary
            // conductance of 1/dy without dt terms (:590-600)
            const size_t on = (size_t)ny * P + gi;
            const double ni = a.ni[on], ne = a.ne[on], nt = a.nt[on];
            const double te = (nt >= 0.0) && (ne >= 0.0) ? nt / ne : 1e-8;
            double mu, de;
            fs_wall_tab(pp, a.tab64, te, mu, de);
            const double E = -a.sig[gi], dh64 = a.m.dy[gj];
            eu = E;
            fi = (float)fs_sg_flux(1.0, E, dh64, pp.mui, pp.Di, ni, 0.0);
            fe = (float)fs_sg_flux(-1.0, E, dh64, mu, de, ne, 0.0);
            cf = idh;
        } else if (gj == ny && tb == 2) {
            const int lc = ly;
            const float te = s_te[lc][lx], ni = s_ni[lc][lx], ne = s_ne[lc][lx], mue = s_mu[lc][lx];
            const int ac = (a.ph[(size_t)(ny + 1) * P + gi] > a.ph[(size_t)ny * P + gi]) ? 1 : 0;
            const float aa = (float)ac;
            const float ve = sqrtf(ve_c * te) * t0_x0;
            fi = (1.0f - aa) * mui * E * ni + 0.25f * vi * ni;
            fe = -(aa * mue * E * ne) + 0.25f * ve * ne - gam * fi;
            const float dfi = (float)(ac - 1) * mui * ni / dh;
            const float dfe = (float)ac * mue * ne / dh - gam * dfi;
            cf = 1.0f / dh - dtf * (dfi - dfe);
        } else {
            const float mue = 0.5f * (s_mu[ly][lx] + s_mu[ly + 1][lx]);
            const float De = 0.5f * (s_de[ly][lx] + s_de[ly + 1][lx]);
            const size_t ol = (size_t)gj * P + gi;
            const bool same = a.phm[ol] == a.ph[ol] && a.phm[ol + P] == a.ph[ol + P];
            const float Emi = same ? E : (float)(-(a.phm[ol + P] - a.phm[ol]) * a.m.inv_dy[gj]);
            const float fc[5] = {E, a.f32[6][of], a.f32[7][of], a.f32[8][of], a.f32[9][of]};
            sg_face_mix(pf, fc, of, E, Emi, same, dh, idh, mue, De, s_ni[ly][lx], s_ni[ly + 1][lx],
                        s_ne[ly][lx], s_ne[ly + 1][lx], dtf, fi, fe, cf);
            if (isnan(cf)) st |= FS_ST_DFDPH_NAN;
        }
        s_yfi[r][c] = fi; s_yfe[r][c] = fe; s_ye[r][c] = eu; s_yc[r][c] = cf;
    }
    __syncthreads();
    const int lx = tid % ABX, ly = tid / ABX;
    const int gi = gx0 + lx, gj = gy0 + ly;
    if (gi <= nx && gj <= ny) {
        const size_t o = (size_t)gj * P + gi;
        const int tx = a.m.tx[(gj - 1) * nx + gi - 1], ty = a.m.ty[(gj - 1) * nx + gi - 1];
        // Gauss-law part in FP64
        const double idlx = a.m.inv_dlx[gi - 1];
        double dfdx = -(s_xe[ly][lx + 1] - s_xe[ly][lx]) * idlx;
        double dfdy;
        if (pp.cyl) {
            const double wr = a.m.r[gj], wn = (a.m.r[gj + 1] + wr) / 2.0, ws = (wr + a.m.r[gj - 1]) / 2.0;
            dfdy = -(s_ye[ly + 1][lx] * wn - s_ye[ly][lx] * ws) / a.m.dly[gj - 1] / wr;
        } else {
            dfdy = -(s_ye[ly + 1][lx] - s_ye[ly][lx]) * a.m.inv_dly[gj - 1];
        }
        // flux divergence and the conductances in FP32
        const float fdlx = a.mf.dlx[gi - 1], fdly = a.mf.dly[gj - 1];
        const float fidlx = a.mf.inv_dlx[gi - 1], fidly = a.mf.inv_dly[gj - 1];
        float fwr = 1.0f, fwn = 1.0f, fws = 1.0f;
        if (pp.cyl) {
            fwr = a.mf.r[gj];
            fwn = 0.5f * (a.mf.r[gj + 1] + fwr);
            fws = 0.5f * (fwr + a.mf.r[gj - 1]);
        }
        float div = ((s_xfi[ly][lx + 1] - s_xfi[ly][lx]) - (s_xfe[ly][lx + 1] - s_xfe[ly][lx])) * fidlx;
        if (pp.cyl)
            div += ((s_yfi[ly + 1][lx] * fwn - s_yfi[ly][lx] * fws) - (s_yfe[ly + 1][lx] * fwn - s_yfe[ly][lx] * fws))
                   * fidly / fwr;
        else
            div += ((s_yfi[ly + 1][lx] - s_yfi[ly][lx]) - (s_yfe[ly + 1][lx] - s_yfe[ly][lx])) * fidly;
        double b = dfdx + dfdy + (a.ni[o] - a.ne[o]) - dt * (double)div;
        if (isnan(b)) st |= FS_ST_BNAN;
        const float cw = s_xc[ly][lx], cee = s_xc[ly][lx + 1], cs = s_yc[ly][lx], cnn = s_yc[ly + 1][lx];
        const float offw = gi > 1 ? cw : 0.0f, offe = gi < nx ? cee : 0.0f;
        const float offs = gj > 1 ? cs : 0.0f, offn = gj < ny ? cnn : 0.0f;
        float gx = 0.0f, gys = 0.0f, gyn = 0.0f;
        if (gi == 1 && tx == -2) gx += cw;
        if (gi == nx && tx == 2) gx += cee;
        if (gj == 1 && ty == -2) gys += cs;
        if (gj == ny && (ty == 2 || ty == 3)) gyn += cnn;
        if (gi == 1 && tx == -1) gx += a.mf.inv_dx[0] - a.mf.inv_dx[1];
        if (gj == 1 && ty == -1) gyn += a.mf.inv_dy[0] - a.mf.inv_dy[1];
        const float sx = fdly * fwr;
        const float extra = gx * sx + (gys * fws + gyn * fwn) * fdlx;
        const float mc = (offw + offe) * sx + (offs * fws + offn * fwn) * fdlx + extra;
        a.mc[o] = mc;
        a.inv_mc[o] = 1.0f / mc;
        a.extra[o] = extra;
        a.ce[o] = offe * sx;
        a.cn[o] = offn * fwn * fdlx;
        // the CG runs on M d = D b, D = dlx dly r; 1/D is written by k_dinv once
        a.rhs[o] = b * (a.m.dlx[gi - 1] * a.m.dly[gj - 1] * (pp.cyl ? a.m.r[gj] : 1.0));
    }
    if (st) atomicOr(&a.ctrl_w->status, st);
}

// 1/D of the row scaling D = dlx dly r (a property of the mesh)
__global__ void k_dinv(const MeshDev m, int nx, int ny, int P, int cyl, double *dinv, float *dinv32) {
    const int gi = blockIdx.x * blockDim.x + threadIdx.x + 1, gj = blockIdx.y * blockDim.y + threadIdx.y + 1;
    if (gi > nx || gj > ny) return;
    const double d = 1.0 / (m.dlx[gi - 1] * m.dly[gj - 1] * (cyl ? m.r[gj] : 1.0));
    dinv[(size_t)gj * P + gi] = d;
    dinv32[(size_t)gj * P + gi] = (float)d;
}

// --------------------------------------------- FP32 CG under FP64 refinement
// Outer loop: r = D b - M x to FP64 accuracy, ||r|| / ||b|| checked against
// lapl_rtol.  Inner loop: flexible PCG with FP32 vectors and the FP32 V-cycle
// on the current residual, the iterate accumulated as a float-float pair
// (~48-bit significand; FP32 arithmetic, which this GPU issues ~60 times
// faster than FP64), run until its FP32
// recurrence residual has fallen by inner_tol = 1e-4 (or just enough to reach
// lapl_rtol, or inner_max iterations); then the refinement recomputes the
// true residual in float-float, and the inner loop goes on from it with its
// search direction kept (CG with reliable updates).  The FP32
// recurrence drifts from the true residual (rounding of the FP32 vectors and
// operator products); the refinement removes the drift, so the converged
// residual is the true FP64 one.  Dot products: FP32 sums in a fixed order
// (grid_sumf), the refinement's of power-of-two scaled values.
struct CgmArgs {
    int nx, ny, P, nblk;
    dim3 grid;
    double *rhs, *dinv, *part;           // FP64: D b, 1/D; reduction partials
    float *xh, *xl;                      // the iterate as a float-float pair xh + xl
    const float *dinv32;                 // 1/D rounded to FP32 (the refinement's norm)
    float *z, *r32, *p, *q, *w;          // FP32 inner vectors (z, r32 are level 0 of the V-cycle; w = M z)
    const float *ce, *cn, *extra;
    Ctrl *ctrl;
    double rtol, inner_tol2;
    int maxit, inner_max;
    int lpc;                             // the learned correction is part of the preconditioner
    int use_cond;
    cudaGraphConditionalHandle cond;
};


// Fixed-order FP32 sums of N per-thread values over the grid (warp shuffles,
// then the eight warps, then the CTAs' partials by the last CTA); true in the
// last CTA, whose thread 0 holds the sums in out.  part needs N * nblk floats.
// The inner iteration's dot products are sums of FP32 products and feed FP32
// updates, so FP32 sums (relative error ~1e-6 over 10^6 terms) lose nothing
// that matters; FP64 sums would cost more than the kernel's streaming: a
// warp-wide FP64 add occupies an SM's FP64 pipe for ~16 cycles on this GPU.
template <int N>
__device__ bool grid_sumf(float (&v)[N], float *part, unsigned int *counter, int nblk, double (&out)[N]) {
    __shared__ float s_p[N][8];
    __shared__ bool s_last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    auto block_sum = [&]() {   // v (per thread) -> s_p[k][0..7] -> v[k] in thread 0
#pragma unroll
        for (int k = 0; k < N; k++)
            for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
        if (lane == 0)
            for (int k = 0; k < N; k++) s_p[k][wid] = v[k];
        __syncthreads();
        if (threadIdx.x == 0)
            for (int k = 0; k < N; k++) {
                float r = 0.0f;
                for (int wv = 0; wv < 8; wv++) r += s_p[k][wv];
                v[k] = r;
            }
    };
    block_sum();
    if (threadIdx.x == 0) {
        for (int k = 0; k < N; k++) part[(size_t)k * nblk + blockIdx.x] = v[k];
        __threadfence();
        s_last = atomicAdd(counter, 1u) == (unsigned int)nblk - 1u;
    }
    __syncthreads();
    if (!s_last) return false;
    __threadfence();
    // all N partials of a stride issued together (one L2 round trip per
    // stride), each value's sum in stride order; loads bypass L1 (the
    // writers' __threadfence and the counter make them visible in L2)
#pragma unroll
    for (int k = 0; k < N; k++) v[k] = 0.0f;
    for (int b = threadIdx.x; b < nblk; b += 256) {
        float t[N];
#pragma unroll
        for (int k = 0; k < N; k++) t[k] = __ldcg(part + (size_t)k * nblk + b);
#pragma unroll
        for (int k = 0; k < N; k++) v[k] += t[k];
    }
    __syncthreads();   // every thread is past its reads of s_p above
    block_sum();
    if (threadIdx.x == 0) {
        for (int k = 0; k < N; k++) out[k] = (double)v[k];
        *counter = 0u;
    }
    return true;
}

// x = 0, r = D b (FP64), r32 = r; ||b||, ||r32||
__global__ void __launch_bounds__(256) k_cgm_init(const CgmArgs a) {
    double v = 0.0, w = 0.0;
    CG_NODES(a, {
        const double b = a.rhs[o];
        const float b32 = (float)b;
        a.xh[o] = 0.0f;
        a.xl[o] = 0.0f;
        a.r32[o] = b32;
        a.p[o] = 0.0f;
        a.q[o] = 0.0f;
        const double u = b * a.dinv[o];
        v += u * u;
        w += (double)(b32 * b32);
    })
    double sv, sw;
    if (grid_sum2(v, w, a.part, &a.ctrl->counter[0], a.nblk, sv, sw) && threadIdx.x == 0) {
        Ctrl *c = a.ctrl;
        c->bnorm2 = sv;
        c->rnorm2 = sv;
        c->r0in2 = sw;
        c->relres = sv > 0.0 ? 1.0 : 0.0;
        c->cg_done = sv == 0.0 ? 1 : 0;
        c->cg_iters = 0;
        c->cg_fail = 0;
        c->inner_it = 0;
        c->refine = 0;
        c->rz = 0.0;
        c->alpha = 0.0;
        c->rr_prev = sw;
        c->lpc_off = 0;
        c->lpc_stalls = 0;
        c->cgm_restarted = 1;
    }
}

__device__ __forceinline__ float4 ld4(const float *p, size_t o) { return *reinterpret_cast<const float4 *>(p + o); }
__device__ __forceinline__ void st4(float *p, size_t o, float4 v) { *reinterpret_cast<float4 *>(p + o) = v; }
__device__ __forceinline__ float dot4(float4 a, float4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }

// The inner-loop kernels stream whole rows 1..ny in float4 steps: every
// inner vector and coefficient is zero on the ghost ring and the row padding,
// so those lanes add nothing to the dot products and stay zero.

// Float-float values hi + lo (|lo| <= ulp(hi) / 2) by error-free
// transformations: Knuth's two-sum, Dekker's fast two-sum and the FMA
// two-product; the _rn intrinsics keep the compiler from contracting them.
struct FF {
    float h, l;
};
__device__ __forceinline__ FF ff_fast2(float a, float b) {   // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ FF ff_sum(FF a, FF b) {
    const float s = __fadd_rn(a.h, b.h), bb = __fsub_rn(s, a.h);
    const float e = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bb)), __fsub_rn(b.h, bb));
    return ff_fast2(s, __fadd_rn(e, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ FF ff_neg(FF a) { return {-a.h, -a.l}; }
__device__ __forceinline__ FF ff_mulf(FF a, float c) {   // (a.h + a.l) c
    const float p = __fmul_rn(a.h, c);
    return ff_fast2(p, __fmaf_rn(a.l, c, __fmaf_rn(a.h, c, -p)));
}
// a double split into a float-float pair (three FP64-pipe instructions)
__device__ __forceinline__ FF ff_from(double d) {
    const float h = __double2float_rn(d);
    return {h, __double2float_rn(d - (double)h)};
}

// Warm start, as in the FP64 solver: the previous solve's correction d (the
// float-float iterate, still in xh + xl) scaled by the alpha that minimises
// |D^-1 (D b - alpha M d)|, the norm the convergence test takes, is the
// initial guess; the refinement kernel then forms its residual in
// float-float arithmetic, so alpha itself needs no more than FP32 accuracy
// (M d of the leading part xh, FP32 sums; a sum that overflows or vanishes
// gives alpha = 0, the zero start).  This kernel: the three sums, alpha
// (spare[1]) and the control block reset of k_cgm_init, with the refinement
// requested (relres starts infinite, so that the refinement's "did the
// residual fall" holds).
__global__ void __launch_bounds__(256) k_cgm_init_warm(const CgmArgs a) {
    float v[3] = {0.0f, 0.0f, 0.0f};
    CG_NODES(a, {
        const float d0 = a.xh[o];
        const float md = a.ce[o] * (d0 - a.xh[o + 1]) + a.ce[o - 1] * (d0 - a.xh[o - 1])
                       + a.cn[o] * (d0 - a.xh[o + a.P]) + a.cn[o - a.P] * (d0 - a.xh[o - a.P]) + a.extra[o] * d0;
        const float bw = (float)a.rhs[o] * a.dinv32[o], mw = md * a.dinv32[o];
        v[0] += bw * bw;
        v[1] += bw * mw;
        v[2] += mw * mw;
    })
    double s[3];
    if (grid_sumf<3>(v, reinterpret_cast<float *>(a.part), &a.ctrl->counter[0], a.nblk, s) && threadIdx.x == 0) {
        Ctrl *c = a.ctrl;
        double al = s[2] > 0.0 ? s[1] / s[2] : 0.0;
        if (!isfinite(al)) al = 0.0;
        c->spare[1] = al;
        c->cg_done = 0;   // decided by the refinement on the exact |D b|
        c->cg_iters = 0;
        c->cg_fail = 0;
        c->inner_it = 0;
        c->refine = 1;
        c->relres = INFINITY;
        c->rz = 0.0;
        c->alpha = 0.0;
        c->pq = 0.0;
        c->lpc_off = 0;
        c->lpc_stalls = 0;
        c->cgm_restarted = 1;
    }
}

// x = alpha d in float-float arithmetic (0 for the zero start); p = q = 0;
// |D b|^2 for the convergence test (FP64 sum), and a zero right-hand side
// ends the solve here
__global__ void __launch_bounds__(256) k_cgm_init_apply(const CgmArgs a) {
    const double al = a.ctrl->spare[1];
    const FF alf = ff_from(al);
    double vb = 0.0;
    CG_NODES(a, {
        const float xh = a.xh[o], xl = a.xl[o];
        const float pr = __fmul_rn(alf.h, xh);
        const float t = __fmaf_rn(alf.h, xl, __fmaf_rn(alf.l, xh, __fmaf_rn(alf.h, xh, -pr)));
        const FF x = ff_fast2(pr, t);
        a.xh[o] = al != 0.0 ? x.h : 0.0f;
        a.xl[o] = al != 0.0 ? x.l : 0.0f;
        a.p[o] = 0.0f;
        a.q[o] = 0.0f;
        const double u = a.rhs[o] * a.dinv[o];
        vb += u * u;
    })
    double sb;
    if (grid_sum<256>(vb, a.part, &a.ctrl->counter[0], a.nblk, &sb) && threadIdx.x == 0) {
        Ctrl *c = a.ctrl;
        c->bnorm2 = sb;
        c->rnorm2 = sb;
        if (sb == 0.0) {
            c->cg_done = 1;
            c->relres = 0.0;
        }
    }
}

// M z at one node in float-float arithmetic: each face term c (z_i - z_j) is
// formed exactly (the difference of neighbouring, similar values is exact,
// the product's rounding error is recovered with an FMA) and the terms are
// summed with error-free additions, so the FP32 result carries an error of
// ~eps |M z| instead of ~eps sum_f |c_f (z_i - z_j)|.  For the smooth
// corrections of the first refinement cycle the face terms are ~1e3 times
// larger than their sum, and a plainly rounded M z lets the FP32 residual
// drift away from the true one by ~5e-4 relative within a few iterations.
__device__ __forceinline__ void ff_add(float &hi, float &lo, float p, float pe) {
    const float s = __fadd_rn(hi, p);
    const float bb = __fsub_rn(s, hi);
    const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    hi = s;
    lo = __fadd_rn(lo, __fadd_rn(e, pe));
}
__device__ __forceinline__ float mz_ff(float z, float ze, float zw, float zn, float zs, float ce, float cw, float cn,
                                       float cs, float ex) {
    float hi = 0.0f, lo = 0.0f;
    float d, p;
    d = __fsub_rn(z, ze); p = __fmul_rn(ce, d); ff_add(hi, lo, p, __fmaf_rn(ce, d, -p));
    d = __fsub_rn(z, zw); p = __fmul_rn(cw, d); ff_add(hi, lo, p, __fmaf_rn(cw, d, -p));
    d = __fsub_rn(z, zn); p = __fmul_rn(cn, d); ff_add(hi, lo, p, __fmaf_rn(cn, d, -p));
    d = __fsub_rn(z, zs); p = __fmul_rn(cs, d); ff_add(hi, lo, p, __fmaf_rn(cs, d, -p));
    p = __fmul_rn(ex, z); ff_add(hi, lo, p, __fmaf_rn(ex, z, -p));
    return __fadd_rn(hi, lo);
}

// After the V-cycle, one pass and one reduction (the Chronopoulos-Gear
// arrangement of the iteration): w = M z (float-float stencil), rz = r32.z,
// zq = z.q and zw = z.w.  The flexible beta = -alpha z.q / rz_old (Notay's
// FCG(1): -z.(M p_old) / p_old.(M p_old)), and p.q of the new directions
// p = z + beta p_old, q = w + beta q_old follows from the same sums:
// p.q = z.w + 2 beta z.q + beta^2 (p_old.q_old), with p_old.(M z) = q_old.z
// for the symmetric M.  alpha = rz / p.q.  The same reduction carries r.r,
// r.w, r.q, w.w, w.q and q.q, from which the norm of the updated residual
// r - alpha q_new follows without a second reduction:
// |r|^2 - 2 alpha (r.w + beta r.q) + alpha^2 (w.w + 2 beta w.q + beta^2 q.q),
// each sum taken fresh from the vectors (no recurrence to drift), so that
// k_cgm_upd is a plain pointwise update; the refinement and stall decisions
// are taken here from that norm.
__global__ void __launch_bounds__(256) k_cgm_rzw(const CgmArgs a) {
    if (a.ctrl->cg_done || a.ctrl->cg_fail) return;
    const int P = a.P;
    float v = 0.0f, u = 0.0f, t = 0.0f, rr = 0.0f, rw = 0.0f, rq = 0.0f, ww = 0.0f, wq = 0.0f, qq = 0.0f;
    CG_VEC4(a, {
        const float4 z = ld4(a.z, o), zn = ld4(a.z, o + P), zs = ld4(a.z, o - P);
        const float zw = a.z[o - 1], ze = a.z[o + 4];
        const float4 ce = ld4(a.ce, o), cn = ld4(a.cn, o), cs = ld4(a.cn, o - P), ex = ld4(a.extra, o);
        const float cw = a.ce[o - 1];
        float4 mz;
        mz.x = mz_ff(z.x, z.y, zw, zn.x, zs.x, ce.x, cw, cn.x, cs.x, ex.x);
        mz.y = mz_ff(z.y, z.z, z.x, zn.y, zs.y, ce.y, ce.x, cn.y, cs.y, ex.y);
        mz.z = mz_ff(z.z, z.w, z.y, zn.z, zs.z, ce.z, ce.y, cn.z, cs.z, ex.z);
        mz.w = mz_ff(z.w, ze, z.z, zn.w, zs.w, ce.w, ce.z, cn.w, cs.w, ex.w);
        st4(a.w, o, mz);
        const float4 r = ld4(a.r32, o), q = ld4(a.q, o);
        v += dot4(r, z);
        u += dot4(z, q);
        t += dot4(z, mz);
        rr += dot4(r, r);
        rw += dot4(r, mz);
        rq += dot4(r, q);
        ww += dot4(mz, mz);
        wq += dot4(mz, q);
        qq += dot4(q, q);
    })
    float in[9] = {v, u, t, rr, rw, rq, ww, wq, qq};
    double s[9];
    if (grid_sumf<9>(in, reinterpret_cast<float *>(a.part), &a.ctrl->counter[1], a.nblk, s) && threadIdx.x == 0) {
        Ctrl *c = a.ctrl;
        c->rz_old = c->rz;
        c->rz = s[0];
        // the search direction carries over a refinement (the true residual
        // replaces the recurrence one, the Krylov recurrence goes on, as in
        // CG with reliable updates); it restarts only at the solve's start
        // and after a breakdown (alpha = 0 there, so beta = 0)
        const bool first = c->cg_iters == 0;   // q_old = 0
        const double be = first ? 0.0 : -c->alpha * s[1] / c->rz_old;
        c->beta = be;
        const double pq = first ? s[2] : s[2] + 2.0 * be * s[1] + be * be * c->pq;
        c->pq = pq;
        const double al = pq > 0.0 ? c->rz / pq : 0.0;
        c->alpha = al;
        const double rqn = s[4] + be * s[5], qqn = s[6] + 2.0 * be * s[7] + be * be * s[8];
        const double out = fmax(s[3] - 2.0 * al * rqn + al * al * qqn, 0.0);
        // the learned correction stalls the iteration: plain MG-PCG for the rest of the solve
        // an iteration with the network whose residual falls by less than 4x
        // stalls (plain MG-PCG takes about 10x per iteration on these
        // systems); after 3 stalls the solve goes on with plain MG-PCG
        if (a.lpc && c->inner_it > 0 && out > 0.0625 * c->rr_prev && ++c->lpc_stalls >= 3) c->lpc_off = 1;
        c->rr_prev = out;
        c->cg_iters += 1;
        c->inner_it += 1;
        c->rnorm2 = out;   // inner recurrence residual (diagnostic)
        // this cycle's target: inner_tol, or just enough to reach rtol overall
        const double need = 0.3 * a.rtol / fmax(c->relres, 1e-300);
        const double tgt2 = fmax(a.inner_tol2, need * need);
        if (!(pq > 0.0) || out <= tgt2 * c->r0in2 || c->inner_it >= a.inner_max || c->cg_iters >= a.maxit ||
            isnan(s[3] + s[6]))
            c->refine = 1;
    }
}

// p = z + beta p ; q = w + beta q ; x += alpha p in float-float ; r32 -= alpha q.
// x is accumulated beyond FP32: an FP32 correction would carry a rounding of
// ~eps |d| that M amplifies by its condition number (~5e-4 relative residual
// at 1024^2), the floor no inner iteration can get below.
__global__ void __launch_bounds__(256) k_cgm_upd(const CgmArgs a) {
    if (a.ctrl->cg_done || a.ctrl->cg_fail) return;
    const float be = (float)a.ctrl->beta;
    const FF alf = ff_from(a.ctrl->alpha);
    const float al = alf.h;
    CG_VEC4(a, {
        const float4 z = ld4(a.z, o), w = ld4(a.w, o), p0 = ld4(a.p, o), q0 = ld4(a.q, o);
        const float4 p = make_float4(z.x + be * p0.x, z.y + be * p0.y, z.z + be * p0.z, z.w + be * p0.w);
        const float4 q = make_float4(w.x + be * q0.x, w.y + be * q0.y, w.z + be * q0.z, w.w + be * q0.w);
        st4(a.p, o, p);
        st4(a.q, o, q);
        float4 xh = ld4(a.xh, o), xl = ld4(a.xl, o);
        FF t;
        t = ff_sum({xh.x, xl.x}, ff_mulf(alf, p.x)); xh.x = t.h; xl.x = t.l;
        t = ff_sum({xh.y, xl.y}, ff_mulf(alf, p.y)); xh.y = t.h; xl.y = t.l;
        t = ff_sum({xh.z, xl.z}, ff_mulf(alf, p.z)); xh.z = t.h; xl.z = t.l;
        t = ff_sum({xh.w, xl.w}, ff_mulf(alf, p.w)); xh.w = t.h; xl.w = t.l;
        st4(a.xh, o, xh);
        st4(a.xl, o, xl);
        float4 r = ld4(a.r32, o);
        r.x -= al * q.x; r.y -= al * q.y; r.z -= al * q.z; r.w -= al * q.w;
        st4(a.r32, o, r);
    })
}

// refinement: r = D b - M x in float-float (each face term c (x_i - x_j) and
// the sum carried to ~48 bits: the terms are up to ~1e3 times larger than
// their sum, which must be right to well below lapl_rtol), r32 = r rounded;
// convergence on |D^-1 r| / |D^-1 D b|.  The norms are FP32 sums of values
// scaled by sc, a power of two near 1 / |D^-1 D b| (so that the summands stay
// far inside the FP32 range for relative residuals from 1e3 down to 1e-15).
__global__ void __launch_bounds__(256) k_cgm_refine(const CgmArgs a) {
    if (!a.ctrl->refine || a.ctrl->cg_done || a.ctrl->cg_fail) return;
    const double bn2 = a.ctrl->bnorm2;
    // sc = 2^-floor(e/2), e the binary exponent of |b|^2: integer arithmetic only
    const int e2 = (int)((__double_as_longlong(bn2) >> 52) & 0x7ff) - 1023;
    const int esc = min(max(-(e2 >> 1), -120), 120);
    const float sc = __int_as_float((127 + esc) << 23);
    float v = 0.0f, w = 0.0f;
    CG_NODES(a, {
        const FF xc = {a.xh[o], a.xl[o]};
        auto face = [&](float c, size_t on) {   // c (x_o - x_on)
            return ff_mulf(ff_sum(xc, ff_neg({a.xh[on], a.xl[on]})), c);
        };
        FF mx = face(a.ce[o], o + 1);
        mx = ff_sum(mx, face(a.ce[o - 1], o - 1));
        mx = ff_sum(mx, face(a.cn[o], o + a.P));
        mx = ff_sum(mx, face(a.cn[o - a.P], o - a.P));
        mx = ff_sum(mx, ff_mulf(xc, a.extra[o]));
        const FF rr = ff_sum(ff_from(a.rhs[o]), ff_neg(mx));
        const float r32 = __fadd_rn(rr.h, rr.l);
        a.r32[o] = r32;
        const float u = r32 * a.dinv32[o] * sc;
        v += u * u;
        w += r32 * r32;
    })
    float in[2] = {v, w};
    double sums[2];
    if (grid_sumf<2>(in, reinterpret_cast<float *>(a.part), &a.ctrl->counter[4], a.nblk, sums) && threadIdx.x == 0) {
        Ctrl *c = a.ctrl;
        const double prev = c->relres, s2 = (double)sc * (double)sc;
        c->rnorm2 = sums[0] / s2;
        c->r0in2 = sums[1];
        c->relres = bn2 > 0.0 ? sqrt(sums[0] / (bn2 * s2)) : 0.0;
        c->inner_it = 0;
        c->refine = 0;
        c->rr_prev = sums[1];
        // the search direction is kept across the refinement unless the
        // cycle broke down (pq <= 0) or the true residual did not fall over
        // it; a cycle that fails to reduce it after a restart fails the solve
        const bool fell = c->relres < prev;
        if (c->relres <= a.rtol) c->cg_done = 1;
        else if (isnan(sums[0]) || c->cg_iters >= a.maxit || (!fell && c->cgm_restarted)) c->cg_fail = 1;
        c->cgm_restarted = !(c->pq > 0.0) || !fell;
        if (c->cgm_restarted) c->alpha = 0.0;   // restart from z (beta = 0)
        if (a.use_cond && (c->cg_done || c->cg_fail)) cudaGraphSetConditional(a.cond, 0u);
    }
}

// phi(interior) += xh + xl ; ph_mi = phi (lapl_lib.F90:112-119), after convergence
__global__ void k_phi_update_ff(double *ph, double *phm, const float *xh, const float *xl, int nx, int ny, int P,
                                const Ctrl *ctrl) {
    if (!ctrl->cg_done || ctrl->cg_fail) return;
    const unsigned n = (unsigned)(ny + 2) * (unsigned)P;   // 32-bit indices, as in k_phi_update
    for (unsigned o = blockIdx.x * blockDim.x + threadIdx.x; o < n; o += gridDim.x * blockDim.x) {
        const int gj = (int)(o / (unsigned)P), gi = (int)(o - (unsigned)gj * (unsigned)P);
        double v = ph[o];
        if (gi >= 1 && gi <= nx && gj >= 1 && gj <= ny) v = v + ((double)xh[o] + (double)xl[o]);
        ph[o] = v;
        phm[o] = v;
    }
}

// ------------------------------------------- learned correction (inference)
// The network works on the fine grid (NN cell (J, I), 0-based, is node
// (I + 1, J + 1); the NN grid is padded to multiples of 8 with zero cells).
// Inputs per cell, x0 [Hn][Wn][16] BF16 (channels 4..15 stay zero):
//   f0 = s / sigma: the residual the V-cycle leaves, s = r - M z, over the
//        current residual's RMS sigma = |r| / sqrt(nx ny);
//   f1, f2 = c_e / m_c, c_n / m_c: the shares of the east and north face
//        conductances in the diagonal -- the grid-spacing map (the
//        permittivity is eps0 everywhere in this model);
//   f3 = asinh(n_i - n_e): the net charge density.
// Output y: the correction a second V-cycle adds for s, scaled by m_c / sigma.
// The preconditioner is z = V(r) + alpha d with d = sigma y / m_c and alpha
// the step that minimises |s - alpha M d| (one more grid reduction): the
// network's correction is taken only as far as it reduces the residual the
// V-cycle left, so a poor prediction costs little.
struct LpcArgs {
    int Hn, Wn;
    float *s;                 // s = r - M V(r), fine FP32 field (kept for the step length)
    float *d;                 // the network's correction d = sigma y / m_c (fine FP32 field)
    const float *mc;          // level-0 diagonal (FP32)
    const double *ni, *ne;    // the current densities, for the charge feature
    __nv_bfloat16 *x0;        // network input
    const float *y;           // network output (channel 0)
    __nv_bfloat16 *feat;      // harvest: feature slot [Hn][Wn][LPC_NFEAT], or null
    float *tgt;               // harvest: target slot [Hn][Wn]
    int s_to_r;               // harvest: write s over r32 (the next V-cycle's input)
};

__device__ __forceinline__ float lpc_sigma(const CgmArgs &a) {
    const double n = (double)a.nx * (double)a.ny, r2 = a.ctrl->rr_prev;
    return r2 > 0.0 ? (float)sqrt(r2 / n) : 0.0f;
}

__global__ void __launch_bounds__(256) k_lpc_feat(const LpcArgs l, const CgmArgs a) {
    const float sg = lpc_sigma(a), is = sg > 0.0f ? 1.0f / sg : 0.0f;
    CG_NODES(a, {
        const int jj = (int)j_, ii = (int)(q_ - j_ * (unsigned)a.nx);
        const float s = a.r32[o] - mz_ff(a.z[o], a.z[o + 1], a.z[o - 1], a.z[o + a.P], a.z[o - a.P], a.ce[o],
                                         a.ce[o - 1], a.cn[o], a.cn[o - a.P], a.extra[o]);
        const float mc = l.mc[o], im = mc > 0.0f ? 1.0f / mc : 0.0f;
        const __nv_bfloat162 f01 = __floats2bfloat162_rn(s * is, a.ce[o] * im);
        const __nv_bfloat162 f23 = __floats2bfloat162_rn(a.cn[o] * im, asinhf((float)(l.ni[o] - l.ne[o])));
        const size_t p = (size_t)jj * l.Wn + ii;
        if (l.s) l.s[o] = s;
        uint2 v;
        v.x = *reinterpret_cast<const uint32_t *>(&f01);
        v.y = *reinterpret_cast<const uint32_t *>(&f23);
        *reinterpret_cast<uint2 *>(l.x0 + p * LPC_CIN0) = v;
        if (l.feat) *reinterpret_cast<uint2 *>(l.feat + p * LPC_NFEAT) = v;
        if (l.s_to_r) a.r32[o] = s;
    })
}

// d = sigma y / m_c; the step alpha = (s . M d) / (M d . M d) into the control
// block (0 for a non-finite correction, which also switches the network off)
__global__ void __launch_bounds__(256) k_lpc_step(const LpcArgs l, const CgmArgs a) {
    Ctrl *c = a.ctrl;
    if (c->lpc_off || c->cg_done || c->cg_fail) return;
    const float sg = lpc_sigma(a);
    float v[2] = {0.0f, 0.0f};
    // M d needs the neighbours' d, recomputed from y (no grid-wide barrier);
    // a non-finite prediction contributes nothing
    CG_NODES(a, {
        auto dn = [&](size_t on, unsigned jj, unsigned ii) {
            const float mc = l.mc[on];
            const float dv = mc > 0.0f ? sg * l.y[(size_t)jj * l.Wn + ii] / mc : 0.0f;
            return isfinite(dv) ? dv : 0.0f;
        };
        const unsigned jj = j_, ii = q_ - j_ * (unsigned)a.nx;
        const float d0 = dn(o, jj, ii);
        const float de = ii + 1 < (unsigned)a.nx ? dn(o + 1, jj, ii + 1) : 0.0f;
        const float dw = ii > 0 ? dn(o - 1, jj, ii - 1) : 0.0f;
        const float dnn = jj + 1 < (unsigned)a.ny ? dn(o + a.P, jj + 1, ii) : 0.0f;
        const float ds = jj > 0 ? dn(o - a.P, jj - 1, ii) : 0.0f;
        l.d[o] = d0;
        const float md = mz_ff(d0, de, dw, dnn, ds, a.ce[o], a.ce[o - 1], a.cn[o], a.cn[o - a.P], a.extra[o]);
        v[0] += l.s[o] * md;
        v[1] += md * md;
    })
    double sums[2];
    if (grid_sumf<2>(v, reinterpret_cast<float *>(a.part), &a.ctrl->counter[6], a.nblk, sums) && threadIdx.x == 0) {
        const double al = sums[1] > 0.0 ? sums[0] / sums[1] : 0.0;
        c->spare[0] = isfinite(al) ? al : 0.0;
        if (!isfinite(al)) c->lpc_off = 1;
    }
}

// z += alpha d, unless the correction is switched off for this solve
__global__ void __launch_bounds__(256) k_lpc_add(const LpcArgs l, const CgmArgs a) {
    Ctrl *c = a.ctrl;
    if (c->lpc_off || c->cg_done || c->cg_fail) return;
    const float al = (float)c->spare[0];
    CG_NODES(a, { a.z[o] += al * l.d[o]; })
}

// harvest: rr_prev = |r32|^2 (the feature scale of the residual in r32)
__global__ void __launch_bounds__(256) k_lpc_norm(const CgmArgs a) {
    double v = 0.0;
    CG_NODES(a, { v += (double)a.r32[o] * (double)a.r32[o]; })
    double out;
    if (grid_sum<256>(v, a.part, &a.ctrl->counter[5], a.nblk, &out) && threadIdx.x == 0) a.ctrl->rr_prev = out;
}

// harvest target: the second V-cycle's correction z = V(s), times m_c / sigma
__global__ void __launch_bounds__(256) k_lpc_target(const LpcArgs l, const CgmArgs a) {
    const float sg = lpc_sigma(a), is = sg > 0.0f ? 1.0f / sg : 0.0f;
    CG_NODES(a, {
        const size_t p = (size_t)j_ * l.Wn + (q_ - j_ * (unsigned)a.nx);
        l.tgt[p] = a.z[o] * l.mc[o] * is;
    })
}

}  // namespace

// ------------------------------------------------------------------ host side
static void destroy_cgm_graphs(fs_ctx *c) {
    for (int v = 0; v < 2; v++)
        if (c->cgm_graph_built[v]) {
            cudaGraphExecDestroy(c->cgm_exec[v]);
            cudaGraphDestroy(c->cgm_graph[v]);
            c->cgm_graph_built[v] = 0;
        }
}

// after a change of the V-cycle's smoother: the graphs are rebuilt at the next
// solve, and the shared memory limits of this translation unit's instances
// of the level kernels follow the context's strips and smoother
int fs_lapl_mixed_reconfigure(fs_ctx *c) {
    destroy_cgm_graphs(c);
    cudaError_t e = mg_level_smem_limits<float>(c);
    return e == cudaSuccess ? FS_OK : fs_cuda_check(c, e, "multigrid shared memory");
}

int fs_lapl_alloc_mixed(fs_ctx *c) {
    for (int l = 0; l < c->mg_nlev; l++) {
        MGLevelF &m = c->mgf[l];
        m.nx = c->mg[l].nx;
        m.ny = c->mg[l].ny;
        m.pitch = c->mg[l].pitch;
        const size_t n = (size_t)(m.ny + 2) * m.pitch;
        float **fields[] = {&m.mc, &m.ce, &m.cn, &m.extra, &m.inv_mc, &m.rhs, &m.x, &m.xd};
        for (float **f : fields) {
            cudaError_t e = cudaMalloc(f, n * sizeof(float));
            if (e == cudaSuccess) e = cudaMemset(*f, 0, n * sizeof(float));
            if (e != cudaSuccess) return fs_cuda_check(c, e, "cudaMalloc (FP32 multigrid)");
        }
        m.res = nullptr;
    }
    float **vecs[] = {&c->p32, &c->q32, &c->w32, &c->xh32, &c->xl32, &c->dinv32};
    for (float **v : vecs) {
        cudaError_t e = cudaMalloc(v, c->field_elems * sizeof(float));
        if (e == cudaSuccess) e = cudaMemset(*v, 0, c->field_elems * sizeof(float));
        if (e != cudaSuccess) return fs_cuda_check(c, e, "cudaMalloc (FP32 CG vectors)");
    }
    {   // nine partials per CTA of the CG reductions (<= 4 CTAs per SM)
        const int need = 9 * 4 * c->nsm;
        if (c->cg_nblk < need) {
            cudaFree(c->d_cg_part);
            cudaError_t e = cudaMalloc(&c->d_cg_part, sizeof(double) * need);
            if (e != cudaSuccess) return fs_cuda_check(c, e, "cudaMalloc (CG partials)");
            c->cg_nblk = need;
        }
    }
    cudaFuncSetAttribute(k_mg_down<float, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mg_down_smem<float>(2));
    cudaFuncSetAttribute(k_mg_up<float, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mg_up_smem<float>(2));
    {   // this translation unit's strip and x-line kernels (the strips and the
        // smoother were chosen with the FP64 hierarchy)
        cudaError_t e = mg_level_smem_limits<float>(c);
        if (e != cudaSuccess) return fs_cuda_check(c, e, "multigrid shared memory");
    }
    {
        BottomArgs<float> ba;
        ba.nl = c->mg_nlev;
        ba.lb = 0;
        while (ba.lb < ba.nl && (c->mgf[ba.lb].nx > BOTTOM_N || c->mgf[ba.lb].ny > BOTTOM_N)) ba.lb++;
        for (int l = 0; l < ba.nl; l++) { ba.L[l].nx = c->mgf[l].nx; ba.L[l].ny = c->mgf[l].ny; }
        ba.dl = bottom_dense_level(ba);
        cudaError_t e = fs_smem_limit((const void *)k_bottom_smem<float>, bottom_smem_bytes(ba));
        if (e != cudaSuccess) return fs_cuda_check(c, e, "bottom solver shared memory");
        if ((e = cudaMalloc(&c->d_ainv32, 64 * 64 * sizeof(float))) != cudaSuccess)
            return fs_cuda_check(c, e, "cudaMalloc (dense inverse)");
    }
    c->launches++;
    k_dinv<<<grid2(c->nx, c->ny, dim3(32, 8)), dim3(32, 8), 0, c->stream>>>(c->mesh, c->nx, c->ny, c->pitch,
                                                                           c->cfg.cyl, c->dinv, c->dinv32);
    return fs_cuda_check(c, cudaGetLastError(), "row scaling");
}

void fs_lapl_free_mixed(fs_ctx *c) {
    destroy_cgm_graphs(c);
    for (int l = 0; l < FS_MG_MAX_LEVELS; l++) {
        MGLevelF &m = c->mgf[l];
        float *fs[] = {m.mc, m.ce, m.cn, m.extra, m.inv_mc, m.rhs, m.x, m.xd};
        for (float *f : fs) cudaFree(f);
        memset(&m, 0, sizeof(m));
    }
    cudaFree(c->p32);
    cudaFree(c->q32);
    cudaFree(c->w32);
    cudaFree(c->xh32);
    cudaFree(c->xl32);
    cudaFree(c->dinv32);
    cudaFree(c->d_ainv32);
}

// FP32 V-cycle on the correction equation: mgf[0].rhs holds the FP64
// residual rounded to FP32, mgf[0].x receives z.
static void vcycle_mixed(fs_ctx *c, const CgmArgs &ca) {
    const int nl = c->mg_nlev, nu = c->cfg.mg_smooth;
    const bool fused = nu == 2;
    int lb = 0;
    while (lb < nl && (c->mgf[lb].nx > BOTTOM_N || c->mgf[lb].ny > BOTTOM_N)) lb++;
    dim3 b(32, 8);
    for (int l = 0; l < lb; l++) {
        LevelT<float> f = level_f(c->mgf[l]), cc = level_f(c->mgf[l + 1]);
        if (l == 0 && c->mg_xline) {   // x-line pre-smoothing, the odd rows' residual restricted
            xline_pairs<float>(c, f, fs_mg_pre0(nu), true, 1.0f);
            fs_prof_begin(c, PROF_TRANSFER);
            k_restrict_odd<float><<<grid2(cc.nx, cc.ny, b), b, 0, c->stream>>>(f, cc);
            fs_prof_end(c);
            continue;
        }
        if (fused) {
            fs_prof_begin(c, PROF_SMOOTH);
            k_mg_down<float, 2><<<grid2(f.nx, f.ny, dim3(MTX, MTY)), 256, mg_down_smem<float>(2), c->stream>>>(
                lvt_f(c->mgf[l]), lvt_f(c->mgf[l + 1]));
            fs_prof_end(c);
            continue;
        }
        dim3 g = grid2((f.nx + 1) / 2, f.ny, b);
        for (int it = 0; it < nu; it++) {
            fs_prof_begin(c, PROF_SMOOTH);
            k_rb<float><<<g, b, 0, c->stream>>>(f, 0, it == 0);
            fs_prof_end(c);
            fs_prof_begin(c, PROF_SMOOTH);
            k_rb<float><<<g, b, 0, c->stream>>>(f, 1, 0);
            fs_prof_end(c);
        }
        fs_prof_begin(c, PROF_TRANSFER);
        k_restrict<float><<<grid2(cc.nx, cc.ny, b), b, 0, c->stream>>>(f, cc);
        fs_prof_end(c);
    }
    BottomArgs<float> ba;
    for (int l = 0; l < nl; l++) ba.L[l] = level_f(c->mgf[l]);
    ba.lb = lb;
    ba.nl = nl;
    ba.nu = nu;
    ba.dl = c->mg_dl;
    ba.ainv = c->d_ainv32;
    ba.om = (float)FS_MG_OMEGA_POST;
    fs_prof_begin(c, PROF_BOTTOM);
    k_bottom_smem<float><<<1, BOTTOM_THREADS, bottom_smem_bytes(ba), c->stream>>>(ba);
    fs_prof_end(c);
    // the finest level's last post-smoothing launch fills the strip snapshot
    const bool strips = lb > 0 && has_strips(c) && !c->mg_xline;
    const StripSnap<float> sn = strips ? strip_snap(c, c->strip_snap32) : StripSnap<float>{};
    for (int l = lb - 1; l >= 0; l--) {
        LevelT<float> f = level_f(c->mgf[l]), cc = level_f(c->mgf[l + 1]);
        if (l == 0 && c->mg_xline) {   // x-line post-smoothing
            fs_prof_begin(c, PROF_TRANSFER);
            k_prolong<float><<<grid2(f.nx, f.ny, b), b, 0, c->stream>>>(f, cc);
            fs_prof_end(c);
            xline_pairs<float>(c, f, nu, false, (float)FS_XL_OMEGA_POST);
            continue;
        }
        if (fused) {
            LvT<float> F = lvt_f(c->mgf[l]);
            if (l == 0) F.sn = sn;
            fs_prof_begin(c, PROF_SMOOTH);
            const dim3 g = grid2(f.nx, f.ny, dim3(MTX, MTY));
            k_mg_up<float, 2><<<g, 256, mg_up_smem<float>(2), c->stream>>>(F, lvt_f(c->mgf[l + 1]));
            fs_prof_end(c);
            continue;
        }
        dim3 g = grid2(f.nx, f.ny, b), gh = grid2((f.nx + 1) / 2, f.ny, b);
        fs_prof_begin(c, PROF_TRANSFER);
        k_prolong<float><<<g, b, 0, c->stream>>>(f, cc);
        fs_prof_end(c);
        for (int it = 0; it < nu; it++) {
            fs_prof_begin(c, PROF_SMOOTH);
            k_rb<float><<<gh, b, 0, c->stream>>>(f, 1, 0, (float)FS_MG_OMEGA_POST);
            fs_prof_end(c);
            fs_prof_begin(c, PROF_SMOOTH);
            k_rb<float><<<gh, b, 0, c->stream>>>(f, 0, 0, (float)FS_MG_OMEGA_POST,
                                                  l == 0 && it == nu - 1 ? sn : StripSnap<float>{});
            fs_prof_end(c);
        }
    }
    if (strips) {   // black-red pairs after the red half sweep
        fs_prof_begin(c, PROF_SMOOTH);
        k_rb_strips<float><<<dim3((c->ny + STRIP_ROWS - 1) / STRIP_ROWS, 2), 256, strip_smem<float>(c->strip_w),
                             c->stream>>>(level_f(c->mgf[0]), sn, 1, (float)FS_MG_OMEGA_POST);
        fs_prof_end(c);
    }
}

static LpcArgs lpc_args(fs_ctx *c) {
    LpcArgs l = {};
    l.Hn = c->lpc->Hn; l.Wn = c->lpc->Wn;
    l.mc = c->mgf[0].mc;
    l.ni = c->sp[0].buf[c->lev[0]];
    l.ne = c->sp[1].buf[c->lev[0]];
    l.x0 = c->lpc->x0; l.y = c->lpc->y;
    return l;
}

// z += the network's correction for the residual the V-cycle leaves
static void lpc_apply(fs_ctx *c, const CgmArgs &ca) {
    LpcArgs l = lpc_args(c);
    fs_prof_begin(c, PROF_OTHER);
    l.s = c->lpc_s32;
    l.d = c->lpc_d32;
    k_lpc_feat<<<ca.grid, 256, 0, c->stream>>>(l, ca);
    lpc_forward(c->lpc, 1, c->lpc->Hn, c->lpc->Wn, c->stream);
    k_lpc_step<<<ca.grid, 256, 0, c->stream>>>(l, ca);
    k_lpc_add<<<ca.grid, 256, 0, c->stream>>>(l, ca);
    // one black-red Gauss-Seidel pass on the fine level removes the
    // cell-scale error the network's correction brings in (M amplifies it
    // most), as post-smoothing does after a coarse-grid correction
    LevelT<float> f0 = level_f(c->mgf[0]);
    dim3 b(32, 8), gh = grid2((f0.nx + 1) / 2, f0.ny, b);
    k_rb<float><<<gh, b, 0, c->stream>>>(f0, 1, 0);
    k_rb<float><<<gh, b, 0, c->stream>>>(f0, 0, 0);
    fs_prof_end(c);
    // features, step, correction, 12 convolutions, 3 pools, 3 upsamplings, 2 half sweeps
    c->launches += 3 + LPC_NLAYER + 6 + 2 - 1;
}

static void cg_iteration_mixed(fs_ctx *c, const CgmArgs &ca) {
    vcycle_mixed(c, ca);
    if (ca.lpc) lpc_apply(c, ca);
    fs_prof_begin(c, PROF_CG);
    k_cgm_rzw<<<ca.grid, 256, 0, c->stream>>>(ca);
    fs_prof_end(c);
    fs_prof_begin(c, PROF_CG);
    k_cgm_upd<<<ca.grid, 256, 0, c->stream>>>(ca);
    fs_prof_end(c);
    fs_prof_begin(c, PROF_CG);
    k_cgm_refine<<<ca.grid, 256, 0, c->stream>>>(ca);
    fs_prof_end(c);
}

// WHILE(cond) { one iteration } -> phi update, as one graph (see fs_lapl.cu)
static int build_cgm_graph(fs_ctx *c, CgmArgs ca) {
    std::lock_guard<std::mutex> lock(fs_graph_mutex());
    cudaGraph_t g = nullptr;
    cudaGraphConditionalHandle h;
    cudaError_t e = cudaGraphCreate(&g, 0);
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h, g, 1u, cudaGraphCondAssignDefault);
    if (e != cudaSuccess) return fs_cuda_check(c, e, "CG graph create");
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t wnode;
    e = cudaGraphAddNode(&wnode, g, nullptr, nullptr, 0, &cp);
    if (e != cudaSuccess) { cudaGraphDestroy(g); return fs_cuda_check(c, e, "CG while node"); }
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    ca.use_cond = 1;
    ca.cond = h;
    const int prof = c->prof_on;
    c->prof_on = 0;
    const int64_t l0 = c->launches;
    e = cudaStreamBeginCaptureToGraph(c->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cg_iteration_mixed(c, ca);
        e = cudaStreamEndCapture(c->stream, &body);
    }
    const int v = ca.lpc ? 1 : 0;
    c->cgm_body_kernels[v] = (int)(c->launches - l0);
    if (e == cudaSuccess)
        e = cudaStreamBeginCaptureToGraph(c->stream, g, &wnode, nullptr, 1, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        k_phi_update_ff<<<4 * c->nsm, 256, 0, c->stream>>>(c->ph, c->ph_mi, c->xh32, c->xl32, c->nx, c->ny, c->pitch,
                                                         c->d_ctrl);
        e = cudaStreamEndCapture(c->stream, &g);
    }
    c->launches = l0;
    c->prof_on = prof;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&c->cgm_exec[v], g, 0);
    if (e != cudaSuccess) {
        // A capture that failed (a launch inside it was refused) leaves the
        // graph holding a conditional body the driver has invalidated, and
        // destroying it then crashed the process: the graph is leaked on
        // this error path, which ends the solve with the error anyway.
        return fs_cuda_check(c, e, "CG graph capture");
    }
    c->cgm_graph[v] = g;
    c->cgm_graph_built[v] = 1;
    return FS_OK;
}

// Solve-level choice with the plain multigrid-PCG as the judge: the host keeps
// moving averages of the wall time of solves with and without the network
// (a solve in which the network stalled counts double) and runs the next
// solve with the faster one.  Every lpc_probe_every solves it tries the other
// once: 25 to start with and after a probe that changed the choice, doubled
// (up to 400) after each probe that did not.
static void lpc_account(fs_ctx *c, const CgmArgs &ca, double ms) {
    if (!c->lpc_on) return;
    c->lpc_solves++;
    if (ca.lpc) c->lpc_nn_solves++;
    const double a = 0.3;
    if (ca.lpc) {
        const double t = c->h_ctrl->lpc_off ? 2.0 * ms : ms;
        c->lpc_t_nn = c->lpc_t_nn < 0.0 ? t : (1.0 - a) * c->lpc_t_nn + a * t;
    } else {
        c->lpc_t_plain = c->lpc_t_plain < 0.0 ? ms : (1.0 - a) * c->lpc_t_plain + a * ms;
    }
    int pref;
    if (c->lpc_t_nn < 0.0) pref = 1;
    else if (c->lpc_t_plain < 0.0) pref = 0;
    else pref = c->lpc_t_nn <= c->lpc_t_plain ? 1 : 0;
    // a network solve more than twice as slow as a plain one: probe rarely
    if (c->lpc_t_nn > 0.0 && c->lpc_t_plain > 0.0 && c->lpc_t_nn > 2.0 * c->lpc_t_plain) c->lpc_probe_every = 400;
    if (c->lpc_probe_pending) {
        c->lpc_probe_pending = 0;
        if (pref == (ca.lpc ? 1 : 0)) c->lpc_probe_every = 25;
        else c->lpc_probe_every = std::min(2 * c->lpc_probe_every, 400);
    }
    int next = pref;
    if (++c->lpc_since_probe >= c->lpc_probe_every) {
        next = !pref;
        c->lpc_since_probe = 0;
        c->lpc_probe_pending = 1;
    }
    c->lpc_use_next = next;
}

static CgmArgs cgm_args(fs_ctx *c) {
    MGLevelF &m0 = c->mgf[0];
    CgmArgs ca;
    ca.nx = c->nx; ca.ny = c->ny; ca.P = c->pitch;
    {
        long nb = ((long)c->nx * c->ny + 255) / 256, cap = 4L * c->nsm;
        ca.nblk = (int)(nb < cap ? nb : cap);
        ca.grid = dim3(ca.nblk);
    }
    ca.xh = c->xh32; ca.xl = c->xl32; ca.dinv32 = c->dinv32;
    ca.rhs = c->bs; ca.dinv = c->dinv; ca.part = c->d_cg_part;
    ca.z = m0.x; ca.r32 = m0.rhs; ca.p = c->p32; ca.q = c->q32; ca.w = c->w32;
    ca.ce = m0.ce; ca.cn = m0.cn; ca.extra = m0.extra;
    ca.ctrl = c->d_ctrl;
    ca.rtol = c->cfg.lapl_rtol;
    // the inner loop hands over to the refinement once its FP32 recurrence
    // residual has fallen 1e4-fold: below ~1e-5 the recurrence no longer
    // follows the true residual (measured at 1024^2: a 1e-5 target left a
    // true relative residual of 5e-5 and cost a ninth iteration per solve;
    // with 1e-4 and the search direction kept across the refinement, 8)
    ca.inner_tol2 = 1e-4 * 1e-4;
    ca.inner_max = 16;
    ca.maxit = c->cfg.lapl_maxit;
    ca.lpc = c->lpc && (c->lpc_on == 2 || (c->lpc_on == 1 && c->lpc_use_next));
    ca.use_cond = 0;
    ca.cond = 0;
    return ca;
}

int fs_lapl_solve_mixed(fs_ctx *c, int *lerr, int *iters, double *relres) {
    const auto t_start = std::chrono::steady_clock::now();
    auto elapsed_ms = [&]() {
        return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
    };
    fs_faces_update_mixed(c);
    AsmMixArgs a;
    a.pp = c->pp;
    a.f = c->pf;
    a.m = c->mesh;
    a.mf = c->meshf;
    a.tab = c->d_tab32;
    a.ni = c->sp[0].buf[c->lev[0]];
    a.ne = c->sp[1].buf[c->lev[0]];
    a.nt = c->sp[2].buf[c->lev[0]];
    a.ph = c->ph;
    a.phm = c->ph_mi;
    a.fx_e = c->fx_e;
    a.fy_e = c->fy_e;
    for (int k = 0; k < 10; k++) a.f32[k] = c->f32[k];
    a.ctrl = c->d_ctrl;
    a.ctrl_w = c->d_ctrl;
    a.tab64 = c->d_tab;
    a.sig = fs_sig(c, 0);
    MGLevelF &m0 = c->mgf[0];
    a.mc = m0.mc; a.ce = m0.ce; a.cn = m0.cn; a.extra = m0.extra; a.inv_mc = m0.inv_mc;
    a.rhs = c->bs;
    cudaMemsetAsync(&c->d_ctrl->status, 0, sizeof(unsigned int), c->stream);
    fs_prof_begin(c, PROF_ASSEMBLE);
    k_assemble_mix<<<grid2(c->nx, c->ny, dim3(ABX, ABY)), ANT, 0, c->stream>>>(a);
    fs_prof_end(c);
    {   // coarse operators: one launch per large level, then one CTA for the
        // small levels and the dense inverse
        CoarsenTail<float> ct;
        for (int l = 0; l < c->mg_nlev; l++) ct.L[l] = level_f(c->mgf[l]);
        ct.nl = c->mg_nlev;
        ct.l0 = coarsen_tail_level(ct.L, ct.nl);
        ct.dl = c->mg_dl;
        ct.ainv = c->d_ainv32;
        dim3 b2(16, 16);
        for (int l = 1; l < ct.l0; l++) {
            fs_prof_begin(c, PROF_COARSEN);
            k_coarsen<float><<<grid2(ct.L[l].nx, ct.L[l].ny, b2), b2, 0, c->stream>>>(ct.L[l - 1], ct.L[l]);
            fs_prof_end(c);
        }
        fs_prof_begin(c, PROF_COARSEN);
        k_coarsen_tail<float><<<1, 1024, 0, c->stream>>>(ct);
        fs_prof_end(c);
    }
    CgmArgs ca = cgm_args(c);
    // warm start: scale the previous correction, then the refinement forms
    // the initial residual
    fs_prof_begin(c, PROF_CG);
    k_cgm_init_warm<<<ca.grid, 256, 0, c->stream>>>(ca);
    fs_prof_end(c);
    fs_prof_begin(c, PROF_CG);
    k_cgm_init_apply<<<ca.grid, 256, 0, c->stream>>>(ca);
    fs_prof_end(c);
    fs_prof_begin(c, PROF_CG);
    k_cgm_refine<<<ca.grid, 256, 0, c->stream>>>(ca);
    fs_prof_end(c);
    int rc = fs_sync_ctrl(c);
    if (rc) return rc;
    if (c->h_ctrl->status & FS_ST_NEG_DENSITY) return fs_set_error(c, FS_ERR_NEG_DENSITY, "negative density in get_Te");
    if (c->h_ctrl->status & FS_ST_DFDPH_NAN) return fs_set_error(c, FS_ERR_NAN, "NaN in dFdPh");
    if (c->h_ctrl->status & FS_ST_BNAN) {
        *lerr = 1; *iters = 0; *relres = NAN;
        return FS_OK;
    }
    bool ok = c->h_ctrl->cg_done != 0;
    static const bool no_graph = getenv("FS_NO_GRAPH") != nullptr;
    const int poisson_classes = (1 << PROF_SMOOTH) | (1 << PROF_TRANSFER) | (1 << PROF_BOTTOM) | (1 << PROF_CG);
    if (!ok && !no_graph && !(c->prof_on & poisson_classes)) {
        const int v = ca.lpc ? 1 : 0;
        if (!c->cgm_graph_built[v] && (rc = build_cgm_graph(c, ca))) return rc;
        cudaError_t e = cudaGraphLaunch(c->cgm_exec[v], c->stream);
        if (e != cudaSuccess) return fs_cuda_check(c, e, "CG graph launch");
        rc = fs_sync_ctrl(c);
        if (rc) return rc;
        c->launches += (int64_t)c->h_ctrl->cg_iters * c->cgm_body_kernels[v] + 1;
        lpc_account(c, ca, elapsed_ms());
        *iters = c->h_ctrl->cg_iters;
        *relres = c->h_ctrl->relres;
        bool conv = c->h_ctrl->cg_done && !c->h_ctrl->cg_fail;
        *lerr = conv ? 0 : 1;
        if (conv) c->faces_valid = 0;
        return FS_OK;
    }
    int it = 0;
    static const bool trace = getenv("FS_TRACE_CG") != nullptr;
    while (!ok && it < c->cfg.lapl_maxit) {
        cg_iteration_mixed(c, ca);
        rc = fs_sync_ctrl(c);
        if (rc) return rc;
        it = c->h_ctrl->cg_iters;
        if (trace)
            fprintf(stderr, "cgm %d inner %d relres %.3e inner_r2 %.3e r0in2 %.3e pq %.3e alpha %.3e beta %.3e\n",
                    it, c->h_ctrl->inner_it, c->h_ctrl->relres, c->h_ctrl->rnorm2, c->h_ctrl->r0in2, c->h_ctrl->pq,
                    c->h_ctrl->alpha, c->h_ctrl->beta);
        if (c->h_ctrl->cg_fail) break;
        ok = c->h_ctrl->cg_done != 0;
    }
    lpc_account(c, ca, elapsed_ms());
    *iters = c->h_ctrl->cg_iters;
    *relres = c->h_ctrl->relres;
    if (!ok) {
        *lerr = 1;
        return FS_OK;
    }
    *lerr = 0;
    c->faces_valid = 0;
    c->launches++;
    k_phi_update_ff<<<4 * c->nsm, 256, 0, c->stream>>>(c->ph, c->ph_mi, c->xh32, c->xl32, c->nx, c->ny, c->pitch,
                                                         c->d_ctrl);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fs_cuda_check(c, e, "Poisson kernels (mixed)");
    return FS_OK;
}

// ---------------------------------------------------- learned preconditioner
static int round8(int v) { return (v + 7) / 8 * 8; }

// crop: edge of the training crops in cells (a multiple of 8; 0: 128), at most the grid's
int fs_lpc_init_impl(fs_ctx *c, int crop, int max_batch, int max_samples, uint64_t seed) {
    if (!c->mixed) return fs_set_error(c, FS_ERR_UNSUPPORTED, "the learned preconditioner needs the mixed solver");
    if (max_batch < 1 || max_samples < 1) return fs_set_error(c, FS_ERR_INVALID, "batch and sample counts must be positive");
    if (crop < 0 || crop % 8) return fs_set_error(c, FS_ERR_INVALID, "crop %d is not a multiple of 8", crop);
    fs_lpc_free_impl(c);
    const int Hn = round8(c->ny), Wn = round8(c->nx);
    const int cr = crop ? crop : 128, Hc = std::min(cr, Hn), Wc = std::min(cr, Wn);
    LpcState *L = nullptr;
    int e = lpc_alloc(&L, Hn, Wn, Hc, Wc, max_batch, max_samples, seed, c->stream);
    if (e == (int)cudaErrorNotSupported)
        return fs_set_error(c, FS_ERR_UNSUPPORTED, "tensor-core convolutions unavailable (no TMA descriptor encoder)");
    if (e) return fs_cuda_check(c, (cudaError_t)e, "learned preconditioner buffers");
    c->lpc = L;
    c->lpc_snap_max = 8;
    cudaError_t ce = cudaMalloc(&c->lpc_snap, (size_t)c->lpc_snap_max * c->field_elems * sizeof(float));
    if (ce == cudaSuccess) ce = cudaMalloc(&c->lpc_s32, c->field_elems * sizeof(float));
    if (ce == cudaSuccess) ce = cudaMemset(c->lpc_s32, 0, c->field_elems * sizeof(float));
    if (ce == cudaSuccess) ce = cudaMalloc(&c->lpc_d32, c->field_elems * sizeof(float));
    if (ce == cudaSuccess) ce = cudaMemset(c->lpc_d32, 0, c->field_elems * sizeof(float));
    if (ce != cudaSuccess) { fs_lpc_free_impl(c); return fs_cuda_check(c, ce, "learned preconditioner buffers"); }
    // interior cells of the padded NN grid
    std::vector<float> mk((size_t)Hn * Wn, 0.0f);
    for (int j = 0; j < c->ny; j++)
        for (int i = 0; i < c->nx; i++) mk[(size_t)j * Wn + i] = 1.0f;
    ce = cudaMemcpyAsync(L->mask, mk.data(), mk.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(c->stream);
    return fs_cuda_check(c, ce, "learned preconditioner init");
}

void fs_lpc_free_impl(fs_ctx *c) {
    destroy_cgm_graphs(c);   // a graph may hold the network's kernels
    lpc_free(c->lpc);
    c->lpc = nullptr;
    c->lpc_on = 0;
    cudaFree(c->lpc_snap);
    cudaFree(c->lpc_s32);
    cudaFree(c->lpc_d32);
    c->lpc_snap = nullptr;
    c->lpc_s32 = c->lpc_d32 = nullptr;
}

// Host-driven solve of the current (assembled) system with the plain mixed
// MG-PCG to lapl_rtol; returns the iterations, or a negative error.
static int solve_plain(fs_ctx *c, CgmArgs ca, std::vector<int> *snap_iters) {
    ca.lpc = 0;
    k_cgm_init<<<ca.grid, 256, 0, c->stream>>>(ca);
    int rc = fs_sync_ctrl(c);
    if (rc) return rc;
    int taken = 0;
    for (int it = 0; !c->h_ctrl->cg_done && !c->h_ctrl->cg_fail && it < c->cfg.lapl_maxit; it++) {
        if (snap_iters && taken < c->lpc_snap_max && it % 2 == 0) {   // the residual the preconditioner sees
            cudaMemcpyAsync(c->lpc_snap + (size_t)taken * c->field_elems, ca.r32, c->field_elems * sizeof(float),
                            cudaMemcpyDeviceToDevice, c->stream);
            snap_iters->push_back(it);
            taken++;
        }
        cg_iteration_mixed(c, ca);
        if ((rc = fs_sync_ctrl(c))) return rc;
        static const bool trace = getenv("FS_TRACE_CG") != nullptr;
        if (trace)
            fprintf(stderr, "harvest cg %d inner %d relres %.3e inner_r2 %.3e r0in2 %.3e pq %.3e fail %d\n",
                    c->h_ctrl->cg_iters, c->h_ctrl->inner_it, c->h_ctrl->relres, c->h_ctrl->rnorm2,
                    c->h_ctrl->r0in2, c->h_ctrl->pq, c->h_ctrl->cg_fail);
    }
    if (!c->h_ctrl->cg_done)
        return fs_set_error(c, FS_ERR_INVALID, "harvest solve did not converge (relres %.3e after %d iterations)",
                            c->h_ctrl->relres, c->h_ctrl->cg_iters);
    return c->h_ctrl->cg_iters;
}

// Training pairs from the plain solver: the step's assembled system is
// re-solved with the plain multigrid-PCG, and for up to per_solve of its
// residuals r: z = V(r), s = r - M z (the residual the first V-cycle leaves,
// its features stored), then the target: the second V-cycle's correction
// V(s), scaled as the network's output.
int fs_lpc_harvest_impl(fs_ctx *c, int per_solve, int *added) {
    if (!c->lpc) return fs_set_error(c, FS_ERR_INVALID, "learned preconditioner not initialised");
    LpcState *L = c->lpc;
    *added = 0;
    CgmArgs ca = cgm_args(c);
    std::vector<int> its;
    int rc = solve_plain(c, ca, &its);
    if (rc < 0) return rc;
    const size_t px = (size_t)L->Hn * L->Wn;
    const int n = std::min((int)its.size(), std::min(per_solve, c->lpc_snap_max));
    for (int k = 0; k < n; k++) {
        const int slot = L->nsamp % L->Nmax;
        cudaMemcpyAsync(ca.r32, c->lpc_snap + (size_t)k * c->field_elems, c->field_elems * sizeof(float),
                        cudaMemcpyDeviceToDevice, c->stream);
        k_lpc_norm<<<ca.grid, 256, 0, c->stream>>>(ca);
        vcycle_mixed(c, ca);
        LpcArgs l = lpc_args(c);
        l.feat = L->dfeat + slot * px * LPC_NFEAT;
        l.s_to_r = 1;
        k_lpc_feat<<<ca.grid, 256, 0, c->stream>>>(l, ca);
        vcycle_mixed(c, ca);   // z = V(s)
        l.tgt = L->dtgt + slot * px;
        k_lpc_target<<<ca.grid, 256, 0, c->stream>>>(l, ca);
        L->nsamp++;
        (*added)++;
    }
    return fs_cuda_check(c, cudaStreamSynchronize(c->stream), "harvest");
}

// iters Adam steps on batches of random Hc x Wc crops (origins on the
// 8-cell pooling grid) of the stored pairs
int fs_lpc_train_impl(fs_ctx *c, int iters, int batch, float lr, uint64_t seed, float *loss_hist) {
    if (!c->lpc) return fs_set_error(c, FS_ERR_INVALID, "learned preconditioner not initialised");
    LpcState *L = c->lpc;
    const int n = std::min(L->nsamp, L->Nmax);
    if (n < 1) return fs_set_error(c, FS_ERR_INVALID, "no harvested samples");
    if (batch < 1 || batch > L->Bmax) return fs_set_error(c, FS_ERR_INVALID, "batch %d outside 1..%d", batch, L->Bmax);
    uint64_t st = seed * 0x9E3779B97F4A7C15ull + 7;
    auto draw = [&](uint64_t m) {
        st += 0x9E3779B97F4A7C15ull;
        uint64_t z = st;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return (int)((z ^ (z >> 31)) % m);
    };
    const int ny8 = (L->Hn - L->Hc) / 8 + 1, nx8 = (L->Wn - L->Wc) / 8 + 1;
    std::vector<int> idx(batch), y0(batch), x0(batch);
    float *h_loss = nullptr;
    cudaMallocHost(&h_loss, sizeof(float) * (size_t)std::max(iters, 1));
    for (int it = 0; it < iters; it++) {
        for (int b = 0; b < batch; b++) {
            idx[b] = draw((uint64_t)n);
            y0[b] = 8 * draw((uint64_t)ny8);
            x0[b] = 8 * draw((uint64_t)nx8);
        }
        lpc_gather(L, idx.data(), y0.data(), x0.data(), batch, c->stream);
        int e = lpc_forward(L, batch, L->Hc, L->Wc, c->stream);
        if (!e) e = lpc_loss_backward(L, batch, L->Hc, L->Wc, c->stream);
        if (e) { cudaFreeHost(h_loss); return fs_cuda_check(c, (cudaError_t)e, "training step"); }
        cudaMemcpyAsync(h_loss + it, L->d_loss, sizeof(float), cudaMemcpyDeviceToHost, c->stream);
        lpc_adam(L, lr, c->stream);
    }
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e == cudaSuccess && loss_hist) memcpy(loss_hist, h_loss, sizeof(float) * (size_t)iters);
    cudaFreeHost(h_loss);
    if (e == cudaSuccess && lpc_tc_error(L, c->stream))
        return fs_set_error(c, FS_ERR_CUDA, "tensor-core convolution failed (a bounded wait ran out)");
    return fs_cuda_check(c, e, "training");
}

// loss and gradient of given features/targets (host arrays), for checks
int fs_lpc_grad_impl(fs_ctx *c, const float *feat, const float *tgt, const float *mask, int batch, float *grad,
                     float *loss, float *pred) {
    if (!c->lpc) return fs_set_error(c, FS_ERR_INVALID, "learned preconditioner not initialised");
    LpcState *L = c->lpc;
    if (batch < 1 || batch > L->Bmax) return fs_set_error(c, FS_ERR_INVALID, "batch %d outside 1..%d", batch, L->Bmax);
    const size_t px = (size_t)L->Hn * L->Wn, P = px * batch;
    std::vector<__nv_bfloat16> x0(P * LPC_CIN0, __float2bfloat16(0.0f));
    for (size_t p = 0; p < P; p++)
        for (int k = 0; k < LPC_NFEAT; k++) x0[p * LPC_CIN0 + k] = __float2bfloat16(feat[p * LPC_NFEAT + k]);
    std::vector<float> bm(P);
    for (size_t p = 0; p < P; p++) bm[p] = mask[p % px];
    cudaError_t e = cudaMemcpyAsync(L->x0, x0.data(), x0.size() * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(L->btgt, tgt, P * sizeof(float), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(L->bmask, bm.data(), P * sizeof(float), cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return fs_cuda_check(c, e, "gradient inputs");
    if ((long)batch * L->Hn * L->Wn > L->cap0)
        return fs_set_error(c, FS_ERR_INVALID, "batch %d of full grids exceeds the activation buffers", batch);
    int r = lpc_forward(L, batch, L->Hn, L->Wn, c->stream);
    if (!r) r = lpc_loss_backward(L, batch, L->Hn, L->Wn, c->stream);
    if (r) return fs_cuda_check(c, (cudaError_t)r, "gradient");
    if (grad) e = cudaMemcpyAsync(grad, L->g, L->net.nparam * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && loss) e = cudaMemcpyAsync(loss, L->d_loss, sizeof(float), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && pred) e = cudaMemcpyAsync(pred, L->y, P * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e == cudaSuccess && lpc_tc_error(L, c->stream))
        return fs_set_error(c, FS_ERR_CUDA, "tensor-core convolution failed (a bounded wait ran out)");
    return fs_cuda_check(c, e, "gradient outputs");
}
