// fs_lapl.cu -- the semi-implicit Poisson solve on the GPU (plain FP64 path).
//
// lapl_solve (lapl_lib.F90:57-121) assembles A d = -b every step (laplEqn
// :123-379 for b, laplJ :381-609 and dFdPh :611-636 for A) and hands it to
// PETSc KSP.  Here:
//   * k_assemble evaluates, per face once, the Scharfetter-Gummel fluxes of
//     laplEqn and the flux derivatives of dFdPh, and writes the system in
//     its row-scaled symmetric form M d = D b with D = diag(dlx*dly),
//     M = -D A: per node the diagonal M_c, the east and north face
//     conductances c_e*dly and c_n*dlx (each face conductance
//     1/dx + dt (dFi - dFe) is shared by the two rows of the face, so M is
//     symmetric), and the Dirichlet/boundary remainder of the diagonal;
//   * the preconditioner is a geometric multigrid V-cycle on 2x2 node
//     aggregates: coarse face conductances are the series (along the face
//     normal) and parallel (across it) combination of the fine ones, red-black
//     Gauss-Seidel smoothing (red-black before, black-red after, so the cycle
//     is symmetric), restriction by summation and prolongation by injection;
//     levels with at most 32x32 nodes are handled by one CTA;
//   * CG runs to ||A d + b||_2 / ||b||_2 <= lapl_rtol on the unscaled rows,
//     the residual PETSc reports with -ksp_norm_type unpreconditioned;
//   * phi += d and ph_mi = phi (lapl_lib.F90:112-119).
// All reductions are two-level and fixed-order: per-CTA partials, then the
// last CTA to finish sums them in index order.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <cuda_runtime.h>

#include "fs_fastmath.cuh"
#include "fs_internal.h"

#include "fs_mg.cuh"
#include "fs_sg.cuh"

#define LBX 32
#define LBY 8
#define LNT (LBX * LBY)

namespace {

// ----------------------------------------------------------------- assembly
struct AsmArgs {
    PhysParams pp;
    MeshDev m;
    const double *tab;
    const double *ni, *ne, *nt, *ph, *phm;
    const double *fx_e, *fx_cl, *fx_cr, *fx_dl, *fx_dr, *fy_e, *fy_cl, *fy_cr, *fy_dl, *fy_dr;
    const Ctrl *ctrl;
    Ctrl *ctrl_w;
    const double *sig;   // sig_pl of the dielectric wall, nx+2
    double *mc, *ce, *cn, *extra, *inv_mc, *rhs, *dinv;
    float *mc32, *ce32, *cn32, *extra32, *inv_mc32;   // FP32 copy of the operator (the FP32 finest level), or null
};

__device__ __forceinline__ void tab_index(const PhysParams &pp, double T, int &k, double &w) {
    double x = fs_log(T * pp.ph0);
    double u = (x - pp.lemin) * pp.inv_h;
    if (!(u >= 0.0)) u = 0.0;
    if (u > (double)(pp.ntab - 1)) u = (double)(pp.ntab - 1);
    int i = (int)u;
    if (i > pp.ntab - 2) i = pp.ntab - 2;
    k = i;
    w = u - (double)i;
}
__device__ __forceinline__ double tab_val(const double *tab, int k, double w, int row) {
    const double *t = tab + (size_t)k * FS_TAB_STRIDE;
    return __ldg(t + row) + w * __ldg(t + 8 + row);
}

// SG flux (get_Flux, ptcl_props.F90:142-165) for charge q, and dFdPh of the
// same face at E_mi (lapl_lib.F90:611-636); the exponential is shared when
// the two fields agree, which they do for every interior face because
// ph_mi equals ph on the interior.
__device__ __forceinline__ void sg_and_dfdph(int q, double E, double Emi, double dh, double mu,
                                             double D, double nl, double nr, double &flux,
                                             double &df, unsigned int &st) {
    const double tolf = 9.9999999600419720025e-13;   // REAL(4) 1e-12 of get_Flux
    double v = (double)q * mu * E;
    double arg = v * dh / D;
    double exa = fs_exp(-fabs(arg));
    if (fabs((double)q * E) < tolf) {
        flux = D * (nl - nr) / dh;
    } else if (fabs(arg) < 1e-2) {   // Bernoulli form near a = 0
        double a2 = arg * arg;
        flux = D * ((nl - nr) + 0.5 * arg * (nl + nr) + a2 * (1.0 / 12.0 - a2 / 720.0) * (nl - nr)) / dh;
    } else {
        double ex = fabs(arg) > 100.0 ? exp(-100.0) : exa;
        if (arg > 0) flux = v * (nl - nr * ex) / (1.0 - ex);
        else flux = v * (nr - nl * ex) / (1.0 - ex);
    }
    double vm = (double)q * mu * Emi;
    double am = vm * dh / D;
    if (fabs(vm) < 1e-12) {
        df = 0.0;
    } else if (fabs(am) < 0.05) {
        // series of the same function near a = 0, where the closed form
        // cancels catastrophically: (n1+n2)/2 + (n1-n2)(a/6 - a^3/180 + a^5/5040)
        double dn = nl - nr, a2 = am * am;
        df = 0.5 * (nl + nr) + dn * am * (1.0 / 6.0 - a2 * (1.0 / 180.0 - a2 / 5040.0));
    } else {
        double ex = (Emi == E) ? exa : fs_exp(-fabs(am));
        double one = 1.0 - ex;
        if (am > 0) df = (nl - nr * ex) / one + vm * ex * (nr - nl) / (one * one) * dh / D;
        else df = (nr - nl * ex) / one + vm * ex * (nr - nl) / (one * one) * dh / D;
    }
    if (isnan(df)) st |= FS_ST_DFDPH_NAN;
}

// Electron flux of laplEqn and dFdPh of laplJ on one face when E_mi == E (the
// interior faces: ph_mi equals ph there), sharing one exponential.
__device__ __forceinline__ void elec_face(double E, double dh, double idh, double mue, double De,
                                          double nl, double nr, double e100, double &flux,
                                          double &df) {
    const double tolf = 9.9999999600419720025e-13;
    double v = -mue * E;
    double arg = v * dh / De;
    double aa = fabs(arg);
    double ex = aa >= 1e-2 ? fs_exp(-aa) : 0.0;
    if (fabs(E) < tolf) {
        flux = De * (nl - nr) * idh;
    } else if (aa < 1e-2) {
        double a2 = arg * arg;
        flux = De * ((nl - nr) + 0.5 * arg * (nl + nr) + a2 * (1.0 / 12.0 - a2 / 720.0) * (nl - nr)) * idh;
    } else {
        double exf = aa > 100.0 ? e100 : ex;
        double i1 = 1.0 / (1.0 - exf);
        flux = arg > 0 ? v * (nl - nr * exf) * i1 : v * (nr - nl * exf) * i1;
    }
    if (fabs(v) < 1e-12) {
        df = 0.0;
    } else if (aa < 0.05) {
        double a2 = arg * arg;
        df = 0.5 * (nl + nr) + (nl - nr) * arg * (1.0 / 6.0 - a2 * (1.0 / 180.0 - a2 / 5040.0));
    } else {
        double i1 = 1.0 / (1.0 - ex), t = arg * ex * (nr - nl) * i1 * i1;
        df = (arg > 0 ? (nl - nr * ex) : (nr - nl * ex)) * i1 + t;
    }
}

__global__ void __launch_bounds__(LNT, 2) k_assemble(const AsmArgs a) {
    __shared__ double s_ni[LBY + 2][LBX + 2], s_ne[LBY + 2][LBX + 2], s_nt[LBY + 2][LBX + 2];
    __shared__ double s_ph[LBY + 2][LBX + 2], s_pm[LBY + 2][LBX + 2];
    __shared__ double s_te[LBY + 2][LBX + 2], s_mu[LBY + 2][LBX + 2], s_de[LBY + 2][LBX + 2];
    // per face: ion flux, electron flux, field (as used by dfdx), conductance c, boundary g
    __shared__ double s_xfi[LBY][LBX + 1], s_xfe[LBY][LBX + 1], s_xe[LBY][LBX + 1], s_xc[LBY][LBX + 1];
    __shared__ double s_yfi[LBY + 1][LBX], s_yfe[LBY + 1][LBX], s_ye[LBY + 1][LBX], s_yc[LBY + 1][LBX];
    const PhysParams &pp = a.pp;
    const int nx = pp.nx, ny = pp.ny, P = pp.pitch;
    const int tid = threadIdx.x;
    const int gx0 = blockIdx.x * LBX + 1, gy0 = blockIdx.y * LBY + 1;
    const double dt = a.ctrl->dt;
    unsigned int st = 0;
    for (int q = tid; q < (LBX + 2) * (LBY + 2); q += LNT) {
        int lx = q % (LBX + 2), ly = q / (LBX + 2);
        int gi = gx0 - 1 + lx, gj = gy0 - 1 + ly;
        bool in = gi <= nx + 1 && gj <= ny + 1;
        size_t o = (size_t)gj * P + gi;
        s_ni[ly][lx] = in ? a.ni[o] : 0.0;
        s_ne[ly][lx] = in ? a.ne[o] : 0.0;
        s_nt[ly][lx] = in ? a.nt[o] : 0.0;
        s_ph[ly][lx] = in ? a.ph[o] : 0.0;
        s_pm[ly][lx] = in ? a.phm[o] : 0.0;
    }
    __syncthreads();
    for (int q = tid; q < (LBX + 2) * (LBY + 2); q += LNT) {
        int lx = q % (LBX + 2), ly = q / (LBX + 2);
        int gi = gx0 - 1 + lx, gj = gy0 - 1 + ly;
        double te = 0, mu = 0, de = 0;
        if (gi >= 1 && gi <= nx && gj >= 1 && gj <= ny) {
            double nte = s_nt[ly][lx], nee = s_ne[ly][lx];
            if ((nte >= 0.0) && (nee >= 0.0)) te = nte / nee;
            else { st |= FS_ST_NEG_DENSITY; te = 1e-8; }
            int k; double w;
            if (pp.fits) {
                mu = pp.fit.mue(te);
                de = pp.fit.De(te);
            } else {
                tab_index(pp, te, k, w);
                mu = tab_val(a.tab, k, w, 0);
                de = tab_val(a.tab, k, w, 1);
            }
        }
        s_te[ly][lx] = te; s_mu[ly][lx] = mu; s_de[ly][lx] = de;
    }
    __syncthreads();
    // x faces between gi and gi+1
    for (int q = tid; q < LBY * (LBX + 1); q += LNT) {
        int c = q % (LBX + 1), r = q / (LBX + 1);
        int gi = gx0 - 1 + c, gj = gy0 + r;
        if (gj > ny || gi > nx) continue;
        int lx = c, ly = r + 1;
        const size_t of = (size_t)gj * P + gi;
        double dh = a.m.dx[gi], idh = a.m.inv_dx[gi];
        double E = a.fx_e[of];
        int tl = gi >= 1 ? a.m.tx[(gj - 1) * nx + gi - 1] : 0;
        int tr = gi + 1 <= nx ? a.m.tx[(gj - 1) * nx + gi] : 0;
        double fi = 0, fe = 0, eu = E, cf = 0;
        if (gi == 0 && tr == -1) {
            eu = 0.0;
        } else if (gi == nx && tl == 1) {
            eu = 0.0;
        } else if (gi == 0 && tr == -2) {           // cathode-side electrode row
            int lc = lx + 1;
            double te = s_te[ly][lc], ni = s_ni[ly][lc], ne = s_ne[ly][lc], mue = s_mu[ly][lc];
            double aa = (s_ph[ly][lx] > s_ph[ly][lc]) ? 1.0 : 0.0;
            double ve = sqrt(pp.ve_coef * te) * pp.t0 / pp.x0;
            fi = (1.0 - aa) * pp.mui * E * ni - 2.5e-1 * pp.vi * ni;
            fe = -(aa * mue * E * ne) - 2.5e-1 * ve * ne - pp.gam * fi;
            int ac = (s_ph[ly][lx] > s_ph[ly][lc]) ? 1 : 0;
            double dfi = (double)(1 - ac) * pp.mui * ni * idh;
            double dfe = -((double)ac * mue * ne * idh) - pp.gam * dfi;
            cf = idh + dt * (dfi - dfe);              // Dirichlet conductance of the row
        } else if (gi == nx && tl == 2) {          // anode-side electrode row
            int lc = lx;
            double te = s_te[ly][lc], ni = s_ni[ly][lc], ne = s_ne[ly][lc], mue = s_mu[ly][lc];
            double aa = (s_ph[ly][lx + 1] > s_ph[ly][lc]) ? 1.0 : 0.0;
            double ve = sqrt(pp.ve_coef * te) * pp.t0 / pp.x0;
            fi = (1.0 - aa) * pp.mui * E * ni + 2.5e-1 * pp.vi * ni;
            fe = -(aa * mue * E * ne) + 2.5e-1 * ve * ne - pp.gam * fi;
            int ac = (s_ph[ly][lx + 1] > s_ph[ly][lc]) ? 1 : 0;
            double dfi = (double)(ac - 1) * pp.mui * ni * idh;
            double dfe = (double)ac * mue * ne * idh - pp.gam * dfi;
            cf = idh - dt * (dfi - dfe);
        } else {
            double mue = 5e-1 * (s_mu[ly][lx] + s_mu[ly][lx + 1]);
            double De = 5e-1 * (s_de[ly][lx] + s_de[ly][lx + 1]);
            const double nil = s_ni[ly][lx], nir = s_ni[ly][lx + 1], nel = s_ne[ly][lx], ner = s_ne[ly][lx + 1];
            double dFi, dFe;
            if (s_pm[ly][lx] == s_ph[ly][lx] && s_pm[ly][lx + 1] == s_ph[ly][lx + 1]) {
                fi = a.fx_cl[of] * nil - a.fx_cr[of] * nir;
                dFi = a.fx_dl[of] * nil + a.fx_dr[of] * nir;
                elec_face(E, dh, idh, mue, De, nel, ner, pp.e100, fe, dFe);
            } else {
                double Emi = -(s_pm[ly][lx + 1] - s_pm[ly][lx]) / dh;
                sg_and_dfdph(1, E, Emi, dh, pp.mui, pp.Di, nil, nir, fi, dFi, st);
                sg_and_dfdph(-1, E, Emi, dh, mue, De, nel, ner, fe, dFe, st);
            }
            if (isnan(dFi) || isnan(dFe)) st |= FS_ST_DFDPH_NAN;
            double dfi_mi = pp.mui * idh * dFi;
            double dfe_mi = -(mue * idh * dFe);
            cf = idh + dt * (dfi_mi - dfe_mi);
        }
        s_xfi[r][c] = fi; s_xfe[r][c] = fe; s_xe[r][c] = eu; s_xc[r][c] = cf;
    }
    // y faces between gj and gj+1
    for (int q = tid; q < (LBY + 1) * LBX; q += LNT) {
        int c = q % LBX, r = q / LBX;
        int gi = gx0 + c, gj = gy0 - 1 + r;
        if (gi > nx || gj > ny) continue;
        int lx = c + 1, ly = r;
        const size_t of = (size_t)gj * P + gi;
        double dh = a.m.dy[gj], idh = a.m.inv_dy[gj];
        double E = a.fy_e[of];
        int tb = gj >= 1 ? a.m.ty[(gj - 1) * nx + gi - 1] : 0;
        int tt = gj + 1 <= ny ? a.m.ty[gj * nx + gi - 1] : 0;
        double fi = 0, fe = 0, eu = E, cf = 0;
        if (gj == 0 && tt == -1) {
            eu = 0.0;
        } else if (gj == 0 && tt == -2) {
            // laplEqn has no lower y electrode flux (zero); laplJ has its derivative
            int lc = ly + 1;
            double ni = s_ni[lc][lx], ne = s_ne[lc][lx], mue = s_mu[lc][lx];
            int ac = (s_ph[ly][lx] > s_ph[lc][lx]) ? 1 : 0;
            double dfi = (double)(1 - ac) * pp.mui * ni / dh;
            double dfe = -((double)ac * mue * ne / dh) - pp.gam * dfi;
            cf = 1.0 / dh + dt * (dfi - dfe);
        } else if (gj == ny && tb == 1) {
            eu = 0.0;
        } else if (gj == ny && tb == 3) {
            // dielectric wall: field -sig (lapl_lib.F90:72-76,263-265), fluxes into an
            // empty wall node with the node's own coefficients (:322-331); laplJ
            // sets no column and no flux derivative for it (:548-559) but keeps
            // the interior form of the diagonal (:590-600): a boundary
            // conductance of 1/dy without dt terms
            const int lc = ly;
            E = -a.sig[gi];
            eu = E;
            fi = fs_sg_flux(1.0, E, dh, pp.mui, pp.Di, s_ni[lc][lx], 0.0);
            fe = fs_sg_flux(-1.0, E, dh, s_mu[lc][lx], s_de[lc][lx], s_ne[lc][lx], 0.0);
            cf = idh;
        } else if (gj == ny && tb == 2) {
            int lc = ly;
            double te = s_te[lc][lx], ni = s_ni[lc][lx], ne = s_ne[lc][lx], mue = s_mu[lc][lx];
            double aa = (s_ph[ly + 1][lx] > s_ph[lc][lx]) ? 1.0 : 0.0;
            double ve = sqrt(pp.ve_coef * te) * pp.t0 / pp.x0;
            fi = (1.0 - aa) * pp.mui * E * ni + 2.5e-1 * pp.vi * ni;
            fe = -(aa * mue * E * ne) + 2.5e-1 * ve * ne - pp.gam * fi;
            int ac = (s_ph[ly + 1][lx] > s_ph[lc][lx]) ? 1 : 0;
            double dfi = (double)(ac - 1) * pp.mui * ni / dh;
            double dfe = (double)ac * mue * ne / dh - pp.gam * dfi;
            cf = 1.0 / dh - dt * (dfi - dfe);
        } else {
            double mue = 5e-1 * (s_mu[ly][lx] + s_mu[ly + 1][lx]);
            double De = 5e-1 * (s_de[ly][lx] + s_de[ly + 1][lx]);
            const double nil = s_ni[ly][lx], nir = s_ni[ly + 1][lx], nel = s_ne[ly][lx], ner = s_ne[ly + 1][lx];
            double dFi, dFe;
            if (s_pm[ly][lx] == s_ph[ly][lx] && s_pm[ly + 1][lx] == s_ph[ly + 1][lx]) {
                fi = a.fy_cl[of] * nil - a.fy_cr[of] * nir;
                dFi = a.fy_dl[of] * nil + a.fy_dr[of] * nir;
                elec_face(E, dh, idh, mue, De, nel, ner, pp.e100, fe, dFe);
            } else {
                double Emi = -(s_pm[ly + 1][lx] - s_pm[ly][lx]) / dh;
                sg_and_dfdph(1, E, Emi, dh, pp.mui, pp.Di, nil, nir, fi, dFi, st);
                sg_and_dfdph(-1, E, Emi, dh, mue, De, nel, ner, fe, dFe, st);
            }
            if (isnan(dFi) || isnan(dFe)) st |= FS_ST_DFDPH_NAN;
            double dfi_mi = pp.mui * idh * dFi;
            double dfe_mi = -(mue * idh * dFe);
            cf = idh + dt * (dfi_mi - dfe_mi);
        }
        s_yfi[r][c] = fi; s_yfe[r][c] = fe; s_ye[r][c] = eu; s_yc[r][c] = cf;
    }
    __syncthreads();
    const int lx = tid % LBX, ly = tid / LBX;
    const int gi = gx0 + lx, gj = gy0 + ly;
    if (gi <= nx && gj <= ny) {
        const size_t o = (size_t)gj * P + gi;
        const double dlx = a.m.dlx[gi - 1], dly = a.m.dly[gj - 1];
        const double idlx = a.m.inv_dlx[gi - 1], idly = a.m.inv_dly[gj - 1];
        const int tx = a.m.tx[(gj - 1) * nx + gi - 1], ty = a.m.ty[(gj - 1) * nx + gi - 1];
        // cylindrical weights: r(j) of the row, face radii of the y faces
        const double wr = pp.cyl ? a.m.r[gj] : 1.0;
        const double wn = pp.cyl ? (a.m.r[gj + 1] + a.m.r[gj]) / 2.0 : 1.0;
        const double ws = pp.cyl ? (a.m.r[gj] + a.m.r[gj - 1]) / 2.0 : 1.0;
        // b of laplEqn (lapl_lib.F90:250-375)
        double dfdx = -(s_xe[ly][lx + 1] - s_xe[ly][lx]) * idlx;
        double dflxe_x = (s_xfe[ly][lx + 1] - s_xfe[ly][lx]) * idlx;
        double dflxi_x = (s_xfi[ly][lx + 1] - s_xfi[ly][lx]) * idlx;
        double dfdy, dflxi_y, dflxe_y;
        if (pp.cyl) {
            dfdy = -(s_ye[ly + 1][lx] * wn - s_ye[ly][lx] * ws) / dly / wr;
            dflxi_y = (s_yfi[ly + 1][lx] * wn - s_yfi[ly][lx] * ws) / dly / wr;
            dflxe_y = (s_yfe[ly + 1][lx] * wn - s_yfe[ly][lx] * ws) / dly / wr;
        } else {
            dfdy = -(s_ye[ly + 1][lx] - s_ye[ly][lx]) * idly;
            dflxi_y = (s_yfi[ly + 1][lx] - s_yfi[ly][lx]) * idly;
            dflxe_y = (s_yfe[ly + 1][lx] - s_yfe[ly][lx]) * idly;
        }
        double b = dfdx + dfdy + s_ni[ly + 1][lx + 1] - s_ne[ly + 1][lx + 1]
                 - dt * (dflxi_x + dflxi_y - dflxe_x - dflxe_y);
        if (isnan(b)) st |= FS_ST_BNAN;
        // Row of M = -D A with D = dlx*dly*r: a face shared with an interior
        // neighbour is an off-diagonal conductance; a boundary face enters the
        // diagonal only (laplJ, lapl_lib.F90:566-607).
        const double cw = s_xc[ly][lx], cee = s_xc[ly][lx + 1], cs = s_yc[ly][lx], cnn = s_yc[ly + 1][lx];
        const double offw = gi > 1 ? cw : 0.0, offe = gi < nx ? cee : 0.0;
        const double offs = gj > 1 ? cs : 0.0, offn = gj < ny ? cnn : 0.0;
        double gx = 0.0, gys = 0.0, gyn = 0.0;
        // electrode rows: Dirichlet conductance of the boundary face
        if (gi == 1 && tx == -2) gx += cw;
        if (gi == nx && tx == 2) gx += cee;
        if (gj == 1 && ty == -2) gys += cs;
        if (gj == ny && (ty == 2 || ty == 3)) gyn += cnn;
        // lower Neumann rows: the reference's diagonal takes the ghost spacing
        // dx(i-1) / dy(j-1) where the off-diagonal takes dx(i) / dy(j)
        if (gi == 1 && tx == -1) gx += 1.0 / a.m.dx[0] - 1.0 / a.m.dx[1];
        if (gj == 1 && ty == -1) gyn += 1.0 / a.m.dy[0] - 1.0 / a.m.dy[1];
        const double sx = dly * wr;
        const double extra = gx * sx + (gys * ws + gyn * wn) * dlx;
        const double mc = (offw + offe) * sx + (offs * ws + offn * wn) * dlx + extra;
        const double D = dlx * dly * wr;
        a.mc[o] = mc;
        if (a.inv_mc) a.inv_mc[o] = 1.0 / mc;   // the FP64 finest level's smoother only
        a.extra[o] = extra;
        if (a.mc32) {
            const float mc32 = (float)mc;
            a.mc32[o] = mc32;
            a.inv_mc32[o] = 1.0f / mc32;
            a.extra32[o] = (float)extra;
            a.ce32[o] = (float)(offe * sx);
            a.cn32[o] = (float)(offn * wn * dlx);
        }
        a.ce[o] = offe * sx;
        a.cn[o] = offn * wn * dlx;
        a.rhs[o] = b * D;
        if (a.dinv) a.dinv[o] = 1.0 / D;   // a property of the mesh: the first assembly writes it
    }
    if (st) atomicOr(&a.ctrl_w->status, st);
}


// ------------------------------------------------------------------------ CG
struct CgArgs {
    int nx, ny, P, nblk;
    dim3 grid;                             // nblk CTAs of 256 threads, grid-stride over nodes
    double *x, *r, *z, *p, *q, *rhs, *dinv, *part;
    const double *mc, *ce, *cn;
    float *r32;                            // FP32 finest level: its right-hand side, a copy of r (or null)
    const float *x32;                      // ... and its iterate, z in FP32
    Ctrl *ctrl;
    double rtol;
    int maxit;
    int use_cond;                          // loop runs under a conditional WHILE node
    cudaGraphConditionalHandle cond;
};

// Warm start.  The previous solve's correction d (still in x) scaled by the
// alpha that minimises the D^-1-weighted norm of b - alpha M d -- the norm
// the convergence test takes -- is the initial guess: never a larger initial
// residual than the zero start, which it becomes when M d vanishes or the
// sums are not finite.  The corrections of consecutive steps are alike (the
// discharge moves little in one dt), so the CG starts from a residual
// several times smaller.  Here M d (into q) and the three sums; alpha goes
// to the control block (spare[1]).
__global__ void __launch_bounds__(256) k_cg_init_warm(const CgArgs a) {
    double v[3] = {0.0, 0.0, 0.0};
    CG_NODES(a, {
        const double d = a.x[o];
        const double md = a.mc[o] * d - a.ce[o] * a.x[o + 1] - a.ce[o - 1] * a.x[o - 1] - a.cn[o] * a.x[o + a.P]
                        - a.cn[o - a.P] * a.x[o - a.P];
        a.q[o] = md;
        const double bw = a.rhs[o] * a.dinv[o], mw = md * a.dinv[o];
        v[0] += bw * bw;
        v[1] += bw * mw;
        v[2] += mw * mw;
    })
    double s[3];
    if (grid_sum3(v, a.part, &a.ctrl->counter[0], a.nblk, s) && threadIdx.x == 0) {
        Ctrl *c = a.ctrl;
        double al = s[2] > 0.0 ? s[1] / s[2] : 0.0;
        if (!isfinite(al)) al = 0.0;
        const double rr = al != 0.0 ? fmax(s[0] - al * s[1], 0.0) : s[0];
        c->spare[1] = al;
        c->bnorm2 = s[0];
        c->rnorm2 = rr;
        c->relres = s[0] > 0.0 ? sqrt(rr / s[0]) : 0.0;
        c->cg_done = s[0] == 0.0 ? 1 : 0;
        c->cg_iters = 0;
        c->cg_fail = 0;
        c->rz = 0.0;
    }
}

// x = alpha d, r = b - alpha M d (or the zero start), p = q = 0
__global__ void __launch_bounds__(256) k_cg_init_apply(const CgArgs a) {
    const double al = a.ctrl->spare[1];
    const bool warm = al != 0.0;
    CG_NODES(a, {
        const double r = warm ? a.rhs[o] - al * a.q[o] : a.rhs[o];
        a.x[o] = warm ? al * a.x[o] : 0.0;
        a.r[o] = r;
        if (a.r32) a.r32[o] = (float)r;
        a.p[o] = 0.0;
        a.q[o] = 0.0;
    })
}

// rz = r.z and zq = z.q (q = M p_old) of the preconditioned residual, then the
// flexible beta = -zq / p_old.q (Notay's FCG(1); 0 on the first iteration).
// Plain CG's rz / rz_old assumes a symmetric preconditioner, and the V-cycle
// is not one: its post-smoothing is over-relaxed and its pre-smoothing not,
// the electrode strips get sweeps after the post-smoothing only, and the
// finest level pre-smooths with fewer sweeps than it post-smooths.
__device__ __forceinline__ void cg_beta(Ctrl *c, double rz, double zq) {
    c->rz_old = c->rz;
    c->rz = rz;
    c->beta = c->cg_iters == 0 ? 0.0 : -zq / c->pq;
}

// z = the FP32 finest level's iterate, with rz = r.z and zq = z.q in FP64.
// (k_cg_pq reading z from the FP32 iterate instead, its five conversions
// per node on the FP64 pipe, was slower than this write and read of z.)
__global__ void __launch_bounds__(256) k_cg_rz32(const CgArgs a) {
    double v = 0.0, u = 0.0;
    CG_NODES(a, {
        const double z = (double)a.x32[o];
        a.z[o] = z;
        v += a.r[o] * z;
        u += z * a.q[o];
    })
    double sv, su;
    if (grid_sum2(v, u, a.part, &a.ctrl->counter[1], a.nblk, sv, su) && threadIdx.x == 0) cg_beta(a.ctrl, sv, su);
}

__global__ void __launch_bounds__(256) k_cg_rz(const CgArgs a) {
    double v = 0.0, u = 0.0;
    CG_NODES(a, {
        v += a.r[o] * a.z[o];
        u += a.z[o] * a.q[o];
    })
    double sv, su;
    if (grid_sum2(v, u, a.part, &a.ctrl->counter[1], a.nblk, sv, su) && threadIdx.x == 0) cg_beta(a.ctrl, sv, su);
}

// Last half sweep of the fine level (red, after the black one) fused with
// rz = r.z and zq = z.q over all nodes and the flexible beta (cg_beta).
__global__ void __launch_bounds__(256) k_rb_rz(const LevelDev L, const CgArgs a, double om) {
    double v = 0.0, u = 0.0;
    CG_NODES(a, {
        const int J = (int)j_ + 1, I = (int)(q_ - j_ * (unsigned)a.nx) + 1;
        double z = L.x[o];
        if (((I + J) & 1) == 0) {
            z = relax(z, gs_node(L, o), om);
            L.x[o] = z;
        }
        v += L.rhs[o] * z;   // black nodes are final after the previous half sweep
        u += a.q[o] * z;
    })
    double sv, su;
    if (grid_sum2(v, u, a.part, &a.ctrl->counter[1], a.nblk, sv, su) && threadIdx.x == 0) cg_beta(a.ctrl, sv, su);
}

// p = z + beta p ; q = M z + beta q (= M p, since q held M p_old) ; pq = p.q ;
// alpha = rz / pq.  Pointwise in p and q, so no halo of p is needed.
__global__ void __launch_bounds__(256) k_cg_pq(const CgArgs a) {
    double v = 0.0;
    const double be = a.ctrl->beta;
    CG_NODES(a, {
        double mz = a.mc[o] * a.z[o] - a.ce[o] * a.z[o + 1] - a.ce[o - 1] * a.z[o - 1]
                  - a.cn[o] * a.z[o + a.P] - a.cn[o - a.P] * a.z[o - a.P];
        double pn = a.z[o] + be * a.p[o];
        double qn = mz + be * a.q[o];
        a.p[o] = pn;
        a.q[o] = qn;
        v += pn * qn;
    })
    double out;
    if (grid_sum<256>(v, a.part, &a.ctrl->counter[2], a.nblk, &out) && threadIdx.x == 0) {
        Ctrl *c = a.ctrl;
        c->pq = out;
        if (c->cg_done) c->alpha = 0.0;   // right-hand side was zero: nothing to do
        else if (!(out > 0.0)) { c->cg_fail = 1; c->alpha = 0.0; }
        else c->alpha = c->rz / out;
    }
}

__global__ void __launch_bounds__(256) k_cg_xr(const CgArgs a) {
    double v = 0.0;
    const double al = a.ctrl->alpha;
    CG_NODES(a, {
        a.x[o] += al * a.p[o];
        double rr = a.r[o] - al * a.q[o];
        a.r[o] = rr;
        if (a.r32) a.r32[o] = (float)rr;
        double u = rr * a.dinv[o];
        v += u * u;
    })
    double out;
    if (grid_sum<256>(v, a.part, &a.ctrl->counter[3], a.nblk, &out) && threadIdx.x == 0) {
        Ctrl *c = a.ctrl;
        c->rnorm2 = out;
        c->cg_iters += 1;
        c->relres = c->bnorm2 > 0.0 ? sqrt(out / c->bnorm2) : 0.0;
        if (c->relres <= a.rtol) c->cg_done = 1;
        if (isnan(out)) c->cg_fail = 1;
        if (a.use_cond && (c->cg_done || c->cg_fail || c->cg_iters >= a.maxit))
            cudaGraphSetConditional(a.cond, 0u);
    }
}

LevelDev level_dev(const MGLevel &m) {
    LevelDev L;
    L.nx = m.nx; L.ny = m.ny; L.P = m.pitch;
    L.mc = m.mc; L.ce = m.ce; L.cn = m.cn; L.extra = m.extra; L.inv_mc = m.inv_mc;
    L.rhs = m.rhs; L.x = m.x; L.res = m.res;
    return L;
}

LvT<double> lvt(const MGLevel &m) {
    LvT<double> L;
    L.nx = m.nx; L.ny = m.ny; L.P = m.pitch;
    L.mc = m.mc; L.ce = m.ce; L.cn = m.cn; L.inv_mc = m.inv_mc; L.rhs = m.rhs; L.x = m.x; L.xd = m.xd;
    L.om = FS_MG_OMEGA_POST;
    return L;
}

}  // namespace

// ------------------------------------------------------------------ host side
static int alloc_zero(fs_ctx *c, double **p, size_t n) {
    cudaError_t e = cudaMalloc(p, n * sizeof(double));
    if (e != cudaSuccess) return fs_cuda_check(c, e, "cudaMalloc (Poisson)");
    e = cudaMemset(*p, 0, n * sizeof(double));
    return e == cudaSuccess ? FS_OK : fs_cuda_check(c, e, "cudaMemset");
}

// x-line smoothing where the mesh is anisotropic in the bulk (mg_aniso)
// or where fs_set_line_smoother asked for it; rows that fit a warp's shared
// memory (xline_fits: 4715 nodes in FP64, 9680 in FP32)
static bool xline_fits_ctx(const fs_ctx *c) {
    return xline_fits(c->nx);
}
static void xline_select(fs_ctx *c) {
    c->mg_xline = c->mg_xline_mode == 2 || (c->mg_xline_mode == 0 && c->mg_aniso);
    if (!xline_fits_ctx(c)) c->mg_xline = 0;
}

// the shared memory limits of the level kernels the FP64 solver launches (the
// mixed solver's are set in its own translation unit)
static int fp64_level_limits(fs_ctx *c) {
    if (c->mixed) return FS_OK;
    cudaError_t e = mg_level_smem_limits<double>(c);
    if (e == cudaSuccess) e = mg_level_smem_limits<float>(c);
    return e == cudaSuccess ? FS_OK : fs_cuda_check(c, e, "multigrid shared memory");
}

// Electrode strips of the finest level (k_rb_strips): the leading and trailing
// columns whose x faces conduct more than twice as well as their y faces, by
// the mesh spacings of the middle row; none when either is wider than
// FS_STRIP_MAX columns.  Allocates their snapshot in the solver's type.
// A mesh anisotropic in the middle of the grid takes x-line smoothing of the
// finest level (mg_xline) instead, unless fs_set_line_smoother chose
// otherwise.
int fs_mg_strips(fs_ctx *c) {
    const int nx = c->nx, j = c->ny / 2 + 1;
    const std::vector<double> &x = c->h_x, &y = c->h_y;
    const double dy = y[j + 1] - y[j], dly = 0.5 * (y[j + 1] - y[j - 1]);
    auto stretched = [&](int i) {
        double cx = 0.0;
        if (i > 1) cx = fmax(cx, dly / (x[i] - x[i - 1]));
        if (i < nx) cx = fmax(cx, dly / (x[i + 1] - x[i]));
        return cx > 2.0 * (0.5 * (x[i + 1] - x[i - 1]) / dy);
    };
    int kl = 0, kr = nx + 1;
    while (kl < nx / 2 && stretched(kl + 1)) kl++;
    while (kr - 1 > nx / 2 + 1 && stretched(kr - 1)) kr--;
    const bool wide = kl > FS_STRIP_MAX || nx + 1 - kr > FS_STRIP_MAX;
    if (wide) { kl = 0; kr = nx + 1; }
    // anisotropic in the bulk too: the middle column's x faces conduct more
    // than twice as well as its y faces (a 301x173 grid on the square glow
    // domain).  A mesh stretched near the electrodes over more than
    // FS_STRIP_MAX columns but isotropic in the middle (the tanh mesh) keeps
    // point smoothing: there x-lines took as many iterations (8 per step at
    // 1024^2) at more cost per V-cycle.
    c->mg_aniso = stretched(std::max(1, nx / 2));
    xline_select(c);
    c->strip_kl = kl;
    c->strip_kr = kr;
    c->strip_w = std::max(kl + 2, nx - kr + 3);
    if (!has_strips(c)) return fp64_level_limits(c);
    const size_t n = (size_t)2 * (c->ny + 2) * c->strip_w;
    cudaError_t e;
    if (c->mixed) {
        e = cudaMalloc(&c->strip_snap32, n * sizeof(float));
        if (e == cudaSuccess) e = cudaMemset(c->strip_snap32, 0, n * sizeof(float));
    } else {
        e = cudaMalloc(&c->strip_snap64, n * sizeof(double));
        if (e == cudaSuccess) e = cudaMemset(c->strip_snap64, 0, n * sizeof(double));
    }
    return e == cudaSuccess ? fp64_level_limits(c) : fs_cuda_check(c, e, "strip snapshot");
}

// Smoother of the V-cycles: -1 chosen from the mesh, 0 point red-black, 1
// zebra x-line.  The solvers' CUDA graphs are rebuilt at their next use.
int fs_set_line_smoother_impl(fs_ctx *c, int mode) {
    if (mode < -1 || mode > 1) return fs_set_error(c, FS_ERR_INVALID, "line smoother mode must be -1, 0 or 1");
    if (mode == 1 && !xline_fits_ctx(c))
        return fs_set_error(c, FS_ERR_UNSUPPORTED, "x-line smoothing takes rows of up to %d nodes (%s)",
                            c->mixed ? 9680 : 4715, c->mixed ? "FP32" : "FP64");
    c->mg_xline_mode = mode + 1;
    if (c->cg_graph_built) {
        cudaGraphExecDestroy(c->cg_exec);
        cudaGraphDestroy(c->cg_graph);
        c->cg_graph_built = 0;
    }
    xline_select(c);
    if (c->mixed) return fs_lapl_mixed_reconfigure(c);
    return fp64_level_limits(c);
}

int fs_lapl_alloc(fs_ctx *c) {
    if (int rs = fs_mg_strips(c)) return rs;
    int nx = c->nx, ny = c->ny, nl = 0;
    for (;;) {
        MGLevel &m = c->mg[nl];
        m.nx = nx; m.ny = ny;
        m.pitch = ((nx + 2 + 31) / 32) * 32;
        size_t n = (size_t)(ny + 2) * m.pitch;
        int rc;
        double **fields[] = {&m.mc, &m.ce, &m.cn, &m.extra, &m.inv_mc, &m.res};
        for (double **f : fields)
            if ((rc = alloc_zero(c, f, n))) return rc;
        if (nl == 0) {
            m.rhs = nullptr;   // bound to the CG vectors below
            m.x = nullptr;
        } else {
            if ((rc = alloc_zero(c, &m.rhs, n))) return rc;
            if ((rc = alloc_zero(c, &m.x, n))) return rc;
            if ((rc = alloc_zero(c, &m.xd, n))) return rc;   // fused levels (1 and coarser)
        }
        nl++;
        if ((nx == 1 && ny == 1) || nl == FS_MG_MAX_LEVELS) break;
        nx = (nx + 1) / 2;
        ny = (ny + 1) / 2;
    }
    c->mg_nlev = nl;
    c->mg_fused = c->cfg.mg_smooth == 2;
    cudaFuncSetAttribute(k_mg_down<double, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mg_down_smem<double>(2));
    cudaFuncSetAttribute(k_mg_up<double, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mg_up_smem<double>(2));
    {
        BottomArgs<double> ba;
        ba.nl = nl;
        ba.lb = 0;
        while (ba.lb < nl && (c->mg[ba.lb].nx > BOTTOM_N || c->mg[ba.lb].ny > BOTTOM_N)) ba.lb++;
        for (int l = 0; l < nl; l++) { ba.L[l].nx = c->mg[l].nx; ba.L[l].ny = c->mg[l].ny; }
        ba.dl = bottom_dense_level(ba);
        c->mg_lb = ba.lb;
        c->mg_dl = ba.dl;
        cudaError_t e = fs_smem_limit((const void *)k_bottom_smem<double>, bottom_smem_bytes(ba));
        if (e != cudaSuccess) return fs_cuda_check(c, e, "bottom solver shared memory");
        if ((e = cudaMalloc(&c->d_ainv64, 64 * 64 * sizeof(double))) != cudaSuccess)
            return fs_cuda_check(c, e, "cudaMalloc (dense inverse)");
    }
    // the preconditioner's levels in FP32 (see vcycle): all of them with the
    // fused smoother and at least two levels above the bottom solver
    c->mg_lf = nl;
    if (!c->mixed && c->mg_fused && c->mg_lb >= 2) {
        c->mg_lf = 0;
        for (int l = c->mg_lf; l < nl; l++) {
            MGLevelF &m = c->mgc[l];
            m.nx = c->mg[l].nx;
            m.ny = c->mg[l].ny;
            m.pitch = c->mg[l].pitch;
            m.res = nullptr;
            const size_t n = (size_t)(m.ny + 2) * m.pitch;
            float **fields[] = {&m.mc, &m.ce, &m.cn, &m.extra, &m.inv_mc, &m.rhs, &m.x, &m.xd};
            for (float **f : fields) {
                cudaError_t e = cudaMalloc(f, n * sizeof(float));
                if (e == cudaSuccess) e = cudaMemset(*f, 0, n * sizeof(float));
                if (e != cudaSuccess) return fs_cuda_check(c, e, "cudaMalloc (FP32 coarse levels)");
            }
        }
        cudaError_t e = cudaMalloc(&c->d_ainvc, 64 * 64 * sizeof(float));
        if (e != cudaSuccess) return fs_cuda_check(c, e, "cudaMalloc (dense inverse)");
        if (has_strips(c)) {   // the FP32 finest level's strip snapshot
            const size_t ns = (size_t)2 * (c->ny + 2) * c->strip_w;
            e = cudaMalloc(&c->strip_snap32, ns * sizeof(float));
            if (e == cudaSuccess) e = cudaMemset(c->strip_snap32, 0, ns * sizeof(float));
            if (e != cudaSuccess) return fs_cuda_check(c, e, "strip snapshot");
        }
        cudaFuncSetAttribute(k_mg_down<float, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)mg_down_smem<float>(2));
        cudaFuncSetAttribute(k_mg_up<float, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mg_up_smem<float>(2));
        BottomArgs<float> bf;
        bf.nl = nl;
        bf.lb = c->mg_lb;
        bf.dl = c->mg_dl;
        for (int l = 0; l < nl; l++) { bf.L[l].nx = c->mg[l].nx; bf.L[l].ny = c->mg[l].ny; }
        e = fs_smem_limit((const void *)k_bottom_smem<float>, bottom_smem_bytes(bf));
        if (e != cudaSuccess) return fs_cuda_check(c, e, "bottom solver shared memory");
    }
    size_t n0 = (size_t)(c->ny + 2) * c->pitch;
    double **vecs[] = {&c->p, &c->q, &c->z, &c->r, &c->xs, &c->bs, &c->dinv};
    for (double **v : vecs) {
        int rc = alloc_zero(c, v, n0);
        if (rc) return rc;
    }
    c->mg[0].rhs = c->r;
    c->mg[0].x = c->z;
    dim3 g = grid2(c->nx, c->ny, dim3(32, 8));
    // partials of the CG reductions: three per CTA of the (<= 4 per SM) CG grids
    c->cg_nblk = std::max((int)(g.x * g.y), 3 * 4 * c->nsm);
    return alloc_zero(c, &c->d_cg_part, (size_t)c->cg_nblk);
}

void fs_lapl_free(fs_ctx *c) {
    if (c->cg_graph_built) {
        cudaGraphExecDestroy(c->cg_exec);
        cudaGraphDestroy(c->cg_graph);
        c->cg_graph_built = 0;
    }
    for (int l = 0; l < c->mg_nlev; l++) {
        MGLevel &m = c->mg[l];
        double *fs[] = {m.mc, m.ce, m.cn, m.extra, m.inv_mc, m.res};
        for (double *f : fs) cudaFree(f);
        if (l > 0) { cudaFree(m.rhs); cudaFree(m.x); cudaFree(m.xd); }
    }
    double *vs[] = {c->p, c->q, c->z, c->r, c->xs, c->bs, c->dinv, c->d_cg_part, c->d_ainv64};
    for (double *v : vs) cudaFree(v);
    for (int l = c->mg_lf; l < c->mg_nlev; l++) {
        MGLevelF &m = c->mgc[l];
        float *fs[] = {m.mc, m.ce, m.cn, m.extra, m.inv_mc, m.rhs, m.x, m.xd};
        for (float *f : fs) cudaFree(f);
        memset(&m, 0, sizeof(m));
    }
    cudaFree(c->d_ainvc);
    c->d_ainvc = nullptr;
    cudaFree(c->strip_snap64);
    cudaFree(c->strip_snap32);
    c->strip_snap64 = nullptr;
    c->strip_snap32 = nullptr;
    c->mg_nlev = 0;
}

// The V-cycle of the FP64 solver's preconditioner.  Levels mg_lf.. run in
// FP32 with the mixed solver's fused level kernels, strip sweeps and bottom
// solver -- on grids with at least two levels above the bottom solver all of
// them (mg_lf = 0): the V-cycle only shapes the preconditioner of the FP64
// CG, whose iterate, residual, operator product and convergence test stay
// FP64, and its FP64 kernels were FP64-issue-bound on this GPU (the FP64
// fused levels and bottom solve took ~2.5x their FP32 time, the FP64
// finest-level sweeps ~1.4x).  The finest level's operator is the FP64
// assembly's, rounded to FP32 as the assembly writes it; its right-hand
// side is r rounded by the CG kernels that update r, and z comes back in
// FP64 with r.z (k_cg_rz32).  On smaller grids (mg_lf = mg_nlev) every
// level runs in FP64.
static void vcycle(fs_ctx *c, const CgArgs *ca) {
    const int nl = c->mg_nlev, nu = c->cfg.mg_smooth, lf = c->mg_lf;
    int lb = 0;
    while (lb < nl && (c->mg[lb].nx > BOTTOM_N || c->mg[lb].ny > BOTTOM_N)) lb++;
    dim3 b(32, 8);
    for (int l = 0; l < lb; l++) {
        if (l >= lf) {
            if (l == 0 && c->mg_xline) {   // x-line pre-smoothing, the odd rows' residual restricted
                const LevelT<float> f = level_f(c->mgc[0]), cc = level_f(c->mgc[1]);
                xline_pairs<float>(c, f, fs_mg_pre0(nu), true, 1.0f);
                fs_prof_begin(c, PROF_TRANSFER);
                k_restrict_odd<float><<<grid2(cc.nx, cc.ny, b), b, 0, c->stream>>>(f, cc);
                fs_prof_end(c);
                continue;
            }
            fs_prof_begin(c, PROF_SMOOTH);
            k_mg_down<float, 2><<<grid2(c->mgc[l].nx, c->mgc[l].ny, dim3(MTX, MTY)), 256, mg_down_smem<float>(2),
                                  c->stream>>>(lvt_f(c->mgc[l]), lvt_f(c->mgc[l + 1]));
            fs_prof_end(c);
            continue;
        }
        LevelDev f = level_dev(c->mg[l]), cc = level_dev(c->mg[l + 1]);
        if (l == 0 && c->mg_xline) {   // x-line pre-smoothing, the odd rows' residual restricted
            xline_pairs<double>(c, f, fs_mg_pre0(nu), true, 1.0);
            fs_prof_begin(c, PROF_TRANSFER);
            if (l + 1 == lf) k_restrict_odd<double, float><<<grid2(cc.nx, cc.ny, b), b, 0, c->stream>>>(f, level_f(c->mgc[lf]));
            else k_restrict_odd<double><<<grid2(cc.nx, cc.ny, b), b, 0, c->stream>>>(f, cc);
            fs_prof_end(c);
            continue;
        }
        // fused (temporally blocked) levels only where launches dominate: the
        // FP64 levels above 256^2 are FP64-issue-bound, and the fused kernel's
        // redundant halo sweeps cost more there than the launches they save
        if (c->mg_fused && l > 0 && c->mg[l].nx <= 256 && c->mg[l].ny <= 256) {
            LvT<double> F = lvt(c->mg[l]), C = lvt(c->mg[l + 1]);
            fs_prof_begin(c, PROF_SMOOTH);
            k_mg_down<double, 2><<<grid2(f.nx, f.ny, dim3(MTX, MTY)), 256, mg_down_smem<double>(2), c->stream>>>(F, C);
            fs_prof_end(c);
            continue;
        }
        dim3 g = grid2((f.nx + 1) / 2, f.ny, b);
        fs_prof_begin(c, PROF_SMOOTH);
        k_rb_pair0<<<g, b, 0, c->stream>>>(f);   // the first red-black pair, from x = 0
        fs_prof_end(c);
        for (int it = 1; it < (l == 0 ? fs_mg_pre0(nu) : nu); it++) {
            fs_prof_begin(c, PROF_SMOOTH);
            k_rb<<<g, b, 0, c->stream>>>(f, 0, 0);
            fs_prof_end(c);
            fs_prof_begin(c, PROF_SMOOTH);
            k_rb<<<g, b, 0, c->stream>>>(f, 1, 0);
            fs_prof_end(c);
        }
        fs_prof_begin(c, PROF_TRANSFER);
        if (l + 1 == lf) k_restrict<double, float><<<grid2(cc.nx, cc.ny, b), b, 0, c->stream>>>(f, level_f(c->mgc[lf]));
        else if (l == 0) k_restrict<<<grid2(cc.nx, cc.ny, b), b, 0, c->stream>>>(f, cc);
        else k_restrict_t<double><<<grid2(cc.nx, cc.ny, b), b, 0, c->stream>>>(f, cc);
        fs_prof_end(c);
    }
    if (lf < nl) {
        BottomArgs<float> ba;
        for (int l = 0; l < nl; l++) ba.L[l] = level_f(c->mgc[l]);
        ba.lb = lb;
        ba.nl = nl;
        ba.nu = nu;
        ba.dl = c->mg_dl;
        ba.ainv = c->d_ainvc;
        ba.om = (float)FS_MG_OMEGA_POST;
        fs_prof_begin(c, PROF_BOTTOM);
        k_bottom_smem<float><<<1, BOTTOM_THREADS, bottom_smem_bytes(ba), c->stream>>>(ba);
        fs_prof_end(c);
    } else {
        BottomArgs<double> ba;
        for (int l = 0; l < nl; l++) ba.L[l] = level_dev(c->mg[l]);
        ba.lb = lb;
        ba.nl = nl;
        ba.nu = nu;
        ba.dl = c->mg_dl;
        ba.ainv = c->d_ainv64;
        ba.om = FS_MG_OMEGA_POST;
        fs_prof_begin(c, PROF_BOTTOM);
        k_bottom_smem<double><<<1, BOTTOM_THREADS, bottom_smem_bytes(ba), c->stream>>>(ba);
        fs_prof_end(c);
    }
    for (int l = lb - 1; l >= 0; l--) {
        if (l >= lf) {
            if (l == 0 && c->mg_xline) {   // x-line post-smoothing
                const LevelT<float> f = level_f(c->mgc[0]);
                fs_prof_begin(c, PROF_TRANSFER);
                k_prolong<float><<<grid2(f.nx, f.ny, b), b, 0, c->stream>>>(f, level_f(c->mgc[1]));
                fs_prof_end(c);
                xline_pairs<float>(c, f, nu, false, (float)FS_XL_OMEGA_POST);
            } else {
                // the finest level's post-smoothing fills the strip snapshot, and
                // the strips get their extra sweep pairs after it
                const bool strips = l == 0 && has_strips(c);
                LvT<float> F = lvt_f(c->mgc[l]);
                if (strips) F.sn = strip_snap(c, c->strip_snap32);
                fs_prof_begin(c, PROF_SMOOTH);
                k_mg_up<float, 2><<<grid2(c->mgc[l].nx, c->mgc[l].ny, dim3(MTX, MTY)), 256, mg_up_smem<float>(2),
                                    c->stream>>>(F, lvt_f(c->mgc[l + 1]));
                fs_prof_end(c);
                if (strips) {
                    fs_prof_begin(c, PROF_SMOOTH);
                    k_rb_strips<float><<<dim3((c->ny + STRIP_ROWS - 1) / STRIP_ROWS, 2), 256,
                                         strip_smem<float>(c->strip_w), c->stream>>>(
                        level_f(c->mgc[0]), F.sn, 1, (float)FS_MG_OMEGA_POST);
                    fs_prof_end(c);
                }
            }
            if (l == 0) {   // z in FP64 from the FP32 iterate, r.z and z.q
                fs_prof_begin(c, PROF_CG);
                k_cg_rz32<<<ca->grid, 256, 0, c->stream>>>(*ca);
                fs_prof_end(c);
            }
            continue;
        }
        LevelDev f = level_dev(c->mg[l]), cc = level_dev(c->mg[l + 1]);
        if (c->mg_fused && l > 0 && c->mg[l].nx <= 256 && c->mg[l].ny <= 256) {
            LvT<double> F = lvt(c->mg[l]), C = lvt(c->mg[l + 1]);
            fs_prof_begin(c, PROF_SMOOTH);
            k_mg_up<double, 2><<<grid2(f.nx, f.ny, dim3(MTX, MTY)), 256, mg_up_smem<double>(2), c->stream>>>(F, C);
            fs_prof_end(c);
            continue;
        }
        dim3 g = grid2(f.nx, f.ny, b), gh = grid2((f.nx + 1) / 2, f.ny, b);
        fs_prof_begin(c, PROF_TRANSFER);
        if (l + 1 == lf) k_prolong<double, float><<<g, b, 0, c->stream>>>(f, level_f(c->mgc[lf]));
        else k_prolong<<<g, b, 0, c->stream>>>(f, cc);
        fs_prof_end(c);
        if (l == 0 && c->mg_xline) {   // x-line post-smoothing, then r.z
            xline_pairs<double>(c, f, nu, false, FS_XL_OMEGA_POST);
            fs_prof_begin(c, PROF_CG);
            k_cg_rz<<<ca->grid, 256, 0, c->stream>>>(*ca);
            fs_prof_end(c);
            continue;
        }
        for (int it = 0; it < nu; it++) {
            // the strip sweeps go before the last half sweep, which is fused
            // with r.z: red-black pairs after the black half sweep, which
            // fills their snapshot
            const bool strips = l == 0 && it == nu - 1 && has_strips(c);
            const StripSnap<double> sn = strips ? strip_snap(c, c->strip_snap64) : StripSnap<double>{};
            fs_prof_begin(c, PROF_SMOOTH);
            k_rb<<<gh, b, 0, c->stream>>>(f, 1, 0, FS_MG_OMEGA_POST, sn);
            fs_prof_end(c);
            if (l == 0 && it == nu - 1) {
                if (strips) {
                    fs_prof_begin(c, PROF_SMOOTH);
                    k_rb_strips<double><<<dim3((f.ny + STRIP_ROWS - 1) / STRIP_ROWS, 2), 256,
                                          strip_smem<double>(c->strip_w), c->stream>>>(f, sn, 0, FS_MG_OMEGA_POST);
                    fs_prof_end(c);
                }
                fs_prof_begin(c, PROF_SMOOTH);
                k_rb_rz<<<ca->grid, 256, 0, c->stream>>>(f, *ca, FS_MG_OMEGA_POST);
                fs_prof_end(c);
            } else {
                fs_prof_begin(c, PROF_SMOOTH);
                k_rb<<<gh, b, 0, c->stream>>>(f, 0, 0, FS_MG_OMEGA_POST);
                fs_prof_end(c);
            }
        }
    }
    if (lb == 0) {   // the whole V-cycle ran in the bottom kernel: r.z separately
        fs_prof_begin(c, PROF_CG);
        k_cg_rz<<<ca->grid, 256, 0, c->stream>>>(*ca);
        fs_prof_end(c);
    }
}

// One PCG iteration: z = B r, rz, p = z + beta p, q = M p, x/r update.
static void cg_iteration(fs_ctx *c, const CgArgs &ca, dim3 gb) {
    vcycle(c, &ca);
    fs_prof_begin(c, PROF_CG);
    k_cg_pq<<<ca.grid, 256, 0, c->stream>>>(ca);
    fs_prof_end(c);
    fs_prof_begin(c, PROF_CG);
    k_cg_xr<<<ca.grid, 256, 0, c->stream>>>(ca);
    fs_prof_end(c);
}

// Graph: WHILE(cond) { one PCG iteration } -> phi update.  The last CTA of the
// residual reduction clears cond on convergence, breakdown or the iteration cap.
static int build_cg_graph(fs_ctx *c, CgArgs ca) {
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
    dim3 gb = grid2(c->nx, c->ny, dim3(32, 8));
    e = cudaStreamBeginCaptureToGraph(c->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cg_iteration(c, ca, gb);
        e = cudaStreamEndCapture(c->stream, &body);
    }
    c->cg_body_kernels = (int)(c->launches - l0);
    if (e == cudaSuccess)
        e = cudaStreamBeginCaptureToGraph(c->stream, g, &wnode, nullptr, 1, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        k_phi_update<<<4 * 152, 256, 0, c->stream>>>(c->ph, c->ph_mi, c->xs, c->nx, c->ny, c->pitch, c->d_ctrl);
        e = cudaStreamEndCapture(c->stream, &g);
    }
    c->launches = l0;
    c->prof_on = prof;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&c->cg_exec, g, 0);
    if (e != cudaSuccess) {
        // A capture that failed (a launch inside it was refused) leaves the
        // graph holding a conditional body the driver has invalidated, and
        // destroying it then crashed the process: the graph is leaked on
        // this error path, which ends the solve with the error anyway.
        return fs_cuda_check(c, e, "CG graph capture");
    }
    c->cg_graph = g;
    c->cg_graph_built = 1;
    return FS_OK;
}

int fs_lapl_solve_impl(fs_ctx *c, int *lerr, int *iters, double *relres) {
    static const bool trace = getenv("FS_TRACE_CG") != nullptr;
    AsmArgs a;
    a.pp = c->pp;
    a.m = c->mesh;
    a.tab = c->d_tab;
    a.ni = c->sp[0].buf[c->lev[0]];
    a.ne = c->sp[1].buf[c->lev[0]];
    a.nt = c->sp[2].buf[c->lev[0]];
    a.ph = c->ph;
    a.phm = c->ph_mi;
    fs_faces_update(c);   // E and the ion coefficients of the current phi
    a.fx_e = c->fx_e; a.fx_cl = c->fx_cl; a.fx_cr = c->fx_cr; a.fx_dl = c->fx_dl; a.fx_dr = c->fx_dr;
    a.fy_e = c->fy_e; a.fy_cl = c->fy_cl; a.fy_cr = c->fy_cr; a.fy_dl = c->fy_dl; a.fy_dr = c->fy_dr;
    a.ctrl = c->d_ctrl;
    a.ctrl_w = c->d_ctrl;
    a.sig = fs_sig(c, 0);
    MGLevel &m0 = c->mg[0];
    a.mc = m0.mc; a.ce = m0.ce; a.cn = m0.cn; a.extra = m0.extra; a.inv_mc = m0.inv_mc;
    a.rhs = c->bs;   // scaled right-hand side D b
    a.dinv = c->dinv;
    a.mc32 = a.ce32 = a.cn32 = a.extra32 = a.inv_mc32 = nullptr;
    if (c->mg_lf == 0) {   // the FP32 finest level of the preconditioner (no FP64 smoothing there)
        MGLevelF &f0 = c->mgc[0];
        a.mc32 = f0.mc; a.ce32 = f0.ce; a.cn32 = f0.cn; a.extra32 = f0.extra; a.inv_mc32 = f0.inv_mc;
        a.inv_mc = nullptr;
    }
    if (c->dinv_done) a.dinv = nullptr;
    // status bits of the assembly
    cudaMemsetAsync(&c->d_ctrl->status, 0, sizeof(unsigned int), c->stream);   // not a kernel
    dim3 g = grid2(c->nx, c->ny, dim3(LBX, LBY));
    fs_prof_begin(c, PROF_ASSEMBLE);
    k_assemble<<<g, LNT, 0, c->stream>>>(a);
    fs_prof_end(c);
    c->dinv_done = 1;
    // coarse operators: one launch per large level, then one CTA for the
    // small levels and the dense inverse
    if (c->mg_lf < c->mg_nlev) {   // FP32 levels: level 1 from the FP64 level 0 (level 0 came with the assembly)
        const int lf = std::max(c->mg_lf, 1);
        CoarsenTail<float> ct;
        for (int l = 0; l < c->mg_nlev; l++) {
            ct.L[l] = level_f(c->mgc[l]);
            ct.L[l].nx = c->mg[l].nx;
            ct.L[l].ny = c->mg[l].ny;
        }
        ct.nl = c->mg_nlev;
        ct.l0 = std::max(coarsen_tail_level(ct.L, ct.nl), lf + 1);
        ct.dl = c->mg_dl;
        ct.ainv = c->d_ainvc;
        dim3 b2(16, 16);
        fs_prof_begin(c, PROF_COARSEN);
        k_coarsen<double, float><<<grid2(ct.L[lf].nx, ct.L[lf].ny, b2), b2, 0, c->stream>>>(
            level_dev(c->mg[lf - 1]), ct.L[lf]);
        fs_prof_end(c);
        for (int l = lf + 1; l < ct.l0; l++) {
            fs_prof_begin(c, PROF_COARSEN);
            k_coarsen<float><<<grid2(ct.L[l].nx, ct.L[l].ny, b2), b2, 0, c->stream>>>(ct.L[l - 1], ct.L[l]);
            fs_prof_end(c);
        }
        fs_prof_begin(c, PROF_COARSEN);
        k_coarsen_tail<float><<<1, 1024, 0, c->stream>>>(ct);
        fs_prof_end(c);
    } else {
        CoarsenTail<double> ct;
        for (int l = 0; l < c->mg_nlev; l++) ct.L[l] = level_dev(c->mg[l]);
        ct.nl = c->mg_nlev;
        ct.l0 = coarsen_tail_level(ct.L, ct.nl);
        ct.dl = c->mg_dl;
        ct.ainv = c->d_ainv64;
        dim3 b2(16, 16);
        for (int l = 1; l < ct.l0; l++) {
            fs_prof_begin(c, PROF_COARSEN);
            k_coarsen<<<grid2(ct.L[l].nx, ct.L[l].ny, b2), b2, 0, c->stream>>>(ct.L[l - 1], ct.L[l]);
            fs_prof_end(c);
        }
        fs_prof_begin(c, PROF_COARSEN);
        k_coarsen_tail<double><<<1, 1024, 0, c->stream>>>(ct);
        fs_prof_end(c);
    }
    // CG on M d = D b
    CgArgs ca;
    ca.nx = c->nx; ca.ny = c->ny; ca.P = c->pitch;
    {
        long nb = ((long)c->nx * c->ny + 255) / 256, cap = 4L * c->nsm;
        ca.nblk = (int)(nb < cap ? nb : cap);
        ca.grid = dim3(ca.nblk);
    }
    ca.x = c->xs; ca.r = c->r; ca.z = c->z; ca.p = c->p; ca.q = c->q;
    ca.rhs = c->bs; ca.dinv = c->dinv; ca.part = c->d_cg_part;
    ca.mc = m0.mc; ca.ce = m0.ce; ca.cn = m0.cn;
    ca.r32 = c->mg_lf == 0 ? c->mgc[0].rhs : nullptr;
    ca.x32 = c->mg_lf == 0 ? c->mgc[0].x : nullptr;
    ca.ctrl = c->d_ctrl;
    ca.rtol = c->cfg.lapl_rtol;
    ca.maxit = c->cfg.lapl_maxit;
    ca.use_cond = 0;
    ca.cond = 0;
    dim3 gb = grid2(c->nx, c->ny, dim3(32, 8));
    fs_prof_begin(c, PROF_CG);
    k_cg_init_warm<<<ca.grid, 256, 0, c->stream>>>(ca);
    fs_prof_end(c);
    fs_prof_begin(c, PROF_CG);
    k_cg_init_apply<<<ca.grid, 256, 0, c->stream>>>(ca);
    fs_prof_end(c);
    int rc = fs_sync_ctrl(c);
    if (rc) return rc;
    if (c->h_ctrl->status & FS_ST_NEG_DENSITY) return fs_set_error(c, FS_ERR_NEG_DENSITY, "negative density in get_Te");
    if (c->h_ctrl->status & FS_ST_DFDPH_NAN) return fs_set_error(c, FS_ERR_NAN, "NaN in dFdPh");
    int it = 0;
    bool ok = c->h_ctrl->cg_done != 0;
    if (c->h_ctrl->status & FS_ST_BNAN) {
        *lerr = 1; *iters = 0; *relres = NAN;
        return FS_OK;
    }
    // FS_NO_GRAPH=1 keeps the loop on the host so that a profiler sees each kernel
    static const bool no_graph = getenv("FS_NO_GRAPH") != nullptr;
    const int poisson_classes = (1 << PROF_SMOOTH) | (1 << PROF_TRANSFER) | (1 << PROF_BOTTOM) | (1 << PROF_CG);
    if (!ok && !no_graph && !(c->prof_on & poisson_classes)) {
        // whole CG loop and the phi update as one graph launch
        if (!c->cg_graph_built && (rc = build_cg_graph(c, ca))) return rc;
        int before = 0;
        cudaError_t e = cudaGraphLaunch(c->cg_exec, c->stream);
        if (e != cudaSuccess) return fs_cuda_check(c, e, "CG graph launch");
        (void)before;
        rc = fs_sync_ctrl(c);
        if (rc) return rc;
        c->launches += (int64_t)c->h_ctrl->cg_iters * c->cg_body_kernels + 1;
        *iters = c->h_ctrl->cg_iters;
        *relres = c->h_ctrl->relres;
        bool conv = c->h_ctrl->cg_done && !c->h_ctrl->cg_fail;
        *lerr = conv ? 0 : 1;
        if (conv) c->faces_valid = 0;   // phi += d happened in the graph
        return FS_OK;
    }
    while (!ok && it < c->cfg.lapl_maxit) {
        cg_iteration(c, ca, gb);
        rc = fs_sync_ctrl(c);
        if (rc) return rc;
        it = c->h_ctrl->cg_iters;
        if (trace)
            fprintf(stderr, "cg %d relres %.3e rz %.3e pq %.3e alpha %.3e beta %.3e fail %d\n", it,
                    c->h_ctrl->relres, c->h_ctrl->rz, c->h_ctrl->pq, c->h_ctrl->alpha, c->h_ctrl->beta,
                    c->h_ctrl->cg_fail);
        if (c->h_ctrl->cg_fail) break;
        ok = c->h_ctrl->cg_done != 0;
    }
    *iters = c->h_ctrl->cg_iters;
    *relres = c->h_ctrl->relres;
    if (!ok) {
        *lerr = 1;
        return FS_OK;
    }
    *lerr = 0;
    c->faces_valid = 0;
    c->launches++;
    k_phi_update<<<4 * 152, 256, 0, c->stream>>>(c->ph, c->ph_mi, c->xs, c->nx, c->ny, c->pitch, c->d_ctrl);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fs_cuda_check(c, e, "Poisson kernels");
    return FS_OK;
}
