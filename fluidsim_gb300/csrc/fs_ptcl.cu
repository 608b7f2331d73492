// fs_ptcl.cu -- the particle step on the GPU (plain FP64 path).
//
// One launch per RK-Merson stage does what the reference does in the cell
// loop of ptcl_step plus rk_step for every species (ptcl_lib.F90:44-57,
// ptclEqn ptcl_lib.F90:99-550, rk_step ptcl_props.F90:71-139):
//   * a CTA owns a 32x8 tile of interior nodes and stages the tile plus a
//     one-node halo of n_i, n_e, n_t (, n_m) and phi in shared memory;
//   * per node it evaluates the mean energy Te = nt/ne and the table
//     coefficients once (the reference re-evaluates them for every face);
//   * per face it evaluates the Scharfetter-Gummel flux once (get_Flux,
//     ptcl_props.F90:142-165) -- both nodes of a face see the same value,
//     as in the reference, where the two nodes compute identical expressions;
//     the electron and energy fluxes share one exponential because
//     mut/Dt = mue/De (ptcl_lib.F90:142-143);
//   * per node it forms the divergence, the sources and k_s, and applies the
//     Merson stage combination with the density floor; stage 5 also produces
//     per-CTA partial sums of the error norm, the dielectric relaxation time
//     t_m and the electrode-current rows of circ_step (circ_lib.F90:87-151).
// A one-CTA controller kernel then applies the PI step-size control of
// ptcl_lib.F90:59-95 on the device.
#include <cstdio>
#include <cstring>
#include <cuda_runtime.h>

#include "fs_fastmath.cuh"
#include "fs_internal.h"
#include "fs_sg.cuh"
#include "fs_wall.cuh"

// stage tiles: 32 x 8 nodes by default; 32 x 4 and 64 x 4 selectable per
// context (fs_set_stage_tile); the partial sums are sized for the most tiles
#define DEF_BX 32
#define DEF_BY 8

namespace {

struct StageArgs {
    PhysParams pp;
    MeshDev m;
    const double *tab;
    const double *nin[FS_MAX_SPECIES];
    const double *nbase[FS_MAX_SPECIES];
    double *nout[FS_MAX_SPECIES];
    const double *k1[FS_MAX_SPECIES];
    const double *k3[FS_MAX_SPECIES];
    const double *k4[FS_MAX_SPECIES];
    double *kout[FS_MAX_SPECIES];
    const double *ph;
    const double *fx_e, *fx_cl, *fx_cr, *fy_e, *fy_cl, *fy_cr;
    Ctrl *ctrl;
    double *part;     // [species][nblk] partial error sums
    double *rows;     // [2][ny+2] current rows
    double *sig_mi, *sig_pl, *ks;   // dielectric wall charge (nx+2 each) and its 5 stage slopes
    const double *sig_or;
    int rows_every_stage;   // the RC circuit needs the electrode current after every stage
    int stage;
    int nblk;
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

// get_Flux for q = -1 with (mue, De) and (5/3 mue, 5/3 De): one exponential
__device__ __forceinline__ void sg_elec(double E, double dh, double inv_dh, double mue, double De,
                                        double nel, double ner, double ntl, double ntr,
                                        double &fe, double &ft) {
    const double tol = 9.9999999600419720025e-13;
    const double f53 = 5.0 / 3.0;
    double mut = f53 * mue, Dt = f53 * De;
    double ve = -mue * E, vt = -mut * E;
    double arg = ve * dh / De;
    if (fabs(E) < tol) {
        fe = De * (nel - ner) * inv_dh;
        ft = Dt * (ntl - ntr) * inv_dh;
        return;
    }
    if (fabs(arg) < 1e-2) {   // Bernoulli form near a = 0
        double a2 = arg * arg, c2 = a2 * (1.0 / 12.0 - a2 / 720.0);
        fe = De * ((nel - ner) + 0.5 * arg * (nel + ner) + c2 * (nel - ner)) * inv_dh;
        ft = Dt * ((ntl - ntr) + 0.5 * arg * (ntl + ntr) + c2 * (ntl - ntr)) * inv_dh;
        return;
    }
    double ex;
    if (arg > 0) {
        ex = fs_exp(fmax(-arg, -100.0));
        double inv = 1.0 / (1.0 - ex);
        fe = ve * (nel - ner * ex) * inv;
        ft = vt * (ntl - ntr * ex) * inv;
    } else {
        ex = fs_exp(fmax(arg, -100.0));
        double inv = 1.0 / (1.0 - ex);
        fe = ve * (ner - nel * ex) * inv;
        ft = vt * (ntr - ntl * ex) * inv;
    }
}

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Dielectric wall face of column gi (type_y == 3 on the last row) and the
// column's surface-charge step: fs_wall.cuh.
template <int NS>
__device__ __forceinline__ double wall_face(const StageArgs &a, int gi, double te, double ni, double ne, double nt,
                                            double nm, double mue, double de, double &fi, double &fe, double &ft,
                                            double &fm, unsigned int &st) {
    const WallArgs w = {a.tab, a.sig_or, a.sig_mi, a.sig_pl, a.ks};
    return fs_wall_face<NS>(a.pp, w, a.m.dy[a.pp.ny], a.ctrl->dt, a.stage, gi, te, ni, ne, nt, nm, mue, de, fi, fe,
                            ft, fm, st);
}

// One RK stage on the tile (bx, by) of the grid (BX x BY nodes); blk is the
// tile's index among the grid's tiles (its slot in the error partials).
template <int NS, int TBX, int TBY>
__device__ __forceinline__ void stage_tile(const StageArgs &a, int bx, int by, int blk) {
    constexpr int BX = TBX, BY = TBY, NT = BX * BY, HX = BX + 2, HY = BY + 2;
    __shared__ double s_n[NS][HY][HX];
    __shared__ double s_ph[HY][HX];
    __shared__ double s_te[HY][HX];
    __shared__ double s_mue[HY][HX];
    __shared__ double s_de[HY][HX];
    __shared__ double s_w[BY][BX];
    __shared__ int s_k[BY][BX];
    __shared__ double s_fx[NS][BY][BX + 1];   // x-face left of tile column c
    __shared__ double s_fy[NS][BY + 1][BX];   // y-face below tile row r
    __shared__ double s_ex[BY][BX + 1];       // face field as used by the Joule term
    __shared__ double s_ey[BY + 1][BX];
    __shared__ double s_red[NS][NT / 32];
    __shared__ double s_tm[NT / 32];

    const PhysParams &pp = a.pp;
    const int nx = pp.nx, ny = pp.ny, P = pp.pitch;
    const int tid = threadIdx.x;
    const int gx0 = bx * BX + 1, gy0 = by * BY + 1;
    unsigned int st = 0;

    // phase 1: tile + halo of the stage state and phi
    for (int q = tid; q < HX * HY; q += NT) {
        int lx = q % HX, ly = q / HX;
        int gi = gx0 - 1 + lx, gj = gy0 - 1 + ly;
        bool in = gi <= nx + 1 && gj <= ny + 1;
        size_t o = (size_t)gj * P + gi;
#pragma unroll
        for (int s = 0; s < NS; s++) s_n[s][ly][lx] = in ? a.nin[s][o] : 0.0;
        s_ph[ly][lx] = in ? a.ph[o] : 0.0;
    }
    __syncthreads();
    // phase 2: mean energy and table coefficients of every interior node of the tile+halo
    for (int q = tid; q < HX * HY; q += NT) {
        int lx = q % HX, ly = q / HX;
        int gi = gx0 - 1 + lx, gj = gy0 - 1 + ly;
        double te = 0, mu = 0, de = 0;
        if (gi >= 1 && gi <= nx && gj >= 1 && gj <= ny) {
            double nte = s_n[2][ly][lx], nee = s_n[1][ly][lx];
            if ((nte >= 0.0) && (nee >= 0.0)) te = nte / nee;
            else { st |= FS_ST_NEG_DENSITY; te = 1e-8; }
            int k; double w;
            if (pp.fits) {
                k = 0; w = 0.0;
                mu = pp.fit.mue(te);
                de = pp.fit.De(te);
            } else {
                tab_index(pp, te, k, w);
                mu = tab_val(a.tab, k, w, 0);
                de = tab_val(a.tab, k, w, 1);
            }
            if (lx >= 1 && lx <= BX && ly >= 1 && ly <= BY) { s_k[ly - 1][lx - 1] = k; s_w[ly - 1][lx - 1] = w; }
        }
        s_te[ly][lx] = te; s_mue[ly][lx] = mu; s_de[ly][lx] = de;
    }
    __syncthreads();

    // phase 3a: x faces.  Face c of tile row r lies between nodes gi = gx0-1+c and gi+1.
    for (int q = tid; q < BY * (BX + 1); q += NT) {
        int c = q % (BX + 1), r = q / (BX + 1);
        int gi = gx0 - 1 + c, gj = gy0 + r;
        if (gj > ny || gi > nx) continue;
        int lx = c, ly = r + 1;   // left node in halo coordinates
        const size_t of = (size_t)gj * P + gi;
        double E = a.fx_e[of];
        double fi = 0, fe = 0, ft = 0, fm = 0, eu = E;
        int tl = gi >= 1 ? a.m.tx[(gj - 1) * nx + gi - 1] : 0;       // type of left node
        int tr = gi + 1 <= nx ? a.m.tx[(gj - 1) * nx + gi] : 0;      // type of right node
        if (gi == 0 && tr == -1) {           // vacuum face of the first node
            eu = 0.0;
        } else if (gi == nx && tl == 1) {    // vacuum face of the last node
            eu = 0.0;
        } else if ((gi == 0 && tr == -2) || (gi == nx && tl == 2)) {   // electrode face
            const bool left = gi == 0;
            const int lc = left ? lx + 1 : lx;     // the interior node
            double te = s_te[ly][lc], ni = s_n[0][ly][lc], ne = s_n[1][ly][lc], nt = s_n[2][ly][lc];
            double phg = left ? s_ph[ly][lx] : s_ph[ly][lx + 1];
            double aa = (phg > s_ph[ly][lc]) ? 1.0 : 0.0;
            double mue = s_mue[ly][lc], mut = (5.0 / 3.0) * mue;
            double ve = sqrt(pp.ve_coef * te) * pp.t0 / pp.x0;
            double sgn = left ? -1.0 : 1.0;
            fi = (1.0 - aa) * pp.mui * E * ni + sgn * (2.5e-1 * pp.vi * ni);
            fe = -(aa * mue * E * ne) + sgn * (2.5e-1 * ve * ne) - pp.gam * fi;
            ft = -(aa * mut * E * nt) + sgn * (1.0 / 3.0 * ve * nt) - pp.gam * te * fi;
            if (NS == 4) fm = sgn * (5e-1 * pp.vi * s_n[3][ly][lc]);
        } else {                              // Scharfetter-Gummel face
            double dh = a.m.dx[gi], idh = a.m.inv_dx[gi];
            double mue = 5e-1 * (s_mue[ly][lx] + s_mue[ly][lx + 1]);
            double De = 5e-1 * (s_de[ly][lx] + s_de[ly][lx + 1]);
            fi = a.fx_cl[of] * s_n[0][ly][lx] - a.fx_cr[of] * s_n[0][ly][lx + 1];
            sg_elec(E, dh, idh, mue, De, s_n[1][ly][lx], s_n[1][ly][lx + 1],
                    s_n[2][ly][lx], s_n[2][ly][lx + 1], fe, ft);
            if (NS == 4) fm = -pp.Dm * (s_n[3][ly][lx + 1] - s_n[3][ly][lx]) * idh;
            if (a.stage == 5 || a.rows_every_stage) {
                if (gi == 1 && a.m.dr_a[gj] != 0.0) a.rows[gj] = a.m.dr_a[gj] * (fi - fe);
                if (gi == nx - 1 && a.m.dr_c[gj] != 0.0) a.rows[(ny + 2) + gj] = a.m.dr_c[gj] * (fi - fe);
            }
        }
        s_fx[0][r][c] = fi; s_fx[1][r][c] = fe; s_fx[2][r][c] = ft;
        if (NS == 4) s_fx[3][r][c] = fm;
        s_ex[r][c] = eu;
    }
    __syncthreads();
    // phase 3b: y faces.  Face r of tile column c lies between gj = gy0-1+r and gj+1.
    for (int q = tid; q < (BY + 1) * BX; q += NT) {
        int c = q % BX, r = q / BX;
        int gi = gx0 + c, gj = gy0 - 1 + r;
        if (gi > nx || gj > ny) continue;
        int lx = c + 1, ly = r;     // lower node in halo coordinates
        const size_t of = (size_t)gj * P + gi;
        double E = a.fy_e[of];
        double fi = 0, fe = 0, ft = 0, fm = 0, eu = E;
        int tb = gj >= 1 ? a.m.ty[(gj - 1) * nx + gi - 1] : 0;
        int tt = gj + 1 <= ny ? a.m.ty[gj * nx + gi - 1] : 0;
        if (gj == 0 && tt == -1) {
            eu = 0.0;
        } else if (gj == 0 && tt == -2) {
            // ptclEqn has no lower y electrode: zero flux, face field kept (ptcl_lib.F90:287-367)
        } else if (gj == ny && tb == 1) {
            eu = 0.0;
        } else if (gj == ny && tb == 3) {
            const int lc = ly;
            eu = wall_face<NS>(a, gi, s_te[lc][lx], s_n[0][lc][lx], s_n[1][lc][lx], s_n[2][lc][lx],
                               NS == 4 ? s_n[3][lc][lx] : 0.0, s_mue[lc][lx], s_de[lc][lx], fi, fe, ft, fm, st);
        } else if (gj == ny && tb == 2) {
            const bool low = false;
            const int lc = low ? ly + 1 : ly;
            double te = s_te[lc][lx], ni = s_n[0][lc][lx], ne = s_n[1][lc][lx], nt = s_n[2][lc][lx];
            double phg = low ? s_ph[ly][lx] : s_ph[ly + 1][lx];
            double aa = (phg > s_ph[lc][lx]) ? 1.0 : 0.0;
            double mue = s_mue[lc][lx], mut = (5.0 / 3.0) * mue;
            double ve = sqrt(pp.ve_coef * te) * pp.t0 / pp.x0;
            double sgn = low ? -1.0 : 1.0;
            fi = (1.0 - aa) * pp.mui * E * ni + sgn * (2.5e-1 * pp.vi * ni);
            // the reference's upper y electrode takes gamma times the x-direction
            // ion flux of the node's upper x face (ptcl_lib.F90:427-433)
            double fix = low ? fi : s_fx[0][lc - 1][lx];
            fe = -(aa * mue * E * ne) + sgn * (2.5e-1 * ve * ne) - pp.gam * fix;
            ft = -(aa * mut * E * nt) + sgn * (1.0 / 3.0 * ve * nt) - pp.gam * te * fix;
            if (NS == 4) fm = sgn * (5e-1 * pp.vi * s_n[3][lc][lx]);
        } else {
            double dh = a.m.dy[gj], idh = a.m.inv_dy[gj];
            double mue = 5e-1 * (s_mue[ly][lx] + s_mue[ly + 1][lx]);
            double De = 5e-1 * (s_de[ly][lx] + s_de[ly + 1][lx]);
            fi = a.fy_cl[of] * s_n[0][ly][lx] - a.fy_cr[of] * s_n[0][ly + 1][lx];
            sg_elec(E, dh, idh, mue, De, s_n[1][ly][lx], s_n[1][ly + 1][lx],
                    s_n[2][ly][lx], s_n[2][ly + 1][lx], fe, ft);
            if (NS == 4) fm = -pp.Dm * (s_n[3][ly + 1][lx] - s_n[3][ly][lx]) * idh;
        }
        s_fy[0][r][c] = fi; s_fy[1][r][c] = fe; s_fy[2][r][c] = ft;
        if (NS == 4) s_fy[3][r][c] = fm;
        s_ey[r][c] = eu;
    }
    __syncthreads();

    // phase 4: one node per thread
    const int lx = tid % BX, ly = tid / BX;
    const int gi = gx0 + lx, gj = gy0 + ly;
    double qerr[NS];
#pragma unroll
    for (int s = 0; s < NS; s++) qerr[s] = 0.0;
    double tm = 1e300;
    if (gi <= nx && gj <= ny) {
        const size_t o = (size_t)gj * P + gi;
        const int hx = lx + 1, hy = ly + 1;
        const double te = s_te[hy][hx];
        const double ni = s_n[0][hy][hx], ne = s_n[1][hy][hx];
        const double nm = NS == 4 ? s_n[3][hy][hx] : 0.0;
        const int kk = s_k[ly][lx];
        const double w = s_w[ly][lx];
        const bool fits = pp.fits;
        const double k_ir = fits ? pp.fit.k_ir_fit(te) : tab_val(a.tab, kk, w, 2);
        const double k_ex = fits ? pp.fit.k_ex(te) : tab_val(a.tab, kk, w, 3);
        const double nu = fits ? pp.fit.nu(te) : tab_val(a.tab, kk, w, 4);
        const double beta = fits ? pp.fit.beta(te) : tab_val(a.tab, kk, w, 5);
        const double idlx = a.m.inv_dlx[gi - 1], idly = a.m.inv_dly[gj - 1];
        double dfdx[NS], dfdy[NS];
        if (pp.cyl) {
            double r0 = a.m.r[gj], rp = (a.m.r[gj + 1] + r0), rm = (r0 + a.m.r[gj - 1]);
#pragma unroll
            for (int s = 0; s < NS; s++) {
                dfdx[s] = (s_fx[s][ly][lx + 1] - s_fx[s][ly][lx]) * idlx;
                dfdy[s] = (s_fy[s][ly + 1][lx] * rp / 2.0 - s_fy[s][ly][lx] * rm / 2.0) * idly / r0;
            }
        } else {
#pragma unroll
            for (int s = 0; s < NS; s++) {
                dfdx[s] = (s_fx[s][ly][lx + 1] - s_fx[s][ly][lx]) * idlx;
                dfdy[s] = (s_fy[s][ly + 1][lx] - s_fy[s][ly][lx]) * idly;
            }
        }
        const double fex = (s_fx[1][ly][lx + 1] + s_fx[1][ly][lx]) * 0.5;
        const double exa = (s_ex[ly][lx] + s_ex[ly][lx + 1]) * 0.5;
        const double fey = (s_fy[1][ly + 1][lx] + s_fy[1][ly][lx]) * 0.5;
        const double eya = (s_ey[ly][lx] + s_ey[ly + 1][lx]) * 0.5;
        double term_sie = k_ir * pp.ninf * ne - beta * ni * ne;
        double k_si = 0, k_sc = 0;
        if (NS == 4) {
            k_sc = fits ? pp.fit.k_sc(te) : tab_val(a.tab, kk, w, 6);
            k_si = fits ? pp.fit.k_si(te) : tab_val(a.tab, kk, w, 7);
            term_sie = term_sie + k_si * nm * ne + pp.k_mp * (nm * nm);
        }
        const double term_st1 = -(fex * exa + fey * eya);
        // Tg kb / e / ph0 folded on the host (same operations, same value); the
        // divisions by mi and by 1.5 as products with reciprocals (<= 1 ulp each)
        const double term_st2 = -(ne * nu * pp.me * pp.inv_mi * (te * (2.0 / 3.0) - pp.tg_term));
        double term_st3 = -(pp.h_ir * k_ir * pp.ninf * ne) - pp.h_si * k_si * nm * ne
                        - pp.h_ex * k_ex * pp.ninf * ne;
        double kv[NS];
        kv[0] = -dfdx[0] - dfdy[0] + term_sie;
        kv[1] = -dfdx[1] - dfdy[1] + term_sie;
        kv[2] = -dfdx[2] - dfdy[2] + term_st1 + term_st2 + term_st3;
        if (NS == 4) {
            double term_sm = k_ex * pp.ninf * ne - k_si * nm * ne - k_sc * nm * ne - pp.k_r * nm * ne
                           - 2.0 * pp.k_mp * (nm * nm) - pp.k_2q * pp.ninf * nm
                           - pp.k_3q * (pp.ninf * pp.ninf) * nm;
            kv[3] = -dfdx[3] - dfdy[3] + term_sm;
        }
        const double dt = a.ctrl->dt;
        const int stg = a.stage;
#pragma unroll
        for (int s = 0; s < NS; s++) {
            if (isnan(kv[s])) st |= FS_ST_NAN;
            if (a.kout[s]) a.kout[s][o] = kv[s];
            const double n3 = a.nbase[s][o];
            double v;
            if (stg == 1) v = n3 + kv[s] * dt * (1.0 / 3.0);
            else if (stg == 2) v = n3 + dt * (a.k1[s][o] + kv[s]) * (1.0 / 6.0);
            else if (stg == 3) v = n3 + dt * (a.k1[s][o] + kv[s] * 3.0) * 0.125;
            else if (stg == 4) v = n3 + dt * (a.k1[s][o] - a.k3[s][o] * 3.0 + kv[s] * 4.0) * 0.5;
            else {
                const double k1 = a.k1[s][o], k3 = a.k3[s][o], k4 = a.k4[s][o];
                v = n3 + dt * (k1 + k4 * 4.0 + kv[s]) * (1.0 / 6.0);
                double err = fabs(dt * (k1 * (2.0 / 30.0) - k3 * (3.0 / 10.0) + k4 * (4.0 / 15.0)
                                        - kv[s] * (1.0 / 30.0)));
                double qq = err / (pp.abs_tol + pp.rel_tol * fabs(n3));
                qerr[s] = qq * qq;
            }
            a.nout[s][o] = fmax(v, pp.nmin[s]);
        }
        if (stg == 5) {
            // mue(2) as the reference leaves it when t_m is evaluated (ptcl_lib.F90:527)
            const int ty = a.m.ty[(gj - 1) * nx + gi - 1], tx = a.m.tx[(gj - 1) * nx + gi - 1];
            double mue2;
            if (ty == 0 || ty < 0) mue2 = 5e-1 * (s_mue[hy][hx] + s_mue[hy + 1][hx]);
            else if (ty == 1 && (tx == 0 || tx < 0)) mue2 = 5e-1 * (s_mue[hy][hx] + s_mue[hy][hx + 1]);
            else mue2 = s_mue[hy][hx];
            tm = 1.0 / (mue2 * ne + pp.mui * ni);
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
            a.part[(size_t)tid * a.nblk + blk] = v;
        }
        if (tid == 0) {
            double m = s_tm[0];
            for (int wv = 1; wv < NT / 32; wv++) m = fmin(m, s_tm[wv]);
            if (m > 0.0 && m < 1e300)
                atomicMin((unsigned long long *)&a.ctrl->t_m, (unsigned long long)__double_as_longlong(m));
        }
    }
}

template <int NS, int TBX, int TBY>
__global__ void __launch_bounds__(TBX * TBY, 2) k_stage(const StageArgs a) {
    stage_tile<NS, TBX, TBY>(a, blockIdx.x, blockIdx.y, blockIdx.y * gridDim.x + blockIdx.x);
}

// Ion face coefficients while phi is frozen.  get_Flux for q = +1
// (ptcl_props.F90:142-165): mui and Di are constants, so on a face the flux is
// linear in the two densities, flux = cl n_left - cr n_right, with the
// Bernoulli form near a = 0 where 1 - exp(-a) cancels and the exponent clamped
// at -100 as get_Flux clamps it.  dFdPh for ions (lapl_lib.F90:611-636) is
// linear too, dF/dv = dl n1 + dr n2, with its own small-|a| series.  The two
// share the Bernoulli argument, so the exponential and 1 / (1 - exp(-|a|))
// are formed once.
__device__ __forceinline__ void ion_face(const PhysParams &pp, double E, double dh, double inv_dh, double &cl,
                                         double &cr, double &dl, double &dr) {
    const double tol = 9.9999999600419720025e-13;   // REAL(4) 1e-12
    const double v = pp.mui * E;
    const double a = v * dh / pp.Di, aa = fabs(a);
    double ex = 0.0, inv = 0.0;
    if (aa >= 1e-2) {
        ex = fs_exp(-aa);
        inv = 1.0 / (1.0 - ex);
    }
    if (fabs(E) < tol) {
        cl = cr = pp.Di * inv_dh;
    } else if (aa < 1e-2) {
        double a2 = a * a, c2 = a2 * (1.0 / 12.0 - a2 / 720.0), d = pp.Di * inv_dh;
        cl = d * (1.0 + 0.5 * a + c2);
        cr = d * (1.0 - 0.5 * a + c2);
    } else {
        double exc = ex, ic = inv;
        if (aa > 100.0) {
            exc = exp(-100.0);
            ic = 1.0 / (1.0 - exc);
        }
        if (a > 0) {
            cl = v * ic;
            cr = v * exc * ic;
        } else {
            cl = -(v * exc * ic);
            cr = -(v * ic);
        }
    }
    if (fabs(v) < 1e-12) {
        dl = dr = 0.0;
    } else if (aa < 0.05) {
        double a2 = a * a, sres = a * (1.0 / 6.0 - a2 * (1.0 / 180.0 - a2 / 5040.0));
        dl = 0.5 + sres;
        dr = 0.5 - sres;
    } else {
        const double t = a * ex * inv * inv;
        if (a > 0) {
            dl = inv - t;
            dr = -(ex * inv) + t;
        } else {
            dl = -(ex * inv) - t;
            dr = inv + t;
        }
    }
}

struct FaceArgs {
    double *fx_e, *fx_cl, *fx_cr, *fx_dl, *fx_dr, *fy_e, *fy_cl, *fy_cr, *fy_dl, *fy_dr;
};

// Face data while phi is frozen: E = -(phi_R - phi_L)/h as ptclEqn forms it
// (ptcl_lib.F90:112-121,286-298), the ion flux coefficients and the ion dFdPh
// coefficients.  x face east of (gi,gj) for gi = 0..nx, y face north of it for gj = 0..ny.
__global__ void k_faces(const PhysParams pp, const MeshDev m, const double *ph, const FaceArgs f) {
    const int gi = blockIdx.x * blockDim.x + threadIdx.x, gj = blockIdx.y * blockDim.y + threadIdx.y;
    const int nx = pp.nx, ny = pp.ny, P = pp.pitch;
    if (gi > nx || gj > ny) return;
    const size_t o = (size_t)gj * P + gi;
    if (gj >= 1) {
        double E = -(ph[o + 1] - ph[o]) * m.inv_dx[gi];   // reciprocal product (<= 1 ulp from the division)
        double cl, cr, dl, dr;
        ion_face(pp, E, m.dx[gi], m.inv_dx[gi], cl, cr, dl, dr);
        f.fx_e[o] = E; f.fx_cl[o] = cl; f.fx_cr[o] = cr; f.fx_dl[o] = dl; f.fx_dr[o] = dr;
    }
    if (gi >= 1) {
        double E = -(ph[o + P] - ph[o]) * m.inv_dy[gj];
        double cl, cr, dl, dr;
        ion_face(pp, E, m.dy[gj], m.inv_dy[gj], cl, cr, dl, dr);
        f.fy_e[o] = E; f.fy_cl[o] = cl; f.fy_cr[o] = cr; f.fy_dl[o] = dl; f.fy_dr[o] = dr;
    }
}

// circ_step ghost potentials (circ_lib.F90:178-198): DC, so Vd_mi = Vd_pl = Vsrc.
// The fields of the two electrode faces of the row follow the new ghosts.
__global__ void k_circ_ghost(double *ph, const int8_t *tx, const double *r, const double *dx,
                             double *fx_e, int nx, int ny, int P, double ew, double vd) {
    int gj = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (gj > ny) return;
    const size_t o = (size_t)gj * P;
    if (r[gj] <= ew) {
        if (tx[(gj - 1) * nx + 0] == -2) {
            ph[o + 0] = vd / 2.0;
            fx_e[o + 0] = -(ph[o + 1] - ph[o + 0]) / dx[0];
        }
        if (tx[(gj - 1) * nx + nx - 1] == 2) {
            ph[o + nx + 1] = vd / (-2.0);
            fx_e[o + nx] = -(ph[o + nx + 1] - ph[o + nx]) / dx[nx];
        }
    }
}

// RC circuit of circ_step for the AC source (circ_lib.F90:156-198), after each
// stage: Idc from the stage's current rows (fixed-order sum), the slope
// kv(stage) = -(Idc - (Vsrc - Vd_mi)/Res)/Cap, the Merson combination into
// Vd_mi (stages 1-4) or Vd_pl (stage 5), then the ghost potentials +-Vd/2 of
// the electrode rows and the fields of their electrode faces.  vd_mi0 is
// Vd_mi at the start of the attempt (a host value); later stages read the
// device's.
__global__ void __launch_bounds__(256) k_circuit(Ctrl *c, const double *rows, double *ph, double *fx_e,
                                                 float *fx_e32, const int8_t *tx, const double *r, const double *dx, int nx,
                                                 int ny, int P, double ew, int stage, double vsrc, double vd_or,
                                                 double vd_mi0, double res, double cap) {
    __shared__ double s[256];
    __shared__ double s_vd;
    const int t = threadIdx.x;
    double rc = 0.0;
    for (int j = 1 + t; j <= ny; j += 256) rc += rows[(ny + 2) + j];
    s[t] = rc;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (t < w) s[t] += s[t + w];
        __syncthreads();
    }
    if (t == 0) {
        const double idc = s[0], dt = c->dt;
        const double vd_mi = stage == 1 ? vd_mi0 : c->vd_mi;
        const double kv = -(idc - (vsrc - vd_mi) / res) / cap;
        c->kv[stage] = kv;
        const double *k = c->kv;
        double v;
        if (stage == 1) v = vd_or + dt * k[1] / 3.0;
        else if (stage == 2) v = vd_or + dt * (k[1] + k[2]) / 6.0;
        else if (stage == 3) v = vd_or + dt * (k[1] + k[3] * 3.0) / 8.0;
        else if (stage == 4) v = vd_or + dt * (k[1] - k[3] * 3.0 + k[4] * 4.0) / 2.0;
        else v = vd_or + dt * (k[1] + k[4] * 4.0 + k[5]) / 6.0;
        if (stage == 5) c->vd_pl = v;
        else c->vd_mi = v;
        s_vd = v;
    }
    __syncthreads();
    const double vd = s_vd;
    for (int gj = 1 + t; gj <= ny; gj += 256) {
        const size_t o = (size_t)gj * P;
        if (r[gj] <= ew) {
            if (tx[(gj - 1) * nx + 0] == -2) {
                ph[o + 0] = vd / 2.0;
                fx_e[o + 0] = -(ph[o + 1] - ph[o + 0]) / dx[0];
                if (fx_e32) fx_e32[o + 0] = (float)fx_e[o + 0];
            }
            if (tx[(gj - 1) * nx + nx - 1] == 2) {
                ph[o + nx + 1] = vd / (-2.0);
                fx_e[o + nx] = -(ph[o + nx + 1] - ph[o + nx]) / dx[nx];
                if (fx_e32) fx_e32[o + nx] = (float)fx_e[o + nx];
            }
        }
    }
}

// PI controller of ptcl_lib.F90:59-95 plus the current sums of circ_step.
// All sums are fixed-order: strided per-thread partials, then a fixed tree.
// One CTA of 256 threads.
__device__ __forceinline__ void controller_body(Ctrl *c, const double *part, int nblk, int ns, const double *rows,
                                                int ny, int adaptive, double dt_min) {
    __shared__ double s[FS_MAX_SPECIES + 2][256];
    const int t = threadIdx.x;
    for (int sp = 0; sp < ns; sp++) {
        double v = 0.0;
        for (int b = t; b < nblk; b += 256) v += part[(size_t)sp * nblk + b];
        s[sp][t] = v;
    }
    double ra = 0.0, rc = 0.0;
    for (int j = 1 + t; j <= ny; j += 256) { ra += rows[j]; rc += rows[(ny + 2) + j]; }
    s[FS_MAX_SPECIES][t] = ra;
    s[FS_MAX_SPECIES + 1][t] = rc;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (t < w) {
            for (int sp = 0; sp < ns; sp++) s[sp][t] += s[sp][t + w];
            s[FS_MAX_SPECIES][t] += s[FS_MAX_SPECIES][t + w];
            s[FS_MAX_SPECIES + 1][t] += s[FS_MAX_SPECIES + 1][t + w];
        }
        __syncthreads();
    }
    if (t != 0) return;
    // species order of the reference's sum: ni, ne, nm, nt
    double e_ni = s[0][0], e_ne = s[1][0], e_nt = s[2][0], e_nm = ns == 4 ? s[3][0] : 0.0;
    double err_cur = sqrt(e_ni + e_ne + e_nm + e_nt);
    c->err_cur = err_cur;
    c->dt_step = c->dt;
    c->ida = s[FS_MAX_SPECIES][0];
    c->idc = s[FS_MAX_SPECIES + 1][0];
    c->rejected = 0;
    if (!adaptive) return;
    double scfac = 8e-1 * pow(err_cur, -7e-1 / 4.0) * pow(c->err_prev, 4e-1 / 4.0);
    scfac = fmin(2.5, fmax(3e-1, scfac));
    c->scfac = scfac;
    c->dt = scfac * c->dt;
    if (c->dt <= dt_min) { c->min_dt = 1; return; }
    if (err_cur <= 1.0) c->err_prev = err_cur;
    else c->rejected = 1;
}

__global__ void __launch_bounds__(256) k_controller(Ctrl *c, const double *part, int nblk, int ns,
                                                    const double *rows, int ny, int adaptive, double dt_min) {
    controller_body(c, part, nblk, ns, rows, ny, adaptive, dt_min);
}

__global__ void k_reset_step(Ctrl *c, double *rows, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) { c->t_m = 1e9; c->status = 0; c->rejected = 0; c->min_dt = 0; }
    if (i < n) rows[i] = 0.0;
}

// ---- many discharges in one launch per RK stage (fs_ptcl_batch_attempt)
// Tile q of the batch: x = discharge, (y, z) = tile coordinates in its grid,
// w = the tile's index among that grid's tiles.
template <int NS, int TBX, int TBY>
__global__ void __launch_bounds__(TBX * TBY, 2) k_stage_batch(const StageArgs *args, const int4 *tiles,
                                                              const int *act) {
    const int4 t = tiles[blockIdx.x];
    if (!act[t.x]) return;   // uniform over the CTA
    stage_tile<NS, TBX, TBY>(args[t.x], t.y, t.z, t.w);
}

struct BatchCtl {
    Ctrl *ctrl;
    const double *part, *rows;
    double *rows_w;
    int nblk, ns, ny, adaptive;
    double dt_min;
    // circ_step ghosts (DC)
    double *ph, *fx_e;
    const int8_t *tx;
    const double *r, *dx;
    int nx, P;
    double ew, vd;
};

// start of a step of discharge b (fresh[b]): t_m, status and current rows
__global__ void __launch_bounds__(256) k_reset_batch(const BatchCtl *bc, const int *act, const int *fresh) {
    const int b = blockIdx.x;
    if (!act[b] || !fresh[b]) return;
    const BatchCtl &q = bc[b];
    if (threadIdx.x == 0) { q.ctrl->t_m = 1e9; q.ctrl->status = 0; q.ctrl->rejected = 0; q.ctrl->min_dt = 0; }
    for (int i = threadIdx.x; i < 2 * (q.ny + 2); i += blockDim.x) q.rows_w[i] = 0.0;
}

__global__ void __launch_bounds__(128) k_circ_ghost_batch(const BatchCtl *bc, const int *act) {
    const int b = blockIdx.x;
    if (!act[b]) return;
    const BatchCtl &q = bc[b];
    for (int gj = 1 + threadIdx.x; gj <= q.ny; gj += blockDim.x) {
        const size_t o = (size_t)gj * q.P;
        if (q.r[gj] <= q.ew) {
            if (q.tx[(gj - 1) * q.nx + 0] == -2) {
                q.ph[o + 0] = q.vd / 2.0;
                q.fx_e[o + 0] = -(q.ph[o + 1] - q.ph[o + 0]) / q.dx[0];
            }
            if (q.tx[(gj - 1) * q.nx + q.nx - 1] == 2) {
                q.ph[o + q.nx + 1] = q.vd / (-2.0);
                q.fx_e[o + q.nx] = -(q.ph[o + q.nx + 1] - q.ph[o + q.nx]) / q.dx[q.nx];
            }
        }
    }
}

// the controller of every discharge in the batch (one CTA each), then its
// control block copied into the batch's gathered array
__global__ void __launch_bounds__(256) k_controller_batch(const BatchCtl *bc, const int *act, Ctrl *gathered) {
    const int b = blockIdx.x;
    if (!act[b]) return;
    const BatchCtl &q = bc[b];
    controller_body(q.ctrl, q.part, q.nblk, q.ns, q.rows, q.ny, q.adaptive, q.dt_min);
    __syncthreads();
    __threadfence_block();
    const uint64_t *src = reinterpret_cast<const uint64_t *>(q.ctrl);
    uint64_t *dst = reinterpret_cast<uint64_t *>(gathered + b);
    for (int i = threadIdx.x; i < (int)(sizeof(Ctrl) / 8); i += blockDim.x) dst[i] = src[i];
}

}  // namespace

void fs_faces_update(fs_ctx *c) {
    if (c->faces_valid) return;
    dim3 b(32, 8), g((c->nx + 1 + 31) / 32, (c->ny + 1 + 7) / 8);
    FaceArgs f = {c->fx_e, c->fx_cl, c->fx_cr, c->fx_dl, c->fx_dr, c->fy_e, c->fy_cl, c->fy_cr, c->fy_dl, c->fy_dr};
    fs_prof_begin(c, PROF_OTHER);
    k_faces<<<g, b, 0, c->stream>>>(c->pp, c->mesh, c->ph, f);
    fs_prof_end(c);
    c->faces_valid = 1;
}

int fs_sig_copy(fs_ctx *c, int dst, int src) {
    cudaError_t e = cudaMemcpyAsync(fs_sig(c, dst), fs_sig(c, src), sizeof(double) * (c->nx + 2),
                                    cudaMemcpyDeviceToDevice, c->stream);
    return e == cudaSuccess ? FS_OK : fs_cuda_check(c, e, "surface charge copy");
}

static int stage_tiles(const fs_ctx *c, int bx, int by) { return ((c->nx + bx - 1) / bx) * ((c->ny + by - 1) / by); }

int fs_ptcl_alloc(fs_ctx *c) {
    c->stage_bx = DEF_BX;
    c->stage_by = DEF_BY;
    c->nblk_stage = stage_tiles(c, c->stage_bx, c->stage_by);
    const int nblk_max = stage_tiles(c, 32, 4);   // the shape with the most tiles
    cudaError_t e = cudaMalloc(&c->d_sig, sizeof(double) * 8 * (c->nx + 2));
    if (e == cudaSuccess) e = cudaMemset(c->d_sig, 0, sizeof(double) * 8 * (c->nx + 2));
    if (e != cudaSuccess) return fs_cuda_check(c, e, "cudaMalloc surface charge");
    for (int q = 0; q < 3; q++) c->sig_slot[q] = q;
    e = cudaMalloc(&c->d_part, sizeof(double) * FS_MAX_SPECIES * nblk_max);
    if (e != cudaSuccess) return fs_cuda_check(c, e, "cudaMalloc partials");
    e = cudaMalloc(&c->d_rows, sizeof(double) * 2 * (c->ny + 2));
    if (e != cudaSuccess) return fs_cuda_check(c, e, "cudaMalloc rows");
    double **faces[] = {&c->fx_e, &c->fx_cl, &c->fx_cr, &c->fy_e, &c->fy_cl, &c->fy_cr,
                        &c->fx_dl, &c->fx_dr, &c->fy_dl, &c->fy_dr};
    for (double **f : faces) {
        e = cudaMalloc(f, sizeof(double) * c->field_elems);
        if (e == cudaSuccess) e = cudaMemset(*f, 0, sizeof(double) * c->field_elems);
        if (e != cudaSuccess) return fs_cuda_check(c, e, "cudaMalloc faces");
    }
    return cudaMemset(c->d_rows, 0, sizeof(double) * 2 * (c->ny + 2)) == cudaSuccess ? FS_OK
                                                                                   : FS_ERR_CUDA;
}

int fs_set_stage_tile_impl(fs_ctx *c, int bx, int by) {
    if (!((bx == 32 && (by == 8 || by == 4)) || (bx == 64 && by == 4)))
        return fs_set_error(c, FS_ERR_INVALID, "stage tile %dx%d not one of 32x8, 32x4, 64x4", bx, by);
    if (bx == 64 && c->cfg.nspecies == 4)   // its shared memory would exceed 48 KB
        return fs_set_error(c, FS_ERR_UNSUPPORTED, "the 64x4 stage tile takes 3 species");
    c->stage_bx = bx;
    c->stage_by = by;
    c->nblk_stage = stage_tiles(c, bx, by);
    return FS_OK;
}

template <int NS>
static void launch_stage_ns(fs_ctx *c, StageArgs &a) {
    const dim3 grid((c->nx + c->stage_bx - 1) / c->stage_bx, (c->ny + c->stage_by - 1) / c->stage_by);
    if constexpr (NS == 3) {
        if (c->stage_bx == 64) { k_stage<NS, 64, 4><<<grid, 256, 0, c->stream>>>(a); return; }
    }
    if (c->stage_by == 4) k_stage<NS, 32, 4><<<grid, 128, 0, c->stream>>>(a);
    else k_stage<NS, 32, 8><<<grid, 256, 0, c->stream>>>(a);
}

static void launch_stage(fs_ctx *c, StageArgs &a) {
    if (c->cfg.nspecies == 4) launch_stage_ns<4>(c, a);
    else launch_stage_ns<3>(c, a);
}

// Start of a particle step: t_m, status and the current rows reset on the device.
void fs_ptcl_reset(fs_ctx *c) {
    c->launches++;
    k_reset_step<<<(2 * (c->ny + 2) + 255) / 256, 256, 0, c->stream>>>(c->d_ctrl, c->d_rows, 2 * (c->ny + 2));
}

// End of one five-stage attempt: the controller, then the host reads the
// control block and turns its status bits into errors.
int fs_ptcl_control(fs_ctx *c) {
    c->launches++;
    k_controller<<<1, 256, 0, c->stream>>>(c->d_ctrl, c->d_part, c->nblk_stage, c->cfg.nspecies, c->d_rows,
                                           c->ny, c->cfg.adaptive, c->cfg.dt_min);
    int rc = fs_sync_ctrl(c);
    if (rc) return rc;
    const Ctrl &h = *c->h_ctrl;
    if (h.status & FS_ST_NEG_DENSITY) return fs_set_error(c, FS_ERR_NEG_DENSITY, "negative density in get_Te");
    if (h.status & FS_ST_NAN) return fs_set_error(c, FS_ERR_NAN, "NaN in particle right-hand side");
    if (h.min_dt) return fs_set_error(c, FS_ERR_MIN_DT, "minimum timestep reached");
    return FS_OK;
}

// The RC circuit after stage stg (k_circuit); fx_e32, when not null, also
// receives the electrode faces' fields in FP32 (the mixed path's face field).
void fs_circuit_launch(fs_ctx *c, int stg, float *fx_e32) {
    c->launches++;
    k_circuit<<<1, 256, 0, c->stream>>>(c->d_ctrl, c->d_rows, c->ph, c->fx_e, fx_e32, c->mesh.tx, c->mesh.r,
                                        c->mesh.dx, c->nx, c->ny, c->pitch, c->cfg.ew, stg, c->Vsrc, c->Vd_or,
                                        c->Vd_mi, c->cfg.res, c->k.cap);
}

// ptcl_step: five stages, restart on rejection (ptcl_lib.F90:32-97).
int fs_ptcl_step_impl(fs_ctx *c, int *attempts_out) {
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
    fs_faces_update(c);
    for (;;) {
        attempts++;
        StageArgs a;
        memset(&a, 0, sizeof(a));
        a.pp = c->pp;
        a.m = c->mesh;
        a.tab = c->d_tab;
        a.ph = c->ph;
        a.fx_e = c->fx_e; a.fx_cl = c->fx_cl; a.fx_cr = c->fx_cr;
        a.fy_e = c->fy_e; a.fy_cl = c->fy_cl; a.fy_cr = c->fy_cr;
        a.ctrl = c->d_ctrl;
        a.part = c->d_part;
        a.rows = c->d_rows;
        a.sig_pl = fs_sig(c, 0);
        a.sig_mi = fs_sig(c, 1);
        a.sig_or = fs_sig(c, 2);
        a.ks = fs_sig_ks(c);
        a.rows_every_stage = rc_circuit;
        a.nblk = c->nblk_stage;
        const int ins[5] = {in1, SA, SB, SA, SB};
        const int outs[5] = {SA, SB, SA, SB, OUT};
        for (int stg = 1; stg <= 5; stg++) {
            a.stage = stg;
            for (int s = 0; s < ns; s++) {
                SpeciesBufs &b = c->sp[s];
                a.nin[s] = b.buf[ins[stg - 1]];
                a.nbase[s] = b.buf[L3];
                a.nout[s] = b.buf[outs[stg - 1]];
                a.k1[s] = b.k[0];
                a.k3[s] = b.k[1];
                a.k4[s] = b.k[2];
                a.kout[s] = stg == 1 ? b.k[0] : stg == 3 ? b.k[1] : stg == 4 ? b.k[2] : nullptr;
            }
            fs_prof_begin(c, PROF_STAGE);
            launch_stage(c, a);
            fs_prof_end(c);
            if (rc_circuit) {
                fs_circuit_launch(c, stg, nullptr);
            } else if (stg == 1 && ++c->launches) {
                k_circ_ghost<<<(c->ny + 127) / 128, 128, 0, c->stream>>>(
                    c->ph, c->mesh.tx, c->mesh.r, c->mesh.dx, c->fx_e, c->nx, c->ny, c->pitch, c->cfg.ew,
                    c->Vsrc);
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
        in1 = L3;   // n(:,:,1) = n(:,:,2) = n(:,:,3): restart from the base state
        if (attempts > 100000) return fs_set_error(c, FS_ERR_MIN_DT, "RK restart limit");
    }
    c->lev[0] = OUT;
    c->lev[1] = SB;
    c->dt = c->h_ctrl->dt;
    c->st.attempts += attempts;
    if (attempts_out) *attempts_out = attempts;
    return FS_OK;
}

// ---------------------------------------------------------------- batches
// group of a stage tile shape in a batch: 0 = 32x8, 1 = 32x4, 2 = 64x4
static int shape_group(int bx, int by) { return bx == 64 ? 2 : by == 4 ? 1 : 0; }

// Work buffers of fs_ptcl_batch_attempt for one set of contexts.
struct FsBatchWork {
    int n = 0, device = 0;
    // the discharges grouped by stage tile shape: one launch per group and stage
    static constexpr int kShapes = 3;
    int ntiles[kShapes] = {0, 0, 0};
    int4 *d_tiles_g[kShapes] = {nullptr, nullptr, nullptr};
    std::vector<int> nblk;   // tiles of each discharge (its own tile shape)
    cudaStream_t st = nullptr;
    StageArgs *h_args = nullptr, *d_args = nullptr;   // [5][n]
    BatchCtl *h_ctl = nullptr, *d_ctl = nullptr;
    int *h_flags = nullptr, *d_flags = nullptr;       // act[n], fresh[n]
    Ctrl *h_gather = nullptr, *d_gather = nullptr;
    std::vector<cudaEvent_t> ev;
    std::vector<int> in1, attempts;
};

void fs_batch_work_free(FsBatchWork *w) {
    if (!w) return;
    cudaFreeHost(w->h_args); cudaFree(w->d_args);
    cudaFreeHost(w->h_ctl); cudaFree(w->d_ctl);
    cudaFreeHost(w->h_flags); cudaFree(w->d_flags);
    for (int g = 0; g < FsBatchWork::kShapes; g++) cudaFree(w->d_tiles_g[g]);
    cudaFreeHost(w->h_gather); cudaFree(w->d_gather);
    for (cudaEvent_t e : w->ev) cudaEventDestroy(e);
    if (w->st) cudaStreamDestroy(w->st);
    delete w;
}

int fs_batch_work_alloc(fs_ctx **cs, int n, FsBatchWork **out) {
    FsBatchWork *w = new FsBatchWork();
    w->n = n;
    w->device = cs[0]->device;
    std::vector<int4> tiles[FsBatchWork::kShapes];
    w->nblk.resize(n);
    for (int b = 0; b < n; b++) {
        const fs_ctx *c = cs[b];
        const int bx = c->stage_bx, by = c->stage_by, g = shape_group(bx, by);
        const int gx = (c->nx + bx - 1) / bx, gy = (c->ny + by - 1) / by;
        w->nblk[b] = gx * gy;
        for (int y = 0; y < gy; y++)
            for (int x = 0; x < gx; x++) tiles[g].push_back(make_int4(b, x, y, y * gx + x));
    }
    w->ev.resize(n, nullptr);
    w->in1.assign(n, 0);
    w->attempts.assign(n, 0);
    cudaError_t e = cudaStreamCreateWithFlags(&w->st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMallocHost(&w->h_args, sizeof(StageArgs) * 5 * n);
    if (e == cudaSuccess) e = cudaMalloc(&w->d_args, sizeof(StageArgs) * 5 * n);
    if (e == cudaSuccess) e = cudaMallocHost(&w->h_ctl, sizeof(BatchCtl) * n);
    if (e == cudaSuccess) e = cudaMalloc(&w->d_ctl, sizeof(BatchCtl) * n);
    if (e == cudaSuccess) e = cudaMallocHost(&w->h_flags, sizeof(int) * 2 * n);
    if (e == cudaSuccess) e = cudaMalloc(&w->d_flags, sizeof(int) * 2 * n);
    for (int g = 0; g < FsBatchWork::kShapes && e == cudaSuccess; g++) {
        w->ntiles[g] = (int)tiles[g].size();
        if (tiles[g].empty()) continue;
        e = cudaMalloc(&w->d_tiles_g[g], sizeof(int4) * tiles[g].size());
        if (e == cudaSuccess)
            e = cudaMemcpy(w->d_tiles_g[g], tiles[g].data(), sizeof(int4) * tiles[g].size(), cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) e = cudaMallocHost(&w->h_gather, sizeof(Ctrl) * n);
    if (e == cudaSuccess) e = cudaMalloc(&w->d_gather, sizeof(Ctrl) * n);
    for (int b = 0; b < n && e == cudaSuccess; b++) e = cudaEventCreateWithFlags(&w->ev[b], cudaEventDisableTiming);
    if (e != cudaSuccess) { fs_batch_work_free(w); return FS_ERR_NOMEM; }
    *out = w;
    return FS_OK;
}

// One RK-Merson attempt (ptcl_step, ptcl_lib.F90:32-97) of every context b
// with act[b] != 0, the five stages each as one launch over the tiles of all
// of them, the controllers as one launch: the kernels and the arithmetic of
// fs_ptcl_step_impl, so every discharge takes the same steps as alone.
// fresh[b]: the attempt starts a step (else it retries one the controller
// rejected).  On return rej[b] = 1 for a rejected attempt (its retry is the
// caller's next call), 0 for an accepted one (levels and dt advanced as
// fs_ptcl_step_impl leaves them); rc[b] an error of discharge b.  DC source,
// FP64 path, no dielectric wall.
int fs_ptcl_batch_attempt(fs_ctx **cs, int n, FsBatchWork *w, const int *act, const int *fresh, int *rej, int *rc) {
    const int ns = 3;
    int any = 0;
    for (int b = 0; b < n; b++) {
        rej[b] = 0;
        if (!act[b]) continue;
        any = 1;
        fs_ctx *c = cs[b];
        // order after the discharge's own stream (its last Poisson solve)
        cudaEventRecord(w->ev[b], c->stream);
        cudaStreamWaitEvent(w->st, w->ev[b], 0);
        if (fresh[b]) {
            c->Vsrc = fs_circ_source(c->cfg, c->k, c->t);
            if (!c->faces_valid) {   // E and ion face data of the current phi, on the batch stream
                dim3 bl(32, 8), g((c->nx + 1 + 31) / 32, (c->ny + 1 + 7) / 8);
                FaceArgs f = {c->fx_e, c->fx_cl, c->fx_cr, c->fx_dl, c->fx_dr,
                              c->fy_e, c->fy_cl, c->fy_cr, c->fy_dl, c->fy_dr};
                k_faces<<<g, bl, 0, w->st>>>(c->pp, c->mesh, c->ph, f);
                c->launches++;
                c->faces_valid = 1;
            }
            w->in1[b] = c->lev[1];
            w->attempts[b] = 0;
        }
        w->attempts[b]++;
        const int L2 = c->lev[1], L3 = c->lev[2];
        int freeb[FS_NBUF], nf = 0;
        for (int q = 0; q < FS_NBUF; q++)
            if (q != L2 && q != L3) freeb[nf++] = q;
        const int SA = freeb[0], SB = freeb[1], OUT = freeb[2];
        const int ins[5] = {w->in1[b], SA, SB, SA, SB};
        const int outs[5] = {SA, SB, SA, SB, OUT};
        for (int stg = 1; stg <= 5; stg++) {
            StageArgs &a = w->h_args[(size_t)(stg - 1) * n + b];
            memset(&a, 0, sizeof(a));
            a.pp = c->pp;
            a.m = c->mesh;
            a.tab = c->d_tab;
            a.ph = c->ph;
            a.fx_e = c->fx_e; a.fx_cl = c->fx_cl; a.fx_cr = c->fx_cr;
            a.fy_e = c->fy_e; a.fy_cl = c->fy_cl; a.fy_cr = c->fy_cr;
            a.ctrl = c->d_ctrl;
            a.part = c->d_part;
            a.rows = c->d_rows;
            a.sig_pl = fs_sig(c, 0);
            a.sig_mi = fs_sig(c, 1);
            a.sig_or = fs_sig(c, 2);
            a.ks = fs_sig_ks(c);
            a.nblk = w->nblk[b];
            a.stage = stg;
            for (int sp = 0; sp < ns; sp++) {
                SpeciesBufs &bf = c->sp[sp];
                a.nin[sp] = bf.buf[ins[stg - 1]];
                a.nbase[sp] = bf.buf[L3];
                a.nout[sp] = bf.buf[outs[stg - 1]];
                a.k1[sp] = bf.k[0];
                a.k3[sp] = bf.k[1];
                a.k4[sp] = bf.k[2];
                a.kout[sp] = stg == 1 ? bf.k[0] : stg == 3 ? bf.k[1] : stg == 4 ? bf.k[2] : nullptr;
            }
        }
        BatchCtl &q = w->h_ctl[b];
        q.ctrl = c->d_ctrl; q.part = c->d_part; q.rows = c->d_rows; q.rows_w = c->d_rows;
        q.nblk = w->nblk[b]; q.ns = ns; q.ny = c->ny; q.adaptive = c->cfg.adaptive; q.dt_min = c->cfg.dt_min;
        q.ph = c->ph; q.fx_e = c->fx_e; q.tx = c->mesh.tx; q.r = c->mesh.r; q.dx = c->mesh.dx;
        q.nx = c->nx; q.P = c->pitch; q.ew = c->cfg.ew; q.vd = c->Vsrc;
        c->launches += 7;   // reset, five stages, ghosts (the controller is counted below)
    }
    if (!any) return FS_OK;
    for (int b = 0; b < n; b++) { w->h_flags[b] = act[b]; w->h_flags[n + b] = fresh[b]; }
    cudaMemcpyAsync(w->d_args, w->h_args, sizeof(StageArgs) * 5 * n, cudaMemcpyHostToDevice, w->st);
    cudaMemcpyAsync(w->d_ctl, w->h_ctl, sizeof(BatchCtl) * n, cudaMemcpyHostToDevice, w->st);
    cudaMemcpyAsync(w->d_flags, w->h_flags, sizeof(int) * 2 * n, cudaMemcpyHostToDevice, w->st);
    const int *d_act = w->d_flags, *d_fresh = w->d_flags + n;
    k_reset_batch<<<n, 256, 0, w->st>>>(w->d_ctl, d_act, d_fresh);
    for (int stg = 1; stg <= 5; stg++) {
        const StageArgs *sa = w->d_args + (size_t)(stg - 1) * n;
        if (w->ntiles[0]) k_stage_batch<3, 32, 8><<<w->ntiles[0], 256, 0, w->st>>>(sa, w->d_tiles_g[0], d_act);
        if (w->ntiles[1]) k_stage_batch<3, 32, 4><<<w->ntiles[1], 128, 0, w->st>>>(sa, w->d_tiles_g[1], d_act);
        if (w->ntiles[2]) k_stage_batch<3, 64, 4><<<w->ntiles[2], 256, 0, w->st>>>(sa, w->d_tiles_g[2], d_act);
        if (stg == 1) k_circ_ghost_batch<<<n, 128, 0, w->st>>>(w->d_ctl, d_act);
    }
    k_controller_batch<<<n, 256, 0, w->st>>>(w->d_ctl, d_act, w->d_gather);
    cudaMemcpyAsync(w->h_gather, w->d_gather, sizeof(Ctrl) * n, cudaMemcpyDeviceToHost, w->st);
    cudaError_t e = cudaStreamSynchronize(w->st);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
        for (int b = 0; b < n; b++)
            if (act[b]) rc[b] = fs_cuda_check(cs[b], e, "batched RK attempt");
        return FS_ERR_CUDA;
    }
    for (int b = 0; b < n; b++) {
        if (!act[b]) continue;
        fs_ctx *c = cs[b];
        c->launches++;
        *c->h_ctrl = w->h_gather[b];
        const Ctrl &h = *c->h_ctrl;
        if (h.status & FS_ST_NEG_DENSITY) { rc[b] = fs_set_error(c, FS_ERR_NEG_DENSITY, "negative density in get_Te"); continue; }
        if (h.status & FS_ST_NAN) { rc[b] = fs_set_error(c, FS_ERR_NAN, "NaN in particle right-hand side"); continue; }
        if (h.min_dt) { rc[b] = fs_set_error(c, FS_ERR_MIN_DT, "minimum timestep reached"); continue; }
        c->Vd_pl = c->Vd_mi = c->Vsrc;
        if (h.rejected) {
            c->st.rk_rejects++;
            c->Vd_pl = c->Vd_or;
            c->Vd_mi = c->Vd_or;
            w->in1[b] = c->lev[2];   // restart from the base state
            rej[b] = 1;
            if (w->attempts[b] > 100000) rc[b] = fs_set_error(c, FS_ERR_MIN_DT, "RK restart limit");
            continue;
        }
        const int L2 = c->lev[1], L3 = c->lev[2];
        int freeb[FS_NBUF], nf = 0;
        for (int q = 0; q < FS_NBUF; q++)
            if (q != L2 && q != L3) freeb[nf++] = q;
        c->lev[0] = freeb[2];
        c->lev[1] = freeb[1];
        c->dt = h.dt;
        c->st.attempts += w->attempts[b];
    }
    return FS_OK;
}
