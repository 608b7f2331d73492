// fs_wall.cuh -- the dielectric wall on the last row (type_y == 3), shared by
// the FP64 and the mixed-precision RK stage: the wall face's fluxes
// (ptcl_lib.F90:292-294 and :392-406) and the surface-charge step sfc_step
// (sfc_lib.F90:19-80).  Both precision paths evaluate it in FP64: it runs on
// one row of the grid, and the surface charge it integrates is a running sum
// over the whole discharge.
#pragma once
#include <cuda_runtime.h>

#include "fs_fastmath.cuh"
#include "fs_internal.h"
#include "fs_sg.cuh"

struct WallArgs {
    const double *tab;          // FP64 coefficient table, FS_TAB_STRIDE doubles per node
    const double *sig_or;       // charge at the start of the step (nx+2)
    double *sig_mi, *sig_pl;    // the stages' charge (stages 1-4) and the step's result (stage 5)
    double *ks;                 // the five stage slopes, [5][nx+2]
};

// mue, De of the rate table at mean energy T (nondimensional)
__device__ __forceinline__ void fs_wall_tab(const PhysParams &pp, const double *tab, double T, double &mu,
                                            double &de) {
    const double x = fs_log(T * pp.ph0);
    double u = (x - pp.lemin) * pp.inv_h;
    if (!(u >= 0.0)) u = 0.0;
    if (u > (double)(pp.ntab - 1)) u = (double)(pp.ntab - 1);
    int i = (int)u;
    if (i > pp.ntab - 2) i = pp.ntab - 2;
    const double w = u - (double)i;
    const double *t = tab + (size_t)i * FS_TAB_STRIDE;
    mu = __ldg(t + 0) + w * __ldg(t + 8);
    de = __ldg(t + 1) + w * __ldg(t + 9);
}

// Wall face of column gi: field -sig_mi(i), fluxes into an empty wall node
// with the node's own coefficients and get_mut / get_Dt for the energy.  The
// calling thread is the only reader and writer of column gi's charge, so
// sfc_step runs here too: its slope from the same stage state, then the
// Merson combination into sig_mi (stages 1-4) or sig_pl (stage 5).  Returns
// the face field.  Kept out of line: it runs on one row.
template <int NS>
__device__ __noinline__ double fs_wall_face(const PhysParams &pp, const WallArgs &w, double dh, double dt,
                                            int stage, int gi, double te, double ni, double ne, double nt,
                                            double nm, double mue, double de, double &fi, double &fe, double &ft,
                                            double &fm, unsigned int &st) {
    const double E = -w.sig_mi[gi];
    fi = fs_sg_flux(1.0, E, dh, pp.mui, pp.Di, ni, 0.0);
    fe = fs_sg_flux(-1.0, E, dh, mue, de, ne, 0.0);
    ft = fs_sg_flux(-1.0, E, dh, pp.fit.mut(te), pp.fit.Dt(te), nt, 0.0);
    fm = NS == 4 ? pp.Dm * nm / dh : 0.0;
    // sfc_step receives (ni, ne, nt) in its (ne, ni, nt) arguments
    // (ptcl_lib.F90:52): its mean energy is nt/ni, its "ion" flux carries n_e
    // and its "electron" flux n_i
    double tes;
    if ((nt >= 0.0) && (ni >= 0.0)) tes = nt / ni;
    else { st |= FS_ST_NEG_DENSITY; tes = 1e-8; }
    double mus, des;
    if (pp.fits) {
        mus = pp.fit.mue(tes);
        des = pp.fit.De(tes);
    } else {
        fs_wall_tab(pp, w.tab, tes, mus, des);
    }
    const double ksv = fs_sg_flux(1.0, E, dh, pp.mui, pp.Di, ne, 0.0) - fs_sg_flux(-1.0, E, dh, mus, des, ni, 0.0);
    const int W = pp.nx + 2;
    w.ks[(size_t)(stage - 1) * W + gi] = ksv;
    const double so = w.sig_or[gi];
    const double k1 = stage > 1 ? w.ks[gi] : ksv;
    if (stage == 1) w.sig_mi[gi] = so + dt * k1 / 3.0;
    else if (stage == 2) w.sig_mi[gi] = so + dt * (k1 + ksv) / 6.0;
    else if (stage == 3) w.sig_mi[gi] = so + dt * (k1 + ksv * 3.0) / 8.0;
    else if (stage == 4) w.sig_mi[gi] = so + dt * (k1 - w.ks[(size_t)2 * W + gi] * 3.0 + ksv * 4.0) / 2.0;
    else w.sig_pl[gi] = so + dt * (k1 + w.ks[(size_t)3 * W + gi] * 4.0 + ksv) / 6.0;
    return E;
}
