// fs_output.cpp -- the reference's on-disk output, written from device state.
//
// Same files, units and layout as the reference's g_init output set-up
// (props.F90:239-320) and writeOut (main.F90:297-333), so its post-processing
// (save.py) reads a GPU run unchanged: raw native FP64 with no record
// markers; meshx.dat / meshy.dat hold the interior node coordinates in metres;
// every call appends one record to f1..f5.dat (the interior (nx, ny) block,
// x fastest: phi in V, n_e, n_i in m^-3, the energy density as n_eps ph0 / 1.5,
// n_m in m^-3) and one value to time.dat (nondimensional t), vd.dat (V),
// ida.dat / idc.dat (A), dt.dat (nondimensional) and flx.dat (the EM flux,
// zero: the EM module is not part of the path).  With three species f5.dat
// gets zeros.
#include <cstdio>
#include <string>
#include <vector>

#include "fs_internal.h"

static int put(fs_ctx *c, const std::string &path, const double *v, size_t n, bool append) {
    FILE *f = fopen(path.c_str(), append ? "ab" : "wb");
    if (!f) return fs_set_error(c, FS_ERR_INVALID, "cannot open %s", path.c_str());
    const size_t w = n ? fwrite(v, sizeof(double), n, f) : 0;
    const int rc = fclose(f);
    if (w != n || rc != 0) return fs_set_error(c, FS_ERR_INVALID, "cannot write %s", path.c_str());
    return FS_OK;
}

int fs_write_output(fs_ctx *c, const char *dir, int32_t init) {
    if (!c || !dir) return FS_ERR_INVALID;
    const std::string p = std::string(dir) + "/";
    const int nx = c->nx, ny = c->ny, ld = nx + 2;
    const double x0 = c->k.x0, ph0 = c->k.ph0, x03 = x0 * x0 * x0;
    int rc;
    static const char *series[] = {"f1.dat", "f2.dat", "f3.dat", "f4.dat", "f5.dat", "time.dat", "vd.dat",
                                   "ida.dat", "idc.dat", "dt.dat", "flx.dat"};
    if (init) {   // g_init: fresh files, mesh coordinates
        std::vector<double> xs(nx), ys(ny);
        for (int i = 0; i < nx; i++) xs[i] = c->h_x[i + 1] * x0;
        for (int j = 0; j < ny; j++) ys[j] = c->h_y[j + 1] * x0;
        if ((rc = put(c, p + "meshx.dat", xs.data(), xs.size(), false))) return rc;
        if ((rc = put(c, p + "meshy.dat", ys.data(), ys.size(), false))) return rc;
        for (const char *s : series)
            if ((rc = put(c, p + s, nullptr, 0, false))) return rc;
        return FS_OK;
    }
    const size_t ng = (size_t)ld * (ny + 2);
    std::vector<double> ni(ng), ne(ng), nt(ng), nm(ng, 0.0), ph(ng);
    if ((rc = fs_download_state(c, ni.data(), ne.data(), nt.data(), c->cfg.nspecies == 4 ? nm.data() : nullptr,
                                ph.data(), ld, 1)))
        return rc;
    std::vector<double> blk((size_t)nx * ny);
    // the interior block, each value converted as writeOut converts it
    auto interior = [&](const std::vector<double> &a, auto conv) {
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) blk[(size_t)(j - 1) * nx + (i - 1)] = conv(a[(size_t)j * ld + i]);
    };
    interior(ph, [&](double v) { return v * ph0; });
    if ((rc = put(c, p + "f1.dat", blk.data(), blk.size(), true))) return rc;
    interior(ne, [&](double v) { return v / x03; });
    if ((rc = put(c, p + "f2.dat", blk.data(), blk.size(), true))) return rc;
    interior(ni, [&](double v) { return v / x03; });
    if ((rc = put(c, p + "f3.dat", blk.data(), blk.size(), true))) return rc;
    interior(nt, [&](double v) { return v / x03 * ph0 / 1.5; });
    if ((rc = put(c, p + "f4.dat", blk.data(), blk.size(), true))) return rc;
    interior(nm, [&](double v) { return v / x03; });
    if ((rc = put(c, p + "f5.dat", blk.data(), blk.size(), true))) return rc;
    const double e = c->k.e, t0 = c->k.t0;
    const double vals[6] = {c->t, c->Vd_pl * ph0, c->h_ctrl->ida * e / t0, c->h_ctrl->idc * e / t0, c->dt, 0.0};
    static const char *names[6] = {"time.dat", "vd.dat", "ida.dat", "idc.dat", "dt.dat", "flx.dat"};
    for (int k = 0; k < 6; k++)
        if ((rc = put(c, p + names[k], &vals[k], 1, true))) return rc;
    return FS_OK;
}
