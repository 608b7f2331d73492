// fs_output.cpp -- the reference's on-disk output, written from device state.
//
// Same files, units and layout as the reference's g_init output set-up
// (props.F90:239-320) and writeOut (main.F90:297-333), so its post-processing
// (save.py) reads a GPU run unchanged: raw native FP64 with no record
// markers; meshx.dat / meshy.dat hold the interior node coordinates in metres;
// every record appends to f1..f5.dat the interior (nx, ny) block, x fastest:
// phi in V, n_e, n_i in m^-3, the energy density as n_eps ph0 / 1.5, n_m in
// m^-3 (zeros with three species); and one value to time.dat (nondimensional
// t), vd.dat (V), ida.dat / idc.dat (A), dt.dat (nondimensional) and flx.dat
// (the EM flux, zero: the EM module is not part of the path).
//
// A record is written asynchronously: fs_write_output queues a device-to-host
// copy of the level-1 fields into a pinned staging buffer on the context's
// stream, records an event and hands the record to the context's writer
// thread, which waits for the event, converts and appends while the caller
// keeps stepping (stream order makes the copy see the state as of the call).
// One record is in flight at a time: the next call, fs_output_wait and
// fs_destroy wait for it.
#include <condition_variable>
#include <cstdio>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "fs_internal.h"

struct fs_output {
    std::thread th;
    std::mutex m;
    std::condition_variable cv;
    bool busy = false, quit = false;
    int status = FS_OK;
    std::string err;
    // the record in flight
    std::string dir;
    double vals[6] = {0, 0, 0, 0, 0, 0};
    double *stage = nullptr;     // pinned: ni, ne, nt, nm, ph at (nx+2, ny+2) each
    cudaEvent_t ev = nullptr;
    int nx = 0, ny = 0, ns = 3;
    int device = 0;
    double x0 = 0, ph0 = 0;
};

namespace {

int put(std::string &err, const std::string &path, const double *v, size_t n, bool append) {
    FILE *f = fopen(path.c_str(), append ? "ab" : "wb");
    if (!f) { err = "cannot open " + path; return FS_ERR_INVALID; }
    const size_t w = n ? fwrite(v, sizeof(double), n, f) : 0;
    const int rc = fclose(f);
    if (w != n || rc != 0) { err = "cannot write " + path; return FS_ERR_INVALID; }
    return FS_OK;
}

// writeOut for the staged record (runs on the writer thread)
int write_record(fs_output &o) {
    const int nx = o.nx, ny = o.ny, ld = nx + 2;
    const size_t ng = (size_t)ld * (ny + 2);
    const double x03 = o.x0 * o.x0 * o.x0, ph0 = o.ph0;
    const std::string p = o.dir + "/";
    std::vector<double> blk((size_t)nx * ny);
    auto field = [&](int q) { return o.stage + (size_t)q * ng; };
    // the interior block, each value converted as writeOut converts it
    auto interior = [&](const double *a, auto conv) {
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) blk[(size_t)(j - 1) * nx + (i - 1)] = conv(a[(size_t)j * ld + i]);
    };
    int rc;
    interior(field(4), [&](double v) { return v * ph0; });
    if ((rc = put(o.err, p + "f1.dat", blk.data(), blk.size(), true))) return rc;
    interior(field(1), [&](double v) { return v / x03; });
    if ((rc = put(o.err, p + "f2.dat", blk.data(), blk.size(), true))) return rc;
    interior(field(0), [&](double v) { return v / x03; });
    if ((rc = put(o.err, p + "f3.dat", blk.data(), blk.size(), true))) return rc;
    interior(field(2), [&](double v) { return v / x03 * ph0 / 1.5; });
    if ((rc = put(o.err, p + "f4.dat", blk.data(), blk.size(), true))) return rc;
    if (o.ns == 4) interior(field(3), [&](double v) { return v / x03; });
    else std::fill(blk.begin(), blk.end(), 0.0);
    if ((rc = put(o.err, p + "f5.dat", blk.data(), blk.size(), true))) return rc;
    static const char *names[6] = {"time.dat", "vd.dat", "ida.dat", "idc.dat", "dt.dat", "flx.dat"};
    for (int k = 0; k < 6; k++)
        if ((rc = put(o.err, p + names[k], &o.vals[k], 1, true))) return rc;
    return FS_OK;
}

void writer_loop(fs_output *o) {
    cudaSetDevice(o->device);   // the context's device, for the event waits
    std::unique_lock<std::mutex> lk(o->m);
    for (;;) {
        o->cv.wait(lk, [o] { return o->quit || o->busy; });
        if (o->busy) {
            lk.unlock();
            int rc;
            cudaError_t e = cudaEventSynchronize(o->ev);
            if (e != cudaSuccess) {
                rc = FS_ERR_CUDA;
                o->err = std::string("output copy: ") + cudaGetErrorString(e);
            } else {
                rc = write_record(*o);
            }
            lk.lock();
            if (rc && o->status == FS_OK) o->status = rc;
            o->busy = false;
            o->cv.notify_all();
        } else if (o->quit) {
            return;
        }
    }
}

// wait for the record in flight; returns (and clears) the writer's status
int wait_record(fs_ctx *c) {
    fs_output *o = c->out;
    if (!o) return FS_OK;
    std::unique_lock<std::mutex> lk(o->m);
    o->cv.wait(lk, [o] { return !o->busy; });
    const int rc = o->status;
    o->status = FS_OK;
    if (rc) return fs_set_error(c, rc, "%s", o->err.c_str());
    return FS_OK;
}

int start(fs_ctx *c) {
    if (c->out) return FS_OK;
    fs_output *o = new fs_output();
    o->nx = c->nx;
    o->ny = c->ny;
    o->device = c->device;
    o->ns = c->cfg.nspecies;
    o->x0 = c->k.x0;
    o->ph0 = c->k.ph0;
    const size_t ng = (size_t)(c->nx + 2) * (c->ny + 2);
    cudaError_t e = cudaMallocHost(&o->stage, sizeof(double) * 5 * ng);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&o->ev, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        if (o->stage) cudaFreeHost(o->stage);
        delete o;
        return fs_cuda_check(c, e, "output staging");
    }
    o->th = std::thread(writer_loop, o);
    c->out = o;
    return FS_OK;
}

}  // namespace

void fs_output_free(fs_ctx *c) {
    fs_output *o = c->out;
    if (!o) return;
    {
        std::unique_lock<std::mutex> lk(o->m);
        o->cv.wait(lk, [o] { return !o->busy; });
        o->quit = true;
        o->cv.notify_all();
    }
    o->th.join();
    cudaEventDestroy(o->ev);
    cudaFreeHost(o->stage);
    delete o;
    c->out = nullptr;
}

int fs_output_wait(fs_ctx *c) {
    if (!c) return FS_ERR_INVALID;
    return wait_record(c);
}

int fs_write_output(fs_ctx *c, const char *dir, int32_t init) {
    if (!c || !dir) return FS_ERR_INVALID;
    int rc;
    if ((rc = wait_record(c))) return rc;
    const std::string p = std::string(dir) + "/";
    if (init) {   // g_init: fresh files, mesh coordinates (synchronous)
        const int nx = c->nx, ny = c->ny;
        const double x0 = c->k.x0;
        std::string err;
        std::vector<double> xs(nx), ys(ny);
        for (int i = 0; i < nx; i++) xs[i] = c->h_x[i + 1] * x0;
        for (int j = 0; j < ny; j++) ys[j] = c->h_y[j + 1] * x0;
        static const char *series[] = {"f1.dat", "f2.dat", "f3.dat", "f4.dat", "f5.dat", "time.dat", "vd.dat",
                                       "ida.dat", "idc.dat", "dt.dat", "flx.dat"};
        if (!(rc = put(err, p + "meshx.dat", xs.data(), xs.size(), false)) &&
            !(rc = put(err, p + "meshy.dat", ys.data(), ys.size(), false)))
            for (const char *s : series)
                if ((rc = put(err, p + s, nullptr, 0, false))) break;
        return rc ? fs_set_error(c, rc, "%s", err.c_str()) : FS_OK;
    }
    if ((rc = start(c))) return rc;
    fs_output *o = c->out;
    // stage the level-1 fields on the stream: ni, ne, nt, nm, ph
    const size_t ld = (size_t)c->nx + 2, rows = (size_t)c->ny + 2, ng = ld * rows;
    const size_t w = ld * sizeof(double), dp = (size_t)c->pitch * sizeof(double);
    cudaError_t e = cudaSuccess;
    for (int s = 0; s < c->cfg.nspecies && e == cudaSuccess; s++)
        e = cudaMemcpy2DAsync(o->stage + (size_t)s * ng, w, c->sp[s].buf[c->lev[0]], dp, w, rows,
                              cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpy2DAsync(o->stage + 4 * ng, w, c->ph, dp, w, rows, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaEventRecord(o->ev, c->stream);
    if (e != cudaSuccess) return fs_cuda_check(c, e, "output staging copy");
    std::lock_guard<std::mutex> lk(o->m);
    o->dir = dir;
    const double ec = c->k.e, t0 = c->k.t0;
    const double vals[6] = {c->t, c->Vd_pl * c->k.ph0, c->h_ctrl->ida * ec / t0, c->h_ctrl->idc * ec / t0, c->dt,
                            0.0};
    for (int k = 0; k < 6; k++) o->vals[k] = vals[k];
    o->busy = true;
    o->cv.notify_all();
    return FS_OK;
}
