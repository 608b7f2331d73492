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
// A record is written asynchronously: fs_write_output queues on the context's
// stream a kernel that converts the level-1 fields into the files' units and
// layout (fs_output_stage; stream order makes it see the state as of the
// call), then on the writer's own copy stream, after that kernel, one
// device-to-host copy of the result into a pinned block, so that the copy
// overlaps the steps that follow; the writer thread waits for the copy and
// appends the five blocks to their files, one thread per file, while the
// caller keeps stepping.  One record is in flight at a time: the next call,
// fs_output_wait and fs_destroy wait for it.
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
    double *stage = nullptr;     // pinned: the f1..f5 blocks, nx ny values each
    double *dstage = nullptr;    // device: the same blocks, converted by fs_output_stage
    cudaEvent_t ev = nullptr;    // the record's copy is complete (copy stream)
    cudaEvent_t conv = nullptr;  // the record's conversion is complete (context's stream)
    cudaStream_t cs = nullptr;   // copy stream
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

// writeOut for the staged record (runs on the writer thread): the five field
// blocks, already in the files' units and layout, appended by one thread each,
// then the six scalars
int write_record(fs_output &o) {
    const size_t n = (size_t)o.nx * o.ny;
    const std::string p = o.dir + "/";
    static const char *fields[5] = {"f1.dat", "f2.dat", "f3.dat", "f4.dat", "f5.dat"};
    int rcs[5] = {FS_OK, FS_OK, FS_OK, FS_OK, FS_OK};
    std::string errs[5];
    auto one = [&](int q) { rcs[q] = put(errs[q], p + fields[q], o.stage + q * n, n, true); };
    std::thread th[4];
    int started = 0;
    try {
        for (; started < 4; started++) th[started] = std::thread(one, started + 1);
    } catch (...) {   // no thread to be had: the rest on this one
    }
    for (int q = started + 1; q < 5; q++) one(q);
    one(0);
    for (int t = 0; t < started; t++) th[t].join();
    for (int q = 0; q < 5; q++)
        if (rcs[q]) { o.err = errs[q]; return rcs[q]; }
    static const char *names[6] = {"time.dat", "vd.dat", "ida.dat", "idc.dat", "dt.dat", "flx.dat"};
    int rc;
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
    const size_t n = (size_t)c->nx * c->ny;
    cudaError_t e = cudaMallocHost(&o->stage, sizeof(double) * 5 * n);
    if (e == cudaSuccess) e = cudaMalloc(&o->dstage, sizeof(double) * 5 * n);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&o->ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&o->conv, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&o->cs, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        if (o->stage) cudaFreeHost(o->stage);
        if (o->dstage) cudaFree(o->dstage);
        if (o->ev) cudaEventDestroy(o->ev);
        if (o->conv) cudaEventDestroy(o->conv);
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
    cudaStreamSynchronize(o->cs);
    cudaStreamDestroy(o->cs);
    cudaEventDestroy(o->ev);
    cudaEventDestroy(o->conv);
    cudaFreeHost(o->stage);
    cudaFree(o->dstage);
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
    // the level-1 fields converted on the device (context's stream), then
    // copied to the pinned block on the copy stream
    const size_t n = (size_t)c->nx * c->ny;
    cudaError_t e = fs_output_stage(c, o->dstage, o->x0 * o->x0 * o->x0);
    if (e == cudaSuccess) e = cudaEventRecord(o->conv, c->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(o->cs, o->conv, 0);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(o->stage, o->dstage, 5 * n * sizeof(double), cudaMemcpyDeviceToHost, o->cs);
    if (e == cudaSuccess) e = cudaEventRecord(o->ev, o->cs);
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
