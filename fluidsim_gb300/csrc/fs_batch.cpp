// fs_batch.cpp -- advance many independent discharges concurrently.
//
// The reference runs one discharge per program invocation; its I-V curves
// (voltage and pressure sweeps, plot-idvd.py) come from many such runs.  Here
// each discharge is an ordinary context (own CUDA stream, own CUDA graphs,
// own adaptive dt and convergence), and a pool of host threads advances them:
// a worker takes the next unfinished discharge (largest grids first), runs it
// to its step count or end time, and takes the next.  The GPU overlaps the
// kernels of the streams in flight, which keeps the SMs busy on grids too
// small to fill them alone.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "fs_internal.h"

int fs_batch_run(fs_ctx **ctx, int32_t n, int32_t steps, double t_end, int32_t nthreads, fs_stats *out,
                 int32_t *rc_out) {
    if (!ctx || n < 0 || steps < 0 || nthreads < 1) return FS_ERR_INVALID;
    for (int i = 0; i < n; i++)
        if (!ctx[i]) return FS_ERR_INVALID;
    std::vector<int> order(n);
    for (int i = 0; i < n; i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return (long)ctx[a]->nx * ctx[a]->ny > (long)ctx[b]->nx * ctx[b]->ny;
    });
    std::atomic<int> next(0);
    std::atomic<int> first_rc(0);
    auto worker = [&]() {
        for (;;) {
            const int k = next.fetch_add(1);
            if (k >= n) return;
            const int i = order[k];
            fs_ctx *c = ctx[i];
            cudaSetDevice(c->device);
            int rc = FS_OK;
            fs_stats st;
            memset(&st, 0, sizeof(st));
            for (int s = 0; s < steps && rc == FS_OK; s++) {
                if (t_end > 0.0 && c->t >= t_end) break;
                rc = fs_run(c, 1, &st);
            }
            if (rc == FS_OK) rc = fs_get_stats(c, &st);
            if (out) out[i] = st;
            if (rc_out) rc_out[i] = rc;
            if (rc != FS_OK) {
                int expect = 0;
                first_rc.compare_exchange_strong(expect, rc);
            }
        }
    };
    const int nt = std::min<int>(nthreads, std::max(n, 1));
    std::vector<std::thread> pool;
    for (int t = 1; t < nt; t++) pool.emplace_back(worker);
    worker();
    for (auto &th : pool) th.join();
    return first_rc.load();
}
