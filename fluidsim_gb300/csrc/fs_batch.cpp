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
#include <cstdlib>
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

// One group of the fused advance: rounds of one fused RK-Merson attempt of
// every unfinished discharge of the group that is past its two Poisson-only
// start-up iterations (fs_ptcl_batch_attempt: one launch per stage and tile
// shape over the tiles of all of them, per-discharge dt, its own accept or
// reject), then -- host threads in parallel, one discharge each -- the
// Poisson solve (the CUDA graph of its CG loop) and the accept/reject
// rotation of every discharge whose attempt was accepted.  A rejected attempt
// is retried in the next round.  rc holds the group's return codes.
static int fused_group(fs_ctx **ctx, int n, int32_t steps, double t_end, int nthreads, int32_t *rc) {
    FsBatchWork *w = nullptr;
    int rc0 = fs_batch_work_alloc(ctx, n, &w);
    if (rc0) {
        for (int i = 0; i < n; i++) rc[i] = rc0;
        return rc0;
    }
    std::vector<int> act(n), fresh(n, 1), rej(n, 0), done(n, 0), rk(n), pois(n), rci(n, FS_OK);
    std::vector<int> order(n);
    for (int i = 0; i < n; i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return (long)ctx[a]->nx * ctx[a]->ny > (long)ctx[b]->nx * ctx[b]->ny;
    });
    int err = FS_OK;
    for (int round = 0;; round++) {
        int nact = 0, nrk = 0;
        for (int i = 0; i < n; i++) {
            fs_ctx *c = ctx[i];
            act[i] = rci[i] == FS_OK && done[i] < steps && !(t_end > 0.0 && c->t >= t_end);
            rk[i] = act[i] && c->ts > 1;
            nact += act[i];
            nrk += rk[i];
        }
        if (!nact) break;
        if (nrk) {
            err = fs_ptcl_batch_attempt(ctx, n, w, rk.data(), fresh.data(), rej.data(), rci.data());
            if (err) break;
        }
        for (int i = 0; i < n; i++) {
            pois[i] = act[i] && rci[i] == FS_OK && !(rk[i] && rej[i]);
            fresh[i] = !(rk[i] && rej[i] && rci[i] == FS_OK);
        }
        std::atomic<int> next(0);
        auto worker = [&]() {
            cudaSetDevice(ctx[0]->device);
            for (;;) {
                const int k = next.fetch_add(1);
                if (k >= n) return;
                const int i = order[k];
                if (!pois[i]) continue;
                fs_ctx *c = ctx[i];
                int lerr = 1, iters = 0;
                double relres = 0;
                int r = fs_lapl_solve_impl(c, &lerr, &iters, &relres);
                if (r == FS_OK) {
                    c->st.lapl_iters += iters;
                    c->st.last_lapl_iters = iters;
                    c->st.lapl_relres = relres;
                    c->st.lerr = lerr;
                    if (lerr == 0) r = fs_accept(c);
                    else {
                        c->st.lapl_rejects++;
                        r = fs_reject(c);
                    }
                }
                rci[i] = r;
                done[i]++;
            }
        };
        // the first round builds the discharges' CUDA graphs: one thread
        const int nt = round == 0 ? 1 : std::min<int>(nthreads, nact);
        std::vector<std::thread> pool;
        for (int t = 1; t < nt; t++) pool.emplace_back(worker);
        worker();
        for (auto &th : pool) th.join();
    }
    fs_batch_work_free(w);
    for (int i = 0; i < n; i++) rc[i] = err != FS_OK && rci[i] == FS_OK ? err : rci[i];
    return err;
}

// The same advance with the RK stages fused across discharges.  The
// discharges are dealt, largest first, into groups of about equal node count
// (eight by default; FS_FUSED_GROUPS in the environment sets 1..16), each
// driven by its own host thread (fused_group): while one group's Poisson
// solves run, another's fused stages do, so neither phase leaves the GPU
// idle.  On the 192-discharge sweep (grids 64-512^2, 32 host threads) one
// group ran at 0.88x the concurrent driver, two at 0.92x, four at 0.95x,
// eight at 0.97x; with every grid capped at 96^2 one group ran at 0.71x and
// eight at 1.04x.  Each discharge takes exactly the steps it takes alone.
int fs_batch_run_fused(fs_ctx **ctx, int32_t n, int32_t steps, double t_end, int32_t nthreads, fs_stats *out,
                       int32_t *rc_out) {
    if (!ctx || n < 1 || steps < 0 || nthreads < 1) return FS_ERR_INVALID;
    for (int i = 0; i < n; i++) {
        fs_ctx *c = ctx[i];
        if (!c) return FS_ERR_INVALID;
        if (c->mixed || c->cfg.nspecies != 3 || c->cfg.rf != 0 || c->rwall || c->device != ctx[0]->device)
            return fs_set_error(c, FS_ERR_UNSUPPORTED,
                                "fused batches take FP64 contexts with 3 species, a DC source, no dielectric wall "
                                "and one device");
    }
    cudaSetDevice(ctx[0]->device);
    std::vector<int> order(n);
    for (int i = 0; i < n; i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return (long)ctx[a]->nx * ctx[a]->ny > (long)ctx[b]->nx * ctx[b]->ny;
    });
    int ng = 8;
    if (const char *env = getenv("FS_FUSED_GROUPS")) ng = atoi(env);
    ng = std::max(1, std::min(ng, std::min<int>(n, 16)));
    std::vector<std::vector<fs_ctx *>> gctx(ng);
    std::vector<std::vector<int>> gidx(ng);
    std::vector<long> load(ng, 0);
    for (int i : order) {
        const int g = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        gctx[g].push_back(ctx[i]);
        gidx[g].push_back(i);
        load[g] += (long)ctx[i]->nx * ctx[i]->ny;
    }
    std::vector<std::vector<int32_t>> grc(ng);
    std::vector<int> gerr(ng, FS_OK);
    const int nt = std::max(1, nthreads / ng);
    auto run = [&](int g) {
        cudaSetDevice(ctx[0]->device);
        grc[g].assign(gctx[g].size(), FS_OK);
        gerr[g] = fused_group(gctx[g].data(), (int)gctx[g].size(), steps, t_end, nt, grc[g].data());
    };
    std::vector<std::thread> drivers;
    for (int g = 1; g < ng; g++) drivers.emplace_back(run, g);
    run(0);
    for (auto &th : drivers) th.join();
    std::vector<int32_t> rc(n, FS_OK);
    for (int g = 0; g < ng; g++)
        for (size_t k = 0; k < gidx[g].size(); k++) rc[gidx[g][k]] = grc[g][k];
    int first = FS_OK;
    for (int i = 0; i < n; i++) {
        fs_stats st;
        memset(&st, 0, sizeof(st));
        if (rc[i] == FS_OK) rc[i] = fs_get_stats(ctx[i], &st);
        if (out) out[i] = st;
        if (rc_out) rc_out[i] = rc[i];
        if (rc[i] != FS_OK && first == FS_OK) first = rc[i];
    }
    for (int g = 0; g < ng && first == FS_OK; g++) first = gerr[g];
    return first;
}
