// fs_mg.cuh -- multigrid building blocks shared by the FP64 and the mixed
// precision Poisson solvers: deterministic grid reductions, the 2x2
// aggregation hierarchy (coarse operators, red-black Gauss-Seidel, restriction,
// prolongation), the temporally blocked level kernels and the one-CTA bottom
// solver, each templated on the arithmetic type of the level.
#pragma once
#include <algorithm>
#include <cuda_runtime.h>

#include "fs_internal.h"

#define BOTTOM_N 32
#define BOTTOM_THREADS 1024

// Post-smoothing of both solvers' V-cycles: every half sweep after the
// coarse-grid correction is over-relaxed by FS_MG_OMEGA_POST, and the finest
// level's electrode strips (k_rb_strips) get FS_STRIP_PAIRS more red-black
// sweep pairs; strips wider than FS_STRIP_MAX columns (a mesh stretched
// everywhere) get none.  The pre-smoothing stays plain Gauss-Seidel, so the
// black residuals the down sweeps leave are still zero.  On the 1024^2 glow
// Jacobians this takes the CG from 11-12 iterations to 8.
#define FS_MG_OMEGA_POST 1.3
#define FS_STRIP_PAIRS 2
// The FP64 solver's finest level pre-smooths with one sweep pair fewer than
// the others (at least one): its FP64 sweeps are the costliest of the cycle,
// and with the strip sweeps after its post-smoothing the CG needs no more
// iterations for it (8 at 1024^2 with 1 or 2 pre-sweeps there; 9 with 1
// post-sweep, 10 with 1 + 1).  The mixed solver keeps both: its FP32 inner
// iteration, restarted at each refinement, went from 8 to 9.2 iterations.
inline int fs_mg_pre0(int nu) { return nu > 1 ? nu - 1 : 1; }
#define FS_STRIP_MAX 64

namespace {

__device__ __forceinline__ double warp_sum_d(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// part[tid] + part[tid + NTH] + part[tid + 2 NTH] + ... (< nblk), summed in
// that order, the loads issued four at a time: the partials were just written
// by other CTAs, so each load is an L2 round trip, and a chain of dependent
// ones is what the last CTA of a grid reduction would otherwise wait on.  The
// loads bypass L1 (ld.global.cg): the writers' __threadfence and the counter
// make their values visible in L2.
template <int NTH>
__device__ __forceinline__ double strided_sum(const double *part, int nblk, int tid) {
    double s = 0.0;
    for (int b = tid; b < nblk; b += 4 * NTH) {
        double v[4];
#pragma unroll
        for (int k = 0; k < 4; k++) v[k] = b + k * NTH < nblk ? __ldcg(part + b + k * NTH) : 0.0;
#pragma unroll
        for (int k = 0; k < 4; k++) s += v[k];
    }
    return s;
}

// Block sum of v, then deterministic grid sum by the last CTA.  Returns true
// in the last CTA (all threads), with *out written.
template <int NTH>
__device__ bool grid_sum(double v, double *part, unsigned int *counter, int nblk, double *out) {
    __shared__ double s_w[NTH / 32];
    __shared__ bool s_last;
    const int tid = threadIdx.x + threadIdx.y * blockDim.x;
    const int bid = blockIdx.x + blockIdx.y * gridDim.x;
    v = warp_sum_d(v);
    if ((tid & 31) == 0) s_w[tid >> 5] = v;
    __syncthreads();
    if (tid == 0) {
        double s = 0.0;
        for (int w = 0; w < NTH / 32; w++) s += s_w[w];
        part[bid] = s;
        __threadfence();
        unsigned int prev = atomicAdd(counter, 1u);
        s_last = (prev == (unsigned int)nblk - 1u);
    }
    __syncthreads();
    if (!s_last) return false;
    __threadfence();
    __shared__ double s_r[NTH];
    s_r[tid] = strided_sum<NTH>(part, nblk, tid);
    __syncthreads();
    for (int w = NTH / 2; w > 0; w >>= 1) {
        if (tid < w) s_r[tid] += s_r[tid + w];
        __syncthreads();
    }
    if (tid == 0) {
        *out = s_r[0];
        *counter = 0u;
    }
    __syncthreads();
    return true;
}

// Fixed-order sum of two per-thread values over the grid (256-thread CTAs);
// true in the last CTA (thread 0 holds the sums).  part needs 2 * nblk entries.
__device__ bool grid_sum2(double v, double w, double *part, unsigned int *counter, int nblk, double &sv,
                          double &sw) {
    __shared__ double s_a[8], s_b[8];
    __shared__ bool s_last;
    for (int o = 16; o > 0; o >>= 1) {
        v += __shfl_down_sync(0xffffffffu, v, o);
        w += __shfl_down_sync(0xffffffffu, w, o);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { s_a[wid] = v; s_b[wid] = w; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ra = 0.0, rb = 0.0;
        for (int k = 0; k < 8; k++) { ra += s_a[k]; rb += s_b[k]; }
        part[blockIdx.x] = ra;
        part[nblk + blockIdx.x] = rb;
        __threadfence();
        s_last = atomicAdd(counter, 1u) == (unsigned int)nblk - 1u;
    }
    __syncthreads();
    if (!s_last) return false;
    __threadfence();
    __shared__ double s_r[256], s_w[256];
    s_r[threadIdx.x] = strided_sum<256>(part, nblk, threadIdx.x);
    s_w[threadIdx.x] = strided_sum<256>(part + nblk, nblk, threadIdx.x);
    __syncthreads();
    for (int k = 128; k > 0; k >>= 1) {
        if (threadIdx.x < k) { s_r[threadIdx.x] += s_r[threadIdx.x + k]; s_w[threadIdx.x] += s_w[threadIdx.x + k]; }
        __syncthreads();
    }
    sv = s_r[0];
    sw = s_w[0];
    if (threadIdx.x == 0) *counter = 0u;
    return true;
}

// Fixed-order sum of three per-thread values over the grid (256-thread CTAs);
// true in the last CTA (thread 0 holds the sums).  part needs 3 * nblk entries.
__device__ bool grid_sum3(double (&v)[3], double *part, unsigned int *counter, int nblk, double (&out)[3]) {
    __shared__ double s_p[3][8];
    __shared__ bool s_last;
#pragma unroll
    for (int k = 0; k < 3; k++)
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0)
        for (int k = 0; k < 3; k++) s_p[k][wid] = v[k];
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 0; k < 3; k++) {
            double r = 0.0;
            for (int w = 0; w < 8; w++) r += s_p[k][w];
            part[(size_t)k * nblk + blockIdx.x] = r;
        }
        __threadfence();
        s_last = atomicAdd(counter, 1u) == (unsigned int)nblk - 1u;
    }
    __syncthreads();
    if (!s_last) return false;
    __threadfence();
    __shared__ double s_r[3][256];
    for (int k = 0; k < 3; k++) s_r[k][threadIdx.x] = strided_sum<256>(part + (size_t)k * nblk, nblk, threadIdx.x);
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if (threadIdx.x < h)
            for (int k = 0; k < 3; k++) s_r[k][threadIdx.x] += s_r[k][threadIdx.x + h];
        __syncthreads();
    }
    for (int k = 0; k < 3; k++) out[k] = s_r[k][0];
    if (threadIdx.x == 0) *counter = 0u;
    return true;
}

// ---------------------------------------------------------------- multigrid
template <typename T>
struct LevelT {
    int nx, ny, P;
    T *mc, *ce, *cn, *extra, *inv_mc, *rhs, *x, *res;
};
using LevelDev = LevelT<double>;

// Coarse operators of the 2x2 aggregation: an aggregate's x face conducts as
// the fine x faces across it in parallel, each in series with half of the
// fine faces inside the two aggregates it joins (y alike), and the boundary
// remainder of a fine cell, in series with half of its aggregate's inner
// face, adds up.  The arithmetic is FP32 on every level, also under the FP64
// solver: the coarse operators only shape its preconditioner (a fixed linear
// map either way), and the FP64 divisions cost ~20 us a level on this GPU.
template <typename T>
__device__ __forceinline__ float inv_or_big(T c) {
    const float cf = (float)c;
    return cf > 1e-37f ? 1.0f / cf : 1e37f;
}
// The face functions issue all their loads before any arithmetic, so that a
// thread's loads overlap (otherwise each waits for the division before it).
// x face between aggregates (I, J) and (I + 1, J); 0 at the grid's edges
template <typename T>
__device__ __forceinline__ float coarse_ce(const LevelT<T> &f, int cnx, int I, int J) {
    if (I < 1 || I >= cnx) return 0.0f;
    const int fx0 = 2 * I - 1, fx1 = min(2 * I, f.nx), fy0 = 2 * J - 1, fy1 = min(2 * J, f.ny);
    const int gx0 = fx1 + 1, gx1 = min(fx1 + 2, f.nx);
    float cross[2], own[2], next[2];   // ce at fx1 (the face), fx0 and gx0 of rows fy0, fy1
#pragma unroll
    for (int r = 0; r < 2; r++) {
        const size_t o = (size_t)(r ? fy1 : fy0) * f.P;
        cross[r] = (float)f.ce[o + fx1];
        own[r] = (float)f.ce[o + fx0];
        next[r] = (float)f.ce[o + gx0];
    }
    float ce = 0.0f;
#pragma unroll
    for (int r = 0; r < 2; r++) {
        if (r && fy1 == fy0) break;
        float R = inv_or_big(cross[r]);
        if (fx1 > fx0) R += 0.5f * inv_or_big(own[r]);
        if (gx1 > gx0) R += 0.5f * inv_or_big(next[r]);
        ce += 1.0f / R;
    }
    return ce;
}
// y face between aggregates (I, J) and (I, J + 1)
template <typename T>
__device__ __forceinline__ float coarse_cn(const LevelT<T> &f, int cny, int I, int J) {
    if (J < 1 || J >= cny) return 0.0f;
    const int fx0 = 2 * I - 1, fx1 = min(2 * I, f.nx), fy0 = 2 * J - 1, fy1 = min(2 * J, f.ny);
    const int gy0 = fy1 + 1, gy1 = min(fy1 + 2, f.ny);
    float cross[2], own[2], next[2];   // cn at rows fy1 (the face), fy0 and gy0 of columns fx0, fx1
#pragma unroll
    for (int k = 0; k < 2; k++) {
        const int fx = k ? fx1 : fx0;
        cross[k] = (float)f.cn[(size_t)fy1 * f.P + fx];
        own[k] = (float)f.cn[(size_t)fy0 * f.P + fx];
        next[k] = (float)f.cn[(size_t)gy0 * f.P + fx];
    }
    float cn = 0.0f;
#pragma unroll
    for (int k = 0; k < 2; k++) {
        if (k && fx1 == fx0) break;
        float R = inv_or_big(cross[k]);
        if (fy1 > fy0) R += 0.5f * inv_or_big(own[k]);
        if (gy1 > gy0) R += 0.5f * inv_or_big(next[k]);
        cn += 1.0f / R;
    }
    return cn;
}
template <typename T>
__device__ __forceinline__ float coarse_extra(const LevelT<T> &f, int I, int J) {
    const int fx0 = 2 * I - 1, fx1 = min(2 * I, f.nx), fy0 = 2 * J - 1, fy1 = min(2 * J, f.ny);
    float e[2][2], ci[2];   // extra of the aggregate's cells; ce at fx0 of its rows
#pragma unroll
    for (int r = 0; r < 2; r++) {
        const size_t o = (size_t)(r ? fy1 : fy0) * f.P;
        e[r][0] = (float)f.extra[o + fx0];
        e[r][1] = (float)f.extra[o + fx1];
        ci[r] = (float)f.ce[o + fx0];
    }
    float ex = 0.0f;
#pragma unroll
    for (int r = 0; r < 2; r++) {
        if (r && fy1 == fy0) break;
#pragma unroll
        for (int k = 0; k < 2; k++) {
            if (k && fx1 == fx0) break;
            float v = e[r][k];
            if (v > 0.0f && fx1 > fx0) v = 1.0f / (1.0f / v + 0.5f * inv_or_big(ci[r]));
            ex += v;
        }
    }
    return ex;
}
// the whole coarse row of aggregate (I, J): its faces, remainder, diagonal
// and inverse diagonal (the west and south faces recomputed, not read back,
// so one pass builds a level)
template <typename T, typename TC>
__device__ void coarsen_cell(const LevelT<T> &f, const LevelT<TC> &c, int I, int J) {
    const size_t oc = (size_t)J * c.P + I;
    const float ce = coarse_ce(f, c.nx, I, J), cn = coarse_cn(f, c.ny, I, J), ex = coarse_extra(f, I, J);
    const float mc = ce + coarse_ce(f, c.nx, I - 1, J) + cn + coarse_cn(f, c.ny, I, J - 1) + ex;
    c.ce[oc] = (TC)ce;
    c.cn[oc] = (TC)cn;
    c.extra[oc] = (TC)ex;
    c.mc[oc] = (TC)mc;
    c.inv_mc[oc] = mc > 0.0f ? (TC)(1.0f / mc) : TC(0);
}

template <typename T, typename TC = T>
__global__ void k_coarsen(const LevelT<T> f, const LevelT<TC> c) {
    int I = blockIdx.x * blockDim.x + threadIdx.x + 1, J = blockIdx.y * blockDim.y + threadIdx.y + 1;
    if (I <= c.nx && J <= c.ny) coarsen_cell(f, c, I, J);
}

// Gauss-Seidel update of one node
template <typename T>
__device__ __forceinline__ T gs_node(const LevelT<T> &L, size_t o) {
    return (L.rhs[o] + L.ce[o] * L.x[o + 1] + L.ce[o - 1] * L.x[o - 1] + L.cn[o] * L.x[o + L.P]
            + L.cn[o - L.P] * L.x[o - L.P]) * L.inv_mc[o];
}

// Over-relaxed update x + om (g - x) of a node whose Gauss-Seidel value is g
// (om = 1: plain Gauss-Seidel, g itself)
template <typename T>
__device__ __forceinline__ T relax(T x, T g, T om) {
    return om == T(1) ? g : x + om * (g - x);
}

// Electrode strips.  Where the mesh is stretched along x next to the
// electrodes (x faces conducting several times better than y faces), point
// Gauss-Seidel barely damps error that is smooth in x and oscillates in y, and
// the coarse grids, which see the same stretching, do not remove it either: on
// the 1024^2 glow mesh (spacing 1/4 of the bulk's over ~28 cells at each
// electrode) these strips alone raise the CG iterations from 7 to 10.  Two
// more over-relaxed sweep pairs confined to the strip columns of the finest
// level (1..kl and kr..nx), in its post-smoothing, bring them back.
//
// They run as one launch (k_rb_strips) on row tiles with a halo of one row per
// half sweep.  So that no tile reads a value another tile of the launch
// writes, the kernel before it copies the strips, with their inner neighbour
// column, into a snapshot as it writes them, and k_rb_strips reads only the
// snapshot.  Strip s (0: columns 0..kl+1, 1: columns kr-1..nx+1), row gj
// (0..ny+1), column gi is at v[(s (ny + 2) + gj) w + gi - c0], c0 = 0 or
// kr - 1; the ghost entries stay zero.
template <typename T>
struct StripSnap {
    T *v = nullptr;   // no snapshot
    int kl = 0, kr = 0, w = 0;
    __device__ __forceinline__ bool holds(int gi) const {
        return (kl > 0 && gi <= kl + 1) || (kr > 0 && gi >= kr - 1);
    }
    __device__ __forceinline__ void put(int gi, int gj, int ny, T val) const {
        if (kl > 0 && gi <= kl + 1) v[(size_t)gj * w + gi] = val;
        if (kr > 0 && gi >= kr - 1) v[((size_t)(ny + 2) + gj) * w + (gi - kr + 1)] = val;
    }
};

// one red (color 0) or black (color 1) half sweep; zero_init: x starts at 0;
// om: relaxation factor (1 before the coarse-grid correction); sn: the strip
// snapshot to fill, before k_rb_strips
// Each thread owns the column pair (2t+1, 2t+2) of a row and updates the
// node of the swept colour in it, so every lane does useful FP64 work.
template <typename T>
__global__ void k_rb(const LevelT<T> L, int color, int zero_init, T om = T(1), StripSnap<T> sn = {}) {
    const int J = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int c0 = blockIdx.x * (2 * blockDim.x) + 2 * threadIdx.x + 1;
    if (J > L.ny || c0 > L.nx) return;
    const int I = ((c0 + J) & 1) == color ? c0 : c0 + 1, Io = I == c0 ? c0 + 1 : c0;
    if (zero_init && Io <= L.nx) L.x[(size_t)J * L.P + Io] = T(0);
    if (I > L.nx) return;
    const size_t o = (size_t)J * L.P + I;
    const T v = zero_init ? L.rhs[o] * L.inv_mc[o] : relax(L.x[o], gs_node(L, o), om);
    L.x[o] = v;
    if (sn.v && (sn.holds(c0) || sn.holds(c0 + 1))) {
        sn.put(I, J, L.ny, v);
        if (Io <= L.nx) sn.put(Io, J, L.ny, L.x[(size_t)J * L.P + Io]);
    }
}

// One red-black sweep pair from x = 0 in one pass: the red half sweep gives
// x = rhs / mc on the red nodes, and the black half sweep after it reads only
// those, so each black node forms its red neighbours' values from their rhs
// and 1/mc itself (the same products as the two launches, bit for bit; the
// ghost ring counts as zero, as x is there).  Threads own column pairs as in
// k_rb.
template <typename T>
__global__ void k_rb_pair0(const LevelT<T> L) {
    const int J = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int c0 = blockIdx.x * (2 * blockDim.x) + 2 * threadIdx.x + 1;
    if (J > L.ny || c0 > L.nx) return;
    auto xr = [&](int i, int j) -> T {
        if (i < 1 || i > L.nx || j < 1 || j > L.ny) return T(0);
        const size_t o = (size_t)j * L.P + i;
        return L.rhs[o] * L.inv_mc[o];
    };
#pragma unroll
    for (int d = 0; d < 2; d++) {
        const int I = c0 + d;
        if (I > L.nx) break;
        const size_t o = (size_t)J * L.P + I;
        L.x[o] = ((I + J) & 1) == 0
                     ? xr(I, J)
                     : (L.rhs[o] + L.ce[o] * xr(I + 1, J) + L.ce[o - 1] * xr(I - 1, J) + L.cn[o] * xr(I, J + 1)
                        + L.cn[o - L.P] * xr(I, J - 1)) * L.inv_mc[o];
    }
}

// The 2 FS_STRIP_PAIRS half sweeps (colours color0, 1 - color0, ...) over both
// strips of level L, from the snapshot sn, into L.x.  Grid (row tiles of
// STRIP_ROWS, 2 strips), 256 threads, strip_smem() bytes of shared memory.
#define STRIP_ROWS 32
template <typename T>
inline size_t strip_smem(int w) {
    return (size_t)5 * w * (STRIP_ROWS + 4 * FS_STRIP_PAIRS) * sizeof(T);
}
template <typename T>
__global__ void __launch_bounds__(256) k_rb_strips(const LevelT<T> L, const StripSnap<T> sn, int color0, T om) {
    constexpr int H = 2 * FS_STRIP_PAIRS, WY = STRIP_ROWS + 2 * H;
    extern __shared__ __align__(16) unsigned char sm_raw[];
    const int s = blockIdx.y;
    if ((s == 0 && sn.kl == 0) || (s == 1 && sn.kr == 0)) return;
    const int c0 = s == 0 ? 0 : sn.kr - 1;                    // first column held
    const int nc = s == 0 ? sn.kl + 2 : L.nx - sn.kr + 3;     // the strip, its inner neighbour, the ghost
    const int nu = nc - 2;                                    // columns updated: local 1..nu
    const int W = nc * WY;
    T *sx = (T *)sm_raw, *srhs = sx + W, *simc = srhs + W, *sce = simc + W, *scn = sce + W;
    const int gy0 = blockIdx.x * STRIP_ROWS + 1;
    const T *snap = sn.v + (size_t)s * (L.ny + 2) * sn.w;
    for (int q = threadIdx.x; q < W; q += blockDim.x) {
        const int k = q % nc, ly = q / nc, gi = c0 + k, gj = gy0 - H + ly;
        const bool row = gj >= 0 && gj <= L.ny + 1;
        const bool in = gj >= 1 && gj <= L.ny && gi >= 1 && gi <= L.nx;
        const size_t o = (size_t)gj * L.P + gi;
        sx[q] = in ? snap[(size_t)gj * sn.w + k] : T(0);
        srhs[q] = in ? L.rhs[o] : T(0);
        simc[q] = in ? L.inv_mc[o] : T(0);
        sce[q] = row ? L.ce[o] : T(0);
        scn[q] = row ? L.cn[o] : T(0);
    }
    __syncthreads();
    for (int st = 0; st < 2 * FS_STRIP_PAIRS; st++) {
        const int color = color0 ^ (st & 1), lo = st + 1, n = (WY - 2 - 2 * st) * nu;
        for (int q = threadIdx.x; q < n; q += blockDim.x) {
            const int k = 1 + q % nu, ly = lo + q / nu, gi = c0 + k, gj = gy0 - H + ly;
            if (gj < 1 || gj > L.ny || ((gi + gj) & 1) != color) continue;
            const int i = ly * nc + k;
            const T g = (srhs[i] + sce[i] * sx[i + 1] + sce[i - 1] * sx[i - 1] + scn[i] * sx[i + nc]
                         + scn[i - nc] * sx[i - nc]) * simc[i];
            sx[i] = relax(sx[i], g, om);
        }
        __syncthreads();
    }
    for (int q = threadIdx.x; q < STRIP_ROWS * nu; q += blockDim.x) {
        const int k = 1 + q % nu, ty = q / nu, gj = gy0 + ty;
        if (gj <= L.ny) L.x[(size_t)gj * L.P + c0 + k] = sx[(H + ty) * nc + k];
    }
}

// coarse rhs = sum over the aggregate of the fine residual rhs - M x.  The
// pre-smoothing ends with a black half sweep, after which every black node's
// residual is zero (to rounding), so only the red nodes are summed.
template <typename T>
__device__ __forceinline__ T resid(const LevelT<T> &L, size_t o) {
    return L.rhs[o] - (L.mc[o] * L.x[o] - L.ce[o] * L.x[o + 1] - L.ce[o - 1] * L.x[o - 1]
                       - L.cn[o] * L.x[o + L.P] - L.cn[o - L.P] * L.x[o - L.P]);
}
// (the coarse level may be FP32 under an FP64 fine level: the sum is formed
// in the fine level's type and rounded once)
template <typename T, typename TC = T>
__global__ void k_restrict(const LevelT<T> f, const LevelT<TC> c) {
    int I = blockIdx.x * blockDim.x + threadIdx.x + 1, J = blockIdx.y * blockDim.y + threadIdx.y + 1;
    if (I > c.nx || J > c.ny) return;
    const int fx0 = 2 * I - 1, fx1 = min(2 * I, f.nx), fy0 = 2 * J - 1, fy1 = min(2 * J, f.ny);
    T s = T(0);
    for (int fy = fy0; fy <= fy1; fy++)
        for (int fx = fx0; fx <= fx1; fx++)
            if (((fx + fy) & 1) == 0) s += resid(f, (size_t)fy * f.P + fx);
    c.rhs[(size_t)J * c.P + I] = (TC)s;
}
// Coarse-grid correction at fine node (gi, gj): cell-centred bilinear
// interpolation of the coarse iterate -- weights 9/16, 3/16, 3/16, 1/16 from
// the aggregate holding the node and its neighbours on the node's side --
// constant beyond the coarse grid's edge.  (With piecewise-constant
// prolongation and restriction the orders add up to the PDE's order and the
// V-cycle converges slowly; a second-order prolongation fixes that.)
template <typename T>
__device__ __forceinline__ T prolong_at(const T *cx, int cP, int cnx, int cny, int gi, int gj) {
    const int I = (gi + 1) >> 1, J = (gj + 1) >> 1;
    int In = (gi & 1) ? I - 1 : I + 1, Jn = (gj & 1) ? J - 1 : J + 1;
    if (In < 1 || In > cnx) In = I;
    if (Jn < 1 || Jn > cny) Jn = J;
    const T a = cx[(size_t)J * cP + I], b = cx[(size_t)J * cP + In], d = cx[(size_t)Jn * cP + I],
            e = cx[(size_t)Jn * cP + In];
    return T(0.5625) * a + T(0.1875) * (b + d) + T(0.0625) * e;
}

// Weight of coarse index I in prolong_at's interpolation at fine index fi
// (one direction; the 2D weight is the product): restriction with these
// weights is the transpose of the prolongation.
template <typename T>
__device__ __forceinline__ T prolong_w(int fi, int I, int cn) {
    const int Ic = (fi + 1) >> 1;
    int In = (fi & 1) ? Ic - 1 : Ic + 1;
    if (In < 1 || In > cn) In = Ic;
    return (I == Ic ? T(0.75) : T(0)) + (I == In ? T(0.25) : T(0));
}

template <typename T, typename TC = T>
__global__ void k_prolong(const LevelT<T> f, const LevelT<TC> c) {
    int I = blockIdx.x * blockDim.x + threadIdx.x + 1, J = blockIdx.y * blockDim.y + threadIdx.y + 1;
    if (I > f.nx || J > f.ny) return;
    f.x[(size_t)J * f.P + I] += (T)prolong_at(c.x, c.P, c.nx, c.ny, I, J);
}

// ---------------------------------------------- fused (temporally blocked) levels
// One CTA owns an MTX x MTY tile of a level plus a halo of 2*nu nodes held in
// shared memory.  Down: nu red-black sweeps from x = 0, the residual and its
// 2x2 aggregate sums (the coarse right-hand side) in one launch.  Up: the
// coarse correction and nu black-red sweeps in one launch.  With x = 0 the
// first sweep needs no neighbours, and each later sweep updates a region one
// ring smaller, so after 2*nu sweeps the tile (and, going down, its first
// ring) holds exactly the values the unfused sweeps produce.  The halo of the
// up kernel must hold the down-smoothed values of the neighbouring tiles, so
// down writes its iterate to xd and up reads xd and writes x: no tile reads
// a value another tile of the same launch writes.
#define MTX 32
#define MTY 16

template <typename T>
struct LvT {
    int nx, ny, P;
    const T *mc, *ce, *cn, *inv_mc;
    T *rhs, *x, *xd;
    T om;             // relaxation factor of the up (post-smoothing) sweeps
    StripSnap<T> sn;  // the up kernel fills it (the finest level, before k_rb_strips)
};

// Restriction.  FP64 levels below the finest (the FP64 solver's coarse levels
// on grids too small for FP32 ones) restrict with the transpose of the
// bilinear prolongation (it took the FP64 solver from 13 to 11 CG iterations
// at 1024^2 when that solver was plain CG and its coarse levels FP64); FP32
// levels sum the aggregate's residuals, which costs less and needs the same
// iterations under the flexible CG.  With the transpose the down kernel keeps
// one more halo ring than the sweeps need, so that the residuals of the
// tile's first ring, which the transpose reaches, are exact too.
template <typename T>
struct RestrictFW { static constexpr bool value = sizeof(T) == 8; };

// coarse right-hand side at (I, J) from the fine residuals (the red ones:
// black residuals vanish after the last, black, half sweep)
template <typename T>
__device__ __forceinline__ T restrict_at(const LevelT<T> &f, const LevelT<T> &c, int I, int J) {
    T s = T(0);
    if (RestrictFW<T>::value) {
        for (int fy = max(2 * J - 2, 1); fy <= min(2 * J + 1, f.ny); fy++)
            for (int fx = max(2 * I - 2, 1); fx <= min(2 * I + 1, f.nx); fx++)
                if (((fx + fy) & 1) == 0)
                    s += prolong_w<T>(fy, J, c.ny) * prolong_w<T>(fx, I, c.nx) * resid(f, (size_t)fy * f.P + fx);
    } else {
        for (int fy = 2 * J - 1; fy <= min(2 * J, f.ny); fy++)
            for (int fx = 2 * I - 1; fx <= min(2 * I, f.nx); fx++)
                if (((fx + fy) & 1) == 0) s += resid(f, (size_t)fy * f.P + fx);
    }
    return s;
}

// coarse right-hand sides by restrict_at (the unfused FP64 levels below the
// finest: the transpose of the prolongation, as the fused levels restrict)
template <typename T>
__global__ void k_restrict_t(const LevelT<T> f, const LevelT<T> c) {
    int I = blockIdx.x * blockDim.x + threadIdx.x + 1, J = blockIdx.y * blockDim.y + threadIdx.y + 1;
    if (I > c.nx || J > c.ny) return;
    c.rhs[(size_t)J * c.P + I] = restrict_at(f, c, I, J);
}

template <typename T, int NU>
__global__ void __launch_bounds__(256) k_mg_down(const LvT<T> f, const LvT<T> c) {
    constexpr bool FW = RestrictFW<T>::value;
    constexpr int E = FW ? 1 : 0;    // residual ring beyond the tile
    constexpr int H = 2 * NU + E, WX = MTX + 2 * H, WY = MTY + 2 * H, W = WX * WY;
    constexpr int RX = MTX + 2 * E;  // residual block: the tile (and its first ring)
    extern __shared__ __align__(16) unsigned char sm_raw[];
    T *sx = (T *)sm_raw, *srhs = sx + W, *simc = srhs + W, *smc = simc + W, *sce = smc + W,
      *scn = sce + W, *sr = scn + W;
    const int gx0 = blockIdx.x * MTX + 1, gy0 = blockIdx.y * MTY + 1;
    for (int q = threadIdx.x; q < W; q += blockDim.x) {
        const int lx = q % WX, ly = q / WX, gi = gx0 - H + lx, gj = gy0 - H + ly;
        const bool in = gi >= 1 && gj >= 1 && gi <= f.nx && gj <= f.ny;
        const bool arr = gi >= 0 && gj >= 0 && gi <= f.nx + 1 && gj <= f.ny + 1;
        const size_t o = (size_t)gj * f.P + gi;
        sx[q] = T(0);
        srhs[q] = in ? f.rhs[o] : T(0);
        simc[q] = in ? f.inv_mc[o] : T(0);
        smc[q] = in ? f.mc[o] : T(0);
        sce[q] = arr ? f.ce[o] : T(0);
        scn[q] = arr ? f.cn[o] : T(0);
    }
    __syncthreads();
    for (int s = 0; s < 2 * NU; s++) {
        const int color = s & 1, lo = s, hx = WX - 1 - s, hy = WY - 1 - s;
        const int nxr = hx - lo + 1, n = nxr * (hy - lo + 1);
        for (int q = threadIdx.x; q < n; q += blockDim.x) {
            const int lx = lo + q % nxr, ly = lo + q / nxr;
            const int gi = gx0 - H + lx, gj = gy0 - H + ly;
            if (((gi + gj) & 1) != color) continue;
            const int k = ly * WX + lx;
            if (s == 0) sx[k] = srhs[k] * simc[k];
            else sx[k] = (srhs[k] + sce[k] * sx[k + 1] + sce[k - 1] * sx[k - 1] + scn[k] * sx[k + WX]
                          + scn[k - WX] * sx[k - WX]) * simc[k];
        }
        __syncthreads();
    }
    for (int q = threadIdx.x; q < RX * (MTY + 2 * E); q += blockDim.x) {
        const int tx = q % RX - E, ty = q / RX - E, lx = H + tx, ly = H + ty;
        const int gi = gx0 + tx, gj = gy0 + ty;
        const int k = ly * WX + lx;
        T r = T(0);
        if (gi >= 1 && gj >= 1 && gi <= f.nx && gj <= f.ny) {
            if (((gi + gj) & 1) == 0)   // black residuals vanish after the last (black) sweep
                r = srhs[k] - (smc[k] * sx[k] - sce[k] * sx[k + 1] - sce[k - 1] * sx[k - 1]
                               - scn[k] * sx[k + WX] - scn[k - WX] * sx[k - WX]);
            if (tx >= 0 && ty >= 0 && tx < MTX && ty < MTY) f.xd[(size_t)gj * f.P + gi] = sx[k];
        }
        sr[q] = r;
    }
    __syncthreads();
    for (int q = threadIdx.x; q < (MTX / 2) * (MTY / 2); q += blockDim.x) {
        const int ci = q % (MTX / 2), cj = q / (MTX / 2);
        const int I = (gx0 - 1) / 2 + 1 + ci, J = (gy0 - 1) / 2 + 1 + cj;
        if (I > c.nx || J > c.ny) continue;
        if (!FW) {
            const int t0 = (2 * cj) * MTX + 2 * ci;
            c.rhs[(size_t)J * c.P + I] = sr[t0] + sr[t0 + 1] + sr[t0 + MTX] + sr[t0 + MTX + 1];
            continue;
        }
        T acc = T(0);
        for (int dy = -1; dy <= 2; dy++) {
            const int fy = 2 * J - 1 + dy;
            if (fy < 1 || fy > f.ny) continue;
            const T wy = prolong_w<T>(fy, J, c.ny);
            for (int dx = -1; dx <= 2; dx++) {
                const int fx = 2 * I - 1 + dx;
                if (fx < 1 || fx > f.nx) continue;
                acc += wy * prolong_w<T>(fx, I, c.nx) * sr[(2 * cj + dy + 1) * RX + 2 * ci + dx + 1];
            }
        }
        c.rhs[(size_t)J * c.P + I] = acc;
    }
}

template <typename T, int NU>
__global__ void __launch_bounds__(256) k_mg_up(const LvT<T> f, const LvT<T> c) {
    constexpr int H = 2 * NU, WX = MTX + 2 * H, WY = MTY + 2 * H, W = WX * WY;
    extern __shared__ __align__(16) unsigned char sm_raw[];
    T *sx = (T *)sm_raw, *srhs = sx + W, *simc = srhs + W, *sce = simc + W, *scn = sce + W;
    const int gx0 = blockIdx.x * MTX + 1, gy0 = blockIdx.y * MTY + 1;
    for (int q = threadIdx.x; q < W; q += blockDim.x) {
        const int lx = q % WX, ly = q / WX, gi = gx0 - H + lx, gj = gy0 - H + ly;
        const bool in = gi >= 1 && gj >= 1 && gi <= f.nx && gj <= f.ny;
        const bool arr = gi >= 0 && gj >= 0 && gi <= f.nx + 1 && gj <= f.ny + 1;
        const size_t o = (size_t)gj * f.P + gi;
        sx[q] = in ? f.xd[o] + prolong_at(c.x, c.P, c.nx, c.ny, gi, gj) : T(0);
        srhs[q] = in ? f.rhs[o] : T(0);
        simc[q] = in ? f.inv_mc[o] : T(0);
        sce[q] = arr ? f.ce[o] : T(0);
        scn[q] = arr ? f.cn[o] : T(0);
    }
    __syncthreads();
    for (int s = 0; s < 2 * NU; s++) {
        const int color = (s & 1) ? 0 : 1, lo = s + 1, hx = WX - 2 - s, hy = WY - 2 - s;
        const int nxr = hx - lo + 1, n = nxr * (hy - lo + 1);
        for (int q = threadIdx.x; q < n; q += blockDim.x) {
            const int lx = lo + q % nxr, ly = lo + q / nxr;
            const int gi = gx0 - H + lx, gj = gy0 - H + ly;
            if (((gi + gj) & 1) != color) continue;
            const int k = ly * WX + lx;
            sx[k] = relax(sx[k], (srhs[k] + sce[k] * sx[k + 1] + sce[k - 1] * sx[k - 1] + scn[k] * sx[k + WX]
                                  + scn[k - WX] * sx[k - WX]) * simc[k], f.om);
        }
        __syncthreads();
    }
    for (int q = threadIdx.x; q < MTX * MTY; q += blockDim.x) {
        const int tx = q % MTX, ty = q / MTX, gi = gx0 + tx, gj = gy0 + ty;
        if (gi <= f.nx && gj <= f.ny) {
            const T v = sx[(H + ty) * WX + H + tx];
            f.x[(size_t)gj * f.P + gi] = v;
            if (f.sn.v) f.sn.put(gi, gj, f.ny, v);
        }
    }
}

// V-cycle over levels [lb, dl] inside one CTA (levels of at most 32x32 nodes).
template <typename T>
struct BottomArgs {
    LevelT<T> L[FS_MG_MAX_LEVELS];
    int lb, nl, nu;
    int dl;              // k_bottom_smem: level solved exactly with the dense inverse ainv
    const T *ainv;       // (nx*ny)^2 of level dl, row-major over the compact index (J-1)*nx + I-1
    T om;                // relaxation factor of the post-smoothing sweeps
};
// The V-cycle over levels [lb, dl] with every level held in shared memory
// (operators, right-hand sides, iterates), and level dl -- the first with at
// most 64 unknowns -- solved exactly with its dense inverse (dense_inverse, once
// per solve) instead of recursing further: ~20 dependent phases instead of
// ~50.  Only the top level's right-hand side is read from, and its iterate
// written to, global memory.
template <typename T>
__host__ __device__ inline int bottom_smem_elems(const BottomArgs<T> &a) {
    int n = 0;
    for (int l = a.lb; l <= a.dl; l++) n += (a.L[l].nx + 2) * (a.L[l].ny + 2);
    return n;
}
// shared memory of k_bottom_smem: six arrays per level, the dense inverse and
// the residuals of the top level (the largest)
template <typename T>
inline size_t bottom_smem_bytes(const BottomArgs<T> &a) {
    return (6 * (size_t)bottom_smem_elems(a) + 64 * 64 + (size_t)(a.L[a.lb].nx + 2) * (a.L[a.lb].ny + 2)) * sizeof(T);
}
// first level at or below lb with at most 64 unknowns (the coarsest is 1 x 1)
template <typename T>
inline int bottom_dense_level(const BottomArgs<T> &a) {
    int l = a.lb;
    while (l < a.nl - 1 && a.L[l].nx * a.L[l].ny > 64) l++;
    return l;
}

// Inverse of the operator of level L (at most 64 unknowns), once per solve,
// by Gauss-Jordan elimination without pivoting (the operator is symmetric
// positive definite) on a 64 x 64 matrix (identity beyond the n unknowns),
// in FP32 on every level type: it is the preconditioner's exact coarsest
// solve, to FP32 accuracy.  The 1024 threads of the CTA hold the matrix in
// registers, thread t the four entries (t / 16, 4 (t % 16) .. + 3); pivot k
// reads row k and column k from shared buffers that the previous pivot's
// owners wrote (double-buffered: one barrier per pivot).  A node without a
// positive pivot gets x = 0.  ainv is row-major over the compact index
// (J-1)*nx + I-1.
#define DENSE_N 64
template <typename T>
__device__ void dense_inverse(const LevelT<T> &L, T *ainv) {
    __shared__ float rowb[2][DENSE_N], colb[2][DENSE_N];
    const int nx = L.nx, n = L.nx * L.ny, t = threadIdx.x;
    const int i = t >> 4, j0 = (t & 15) * 4;
    float a[4];
#pragma unroll
    for (int m = 0; m < 4; m++) {
        const int cidx = j0 + m;
        float v = 0.0f;
        if (i >= n || cidx >= n) {
            v = i == cidx ? 1.0f : 0.0f;
        } else {
            const int I = i % nx + 1, J = i / nx + 1;
            const size_t o = (size_t)J * L.P + I;
            if (cidx == i) v = (float)L.mc[o];
            else if (cidx == i + 1 && I < nx) v = -(float)L.ce[o];
            else if (cidx == i - 1 && I > 1) v = -(float)L.ce[o - 1];
            else if (cidx == i + nx) v = -(float)L.cn[o];
            else if (cidx == i - nx) v = -(float)L.cn[o - L.P];
        }
        a[m] = v;
    }
    auto publish = [&](int k, int b) {   // row k and column k as they stand
        if (i == k)
            for (int m = 0; m < 4; m++) rowb[b][j0 + m] = a[m];
        if (k >= j0 && k < j0 + 4) colb[b][i] = a[k - j0];
    };
    publish(0, 0);
    __syncthreads();
    for (int k = 0; k < n; k++) {
        const int b = k & 1;
        const float piv = colb[b][k], ip = piv > 0.0f ? 1.0f / piv : 0.0f;
        const float cip = colb[b][i] * ip;
#pragma unroll
        for (int m = 0; m < 4; m++) {
            const int j = j0 + m;
            const float rkj = rowb[b][j];
            if (i == k) a[m] = j == k ? ip : rkj * ip;
            else a[m] = j == k ? -cip : a[m] - cip * rkj;
        }
        if (k + 1 < n) publish(k + 1, b ^ 1);
        __syncthreads();
    }
#pragma unroll
    for (int m = 0; m < 4; m++) ainv[i * DENSE_N + j0 + m] = (T)a[m];
}
// The coarse levels of at most COARSEN_TAIL_CELLS aggregates, built one after
// another by a single CTA (a barrier between levels instead of a launch per
// level), then the dense inverse of level dl.
#define COARSEN_TAIL_CELLS 4096
template <typename T>
struct CoarsenTail {
    LevelT<T> L[FS_MG_MAX_LEVELS];
    int l0, nl;   // build levels l0 .. nl-1 (each from the one above)
    int dl;       // then invert level dl into ainv
    T *ainv;
};
template <typename T>
__global__ void __launch_bounds__(1024) k_coarsen_tail(const CoarsenTail<T> a) {
    for (int l = a.l0; l < a.nl; l++) {
        const LevelT<T> &f = a.L[l - 1], &c = a.L[l];
        for (int q = threadIdx.x; q < c.nx * c.ny; q += 1024) coarsen_cell(f, c, q % c.nx + 1, q / c.nx + 1);
        __syncthreads();   // the CTA's global writes of level l are visible to it
    }
    dense_inverse(a.L[a.dl], a.ainv);
}
// first level built by k_coarsen_tail: the finest with at most
// COARSEN_TAIL_CELLS aggregates, never level 0 (assembled, not coarsened)
template <typename T>
inline int coarsen_tail_level(const LevelT<T> *L, int nl) {
    int l = 1;
    while (l < nl && L[l].nx * L[l].ny > COARSEN_TAIL_CELLS) l++;
    return l;
}

template <typename T>
__global__ void __launch_bounds__(BOTTOM_THREADS) k_bottom_smem(const BottomArgs<T> a) {
    static_assert(BOTTOM_THREADS == BOTTOM_N * BOTTOM_N && BOTTOM_N == 32, "one node per thread");
    extern __shared__ __align__(16) unsigned char sm_raw[];
    __shared__ T scr[DENSE_N];
    const int t = threadIdx.x;
    int I, J;   // this thread's node of the level set by at()
    auto at = [&](const LevelT<T> &L) {
        const int sh = 32 - __clz(L.nx - 1);
        I = (t & ((1 << sh) - 1)) + 1;
        J = (t >> sh) + 1;
        return I <= L.nx && J <= L.ny;
    };
    const int tot = bottom_smem_elems(a);
    T *base = (T *)sm_raw;
    const int nd = a.L[a.dl].nx * a.L[a.dl].ny;
    T *sinv = base + 6 * tot;   // DENSE_N x DENSE_N, transposed: sinv[j * DENSE_N + i] = ainv[i][j]
    T *sres = sinv + DENSE_N * DENSE_N;   // fine residuals of the level being restricted
    LevelT<T> S[FS_MG_MAX_LEVELS];
    {
        int off = 0;
        for (int l = a.lb; l <= a.dl; l++) {
            const LevelT<T> &G = a.L[l];
            LevelT<T> &L = S[l];
            L.nx = G.nx; L.ny = G.ny; L.P = G.nx + 2;
            L.mc = base + off; L.ce = base + tot + off; L.cn = base + 2 * tot + off;
            L.inv_mc = base + 3 * tot + off; L.rhs = base + 4 * tot + off; L.x = base + 5 * tot + off;
            L.extra = nullptr; L.res = nullptr;
            const int n = (G.nx + 2) * (G.ny + 2);
            for (int q = t; q < n; q += BOTTOM_THREADS) {
                const int i = q % (G.nx + 2), j = q / (G.nx + 2);
                const size_t o = (size_t)j * G.P + i;
                L.mc[q] = G.mc[o]; L.ce[q] = G.ce[o]; L.cn[q] = G.cn[o]; L.inv_mc[q] = G.inv_mc[o];
                L.rhs[q] = l == a.lb ? G.rhs[o] : T(0);
                L.x[q] = T(0);
            }
            off += n;
        }
        for (int q = t; q < DENSE_N * DENSE_N; q += BOTTOM_THREADS)
            sinv[(q & (DENSE_N - 1)) * DENSE_N + (q >> 6)] = a.ainv[q];
    }
    __syncthreads();
    auto sweep = [&](const LevelT<T> &L, int color, int zero, T om) {
        if (at(L)) {
            const int o = J * L.P + I;
            if (((I + J) & 1) == color)
                L.x[o] = zero ? L.rhs[o] * L.inv_mc[o] : relax(L.x[o], gs_node(L, (size_t)o), om);
            else if (zero) L.x[o] = T(0);
        }
        __syncthreads();
    };
    for (int l = a.lb; l < a.dl; l++) {
        const LevelT<T> f = S[l], c = S[l + 1];
        sweep(f, 0, 1, T(1));
        sweep(f, 1, 0, T(1));
        for (int it = 1; it < a.nu; it++) { sweep(f, 0, 0, T(1)); sweep(f, 1, 0, T(1)); }
        if (RestrictFW<T>::value) {   // each fine residual once, then the transpose weights
            if (at(f)) {
                const int o = J * f.P + I;
                sres[o] = ((I + J) & 1) == 0 ? resid(f, (size_t)o) : T(0);
            }
            __syncthreads();
            if (at(c)) {
                T s = T(0);
                for (int fy = max(2 * J - 2, 1); fy <= min(2 * J + 1, f.ny); fy++) {
                    const T wy = prolong_w<T>(fy, J, c.ny);
                    for (int fx = max(2 * I - 2, 1); fx <= min(2 * I + 1, f.nx); fx++)
                        s += wy * prolong_w<T>(fx, I, c.nx) * sres[fy * f.P + fx];
                }
                c.rhs[J * c.P + I] = s;
            }
        } else {
            if (at(c)) c.rhs[J * c.P + I] = restrict_at(f, c, I, J);
        }
        __syncthreads();
    }
    {   // level dl: x = A^-1 rhs with the precomputed dense inverse
        const LevelT<T> c = S[a.dl];
        if (t < nd) scr[t] = c.rhs[(t / c.nx + 1) * c.P + t % c.nx + 1];
        __syncthreads();
        if (t < nd) {
            T acc = T(0);
            for (int j = 0; j < nd; j++) acc += sinv[j * DENSE_N + t] * scr[j];
            c.x[(t / c.nx + 1) * c.P + t % c.nx + 1] = acc;
        }
        __syncthreads();
    }
    for (int l = a.dl - 1; l >= a.lb; l--) {
        const LevelT<T> f = S[l], c = S[l + 1];
        if (at(f)) f.x[J * f.P + I] += prolong_at(c.x, c.P, c.nx, c.ny, I, J);
        __syncthreads();
        for (int it = 0; it < a.nu; it++) { sweep(f, 1, 0, a.om); sweep(f, 0, 0, a.om); }
    }
    const LevelT<T> G = a.L[a.lb], L = S[a.lb];
    if (at(L)) G.x[(size_t)J * G.P + I] = L.x[J * L.P + I];
}

// grid-stride loop over the interior nodes; o is the node's field offset
// (32-bit index arithmetic: grids are limited to 2^28 nodes)
#define CG_NODES(a, ...)                                                                   \
    for (unsigned q_ = blockIdx.x * 256u + threadIdx.x; q_ < (unsigned)((a).nx * (a).ny); \
         q_ += gridDim.x * 256u) {                                                         \
        const unsigned j_ = q_ / (unsigned)(a).nx;                                         \
        const size_t o = (size_t)(j_ + 1) * (a).P + (q_ - j_ * (unsigned)(a).nx + 1);      \
        __VA_ARGS__                                                                        \
    }

// grid-stride loop over rows 1..ny of a pitched FP32 field in float4 steps
// (ghost columns and row padding included; o is the offset of the first of
// the four elements, a multiple of 4 since the pitch is a multiple of 32)
#define CG_VEC4(a, ...)                                                                    \
    for (unsigned t4_ = blockIdx.x * 256u + threadIdx.x; t4_ < (unsigned)((a).ny * (a).P / 4); \
         t4_ += gridDim.x * 256u) {                                                        \
        const size_t o = (size_t)(a).P + 4 * (size_t)t4_;                                  \
        __VA_ARGS__                                                                        \
    }

// phi(interior) += d ; ph_mi = phi (lapl_lib.F90:112-119), only after convergence
__global__ void k_phi_update(double *ph, double *phm, const double *x, int nx, int ny, int P,
                             const Ctrl *ctrl) {
    if (!ctrl->cg_done || ctrl->cg_fail) return;
    // 32-bit index arithmetic (grids are limited to 2^28 nodes): a 64-bit
    // division per element costs more than the update
    const unsigned n = (unsigned)(ny + 2) * (unsigned)P;
    for (unsigned o = blockIdx.x * blockDim.x + threadIdx.x; o < n; o += gridDim.x * blockDim.x) {
        const int gj = (int)(o / (unsigned)P), gi = (int)(o - (unsigned)gj * (unsigned)P);
        double v = ph[o];
        if (gi >= 1 && gi <= nx && gj >= 1 && gj <= ny) v = v + x[o];
        ph[o] = v;
        phm[o] = v;
    }
}

inline dim3 grid2(int nx, int ny, dim3 b) { return dim3((nx + b.x - 1) / b.x, (ny + b.y - 1) / b.y); }

// device views of an FP32 level
inline LevelT<float> level_f(const MGLevelF &m) {
    LevelT<float> L;
    L.nx = m.nx; L.ny = m.ny; L.P = m.pitch;
    L.mc = m.mc; L.ce = m.ce; L.cn = m.cn; L.extra = m.extra; L.inv_mc = m.inv_mc;
    L.rhs = m.rhs; L.x = m.x; L.res = nullptr;
    return L;
}
inline LvT<float> lvt_f(const MGLevelF &m) {
    LvT<float> L;
    L.nx = m.nx; L.ny = m.ny; L.P = m.pitch;
    L.mc = m.mc; L.ce = m.ce; L.cn = m.cn; L.inv_mc = m.inv_mc; L.rhs = m.rhs; L.x = m.x; L.xd = m.xd;
    L.om = (float)FS_MG_OMEGA_POST;
    return L;
}

// the strip snapshot of a context (kl, kr = 0 for a side without a strip)
template <typename T>
inline StripSnap<T> strip_snap(const fs_ctx *c, T *v) {
    StripSnap<T> s;
    s.v = v;
    s.kl = c->strip_kl;
    s.kr = c->strip_kr <= c->nx ? c->strip_kr : 0;
    s.w = c->strip_w;
    return s;
}
inline bool has_strips(const fs_ctx *c) { return c->strip_kl > 0 || c->strip_kr <= c->nx; }

template <typename T>
size_t mg_down_smem(int nu) {
    const int e = RestrictFW<T>::value ? 1 : 0;
    size_t W = (size_t)(MTX + 4 * nu + 2 * e) * (MTY + 4 * nu + 2 * e);
    return (6 * W + (size_t)(MTX + 2 * e) * (MTY + 2 * e)) * sizeof(T);
}
template <typename T>
size_t mg_up_smem(int nu) {
    size_t W = (size_t)(MTX + 4 * nu) * (MTY + 4 * nu);
    return 5 * W * sizeof(T);
}


// ------------------------------------------------------------ x-line smoother
// Zebra line Gauss-Seidel along x, for grids whose x faces conduct several
// times better than their y faces across the whole grid (a square domain on a
// grid with nx > ny, a mesh stretched along x far beyond the electrode
// strips).  There point Gauss-Seidel barely damps error that is smooth along
// x, and the 2x2 aggregates keep the cells' aspect ratio on every level; a
// line solve removes that error exactly.  Each row of one parity is solved
// for its x couplings given the rows above and below:
//   -ce(i-1) x(i-1) + mc(i) x(i) - ce(i) x(i+1) = rhs(i) + cn(i) x_n(i) + cn_s(i) x_s(i).
//
// One CTA per row, xline_threads(nx) threads (32..256, about one per 8
// nodes).  The row is cut into K = ceil(nx / m) chunks of m = ceil(nx /
// threads) nodes; the last node of a chunk is its separator.  Thread k
// eliminates its chunk's interior (Thomas) for the right-hand side and for
// unit values of the two separators that bound it, which leaves a
// tridiagonal system in the K separators, solved by parallel cyclic
// reduction in shared memory; the interior follows from the separators.  The
// matrix is an M-matrix with a dominant diagonal, so neither elimination
// pivots.  The row is staged in five shared-memory arrays (coalesced loads
// and stores; the eliminations work in place).  A single warp per row was
// tried first: with one warp streaming a whole row the loads and stores are
// latency-bound (a 1024-node row took ~13 us per half sweep).
#define XL_SMEM_MAX (200 * 1024)
// Only the finest level smooths with x-lines; the coarser levels keep the
// point sweeps (fused level kernels).  Measured on the mixed solver, CG
// iterations per step (301x173 glow / 1024^2 tanh mesh / 1024^2 glow): point
// smoothing 13 / 8 / 7; x-lines on every level above the bottom 11 / 11 / 11;
// on the finest level only 8 / 7.8 / 8 with plain post-smoothing, 9 / 7 / 7
// over-relaxed by 1.15, 9 / 8 / 8 by 1.3 -- plain it is.  Sweep pairs on the
// finest level (pre + post, 301x173, iterations and ms per step, FP64 /
// mixed): 2 + 2: 8, 1.72 / 8, 1.27; 1 + 2: 8, 1.53 / 8, 1.12; 1 + 1: 9, 1.49 /
// 10, 1.14; point smoothing 15, 1.70 / 13, 1.06.  Both solvers take 1 + 2
// (fs_mg_pre0 pre-sweep pairs).
#define FS_XL_OMEGA_POST 1.0

// Thread k works on the nodes k m + 1 .. (k + 1) m of the row, so a plain
// layout would put a warp's accesses m words apart -- all on one bank for
// m = 32.  Element i is stored at i + i / 32 instead.
__host__ __device__ __forceinline__ int xl_idx(int i) { return i + (i >> 5); }
inline int xline_row_len(int nx) { return xl_idx(nx + 1) + 1; }
inline int xline_threads(int nx) {
    int t = 32;
    while (t < 256 && t * 8 < nx) t *= 2;
    return t;
}
// The line solves compute in FP32 on either level type: they only shape the
// preconditioner, and FP64 divisions, of which a row solve has one or two
// per node, would make the FP64 solver's finest level ~2x dearer than its
// point sweeps on this GPU.
inline size_t xline_smem(int nx) {
    return ((size_t)5 * xline_row_len(nx) + (size_t)5 * xline_threads(nx)) * sizeof(float);
}
// rows of up to this many nodes take x-line smoothing
inline bool xline_fits(int nx) { return xline_smem(nx) <= XL_SMEM_MAX; }

// one half sweep over the rows J = 1 + color, 3 + color, ... (grid: one CTA
// per row); zero_init: x starts at 0 (the other parity's rows are zeroed and
// not read); om: over-relaxation of the line solution
template <typename T>
__global__ void __launch_bounds__(256) k_xline(const LevelT<T> L, int color, int zero_init, T om) {
    typedef float XF;   // arithmetic of the line solve
    extern __shared__ __align__(16) unsigned char xl_raw[];
    const int nx = L.nx, P = L.P, t = threadIdx.x, NT = blockDim.x;
    const int J = 1 + color + 2 * (int)blockIdx.x;
    if (J > L.ny) return;   // whole CTA
    const int R = xl_idx(nx + 1) + 1;
    XF *sb = reinterpret_cast<XF *>(xl_raw);   // mc, then the eliminated c'
    XF *sc = sb + R;             // ce: the face between i and i + 1 (0 at both ends)
    XF *sd = sc + R;             // right-hand side, then y, then the line solution
    XF *sa = sd + R;             // response to the chunk's left separator
    XF *sz = sa + R;             // response to the chunk's own separator
    XF *rA = sz + R, *rB = rA + NT, *rC = rB + NT, *rD = rC + NT, *sx = rD + NT;   // the separators' system
    const size_t row = (size_t)J * P;
    for (int i = t; i <= nx + 1; i += NT) {
        const size_t o = row + i;
        const bool in = i >= 1 && i <= nx;
        T d = T(0);
        if (in) {
            d = L.rhs[o];
            if (!zero_init) d += L.cn[o] * L.x[o + P] + L.cn[o - P] * L.x[o - P];
        }
        sb[xl_idx(i)] = in ? (XF)L.mc[o] : XF(1);
        sc[xl_idx(i)] = i >= 1 && i < nx ? (XF)L.ce[o] : XF(0);
        sd[xl_idx(i)] = (XF)d;
    }
    if (zero_init && J + 1 <= L.ny)
        for (int i = 1 + t; i <= nx; i += NT) L.x[row + P + i] = T(0);
    __syncthreads();
    const int m = (nx + NT - 1) / NT, K = (nx + m - 1) / m;
    const int s0 = t * m + 1, e0 = min((t + 1) * m, nx);
    const int mi = t < K ? e0 - s0 : 0;
    // interior rows s0 .. e0-1, in place: sb <- c', sd <- y, sa <- alpha, sz <- beta
    for (int q = 0; q < mi; q++) {
        const int i = s0 + q;
        const XF a = -sc[xl_idx(i - 1)], c = q == mi - 1 ? XF(0) : -sc[xl_idx(i)];
        const XF inv = XF(1) / (q > 0 ? sb[xl_idx(i)] - a * sb[xl_idx(i - 1)] : sb[xl_idx(i)]);
        XF ry = sd[xl_idx(i)], ra = q == 0 ? -a : XF(0), rz = q == mi - 1 ? sc[xl_idx(i)] : XF(0);
        if (q > 0) {
            ry -= a * sd[xl_idx(i - 1)];
            ra -= a * sa[xl_idx(i - 1)];
            rz -= a * sz[xl_idx(i - 1)];
        }
        sb[xl_idx(i)] = c * inv;
        sd[xl_idx(i)] = ry * inv;
        sa[xl_idx(i)] = ra * inv;
        sz[xl_idx(i)] = rz * inv;
    }
    for (int q = mi - 2; q >= 0; q--) {
        const int i = s0 + q;
        const XF cpv = sb[xl_idx(i)];
        sd[xl_idx(i)] -= cpv * sd[xl_idx(i + 1)];
        sa[xl_idx(i)] -= cpv * sa[xl_idx(i + 1)];
        sz[xl_idx(i)] -= cpv * sz[xl_idx(i + 1)];
    }
    __syncthreads();
    // the separator equation of each chunk, in terms of the separators
    if (t < K) {
        const XF a = -sc[xl_idx(e0 - 1)], c = -sc[xl_idx(e0)];
        XF A = a, B = sb[xl_idx(e0)], C = c, D = sd[xl_idx(e0)];
        if (mi > 0) {
            const int il = e0 - 1;
            A = a * sa[xl_idx(il)];
            B += a * sz[xl_idx(il)];
            D -= a * sd[xl_idx(il)];
        }
        if (t + 1 < K && e0 + 1 < min((t + 2) * m, nx)) {
            const int f = e0 + 1;   // the next chunk's first interior node (it has one)
            B += c * sa[xl_idx(f)];
            C = c * sz[xl_idx(f)];
            D -= c * sd[xl_idx(f)];
        }
        rA[t] = t == 0 ? XF(0) : A;
        rB[t] = B;
        rC[t] = t + 1 < K ? C : XF(0);
        rD[t] = D;
    }
    __syncthreads();
    // parallel cyclic reduction: after the stride passes every equation holds
    // its separator alone
    for (int st = 1; st < K; st <<= 1) {
        XF nA = XF(0), nB = XF(1), nC = XF(0), nD = XF(0);
        if (t < K) {
            const int lo = t - st, hi = t + st;
            const XF Al = lo >= 0 ? rA[lo] : XF(0), Bl = lo >= 0 ? rB[lo] : XF(1), Cl = lo >= 0 ? rC[lo] : XF(0),
                    Dl = lo >= 0 ? rD[lo] : XF(0);
            const XF Ah = hi < K ? rA[hi] : XF(0), Bh = hi < K ? rB[hi] : XF(1), Ch = hi < K ? rC[hi] : XF(0),
                    Dh = hi < K ? rD[hi] : XF(0);
            const XF k1 = rA[t] / Bl, k2 = rC[t] / Bh;
            nA = -Al * k1;
            nB = rB[t] - Cl * k1 - Ah * k2;
            nC = -Ch * k2;
            nD = rD[t] - Dl * k1 - Dh * k2;
        }
        __syncthreads();
        if (t < K) {
            rA[t] = nA;
            rB[t] = nB;
            rC[t] = nC;
            rD[t] = nD;
        }
        __syncthreads();
    }
    if (t < K) sx[t] = rD[t] / rB[t];
    __syncthreads();
    if (t < K) {
        const XF xr = sx[t], xl = t > 0 ? sx[t - 1] : XF(0);
        for (int q = 0; q < mi; q++) {
            const int i = s0 + q;
            sd[xl_idx(i)] = sd[xl_idx(i)] + sa[xl_idx(i)] * xl + sz[xl_idx(i)] * xr;
        }
        sd[xl_idx(e0)] = xr;
    }
    __syncthreads();
    for (int i = 1 + t; i <= nx; i += NT) {
        const size_t o = row + i;
        const T v = (T)sd[xl_idx(i)];
        L.x[o] = zero_init ? v : relax(L.x[o], v, om);
    }
}

// coarse rhs = the aggregate's sum of the fine residual after x-line
// pre-smoothing, which ends with the even rows' half sweep: their residual is
// zero (to rounding), so only the odd row 2J - 1 of each aggregate is summed
template <typename T, typename TC = T>
__global__ void k_restrict_odd(const LevelT<T> f, const LevelT<TC> c) {
    int I = blockIdx.x * blockDim.x + threadIdx.x + 1, J = blockIdx.y * blockDim.y + threadIdx.y + 1;
    if (I > c.nx || J > c.ny) return;
    const int fx0 = 2 * I - 1, fx1 = min(2 * I, f.nx), fy = 2 * J - 1;
    T s = T(0);
    for (int fx = fx0; fx <= fx1; fx++) s += resid(f, (size_t)fy * f.P + fx);
    c.rhs[(size_t)J * c.P + I] = (TC)s;
}


// Dynamic shared memory limits of the strip and x-line kernels at type T.
// The templates live in an anonymous namespace, so every translation unit
// that launches them has its own instances with their own attributes: each
// sets the limits of the instances it launches.
template <typename T>
inline cudaError_t mg_level_smem_limits(const fs_ctx *c) {
    cudaError_t e = cudaSuccess;
    if (has_strips(c)) e = fs_smem_limit((const void *)k_rb_strips<T>, strip_smem<T>(c->strip_w));
    if (e == cudaSuccess && c->mg_xline) e = fs_smem_limit((const void *)k_xline<T>, xline_smem(c->nx));
    return e;
}

// x-line half sweeps on one level, timed and counted like the other levels'
// kernels: `pairs` sweep pairs, odd rows then even rows (pre-smoothing, the
// first from x = 0), or even rows then odd rows (post-smoothing, over-relaxed)
template <typename T>
inline void xline_pairs(fs_ctx *c, const LevelT<T> &f, int pairs, bool pre, T om) {
    for (int it = 0; it < pairs; it++)
        for (int h = 0; h < 2; h++) {
            const int color = pre ? h : 1 - h, rows = (f.ny + 1 - color) / 2;
            if (rows == 0) continue;   // a level one row high has no even rows
            fs_prof_begin(c, PROF_SMOOTH);
            k_xline<T><<<rows, xline_threads(f.nx), xline_smem(f.nx), c->stream>>>(f, color,
                                                                                  pre && it == 0 && h == 0, om);
            fs_prof_end(c);
        }
}

}  // namespace
