// fs_lpc.cu -- kernels of the learned Poisson preconditioner (see fs_lpc.cuh).
//
// Network (a two-level U-Net, ~250k parameters, 3x3 convolutions, ReLU):
//   e1a 16->32, e1b 32->32                    (full NN grid; e1b output = skip s1)
//   pool, e2a 32->64, e2b 64->64              (1/2; e2b output = skip s2)
//   pool, b1 64->64, b2 64->64                (1/4)
//   up, d2 [up(b2), s2] 128->64               (1/2)
//   up, d1 [up(d2), s1] 96->32                (full)
//   out 32->8 (channel 0 is the prediction, no ReLU)
// Activations are NHWC BF16 tensors [B][H][W][C]; every convolution is an
// implicit GEMM on the tensor cores (mma.sync m16n8k16, BF16 operands, FP32
// accumulation) with zero padding at the grid edge.  Backward: data gradients
// by the transposed implicit GEMM, weight gradients by a split-K GEMM over
// pixels with a fixed-order reduction; Adam on FP32 master weights, from
// which the two BF16 copies (forward [tap][cout][cin], backward
// [tap][cin][cout]) are refreshed.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <vector>

#include "fs_lpc.cuh"

typedef __nv_bfloat16 bf16;

namespace {

__device__ __forceinline__ uint32_t ld_b32(const bf16 *p) { return *reinterpret_cast<const uint32_t *>(p); }
__device__ __forceinline__ uint32_t pack2(bf16 lo, bf16 hi) {
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}
__device__ __forceinline__ void mma_bf16(float *c, const uint32_t *a, const uint32_t *b) {
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};\n"
                 : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

struct Pix {
    int b, y, x;
    bool ok;
};
__device__ __forceinline__ Pix pix_of(long p, int H, int W, long P) {
    Pix q;
    q.ok = p < P;
    long pp = q.ok ? p : 0;
    q.b = (int)(pp / ((long)H * W));
    int rem = (int)(pp - (long)q.b * H * W);
    q.y = rem / W;
    q.x = rem - q.y * W;
    return q;
}
// pixel index of the neighbour at tap t (dy = t/3-1, dx = t%3-1), -1 outside
__device__ __forceinline__ long nbr(const Pix &q, int t, int H, int W) {
    const int y = q.y + t / 3 - 1, x = q.x + t % 3 - 1;
    if (!q.ok || y < 0 || y >= H || x < 0 || x >= W) return -1;
    return ((long)q.b * H + y) * W + x;
}

struct ConvArgs {
    const bf16 *in1, *in2;       // input channels [0, c1) from in1, [c1, c1 + c2) from in2
    int c1, c2, cout;
    const bf16 *w;               // forward: [9][cout][cin]; backward data: [9][cin][cout]
    const float *bias;
    bf16 *out;                   // BF16 output, or
    float *out32;                // FP32 output (last layer)
    const bf16 *mask1, *mask2;   // backward data: ReLU masks of the two input tensors (may be null)
    bf16 *dout2;                 // backward data: gradient of in2's channels
    int relu;
    int B, H, W;
};

// Forward 3x3 convolution.  A warp computes 16 output pixels x 8*NT output
// channels; the warps of a CTA split the output channels of one 16-pixel tile
// (wpt = cout / (8 NT) warps per tile, 4 / wpt tiles per CTA), which keeps
// enough warps in flight on the small grids of the coarse levels.
template <int NT>
__global__ void __launch_bounds__(128) k_conv_fwd(const ConvArgs a) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, tq = lane & 3;
    const int wpt = a.cout / (8 * NT), tpc = 4 / wpt;
    const int co_base = (warp % wpt) * 8 * NT;
    const long P = (long)a.B * a.H * a.W;
    const long p0 = ((long)blockIdx.x * tpc + warp / wpt) * 16 + g, p1 = p0 + 8;
    const Pix q0 = pix_of(p0, a.H, a.W, P), q1 = pix_of(p1, a.H, a.W, P);
    const int cin = a.c1 + a.c2;
    float acc[NT][4];
#pragma unroll
    for (int j = 0; j < NT; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
    for (int t = 0; t < 9; t++) {
        const long n0 = nbr(q0, t, a.H, a.W), n1 = nbr(q1, t, a.H, a.W);
        for (int ci0 = 0; ci0 < cin; ci0 += 16) {
            const bf16 *src;
            int cs, cc;
            if (ci0 < a.c1) { src = a.in1; cs = a.c1; cc = ci0; }
            else { src = a.in2; cs = a.c2; cc = ci0 - a.c1; }
            uint32_t af[4];
            const int ca = cc + tq * 2;
            af[0] = n0 >= 0 ? ld_b32(src + n0 * cs + ca) : 0u;
            af[1] = n1 >= 0 ? ld_b32(src + n1 * cs + ca) : 0u;
            af[2] = n0 >= 0 ? ld_b32(src + n0 * cs + ca + 8) : 0u;
            af[3] = n1 >= 0 ? ld_b32(src + n1 * cs + ca + 8) : 0u;
#pragma unroll
            for (int j = 0; j < NT; j++) {
                const bf16 *wr = a.w + ((size_t)t * a.cout + co_base + j * 8 + g) * cin + ci0 + tq * 2;
                uint32_t bfr[2] = {ld_b32(wr), ld_b32(wr + 8)};
                mma_bf16(acc[j], af, bfr);
            }
        }
    }
#pragma unroll
    for (int j = 0; j < NT; j++) {
        const int co = co_base + j * 8 + tq * 2;
        float v[4] = {acc[j][0] + a.bias[co], acc[j][1] + a.bias[co + 1], acc[j][2] + a.bias[co],
                      acc[j][3] + a.bias[co + 1]};
        if (a.relu)
            for (int k = 0; k < 4; k++) v[k] = fmaxf(v[k], 0.0f);
        if (a.out32) {
            if (q0.ok) { a.out32[p0 * a.cout + co] = v[0]; a.out32[p0 * a.cout + co + 1] = v[1]; }
            if (q1.ok) { a.out32[p1 * a.cout + co] = v[2]; a.out32[p1 * a.cout + co + 1] = v[3]; }
        } else {
            if (q0.ok) *reinterpret_cast<uint32_t *>(a.out + p0 * a.cout + co) =
                pack2(__float2bfloat16_rn(v[0]), __float2bfloat16_rn(v[1]));
            if (q1.ok) *reinterpret_cast<uint32_t *>(a.out + p1 * a.cout + co) =
                pack2(__float2bfloat16_rn(v[2]), __float2bfloat16_rn(v[3]));
        }
    }
}

// Backward data: dIn[q][ci] = sum_t sum_co dOut[q - off_t][co] W[t][co][ci],
// with the ReLU mask of the input tensor applied in the epilogue.
// A CTA computes 16 pixels; its 4 warps take 8*NT input channels each
// (NT = cin / 32).  cout a multiple of 16.
template <int NT>
__global__ void __launch_bounds__(128) k_conv_bwd_data(const ConvArgs a, const bf16 *dout) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, tq = lane & 3;
    const int ci_base = warp * 8 * NT;
    const long P = (long)a.B * a.H * a.W;
    const long p0 = (long)blockIdx.x * 16 + g, p1 = p0 + 8;
    const Pix q0 = pix_of(p0, a.H, a.W, P), q1 = pix_of(p1, a.H, a.W, P);
    const int cin = a.c1 + a.c2, cout = a.cout;
    float acc[NT][4];
#pragma unroll
    for (int j = 0; j < NT; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
    for (int t = 0; t < 9; t++) {
        const long n0 = nbr(q0, 8 - t, a.H, a.W), n1 = nbr(q1, 8 - t, a.H, a.W);
        for (int co0 = 0; co0 < cout; co0 += 16) {
            uint32_t af[4];
            const int ca = co0 + tq * 2;
            af[0] = n0 >= 0 ? ld_b32(dout + n0 * cout + ca) : 0u;
            af[1] = n1 >= 0 ? ld_b32(dout + n1 * cout + ca) : 0u;
            af[2] = n0 >= 0 ? ld_b32(dout + n0 * cout + ca + 8) : 0u;
            af[3] = n1 >= 0 ? ld_b32(dout + n1 * cout + ca + 8) : 0u;
#pragma unroll
            for (int j = 0; j < NT; j++) {
                const bf16 *wr = a.w + ((size_t)t * cin + ci_base + j * 8 + g) * cout + ca;
                uint32_t bfr[2] = {ld_b32(wr), ld_b32(wr + 8)};
                mma_bf16(acc[j], af, bfr);
            }
        }
    }
#pragma unroll
    for (int j = 0; j < NT; j++) {
        const int ci = ci_base + j * 8 + tq * 2;
        bf16 *dst;
        const bf16 *msk;
        int cs, cc;
        if (ci < a.c1) { dst = a.out; msk = a.mask1; cs = a.c1; cc = ci; }
        else { dst = a.dout2; msk = a.mask2; cs = a.c2; cc = ci - a.c1; }
        float v[4] = {acc[j][0], acc[j][1], acc[j][2], acc[j][3]};
        if (msk) {
            if (q0.ok) {
                if (!(__bfloat162float(msk[p0 * cs + cc]) > 0.0f)) v[0] = 0.0f;
                if (!(__bfloat162float(msk[p0 * cs + cc + 1]) > 0.0f)) v[1] = 0.0f;
            }
            if (q1.ok) {
                if (!(__bfloat162float(msk[p1 * cs + cc]) > 0.0f)) v[2] = 0.0f;
                if (!(__bfloat162float(msk[p1 * cs + cc + 1]) > 0.0f)) v[3] = 0.0f;
            }
        }
        if (q0.ok) *reinterpret_cast<uint32_t *>(dst + p0 * cs + cc) =
            pack2(__float2bfloat16_rn(v[0]), __float2bfloat16_rn(v[1]));
        if (q1.ok) *reinterpret_cast<uint32_t *>(dst + p1 * cs + cc) =
            pack2(__float2bfloat16_rn(v[2]), __float2bfloat16_rn(v[3]));
    }
}

// Backward data of the last layer (one live output channel): CUDA cores.
// dIn[q][ci] = sum_t dy[q - off_t] W[t][0][ci], masked by the input's ReLU.
__global__ void k_out_bwd_data(const bf16 *dy, int cy, const float *w32, int cin, const bf16 *mask, bf16 *din,
                               int B, int H, int W) {
    const long P = (long)B * H * W;
    const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= P) return;
    const Pix qq = pix_of(q, H, W, P);
    float d[9];
    for (int t = 0; t < 9; t++) {
        const long n = nbr(qq, 8 - t, H, W);
        d[t] = n >= 0 ? __bfloat162float(dy[n * cy]) : 0.0f;
    }
    for (int ci = 0; ci < cin; ci++) {
        float s = 0.0f;
        for (int t = 0; t < 9; t++) s += d[t] * __bfloat162float(__float2bfloat16_rn(w32[(size_t)t * LPC_COUT_LAST * cin + ci]));
        if (!(__bfloat162float(mask[q * cin + ci]) > 0.0f)) s = 0.0f;
        din[q * cin + ci] = __float2bfloat16_rn(s);
    }
}

// Weight gradient, split over pixel chunks: part[chunk][t][ci][co] =
// sum_{p in chunk} In[p + off_t][ci] dOut[p][co].  One CTA per (tap, chunk);
// warps own 16-row blocks of ci, all co.
template <int NT>   // NT = cout / 8
__global__ void __launch_bounds__(128) k_conv_bwd_w(const ConvArgs a, const bf16 *dout, float *part, long chunk) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, tq = lane & 3;
    const int t = blockIdx.x, ch = blockIdx.y;
    const long P = (long)a.B * a.H * a.W;
    const int cin = a.c1 + a.c2, cout = a.cout;
    const long pb = (long)ch * chunk, pe = min(P, pb + chunk);
    for (int mt = warp; mt < cin / 16; mt += 4) {
        float acc[NT][4];
#pragma unroll
        for (int j = 0; j < NT; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
        const int r0 = mt * 16 + g, r1 = r0 + 8;   // input channels of this thread's A rows
        const bf16 *s0 = r0 < a.c1 ? a.in1 + r0 : a.in2 + (r0 - a.c1);
        const bf16 *s1 = r1 < a.c1 ? a.in1 + r1 : a.in2 + (r1 - a.c1);
        const int st0 = r0 < a.c1 ? a.c1 : a.c2, st1 = r1 < a.c1 ? a.c1 : a.c2;
        for (long k0 = pb; k0 < pe; k0 += 16) {
            // this thread's four pixels of the K step
            long pk[4] = {k0 + tq * 2, k0 + tq * 2 + 1, k0 + tq * 2 + 8, k0 + tq * 2 + 9};
            long nb[4];
            bool in[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                in[u] = pk[u] < pe;
                const Pix q = pix_of(in[u] ? pk[u] : pb, a.H, a.W, P);
                nb[u] = in[u] ? nbr(q, t, a.H, a.W) : -1;
            }
            auto av = [&](const bf16 *s, int st, int u) {
                return nb[u] >= 0 ? s[nb[u] * st] : __float2bfloat16_rn(0.0f);
            };
            uint32_t af[4] = {pack2(av(s0, st0, 0), av(s0, st0, 1)), pack2(av(s1, st1, 0), av(s1, st1, 1)),
                              pack2(av(s0, st0, 2), av(s0, st0, 3)), pack2(av(s1, st1, 2), av(s1, st1, 3))};
#pragma unroll
            for (int j = 0; j < NT; j++) {
                const int co = j * 8 + g;
                auto bv = [&](int u) { return in[u] ? dout[pk[u] * cout + co] : __float2bfloat16_rn(0.0f); };
                uint32_t bfr[2] = {pack2(bv(0), bv(1)), pack2(bv(2), bv(3))};
                mma_bf16(acc[j], af, bfr);
            }
        }
        float *dst = part + ((size_t)ch * 9 + t) * cin * cout;
#pragma unroll
        for (int j = 0; j < NT; j++) {
            const int co = j * 8 + tq * 2;
            dst[(size_t)r0 * cout + co] = acc[j][0];
            dst[(size_t)r0 * cout + co + 1] = acc[j][1];
            dst[(size_t)r1 * cout + co] = acc[j][2];
            dst[(size_t)r1 * cout + co + 1] = acc[j][3];
        }
    }
}

// grad[w_off + (t*cout + co)*cin + ci] = sum over chunks (fixed order);
// grad[b_off + co] = sum_p dOut[p][co] from per-chunk partials in bpart.
__global__ void k_wgrad_reduce(const float *part, int nchunk, int cin, int cout, float *gw) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 9 * cin * cout) return;
    const int t = i / (cin * cout), rem = i - t * cin * cout, ci = rem / cout, co = rem - ci * cout;
    float s = 0.0f;
    for (int c = 0; c < nchunk; c++) s += part[((size_t)c * 9 + t) * cin * cout + (size_t)ci * cout + co];
    gw[((size_t)t * cout + co) * cin + ci] = s;
}
__global__ void k_bgrad(const bf16 *dout, int cout, long P, float *gb) {
    // one CTA per output channel, fixed-order tree
    __shared__ float s[256];
    const int co = blockIdx.x;
    float v = 0.0f;
    for (long p = threadIdx.x; p < P; p += 256) v += __bfloat162float(dout[p * cout + co]);
    s[threadIdx.x] = v;
    __syncthreads();
    for (int k = 128; k > 0; k >>= 1) {
        if (threadIdx.x < k) s[threadIdx.x] += s[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) gb[co] = s[0];
}

// 2x2 average pool, [B][H][W][C] -> [B][H/2][W/2][C] (H, W even)
__global__ void k_pool(const bf16 *in, bf16 *out, int B, int H, int W, int C) {
    const long n = (long)B * (H / 2) * (W / 2) * C;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const long pix = i / C;
        const int x = (int)(pix % (W / 2)), y = (int)((pix / (W / 2)) % (H / 2)), b = (int)(pix / ((long)(W / 2) * (H / 2)));
        const long s = (((long)b * H + 2 * y) * W + 2 * x) * C + c;
        const float v = __bfloat162float(in[s]) + __bfloat162float(in[s + C]) + __bfloat162float(in[s + (long)W * C]) +
                        __bfloat162float(in[s + (long)W * C + C]);
        out[i] = __float2bfloat16_rn(0.25f * v);
    }
}
// nearest 2x upsample, [B][h][w][C] -> [B][2h][2w][C]
__global__ void k_up(const bf16 *in, bf16 *out, int B, int h, int w, int C) {
    const long n = (long)B * (2 * h) * (2 * w) * C;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const long pix = i / C;
        const int x = (int)(pix % (2 * w)), y = (int)((pix / (2 * w)) % (2 * h)), b = (int)(pix / ((long)(2 * w) * (2 * h)));
        out[i] = in[(((long)b * h + y / 2) * w + x / 2) * C + c];
    }
}
// gradient through a pool plus a second contribution, then the ReLU mask:
// ds = (dp[pix/2] / 4 + dadd) * (s > 0)        (all [B][H][W][C])
__global__ void k_pool_bwd(const bf16 *dp, const bf16 *dadd, const bf16 *s, bf16 *ds, int B, int H, int W, int C) {
    const long n = (long)B * H * W * C;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const long pix = i / C;
        const int x = (int)(pix % W), y = (int)((pix / W) % H), b = (int)(pix / ((long)W * H));
        float v = 0.25f * __bfloat162float(dp[(((long)b * (H / 2) + y / 2) * (W / 2) + x / 2) * C + c]);
        v += __bfloat162float(dadd[i]);
        if (!(__bfloat162float(s[i]) > 0.0f)) v = 0.0f;
        ds[i] = __float2bfloat16_rn(v);
    }
}
// gradient through a nearest upsample, then the ReLU mask of the source:
// da[b][y][x] = sum of du over the 2x2 block, times (a > 0)
__global__ void k_up_bwd(const bf16 *du, const bf16 *a, bf16 *da, int B, int h, int w, int C) {
    const long n = (long)B * h * w * C;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const long pix = i / C;
        const int x = (int)(pix % w), y = (int)((pix / w) % h), b = (int)(pix / ((long)w * h));
        const long s = (((long)b * 2 * h + 2 * y) * (2 * w) + 2 * x) * C + c;
        float v = __bfloat162float(du[s]) + __bfloat162float(du[s + C]) + __bfloat162float(du[s + (long)2 * w * C]) +
                  __bfloat162float(du[s + (long)2 * w * C + C]);
        if (!(__bfloat162float(a[i]) > 0.0f)) v = 0.0f;
        da[i] = __float2bfloat16_rn(v);
    }
}

// MSE over the valid pixels: loss = sum m (y - t)^2 / sum m; dy = 2 m (y - t) / sum m
// in channel 0 of [P][LPC_COUT_LAST] (other channels 0).  One CTA, fixed order.
__global__ void k_loss(const float *y, const float *tgt, const float *msk, long P, bf16 *dy, float *loss) {
    __shared__ float s_l[1024], s_m[1024];
    float l = 0.0f, m = 0.0f;
    for (long p = threadIdx.x; p < P; p += 1024) {
        const float d = y[p * LPC_COUT_LAST] - tgt[p];
        l += msk[p] * d * d;
        m += msk[p];
    }
    s_l[threadIdx.x] = l;
    s_m[threadIdx.x] = m;
    __syncthreads();
    for (int k = 512; k > 0; k >>= 1) {
        if (threadIdx.x < k) { s_l[threadIdx.x] += s_l[threadIdx.x + k]; s_m[threadIdx.x] += s_m[threadIdx.x + k]; }
        __syncthreads();
    }
    const float inv = s_m[0] > 0.0f ? 1.0f / s_m[0] : 0.0f;
    if (threadIdx.x == 0) *loss = s_l[0] * inv;
    for (long p = threadIdx.x; p < P; p += 1024) {
        const float d = y[p * LPC_COUT_LAST] - tgt[p];
        dy[p * LPC_COUT_LAST] = __float2bfloat16_rn(2.0f * msk[p] * d * inv);
        for (int c = 1; c < LPC_COUT_LAST; c++) dy[p * LPC_COUT_LAST + c] = __float2bfloat16_rn(0.0f);
    }
}

// Adam on the FP32 master parameters (step t, 1-based)
__global__ void k_adam(float *w, const float *gr, float *m, float *v, size_t n, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float g = gr[i];
        const float mi = b1 * m[i] + (1.0f - b1) * g;
        const float vi = b2 * v[i] + (1.0f - b2) * g * g;
        m[i] = mi;
        v[i] = vi;
        w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

// BF16 copies of the weights: wf[l][t][co][ci] and wb[l][t][ci][co]
__global__ void k_refresh(const LpcNet net, const float *w, bf16 *wf, bf16 *wb) {
    for (int l = 0; l < LPC_NLAYER; l++) {
        const LpcLayer &L = net.L[l];
        const int cin = L.c1 + L.c2, n = 9 * cin * L.cout;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
            const int t = i / (L.cout * cin), rem = i - t * L.cout * cin, co = rem / cin, ci = rem - co * cin;
            const bf16 v = __float2bfloat16_rn(w[L.w_off + i]);
            wf[L.wf_off + i] = v;
            wb[L.wb_off + ((size_t)t * cin + ci) * L.cout + co] = v;
        }
    }
}

}  // namespace

// ------------------------------------------------------------------ host side
void lpc_describe(LpcNet &net) {
    // c1, c2, cout, resolution level
    const int spec[LPC_NLAYER][4] = {{LPC_CIN0, 0, 32, 0}, {32, 0, 32, 0}, {32, 0, 64, 1}, {64, 0, 64, 1},
                                     {64, 0, 64, 2},       {64, 0, 64, 2}, {64, 64, 64, 1}, {64, 32, 32, 0},
                                     {32, 0, LPC_COUT_LAST, 0}};
    size_t wp = 0, w16 = 0;
    for (int l = 0; l < LPC_NLAYER; l++) {
        LpcLayer &L = net.L[l];
        L.c1 = spec[l][0]; L.c2 = spec[l][1]; L.cout = spec[l][2]; L.res = spec[l][3];
        const size_t nw = (size_t)9 * (L.c1 + L.c2) * L.cout;
        L.w_off = wp; wp += nw;
        L.b_off = wp; wp += L.cout;
        L.wf_off = w16; L.wb_off = w16; w16 += nw;
    }
    net.nparam = wp;
    net.nw16 = w16;
}

namespace {

template <typename T>
cudaError_t dalloc(T **p, size_t n) {
    cudaError_t e = cudaMalloc(p, n * sizeof(T) + 16);
    if (e == cudaSuccess) e = cudaMemset(*p, 0, n * sizeof(T) + 16);
    return e;
}

uint64_t sm64(uint64_t &s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
double unif(uint64_t &s) { return ((sm64(s) >> 11) + 0.5) * (1.0 / 9007199254740992.0); }

inline int nblk(long n, int t) { return (int)((n + t - 1) / t); }

void conv_fwd(const LpcState *L, int l, const bf16 *in1, const bf16 *in2, bf16 *out, float *out32, int B, int H,
              int W, cudaStream_t st) {
    const LpcLayer &Y = L->net.L[l];
    ConvArgs a = {};
    a.in1 = in1; a.in2 = in2; a.c1 = Y.c1; a.c2 = Y.c2; a.cout = Y.cout;
    a.w = L->wf + Y.wf_off; a.bias = L->w + Y.b_off;
    a.out = out; a.out32 = out32; a.relu = out32 ? 0 : 1;
    a.B = B; a.H = H; a.W = W;
    const long P = (long)B * H * W;
    // warps per 16-pixel tile: cout / 16 for cout >= 16 (two 8-channel tiles a warp), 1 for the last layer
    if (Y.cout == LPC_COUT_LAST) k_conv_fwd<1><<<nblk(P, 64), 128, 0, st>>>(a);
    else if (Y.cout == 32) k_conv_fwd<2><<<nblk(P, 32), 128, 0, st>>>(a);
    else k_conv_fwd<2><<<nblk(P, 16), 128, 0, st>>>(a);   // cout 64
}

void conv_bwd_data(const LpcState *L, int l, const bf16 *dout, bf16 *din1, bf16 *din2, const bf16 *m1, const bf16 *m2,
                   int B, int H, int W, cudaStream_t st) {
    const LpcLayer &Y = L->net.L[l];
    ConvArgs a = {};
    a.c1 = Y.c1; a.c2 = Y.c2; a.cout = Y.cout;
    a.w = L->wb + Y.wb_off;
    a.out = din1; a.dout2 = din2; a.mask1 = m1; a.mask2 = m2;
    a.B = B; a.H = H; a.W = W;
    const int g = nblk((long)B * H * W, 16);
    switch ((Y.c1 + Y.c2) / 32) {
        case 1: k_conv_bwd_data<1><<<g, 128, 0, st>>>(a, dout); break;
        case 2: k_conv_bwd_data<2><<<g, 128, 0, st>>>(a, dout); break;
        case 3: k_conv_bwd_data<3><<<g, 128, 0, st>>>(a, dout); break;
        case 4: k_conv_bwd_data<4><<<g, 128, 0, st>>>(a, dout); break;
    }
}

void conv_bwd_w(LpcState *L, int l, const bf16 *in1, const bf16 *in2, const bf16 *dout, int B, int H, int W,
                cudaStream_t st) {
    const LpcLayer &Y = L->net.L[l];
    ConvArgs a = {};
    a.in1 = in1; a.in2 = in2; a.c1 = Y.c1; a.c2 = Y.c2; a.cout = Y.cout;
    a.B = B; a.H = H; a.W = W;
    const long P = (long)B * H * W;
    long chunk = (P + L->nchunk_max - 1) / L->nchunk_max;
    if (chunk < 1024) chunk = 1024;
    const int nch = (int)((P + chunk - 1) / chunk);
    dim3 g(9, nch);
    switch (Y.cout / 8) {
        case 1: k_conv_bwd_w<1><<<g, 128, 0, st>>>(a, dout, L->part, chunk); break;
        case 4: k_conv_bwd_w<4><<<g, 128, 0, st>>>(a, dout, L->part, chunk); break;
        case 8: k_conv_bwd_w<8><<<g, 128, 0, st>>>(a, dout, L->part, chunk); break;
    }
    const int cin = Y.c1 + Y.c2;
    k_wgrad_reduce<<<nblk(9L * cin * Y.cout, 256), 256, 0, st>>>(L->part, nch, cin, Y.cout, L->g + Y.w_off);
    k_bgrad<<<Y.cout, 256, 0, st>>>(dout, Y.cout, P, L->g + Y.b_off);
}

}  // namespace

int lpc_alloc(LpcState **out, int Hn, int Wn, int Bmax, int Nmax, uint64_t seed, cudaStream_t st) {
    LpcState *L = new LpcState();
    lpc_describe(L->net);
    L->Hn = Hn; L->Wn = Wn; L->Bmax = Bmax; L->Nmax = Nmax; L->nsamp = 0; L->adam_t = 0;
    const long P0 = (long)Bmax * Hn * Wn, P1 = P0 / 4, P2 = P0 / 16;
    const size_t np = L->net.nparam, nw = L->net.nw16;
    L->nchunk_max = 64;
    L->part_n = (size_t)L->nchunk_max * 9 * 128 * 64;
    cudaError_t e = cudaSuccess;
#define A(ptr, n) if (e == cudaSuccess) e = dalloc(&(ptr), (size_t)(n))
    A(L->w, np); A(L->g, np); A(L->m, np); A(L->v, np); A(L->wf, nw); A(L->wb, nw);
    A(L->x0, P0 * LPC_CIN0); A(L->a1, P0 * 32); A(L->s1, P0 * 32); A(L->p1, P1 * 32); A(L->a2, P1 * 64);
    A(L->s2, P1 * 64); A(L->p2, P2 * 64); A(L->a3, P2 * 64); A(L->a4, P2 * 64); A(L->u2, P1 * 64);
    A(L->a5, P1 * 64); A(L->u1, P0 * 64); A(L->a6, P0 * 32); A(L->y, P0 * LPC_COUT_LAST);
    A(L->dy, P0 * LPC_COUT_LAST); A(L->da6, P0 * 32); A(L->du1, P0 * 64); A(L->ds1b, P0 * 32); A(L->da5, P1 * 64);
    A(L->du2, P1 * 64); A(L->ds2b, P1 * 64); A(L->da4, P2 * 64); A(L->da3, P2 * 64); A(L->dp2, P2 * 64);
    A(L->ds2, P1 * 64); A(L->da2, P1 * 64); A(L->dp1, P1 * 32); A(L->ds1, P0 * 32); A(L->da1, P0 * 32);
    A(L->part, L->part_n);
    A(L->dfeat, (size_t)Nmax * Hn * Wn * LPC_CIN0); A(L->dtgt, (size_t)Nmax * Hn * Wn);
    A(L->mask, (size_t)Hn * Wn); A(L->btgt, P0); A(L->bmask, P0); A(L->d_loss, 4);
#undef A
    if (e != cudaSuccess) { lpc_free(L); return (int)e; }
    // He-normal weights from a seeded generator, zero biases; the last layer
    // starts 10x smaller so that the untrained correction is nearly zero
    std::vector<float> hw(np, 0.0f);
    uint64_t s = seed * 0x100000001B3ull + 12345;
    for (int l = 0; l < LPC_NLAYER; l++) {
        const LpcLayer &Y = L->net.L[l];
        const int cin = Y.c1 + Y.c2, cin_eff = l == 0 ? LPC_NFEAT : cin;
        const double sd = std::sqrt(2.0 / (9.0 * cin_eff)) * (l == LPC_NLAYER - 1 ? 0.1 : 1.0);
        for (int t = 0; t < 9; t++)
            for (int co = 0; co < Y.cout; co++)
                for (int ci = 0; ci < cin; ci++) {
                    const double u1 = unif(s), u2 = unif(s);
                    const double z = std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
                    const bool live = (l > 0 || ci < LPC_NFEAT) && (l < LPC_NLAYER - 1 || co == 0);
                    hw[Y.w_off + ((size_t)t * Y.cout + co) * cin + ci] = live ? (float)(sd * z) : 0.0f;
                }
    }
    e = cudaMemcpyAsync(L->w, hw.data(), np * sizeof(float), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) { lpc_free(L); return (int)e; }
    lpc_refresh(L, st);
    *out = L;
    return 0;
}

void lpc_free(LpcState *L) {
    if (!L) return;
    void *ps[] = {L->w, L->g, L->m, L->v, L->wf, L->wb, L->x0, L->a1, L->s1, L->p1, L->a2, L->s2, L->p2, L->a3,
                  L->a4, L->u2, L->a5, L->u1, L->a6, L->y, L->dy, L->da6, L->du1, L->ds1b, L->da5, L->du2,
                  L->ds2b, L->da4, L->da3, L->dp2, L->ds2, L->da2, L->dp1, L->ds1, L->da1, L->part, L->dfeat,
                  L->dtgt, L->mask, L->btgt, L->bmask, L->d_loss};
    for (void *p : ps) cudaFree(p);
    delete L;
}

void lpc_refresh(LpcState *L, cudaStream_t st) { k_refresh<<<256, 256, 0, st>>>(L->net, L->w, L->wf, L->wb); }

void lpc_forward(LpcState *L, int B, cudaStream_t st) {
    const int H0 = L->Hn, W0 = L->Wn, H1 = H0 / 2, W1 = W0 / 2, H2 = H1 / 2, W2 = W1 / 2;
    const int ew = 1024;
    conv_fwd(L, 0, L->x0, nullptr, L->a1, nullptr, B, H0, W0, st);
    conv_fwd(L, 1, L->a1, nullptr, L->s1, nullptr, B, H0, W0, st);
    k_pool<<<ew, 256, 0, st>>>(L->s1, L->p1, B, H0, W0, 32);
    conv_fwd(L, 2, L->p1, nullptr, L->a2, nullptr, B, H1, W1, st);
    conv_fwd(L, 3, L->a2, nullptr, L->s2, nullptr, B, H1, W1, st);
    k_pool<<<ew, 256, 0, st>>>(L->s2, L->p2, B, H1, W1, 64);
    conv_fwd(L, 4, L->p2, nullptr, L->a3, nullptr, B, H2, W2, st);
    conv_fwd(L, 5, L->a3, nullptr, L->a4, nullptr, B, H2, W2, st);
    k_up<<<ew, 256, 0, st>>>(L->a4, L->u2, B, H2, W2, 64);
    conv_fwd(L, 6, L->u2, L->s2, L->a5, nullptr, B, H1, W1, st);
    k_up<<<ew, 256, 0, st>>>(L->a5, L->u1, B, H1, W1, 64);
    conv_fwd(L, 7, L->u1, L->s1, L->a6, nullptr, B, H0, W0, st);
    conv_fwd(L, 8, L->a6, nullptr, nullptr, L->y, B, H0, W0, st);
}

int lpc_loss_backward(LpcState *L, int B, cudaStream_t st) {
    const int H0 = L->Hn, W0 = L->Wn, H1 = H0 / 2, W1 = W0 / 2, H2 = H1 / 2, W2 = W1 / 2;
    const long P0 = (long)B * H0 * W0;
    const int ew = 1024;
    k_loss<<<1, 1024, 0, st>>>(L->y, L->btgt, L->bmask, P0, L->dy, L->d_loss);
    const LpcLayer &Lo = L->net.L[8];
    conv_bwd_w(L, 8, L->a6, nullptr, L->dy, B, H0, W0, st);
    k_out_bwd_data<<<nblk(P0, 256), 256, 0, st>>>(L->dy, LPC_COUT_LAST, L->w + Lo.w_off, Lo.c1, L->a6, L->da6, B,
                                                   H0, W0);
    conv_bwd_w(L, 7, L->u1, L->s1, L->da6, B, H0, W0, st);
    conv_bwd_data(L, 7, L->da6, L->du1, L->ds1b, nullptr, nullptr, B, H0, W0, st);
    k_up_bwd<<<ew, 256, 0, st>>>(L->du1, L->a5, L->da5, B, H1, W1, 64);
    conv_bwd_w(L, 6, L->u2, L->s2, L->da5, B, H1, W1, st);
    conv_bwd_data(L, 6, L->da5, L->du2, L->ds2b, nullptr, nullptr, B, H1, W1, st);
    k_up_bwd<<<ew, 256, 0, st>>>(L->du2, L->a4, L->da4, B, H2, W2, 64);
    conv_bwd_w(L, 5, L->a3, nullptr, L->da4, B, H2, W2, st);
    conv_bwd_data(L, 5, L->da4, L->da3, nullptr, L->a3, nullptr, B, H2, W2, st);
    conv_bwd_w(L, 4, L->p2, nullptr, L->da3, B, H2, W2, st);
    conv_bwd_data(L, 4, L->da3, L->dp2, nullptr, nullptr, nullptr, B, H2, W2, st);
    k_pool_bwd<<<ew, 256, 0, st>>>(L->dp2, L->ds2b, L->s2, L->ds2, B, H1, W1, 64);
    conv_bwd_w(L, 3, L->a2, nullptr, L->ds2, B, H1, W1, st);
    conv_bwd_data(L, 3, L->ds2, L->da2, nullptr, L->a2, nullptr, B, H1, W1, st);
    conv_bwd_w(L, 2, L->p1, nullptr, L->da2, B, H1, W1, st);
    conv_bwd_data(L, 2, L->da2, L->dp1, nullptr, nullptr, nullptr, B, H1, W1, st);
    k_pool_bwd<<<ew, 256, 0, st>>>(L->dp1, L->ds1b, L->s1, L->ds1, B, H0, W0, 32);
    conv_bwd_w(L, 1, L->a1, nullptr, L->ds1, B, H0, W0, st);
    conv_bwd_data(L, 1, L->ds1, L->da1, nullptr, L->a1, nullptr, B, H0, W0, st);
    conv_bwd_w(L, 0, L->x0, nullptr, L->da1, B, H0, W0, st);
    return (int)cudaGetLastError();
}

void lpc_adam(LpcState *L, float lr, cudaStream_t st) {
    L->adam_t++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - (float)std::pow(b1, L->adam_t), c2 = 1.0f - (float)std::pow(b2, L->adam_t);
    k_adam<<<256, 256, 0, st>>>(L->w, L->g, L->m, L->v, L->net.nparam, lr, b1, b2, 1e-8f, c1, c2);
    lpc_refresh(L, st);
}

void lpc_gather(LpcState *L, const int *h_idx, int B, cudaStream_t st) {
    const size_t px = (size_t)L->Hn * L->Wn;
    for (int b = 0; b < B; b++) {
        const size_t i = (size_t)h_idx[b];
        cudaMemcpyAsync(L->x0 + b * px * LPC_CIN0, L->dfeat + i * px * LPC_CIN0, px * LPC_CIN0 * sizeof(bf16),
                        cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(L->btgt + b * px, L->dtgt + i * px, px * sizeof(float), cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(L->bmask + b * px, L->mask, px * sizeof(float), cudaMemcpyDeviceToDevice, st);
    }
}
