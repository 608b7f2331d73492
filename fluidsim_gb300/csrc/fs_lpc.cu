// fs_lpc.cu -- the learned Poisson preconditioner's network (see fs_lpc.cuh).
//
// A four-level U-Net, 3x3 convolutions, ReLU, 2x2 average pooling, nearest
// upsampling, 258,528 parameters:
//   enc0 16->16->16 (skip s0)  | pool | enc1 16->32->32 (skip s1) | pool |
//   enc2 32->64->64 (skip s2)  | pool | bottleneck 64->64->64 | up |
//   dec2 [up, s2] 128->64 | up | dec1 [up, s1] 96->32 | up |
//   dec0 [up, s0] 48->16 | out 16->16 (channel 0 is the prediction, no ReLU)
// Activations are NHWC BF16 tensors [B][H][W][C].  Every convolution runs on
// the tcgen05 tensor cores (fs_conv_tc.cu: TMA-staged BF16 operands, FP32
// accumulators in tensor memory): the forward pass, and the data gradient as
// the convolution of the output gradient with the flipped, transposed
// weights (ReLU masks applied in its epilogue).  Weight gradients: a split-K
// GEMM over pixels on mma.sync with a fixed-order reduction.  Adam on FP32
// master weights, from which the BF16 weight images are rebuilt.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "fluidsim_gpu.h"
#include "fs_lpc.cuh"

typedef __nv_bfloat16 bf16;

namespace {

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
        const float d = y[p] - tgt[p];
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
        const float d = y[p] - tgt[p];
        uint4 *o = reinterpret_cast<uint4 *>(dy + p * LPC_COUT_LAST);
        const uint32_t v0 = (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(2.0f * msk[p] * d * inv));
        o[0] = make_uint4(v0, 0u, 0u, 0u);
        o[1] = make_uint4(0u, 0u, 0u, 0u);
    }
}

// B crops of Hc x Wc cells from the training pairs: crop b of pair idx[b] at
// (y0[b], x0[b]) -> x0 [b][y][x][16] (the LPC_NFEAT features, zeros after),
// batch target and mask (interior cells of the padded grid)
__global__ void k_gather(const bf16 *feat, const float *tgt, const float *mask, int Hn, int Wn, const int *crops,
                         int B, int Hc, int Wc, bf16 *x0, float *btgt, float *bmask) {
    const long n = (long)B * Hc * Wc;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) {
        const int b = (int)(q / ((long)Hc * Wc)), r = (int)(q - (long)b * Hc * Wc), y = r / Wc, x = r - y * Wc;
        const int i = crops[3 * b], yy = crops[3 * b + 1] + y, xx = crops[3 * b + 2] + x;
        const size_t src = ((size_t)i * Hn + yy) * Wn + xx, cell = (size_t)yy * Wn + xx;
        const uint2 f = *reinterpret_cast<const uint2 *>(feat + src * LPC_NFEAT);
        uint4 *o = reinterpret_cast<uint4 *>(x0 + q * LPC_CIN0);
        o[0] = make_uint4(f.x, f.y, 0u, 0u);
        o[1] = make_uint4(0u, 0u, 0u, 0u);
        btgt[q] = tgt[src];
        bmask[q] = mask[cell];
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

}  // namespace

// ------------------------------------------------------------------ host side
void lpc_describe(LpcNet &net) {
    // c1, c2, cout, resolution level
    const int spec[LPC_NLAYER][4] = {{LPC_CIN0, 0, 16, 0}, {16, 0, 16, 0},  {16, 0, 32, 1},  {32, 0, 32, 1},
                                     {32, 0, 64, 2},       {64, 0, 64, 2},  {64, 0, 64, 3},  {64, 0, 64, 3},
                                     {64, 64, 64, 2},      {64, 32, 32, 1}, {32, 16, 16, 0}, {16, 0, LPC_COUT_LAST, 0}};
    size_t wp = 0, img = 0;
    for (int l = 0; l < LPC_NLAYER; l++) {
        LpcLayer &L = net.L[l];
        L.c1 = spec[l][0]; L.c2 = spec[l][1]; L.cout = spec[l][2]; L.res = spec[l][3];
        const size_t nw = (size_t)9 * (L.c1 + L.c2) * L.cout;
        L.w_off = wp; wp += nw;
        L.b_off = wp; wp += L.cout;
        TcConvArgs t = {};
        L.bytes_f = tc_weight_layout(L.c1, L.c2, L.cout, t.boff, t.kc, t.nchunk);
        L.bytes_b = l > 0 ? tc_weight_layout(L.cout, 0, L.c1 + L.c2, t.boff, t.kc, t.nchunk) : 0;
        L.img_f = img; img += (size_t)L.bytes_f;
        L.img_b = img; img += (size_t)L.bytes_b;
    }
    net.nparam = wp;
    net.img_bytes = img;
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

// One tensor-core convolution over B images of H x W cells.  Forward (bwd = 0):
// inputs in1 (c1 channels), in2 (c2), output out (BF16, bias, ReLU) or y
// (FP32 channel 0, bias).  Data gradient (bwd = 1): input in1 = the output
// gradient (cout channels), outputs out (c1 channels, ReLU mask m1) and out2
// (c2 channels, mask m2).
int tc_layer(LpcState *L, int l, int bwd, int B, int H, int W, const bf16 *in1, const bf16 *in2, bf16 *out,
             bf16 *out2, const bf16 *m1, const bf16 *m2, float *y, cudaStream_t st) {
    const LpcLayer &Y = L->net.L[l];
    TcConvArgs a = {};
    int ci1, ci2, co;
    if (!bwd) { ci1 = Y.c1; ci2 = Y.c2; co = Y.cout; }
    else { ci1 = Y.cout; ci2 = 0; co = Y.c1 + Y.c2; }
    a.wbytes = tc_weight_layout(ci1, ci2, co, a.boff, a.kc, a.nchunk);
    a.cout = co;
    a.B = B; a.H = H; a.W = W;
    a.halo = tc_halo_fits(a);
    CUtensorMap m[2];
    if (tc_make_map(&m[0], in1, B, H, W, ci1, a.kc[0], a.halo) ||
        (ci2 && tc_make_map(&m[1], in2, B, H, W, ci2, a.kc[1], a.halo)))
        return -1;
    a.tmem_cols = tc_tmem_cols(co);
    tc_set_tiles(a);
    a.wimg = L->img + (bwd ? Y.img_b : Y.img_f);
    a.err = L->d_tc_err;
    if (!bwd) {
        a.bias = L->w + Y.b_off;
        if (y) { a.out32 = y; a.out32_ch = 1; }
        else { a.out = out; a.relu = 1; }
        a.split = co;
    } else {
        a.out = out; a.out2 = out2; a.split = Y.c1;
        a.mask = m1; a.mask2 = m2;
    }
    return tc_conv(&m[0], ci2 ? &m[1] : nullptr, a, st);
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
        case 2: k_conv_bwd_w<2><<<g, 128, 0, st>>>(a, dout, L->part, chunk); break;
        case 4: k_conv_bwd_w<4><<<g, 128, 0, st>>>(a, dout, L->part, chunk); break;
        case 8: k_conv_bwd_w<8><<<g, 128, 0, st>>>(a, dout, L->part, chunk); break;
    }
    const int cin = Y.c1 + Y.c2;
    k_wgrad_reduce<<<nblk(9L * cin * Y.cout, 256), 256, 0, st>>>(L->part, nch, cin, Y.cout, L->g + Y.w_off);
    k_bgrad<<<Y.cout, 256, 0, st>>>(dout, Y.cout, P, L->g + Y.b_off);
}

}  // namespace

int lpc_alloc(LpcState **out, int Hn, int Wn, int Hc, int Wc, int Bmax, int Nmax, uint64_t seed, cudaStream_t st) {
    if (Hn % 8 || Wn % 8 || Hc % 8 || Wc % 8 || Hc > Hn || Wc > Wn || Bmax < 1 || Nmax < 1) return (int)cudaErrorInvalidValue;
    if (tc_init()) return (int)cudaErrorNotSupported;
    LpcState *L = new LpcState();
    lpc_describe(L->net);
    L->Hn = Hn; L->Wn = Wn; L->Hc = Hc; L->Wc = Wc; L->Bmax = Bmax; L->Nmax = Nmax; L->nsamp = 0; L->adam_t = 0;
    const long c0 = std::max((long)Bmax * Hc * Wc, (long)Hn * Wn), c1 = c0 / 4, c2 = c0 / 16, c3 = c0 / 64;
    L->cap0 = c0;
    const size_t np = L->net.nparam;
    L->nchunk_max = 64;
    L->part_n = (size_t)L->nchunk_max * 9 * 128 * 64;
    cudaError_t e = cudaSuccess;
#define A(ptr, n) if (e == cudaSuccess) e = dalloc(&(ptr), (size_t)(n))
    A(L->w, np); A(L->g, np); A(L->m, np); A(L->v, np); A(L->img, L->net.img_bytes);
    A(L->x0, c0 * LPC_CIN0); A(L->a0, c0 * 16); A(L->s0, c0 * 16); A(L->p0, c1 * 16); A(L->a1, c1 * 32);
    A(L->s1, c1 * 32); A(L->p1, c2 * 32); A(L->a2, c2 * 64); A(L->s2, c2 * 64); A(L->p2, c3 * 64);
    A(L->a3, c3 * 64); A(L->b3, c3 * 64); A(L->u2, c2 * 64); A(L->d2, c2 * 64); A(L->u1, c1 * 64);
    A(L->d1, c1 * 32); A(L->u0, c0 * 32); A(L->d0, c0 * 16); A(L->y, c0);
    A(L->dy, c0 * LPC_COUT_LAST); A(L->dd0, c0 * 16); A(L->du0, c0 * 32); A(L->ds0b, c0 * 16); A(L->dd1, c1 * 32);
    A(L->du1, c1 * 64); A(L->ds1b, c1 * 32); A(L->dd2, c2 * 64); A(L->du2, c2 * 64); A(L->ds2b, c2 * 64);
    A(L->db3, c3 * 64); A(L->da3, c3 * 64); A(L->dp2, c3 * 64); A(L->ds2, c2 * 64); A(L->da2, c2 * 64);
    A(L->dp1, c2 * 32); A(L->ds1, c1 * 32); A(L->da1, c1 * 32); A(L->dp0, c1 * 16); A(L->ds0, c0 * 16);
    A(L->da0, c0 * 16);
    A(L->part, L->part_n);
    A(L->dfeat, (size_t)Nmax * Hn * Wn * LPC_NFEAT); A(L->dtgt, (size_t)Nmax * Hn * Wn);
    A(L->mask, (size_t)Hn * Wn); A(L->btgt, c0); A(L->bmask, c0); A(L->d_loss, 4); A(L->d_tc_err, 4);
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
    void *ps[] = {L->w,   L->g,    L->m,    L->v,    L->img,  L->x0,  L->a0,  L->s0,    L->p0,    L->a1,   L->s1,
                  L->p1,  L->a2,   L->s2,   L->p2,   L->a3,   L->b3,  L->u2,  L->d2,    L->u1,    L->d1,   L->u0,
                  L->d0,  L->y,    L->dy,   L->dd0,  L->du0,  L->ds0b, L->dd1, L->du1,  L->ds1b,  L->dd2,  L->du2,
                  L->ds2b, L->db3, L->da3,  L->dp2,  L->ds2,  L->da2, L->dp1, L->ds1,   L->da1,   L->dp0,  L->ds0,
                  L->da0, L->part, L->dfeat, L->dtgt, L->mask, L->btgt, L->bmask, L->d_loss, L->d_tc_err};
    for (void *p : ps) cudaFree(p);
    delete L;
}

void lpc_refresh(LpcState *L, cudaStream_t st) {
    for (int l = 0; l < LPC_NLAYER; l++) {
        const LpcLayer &Y = L->net.L[l];
        tc_build_weights(L->w + Y.w_off, Y.c1, Y.c2, Y.cout, L->img + Y.img_f, st);
        if (l > 0) tc_build_weights_bwd(L->w + Y.w_off, Y.c1 + Y.c2, Y.cout, L->img + Y.img_b, st);
    }
}

int lpc_forward(LpcState *L, int B, int H, int W, cudaStream_t st) {
    if ((long)B * H * W > L->cap0 || H % 8 || W % 8) return (int)cudaErrorInvalidValue;
    const int H1 = H / 2, W1 = W / 2, H2 = H / 4, W2 = W / 4, H3 = H / 8, W3 = W / 8;
    const int ew = 1024;
    int r = 0;
    r |= tc_layer(L, 0, 0, B, H, W, L->x0, nullptr, L->a0, nullptr, nullptr, nullptr, nullptr, st);
    r |= tc_layer(L, 1, 0, B, H, W, L->a0, nullptr, L->s0, nullptr, nullptr, nullptr, nullptr, st);
    k_pool<<<ew, 256, 0, st>>>(L->s0, L->p0, B, H, W, 16);
    r |= tc_layer(L, 2, 0, B, H1, W1, L->p0, nullptr, L->a1, nullptr, nullptr, nullptr, nullptr, st);
    r |= tc_layer(L, 3, 0, B, H1, W1, L->a1, nullptr, L->s1, nullptr, nullptr, nullptr, nullptr, st);
    k_pool<<<ew, 256, 0, st>>>(L->s1, L->p1, B, H1, W1, 32);
    r |= tc_layer(L, 4, 0, B, H2, W2, L->p1, nullptr, L->a2, nullptr, nullptr, nullptr, nullptr, st);
    r |= tc_layer(L, 5, 0, B, H2, W2, L->a2, nullptr, L->s2, nullptr, nullptr, nullptr, nullptr, st);
    k_pool<<<ew, 256, 0, st>>>(L->s2, L->p2, B, H2, W2, 64);
    r |= tc_layer(L, 6, 0, B, H3, W3, L->p2, nullptr, L->a3, nullptr, nullptr, nullptr, nullptr, st);
    r |= tc_layer(L, 7, 0, B, H3, W3, L->a3, nullptr, L->b3, nullptr, nullptr, nullptr, nullptr, st);
    k_up<<<ew, 256, 0, st>>>(L->b3, L->u2, B, H3, W3, 64);
    r |= tc_layer(L, 8, 0, B, H2, W2, L->u2, L->s2, L->d2, nullptr, nullptr, nullptr, nullptr, st);
    k_up<<<ew, 256, 0, st>>>(L->d2, L->u1, B, H2, W2, 64);
    r |= tc_layer(L, 9, 0, B, H1, W1, L->u1, L->s1, L->d1, nullptr, nullptr, nullptr, nullptr, st);
    k_up<<<ew, 256, 0, st>>>(L->d1, L->u0, B, H1, W1, 32);
    r |= tc_layer(L, 10, 0, B, H, W, L->u0, L->s0, L->d0, nullptr, nullptr, nullptr, nullptr, st);
    r |= tc_layer(L, 11, 0, B, H, W, L->d0, nullptr, nullptr, nullptr, nullptr, nullptr, L->y, st);
    if (r) L->tc_bad = 1;
    return r ? (int)cudaErrorLaunchFailure : 0;
}

int lpc_loss_backward(LpcState *L, int B, int H, int W, cudaStream_t st) {
    const int H1 = H / 2, W1 = W / 2, H2 = H / 4, W2 = W / 4, H3 = H / 8, W3 = W / 8;
    const long P0 = (long)B * H * W;
    const int ew = 1024;
    int r = 0;
    k_loss<<<1, 1024, 0, st>>>(L->y, L->btgt, L->bmask, P0, L->dy, L->d_loss);
    // output layer
    conv_bwd_w(L, 11, L->d0, nullptr, L->dy, B, H, W, st);
    r |= tc_layer(L, 11, 1, B, H, W, L->dy, nullptr, L->dd0, nullptr, L->d0, nullptr, nullptr, st);
    // dec0 [u0, s0] -> d0
    conv_bwd_w(L, 10, L->u0, L->s0, L->dd0, B, H, W, st);
    r |= tc_layer(L, 10, 1, B, H, W, L->dd0, nullptr, L->du0, L->ds0b, nullptr, nullptr, nullptr, st);
    k_up_bwd<<<ew, 256, 0, st>>>(L->du0, L->d1, L->dd1, B, H1, W1, 32);
    // dec1 [u1, s1] -> d1
    conv_bwd_w(L, 9, L->u1, L->s1, L->dd1, B, H1, W1, st);
    r |= tc_layer(L, 9, 1, B, H1, W1, L->dd1, nullptr, L->du1, L->ds1b, nullptr, nullptr, nullptr, st);
    k_up_bwd<<<ew, 256, 0, st>>>(L->du1, L->d2, L->dd2, B, H2, W2, 64);
    // dec2 [u2, s2] -> d2
    conv_bwd_w(L, 8, L->u2, L->s2, L->dd2, B, H2, W2, st);
    r |= tc_layer(L, 8, 1, B, H2, W2, L->dd2, nullptr, L->du2, L->ds2b, nullptr, nullptr, nullptr, st);
    k_up_bwd<<<ew, 256, 0, st>>>(L->du2, L->b3, L->db3, B, H3, W3, 64);
    // bottleneck
    conv_bwd_w(L, 7, L->a3, nullptr, L->db3, B, H3, W3, st);
    r |= tc_layer(L, 7, 1, B, H3, W3, L->db3, nullptr, L->da3, nullptr, L->a3, nullptr, nullptr, st);
    conv_bwd_w(L, 6, L->p2, nullptr, L->da3, B, H3, W3, st);
    r |= tc_layer(L, 6, 1, B, H3, W3, L->da3, nullptr, L->dp2, nullptr, nullptr, nullptr, nullptr, st);
    k_pool_bwd<<<ew, 256, 0, st>>>(L->dp2, L->ds2b, L->s2, L->ds2, B, H2, W2, 64);
    // enc2
    conv_bwd_w(L, 5, L->a2, nullptr, L->ds2, B, H2, W2, st);
    r |= tc_layer(L, 5, 1, B, H2, W2, L->ds2, nullptr, L->da2, nullptr, L->a2, nullptr, nullptr, st);
    conv_bwd_w(L, 4, L->p1, nullptr, L->da2, B, H2, W2, st);
    r |= tc_layer(L, 4, 1, B, H2, W2, L->da2, nullptr, L->dp1, nullptr, nullptr, nullptr, nullptr, st);
    k_pool_bwd<<<ew, 256, 0, st>>>(L->dp1, L->ds1b, L->s1, L->ds1, B, H1, W1, 32);
    // enc1
    conv_bwd_w(L, 3, L->a1, nullptr, L->ds1, B, H1, W1, st);
    r |= tc_layer(L, 3, 1, B, H1, W1, L->ds1, nullptr, L->da1, nullptr, L->a1, nullptr, nullptr, st);
    conv_bwd_w(L, 2, L->p0, nullptr, L->da1, B, H1, W1, st);
    r |= tc_layer(L, 2, 1, B, H1, W1, L->da1, nullptr, L->dp0, nullptr, nullptr, nullptr, nullptr, st);
    k_pool_bwd<<<ew, 256, 0, st>>>(L->dp0, L->ds0b, L->s0, L->ds0, B, H, W, 16);
    // enc0
    conv_bwd_w(L, 1, L->a0, nullptr, L->ds0, B, H, W, st);
    r |= tc_layer(L, 1, 1, B, H, W, L->ds0, nullptr, L->da0, nullptr, L->a0, nullptr, nullptr, st);
    conv_bwd_w(L, 0, L->x0, nullptr, L->da0, B, H, W, st);
    if (r) { L->tc_bad = 1; return (int)cudaErrorLaunchFailure; }
    return (int)cudaGetLastError();
}

void lpc_adam(LpcState *L, float lr, cudaStream_t st) {
    L->adam_t++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - (float)std::pow(b1, L->adam_t), c2 = 1.0f - (float)std::pow(b2, L->adam_t);
    k_adam<<<256, 256, 0, st>>>(L->w, L->g, L->m, L->v, L->net.nparam, lr, b1, b2, 1e-8f, c1, c2);
    lpc_refresh(L, st);
}

void lpc_gather(LpcState *L, const int *h_idx, const int *h_y0, const int *h_x0, int B, cudaStream_t st) {
    // crop table through a small pinned-free staging: B <= Bmax triples in the loss slot's neighbour
    std::vector<int> cr(3 * (size_t)B);
    for (int b = 0; b < B; b++) { cr[3 * b] = h_idx[b]; cr[3 * b + 1] = h_y0[b]; cr[3 * b + 2] = h_x0[b]; }
    int *d_cr = reinterpret_cast<int *>(L->part);   // the weight-gradient partials are free here
    cudaMemcpyAsync(d_cr, cr.data(), cr.size() * sizeof(int), cudaMemcpyHostToDevice, st);
    const long n = (long)B * L->Hc * L->Wc;
    k_gather<<<nblk(n, 256) < 4096 ? nblk(n, 256) : 4096, 256, 0, st>>>(L->dfeat, L->dtgt, L->mask, L->Hn, L->Wn, d_cr,
                                                                       B, L->Hc, L->Wc, L->x0, L->btgt, L->bmask);
    cudaStreamSynchronize(st);   // the host table must outlive the copy
}

int lpc_tc_error(LpcState *L, cudaStream_t st) {
    int err = 0;
    if (cudaMemcpyAsync(&err, L->d_tc_err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return FS_ERR_CUDA;
    if (err || L->tc_bad) { L->tc_bad = 1; return FS_ERR_CUDA; }
    return 0;
}
