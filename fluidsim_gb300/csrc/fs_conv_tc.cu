// fs_conv_tc.cu -- 3x3 convolutions of the learned preconditioner on the
// Blackwell tensor cores (tcgen05), fed by the tensor memory accelerator.
//
// Implicit GEMM over tiles of 128 output pixels (TW x TH pixels of one image,
// TW = min(128, W) rounded up to a power of two): D[128 px][cout] = sum over
// the 9 taps and the input channels of A[px][cin] W[cin][cout].  Persistent
// CTAs (as many as fit on the SMs) take the tiles in turn.
//   * A: for each tap (dy, dx) and each source tensor (the decoder's
//     concatenation has two), the tile's input pixels shifted by (dy, dx) --
//     one TMA load of a TW x TH x kc box of the NHWC BF16 activations, with
//     the 128-byte / 64-byte / 32-byte swizzle the MMA descriptor names; the
//     zero padding at the grid edge is TMA's out-of-bounds fill;
//   * B: the layer's weights, stored once per refresh as the exact shared-
//     memory image the MMA reads (K-major, swizzled, one block per tap and
//     source), copied in by one bulk copy;
//   * one thread issues the TMA loads into a ring of A stages that runs on
//     across the CTA's tiles, one thread issues tcgen05.mma (kind::f16,
//     BF16 x BF16 -> FP32, M = 128, N = cout) into one of two accumulators
//     in tensor memory, and tcgen05.commit frees each A stage when its MMAs
//     are done and hands a finished accumulator to the epilogue;
//   * four warps read the other accumulator (tcgen05.ld, one pixel per
//     thread) and apply bias, ReLU (or the ReLU mask of the backward pass)
//     and the BF16 store while the next tile's MMAs run.
// Halo rows (grids at least 128 wide, when three row slots fit): a tile is
// one 128-pixel row segment and each CTA takes a contiguous run of rows.  The
// producer loads each input row once, 130 pixels wide (the segment and one
// pixel either side), into a ring of row slots; the MMAs of output row y read
// rows y - 1, y, y + 1, the three x taps of a row being the same slot at
// start addresses one pixel (one swizzled K-major row) apart.  A row slot is
// freed by the commit after its last output row, so an input row crosses
// from L2 once per run instead of three times per tap row.
// Every wait on an mbarrier is bounded: a wait that runs out sets *err and
// the CTA skips the rest of its work (after a bounded wait for its own
// copies and MMAs in flight) and frees its tensor memory.
#include <cuda.h>   // CUtensorMap and its enums; the encoder is fetched through the runtime
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "fs_conv_tc.cuh"

namespace {

constexpr int kMaxStages = 32;             // A ring depth at most
constexpr int kRingBudget = 96 * 1024;     // shared memory the A ring may take
// epilogue staging: per epilogue warp 32 pixels x 16 channels in FP32, rows
// of kEpiRow floats (80 bytes: the lanes' 16-byte accesses fall on distinct
// banks), then the bias (up to 128 channels)
constexpr int kEpiRow = 20;
constexpr int kEpiBytes = 4 * 32 * kEpiRow * 4 + 128 * 4 + 16;
constexpr long kSpinLimit = 1L << 20;      // bounded waits (each try_wait may sleep ~us)

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *b, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes)
                 : "memory");
}

// true once the phase with this parity has completed; false if the wait ran out
__device__ __forceinline__ bool mbar_wait(uint64_t *b, uint32_t parity) {
    const uint32_t a = smem_u32(b);
    for (long i = 0; i < kSpinLimit; ++i) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(a), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

__device__ __forceinline__ void tma_load_4d(void *dst, const CUtensorMap *map, int c, int x, int y, int b,
                                            uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
        "%5}], [%6];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c), "r"(x), "r"(y), "r"(b), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void bulk_copy(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// Shared-memory matrix descriptor (tcgen05): start address, leading byte
// offset (unused by the swizzled K-major layouts: 1), stride byte offset
// (one 8-row swizzle atom), descriptor version 1, swizzle mode in bits 61-63.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t sbo, uint32_t mode) {
    uint64_t d = (uint64_t)((addr & 0x3FFFF) >> 4);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)mode << 61;
    return d;
}

// Coordinates of the CTA's it-th tile.  Halo rows: contiguous runs of the
// linear tile index with y fastest; otherwise tiles blockIdx.x + it * gridDim.x
// with x fastest.
__device__ __forceinline__ void tile_at(const TcConvArgs &a, int it, int &tx, int &ty, int &b) {
    long t;
    if (a.halo) {
        t = (long)blockIdx.x * a.ntiles / gridDim.x + it;
        ty = (int)(t % a.tiles_y);
        t /= a.tiles_y;
        tx = (int)(t % a.tiles_x);
        b = (int)(t / a.tiles_x);
    } else {
        t = blockIdx.x + (long)it * gridDim.x;
        tx = (int)(t % a.tiles_x);
        t /= a.tiles_x;
        ty = (int)(t % a.tiles_y);
        b = (int)(t / a.tiles_y);
    }
}

// halo rows: the run of consecutive output rows starting at the CTA's tile it
// (same image and x segment), its first row y0 and x segment tx, b
__device__ __forceinline__ int run_at(const TcConvArgs &a, int it, int ntile_cta, int &tx, int &y0, int &b) {
    tile_at(a, it, tx, y0, b);
    int n = 1;
    for (; it + n < ntile_cta; ++n) {
        int t2, y2, b2;
        tile_at(a, it + n, t2, y2, b2);
        if (y2 != y0 + n) break;
    }
    return n;
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accum) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 16 consecutive FP32 accumulator columns of this thread's TMEM lane: the
// load is issued here and its registers hold the values only after
// tmem_wait_ld, which names them as operands so that no use moves above it
__device__ __forceinline__ void tmem_ld16_issue(uint32_t addr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(addr));
}

__device__ __forceinline__ void tmem_wait_ld(uint32_t (&r)[16]) {
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                   "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                   "+r"(r[15])
                 :
                 : "memory");
}

// swizzle mode field and atom size of a K chunk of kc BF16 channels
__device__ __host__ __forceinline__ uint32_t swz_mode(int kc) { return kc == 64 ? 2u : kc == 32 ? 4u : 6u; }
__device__ __host__ __forceinline__ uint32_t swz_atom(int kc) { return 8u * 2u * (uint32_t)kc; }

// Persistent: each CTA loops over tiles blockIdx.x, + gridDim.x, ...  Warp 4
// (one thread) streams the A chunks of its tiles through a ring of nst
// stages; warp 5 (one thread) issues the MMAs of a tile into one of two
// accumulators in tensor memory while warps 0-3 drain the other (TMEM lane
// quarter w to warp w), so loads, MMAs and the epilogue of consecutive tiles
// overlap.
__global__ void __launch_bounds__(192, 4) k_conv_tc(const __grid_constant__ CUtensorMap tm0,
                                                    const __grid_constant__ CUtensorMap tm1, const TcConvArgs a) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    const int nst = a.nst;
    uint8_t *sw = smem;                               // weight image
    uint8_t *sa = smem + a.wbytes;                    // A stages (wbytes and stage_bytes are multiples of 1024)
    uint64_t *full = reinterpret_cast<uint64_t *>(sa + (size_t)nst * a.stage_bytes);
    uint64_t *empty = full + nst;
    uint64_t *tfull = empty + nst;                    // accumulator b ready (MMA -> epilogue)
    uint64_t *tempty = tfull + 2;                     // accumulator b drained (epilogue -> MMA)
    uint64_t *wbar = tempty + 2;
    uint64_t *fin = wbar + 1;                         // every MMA of this CTA complete
    uint32_t *tslot = reinterpret_cast<uint32_t *>(fin + 1);
    float *sstage = reinterpret_cast<float *>((reinterpret_cast<uintptr_t>(tslot + 1) + 15) & ~(uintptr_t)15);
    float *sbias = sstage + 4 * 32 * kEpiRow;
    __shared__ int s_fail;
    __shared__ uint64_t s_bdesc[TC_MAX_CHUNKS];      // B descriptor of each (tap, chunk) weight block
    volatile int *vfail = &s_fail;   // raised by any role whose wait ran out

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nper = a.nchunk[0] + a.nchunk[1];       // K chunks per tap
    const int nk = 9 * nper;
    const int ntile_cta =
        a.halo ? (int)((long)(blockIdx.x + 1) * a.ntiles / gridDim.x - (long)blockIdx.x * a.ntiles / gridDim.x)
               : blockIdx.x < a.ntiles ? (a.ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;

    if (threadIdx.x == 0) {
        // a CTA of this launch whose wait ran out voids the result: skip the work
        s_fail = *reinterpret_cast<volatile int *>(a.err) ? 2 : 0;
        for (int s = 0; s < nst; ++s) { mbar_init(full + s, 1); mbar_init(empty + s, 1); }
        for (int s = 0; s < 2; ++s) { mbar_init(tfull + s, 1); mbar_init(tempty + s, 4); }
        mbar_init(wbar, 1);
        mbar_init(fin, 1);
    }
    for (int i = threadIdx.x; i < a.cout; i += blockDim.x) sbias[i] = a.bias ? a.bias[i] : 0.0f;
    // the MMA descriptors of the weight blocks, once per CTA: the issuing
    // thread then adds offsets to precomputed descriptors (a descriptor's
    // start field is the address / 16, so address + 32 k is descriptor + 2 k)
    for (int i = threadIdx.x; i < 9 * (a.nchunk[0] + a.nchunk[1]); i += blockDim.x) {
        const int q = i % (a.nchunk[0] + a.nchunk[1]), kcw = a.kc[q < a.nchunk[0] ? 0 : 1];
        s_bdesc[i] = smem_desc(smem_u32(sw + a.boff[i]), swz_atom(kcw), swz_mode(kcw));
    }
    if (threadIdx.x == 0) {
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    if (s_fail == 2 || ntile_cta == 0) return;   // uniform over the CTA
    if (warp == 4) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                     "r"((uint32_t)(2 * a.tmem_cols))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;

    if (warp == 4 && lane == 0 && a.halo) {
        // producer, halo rows: the weight image, then for each run of output
        // rows y0 .. y0 + n - 1 the input rows y0 - 1 .. y0 + n, one slot each
        // (all K chunks of the row; rows outside the grid read TMA's zero fill)
        mbar_expect_tx(wbar, (uint32_t)a.wbytes);
        bulk_copy(sw, a.wimg, (uint32_t)a.wbytes, wbar);
        long g = 0;   // rows issued
        bool go = true;
        for (int it = 0; go && it < ntile_cta && !*vfail;) {
            int tx, y0, b;
            const int n = run_at(a, it, ntile_cta, tx, y0, b);
            for (int r = y0 - 1; r <= y0 + n; ++r, ++g) {
                const int s = (int)(g % nst);
                const long u = g / nst;
                if (u > 0 && !mbar_wait(empty + s, (uint32_t)((u - 1) & 1))) { atomicExch(&s_fail, 1); go = false; break; }
                mbar_expect_tx(full + s, (uint32_t)a.row_tx);
                uint8_t *dst = sa + (size_t)s * a.stage_bytes;
                for (int q = 0; q < nper; ++q) {
                    const int src = q < a.nchunk[0] ? 0 : 1, j = src ? q - a.nchunk[0] : q;
                    tma_load_4d(dst + a.qoff[q], src ? &tm1 : &tm0, j * a.kc[src], tx * a.TW - 1, r, b, full + s);
                }
            }
            it += n;
        }
        for (long h = g - nst > 0 ? g - nst : 0; h < g; ++h)
            mbar_wait(full + (int)(h % nst), (uint32_t)((h / nst) & 1));
    } else if (warp == 5 && lane == 0 && a.halo) {
        // MMA issuer, halo rows: output row y of a run reads row slots of
        // input rows y - 1, y, y + 1 (row loads g + k, g + k + 1, g + k + 2);
        // tap (dy, dx) = that slot at dx pixels' offset
        const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(a.cout >> 3) << 17) |
                               ((uint32_t)(128 >> 4) << 24);
        bool ok = mbar_wait(wbar, 0);
        long g = 0;   // row load of the current run's first input row
        for (int it = 0; ok && it < ntile_cta;) {
            int tx, y0, b;
            const int n = run_at(a, it, ntile_cta, tx, y0, b);
            for (int k = 0; ok && k < n; ++k, ++it) {
                const int bs = it & 1, u = it >> 1;
                if (u > 0 && !mbar_wait(tempty + bs, (uint32_t)((u - 1) & 1))) { ok = false; break; }
                tc_fence_after();
                const uint32_t acc = tmem + (uint32_t)(bs * a.tmem_cols);
                uint32_t accum = 0;
                for (int dr = 0; ok && dr < 3; ++dr) {
                    const long L = g + k + dr;
                    const int s = (int)(L % nst);
                    if (!mbar_wait(full + s, (uint32_t)((L / nst) & 1)) || *vfail) { ok = false; break; }
                    tc_fence_after();
                    const uint32_t rbase = smem_u32(sa + (size_t)s * a.stage_bytes);
                    for (int q = 0; q < nper; ++q) {
                        const int kcw = a.kc[q < a.nchunk[0] ? 0 : 1], nk16 = kcw / 16;
                        // the chunk's A descriptor at dx = 0; each dx one pixel row (2 kcw bytes) on
                        const uint64_t a0 = smem_desc(rbase + (uint32_t)a.qoff[q], swz_atom(kcw), swz_mode(kcw));
                        const uint64_t *bd = s_bdesc + dr * 3 * nper + q;
                        for (int dx = 0; dx < 3; ++dx) {
                            const uint64_t ad = a0 + (uint64_t)(dx * kcw / 8), bdx = bd[dx * nper];
                            for (int kk = 0; kk < nk16; ++kk) {
                                mma_bf16(acc, ad + 2 * kk, bdx + 2 * kk, idesc, accum);
                                accum = 1;
                            }
                        }
                    }
                }
                if (!ok) break;
                mma_commit(tfull + bs);
                // input row y - 1 has no later reader; at the run's end neither have y, y + 1
                mma_commit(empty + (int)((g + k) % nst));
                if (k == n - 1) {
                    mma_commit(empty + (int)((g + k + 1) % nst));
                    mma_commit(empty + (int)((g + k + 2) % nst));
                }
            }
            g += n + 2;
        }
        if (!ok) atomicExch(&s_fail, 1);
        mma_commit(fin);
        mbar_wait(fin, 0);
    } else if (warp == 4 && lane == 0) {
        // producer: the weight image, then the A chunks of each tile, tap by tap
        mbar_expect_tx(wbar, (uint32_t)a.wbytes);
        bulk_copy(sw, a.wimg, (uint32_t)a.wbytes, wbar);
        long g = 0;   // chunks issued
        for (int it = 0; it < ntile_cta && !*vfail; ++it) {
            int tx, ty, b;
            tile_at(a, it, tx, ty, b);
            const int x0 = tx * a.TW, y0 = ty * a.TH;
            for (int kc = 0; kc < nk; ++kc, ++g) {
                const int s = (int)(g % nst);
                const long n = g / nst;
                if (n > 0 && !mbar_wait(empty + s, (uint32_t)((n - 1) & 1))) { atomicExch(&s_fail, 1); break; }
                const int t = kc / nper, q = kc - t * nper;
                const int src = q < a.nchunk[0] ? 0 : 1, j = src ? q - a.nchunk[0] : q;
                const int kcw = a.kc[src];
                mbar_expect_tx(full + s, (uint32_t)(128 * kcw * 2));
                tma_load_4d(sa + (size_t)s * a.stage_bytes, src ? &tm1 : &tm0, j * kcw, x0 + t % 3 - 1,
                            y0 + t / 3 - 1, b, full + s);
            }
        }
        // leave no copy in flight: the last nst chunks issued are complete
        for (long h = g - nst > 0 ? g - nst : 0; h < g; ++h)
            mbar_wait(full + (int)(h % nst), (uint32_t)((h / nst) & 1));
    } else if (warp == 5 && lane == 0) {
        // MMA issuer
        const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(a.cout >> 3) << 17) |
                               ((uint32_t)(128 >> 4) << 24);
        bool ok = mbar_wait(wbar, 0);
        long g = 0;
        for (int it = 0; ok && it < ntile_cta; ++it) {
            const int bs = it & 1, u = it >> 1;
            if (u > 0 && !mbar_wait(tempty + bs, (uint32_t)((u - 1) & 1))) { ok = false; break; }
            tc_fence_after();
            const uint32_t acc = tmem + (uint32_t)(bs * a.tmem_cols);
            for (int kc = 0; kc < nk; ++kc, ++g) {
                const int s = (int)(g % nst);
                if (!mbar_wait(full + s, (uint32_t)((g / nst) & 1)) || *vfail) { ok = false; break; }
                tc_fence_after();
                const int t = kc / nper, q = kc - t * nper;
                const int src = q < a.nchunk[0] ? 0 : 1;
                const int kcw = a.kc[src];
                const uint64_t ad = smem_desc(smem_u32(sa + (size_t)s * a.stage_bytes), swz_atom(kcw), swz_mode(kcw));
                const uint64_t bd = s_bdesc[t * nper + q];
                for (int k = 0; k < kcw / 16; ++k)
                    mma_bf16(acc, ad + 2 * k, bd + 2 * k, idesc, (kc > 0 || k > 0) ? 1u : 0u);
                mma_commit(empty + s);
            }
            if (ok) mma_commit(tfull + bs);
        }
        if (!ok) atomicExch(&s_fail, 1);
        // every MMA this thread issued has completed before the memory goes back
        mma_commit(fin);
        mbar_wait(fin, 0);
    } else if (warp < 4) {
        // epilogue: thread = one pixel of the tile (its TMEM lane).  The
        // accumulator is read 16 columns at a time, the next group's load in
        // flight while the current one is written out.
        const int p = warp * 32 + lane;
        const int lgw = __ffs(a.TW) - 1;                 // TW is a power of two
        const int ps = a.out32 ? 2 : 1;                 // log2 lanes per pixel in the coalesced stores
        const int sub = lane & ((1 << ps) - 1);          // the lane's 16-byte piece of a pixel's row
        const int q0 = warp * 32;                        // first tile pixel of the warp
        float *st = sstage + warp * 32 * kEpiRow;       // this warp's staging rows
        const bool narrow = a.out32 && !((a.out32_ch & 3) == 0 && a.out32_ch >= 16);
        for (int it = 0; it < ntile_cta; ++it) {
            const int bs = it & 1, u = it >> 1;
            bool ok = mbar_wait(tfull + bs, (uint32_t)(u & 1));
            ok = __all_sync(0xffffffffu, ok);   // warp-uniform (tcgen05.ld is warp-collective)
            if (!ok) { atomicExch(&s_fail, 1); break; }
            tc_fence_after();
            int tx, ty, b;
            tile_at(a, it, tx, ty, b);
            const int xb = tx * a.TW, yb = ty * a.TH;
            const int px = xb + (p & (a.TW - 1)), py = yb + (p >> lgw);
            const bool in = px < a.W && py < a.H;
            const long pix = ((long)b * a.H + py) * a.W + px;
            // the pixels this lane stores in the coalesced passes (4 FP32 passes
            // of 8 pixels, or 2 BF16 passes of 16), -1 outside the grid
            long qp[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int pq = q0 + (lane >> ps) + i * (32 >> ps);
                const int qx = xb + (pq & (a.TW - 1)), qy = yb + (pq >> lgw);
                qp[i] = (i < (1 << ps) && qx < a.W && qy < a.H) ? ((long)b * a.H + qy) * a.W + qx : -1;
            }
            const uint32_t acc = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(bs * a.tmem_cols);
            uint32_t r[16];
            __syncwarp();
            tmem_ld16_issue(acc, r);
            for (int c0 = 0; c0 < a.cout; c0 += 16) {
                __syncwarp();
                tmem_wait_ld(r);
                float v[16];
#pragma unroll
                for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
                if (c0 + 16 < a.cout) tmem_ld16_issue(acc + (uint32_t)(c0 + 16), r);   // next group in flight
                const float4 *b4 = reinterpret_cast<const float4 *>(sbias + c0);
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const float4 bb = b4[j];
                    v[4 * j] += bb.x; v[4 * j + 1] += bb.y; v[4 * j + 2] += bb.z; v[4 * j + 3] += bb.w;
                }
                if (a.out32 && !narrow && c0 + 16 > a.out32_ch) continue;   // past the output's channels
                if (narrow) {   // a narrow FP32 output (the prediction channel)
                    if (in) {
#pragma unroll
                        for (int i = 0; i < 16; ++i)
                            if (c0 + i < a.out32_ch) a.out32[pix * a.out32_ch + c0 + i] = v[i];
                    }
                    continue;
                }
                // bias and ReLU on this lane's pixel, staged; then the warp
                // writes its 32 pixels with 16-byte stores, consecutive lanes
                // on consecutive addresses
                if (a.relu && !a.out32) {
#pragma unroll
                    for (int i = 0; i < 16; ++i) v[i] = fmaxf(v[i], 0.0f);
                }
                __syncwarp();   // the previous group's staging rows are read
                float4 *row = reinterpret_cast<float4 *>(st + lane * kEpiRow);
#pragma unroll
                for (int j = 0; j < 4; ++j) row[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
                __syncwarp();
                if (a.out32) {
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        if (qp[i] < 0) continue;
                        const int q = (lane >> 2) + 8 * i;
                        *reinterpret_cast<float4 *>(a.out32 + qp[i] * a.out32_ch + c0 + 4 * sub) =
                            reinterpret_cast<const float4 *>(st + q * kEpiRow)[sub];
                    }
                    continue;
                }
                // BF16 output, split over up to two tensors (the backward pass's
                // concatenated inputs): channels [0, split) to out, the rest to out2
                __nv_bfloat16 *dst;
                int cc, cs;
                const __nv_bfloat16 *msk;
                if (c0 < a.split) { dst = a.out; cc = c0; cs = a.split; msk = a.mask; }
                else { dst = a.out2; cc = c0 - a.split; cs = a.cout - a.split; msk = a.mask2; }
#pragma unroll
                for (int i = 0; i < 2; ++i) {
                    if (qp[i] < 0) continue;
                    const int q = (lane >> 1) + 16 * i;
                    const float *f = st + q * kEpiRow + 8 * sub;
                    float w[8];
#pragma unroll
                    for (int k = 0; k < 8; ++k) w[k] = f[k];
                    const long off = qp[i] * cs + cc + 8 * sub;
                    if (msk) {   // ReLU mask of the backward pass: 8 BF16 values in one load
                        const uint4 mk = *reinterpret_cast<const uint4 *>(msk + off);
                        const uint32_t mw[4] = {mk.x, mk.y, mk.z, mk.w};
#pragma unroll
                        for (int k = 0; k < 8; ++k) {
                            const uint16_t hb = (uint16_t)(mw[k >> 1] >> (16 * (k & 1)));
                            if (!(__bfloat162float(__ushort_as_bfloat16(hb)) > 0.0f)) w[k] = 0.0f;
                        }
                    }
                    uint32_t pk[4];
#pragma unroll
                    for (int k = 0; k < 8; k += 2) {
                        const __nv_bfloat162 h = __floats2bfloat162_rn(w[k], w[k + 1]);
                        pk[k / 2] = *reinterpret_cast<const uint32_t *>(&h);
                    }
                    *reinterpret_cast<uint4 *>(dst + off) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
                }
            }
            // this warp's lanes of accumulator bs are read: hand it back
            tc_fence_before();
            __syncwarp();
            if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(tempty + bs))
                                        : "memory");
        }
    }
    tc_fence_before();
    __syncthreads();
    if (s_fail && threadIdx.x == 0) atomicExch(a.err, 1);
    tc_fence_after();
    __syncwarp();
    if (warp == 4)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"((uint32_t)(2 * a.tmem_cols))
                     : "memory");
}

// The weight image of one layer from FP32 weights w[9][cout][c1 + c2]: per
// (tap, K chunk) block, row co holds the chunk's kc input channels in BF16,
// rows of 2 kc bytes with the 16-byte pieces of row r permuted as the
// swizzle mode permutes them (128 B: piece ^ (r & 7); 64 B: ^ ((r >> 1) & 3);
// 32 B: ^ ((r >> 2) & 1)) -- the layout the MMA descriptor reads.
// transposed = 1: the image of the data-gradient convolution of a layer
// w[9][cin][cout] (input channels = that layer's cout = c1 here, outputs its
// cin = cout here): entry (t, co, ci) = w[8 - t][ci][co], the flipped taps.
__global__ void k_tc_weights(const float *w, int c1, int c2, int cout, TcConvArgs lay, uint8_t *img, int transposed) {
    const int cin = c1 + c2, nper = lay.nchunk[0] + lay.nchunk[1];
    const int n = 9 * cout * cin;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int t = i / (cout * cin), rem = i - t * cout * cin, co = rem / cin, ci = rem - co * cin;
        const float wv = transposed ? w[((size_t)(8 - t) * cin + ci) * cout + co] : w[i];
        const int src = ci < c1 ? 0 : 1, cl = src ? ci - c1 : ci, kc = lay.kc[src];
        const int j = cl / kc, e = cl - j * kc;
        const int q = src ? lay.nchunk[0] + j : j;
        const int piece = e >> 3, f = kc == 64 ? (co & 7) : kc == 32 ? ((co >> 1) & 3) : ((co >> 2) & 1);
        const size_t off = (size_t)lay.boff[t * nper + q] + (size_t)co * (2 * kc) + (size_t)(piece ^ f) * 16 +
                           (size_t)(e & 7) * 2;
        *reinterpret_cast<__nv_bfloat16 *>(img + off) = __float2bfloat16_rn(wv);
    }
}

// tcgen05.mma issue rate, the bound of the convolutions: one thread issues
// nmma MMAs (M = 128, N = n, K = 16, BF16 x BF16 -> FP32, both operands in
// zeroed shared memory with the 128-byte swizzle) into one accumulator;
// out = SM cycles from the first issue to the completion of the last.
__global__ void __launch_bounds__(128) k_mma_rate(int nmma, int n, unsigned long long *out, int *err) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *sm = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    __shared__ uint64_t bar;
    __shared__ uint32_t slot;
    for (int i = threadIdx.x; i < 48 * 1024 / 4; i += blockDim.x) reinterpret_cast<uint32_t *>(sm)[i] = 0u;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (threadIdx.x < 32) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" ::"r"(smem_u32(&slot))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = slot;
    if (threadIdx.x == 0) {
        const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
                               ((uint32_t)(128 >> 4) << 24);
        const uint32_t a = smem_u32(sm), b = smem_u32(sm + 16384);   // 128 rows of A, up to 256 of B
        const long long t0 = clock64();
        for (int i = 0; i < nmma; ++i)
            mma_bf16(tmem, smem_desc(a + 32 * (i & 3), 1024, 2), smem_desc(b + 32 * (i & 3), 1024, 2), idesc,
                     i > 0 ? 1u : 0u);
        mma_commit(&bar);
        const bool ok = mbar_wait(&bar, 0);
        out[0] = (unsigned long long)(clock64() - t0);
        if (!ok) atomicExch(err, 1);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (threadIdx.x < 32)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(tmem) : "memory");
}

}  // namespace

// SM cycles per tcgen05.mma (M = 128, N = n, K = 16, BF16) issued back to back
// by one thread, on the current device: 2048 instructions after a warm-up
// launch, one CTA, timed with clock64 (no clocks or settings touched).
extern "C" int fs_mma_rate(int32_t n, double *cycles_per_mma) {
    if (!cycles_per_mma || n < 16 || n > 256 || n % 16) return -1;
    const int smem = 49 * 1024 + 1024;
    if (cudaFuncSetAttribute(k_mma_rate, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
        return -2;
    unsigned long long *d = nullptr;
    if (cudaMalloc(&d, 16) != cudaSuccess) return -2;
    int *err = reinterpret_cast<int *>(d + 1);
    int rc = cudaMemset(d, 0, 16) == cudaSuccess ? 0 : -2;
    const int nmma = 2048;
    for (int rep = 0; rep < 2 && !rc; ++rep) {
        k_mma_rate<<<1, 128, smem>>>(nmma, n, d, err);
        if (cudaDeviceSynchronize() != cudaSuccess) rc = -3;
    }
    unsigned long long h[2] = {0, 0};
    if (!rc && cudaMemcpy(h, d, 16, cudaMemcpyDeviceToHost) != cudaSuccess) rc = -3;
    if (!rc && (int)h[1]) rc = -6;   // the wait for the MMAs ran out
    if (!rc) *cycles_per_mma = (double)h[0] / nmma;
    cudaFree(d);
    return rc;
}

// ----------------------------------------------------------------------- host
namespace {
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn g_encode = nullptr;

int load_encoder() {
    if (g_encode) return 0;
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn)
        return -1;
    g_encode = reinterpret_cast<EncodeTiledFn>(fn);
    return 0;
}
}  // namespace

int tc_tmem_cols(int n) {
    int c = 32;
    while (c < n) c *= 2;
    return c;
}

void tc_tile_shape(int W, int &TW, int &TH) {
    TW = 16;
    while (TW < 128 && TW < W) TW *= 2;
    TH = 128 / TW;
}

int tc_make_map(CUtensorMap *m, const void *base, int B, int H, int W, int C, int kc, int halo) {
    if (load_encoder()) return -1;
    if (!(kc == 16 || kc == 32 || kc == 64) || C % kc || (reinterpret_cast<uintptr_t>(base) & 15)) return -2;
    int TW, TH;
    tc_tile_shape(W, TW, TH);
    if (halo) {   // one input row: the segment and one pixel either side
        if (TH != 1) return -2;
        TW += 2;
    }
    const cuuint64_t dims[4] = {(cuuint64_t)C, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)B};
    const cuuint64_t strides[3] = {(cuuint64_t)C * 2, (cuuint64_t)W * C * 2, (cuuint64_t)H * W * C * 2};
    const cuuint32_t box[4] = {(cuuint32_t)kc, (cuuint32_t)TW, (cuuint32_t)TH, 1};
    const cuuint32_t es[4] = {1, 1, 1, 1};
    const CUtensorMapSwizzle sw = kc == 64 ? CU_TENSOR_MAP_SWIZZLE_128B
                                  : kc == 32 ? CU_TENSOR_MAP_SWIZZLE_64B
                                             : CU_TENSOR_MAP_SWIZZLE_32B;
    const CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void *>(base), dims, strides, box,
                                es, CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? 0 : -3;
}

int tc_weight_layout(int c1, int c2, int cout, int *boff, int *kc, int *nchunk) {
    kc[0] = c1 >= 64 ? 64 : c1;
    kc[1] = c2 >= 64 ? 64 : c2;
    nchunk[0] = c1 / (kc[0] ? kc[0] : 1);
    nchunk[1] = c2 ? c2 / kc[1] : 0;
    const int nper = nchunk[0] + nchunk[1];
    int off = 0;
    for (int t = 0; t < 9; ++t)
        for (int q = 0; q < nper; ++q) {
            const int src = q < nchunk[0] ? 0 : 1;
            boff[t * nper + q] = off;
            const int bytes = cout * kc[src] * 2;
            off += (bytes + 1023) / 1024 * 1024;
        }
    return off;
}

void tc_set_tiles(TcConvArgs &a) {
    tc_tile_shape(a.W, a.TW, a.TH);
    a.tiles_x = (a.W + a.TW - 1) / a.TW;
    a.tiles_y = (a.H + a.TH - 1) / a.TH;
}

static void build_image(const float *w, int c1, int c2, int cout, void *img, int transposed, cudaStream_t st) {
    TcConvArgs lay = {};
    const int bytes = tc_weight_layout(c1, c2, cout, lay.boff, lay.kc, lay.nchunk);
    cudaMemsetAsync(img, 0, (size_t)bytes, st);
    const int n = 9 * cout * (c1 + c2);
    k_tc_weights<<<(n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024, 256, 0, st>>>(
        w, c1, c2, cout, lay, reinterpret_cast<uint8_t *>(img), transposed);
}

void tc_build_weights(const float *w, int c1, int c2, int cout, void *img, cudaStream_t st) {
    build_image(w, c1, c2, cout, img, 0, st);
}

void tc_build_weights_bwd(const float *w, int cin, int cout, void *img, cudaStream_t st) {
    build_image(w, cout, 0, cin, img, 1, st);
}

// A ring of a layer: stages of 128 pixels x the larger K chunk, as many as
// fit the budget and the limit left by the weight image (at least 2, at most
// the chunks of one tile)
static void ring_shape(const TcConvArgs &a, size_t limit, int &nst, int &stage_bytes) {
    const int kcmax = a.kc[0] > a.kc[1] ? a.kc[0] : a.kc[1];
    stage_bytes = 128 * kcmax * 2;
    const int nk = 9 * (a.nchunk[0] + a.nchunk[1]);
    long room = (long)limit - 1024 - a.wbytes - 256 - kEpiBytes;
    if (room > kRingBudget) room = kRingBudget;
    nst = (int)(room / stage_bytes);
    if (nst > kMaxStages) nst = kMaxStages;
    if (nst > nk) nst = nk;   // one tile ahead: a deeper ring costs CTAs per SM (measured slower)
    if (nst < 2) nst = 2;
}

// halo rows: a row slot holds each K chunk of one input row (130 pixels) in a
// block of its own, 1024-aligned for the swizzle; fills qoff and row_tx
static int halo_slot(TcConvArgs &a) {
    const int nper = a.nchunk[0] + a.nchunk[1];
    int off = 0, tx = 0;
    for (int q = 0; q < nper && q < 4; ++q) {
        const int kc = a.kc[q < a.nchunk[0] ? 0 : 1], bytes = 130 * kc * 2;
        a.qoff[q] = off;
        tx += bytes;
        off += (bytes + 1023) / 1024 * 1024;
    }
    a.row_tx = tx;
    return off;
}

size_t tc_smem_bytes(int wbytes, int nst, int stage_bytes) {
    return 1024 + (size_t)wbytes + (size_t)nst * stage_bytes + 8 * (2 * (size_t)nst + 6) + 16 + kEpiBytes;
}

namespace {
// the dynamic shared memory a launch may take: the device's opt-in limit
// per block less the kernel's static shared memory; the SM count
size_t g_smem_max = 0;
size_t g_smem_sm = 0;   // shared memory per SM
int g_nsm = 0;
int g_regs = 0;         // registers per thread of the kernel
}  // namespace

int tc_init() {
    if (g_smem_max) return 0;
    if (load_encoder()) return -1;
    int dev = 0, optin = 0;
    cudaFuncAttributes fa;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
        cudaFuncGetAttributes(&fa, k_conv_tc) != cudaSuccess)
        return -2;
    const int dyn = optin - (int)fa.sharedSizeBytes;
    if (cudaFuncSetAttribute(k_conv_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn) != cudaSuccess) return -2;
    // all of the unified L1/shared storage as shared memory, so that several
    // CTAs fit on an SM (the kernel reads nothing through L1)
    if (cudaFuncSetAttribute(k_conv_tc, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared) != cudaSuccess)
        return -2;
    int smsm = 0;
    if (cudaDeviceGetAttribute(&g_nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&smsm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess)
        return -2;
    g_smem_sm = (size_t)smsm;
    g_regs = fa.numRegs;
    g_smem_max = (size_t)dyn;
    return 0;
}

size_t tc_smem_limit() { return g_smem_max; }

int tc_halo_fits(const TcConvArgs &a0) {
    if (!g_smem_max || a0.W < 128 || a0.nchunk[0] + a0.nchunk[1] > 4) return 0;
    TcConvArgs a = a0;
    const long room = (long)g_smem_max - 1024 - a.wbytes - 256 - kEpiBytes;
    return room >= 3L * halo_slot(a) ? 1 : 0;
}

int tc_conv(const CUtensorMap *m0, const CUtensorMap *m1, const TcConvArgs &a0, cudaStream_t st) {
    if (!g_smem_max) return -2;
    TcConvArgs a = a0;
    if (a.halo) {
        // row slots: three in use and up to two loading ahead
        if (!tc_halo_fits(a)) return -2;
        a.stage_bytes = halo_slot(a);
        const long room = (long)g_smem_max - 1024 - a.wbytes - 256 - kEpiBytes;
        a.nst = (int)(room / a.stage_bytes);
        if (a.nst > 5) a.nst = 5;
    } else {
        ring_shape(a, g_smem_max, a.nst, a.stage_bytes);
    }
    const size_t smem = tc_smem_bytes(a.wbytes, a.nst, a.stage_bytes);
    if (smem > g_smem_max) return -2;
    a.ntiles = a.tiles_x * a.tiles_y * a.B;
    // CTAs per SM: what shared memory allows, and two accumulators each in
    // the 512 tensor-memory columns
    // (counted here from the kernel's registers and the SM's shared memory:
    // the occupancy query answers 1 for this kernel, while three 47 KB CTAs
    // are resident at once when launched one tile per CTA)
    const int by_smem = (int)(g_smem_sm / (smem + 1024));
    const int regs_cta = ((g_regs + 7) / 8 * 8) * 192;
    const int by_regs = 65536 / regs_cta;
    int per_sm = by_smem < by_regs ? by_smem : by_regs;
    const int tmem_cap = 512 / (2 * a.tmem_cols);
    if (per_sm > tmem_cap) per_sm = tmem_cap;
    if (per_sm < 1) return -2;
    const long grid = (long)g_nsm * per_sm < a.ntiles ? (long)g_nsm * per_sm : a.ntiles;
    k_conv_tc<<<(int)grid, 192, smem, st>>>(*m0, m1 ? *m1 : *m0, a);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : -100 - (int)e;
}

// One 3x3 convolution through the tcgen05 path on host arrays (tests): in1
// [B][H][W][c1] and in2 [B][H][W][c2] (may be null) as BF16 bit patterns,
// w [9][cout][c1 + c2] and bias [cout] in FP32; mode 0 writes FP32
// out[B][H][W][cout] (bias, no ReLU), mode 1 BF16 bit patterns (bias, ReLU).
extern "C" int fs_conv3x3_tc(int32_t B, int32_t H, int32_t W, int32_t c1, int32_t c2, int32_t cout,
                             const uint16_t *in1, const uint16_t *in2, const float *w, const float *bias,
                             int32_t mode, void *out) {
    if (B < 1 || H < 1 || W < 1 || cout < 16 || cout > 128 || cout % 16 || !in1 || !w || !out ||
        (c2 > 0 && !in2) || c1 < 16 || c1 % 16 || c2 < 0 || c2 % 16 || (c1 > 64 && c1 % 64) ||
        (c2 > 64 && c2 % 64) || (mode != 0 && mode != 1))
        return -1;
    const size_t P = (size_t)B * H * W, cin = (size_t)c1 + c2;
    TcConvArgs a = {};
    a.wbytes = tc_weight_layout(c1, c2, cout, a.boff, a.kc, a.nchunk);
    if (9 * (a.nchunk[0] + a.nchunk[1]) > TC_MAX_CHUNKS) return -1;
    uint8_t *d = nullptr;
    const size_t o_in1 = 0, o_in2 = o_in1 + (P * c1 * 2 + 1023) / 1024 * 1024,
                 o_w = o_in2 + (P * c2 * 2 + 1023) / 1024 * 1024, o_b = o_w + 9 * cin * cout * 4,
                 o_img = (o_b + cout * 4 + 1023) / 1024 * 1024, o_out = o_img + (size_t)a.wbytes,
                 o_err = o_out + P * cout * 4, total = o_err + 16;
    if (tc_init()) return -3;
    if (cudaMalloc(&d, total) != cudaSuccess) return -2;
    int rc = 0;
    cudaStream_t st = 0;
    cudaMemcpy(d + o_in1, in1, P * c1 * 2, cudaMemcpyHostToDevice);
    if (c2) cudaMemcpy(d + o_in2, in2, P * c2 * 2, cudaMemcpyHostToDevice);
    cudaMemcpy(d + o_w, w, 9 * cin * cout * 4, cudaMemcpyHostToDevice);
    if (bias) cudaMemcpy(d + o_b, bias, cout * 4, cudaMemcpyHostToDevice);
    else cudaMemset(d + o_b, 0, cout * 4);
    cudaMemset(d + o_err, 0, 16);
    tc_build_weights(reinterpret_cast<float *>(d + o_w), c1, c2, cout, d + o_img, st);
    a.cout = cout;
    a.B = B; a.H = H; a.W = W;
    a.halo = tc_halo_fits(a);
    CUtensorMap m0, m1;
    if (tc_make_map(&m0, d + o_in1, B, H, W, c1, a.kc[0], a.halo) ||
        (c2 && tc_make_map(&m1, d + o_in2, B, H, W, c2, a.kc[1], a.halo)))
        rc = -3;
    if (!rc) {
        a.tmem_cols = tc_tmem_cols(cout);
        tc_set_tiles(a);
        a.wimg = d + o_img;
        a.bias = reinterpret_cast<float *>(d + o_b);
        a.relu = mode == 1;
        a.split = cout;
        if (mode == 0) { a.out32 = reinterpret_cast<float *>(d + o_out); a.out32_ch = cout; }
        else a.out = reinterpret_cast<__nv_bfloat16 *>(d + o_out);
        a.err = reinterpret_cast<int *>(d + o_err);
        const cudaError_t pre = cudaGetLastError();   // anything the set-up left
        rc = pre != cudaSuccess ? -100 - (int)pre : tc_conv(&m0, c2 ? &m1 : nullptr, a, st);
    }
    int err = 0;
    if (!rc) {
        const cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) rc = -100 - (int)e;
    }
    if (!rc) cudaMemcpy(&err, d + o_err, 4, cudaMemcpyDeviceToHost);
    if (!rc && err) rc = -6;
    if (!rc) cudaMemcpy(out, d + o_out, P * cout * (mode == 0 ? 4 : 2), cudaMemcpyDeviceToHost);
    cudaFree(d);
    return rc;
}
