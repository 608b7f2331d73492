// fs_conv_tc.cuh -- 3x3 convolution on the tcgen05 tensor cores (see
// fs_conv_tc.cu).  Internal to the library.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stddef.h>

#define TC_MAX_CHUNKS 36   // 9 taps x up to 4 K chunks

struct TcConvArgs {
    int kc[2];                 // channels per K chunk of each source (16, 32 or 64)
    int nchunk[2];             // K chunks per tap of each source (0 for a missing second source)
    int boff[TC_MAX_CHUNKS];   // byte offset of each (tap, chunk) block in the weight image
    int cout;                  // output channels: a multiple of 16, at most 128
    int tmem_cols;             // tc_tmem_cols(cout)
    int B, H, W, TW, TH, tiles_x, tiles_y;
    const void *wimg;          // weight image (tc_weight_layout), 16-byte aligned
    int wbytes;                // its size, a multiple of 1024
    const float *bias;         // cout values or null
    int relu;
    __nv_bfloat16 *out;        // BF16 NHWC output: channels [0, split) ...
    __nv_bfloat16 *out2;       // ... and [split, cout) (split = cout: out2 unused)
    int split;
    const __nv_bfloat16 *mask, *mask2;   // ReLU masks of out / out2 (backward pass), or null
    float *out32;              // FP32 output [pix][out32_ch] instead of BF16 (null: BF16)
    int out32_ch;
    int *err;                  // set to 1 if a wait ran out
    int halo;                  // 1: halo-row tiles, 0: tap tiles (tc_halo_fits)
    int nst, stage_bytes, ntiles;   // A ring and tile count (set by tc_conv)
    int qoff[4];               // halo rows: byte offset of each K chunk in a row slot (set by tc_conv)
    int row_tx;                // halo rows: bytes one row slot receives (set by tc_conv)
};

// pixel tile of a grid W wide: TW = min(128, W) rounded up to a power of two
// (at least 16), TH = 128 / TW
void tc_tile_shape(int W, int &TW, int &TH);
// TMA descriptor of an NHWC BF16 tensor [B][H][W][C] read in chunks of kc
// channels over the tile box (halo = 0) or over one input row of TW + 2
// pixels (halo = 1); 0 or a negative error
int tc_make_map(CUtensorMap *m, const void *base, int B, int H, int W, int C, int kc, int halo);
// 1 if a layer (kc, nchunk, wbytes, W set; after tc_init) runs with halo
// rows: tiles of one 128-pixel row segment, each input row loaded once and
// shared by the three output rows that read it; needs a grid at least 128
// wide and three row slots beside the weight image
int tc_halo_fits(const TcConvArgs &a);
// tile geometry of a layer (W, H, halo set): TW, TH, tiles_x, tiles_y
void tc_set_tiles(TcConvArgs &a);
// block offsets of the weight image of a layer with sources of c1 and c2
// channels and cout outputs; fills kc, nchunk; returns the image size in bytes
int tc_weight_layout(int c1, int c2, int cout, int *boff, int *kc, int *nchunk);
// the weight image of a layer (FP32 w[9][cout][c1 + c2] on the device)
void tc_build_weights(const float *w, int c1, int c2, int cout, void *img, cudaStream_t st);
// the image of its data-gradient convolution (input channels cout, outputs
// cin; layout tc_weight_layout(cout, 0, cin))
void tc_build_weights_bwd(const float *w, int cin, int cout, void *img, cudaStream_t st);
// tensor-memory columns of an accumulator of n FP32 columns (a power of two >= 32)
int tc_tmem_cols(int n);
// dynamic shared memory of a launch with an A ring of nst stages
size_t tc_smem_bytes(int wbytes, int nst, int stage_bytes);
// once per process before the first launch (outside any stream capture):
// the kernel's shared-memory limit; 0 or a negative error
int tc_init();
// the dynamic shared memory a launch may take (0 before tc_init)
size_t tc_smem_limit();
// launch: persistent CTAs over every tile; m1 may be null (one source)
int tc_conv(const CUtensorMap *m0, const CUtensorMap *m1, const TcConvArgs &a, cudaStream_t st);
