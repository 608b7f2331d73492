// fs_lpc.cuh -- the learned Poisson preconditioner: a BF16 U-Net on the fine
// grid of the Poisson system, evaluated on the tcgen05 tensor cores with FP32
// accumulation, trained on the GPU by its own forward, backward and Adam
// kernels.  No counterpart in the reference (which hands the system to
// PETSc); this header is internal to the library.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "fs_conv_tc.cuh"

#define LPC_NLAYER 12
#define LPC_NLEV 4       // resolution levels (three 2x2 poolings)
#define LPC_CIN0 16      // input features, LPC_NFEAT used, padded to the MMA K step
#define LPC_COUT_LAST 16 // output channels of the last layer, 1 used (the MMA's smallest N)
#define LPC_NFEAT 4      // residual, the two face-coupling shares (grid spacing), net charge

// Layer table: input channels (two inputs for the decoder's concatenations),
// output channels and the resolution level (0: the fine grid, l: / 2^l).
struct LpcLayer {
    int c1, c2, cout, res;
    size_t w_off, b_off;      // offsets into the FP32 parameter vector
    size_t img_f, img_b;      // byte offsets of the forward / backward-data weight images
    int bytes_f, bytes_b;     // their sizes
};

struct LpcNet {
    LpcLayer L[LPC_NLAYER];
    size_t nparam;            // FP32 parameters (weights + biases)
    size_t img_bytes;         // all weight images
};

void lpc_describe(LpcNet &net);

// Network state, activations, gradients and the harvested training set of one
// context.  Activations and gradients hold up to cap0 fine-level pixels (the
// larger of one full grid and a training batch of crops); the training pairs
// are full grids of Hn x Wn (multiples of 8) cells.
struct LpcState {
    LpcNet net;
    int Hn, Wn, Hc, Wc, Bmax, Nmax, nsamp;
    long cap0;
    int adam_t;
    float *w, *g, *m, *v;                       // FP32 master parameters, gradient, Adam moments
    uint8_t *img;                               // BF16 weight images (forward, backward data)
    // activations (NHWC BF16): x0 input; a*/s* encoder, p* pooled, b3
    // bottleneck, u* upsampled, d* decoder outputs
    __nv_bfloat16 *x0, *a0, *s0, *p0, *a1, *s1, *p1, *a2, *s2, *p2, *a3, *b3, *u2, *d2, *u1, *d1, *u0, *d0;
    float *y;                                   // [P] FP32 output (channel 0)
    // gradients
    __nv_bfloat16 *dy, *dd0, *du0, *ds0b, *dd1, *du1, *ds1b, *dd2, *du2, *ds2b, *db3, *da3, *dp2, *ds2, *da2,
        *dp1, *ds1, *da1, *dp0, *ds0, *da0;
    float *part;                                // weight-gradient partials
    size_t part_n;
    int nchunk_max;
    __nv_bfloat16 *dfeat;                       // [Nmax][Hn][Wn][LPC_NFEAT] harvested inputs
    float *dtgt;                                // [Nmax][Hn][Wn] harvested targets
    float *mask;                                // [Hn][Wn] interior cells of the padded grid
    float *btgt, *bmask;                        // batch targets and masks [cap0]
    float *d_loss;
    int *d_tc_err;                              // set by a tensor-core convolution whose wait ran out
    int tc_bad;                                 // a convolution failed: the network stays off
};

int lpc_alloc(LpcState **out, int Hn, int Wn, int Hc, int Wc, int Bmax, int Nmax, uint64_t seed, cudaStream_t st);
void lpc_free(LpcState *L);
// forward over B images of H x W cells already in x0 (training: the batch targets too)
int lpc_forward(LpcState *L, int B, int H, int W, cudaStream_t st);
// loss and gradient of the batch (after lpc_forward); returns 0 or an error
int lpc_loss_backward(LpcState *L, int B, int H, int W, cudaStream_t st);
void lpc_adam(LpcState *L, float lr, cudaStream_t st);
void lpc_refresh(LpcState *L, cudaStream_t st);
// B random crops of Hc x Wc cells from the training pairs (host-drawn pair
// indices and crop origins) into the batch buffers
void lpc_gather(LpcState *L, const int *h_idx, const int *h_y0, const int *h_x0, int B, cudaStream_t st);
// 0, or FS_ERR_CUDA after a tensor-core convolution failed (its bounded wait
// ran out or it could not be launched): the network is then left off
int lpc_tc_error(LpcState *L, cudaStream_t st);
