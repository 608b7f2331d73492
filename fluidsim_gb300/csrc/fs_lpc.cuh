// fs_lpc.cuh -- the learned Poisson preconditioner: a small BF16 U-Net on the
// grid of one multigrid level, evaluated on the tensor cores with FP32
// accumulation, trained on the GPU by its own forward, backward and Adam
// kernels.  No counterpart in the reference (which hands the system to
// PETSc); this header is internal to the library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define LPC_NLAYER 9
#define LPC_CIN0 16      // input features, 4 used, padded to the MMA K step
#define LPC_COUT_LAST 8  // output channels of the last layer, 1 used (MMA N step)
#define LPC_NFEAT 4      // residual, ce/mc, cn/mc, extra/mc

// Layer table: input channels (two inputs for the decoder's concatenations),
// output channels and the resolution level (0: full NN grid, 1: /2, 2: /4).
struct LpcLayer {
    int c1, c2, cout, res;
    size_t w_off, b_off;      // offsets into the FP32 parameter vector
    size_t wf_off, wb_off;    // offsets into the BF16 weight copies
};

struct LpcNet {
    LpcLayer L[LPC_NLAYER];
    size_t nparam;            // FP32 parameters (weights + biases)
    size_t nw16;              // BF16 elements of one weight copy
};

void lpc_describe(LpcNet &net);

#include <cuda_bf16.h>

// Network state, activations, gradients and the harvested training set of one
// context.  The NN grid is Hn x Wn (multiples of 4), batch up to Bmax.
struct LpcState {
    LpcNet net;
    int Hn, Wn, Bmax, Nmax, nsamp, level;
    int adam_t;
    float *w, *g, *m, *v;                       // FP32 master parameters, gradient, Adam moments
    __nv_bfloat16 *wf, *wb;                     // BF16 weight copies
    __nv_bfloat16 *x0, *a1, *s1, *p1, *a2, *s2, *p2, *a3, *a4, *u2, *a5, *u1, *a6;
    float *y;                                   // [P][LPC_COUT_LAST] FP32 output
    __nv_bfloat16 *dy, *da6, *du1, *ds1b, *da5, *du2, *ds2b, *da4, *da3, *dp2, *ds2, *da2, *dp1, *ds1, *da1;
    float *part;                                // weight-gradient partials
    size_t part_n;
    int nchunk_max;
    __nv_bfloat16 *dfeat;                       // [Nmax][Hn][Wn][LPC_CIN0]
    float *dtgt;                                // [Nmax][Hn][Wn]
    float *mask;                                // [Hn][Wn] valid cells of the padded grid
    float *btgt, *bmask;                        // batch targets and masks [Bmax][Hn][Wn]
    float *d_loss;
};

int lpc_alloc(LpcState **out, int Hn, int Wn, int Bmax, int Nmax, uint64_t seed, cudaStream_t st);
void lpc_free(LpcState *L);
// forward over B samples already in x0 (and, for training, the batch targets)
void lpc_forward(LpcState *L, int B, cudaStream_t st);
// loss and gradient of the batch (after lpc_forward); returns 0 or a CUDA error
int lpc_loss_backward(LpcState *L, int B, cudaStream_t st);
void lpc_adam(LpcState *L, float lr, cudaStream_t st);
void lpc_refresh(LpcState *L, cudaStream_t st);
// copy samples idx[0..B) of the training set into the batch buffers
void lpc_gather(LpcState *L, const int *h_idx, int B, cudaStream_t st);
