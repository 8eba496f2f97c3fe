// Host-side entry points of the surrogate kernels (nn_kernels.cu, nn_fused.cu).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

#include "nn.cuh"

namespace sbs {
namespace nn {

// Packed weights derived from the FP32 parameter vector by pack().
struct Packed {
    bf16 *wf1;  // [32][144] layer 1, [oc][tap*16 + ic]
    bf16 *wf2;  // [32][288] layer 2 forward  [oc][tap*32 + ic]
    bf16 *wf3;  // [32][288] layer 3 forward
    bf16 *wb2;  // [32][288] layer 2 transpose [ic][tap*32 + oc]
    bf16 *wb3;  // [32][288] layer 3 transpose
    float *w4;  // [9][32]   layer 4, BF16-rounded values in FP32
    float *b;   // [97]      b1 | b2 | b3 | b4
    int act;    // SBS_NN_ACT_* of the network
    unsigned *err;  // device word: nonzero after a timed-out wait of the tensor-core convolutions
};

cudaError_t features(const Fields &fs, int nf, const GridTab &g, bf16 *x, cudaStream_t st);
cudaError_t conv_forward(int layer, const bf16 *in, const Packed &p, float *y, bf16 *a, int nf, int nt, int np,
                         cudaStream_t st);
cudaError_t conv_backward_data(int layer, const bf16 *g, const Packed &p, const float *yprev, bf16 *gprev, int nf,
                               int nt, int np, cudaStream_t st);
cudaError_t conv_backward_weight(int layer, const bf16 *g, const bf16 *x, float *partial, int nblocks, float *grad,
                                 unsigned *err, int nf, int nt, int np, cudaStream_t st);
// tcgen05 weight gradients of a 3x3 layer with cin input channels: one partial row per block
// (nblocks of them, [32 * 9 * cin + 32] each) for the fixed-order reduction (nn_conv_tc.cu)
cudaError_t wgrad_tc(int cin, const bf16 *g, const bf16 *x, float *partial, int nblocks, unsigned *err, int nf, int nt,
                     int np, cudaStream_t st);
// target == null: forward only (y4). Otherwise also g4 and per-block loss partials; *nblocks_out
// receives the number of loss partials.
cudaError_t output_layer(const bf16 *a3, const Packed &p, float *y4, const float *target, float *g4,
                         double *loss_part, float inv_nmask2, const GridTab &g, int nf, cudaStream_t st,
                         int *nblocks_out);
cudaError_t output_backward(const float *g4, const bf16 *a3, const float *y3, const Packed &p, bf16 *g3,
                            float *partial, int nblocks, float *grad, const GridTab &g, int nf, cudaStream_t st);
cudaError_t adam(float *theta, float *m, float *v, const float *grad, float lr, float b1, float b2, float eps,
                 int step, cudaStream_t st);
cudaError_t pack(const float *theta, const Packed &p, cudaStream_t st);
cudaError_t apply(const float *h, size_t pitch_in, const float *y, float kout, int nt, int np, float *out,
                  size_t pitch_out, cudaStream_t st);
// target[b] = (h1[b] - h0[b]) / kout[b] for nf contiguous nt x np fields
cudaError_t targets(const float *const *h0, const float *const *h1, const float *kout, int nf, int nt, int np,
                    float *target, cudaStream_t st);
// out2[0] = max |a - b|, out2[1] = max |b| (float bits) over the masked rows of g
cudaError_t masked_error(const float *a, size_t pa, const float *b, size_t pb, const GridTab &g, unsigned *out2,
                         cudaStream_t st);

}  // namespace nn
}  // namespace sbs
