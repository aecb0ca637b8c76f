// The tensor-core (tcgen05) path of the U-Net's 3x3 convolution products
// (forward, data gradient, weight gradient), defined in unet_tc.cu.
#pragma once
#include "common.cuh"

namespace dyfox {

// One forward (mode 0) or data-gradient (mode 1) product.
//   act: (N, H, W, Ck) bf16, the forward input X or the masked output
//        gradient G;
//   wk:  (Ncols, 9 Ck) bf16, W[co][tap][ci] (forward) or Wt[ci][tap][co];
//   out: (N H W, Ncols), bf16 relu(conv + bias) (forward) or float.
struct TcConv {
    int mode;
    const void *act;
    const void *wk;
    const float *bias;
    void *out;
    int N, H, W, Ck, Ncols;
};

// Whether the shapes fit the kernel: Ck a multiple of 32, Ncols of 16,
// rows of 128 pixels or rows dividing 128 (a tile never crosses an image),
// 16-byte aligned buffers, and the driver's tensor-map encoder available.
bool conv_tc_supported(const TcConv &c);
cudaError_t conv_tc_launch(const TcConv &c, cudaStream_t stream);

// The weight-gradient product: FP32 partials (splits, 9 Cin, Cout) of
// sum_p X[p + t][ci] G[p][co] over shares of the pixels, for
// wgrad_reduce_kernel.  X (N, H, W, Cin) and G (N, H, W, Cout) bf16;
// part: part_floats floats.
struct TcWgrad {
    const void *X, *G;
    float *part;
    size_t part_floats;
    int N, H, W, Cin, Cout;
};

// Whether the shapes fit (channels multiples of 32, the image rows as for
// the other products, 16-byte aligned buffers, the encoder available).
bool conv_tc_wgrad_supported(const TcWgrad &w);
// Launches the partial products; *splits receives the partials written.
cudaError_t conv_tc_wgrad_launch(const TcWgrad &w, int *splits,
                                 cudaStream_t stream);

}  // namespace dyfox
