// closure_net.h -- the closure network's device state (internal).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stddef.h>

struct NetGeom {
    int nx, ny, nz, nb;     // grid and samples per batch
    int R;                  // rows per 128-point tile (128 / nx)
    long long tiles;        // nb * nz * nx * ny / 128
};

struct vec_net {
    NetGeom g;
    size_t npts = 0;        // nx * ny * nz
    int cout_real = 8;      // output channels (padded to 16 inside)
    int num_sms = 152;
    int conv_mt = 2;        // m-tiles per warp in the convolution kernels (VEC_NET_MT=1: one)
    int conv_tc = 1;        // forward / input gradient on tcgen05 for nx = 128 (VEC_NET_TC=0: mma.sync)
    int *err = nullptr;     // set by a kernel whose bounded wait ran out
    cudaStream_t stream = nullptr;
    int own_stream = 0;
    long long launches = 0;
    long long step = 0;     // Adam steps taken
    // FP32 master parameters, gradients, Adam moments; layer l has weights
    // [27][cout][cin] at off_w[l] and biases at off_b[l]
    float *p = nullptr, *gr = nullptr, *m = nullptr, *v = nullptr;
    size_t nparam = 0;
    size_t off_w[4] = {}, off_b[4] = {};
    // BF16 forward weights and tap-flipped transposed weights
    __nv_bfloat16 *wf[4] = {}, *wb[4] = {};
    // activations of one batch (channel-last)
    __nv_bfloat16 *x0 = nullptr;                 // [P][16] input
    __nv_bfloat16 *pre[3] = {}, *act[3] = {};    // [P][32] pre-activation and GELU output
    __nv_bfloat16 *d[2] = {};                    // [P][32] gradients
    __nv_bfloat16 *dout = nullptr;               // [P][16] output gradient
    float *out = nullptr;                        // [P][8]
    float *tgt = nullptr;                        // [P][8]
    float *xin = nullptr;                        // [P][16] FP32 staging
    float *part = nullptr;                       // per-CTA weight-gradient partials
    double *loss_d = nullptr;
};

// cuTensorMapEncodeTiled (lines_ct.cu), null if unavailable
void *tma_encode_fn();

int net_pack(vec_net *N);
int net_forward(vec_net *N);
int net_backward(vec_net *N, const float *tgt);
int net_adam(vec_net *N, float lr);
