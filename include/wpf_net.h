/* wpf_net.h -- C ABI of the learned warm start of the Darcy solve.
 *
 * No counterpart in the reference: wPFAW3D starts every pressure solve from
 * the previous pressure (wPFAW3D.f90:980).  This small 3-D U-Net maps, at half
 * the simulation resolution, the fields (log K_rock, phase, pressure, the
 * phase change of the last step, the last two pressure increments and their
 * time extrapolation) to a correction of the extrapolated pressure increment.
 * The solve still ends at the same FP64 residual tolerance, so the network
 * changes only where the iteration starts; the FP64 residual decides, every
 * solve, whether its start is kept (see WPF_SOLVER_EXTRAPOLATE in wpf.h).
 *
 * Network: 7 convolutions 3x3x3 ("same", zero padding), 4 levels with
 * 16/32/64/64 channels, 2x2x2 average pooling down, nearest upsampling plus
 * skip addition up, ReLU after every convolution but the last.  Activations
 * and weights are BF16 (NDHWC: channel innermost, then x, y, z), accumulation
 * FP32 in tensor memory (tcgen05 implicit GEMM, sm_103a); master weights and
 * the Adam moments are FP32.  Training and inference run on the GPU through
 * these kernels only.
 *
 * Device pointers are plain CUDA device addresses; `stream` is a cudaStream_t
 * (NULL = the legacy default stream).  Status codes are wpf.h's.
 */
#ifndef WPF_NET_H
#define WPF_NET_H

#include <stdint.h>

#include "wpf.h"

#ifdef __cplusplus
extern "C" {
#endif

#define WPF_NET_IN_CHANNELS 16   /* input tensor channels (WPF_NET_FEATURES used, rest zero) */
#define WPF_NET_FEATURES 6
#define WPF_NET_LAYERS 7

typedef struct wpf_net wpf_net;

/* A network for a grid of nx x ny x nz voxels (each a multiple of 8). */
int wpf_net_create(int32_t nx, int32_t ny, int32_t nz, wpf_net** net);
int wpf_net_destroy(wpf_net* net);
/* He-normal initial weights from a seed (host RNG, deterministic), zero bias. */
int wpf_net_init(wpf_net* net, uint64_t seed);
/* Number of FP32 parameters (weights [Cout][27][Cin] of each layer, then its
 * bias [Cout], layer by layer) and their host copy in / out.               */
int wpf_net_param_count(const wpf_net* net, int64_t* n);
int wpf_net_get_params(wpf_net* net, float* host);
int wpf_net_set_params(wpf_net* net, const float* host);
/* Forward pass: in = bf16 [nz][ny][nx][16] (device), out = fp32 [nz][ny][nx]
 * (device): channel 0 of the last layer.                                    */
int wpf_net_forward(wpf_net* net, const uint16_t* in, float* out, void* stream);
/* One Adam step on the loss  sum_v mask_v (out_v - target_v)^2 / sum_v mask_v
 * (mask = NULL: all ones); *loss (host, may be NULL) gets the loss before the
 * step.  lr, beta1 0.9, beta2 0.999, eps 1e-8.                              */
int wpf_net_train_step(wpf_net* net, const uint16_t* in, const float* target, const float* mask,
                       float lr, float* loss, void* stream);
/* Gradients of the last train step (same layout as the parameters), for the
 * gradient checks against the CPU restatement.                              */
int wpf_net_get_grads(wpf_net* net, float* host);
/* The activations (bf16) of a layer after the last forward pass: index 0..6 =
 * the outputs of the seven convolutions (the last one rounded to bf16).    */
int wpf_net_get_activation(wpf_net* net, int32_t layer, uint16_t* host, int64_t n);

/* Single kernels, exposed for the tests.
 * wpf_conv3d: out[v][co] = act(bias[co] + sum_{t,ci} in[v+d_t][ci] w[co][t][ci]),
 * tap t = (dz+1)*9 + (dy+1)*3 + (dx+1); act = ReLU if relu; bf16 out (out16)
 * or fp32 out (out32), one of them non-null.  cin, cout in {16, 32, 64}.    */
int wpf_conv3d(int32_t cin, int32_t cout, int32_t nx, int32_t ny, int32_t nz, const uint16_t* in,
               const uint16_t* w, const float* bias, int32_t relu, uint16_t* out16, float* out32,
               void* stream);
/* Weight gradient, accumulated (+=) into fp32 gw[co][t][ci] and gb[co]:
 * gw += sum_v gy[v][co] x[v+d_t][ci], gb += sum_v gy[v][co].               */
int wpf_conv3d_wgrad(int32_t cin, int32_t cout, int32_t nx, int32_t ny, int32_t nz,
                     const uint16_t* x, const uint16_t* gy, float* gw, float* gb, void* stream);

/* Attach a trained network to a simulation handle: the net grid must be half
 * the simulation grid per axis.  net = NULL detaches.  The handle does not own
 * the net.  The solve uses it when WPF_SOLVER_EXTRAPOLATE is set and two
 * increments are held; wpf_step_stats.warm_start is then 2 when the net's
 * start was kept.                                                          */
int wpf_set_warm_start_net(wpf_handle* h, wpf_net* net);
/* Training data from a running simulation (WPF_SOLVER_EXTRAPOLATE set, two
 * increments held): the net input for the coming solve (bf16, net grid, 16
 * channels, device) and, after that solve, the target (fp32, net grid,
 * device): the solve's increment minus the extrapolation, over the same
 * scale.  wpf_ws_features fills `in` from the current state between steps,
 * with dt_next the step size wpf_step will use; wpf_ws_target fills `target`
 * after that wpf_step.  WPF_ERR_ARG when fewer than two increments are held. */
int wpf_ws_features(wpf_handle* h, double dt_next, uint16_t* in);
int wpf_ws_target(wpf_handle* h, float* target);

#ifdef __cplusplus
}
#endif
#endif
