/* Learned warm start: device kernels of the convolutional encoder-decoder
 * that predicts an initial rho / u field from a signed-distance field and
 * inlet parameters, and the signed-distance field itself.  No counterpart in
 * the reference (it always starts from rest, Node.cpp:30-37); the lattice is
 * then warm-started through lbm_init_from_macro (lbm_gb300.h).
 *
 * All pointers are device pointers; calls are asynchronous on `stream`
 * (a cudaStream_t, NULL = the default stream) and allocate nothing.
 * Tensors are channels-last ([z][y][x][c]) BF16 with c a multiple of 16
 * (16, 32 or 64); weights are BF16 [co][tap][ci] (tap = (tz*k + ty)*k + tx),
 * FP32 biases [co].  Kernel size 3 (padding 1, stride 1 or 2) or 1.  The
 * convolutions take 16-byte aligned tensors (activations, weights, FP32
 * outputs) and return LBM_ERR_ARG for others. */
#ifndef LBM_NN_H
#define LBM_NN_H

#include "lbm_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* y = act(conv(x, w) + bias), act = ReLU if relu != 0; dims_in = {D, H, W}
 * of x; y has ((D - 1)/stride + 1, ...) voxels and co channels.  y_f32
 * (optional) receives the same values in FP32. */
lbm_status lbm_nn_conv3d_fwd(const void* x, const int dims_in[3], int ci, const void* w, const float* bias, int co,
                             int ksize, int stride, int relu, void* y, float* y_f32, void* stream);

/* Convolution engine.  LBM_NN_ENGINE_AUTO (default): 3x3x3 convolutions
 * run on the tcgen05 tensor cores with tensor-memory accumulators
 * (conv_tc.cu) -- the forward pass at stride 1 on input grids with D % 4,
 * H % 16 and W % 8 == 0 and at stride 2 on even grids whose output has
 * H % 16 and W % 8 == 0, the stride-1 input gradient on the same grids,
 * and the weight gradient wherever the output's W is a multiple of 16
 * (16-byte aligned activations); the others on mma.sync.
 * LBM_NN_ENGINE_MMA_SYNC: mma.sync everywhere (the comparison path).
 * Process-wide. */
#define LBM_NN_ENGINE_AUTO 0
#define LBM_NN_ENGINE_MMA_SYNC 1
lbm_status lbm_nn_set_conv_engine(int engine);
/* Waits for the device, then reports (LBM_ERR_CUDA) and clears a bounded
 * wait of a tensor-core convolution that gave up since the last call. */
lbm_status lbm_nn_conv_status(void);

/* Gradients of the convolution above (before its activation): dx = dL/dx
 * (BF16, written; needs w_t, scratch of the weight's size), dw += dL/dw and
 * db += dL/db (FP32, accumulated); any of dx / dw / db may be NULL. */
lbm_status lbm_nn_conv3d_bwd(const void* x, const int dims_in[3], int ci, const void* w, void* w_t, int co,
                             int ksize, int stride, const void* dy, void* dx, float* dw, float* db, void* stream);

/* dy *= (y > 0) over n elements (ReLU backward from the stored output). */
lbm_status lbm_nn_relu_bwd(const void* y, void* dy, int64_t n, void* stream);

/* Nearest-neighbour x2 upsampling of x (dims_in, c channels) into y; with
 * adjoint != 0, x is the gradient of the fine tensor and y receives the
 * gradient of the coarse one (dims_in). */
lbm_status lbm_nn_upsample2(const void* x, const int dims_in[3], int c, void* y, int adjoint, void* stream);

/* out = a + b over n BF16 elements. */
lbm_status lbm_nn_add(const void* a, const void* b, void* out, int64_t n, void* stream);

/* Masked squared error: for voxels with mask != 0 and channels < nc,
 * *loss += sum (pred - target)^2 * inv_norm; dpred = 2 (pred - target) *
 * inv_norm (BF16, zero elsewhere).  pred is [nvox][c] FP32, target
 * [nvox][nc] FP32. */
lbm_status lbm_nn_mse(const float* pred, const float* target, const uint8_t* mask, int64_t nvox, int c, int nc,
                      float inv_norm, void* dpred, float* loss, void* stream);

/* One Adam step (bias-corrected, step >= 1) on FP32 master weights w; the
 * BF16 copy w_bf16 (optional) follows. */
lbm_status lbm_nn_adam(float* w, void* w_bf16, const float* grad, float* m, float* v, int64_t n, float lr,
                       float beta1, float beta2, float eps, int64_t step, void* stream);

/* Signed distance (lattice spacings, > 0 in fluid) of every voxel of a
 * D x H x W mask ([z][y][x], nonzero = fluid) to the fluid boundary, by
 * jump flooding; scratch holds 2 * D * H * W int32. */
lbm_status lbm_sdf_from_mask(const uint8_t* mask, const int dims[3], float* sdf, void* scratch, void* stream);

/* Slice-wise Hagen-Poiseuille prior of a vessel along +z (inlet on the
 * first fluid slice with peak velocity `inlet`, density 1 after the last):
 * dist = in-slice distance to the wall (jump flooding per z slice, 0 on
 * solid), R(z) = its slice maximum, u_z = 2 Q / (pi R^2) (1 - (R - dist)^2 /
 * R^2) with Q = pi R0^2 inlet / 2, and drho = rho - 1 from d rho / dz =
 * -3 * 8 nu Q / (pi R^4).  scratch: 2 * D * H * W int32 + 3 * D floats. */
lbm_status lbm_ws_prior(const uint8_t* mask, const int dims[3], double inlet, double nu, float* dist, float* drho,
                        float* uz, void* scratch, void* stream);

/* `rounds` passes of a masked [1, 2, 1] / 4 filter along z, y and x over an
 * FP32 field v (weights renormalised next to solid voxels or the box face,
 * zero on solid); tmp: scratch of v's size. */
lbm_status lbm_ws_smooth(const uint8_t* mask, const int dims[3], float* v, float* tmp, int rounds, void* stream);

/* The network's BF16 input [nvox][16] for a D x H x W grid (dims) in one
 * pass: channel 0 clamp(sdf * sdf_scale, -3, 3), 1 the mask (0 / 1), 2
 * mean_in and 3 period_in (the scaled inlet mean and period, the same for
 * every voxel), 4 z / D, 5 uz_p / inlet, 6 drho_p / inlet * rho_scale,
 * 7..15 zero; every value computed in FP32 and rounded to BF16 once.  x
 * 16-byte aligned. */
lbm_status lbm_ws_features(const float* sdf, const uint8_t* mask, const float* uz_p, const float* drho_p,
                           const int dims[3], float sdf_scale, float mean_in, float period_in, float inlet,
                           float rho_scale, void* x, void* stream);

/* Network output y ([nvox][c] FP32, c >= 4) to fields [4][nvox]: rho - 1 =
 * drho_p + y0 inlet / rho_scale, u = y1..3 inlet / u_scale, u_z += uz_p;
 * zero on solid voxels. */
lbm_status lbm_ws_output(const float* y, int c, const uint8_t* mask, const float* drho_p, const float* uz_p,
                         int64_t nvox, float inlet, float rho_scale, float u_scale, float* fields, void* stream);

/* rho[a] = 1 + fields[0][idx[a]], u[3a + k] = fields[1 + k][idx[a]]: the
 * per-node input of lbm_init_from_macro_device (idx = the fluid voxels in
 * raster order, which is the lattice's active-node order). */
lbm_status lbm_ws_gather(const float* fields, int64_t nvox, const int64_t* idx, int64_t nact, float* rho, float* u,
                         void* stream);

#ifdef __cplusplus
}
#endif

#endif /* LBM_NN_H */
