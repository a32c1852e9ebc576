/*
 * lbm_unet.h -- C ABI of the learned warm start's kernels (GB300, sm_103a).
 *
 * No reference counterpart: the reference has no learned component.  A small
 * convolutional U-Net predicts the steady (rho, u) of a D2Q9 channel from its
 * geometry mask and Reynolds number; the prediction initialises the
 * populations of the plain LBM (lbm_gpu_set_populations), which then iterates
 * to the reference's convergence criterion.  These entry points are the
 * network's forward and backward building blocks; the training loop and the
 * warm start itself live in lbm_gb300/warmstart.py.
 *
 * Conventions: device pointers; tensors NHWC; activations and activation
 * gradients BF16 (passed as void*), weights [cout][3][3][cin] BF16 with FP32
 * master copies, gradients FP32; every convolution is 3x3, stride 1, zero
 * padding 1, with cin and cout multiples of 32.  `ld*` is the channel stride
 * of a tensor (>= its channel count) and `off*` a channel offset into it, so
 * concatenations are views.  `stream` is a cudaStream_t.  Return 0 on success,
 * -1 for invalid arguments, -2 for a CUDA launch error, -6 (lbm_nn_conv_status
 * only) for a bounded device wait that ran out.
 */
#ifndef LBM_UNET_H
#define LBM_UNET_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* y[:, offy:offy+cout] = act(conv(x[:, :cin], w) + bias); out_f32 selects FP32 output.  Runs on the tcgen05
 * tensor-core kernel where the shape qualifies (cout <= 256; W a multiple of 128, or a divisor of 128 with
 * H a multiple of 128 / W; x, w, y 16-byte aligned; ldy, offy multiples of 8 for BF16 output, of 4 for FP32),
 * else on the mma.sync kernel */
int lbm_nn_conv3x3_fwd(const void* x, int ldx, const void* w, const float* bias, void* y, int ldy, int offy, int B, int H, int W, int cin,
                       int cout, int relu, int out_f32, void* stream);
/* dw [cout][9 cin] = sum over pixels of dy (x) shifted x; partial: FP32 scratch of partial_floats */
int lbm_nn_conv3x3_wgrad(const void* x, int ldx, const void* dy, int lddy, float* partial, int64_t partial_floats, float* dw, int B, int H,
                         int W, int cin, int cout, void* stream);
/* db[c] = sum over npix pixels of dy[:, c] */
int lbm_nn_bias_grad(const void* dy, int lddy, int64_t npix, int c, float* db, void* stream);
/* wt [cin][3][3][cout] = w [cout][2-ky][2-kx][cin]: the data-gradient weights */
int lbm_nn_flip_weights(const void* w, void* wt, int cin, int cout, void* stream);
/* dx[:, :c] = dy[:, offdy:offdy+c] * (y[:, offy:offy+c] > 0) */
int lbm_nn_relu_bwd(const void* dy, int lddy, int offdy, const void* y, int ldy, int offy, void* dx, int lddx, int64_t npix, int c,
                    void* stream);
/* 2x2 max pooling of x[:, offx:offx+C] (H, W even) into dense y, and its gradient added into dx[:, offdx:offdx+C] */
int lbm_nn_pool_fwd(const void* x, int ldx, int offx, void* y, int B, int H, int W, int C, void* stream);
int lbm_nn_pool_bwd(const void* x, int ldx, int offx, const void* dy, void* dx, int lddx, int offdx, int B, int H, int W, int C, void* stream);
/* nearest 2x upsampling of dense x [B,h,w,C] into y[:, :C], and its gradient */
int lbm_nn_up_fwd(const void* x, void* y, int ldy, int B, int h, int w, int C, void* stream);
int lbm_nn_up_bwd(const void* dy, int lddy, void* dx, int B, int h, int w, int C, void* stream);
/* masked mean-square error of pred[:, :nout] (FP32, stride ldp) against target [npix][nout] over fluid
 * pixels, scaled by inv_count; writes dpred (BF16, stride ldp) and one partial sum per block */
int lbm_nn_mse(const float* pred, int ldp, const float* target, const uint8_t* fluid, int64_t npix, int nout, float inv_count, void* dpred,
               float* partial, int nblocks, void* stream);
/* Adam step (bias-corrected, step >= 1) on FP32 master weights w, refreshing the BF16 copy w16 if not null */
int lbm_nn_adam(float* w, void* w16, const float* g, float* m, float* v, int64_t n, float lr, float b1, float b2, float eps, int step,
                void* stream);
int lbm_nn_to_bf16(const float* a, void* b, int64_t n, void* stream);
/* 0: the tensor-core convolution where it qualifies (default); 1: the mma.sync kernel only */
int lbm_nn_set_conv_path(int path);
/* 1 if lbm_nn_conv3x3_fwd with these arguments runs on the tensor-core kernel, else 0 */
int lbm_nn_conv_uses_tc(const void* x, int ldx, const void* w, const void* y, int ldy, int offy, int B, int H, int W, int cin, int cout,
                        int out_f32);
/* synchronises the stream; -6 (a bounded pipeline wait of a tensor-core convolution ran out since the last
 * call) or 0, and clears the flag */
int lbm_nn_conv_status(void* stream);
/* TEST ONLY.  The tensor-core convolution's pipeline waits are bounded (0.2 s each); when one runs out the
 * CTA records the flag lbm_nn_conv_status reports, lets its copies and MMAs in flight complete, frees its
 * tensor memory and returns (its output is then invalid).  This sets the limit (1 ns .. 0.5 s) and, with
 * starve = 1, leaves every CTA's first K chunk unloaded, so the waits on it run out: a device-side timeout
 * without a fault.  limit 200000000 and starve 0 restore the defaults. */
int lbm_nn_conv_test_wait(int64_t limit_ns, int32_t starve);

#ifdef __cplusplus
}
#endif

#endif
