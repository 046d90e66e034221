/*
 * rc_mlp.h -- the learned chemistry surrogate: a small MLP
 *   7 inputs (T, p, Y_1..Y_4, dt) -> 4 x 128 hidden (GELU) -> 4 outputs
 * with BF16 weights and activations and FP32 accumulation on the tcgen05
 * tensor cores, trained on the GPU by the project's own forward, backward and
 * Adam kernels.  The inputs enter as the features (1000/T, log10 p,
 * log10(Y_k + 1e-10), log10 dt), normalised by a mean and standard deviation
 * set with the network.  The outputs are, per species k,
 *   z_k = dY_k / (c_k xi_s),
 * the change over dt from the per-cell integrator normalised by the progress
 * scale of the one global reaction: omega_k = c_k k_f (c_k = 1000 M_k
 * (nu''_k - nu'_k)), and xi_s is the smaller of the explicit progress
 * dt k_f / rho and the progress min(Y_k / -c_k) that exhausts the limiting
 * reactant.  z_k is near 1 while the explicit rate holds and is the consumed
 * fraction of the limiting reactant once it runs out.
 *
 * The reference has no surrogate and no chemistry integrator: both are new.
 * All d_* arguments are DEVICE pointers; stream may be null (default stream).
 */
#ifndef RC_MLP_H
#define RC_MLP_H

#ifdef __cplusplus
extern "C" {
#endif

#define RC_MLP_NIN 7
#define RC_MLP_NOUT 4
#define RC_MLP_HIDDEN 128
/* flat FP32 parameter vector: W0(128x7) b0(128) W1(128x128) b1 W2 b2 W3 b3
 * W4(4x128) b4(4); W_l[o][i] row-major (output o, input i) */
#define RC_MLP_NPARAM 51076

typedef struct rc_mlp rc_mlp;

int rc_mlp_create(int device, rc_mlp** out);
int rc_mlp_destroy(rc_mlp* net);
/* host FP32 parameter vectors of RC_MLP_NPARAM values */
int rc_mlp_set_params(rc_mlp* net, const float* params);
int rc_mlp_get_params(rc_mlp* net, float* params);
/* feature normalisation x_n = (f - mean) / std (7 + 7 values, f the features) and the
 * training domain used by the surrogate's error indicator: T_lo, T_hi,
 * p_lo, p_hi, dt_lo, dt_hi (6 values, raw units) */
int rc_mlp_set_norm(rc_mlp* net, const float* mean, const float* std, const float* domain);
/* y(n x 4) = net(x(n x 7)); raw features, row-major; fused tcgen05 kernel */
int rc_mlp_forward(rc_mlp* net, const float* d_x, int n, float* d_y, void* stream);
/* mean squared error of net(x) against t (n x 4) and its gradient with
 * respect to the parameters (d_grad: RC_MLP_NPARAM floats); n a multiple of
 * 128; loss (host, may be null) synchronises */
int rc_mlp_gradient(rc_mlp* net, const float* d_x, const float* d_t, int n, float* d_grad, float* loss,
                    void* stream);
/* one Adam step (bias-corrected, step counted from 1) with the given gradient */
int rc_mlp_adam(rc_mlp* net, const float* d_grad, float lr, float beta1, float beta2, float eps, void* stream);
/* `steps` Adam steps on batches of `batch` (a multiple of 128) pairs drawn
 * with replacement on the device from the n pairs (d_x: n x 7 raw features,
 * d_t: n x 4 targets, row-major; seed selects the draws), learning rate
 * decaying from lr to lr_end on a cosine; d_loss (device, steps floats, may be
 * null) receives each step's loss.  One CUDA graph per step; returns when the
 * steps are done. */
int rc_mlp_train(rc_mlp* net, const float* d_x, const float* d_t, long long n, int steps, int batch, float lr,
                 float lr_end, float beta1, float beta2, float eps, unsigned long long seed, float* d_loss,
                 void* stream);
const char* rc_mlp_last_error(rc_mlp* net);

#ifdef __cplusplus
}
#endif
#endif
