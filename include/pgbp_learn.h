/* pgbp_learn: the kernels of the learned warm start for loopy BP.
 *
 * No counterpart in PGMax: the reference has no learned initialisation. A small convolutional
 * network (pgmax_gb300/warmstart) maps each variable's unaries and couplings to initial
 * log-messages of its edges; plain BP (pgbp_run) then runs from them. These entry points are the
 * network's training and inference kernels: its input features, 3x3 convolutions with circular
 * padding (toroidal grids) over NHWC BF16 images with FP32 accumulation on the tensor cores, their
 * gradients, a mean-centred squared-error loss and Adam. Conventions as in pgbp.h (status codes, caller's
 * stream, caller-owned device buffers, pgbp_last_error).
 *
 * Layouts: images [n][h][w][c] BF16, c contiguous; weights [9][co][ci] BF16, tap
 * t = (dy + 1) * 3 + (dx + 1), out[p][o] = bias[o] + sum_t sum_i in[p + (dy, dx)][i] * w[t][o][i]
 * with coordinates modulo h and w. Supported (ci, co): (16, 64), (64, 64), (64, 32), (32, 64);
 * w a multiple of 16, at most 128.
 */
#ifndef PGBP_LEARN_H_
#define PGBP_LEARN_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* out = conv3x3(in, weights) + bias (bias may be NULL); relu != 0: max(0, .); mask (may be NULL,
 * [n][h][w][co] BF16): outputs where mask <= 0 are set to 0 (the ReLU backward of the layer below,
 * for input gradients). out is FP32 when out_f32 != 0, else BF16. */
int pgbp_conv3x3(void* stream, int64_t n, int h, int w, int ci, int co, const void* in,
                 const void* weights, const float* bias, void* out, int out_f32, int relu,
                 const void* mask);

/* Weight and bias gradients of pgbp_conv3x3: dw[9][co][ci] (FP32) = sum over pixels p of
 * dout[p][o] * in[p + (dy, dx)][i]; db[co] (FP32, may be NULL) = sum over pixels of dout.
 * Deterministic (fixed-order reduction of per-CTA partial sums held in the workspace). */
size_t pgbp_conv3x3_wgrad_workspace(int ci, int co);
int pgbp_conv3x3_wgrad(void* stream, int64_t n, int h, int w, int ci, int co, const void* in,
                       const void* dout, float* dw, float* db, void* workspace,
                       size_t workspace_bytes);

/* flipped[t][i][o] = weights[8 - t][o][i]: the weights whose convolution of an output gradient
 * is the input gradient (ci and co of the forward layer). */
int pgbp_conv3x3_flip(void* stream, int ci, int co, const void* weights, void* flipped);

/* Over groups of `group` consecutive FP32 values: d = (pred - mean pred) - (target - mean
 * target); *loss += sum d^2 (double, may be NULL); grad (BF16) = scale * 2 d. */
int pgbp_center_mse(void* stream, int64_t groups, int group, const float* pred,
                    const float* target, void* grad, double* loss, float scale);

/* One Adam step (step >= 1) on FP32 master weights w with gradient g and moments m, v; writes
 * the BF16 copy w_bf16 when it is not NULL. */
int pgbp_adam(void* stream, int64_t n, float* w, const float* g, float* m, float* v, void* w_bf16,
              float lr, float beta1, float beta2, float eps, int64_t step);

/* The network's inputs for toroidal L x L Potts grids with K-state variables and per-edge tables
 * J_e I_K (the warm-start family): J [n][2 L^2] FP32 (down factors (i, j)-(i+1, j), then right
 * factors (i, j)-(i, j+1)), u [n][L^2][K] FP32 unaries. Per variable and each of its factors in
 * the order down, right, up, left (coupling J_k, other variable's unaries a_k): the closed-form
 * one-step message m_k(s) = log(exp(logsumexp(a_k)) + expm1(J_k) exp(a_k(s))) minus its maximum.
 * x [n][L][L][64] BF16 = (unaries minus their mean, the four couplings, the four messages, zeros);
 * m1 [n][L][L][4 K] FP32 = the four messages. Supported: K = 8, L >= 3. */
int pgbp_potts_features(void* stream, int64_t n, int L, int K, const float* J, const float* u,
                        void* x, float* m1);

#ifdef __cplusplus
}
#endif

#endif /* PGBP_LEARN_H_ */
