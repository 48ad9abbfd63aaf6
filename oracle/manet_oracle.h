/*
 * manet_oracle.h -- FP64 CPU restatement of the Monge-Ampere warm-start network.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU network kernels (forward, backward,
 * weight gradients).  The GPU library never links or calls it.
 *
 * The network has no reference counterpart.  Definition (the GPU kernels implement the same):
 *   4 periodic 3x3x3 convolutions, channels 3 -> 16 -> 16 -> 16 -> 1, ReLU after the first three;
 *   voxel v = (x*N + y)*N + z, tensors channel-last [N^3][c];
 *   tap t = (dx+1)*9 + (dy+1)*3 + (dz+1), dx, dy, dz in {-1, 0, 1};
 *   out[v][co] = b[co] + sum_t sum_ci in[v + d_t][ci] * w[(t*cin + ci)*cout + co]  (periodic);
 *   loss = sum_v (pred[v] - target[v])^2 / N^3.
 */
#ifndef MANET_ORACLE_H
#define MANET_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* round to the nearest bfloat16 (through float, ties to even), returned as a double */
double orc_bf16(double x);

void orc_conv3d(int N, int cin, int cout, const double *in, const double *w, const double *b, int relu,
                double *out);
/* din[v][ci] = sum_t sum_co dout[v - d_t][co] * w[t][ci][co] */
void orc_conv3d_bwd_data(int N, int cin, int cout, const double *dout, const double *w, double *din);
/* dw[t][ci][co] = sum_v in[v + d_t][ci] * dout[v][co];  db[co] = sum_v dout[v][co] */
void orc_conv3d_bwd_weight(int N, int cin, int cout, const double *in, const double *dout, double *dw,
                           double *db);

/* Whole network: forward, MSE loss, gradients of all weights and biases.  x: [N^3][3], target:
 * [N^3]; w[l], b[l] as above; pred (optional): [N^3].  round_bf16 != 0 mirrors the GPU's storage:
 * inputs, weights, hidden activations and the back-propagated activation gradients are rounded
 * to bfloat16 where the GPU stores them in bfloat16.  Returns the loss. */
double orc_manet_loss_grad(int N, const double *x, const double *target, const double *const *w,
                           const double *const *b, int round_bf16, double *pred, double *const *dw,
                           double *const *db);

#ifdef __cplusplus
}
#endif
#endif
