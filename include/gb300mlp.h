/* FP32 kernels of the learned initial-guess network (libgb300jk.so).
 *
 * No counterpart in the reference: gpu4pyscf's initial guesses are minao,
 * atom, huckel, 1e and chkfile (gpu4pyscf/scf/hf.py:414-561, 828-831).
 * These entry points train and run the atom-pair network that predicts
 * density blocks (gpu4pyscf_gb300/scf/learned_guess.py).  Device pointers,
 * caller's stream; 0 on success, negative on error (mlp_last_error()).
 */
#ifndef GB300MLP_H
#define GB300MLP_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* C[M,N] = op(A)[M,K] op(B)[K,N] (+ beta*C) (+ bias[N]); act 1 applies SiLU
 * after storing the pre-activation in Z (Z may be NULL).  Element (m,k) of A
 * is A[m*sam + k*sak], element (k,n) of B is B[k*sbk + n*sbn]; C and Z are
 * row-major with N columns. */
int mlp_gemm(int M, int N, int K, const float *A, int64_t sam, int64_t sak,
             const float *B, int64_t sbk, int64_t sbn, const float *bias, int act,
             float beta, float *Z, float *C, void *stream);

/* dZ = dY * d SiLU(Z)/dZ, elementwise over n entries. */
int mlp_silu_backward(int64_t n, const float *dY, const float *Z, float *dZ, void *stream);

/* out[n] = sum over the M rows of X[M,N]. */
int mlp_colsum(int M, int N, const float *X, float *out, void *stream);

/* grad = 2*mask*(y-t)*inv_count; *loss += sum mask*(y-t)^2*inv_count
 * (mask may be NULL, loss may be NULL). */
int mlp_mse(int64_t n, const float *y, const float *t, const float *mask, float inv_count,
            float *grad, float *loss, void *stream);

/* One Adam step (bias-corrected, step counts from 1) on n parameters. */
int mlp_adam(int64_t n, float *p, const float *g, float *m, float *v, float lr, float b1,
             float b2, float eps, int step, void *stream);

const char *mlp_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* GB300MLP_H */
