/* emt6ro_surrogate.h -- C ABI of the protocol-outcome surrogate.
 *
 * No reference counterpart: the reference scores every GA protocol by full
 * simulation (python/emt6ro/ga_model/model.py, EMT6RoModel.predict).  This
 * MLP maps a protocol's dose-time vector and summary features of the initial
 * tumour to the mean final living-cell count, so a GA can pre-screen a
 * population and simulate only the most promising protocols.
 *
 * Network: 100 -> 512 -> 512 -> 512 -> 1, exact-erf GELU after each hidden
 * layer.  Inputs are 100 FP32 features per row (the library pads them to 128
 * with zeros); weights, activations and gradients of the hidden layers are
 * BF16 with FP32 accumulation on the tensor cores (tcgen05); the output
 * layer, loss and all Adam state are FP32.
 *
 * Parameter arrays (host, FP32, row-major), in this order everywhere:
 *   [0] W1 512 x 128 (columns 100..127 must stay zero)   [1] b1 512
 *   [2] W2 512 x 512                                      [3] b2 512
 *   [4] W3 512 x 512                                      [5] b3 512
 *   [6] w4 512                                            [7] b4 1
 *
 * Batches are B rows, B a positive multiple of 128 up to max_batch.  Device
 * pointers are plain CUDA allocations on the handle's device; the calls run
 * on the handle's stream (emt6_mlp_stream) and are stream-ordered.
 * Return codes and emt6_last_error() as in emt6ro_gb300.h.
 */
#ifndef EMT6RO_SURROGATE_H_
#define EMT6RO_SURROGATE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EMT6_MLP_IN 100
#define EMT6_MLP_IN_PAD 128
#define EMT6_MLP_HIDDEN 512

typedef struct emt6_mlp emt6_mlp;

/* Allocates parameters, Adam moments and activations for max_batch rows;
 * He-normal weights from `seed`, zero biases. */
int emt6_mlp_create(int max_batch, uint64_t seed, int device, emt6_mlp **out);
void emt6_mlp_destroy(emt6_mlp *net);
/* cudaStream_t of the handle */
void *emt6_mlp_stream(emt6_mlp *net);

/* Host copies of the 8 parameter arrays (order above). */
int emt6_mlp_set_params(emt6_mlp *net, const float *const *host);
int emt6_mlp_get_params(emt6_mlp *net, float *const *host);

/* d_y[B] = network(d_x[B][100]); asynchronous. */
int emt6_mlp_predict(emt6_mlp *net, const float *d_x, int B, float *d_y);

/* One Adam step (beta1 0.9, beta2 0.999, eps 1e-8, learning rate lr) on the
 * mean squared error of d_x[B][100] against d_target[B].  When h_loss is not
 * NULL, waits and stores the batch's loss (before the update) there. */
int emt6_mlp_train_step(emt6_mlp *net, const float *d_x, const float *d_target, int B, float lr,
                        float *h_loss);

/* Gradients of the mean squared error with respect to the 8 parameter arrays
 * (host buffers shaped as above) without updating anything; waits. */
int emt6_mlp_gradients(emt6_mlp *net, const float *d_x, const float *d_target, int B,
                       float *const *host_grads, float *h_loss);

/* Split of the weight-gradient GEMMs' reduction (batch) dimension over CTAs:
 * 0 chooses per batch size (default), or 1, 2, 4, 8.  Partial tiles are summed
 * in a fixed order, so results are deterministic for a given split. */
int emt6_mlp_set_splitk(emt6_mlp *net, int splits);

/* Waits for the handle's stream; EMT6_ERR_DEVICE if a GEMM's pipeline wait
 * timed out since the last check. */
int emt6_mlp_sync(emt6_mlp *net);

/* Test hook: d_c[M][N] (FP32) = d_a[M][K] d_b[N][K]^T with BF16 d_a, d_b
 * (row-major); M, N multiples of 128, K of 64.  Waits. */
int emt6_test_mlp_gemm(const void *d_a, const void *d_b, float *d_c, int M, int N, int K,
                       void *stream);
/* Failure-path hook of the same GEMM (no reference counterpart): the MMA
 * issuer first waits stall_us (1..100000) microseconds on an mbarrier nothing
 * arrives on, gives up as a timed-out pipeline wait does, the CTA waits for
 * the loads it issued, frees its tensor memory and returns; the call reports
 * EMT6_ERR_DEVICE and the context stays usable. */
int emt6_test_mlp_gemm_timeout(const void *d_a, const void *d_b, float *d_c, int M, int N,
                               int K, uint32_t stall_us, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* EMT6RO_SURROGATE_H_ */
