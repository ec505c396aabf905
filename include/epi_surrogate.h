/* epi_surrogate.h -- C ABI of the learned surrogate: an MLP from an epidemic's parameter
 * vector to its daily compartment curves, trained and evaluated on the GPU.
 *
 * The reference engine has no surrogate; this interface is an addition that sits beside
 * the engine ABI (epi_engine.h).  The network is in_dim -> hidden (x hidden_layers, GELU)
 * -> out_dim, with BF16 weights and activations, FP32 accumulation in tensor memory and
 * FP32 master weights updated by Adam.  Every matrix product runs in one hand-written
 * sm_103a kernel (tcgen05.mma, operands staged by TMA); bias gradients, the loss, the
 * minibatch gather and Adam are their own kernels.
 *
 * A handle holds `members` networks of the same shape (an ensemble), trained and evaluated
 * together: every kernel launch covers all members.  Member m is initialised from seed + m
 * and draws its minibatches from shuffle_seed + m, so it equals a one-member handle created
 * and trained with those seeds.  Per-member host arrays are member-major: member m's block
 * follows member m-1's.
 *
 * Conventions follow epi_engine.h: every function returns EPI_OK (0) or an EPI_ERR_* code
 * and never aborts; epi_mlp_last_error gives the message.  Host arrays are row-major
 * float32.  A handle is not thread-safe.
 */
#ifndef EPI_SURROGATE_H
#define EPI_SURROGATE_H

#include <stdint.h>

#include "epi_engine.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct epi_mlp epi_mlp;

typedef struct {
    uint32_t in_dim;         /* parameters per sample (<= 64) */
    uint32_t hidden;         /* width of every hidden layer (multiple of 64) */
    uint32_t hidden_layers;  /* number of hidden layers (>= 1) */
    uint32_t out_dim;        /* outputs per sample */
    uint32_t batch;          /* training minibatch (multiple of 128) */
    float lr, beta1, beta2, eps;  /* Adam */
    uint32_t members;        /* networks in the handle (0 means 1; at most 64) */
    uint64_t seed;           /* weight initialisation of member 0 (member m: seed + m) */
} epi_mlp_config;

/* Create a network with weights drawn like torch.nn.Linear's default (uniform in
 * +-1/sqrt(fan_in)) from cfg->seed. */
int epi_mlp_create(const epi_mlp_config* cfg, epi_mlp** out);
int epi_mlp_destroy(epi_mlp* h);
const char* epi_mlp_last_error(const epi_mlp* h);
/* Run on a caller's CUDA stream (cudaStream_t) instead of the handle's own. */
int epi_mlp_set_stream(epi_mlp* h, void* cuda_stream);

/* Number of networks in the handle. */
int epi_mlp_members(const epi_mlp* h, uint32_t* out);
/* Parameters of ONE member: sum over layers of out * in + out (unpadded). */
int epi_mlp_param_count(const epi_mlp* h, uint64_t* out);
/* FP32 master weights, members x param_count: per member, layer by layer, W (out x in,
 * row-major) then b (out). */
int epi_mlp_get_params(epi_mlp* h, float* out);
/* Replace the master weights (and their BF16 copies); Adam moments are reset. */
int epi_mlp_set_params(epi_mlp* h, const float* in);

/* Upload a training set: x is n x in_dim, y is n x out_dim (host arrays). */
int epi_mlp_set_dataset(epi_mlp* h, const float* x, const float* y, uint32_t n);
/* Run `steps` Adam steps on minibatches of the uploaded set, reshuffled every epoch from
 * shuffle_seed (+ m for member m); losses (may be NULL, else members x steps) receives the
 * mean squared error of every member's every step. */
int epi_mlp_train(epi_mlp* h, uint32_t steps, uint64_t shuffle_seed, float* losses);
/* Losses (members values) and gradients (same layout as epi_mlp_get_params) of every member
 * on one minibatch of exactly `batch` samples, without updating the weights. */
int epi_mlp_gradients(epi_mlp* h, const float* x, const float* y, uint32_t n, float* grads, float* loss);

/* Forward pass of every member for n samples: y (members x n x out_dim). */
int epi_mlp_predict(epi_mlp* h, const float* x, uint32_t n, float* y);
/* Forward pass scored against one target curve: score[m][i] = sum_j (y_mij - target_j)^2
 * (members x n), computed on the device (the outputs themselves stay there). */
int epi_mlp_score(epi_mlp* h, const float* x, uint32_t n, const float* target, float* score);

/* Kernel launches so far (the GEMM, gather, bias-gradient, Adam and step kernels). */
int epi_mlp_kernels_launched(const epi_mlp* h, uint64_t* out);

#ifdef __cplusplus
}
#endif

#endif /* EPI_SURROGATE_H */
