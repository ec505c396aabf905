// surrogate.cu -- the learned surrogate of include/epi_surrogate.h: a BF16 MLP trained and
// evaluated on the sm_103a tensor cores.
//
// Layers l = 0 .. L-1 map K_l inputs to N_l outputs (K_0 = in_dim padded to 64, N_{L-1} =
// out_dim padded to a multiple of 128, hidden widths in between).  Padding rows and columns
// are zero and stay zero: their inputs are zero, so are their gradients and Adam updates.
// Per layer the device holds the FP32 master weights W (N x K) and b, Adam moments, and two
// BF16 copies: W (the B operand of the forward product) and W^T (the B operand of the
// input-gradient product).  Activations are kept in both orientations, written by the
// epilogues, so every product takes K-major operands:
//   forward  H_{l+1} = gelu(H_l W_l^T + b_l)          A = H_l      B = W_l
//   output   Y = H_{L-1} W^T + b, dY = 2 (Y - T) / (B * out_dim)   (fused, with the loss)
//   weights  dW_l = dZ_l^T H_l                         A = dZ_l^T   B = H_l^T
//   inputs   dZ_{l-1} = (dZ_l W_l) * gelu'(Z_{l-1})    A = dZ_l     B = W_l^T
// A training step is one CUDA graph: gather, 2L + (L-1) products, L bias reductions, L Adam
// updates and the step counter, replayed once per step.
//
// A handle holds E = cfg.members networks of the same shape (an ensemble).  Every buffer
// carries a leading member axis and every kernel covers all members in one launch: the
// products through the third grid dimension and 3-D tensor maps {cols, rows, E}, the small
// kernels through blockIdx.y.  Member m is initialised from seed + m and, in training, draws
// its minibatches from shuffle_seed + m, so it equals a one-member network created and
// trained with those seeds.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/epi_surrogate.h"
#include "tc_gemm.cuh"

using namespace epi::tc;

namespace {

constexpr uint32_t kInPad = 64;
constexpr uint32_t kMaxMembers = 64;
constexpr int kSmallThreads = 256;

// ---------------------------------------------------------------- small kernels
// Minibatch row r of member e (grid B x E) <- sample idx[e][step - step_base][r]: X rows (bf16,
// already padded) in both orientations and the padded FP32 targets.
__global__ void k_gather(const __nv_bfloat16* __restrict__ xs, const float* __restrict__ ys,
                         const uint32_t* __restrict__ idx, uint32_t steps, const uint32_t* __restrict__ step,
                         uint32_t step_base, uint32_t B, uint32_t out_pad, __nv_bfloat16* __restrict__ h0,
                         __nv_bfloat16* __restrict__ h0t, float* __restrict__ t) {
    const uint32_t r = blockIdx.x, e = blockIdx.y;
    const uint32_t s = idx[((size_t)e * steps + (*step - step_base)) * B + r];
    h0 += (size_t)e * B * kInPad;
    h0t += (size_t)e * B * kInPad;
    t += (size_t)e * B * out_pad;
    for (uint32_t c = threadIdx.x; c < kInPad; c += blockDim.x) {
        const __nv_bfloat16 v = xs[(size_t)s * kInPad + c];
        h0[(size_t)r * kInPad + c] = v;
        h0t[(size_t)c * B + r] = v;
    }
    for (uint32_t c = threadIdx.x; c < out_pad; c += blockDim.x) t[(size_t)r * out_pad + c] = ys[(size_t)s * out_pad + c];
}

// db[n] = sum over the batch of dZ^T[n][:] (one warp per row; the members' rows follow one
// another, so N counts the rows of all members).
__global__ void k_bias_grad(const __nv_bfloat16* __restrict__ dzt, uint32_t N, uint32_t B, float* __restrict__ db) {
    const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
    if (w >= N) return;
    float s = 0.f;
    for (uint32_t b = lane; b < B; b += 32) s += __bfloat162float(dzt[(size_t)w * B + b]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, o);
    if (lane == 0) db[w] = s;
}

struct AdamHyper {
    float lr, beta1, beta2, eps;
};

// One Adam step (Kingma & Ba 2015, with bias correction) of member blockIdx.y; t = *step + 1.
// Blocks below (N / 32) * (K / 32) take a 32 x 32 tile of W (N x K; both multiples of 32) and
// write its BF16 copies W and W^T, the transpose through shared memory so that both stores
// are coalesced; the blocks after them take 256 entries of b each.  256 threads.
__device__ __forceinline__ float adam_update(float* p, float* m, float* v, float g, float c1, float c2, const AdamHyper& hp) {
    const float mi = hp.beta1 * *m + (1.f - hp.beta1) * g;
    const float vi = hp.beta2 * *v + (1.f - hp.beta2) * g * g;
    *m = mi;
    *v = vi;
    const float np = *p - hp.lr * (mi / c1) / (sqrtf(vi / c2) + hp.eps);
    *p = np;
    return np;
}

__global__ void __launch_bounds__(256) k_adam(float* __restrict__ w, const float* __restrict__ gw, float* __restrict__ mw,
                                              float* __restrict__ vw, float* __restrict__ b, const float* __restrict__ gb,
                                              float* __restrict__ mb, float* __restrict__ vb, __nv_bfloat16* __restrict__ wb,
                                              __nv_bfloat16* __restrict__ wtb, uint32_t N, uint32_t K,
                                              const uint32_t* __restrict__ step, AdamHyper hp) {
    __shared__ __nv_bfloat16 tile[32][34];
    const float t = (float)(*step + 1u);
    const float c1 = 1.f - powf(hp.beta1, t), c2 = 1.f - powf(hp.beta2, t);
    const size_t nw = (size_t)N * K, ow = (size_t)blockIdx.y * nw, ob = (size_t)blockIdx.y * N;
    const uint32_t tiles_k = K / 32u, n_tiles = N / 32u * tiles_k;
    if (blockIdx.x < n_tiles) {
        w += ow; gw += ow; mw += ow; vw += ow; wb += ow; wtb += ow;
        const uint32_t n0 = blockIdx.x / tiles_k * 32u, k0 = blockIdx.x % tiles_k * 32u;
        const uint32_t tx = threadIdx.x & 31u, ty = threadIdx.x >> 5;
        for (uint32_t r = ty; r < 32u; r += 8u) {
            const size_t i = (size_t)(n0 + r) * K + k0 + tx;
            const __nv_bfloat16 q = __float2bfloat16_rn(adam_update(w + i, mw + i, vw + i, gw[i], c1, c2, hp));
            wb[i] = q;
            tile[r][tx] = q;
        }
        __syncthreads();
        for (uint32_t r = ty; r < 32u; r += 8u) wtb[(size_t)(k0 + r) * N + n0 + tx] = tile[tx][r];
    } else {
        const uint32_t j = (blockIdx.x - n_tiles) * blockDim.x + threadIdx.x;
        if (j < N) adam_update(b + ob + j, mb + ob + j, vb + ob + j, gb[ob + j], c1, c2, hp);
    }
}

// BF16 copies of the master weights of member blockIdx.y (after initialisation or set_params).
__global__ void k_cast_weights(const float* __restrict__ w, __nv_bfloat16* __restrict__ wb, __nv_bfloat16* __restrict__ wtb,
                               uint32_t N, uint32_t K) {
    const size_t nw = (size_t)N * K, ow = (size_t)blockIdx.y * nw;
    w += ow; wb += ow; wtb += ow;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < nw; i += (size_t)gridDim.x * blockDim.x) {
        const __nv_bfloat16 q = __float2bfloat16_rn(w[i]);
        wb[i] = q;
        wtb[(i % K) * N + i / K] = q;
    }
}

__global__ void k_step_end(uint32_t* step) { *step += 1u; }

// ---------------------------------------------------------------- host helpers
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    return fn;
}

uint32_t round_up(uint32_t v, uint32_t a) { return (v + a - 1) / a * a; }

// splitmix64 (Steele, Lea & Flood 2014): the host stream for weight init and shuffles.
struct SplitMix {
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

}  // namespace

struct MlpLayer {
    uint32_t K = 0, N = 0;        // padded
    uint32_t k_real = 0, n_real = 0;
    // parameters, gradients and Adam moments, E members each
    float *w = nullptr, *b = nullptr, *mw = nullptr, *vw = nullptr, *mb = nullptr, *vb = nullptr;
    float *gw = nullptr, *gb = nullptr;
    __nv_bfloat16 *wb = nullptr, *wtb = nullptr;
    // training activations (batch rows, E members each)
    __nv_bfloat16 *h = nullptr, *ht = nullptr;     // input of this layer, B x K and K x B
    float* z = nullptr;                             // pre-activation output, B x N (hidden layers)
    __nv_bfloat16 *dz = nullptr, *dzt = nullptr;    // gradient at the pre-activation, B x N and N x B
    CUtensorMap t_h, t_w, t_dzt, t_ht, t_dz, t_wt;  // product operands
    // inference activations: the input layer's rows are shared by all members
    __nv_bfloat16* ph = nullptr;
    CUtensorMap t_ph;
};

struct epi_mlp {
    epi_mlp_config cfg{};
    uint32_t E = 1;  // members
    uint32_t L = 0, in_pad = kInPad, out_pad = 0, B = 0;
    std::vector<MlpLayer> layers;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::string err;
    int* d_err = nullptr;
    uint32_t* d_step = nullptr;
    float* d_t = nullptr;        // batch targets, E x B x out_pad
    float* d_loss = nullptr;     // per-step losses, steps x E
    float* d_step_loss = nullptr;  // losses of the step in flight, E
    uint32_t loss_cap = 0;
    uint32_t* d_idx = nullptr;   // minibatch indices of a train call, E x steps x B
    size_t idx_cap = 0;
    __nv_bfloat16* d_xs = nullptr;  // dataset, n x 64 (bf16, padded)
    float* d_ys = nullptr;          // dataset, n x out_pad
    uint32_t n_data = 0;
    // inference
    uint32_t p_cap = 0;
    float* d_py = nullptr;        // E x n x out_pad
    float* d_pscore = nullptr;    // E x n
    float* d_ptarget = nullptr;   // out_pad
    cudaGraphExec_t step_graph = nullptr;
    uint64_t launches = 0;
};

#define MCK(call)                                                                       \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess) {                                                        \
            h->err = std::string(#call) + ": " + cudaGetErrorString(e_);                \
            return EPI_ERR_CUDA;                                                        \
        }                                                                               \
    } while (0)

namespace {

// 3-D map {cols, rows, depth} of depth stacked row-major BF16 matrices; a box is 64 columns
// x box_rows rows of one matrix.
int make_map(epi_mlp* h, CUtensorMap* map, const void* base, uint32_t rows, uint32_t cols, uint32_t box_rows,
             uint32_t depth) {
    EncodeTiledFn enc = encode_fn();
    if (!enc) { h->err = "cuTensorMapEncodeTiled unavailable"; return EPI_ERR_CUDA; }
    const cuuint64_t dims[3] = {cols, rows, depth};
    const cuuint64_t strides[2] = {(cuuint64_t)cols * 2u, (cuuint64_t)cols * rows * 2u};
    const cuuint32_t box[3] = {(cuuint32_t)kBK, box_rows, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        h->err = "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")";
        return EPI_ERR_CUDA;
    }
    return EPI_OK;
}

// One product per member (grid z = E); za = 0 when every member reads member 0's A.
template <int BN, int EP>
int gemm(epi_mlp* h, const CUtensorMap& ta, const CUtensorMap& tb, uint32_t M, uint32_t N, uint32_t K, const EpiArgs& a,
         uint32_t za = 1) {
    if (M % kBM || N % BN || K % kBK || K == 0) {
        h->err = "gemm shape " + std::to_string(M) + "x" + std::to_string(N) + "x" + std::to_string(K);
        return EPI_ERR_ARG;
    }
    constexpr uint32_t smem = gemm_smem_bytes<BN>();
    k_gemm<BN, EP><<<dim3(M / kBM, N / BN, h->E), kGemmThreads, smem, h->stream>>>(ta, tb, M, N, K, a, za, 1u, h->d_err);
    MCK(cudaGetLastError());
    h->launches++;
    return EPI_OK;
}

#define MRC(x)                 \
    do {                       \
        int rc_ = (x);         \
        if (rc_) return rc_;   \
    } while (0)

int blocks_for(size_t n) { return (int)std::min<size_t>((n + kSmallThreads - 1) / kSmallThreads, 4096); }

int cast_all(epi_mlp* h) {
    for (auto& ly : h->layers) {
        k_cast_weights<<<dim3(blocks_for((size_t)ly.N * ly.K), h->E), kSmallThreads, 0, h->stream>>>(ly.w, ly.wb, ly.wtb,
                                                                                                     ly.N, ly.K);
        MCK(cudaGetLastError());
        h->launches++;
    }
    return EPI_OK;
}

// Forward + backward of one minibatch per member already in layers[0].h / .ht and d_t;
// member e's loss added to loss[e].
int enqueue_fwd_bwd(epi_mlp* h, float* loss) {
    const uint32_t B = h->B, L = h->L;
    for (uint32_t l = 0; l < L; ++l) {
        MlpLayer& ly = h->layers[l];
        EpiArgs a;
        a.bias = ly.b;
        a.ms_bias = ly.N;
        if (l + 1 < L) {
            MlpLayer& nx = h->layers[l + 1];
            a.z = ly.z;
            a.out = nx.h;
            a.out_t = nx.ht;
            a.ms_z = a.ms_out = (uint64_t)B * ly.N;
            MRC((gemm<128, kEpHidden>(h, ly.t_h, ly.t_w, B, ly.N, ly.K, a)));
        } else {
            a.target = h->d_t;
            a.out = ly.dz;
            a.out_t = ly.dzt;
            a.loss = loss;
            a.n_valid = h->cfg.out_dim;
            a.m_valid = B;
            a.grad_scale = 2.0f / ((float)B * (float)h->cfg.out_dim);
            a.ms_target = a.ms_out = (uint64_t)B * ly.N;
            a.ms_loss = 1;
            MRC((gemm<128, kEpOut>(h, ly.t_h, ly.t_w, B, ly.N, ly.K, a)));
        }
    }
    for (int l = (int)L - 1; l >= 0; --l) {
        MlpLayer& ly = h->layers[l];
        EpiArgs g;
        g.outf = ly.gw;
        g.ms_outf = (uint64_t)ly.N * ly.K;
        if (ly.K == 64) MRC((gemm<64, kEpDw>(h, ly.t_dzt, ly.t_ht, ly.N, ly.K, B, g)));
        else MRC((gemm<128, kEpDw>(h, ly.t_dzt, ly.t_ht, ly.N, ly.K, B, g)));
        const uint32_t rows = ly.N * h->E;
        k_bias_grad<<<(rows * 32 + kSmallThreads - 1) / kSmallThreads, kSmallThreads, 0, h->stream>>>(ly.dzt, rows, B,
                                                                                                      ly.gb);
        MCK(cudaGetLastError());
        h->launches++;
        if (l > 0) {
            MlpLayer& pv = h->layers[l - 1];
            EpiArgs d;
            d.zin = pv.z;
            d.out = pv.dz;
            d.out_t = pv.dzt;
            d.ms_zin = d.ms_out = (uint64_t)B * ly.K;
            MRC((gemm<128, kEpDh>(h, ly.t_dz, ly.t_wt, B, ly.K, ly.N, d)));
        }
    }
    return EPI_OK;
}

int enqueue_adam(epi_mlp* h) {
    const AdamHyper hp{h->cfg.lr, h->cfg.beta1, h->cfg.beta2, h->cfg.eps};
    for (auto& ly : h->layers) {
        const uint32_t blocks = ly.N / 32u * (ly.K / 32u) + (ly.N + kSmallThreads - 1) / kSmallThreads;
        k_adam<<<dim3(blocks, h->E), kSmallThreads, 0, h->stream>>>(
            ly.w, ly.gw, ly.mw, ly.vw, ly.b, ly.gb, ly.mb, ly.vb, ly.wb, ly.wtb, ly.N, ly.K, h->d_step, hp);
        MCK(cudaGetLastError());
        h->launches++;
    }
    return EPI_OK;
}

int check_err(epi_mlp* h) {
    int e = 0;
    MCK(cudaMemcpyAsync(&e, h->d_err, sizeof e, cudaMemcpyDeviceToHost, h->stream));
    MCK(cudaStreamSynchronize(h->stream));
    if (e) {
        h->err = "tensor-core product: a bounded wait expired (flag " + std::to_string(e) + ")";
        MCK(cudaMemsetAsync(h->d_err, 0, sizeof(int), h->stream));
        return EPI_ERR_TIMEOUT;
    }
    return EPI_OK;
}

// Pad host inputs (n x in_dim, float) into BF16 rows of 64.
std::vector<__nv_bfloat16> pad_inputs(const float* x, uint32_t n, uint32_t n_rows, uint32_t in_dim) {
    std::vector<__nv_bfloat16> v((size_t)n_rows * kInPad, __float2bfloat16_rn(0.f));
    for (uint32_t i = 0; i < n; ++i)
        for (uint32_t c = 0; c < in_dim; ++c) v[(size_t)i * kInPad + c] = __float2bfloat16_rn(x[(size_t)i * in_dim + c]);
    return v;
}

int ensure_predict(epi_mlp* h, uint32_t n_pad) {
    if (n_pad <= h->p_cap) return EPI_OK;
    for (auto& ly : h->layers) {
        if (ly.ph) cudaFree(ly.ph);
        ly.ph = nullptr;
    }
    cudaFree(h->d_py);
    cudaFree(h->d_pscore);
    h->d_py = nullptr;
    h->d_pscore = nullptr;
    h->p_cap = 0;
    for (uint32_t l = 0; l < h->L; ++l) {
        MlpLayer& ly = h->layers[l];
        const uint32_t depth = l == 0 ? 1u : h->E;
        MCK(cudaMalloc(&ly.ph, (size_t)depth * n_pad * ly.K * sizeof(__nv_bfloat16)));
        MRC(make_map(h, &ly.t_ph, ly.ph, n_pad, ly.K, kBM, depth));
    }
    MCK(cudaMalloc(&h->d_py, (size_t)h->E * n_pad * h->out_pad * sizeof(float)));
    MCK(cudaMalloc(&h->d_pscore, (size_t)h->E * n_pad * sizeof(float)));
    h->p_cap = n_pad;
    return EPI_OK;
}

// Forward pass of n host samples through every member; outputs stay in d_py (and scores in
// d_pscore when target).  The buffers hold p_cap rows per member (the largest call so far):
// member m's rows start at m * p_cap in every buffer and tensor map, whatever n is.
int forward_n(epi_mlp* h, const float* x, uint32_t n, const float* target) {
    const uint32_t n_pad = std::max<uint32_t>(round_up(n, kBM), kBM);
    MRC(ensure_predict(h, n_pad));
    const uint64_t cap = h->p_cap;
    std::vector<__nv_bfloat16> xs = pad_inputs(x, n, n_pad, h->cfg.in_dim);
    MCK(cudaMemcpyAsync(h->layers[0].ph, xs.data(), xs.size() * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice, h->stream));
    if (target) {
        MCK(cudaMemcpyAsync(h->d_ptarget, target, h->cfg.out_dim * sizeof(float), cudaMemcpyHostToDevice, h->stream));
        MCK(cudaMemsetAsync(h->d_pscore, 0, (size_t)h->E * cap * sizeof(float), h->stream));
    }
    for (uint32_t l = 0; l < h->L; ++l) {
        MlpLayer& ly = h->layers[l];
        EpiArgs a;
        a.bias = ly.b;
        a.ms_bias = ly.N;
        const uint32_t za = l == 0 ? 0u : 1u;  // the input rows are shared
        if (l + 1 < h->L) {
            a.out = h->layers[l + 1].ph;
            a.ms_out = cap * ly.N;
            MRC((gemm<128, kEpHidden>(h, ly.t_ph, ly.t_w, n_pad, ly.N, ly.K, a, za)));
        } else {
            a.outf = target ? nullptr : h->d_py;
            a.score_target = target ? h->d_ptarget : nullptr;
            a.score = target ? h->d_pscore : nullptr;
            a.n_valid = h->cfg.out_dim;
            a.m_valid = n;
            a.ms_outf = cap * ly.N;
            a.ms_score = cap;
            MRC((gemm<128, kEpOut>(h, ly.t_ph, ly.t_w, n_pad, ly.N, ly.K, a, za)));
        }
    }
    return EPI_OK;
}

void free_all(epi_mlp* h) {
    if (h->step_graph) cudaGraphExecDestroy(h->step_graph);
    for (auto& ly : h->layers) {
        cudaFree(ly.w); cudaFree(ly.b); cudaFree(ly.mw); cudaFree(ly.vw); cudaFree(ly.mb); cudaFree(ly.vb);
        cudaFree(ly.gw); cudaFree(ly.gb); cudaFree(ly.wb); cudaFree(ly.wtb);
        cudaFree(ly.h); cudaFree(ly.ht); cudaFree(ly.z); cudaFree(ly.dz); cudaFree(ly.dzt); cudaFree(ly.ph);
    }
    cudaFree(h->d_err); cudaFree(h->d_step); cudaFree(h->d_t); cudaFree(h->d_loss); cudaFree(h->d_step_loss);
    cudaFree(h->d_idx);
    cudaFree(h->d_xs); cudaFree(h->d_ys); cudaFree(h->d_py); cudaFree(h->d_pscore); cudaFree(h->d_ptarget);
    if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
}

template <int BN, int EP>
int allow_smem(epi_mlp* h) {
    MCK(cudaFuncSetAttribute(k_gemm<BN, EP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gemm_smem_bytes<BN>()));
    return EPI_OK;
}

int init(epi_mlp* h) {
    const epi_mlp_config& c = h->cfg;
    MRC((allow_smem<128, kEpHidden>(h)));
    MRC((allow_smem<128, kEpOut>(h)));
    MRC((allow_smem<128, kEpDh>(h)));
    MRC((allow_smem<128, kEpDw>(h)));
    MRC((allow_smem<64, kEpDw>(h)));
    const uint32_t E = h->E;
    h->L = c.hidden_layers + 1;
    h->B = c.batch;
    h->out_pad = round_up(c.out_dim, 128);
    MCK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    h->own_stream = true;
    MCK(cudaMalloc(&h->d_err, sizeof(int)));
    MCK(cudaMalloc(&h->d_step, sizeof(uint32_t)));
    MCK(cudaMemset(h->d_err, 0, sizeof(int)));
    MCK(cudaMemset(h->d_step, 0, sizeof(uint32_t)));
    MCK(cudaMalloc(&h->d_t, (size_t)E * h->B * h->out_pad * sizeof(float)));
    MCK(cudaMalloc(&h->d_step_loss, (size_t)E * sizeof(float)));
    MCK(cudaMalloc(&h->d_ptarget, (size_t)h->out_pad * sizeof(float)));
    h->layers.resize(h->L);
    for (uint32_t l = 0; l < h->L; ++l) {
        MlpLayer& ly = h->layers[l];
        ly.k_real = l == 0 ? c.in_dim : c.hidden;
        ly.n_real = l + 1 == h->L ? c.out_dim : c.hidden;
        ly.K = l == 0 ? kInPad : c.hidden;
        ly.N = l + 1 == h->L ? h->out_pad : c.hidden;
        const size_t nw = (size_t)E * ly.N * ly.K, nb = (size_t)E * ly.N, act_in = (size_t)E * h->B * ly.K,
                     act_out = (size_t)E * h->B * ly.N;
        for (float** p : {&ly.w, &ly.mw, &ly.vw, &ly.gw}) MCK(cudaMalloc(p, nw * sizeof(float)));
        for (float** p : {&ly.b, &ly.mb, &ly.vb, &ly.gb}) MCK(cudaMalloc(p, nb * sizeof(float)));
        MCK(cudaMalloc(&ly.wb, nw * sizeof(__nv_bfloat16)));
        MCK(cudaMalloc(&ly.wtb, nw * sizeof(__nv_bfloat16)));
        MCK(cudaMalloc(&ly.h, act_in * sizeof(__nv_bfloat16)));
        MCK(cudaMalloc(&ly.ht, act_in * sizeof(__nv_bfloat16)));
        if (l + 1 < h->L) MCK(cudaMalloc(&ly.z, act_out * sizeof(float)));
        MCK(cudaMalloc(&ly.dz, act_out * sizeof(__nv_bfloat16)));
        MCK(cudaMalloc(&ly.dzt, act_out * sizeof(__nv_bfloat16)));
        for (float* p : {ly.mw, ly.vw, ly.gw}) MCK(cudaMemset(p, 0, nw * sizeof(float)));
        for (float* p : {ly.mb, ly.vb, ly.gb}) MCK(cudaMemset(p, 0, nb * sizeof(float)));
        // operands: forward A = h (B x K), B = W (N x K); weights A = dZ^T (N x B), B = H^T (K x B);
        // inputs A = dZ (B x N), B = W^T (K x N)
        MRC(make_map(h, &ly.t_h, ly.h, h->B, ly.K, kBM, E));
        MRC(make_map(h, &ly.t_w, ly.wb, ly.N, ly.K, 128, E));
        MRC(make_map(h, &ly.t_dzt, ly.dzt, ly.N, h->B, kBM, E));
        MRC(make_map(h, &ly.t_ht, ly.ht, ly.K, h->B, ly.K == 64 ? 64 : 128, E));
        MRC(make_map(h, &ly.t_dz, ly.dz, h->B, ly.N, kBM, E));
        MRC(make_map(h, &ly.t_wt, ly.wtb, ly.K, ly.N, 128, E));
    }
    // torch.nn.Linear's default: W and b uniform in +-1/sqrt(fan_in); member m draws from
    // seed + m, layer by layer (W row by row, then b)
    for (uint32_t m = 0; m < E; ++m) {
        SplitMix rng{c.seed + m};
        for (auto& ly : h->layers) {
            const size_t nw = (size_t)ly.N * ly.K;
            const double bound = 1.0 / std::sqrt((double)ly.k_real);
            std::vector<float> w(nw, 0.f), b(ly.N, 0.f);
            for (uint32_t n = 0; n < ly.n_real; ++n)
                for (uint32_t k = 0; k < ly.k_real; ++k) w[(size_t)n * ly.K + k] = (float)((2.0 * rng.uniform() - 1.0) * bound);
            for (uint32_t n = 0; n < ly.n_real; ++n) b[n] = (float)((2.0 * rng.uniform() - 1.0) * bound);
            MCK(cudaMemcpy(ly.w + m * nw, w.data(), nw * sizeof(float), cudaMemcpyHostToDevice));
            MCK(cudaMemcpy(ly.b + (size_t)m * ly.N, b.data(), ly.N * sizeof(float), cudaMemcpyHostToDevice));
        }
    }
    MRC(cast_all(h));
    MCK(cudaStreamSynchronize(h->stream));
    return EPI_OK;
}

uint64_t member_params(const epi_mlp* h) {
    uint64_t n = 0;
    for (auto& ly : h->layers) n += (uint64_t)ly.n_real * ly.k_real + ly.n_real;
    return n;
}

// Device W / b arrays of every layer (E padded members each) -> member-major unpadded host layout.
int download_params(epi_mlp* h, float* const MlpLayer::*wp, float* const MlpLayer::*bp, float* out) {
    const uint64_t count = member_params(h);
    size_t o = 0;
    for (auto& ly : h->layers) {
        const size_t nw = (size_t)ly.N * ly.K;
        std::vector<float> w(nw * h->E), b((size_t)ly.N * h->E);
        MCK(cudaMemcpy(w.data(), ly.*wp, w.size() * sizeof(float), cudaMemcpyDeviceToHost));
        MCK(cudaMemcpy(b.data(), ly.*bp, b.size() * sizeof(float), cudaMemcpyDeviceToHost));
        for (uint32_t m = 0; m < h->E; ++m) {
            size_t q = m * count + o;
            for (uint32_t n = 0; n < ly.n_real; ++n)
                for (uint32_t k = 0; k < ly.k_real; ++k) out[q++] = w[m * nw + (size_t)n * ly.K + k];
            for (uint32_t n = 0; n < ly.n_real; ++n) out[q++] = b[(size_t)m * ly.N + n];
        }
        o += (size_t)ly.n_real * ly.k_real + ly.n_real;
    }
    return EPI_OK;
}

}  // namespace

// ---------------------------------------------------------------- C ABI
extern "C" {

int epi_mlp_create(const epi_mlp_config* cfg, epi_mlp** out) {
    if (!cfg || !out) return EPI_ERR_ARG;
    *out = nullptr;
    if (cfg->in_dim == 0 || cfg->in_dim > kInPad || cfg->hidden == 0 || cfg->hidden % 128 || cfg->hidden_layers == 0 ||
        cfg->out_dim == 0 || cfg->batch == 0 || cfg->batch % 128 || !(cfg->lr > 0.f) || cfg->members > kMaxMembers)
        return EPI_ERR_CONFIG;
    epi_mlp* h = new epi_mlp();
    h->cfg = *cfg;
    h->E = cfg->members ? cfg->members : 1u;
    h->cfg.members = h->E;
    int rc = init(h);
    // on failure the handle is kept so that the caller can read the message, then destroy it
    *out = h;
    return rc;
}

int epi_mlp_destroy(epi_mlp* h) {
    if (!h) return EPI_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    free_all(h);
    delete h;
    return EPI_OK;
}

const char* epi_mlp_last_error(const epi_mlp* h) { return h ? h->err.c_str() : "null handle"; }

int epi_mlp_set_stream(epi_mlp* h, void* cuda_stream) {
    if (!h) return EPI_ERR_ARG;
    MCK(cudaStreamSynchronize(h->stream));
    if (h->own_stream) cudaStreamDestroy(h->stream);
    h->stream = static_cast<cudaStream_t>(cuda_stream);
    h->own_stream = false;
    if (h->step_graph) {
        cudaGraphExecDestroy(h->step_graph);
        h->step_graph = nullptr;
    }
    return EPI_OK;
}

int epi_mlp_members(const epi_mlp* h, uint32_t* out) {
    if (!h || !out) return EPI_ERR_ARG;
    *out = h->E;
    return EPI_OK;
}

int epi_mlp_param_count(const epi_mlp* h, uint64_t* out) {
    if (!h || !out) return EPI_ERR_ARG;
    *out = member_params(h);
    return EPI_OK;
}

int epi_mlp_get_params(epi_mlp* h, float* out) {
    if (!h || !out) return EPI_ERR_ARG;
    MCK(cudaStreamSynchronize(h->stream));
    return download_params(h, &MlpLayer::w, &MlpLayer::b, out);
}

int epi_mlp_set_params(epi_mlp* h, const float* in) {
    if (!h || !in) return EPI_ERR_ARG;
    MCK(cudaStreamSynchronize(h->stream));
    const uint64_t count = member_params(h);
    size_t o = 0;
    for (auto& ly : h->layers) {
        const size_t nw = (size_t)ly.N * ly.K;
        std::vector<float> w(nw * h->E, 0.f), b((size_t)ly.N * h->E, 0.f);
        for (uint32_t m = 0; m < h->E; ++m) {
            size_t q = m * count + o;
            for (uint32_t n = 0; n < ly.n_real; ++n)
                for (uint32_t k = 0; k < ly.k_real; ++k) w[m * nw + (size_t)n * ly.K + k] = in[q++];
            for (uint32_t n = 0; n < ly.n_real; ++n) b[(size_t)m * ly.N + n] = in[q++];
        }
        o += (size_t)ly.n_real * ly.k_real + ly.n_real;
        MCK(cudaMemcpy(ly.w, w.data(), w.size() * sizeof(float), cudaMemcpyHostToDevice));
        MCK(cudaMemcpy(ly.b, b.data(), b.size() * sizeof(float), cudaMemcpyHostToDevice));
        for (float* p : {ly.mw, ly.vw}) MCK(cudaMemset(p, 0, w.size() * sizeof(float)));
        for (float* p : {ly.mb, ly.vb}) MCK(cudaMemset(p, 0, b.size() * sizeof(float)));
    }
    MCK(cudaMemset(h->d_step, 0, sizeof(uint32_t)));
    MRC(cast_all(h));
    MCK(cudaStreamSynchronize(h->stream));
    return EPI_OK;
}

int epi_mlp_set_dataset(epi_mlp* h, const float* x, const float* y, uint32_t n) {
    if (!h || !x || !y || n == 0) return EPI_ERR_ARG;
    MCK(cudaStreamSynchronize(h->stream));
    cudaFree(h->d_xs);
    cudaFree(h->d_ys);
    h->d_xs = nullptr;
    h->d_ys = nullptr;
    h->n_data = 0;
    std::vector<__nv_bfloat16> xs = pad_inputs(x, n, n, h->cfg.in_dim);
    std::vector<float> ys((size_t)n * h->out_pad, 0.f);
    for (uint32_t i = 0; i < n; ++i)
        std::memcpy(&ys[(size_t)i * h->out_pad], y + (size_t)i * h->cfg.out_dim, h->cfg.out_dim * sizeof(float));
    MCK(cudaMalloc(&h->d_xs, xs.size() * sizeof(__nv_bfloat16)));
    MCK(cudaMalloc(&h->d_ys, ys.size() * sizeof(float)));
    MCK(cudaMemcpy(h->d_xs, xs.data(), xs.size() * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice));
    MCK(cudaMemcpy(h->d_ys, ys.data(), ys.size() * sizeof(float), cudaMemcpyHostToDevice));
    h->n_data = n;
    return EPI_OK;
}

int epi_mlp_train(epi_mlp* h, uint32_t steps, uint64_t shuffle_seed, float* losses) {
    if (!h) return EPI_ERR_ARG;
    if (steps == 0) return EPI_OK;
    if (h->n_data < h->B) { h->err = "training set smaller than one minibatch"; return EPI_ERR_ARG; }
    const uint32_t E = h->E, B = h->B;
    // minibatch indices: member m shuffles from shuffle_seed + m, a fresh permutation every
    // epoch, whole batches only
    const uint32_t per_epoch = h->n_data / B;
    std::vector<uint32_t> idx((size_t)E * steps * B), perm(h->n_data);
    for (uint32_t m = 0; m < E; ++m) {
        SplitMix rng{shuffle_seed + m};
        uint32_t* dst = &idx[(size_t)m * steps * B];
        for (uint32_t s = 0; s < steps; ++s) {
            if (s % per_epoch == 0) {
                for (uint32_t i = 0; i < h->n_data; ++i) perm[i] = i;
                for (uint32_t i = h->n_data - 1; i > 0; --i) std::swap(perm[i], perm[rng.next() % (i + 1)]);  // Fisher-Yates
            }
            std::memcpy(dst + (size_t)s * B, &perm[(size_t)(s % per_epoch) * B], B * sizeof(uint32_t));
        }
    }
    MCK(cudaStreamSynchronize(h->stream));
    if (idx.size() > h->idx_cap) {
        cudaFree(h->d_idx);
        h->d_idx = nullptr;
        h->idx_cap = 0;
        MCK(cudaMalloc(&h->d_idx, idx.size() * sizeof(uint32_t)));
        h->idx_cap = idx.size();
    }
    if ((size_t)steps * E > h->loss_cap) {
        cudaFree(h->d_loss);
        h->d_loss = nullptr;
        h->loss_cap = 0;
        MCK(cudaMalloc(&h->d_loss, (size_t)steps * E * sizeof(float)));
        h->loss_cap = steps * E;
    }
    MCK(cudaMemcpyAsync(h->d_idx, idx.data(), idx.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, h->stream));
    // Adam's step counter keeps counting across calls; this call's minibatch s is read at
    // (*d_step - t0)
    uint32_t t0 = 0;
    MCK(cudaMemcpyAsync(&t0, h->d_step, sizeof t0, cudaMemcpyDeviceToHost, h->stream));
    MCK(cudaStreamSynchronize(h->stream));
    if (h->step_graph) {
        cudaGraphExecDestroy(h->step_graph);
        h->step_graph = nullptr;
    }
    cudaGraph_t g;
    MCK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    int rc = EPI_OK;
    {
        MlpLayer& l0 = h->layers[0];
        cudaError_t me = cudaMemsetAsync(h->d_step_loss, 0, (size_t)E * sizeof(float), h->stream);
        if (me != cudaSuccess) rc = EPI_ERR_CUDA;
        k_gather<<<dim3(B, E), 128, 0, h->stream>>>(h->d_xs, h->d_ys, h->d_idx, steps, h->d_step, t0, B, h->out_pad, l0.h,
                                                    l0.ht, h->d_t);
        if (!rc) rc = enqueue_fwd_bwd(h, h->d_step_loss);
        if (!rc) rc = enqueue_adam(h);
        if (!rc) k_step_end<<<1, 1, 0, h->stream>>>(h->d_step);
    }
    cudaError_t ce = cudaStreamEndCapture(h->stream, &g);
    if (rc) return rc;
    if (ce != cudaSuccess) { h->err = std::string("capture: ") + cudaGetErrorString(ce); return EPI_ERR_CUDA; }
    ce = cudaGraphInstantiate(&h->step_graph, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) { h->err = std::string("instantiate: ") + cudaGetErrorString(ce); return EPI_ERR_CUDA; }
    // kernels per step (each covering all members): gather, L forward + L weight + (L - 1)
    // input products, L bias reductions, L Adam updates, the step counter
    const uint64_t per_step = 2 + 4 * (uint64_t)h->L + (h->L - 1);
    for (uint32_t s = 0; s < steps; ++s) {
        MCK(cudaGraphLaunch(h->step_graph, h->stream));
        MCK(cudaMemcpyAsync(h->d_loss + (size_t)s * E, h->d_step_loss, E * sizeof(float), cudaMemcpyDeviceToDevice,
                            h->stream));
        h->launches += per_step;
    }
    MRC(check_err(h));
    if (losses) {
        std::vector<float> l((size_t)steps * E);
        MCK(cudaMemcpy(l.data(), h->d_loss, l.size() * sizeof(float), cudaMemcpyDeviceToHost));
        const float inv = 1.0f / ((float)B * (float)h->cfg.out_dim);
        for (uint32_t m = 0; m < E; ++m)
            for (uint32_t s = 0; s < steps; ++s) losses[(size_t)m * steps + s] = l[(size_t)s * E + m] * inv;
    }
    return EPI_OK;
}

int epi_mlp_gradients(epi_mlp* h, const float* x, const float* y, uint32_t n, float* grads, float* loss) {
    if (!h || !x || !y || !grads) return EPI_ERR_ARG;
    if (n != h->B) { h->err = "gradients take exactly one minibatch"; return EPI_ERR_ARG; }
    MCK(cudaStreamSynchronize(h->stream));
    const uint32_t E = h->E;
    MlpLayer& l0 = h->layers[0];
    std::vector<__nv_bfloat16> xs = pad_inputs(x, n, n, h->cfg.in_dim), xt((size_t)kInPad * n);
    for (uint32_t r = 0; r < n; ++r)
        for (uint32_t c = 0; c < kInPad; ++c) xt[(size_t)c * n + r] = xs[(size_t)r * kInPad + c];
    std::vector<float> ys((size_t)n * h->out_pad, 0.f);
    for (uint32_t i = 0; i < n; ++i)
        std::memcpy(&ys[(size_t)i * h->out_pad], y + (size_t)i * h->cfg.out_dim, h->cfg.out_dim * sizeof(float));
    for (uint32_t m = 0; m < E; ++m) {  // every member sees the same minibatch
        MCK(cudaMemcpyAsync(l0.h + (size_t)m * xs.size(), xs.data(), xs.size() * sizeof(__nv_bfloat16),
                            cudaMemcpyHostToDevice, h->stream));
        MCK(cudaMemcpyAsync(l0.ht + (size_t)m * xt.size(), xt.data(), xt.size() * sizeof(__nv_bfloat16),
                            cudaMemcpyHostToDevice, h->stream));
        MCK(cudaMemcpyAsync(h->d_t + (size_t)m * ys.size(), ys.data(), ys.size() * sizeof(float), cudaMemcpyHostToDevice,
                            h->stream));
    }
    float* d_l = nullptr;
    MCK(cudaMalloc(&d_l, E * sizeof(float)));
    MCK(cudaMemsetAsync(d_l, 0, E * sizeof(float), h->stream));
    int rc = enqueue_fwd_bwd(h, d_l);
    if (!rc) rc = check_err(h);
    std::vector<float> lsum(E, 0.f);
    if (!rc && cudaMemcpy(lsum.data(), d_l, E * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess) rc = EPI_ERR_CUDA;
    cudaFree(d_l);
    if (rc) {
        if (rc == EPI_ERR_CUDA && h->err.empty()) h->err = "gradients: device copy failed";
        return rc;
    }
    if (loss)
        for (uint32_t m = 0; m < E; ++m) loss[m] = lsum[m] / ((float)n * (float)h->cfg.out_dim);
    return download_params(h, &MlpLayer::gw, &MlpLayer::gb, grads);
}

int epi_mlp_predict(epi_mlp* h, const float* x, uint32_t n, float* y) {
    if (!h || !x || !y) return EPI_ERR_ARG;
    if (n == 0) return EPI_OK;
    MRC(forward_n(h, x, n, nullptr));
    MRC(check_err(h));
    const size_t per = (size_t)h->p_cap * h->out_pad;
    std::vector<float> tmp((size_t)n * h->out_pad);
    for (uint32_t m = 0; m < h->E; ++m) {
        MCK(cudaMemcpy(tmp.data(), h->d_py + m * per, tmp.size() * sizeof(float), cudaMemcpyDeviceToHost));
        float* ym = y + (size_t)m * n * h->cfg.out_dim;
        for (uint32_t i = 0; i < n; ++i)
            std::memcpy(ym + (size_t)i * h->cfg.out_dim, &tmp[(size_t)i * h->out_pad], h->cfg.out_dim * sizeof(float));
    }
    return EPI_OK;
}

int epi_mlp_score(epi_mlp* h, const float* x, uint32_t n, const float* target, float* score) {
    if (!h || !x || !target || !score) return EPI_ERR_ARG;
    if (n == 0) return EPI_OK;
    MRC(forward_n(h, x, n, target));
    MRC(check_err(h));
    for (uint32_t m = 0; m < h->E; ++m)
        MCK(cudaMemcpy(score + (size_t)m * n, h->d_pscore + (size_t)m * h->p_cap, (size_t)n * sizeof(float),
                       cudaMemcpyDeviceToHost));
    return EPI_OK;
}

int epi_mlp_kernels_launched(const epi_mlp* h, uint64_t* out) {
    if (!h || !out) return EPI_ERR_ARG;
    *out = h->launches;
    return EPI_OK;
}

}  // extern "C"
