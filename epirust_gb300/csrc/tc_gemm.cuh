// tc_gemm.cuh -- BF16 matrix products on the sm_103a tensor cores (tcgen05 + TMA), with the
// fused epilogues of the surrogate MLP.
//
// D[m][n] = sum_k A[m][k] * B[n][k]: A is M x K and B is N x K, both row-major BF16 with K
// contiguous ("K-major").  One CTA of 128 threads computes a 128 x BN tile of D:
//   thread 0      issues TMA loads of 128 x 64 (A) and BN x 64 (B) tiles into a 2-stage ring
//                 of shared memory (128-byte swizzle), and tcgen05.mma (M = 128, N = BN,
//                 K = 16) on each stage, accumulating in FP32 in tensor memory;
//   all 4 warps   wait for the last MMA, read their 32 lanes (rows) of the accumulator with
//                 tcgen05.ld, apply the epilogue and store.
// Every wait on an mbarrier is bounded: on expiry the kernel raises a flag in *err, waits
// (again bounded) for its own copies and MMAs still in flight, frees tensor memory and exits.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <stdint.h>

namespace epi {
namespace tc {

constexpr int kBM = 128;         // rows of a tile (MMA M)
constexpr int kBK = 64;          // K per stage: one 128-byte row of BF16
constexpr int kStages = 2;
constexpr int kGemmThreads = 128;
constexpr uint32_t kSpinLimit = 1u << 22;  // polls (about 0.3 s with the back-off) before a wait fails

// Epilogues.
enum Epilogue : int {
    kEpHidden = 0,  // x = acc + bias; z = x (fp32, optional); out = gelu(x) (bf16) and out_t = its transpose
    kEpOut = 1,     // x = acc + bias; outf = x (optional); with targets: loss += (x - t)^2 and
                    // out/out_t = bf16(2 (x - t) / (rows * outputs)); with a score target: score[m] += (x - s)^2
    kEpDh = 2,      // out/out_t = bf16(acc * gelu'(zin))
    kEpDw = 3       // outf = acc (fp32)
};

// Pointers are those of member 0 of a stack of networks; member m (blockIdx.z) adds m times
// the ms_* element stride of each (0: shared by all members).
struct EpiArgs {
    const float* bias = nullptr;        // [N]
    float* z = nullptr;                 // [M x N]
    const float* zin = nullptr;         // [M x N]
    __nv_bfloat16* out = nullptr;       // [M x N]
    __nv_bfloat16* out_t = nullptr;     // [N x M]
    float* outf = nullptr;              // [M x N]
    const float* target = nullptr;      // [M x N] training targets (padding columns ignored)
    const float* score_target = nullptr;  // [n_valid]
    float* loss = nullptr;              // one float, accumulated
    float* score = nullptr;             // [M], accumulated
    uint32_t n_valid = 0;               // real output columns
    uint32_t m_valid = 0;               // real sample rows
    float grad_scale = 0.f;
    uint64_t ms_bias = 0, ms_z = 0, ms_zin = 0, ms_out = 0, ms_outf = 0, ms_target = 0, ms_score = 0, ms_loss = 0;
};

// The member-m view of a.
__device__ __forceinline__ EpiArgs member_args(const EpiArgs& a, uint32_t m) {
    EpiArgs b = a;
    if (b.bias) b.bias += m * a.ms_bias;
    if (b.z) b.z += m * a.ms_z;
    if (b.zin) b.zin += m * a.ms_zin;
    if (b.out) b.out += m * a.ms_out;
    if (b.out_t) b.out_t += m * a.ms_out;  // both orientations hold M x N elements
    if (b.outf) b.outf += m * a.ms_outf;
    if (b.target) b.target += m * a.ms_target;
    if (b.score) b.score += m * a.ms_score;
    if (b.loss) b.loss += m * a.ms_loss;
    return b;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// Bounded wait for the phase with the given parity to complete; false when it did not.
// test_wait never suspends, so the poll count bounds the time spent.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    const uint32_t addr = smem_u32(bar);
    for (uint32_t it = 0; it < kSpinLimit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(addr), "r"(parity)
            : "memory");
        if (done) return true;
        if (it >= 64) __nanosleep(32);
    }
    return false;
}

// Tile (x, y) of member z of a 3-D tensor map {K, rows, members}.
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int32_t x, int32_t y, int32_t z,
                                            uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor of a K-major operand tile written by TMA with the 128-byte
// swizzle: rows 128 bytes apart, 8-row groups 1024 bytes apart (stride byte offset), the
// leading byte offset unused for swizzled K-major layouts, descriptor version 1, swizzle
// mode 2 (128 B).  The tile base is 1024-byte aligned, so the base offset field is 0.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(1024u >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), BF16 A and B
// (bits 7-9 = 1, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 in bits 17-22 and
// M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t instr_desc(uint32_t m, uint32_t n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((m >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
        : "memory");
}
// Arrive on bar once every tcgen05 operation this thread issued before has completed.
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float v[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
        "[%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

// GELU(x) = x * Phi(x) and its derivative Phi(x) + x * phi(x), with the CUDA erff / expf.
__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
    return 0.5f * (1.0f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

template <int EP>
__device__ __forceinline__ void epilogue16(const EpiArgs& a, uint32_t M, uint32_t N, uint32_t m, uint32_t n,
                                           const float v[16], float& lsum, float& ssum) {
    if (EP == kEpDw) {
        float4* o = reinterpret_cast<float4*>(a.outf + (size_t)m * N + n);
#pragma unroll
        for (int q = 0; q < 4; ++q) o[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
        return;
    }
    float x[16];
    __align__(16) __nv_bfloat16 hb[16];
    bool write_bf16 = true;
    if (EP == kEpHidden) {
#pragma unroll
        for (int j = 0; j < 16; ++j) x[j] = v[j] + __ldg(a.bias + n + j);
        if (a.z) {
            float4* o = reinterpret_cast<float4*>(a.z + (size_t)m * N + n);
#pragma unroll
            for (int q = 0; q < 4; ++q) o[q] = make_float4(x[4 * q], x[4 * q + 1], x[4 * q + 2], x[4 * q + 3]);
        }
#pragma unroll
        for (int j = 0; j < 16; ++j) hb[j] = __float2bfloat16_rn(gelu(x[j]));
    } else if (EP == kEpOut) {
#pragma unroll
        for (int j = 0; j < 16; ++j) x[j] = v[j] + __ldg(a.bias + n + j);
        if (a.outf) {
            float4* o = reinterpret_cast<float4*>(a.outf + (size_t)m * N + n);
#pragma unroll
            for (int q = 0; q < 4; ++q) o[q] = make_float4(x[4 * q], x[4 * q + 1], x[4 * q + 2], x[4 * q + 3]);
        }
        const bool row_ok = m < a.m_valid;
        if (a.score_target && row_ok) {
#pragma unroll
            for (int j = 0; j < 16; ++j)
                if (n + j < a.n_valid) {
                    const float e = x[j] - __ldg(a.score_target + n + j);
                    ssum += e * e;
                }
        }
        write_bf16 = a.target != nullptr;
        if (write_bf16) {
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                float d = 0.f;
                if (row_ok && n + j < a.n_valid) d = x[j] - __ldg(a.target + (size_t)m * N + n + j);
                lsum += d * d;
                hb[j] = __float2bfloat16_rn(d * a.grad_scale);
            }
        }
    } else {  // kEpDh
        const float4* zi = reinterpret_cast<const float4*>(a.zin + (size_t)m * N + n);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float4 zz = zi[q];
            hb[4 * q + 0] = __float2bfloat16_rn(v[4 * q + 0] * gelu_grad(zz.x));
            hb[4 * q + 1] = __float2bfloat16_rn(v[4 * q + 1] * gelu_grad(zz.y));
            hb[4 * q + 2] = __float2bfloat16_rn(v[4 * q + 2] * gelu_grad(zz.z));
            hb[4 * q + 3] = __float2bfloat16_rn(v[4 * q + 3] * gelu_grad(zz.w));
        }
    }
    if (!write_bf16) return;
    if (a.out) {
        uint4* o = reinterpret_cast<uint4*>(a.out + (size_t)m * N + n);
        o[0] = *reinterpret_cast<const uint4*>(&hb[0]);
        o[1] = *reinterpret_cast<const uint4*>(&hb[8]);
    }
    if (a.out_t) {  // lanes hold consecutive rows m: each column's 32 values land side by side
#pragma unroll
        for (int j = 0; j < 16; ++j) a.out_t[(size_t)(n + j) * M + m] = hb[j];
    }
}

// Stage ring + 1 KB for the 1024-byte alignment of the swizzled tiles: 65 KB with BN = 128,
// so three CTAs share an SM and one's epilogue overlaps the others' copies and products.
// (Measured on the screen of 65,536 candidates by 5 members: a hidden 512 x 512 product took
// 650 us with 3 stages and one CTA per SM, 418 us with two CTAs, 347 us with 2 stages and
// three CTAs.)
template <int BN>
constexpr uint32_t gemm_smem_bytes() {
    return (uint32_t)kStages * (uint32_t)(kBM + BN) * kBK * 2u + 1024u;
}

// Grid (M / 128, N / BN, members); M % 128 == 0, N % BN == 0, K % 64 == 0 (checked by the
// host).  za / zb: 1 when A / B differ per member, 0 when the member stack shares member 0's.
template <int BN, int EP>
__global__ void __launch_bounds__(kGemmThreads, 3)
    k_gemm(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, uint32_t M, uint32_t N,
           uint32_t K, EpiArgs margs, uint32_t za, uint32_t zb, int* err) {
    const EpiArgs args = member_args(margs, blockIdx.z);
    static_assert(BN == 64 || BN == 128 || BN == 256, "UMMA N");
    constexpr uint32_t kABytes = kBM * kBK * 2, kBBytes = BN * kBK * 2, kStageBytes = kABytes + kBBytes;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    __shared__ __align__(8) uint64_t full_bar[kStages];
    __shared__ __align__(8) uint64_t empty_bar[kStages];
    __shared__ __align__(8) uint64_t done_bar;
    __shared__ uint32_t tmem_base;

    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t m0 = blockIdx.x * kBM, n0 = blockIdx.y * BN;
    const uint32_t nk = K / kBK;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&full_bar[s], 1);
            mbar_init(&empty_bar[s], 1);
        }
        mbar_init(&done_bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"((uint32_t)BN)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base;

    if (threadIdx.x == 0) {
        const uint32_t idesc = instr_desc(kBM, BN);
        uint32_t issued = 0, consumed = 0;
        bool ok = true;
        auto load_stage = [&](uint32_t kb) {
            const uint32_t s = kb % kStages;
            uint8_t* sa = smem + s * kStageBytes;
            mbar_expect_tx(&full_bar[s], kStageBytes);
            tma_load_3d(sa, &ta, (int32_t)(kb * kBK), (int32_t)m0, (int32_t)(blockIdx.z * za), &full_bar[s]);
            tma_load_3d(sa + kABytes, &tb, (int32_t)(kb * kBK), (int32_t)n0, (int32_t)(blockIdx.z * zb), &full_bar[s]);
            ++issued;
        };
        for (uint32_t kb = 0; kb < nk && kb < (uint32_t)kStages; ++kb) load_stage(kb);
        for (uint32_t kb = 0; kb < nk; ++kb) {
            const uint32_t s = kb % kStages, ph = (kb / kStages) & 1u;
            if (!mbar_wait(&full_bar[s], ph)) { ok = false; break; }
            ++consumed;
            tc_fence_after();
            const uint32_t sa = smem_u32(smem + s * kStageBytes), sb = sa + kABytes;
#pragma unroll
            for (int j = 0; j < kBK / 16; ++j)  // K = 16 per MMA: advance 32 bytes within the swizzled row
                mma_bf16(tmem, smem_desc(sa + 32u * j), smem_desc(sb + 32u * j), idesc, (kb | (uint32_t)j) != 0u);
            mma_commit(&empty_bar[s]);
            if (kb + kStages < nk) {
                if (!mbar_wait(&empty_bar[s], ph)) { ok = false; break; }  // stage s read by its MMAs
                load_stage(kb + kStages);
            }
        }
        if (!ok) {
            atomicOr(err, 1);
            // drain: copies issued but not consumed
            for (uint32_t kb = consumed; kb < issued; ++kb) mbar_wait(&full_bar[kb % kStages], (kb / kStages) & 1u);
        }
        mma_commit(&done_bar);  // arrives when every MMA issued above has completed
    }
    __syncwarp();
    // warp-uniform, so that tcgen05.ld below runs on all 32 lanes or none
    const bool done = __all_sync(0xFFFFFFFFu, mbar_wait(&done_bar, 0));
    tc_fence_after();
    if (!done) {
        if (lane == 0) atomicOr(err, 2);
    } else {
        const uint32_t m = m0 + warp * 32u + lane;
        float lsum = 0.f, ssum = 0.f;
#pragma unroll 1
        for (uint32_t c = 0; c < (uint32_t)BN; c += 16) {
            float v[16];
            tmem_ld16(tmem + ((warp * 32u) << 16) + c, v);
            epilogue16<EP>(args, M, N, m, n0 + c, v, lsum, ssum);
        }
        if (EP == kEpOut) {
            if (args.score && m < args.m_valid) atomicAdd(args.score + m, ssum);
            if (args.loss && args.target) {
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xFFFFFFFFu, lsum, o);
                if (lane == 0) atomicAdd(args.loss, lsum);
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)BN) : "memory");
}

}  // namespace tc
}  // namespace epi
