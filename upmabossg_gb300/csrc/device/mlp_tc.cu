// Surrogate GEMM on the fifth-generation tensor cores (tcgen05, sm_103a):
//   C[M x N] = alpha * A[M x K] . B[K x N] (+ bias[n]) (ReLU), A and B BF16, accumulation FP32 in
//   tensor memory (TMEM).
// One CTA (4 warps) computes a 128 x TN tile (TN = 128 or 256). K is consumed in 64-wide blocks:
// one thread issues TMA copies (cp.async.bulk.tensor, 128-byte swizzle) of the A and B^T tiles into
// a STAGES-deep shared-memory ring, another issues 128 x TN x 16 tcgen05.mma instructions from the
// swizzled K-major descriptors and commits each block to the stage's "empty" mbarrier, and the
// two meet only through the ring's mbarriers. The epilogue reads the accumulator with tcgen05.ld
// (warp w owns TMEM lanes 32w .. 32w + 31 = tile rows), applies alpha, bias and ReLU and writes
// each thread's 32-column runs with 16-byte stores. Requirements (mlp_gemm_tc_supported): A rows
// K-contiguous (a_k == 1) with no device-side row offset, B given transposed (element (k, n) at
// B[n * b_n + k], b_k == 1), K, a_m and b_n multiples of 8, 16-byte aligned A and B.
#include <cuda.h>  // CUtensorMap and its encoder's signature (the encoder is fetched at run time)
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "mlp.h"

namespace mbg {

namespace {

constexpr int TM = 128, TK = 64;
constexpr int kTileBytesA = TM * TK * 2;  // 16 KiB A tile per stage
constexpr unsigned kSpinLimit = 1u << 22;  // bounded mbarrier waits

// Shapes: TN output columns per CTA (the MMA's N and the TMEM columns it holds), STAGES deep ring.
template <int TN, int STAGES>
struct TcShape {
    static constexpr int kTileBytesB = TN * TK * 2;
    static constexpr int kStageBytes = kTileBytesA + kTileBytesB;       // A tile, then B tile
    static constexpr int kSmemBytes = STAGES * kStageBytes + 1024;      // + alignment slack
    // Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), BF16 A and B (bits 7-9
    // and 10-12 = 1), both K-major (bits 15, 16 = 0), N / 8 at bits 17-22, M / 16 at bits 24-28.
    static constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TN >> 3) << 17) |
                                       ((uint32_t)(TM >> 4) << 24);
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Waits until the phase with parity `parity` of the mbarrier has completed; false after the
// spin limit.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) {
    const uint32_t a = smem_u32(bar);
    for (unsigned i = 0; i < kSpinLimit; ++i) {
        uint32_t done = 0;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void mma_bf16_tc(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                            uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// 32 consecutive FP32 accumulator columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace

// ---------------------------------------------------------------------------------------------
// TMA form: the A and B^T tiles arrive by cp.async.bulk.tensor (128-byte swizzle, box 64 x rows)
// into a STAGES-deep ring; one thread issues the copies, another the MMAs, and the ring is driven
// by mbarriers alone (full: the copy's bytes landed; empty: the MMAs that read the stage are done),
// so neither thread waits for the other except through those barriers. The shared-memory
// descriptors use the 128-byte swizzle layout (8-row groups 1024 bytes apart; a K step of 16
// elements advances the start address by 32 bytes inside the swizzle atom).

namespace {

__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | (1ull << 16) | ((uint64_t)(1024u >> 4) << 32) | (1ull << 46) |
           (2ull << 61);
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

}  // namespace

template <int TN, int STAGES>
__global__ void __launch_bounds__(128) mlp_gemm_tma_kernel(const __grid_constant__ CUtensorMap tmA,
                                                           const __grid_constant__ CUtensorMap tmB,
                                                           const GemmArgs g, unsigned* error_flag) {
    using S = TcShape<TN, STAGES>;
    constexpr int kStageBytes = S::kStageBytes;
    extern __shared__ unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t full[STAGES], empty[STAGES], done;
    __shared__ uint32_t tmem_slot;
    __shared__ unsigned fail;
    unsigned char* smem = reinterpret_cast<unsigned char*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const uint32_t sbase = smem_u32(smem);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.y * TM, n0 = blockIdx.x * TN;
    const int nk = (g.K + TK - 1) / TK;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"(TN)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (threadIdx.x == 0) {
        for (int i = 0; i < STAGES; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], 1);
        }
        mbar_init(&done, 1);
        fail = 0u;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;

    if (threadIdx.x == 0) {
        // producer: stage kb % STAGES gets K block kb once the MMAs of block kb - STAGES are done
        for (int kb = 0; kb < nk; ++kb) {
            const int st = kb % STAGES;
            if (kb >= STAGES && !mbar_wait(&empty[st], (unsigned)(((kb / STAGES) - 1) & 1))) {
                fail = 1u;
                break;
            }
            const uint32_t a = sbase + st * kStageBytes;
            mbar_expect_tx(&full[st], (uint32_t)kStageBytes);
            tma_load_2d(a, &tmA, kb * TK, m0, &full[st]);
            tma_load_2d(a + kTileBytesA, &tmB, kb * TK, n0, &full[st]);
        }
    } else if (threadIdx.x == 32) {
        // MMA issuer: four 128 x TN x 16 products per K block, then the stage is released
        for (int kb = 0; kb < nk; ++kb) {
            const int st = kb % STAGES;
            if (!mbar_wait(&full[st], (unsigned)((kb / STAGES) & 1))) {
                fail = 1u;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t a = sbase + st * kStageBytes, b = a + kTileBytesA;
            const int steps = (min(TK, g.K - kb * TK) + 15) / 16;
            for (int s = 0; s < steps; ++s)
                mma_bf16_tc(tmem, smem_desc_sw128(a + 32u * s), smem_desc_sw128(b + 32u * s), S::kIdesc,
                            (kb > 0 || s > 0) ? 1u : 0u);
            mma_commit(&empty[st]);
        }
        mma_commit(&done);
    }
    // everyone: the accumulator is complete once the last commit has arrived
    bool ok = nk == 0 || mbar_wait(&done, 0u);
    __syncwarp();
    ok = ok && !*((volatile unsigned*)&fail);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!ok && lane == 0) atomicOr(error_flag, 1u);

    const int row = m0 + warp * 32 + lane;
    const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
    const bool vec_b = g.Cb && (g.ldcb % 8) == 0 && ((uintptr_t)g.Cb & 15u) == 0;
    const bool vec_f = g.C && !g.accumulate && (g.ldc % 4) == 0 && ((uintptr_t)g.C & 15u) == 0;
    const bool vec_bias = ((uintptr_t)g.bias & 15u) == 0 && (n0 % 4) == 0;
#pragma unroll 1
    for (int c0 = 0; c0 < TN; c0 += 32) {
        float v[32];
        __syncwarp();  // tcgen05.ld is warp-collective: reconverge after the previous chunk's exits
        tmem_ld32(lane_addr + (uint32_t)c0, v);
        const int col0 = n0 + c0;
        if (!ok || row >= g.M || col0 >= g.N) continue;
        const bool full_cols = col0 + 32 <= g.N;
        float bias[32];
        if (g.bias && full_cols && vec_bias) {
            // the same 32 values for every lane: eight 16-byte broadcast loads
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const float4 b4 = __ldg(reinterpret_cast<const float4*>(g.bias + col0) + q);
                bias[4 * q] = b4.x;
                bias[4 * q + 1] = b4.y;
                bias[4 * q + 2] = b4.z;
                bias[4 * q + 3] = b4.w;
            }
        } else {
#pragma unroll
            for (int i = 0; i < 32; ++i) bias[i] = g.bias && col0 + i < g.N ? __ldg(g.bias + col0 + i) : 0.f;
        }
#pragma unroll
        for (int i = 0; i < 32; ++i) {
            float x = g.alpha * (nk > 0 ? v[i] : 0.f) + bias[i];
            if (g.relu) x = x > 0.f ? x : 0.f;
            v[i] = x;
        }
        if (g.Cb) {
            __nv_bfloat16* dst = g.Cb + (long long)row * g.ldcb + col0;
            if (full_cols && vec_b) {
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    uint4 w;
                    unsigned* wp = reinterpret_cast<unsigned*>(&w);
#pragma unroll
                    for (int h = 0; h < 4; ++h) {
                        const __nv_bfloat162 b2 = __floats2bfloat162_rn(v[8 * q + 2 * h], v[8 * q + 2 * h + 1]);
                        wp[h] = *reinterpret_cast<const unsigned*>(&b2);
                    }
                    reinterpret_cast<uint4*>(dst)[q] = w;
                }
            } else {
#pragma unroll
                for (int i = 0; i < 32; ++i)
                    if (col0 + i < g.N) dst[i] = __float2bfloat16(v[i]);
            }
        }
        if (g.C) {
            float* dst = g.C + (long long)row * g.ldc + col0;
            if (full_cols && vec_f) {
#pragma unroll
                for (int q = 0; q < 8; ++q)
                    reinterpret_cast<float4*>(dst)[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
            } else {
#pragma unroll
                for (int i = 0; i < 32; ++i)
                    if (col0 + i < g.N) dst[i] = g.accumulate ? dst[i] + v[i] : v[i];
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TN) : "memory");
}

// ---------------------------------------------------------------------------------------------
// Persistent form for products of many tiles (the surrogate's prediction chunks): one CTA per SM
// walks the 128 x 256 output tiles i = blockIdx.x, + gridDim.x, ... with three roles on separate
// warps that meet only through mbarriers — warp 0 issues the TMA copies into a 4-stage ring,
// warp 1 issues the MMAs, warps 2-5 run the epilogue — and two accumulators of 256 TMEM columns
// each (the whole 512-column tensor memory), so that the epilogue of tile i (TMEM -> registers ->
// bias/ReLU -> global) overlaps the MMAs of tile i + 1. acc_full[a] is committed by the MMAs of
// a tile that used accumulator a; acc_empty[a] collects one arrival per epilogue warp once it
// has read accumulator a out. Every wait is bounded and also gives up as soon as another role
// has failed (a shared flag), so a failed wait ends the kernel quickly with the error flag set.

namespace {

constexpr int kPStages = 4, kPTN = 256;
constexpr int kPStageBytes = kTileBytesA + kPTN * TK * 2;  // 48 KiB
constexpr int kPSmemBytes = kPStages * kPStageBytes + 1024;
constexpr uint32_t kPIdesc = TcShape<kPTN, 2>::kIdesc;

__device__ __forceinline__ bool mbar_wait_or_fail(uint64_t* bar, unsigned parity, volatile unsigned* fail) {
    const uint32_t a = smem_u32(bar);
    for (unsigned i = 0; i < kSpinLimit; ++i) {
        uint32_t done = 0;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        if ((i & 255u) == 255u && *fail) return false;
    }
    *fail = 1u;
    return false;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

}  // namespace

__global__ void __launch_bounds__(192, 1) mlp_gemm_tma_persistent(const __grid_constant__ CUtensorMap tmA,
                                                                  const __grid_constant__ CUtensorMap tmB,
                                                                  const GemmArgs g, unsigned* error_flag,
                                                                  int tiles_n, int tiles) {
    extern __shared__ unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t full[kPStages], empty[kPStages], acc_full[2], acc_empty[2], drain;
    __shared__ uint32_t tmem_slot;
    __shared__ unsigned fail;
    unsigned char* smem = reinterpret_cast<unsigned char*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const uint32_t sbase = smem_u32(smem);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nk = (g.K + TK - 1) / TK;
    volatile unsigned* vfail = &fail;

    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"(2 * kPTN)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (threadIdx.x == 0) {
        for (int i = 0; i < kPStages; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], 1);
        }
        for (int i = 0; i < 2; ++i) {
            mbar_init(&acc_full[i], 1);
            mbar_init(&acc_empty[i], 4);  // one arrival per epilogue warp
        }
        mbar_init(&drain, 1);
        fail = 0u;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;

    if (warp == 0) {
        if (lane == 0) {  // producer: K block `it` of this CTA's run goes to stage it % kPStages
            int it = 0;
            for (int tile = blockIdx.x; tile < tiles && !*vfail; tile += gridDim.x) {
                const int m0 = (tile / tiles_n) * TM, n0 = (tile % tiles_n) * kPTN;
                for (int kb = 0; kb < nk; ++kb, ++it) {
                    const int st = it % kPStages;
                    if (it >= kPStages && !mbar_wait_or_fail(&empty[st], (unsigned)(((it / kPStages) - 1) & 1), vfail))
                        break;
                    const uint32_t a = sbase + st * kPStageBytes;
                    mbar_expect_tx(&full[st], (uint32_t)kPStageBytes);
                    tma_load_2d(a, &tmA, kb * TK, m0, &full[st]);
                    tma_load_2d(a + kTileBytesA, &tmB, kb * TK, n0, &full[st]);
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {  // MMA issuer: tile j of this CTA accumulates in accumulator j & 1
            int it = 0, j = 0;
            for (int tile = blockIdx.x; tile < tiles && !*vfail; tile += gridDim.x, ++j) {
                const int acc = j & 1;
                if (j >= 2 && !mbar_wait_or_fail(&acc_empty[acc], (unsigned)(((j >> 1) - 1) & 1), vfail)) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t d = tmem + (uint32_t)(acc * kPTN);
                bool ok = true;
                for (int kb = 0; kb < nk; ++kb, ++it) {
                    const int st = it % kPStages;
                    if (!mbar_wait_or_fail(&full[st], (unsigned)((it / kPStages) & 1), vfail)) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t a = sbase + st * kPStageBytes, b = a + kTileBytesA;
                    const int steps = (min(TK, g.K - kb * TK) + 15) / 16;
                    for (int s = 0; s < steps; ++s)
                        mma_bf16_tc(d, smem_desc_sw128(a + 32u * s), smem_desc_sw128(b + 32u * s), kPIdesc,
                                    (kb > 0 || s > 0) ? 1u : 0u);
                    mma_commit(&empty[st]);
                }
                if (!ok) break;
                mma_commit(&acc_full[acc]);
            }
            // every MMA issued here has completed before the tensor memory is released, even when
            // a failed wait cut the loop short
            mma_commit(&drain);
            mbar_wait(&drain, 0u);
        }
    } else {  // epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31, the tile's rows of that quarter
        const int q = warp & 3;
        const bool vec_b = g.Cb && (g.ldcb % 8) == 0 && ((uintptr_t)g.Cb & 15u) == 0;
        const bool vec_f = g.C && !g.accumulate && (g.ldc % 4) == 0 && ((uintptr_t)g.C & 15u) == 0;
        int j = 0;
        for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x, ++j) {
            const int acc = j & 1;
            bool ok = mbar_wait_or_fail(&acc_full[acc], (unsigned)((j >> 1) & 1), vfail);
            ok = __all_sync(0xffffffffu, ok);
            if (!ok) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int m0 = (tile / tiles_n) * TM, n0 = (tile % tiles_n) * kPTN;
            const int row = m0 + q * 32 + lane;
            const uint32_t lane_addr = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(acc * kPTN);
            const bool vec_bias = ((uintptr_t)g.bias & 15u) == 0 && (n0 % 4) == 0;
#pragma unroll 1
            for (int c0 = 0; c0 < kPTN; c0 += 32) {
                float v[32];
                __syncwarp();
                tmem_ld32(lane_addr + (uint32_t)c0, v);
                const int col0 = n0 + c0;
                if (row >= g.M || col0 >= g.N) continue;
                const bool full_cols = col0 + 32 <= g.N;
                float bias[32];
                if (g.bias && full_cols && vec_bias) {
#pragma unroll
                    for (int k4 = 0; k4 < 8; ++k4) {
                        const float4 b4 = __ldg(reinterpret_cast<const float4*>(g.bias + col0) + k4);
                        bias[4 * k4] = b4.x;
                        bias[4 * k4 + 1] = b4.y;
                        bias[4 * k4 + 2] = b4.z;
                        bias[4 * k4 + 3] = b4.w;
                    }
                } else {
#pragma unroll
                    for (int i = 0; i < 32; ++i) bias[i] = g.bias && col0 + i < g.N ? __ldg(g.bias + col0 + i) : 0.f;
                }
#pragma unroll
                for (int i = 0; i < 32; ++i) {
                    float x = g.alpha * v[i] + bias[i];
                    if (g.relu) x = x > 0.f ? x : 0.f;
                    v[i] = x;
                }
                if (g.Cb) {
                    __nv_bfloat16* dst = g.Cb + (long long)row * g.ldcb + col0;
                    if (full_cols && vec_b) {
#pragma unroll
                        for (int k4 = 0; k4 < 4; ++k4) {
                            uint4 w;
                            unsigned* wp = reinterpret_cast<unsigned*>(&w);
#pragma unroll
                            for (int h = 0; h < 4; ++h) {
                                const __nv_bfloat162 b2 = __floats2bfloat162_rn(v[8 * k4 + 2 * h], v[8 * k4 + 2 * h + 1]);
                                wp[h] = *reinterpret_cast<const unsigned*>(&b2);
                            }
                            reinterpret_cast<uint4*>(dst)[k4] = w;
                        }
                    } else {
#pragma unroll
                        for (int i = 0; i < 32; ++i)
                            if (col0 + i < g.N) dst[i] = __float2bfloat16(v[i]);
                    }
                }
                if (g.C) {
                    float* dst = g.C + (long long)row * g.ldc + col0;
                    if (full_cols && vec_f) {
#pragma unroll
                        for (int k4 = 0; k4 < 8; ++k4)
                            reinterpret_cast<float4*>(dst)[k4] =
                                make_float4(v[4 * k4], v[4 * k4 + 1], v[4 * k4 + 2], v[4 * k4 + 3]);
                    } else {
#pragma unroll
                        for (int i = 0; i < 32; ++i)
                            if (col0 + i < g.N) dst[i] = g.accumulate ? dst[i] + v[i] : v[i];
                    }
                }
            }
            // the accumulator is read out: the MMAs of tile j + 2 may overwrite it
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(&acc_empty[acc]);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (threadIdx.x == 0 && fail) atomicOr(error_flag, 1u);
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * kPTN) : "memory");
}

namespace {

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encoder() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
        else
            cudaGetLastError();
    });
    return fn;
}

// A K-contiguous BF16 matrix of `rows` rows (row stride ld elements, K columns) as a 2-D tensor
// map with 64 x box_rows boxes and the 128-byte swizzle; rows and columns outside read as zero.
bool encode_kmajor(CUtensorMap* map, const __nv_bfloat16* base, long long rows, int K, long long ld, int box_rows) {
    EncodeTiledFn fn = encoder();
    if (!fn) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    const cuuint32_t box[2] = {(cuuint32_t)TK, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<__nv_bfloat16*>(base), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

bool mlp_gemm_tc_supported(const GemmArgs& g) {
    auto aligned16 = [](const void* p) { return ((uintptr_t)p & 15u) == 0; };
    return g.M > 0 && g.N > 0 && g.K > 0 && g.a_k == 1 && g.b_k == 1 && g.K % 8 == 0 && g.a_m % 8 == 0 &&
           g.b_n % 8 == 0 && aligned16(g.A) && aligned16(g.B) && !g.a_row_offset && encoder() != nullptr;
}

cudaError_t mlp_gemm_tc_configure() {
    cudaError_t e = cudaFuncSetAttribute(mlp_gemm_tma_kernel<128, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         TcShape<128, 3>::kSmemBytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(mlp_gemm_tma_kernel<256, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 TcShape<256, 2>::kSmemBytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(mlp_gemm_tma_persistent, cudaFuncAttributeMaxDynamicSharedMemorySize, kPSmemBytes);
    return e;
}

namespace {
int sm_count() {
    static int n = 0;
    static std::once_flag once;
    std::call_once(once, [] {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            n = 0;
    });
    return n;
}
}  // namespace

cudaError_t mlp_gemm_tc(const GemmArgs& g, unsigned* error_flag, cudaStream_t s) {
    if (!mlp_gemm_tc_supported(g)) return cudaErrorInvalidValue;
    const int mt = (g.M + TM - 1) / TM;
    // 128 x 256 tiles with a 2-stage ring for products wider than 128 columns, 128 x 128 with 3
    // stages otherwise: 96 KB of shared memory per CTA, so that two CTAs share an SM and one's
    // epilogue overlaps the other's K loop (measured: 295 TFLOP/s on the surrogate's forward pass,
    // against 198 with one 4-stage CTA per SM)
    const int tn = g.N > 128 ? 256 : 128;
    CUtensorMap ma, mb;
    if (!encode_kmajor(&ma, g.A, g.M, g.K, g.a_m, TM) || !encode_kmajor(&mb, g.B, g.N, g.K, g.b_n, tn))
        return cudaErrorInvalidValue;
    // many 128 x 256 tiles (at least two per SM): the persistent CTAs with two accumulators
    const int sms = sm_count();
    const int tiles_n = (g.N + kPTN - 1) / kPTN, tiles = tiles_n * mt;
    if (tn == 256 && !g.accumulate && sms > 0 && tiles >= 2 * sms) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)sms);
        cfg.blockDim = dim3(192);
        cfg.dynamicSmemBytes = kPSmemBytes;
        cfg.stream = s;
        return cudaLaunchKernelEx(&cfg, mlp_gemm_tma_persistent, ma, mb, g, error_flag, tiles_n, tiles);
    }
    if (tn == 256)
        mlp_gemm_tma_kernel<256, 2><<<dim3((g.N + 255) / 256, mt), 128, TcShape<256, 2>::kSmemBytes, s>>>(
            ma, mb, g, error_flag);
    else
        mlp_gemm_tma_kernel<128, 3><<<dim3((g.N + 127) / 128, mt), 128, TcShape<128, 3>::kSmemBytes, s>>>(
            ma, mb, g, error_flag);
    return cudaGetLastError();
}

// y[c][r] = x[r][c] for a rows x cols BF16 matrix, through 32 x 32 shared-memory tiles.
__global__ void mlp_transpose_bf16_kernel(const __nv_bfloat16* __restrict__ x, int rows, int cols,
                                          __nv_bfloat16* __restrict__ y) {
    __shared__ __nv_bfloat16 t[32][33];
    const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int r = r0 + i, c = c0 + threadIdx.x;
        if (r < rows && c < cols) t[i][threadIdx.x] = x[(long long)r * cols + c];
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int c = c0 + i, r = r0 + threadIdx.x;
        if (r < rows && c < cols) y[(long long)c * rows + r] = t[threadIdx.x][i];
    }
}

cudaError_t mlp_transpose_bf16(const __nv_bfloat16* x, int rows, int cols, __nv_bfloat16* y, cudaStream_t s) {
    dim3 grid((cols + 31) / 32, (rows + 31) / 32), block(32, 8);
    mlp_transpose_bf16_kernel<<<grid, block, 0, s>>>(x, rows, cols, y);
    return cudaGetLastError();
}

}  // namespace mbg
