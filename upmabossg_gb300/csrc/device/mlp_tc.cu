// Surrogate GEMM on the fifth-generation tensor cores (tcgen05, sm_103a):
//   C[M x N] = alpha * A[M x K] . B[K x N] (+ bias[n]) (ReLU), A and B BF16, accumulation FP32 in
//   tensor memory (TMEM).
// One CTA (4 warps) computes a 128 x 128 tile. K is consumed in 64-wide blocks through a 3-stage
// shared-memory ring: every thread copies its 16-byte chunks of the A and B tiles with cp.async
// (zero-filled outside the matrices) into the canonical no-swizzle K-major layout (8 x 16-byte
// core matrices; core matrix (row group r, k group q) at byte (r * 8 + q) * 128), so the copies of
// the next two blocks are in flight while the tensor core works on the current one; one thread
// issues four 128x128x16 tcgen05.mma instructions per block and a tcgen05.commit to the stage's
// mbarrier, and a stage is refilled once its mbarrier has flipped. The epilogue reads the
// accumulator with tcgen05.ld (warp w owns TMEM lanes 32w .. 32w + 31 = tile rows), applies alpha,
// bias and ReLU and writes each thread's 32-column run with 16-byte stores. Requirements (checked
// by mlp_gemm_tc_supported): A rows K-contiguous (a_k == 1), B given transposed (element (k, n) at
// B[n * b_n + k], b_k == 1), K, a_m and b_n multiples of 8, 16-byte aligned A and B.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "mlp.h"

namespace mbg {

namespace {

constexpr int TM = 128, TK = 64;
constexpr int kTileBytesA = TM * TK * 2;  // 16 KiB A tile per stage
constexpr unsigned kSpinLimit = 1u << 26;  // bounded mbarrier waits

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

// Shared-memory matrix descriptor (tcgen05): start address, leading-dimension byte offset (between
// core matrices along K for K-major operands), stride byte offset (between 8-row groups), the
// descriptor version (1) at bits 46-47, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

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

// Starts the copies of rows r0 .. r0+127 (of `rows`), k0 .. k0+63 (of K) of a K-contiguous BF16
// matrix (row stride ld elements) into the core-matrix layout at shared address dst: chunk c
// (16 bytes) of the tile is row (c / 64) * 8 + c % 8, k group (c / 8) % 8, stored at byte 16 c, so
// a warp's 32 chunks cover 8 rows x 64 contiguous bytes. Chunks outside the matrix are zero-filled.
template <int ROWS>
__device__ __forceinline__ void load_tile_async(uint32_t dst, const __nv_bfloat16* src, long long ld, int r0,
                                                int rows, int k0, int K) {
#pragma unroll
    for (int i = 0; i < (ROWS * TK / 8) / 128; ++i) {
        const int c = (int)threadIdx.x + 128 * i;
        const int r = (c >> 6) * 8 + (c & 7);
        const int kq = (c >> 3) & 7;
        const int gr = r0 + r, gk = k0 + kq * 8;
        const bool in = gr < rows && gk < K;
        const __nv_bfloat16* p = in ? src + (long long)gr * ld + gk : src;
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst + 16u * c), "l"(p), "r"(in ? 16 : 0)
                     : "memory");
    }
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

}  // namespace

template <int TN, int STAGES>
__global__ void __launch_bounds__(128) mlp_gemm_tc_kernel(const GemmArgs g, unsigned* error_flag) {
    using S = TcShape<TN, STAGES>;
    constexpr int kStages = STAGES, kStageBytes = S::kStageBytes;
    extern __shared__ unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bar[kStages];
    __shared__ uint32_t tmem_slot;
    unsigned char* smem = reinterpret_cast<unsigned char*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const uint32_t sbase = smem_u32(smem);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.y * TM, n0 = blockIdx.x * TN;
    const long long a_base = g.a_row_offset ? (long long)(*g.a_row_offset) * g.a_m : 0;
    const __nv_bfloat16* A = g.A + a_base;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"(TN)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (threadIdx.x == 0) {
        for (int i = 0; i < kStages; ++i) mbar_init(&bar[i], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    const int nk = (g.K + TK - 1) / TK;
    // prologue: the first kStages - 1 blocks in flight (an empty group keeps the counting uniform)
#pragma unroll
    for (int st = 0; st < kStages - 1; ++st) {
        if (st < nk) {
            const uint32_t d = sbase + st * kStageBytes;
            load_tile_async<TM>(d, A, g.a_m, m0, g.M, st * TK, g.K);
            load_tile_async<TN>(d + kTileBytesA, g.B, g.b_n, n0, g.N, st * TK, g.K);
        }
        cp_async_commit();
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;

    bool ok = true;
    for (int kb = 0; kb < nk; ++kb) {
        const int stage = kb % kStages;
        // this thread's copies of block kb have landed (the later kStages - 2 groups may be pending)
        cp_async_wait<kStages - 2>();
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // -> visible to the tensor core
        __syncthreads();
        if (threadIdx.x == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int steps = (min(TK, g.K - kb * TK) + 15) / 16;
            const uint32_t a_addr = sbase + stage * kStageBytes, b_addr = a_addr + kTileBytesA;
            for (int s = 0; s < steps; ++s) {
                // K step s covers k groups 2s and 2s+1: 256 bytes further into each tile
                const uint64_t ad = smem_desc(a_addr + 256u * s, 128u, 1024u);
                const uint64_t bd = smem_desc(b_addr + 256u * s, 128u, 1024u);
                mma_bf16_tc(tmem, ad, bd, S::kIdesc, (kb > 0 || s > 0) ? 1u : 0u);
            }
            mma_commit(&bar[stage]);
        }
        // refill the stage of block kb - 1 with block kb + kStages - 1 once block kb - 1's MMAs are done
        const int next = kb + kStages - 1;
        if (next < nk) {
            const int ns = next % kStages;
            if (kb >= 1 && !mbar_wait(&bar[ns], (unsigned)(((kb - 1) / kStages) & 1))) ok = false;
            const uint32_t d = sbase + ns * kStageBytes;
            load_tile_async<TM>(d, A, g.a_m, m0, g.M, next * TK, g.K);
            load_tile_async<TN>(d + kTileBytesA, g.B, g.b_n, n0, g.N, next * TK, g.K);
        }
        cp_async_commit();
    }
    // every MMA of this thread is tracked by the last commit
    if (nk > 0 && !mbar_wait(&bar[(nk - 1) % kStages], (unsigned)(((nk - 1) / kStages) & 1))) ok = false;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!ok && lane == 0) atomicOr(error_flag, 1u);

    const int row = m0 + warp * 32 + lane;
    const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
    // 16-byte stores need 16-byte aligned rows
    const bool vec_b = g.Cb && (g.ldcb % 8) == 0 && ((uintptr_t)g.Cb & 15u) == 0;
    const bool vec_f = g.C && !g.accumulate && (g.ldc % 4) == 0 && ((uintptr_t)g.C & 15u) == 0;
#pragma unroll 1
    for (int c0 = 0; c0 < TN; c0 += 32) {
        float v[32];
        __syncwarp();  // tcgen05.ld is warp-collective: reconverge after the previous chunk's exits
        tmem_ld32(lane_addr + (uint32_t)c0, v);
        const int col0 = n0 + c0;
        if (!ok || row >= g.M || col0 >= g.N) continue;
#pragma unroll
        for (int i = 0; i < 32; ++i) {
            float x = g.alpha * (nk > 0 ? v[i] : 0.f);
            if (g.bias && col0 + i < g.N) x += __ldg(g.bias + col0 + i);
            if (g.relu) x = x > 0.f ? x : 0.f;
            v[i] = x;
        }
        const bool full = col0 + 32 <= g.N;
        if (g.Cb) {
            __nv_bfloat16* dst = g.Cb + (long long)row * g.ldcb + col0;
            if (full && vec_b) {
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
            if (full && vec_f) {
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

bool mlp_gemm_tc_supported(const GemmArgs& g) {
    auto aligned16 = [](const void* p) { return ((uintptr_t)p & 15u) == 0; };
    return g.M > 0 && g.N > 0 && g.K > 0 && g.a_k == 1 && g.b_k == 1 && g.K % 8 == 0 && g.a_m % 8 == 0 &&
           g.b_n % 8 == 0 && aligned16(g.A) && aligned16(g.B);
}

cudaError_t mlp_gemm_tc_configure() {
    cudaError_t e = cudaFuncSetAttribute(mlp_gemm_tc_kernel<128, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         TcShape<128, 3>::kSmemBytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(mlp_gemm_tc_kernel<256, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 TcShape<256, 2>::kSmemBytes);
    return e;
}

cudaError_t mlp_gemm_tc(const GemmArgs& g, unsigned* error_flag, cudaStream_t s) {
    if (!mlp_gemm_tc_supported(g)) return cudaErrorInvalidValue;
    const dim3 rows(1, (g.M + TM - 1) / TM);
    if (g.N > 128) {
        // 128 x 256 tiles: half the A traffic of 128-wide tiles, two CTAs per SM (96 KB ring each,
        // 256 TMEM columns each)
        mlp_gemm_tc_kernel<256, 2><<<dim3((g.N + 255) / 256, rows.y), 128, TcShape<256, 2>::kSmemBytes, s>>>(
            g, error_flag);
    } else {
        mlp_gemm_tc_kernel<128, 3><<<dim3((g.N + 127) / 128, rows.y), 128, TcShape<128, 3>::kSmemBytes, s>>>(
            g, error_flag);
    }
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
