// Surrogate GEMM on the fifth-generation tensor cores (tcgen05, sm_103a):
//   C[M x N] = alpha * A[M x K] . B[K x N] (+ bias[n]) (ReLU), A and B BF16, accumulation FP32 in
//   tensor memory (TMEM).
// One CTA (4 warps) computes a 128 x 128 tile. Per 64-wide K block, the 128 threads stage the A
// and B tiles into shared memory in the canonical no-swizzle K-major layout (8 x 16-byte core
// matrices; core matrix (row group r, k group q) at byte (r * 8 + q) * 128), two buffers deep, and
// one thread issues four 128x128x16 tcgen05.mma instructions and a tcgen05.commit to the buffer's
// mbarrier; the buffer is refilled once that mbarrier has flipped. The epilogue reads the 128 x 128
// FP32 accumulator with tcgen05.ld (warp w owns TMEM lanes 32w .. 32w + 31 = tile rows) and applies
// alpha, bias and ReLU. Requirements (checked by mlp_gemm_tc): A rows K-contiguous (a_k == 1),
// B given transposed (element (k, n) at B[n * b_n + k], b_k == 1), K, a_m and b_n multiples of 8,
// 16-byte aligned A and B.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "mlp.h"

namespace mbg {

namespace {

constexpr int TM = 128, TN = 128, TK = 64;
constexpr int kTileBytes = TM * TK * 2;            // 16 KiB per operand tile
constexpr int kSmemBytes = 4 * kTileBytes + 1024;  // A0 B0 A1 B1 + alignment slack
constexpr unsigned kSpinLimit = 1u << 26;          // bounded mbarrier waits

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor (tcgen05): start address, leading-dimension byte offset (between
// core matrices along K for K-major operands), stride byte offset (between 8-row groups), the
// descriptor version (1) at bits 46-47, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), BF16 A and B (bits 7-9 and
// 10-12 = 1), both K-major (bits 15, 16 = 0), N / 8 at bits 17-22, M / 16 at bits 24-28.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TN >> 3) << 17) |
                            ((uint32_t)(TM >> 4) << 24);

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

__device__ __forceinline__ void mma_bf16_tc(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate)
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

// Stages rows r0 .. r0+127 (of `rows`), k0 .. k0+63 (of K) of a K-contiguous BF16 matrix (row
// stride ld elements) into the core-matrix layout at dst: chunk c (16 bytes) of the tile is row
// (c / 64) * 8 + c % 8, k group (c / 8) % 8, stored at byte 16 c. Out-of-range chunks are zero.
__device__ __forceinline__ void stage_tile(unsigned char* dst, const __nv_bfloat16* src, long long ld, int r0,
                                           int rows, int k0, int K) {
#pragma unroll
    for (int i = 0; i < (TM * TK / 8) / 128; ++i) {
        const int c = (int)threadIdx.x + 128 * i;
        const int r = (c >> 6) * 8 + (c & 7);
        const int kq = (c >> 3) & 7;
        const int gr = r0 + r, gk = k0 + kq * 8;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (gr < rows && gk < K) v = __ldg(reinterpret_cast<const uint4*>(src + (long long)gr * ld + gk));
        *reinterpret_cast<uint4*>(dst + 16 * c) = v;
    }
}

}  // namespace

__global__ void __launch_bounds__(128) mlp_gemm_tc_kernel(const GemmArgs g, unsigned* error_flag) {
    extern __shared__ unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ uint32_t tmem_slot;
    unsigned char* smem = reinterpret_cast<unsigned char*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.y * TM, n0 = blockIdx.x * TN;
    const long long a_base = g.a_row_offset ? (long long)(*g.a_row_offset) * g.a_m : 0;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"(TN)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;

    bool ok = true;
    const int nk = (g.K + TK - 1) / TK;
    for (int kb = 0; kb < nk; ++kb) {
        const int buf = kb & 1;
        // the MMAs that last read this buffer (K block kb - 2) must be done before it is refilled
        if (kb >= 2 && !mbar_wait(&bar[buf], (unsigned)(((kb - 2) >> 1) & 1))) ok = false;
        const int k0 = kb * TK;
        unsigned char* ta = smem + (2 * buf) * kTileBytes;  // buffer buf: A tile, then B tile
        unsigned char* tb = ta + kTileBytes;
        stage_tile(ta, g.A + a_base, g.a_m, m0, g.M, k0, g.K);
        stage_tile(tb, g.B, g.b_n, n0, g.N, k0, g.K);
        // generic-proxy stores -> visible to the tensor core's async proxy
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (threadIdx.x == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int steps = (min(TK, g.K - k0) + 15) / 16;
            const uint32_t a_addr = smem_u32(ta), b_addr = smem_u32(tb);
            for (int s = 0; s < steps; ++s) {
                // K step s covers k groups 2s and 2s+1: 256 bytes further into each tile
                const uint64_t ad = smem_desc(a_addr + 256u * s, 128u, 1024u);
                const uint64_t bd = smem_desc(b_addr + 256u * s, 128u, 1024u);
                mma_bf16_tc(tmem, ad, bd, (kb > 0 || s > 0) ? 1u : 0u);
            }
            mma_commit(&bar[buf]);
        }
    }
    // every MMA of this thread is tracked by the last commit
    if (nk > 0 && !mbar_wait(&bar[(nk - 1) & 1], (unsigned)(((nk - 1) >> 1) & 1))) ok = false;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!ok && lane == 0) atomicOr(error_flag, 1u);

    const int row = m0 + warp * 32 + lane;
    const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
    for (int c0 = 0; c0 < TN; c0 += 32) {
        float v[32];
        tmem_ld32(lane_addr + (uint32_t)c0, v);
        if (!ok || row >= g.M) continue;
#pragma unroll
        for (int i = 0; i < 32; ++i) {
            const int col = n0 + c0 + i;
            if (col >= g.N) break;
            float x = g.alpha * (nk > 0 ? v[i] : 0.f);
            if (g.bias) x += g.bias[col];
            if (g.relu) x = x > 0.f ? x : 0.f;
            if (g.C) {
                float* dst = g.C + (long long)row * g.ldc + col;
                *dst = g.accumulate ? *dst + x : x;
            }
            if (g.Cb) g.Cb[(long long)row * g.ldcb + col] = __float2bfloat16(x);
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

cudaError_t mlp_gemm_tc(const GemmArgs& g, unsigned* error_flag, cudaStream_t s) {
    if (!mlp_gemm_tc_supported(g)) return cudaErrorInvalidValue;
    static bool configured = false;
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(mlp_gemm_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             kSmemBytes);
        if (e != cudaSuccess) return e;
        configured = true;
    }
    dim3 grid((g.N + TN - 1) / TN, (g.M + TM - 1) / TM);
    mlp_gemm_tc_kernel<<<grid, 128, kSmemBytes, s>>>(g, error_flag);
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
