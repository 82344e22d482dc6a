// Kernels of the learned surrogate: a BF16 multilayer perceptron (FP32 accumulation) that maps a
// sweep point's rate-scaling parameters to the output-state distribution of the final window.
// Here: the general mma.sync product, softmax / cross-entropy, ensemble statistics and small
// helpers; the training step's member-batched products, gather and Adam are in mlp_train.cu, the
// tcgen05 forward product in mlp_tc.cu; the host side is surrogate.cpp.
//
// GEMM: C[M x N] = A[M x K] . B[K x N] with arbitrary element strides for A and B (the forward
// product when the tcgen05 path is off or does not apply). Tiles of 64 x 64 x 32 are staged in
// shared memory as BF16 and multiplied with the m16n8k16 BF16 tensor-core instruction; the
// epilogue adds a bias, applies ReLU and stores FP32 and/or BF16.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "mlp.h"

namespace mbg {

namespace {

constexpr int BM = 64, BN = 64, BK = 32, PAD = 8;

__device__ __forceinline__ unsigned pack2(const __nv_bfloat16* p) { return *reinterpret_cast<const unsigned*>(p); }

__device__ __forceinline__ void mma_bf16(float (&c)[4], const unsigned (&a)[4], const unsigned (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

}  // namespace

__global__ void __launch_bounds__(128) mlp_gemm_kernel(const GemmArgs g) {
    __shared__ __align__(16) __nv_bfloat16 As[BM][BK + PAD];  // [m][k]
    __shared__ __align__(16) __nv_bfloat16 Bs[BN][BK + PAD];  // [n][k]
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    const int gq = lane >> 2, tq = lane & 3;
    const long long a_base = g.a_row_offset ? (long long)(*g.a_row_offset) * g.a_m : 0;
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.f;

    for (int k0 = 0; k0 < g.K; k0 += BK) {
        for (int idx = tid; idx < BM * BK; idx += 128) {
            const int m = idx / BK, k = idx % BK;
            const int gm = m0 + m, gk = k0 + k;
            As[m][k] = (gm < g.M && gk < g.K) ? g.A[a_base + gm * g.a_m + (long long)gk * g.a_k] : __float2bfloat16(0.f);
        }
        for (int idx = tid; idx < BN * BK; idx += 128) {
            const int n = idx / BK, k = idx % BK;
            const int gn = n0 + n, gk = k0 + k;
            Bs[n][k] = (gn < g.N && gk < g.K) ? g.B[(long long)gk * g.b_k + (long long)gn * g.b_n] : __float2bfloat16(0.f);
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; kk += 16) {
            unsigned af[2][4], bf[4][2];
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const int r = wm + i * 16 + gq;
                af[i][0] = pack2(&As[r][kk + 2 * tq]);
                af[i][1] = pack2(&As[r + 8][kk + 2 * tq]);
                af[i][2] = pack2(&As[r][kk + 2 * tq + 8]);
                af[i][3] = pack2(&As[r + 8][kk + 2 * tq + 8]);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int c = wn + j * 8 + gq;
                bf[j][0] = pack2(&Bs[c][kk + 2 * tq]);
                bf[j][1] = pack2(&Bs[c][kk + 2 * tq + 8]);
            }
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], af[i], bf[j]);
        }
        __syncthreads();
    }
    // epilogue: element (row, col) of fragment register r: row = gq (+8 for r >= 2), col = 2 tq (+1)
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const int row = m0 + wm + i * 16 + gq + (r >= 2 ? 8 : 0);
                const int col = n0 + wn + j * 8 + 2 * tq + (r & 1);
                if (row >= g.M || col >= g.N) continue;
                float v = g.alpha * acc[i][j][r];
                if (g.bias) v += g.bias[col];
                if (g.relu) v = v > 0.f ? v : 0.f;
                if (g.C) {
                    float* dst = g.C + (long long)row * g.ldc + col;
                    *dst = g.accumulate ? *dst + v : v;
                }
                if (g.Cb) g.Cb[(long long)row * g.ldcb + col] = __float2bfloat16(v);
            }
}

cudaError_t mlp_gemm(const GemmArgs& g, cudaStream_t s) {
    dim3 grid((g.N + BN - 1) / BN, (g.M + BM - 1) / BM);
    mlp_gemm_kernel<<<grid, 128, 0, s>>>(g);
    return cudaGetLastError();
}

// One warp per row; blockIdx.y selects a stacked [rows x cols] block (member), whose loss goes to
// loss[blockIdx.y].
__global__ void mlp_softmax_xent_kernel(const float* __restrict__ logits, int rows, int cols,
                                        const float* __restrict__ target, float scale, float* __restrict__ probs,
                                        __nv_bfloat16* __restrict__ dlogits, float* __restrict__ loss) {
    const int lane = threadIdx.x & 31;
    const int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (row >= rows) return;
    const long long zo = (long long)blockIdx.y * rows * cols;
    logits += zo;
    if (target) target += zo;
    if (probs) probs += zo;
    if (dlogits) dlogits += zo;
    if (loss) loss += blockIdx.y;
    const float* z = logits + (long long)row * cols;
    float mx = -3.4e38f;
    for (int c = lane; c < cols; c += 32) mx = fmaxf(mx, z[c]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    float sum = 0.f;
    for (int c = lane; c < cols; c += 32) sum += __expf(z[c] - mx);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    const float lse = mx + __logf(sum);
    float l = 0.f;
    for (int c = lane; c < cols; c += 32) {
        const float p = __expf(z[c] - lse);
        if (probs) probs[(long long)row * cols + c] = p;
        if (target) {
            const float y = target[(long long)row * cols + c];
            if (dlogits) dlogits[(long long)row * cols + c] = __float2bfloat16((p - y) * scale);
            if (y > 0.f) l -= y * (z[c] - lse);
        }
    }
    if (loss && target) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
        if (lane == 0) atomicAdd(loss, l);
    }
}

cudaError_t mlp_softmax_xent(const float* logits, int rows, int cols, const float* target, float scale,
                             float* probs, __nv_bfloat16* dlogits, float* loss, cudaStream_t s) {
    const int warps = 8;
    mlp_softmax_xent_kernel<<<(rows + warps - 1) / warps, warps * 32, 0, s>>>(logits, rows, cols, target, scale,
                                                                               probs, dlogits, loss);
    return cudaGetLastError();
}

cudaError_t mlp_softmax_xent_members(const float* logits, int rows, int cols, int members, const float* target,
                                     float scale, __nv_bfloat16* dlogits, float* loss, cudaStream_t s) {
    const int warps = 8;
    mlp_softmax_xent_kernel<<<dim3((rows + warps - 1) / warps, members), warps * 32, 0, s>>>(
        logits, rows, cols, target, scale, nullptr, dlogits, loss);
    return cudaGetLastError();
}




__global__ void mlp_step_advance_kernel(int* t) { *t += 1; }

cudaError_t mlp_step_advance(int* t, cudaStream_t s) {
    mlp_step_advance_kernel<<<1, 1, 0, s>>>(t);
    return cudaGetLastError();
}

__global__ void mlp_to_bf16_kernel(const float* __restrict__ x, __nv_bfloat16* __restrict__ y, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        y[i] = __float2bfloat16(x[i]);
}

cudaError_t mlp_to_bf16(const float* x, __nv_bfloat16* y, long long n, cudaStream_t s) {
    mlp_to_bf16_kernel<<<512, 256, 0, s>>>(x, y, n);
    return cudaGetLastError();
}

// One warp per row.
__global__ void mlp_ensemble_stats_kernel(const float* __restrict__ probs, int members, int rows, int cols,
                                          float* __restrict__ mean, float* __restrict__ spread) {
    const int lane = threadIdx.x & 31;
    const int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (row >= rows) return;
    const long long stride = (long long)rows * cols;
    const float inv = 1.f / (float)members;
    for (int c = lane; c < cols; c += 32) {
        float s = 0.f;
        for (int e = 0; e < members; ++e) s += probs[e * stride + (long long)row * cols + c];
        mean[(long long)row * cols + c] = s * inv;
    }
    __syncwarp();
    float worst = 0.f;
    for (int e = 0; e < members; ++e) {
        float tv = 0.f;
        for (int c = lane; c < cols; c += 32)
            tv += fabsf(probs[e * stride + (long long)row * cols + c] - mean[(long long)row * cols + c]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) tv += __shfl_xor_sync(0xffffffffu, tv, o);
        worst = fmaxf(worst, 0.5f * tv);
    }
    if (lane == 0) spread[row] = worst;
}

__global__ void mlp_gather_column_kernel(const float* __restrict__ x, int rows, int cols, int column,
                                         float* __restrict__ y) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < rows) y[r] = x[(size_t)r * cols + column];
}

cudaError_t mlp_gather_column(const float* x, int rows, int cols, int column, float* y, cudaStream_t s) {
    if (rows <= 0) return cudaSuccess;
    mlp_gather_column_kernel<<<(rows + 255) / 256, 256, 0, s>>>(x, rows, cols, column, y);
    return cudaGetLastError();
}

cudaError_t mlp_ensemble_stats(const float* probs, int members, int rows, int cols, float* mean, float* spread,
                               cudaStream_t s) {
    mlp_ensemble_stats_kernel<<<(rows + 7) / 8, 256, 0, s>>>(probs, members, rows, cols, mean, spread);
    return cudaGetLastError();
}


}  // namespace mbg
