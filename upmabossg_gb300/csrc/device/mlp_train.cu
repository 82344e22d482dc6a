// Member-batched kernels of one surrogate training step (host side: Surrogate::train and
// Surrogate::gradients in surrogate.cpp). Every launch covers all ensemble members at once
// (blockIdx.z selects the member), so a step of the whole ensemble is one short chain of launches
// replayed from a CUDA graph.
//
// The products of a minibatch are small (64 x 512 x 512): they run on mma.sync m16n8k16 BF16
// tiles of 64 x 64 x 32 staged in shared memory through registers with 16-byte loads along the
// operand's contiguous dimension, the fragments read with ldmatrix (transposed for an operand
// that is contiguous along M or N). So the forward product reads W [in][out] as stored and the
// weight gradient reads the activations and output gradients without a transpose. Epilogues fuse
// the bias and ReLU (forward), the ReLU mask of the layer below (data gradient) and, in the weight
// gradient, the bias gradient (column sums of the output gradient, in row order).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "mlp.h"

namespace mbg {

namespace {

constexpr int TBM = 64, TBN = 64, TBK = 32;
constexpr int PITCH_K = TBK + 8;   // [mn][k] tiles: 80-byte rows
constexpr int PITCH_MN = TBM + 8;  // [k][mn] tiles: 144-byte rows
constexpr int TILE_ELEMS = TBM * PITCH_K > TBK * PITCH_MN ? TBM * PITCH_K : TBK * PITCH_MN;

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void ldsm_x4(unsigned (&r)[4], const __nv_bfloat16* p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(smem_addr(p))
                 : "memory");
}

__device__ __forceinline__ void ldsm_x4_trans(unsigned (&r)[4], const __nv_bfloat16* p) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(smem_addr(p))
                 : "memory");
}

__device__ __forceinline__ void mma16816(float (&c)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Chunk c (0..255) of the 64 x 32 tile of an operand X with logical element (p, k), p along M or
// N (extent P), k along K: eight consecutive elements along the contiguous dimension. KC: element
// (p, k) at x[p * ld + k] (K contiguous), otherwise at x[k * ld + p]. Outside the operand: zeros.
template <bool KC>
__device__ __forceinline__ uint4 load_chunk(const __nv_bfloat16* x, long long ld, int P, int K, int p0, int k0,
                                            int c, bool vec) {
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    int p, k;
    if (KC) {
        p = p0 + (c >> 2);
        k = k0 + (c & 3) * 8;
        if (p >= P || k >= K) return v;
    } else {
        k = k0 + (c >> 3);
        p = p0 + (c & 7) * 8;
        if (k >= K || p >= P) return v;
    }
    const __nv_bfloat16* src = KC ? x + (long long)p * ld + k : x + (long long)k * ld + p;
    const int left = KC ? K - k : P - p;  // elements of the chunk inside the operand
    if (vec && left >= 8) return __ldg(reinterpret_cast<const uint4*>(src));
    union {
        uint4 u;
        __nv_bfloat16 h[8];
    } e;
#pragma unroll
    for (int j = 0; j < 8; ++j) e.h[j] = j < left ? src[j] : __float2bfloat16(0.f);
    return e.u;
}

template <bool KC>
__device__ __forceinline__ void store_chunk(__nv_bfloat16* tile, int c, uint4 v) {
    __nv_bfloat16* dst = KC ? tile + (c >> 2) * PITCH_K + (c & 3) * 8 : tile + (c >> 3) * PITCH_MN + (c & 7) * 8;
    *reinterpret_cast<uint4*>(dst) = v;
}

// A fragment (16 x 16 at rows m, columns kk) of a tile: [m][k] (KC) or [k][m].
template <bool KC>
__device__ __forceinline__ void frag_a(unsigned (&a)[4], const __nv_bfloat16* tile, int m, int kk, int lane) {
    if (KC) {
        ldsm_x4(a, tile + (m + (lane & 15)) * PITCH_K + kk + (lane >> 4) * 8);
    } else {
        const int j = lane >> 3, r = lane & 7;
        ldsm_x4_trans(a, tile + (kk + 8 * (j >> 1) + r) * PITCH_MN + m + 8 * (j & 1));
    }
}

// B fragments of two n8 tiles (columns n..n+15, rows kk..kk+15) of a tile: [n][k] (KC) or [k][n].
// b[0], b[1]: first n8 tile; b[2], b[3]: second.
template <bool KC>
__device__ __forceinline__ void frag_b2(unsigned (&b)[4], const __nv_bfloat16* tile, int n, int kk, int lane) {
    const int j = lane >> 3, r = lane & 7;
    if (KC) ldsm_x4(b, tile + (n + 8 * (j >> 1) + r) * PITCH_K + kk + 8 * (j & 1));
    else ldsm_x4_trans(b, tile + (kk + 8 * (j & 1) + r) * PITCH_MN + n + 8 * (j >> 1));
}

// Column sum over the tile's 32 rows of column `col` of a B tile (for the bias gradient).
template <bool KC>
__device__ __forceinline__ float tile_col_sum(const __nv_bfloat16* tile, int col) {
    float s = 0.f;
#pragma unroll 8
    for (int k = 0; k < TBK; ++k) s += __bfloat162float(KC ? tile[col * PITCH_K + k] : tile[k * PITCH_MN + col]);
    return s;
}

}  // namespace

template <bool A_KC, bool B_KC, int EPI>
__global__ void __launch_bounds__(128) mlp_member_gemm_kernel(const MemberGemm g) {
    __shared__ __align__(16) __nv_bfloat16 sa[2][TILE_ELEMS];
    __shared__ __align__(16) __nv_bfloat16 sb[2][TILE_ELEMS];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int z = blockIdx.z;
    const int m0 = blockIdx.y * TBM, n0 = blockIdx.x * TBN;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    const __nv_bfloat16* A = g.A + (long long)z * g.a_z;
    const __nv_bfloat16* B = g.B + (long long)z * g.b_z;
    const bool bias_grad = EPI == kMemberGemmF32 && g.gb != nullptr && blockIdx.y == 0;
    float colsum = 0.f;

    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.f;

    const int kt_n = (g.K + TBK - 1) / TBK;
    uint4 ra[2], rb[2];
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        ra[i] = load_chunk<A_KC>(A, g.lda, g.M, g.K, m0, 0, tid + 128 * i, g.vec_a);
        rb[i] = load_chunk<B_KC>(B, g.ldb, g.N, g.K, n0, 0, tid + 128 * i, g.vec_b);
    }
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        store_chunk<A_KC>(sa[0], tid + 128 * i, ra[i]);
        store_chunk<B_KC>(sb[0], tid + 128 * i, rb[i]);
    }
    __syncthreads();
    for (int kt = 0; kt < kt_n; ++kt) {
        const int cur = kt & 1;
        if (kt + 1 < kt_n) {
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                ra[i] = load_chunk<A_KC>(A, g.lda, g.M, g.K, m0, (kt + 1) * TBK, tid + 128 * i, g.vec_a);
                rb[i] = load_chunk<B_KC>(B, g.ldb, g.N, g.K, n0, (kt + 1) * TBK, tid + 128 * i, g.vec_b);
            }
        }
#pragma unroll
        for (int kk = 0; kk < TBK; kk += 16) {
            unsigned af[2][4], bf[2][4];
            frag_a<A_KC>(af[0], sa[cur], wm, kk, lane);
            frag_a<A_KC>(af[1], sa[cur], wm + 16, kk, lane);
            frag_b2<B_KC>(bf[0], sb[cur], wn, kk, lane);
            frag_b2<B_KC>(bf[1], sb[cur], wn + 16, kk, lane);
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) mma16816(acc[i][j], af[i], bf[j >> 1][2 * (j & 1)], bf[j >> 1][2 * (j & 1) + 1]);
        }
        if (bias_grad && tid < TBN) colsum += tile_col_sum<B_KC>(sb[cur], tid);
        if (kt + 1 < kt_n) {
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                store_chunk<A_KC>(sa[cur ^ 1], tid + 128 * i, ra[i]);
                store_chunk<B_KC>(sb[cur ^ 1], tid + 128 * i, rb[i]);
            }
        }
        __syncthreads();
    }
    if (bias_grad && tid < TBN && n0 + tid < g.N) g.gb[(long long)z * g.gb_z + n0 + tid] = colsum;

    // element (row, col) of accumulator register r: row = gq (+8 for r >= 2), col = 2 tq (+1 for odd r)
    const int gq = lane >> 2, tq = lane & 3;
    const float* bias = g.bias ? g.bias + (long long)z * g.bias_z : nullptr;
    const __nv_bfloat16* act = g.act ? g.act + (long long)z * g.act_z : nullptr;
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const int row = m0 + wm + 16 * i + gq + (r >= 2 ? 8 : 0);
                const int col = n0 + wn + 8 * j + 2 * tq + (r & 1);
                if (row >= g.M || col >= g.N) continue;
                float v = acc[i][j][r];
                const long long o = (long long)z * g.c_z + (long long)row * g.ldc + col;
                if (EPI == kMemberGemmBiasReluBf16) {
                    v += bias[col];
                    g.Cb[o] = __float2bfloat16(v > 0.f ? v : 0.f);
                } else if (EPI == kMemberGemmBiasF32) {
                    g.C[o] = v + bias[col];
                } else if (EPI == kMemberGemmMaskBf16) {
                    const bool on = __bfloat162float(act[(long long)row * g.ldact + col]) > 0.f;
                    g.Cb[o] = __float2bfloat16(on ? v : 0.f);
                } else {
                    g.C[o] = v;
                }
            }
}

cudaError_t mlp_member_gemm(const MemberGemm& g, int members, int epi, bool a_kc, bool b_kc, cudaStream_t s) {
    if (members < 1 || g.M < 1 || g.N < 1 || g.K < 1) return cudaErrorInvalidValue;
    const dim3 grid((g.N + TBN - 1) / TBN, (g.M + TBM - 1) / TBM, members);
    if (a_kc && !b_kc && epi == kMemberGemmBiasReluBf16)
        mlp_member_gemm_kernel<true, false, kMemberGemmBiasReluBf16><<<grid, 128, 0, s>>>(g);
    else if (a_kc && !b_kc && epi == kMemberGemmBiasF32)
        mlp_member_gemm_kernel<true, false, kMemberGemmBiasF32><<<grid, 128, 0, s>>>(g);
    else if (a_kc && b_kc && epi == kMemberGemmMaskBf16)
        mlp_member_gemm_kernel<true, true, kMemberGemmMaskBf16><<<grid, 128, 0, s>>>(g);
    else if (!a_kc && !b_kc && epi == kMemberGemmF32)
        mlp_member_gemm_kernel<false, false, kMemberGemmF32><<<grid, 128, 0, s>>>(g);
    else
        return cudaErrorInvalidValue;
    return cudaGetLastError();
}

// Minibatch (*t mod steps) of every member: member e takes rows perm[e * n + (*t mod steps) * rows + r]
// of x (cols_x per row, to BF16) and y (cols_y per row).
__global__ void mlp_member_gather_kernel(const float* __restrict__ x, int cols_x, const float* __restrict__ y,
                                         int cols_y, const int* __restrict__ perm, long long n,
                                         const int* __restrict__ t, int steps, int rows, int members,
                                         __nv_bfloat16* __restrict__ xb, float* __restrict__ yt) {
    const long long base = (long long)(*t % steps) * rows;
    const int cols = cols_x + cols_y;
    const long long total = (long long)members * rows * cols;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const long long er = i / cols;  // member * rows + row
        const int c = (int)(i - er * cols);
        const int e = (int)(er / rows), r = (int)(er - (long long)e * rows);
        const long long src = perm[e * n + base + r];
        if (c < cols_x) xb[er * cols_x + c] = __float2bfloat16(x[src * cols_x + c]);
        else yt[er * cols_y + (c - cols_x)] = y[src * cols_y + (c - cols_x)];
    }
}

cudaError_t mlp_member_gather(const float* x, int cols_x, const float* y, int cols_y, const int* perm, long long n,
                              const int* t, int steps, int rows, int members, __nv_bfloat16* xb, float* yt,
                              cudaStream_t s) {
    mlp_member_gather_kernel<<<256, 256, 0, s>>>(x, cols_x, y, cols_y, perm, n, t, steps, rows, members, xb, yt);
    return cudaGetLastError();
}

// Adam over the parameter blocks of every member (member e: elements [e * per, (e + 1) * per)),
// with member e's learning rate and bias corrections for step *t read from
// sched[3 * (e * sched_len + *t) ..].
__global__ void mlp_member_adam_kernel(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                                       float* __restrict__ v, __nv_bfloat16* __restrict__ wb, long long per,
                                       int members, const float* __restrict__ sched, long long sched_len,
                                       const int* __restrict__ t, float beta1, float beta2, float eps) {
    const int k = *t;
    const long long n = per * members;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const long long e = i / per;
        const float* sc = sched + 3 * (e * sched_len + k);
        const float lr = sc[0], c1 = sc[1], c2 = sc[2];
        const float gi = g[i];
        const float mi = beta1 * m[i] + (1.f - beta1) * gi;
        const float vi = beta2 * v[i] + (1.f - beta2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float wi = w[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
        w[i] = wi;
        wb[i] = __float2bfloat16(wi);
    }
}

cudaError_t mlp_member_adam(float* w, const float* g, float* m, float* v, __nv_bfloat16* wb, long long per,
                            int members, const float* sched, long long sched_len, const int* t, float beta1,
                            float beta2, float eps, cudaStream_t s) {
    mlp_member_adam_kernel<<<1024, 256, 0, s>>>(w, g, m, v, wb, per, members, sched, sched_len, t, beta1, beta2, eps);
    return cudaGetLastError();
}

}  // namespace mbg
