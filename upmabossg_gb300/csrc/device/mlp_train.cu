// Member-batched kernels of one surrogate training step (host side: Surrogate::train and
// Surrogate::gradients in surrogate.cpp). Every launch covers all ensemble members at once
// (blockIdx.z selects the member), so a step of the whole ensemble is one short chain of launches
// replayed from a CUDA graph.
//
// The products of a minibatch are small (64 x 512 x 512): they run on mma.sync m16n8k16 BF16
// tiles of 64 x 64 x 32 staged in shared memory with 16-byte copies along the operand's contiguous
// dimension (a 4-stage cp.async ring when both operands allow 16-byte copies, so that the K loop of
// a tile keeps three tiles of loads in flight; otherwise element-wise loads staged through
// registers), the fragments read with ldmatrix (transposed for an operand that is contiguous
// along M or N). So the forward product reads W [in][out] as stored and the weight gradient reads
// the activations and output gradients without a transpose. A product with a long K loop and few
// output tiles (64 rows x 512 columns over K = 512: 8 tiles a member) splits K over the four CTAs
// of a thread-block cluster, which add their partial tiles through distributed shared memory
// before the leader's epilogue. Epilogues fuse the bias and ReLU (forward), the ReLU mask of the
// layer below (data gradient) and, in the weight gradient, the bias gradient (column sums of the
// output gradient, in row order).
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
__device__ __forceinline__ __nv_bfloat16* chunk_dst(__nv_bfloat16* tile, int c) {
    return KC ? tile + (c >> 2) * PITCH_K + (c & 3) * 8 : tile + (c >> 3) * PITCH_MN + (c & 7) * 8;
}

template <bool KC>
__device__ __forceinline__ void store_chunk(__nv_bfloat16* tile, int c, uint4 v) {
    *reinterpret_cast<uint4*>(chunk_dst<KC>(tile, c)) = v;
}

// The same chunk as load_chunk, copied by cp.async (16-byte aligned chunks only): the bytes inside
// the operand are read, the rest of the 16 bytes zero-filled (a chunk wholly outside reads nothing
// and points at x itself).
template <bool KC>
__device__ __forceinline__ void copy_chunk(__nv_bfloat16* tile, int c, const __nv_bfloat16* x, long long ld, int P,
                                           int K, int p0, int k0) {
    int p, k;
    if (KC) {
        p = p0 + (c >> 2);
        k = k0 + (c & 3) * 8;
    } else {
        k = k0 + (c >> 3);
        p = p0 + (c & 7) * 8;
    }
    const __nv_bfloat16* src = x;
    unsigned bytes = 0u;
    if (p < P && k < K) {
        src = KC ? x + (long long)p * ld + k : x + (long long)k * ld + p;
        const int left = KC ? K - k : P - p;
        bytes = left >= 8 ? 16u : 2u * (unsigned)left;
    }
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(smem_addr(chunk_dst<KC>(tile, c))), "l"(src),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ unsigned cluster_rank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;\n" : "=r"(r));
    return r;
}
// Every thread of every CTA of the cluster: arrive (releasing its shared-memory writes), then wait.
__device__ __forceinline__ void cluster_sync() {
    asm volatile("barrier.cluster.arrive.release.aligned;\nbarrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}
// Four floats at the shared-memory address `local` of this CTA, read from CTA `rank` of the cluster.
__device__ __forceinline__ float4 ld_cluster_f4(const void* local, unsigned rank) {
    unsigned remote;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;\n" : "=r"(remote) : "r"(smem_addr(local)), "r"(rank));
    float4 v;
    asm volatile("ld.shared::cluster.v4.f32 {%0,%1,%2,%3}, [%4];\n"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "r"(remote)
                 : "memory");
    return v;
}

__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
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

// KS > 1: launched in clusters of KS CTAs along x (blockIdx.x = tile column * KS + rank); CTA
// rank r runs k-tiles [r * per, (r + 1) * per) of the product and rank 0 sums the partial tiles
// and writes the result (no bias gradient in this form).
template <bool A_KC, bool B_KC, int EPI, bool ASYNC, int KS>
__global__ void __launch_bounds__(128) mlp_member_gemm_kernel(const MemberGemm g) {
    constexpr int STAGES = ASYNC ? 4 : 2;
    constexpr int STAGE_ELEMS = 2 * TILE_ELEMS;  // A tile, then B tile
    static_assert(KS == 1 || STAGES * STAGE_ELEMS * 2 >= 128 * 32 * 4, "partial tiles reuse the staging buffers");
    static_assert(KS == 1 || EPI != kMemberGemmF32, "the split form has no bias gradient");
    __shared__ __align__(128) __nv_bfloat16 stage_buf[STAGES * STAGE_ELEMS];
    auto sa = [&](int st) { return stage_buf + st * STAGE_ELEMS; };
    auto sb = [&](int st) { return stage_buf + st * STAGE_ELEMS + TILE_ELEMS; };
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int z = blockIdx.z;
    const int ks = KS > 1 ? (int)cluster_rank() : 0;
    const int m0 = blockIdx.y * TBM, n0 = (int)(blockIdx.x / KS) * TBN;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    const __nv_bfloat16* A = g.A + (long long)z * g.a_z;
    const __nv_bfloat16* B = g.B + (long long)z * g.b_z;
    const bool bias_grad = KS == 1 && EPI == kMemberGemmF32 && g.gb != nullptr && blockIdx.y == 0;
    float colsum = 0.f;

    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.f;

    auto mma_tile = [&](const __nv_bfloat16* ta, const __nv_bfloat16* tb) {
#pragma unroll
        for (int kk = 0; kk < TBK; kk += 16) {
            unsigned af[2][4], bf[2][4];
            frag_a<A_KC>(af[0], ta, wm, kk, lane);
            frag_a<A_KC>(af[1], ta, wm + 16, kk, lane);
            frag_b2<B_KC>(bf[0], tb, wn, kk, lane);
            frag_b2<B_KC>(bf[1], tb, wn + 16, kk, lane);
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    mma16816(acc[i][j], af[i], bf[j >> 1][2 * (j & 1)], bf[j >> 1][2 * (j & 1) + 1]);
        }
        if (bias_grad && tid < TBN) colsum += tile_col_sum<B_KC>(tb, tid);
    };

    const int kt_all = (g.K + TBK - 1) / TBK;
    const int per = (kt_all + KS - 1) / KS;
    const int kt0 = ks * per;  // this CTA's first k-tile
    const int kt_n = kt_all - kt0 < per ? (kt_all - kt0 > 0 ? kt_all - kt0 : 0) : per;
    if (ASYNC) {
        // ring of STAGES k-tiles: tile kt in stage kt % STAGES, STAGES - 1 tiles of copies ahead
        auto issue = [&](int kt) {
            __nv_bfloat16* ta = sa(kt % STAGES);
            __nv_bfloat16* tb = sb(kt % STAGES);
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                copy_chunk<A_KC>(ta, tid + 128 * i, A, g.lda, g.M, g.K, m0, (kt0 + kt) * TBK);
                copy_chunk<B_KC>(tb, tid + 128 * i, B, g.ldb, g.N, g.K, n0, (kt0 + kt) * TBK);
            }
        };
#pragma unroll
        for (int s = 0; s < STAGES - 1; ++s) {
            if (s < kt_n) issue(s);
            cp_commit();  // a group per stage, empty past the end: the wait count stays uniform
        }
        for (int kt = 0; kt < kt_n; ++kt) {
            cp_wait<STAGES - 2>();  // this thread's copies of tile kt landed
            __syncthreads();        // everyone's did, and every thread is done with tile kt - 1
            if (kt + STAGES - 1 < kt_n) issue(kt + STAGES - 1);
            cp_commit();
            mma_tile(sa(kt % STAGES), sb(kt % STAGES));
        }
        cp_wait<0>();
    } else if (kt_n > 0) {
        uint4 ra[2], rb[2];
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            ra[i] = load_chunk<A_KC>(A, g.lda, g.M, g.K, m0, kt0 * TBK, tid + 128 * i, g.vec_a);
            rb[i] = load_chunk<B_KC>(B, g.ldb, g.N, g.K, n0, kt0 * TBK, tid + 128 * i, g.vec_b);
        }
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            store_chunk<A_KC>(sa(0), tid + 128 * i, ra[i]);
            store_chunk<B_KC>(sb(0), tid + 128 * i, rb[i]);
        }
        __syncthreads();
        for (int kt = 0; kt < kt_n; ++kt) {
            const int cur = kt & 1;
            if (kt + 1 < kt_n) {
#pragma unroll
                for (int i = 0; i < 2; ++i) {
                    ra[i] = load_chunk<A_KC>(A, g.lda, g.M, g.K, m0, (kt0 + kt + 1) * TBK, tid + 128 * i, g.vec_a);
                    rb[i] = load_chunk<B_KC>(B, g.ldb, g.N, g.K, n0, (kt0 + kt + 1) * TBK, tid + 128 * i, g.vec_b);
                }
            }
            mma_tile(sa(cur), sb(cur));
            if (kt + 1 < kt_n) {
#pragma unroll
                for (int i = 0; i < 2; ++i) {
                    store_chunk<A_KC>(sa(cur ^ 1), tid + 128 * i, ra[i]);
                    store_chunk<B_KC>(sb(cur ^ 1), tid + 128 * i, rb[i]);
                }
            }
            __syncthreads();
        }
    }

    if (KS > 1) {
        // partial tiles of ranks 1 .. KS-1 into their staging buffers as float4 [8][128 threads],
        // summed by rank 0 in rank order; the second barrier keeps them alive until it has read
        __syncthreads();  // every warp is done with the staging tiles
        float4* part = reinterpret_cast<float4*>(stage_buf);
        if (ks != 0) {
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    part[(i * 4 + j) * 128 + tid] = make_float4(acc[i][j][0], acc[i][j][1], acc[i][j][2], acc[i][j][3]);
        }
        cluster_sync();
        if (ks == 0) {
            for (int r = 1; r < KS; ++r)
#pragma unroll
                for (int i = 0; i < 2; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        const float4 v = ld_cluster_f4(part + (i * 4 + j) * 128 + tid, (unsigned)r);
                        acc[i][j][0] += v.x;
                        acc[i][j][1] += v.y;
                        acc[i][j][2] += v.z;
                        acc[i][j][3] += v.w;
                    }
        }
        cluster_sync();
        if (ks != 0) return;
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

namespace {
// K split over a cluster of 4 CTAs for products of at least 8 k-tiles (both operands 16-byte
// copyable, no bias gradient); otherwise one CTA per output tile.
template <bool A_KC, bool B_KC, int EPI>
cudaError_t launch_member_gemm(const MemberGemm& g, int members, cudaStream_t s) {
    const unsigned nt = (unsigned)((g.N + TBN - 1) / TBN), mt = (unsigned)((g.M + TBM - 1) / TBM);
    const int kt_all = (g.K + TBK - 1) / TBK;
    if constexpr (EPI != kMemberGemmF32) {
        if (g.vec_a && g.vec_b && kt_all >= 8) {
            constexpr int KS = 4;
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(nt * KS, mt, (unsigned)members);
            cfg.blockDim = dim3(128);
            cfg.stream = s;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeClusterDimension;
            attr[0].val.clusterDim.x = KS;
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            return cudaLaunchKernelEx(&cfg, mlp_member_gemm_kernel<A_KC, B_KC, EPI, true, KS>, g);
        }
    }
    const dim3 grid(nt, mt, (unsigned)members);
    if (g.vec_a && g.vec_b) mlp_member_gemm_kernel<A_KC, B_KC, EPI, true, 1><<<grid, 128, 0, s>>>(g);
    else mlp_member_gemm_kernel<A_KC, B_KC, EPI, false, 1><<<grid, 128, 0, s>>>(g);
    return cudaGetLastError();
}
}  // namespace

cudaError_t mlp_member_gemm(const MemberGemm& g, int members, int epi, bool a_kc, bool b_kc, cudaStream_t s) {
    if (members < 1 || g.M < 1 || g.N < 1 || g.K < 1) return cudaErrorInvalidValue;
    if (a_kc && !b_kc && epi == kMemberGemmBiasReluBf16)
        return launch_member_gemm<true, false, kMemberGemmBiasReluBf16>(g, members, s);
    if (a_kc && !b_kc && epi == kMemberGemmBiasF32) return launch_member_gemm<true, false, kMemberGemmBiasF32>(g, members, s);
    if (a_kc && b_kc && epi == kMemberGemmMaskBf16) return launch_member_gemm<true, true, kMemberGemmMaskBf16>(g, members, s);
    if (!a_kc && !b_kc && epi == kMemberGemmF32) return launch_member_gemm<false, false, kMemberGemmF32>(g, members, s);
    return cudaErrorInvalidValue;
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
