// Compaction of the window sums for read-back: the non-zero (window, output state) bins of a
// simulation in increasing bin order, as (bin, sum) pairs, from either the dense windows x 2^n_out
// table or the window hash table (SimParams::hslots). The same passes compact the 2^n_out
// final-state counts into (output state, count) pairs.
//
// The reference reads its dense windows x 2^n_out float table back whole and walks it on the host
// (src/statistics/window_average_small.cpp:99-140, 181-250). Here a bitmap over all bins marks the
// occupied ones; per chunk of 2048 bitmap words a block scan gives every word the number of
// occupied bins before it inside the chunk, one block scans the chunk totals, and each occupied
// bin is written at its rank. No sort: two passes over the occupied slots (or the dense table)
// and three over the bitmap (windows x 2^n_out / 8 bytes).
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "../../../include/mbg.h"
#include "kernels.h"

namespace mbg {

// Records the message for mbg_last_error() and returns `st` (defined with the C ABI, capi.cpp).
mbg_status set_error(mbg_status st, const std::string& msg);

namespace {

constexpr int kCountThreads = 256;
constexpr int kWordsPerThread = 8;
constexpr int kChunkWords = kCountThreads * kWordsPerThread;  // bitmap words per count block

// Hash table: one bit per occupied slot's bin.
__global__ void win_mark_hash(const unsigned long long* __restrict__ slots, unsigned long long n_slots,
                              unsigned* __restrict__ bitmap) {
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n_slots;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned long long key = slots[2 * i];
        if (key) {
            const unsigned long long bin = key - 1ull;
            atomicOr(bitmap + (bin >> 5), 1u << (unsigned)(bin & 31ull));
        }
    }
}

// Dense table (u64 window sums or u32 final-state counts): warp w builds bitmap words 32w .. 32w + 31,
// one ballot per word over 32 coalesced entries (no atomics: every word has one writer).
template <typename T>
__global__ void win_mark_dense(const T* __restrict__ hist, unsigned long long n_bins, unsigned long long n_words,
                               unsigned* __restrict__ bitmap) {
    const unsigned lane = threadIdx.x & 31u;
    const unsigned long long warps = (unsigned long long)gridDim.x * blockDim.x / 32;
    for (unsigned long long g = (blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x) / 32; g * 32 < n_words;
         g += warps) {
        unsigned mine = 0;
        for (unsigned k = 0; k < 32; ++k) {
            const unsigned long long word = g * 32 + k;
            const unsigned long long bin = word * 32 + lane;
            const bool set = word < n_words && bin < n_bins && hist[bin] != T(0);
            const unsigned b = __ballot_sync(0xffffffffu, set);
            if (lane == k) mine = b;
        }
        const unsigned long long word = g * 32 + lane;
        if (word < n_words) bitmap[word] = mine;
    }
}

// Block b of 256 threads: words [2048 b, 2048 (b + 1)). wpre[word] = occupied bins in the chunk
// before the word; chunk[b] = occupied bins in the chunk.
__global__ void __launch_bounds__(kCountThreads) win_count(const unsigned* __restrict__ bitmap,
                                                           unsigned long long n_words, unsigned* __restrict__ wpre,
                                                           unsigned* __restrict__ chunk) {
    __shared__ unsigned warp_tot[kCountThreads / 32];
    const unsigned long long base = (unsigned long long)blockIdx.x * kChunkWords + threadIdx.x * kWordsPerThread;
    unsigned c[kWordsPerThread];
    unsigned mine = 0;
#pragma unroll
    for (int j = 0; j < kWordsPerThread; ++j) {
        c[j] = base + j < n_words ? (unsigned)__popc(bitmap[base + j]) : 0u;
        mine += c[j];
    }
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    unsigned incl = mine;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= (unsigned)d) incl += y;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    unsigned before = 0, total = 0;
    for (int w = 0; w < kCountThreads / 32; ++w) {
        if (w < (int)warp) before += warp_tot[w];
        total += warp_tot[w];
    }
    unsigned run = before + incl - mine;
#pragma unroll
    for (int j = 0; j < kWordsPerThread; ++j) {
        if (base + j < n_words) wpre[base + j] = run;
        run += c[j];
    }
    if (threadIdx.x == 0) chunk[blockIdx.x] = total;
}

// One block: exclusive prefix of the chunk totals in place; *total = their sum.
__global__ void __launch_bounds__(1024) win_scan_chunks(unsigned* __restrict__ chunk, unsigned n_chunks,
                                                         unsigned long long* __restrict__ total) {
    __shared__ unsigned warp_tot[32];
    __shared__ unsigned carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    for (unsigned base = 0; base < n_chunks; base += 1024) {
        const unsigned i = base + threadIdx.x;
        const unsigned v = i < n_chunks ? chunk[i] : 0u;
        unsigned incl = v;
        for (int d = 1; d < 32; d <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= (unsigned)d) incl += y;
        }
        if (lane == 31) warp_tot[warp] = incl;
        __syncthreads();
        unsigned before = carry;
        for (unsigned w = 0; w < warp; ++w) before += warp_tot[w];
        if (i < n_chunks) chunk[i] = before + incl - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry = before + incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

__device__ __forceinline__ unsigned bin_rank(unsigned long long bin, const unsigned* __restrict__ bitmap,
                                             const unsigned* __restrict__ wpre, const unsigned* __restrict__ chunk) {
    const unsigned long long word = bin >> 5;
    const unsigned below = bitmap[word] & ((1u << (unsigned)(bin & 31ull)) - 1u);
    return chunk[word / kChunkWords] + wpre[word] + (unsigned)__popc(below);
}

__global__ void win_emit_hash(const unsigned long long* __restrict__ slots, unsigned long long n_slots,
                              const unsigned* __restrict__ bitmap, const unsigned* __restrict__ wpre,
                              const unsigned* __restrict__ chunk, unsigned* __restrict__ out_bin,
                              unsigned long long* __restrict__ out_sum) {
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n_slots;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned long long key = slots[2 * i];
        if (key) {
            const unsigned long long bin = key - 1ull;
            const unsigned r = bin_rank(bin, bitmap, wpre, chunk);
            out_bin[r] = (unsigned)bin;
            out_sum[r] = slots[2 * i + 1];
        }
    }
}

template <typename T>
__global__ void win_emit_dense(const T* __restrict__ hist, unsigned long long n_words,
                               const unsigned* __restrict__ bitmap, const unsigned* __restrict__ wpre,
                               const unsigned* __restrict__ chunk, unsigned* __restrict__ out_bin,
                               T* __restrict__ out_sum) {
    for (unsigned long long word = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; word < n_words;
         word += (unsigned long long)gridDim.x * blockDim.x) {
        unsigned bits = bitmap[word];
        unsigned r = chunk[word / kChunkWords] + wpre[word];
        while (bits) {
            const unsigned j = (unsigned)__ffs(bits) - 1u;
            bits &= bits - 1u;
            const unsigned long long bin = word * 32 + j;
            out_bin[r] = (unsigned)bin;
            out_sum[r] = hist[bin];
            ++r;
        }
    }
}

}  // namespace

unsigned long long window_bitmap_words(unsigned long long n_bins) { return (n_bins + 31) / 32; }

unsigned window_chunks(unsigned long long n_bins) {
    return (unsigned)((window_bitmap_words(n_bins) + kChunkWords - 1) / kChunkWords);
}

namespace {

// The marking kernel of one table, then the two scans that rank its marked entries.
template <typename Mark>
cudaError_t count_marked(unsigned long long n_bins, unsigned* bitmap, unsigned* wpre, unsigned* chunk,
                         unsigned long long* total, int sms, cudaStream_t stream, Mark mark) {
    const unsigned long long n_words = window_bitmap_words(n_bins);
    const unsigned n_chunks = window_chunks(n_bins);
    cudaError_t e = cudaMemsetAsync(bitmap, 0, n_words * 4, stream);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.stream = stream;
    cfg.gridDim = dim3(sms * 8);
    cfg.blockDim = dim3(256);
    e = mark(cfg, n_words);
    if (e != cudaSuccess) return e;
    cfg.gridDim = dim3(n_chunks);
    cfg.blockDim = dim3(kCountThreads);
    e = cudaLaunchKernelEx(&cfg, win_count, (const unsigned*)bitmap, n_words, wpre, chunk);
    if (e != cudaSuccess) return e;
    cfg.gridDim = dim3(1);
    cfg.blockDim = dim3(1024);
    return cudaLaunchKernelEx(&cfg, win_scan_chunks, chunk, n_chunks, total);
}

}  // namespace

cudaError_t launch_window_count(const unsigned long long* hist, const unsigned long long* hslots, int hash_bits,
                                unsigned long long n_bins, unsigned* bitmap, unsigned* wpre, unsigned* chunk,
                                unsigned long long* total, int sms, cudaStream_t stream) {
    return count_marked(n_bins, bitmap, wpre, chunk, total, sms, stream,
                        [&](cudaLaunchConfig_t& cfg, unsigned long long n_words) {
                            if (hash_bits > 0)
                                return cudaLaunchKernelEx(&cfg, win_mark_hash, hslots, 1ull << hash_bits, bitmap);
                            return cudaLaunchKernelEx(&cfg, win_mark_dense<unsigned long long>, hist, n_bins,
                                                      n_words, bitmap);
                        });
}

cudaError_t launch_final_count(const unsigned* counts, unsigned long long n_states, unsigned* bitmap,
                               unsigned* wpre, unsigned* chunk, unsigned long long* total, int sms,
                               cudaStream_t stream) {
    return count_marked(n_states, bitmap, wpre, chunk, total, sms, stream,
                        [&](cudaLaunchConfig_t& cfg, unsigned long long n_words) {
                            return cudaLaunchKernelEx(&cfg, win_mark_dense<unsigned>, counts, n_states, n_words,
                                                      bitmap);
                        });
}

cudaError_t launch_final_emit(const unsigned* counts, unsigned long long n_states, const unsigned* bitmap,
                              const unsigned* wpre, const unsigned* chunk, unsigned* out_state, unsigned* out_count,
                              int sms, cudaStream_t stream) {
    cudaLaunchConfig_t cfg = {};
    cfg.stream = stream;
    cfg.gridDim = dim3(sms * 8);
    cfg.blockDim = dim3(256);
    return cudaLaunchKernelEx(&cfg, win_emit_dense<unsigned>, counts, window_bitmap_words(n_states), bitmap, wpre,
                              chunk, out_state, out_count);
}

cudaError_t launch_window_emit(const unsigned long long* hist, const unsigned long long* hslots, int hash_bits,
                               unsigned long long n_bins, const unsigned* bitmap, const unsigned* wpre,
                               const unsigned* chunk, unsigned* out_bin, unsigned long long* out_sum, int sms,
                               cudaStream_t stream) {
    cudaLaunchConfig_t cfg = {};
    cfg.stream = stream;
    cfg.gridDim = dim3(sms * 8);
    cfg.blockDim = dim3(256);
    if (hash_bits > 0)
        return cudaLaunchKernelEx(&cfg, win_emit_hash, hslots, 1ull << hash_bits, bitmap, wpre, chunk, out_bin,
                                  out_sum);
    return cudaLaunchKernelEx(&cfg, win_emit_dense<unsigned long long>, hist, window_bitmap_words(n_bins), bitmap,
                              wpre, chunk, out_bin, out_sum);
}

// ---------------------------------------------------------------------------------------------
// One window of many batched instances gathered into one array: block (x, y) copies entries
// x * 256 + threadIdx.x (grid-stride in x) of span y.

namespace {

__global__ void win_gather(const WindowSpan* __restrict__ spans, unsigned long long* __restrict__ out) {
    const WindowSpan s = spans[blockIdx.y];
    for (unsigned long long e = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; e < s.n;
         e += (unsigned long long)gridDim.x * blockDim.x)
        out[s.dst + e] = s.src[e];
}

}  // namespace

cudaError_t launch_window_gather(const WindowSpan* spans, int n_spans, unsigned long long max_n,
                                 unsigned long long* out, cudaStream_t stream) {
    for (int s0 = 0; s0 < n_spans; s0 += 65535) {
        cudaLaunchConfig_t cfg = {};
        cfg.stream = stream;
        cfg.gridDim = dim3((unsigned)std::min<unsigned long long>((max_n + 255) / 256, 1024ull),
                           (unsigned)std::min(65535, n_spans - s0));
        cfg.blockDim = dim3(256);
        const cudaError_t e = cudaLaunchKernelEx(&cfg, win_gather, spans + s0, out);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// ---------------------------------------------------------------------------------------------
// L2 atomic throughput probe: the secondary bound of the simulation kernels, whose window-sum
// flushes are fire-and-forget 64-bit atomic adds (RED) into an L2-resident table.

namespace {

__global__ void l2_red_probe(unsigned long long* __restrict__ buf, unsigned mask, int iters) {
    const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned a = tid * 2654435761u;
    for (int i = 0; i < iters; ++i) {
        atomicAdd(buf + (a & mask), 1ull);
        a += 0x9E3779B9u;
    }
}

}  // namespace

}  // namespace mbg

extern "C" mbg_status mbg_device_l2_atomic_rate(int32_t device, uint32_t distinct, double* atomics_per_s) {
    if (!atomics_per_s || distinct == 0 || (distinct & (distinct - 1)) != 0 || distinct > (1u << 26))
        return mbg::set_error(MBG_ERR_ARG, "mbg_device_l2_atomic_rate: distinct must be a power of two <= 2^26");
    int sms = 0;
    unsigned long long* buf = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaMalloc(&buf, (size_t)distinct * 8);
    if (e == cudaSuccess) e = cudaMemset(buf, 0, (size_t)distinct * 8);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    const int iters = 256, block = 256;
    const unsigned grid = (unsigned)sms * 8u;
    float best = 0.f;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {  // the first is a warm-up
        e = cudaEventRecord(e0, nullptr);
        if (e == cudaSuccess) e = cudaLaunchKernelEx(&cfg, mbg::l2_red_probe, buf, distinct - 1u, iters);
        if (e == cudaSuccess) e = cudaEventRecord(e1, nullptr);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e == cudaSuccess && rep > 0 && (best == 0.f || ms < best)) best = ms;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (buf) cudaFree(buf);
    if (e != cudaSuccess)
        return mbg::set_error(MBG_ERR_CUDA, std::string("mbg_device_l2_atomic_rate: ") + cudaGetErrorString(e));
    *atomics_per_s = (double)grid * block * iters / (best * 1e-3);
    return mbg::set_error(MBG_OK, "");
}
