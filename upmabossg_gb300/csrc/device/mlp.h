// Host-callable launchers of the surrogate MLP kernels (mlp.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace mbg {

// C[M x N] = alpha * A[M x K] . B[K x N] (+ bias[n]) (ReLU), element (m, k) of A at
// A[a_row_offset * a_m + m * a_m + k * a_k] (a_row_offset read on the device, may be null),
// element (k, n) of B at B[k * b_k + n * b_n]. C (FP32) and/or Cb (BF16) may be null.
struct GemmArgs {
    int M = 0, N = 0, K = 0;
    const __nv_bfloat16* A = nullptr;
    long long a_m = 0, a_k = 0;
    const int* a_row_offset = nullptr;
    const __nv_bfloat16* B = nullptr;
    long long b_k = 0, b_n = 0;
    float* C = nullptr;
    int ldc = 0;
    __nv_bfloat16* Cb = nullptr;
    int ldcb = 0;
    const float* bias = nullptr;
    int relu = 0;
    int accumulate = 0;
    float alpha = 1.f;
};

cudaError_t mlp_gemm(const GemmArgs& g, cudaStream_t s);
// The same product on the tcgen05 tensor cores (mlp_tc.cu): requires a_k == 1 and b_k == 1 (B
// given transposed, K-contiguous), K, a_m and b_n multiples of 8 and 16-byte aligned A and B
// (mlp_gemm_tc_supported); sets *error_flag if a completion wait gave up.
bool mlp_gemm_tc_supported(const GemmArgs& g);
// Sets the kernel's shared-memory limit (once per device, before any launch or graph capture).
cudaError_t mlp_gemm_tc_configure();
cudaError_t mlp_gemm_tc(const GemmArgs& g, unsigned* error_flag, cudaStream_t s);
// y = x^T for a rows x cols BF16 matrix.
cudaError_t mlp_transpose_bf16(const __nv_bfloat16* x, int rows, int cols, __nv_bfloat16* y, cudaStream_t s);

// Softmax of logits [rows x cols] (cols <= 1024) into probs (FP32); with a target distribution:
// dlogits = (softmax - target) * scale as BF16 and the summed cross-entropy added to *loss.
cudaError_t mlp_softmax_xent(const float* logits, int rows, int cols, const float* target, float scale,
                             float* probs, __nv_bfloat16* dlogits, float* loss, cudaStream_t s);
// dh = (act > 0) ? da : 0, BF16 out.
cudaError_t mlp_relu_backward(const float* da, const __nv_bfloat16* act, __nv_bfloat16* dh, long long n,
                              cudaStream_t s);
// db[c] = sum over rows of d[r, c] (d BF16, rows x cols row-major).
cudaError_t mlp_bias_grad(const __nv_bfloat16* d, int rows, int cols, float* db, cudaStream_t s);
// Adam whose learning rate and bias corrections come from sched[3 * (*t) .. +2] = (lr, 1 / (1 - b1^k),
// 1 / (1 - b2^k)), and the step counter increment: the step-dependent parts of a replayed graph.
cudaError_t mlp_adam_sched(float* w, const float* g, float* m, float* v, __nv_bfloat16* wb, long long n,
                           const float* sched, const int* t, float beta1, float beta2, float eps, cudaStream_t s);
cudaError_t mlp_step_advance(int* t, cudaStream_t s);
cudaError_t mlp_to_bf16(const float* x, __nv_bfloat16* y, long long n, cudaStream_t s);
// probs: E members x rows x cols. mean = member average; spread[r] = max over members of the
// total-variation distance between the member and the mean.
cudaError_t mlp_ensemble_stats(const float* probs, int members, int rows, int cols, float* mean, float* spread,
                               cudaStream_t s);
// y[r] = x[r, column] for a rows x cols matrix.
cudaError_t mlp_gather_column(const float* x, int rows, int cols, int column, float* y, cudaStream_t s);
// y[i, :] = x[idx[i], :] (rows of `cols` floats), converting to BF16 when yb is set.
cudaError_t mlp_gather_rows(const float* x, const int* idx, int rows, int cols, float* y, __nv_bfloat16* yb,
                            cudaStream_t s);
// Minibatch (*t mod steps) of the permutation perm (rows indices each).
cudaError_t mlp_gather_rows_step(const float* x, const int* perm, const int* t, int steps, int rows, int cols,
                                 float* y, __nv_bfloat16* yb, cudaStream_t s);

}  // namespace mbg
