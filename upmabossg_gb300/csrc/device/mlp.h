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
// *t += 1 (the step counter of a replayed training graph).
cudaError_t mlp_step_advance(int* t, cudaStream_t s);

// ---- member-batched training step (mlp_train.cu): blockIdx.z = ensemble member ----
// Epilogues of mlp_member_gemm: C = relu(A.B + bias) as BF16; C = A.B + bias as FP32;
// C = (act > 0) ? A.B : 0 as BF16; C = A.B as FP32 (plus, with gb set, gb[n] = sum over k of B(k, n)).
enum { kMemberGemmBiasReluBf16 = 0, kMemberGemmBiasF32 = 1, kMemberGemmMaskBf16 = 2, kMemberGemmF32 = 3 };
// C[M x N] = A[M x K] . B[K x N] for every member z (each pointer advanced by z times its *_z stride).
// A(m, k) at A[m * lda + k] when the launch's a_kc is set, else at A[k * lda + m]; B(k, n) at
// B[n * ldb + k] when b_kc is set, else at B[k * ldb + n]. C or Cb at [m * ldc + n]; act at
// [m * ldact + n]. vec_a / vec_b: the operand (and its member stride and leading dimension) allow
// 16-byte loads (16-byte aligned base, lda / ldb and *_z multiples of 8 elements).
struct MemberGemm {
    int M = 0, N = 0, K = 0;
    const __nv_bfloat16* A = nullptr;
    long long lda = 0, a_z = 0;
    const __nv_bfloat16* B = nullptr;
    long long ldb = 0, b_z = 0;
    float* C = nullptr;
    __nv_bfloat16* Cb = nullptr;
    long long ldc = 0, c_z = 0;
    const float* bias = nullptr;
    long long bias_z = 0;
    const __nv_bfloat16* act = nullptr;
    long long ldact = 0, act_z = 0;
    float* gb = nullptr;
    long long gb_z = 0;
    bool vec_a = false, vec_b = false;
};
// Supported (a_kc, b_kc, epilogue): (1, 0, bias+ReLU BF16), (1, 0, bias FP32), (1, 1, mask BF16),
// (0, 0, FP32 with bias gradient): the forward, data-gradient and weight-gradient products. With
// vec_a and vec_b the operands stream through a 4-stage cp.async ring, and products of at least 8
// k-tiles without a bias gradient split K over a 4-CTA cluster.
cudaError_t mlp_member_gemm(const MemberGemm& g, int members, int epi, bool a_kc, bool b_kc, cudaStream_t s);
// Member e's minibatch (*t mod steps): rows perm[e * n + (*t mod steps) * rows + r] of x (to BF16,
// xb [members][rows][cols_x]) and of y (yt [members][rows][cols_y]).
cudaError_t mlp_member_gather(const float* x, int cols_x, const float* y, int cols_y, const int* perm, long long n,
                              const int* t, int steps, int rows, int members, __nv_bfloat16* xb, float* yt,
                              cudaStream_t s);
// Adam over `members` consecutive parameter blocks of `per` elements, member e's learning rate and
// bias corrections at sched[3 * (e * sched_len + *t) ..]; wb receives the BF16 copy.
cudaError_t mlp_member_adam(float* w, const float* g, float* m, float* v, __nv_bfloat16* wb, long long per,
                            int members, const float* sched, long long sched_len, const int* t, float beta1,
                            float beta2, float eps, cudaStream_t s);
// Softmax cross-entropy of `members` stacked [rows x cols] blocks (member stride rows * cols for
// logits, target and dlogits); member z's summed loss is added to loss[z].
cudaError_t mlp_softmax_xent_members(const float* logits, int rows, int cols, int members, const float* target,
                                     float scale, __nv_bfloat16* dlogits, float* loss, cudaStream_t s);
cudaError_t mlp_to_bf16(const float* x, __nv_bfloat16* y, long long n, cudaStream_t s);
// probs: E members x rows x cols. mean = member average; spread[r] = max over members of the
// total-variation distance between the member and the mean.
cudaError_t mlp_ensemble_stats(const float* probs, int members, int rows, int cols, float* mean, float* spread,
                               cudaStream_t s);
// y[r] = x[r, column] for a rows x cols matrix.
cudaError_t mlp_gather_column(const float* x, int rows, int cols, int column, float* y, cudaStream_t s);

}  // namespace mbg
