// Ensemble of BF16 MLPs used to screen sweep points (surrogate.cpp).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "../device/mlp.h"
#include "sim_host.hpp"

namespace mbg {

class Surrogate {
public:
    // A layer's tensors point into its member's parameter block (see `per_member`).
    struct Layer {
        int in = 0, out = 0;
        float *w = nullptr, *b = nullptr;  // FP32 master weights, W row-major [in][out]
        __nv_bfloat16* wb = nullptr;       // BF16 copy used by the GEMMs
        __nv_bfloat16* wtb = nullptr;      // BF16 W^T [out][in]: the K-major operand of the tcgen05 GEMM
        float *gw = nullptr, *gb = nullptr;
    };
    struct Member {
        std::vector<Layer> layers;
        int step = 0;
    };

    ~Surrogate();
    void create(int in_dim, int hidden, int hidden_layers, int out_dim, int ensemble, uint64_t seed, int device);
    float train(const float* x, const float* y, int64_t n, int epochs, int batch, float lr, uint64_t seed);
    // Ensemble mean distribution (probs, n x out; may be null), spread (may be null) and, when
    // score is set, the mean probability of output `column` alone.
    void predict(const float* x, int64_t n, float* probs, float* spread, int column = -1, float* score = nullptr,
                 int chunk = 65536);
    float gradients(int member, const float* x, const float* y, int rows);
    int64_t param_count() const;
    // Device time (ms) of one forward pass of every member over `rows` rows, mean of `reps`.
    double time_forward(int rows, int reps);
    void get_params(int member, float* dst, bool grads);
    void set_params(int member, const float* src);

    int in_dim = 0, hidden = 0, hidden_layers = 0, out_dim = 0, ensemble = 0, device = 0;
    // Parameter blocks: member e's tensors of one kind (weights, gradients, Adam moments, BF16
    // weights) are elements [e * per_member, (e + 1) * per_member) of one allocation per kind, layer
    // l's W at off_w[l] and its bias at off_b[l] (multiples of 8 elements, zero padding between), so
    // that one launch updates every member and every layer.
    long long per_member = 0;
    std::vector<long long> off_w, off_b;
    // forward products on the tcgen05 tensor cores (true) or on the mma.sync kernel
    bool tensor_tc = true;
    std::vector<Member> members;

private:
    // Activations of one member's forward pass over a chunk of prediction rows.
    struct Work {
        int cap_rows = 0;
        __nv_bfloat16* xb = nullptr;
        std::vector<__nv_bfloat16*> acts;
        float* logits = nullptr;
    };
    // Buffers of a training step for every member at once, member z's rows after z * rows * width:
    // inputs, targets, activations, logits, output-layer and hidden-layer gradients, losses.
    struct StepWork {
        int cap_rows = 0;
        __nv_bfloat16* xb = nullptr;
        float* yt = nullptr;
        std::vector<__nv_bfloat16*> acts;
        float* logits = nullptr;
        __nv_bfloat16* dlogits = nullptr;
        __nv_bfloat16* dh[2] = {nullptr, nullptr};
        float* loss = nullptr;
    };
    template <class T>
    T* alloc(size_t n);
    void ensure_batch(int rows);
    void ensure_step(int rows);
    void forward(int member, int rows, Work& w);
    // One training step's products for members m0 .. m0 + count - 1 over `rows` rows in step work
    // slots 0 .. count - 1: forward (activations, logits), then loss, data, weight and bias gradients.
    void step_forward(int rows, int m0, int count, cudaStream_t s);
    void step_backward(int rows, int m0, int count, cudaStream_t s);
    void refresh_transposed(int member, cudaStream_t s);
    void check_tc_error();

    cudaStream_t stream = nullptr;
    Work main;
    StepWork sw;
    float *w_all = nullptr, *g_all = nullptr, *m_all = nullptr, *v_all = nullptr;
    __nv_bfloat16* wb_all = nullptr;
    int cap_rows = 0;  // prediction buffers below
    float* xf = nullptr;
    float* probs = nullptr;
    float* mean = nullptr;
    float* spread = nullptr;
    unsigned* tc_error = nullptr;   // set by a tcgen05 GEMM whose mbarrier wait gave up
    std::vector<bool> wt_stale;     // per member: wtb behind wb
    std::vector<void*> owned;
};

}  // namespace mbg
