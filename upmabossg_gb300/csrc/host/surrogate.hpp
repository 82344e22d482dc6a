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
    struct Layer {
        int in = 0, out = 0;
        float *w = nullptr, *b = nullptr;  // FP32 master weights, W row-major [in][out]
        __nv_bfloat16* wb = nullptr;       // BF16 copy used by the GEMMs
        __nv_bfloat16* wtb = nullptr;      // BF16 W^T [out][in]: the K-major operand of the tcgen05 GEMM
        float *gw = nullptr, *gb = nullptr;
        float *mw = nullptr, *vw = nullptr, *mb = nullptr, *vb = nullptr;  // Adam moments
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
    // forward products on the tcgen05 tensor cores (true) or on the mma.sync kernel
    bool tensor_tc = true;
    std::vector<Member> members;

private:
    // Activations, gradients and the stream of one forward/backward pass. Prediction uses `main`;
    // training gives every member its own, so that the members train concurrently.
    struct Work {
        cudaStream_t stream = nullptr;
        int cap_rows = 0;
        __nv_bfloat16* xb = nullptr;
        float* yt = nullptr;
        std::vector<__nv_bfloat16*> acts;
        float* logits = nullptr;
        __nv_bfloat16* dlogits = nullptr;
        float* da = nullptr;
        __nv_bfloat16 *dh = nullptr, *dh2 = nullptr;
        float* loss = nullptr;
    };
    template <class T>
    T* alloc(size_t n);
    void ensure_work(Work& w, int rows);
    void ensure_batch(int rows);
    void forward(int member, int rows, Work& w);
    void backward(int member, int rows, Work& w);
    void refresh_transposed(int member, cudaStream_t s);
    void check_tc_error();

    cudaStream_t stream = nullptr;
    Work main;
    std::vector<Work> train_work;
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
