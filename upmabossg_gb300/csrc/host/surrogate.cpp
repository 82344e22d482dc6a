// Learned surrogate for sweep screening: an ensemble of BF16 MLPs (FP32 accumulation and FP32
// master weights) mapping a sweep point's parameters to an output-state distribution. Training
// (softmax cross-entropy against simulated distributions, Adam) and inference run on the project's
// own kernels (device/mlp.cu). The reference has no surrogate; this is an addition on top of the
// simulator, which has the last word: every point a screen reports is re-simulated.
#include "surrogate.hpp"

#include <cmath>
#include <cstring>
#include <numeric>
#include <random>

namespace mbg {

namespace {

void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw CudaError(std::string(what) + ": " + cudaGetErrorString(e));
}

}  // namespace

template <class T>
T* Surrogate::alloc(size_t n) {
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, (n ? n : 1) * sizeof(T));
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw NoMemError(std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    owned.push_back(p);
    return static_cast<T*>(p);
}

Surrogate::~Surrogate() {
    for (void* p : owned) cudaFree(p);
    for (Work& w : train_work)
        if (w.stream) cudaStreamDestroy(w.stream);
    if (stream) cudaStreamDestroy(stream);
}

void Surrogate::create(int in, int hid, int n_hidden, int out, int ens, uint64_t seed, int dev) {
    if (in < 1 || hid < 1 || n_hidden < 1 || out < 2 || out > 1024 || ens < 1 || ens > 16)
        throw ArgError("surrogate dimensions out of range");
    in_dim = in;
    hidden = hid;
    hidden_layers = n_hidden;
    out_dim = out;
    ensemble = ens;
    device = dev;
    ck(cudaSetDevice(device), "cudaSetDevice");
    ck(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
    tc_error = alloc<unsigned>(1);
    ck(cudaMemset(tc_error, 0, 4), "cudaMemset");
    ck(mlp_gemm_tc_configure(), "mlp_gemm_tc_configure");  // kernel attributes before any graph capture
    std::mt19937_64 rng(seed);
    members.resize(ens);
    wt_stale.assign(ens, true);
    for (int e = 0; e < ens; ++e) {
        Member& mb = members[e];
        for (int l = 0; l <= n_hidden; ++l) {
            Layer L;
            L.in = l == 0 ? in : hid;
            L.out = l == n_hidden ? out : hid;
            const size_t nw = (size_t)L.in * L.out;
            L.w = alloc<float>(nw);
            L.b = alloc<float>(L.out);
            L.wb = alloc<__nv_bfloat16>(nw);
            L.wtb = alloc<__nv_bfloat16>(nw);
            L.gw = alloc<float>(nw);
            L.gb = alloc<float>(L.out);
            L.mw = alloc<float>(nw);
            L.vw = alloc<float>(nw);
            L.mb = alloc<float>(L.out);
            L.vb = alloc<float>(L.out);
            // He initialisation for the ReLU layers, Glorot-like for the output layer
            const double sd = l == n_hidden ? std::sqrt(1.0 / L.in) : std::sqrt(2.0 / L.in);
            std::normal_distribution<double> nd(0.0, sd);
            std::vector<float> hw(nw), hb(L.out, 0.f);
            for (auto& x : hw) x = (float)nd(rng);
            ck(cudaMemcpy(L.w, hw.data(), nw * 4, cudaMemcpyHostToDevice), "cudaMemcpy H2D");
            ck(cudaMemcpy(L.b, hb.data(), L.out * 4, cudaMemcpyHostToDevice), "cudaMemcpy H2D");
            ck(cudaMemset(L.mw, 0, nw * 4), "cudaMemset");
            ck(cudaMemset(L.vw, 0, nw * 4), "cudaMemset");
            ck(cudaMemset(L.mb, 0, L.out * 4), "cudaMemset");
            ck(cudaMemset(L.vb, 0, L.out * 4), "cudaMemset");
            ck(mlp_to_bf16(L.w, L.wb, (long long)nw, stream), "mlp_to_bf16");
            mb.layers.push_back(L);
        }
    }
    ck(cudaStreamSynchronize(stream), "surrogate init");
}

void Surrogate::ensure_work(Work& w, int rows) {
    if (rows <= w.cap_rows) return;
    w.cap_rows = rows;
    w.xb = alloc<__nv_bfloat16>((size_t)rows * in_dim);
    w.yt = alloc<float>((size_t)rows * out_dim);
    w.acts.clear();
    for (int l = 0; l < hidden_layers; ++l) w.acts.push_back(alloc<__nv_bfloat16>((size_t)rows * hidden));
    w.logits = alloc<float>((size_t)rows * out_dim);
    w.dlogits = alloc<__nv_bfloat16>((size_t)rows * out_dim);
    w.da = alloc<float>((size_t)rows * hidden);
    w.dh = alloc<__nv_bfloat16>((size_t)rows * hidden);
    w.dh2 = alloc<__nv_bfloat16>((size_t)rows * hidden);
    w.loss = alloc<float>(1);
}

void Surrogate::ensure_batch(int rows) {
    main.stream = stream;
    ensure_work(main, rows);
    if (rows <= cap_rows) return;
    cap_rows = rows;
    xf = alloc<float>((size_t)rows * in_dim);
    probs = alloc<float>((size_t)rows * out_dim * ensemble);
    mean = alloc<float>((size_t)rows * out_dim);
    spread = alloc<float>((size_t)rows);
}

void Surrogate::refresh_transposed(int e, cudaStream_t s) {
    if (!wt_stale[e]) return;
    for (const Layer& L : members[e].layers)
        ck(mlp_transpose_bf16(L.wb, L.in, L.out, L.wtb, s), "mlp_transpose_bf16");
    wt_stale[e] = false;
}

void Surrogate::check_tc_error() {
    unsigned flag = 0;
    ck(cudaMemcpy(&flag, tc_error, 4, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
    if (flag) throw DeviceError("tcgen05 GEMM: a tensor-core completion wait gave up");
}

// logits = MLP(xb) for `rows` rows of member e; hidden activations kept for the backward pass.
void Surrogate::forward(int e, int rows, Work& w) {
    Member& mb = members[e];
    if (tensor_tc) refresh_transposed(e, w.stream);
    const __nv_bfloat16* a = w.xb;
    int a_cols = in_dim;
    for (int l = 0; l <= hidden_layers; ++l) {
        const Layer& L = mb.layers[l];
        GemmArgs g;
        g.M = rows;
        g.N = L.out;
        g.K = L.in;
        g.A = a;
        g.a_m = a_cols;
        g.a_k = 1;
        g.B = L.wb;
        g.b_k = L.out;
        g.b_n = 1;
        g.bias = L.b;
        GemmArgs gt = g;  // the tcgen05 form reads W^T
        gt.B = L.wtb;
        gt.b_k = 1;
        gt.b_n = L.in;
        if (l < hidden_layers) {
            g.relu = 1;
            g.Cb = w.acts[l];
            g.ldcb = L.out;
        } else {
            g.C = w.logits;
            g.ldc = L.out;
        }
        gt.relu = g.relu;
        gt.Cb = g.Cb;
        gt.ldcb = g.ldcb;
        gt.C = g.C;
        gt.ldc = g.ldc;
        if (tensor_tc && mlp_gemm_tc_supported(gt)) ck(mlp_gemm_tc(gt, tc_error, w.stream), "mlp_gemm_tc forward");
        else ck(mlp_gemm(g, w.stream), "mlp_gemm forward");
        if (l < hidden_layers) {
            a = w.acts[l];
            a_cols = L.out;
        }
    }
}

// Gradients of the mean cross-entropy of member e on `rows` rows (targets in yt) into gw, gb;
// the summed loss is added to *loss.
void Surrogate::backward(int e, int rows, Work& w) {
    Member& mb = members[e];
    ck(mlp_softmax_xent(w.logits, rows, out_dim, w.yt, 1.f / (float)rows, nullptr, w.dlogits, w.loss, w.stream),
       "mlp_softmax_xent");
    const __nv_bfloat16* d = w.dlogits;  // gradient w.r.t. the current layer's output
    int d_cols = out_dim;
    __nv_bfloat16* bufs[2] = {w.dh, w.dh2};
    for (int l = hidden_layers; l >= 0; --l) {
        Layer& L = mb.layers[l];
        const __nv_bfloat16* a_in = l == 0 ? w.xb : w.acts[l - 1];
        // dW = a_in^T . d
        GemmArgs gw;
        gw.M = L.in;
        gw.N = L.out;
        gw.K = rows;
        gw.A = a_in;
        gw.a_m = 1;
        gw.a_k = L.in;
        gw.B = d;
        gw.b_k = d_cols;
        gw.b_n = 1;
        gw.C = L.gw;
        gw.ldc = L.out;
        ck(mlp_gemm(gw, w.stream), "mlp_gemm weight gradient");
        ck(mlp_bias_grad(d, rows, L.out, L.gb, w.stream), "mlp_bias_grad");
        if (l > 0) {
            // da = d . W^T, then through the ReLU of the layer below
            GemmArgs gd;
            gd.M = rows;
            gd.N = L.in;
            gd.K = L.out;
            gd.A = d;
            gd.a_m = d_cols;
            gd.a_k = 1;
            gd.B = L.wb;
            gd.b_k = 1;
            gd.b_n = L.out;
            gd.C = w.da;
            gd.ldc = L.in;
            ck(mlp_gemm(gd, w.stream), "mlp_gemm data gradient");
            __nv_bfloat16* next = bufs[l & 1];
            ck(mlp_relu_backward(w.da, w.acts[l - 1], next, (long long)rows * L.in, w.stream), "mlp_relu_backward");
            d = next;
            d_cols = L.in;
        }
    }
}

float Surrogate::train(const float* x, const float* y, int64_t n, int epochs, int batch, float lr, uint64_t seed) {
    if (n < 1 || batch < 1 || epochs < 1) throw ArgError("empty training set or batch");
    ck(cudaSetDevice(device), "cudaSetDevice");
    batch = (int)std::min<int64_t>(batch, n);
    const int steps = (int)(n / batch);
    const int64_t total = (int64_t)epochs * steps;
    // every member trains on its own stream with its own buffers, so that the members' small
    // kernels run side by side
    if ((int)train_work.size() < ensemble) train_work.resize(ensemble);
    for (Work& w : train_work) {
        if (!w.stream) ck(cudaStreamCreateWithFlags(&w.stream, cudaStreamNonBlocking), "cudaStreamCreate");
        ensure_work(w, batch);
    }
    ck(cudaStreamSynchronize(stream), "surrogate");  // weights written on the main stream
    float* dx = alloc<float>((size_t)n * in_dim);
    float* dy = alloc<float>((size_t)n * out_dim);
    int* didx = alloc<int>((size_t)n * ensemble);
    float* sched = alloc<float>((size_t)3 * total * ensemble);
    int* tdev = alloc<int>((size_t)ensemble);
    ck(cudaMemcpy(dx, x, (size_t)n * in_dim * 4, cudaMemcpyHostToDevice), "cudaMemcpy H2D");
    ck(cudaMemcpy(dy, y, (size_t)n * out_dim * 4, cudaMemcpyHostToDevice), "cudaMemcpy H2D");
    ck(cudaMemset(tdev, 0, 4 * (size_t)ensemble), "cudaMemset");
    // per member and step: learning rate (half-cosine decay over the call, floored at lr / 100) and
    // Adam's bias corrections, which continue the member's step count
    {
        std::vector<float> hs((size_t)3 * total * ensemble);
        for (int e = 0; e < ensemble; ++e)
            for (int64_t k = 0; k < total; ++k) {
                const double f =
                    std::max(0.01, 0.5 * (1.0 + std::cos(3.141592653589793 * (double)k / (double)total)));
                const double t = (double)(members[e].step + k + 1);
                float* h = hs.data() + 3 * ((size_t)e * total + k);
                h[0] = (float)(lr * f);
                h[1] = (float)(1.0 / (1.0 - std::pow(0.9, t)));
                h[2] = (float)(1.0 / (1.0 - std::pow(0.999, t)));
            }
        ck(cudaMemcpy(sched, hs.data(), hs.size() * 4, cudaMemcpyHostToDevice), "cudaMemcpy H2D");
    }
    // one training step per member, captured once and replayed: minibatch gather, W^T refresh,
    // forward, backward, Adam, step counter
    std::vector<cudaGraphExec_t> execs(ensemble, nullptr);
    auto release = [&]() {
        for (cudaGraphExec_t& x : execs)
            if (x) cudaGraphExecDestroy(x);
    };
    try {
        for (int e = 0; e < ensemble; ++e) {
            Work& w = train_work[e];
            Member& mb = members[e];
            const int* perm_e = didx + (size_t)e * n;
            const float* sched_e = sched + (size_t)3 * total * e;
            wt_stale[e] = true;
            ck(cudaStreamBeginCapture(w.stream, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
            try {
                ck(mlp_gather_rows_step(dx, perm_e, tdev + e, steps, batch, in_dim, nullptr, w.xb, w.stream),
                   "gather x");
                ck(mlp_gather_rows_step(dy, perm_e, tdev + e, steps, batch, out_dim, w.yt, nullptr, w.stream),
                   "gather y");
                forward(e, batch, w);
                backward(e, batch, w);
                for (Layer& L : mb.layers) {
                    ck(mlp_adam_sched(L.w, L.gw, L.mw, L.vw, L.wb, (long long)L.in * L.out, sched_e, tdev + e, 0.9f,
                                      0.999f, 1e-8f, w.stream),
                       "mlp_adam_sched");
                    ck(mlp_adam_sched(L.b, L.gb, L.mb, L.vb, nullptr, L.out, sched_e, tdev + e, 0.9f, 0.999f, 1e-8f,
                                      w.stream),
                       "mlp_adam_sched");
                }
                ck(mlp_step_advance(tdev + e, w.stream), "mlp_step_advance");
            } catch (...) {
                cudaGraph_t g = nullptr;
                cudaStreamEndCapture(w.stream, &g);
                if (g) cudaGraphDestroy(g);
                throw;
            }
            cudaGraph_t graph = nullptr;
            ck(cudaStreamEndCapture(w.stream, &graph), "cudaStreamEndCapture");
            const cudaError_t ie = cudaGraphInstantiate(&execs[e], graph, 0);
            cudaGraphDestroy(graph);
            ck(ie, "cudaGraphInstantiate");
        }
        std::mt19937_64 rng(seed);
        std::vector<int> perm(n);
        std::vector<float> last_loss(ensemble, 0.f);
        for (int ep = 0; ep < epochs; ++ep) {
            for (int e = 0; e < ensemble; ++e) {
                Work& w = train_work[e];
                std::iota(perm.begin(), perm.end(), 0);
                std::shuffle(perm.begin(), perm.end(), rng);
                // pageable source: the copy is staged before the call returns, so perm can be refilled
                ck(cudaMemcpyAsync(didx + (size_t)e * n, perm.data(), (size_t)n * 4, cudaMemcpyHostToDevice,
                                   w.stream),
                   "cudaMemcpyAsync");
                ck(cudaMemsetAsync(w.loss, 0, 4, w.stream), "cudaMemsetAsync");
            }
            for (int st = 0; st < steps; ++st)
                for (int e = 0; e < ensemble; ++e) ck(cudaGraphLaunch(execs[e], train_work[e].stream), "cudaGraphLaunch");
            if (ep == epochs - 1)
                for (int e = 0; e < ensemble; ++e) {
                    Work& w = train_work[e];
                    ck(cudaMemcpyAsync(&last_loss[e], w.loss, 4, cudaMemcpyDeviceToHost, w.stream), "cudaMemcpyAsync");
                }
        }
        for (Work& w : train_work) ck(cudaStreamSynchronize(w.stream), "training");
        release();
        float last = 0.f;
        for (int e = 0; e < ensemble; ++e) {
            members[e].step += (int)total;
            wt_stale[e] = true;
            last += last_loss[e] / (float)(steps * batch) / (float)ensemble;
        }
        check_tc_error();
        for (void* p : {(void*)dx, (void*)dy, (void*)didx, (void*)sched, (void*)tdev}) {
            cudaFree(p);
            owned.erase(std::find(owned.begin(), owned.end(), p));
        }
        return last;
    } catch (...) {
        for (Work& w : train_work) cudaStreamSynchronize(w.stream);
        release();
        throw;
    }
}

void Surrogate::predict(const float* x, int64_t n, float* out_probs, float* out_spread, int column,
                        float* out_score, int chunk) {
    ck(cudaSetDevice(device), "cudaSetDevice");
    if (out_score && (column < 0 || column >= out_dim)) throw ArgError("output column out of range");
    chunk = (int)std::max<int64_t>(1, std::min<int64_t>(chunk, n));
    ensure_batch(chunk);
    for (int64_t r0 = 0; r0 < n; r0 += chunk) {
        const int rows = (int)std::min<int64_t>(chunk, n - r0);
        ck(cudaMemcpyAsync(xf, x + r0 * in_dim, (size_t)rows * in_dim * 4, cudaMemcpyHostToDevice, stream),
           "cudaMemcpyAsync");
        ck(mlp_to_bf16(xf, main.xb, (long long)rows * in_dim, stream), "mlp_to_bf16");
        for (int e = 0; e < ensemble; ++e) {
            forward(e, rows, main);
            ck(mlp_softmax_xent(main.logits, rows, out_dim, nullptr, 0.f, probs + (size_t)e * rows * out_dim, nullptr,
                                nullptr, stream),
               "mlp_softmax");
        }
        ck(mlp_ensemble_stats(probs, ensemble, rows, out_dim, mean, spread, stream), "mlp_ensemble_stats");
        if (out_probs)
            ck(cudaMemcpyAsync(out_probs + r0 * out_dim, mean, (size_t)rows * out_dim * 4, cudaMemcpyDeviceToHost,
                               stream),
               "cudaMemcpyAsync");
        if (out_spread)
            ck(cudaMemcpyAsync(out_spread + r0, spread, (size_t)rows * 4, cudaMemcpyDeviceToHost, stream),
               "cudaMemcpyAsync");
        if (out_score) {
            // the column is gathered into the first rows of the (already copied) per-member buffer
            ck(mlp_gather_column(mean, rows, out_dim, column, probs, stream), "mlp_gather_column");
            ck(cudaMemcpyAsync(out_score + r0, probs, (size_t)rows * 4, cudaMemcpyDeviceToHost, stream),
               "cudaMemcpyAsync");
        }
        ck(cudaStreamSynchronize(stream), "prediction");
    }
    check_tc_error();
}

double Surrogate::time_forward(int rows, int reps) {
    ck(cudaSetDevice(device), "cudaSetDevice");
    if (rows < 1 || reps < 1) throw ArgError("rows and reps must be positive");
    ensure_batch(rows);
    // inputs: whatever the last batch left (the products' cost does not depend on the values)
    ck(cudaMemsetAsync(main.xb, 0, (size_t)rows * in_dim * sizeof(__nv_bfloat16), stream), "cudaMemsetAsync");
    cudaEvent_t e0, e1;
    ck(cudaEventCreate(&e0), "cudaEventCreate");
    ck(cudaEventCreate(&e1), "cudaEventCreate");
    for (int e = 0; e < ensemble; ++e) forward(e, rows, main);  // warm-up (and W^T refresh)
    ck(cudaEventRecord(e0, stream), "cudaEventRecord");
    for (int r = 0; r < reps; ++r)
        for (int e = 0; e < ensemble; ++e) forward(e, rows, main);
    ck(cudaEventRecord(e1, stream), "cudaEventRecord");
    ck(cudaEventSynchronize(e1), "forward timing");
    float ms = 0.f;
    ck(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    check_tc_error();
    return (double)ms / reps;
}

int64_t Surrogate::param_count() const {
    int64_t c = 0;
    for (const Layer& L : members[0].layers) c += (int64_t)L.in * L.out + L.out;
    return c;
}

void Surrogate::get_params(int e, float* dst, bool grads) {
    ck(cudaSetDevice(device), "cudaSetDevice");
    ck(cudaStreamSynchronize(stream), "surrogate");
    for (const Layer& L : members.at(e).layers) {
        const size_t nw = (size_t)L.in * L.out;
        ck(cudaMemcpy(dst, grads ? L.gw : L.w, nw * 4, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
        dst += nw;
        ck(cudaMemcpy(dst, grads ? L.gb : L.b, L.out * 4, cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
        dst += L.out;
    }
}

void Surrogate::set_params(int e, const float* src) {
    ck(cudaSetDevice(device), "cudaSetDevice");
    for (Layer& L : members.at(e).layers) {
        const size_t nw = (size_t)L.in * L.out;
        ck(cudaMemcpy(L.w, src, nw * 4, cudaMemcpyHostToDevice), "cudaMemcpy H2D");
        src += nw;
        ck(cudaMemcpy(L.b, src, L.out * 4, cudaMemcpyHostToDevice), "cudaMemcpy H2D");
        src += L.out;
        ck(mlp_to_bf16(L.w, L.wb, (long long)nw, stream), "mlp_to_bf16");
    }
    wt_stale[e] = true;
    ck(cudaStreamSynchronize(stream), "surrogate");
}

float Surrogate::gradients(int e, const float* x, const float* y, int rows) {
    ck(cudaSetDevice(device), "cudaSetDevice");
    if (e < 0 || e >= ensemble) throw ArgError("ensemble member out of range");
    ensure_batch(rows);
    ck(cudaMemcpyAsync(xf, x, (size_t)rows * in_dim * 4, cudaMemcpyHostToDevice, stream), "cudaMemcpyAsync");
    ck(mlp_to_bf16(xf, main.xb, (long long)rows * in_dim, stream), "mlp_to_bf16");
    ck(cudaMemcpyAsync(main.yt, y, (size_t)rows * out_dim * 4, cudaMemcpyHostToDevice, stream), "cudaMemcpyAsync");
    ck(cudaMemsetAsync(main.loss, 0, 4, stream), "cudaMemsetAsync");
    forward(e, rows, main);
    backward(e, rows, main);
    float h = 0.f;
    ck(cudaMemcpyAsync(&h, main.loss, 4, cudaMemcpyDeviceToHost, stream), "cudaMemcpyAsync");
    ck(cudaStreamSynchronize(stream), "gradients");
    return h / (float)rows;
}

}  // namespace mbg
