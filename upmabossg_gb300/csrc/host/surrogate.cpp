// Learned surrogate for sweep screening: an ensemble of BF16 MLPs (FP32 accumulation and FP32
// master weights) mapping a sweep point's parameters to an output-state distribution. Training
// (softmax cross-entropy against simulated distributions, Adam; device/mlp_train.cu, every launch
// covering all members) and inference (device/mlp.cu, device/mlp_tc.cu) run on the project's own
// kernels. The reference has no surrogate; this is an addition on top of the simulator, which has
// the last word: every point a screen reports is re-simulated.
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
    if (stream) cudaStreamDestroy(stream);
}

namespace {
long long round8(long long x) { return (x + 7) & ~7ll; }
bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }
}  // namespace

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
    off_w.clear();
    off_b.clear();
    per_member = 0;
    for (int l = 0; l <= n_hidden; ++l) {
        const long long li = l == 0 ? in : hid, lo = l == n_hidden ? out : hid;
        off_w.push_back(per_member);
        per_member = round8(per_member + li * lo);
        off_b.push_back(per_member);
        per_member = round8(per_member + lo);
    }
    const size_t all = (size_t)per_member * ens;
    w_all = alloc<float>(all);
    g_all = alloc<float>(all);
    m_all = alloc<float>(all);
    v_all = alloc<float>(all);
    wb_all = alloc<__nv_bfloat16>(all);
    for (float* p : {w_all, g_all, m_all, v_all}) ck(cudaMemset(p, 0, all * 4), "cudaMemset");
    for (int e = 0; e < ens; ++e) {
        Member& mb = members[e];
        const long long base = (long long)e * per_member;
        for (int l = 0; l <= n_hidden; ++l) {
            Layer L;
            L.in = l == 0 ? in : hid;
            L.out = l == n_hidden ? out : hid;
            const size_t nw = (size_t)L.in * L.out;
            L.w = w_all + base + off_w[l];
            L.b = w_all + base + off_b[l];
            L.wb = wb_all + base + off_w[l];
            L.gw = g_all + base + off_w[l];
            L.gb = g_all + base + off_b[l];
            L.wtb = alloc<__nv_bfloat16>(nw);
            // He initialisation for the ReLU layers, Glorot-like for the output layer
            const double sd = l == n_hidden ? std::sqrt(1.0 / L.in) : std::sqrt(2.0 / L.in);
            std::normal_distribution<double> nd(0.0, sd);
            std::vector<float> hw(nw);
            for (auto& x : hw) x = (float)nd(rng);
            ck(cudaMemcpy(L.w, hw.data(), nw * 4, cudaMemcpyHostToDevice), "cudaMemcpy H2D");
            mb.layers.push_back(L);
        }
    }
    ck(mlp_to_bf16(w_all, wb_all, (long long)all, stream), "mlp_to_bf16");
    ck(cudaStreamSynchronize(stream), "surrogate init");
}

void Surrogate::ensure_batch(int rows) {
    if (rows > main.cap_rows) {
        main.cap_rows = rows;
        main.xb = alloc<__nv_bfloat16>((size_t)rows * in_dim);
        main.acts.clear();
        for (int l = 0; l < hidden_layers; ++l) main.acts.push_back(alloc<__nv_bfloat16>((size_t)rows * hidden));
        main.logits = alloc<float>((size_t)rows * out_dim);
    }
    if (rows <= cap_rows) return;
    cap_rows = rows;
    xf = alloc<float>((size_t)rows * in_dim);
    probs = alloc<float>((size_t)rows * out_dim * ensemble);
    mean = alloc<float>((size_t)rows * out_dim);
    spread = alloc<float>((size_t)rows);
}

void Surrogate::ensure_step(int rows) {
    if (rows <= sw.cap_rows) return;
    sw.cap_rows = rows;
    const size_t r = (size_t)rows * ensemble;
    sw.xb = alloc<__nv_bfloat16>(r * in_dim);
    sw.yt = alloc<float>(r * out_dim);
    sw.acts.clear();
    for (int l = 0; l < hidden_layers; ++l) sw.acts.push_back(alloc<__nv_bfloat16>(r * hidden));
    sw.logits = alloc<float>(r * out_dim);
    sw.dlogits = alloc<__nv_bfloat16>(r * out_dim);
    sw.dh[0] = alloc<__nv_bfloat16>(r * hidden);
    sw.dh[1] = alloc<__nv_bfloat16>(r * hidden);
    sw.loss = alloc<float>(ensemble);
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
    if (tensor_tc) refresh_transposed(e, stream);
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
        if (tensor_tc && mlp_gemm_tc_supported(gt)) ck(mlp_gemm_tc(gt, tc_error, stream), "mlp_gemm_tc forward");
        else ck(mlp_gemm(g, stream), "mlp_gemm forward");
        if (l < hidden_layers) {
            a = w.acts[l];
            a_cols = L.out;
        }
    }
}

void Surrogate::step_forward(int rows, int m0, int count, cudaStream_t s) {
    const __nv_bfloat16* a = sw.xb;
    int a_cols = in_dim;
    const long long pb = (long long)m0 * per_member;
    for (int l = 0; l <= hidden_layers; ++l) {
        const Layer& L = members[m0].layers[l];
        MemberGemm g;
        g.M = rows;
        g.N = L.out;
        g.K = L.in;
        g.A = a;
        g.lda = a_cols;
        g.a_z = (long long)rows * a_cols;
        g.B = wb_all + pb + off_w[l];  // W [in][out]: B(k, n) at W[k * out + n]
        g.ldb = L.out;
        g.b_z = per_member;
        g.bias = w_all + pb + off_b[l];
        g.bias_z = per_member;
        g.vec_a = aligned16(a) && a_cols % 8 == 0 && g.a_z % 8 == 0;
        g.vec_b = aligned16(g.B) && L.out % 8 == 0 && per_member % 8 == 0;
        const bool hid = l < hidden_layers;
        if (hid) g.Cb = sw.acts[l];
        else g.C = sw.logits;
        g.ldc = L.out;
        g.c_z = (long long)rows * L.out;
        ck(mlp_member_gemm(g, count, hid ? kMemberGemmBiasReluBf16 : kMemberGemmBiasF32, true, false, s),
           "mlp_member_gemm forward");
        if (hid) {
            a = sw.acts[l];
            a_cols = L.out;
        }
    }
}

// Gradients of the mean cross-entropy (targets in yt) into the members' gradient blocks; the
// summed loss of slot z is added to sw.loss[z].
void Surrogate::step_backward(int rows, int m0, int count, cudaStream_t s) {
    ck(mlp_softmax_xent_members(sw.logits, rows, out_dim, count, sw.yt, 1.f / (float)rows, sw.dlogits, sw.loss, s),
       "mlp_softmax_xent_members");
    const long long pb = (long long)m0 * per_member;
    const __nv_bfloat16* d = sw.dlogits;  // gradient w.r.t. the current layer's output
    int d_cols = out_dim;
    for (int l = hidden_layers; l >= 0; --l) {
        const Layer& L = members[m0].layers[l];
        const __nv_bfloat16* a_in = l == 0 ? sw.xb : sw.acts[l - 1];
        __nv_bfloat16* next = sw.dh[l & 1];
        if (l > 0) {
            // da[r][i] = sum over o of d[r][o] W[i][o], through the ReLU of the layer below
            MemberGemm gd;
            gd.M = rows;
            gd.N = L.in;
            gd.K = L.out;
            gd.A = d;
            gd.lda = d_cols;
            gd.a_z = (long long)rows * d_cols;
            gd.B = wb_all + pb + off_w[l];  // B(o, i) at W[i * out + o]
            gd.ldb = L.out;
            gd.b_z = per_member;
            gd.act = sw.acts[l - 1];
            gd.ldact = L.in;
            gd.act_z = (long long)rows * L.in;
            gd.Cb = next;
            gd.ldc = L.in;
            gd.c_z = (long long)rows * L.in;
            gd.vec_a = aligned16(d) && d_cols % 8 == 0 && gd.a_z % 8 == 0;
            gd.vec_b = aligned16(gd.B) && L.out % 8 == 0 && per_member % 8 == 0;
            ck(mlp_member_gemm(gd, count, kMemberGemmMaskBf16, true, true, s), "mlp_member_gemm data gradient");
        }
        // dW[i][o] = sum over rows of a_in[r][i] d[r][o], db[o] = sum over rows of d[r][o]
        MemberGemm gw;
        gw.M = L.in;
        gw.N = L.out;
        gw.K = rows;
        gw.A = a_in;  // A(i, r) at a_in[r * in + i]
        gw.lda = L.in;
        gw.a_z = (long long)rows * L.in;
        gw.B = d;  // B(r, o) at d[r * out + o]
        gw.ldb = d_cols;
        gw.b_z = (long long)rows * d_cols;
        gw.C = g_all + pb + off_w[l];
        gw.ldc = L.out;
        gw.c_z = per_member;
        gw.gb = g_all + pb + off_b[l];
        gw.gb_z = per_member;
        gw.vec_a = aligned16(a_in) && L.in % 8 == 0 && gw.a_z % 8 == 0;
        gw.vec_b = aligned16(d) && d_cols % 8 == 0 && gw.b_z % 8 == 0;
        ck(mlp_member_gemm(gw, count, kMemberGemmF32, false, false, s), "mlp_member_gemm weight gradient");
        if (l > 0) {
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
    ensure_step(batch);
    ck(cudaStreamSynchronize(stream), "surrogate");
    float* dx = alloc<float>((size_t)n * in_dim);
    float* dy = alloc<float>((size_t)n * out_dim);
    int* didx = alloc<int>((size_t)n * ensemble);
    float* sched = alloc<float>((size_t)3 * total * ensemble);
    int* tdev = alloc<int>(1);
    auto release_scratch = [&]() {
        for (void* p : {(void*)dx, (void*)dy, (void*)didx, (void*)sched, (void*)tdev}) {
            cudaFree(p);
            owned.erase(std::find(owned.begin(), owned.end(), p));
        }
    };
    cudaGraphExec_t exec = nullptr;
    try {
        ck(cudaMemcpy(dx, x, (size_t)n * in_dim * 4, cudaMemcpyHostToDevice), "cudaMemcpy H2D");
        ck(cudaMemcpy(dy, y, (size_t)n * out_dim * 4, cudaMemcpyHostToDevice), "cudaMemcpy H2D");
        ck(cudaMemset(tdev, 0, 4), "cudaMemset");
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
        // one training step of every member, captured once and replayed: minibatch gather, forward,
        // backward, Adam over all parameter blocks, step counter
        ck(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
        try {
            ck(mlp_member_gather(dx, in_dim, dy, out_dim, didx, n, tdev, steps, batch, ensemble, sw.xb, sw.yt, stream),
               "mlp_member_gather");
            step_forward(batch, 0, ensemble, stream);
            step_backward(batch, 0, ensemble, stream);
            ck(mlp_member_adam(w_all, g_all, m_all, v_all, wb_all, per_member, ensemble, sched, total, tdev, 0.9f,
                               0.999f, 1e-8f, stream),
               "mlp_member_adam");
            ck(mlp_step_advance(tdev, stream), "mlp_step_advance");
        } catch (...) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(stream, &g);
            if (g) cudaGraphDestroy(g);
            throw;
        }
        cudaGraph_t graph = nullptr;
        ck(cudaStreamEndCapture(stream, &graph), "cudaStreamEndCapture");
        const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        ck(ie, "cudaGraphInstantiate");
        std::mt19937_64 rng(seed);
        std::vector<int> perm(n);
        std::vector<float> last_loss(ensemble, 0.f);
        for (int ep = 0; ep < epochs; ++ep) {
            for (int e = 0; e < ensemble; ++e) {
                std::iota(perm.begin(), perm.end(), 0);
                std::shuffle(perm.begin(), perm.end(), rng);
                // pageable source: the copy is staged before the call returns, so perm can be refilled
                ck(cudaMemcpyAsync(didx + (size_t)e * n, perm.data(), (size_t)n * 4, cudaMemcpyHostToDevice, stream),
                   "cudaMemcpyAsync");
            }
            ck(cudaMemsetAsync(sw.loss, 0, 4 * (size_t)ensemble, stream), "cudaMemsetAsync");
            for (int st = 0; st < steps; ++st) ck(cudaGraphLaunch(exec, stream), "cudaGraphLaunch");
            if (ep == epochs - 1)
                ck(cudaMemcpyAsync(last_loss.data(), sw.loss, 4 * (size_t)ensemble, cudaMemcpyDeviceToHost, stream),
                   "cudaMemcpyAsync");
        }
        ck(cudaStreamSynchronize(stream), "training");
        cudaGraphExecDestroy(exec);
        exec = nullptr;
        float last = 0.f;
        for (int e = 0; e < ensemble; ++e) {
            members[e].step += (int)total;
            wt_stale[e] = true;
            last += last_loss[e] / (float)(steps * batch) / (float)ensemble;
        }
        release_scratch();
        return last;
    } catch (...) {
        cudaStreamSynchronize(stream);
        if (exec) cudaGraphExecDestroy(exec);
        release_scratch();
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
    if (rows < 1) throw ArgError("no rows");
    ensure_batch(rows);
    ensure_step(rows);
    // the training step's member-batched kernels over every member, each on the same rows (the
    // gradients of all members are refreshed; member e's loss is returned)
    ck(cudaMemcpyAsync(xf, x, (size_t)rows * in_dim * 4, cudaMemcpyHostToDevice, stream), "cudaMemcpyAsync");
    ck(mlp_to_bf16(xf, sw.xb, (long long)rows * in_dim, stream), "mlp_to_bf16");
    ck(cudaMemcpyAsync(sw.yt, y, (size_t)rows * out_dim * 4, cudaMemcpyHostToDevice, stream), "cudaMemcpyAsync");
    for (int z = 1; z < ensemble; ++z) {
        ck(cudaMemcpyAsync(sw.xb + (size_t)z * rows * in_dim, sw.xb, (size_t)rows * in_dim * sizeof(__nv_bfloat16),
                           cudaMemcpyDeviceToDevice, stream),
           "cudaMemcpyAsync");
        ck(cudaMemcpyAsync(sw.yt + (size_t)z * rows * out_dim, sw.yt, (size_t)rows * out_dim * 4,
                           cudaMemcpyDeviceToDevice, stream),
           "cudaMemcpyAsync");
    }
    ck(cudaMemsetAsync(sw.loss, 0, 4 * (size_t)ensemble, stream), "cudaMemsetAsync");
    step_forward(rows, 0, ensemble, stream);
    step_backward(rows, 0, ensemble, stream);
    float h = 0.f;
    ck(cudaMemcpyAsync(&h, sw.loss + e, 4, cudaMemcpyDeviceToHost, stream), "cudaMemcpyAsync");
    ck(cudaStreamSynchronize(stream), "gradients");
    return h / (float)rows;
}

}  // namespace mbg
