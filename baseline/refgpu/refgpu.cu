// Reference-kernel harness: BASELINE MEASUREMENT ONLY.
//
// Runs the reference MaBoSSG's own device kernels on this GPU: src/jit_kernels/simulation.cu,
// window_average_small.cu and final_states.cu of the reference, compiled unmodified from its
// sources to LTO fatbins (`-arch=lto_103 -rdc=true -fatbin`, build_kernels.sh). The reference's host
// side cannot be built here (its parser is Flex/Bison output, its build is cmake with a network
// fetch, and two of its files no longer compile against CUDA 13), so the host path that drives
// those kernels is restated here, call for call:
//   generated rate source  src/generator.cpp:11-235 with the AST code of src/parser/expressions.cpp:25-231
//   JIT and link           src/kernel_compiler.cpp:61-164: NVRTC -dlto -rdc, nvJitLink -dlto -arch=sm_103
//                          with the three fatbins, cuModuleLoadData, the five kernels by name
//   batch loop             src/simulation_runner.cu:42-180: batches of <= 1e6 trajectories, <= 99 steps per
//                          launch, thrust stable_partition / partition of the unfinished trajectories,
//                          refill, memset of the record times
//   statistics per batch   final_states.cpp:36-43, fixed_states.cu:49-125 (CUB select, merge sort,
//                          run-length encode, two blocking copies, host map merge),
//                          window_average_small.cpp:58-89 (the 10 KiB shared-memory rule)
//   finalize               final_states.cpp:45-51, window_average_small.cpp:91-107
// The timed phase is the reference's "main> simulation" scope (main.cpp:54-83): runner and
// statistics set-up, the batch loop and finalize. Transitions are counted from the records each
// launch writes (a record per loop iteration, a flip after every record but the last) by a
// kernel of this harness whose own time is measured separately and taken out.
//
// Nothing in the product (upmabossg_gb300) links, loads or calls this file.
#include <cuda_runtime.h>
#include <curand_kernel.h>
#include <nvJitLink.h>
#include <nvrtc.h>

#include <cub/device/device_merge_sort.cuh>
#include <cub/device/device_run_length_encode.cuh>
#include <cub/device/device_select.cuh>
#include <thrust/device_ptr.h>
#include <thrust/execution_policy.h>
#include <thrust/iterator/counting_iterator.h>
#include <thrust/iterator/permutation_iterator.h>
#include <thrust/iterator/transform_iterator.h>
#include <thrust/iterator/zip_iterator.h>
#include <thrust/partition.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../upmabossg_gb300/csrc/host/model.hpp"

namespace {

struct Fail : std::runtime_error {
    using std::runtime_error::runtime_error;
};

void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw Fail(std::string(what) + ": " + cudaGetErrorString(e));
}

enum Status : uint8_t { CONTINUE = 0, FINISHED = 1, FIXED_POINT = 2 };  // trajectory_status.h:3-8

// ---------------------------------------------------------------------------------------------
// Generated source in the reference's layout (generator.cpp). Floats print with the default
// stream precision, as the reference's `os << float` does.

std::string fstr(float v) {
    std::ostringstream os;
    os << v;
    return os.str();
}

void gen_expr(const mbg::Expr& e, const mbg::Model& m, int cur, std::ostream& os, int depth = 0) {
    using K = mbg::Expr::Kind;
    using mbg::Op;
    if (depth > 64) throw Fail("alias recursion too deep");
    switch (e.kind) {
        case K::Literal: os << fstr((float)e.value); break;
        case K::Var: {
            auto it = m.variables.find(e.name);
            if (it == m.variables.end()) throw Fail("unknown variable " + e.name);
            os << fstr((float)it->second);
            break;
        }
        case K::Ident: {  // expressions.cpp:194-205
            const int i = m.node_index(e.name);
            if (i < 0) throw Fail("unknown node name: " + e.name);
            os << "((state[" << i / 32 << "] & " << (1u << (i % 32)) << "u) != 0)";
            break;
        }
        case K::Alias: {  // expressions.cpp:223-231
            const mbg::Expr* a = m.nodes[cur].attr(e.name.substr(1));
            if (!a) throw Fail("missing attribute " + e.name);
            gen_expr(*a, m, cur, os, depth + 1);
            break;
        }
        case K::Paren:
            os << "(";
            gen_expr(*e.a, m, cur, os, depth);
            os << ")";
            break;
        case K::Unary:
            os << (e.op == Op::Minus ? "-" : e.op == Op::Not ? "!" : "+");
            gen_expr(*e.a, m, cur, os, depth);
            break;
        case K::Binary: {
            const char* s = nullptr;
            switch (e.op) {
                case Op::Plus: s = " + "; break;
                case Op::Minus: s = " - "; break;
                case Op::Star: s = " * "; break;
                case Op::Slash: s = " / "; break;
                case Op::And: s = " & "; break;
                case Op::Or: s = " | "; break;
                case Op::Xor: s = " ^ "; break;  // the reference throws (expressions.cpp:79,148)
                case Op::Eq: s = " == "; break;
                case Op::Ne: s = " != "; break;
                case Op::Le: s = " <= "; break;
                case Op::Lt: s = " < "; break;
                case Op::Ge: s = " >= "; break;
                case Op::Gt: s = " > "; break;
                default: throw Fail("unknown binary operator");
            }
            gen_expr(*e.a, m, cur, os, depth);
            os << s;
            gen_expr(*e.b, m, cur, os, depth);
            break;
        }
        case K::Ternary:
            gen_expr(*e.a, m, cur, os, depth);
            os << " ? ";
            gen_expr(*e.b, m, cur, os, depth);
            os << " : ";
            gen_expr(*e.c, m, cur, os, depth);
            break;
    }
}

float eval_f(const mbg::Expr& e, const mbg::Model& m) { return (float)mbg::eval_const(e, m); }

// generator.cpp:57-82: `@logic ? v : 0` (up) or `@logic ? 0 : v` (down), v constant.
bool logic_ternary(const mbg::Expr* e, const mbg::Model& m, bool up, float& val) {
    if (!e || e->kind != mbg::Expr::Kind::Ternary) return false;
    if (e->a->kind != mbg::Expr::Kind::Alias || e->a->name != "@logic") return false;
    float l, r;
    try {
        l = eval_f(*e->b, m);
        r = eval_f(*e->c, m);
    } catch (const mbg::Error&) {
        return false;  // not a constant
    }
    const float zero = up ? r : l;
    val = up ? l : r;
    return zero == 0.f;
}

std::string generate(const mbg::Model& m) {
    const int n = (int)m.nodes.size();
    std::ostringstream ss;
    ss << "using uint8_t = unsigned char;\nusing uint32_t = unsigned int;\n\n";
    ss << "constexpr int state_size = " << n << ";\n";
    ss << "constexpr int state_words = " << (n + 31) / 32 << ";\n";
    ss << "constexpr bool discrete_time = " << (m.constant("discrete_time") != 0) << ";\n";
    ss << "constexpr float max_time = " << fstr((float)m.constant("max_time")) << ";\n";
    ss << "constexpr float time_tick = " << fstr((float)m.constant("time_tick")) << ";\n";
    ss << "using state_word_t = uint32_t;\n";
    for (int i = 0; i < n; ++i) {  // generate_node_transitions, generator.cpp:84-122
        const mbg::Node& nd = m.nodes[i];
        ss << "__device__ float " << nd.name << "_rate(const state_word_t* __restrict__ state)\n{\n";
        float up = 0, down = 0;
        const std::string self = "((state[" + std::to_string(i / 32) + "] & " + std::to_string(1u << (i % 32)) +
                                 "u) != 0)";
        if (logic_ternary(nd.attr("rate_up"), m, true, up) && logic_ternary(nd.attr("rate_down"), m, false, down)) {
            ss << "    const bool is_up = " << self << ";\n";
            ss << "    const bool logic = ";
            const mbg::Expr* lg = nd.attr("logic");
            if (!lg) throw Fail("node " + nd.name + " has no logic");
            gen_expr(*lg, m, i, ss);
            ss << ";\n";
            if (up == down)
                ss << "    return is_up == logic ? 0 : " << fstr(up) << ";\n";
            else
                ss << "    return is_up == logic ? 0 : (is_up ? " << fstr(down) << " : " << fstr(up) << ");\n";
        } else {
            ss << "    return " << self << " ?\n          (";
            gen_expr(*nd.attr("rate_down"), m, i, ss);
            ss << ")\n        : (";
            gen_expr(*nd.attr("rate_up"), m, i, ss);
            ss << ");\n";
        }
        ss << "}\n\n";
    }
    // generate_aggregate_function, generator.cpp:124-144
    ss << "__device__ float compute_transition_rates(float* __restrict__ transition_rates, const state_word_t* "
          "__restrict__ state)\n{\n    float sum = 0;\n    float tmp;\n";
    for (int i = 0; i < n; ++i)
        ss << "    tmp = " << m.nodes[i].name << "_rate(state);\n    transition_rates[" << i
           << "] = tmp;\n    sum += tmp;\n";
    ss << "    return sum;\n}\n";
    // generate_transition_entropy_function, generator.cpp:146-175
    ss << "__device__ float compute_transition_entropy(const float* __restrict__ transition_rates)\n{\n"
          "    float entropy = 0.f;\n    float non_internal_total_rate = 0.f;\n    float tmp_prob;\n";
    for (int i = 0; i < n; ++i)
        if (!m.is_internal(i)) ss << "    non_internal_total_rate += transition_rates[" << i << "];\n";
    ss << "    if (non_internal_total_rate == 0.f) return 0.f;\n";
    for (int i = 0; i < n; ++i)
        if (!m.is_internal(i))
            ss << "    tmp_prob = transition_rates[" << i << "] / non_internal_total_rate;\n"
               << "    entropy -= (tmp_prob == 0.f) ? 0.f : log2f(tmp_prob) * tmp_prob;\n";
    ss << "    return entropy;\n}\n";
    ss << "enum class trajectory_status : uint8_t { CONTINUE, FINISHED, FIXED_POINT };\n";
    // generate_simulate, generator.cpp:177-205
    ss << R"(
extern __device__ void simulate_inner(int trajectories_count, int state_size, int trajectory_limit, float time_tick,
    float max_time, bool discrete_time, state_word_t* __restrict__ last_states, float* __restrict__ last_times,
    void* __restrict__ rands, state_word_t* __restrict__ trajectory_states, float* __restrict__ trajectory_times,
    float* __restrict__ trajectory_transition_entropies, trajectory_status* __restrict__ trajectory_statuses,
    float* __restrict__ transition_rates, state_word_t* __restrict__ state);

extern "C" __global__ void simulate(int trajectories_count, int trajectory_limit, state_word_t* __restrict__ last_states,
    float* __restrict__ last_times, void* __restrict__ rands, state_word_t* __restrict__ trajectory_states,
    float* __restrict__ trajectory_times, float* __restrict__ trajectory_transition_entropies,
    trajectory_status* __restrict__ trajectory_statuses)
{
    float transition_rates[state_size];
    state_word_t state[state_words];
    simulate_inner(trajectories_count, state_size, trajectory_limit, time_tick, max_time, discrete_time, last_states,
                   last_times, rands, trajectory_states, trajectory_times, trajectory_transition_entropies,
                   trajectory_statuses, transition_rates, state);
}
)";
    // generate_non_internal_index, generator.cpp:207-235
    ss << "__device__ uint32_t get_non_internal_index(const state_word_t* __restrict__ state)\n{\n    return 0";
    int k = 0;
    for (int i = 0; i < n; ++i) {
        if (m.is_internal(i)) continue;
        ss << " | ((state[" << i / 32 << "] & " << (1u << (i % 32)) << "u)";
        const int shift = i % 32 - k++;
        if (shift > 0) ss << " >> " << shift;
        else if (shift < 0) ss << " << " << -shift;
        ss << ")";
    }
    ss << ";\n}\n";
    return ss.str();
}

std::vector<char> read_bin(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw Fail("cannot read " + path + " (build the reference kernels with baseline/refgpu/build_kernels.sh)");
    return std::vector<char>((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
}

// The linked module is loaded through the runtime's library API (the reference uses the driver's
// cuModuleLoadData / cuModuleGetFunction / cuLaunchKernel: the same load and launch), so that the
// harness needs no link against libcuda and loads on a machine without a driver.
struct Kernels {
    cudaLibrary_t lib = nullptr;
    cudaKernel_t init_random = nullptr, init_state = nullptr, simulate = nullptr, window = nullptr,
                 final_states = nullptr;
};

// kernel_compiler::compile_simulation, kernel_compiler.cpp:61-164: NVRTC with the reference's
// options (its default virtual architecture), then nvJitLink for sm_103. Needs no GPU.
std::vector<char> compile_and_link(const std::string& code, const std::string& dir) {
    nvrtcProgram prog;
    if (nvrtcCreateProgram(&prog, code.c_str(), "simulation.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS)
        throw Fail("nvrtcCreateProgram");
    const char* opts[] = {"-dlto", "--relocatable-device-code=true"};
    nvrtcResult r = nvrtcCompileProgram(prog, 2, opts);
    if (r != NVRTC_SUCCESS) {
        size_t ls = 0;
        nvrtcGetProgramLogSize(prog, &ls);
        std::string log(ls, '\0');
        nvrtcGetProgramLog(prog, &log[0]);
        nvrtcDestroyProgram(&prog);
        throw Fail("NVRTC: " + log.substr(0, 2000));
    }
    size_t lsz = 0;
    nvrtcGetLTOIRSize(prog, &lsz);
    std::vector<char> ltoir(lsz);
    nvrtcGetLTOIR(prog, ltoir.data());
    nvrtcDestroyProgram(&prog);

    nvJitLinkHandle h;
    const char* lopts[] = {"-dlto", "-arch=sm_103"};
    if (nvJitLinkCreate(&h, 2, lopts) != NVJITLINK_SUCCESS) throw Fail("nvJitLinkCreate");
    std::vector<std::vector<char>> fat;
    for (const char* f : {"simulation", "final_states", "window_average_small"}) {
        fat.push_back(read_bin(dir + "/" + f + ".fatbin"));
        if (nvJitLinkAddData(h, NVJITLINK_INPUT_FATBIN, fat.back().data(), fat.back().size(), f) != NVJITLINK_SUCCESS)
            throw Fail(std::string("nvJitLinkAddData ") + f);
    }
    if (nvJitLinkAddData(h, NVJITLINK_INPUT_LTOIR, ltoir.data(), ltoir.size(), "simulation_formulae.cu") !=
            NVJITLINK_SUCCESS ||
        nvJitLinkComplete(h) != NVJITLINK_SUCCESS) {
        size_t ls = 0;
        nvJitLinkGetErrorLogSize(h, &ls);
        std::string log(ls, '\0');
        if (ls) nvJitLinkGetErrorLog(h, &log[0]);
        nvJitLinkDestroy(&h);
        throw Fail("nvJitLink: " + log.substr(0, 2000));
    }
    size_t csz = 0;
    nvJitLinkGetLinkedCubinSize(h, &csz);
    std::vector<char> cubin(csz);
    nvJitLinkGetLinkedCubin(h, cubin.data());
    nvJitLinkDestroy(&h);
    return cubin;
}

void compile(const std::string& code, bool discrete, const std::string& dir, Kernels& k) {
    std::vector<char> cubin = compile_and_link(code, dir);
    ck(cudaLibraryLoadData(&k.lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0), "cudaLibraryLoadData");
    ck(cudaLibraryGetKernel(&k.init_random, k.lib, "initialize_random"), "initialize_random");
    ck(cudaLibraryGetKernel(&k.init_state, k.lib, "initialize_initial_state"), "initialize_initial_state");
    ck(cudaLibraryGetKernel(&k.simulate, k.lib, "simulate"), "simulate");
    ck(cudaLibraryGetKernel(&k.window, k.lib, discrete ? "window_average_small_discrete" : "window_average_small"),
       "window_average_small");
    ck(cudaLibraryGetKernel(&k.final_states, k.lib, "final_states"), "final_states");
}

// kernel_wrapper::run / run_shared, src/kernel.h:9-23: a launch on the legacy stream with the
// arguments passed by address.
template <class... A>
void launch(cudaKernel_t f, unsigned grid, unsigned block, unsigned smem, A... args) {
    void* p[] = {(void*)&args...};
    ck(cudaLaunchKernel((const void*)f, dim3(grid), dim3(block), p, smem, nullptr), "cudaLaunchKernel");
}

unsigned div_up(uint64_t a, uint64_t b) { return (unsigned)((a + b - 1) / b); }

// Flips in one launch: every trajectory writes slot 0 (its start time) and then a record per loop
// iteration; every record but the last is followed by a flip. Unused slots hold time 0.
__global__ void count_flips(int n, int len, const float* __restrict__ times, unsigned long long* __restrict__ out) {
    unsigned long long mine = 0;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        int r = 0;
        for (int j = 1; j < len; ++j) r += times[(size_t)t * len + j] != 0.f;
        mine += r > 0 ? (unsigned long long)(r - 1) : 0ull;
    }
    for (int d = 16; d > 0; d >>= 1) mine += __shfl_down_sync(0xffffffffu, mine, d);
    if ((threadIdx.x & 31) == 0 && mine) atomicAdd(out, mine);
}

struct IsFixed {
    __host__ __device__ bool operator()(uint8_t s) const { return s == FIXED_POINT; }
};
struct IsContinue {
    __host__ __device__ bool operator()(uint8_t s) const { return s == CONTINUE; }
};
struct DivBy {
    int w;
    __host__ __device__ int operator()(int i) const { return i / w; }
};

template <int W>
struct WState {
    uint32_t d[W];
    __host__ __device__ bool operator==(const WState& o) const {
        for (int i = 0; i < W; ++i)
            if (d[i] != o.d[i]) return false;
        return true;
    }
};
template <int W>
struct WLess {  // static_state_t order, fixed_states.cu:23-33: highest word first
    __device__ bool operator()(const WState<W>& a, const WState<W>& b) const {
        for (int i = W - 1; i >= 0; --i)
            if (a.d[i] != b.d[i]) return a.d[i] < b.d[i];
        return false;
    }
};

// fixed_states_stats<W>, fixed_states.cu:49-125
struct FixedBase {
    virtual ~FixedBase() = default;
    virtual void process(const uint32_t* last_states, const uint8_t* statuses, int n) = 0;
    std::map<std::vector<uint32_t>, int> result;
};

template <int W>
struct Fixed : FixedBase {
    void* tmp = nullptr;
    size_t tmp_bytes = 0;
    int* d_num = nullptr;
    WState<W>* copy = nullptr;
    WState<W>* uniq = nullptr;
    int* cnt = nullptr;
    ~Fixed() override {
        for (void* p : {tmp, (void*)d_num, (void*)copy, (void*)uniq, (void*)cnt})
            if (p) cudaFree(p);
    }
    void process(const uint32_t* last_states, const uint8_t* statuses, int n) override {
        const WState<W>* in = reinterpret_cast<const WState<W>*>(last_states);
        auto flags = thrust::make_transform_iterator(statuses, IsFixed());
        if (!tmp) {
            size_t a = 0, b = 0, c = 0;
            cub::DeviceSelect::Flagged(nullptr, a, in, flags, copy, d_num, n);
            cub::DeviceMergeSort::SortKeys(nullptr, b, copy, n, WLess<W>());
            cub::DeviceRunLengthEncode::Encode(nullptr, c, copy, uniq, cnt, d_num, n);
            tmp_bytes = std::max({a, b, c});
            ck(cudaMalloc(&tmp, tmp_bytes), "cudaMalloc");
            ck(cudaMalloc(&d_num, sizeof(int)), "cudaMalloc");
            ck(cudaMalloc(&copy, (size_t)n * sizeof(WState<W>)), "cudaMalloc");
            ck(cudaMalloc(&uniq, (size_t)n * sizeof(WState<W>)), "cudaMalloc");
            ck(cudaMalloc(&cnt, (size_t)n * sizeof(int)), "cudaMalloc");
        }
        ck(cub::DeviceSelect::Flagged(tmp, tmp_bytes, in, flags, copy, d_num, n), "DeviceSelect::Flagged");
        int fixed_count = 0;
        ck(cudaMemcpy(&fixed_count, d_num, sizeof(int), cudaMemcpyDeviceToHost), "cudaMemcpy");
        ck(cub::DeviceMergeSort::SortKeys(tmp, tmp_bytes, copy, fixed_count, WLess<W>()), "DeviceMergeSort");
        ck(cub::DeviceRunLengthEncode::Encode(tmp, tmp_bytes, copy, uniq, cnt, d_num, fixed_count),
           "DeviceRunLengthEncode");
        int nu = 0;
        ck(cudaMemcpy(&nu, d_num, sizeof(int), cudaMemcpyDeviceToHost), "cudaMemcpy");
        std::vector<WState<W>> hs(nu);
        std::vector<int> hc(nu);
        ck(cudaMemcpy(hs.data(), uniq, nu * sizeof(WState<W>), cudaMemcpyDeviceToHost), "cudaMemcpy");
        ck(cudaMemcpy(hc.data(), cnt, nu * sizeof(int), cudaMemcpyDeviceToHost), "cudaMemcpy");
        for (int i = 0; i < nu; ++i) result[std::vector<uint32_t>(hs[i].d, hs[i].d + W)] += hc[i];
    }
};

std::unique_ptr<FixedBase> make_fixed(int words) {
    switch (words) {  // the reference instantiates every width up to MAX_WORDS (fixed_states.cu:189-209)
        case 1: return std::make_unique<Fixed<1>>();
        case 2: return std::make_unique<Fixed<2>>();
        case 3: return std::make_unique<Fixed<3>>();
        case 5: return std::make_unique<Fixed<5>>();
        case 7: return std::make_unique<Fixed<7>>();
        case 32: return std::make_unique<Fixed<32>>();
        // 157 words (5000 nodes) does not build: CUB's run-length encode of 628-byte keys needs
        // 161 KB of static shared memory (ptxas: "uses too much shared data"), in the reference's
        // fixed_states.cu as here
        default: throw Fail("no fixed-point width instantiated for " + std::to_string(words) + " state words");
    }
}

}  // namespace

struct rg_result {
    int n = 0, words = 0, n_out = 0, windows = 0, discrete = 0;
    uint64_t n_traj = 0, transitions = 0;
    int iterations = 0;
    double sim_ms = 0, compile_ms = 0, count_ms = 0;
    std::vector<float> probs;     // windows x 2^n_out raw sums (time, or counts if discrete)
    std::vector<int> probs_discrete;
    std::vector<float> tr_entropy;
    std::vector<int> final_counts;
    std::map<std::vector<uint32_t>, int> fixed;
};

extern "C" {

// Runs the reference kernels on .bnd/.cfg texts (n_traj 0: the cfg's sample_count; seed: the cfg's
// seed_pseudorandom). Returns NULL on error with the message in err.
rg_result* rg_run(const char* bnd, const char* cfg, const char* fatbin_dir, uint64_t n_traj_override, char* err,
                  size_t errlen) {
    try {
        auto res = std::make_unique<rg_result>();
        mbg::Model m;
        mbg::parse_bnd(m, bnd, "model.bnd");
        mbg::parse_cfg(m, cfg, "model.cfg");
        const int n = (int)m.nodes.size();
        const int W = (n + 31) / 32;
        int n_out = 0;
        for (int i = 0; i < n; ++i) n_out += !m.is_internal(i);
        if (n_out > 20) throw Fail("the reference supports at most 20 output nodes (main.cpp:142-146)");
        const bool discrete = m.constant("discrete_time") != 0;
        const float max_time = (float)m.constant("max_time"), tick = (float)m.constant("time_tick");
        int n_traj = (int)m.constant("sample_count");
        if (n_traj_override) n_traj = (int)n_traj_override;
        const unsigned long long seed = (unsigned long long)m.constant("seed_pseudorandom");
        std::vector<float> istate;
        for (auto& nd : m.nodes) istate.push_back((float)nd.istate);
        res->n = n;
        res->words = W;
        res->n_out = n_out;
        res->discrete = discrete;
        res->n_traj = (uint64_t)n_traj;

        // compilation (main.cpp:38-52)
        ck(cudaSetDevice(0), "cudaSetDevice");
        ck(cudaFree(nullptr), "context");
        auto t0 = std::chrono::steady_clock::now();
        Kernels k;
        compile(generate(m), discrete, fatbin_dir, k);
        auto t1 = std::chrono::steady_clock::now();
        res->compile_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();

        // ---- "main> simulation" (main.cpp:54-83)
        ck(cudaDeviceSynchronize(), "sync");
        auto ts = std::chrono::steady_clock::now();
        const int batch_limit = std::min(1000000, n_traj);  // simulation_runner.cu:50
        const int len = 100;                                 // simulation_runner.cu:51
        // The reference's window kernel addresses a record as `traj_states + id * state_words` with
        // a 32-bit signed `id` (window_average_small.cu:66,70,116,120): at batch x 100 x words >=
        // 2^31 the product overflows and the kernel reads outside the record buffer (it faulted
        // the GPU at 1e6 trajectories of the 1000-node workload). Such runs are refused here.
        if ((uint64_t)batch_limit * len * (uint64_t)W >= (1ull << 31))
            throw Fail("the reference's window kernel would overflow its 32-bit record index: batch " +
                       std::to_string(batch_limit) + " x 100 records x " + std::to_string(W) +
                       " words >= 2^31 (window_average_small.cu:66,70); at most " +
                       std::to_string((unsigned long long)(((1ull << 31) - 1) / (100ull * W))) +
                       " trajectories at this model size");
        const uint32_t S = 1u << n_out;
        const int K = (int)std::ceil(max_time / tick);       // window_average_small.cpp:26
        res->windows = K;
        // statistics set-up
        int* d_final = nullptr;
        ck(cudaMalloc(&d_final, S * sizeof(int)), "cudaMalloc");
        ck(cudaMemset(d_final, 0, S * sizeof(int)), "cudaMemset");
        std::unique_ptr<FixedBase> fixed = make_fixed(W);
        float* d_th = nullptr;
        void* d_probs = nullptr;
        ck(cudaMalloc(&d_th, K * sizeof(float)), "cudaMalloc");
        ck(cudaMemset(d_th, 0, K * sizeof(float)), "cudaMemset");
        ck(cudaMalloc(&d_probs, (size_t)K * S * 4), "cudaMalloc");
        ck(cudaMemset(d_probs, 0, (size_t)K * S * 4), "cudaMemset");
        // run_simulation (simulation_runner.cu:54-180)
        uint32_t* d_last_states = nullptr;
        float* d_last_times = nullptr;
        curandState* d_rands = nullptr;
        float* d_istate = nullptr;
        uint32_t* d_traj_states = nullptr;
        float* d_traj_times = nullptr;
        float* d_traj_h = nullptr;
        uint8_t* d_status = nullptr;
        ck(cudaMalloc(&d_last_states, (size_t)batch_limit * W * 4), "cudaMalloc");
        ck(cudaMalloc(&d_last_times, (size_t)batch_limit * 4), "cudaMalloc");
        ck(cudaMalloc(&d_rands, (size_t)batch_limit * sizeof(curandState)), "cudaMalloc");
        ck(cudaMalloc(&d_istate, istate.size() * 4), "cudaMalloc");
        ck(cudaMalloc(&d_traj_states, (size_t)batch_limit * len * W * 4), "cudaMalloc");
        ck(cudaMalloc(&d_traj_times, (size_t)batch_limit * len * 4), "cudaMalloc");
        ck(cudaMalloc(&d_traj_h, (size_t)batch_limit * len * 4), "cudaMalloc");
        ck(cudaMalloc(&d_status, (size_t)batch_limit), "cudaMalloc");
        ck(cudaMemcpy(d_istate, istate.data(), istate.size() * 4, cudaMemcpyHostToDevice), "cudaMemcpy");
        launch(k.init_random, div_up(batch_limit, 256), 256, 0, batch_limit, seed, (void*)d_rands);
        launch(k.init_state, div_up(batch_limit, 256), 256, 0, batch_limit, n, (const float*)d_istate,
               d_last_states, d_last_times, (void*)d_rands);
        ck(cudaMemset(d_traj_times, 0, (size_t)batch_limit * len * 4), "cudaMemset");

        unsigned long long* d_flips = nullptr;
        ck(cudaMalloc(&d_flips, 8), "cudaMalloc");
        ck(cudaMemset(d_flips, 0, 8), "cudaMemset");
        cudaEvent_t c0, c1;
        ck(cudaEventCreate(&c0), "cudaEventCreate");
        ck(cudaEventCreate(&c1), "cudaEventCreate");
        double count_ms = 0;

        int remaining = n_traj;
        int in_batch = std::min(n_traj, batch_limit);
        int to_start = n_traj - in_batch;
        // window kernel shared memory (window_average_small.cpp:67-82)
        int smem = (int)sizeof(float) * K;
        bool use_shared = false;
        if (smem + sizeof(float) * (size_t)S * K < 10 * 1024) {
            smem += (int)(sizeof(float) * S * K);
            use_shared = true;
        }
        while (in_batch) {
            launch(k.simulate, div_up(in_batch, 256), 256, 0, in_batch, len, d_last_states, d_last_times,
                   (void*)d_rands, d_traj_states, d_traj_times, d_traj_h, (void*)d_status);
            ++res->iterations;
            // the harness's own transition count, timed apart
            ck(cudaEventRecord(c0, nullptr), "cudaEventRecord");
            count_flips<<<std::min(div_up(in_batch, 256), 4096u), 256>>>(in_batch, len, d_traj_times, d_flips);
            ck(cudaGetLastError(), "count_flips");
            ck(cudaEventRecord(c1, nullptr), "cudaEventRecord");
            // stats_composite::process_batch: final, fixed, window (main.cpp:65-74)
            launch(k.final_states, div_up(in_batch, 256), 256, 0, in_batch, W, (const uint32_t*)d_last_states,
                   (const uint8_t*)d_status, d_final);
            fixed->process(d_last_states, d_status, in_batch);
            launch(k.window, div_up((uint64_t)in_batch * (len - 1), 256), 256, (unsigned)smem, len, in_batch, W, S,
                   tick, K, use_shared, (const uint32_t*)d_traj_states, (const float*)d_traj_times,
                   (const float*)d_traj_h, d_probs, d_th);
            float cms = 0;
            ck(cudaEventSynchronize(c1), "cudaEventSynchronize");
            ck(cudaEventElapsedTime(&cms, c0, c1), "cudaEventElapsedTime");
            count_ms += cms;
            // prepare the next iteration: unfinished trajectories to the front
            {
                thrust::device_ptr<uint32_t> ls(d_last_states);
                thrust::device_ptr<uint8_t> st(d_status);
                auto stencil = thrust::make_permutation_iterator(
                    st, thrust::make_transform_iterator(thrust::counting_iterator<int>(0), DivBy{W}));
                thrust::stable_partition(thrust::device, ls, ls + (size_t)in_batch * W, stencil, IsContinue());
                auto zb = thrust::make_zip_iterator(thrust::make_tuple(thrust::device_ptr<float>(d_last_times),
                                                                       thrust::device_ptr<curandState>(d_rands)));
                const int still = (int)(thrust::partition(thrust::device, zb, zb + in_batch, st, IsContinue()) - zb);
                remaining -= in_batch - still;
                in_batch = still;
            }
            {
                const int add = std::min(batch_limit - in_batch, to_start);
                if (add) {
                    launch(k.init_state, div_up(add, 256), 256, 0, add, n, (const float*)d_istate,
                           d_last_states + (size_t)in_batch * W, d_last_times + in_batch, (void*)(d_rands + in_batch));
                    in_batch += add;
                    to_start -= add;
                }
            }
            ck(cudaMemset(d_traj_times, 0, (size_t)in_batch * len * 4), "cudaMemset");
        }
        // finalize (final_states.cpp:45-51, window_average_small.cpp:91-107)
        res->final_counts.resize(S);
        ck(cudaMemcpy(res->final_counts.data(), d_final, S * sizeof(int), cudaMemcpyDeviceToHost), "cudaMemcpy");
        if (discrete) {
            res->probs_discrete.resize((size_t)K * S);
            ck(cudaMemcpy(res->probs_discrete.data(), d_probs, (size_t)K * S * 4, cudaMemcpyDeviceToHost), "cudaMemcpy");
        } else {
            res->probs.resize((size_t)K * S);
            ck(cudaMemcpy(res->probs.data(), d_probs, (size_t)K * S * 4, cudaMemcpyDeviceToHost), "cudaMemcpy");
        }
        res->tr_entropy.resize(K);
        ck(cudaMemcpy(res->tr_entropy.data(), d_th, K * 4, cudaMemcpyDeviceToHost), "cudaMemcpy");
        for (void* p : {(void*)d_last_states, (void*)d_last_times, (void*)d_rands, (void*)d_istate,
                        (void*)d_traj_states, (void*)d_traj_times, (void*)d_traj_h, (void*)d_status})
            ck(cudaFree(p), "cudaFree");
        ck(cudaDeviceSynchronize(), "simulation");
        auto te = std::chrono::steady_clock::now();
        res->sim_ms = std::chrono::duration<double, std::milli>(te - ts).count() - count_ms;
        res->count_ms = count_ms;
        ck(cudaMemcpy(&res->transitions, d_flips, 8, cudaMemcpyDeviceToHost), "cudaMemcpy");
        res->fixed = fixed->result;
        fixed.reset();
        for (void* p : {(void*)d_final, (void*)d_th, d_probs, (void*)d_flips}) cudaFree(p);
        cudaEventDestroy(c0);
        cudaEventDestroy(c1);
        cudaLibraryUnload(k.lib);
        if (remaining != 0) throw Fail("batch loop ended with trajectories left");
        return res.release();
    } catch (const std::exception& e) {
        if (err && errlen) {
            std::strncpy(err, e.what(), errlen - 1);
            err[errlen - 1] = 0;
        }
        return nullptr;
    }
}

void rg_free(rg_result* r) { delete r; }

// Generates the model's rate source and links it with the reference kernels (no GPU needed).
// Returns the cubin size, 0 on error (message in err).
size_t rg_link_check(const char* bnd, const char* cfg, const char* fatbin_dir, char* err, size_t errlen) {
    try {
        mbg::Model m;
        mbg::parse_bnd(m, bnd, "model.bnd");
        mbg::parse_cfg(m, cfg, "model.cfg");
        return compile_and_link(generate(m), fatbin_dir).size();
    } catch (const std::exception& e) {
        if (err && errlen) {
            std::strncpy(err, e.what(), errlen - 1);
            err[errlen - 1] = 0;
        }
        return 0;
    }
}

// n, words, n_out, windows, discrete, iterations
void rg_dims(const rg_result* r, int* out6) {
    out6[0] = r->n;
    out6[1] = r->words;
    out6[2] = r->n_out;
    out6[3] = r->windows;
    out6[4] = r->discrete;
    out6[5] = r->iterations;
}

// sim_ms, compile_ms, count_ms, transitions, n_traj
void rg_times(const rg_result* r, double* out5) {
    out5[0] = r->sim_ms;
    out5[1] = r->compile_ms;
    out5[2] = r->count_ms;
    out5[3] = (double)r->transitions;
    out5[4] = (double)r->n_traj;
}

// Window sums (windows x 2^n_out floats; counts converted to float in discrete time) and TH sums.
void rg_windows(const rg_result* r, float* probs, float* th) {
    if (probs) {
        if (r->discrete)
            for (size_t i = 0; i < r->probs_discrete.size(); ++i) probs[i] = (float)r->probs_discrete[i];
        else
            std::memcpy(probs, r->probs.data(), r->probs.size() * 4);
    }
    if (th) std::memcpy(th, r->tr_entropy.data(), r->tr_entropy.size() * 4);
}

void rg_final(const rg_result* r, int* counts) {
    std::memcpy(counts, r->final_counts.data(), r->final_counts.size() * 4);
}

size_t rg_fixed_count(const rg_result* r) { return r->fixed.size(); }

// Fixed points in the reference's order (highest word first): states (count x words), counts.
void rg_fixed(const rg_result* r, uint32_t* states, int* counts) {
    std::vector<std::pair<std::vector<uint32_t>, int>> v(r->fixed.begin(), r->fixed.end());
    std::sort(v.begin(), v.end(), [](const auto& a, const auto& b) {
        for (size_t w = a.first.size(); w-- > 0;)
            if (a.first[w] != b.first[w]) return a.first[w] < b.first[w];
        return false;
    });
    size_t i = 0;
    for (auto& p : v) {
        std::memcpy(states + i * r->words, p.first.data(), r->words * 4);
        counts[i++] = p.second;
    }
}

}  // extern "C"
