// NVRTC compilation of the per-model thread-per-trajectory kernel.
//
// Replaces src/kernel_compiler.cpp:61-164, which compiles the generated source to LTO IR and
// links it with nvJitLink against prebuilt fatbins of the fixed kernels. Here the fixed device
// code is compiled into the same NVRTC program from the project's own headers (embedded at build
// time), straight to an sm_103a cubin, loaded with the runtime's library API. Compiled cubins are
// cached in process and on disk (MBG_JIT_CACHE, default ~/.cache/mbg_gb300).
#include <cuda_runtime.h>
#include <nvrtc.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <sys/stat.h>
#include <unistd.h>

#include "sim_host.hpp"

namespace mbg {

#include "../_gen/jit_src.inc"  // kJitHeaders[], kJitHeaderCount

namespace {

std::mutex g_mu;
std::map<uint64_t, cudaLibrary_t> g_libs;

uint64_t fnv1a(const std::string& s) {
    uint64_t h = 1469598103934665603ull;
    for (unsigned char c : s) {
        h ^= c;
        h *= 1099511628211ull;
    }
    return h;
}

void mkdirs(const std::string& d) {
    std::string cur;
    std::stringstream ss(d);
    std::string part;
    if (!d.empty() && d[0] == '/') cur = "/";
    while (std::getline(ss, part, '/')) {
        if (part.empty()) continue;
        cur += part + "/";
        ::mkdir(cur.c_str(), 0755);
    }
}

bool read_bytes(const std::string& path, std::string& out) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    std::ostringstream ss;
    ss << f.rdbuf();
    out = ss.str();
    return !out.empty();
}

const char* kOpts[] = {"--gpu-architecture=sm_103a", "--std=c++17", "-lineinfo", "-DMBG_JIT=1"};

std::string compile(const std::string& src) {
    nvrtcProgram prog;
    if (nvrtcCreateProgram(&prog, src.c_str(), "mbg_model.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS)
        throw JitError("nvrtcCreateProgram failed");
    nvrtcResult rc = nvrtcCompileProgram(prog, (int)(sizeof kOpts / sizeof kOpts[0]), kOpts);
    size_t log_size = 0;
    nvrtcGetProgramLogSize(prog, &log_size);
    std::string log(log_size, '\0');
    if (log_size > 1) nvrtcGetProgramLog(prog, &log[0]);
    if (rc != NVRTC_SUCCESS) {
        nvrtcDestroyProgram(&prog);
        throw JitError(std::string("NVRTC compilation failed: ") + nvrtcGetErrorString(rc) + "\n" + log);
    }
    size_t n = 0;
    nvrtcGetCUBINSize(prog, &n);
    std::string cubin(n, '\0');
    nvrtcGetCUBIN(prog, &cubin[0]);
    nvrtcDestroyProgram(&prog);
    return cubin;
}

}  // namespace

std::string cache_dir() {
    const char* e = std::getenv("MBG_JIT_CACHE");
    if (e && *e) return e;
    const char* home = std::getenv("HOME");
    return std::string(home && *home ? home : "/tmp") + "/.cache/mbg_gb300";
}

void cache_mkdirs(const std::string& d) { mkdirs(d); }

double jit_compile_only(const std::string& model_src) {
    std::string src;
    for (int i = 0; i < kJitHeaderCount; ++i) src += kJitHeaders[i];
    src += model_src;
    auto t0 = std::chrono::steady_clock::now();
    compile(src);
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

void* jit_thread_kernel(const std::string& model_src, double& compile_ms, bool window_hash) {
    // the window-table variant is chosen when the kernel is compiled (sim_core.cuh: MBG_WINDOW_HASH)
    std::string src = window_hash ? "#define MBG_WINDOW_HASH 1\n" : "";
    for (int i = 0; i < kJitHeaderCount; ++i) src += kJitHeaders[i];
    src += model_src;
    int major = 0, minor = 0;
    nvrtcVersion(&major, &minor);
    std::string key_text = src;
    for (const char* o : kOpts) key_text += o;
    key_text += std::to_string(major) + "." + std::to_string(minor);
    const uint64_t key = fnv1a(key_text);
    compile_ms = 0;

    std::lock_guard<std::mutex> lock(g_mu);
    cudaLibrary_t lib = nullptr;
    auto it = g_libs.find(key);
    if (it != g_libs.end()) {
        lib = it->second;
    } else {
        char name[32];
        std::snprintf(name, sizeof name, "%016llx.cubin", (unsigned long long)key);
        const std::string dir = cache_dir(), path = dir + "/" + name;
        std::string cubin;
        if (!read_bytes(path, cubin)) {
            auto t0 = std::chrono::steady_clock::now();
            cubin = compile(src);
            compile_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
            mkdirs(dir);
            const std::string tmp = path + ".tmp" + std::to_string((unsigned long long)::getpid());
            {
                std::ofstream f(tmp, std::ios::binary);
                f.write(cubin.data(), (std::streamsize)cubin.size());
            }
            std::rename(tmp.c_str(), path.c_str());
        }
        cudaError_t e = cudaLibraryLoadData(&lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
        if (e != cudaSuccess) throw CudaError(std::string("cudaLibraryLoadData: ") + cudaGetErrorString(e));
        g_libs[key] = lib;
    }
    cudaKernel_t k = nullptr;
    cudaError_t e = cudaLibraryGetKernel(&k, lib, "mbg_sim_thread");
    if (e != cudaSuccess) throw CudaError(std::string("cudaLibraryGetKernel: ") + cudaGetErrorString(e));
    return (void*)k;
}

}  // namespace mbg
