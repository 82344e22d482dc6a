// Process-wide cache of device and pinned host blocks (devmem.hpp).
#include "devmem.hpp"

#include <cuda.h>  // driver types only: the two driver calls come through cudaGetDriverEntryPoint
#include <cuda_runtime.h>

#include <cstdlib>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <unordered_map>

#include "sim_host.hpp"

namespace mbg {

bool current_context_id(unsigned long long* id) {
    using GetCurrentFn = CUresult (*)(CUcontext*);
    using GetIdFn = CUresult (*)(CUcontext, unsigned long long*);
    static GetCurrentFn get_current = nullptr;
    static GetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<GetCurrentFn>(p);
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<GetIdFn>(p);
    });
    CUcontext ctx = nullptr;
    if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx) return false;
    return get_id(ctx, id) == CUDA_SUCCESS && *id != 0;
}

namespace {

// (context id, bytes, pinned): context 0 = unknown (never cached)
using Key = std::tuple<unsigned long long, size_t, bool>;

struct Cache {
    std::mutex mu;
    std::multimap<Key, void*> spare;
    std::unordered_map<void*, Key> live;
    size_t spare_dev = 0, spare_pinned = 0;
};

Cache& cache() {
    static Cache* c = new Cache();  // never destroyed: blocks may be freed from static destructors
    return *c;
}

void* take_spare(const Key& k) {
    Cache& c = cache();
    std::lock_guard<std::mutex> lock(c.mu);
    auto it = c.spare.find(k);
    if (it == c.spare.end()) return nullptr;
    void* p = it->second;
    c.spare.erase(it);
    (std::get<2>(k) ? c.spare_pinned : c.spare_dev) -= std::get<1>(k);
    c.live.emplace(p, k);
    return p;
}

bool cache_enabled() {
    static const bool on = [] {
        const char* e = std::getenv("MBG_DEVICE_CACHE");
        return !(e && e[0] == '0');
    }();
    return on;
}

void* alloc(size_t bytes, bool pinned, const char* what) {
    if (bytes == 0) bytes = 1;
    unsigned long long ctx = 0;
    bool have = cache_enabled() && current_context_id(&ctx);
    if (have)
        if (void* p = take_spare(Key{ctx, bytes, pinned})) return p;
    void* p = nullptr;
    cudaError_t e = pinned ? cudaMallocHost(&p, bytes) : cudaMalloc(&p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();  // the failed allocation's own error
        throw NoMemError(std::string(pinned ? "cudaMallocHost" : "cudaMalloc") + " of " + std::to_string(bytes) +
                         " bytes (" + what + "): " + cudaGetErrorString(e));
    }
    if (!have && cache_enabled()) have = current_context_id(&ctx);  // the allocation may have created the context
    Cache& c = cache();
    std::lock_guard<std::mutex> lock(c.mu);
    c.live.emplace(p, Key{have ? ctx : 0ull, bytes, pinned});
    return p;
}

void release(void* p, bool pinned) {
    if (!p) return;
    Cache& c = cache();
    {
        std::lock_guard<std::mutex> lock(c.mu);
        auto it = c.live.find(p);
        if (it != c.live.end()) {
            const Key k = it->second;
            c.live.erase(it);
            size_t& spare = pinned ? c.spare_pinned : c.spare_dev;
            const size_t cap = pinned ? kPinnedCacheBytes : kDevCacheBytes;
            if (std::get<0>(k) != 0 && spare + std::get<1>(k) <= cap) {
                c.spare.emplace(k, p);
                spare += std::get<1>(k);
                return;
            }
        }
    }
    if (pinned) cudaFreeHost(p);
    else cudaFree(p);
}

}  // namespace

void* dev_alloc(size_t bytes, const char* what) { return alloc(bytes, false, what); }
void dev_free(void* p) { release(p, false); }
void* pinned_alloc(size_t bytes) { return alloc(bytes, true, "pinned host block"); }
void pinned_free(void* p) { release(p, true); }

}  // namespace mbg
