// Host-side parallel loop over independent items (the nodes of a model being compiled, the
// instances of a batch being laid out).
#pragma once

#include <algorithm>
#include <atomic>
#include <exception>
#include <mutex>
#include <thread>
#include <vector>

namespace mbg {

// f(i, scratch) for every i in [0, n) on up to 16 host threads (one thread when n < serial_below),
// each thread with its own value-initialised Scratch. An exception in f is rethrown here: the one of
// the lowest-numbered item when several fail, as a single thread would have thrown it.
template <class Scratch, class F>
void parallel_items(int n, int serial_below, F&& f) {
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const int threads = n < serial_below ? 1 : (int)std::min<unsigned>(hw, 16u);
    std::atomic<int> next{0};
    std::mutex mu;
    int err_item = n;
    std::exception_ptr err;
    auto worker = [&]() {
        Scratch sc{};
        for (int i; (i = next.fetch_add(1)) < n;) {
            try {
                f(i, sc);
            } catch (...) {
                std::lock_guard<std::mutex> lock(mu);
                if (i < err_item) {
                    err_item = i;
                    err = std::current_exception();
                }
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; ++t) pool.emplace_back(worker);
    worker();
    for (auto& th : pool) th.join();
    if (err) std::rethrow_exception(err);
}

}  // namespace mbg
