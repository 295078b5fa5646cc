// vgb::parallel_for_each and the entry-point pattern (function-try-block + status_of_exception),
// host only.  Prints one line per check; exits non-zero on the first failure.
#include <atomic>
#include <chrono>
#include <cstdio>
#include <stdexcept>
#include <thread>
#include <vector>

#include "../../vira_gb300/csrc/vgb_internal.h"

static vgb_status entry(uint32_t n, uint32_t throw_at, std::atomic<uint32_t>& done, std::string& err) try {
    vgb::parallel_for_each(n, [&](uint32_t k) {
        if (k == throw_at) throw std::bad_alloc();
        std::this_thread::sleep_for(std::chrono::milliseconds(20));  // still running when k throws
        done.fetch_add(1);
    });
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(&err);
}

int main() {
    std::atomic<uint32_t> done{0};
    std::string err;
    // every body runs once
    std::vector<std::atomic<int>> hits(16);
    vgb::parallel_for_each(16, [&](uint32_t k) { hits[k].fetch_add(1); });
    for (auto& h : hits)
        if (h.load() != 1) { std::printf("FAIL each body once\n"); return 1; }
    std::printf("each body once\n");
    // a worker's exception reaches the caller after every other body has finished
    vgb_status s = entry(8, 3, done, err);
    if (s != VGB_ERR_OUT_OF_MEMORY || done.load() != 7 || err != "host allocation failed") {
        std::printf("FAIL worker exception: status %d, done %u, '%s'\n", (int)s, done.load(), err.c_str());
        return 1;
    }
    std::printf("worker exception -> status %d after %u bodies\n", (int)s, done.load());
    // the caller's own body (k = 0) throwing is handled the same way
    done = 0;
    s = entry(4, 0, done, err);
    if (s != VGB_ERR_OUT_OF_MEMORY || done.load() != 3) { std::printf("FAIL caller exception\n"); return 1; }
    std::printf("caller exception -> status %d after %u bodies\n", (int)s, done.load());
    // a std::exception other than bad_alloc keeps its message and is an internal error
    std::string msg;
    s = [&]() -> vgb_status {
        try {
            vgb::parallel_for_each(2, [](uint32_t k) { if (k == 1) throw std::runtime_error("bad block"); });
            return VGB_OK;
        } catch (...) {
            return vgb::status_of_exception(&msg);
        }
    }();
    if (s != VGB_ERR_INTERNAL || msg != "bad block") { std::printf("FAIL runtime_error\n"); return 1; }
    std::printf("runtime_error -> status %d '%s'\n", (int)s, msg.c_str());
    return 0;
}
