/* prof.cpp -- event pool behind prof.h. */
#include "prof.h"

#include <atomic>
#include <mutex>
#include <vector>

namespace mg {

namespace {
struct Mark { int kid; cudaEvent_t a, b; };
std::mutex m;
std::atomic<int> enabled{0};
std::vector<cudaEvent_t> pool;
std::vector<Mark> marks;
size_t next_event = 0;
double total[K_NUM_KERNELS];
long long count[K_NUM_KERNELS];
const size_t kPool = 1 << 14;
}  // namespace

const char *kernel_name(int kid) {
    static const char *const n[K_NUM_KERNELS] = {"k_setup_xo", "k_setup_legacy", "k_setup_end", "k_points", "k_grid",
                                                 "k_chain_resolve", "k_blockgrid", "k_end_chunks", "k_end_lookup",
                                                 "k_ow_seed_climate", "k_ow_finish_tree", "k_batch", "k_search_cells",
                                                 "k_ow_search_first", "k_search_rest", "k_density", "k_batch_exact"};
    return (kid >= 0 && kid < K_NUM_KERNELS) ? n[kid] : "?";
}

static void drain_locked() {
    for (auto &mk : marks) {
        float ms = 0.0f;
        if (cudaEventSynchronize(mk.b) == cudaSuccess && cudaEventElapsedTime(&ms, mk.a, mk.b) == cudaSuccess) {
            total[mk.kid] += ms;
            count[mk.kid] += 1;
        }
    }
    marks.clear();
    next_event = 0;
}

void prof_mark(int kid, cudaStream_t st, bool end) {
    if (!enabled.load(std::memory_order_relaxed)) return;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return; /* graphs: not timed */
    std::lock_guard<std::mutex> lk(m);
    if (!end) {
        if (next_event + 2 > pool.size()) drain_locked();
        Mark mk{kid, pool[next_event], pool[next_event + 1]};
        next_event += 2;
        cudaEventRecord(mk.a, st);
        marks.push_back(mk);
    } else if (!marks.empty() && marks.back().kid == kid) {
        cudaEventRecord(marks.back().b, st);
    }
}

int prof_enable(int on) {
    std::lock_guard<std::mutex> lk(m);
    if (on) {
        if (pool.empty()) {
            pool.resize(kPool);
            for (auto &e : pool)
                if (cudaEventCreate(&e) != cudaSuccess) return -1;
        }
        marks.clear();
        next_event = 0;
        for (int k = 0; k < K_NUM_KERNELS; k++) { total[k] = 0.0; count[k] = 0; }
        enabled.store(1);
    } else {
        enabled.store(0);
        drain_locked();
    }
    return 0;
}

int prof_read(int kid, double *total_ms, long long *launches) {
    std::lock_guard<std::mutex> lk(m);
    drain_locked();
    if (kid < 0 || kid >= K_NUM_KERNELS) return -1;
    if (total_ms) *total_ms = total[kid];
    if (launches) *launches = count[kid];
    return 0;
}

}  // namespace mg
