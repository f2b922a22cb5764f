// Per-kernel-family device timing with CUDA events (measurement aid).

#include <cuda_runtime.h>

#include <atomic>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "tbgpu_internal.cuh"

namespace tbg {
namespace {

std::atomic<bool> g_enabled{false};
std::mutex g_mu;
struct Acc {
    int64_t launches = 0;
    double ms = 0.0;
    double work = 0.0;
};
std::map<std::string, Acc> g_table;
struct Pending {
    std::string name;
    double work;
    cudaEvent_t e0, e1;
};
thread_local std::vector<Pending> t_pending;

}  // namespace

bool timing_enabled() { return g_enabled.load(std::memory_order_relaxed); }

KTimer::KTimer(cudaStream_t s, const char* n, double work_flops) : st(s), name(n), work(work_flops) {
    if (!timing_enabled()) return;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        e0 = e1 = nullptr;
        return;
    }
    cudaEventRecord(e0, st);
}

KTimer::~KTimer() {
    if (!e0) return;
    cudaEventRecord(e1, st);
    t_pending.push_back({name, work, e0, e1});
}

void timing_flush() {
    if (t_pending.empty()) return;
    std::lock_guard<std::mutex> lk(g_mu);
    for (auto& p : t_pending) {
        float ms = 0.f;
        if (cudaEventSynchronize(p.e1) == cudaSuccess && cudaEventElapsedTime(&ms, p.e0, p.e1) == cudaSuccess) {
            Acc& a = g_table[p.name];
            a.launches += 1;
            a.ms += ms;
            a.work += p.work;
        }
        cudaEventDestroy(p.e0);
        cudaEventDestroy(p.e1);
    }
    t_pending.clear();
}

}  // namespace tbg

extern "C" int tbg_kernel_timing_enable(int enable) {
    tbg::g_enabled.store(enable != 0);
    return TBG_OK;
}

extern "C" int tbg_kernel_timing_read(char* names, int64_t* launches, double* total_ms, double* total_work,
                                      int max_entries, int reset) {
    tbg::timing_flush();
    std::lock_guard<std::mutex> lk(tbg::g_mu);
    int i = 0;
    for (auto& kv : tbg::g_table) {
        if (i >= max_entries) break;
        if (names) {
            std::strncpy(names + 64 * i, kv.first.c_str(), 63);
            names[64 * i + 63] = '\0';
        }
        if (launches) launches[i] = kv.second.launches;
        if (total_ms) total_ms[i] = kv.second.ms;
        if (total_work) total_work[i] = kv.second.work;
        ++i;
    }
    if (reset) tbg::g_table.clear();
    return i;
}

extern "C" int tbg_set_device(int device) {
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return tbg::cuda_error(e, "tbg_set_device");
    return TBG_OK;
}
