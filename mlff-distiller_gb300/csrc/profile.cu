// Host side of the optional kernel timing (see profile.h).
#include <mutex>
#include <vector>
#include "common.cuh"
#include "profile.h"

namespace mlff {

namespace {
struct Region {
    int kind;
    cudaEvent_t a, b;
};
std::mutex g_mu;
bool g_on = false;
std::vector<Region> g_regions;     // recorded since mlff_profile_begin
std::vector<cudaEvent_t> g_pool;   // spare events
int64_t g_launches[PK_COUNT] = {};
thread_local int g_kind = PK_OTHER;

cudaEvent_t take_event() {
    if (!g_pool.empty()) {
        cudaEvent_t e = g_pool.back();
        g_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}
}  // namespace

bool prof_enabled() { return g_on; }

void prof_launch(int kind, int n) {
    if (g_on && kind >= 0 && kind < PK_COUNT) g_launches[kind] += n;
}

void prof_count_launch() { prof_launch(g_kind, 1); }

ProfScope::ProfScope(int k, cudaStream_t s) : kind(k), prev_kind(g_kind), st(s), slot(-1) {
    g_kind = k;
    if (!g_on) return;
    std::lock_guard<std::mutex> lk(g_mu);
    Region r{k, take_event(), take_event()};
    cudaEventRecord(r.a, s);
    g_regions.push_back(r);
    slot = (int)g_regions.size() - 1;
}

ProfScope::~ProfScope() {
    g_kind = prev_kind;
    if (slot < 0) return;
    std::lock_guard<std::mutex> lk(g_mu);
    cudaEventRecord(g_regions[slot].b, st);
}

}  // namespace mlff

using namespace mlff;

extern "C" int mlff_profile_begin(void) {
    std::lock_guard<std::mutex> lk(g_mu);
    for (auto& r : g_regions) {
        g_pool.push_back(r.a);
        g_pool.push_back(r.b);
    }
    g_regions.clear();
    for (auto& c : g_launches) c = 0;
    g_on = true;
    return MLFF_OK;
}

extern "C" int mlff_profile_end(double* ms_by_kind, int64_t* launches_by_kind, int32_t n_kinds) {
    std::lock_guard<std::mutex> lk(g_mu);
    g_on = false;
    for (int i = 0; i < n_kinds; ++i) {
        if (ms_by_kind) ms_by_kind[i] = 0.0;
        if (launches_by_kind) launches_by_kind[i] = i < PK_COUNT ? g_launches[i] : 0;
    }
    for (auto& r : g_regions) {
        cudaError_t e = cudaEventSynchronize(r.b);
        if (e != cudaSuccess) return cuda_status(e, "mlff_profile_end");
        float ms = 0.f;
        e = cudaEventElapsedTime(&ms, r.a, r.b);
        if (e != cudaSuccess) return cuda_status(e, "mlff_profile_end");
        if (ms_by_kind && r.kind < n_kinds) ms_by_kind[r.kind] += ms;
    }
    return MLFF_OK;
}
