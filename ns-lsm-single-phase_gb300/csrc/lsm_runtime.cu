// lsm_runtime.cu -- launch bookkeeping shared by every kernel translation
// unit: the launch counter and the optional per-kernel CUDA-event timer.
//
// The timer records an event pair on the launching stream around each
// launch while it is enabled (lsm_profile_enable), and folds the pairs into
// per-kernel totals when they are read; with it disabled a launch costs one
// branch.
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "lsm_c.h"
#include "lsm_kernels.h"

namespace lsm {

unsigned long long g_launches = 0;

namespace {
struct Pending { std::string name; cudaEvent_t a, b; };
struct Acc { long long n = 0; double ms = 0.0; };
std::mutex g_mu;
bool g_on = false;
std::vector<Pending> g_pending;
std::map<std::string, Acc> g_acc;
std::vector<cudaEvent_t> g_free;

cudaEvent_t take_event() {
    if (!g_free.empty()) { cudaEvent_t e = g_free.back(); g_free.pop_back(); return e; }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}

void fold() {
    for (auto& p : g_pending) {
        cudaEventSynchronize(p.b);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, p.a, p.b);
        auto& a = g_acc[p.name];
        a.n += 1;
        a.ms += ms;
        g_free.push_back(p.a);
        g_free.push_back(p.b);
    }
    g_pending.clear();
}
}  // namespace

ProfScope::ProfScope(const char* name, cudaStream_t s) : name_(name), s_(s) {
    // launches recorded into a CUDA graph are counted when the graph is replayed
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s_, &cs) != cudaSuccess) cudaGetLastError();
    if (cs != cudaStreamCaptureStatusNone) return;
    ++g_launches;
    if (!g_on) return;
    std::lock_guard<std::mutex> lk(g_mu);
    a_ = take_event();
    b_ = take_event();
    cudaEventRecord((cudaEvent_t)a_, s_);
    active_ = true;
}

ProfScope::~ProfScope() {
    if (!active_) return;
    std::lock_guard<std::mutex> lk(g_mu);
    cudaEventRecord((cudaEvent_t)b_, s_);
    g_pending.push_back({name_, (cudaEvent_t)a_, (cudaEvent_t)b_});
    if (g_pending.size() > 4096) fold();
}

}  // namespace lsm

extern "C" {

int lsm_profile_enable(int on) {
    std::lock_guard<std::mutex> lk(lsm::g_mu);
    lsm::g_on = on != 0;
    return LSM_OK;
}

int lsm_profile_reset(void) {
    std::lock_guard<std::mutex> lk(lsm::g_mu);
    lsm::fold();
    lsm::g_acc.clear();
    return LSM_OK;
}

int lsm_profile_count(void) {
    std::lock_guard<std::mutex> lk(lsm::g_mu);
    lsm::fold();
    return (int)lsm::g_acc.size();
}

int lsm_profile_entry(int i, char* name, int name_len, long long* launches, double* total_ms) {
    std::lock_guard<std::mutex> lk(lsm::g_mu);
    lsm::fold();
    if (i < 0 || i >= (int)lsm::g_acc.size()) return LSM_ERR_BAD_PARAM;
    auto it = lsm::g_acc.begin();
    std::advance(it, i);
    if (name && name_len > 0) {
        size_t n = it->first.copy(name, (size_t)name_len - 1);
        name[n] = '\0';
    }
    if (launches) *launches = it->second.n;
    if (total_ms) *total_ms = it->second.ms;
    return LSM_OK;
}

}  // extern "C"
