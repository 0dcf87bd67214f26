// profile.cu — optional per-launch device timing with CUDA events (the library's tracing hook).
//
// When enabled, every kernel launch site records an event pair on the launching stream together with
// the launch's algorithmic bytes (one read and one write of each cell it updates).  stc_profile_report
// synchronises on the recorded events and returns, per kernel name, the launch count, the summed
// device time and the summed algorithmic bytes as a JSON object.
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "dispatch.h"
#include "profile.h"

namespace stc {

namespace {
struct Rec {
    std::string name;
    cudaEvent_t a, b;
    double bytes;
    double updates;
};
std::mutex g_mu;
bool g_on = false;
std::vector<Rec> g_recs;
std::vector<cudaEvent_t> g_pool;

cudaEvent_t get_event() {
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

bool profiling() { return g_on; }

void* prof_begin(cudaStream_t s) {
    if (!g_on) return nullptr;
    std::lock_guard<std::mutex> g(g_mu);
    Rec* r = new Rec();
    r->a = get_event();
    r->b = get_event();
    cudaEventRecord(r->a, s);
    return r;
}

void prof_end(void* token, cudaStream_t s, const char* name, double alg_bytes, double updates) {
    if (!token) return;
    Rec* r = (Rec*)token;
    cudaEventRecord(r->b, s);
    std::lock_guard<std::mutex> g(g_mu);
    r->name = name;
    r->bytes = alg_bytes;
    r->updates = updates;
    g_recs.push_back(*r);
    delete r;
}

}  // namespace stc

using namespace stc;

extern "C" int stc_profile_enable(int32_t on) {
    std::lock_guard<std::mutex> g(g_mu);
    for (auto& r : g_recs) {
        g_pool.push_back(r.a);
        g_pool.push_back(r.b);
    }
    g_recs.clear();
    g_on = on != 0;
    return STC_OK;
}

extern "C" int stc_profile_report(char* buf, size_t len) {
    std::lock_guard<std::mutex> g(g_mu);
    struct Acc { long long n = 0; double ms = 0, bytes = 0, updates = 0; };
    std::map<std::string, Acc> acc;
    for (auto& r : g_recs) {
        cudaError_t e = cudaEventSynchronize(r.b);
        if (e != cudaSuccess) return cuda_fail(e);
        float ms = 0.f;
        e = cudaEventElapsedTime(&ms, r.a, r.b);
        if (e != cudaSuccess) return cuda_fail(e);
        Acc& x = acc[r.name];
        x.n += 1;
        x.ms += ms;
        x.bytes += r.bytes;
        x.updates += r.updates;
    }
    std::string out = "{";
    bool first = true;
    for (auto& kv : acc) {
        char tmp[512];
        snprintf(tmp, sizeof(tmp), "%s\"%s\": {\"launches\": %lld, \"ms\": %.6f, \"alg_bytes\": %.1f, \"updates\": %.1f}",
                 first ? "" : ", ", kv.first.c_str(), kv.second.n, kv.second.ms, kv.second.bytes, kv.second.updates);
        out += tmp;
        first = false;
    }
    out += "}";
    if (!buf || len <= out.size()) return (int)out.size() + 1;
    memcpy(buf, out.c_str(), out.size() + 1);
    return STC_OK;
}
