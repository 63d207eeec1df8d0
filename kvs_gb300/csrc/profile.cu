// profile.cu -- per-kernel timing with CUDA events recorded on the stream
// each kernel is launched on (the tracing hook of the library; the
// reference's own timing is host-side kvs::Timer around whole calls).
#include <cstring>
#include <string>
#include <vector>

#include "context.h"

namespace kvsmc {

struct Profiler {
    bool on = false;
    struct Rec {
        const char* name;
        cudaEvent_t a, b;
    };
    std::vector<Rec> recs;
    std::vector<cudaEvent_t> pool;
    const char* open = nullptr;
    cudaEvent_t open_a = nullptr;
    // accumulated results
    std::vector<std::string> names;
    std::vector<uint64_t> launches;
    std::vector<double> ms;

    cudaEvent_t take()
    {
        if (!pool.empty()) {
            cudaEvent_t e = pool.back();
            pool.pop_back();
            return e;
        }
        cudaEvent_t e = nullptr;
        cudaEventCreate(&e);
        return e;
    }

    void collect()
    {
        for (Rec& r : recs) {
            float t = 0.0f;
            cudaEventSynchronize(r.b);
            cudaEventElapsedTime(&t, r.a, r.b);
            size_t i = 0;
            while (i < names.size() && names[i] != r.name) ++i;
            if (i == names.size()) {
                names.push_back(r.name);
                launches.push_back(0);
                ms.push_back(0.0);
            }
            launches[i] += 1;
            ms[i] += t;
            pool.push_back(r.a);
            pool.push_back(r.b);
        }
        recs.clear();
    }

    ~Profiler()
    {
        for (Rec& r : recs) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
        for (cudaEvent_t e : pool) cudaEventDestroy(e);
    }
};

void prof_begin(const Launch& L, const char* name)
{
    if (!L.prof || !L.prof->on) return;
    L.prof->open = name;
    L.prof->open_a = L.prof->take();
    cudaEventRecord(L.prof->open_a, L.stream);
}

void prof_end(const Launch& L)
{
    if (!L.prof || !L.prof->on || !L.prof->open) return;
    cudaEvent_t b = L.prof->take();
    cudaEventRecord(b, L.stream);
    L.prof->recs.push_back({L.prof->open, L.prof->open_a, b});
    L.prof->open = nullptr;
}

Profiler* profiler_create() { return new Profiler(); }
void profiler_destroy(Profiler* p) { delete p; }

}  // namespace kvsmc

extern "C" {

kvsmc_status kvsmc_profile_enable(kvsmc_context* ctx, int32_t on)
{
    if (!ctx) return KVSMC_ERR_INVALID_ARGUMENT;
    kvsmc::Profiler* p = ctx->prof;
    p->collect();
    p->names.clear();
    p->launches.clear();
    p->ms.clear();
    p->on = on != 0;
    return KVSMC_OK;
}

int32_t kvsmc_profile_read(kvsmc_context* ctx, int32_t max, const char** names, uint64_t* launches, double* ms)
{
    if (!ctx) return -1;
    kvsmc::Profiler* p = ctx->prof;
    p->collect();
    const int32_t n = (int32_t)p->names.size();
    for (int32_t i = 0; i < n && i < max; ++i) {
        if (names) names[i] = p->names[i].c_str();
        if (launches) launches[i] = p->launches[i];
        if (ms) ms[i] = p->ms[i];
    }
    return n;
}

}  // extern "C"
