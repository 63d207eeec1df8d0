// server.cu -- kvsmc_server: a request loop over resident volumes with
// continuous batching (see include/kvsmc.h).
//
// Clients push requests into one pending queue.  Each worker thread owns a
// context (its own stream, scratch and auxiliary streams) and loops: take
// every pending request up to max_batch, count them in one fused pass,
// admit them against the output budget, allocate their outputs from the
// server's stream-ordered memory pool, emit them in one fused pass, publish
// the completions.  With several workers, one batch counts while another
// emits, so new arrivals never wait for a whole batch in flight.  The
// budget counts the bytes of results the clients have not released yet; a
// batch that does not fit waits for releases (its requests that could
// never fit alone complete with KVSMC_ERR_BUDGET).
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "batch.h"

namespace {

struct Pending {
    uint64_t ticket;
    kvsmc_volume* vol;
    kvsmc_params params;
    double t_submit;
};

struct Held {
    float* coords;
    float* normals;
    uint64_t bytes;
};

constexpr uint64_t kBytesPerTriangle = 48;   // 9 coords + 3 normals, float

}  // namespace

struct kvsmc_server {
    kvsmc_context* ctx = nullptr;       // owner: device, min/max passes at submit
    kvsmc_server_config cfg{};
    std::vector<kvsmc_context*> wctx;   // one per worker
    std::vector<std::thread> threads;
    cudaMemPool_t pool = nullptr;       // outputs of admitted requests
    cudaStream_t free_stream = nullptr; // stream-ordered frees on release
    std::mutex mu;                      // queues, budget, counters
    std::mutex mm_mu;                   // min/max passes and first-use waits on the owner context
    std::condition_variable cv_work, cv_done, cv_budget;
    std::deque<Pending> pending;
    std::deque<kvsmc_completion> done;
    std::unordered_map<uint64_t, Held> held;
    std::unordered_set<kvsmc_volume*> seen;   // volumes whose upload is known to be complete
    uint64_t next_ticket = 1;
    uint64_t in_use = 0, peak = 0, submitted = 0, completed = 0, batches = 0, budget_waits = 0;
    bool stop = false;
    std::chrono::steady_clock::time_point t0;

    double now() const
    {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
};

namespace {

using kvsmc_host::Item;
using kvsmc_host::StreamBatch;

void free_outputs(kvsmc_server* S, float* coords, float* normals)
{
    if (coords) cudaFreeAsync(coords, S->free_stream);
    if (normals) cudaFreeAsync(normals, S->free_stream);
}

void worker(kvsmc_server* S, int w)
{
    kvsmc_context* ctx = S->wctx[w];
    cudaSetDevice(ctx->device);
    const uint64_t budget = S->cfg.output_budget_bytes;
    for (;;) {
        std::vector<Pending> reqs;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            S->cv_work.wait(lk, [&] { return S->stop || !S->pending.empty(); });
            if (S->pending.empty()) return;   // stopping, and nothing left
            const size_t n = std::min(S->pending.size(), (size_t)S->cfg.max_batch);
            reqs.assign(S->pending.begin(), S->pending.begin() + n);
            S->pending.erase(S->pending.begin(), S->pending.begin() + n);
            ++S->batches;
        }
        const double t_start = S->now();
        const size_t n = reqs.size();
        std::vector<Item> items(n);
        std::vector<Item*> live;
        for (size_t i = 0; i < n; ++i) {
            items[i].vol = reqs[i].vol;
            items[i].params = reqs[i].params;
            items[i].status = kvsmc_host::prepare(ctx, items[i]);   // min/max are cached or preset: no GPU work
            if (!items[i].status && items[i].extracted) live.push_back(&items[i]);
        }

        // count, in one fused pass
        StreamBatch b;
        b.ctx = ctx;
        b.items = live;
        kvsmc_status st = KVSMC_OK;
        if (!live.empty()) {
            st = b.plan();
            if (!st) st = b.count();
        }

        // admission: what this batch's results will hold until released
        uint64_t need = 0;
        std::vector<Item*> admit, later;
        if (!st) {
            for (Item* it : live) {
                const uint64_t bytes = it->sizes.ntriangles * kBytesPerTriangle;
                if (bytes > budget) {
                    it->status = kvsmc_host::fail(ctx, KVSMC_ERR_BUDGET, "result of %llu bytes exceeds the budget",
                                                  (unsigned long long)bytes);
                } else if (need + bytes > budget) {
                    later.push_back(it);   // the batch alone would exceed the budget: run it again later
                } else {
                    need += bytes;
                    admit.push_back(it);
                }
            }
        }
        if (need) {
            std::unique_lock<std::mutex> lk(S->mu);
            if (S->in_use + need > budget) ++S->budget_waits;
            S->cv_budget.wait(lk, [&] { return S->in_use + need <= budget || S->stop; });
            S->in_use += need;
            S->peak = std::max(S->peak, S->in_use);
        }

        // outputs (stream-ordered) and emit, in one fused pass
        std::vector<float*> coords(n, nullptr), normals(n, nullptr);
        uint64_t granted = need;
        for (Item* it : admit) {
            const size_t i = (size_t)(it - items.data());
            const uint64_t t = it->sizes.ntriangles;
            it->emit = true;
            if (t == 0) continue;
            cudaError_t e = cudaMallocFromPoolAsync(reinterpret_cast<void**>(&coords[i]), 36 * t, S->pool, ctx->stream);
            if (e == cudaSuccess)
                e = cudaMallocFromPoolAsync(reinterpret_cast<void**>(&normals[i]), 12 * t, S->pool, ctx->stream);
            if (e != cudaSuccess) {
                cudaGetLastError();
                it->status = kvsmc_host::fail(ctx, KVSMC_ERR_OUT_OF_MEMORY, "output allocation: %s",
                                              cudaGetErrorString(e));
                continue;
            }
            it->d_coords = coords[i];
            it->coords_cap = 9 * t;
            it->d_normals = normals[i];
            it->normals_cap = 3 * t;
        }
        if (!st && !admit.empty()) {
            st = b.emit();
            if (!st) st = b.finish();
        }
        if (st)
            for (Item* it : live)
                if (!it->status) it->status = st;

        // publish
        const double t_done = S->now();
        std::unique_lock<std::mutex> lk(S->mu);
        // deferred requests go back to the front, in order, for a later batch
        for (auto r = later.rbegin(); r != later.rend(); ++r) S->pending.push_front(reqs[(size_t)(*r - items.data())]);
        for (size_t i = 0; i < n; ++i) {
            if (std::find(later.begin(), later.end(), &items[i]) != later.end()) continue;
            kvsmc_completion c;
            std::memset(&c, 0, sizeof c);
            c.ticket = reqs[i].ticket;
            c.status = items[i].status;
            c.batch_size = (int32_t)n;
            c.sizes = items[i].sizes;
            c.submit_s = reqs[i].t_submit;
            c.start_s = t_start;
            c.done_s = t_done;
            const uint64_t bytes = coords[i] ? items[i].sizes.ntriangles * kBytesPerTriangle : 0;
            if (c.status || !coords[i]) {
                free_outputs(S, coords[i], normals[i]);
            } else {
                c.d_coords = coords[i];
                c.d_normals = normals[i];
                S->held[c.ticket] = Held{coords[i], normals[i], bytes};
                granted -= bytes;
            }
            S->done.push_back(c);
            ++S->completed;
        }
        // budget reserved for requests that hold nothing (failed, empty) goes back now
        S->in_use -= granted;
        S->cv_done.notify_all();
        if (granted) S->cv_budget.notify_all();
        if (!later.empty()) S->cv_work.notify_one();
    }
}

}  // namespace

extern "C" {

kvsmc_status kvsmc_server_create(kvsmc_context* ctx, const kvsmc_server_config* cfg, kvsmc_server** out)
{
    if (!ctx || !out) return KVSMC_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return kvsmc_host::fail(ctx, KVSMC_ERR_CUDA, "server: cudaSetDevice");
    kvsmc_server* S = new kvsmc_server();
    S->ctx = ctx;
    if (cfg) S->cfg = *cfg;
    if (S->cfg.output_budget_bytes == 0) S->cfg.output_budget_bytes = 40ull << 30;
    if (S->cfg.max_batch <= 0) S->cfg.max_batch = 256;
    if (S->cfg.workers <= 0) S->cfg.workers = 3;
    S->t0 = std::chrono::steady_clock::now();
    cudaMemPoolProps props;
    std::memset(&props, 0, sizeof props);
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = ctx->device;
    cudaError_t e = cudaMemPoolCreate(&S->pool, &props);
    if (e == cudaSuccess) {
        // keep freed blocks mapped for reuse, up to the budget
        uint64_t keep = S->cfg.output_budget_bytes;
        e = cudaMemPoolSetAttribute(S->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&S->free_stream, cudaStreamNonBlocking);
    kvsmc_status st = e == cudaSuccess ? KVSMC_OK : KVSMC_ERR_CUDA;
    for (int w = 0; w < S->cfg.workers && !st; ++w) {
        kvsmc_context* c = nullptr;
        st = kvsmc_create(ctx->device, &c);
        if (!st) S->wctx.push_back(c);
    }
    if (st) {
        for (kvsmc_context* c : S->wctx) kvsmc_destroy(c);
        if (S->free_stream) cudaStreamDestroy(S->free_stream);
        if (S->pool) cudaMemPoolDestroy(S->pool);
        cudaGetLastError();
        delete S;
        return kvsmc_host::fail(ctx, st, "server: set-up failed");
    }
    for (int w = 0; w < S->cfg.workers; ++w) S->threads.emplace_back(worker, S, w);
    *out = S;
    return KVSMC_OK;
}

kvsmc_status kvsmc_server_submit(kvsmc_server* S, kvsmc_volume* vol, const kvsmc_params* p, uint64_t* ticket)
{
    if (!S || !vol || !p || !ticket) return KVSMC_ERR_INVALID_ARGUMENT;
    Item it;
    it.vol = vol;
    it.params = *p;
    if (!kvsmc_host::stream_eligible(S->wctx[0], it))
        return kvsmc_host::fail(S->ctx, KVSMC_ERR_INVALID_ARGUMENT,
                                "server: only duplicated-mode requests on 8/16-bit or float32 volumes of width "
                                "<= 4097 are served");
    {
        std::lock_guard<std::mutex> lk(S->mm_mu);
        if (!S->seen.count(vol) || (!p->has_minmax && !vol->has_minmax)) {
            if (cudaSetDevice(S->ctx->device) != cudaSuccess) return KVSMC_ERR_CUDA;
            if (!p->has_minmax) {
                kvsmc_status st = kvsmc_host::volume_minmax(S->ctx, vol);
                if (st) return st;
            }
            // the workers' streams read the volume (and its brick table): the
            // owner stream's upload must be done
            if (cudaStreamSynchronize(S->ctx->stream) != cudaSuccess)
                return kvsmc_host::fail(S->ctx, KVSMC_ERR_CUDA, "server: synchronize");
            S->seen.insert(vol);
        }
    }
    std::lock_guard<std::mutex> lk(S->mu);
    *ticket = S->next_ticket++;
    S->pending.push_back(Pending{*ticket, vol, *p, S->now()});
    ++S->submitted;
    S->cv_work.notify_one();
    return KVSMC_OK;
}

int32_t kvsmc_server_poll(kvsmc_server* S, kvsmc_completion* out, int32_t max, int32_t timeout_ms)
{
    if (!S || !out || max <= 0) return 0;
    std::unique_lock<std::mutex> lk(S->mu);
    if (timeout_ms > 0)
        S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return !S->done.empty(); });
    int32_t k = 0;
    while (k < max && !S->done.empty()) {
        out[k++] = S->done.front();
        S->done.pop_front();
    }
    return k;
}

kvsmc_status kvsmc_server_release(kvsmc_server* S, uint64_t ticket)
{
    if (!S) return KVSMC_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(S->mu);
    auto f = S->held.find(ticket);
    if (f == S->held.end()) return KVSMC_OK;   // nothing held (empty, failed or already released)
    cudaSetDevice(S->ctx->device);
    free_outputs(S, f->second.coords, f->second.normals);
    S->in_use -= f->second.bytes;
    S->held.erase(f);
    S->cv_budget.notify_all();
    return KVSMC_OK;
}

kvsmc_status kvsmc_server_stats(kvsmc_server* S, uint64_t* out7)
{
    if (!S || !out7) return KVSMC_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(S->mu);
    uint64_t launches = 0;
    for (kvsmc_context* c : S->wctx) launches += c->launches;
    const uint64_t v[7] = {S->submitted, S->completed, S->batches, launches, S->in_use, S->peak, S->budget_waits};
    std::memcpy(out7, v, sizeof v);
    return KVSMC_OK;
}

kvsmc_status kvsmc_copy_to_host(kvsmc_context* ctx, void* host, const void* device, uint64_t bytes)
{
    if (!ctx || (bytes && (!host || !device))) return KVSMC_ERR_INVALID_ARGUMENT;
    if (!bytes) return KVSMC_OK;
    KVSMC_CUDA(ctx, cudaSetDevice(ctx->device));
    KVSMC_CUDA(ctx, cudaMemcpyAsync(host, device, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return KVSMC_OK;
}

void kvsmc_server_destroy(kvsmc_server* S)
{
    if (!S) return;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
    }
    S->cv_work.notify_all();
    S->cv_budget.notify_all();
    for (std::thread& t : S->threads) t.join();
    cudaSetDevice(S->ctx->device);
    for (auto& h : S->held) free_outputs(S, h.second.coords, h.second.normals);
    S->held.clear();
    cudaStreamSynchronize(S->free_stream);
    for (kvsmc_context* c : S->wctx) kvsmc_destroy(c);
    cudaStreamDestroy(S->free_stream);
    cudaMemPoolDestroy(S->pool);
    delete S;
}

}  // extern "C"
