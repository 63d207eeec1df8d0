// server.cu -- kvsmc_server: a request loop over resident volumes with
// continuous batching (see include/kvsmc.h).
//
// Clients push requests into one pending queue.  Each worker thread owns a
// context (its own stream, scratch and auxiliary streams) and loops: take
// every pending request up to max_batch, count them in one fused pass,
// admit them against the output budget, allocate their outputs from the
// server's output arena, emit them in one fused pass, publish the
// completions.  With several workers, one batch counts while another
// emits, so new arrivals never wait for a whole batch in flight.  The
// budget counts the bytes of results the clients have not released yet; a
// batch that does not fit waits for releases (its requests that could
// never fit alone complete with KVSMC_ERR_BUDGET).  The budget is laid out
// once, at creation, as one device arena; results are carved from it by a
// host-side best-fit free list, so admitting and releasing a result costs no
// CUDA allocation call.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
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
    uint64_t coords_off, coords_len, normals_off, normals_len;
    uint64_t bytes;
};

constexpr uint64_t kBytesPerTriangle = 48;   // 9 coords + 3 normals, float
constexpr uint64_t kArenaAlign = 256;

// Best-fit free list over [0, size): offset -> length, neighbours coalesced.
struct FreeList {
    std::map<uint64_t, uint64_t> free_;
    void reset(uint64_t size) { free_.clear(); if (size) free_[0] = size; }
    bool take(uint64_t len, uint64_t* off)
    {
        auto best = free_.end();
        for (auto it = free_.begin(); it != free_.end(); ++it)
            if (it->second >= len && (best == free_.end() || it->second < best->second)) best = it;
        if (best == free_.end()) return false;
        *off = best->first;
        const uint64_t rest = best->second - len;
        const uint64_t at = best->first + len;
        free_.erase(best);
        if (rest) free_[at] = rest;
        return true;
    }
    void give(uint64_t off, uint64_t len)
    {
        auto next = free_.lower_bound(off);
        if (next != free_.end() && off + len == next->first) {
            len += next->second;
            next = free_.erase(next);
        }
        if (next != free_.begin()) {
            auto prev = std::prev(next);
            if (prev->first + prev->second == off) {
                prev->second += len;
                return;
            }
        }
        free_[off] = len;
    }
};

uint64_t arena_len(uint64_t bytes) { return (bytes + kArenaAlign - 1) / kArenaAlign * kArenaAlign; }

}  // namespace

struct kvsmc_server {
    kvsmc_context* ctx = nullptr;       // owner: device, min/max passes at submit
    kvsmc_server_config cfg{};
    std::vector<kvsmc_context*> wctx;   // one per worker
    std::vector<std::thread> threads;
    char* arena = nullptr;              // outputs of admitted requests (the budget, laid out once)
    uint64_t arena_bytes = 0;
    FreeList free_list;                 // guarded by mu
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

// Give a held result's blocks back (caller holds mu).
void give_back(kvsmc_server* S, const Held& h)
{
    if (h.coords_len) S->free_list.give(h.coords_off, h.coords_len);
    if (h.normals_len) S->free_list.give(h.normals_off, h.normals_len);
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

        // Emit in rounds reusing this one count: each round admits the next
        // requests (in order) whose results fit the budget together, waits
        // until the budget and arena blocks are free, emits just those, and
        // publishes them.  A request whose result alone exceeds the budget
        // completes with KVSMC_ERR_BUDGET.
        std::vector<char> published(n, 0);
        size_t next = 0;
        bool first_round = true;
        for (;;) {
            std::vector<Item*> admit;
            uint64_t need = 0;
            if (!st) {
                while (next < live.size()) {
                    Item* it = live[next];
                    const uint64_t bytes = it->sizes.ntriangles * kBytesPerTriangle;
                    if (bytes > budget) {
                        it->status = kvsmc_host::fail(ctx, KVSMC_ERR_BUDGET, "result of %llu bytes exceeds the budget",
                                                      (unsigned long long)bytes);
                        ++next;
                        continue;
                    }
                    if (need + bytes > budget) break;
                    need += bytes;
                    admit.push_back(it);
                    ++next;
                }
            }
            // outputs: carved from the arena once the budget (and a block of
            // each size) is free; with nothing held the arena is whole, so a
            // round that fits the budget always gets its blocks eventually
            std::vector<Held> blocks(n, Held{0, 0, 0, 0, 0});
            std::vector<float*> coords(n, nullptr), normals(n, nullptr);
            if (need) {
                std::unique_lock<std::mutex> lk(S->mu);
                bool waited = false;
                for (;;) {
                    bool ok = S->in_use + need <= budget;
                    size_t taken = 0;
                    for (; ok && taken < admit.size(); ++taken) {
                        Item* it = admit[taken];
                        const size_t i = (size_t)(it - items.data());
                        const uint64_t t = it->sizes.ntriangles;
                        Held& h = blocks[i];
                        h = Held{0, 0, 0, 0, t * kBytesPerTriangle};
                        if (t == 0) continue;
                        h.coords_len = arena_len(36 * t);
                        h.normals_len = arena_len(12 * t);
                        if (!S->free_list.take(h.coords_len, &h.coords_off)) {
                            h.coords_len = h.normals_len = 0;
                            ok = false;
                            break;
                        }
                        if (!S->free_list.take(h.normals_len, &h.normals_off)) {
                            S->free_list.give(h.coords_off, h.coords_len);
                            h.coords_len = h.normals_len = 0;
                            ok = false;
                            break;
                        }
                    }
                    if (ok) break;
                    for (size_t j = 0; j < taken; ++j) {
                        Held& h = blocks[(size_t)(admit[j] - items.data())];
                        give_back(S, h);
                        h.coords_len = h.normals_len = 0;
                    }
                    if (S->stop) {
                        for (Item* it : admit)
                            it->status = kvsmc_host::fail(ctx, KVSMC_ERR_BUDGET, "server stopping before the budget freed");
                        admit.clear();
                        need = 0;
                        break;
                    }
                    if (!waited) {
                        ++S->budget_waits;
                        waited = true;
                    }
                    S->cv_budget.wait(lk);
                }
                S->in_use += need;
                S->peak = std::max(S->peak, S->in_use);
            }
            for (Item* it : live) it->emit = false;
            for (Item* it : admit) {
                const size_t i = (size_t)(it - items.data());
                const uint64_t t = it->sizes.ntriangles;
                it->emit = true;
                if (t == 0) continue;
                coords[i] = reinterpret_cast<float*>(S->arena + blocks[i].coords_off);
                normals[i] = reinterpret_cast<float*>(S->arena + blocks[i].normals_off);
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

            // publish this round: the admitted requests, and (first round) the
            // ones that failed or had nothing to extract; on an error, all
            const double t_done = S->now();
            uint64_t granted = need;
            std::unique_lock<std::mutex> lk(S->mu);
            for (size_t i = 0; i < n; ++i) {
                if (published[i]) continue;
                const bool in_round = std::find(admit.begin(), admit.end(), &items[i]) != admit.end();
                const bool settled = items[i].status != KVSMC_OK || !items[i].extracted ||
                                     (first_round && std::find(live.begin(), live.end(), &items[i]) == live.end());
                if (!in_round && !settled && !st) continue;
                published[i] = 1;
                kvsmc_completion c;
                std::memset(&c, 0, sizeof c);
                c.ticket = reqs[i].ticket;
                c.status = items[i].status;
                c.batch_size = (int32_t)n;
                c.sizes = items[i].sizes;
                c.submit_s = reqs[i].t_submit;
                c.start_s = t_start;
                c.done_s = t_done;
                if (in_round && !c.status && coords[i]) {
                    c.d_coords = coords[i];
                    c.d_normals = normals[i];
                    S->held[c.ticket] = blocks[i];
                    granted -= blocks[i].bytes;
                } else if (in_round) {
                    give_back(S, blocks[i]);
                }
                S->done.push_back(c);
                ++S->completed;
            }
            // budget reserved for requests that hold nothing (failed, empty) goes back now
            S->in_use -= granted;
            S->cv_done.notify_all();
            S->cv_budget.notify_all();
            first_round = false;
            if (st || next >= live.size()) break;
        }
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
    // the arena: the budget plus room for the 256-byte rounding of every block
    // of a full batch in each worker
    S->arena_bytes = S->cfg.output_budget_bytes + 2 * kArenaAlign * (uint64_t)S->cfg.max_batch * S->cfg.workers;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&S->arena), S->arena_bytes);
    S->free_list.reset(e == cudaSuccess ? S->arena_bytes : 0);
    kvsmc_status st = e == cudaSuccess ? KVSMC_OK
                                       : (e == cudaErrorMemoryAllocation ? KVSMC_ERR_OUT_OF_MEMORY : KVSMC_ERR_CUDA);
    for (int w = 0; w < S->cfg.workers && !st; ++w) {
        kvsmc_context* c = nullptr;
        st = kvsmc_create(ctx->device, &c);
        if (!st) {
            // the workers follow the owner's launch shapes
            c->tuning = ctx->tuning;
            c->tune_forced = ctx->tune_forced;
            c->tune_force = ctx->tune_force;
            S->wctx.push_back(c);
        }
    }
    if (st) {
        for (kvsmc_context* c : S->wctx) kvsmc_destroy(c);
        if (S->arena) cudaFree(S->arena);
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
    give_back(S, f->second);
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
    S->held.clear();
    for (kvsmc_context* c : S->wctx) kvsmc_destroy(c);
    cudaFree(S->arena);
    delete S;
}

}  // extern "C"
