// plan.cu -- replayable batch plans: the streaming extraction of a fixed set
// of requests, planned once and captured into one CUDA graph.
//
// The graph holds, for every value type present, the count launch, then the
// unit scan, the plane scan and the per-isolevel totals, then the emit
// launches, and finally the copy of the status word and the totals into a
// pinned host buffer.  Capture runs on a private stream, so the graph does
// not depend on the stream it is later launched on.  The emit kernel never
// writes a request's triangles past the capacity given at creation; the host
// reports the shortfall after the replay.
#include <cstring>
#include <vector>

#include "batch.h"

using kvsmc_host::Item;

struct kvsmc_plan {
    kvsmc_context* ctx = nullptr;
    int device = 0;
    int32_t n = 0;
    std::vector<kvsmc_sizes> base;        // per request: min/max, extracted
    std::vector<kvsmc_status> pre;        // per request: status decided at creation
    std::vector<int32_t> iso_req;         // per planned isolevel: its request
    std::vector<uint64_t> cap;            // per planned isolevel: triangles its outputs hold
    void* d_mem = nullptr;
    uint64_t* h_out = nullptr;            // pinned: [0] status word, [1 + i] total of isolevel i
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint64_t kernels = 0;
    cudaStream_t last = nullptr;
    bool pending = false;
};

namespace {

void plan_free(kvsmc_plan* p)
{
    if (!p) return;
    cudaSetDevice(p->device);
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    if (p->d_mem) cudaFree(p->d_mem);
    if (p->h_out) cudaFreeHost(p->h_out);
    delete p;
}

// Record every launch of one extraction on stream s (being captured).
cudaError_t record(kvsmc_host::StreamBatch& b, cudaStream_t s, int num_sms, uint64_t* counter, uint64_t* h_out)
{
    const kvsmc::Launch L{s, num_sms, counter, nullptr};
    // the per-kind launches of a pass run side by side (parallel graph branches)
    auto per_kind = [&](bool emit) {
        return kvsmc_host::fan_out(b.ctx, s, b.launches.size(), [&](size_t i, cudaStream_t st) {
            const auto& l = b.launches[i];
            kvsmc::Launch Li = L;
            Li.stream = st;
            return kvsmc::launch_stream(emit, l.dtype, l.rows, b.d_groups + l.g0, l.ng, l.ntasks, b.d_isos,
                                        b.d_unit_counts, emit ? b.d_unit_offsets : nullptr,
                                        emit ? b.d_plane_base : nullptr, b.d_status, b.d_next + 2 * i + (emit ? 1 : 0),
                                        Li, l.ctas_per_sm);
        });
    };
    cudaError_t e = cudaMemsetAsync(b.d_status, 0, sizeof(int), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(b.d_unit_counts, 0, b.unit_elems * sizeof(uint16_t), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(b.d_next, 0, b.launches.size() * 16, s);
    if (e == cudaSuccess) e = per_kind(false);
    if (e == cudaSuccess)
        e = kvsmc::launch_unit_scan(b.d_groups, (int)b.groups.size(), b.scan_blocks, b.d_isos, b.d_unit_counts,
                                    b.d_unit_offsets, b.d_plane_totals, L, b.scan_threads);
    if (e == cudaSuccess) e = kvsmc::launch_scan(b.d_plane_totals, b.d_plane_base, b.iso_planes, b.d_scan, b.d_total, L);
    if (e == cudaSuccess)
        e = kvsmc::launch_iso_totals(b.d_isos, (int)b.isos.size(), b.d_plane_base, b.d_total, b.d_totals, L);
    if (e == cudaSuccess) e = per_kind(true);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_out, b.d_status, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h_out + 1, b.d_totals, b.isos.size() * sizeof(uint64_t), cudaMemcpyDeviceToHost, s);
    return e;
}

}  // namespace

extern "C" {

kvsmc_status kvsmc_plan_create(kvsmc_context* ctx, const kvsmc_request* reqs, int32_t n, kvsmc_plan** out)
{
    using namespace kvsmc_host;
    if (!ctx || !out || n < 0 || (n && !reqs)) return KVSMC_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, KVSMC_ERR_CUDA, "plan: cudaSetDevice");
    std::vector<Item> items((size_t)n);
    kvsmc_plan* p = new kvsmc_plan();
    p->ctx = ctx;
    p->device = ctx->device;
    p->n = n;
    p->base.resize((size_t)n);
    p->pre.assign((size_t)n, KVSMC_OK);
    std::vector<Item*> stream_items;
    for (int32_t i = 0; i < n; ++i) {
        Item& it = items[i];
        it.vol = reqs[i].volume;
        it.params = reqs[i].params;
        it.d_coords = reqs[i].d_coords; it.coords_cap = reqs[i].coords_capacity;
        it.d_normals = reqs[i].d_normals; it.normals_cap = reqs[i].normals_capacity;
        it.emit = true;
        kvsmc_status st = prepare(ctx, it);
        if (st) { plan_free(p); return st; }
        p->base[i] = it.sizes;
        if (!it.extracted) continue;
        if (!stream_eligible(ctx, it)) {
            plan_free(p);
            return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT,
                        "plan: request %d is not one the streaming kernels take (duplicated mode, "
                        "8/16-bit or float32 data, width <= 4097)", (int)i);
        }
        it.sizes.extracted = 1;
        p->base[i] = it.sizes;
        stream_items.push_back(&it);
    }
    if (stream_items.empty()) { *out = p; return KVSMC_OK; }

    StreamBatch b;
    b.ctx = ctx;
    b.items = stream_items;
    b.plan_tables();
    for (size_t k = 0; k < b.isos.size(); ++k) {
        Item* it = b.iso_item[k];
        b.isos[k].coords = it->d_coords;
        b.isos[k].normals = it->d_normals;
        b.isos[k].cap_tris = cap_triangles(*it);
        p->iso_req.push_back((int32_t)(it - items.data()));
        p->cap.push_back(b.isos[k].cap_tris);
    }
    cudaStream_t cs = nullptr;
    cudaError_t e = cudaMalloc(&p->d_mem, b.scratch_bytes());
    if (e == cudaSuccess) e = cudaMallocHost(&p->h_out, (b.isos.size() + 1) * sizeof(uint64_t));
    if (e == cudaSuccess) {
        std::memset(p->h_out, 0, (b.isos.size() + 1) * sizeof(uint64_t));
        b.carve(static_cast<char*>(p->d_mem));
        e = cudaMemcpy(b.d_groups, b.groups.data(), b.groups.size() * sizeof(kvsmc::StreamGroup),
                       cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess)
        e = cudaMemcpy(b.d_isos, b.isos.data(), b.isos.size() * sizeof(kvsmc::StreamIso), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        const cudaError_t rec = record(b, cs, ctx->num_sms, &p->kernels, p->h_out);
        const cudaError_t end = cudaStreamEndCapture(cs, &p->graph);
        e = rec != cudaSuccess ? rec : end;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&p->exec, p->graph, 0);
    if (cs) cudaStreamDestroy(cs);
    if (e != cudaSuccess) {
        cudaGetLastError();
        plan_free(p);
        return fail(ctx, e == cudaErrorMemoryAllocation ? KVSMC_ERR_OUT_OF_MEMORY : KVSMC_ERR_CUDA,
                    "plan: %s", cudaGetErrorString(e));
    }
    *out = p;
    return KVSMC_OK;
}

kvsmc_status kvsmc_plan_launch(kvsmc_plan* p, void* stream)
{
    if (!p) return KVSMC_ERR_INVALID_ARGUMENT;
    kvsmc_context* ctx = p->ctx;
    if (cudaSetDevice(p->device) != cudaSuccess) return kvsmc_host::fail(ctx, KVSMC_ERR_CUDA, "plan: cudaSetDevice");
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
    p->last = s;
    p->pending = true;
    if (!p->exec) return KVSMC_OK;   // nothing extracted
    KVSMC_CUDA(ctx, cudaGraphLaunch(p->exec, s));
    ctx->launches += p->kernels;
    return KVSMC_OK;
}

kvsmc_status kvsmc_plan_wait(kvsmc_plan* p, kvsmc_request* reqs, int32_t n)
{
    if (!p || (n && !reqs) || n != p->n) return KVSMC_ERR_INVALID_ARGUMENT;
    kvsmc_context* ctx = p->ctx;
    if (cudaSetDevice(p->device) != cudaSuccess) return kvsmc_host::fail(ctx, KVSMC_ERR_CUDA, "plan: cudaSetDevice");
    if (!p->pending) return kvsmc_host::fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "plan: no replay to wait for");
    if (p->exec) KVSMC_CUDA(ctx, cudaStreamSynchronize(p->last));
    p->pending = false;
    kvsmc_status first = KVSMC_OK;
    for (int32_t i = 0; i < n; ++i) {
        reqs[i].sizes = p->base[i];
        reqs[i].status = p->pre[i];
    }
    int status = 0;
    if (p->h_out) std::memcpy(&status, p->h_out, sizeof(int));
    for (size_t k = 0; k < p->iso_req.size(); ++k) {
        kvsmc_request& r = reqs[p->iso_req[k]];
        const uint64_t t = p->h_out[1 + k];
        r.sizes.ntriangles = t;
        r.sizes.nvertices = 3 * t;
        r.sizes.ncoords = 9 * t;
        r.sizes.nnormals = 3 * t;
        if (status) r.status = KVSMC_ERR_TIMEOUT;
        else if (t > p->cap[k]) r.status = KVSMC_ERR_CAPACITY;
    }
    for (int32_t i = 0; i < n; ++i)
        if (reqs[i].status && !first) first = reqs[i].status;
    if (status) return kvsmc_host::fail(ctx, KVSMC_ERR_TIMEOUT, "plan: a shared-memory load did not complete");
    if (first == KVSMC_ERR_CAPACITY) return kvsmc_host::fail(ctx, first, "plan: a result exceeds its output buffers");
    return first;
}

uint64_t kvsmc_plan_kernels(const kvsmc_plan* p) { return p ? p->kernels : 0; }

void kvsmc_plan_destroy(kvsmc_plan* p) { plan_free(p); }

}  // extern "C"
