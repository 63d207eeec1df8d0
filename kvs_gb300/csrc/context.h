// context.h -- host-side state of libkvsmc shared by api.cu and batch.cu.
#pragma once
#include <cstdint>
#include <functional>
#include <string>
#include <vector>

#include "../../include/kvsmc.h"
#include "mc_internal.h"

struct kvsmc_volume {
    kvsmc::VolumeView view;
    void* dev = nullptr;        // owned device allocation
    size_t bytes = 0;
    bool has_minmax = false;
    double vmin = 0.0, vmax = 0.0;
    // brick min/max table (streaming kernels' empty-space skip), rebuilt after
    // every copy into a resident volume
    float2* bricks = nullptr;
    size_t brick_bytes = 0;
    bool bricks_valid = false;
};

struct kvsmc_context {
    int device = 0;
    int num_sms = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    void* scratch = nullptr;     // grow-only device arena for per-call intermediates
    size_t scratch_bytes = 0;
    void* out_arena = nullptr;   // grow-only device outputs of the host call
    void* arena2 = nullptr;      // grow-only second arena (vertex normals' triangle lists)
    size_t arena2_bytes = 0;
    void* arena3 = nullptr;      // grow-only third arena (a batch's shared streaming count)
    size_t arena3_bytes = 0;
    void* arena4 = nullptr;      // grow-only fourth arena (grouped shared-vertex requests' count arrays)
    size_t arena4_bytes = 0;
    void* arena5 = nullptr;      // grow-only fifth arena (their per-triangle normals)
    size_t arena5_bytes = 0;
    size_t out_bytes = 0;
    kvsmc_volume* host_vol = nullptr;  // staging volume of the host call
    uint64_t* h_small = nullptr; // pinned: small read-backs (totals, min/max, status)
    void* h_stage = nullptr;     // pinned: staging of work tables sent to the device
    size_t h_stage_bytes = 0;
    uint64_t launches = 0;
    int path = 0;                // 0: streaming kernels where eligible, 1: gather kernels only
    // plane-wait poll limits of the streaming count / emit kernels (kvsmc_set_wait_limit)
    uint32_t wait_polls[2] = {kvsmc::kStreamWaitPolls, kvsmc::kStreamWaitPolls};
    kvsmc::Profiler* prof = nullptr;
    std::string last_error;
    // auxiliary streams for launches that may run side by side (created on first use)
    static constexpr int kAux = 6;
    cudaStream_t aux[kAux] = {};
    cudaEvent_t fork_ev = nullptr;
    cudaEvent_t join_ev[kAux] = {};
    bool aux_ready = false;
    // copy stream of the host calls: results leave while later parts are
    // written (created on first use), one event per emit part
    cudaStream_t copy_stream = nullptr;
    static constexpr int kParts = 16;
    cudaEvent_t part_ev[kParts] = {};
    int* d_flag = nullptr;       // device word for checks of export calls (created on first use)
    int* h_flag = nullptr;       // pinned copy of it
    // export staging: two device record buffers, two pinned host buffers (grow-only)
    uint8_t* stl_dbuf[2] = {};
    uint8_t* stl_hbuf[2] = {};
    size_t stl_buf_bytes = 0;
    cudaEvent_t stl_ev[2] = {};
    // ASCII text of the STL writer: two device, two pinned buffers (grow-only)
    char* txt_dbuf[2] = {};
    char* txt_hbuf[2] = {};
    size_t txt_bytes = 0;
    // streaming launch shapes: the tuning table, or one forced shape
    std::vector<kvsmc_tune_entry> tuning;
    bool tune_forced = false;
    kvsmc_tune_choice tune_force{};
};

namespace kvsmc {
Profiler* profiler_create();
void profiler_destroy(Profiler* p);
}  // namespace kvsmc

namespace kvsmc_host {

kvsmc_status fail(kvsmc_context* ctx, kvsmc_status st, const char* fmt, ...);
inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }
inline kvsmc::Launch launch_of(kvsmc_context* ctx)
{
    kvsmc::Launch L{ctx->stream, ctx->num_sms, &ctx->launches, ctx->prof};
    L.wait_polls[0] = ctx->wait_polls[0];
    L.wait_polls[1] = ctx->wait_polls[1];
    return L;
}
kvsmc_status ensure_scratch(kvsmc_context* ctx, size_t bytes);
kvsmc_status ensure_stage(kvsmc_context* ctx, size_t bytes);
kvsmc_status volume_minmax(kvsmc_context* ctx, kvsmc_volume* v);
bool equal_ref(double a, double b);
kvsmc::Classifier make_classifier(double iso);

// Bump allocator over an arena (256-byte aligned pieces).
struct Carve {
    char* base;
    size_t off = 0;
    template <typename P> P* take(size_t bytes)
    {
        P* p = reinterpret_cast<P*>(base + off);
        off = align_up(off + bytes, 256);
        return p;
    }
};

// One request of a batch after host-side planning.
struct Item {
    kvsmc_volume* vol = nullptr;
    kvsmc_params params{};
    double vmin = 0, vmax = 0;
    bool extracted = true;
    float* d_coords = nullptr;
    uint64_t coords_cap = 0;
    float* d_normals = nullptr;
    uint64_t normals_cap = 0;
    uint32_t* d_conn = nullptr;
    uint64_t conn_cap = 0;
    bool emit = false;           // write outputs (false: count only)
    void* h_coords = nullptr;    // host outputs from the allocator (host calls)
    void* h_normals = nullptr;
    void* h_conn = nullptr;
    kvsmc_sizes sizes{};
    kvsmc_status status = KVSMC_OK;
};

// A resident volume of the given shape with uninitialised values (row-padded
// like the uploads); the caller fills it and then calls volume_bricks.
kvsmc_status volume_create(kvsmc_context* ctx, kvsmc_dtype dtype, uint32_t nx, uint32_t ny, uint32_t nz,
                           kvsmc_volume** out);

// (Re)build a resident volume's brick min/max table on the context's stream
// (no-op for value types or widths the streaming kernels do not take).
kvsmc_status volume_bricks(kvsmc_context* ctx, kvsmc_volume* v);

// Run fn(i, stream) for i < n side by side on the context's auxiliary streams,
// forked from and joined back into `origin` (also inside a stream capture).
cudaError_t fan_out(kvsmc_context* ctx, cudaStream_t origin, size_t n,
                    const std::function<cudaError_t(size_t, cudaStream_t)>& fn);

// Decide min/max (MapperBase::setRange, the volume's cache or a preset) and
// the Math::Equal early exit; fills it.vmin/vmax/extracted and clears sizes.
kvsmc_status prepare(kvsmc_context* ctx, Item& it);

// The streaming launch shape for a volume under the context's tuning (zero
// fields resolved by the built-in rules).
kvsmc_tune_choice stream_shape(const kvsmc_context* ctx, const kvsmc::VolumeView& v);

// Requests the streaming kernels can take (duplicated mode, 8/16-bit and
// float32 data, finite isolevel, width <= 4096 cells).
bool stream_eligible(const kvsmc_context* ctx, const Item& it);
// The same volume and isolevel conditions, whatever the mode (the streaming
// count of a shared-vertex request).
bool stream_volume_eligible(const kvsmc_context* ctx, const Item& it);
// Count (and, for items with emit set, emit) all eligible items together.
kvsmc_status stream_run(kvsmc_context* ctx, std::vector<Item*>& items);

}  // namespace kvsmc_host

#define KVSMC_CUDA(ctx, call)                                                                              \
    do {                                                                                                   \
        cudaError_t e_ = (call);                                                                           \
        if (e_ != cudaSuccess)                                                                             \
            return kvsmc_host::fail(ctx, e_ == cudaErrorMemoryAllocation ? KVSMC_ERR_OUT_OF_MEMORY         \
                                                                         : KVSMC_ERR_CUDA,                 \
                                    "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)
