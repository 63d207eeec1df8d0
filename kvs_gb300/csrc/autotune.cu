// autotune.cu -- launch shapes of the streaming kernels: the tuning table
// (size classes, resolution of a volume's shape, install / read back / force)
// and the autotuner that fills it by timing candidate shapes on seeded
// synthetic volumes of each (value type, size class).
//
// A shape changes how the work is cut (rows per warp task, warp tasks per
// SM, resident CTAs per SM, unit-scan tile), never what is computed: output
// positions come from the exact counts, so every shape writes the same bits.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "batch.h"

namespace {

using kvsmc_host::fail;

// ---------------------------------------------------------------- table

bool tuned_dtype(int dt)
{
    return dt == KVSMC_I8 || dt == KVSMC_I16 || dt == KVSMC_U8 || dt == KVSMC_U16 || dt == KVSMC_F32;
}

bool choice_valid(const kvsmc_tune_choice& c)
{
    return (c.rows == 0 || c.rows == 1 || c.rows == 2) && c.tasks_per_sm >= 0 && c.tasks_per_sm <= 65536 &&
           c.ctas_per_sm >= 0 && c.ctas_per_sm <= 64 &&
           (c.scan_threads == 0 || c.scan_threads == 64 || c.scan_threads == 128 || c.scan_threads == 256);
}

bool entry_valid(const kvsmc_tune_entry& e)
{
    return tuned_dtype(e.dtype) && e.size_class >= 0 && e.size_class < KVSMC_SIZE_CLASSES && choice_valid(e.choice);
}

// ------------------------------------------------------ tuning volumes

// Low-bias 32-bit integer hash (C. Wellons' "lowbias32" constants).
__device__ __forceinline__ uint32_t hash32(uint32_t x)
{
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

// A smooth seeded field in [0, 1] (three products of sinusoids with
// wavelengths of 20-40 cells and random phases, plus 2 % hash noise), mapped
// onto the value range of T.  Dense, x fastest.
template <typename T>
__global__ void k_tune_field(T* __restrict__ out, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t seed)
{
    const uint64_t n = (uint64_t)nx * ny * nz;
    const float tw = 6.2831853f;
    const float ph0 = (float)(hash32(seed ^ 0x1111u) & 0xffffu) * (tw / 65536.0f);
    const float ph1 = (float)(hash32(seed ^ 0x2222u) & 0xffffu) * (tw / 65536.0f);
    const float ph2 = (float)(hash32(seed ^ 0x3333u) & 0xffffu) * (tw / 65536.0f);
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t x = (uint32_t)(i % nx), y = (uint32_t)((i / nx) % ny), z = (uint32_t)(i / ((uint64_t)nx * ny));
        const float a = __sinf(x * (tw / 23.0f) + ph0) * __sinf(y * (tw / 31.0f) + ph1);
        const float b = __sinf(y * (tw / 27.0f) + ph2) * __sinf(z * (tw / 37.0f) + ph0);
        const float c = __sinf(z * (tw / 21.0f) + ph1) * __sinf(x * (tw / 33.0f) + ph2);
        const float noise = (float)(hash32((uint32_t)i * 0x9e3779b9u + seed) & 0xffffu) * (1.0f / 65535.0f) - 0.5f;
        float f = 0.5f + 0.16f * (a + b + c) + 0.04f * noise;
        f = fminf(fmaxf(f, 0.0f), 1.0f);
        T v;
        if (sizeof(T) == 4) v = (T)f;
        else if (sizeof(T) == 1) v = (T)(__float2int_rn(f * 255.0f) + ((T)-1 < 0 ? -128 : 0));
        else v = (T)(__float2int_rn(f * 65535.0f) + ((T)-1 < 0 ? -32768 : 0));
        out[i] = v;
    }
}

// Node count per axis of the tuning cube of a size class: about 2^17, 2^20,
// 2^23, 2^26, 2^29 cells (the middle of each class on a log scale).
uint32_t class_side(int cls)
{
    static const uint32_t side[KVSMC_SIZE_CLASSES] = {51, 102, 204, 407, 813};
    return side[cls];
}

double median(std::vector<double> v)
{
    std::sort(v.begin(), v.end());
    return v.empty() ? 0.0 : v[v.size() / 2];
}

// One (dtype, class) tuning run: volume, requests, outputs; times shapes.
struct Trial {
    kvsmc_context* ctx = nullptr;
    kvsmc_volume* vol = nullptr;
    std::vector<kvsmc_request> reqs;
    float* d_out = nullptr;
    int reps = 3;

    kvsmc_status time_shape(const kvsmc_tune_choice* c, double* ms)
    {
        kvsmc_status st = kvsmc_tuning_force(ctx, c);
        if (st) return st;
        std::vector<double> t;
        for (int r = -1; r < reps; ++r) {   // one untimed run first
            const auto t0 = std::chrono::steady_clock::now();
            st = kvsmc_extract_batch(ctx, reqs.data(), (int32_t)reqs.size());
            const auto t1 = std::chrono::steady_clock::now();
            if (st) return st;
            if (r >= 0) t.push_back(std::chrono::duration<double, std::milli>(t1 - t0).count());
        }
        *ms = median(t);
        return KVSMC_OK;
    }

    void release()
    {
        if (vol) kvsmc_volume_free(ctx, vol);
        if (d_out) cudaFree(d_out);
        vol = nullptr;
        d_out = nullptr;
    }
};

// Build the tuning volume and requests of (dtype, class).
kvsmc_status trial_setup(kvsmc_context* ctx, int dt, int cls, int niso, uint64_t seed, Trial& tr)
{
    const uint32_t s = class_side(cls);
    const size_t es = dt == KVSMC_F32 ? 4 : (dt == KVSMC_I16 || dt == KVSMC_U16) ? 2 : 1;
    const uint64_t n = (uint64_t)s * s * s;
    void* raw = nullptr;
    KVSMC_CUDA(ctx, cudaMalloc(&raw, n * es));
    const uint32_t sd = (uint32_t)(seed * 0x9e3779b97f4a7c15ull >> 32) ^ (uint32_t)(dt * 977 + cls * 131);
    const unsigned blocks = (unsigned)std::min<uint64_t>((n + 255) / 256, (uint64_t)ctx->num_sms * 16);
    cudaStream_t stream = static_cast<cudaStream_t>(kvsmc_stream(ctx));
    switch (dt) {
    case KVSMC_I8: k_tune_field<int8_t><<<blocks, 256, 0, stream>>>((int8_t*)raw, s, s, s, sd); break;
    case KVSMC_I16: k_tune_field<int16_t><<<blocks, 256, 0, stream>>>((int16_t*)raw, s, s, s, sd); break;
    case KVSMC_U8: k_tune_field<uint8_t><<<blocks, 256, 0, stream>>>((uint8_t*)raw, s, s, s, sd); break;
    case KVSMC_U16: k_tune_field<uint16_t><<<blocks, 256, 0, stream>>>((uint16_t*)raw, s, s, s, sd); break;
    default: k_tune_field<float><<<blocks, 256, 0, stream>>>((float*)raw, s, s, s, sd); break;
    }
    ctx->launches += 1;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    kvsmc_status st = KVSMC_OK;
    if (e != cudaSuccess) st = fail(ctx, KVSMC_ERR_CUDA, "autotune: field: %s", cudaGetErrorString(e));
    if (!st) st = kvsmc_volume_from_device(ctx, raw, (kvsmc_dtype)dt, s, s, s, &tr.vol);
    cudaFree(raw);
    if (st) return st;
    double lo = 0, hi = 0;
    if ((st = kvsmc_volume_minmax(ctx, tr.vol, &lo, &hi))) return st;
    tr.reqs.assign((size_t)niso, kvsmc_request{});
    for (int k = 0; k < niso; ++k) {
        kvsmc_request& r = tr.reqs[k];
        std::memset(&r, 0, sizeof r);
        r.volume = tr.vol;
        r.params.isolevel = lo + (hi - lo) * (0.3 + 0.4 * (niso > 1 ? (double)k / (niso - 1) : 0.5)) + 0.013;
        r.params.mode = KVSMC_DUP_POLYGON_NORMAL;
        for (int a = 0; a < 3; ++a) r.params.scale[a] = 1.0f;
    }
    // outputs: the counts are the same under every shape
    if ((st = kvsmc_count_batch(ctx, tr.reqs.data(), niso))) return st;
    uint64_t total = 0;
    for (auto& r : tr.reqs) total += r.sizes.ntriangles;
    KVSMC_CUDA(ctx, cudaMalloc(&tr.d_out, std::max<uint64_t>(1, total) * 12 * sizeof(float)));
    uint64_t off = 0;
    for (auto& r : tr.reqs) {
        const uint64_t t = r.sizes.ntriangles;
        r.d_coords = tr.d_out + 12 * off;
        r.coords_capacity = 9 * t;
        r.d_normals = tr.d_out + 12 * off + 9 * t;
        r.normals_capacity = 3 * t;
        off += t;
    }
    return KVSMC_OK;
}

// The tuned fields that differ from what the built-in rules pick for the
// tuning volume (the rest stay 0, so the rules keep adapting per volume).
kvsmc_tune_choice relative_to_rules(const kvsmc_tune_choice& best, const kvsmc_tune_choice& rules)
{
    kvsmc_tune_choice c{};
    c.rows = best.rows != rules.rows ? best.rows : 0;
    c.tasks_per_sm = best.tasks_per_sm != rules.tasks_per_sm ? best.tasks_per_sm : 0;
    c.ctas_per_sm = best.ctas_per_sm != rules.ctas_per_sm ? best.ctas_per_sm : 0;
    c.scan_threads = best.scan_threads != rules.scan_threads ? best.scan_threads : 0;
    return c;
}

kvsmc_status tune_one(kvsmc_context* ctx, int dt, int cls, const kvsmc_autotune_config& cfg, kvsmc_tune_entry& out)
{
    Trial tr;
    tr.ctx = ctx;
    tr.reps = cfg.reps;
    kvsmc_status st = trial_setup(ctx, dt, cls, cfg.isovalues, cfg.seed, tr);
    if (st) { tr.release(); return st; }
    const uint32_t s = class_side(cls);
    kvsmc_tune_choice rules{};
    kvsmc_tune_resolve(nullptr, 0, (kvsmc_dtype)dt, s, s, s, &rules);
    double def_ms = 0;
    st = tr.time_shape(&rules, &def_ms);
    kvsmc_tune_choice best = rules;
    double best_ms = def_ms;
    auto consider = [&](const kvsmc_tune_choice& c) {
        if (st) return;
        if (std::memcmp(&c, &best, sizeof c) == 0) return;
        double ms = 0;
        st = tr.time_shape(&c, &ms);
        if (!st && ms < best_ms) { best = c; best_ms = ms; }
    };
    // rows x tasks per SM, then CTAs per SM, then the scan tile
    const kvsmc_tune_choice base = rules;
    for (int rows : {1, 2})
        for (int tps : {24, 96, 384}) {
            kvsmc_tune_choice c = base;
            c.rows = rows;
            c.tasks_per_sm = tps;
            consider(c);
        }
    { kvsmc_tune_choice c = best; c.ctas_per_sm = 1; consider(c); }
    for (int sc : {64, 128}) { kvsmc_tune_choice c = best; c.scan_threads = sc; consider(c); }
    kvsmc_tuning_force(ctx, nullptr);
    tr.release();
    if (st) return st;
    std::memset(&out, 0, sizeof out);
    out.dtype = dt;
    out.size_class = cls;
    out.default_ms = def_ms;
    if (best_ms < 0.97 * def_ms) {
        out.choice = relative_to_rules(best, rules);
        out.tuned_ms = best_ms;
    } else {
        out.tuned_ms = def_ms;   // within noise of the rules: keep them
    }
    return KVSMC_OK;
}

}  // namespace

extern "C" {

int32_t kvsmc_size_class(uint32_t nx, uint32_t ny, uint32_t nz)
{
    const uint64_t c = (uint64_t)(nx > 1 ? nx - 1 : 0) * (ny > 1 ? ny - 1 : 0) * (nz > 1 ? nz - 1 : 0);
    if (c < (1ull << 18)) return 0;
    if (c < (1ull << 21)) return 1;
    if (c < (1ull << 24)) return 2;
    if (c < (1ull << 27)) return 3;
    return 4;
}

kvsmc_status kvsmc_tune_resolve(const kvsmc_tune_entry* table, int32_t n, kvsmc_dtype dtype, uint32_t nx,
                                uint32_t ny, uint32_t nz, kvsmc_tune_choice* out)
{
    if (!out || n < 0 || (n > 0 && !table)) return KVSMC_ERR_INVALID_ARGUMENT;
    kvsmc_tune_choice c{};
    c.rows = kvsmc_host::stream_rows(nx > 1 ? nx - 1 : 1);
    c.tasks_per_sm = kvsmc_host::kDefaultTasksPerSm;
    c.ctas_per_sm = 0;
    c.scan_threads = 256;
    const int32_t cls = kvsmc_size_class(nx, ny, nz);
    for (int32_t i = 0; i < n; ++i) {
        if (!entry_valid(table[i])) return KVSMC_ERR_INVALID_ARGUMENT;
        if (table[i].dtype != (int32_t)dtype || table[i].size_class != cls) continue;
        const kvsmc_tune_choice& t = table[i].choice;
        if (t.rows) c.rows = t.rows;
        if (t.tasks_per_sm) c.tasks_per_sm = t.tasks_per_sm;
        if (t.ctas_per_sm) c.ctas_per_sm = t.ctas_per_sm;
        if (t.scan_threads) c.scan_threads = t.scan_threads;
        break;
    }
    *out = c;
    return KVSMC_OK;
}

kvsmc_status kvsmc_tuning_set(kvsmc_context* ctx, const kvsmc_tune_entry* table, int32_t n)
{
    if (!ctx || n < 0 || (n > 0 && !table)) return KVSMC_ERR_INVALID_ARGUMENT;
    for (int32_t i = 0; i < n; ++i)
        if (!entry_valid(table[i]))
            return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "tuning entry %d: bad dtype, class or shape", (int)i);
    ctx->tuning.assign(table, table + n);
    return KVSMC_OK;
}

int32_t kvsmc_tuning_get(const kvsmc_context* ctx, kvsmc_tune_entry* out, int32_t cap)
{
    if (!ctx) return 0;
    const int32_t n = (int32_t)ctx->tuning.size();
    for (int32_t i = 0; i < n && i < cap && out; ++i) out[i] = ctx->tuning[i];
    return n;
}

kvsmc_status kvsmc_tuning_force(kvsmc_context* ctx, const kvsmc_tune_choice* choice)
{
    if (!ctx) return KVSMC_ERR_INVALID_ARGUMENT;
    if (!choice) {
        ctx->tune_forced = false;
        return KVSMC_OK;
    }
    if (!choice_valid(*choice)) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "tuning: bad launch shape");
    ctx->tune_force = *choice;
    ctx->tune_forced = true;
    return KVSMC_OK;
}

kvsmc_status kvsmc_autotune(kvsmc_context* ctx, const kvsmc_autotune_config* cfg, kvsmc_tune_entry* out, int32_t cap,
                            int32_t* nout)
{
    if (!ctx || !cfg) return KVSMC_ERR_INVALID_ARGUMENT;
    if (nout) *nout = 0;
    kvsmc_autotune_config c = *cfg;
    static const int32_t all[5] = {KVSMC_U8, KVSMC_U16, KVSMC_F32, KVSMC_I8, KVSMC_I16};
    if (!c.dtypes) { c.dtypes = all; c.ndtypes = 5; }
    if (c.ndtypes < 0 || c.max_class < 0 || c.max_class >= KVSMC_SIZE_CLASSES || c.isovalues < 1 ||
        c.isovalues > 16 || c.reps < 1 || c.reps > 100)
        return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "autotune: bad configuration");
    for (int32_t i = 0; i < c.ndtypes; ++i)
        if (!tuned_dtype(c.dtypes[i]))
            return fail(ctx, KVSMC_ERR_UNSUPPORTED_DTYPE, "autotune: dtype %d has no streaming kernels", (int)c.dtypes[i]);
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, KVSMC_ERR_CUDA, "autotune: cudaSetDevice");
    const std::vector<kvsmc_tune_entry> saved = ctx->tuning;
    const bool was_forced = ctx->tune_forced;
    const kvsmc_tune_choice old_force = ctx->tune_force;
    ctx->tuning.clear();
    std::vector<kvsmc_tune_entry> table;
    kvsmc_status st = KVSMC_OK;
    for (int32_t i = 0; i < c.ndtypes && !st; ++i)
        for (int cls = 0; cls <= c.max_class && !st; ++cls) {
            kvsmc_tune_entry e;
            st = tune_one(ctx, c.dtypes[i], cls, c, e);
            if (!st) table.push_back(e);
        }
    ctx->tune_forced = was_forced;
    ctx->tune_force = old_force;
    if (st) {
        ctx->tuning = saved;
        return st;
    }
    ctx->tuning = table;
    for (int32_t i = 0; i < (int32_t)table.size() && i < cap && out; ++i) out[i] = table[i];
    if (nout) *nout = (int32_t)std::min<size_t>(table.size(), (size_t)(cap > 0 ? cap : 0));
    return KVSMC_OK;
}

}  // extern "C"
