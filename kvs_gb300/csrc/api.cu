// api.cu -- the C ABI of libkvsmc (include/kvsmc.h): contexts, resident
// volumes, and the count -> size -> emit pipeline for one request.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>

#include "../../include/kvsmc.h"
#include "mc_internal.h"

using namespace kvsmc;

struct kvsmc_volume {
    VolumeView view;
    void* dev = nullptr;        // owned device allocation
    size_t bytes = 0;
    bool has_minmax = false;
    double vmin = 0.0, vmax = 0.0;
};

struct kvsmc_context {
    int device = 0;
    int num_sms = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    void* scratch = nullptr;     // grow-only arena for per-request intermediates
    size_t scratch_bytes = 0;
    void* out_arena = nullptr;   // grow-only device outputs of the host call
    size_t out_bytes = 0;
    kvsmc_volume* host_vol = nullptr;  // staging volume of the host call
    uint64_t* h_small = nullptr; // pinned: totals read back from the device
    uint64_t launches = 0;
    std::string last_error;
};

namespace {

kvsmc_status fail(kvsmc_context* ctx, kvsmc_status st, const char* fmt, ...)
{
    if (ctx) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        ctx->last_error = buf;
    }
    return st;
}

#define KVSMC_CUDA(ctx, call)                                                          \
    do {                                                                               \
        cudaError_t e_ = (call);                                                       \
        if (e_ != cudaSuccess)                                                         \
            return fail(ctx, e_ == cudaErrorMemoryAllocation ? KVSMC_ERR_OUT_OF_MEMORY \
                                                             : KVSMC_ERR_CUDA,         \
                        "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

Launch launch_of(kvsmc_context* ctx) { return Launch{ctx->stream, ctx->num_sms, &ctx->launches}; }

kvsmc_status ensure_scratch(kvsmc_context* ctx, size_t bytes)
{
    if (bytes <= ctx->scratch_bytes) return KVSMC_OK;
    if (ctx->scratch) {
        KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        cudaFree(ctx->scratch);
        ctx->scratch = nullptr;
        ctx->scratch_bytes = 0;
    }
    const size_t want = align_up(bytes + bytes / 4, 1 << 20);
    KVSMC_CUDA(ctx, cudaMalloc(&ctx->scratch, want));
    ctx->scratch_bytes = want;
    return KVSMC_OK;
}

// Bump allocator over the scratch arena (256-byte aligned pieces).
struct Carve {
    char* base;
    size_t off = 0;
    template <typename P> P* take(size_t bytes) {
        P* p = reinterpret_cast<P*>(base + off);
        off = align_up(off + bytes, 256);
        return p;
    }
};

uint64_t elems_per_16B(int dtype) { return 16 / dtype_size(dtype); }

kvsmc_status volume_alloc(kvsmc_context* ctx, kvsmc_dtype dtype, uint32_t nx, uint32_t ny, uint32_t nz,
                          kvsmc_volume* v)
{
    const size_t es = dtype_size(dtype);
    const uint64_t pitch = align_up(nx, elems_per_16B(dtype));
    const size_t bytes = (size_t)pitch * ny * nz * es + 256;  // tail slack for vector loads
    v->view.nx = nx; v->view.ny = ny; v->view.nz = nz;
    v->view.dtype = dtype;
    v->view.pitch = pitch;
    v->view.slice = pitch * ny;
    if (bytes > v->bytes) {
        if (v->dev) cudaFree(v->dev);
        v->dev = nullptr;
        v->bytes = 0;
        KVSMC_CUDA(ctx, cudaMalloc(&v->dev, bytes));
        v->bytes = bytes;
    }
    v->view.data = v->dev;
    v->has_minmax = false;
    return KVSMC_OK;
}

kvsmc_status volume_copy_in(kvsmc_context* ctx, kvsmc_volume* v, const void* src, cudaMemcpyKind kind)
{
    const size_t es = dtype_size(v->view.dtype);
    const size_t row = (size_t)v->view.nx * es;
    const size_t rows = (size_t)v->view.ny * v->view.nz;
    if (v->view.pitch == v->view.nx) {
        KVSMC_CUDA(ctx, cudaMemcpyAsync(v->dev, src, row * rows, kind, ctx->stream));
    } else {
        KVSMC_CUDA(ctx, cudaMemcpy2DAsync(v->dev, v->view.pitch * es, src, row, row, rows, kind, ctx->stream));
    }
    v->has_minmax = false;
    return KVSMC_OK;
}

kvsmc_status check_shape(kvsmc_context* ctx, int dtype, uint32_t nx, uint32_t ny, uint32_t nz)
{
    if (dtype_size(dtype) == 0) return fail(ctx, KVSMC_ERR_UNSUPPORTED_DTYPE, "unsupported data type %d", dtype);
    if (nx == 0 || ny == 0 || nz == 0) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "empty volume %ux%ux%u", nx, ny, nz);
    return KVSMC_OK;
}

kvsmc_status volume_minmax(kvsmc_context* ctx, kvsmc_volume* v)
{
    if (v->has_minmax) return KVSMC_OK;
    kvsmc_status st = ensure_scratch(ctx, minmax_scratch_bytes(ctx->num_sms) + 256);
    if (st) return st;
    double* d_out = reinterpret_cast<double*>(static_cast<char*>(ctx->scratch) + align_up(minmax_scratch_bytes(ctx->num_sms), 256));
    KVSMC_CUDA(ctx, launch_minmax(v->view, ctx->scratch, d_out, launch_of(ctx)));
    KVSMC_CUDA(ctx, cudaMemcpyAsync(ctx->h_small, d_out, 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    double mm[2];
    std::memcpy(mm, ctx->h_small, sizeof mm);
    v->vmin = mm[0];
    v->vmax = mm[1];
    v->has_minmax = true;
    return KVSMC_OK;
}

// kvs::Math::Equal for doubles (Utility/Math.h:135-138).
bool equal_ref(double a, double b)
{
    const double d = a - b;
    return ((d < 0) ? -d : d) < 1.e-6;
}

// Exact classification thresholds (see Classifier).
Classifier make_classifier(int dtype, double iso)
{
    Classifier c;
    c.iso = iso;
    c.pad = 0;
    float f = (float)iso;
    if (!std::isnan(iso) && (double)f > iso) f = std::nextafter(f, -INFINITY);
    c.f_thr = f;
    if (std::isnan(iso) || iso >= 4.0e18) c.i_thr = 0x7fffffffffffffffLL;
    else if (iso < -4.0e18) c.i_thr = (long long)(-0x7fffffffffffffffLL - 1);
    else c.i_thr = (long long)std::floor(iso);
    (void)dtype;
    return c;
}

struct Plan {
    Job job;
    bool extracted = true;
    bool shared = false;
    uint64_t ntri = 0, nvert = 0;
    double vmin = 0, vmax = 0;
};

uint32_t rows_for(uint32_t width, uint32_t limit)
{
    if (width == 0 || limit == 0) return 1;
    uint32_t r = (2048 + width - 1) / width;
    if (r < 1) r = 1;
    if (r > limit) r = limit;
    return r;
}

kvsmc_status plan_request(kvsmc_context* ctx, kvsmc_volume* vol, const kvsmc_params* p, Plan& pl)
{
    if (!vol || !p) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "null volume or params");
    if (p->mode < 0 || p->mode > 2) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "bad mode %d", p->mode);
    if (p->has_minmax) {
        pl.vmin = p->min_value;
        pl.vmax = p->max_value;
    } else {
        kvsmc_status st = volume_minmax(ctx, vol);
        if (st) return st;
        pl.vmin = vol->vmin;
        pl.vmax = vol->vmax;
    }
    pl.extracted = !equal_ref(pl.vmin, pl.vmax);
    pl.shared = p->mode != KVSMC_DUP_POLYGON_NORMAL;
    Job& j = pl.job;
    std::memset(&j, 0, sizeof j);
    j.vol = vol->view;
    j.cls = make_classifier(vol->view.dtype, p->isolevel);
    j.vmin = pl.vmin;
    j.vmax = pl.vmax;
    for (int k = 0; k < 3; ++k) { j.min_coord[k] = p->min_coord[k]; j.scale[k] = p->scale[k]; }
    j.mode = p->mode;
    const uint32_t nx = vol->view.nx, ny = vol->view.ny, nz = vol->view.nz;
    const bool has_cells = nx > 1 && ny > 1 && nz > 1;
    j.cell_rows = rows_for(nx - 1, ny - 1);
    j.cell_ytiles = has_cells ? (ny - 1 + j.cell_rows - 1) / j.cell_rows : 0;
    j.cell_tiles = has_cells ? (uint64_t)(nz - 1) * j.cell_ytiles : 0;
    j.node_rows = rows_for(nx, ny);
    j.node_ytiles = (ny + j.node_rows - 1) / j.node_rows;
    j.node_tiles = pl.shared ? (uint64_t)nz * j.node_ytiles : 0;
    j.words_per_row = (nx + 31) / 32;
    return KVSMC_OK;
}

// Count pass: fills pl.ntri / pl.nvert; leaves per-tile offsets in scratch.
kvsmc_status count_request(kvsmc_context* ctx, Plan& pl)
{
    pl.ntri = pl.nvert = 0;
    if (!pl.extracted) return KVSMC_OK;
    Job& j = pl.job;
    const size_t ct = j.cell_tiles, nt = j.node_tiles;
    const uint64_t rank_words = pl.shared ? (uint64_t)j.vol.nz * j.vol.ny * j.words_per_row : 0;
    const size_t need = 8 * 256 + align_up(ct * 4, 256) + align_up(ct * 8, 256) + align_up(nt * 4, 256) +
                        align_up(nt * 8, 256) + align_up(rank_words * 16, 256) +
                        align_up(scan_scratch_bytes(ct), 256) + align_up(scan_scratch_bytes(nt), 256);
    kvsmc_status st = ensure_scratch(ctx, need);
    if (st) return st;
    Carve cv{static_cast<char*>(ctx->scratch)};
    uint64_t* d_totals = cv.take<uint64_t>(256);
    j.tile_counts = cv.take<uint32_t>(ct * 4);
    j.tile_offsets = cv.take<uint64_t>(ct * 8);
    j.vtile_counts = cv.take<uint32_t>(nt * 4);
    j.vtile_offsets = cv.take<uint64_t>(nt * 8);
    j.rank = cv.take<uint4>(rank_words * 16);
    void* scan_a = cv.take<char>(scan_scratch_bytes(ct));
    void* scan_b = cv.take<char>(scan_scratch_bytes(nt));
    const Launch L = launch_of(ctx);
    KVSMC_CUDA(ctx, cudaMemsetAsync(d_totals, 0, 2 * sizeof(uint64_t), ctx->stream));
    if (ct) {
        KVSMC_CUDA(ctx, launch_cell_count(j, L));
        KVSMC_CUDA(ctx, launch_scan(j.tile_counts, j.tile_offsets, ct, scan_a, d_totals, L));
    }
    if (nt) {
        KVSMC_CUDA(ctx, launch_node_count(j, L));
        KVSMC_CUDA(ctx, launch_scan(j.vtile_counts, j.vtile_offsets, nt, scan_b, d_totals + 1, L));
    }
    KVSMC_CUDA(ctx, cudaMemcpyAsync(ctx->h_small, d_totals, 2 * sizeof(uint64_t), cudaMemcpyDeviceToHost, ctx->stream));
    KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    pl.ntri = ctx->h_small[0];
    pl.nvert = pl.shared ? ctx->h_small[1] : 3 * pl.ntri;
    if (pl.shared && pl.nvert > 0xffffffffull)
        return fail(ctx, KVSMC_ERR_TOO_LARGE, "%llu shared vertices exceed 32-bit connection ids",
                    (unsigned long long)pl.nvert);
    return KVSMC_OK;
}

void fill_sizes(const Plan& pl, const kvsmc_params* p, kvsmc_sizes* s)
{
    std::memset(s, 0, sizeof *s);
    s->ntriangles = pl.ntri;
    s->nvertices = pl.nvert;
    s->min_value = pl.vmin;
    s->max_value = pl.vmax;
    s->extracted = pl.extracted ? 1 : 0;
    if (!pl.extracted) return;
    if (!pl.shared) {
        s->ncoords = 9 * pl.ntri;
        s->nnormals = 3 * pl.ntri;
        s->nconnections = 0;
    } else {
        s->ncoords = 3 * pl.nvert;
        s->nconnections = 3 * pl.ntri;
        // calculate_normals_on_polygon sizes by connections, on_vertex by coords;
        // both produce nothing when there are no coords (MarchingCubes.cpp:536,574).
        if (pl.nvert == 0) s->nnormals = 0;
        else s->nnormals = (p->mode == KVSMC_SHARED_VERTEX_NORMAL) ? 3 * pl.nvert : 3 * pl.ntri;
    }
}

kvsmc_status emit_request(kvsmc_context* ctx, Plan& pl, float* coords, float* normals, uint32_t* conn)
{
    if (!pl.extracted) return KVSMC_OK;
    Job& j = pl.job;
    j.coords = coords;
    j.normals = normals;
    j.connections = conn;
    const Launch L = launch_of(ctx);
    if (!pl.shared) {
        if (pl.ntri) KVSMC_CUDA(ctx, launch_emit_dup(j, L));
        return KVSMC_OK;
    }
    if (pl.nvert) KVSMC_CUDA(ctx, launch_node_emit(j, L));
    if (pl.ntri) KVSMC_CUDA(ctx, launch_connect(j, L));
    if (pl.nvert && j.mode == KVSMC_SHARED_VERTEX_NORMAL) KVSMC_CUDA(ctx, launch_vertex_normals(j, L));
    return KVSMC_OK;
}

kvsmc_status use_device(kvsmc_context* ctx)
{
    if (!ctx) return KVSMC_ERR_INVALID_ARGUMENT;
    KVSMC_CUDA(ctx, cudaSetDevice(ctx->device));
    return KVSMC_OK;
}

}  // namespace

// =================================================================== C ABI

extern "C" {

const char* kvsmc_status_string(kvsmc_status st)
{
    switch (st) {
    case KVSMC_OK: return "ok";
    case KVSMC_ERR_INVALID_ARGUMENT: return "invalid argument";
    case KVSMC_ERR_UNSUPPORTED_DTYPE: return "unsupported data type";
    case KVSMC_ERR_OUT_OF_MEMORY: return "out of memory";
    case KVSMC_ERR_CUDA: return "CUDA error";
    case KVSMC_ERR_NO_DEVICE: return "no CUDA device";
    case KVSMC_ERR_CAPACITY: return "output buffer too small";
    case KVSMC_ERR_TOO_LARGE: return "result exceeds 32-bit vertex ids";
    case KVSMC_ERR_TIMEOUT: return "device-side wait timed out";
    case KVSMC_ERR_BUDGET: return "request exceeds the memory budget";
    }
    return "unknown status";
}

kvsmc_status kvsmc_create(int device, kvsmc_context** out)
{
    if (!out) return KVSMC_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return KVSMC_ERR_NO_DEVICE;
    }
    if (device < 0 && cudaGetDevice(&device) != cudaSuccess) return KVSMC_ERR_NO_DEVICE;
    if (device >= n) return KVSMC_ERR_INVALID_ARGUMENT;
    kvsmc_context* ctx = new kvsmc_context();
    ctx->device = device;
    if (cudaSetDevice(device) != cudaSuccess ||
        cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMallocHost(&ctx->h_small, 64 * sizeof(uint64_t)) != cudaSuccess) {
        cudaGetLastError();
        if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
        delete ctx;
        return KVSMC_ERR_CUDA;
    }
    ctx->stream = ctx->own_stream;
    *out = ctx;
    return KVSMC_OK;
}

void kvsmc_destroy(kvsmc_context* ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (ctx->host_vol) { cudaFree(ctx->host_vol->dev); delete ctx->host_vol; }
    if (ctx->scratch) cudaFree(ctx->scratch);
    if (ctx->out_arena) cudaFree(ctx->out_arena);
    if (ctx->h_small) cudaFreeHost(ctx->h_small);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    delete ctx;
}

const char* kvsmc_last_error(const kvsmc_context* ctx) { return ctx ? ctx->last_error.c_str() : ""; }

void* kvsmc_stream(kvsmc_context* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

kvsmc_status kvsmc_set_stream(kvsmc_context* ctx, void* s)
{
    if (!ctx) return KVSMC_ERR_INVALID_ARGUMENT;
    ctx->stream = s ? static_cast<cudaStream_t>(s) : ctx->own_stream;
    return KVSMC_OK;
}

kvsmc_status kvsmc_synchronize(kvsmc_context* ctx)
{
    kvsmc_status st = use_device(ctx);
    if (st) return st;
    KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return KVSMC_OK;
}

uint64_t kvsmc_kernel_launches(const kvsmc_context* ctx) { return ctx ? ctx->launches : 0; }

kvsmc_status kvsmc_volume_upload(kvsmc_context* ctx, const void* host, kvsmc_dtype dtype,
                                 uint32_t nx, uint32_t ny, uint32_t nz, kvsmc_volume** out)
{
    kvsmc_status st = use_device(ctx);
    if (st) return st;
    if (!host || !out) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "null pointer");
    if ((st = check_shape(ctx, dtype, nx, ny, nz))) return st;
    kvsmc_volume* v = new kvsmc_volume();
    if ((st = volume_alloc(ctx, dtype, nx, ny, nz, v)) || (st = volume_copy_in(ctx, v, host, cudaMemcpyHostToDevice))) {
        if (v->dev) cudaFree(v->dev);
        delete v;
        return st;
    }
    *out = v;
    return KVSMC_OK;
}

kvsmc_status kvsmc_volume_from_device(kvsmc_context* ctx, const void* dev, kvsmc_dtype dtype,
                                      uint32_t nx, uint32_t ny, uint32_t nz, kvsmc_volume** out)
{
    kvsmc_status st = use_device(ctx);
    if (st) return st;
    if (!dev || !out) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "null pointer");
    if ((st = check_shape(ctx, dtype, nx, ny, nz))) return st;
    kvsmc_volume* v = new kvsmc_volume();
    if ((st = volume_alloc(ctx, dtype, nx, ny, nz, v)) || (st = volume_copy_in(ctx, v, dev, cudaMemcpyDeviceToDevice))) {
        if (v->dev) cudaFree(v->dev);
        delete v;
        return st;
    }
    *out = v;
    return KVSMC_OK;
}

kvsmc_status kvsmc_volume_update(kvsmc_context* ctx, kvsmc_volume* v, const void* host)
{
    kvsmc_status st = use_device(ctx);
    if (st) return st;
    if (!v || !host) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "null pointer");
    return volume_copy_in(ctx, v, host, cudaMemcpyHostToDevice);
}

void kvsmc_volume_free(kvsmc_context* ctx, kvsmc_volume* v)
{
    if (!v) return;
    if (ctx) {
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
    }
    if (v->dev) cudaFree(v->dev);
    delete v;
}

kvsmc_status kvsmc_volume_minmax(kvsmc_context* ctx, kvsmc_volume* v, double* mn, double* mx)
{
    kvsmc_status st = use_device(ctx);
    if (st) return st;
    if (!v) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "null volume");
    if ((st = volume_minmax(ctx, v))) return st;
    if (mn) *mn = v->vmin;
    if (mx) *mx = v->vmax;
    return KVSMC_OK;
}

kvsmc_status kvsmc_count(kvsmc_context* ctx, kvsmc_volume* vol, const kvsmc_params* p, kvsmc_sizes* sizes)
{
    kvsmc_status st = use_device(ctx);
    if (st) return st;
    if (!sizes) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "null sizes");
    Plan pl;
    if ((st = plan_request(ctx, vol, p, pl))) return st;
    if ((st = count_request(ctx, pl))) return st;
    fill_sizes(pl, p, sizes);
    return KVSMC_OK;
}

kvsmc_status kvsmc_extract_device(kvsmc_context* ctx, kvsmc_volume* vol, const kvsmc_params* p,
                                  float* d_coords, uint64_t coords_cap, float* d_normals, uint64_t normals_cap,
                                  uint32_t* d_conn, uint64_t conn_cap, kvsmc_sizes* sizes)
{
    kvsmc_status st = use_device(ctx);
    if (st) return st;
    if (!sizes) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "null sizes");
    Plan pl;
    if ((st = plan_request(ctx, vol, p, pl))) return st;
    if ((st = count_request(ctx, pl))) return st;
    fill_sizes(pl, p, sizes);
    if (sizes->ncoords > coords_cap || sizes->nnormals > normals_cap || sizes->nconnections > conn_cap)
        return fail(ctx, KVSMC_ERR_CAPACITY, "output needs %llu coords, %llu normals, %llu connections",
                    (unsigned long long)sizes->ncoords, (unsigned long long)sizes->nnormals,
                    (unsigned long long)sizes->nconnections);
    if ((sizes->ncoords && !d_coords) || (sizes->nnormals && !d_normals) || (sizes->nconnections && !d_conn))
        return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "null output buffer");
    if ((st = emit_request(ctx, pl, d_coords, d_normals, d_conn))) return st;
    KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return KVSMC_OK;
}

kvsmc_status kvsmc_marching_cubes_host(kvsmc_context* ctx, const void* host, kvsmc_dtype dtype,
                                       uint32_t nx, uint32_t ny, uint32_t nz, const kvsmc_params* p,
                                       kvsmc_host_alloc_fn alloc, void* user, kvsmc_sizes* sizes)
{
    kvsmc_status st = use_device(ctx);
    if (st) return st;
    if (!host || !p || !alloc || !sizes) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "null pointer");
    if ((st = check_shape(ctx, dtype, nx, ny, nz))) return st;
    if (!ctx->host_vol) ctx->host_vol = new kvsmc_volume();
    kvsmc_volume* v = ctx->host_vol;
    if ((st = volume_alloc(ctx, dtype, nx, ny, nz, v))) return st;
    if ((st = volume_copy_in(ctx, v, host, cudaMemcpyHostToDevice))) return st;
    Plan pl;
    if ((st = plan_request(ctx, v, p, pl))) return st;
    if ((st = count_request(ctx, pl))) return st;
    fill_sizes(pl, p, sizes);
    const size_t bc = align_up(sizes->ncoords * 4, 256), bn = align_up(sizes->nnormals * 4, 256);
    const size_t bk = align_up(sizes->nconnections * 4, 256);
    if (bc + bn + bk > ctx->out_bytes) {
        if (ctx->out_arena) cudaFree(ctx->out_arena);
        ctx->out_arena = nullptr;
        ctx->out_bytes = 0;
        const size_t want = align_up(bc + bn + bk, 1 << 20);
        KVSMC_CUDA(ctx, cudaMalloc(&ctx->out_arena, want));
        ctx->out_bytes = want;
    }
    char* base = static_cast<char*>(ctx->out_arena);
    float* dc = reinterpret_cast<float*>(base);
    float* dn = reinterpret_cast<float*>(base + bc);
    uint32_t* dk = reinterpret_cast<uint32_t*>(base + bc + bn);
    if ((st = emit_request(ctx, pl, dc, dn, dk))) return st;
    void* hc = nullptr;
    void* hn = nullptr;
    void* hk = nullptr;
    if (sizes->ncoords && !(hc = alloc(user, 0, sizes->ncoords))) return fail(ctx, KVSMC_ERR_OUT_OF_MEMORY, "host alloc (coords)");
    if (sizes->nnormals && !(hn = alloc(user, 1, sizes->nnormals))) return fail(ctx, KVSMC_ERR_OUT_OF_MEMORY, "host alloc (normals)");
    if (sizes->nconnections && !(hk = alloc(user, 2, sizes->nconnections))) return fail(ctx, KVSMC_ERR_OUT_OF_MEMORY, "host alloc (connections)");
    if (hc) KVSMC_CUDA(ctx, cudaMemcpyAsync(hc, dc, sizes->ncoords * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (hn) KVSMC_CUDA(ctx, cudaMemcpyAsync(hn, dn, sizes->nnormals * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (hk) KVSMC_CUDA(ctx, cudaMemcpyAsync(hk, dk, sizes->nconnections * 4, cudaMemcpyDeviceToHost, ctx->stream));
    KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return KVSMC_OK;
}

kvsmc_status kvsmc_count_batch(kvsmc_context* ctx, kvsmc_request* reqs, int32_t n)
{
    kvsmc_status st = use_device(ctx);
    if (st) return st;
    if (!reqs || n < 0) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "bad batch");
    kvsmc_status first = KVSMC_OK;
    for (int32_t i = 0; i < n; ++i) {
        reqs[i].status = kvsmc_count(ctx, reqs[i].volume, &reqs[i].params, &reqs[i].sizes);
        if (reqs[i].status && !first) first = reqs[i].status;
    }
    return first;
}

kvsmc_status kvsmc_extract_batch(kvsmc_context* ctx, kvsmc_request* reqs, int32_t n)
{
    kvsmc_status st = use_device(ctx);
    if (st) return st;
    if (!reqs || n < 0) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "bad batch");
    kvsmc_status first = KVSMC_OK;
    for (int32_t i = 0; i < n; ++i) {
        kvsmc_request& r = reqs[i];
        r.status = kvsmc_extract_device(ctx, r.volume, &r.params, r.d_coords, r.coords_capacity, r.d_normals,
                                        r.normals_capacity, r.d_connections, r.connections_capacity, &r.sizes);
        if (r.status && !first) first = r.status;
    }
    return first;
}

}  // extern "C"
