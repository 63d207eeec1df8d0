// api.cu -- the C ABI of libkvsmc (include/kvsmc.h): contexts, resident
// volumes, and request pipelines.  Duplicated-mode requests on 8/16-bit and
// float32 volumes run through the streaming kernels (batch.cu); the others
// through the gather kernels (mc_gather.cu), one request at a time.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <unordered_map>
#include <vector>

#include "batch.h"

using namespace kvsmc;

namespace kvsmc_host {

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

kvsmc_status ensure_stage(kvsmc_context* ctx, size_t bytes)
{
    if (bytes <= ctx->h_stage_bytes) return KVSMC_OK;
    if (ctx->h_stage) {
        KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        cudaFreeHost(ctx->h_stage);
        ctx->h_stage = nullptr;
        ctx->h_stage_bytes = 0;
    }
    const size_t want = align_up(bytes + bytes / 4, 1 << 16);
    KVSMC_CUDA(ctx, cudaMallocHost(&ctx->h_stage, want));
    ctx->h_stage_bytes = want;
    return KVSMC_OK;
}

kvsmc_status volume_minmax(kvsmc_context* ctx, kvsmc_volume* v)
{
    if (v->has_minmax) return KVSMC_OK;
    const size_t part = align_up(minmax_scratch_bytes(ctx->num_sms), 256);
    kvsmc_status st = ensure_scratch(ctx, part + 256);
    if (st) return st;
    double* d_out = reinterpret_cast<double*>(static_cast<char*>(ctx->scratch) + part);
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
Classifier make_classifier(double iso)
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
    return c;
}

cudaError_t fan_out(kvsmc_context* ctx, cudaStream_t origin, size_t n,
                    const std::function<cudaError_t(size_t, cudaStream_t)>& fn)
{
    if (n == 0) return cudaSuccess;
    if (n == 1) return fn(0, origin);
    cudaError_t e = cudaSuccess;
    if (!ctx->aux_ready) {
        for (int i = 0; i < kvsmc_context::kAux && e == cudaSuccess; ++i) {
            e = cudaStreamCreateWithFlags(&ctx->aux[i], cudaStreamNonBlocking);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->join_ev[i], cudaEventDisableTiming);
        }
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->fork_ev, cudaEventDisableTiming);
        if (e != cudaSuccess) return e;
        ctx->aux_ready = true;
    }
    e = cudaEventRecord(ctx->fork_ev, origin);
    const size_t used = n < (size_t)kvsmc_context::kAux ? n : (size_t)kvsmc_context::kAux;
    for (size_t j = 0; j < used && e == cudaSuccess; ++j) e = cudaStreamWaitEvent(ctx->aux[j], ctx->fork_ev, 0);
    for (size_t i = 0; i < n && e == cudaSuccess; ++i) e = fn(i, ctx->aux[i % kvsmc_context::kAux]);
    for (size_t j = 0; j < used && e == cudaSuccess; ++j) e = cudaEventRecord(ctx->join_ev[j], ctx->aux[j]);
    for (size_t j = 0; j < used && e == cudaSuccess; ++j) e = cudaStreamWaitEvent(origin, ctx->join_ev[j], 0);
    return e;
}

kvsmc_status volume_bricks(kvsmc_context* ctx, kvsmc_volume* v)
{
    v->bricks_valid = false;
    const int dt = v->view.dtype;
    const bool ok = (dt == KVSMC_I8 || dt == KVSMC_I16 || dt == KVSMC_U8 || dt == KVSMC_U16 || dt == KVSMC_F32) &&
                    v->view.nx - 1 <= (uint32_t)kvsmc::kStreamMaxCells;
    if (!ok) return KVSMC_OK;
    const size_t bytes = kvsmc::brick_count(v->view) * sizeof(float2);
    if (bytes > v->brick_bytes) {
        if (v->bricks) cudaFree(v->bricks);
        v->bricks = nullptr;
        v->brick_bytes = 0;
        KVSMC_CUDA(ctx, cudaMalloc(&v->bricks, bytes));
        v->brick_bytes = bytes;
    }
    KVSMC_CUDA(ctx, kvsmc::launch_bricks(v->view, v->bricks, launch_of(ctx)));
    v->bricks_valid = true;
    return KVSMC_OK;
}

// Decide min/max (MapperBase::setRange) and the Equal early exit.
kvsmc_status prepare(kvsmc_context* ctx, Item& it)
{
    if (!it.vol) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "null volume");
    if (it.params.mode < 0 || it.params.mode > 2) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "bad mode %d", it.params.mode);
    if (it.params.has_minmax) {
        it.vmin = it.params.min_value;
        it.vmax = it.params.max_value;
    } else {
        kvsmc_status st = volume_minmax(ctx, it.vol);
        if (st) return st;
        it.vmin = it.vol->vmin;
        it.vmax = it.vol->vmax;
    }
    it.extracted = !equal_ref(it.vmin, it.vmax);
    std::memset(&it.sizes, 0, sizeof it.sizes);
    it.sizes.min_value = it.vmin;
    it.sizes.max_value = it.vmax;
    return KVSMC_OK;
}

}  // namespace kvsmc_host

using namespace kvsmc_host;

namespace {

size_t elems_per_16B(int dtype) { return 16 / dtype_size(dtype); }

kvsmc_status volume_alloc(kvsmc_context* ctx, kvsmc_dtype dtype, uint32_t nx, uint32_t ny, uint32_t nz,
                          kvsmc_volume* v)
{
    const size_t es = dtype_size(dtype);
    const uint64_t pitch = align_up(nx, elems_per_16B(dtype));
    const size_t bytes = (size_t)pitch * ny * nz * es + 256;
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

// ------------------------------------------------------------ gather pipeline

struct Plan {
    Job job;
    bool shared = false;
    uint64_t ntri = 0, nvert = 0;
    // shared-vertex node passes on the streaming kernels (8/16-bit and float32
    // volumes): node units (plane, row, 256-node segment), their task shape,
    // the FP32 vertex path's constants, the status word and task counters
    bool snode = false;
    uint32_t wprn = 0, zchunk = 0;
    uint64_t ntasks = 0;
    kvsmc::FastIso f{};
    int* d_status = nullptr;
    unsigned long long* d_next = nullptr;
    // triangles of a shared-vertex request on the streaming count and the
    // streaming connection pass (one row per task): the request is isolevel
    // sb_iso of group sb_group of the count `sb`, either its own (`batch`) or
    // one shared by the batch's requests on the same volume, counted before
    // (set by the caller before gather_count; sb_tasks = the group's tasks)
    Item* item = nullptr;
    bool sconn = false;
    std::unique_ptr<StreamBatch> batch;
    StreamBatch* sb = nullptr;
    int sb_group = 0;
    uint32_t sb_iso = 0;
    uint64_t sb_tasks = 0;
    // the request's vertex counts per node unit from that shared count (null:
    // the node count pass counts them)
    const uint32_t* sb_nodes = nullptr;
    // its vertices and rank words were written by the multi-isolevel node emit
    bool nodes_done = false;
    // its connections and (per-triangle) normals were written by the
    // multi-isolevel connection pass; tri_normals: where its per-triangle
    // normals are (VertexNormal), kept until its vertex normals
    bool conn_done = false;
    float* tri_normals = nullptr;
};

uint32_t rows_for(uint32_t width, uint32_t limit)
{
    if (width == 0 || limit == 0) return 1;
    uint32_t r = (2048 + width - 1) / width;
    if (r < 1) r = 1;
    if (r > limit) r = limit;
    return r;
}

void gather_plan(const Item& it, Plan& pl)
{
    pl.item = const_cast<Item*>(&it);
    pl.shared = it.params.mode != KVSMC_DUP_POLYGON_NORMAL;
    Job& j = pl.job;
    std::memset(&j, 0, sizeof j);
    j.vol = it.vol->view;
    j.cls = make_classifier(it.params.isolevel);
    j.ip.iso = it.params.isolevel;
    j.ip.vmin = it.vmin;
    j.ip.vmax = it.vmax;
    for (int k = 0; k < 3; ++k) { j.ip.min_coord[k] = it.params.min_coord[k]; j.ip.scale[k] = it.params.scale[k]; }
    j.mode = it.params.mode;
    const uint32_t nx = j.vol.nx, ny = j.vol.ny, nz = j.vol.nz;
    const bool has_cells = nx > 1 && ny > 1 && nz > 1;
    j.cell_rows = rows_for(nx - 1, ny - 1);
    j.cell_ytiles = has_cells ? (ny - 1 + j.cell_rows - 1) / j.cell_rows : 0;
    j.cell_tiles = has_cells ? (uint64_t)(nz - 1) * j.cell_ytiles : 0;
    j.node_rows = rows_for(nx, ny);
    j.node_ytiles = (ny + j.node_rows - 1) / j.node_rows;
    j.node_tiles = pl.shared ? (uint64_t)nz * j.node_ytiles : 0;
    j.words_per_row = (nx + 31) / 32;
}

// The pass shapes of one gather request (node units of the streaming node
// passes, the streaming connection pass or the cell tiles).
void gather_setup(kvsmc_context* ctx, Plan& pl)
{
    pl.ntri = pl.nvert = 0;
    Job& j = pl.job;
    const int dt = j.vol.dtype;
    pl.snode = pl.shared && ctx->path == 0 &&
               (dt == KVSMC_I8 || dt == KVSMC_I16 || dt == KVSMC_U8 || dt == KVSMC_U16 || dt == KVSMC_F32);
    if (pl.snode) {
        // node units replace the node tiles: (plane, row, 256-node segment)
        pl.wprn = (j.vol.nx + 255) / 256;
        const uint64_t steps = (uint64_t)j.vol.nz * j.vol.ny * pl.wprn;
        pl.zchunk = kvsmc_host::stream_zchunk(steps, ctx->num_sms);
        pl.ntasks = (uint64_t)((j.vol.nz + pl.zchunk - 1) / pl.zchunk) * j.vol.ny * pl.wprn;
        pl.f = kvsmc_host::make_fast(j.ip.iso, j.ip.vmin, j.ip.vmax, dt);
        j.node_tiles = steps;   // node units, for the counts and their scan
        // the triangles too: the streaming count and the streaming connection
        // pass when the volume takes the streaming layout with one row per task
        if (pl.sb) {
            pl.sconn = true;
            j.cell_tiles = 0;
        } else if (stream_volume_eligible(ctx, *pl.item)) {
            pl.batch.reset(new StreamBatch());
            pl.batch->ctx = ctx;
            pl.batch->items = {pl.item};
            pl.batch->plan_tables();
            pl.sconn = pl.batch->groups.size() == 1 && pl.batch->launches.size() == 1 && pl.batch->groups[0].rows == 1;
            if (pl.sconn) {
                j.cell_tiles = 0;
                pl.sb = pl.batch.get();
                pl.sb_group = 0;
                pl.sb_iso = 0;
                pl.sb_tasks = pl.batch->launches[0].ntasks;
            } else {
                pl.batch.reset();
            }
        }
    }
}

// Bytes of a set-up request's own count arrays (tiles, rank words, scans,
// status words), its own streaming count excluded.
size_t gather_own_bytes(const Plan& pl)
{
    const Job& j = pl.job;
    const size_t ct = j.cell_tiles, nt = j.node_tiles;
    const uint64_t rank_words = pl.shared ? (uint64_t)j.vol.nz * j.vol.ny * j.words_per_row : 0;
    return 10 * 256 + align_up(ct * 4, 256) + align_up(ct * 8, 256) + align_up(nt * 4, 256) + align_up(nt * 8, 256) +
           align_up(rank_words * 16, 256) + align_up(scan_scratch_bytes(ct), 256) + align_up(scan_scratch_bytes(nt), 256);
}

// Count pass of one set-up request with its arrays carved from `base`
// (gather_own_bytes, then its own streaming count): fills pl.ntri / pl.nvert
// and leaves the per-tile offsets there for gather_emit.
kvsmc_status gather_count_at(kvsmc_context* ctx, Plan& pl, char* base)
{
    Job& j = pl.job;
    const size_t ct = j.cell_tiles, nt = j.node_tiles;
    const uint64_t rank_words = pl.shared ? (uint64_t)j.vol.nz * j.vol.ny * j.words_per_row : 0;
    const size_t own = gather_own_bytes(pl);
    Carve cv{base};
    uint64_t* d_totals = cv.take<uint64_t>(256);
    j.tile_counts = cv.take<uint32_t>(ct * 4);
    j.tile_offsets = cv.take<uint64_t>(ct * 8);
    j.vtile_counts = cv.take<uint32_t>(nt * 4);
    j.vtile_offsets = cv.take<uint64_t>(nt * 8);
    j.rank = cv.take<uint4>(rank_words * 16);
    void* scan_a = cv.take<char>(scan_scratch_bytes(ct));
    void* scan_b = cv.take<char>(scan_scratch_bytes(nt));
    pl.d_status = cv.take<int>(256);
    pl.d_next = cv.take<unsigned long long>(256);
    const kvsmc::Launch L = launch_of(ctx);
    KVSMC_CUDA(ctx, cudaMemsetAsync(d_totals, 0, 3 * sizeof(uint64_t), ctx->stream));
    if (pl.sconn && pl.batch) {
        // unit counts, unit scan, plane scan: the streaming count of one request
        pl.batch->carve(base + own);
        kvsmc_status bst = pl.batch->upload_tables();
        if (!bst) bst = pl.batch->count();
        if (bst) return bst;
    }
    if (ct) {
        KVSMC_CUDA(ctx, launch_cell_count(j, L));
        KVSMC_CUDA(ctx, launch_scan(j.tile_counts, j.tile_offsets, ct, scan_a, d_totals, L));
    }
    if (nt && pl.snode) {
        KVSMC_CUDA(ctx, cudaMemsetAsync(pl.d_status, 0, sizeof(int), ctx->stream));
        KVSMC_CUDA(ctx, cudaMemsetAsync(pl.d_next, 0, 3 * sizeof(unsigned long long), ctx->stream));
        if (!pl.sb_nodes)
            KVSMC_CUDA(ctx, kvsmc::launch_snode(false, j, pl.f, pl.wprn, pl.zchunk, pl.ntasks, j.vtile_counts,
                                                nullptr, pl.d_status, pl.d_next, L));
        KVSMC_CUDA(ctx, launch_scan(pl.sb_nodes ? pl.sb_nodes : j.vtile_counts, j.vtile_offsets, nt, scan_b,
                                    d_totals + 1, L));
        KVSMC_CUDA(ctx, cudaMemcpyAsync(d_totals + 2, pl.d_status, sizeof(int), cudaMemcpyDeviceToDevice, ctx->stream));
    } else if (nt) {
        KVSMC_CUDA(ctx, launch_node_count(j, L));
        KVSMC_CUDA(ctx, launch_scan(j.vtile_counts, j.vtile_offsets, nt, scan_b, d_totals + 1, L));
    }
    KVSMC_CUDA(ctx, cudaMemcpyAsync(ctx->h_small, d_totals, 3 * sizeof(uint64_t), cudaMemcpyDeviceToHost, ctx->stream));
    KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (ctx->h_small[2]) return fail(ctx, KVSMC_ERR_TIMEOUT, "shared-vertex count: a shared-memory load did not complete");
    pl.ntri = pl.sconn ? pl.item->sizes.ntriangles : ctx->h_small[0];
    pl.nvert = pl.shared ? ctx->h_small[1] : 3 * pl.ntri;
    if (pl.shared && pl.nvert > 0xffffffffull)
        return fail(ctx, KVSMC_ERR_TOO_LARGE, "%llu shared vertices exceed 32-bit connection ids",
                    (unsigned long long)pl.nvert);
    return KVSMC_OK;
}

// Count pass of one gather request in the context's scratch arena.
kvsmc_status gather_count(kvsmc_context* ctx, Plan& pl)
{
    gather_setup(ctx, pl);
    const size_t need =
        gather_own_bytes(pl) + (pl.sconn && pl.batch ? align_up(pl.batch->scratch_bytes(), 256) : 0);
    kvsmc_status st = ensure_scratch(ctx, need);
    if (st) return st;
    return gather_count_at(ctx, pl, static_cast<char*>(ctx->scratch));
}

void gather_sizes(const Plan& pl, const Item& it, kvsmc_sizes* s)
{
    std::memset(s, 0, sizeof *s);
    s->ntriangles = pl.ntri;
    s->nvertices = pl.nvert;
    s->min_value = it.vmin;
    s->max_value = it.vmax;
    s->extracted = 1;
    if (!pl.shared) {
        s->ncoords = 9 * pl.ntri;
        s->nnormals = 3 * pl.ntri;
    } else {
        s->ncoords = 3 * pl.nvert;
        s->nconnections = 3 * pl.ntri;
        // calculate_normals_on_polygon sizes by connections, on_vertex by
        // coords; both leave nothing when there are no coords (MarchingCubes.cpp:536,574).
        if (pl.nvert == 0) s->nnormals = 0;
        else s->nnormals = (it.params.mode == KVSMC_SHARED_VERTEX_NORMAL) ? 3 * pl.nvert : 3 * pl.ntri;
    }
}

kvsmc_status gather_emit(kvsmc_context* ctx, Plan& pl, float* coords, float* normals, uint32_t* conn)
{
    Job& j = pl.job;
    j.coords = coords;
    j.normals = normals;
    j.connections = conn;
    const kvsmc::Launch L = launch_of(ctx);
    if (!pl.shared) {
        if (pl.ntri) KVSMC_CUDA(ctx, launch_emit_dup(j, L));
        return KVSMC_OK;
    }
    const bool vertex_normals = pl.nvert && pl.ntri && j.mode == KVSMC_SHARED_VERTEX_NORMAL;
    if (vertex_normals) {
        // per-triangle normals and the vertices' triangle lists live in the
        // context's second arena (the first holds this request's tiles and rank words)
        if (pl.ntri > 0xffffffffull)
            return fail(ctx, KVSMC_ERR_TOO_LARGE, "%llu triangles exceed 32-bit triangle ids of the vertex normals",
                        (unsigned long long)pl.ntri);
        const size_t need = kvsmc::vertex_normals_scratch_bytes(pl.ntri, pl.nvert);
        if (need > ctx->arena2_bytes) {
            KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            if (ctx->arena2) cudaFree(ctx->arena2);
            ctx->arena2 = nullptr;
            ctx->arena2_bytes = 0;
            const size_t want = align_up(need + need / 4, 1 << 20);
            KVSMC_CUDA(ctx, cudaMalloc(&ctx->arena2, want));
            ctx->arena2_bytes = want;
        }
        kvsmc::vertex_normals_carve(j, pl.ntri, pl.nvert, ctx->arena2);
        if (pl.conn_done) j.tri_normals = pl.tri_normals;   // written by the connection pass already
    } else {
        j.tri_normals = nullptr;
    }
    // A pass whose bounded waits gave up leaves its outputs unwritten: the next
    // pass would read those as vertex ids, so the status is checked before it.
    auto check_status = [&](const char* what) -> kvsmc_status {
        int* h = reinterpret_cast<int*>(ctx->h_small);
        KVSMC_CUDA(ctx, cudaMemcpyAsync(h, pl.d_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        if (*h == 1) return fail(ctx, KVSMC_ERR_TIMEOUT, "%s: a shared-memory load did not complete", what);
        if (*h) return fail(ctx, KVSMC_ERR_CUDA, "%s: a vertex id out of range", what);
        return KVSMC_OK;
    };
    kvsmc_status st = KVSMC_OK;
    if (pl.nodes_done) {
        // written already
    } else if (pl.nvert && pl.snode) {
        uint32_t* counts = const_cast<uint32_t*>(pl.sb_nodes ? pl.sb_nodes : j.vtile_counts);
        KVSMC_CUDA(ctx, kvsmc::launch_snode(true, j, pl.f, pl.wprn, pl.zchunk, pl.ntasks, counts, j.vtile_offsets,
                                            pl.d_status, pl.d_next + 1, L));
        if ((st = check_status("shared-vertex node emit"))) return st;
    } else if (pl.nvert) {
        KVSMC_CUDA(ctx, launch_node_emit(j, L));
    }
    if (pl.conn_done) {
        // written already
    } else if (pl.ntri && pl.sconn) {
        StreamBatch& b = *pl.sb;
        KVSMC_CUDA(ctx, kvsmc::launch_sconnect(j, b.d_groups + pl.sb_group, b.d_isos, b.d_unit_counts,
                                               b.d_unit_offsets, b.d_plane_base, pl.sb_iso, pl.sb_tasks, pl.nvert,
                                               pl.ntri, pl.d_status, pl.d_next + 2, L));
        if ((st = check_status("shared-vertex connections"))) return st;
    } else if (pl.ntri) {
        KVSMC_CUDA(ctx, launch_connect(j, L));
    }
    if (vertex_normals) {
        KVSMC_CUDA(ctx, launch_vertex_normals(j, pl.ntri, pl.nvert, L));
    } else if (pl.nvert && j.mode == KVSMC_SHARED_VERTEX_NORMAL) {
        // vertices without any triangle (a volume one node thick): zero normals
        // (calculate_normals_on_vertex adds nothing to its zeroed array)
        KVSMC_CUDA(ctx, cudaMemsetAsync(j.normals, 0, 12 * pl.nvert, ctx->stream));
    }
    return KVSMC_OK;
}

// The streaming triangle count of a batch's shared-vertex requests in one
// pass: requests on the same volume share one read of it (up to 16
// isolevels per group), and each request's connection pass takes its
// isolevel's unit offsets from it.  The same pass counts each request's
// vertices per node unit (groups whose node segments are their cell
// segments), so the requests skip their node count passes.  Requests whose
// group does not take one row per task, and a batch with a single such
// request, keep their own counts.
struct SharedCount {
    std::unique_ptr<StreamBatch> sb;
    std::vector<Item*> cand;   // the requests counted here
    struct Ref {
        int group;
        uint32_t iso;
        uint64_t tasks;
        const uint32_t* nodes;
    };
    std::unordered_map<const Item*, Ref> ref;

    // whether the request's group carries its vertex counts
    bool has_nodes(const Item* it) const
    {
        const auto r = ref.find(it);
        return r != ref.end() && r->second.nodes != nullptr;
    }

    void attach(const Item* it, Plan& pl) const
    {
        const auto r = ref.find(it);
        if (r == ref.end()) return;
        pl.sb = sb.get();
        pl.sb_group = r->second.group;
        pl.sb_iso = r->second.iso;
        pl.sb_tasks = r->second.tasks;
        pl.sb_nodes = r->second.nodes;
    }
};

kvsmc_status shared_count(kvsmc_context* ctx, const std::vector<Item*>& items, SharedCount& sc)
{
    for (Item* it : items) {
        const int m = it->params.mode, dt = it->vol->view.dtype;
        if ((m == KVSMC_SHARED_POLYGON_NORMAL || m == KVSMC_SHARED_VERTEX_NORMAL) && ctx->path == 0 &&
            (dt == KVSMC_I8 || dt == KVSMC_I16 || dt == KVSMC_U8 || dt == KVSMC_U16 || dt == KVSMC_F32) &&
            stream_volume_eligible(ctx, *it) && stream_shape(ctx, it->vol->view).rows == 1)
            sc.cand.push_back(it);   // (the connection pass takes one-row tasks only)
    }
    if (sc.cand.size() < 2) {
        sc.cand.clear();
        return KVSMC_OK;
    }
    sc.sb.reset(new StreamBatch());
    StreamBatch& b = *sc.sb;
    b.ctx = ctx;
    b.items = sc.cand;
    b.want_nodes = true;
    b.plan_tables();
    const size_t need = b.scratch_bytes();
    if (need > ctx->arena3_bytes) {
        KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        if (ctx->arena3) cudaFree(ctx->arena3);
        ctx->arena3 = nullptr;
        ctx->arena3_bytes = 0;
        const size_t want = align_up(need, 1 << 20);
        if (cudaMalloc(&ctx->arena3, want) != cudaSuccess) {
            // no room for the shared count: each request counts on its own
            cudaGetLastError();
            ctx->arena3 = nullptr;
            sc.cand.clear();
            sc.sb.reset();
            return KVSMC_OK;
        }
        ctx->arena3_bytes = want;
    }
    b.carve(static_cast<char*>(ctx->arena3));
    kvsmc_status st = b.upload_tables();
    if (!st) st = b.count();
    if (st) return st;
    for (const StreamBatch::Launch1& l : b.launches) {
        for (int g = l.g0; g < l.g0 + l.ng; ++g) {
            const kvsmc::StreamGroup& G = b.groups[g];
            if (G.rows != 1) continue;
            const uint64_t end = g + 1 < l.g0 + l.ng ? b.groups[g + 1].task_begin : l.ntasks;
            for (int k = 0; k < G.niso; ++k) {
                const uint32_t* nodes = G.node_units ? b.d_node_counts + G.node_base + (uint64_t)k * G.node_units
                                                     : nullptr;
                sc.ref[b.iso_item[G.iso_begin + k]] = SharedCount::Ref{g, (uint32_t)k, end - G.task_begin, nodes};
            }
        }
    }
    return KVSMC_OK;
}

// The requests of a shared count whose groups carry their vertex counts, run
// together: each request's count arrays in its own part of the context's
// fourth arena (they live until its connection pass), then (emit) the
// device outputs from `outputs`, one node emit per group for all its
// requests (k_snode_multi: the volume read once, every node classified once),
// and each request's connections and vertex normals.  Per-request failures
// go to it->status; KVSMC_ERR_OUT_OF_MEMORY (an arena could not grow, before
// any output was written) asks the caller to run the requests one by one.
//
// ready(it, what), when given, is called as soon as outputs of a request are
// final on the context's stream (what: 0 its vertices, 1 its connections and
// any polygon normals, 2 all of its outputs), so a caller can start copying
// them while the later passes run.
kvsmc_status grouped_shared(kvsmc_context* ctx, const SharedCount& sc, std::vector<Item*>& items, bool emit,
                            const std::function<kvsmc_status(std::vector<Item*>&)>& outputs,
                            const std::function<kvsmc_status(Item*, int)>& ready = {})
{
    std::vector<Plan> plans(items.size());
    size_t total = 0;
    std::vector<size_t> off(items.size());
    for (size_t i = 0; i < items.size(); ++i) {
        gather_plan(*items[i], plans[i]);
        sc.attach(items[i], plans[i]);
        gather_setup(ctx, plans[i]);
        off[i] = total;
        total += align_up(gather_own_bytes(plans[i]), 256);
    }
    const size_t tables = align_up((size_t)kvsmc::kStreamMaxIso * sizeof(kvsmc::NodeIso), 256) +
                          align_up((size_t)kvsmc::kStreamMaxIso * sizeof(kvsmc::ConnIso), 256);
    const size_t need = total + tables;
    if (need > ctx->arena4_bytes) {
        KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        if (ctx->arena4) cudaFree(ctx->arena4);
        ctx->arena4 = nullptr;
        ctx->arena4_bytes = 0;
        const size_t want = align_up(need, 1 << 20);
        if (cudaMalloc(&ctx->arena4, want) != cudaSuccess) {
            cudaGetLastError();
            ctx->arena4 = nullptr;
            return KVSMC_ERR_OUT_OF_MEMORY;   // the caller runs the requests one by one
        }
        ctx->arena4_bytes = want;
    }
    char* base = static_cast<char*>(ctx->arena4);
    std::vector<Item*> ok;
    for (size_t i = 0; i < items.size(); ++i) {
        Item* it = items[i];
        kvsmc_status st = gather_count_at(ctx, plans[i], base + off[i]);
        if (!st) gather_sizes(plans[i], *it, &it->sizes);
        if (st) it->status = st;
        else ok.push_back(it);
    }
    if (!emit || ok.empty()) return KVSMC_OK;
    if (kvsmc_status st = outputs(ok)) return st;
    // the VertexNormal requests' per-triangle normals, written by the
    // connection pass, summed by their vertex normals afterwards
    size_t tn_total = 0;
    for (size_t i = 0; i < items.size(); ++i)
        if (!items[i]->status && items[i]->emit && plans[i].job.mode == KVSMC_SHARED_VERTEX_NORMAL)
            tn_total += align_up(12 * plans[i].ntri, 256);
    if (tn_total > ctx->arena5_bytes) {
        KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        if (ctx->arena5) cudaFree(ctx->arena5);
        ctx->arena5 = nullptr;
        ctx->arena5_bytes = 0;
        const size_t want = align_up(tn_total, 1 << 20);
        if (cudaMalloc(&ctx->arena5, want) != cudaSuccess) {
            cudaGetLastError();
            ctx->arena5 = nullptr;
            return KVSMC_ERR_OUT_OF_MEMORY;   // the caller runs the requests one by one
        }
        ctx->arena5_bytes = want;
    }
    {
        size_t o = 0;
        for (size_t i = 0; i < items.size(); ++i)
            if (!items[i]->status && items[i]->emit && plans[i].job.mode == KVSMC_SHARED_VERTEX_NORMAL) {
                plans[i].tri_normals = reinterpret_cast<float*>(static_cast<char*>(ctx->arena5) + o);
                o += align_up(12 * plans[i].ntri, 256);
            }
    }
    std::map<const Item*, Plan*> plan_of;
    for (size_t i = 0; i < items.size(); ++i) plan_of[items[i]] = &plans[i];
    // one node emit per group: its requests in threshold order
    const StreamBatch& b = *sc.sb;
    kvsmc::NodeIso* d_node = reinterpret_cast<kvsmc::NodeIso*>(base + total);
    kvsmc::ConnIso* d_conn = reinterpret_cast<kvsmc::ConnIso*>(
        base + total + align_up((size_t)kvsmc::kStreamMaxIso * sizeof(kvsmc::NodeIso), 256));
    const kvsmc::Launch L = launch_of(ctx);
    for (size_t g = 0; g < b.groups.size(); ++g) {
        const kvsmc::StreamGroup& G = b.groups[g];
        std::vector<Plan*> gp;
        for (int k = 0; k < G.niso; ++k) {
            Item* it = b.iso_item[G.iso_begin + k];
            const auto f = plan_of.find(it);
            if (f == plan_of.end() || it->status || !it->emit || !f->second->sb_nodes || !f->second->nvert) continue;
            gp.push_back(f->second);
        }
        if (gp.empty()) continue;
        kvsmc_status st = ensure_stage(ctx, gp.size() * sizeof(kvsmc::NodeIso));
        if (!st) {
            kvsmc::NodeIso* h = static_cast<kvsmc::NodeIso*>(ctx->h_stage);
            for (size_t k = 0; k < gp.size(); ++k) {
                const Plan& pl = *gp[k];
                h[k].f = pl.f;
                h[k].ip = pl.job.ip;
                h[k].coords = pl.item->d_coords;
                h[k].rank = pl.job.rank;
                h[k].offsets = pl.job.vtile_offsets;
                h[k].counts = pl.sb_nodes;
            }
            const Plan& p0 = *gp[0];
            int* d_status = p0.d_status;
            unsigned long long* d_next = p0.d_next + 1;
            KVSMC_CUDA(ctx, cudaMemcpyAsync(d_node, h, gp.size() * sizeof(kvsmc::NodeIso), cudaMemcpyHostToDevice,
                                            ctx->stream));
            KVSMC_CUDA(ctx, cudaMemsetAsync(d_status, 0, sizeof(int), ctx->stream));
            KVSMC_CUDA(ctx, cudaMemsetAsync(d_next, 0, sizeof(unsigned long long), ctx->stream));
            KVSMC_CUDA(ctx, kvsmc::launch_snode_multi(p0.job.vol, d_node, (int)gp.size(), G.bs, G.bo, p0.wprn,
                                                      p0.zchunk, p0.ntasks, p0.job.words_per_row, d_status, d_next, L));
            int* hs = reinterpret_cast<int*>(ctx->h_small);
            KVSMC_CUDA(ctx, cudaMemcpyAsync(hs, d_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
            KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            if (*hs) st = fail(ctx, KVSMC_ERR_TIMEOUT, "shared-vertex node emit: a shared-memory load did not complete");
            if (!st && ready)   // the vertices leave while the connections are written
                for (Plan* p : gp)
                    if ((st = ready(p->item, 0))) break;
            // then the group's connection pass, every request of the group in its
            // isolevel order (the ones not written here disabled)
            if (!st) st = ensure_stage(ctx, (size_t)G.niso * sizeof(kvsmc::ConnIso));
            if (!st) {
                kvsmc::ConnIso* hc = static_cast<kvsmc::ConnIso*>(ctx->h_stage);
                std::memset(hc, 0, (size_t)G.niso * sizeof(kvsmc::ConnIso));
                uint64_t tasks = 0;
                for (int k = 0; k < G.niso; ++k) {
                    Item* it = b.iso_item[G.iso_begin + k];
                    const auto f = plan_of.find(it);
                    if (f == plan_of.end()) continue;
                    const Plan& pl = *f->second;
                    if (std::find(gp.begin(), gp.end(), f->second) == gp.end() || !pl.ntri) continue;
                    hc[k].rank = pl.job.rank;
                    hc[k].coords = it->d_coords;
                    hc[k].connections = it->d_conn;
                    hc[k].tri_out = pl.job.mode == KVSMC_SHARED_VERTEX_NORMAL ? pl.tri_normals : it->d_normals;
                    hc[k].nvert = pl.nvert;
                    hc[k].ntri = pl.ntri;
                    hc[k].enabled = 1;
                    tasks = pl.sb_tasks;
                }
                if (tasks) {
                    KVSMC_CUDA(ctx, cudaMemcpyAsync(d_conn, hc, (size_t)G.niso * sizeof(kvsmc::ConnIso),
                                                    cudaMemcpyHostToDevice, ctx->stream));
                    KVSMC_CUDA(ctx, cudaMemsetAsync(d_status, 0, sizeof(int), ctx->stream));
                    KVSMC_CUDA(ctx, cudaMemsetAsync(d_next, 0, sizeof(unsigned long long), ctx->stream));
                    KVSMC_CUDA(ctx, kvsmc::launch_sconnect_multi(b.d_groups + g, b.d_isos, d_conn, p0.job.vol.dtype,
                                                                 b.d_unit_counts, b.d_unit_offsets, b.d_plane_base,
                                                                 tasks, d_status, d_next, L));
                    KVSMC_CUDA(ctx, cudaMemcpyAsync(hs, d_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
                    KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
                    if (*hs == 1)
                        st = fail(ctx, KVSMC_ERR_TIMEOUT, "shared-vertex connections: a shared-memory load did not complete");
                    else if (*hs)
                        st = fail(ctx, KVSMC_ERR_CUDA, "shared-vertex connections: a vertex id out of range");
                }
            }
        }
        for (Plan* pl : gp) {
            if (st) {
                pl->item->status = st;
            } else {
                pl->nodes_done = true;
                pl->conn_done = pl->ntri != 0;
                if (ready)
                    if (kvsmc_status rs = ready(pl->item, 1)) pl->item->status = rs;
            }
        }
    }
    for (size_t i = 0; i < items.size(); ++i) {
        Item* it = items[i];
        if (it->status || !it->emit) continue;
        kvsmc_status st = gather_emit(ctx, plans[i], it->d_coords, it->d_normals, it->d_conn);
        if (!st && ready) st = ready(it, 2);
        if (!st && !ready) KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        if (st) it->status = st;
    }
    if (ready) KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return KVSMC_OK;
}

// ------------------------------------------------------------ request setup

bool capacity_ok(const Item& it)
{
    return it.sizes.ncoords <= it.coords_cap && it.sizes.nnormals <= it.normals_cap &&
           it.sizes.nconnections <= it.conn_cap && (!it.sizes.ncoords || it.d_coords) &&
           (!it.sizes.nnormals || it.d_normals) && (!it.sizes.nconnections || it.d_conn);
}

// Run a list of prepared items: streaming ones together, the rest one by
// one.  emit=false only counts.  Per-item status in it.status; returns the
// first error.
kvsmc_status run_items(kvsmc_context* ctx, std::vector<Item*>& items, bool emit)
{
    std::vector<Item*> stream_items, gather_items;
    for (Item* it : items) {
        if (it->status) continue;
        if (!it->extracted) continue;
        (stream_eligible(ctx, *it) ? stream_items : gather_items).push_back(it);
    }
    kvsmc_status first = KVSMC_OK;
    if (!stream_items.empty()) {
        StreamBatch b;
        b.ctx = ctx;
        b.items = stream_items;
        kvsmc_status st = b.plan();
        if (!st) st = b.count();
        if (!st && emit) {
            for (Item* it : stream_items) {
                it->emit = true;
                if (!capacity_ok(*it)) {
                    it->status = fail(ctx, KVSMC_ERR_CAPACITY, "output needs %llu coords, %llu normals",
                                      (unsigned long long)it->sizes.ncoords, (unsigned long long)it->sizes.nnormals);
                }
            }
            st = b.emit();
            if (!st) st = b.finish();
        }
        if (st) {
            for (Item* it : stream_items) if (!it->status) it->status = st;
            first = st;
        }
    }
    SharedCount sc;
    if (kvsmc_status st = shared_count(ctx, gather_items, sc)) {
        for (Item* it : sc.cand) it->status = st;
        if (!first) first = st;
    }
    // requests whose group carries their vertex counts: one node emit per group
    std::vector<Item*> grouped;
    for (Item* it : gather_items)
        if (!it->status && sc.has_nodes(it)) grouped.push_back(it);
    if (!grouped.empty()) {
        auto outputs = [&](std::vector<Item*>& its) -> kvsmc_status {
            for (Item* it : its) {
                if (!capacity_ok(*it))
                    it->status = fail(ctx, KVSMC_ERR_CAPACITY, "output needs %llu coords, %llu normals, %llu connections",
                                      (unsigned long long)it->sizes.ncoords, (unsigned long long)it->sizes.nnormals,
                                      (unsigned long long)it->sizes.nconnections);
                else
                    it->emit = true;
            }
            return KVSMC_OK;
        };
        const kvsmc_status st = grouped_shared(ctx, sc, grouped, emit, outputs);
        if (st == KVSMC_ERR_OUT_OF_MEMORY) grouped.clear();   // each request on its own below
        else if (st)
            for (Item* it : grouped)
                if (!it->status) it->status = st;
    }
    for (Item* it : gather_items) {
        if (it->status) continue;
        if (!grouped.empty() && sc.has_nodes(it)) continue;   // done above
        Plan pl;
        gather_plan(*it, pl);
        sc.attach(it, pl);
        kvsmc_status st = gather_count(ctx, pl);
        if (!st) {
            gather_sizes(pl, *it, &it->sizes);
            if (emit) {
                if (!capacity_ok(*it)) {
                    st = fail(ctx, KVSMC_ERR_CAPACITY, "output needs %llu coords, %llu normals, %llu connections",
                              (unsigned long long)it->sizes.ncoords, (unsigned long long)it->sizes.nnormals,
                              (unsigned long long)it->sizes.nconnections);
                } else {
                    st = gather_emit(ctx, pl, it->d_coords, it->d_normals, it->d_conn);
                    if (!st) KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
                }
            }
        }
        if (st) {
            it->status = st;
            if (!first) first = st;
        }
    }
    for (Item* it : items)
        if (it->status && !first) first = it->status;
    return first;
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
    ctx->prof = profiler_create();
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
    if (ctx->d_flag) cudaFree(ctx->d_flag);
    if (ctx->h_flag) cudaFreeHost(ctx->h_flag);
    for (int b = 0; b < 2; ++b) {
        if (ctx->stl_dbuf[b]) cudaFree(ctx->stl_dbuf[b]);
        if (ctx->stl_hbuf[b]) cudaFreeHost(ctx->stl_hbuf[b]);
        if (ctx->stl_ev[b]) cudaEventDestroy(ctx->stl_ev[b]);
        if (ctx->txt_dbuf[b]) cudaFree(ctx->txt_dbuf[b]);
        if (ctx->txt_hbuf[b]) cudaFreeHost(ctx->txt_hbuf[b]);
    }
    if (ctx->out_arena) cudaFree(ctx->out_arena);
    if (ctx->arena2) cudaFree(ctx->arena2);
    if (ctx->arena3) cudaFree(ctx->arena3);
    if (ctx->arena4) cudaFree(ctx->arena4);
    if (ctx->arena5) cudaFree(ctx->arena5);
    if (ctx->h_small) cudaFreeHost(ctx->h_small);
    if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
    profiler_destroy(ctx->prof);
    if (ctx->aux_ready) {
        for (int i = 0; i < kvsmc_context::kAux; ++i) {
            cudaStreamSynchronize(ctx->aux[i]);
            cudaStreamDestroy(ctx->aux[i]);
            cudaEventDestroy(ctx->join_ev[i]);
        }
        cudaEventDestroy(ctx->fork_ev);
    }
    if (ctx->copy_stream) {
        cudaStreamSynchronize(ctx->copy_stream);
        cudaStreamDestroy(ctx->copy_stream);
        for (int i = 0; i < kvsmc_context::kParts; ++i) cudaEventDestroy(ctx->part_ev[i]);
    }
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

kvsmc_status kvsmc_set_kernel_path(kvsmc_context* ctx, int32_t path)
{
    if (!ctx || path < 0 || path > 1) return KVSMC_ERR_INVALID_ARGUMENT;
    ctx->path = path;
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
    if ((st = volume_alloc(ctx, dtype, nx, ny, nz, v)) || (st = volume_copy_in(ctx, v, host, cudaMemcpyHostToDevice)) ||
        (st = volume_bricks(ctx, v))) {
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
    if ((st = volume_alloc(ctx, dtype, nx, ny, nz, v)) || (st = volume_copy_in(ctx, v, dev, cudaMemcpyDeviceToDevice)) ||
        (st = volume_bricks(ctx, v))) {
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
    if ((st = volume_copy_in(ctx, v, host, cudaMemcpyHostToDevice))) return st;
    return v->bricks_valid ? volume_bricks(ctx, v) : KVSMC_OK;
}

void kvsmc_volume_free(kvsmc_context* ctx, kvsmc_volume* v)
{
    if (!v) return;
    if (ctx) {
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
    }
    if (v->dev) cudaFree(v->dev);
    if (v->bricks) cudaFree(v->bricks);
    delete v;
}

kvsmc_status kvsmc_volume_download(kvsmc_context* ctx, const kvsmc_volume* v, void* host_values)
{
    kvsmc_status st = use_device(ctx);
    if (st) return st;
    if (!v || !host_values) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "null pointer");
    const size_t es = dtype_size(v->view.dtype);
    const size_t row = (size_t)v->view.nx * es;
    KVSMC_CUDA(ctx, cudaMemcpy2DAsync(host_values, row, v->dev, v->view.pitch * es, row,
                                      (size_t)v->view.ny * v->view.nz, cudaMemcpyDeviceToHost, ctx->stream));
    KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return KVSMC_OK;
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
    if (!sizes || !p) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "null pointer");
    Item it;
    it.vol = vol;
    it.params = *p;
    if ((st = prepare(ctx, it))) return st;
    std::vector<Item*> v{&it};
    st = run_items(ctx, v, false);
    *sizes = it.sizes;
    return st;
}

kvsmc_status kvsmc_extract_device(kvsmc_context* ctx, kvsmc_volume* vol, const kvsmc_params* p,
                                  float* d_coords, uint64_t coords_cap, float* d_normals, uint64_t normals_cap,
                                  uint32_t* d_conn, uint64_t conn_cap, kvsmc_sizes* sizes)
{
    kvsmc_status st = use_device(ctx);
    if (st) return st;
    if (!sizes || !p) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "null pointer");
    Item it;
    it.vol = vol;
    it.params = *p;
    it.d_coords = d_coords; it.coords_cap = coords_cap;
    it.d_normals = d_normals; it.normals_cap = normals_cap;
    it.d_conn = d_conn; it.conn_cap = conn_cap;
    if ((st = prepare(ctx, it))) return st;
    std::vector<Item*> v{&it};
    st = run_items(ctx, v, true);
    *sizes = it.sizes;
    return st;
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
    Item it;
    it.vol = v;
    it.params = *p;
    if ((st = prepare(ctx, it))) return st;
    *sizes = it.sizes;
    if (!it.extracted) return KVSMC_OK;
    // count, size the device outputs, emit
    std::vector<Item*> items{&it};
    const bool streaming = stream_eligible(ctx, it);
    StreamBatch b;
    Plan pl;
    if (streaming) {
        b.ctx = ctx;
        b.items = items;
        if ((st = b.plan()) || (st = b.count())) return st;
    } else {
        gather_plan(it, pl);
        if ((st = gather_count(ctx, pl))) return st;
        gather_sizes(pl, it, &it.sizes);
    }
    *sizes = it.sizes;
    const size_t bc = align_up(sizes->ncoords * 4, 256), bn = align_up(sizes->nnormals * 4, 256);
    const size_t bk = align_up(sizes->nconnections * 4, 256);
    if (bc + bn + bk > ctx->out_bytes) {
        KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        if (ctx->out_arena) cudaFree(ctx->out_arena);
        ctx->out_arena = nullptr;
        ctx->out_bytes = 0;
        const size_t want = align_up(bc + bn + bk, 1 << 20);
        KVSMC_CUDA(ctx, cudaMalloc(&ctx->out_arena, want));
        ctx->out_bytes = want;
    }
    char* base = static_cast<char*>(ctx->out_arena);
    it.d_coords = reinterpret_cast<float*>(base);
    it.d_normals = reinterpret_cast<float*>(base + bc);
    it.d_conn = reinterpret_cast<uint32_t*>(base + bc + bn);
    it.coords_cap = sizes->ncoords;
    it.normals_cap = sizes->nnormals;
    it.conn_cap = sizes->nconnections;
    it.emit = true;
    if (streaming) {
        if ((st = b.emit()) || (st = b.finish())) return st;
    } else {
        if ((st = gather_emit(ctx, pl, it.d_coords, it.d_normals, it.d_conn))) return st;
    }
    void* hc = nullptr;
    void* hn = nullptr;
    void* hk = nullptr;
    if (sizes->ncoords && !(hc = alloc(user, 0, sizes->ncoords))) return fail(ctx, KVSMC_ERR_OUT_OF_MEMORY, "host alloc (coords)");
    if (sizes->nnormals && !(hn = alloc(user, 1, sizes->nnormals))) return fail(ctx, KVSMC_ERR_OUT_OF_MEMORY, "host alloc (normals)");
    if (sizes->nconnections && !(hk = alloc(user, 2, sizes->nconnections))) return fail(ctx, KVSMC_ERR_OUT_OF_MEMORY, "host alloc (connections)");
    if (hc) KVSMC_CUDA(ctx, cudaMemcpyAsync(hc, it.d_coords, sizes->ncoords * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (hn) KVSMC_CUDA(ctx, cudaMemcpyAsync(hn, it.d_normals, sizes->nnormals * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (hk) KVSMC_CUDA(ctx, cudaMemcpyAsync(hk, it.d_conn, sizes->nconnections * 4, cudaMemcpyDeviceToHost, ctx->stream));
    KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return KVSMC_OK;
}

// Point the items' device outputs into the (grow-only) output arena.
static kvsmc_status arena_outputs(kvsmc_context* ctx, std::vector<Item*>& its)
{
    size_t total = 0;
    for (Item* it : its)
        total += align_up(it->sizes.ncoords * 4, 256) + align_up(it->sizes.nnormals * 4, 256) +
                 align_up(it->sizes.nconnections * 4, 256);
    if (total > ctx->out_bytes) {
        KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        if (ctx->out_arena) cudaFree(ctx->out_arena);
        ctx->out_arena = nullptr;
        ctx->out_bytes = 0;
        const size_t want = align_up(total, 1 << 20);
        KVSMC_CUDA(ctx, cudaMalloc(&ctx->out_arena, want));
        ctx->out_bytes = want;
    }
    Carve cv{static_cast<char*>(ctx->out_arena)};
    for (Item* it : its) {
        it->d_coords = cv.take<float>(it->sizes.ncoords * 4);
        it->d_normals = cv.take<float>(it->sizes.nnormals * 4);
        it->d_conn = cv.take<uint32_t>(it->sizes.nconnections * 4);
        it->coords_cap = it->sizes.ncoords;
        it->normals_cap = it->sizes.nnormals;
        it->conn_cap = it->sizes.nconnections;
        it->emit = true;
    }
    return KVSMC_OK;
}

// Allocate each item's host arrays through the callback (once per item).
static kvsmc_status host_alloc(kvsmc_context* ctx, std::vector<Item*>& its, const Item* first_item,
                               kvsmc_host_alloc_fn alloc, void* user)
{
    for (Item* it : its) {
        if (it->h_coords || it->h_normals || it->h_conn) continue;
        const int32_t base = 3 * (int32_t)(it - first_item);
        const kvsmc_sizes& s = it->sizes;
        if (s.ncoords && !(it->h_coords = alloc(user, base + 0, s.ncoords)))
            return fail(ctx, KVSMC_ERR_OUT_OF_MEMORY, "host alloc (coords)");
        if (s.nnormals && !(it->h_normals = alloc(user, base + 1, s.nnormals)))
            return fail(ctx, KVSMC_ERR_OUT_OF_MEMORY, "host alloc (normals)");
        if (s.nconnections && !(it->h_conn = alloc(user, base + 2, s.nconnections)))
            return fail(ctx, KVSMC_ERR_OUT_OF_MEMORY, "host alloc (connections)");
    }
    return KVSMC_OK;
}

// Allocate each item's host arrays through the callback and copy them back.
static kvsmc_status copy_back(kvsmc_context* ctx, std::vector<Item*>& its, const Item* first_item,
                              kvsmc_host_alloc_fn alloc, void* user)
{
    kvsmc_status st = host_alloc(ctx, its, first_item, alloc, user);
    if (st) return st;
    for (Item* it : its) {
        const kvsmc_sizes& s = it->sizes;
        void* hc = it->h_coords;
        void* hn = it->h_normals;
        void* hk = it->h_conn;
        if (hc) KVSMC_CUDA(ctx, cudaMemcpyAsync(hc, it->d_coords, s.ncoords * 4, cudaMemcpyDeviceToHost, ctx->stream));
        if (hn) KVSMC_CUDA(ctx, cudaMemcpyAsync(hn, it->d_normals, s.nnormals * 4, cudaMemcpyDeviceToHost, ctx->stream));
        if (hk) KVSMC_CUDA(ctx, cudaMemcpyAsync(hk, it->d_conn, s.nconnections * 4, cudaMemcpyDeviceToHost, ctx->stream));
    }
    KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return KVSMC_OK;
}

// Emit launches of a host call's streaming batch (ranges of cell planes): the
// first part's outputs start crossing the host link after 1/8 of the emit.
constexpr int kStreamHostParts = 8;

// Streaming items of a host call: count, then the emit in parts by ranges of
// cell planes, each part's triangles copied into the host arrays on the copy
// stream while the next part is written.
static kvsmc_status stream_host_pipeline(kvsmc_context* ctx, std::vector<Item*>& s_items, const Item* first_item,
                                         kvsmc_host_alloc_fn alloc, void* user)
{
    StreamBatch b;
    b.ctx = ctx;
    b.items = s_items;
    kvsmc_status st;
    if ((st = b.plan()) || (st = b.count()) || (st = arena_outputs(ctx, s_items)) ||
        (st = host_alloc(ctx, s_items, first_item, alloc, user)))
        return st;
    if (!ctx->copy_stream) {
        KVSMC_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
        for (int i = 0; i < kvsmc_context::kParts; ++i)
            KVSMC_CUDA(ctx, cudaEventCreateWithFlags(&ctx->part_ev[i], cudaEventDisableTiming));
    }
    // first triangle of every (isolevel, z) plane, relative to its isolevel
    std::vector<uint64_t> pb(b.iso_planes);
    if (b.iso_planes)
        KVSMC_CUDA(ctx, cudaMemcpyAsync(pb.data(), b.d_plane_base, b.iso_planes * 8, cudaMemcpyDeviceToHost,
                                        ctx->stream));
    KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    kvsmc::Launch Lc = launch_of(ctx);
    Lc.stream = ctx->copy_stream;
    int part = 0;
    auto copy = [&](uint32_t z0, uint32_t z1, bool whole) -> kvsmc_status {
        cudaEvent_t ev = ctx->part_ev[part++ % kvsmc_context::kParts];
        KVSMC_CUDA(ctx, cudaEventRecord(ev, ctx->stream));
        KVSMC_CUDA(ctx, cudaStreamWaitEvent(ctx->copy_stream, ev, 0));
        kvsmc::prof_begin(Lc, "copy_d2h");
        for (size_t i = 0; i < b.isos.size(); ++i) {
            Item* it = b.iso_item[i];
            const uint64_t total = it->sizes.ntriangles;
            uint64_t t0 = 0, t1 = total;
            if (!whole) {
                const uint64_t first = pb[b.isos[i].plane_index];
                t0 = pb[b.isos[i].plane_index + z0] - first;
                const uint32_t cz = it->vol->view.nz - 1;
                t1 = z1 < cz ? pb[b.isos[i].plane_index + z1] - first : total;
            }
            if (t1 <= t0) continue;
            if (it->h_coords)
                KVSMC_CUDA(ctx, cudaMemcpyAsync(static_cast<float*>(it->h_coords) + 9 * t0, it->d_coords + 9 * t0,
                                                (t1 - t0) * 36, cudaMemcpyDeviceToHost, ctx->copy_stream));
            if (it->h_normals)
                KVSMC_CUDA(ctx, cudaMemcpyAsync(static_cast<float*>(it->h_normals) + 3 * t0, it->d_normals + 3 * t0,
                                                (t1 - t0) * 12, cudaMemcpyDeviceToHost, ctx->copy_stream));
        }
        kvsmc::prof_end(Lc);
        return KVSMC_OK;
    };
    st = b.emit_parts(kStreamHostParts, copy);
    if (!st) st = b.finish();
    const cudaError_t e = cudaStreamSynchronize(ctx->copy_stream);
    if (!st && e != cudaSuccess)
        st = fail(ctx, KVSMC_ERR_CUDA, "copy stream: %s", cudaGetErrorString(e));
    return st;
}

kvsmc_status kvsmc_extract_batch_host(kvsmc_context* ctx, const void* host, kvsmc_dtype dtype, uint32_t nx,
                                      uint32_t ny, uint32_t nz, const kvsmc_params* params, int32_t n,
                                      kvsmc_host_alloc_fn alloc, void* user, kvsmc_sizes* sizes)
{
    kvsmc_status st = use_device(ctx);
    if (st) return st;
    if (!host || (!params && n) || !alloc || (!sizes && n) || n < 0) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "null pointer");
    if ((st = check_shape(ctx, dtype, nx, ny, nz))) return st;
    if (!ctx->host_vol) ctx->host_vol = new kvsmc_volume();
    kvsmc_volume* v = ctx->host_vol;
    if ((st = volume_alloc(ctx, dtype, nx, ny, nz, v))) return st;
    {
        const kvsmc::Launch L = launch_of(ctx);
        kvsmc::prof_begin(L, "copy_h2d");
        st = volume_copy_in(ctx, v, host, cudaMemcpyHostToDevice);
        kvsmc::prof_end(L);
        if (st) return st;
    }
    std::vector<Item> items((size_t)n);
    std::vector<Item*> s_items, g_items;
    kvsmc_status first = KVSMC_OK;
    for (int32_t i = 0; i < n; ++i) {
        items[i].vol = v;
        items[i].params = params[i];
        items[i].status = prepare(ctx, items[i]);
        if (items[i].status) { if (!first) first = items[i].status; continue; }
        if (!items[i].extracted) continue;
        (stream_eligible(ctx, items[i]) ? s_items : g_items).push_back(&items[i]);
    }
    if (!s_items.empty()) {
        if ((st = stream_host_pipeline(ctx, s_items, items.data(), alloc, user))) {
            for (Item* it : s_items) it->status = st;
            if (!first) first = st;
        }
    }
    SharedCount sc;
    if ((st = shared_count(ctx, g_items, sc))) {
        for (Item* it : sc.cand) it->status = st;
        if (!first) first = st;
    }
    std::vector<Item*> grouped;
    for (Item* it : g_items)
        if (!it->status && sc.has_nodes(it)) grouped.push_back(it);
    if (!grouped.empty()) {
        // device outputs and the caller's host arrays once the sizes are known;
        // each array leaves on the copy stream as soon as it is final, while
        // the later passes run
        // (a failure of the caller's allocator fails these requests; it is not
        // the arena shortage on which they would run again one by one)
        bool host_failed = false;
        auto outputs = [&](std::vector<Item*>& its) -> kvsmc_status {
            kvsmc_status s2 = arena_outputs(ctx, its);
            if (!s2 && (s2 = host_alloc(ctx, its, items.data(), alloc, user))) host_failed = true;
            return s2;
        };
        if (!ctx->copy_stream) {
            KVSMC_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
            for (int i = 0; i < kvsmc_context::kParts; ++i)
                KVSMC_CUDA(ctx, cudaEventCreateWithFlags(&ctx->part_ev[i], cudaEventDisableTiming));
        }
        int ev = 0;
        const kvsmc::Launch Lc = [&] { kvsmc::Launch l = launch_of(ctx); l.stream = ctx->copy_stream; return l; }();
        auto ready = [&](Item* it, int what) -> kvsmc_status {
            cudaEvent_t e = ctx->part_ev[ev++ % kvsmc_context::kParts];
            KVSMC_CUDA(ctx, cudaEventRecord(e, ctx->stream));
            KVSMC_CUDA(ctx, cudaStreamWaitEvent(ctx->copy_stream, e, 0));
            const kvsmc_sizes& z = it->sizes;
            const bool pn = it->params.mode == KVSMC_SHARED_POLYGON_NORMAL;
            kvsmc::prof_begin(Lc, "copy_d2h");
            if (what == 0 && it->h_coords)
                KVSMC_CUDA(ctx, cudaMemcpyAsync(it->h_coords, it->d_coords, z.ncoords * 4, cudaMemcpyDeviceToHost,
                                                ctx->copy_stream));
            if (what == 1 && it->h_conn)
                KVSMC_CUDA(ctx, cudaMemcpyAsync(it->h_conn, it->d_conn, z.nconnections * 4, cudaMemcpyDeviceToHost,
                                                ctx->copy_stream));
            if (((what == 1 && pn) || (what == 2 && !pn)) && it->h_normals)
                KVSMC_CUDA(ctx, cudaMemcpyAsync(it->h_normals, it->d_normals, z.nnormals * 4, cudaMemcpyDeviceToHost,
                                                ctx->copy_stream));
            kvsmc::prof_end(Lc);
            return KVSMC_OK;
        };
        st = grouped_shared(ctx, sc, grouped, true, outputs, ready);
        const cudaError_t ce = cudaStreamSynchronize(ctx->copy_stream);
        if (st == KVSMC_ERR_OUT_OF_MEMORY && !host_failed) grouped.clear();   // each request on its own below
        else if (st)
            for (Item* it : grouped)
                if (!it->status) it->status = st;
        if (ce != cudaSuccess && !grouped.empty()) {
            st = fail(ctx, KVSMC_ERR_CUDA, "copy stream: %s", cudaGetErrorString(ce));
            for (Item* it : grouped)
                if (!it->status) it->status = st;
        }
        for (Item* it : grouped)
            if (it->status && !first) first = it->status;
    }
    for (Item* it : g_items) {
        if (it->status) continue;
        if (!grouped.empty() && sc.has_nodes(it)) continue;   // done above
        Plan pl;
        gather_plan(*it, pl);
        sc.attach(it, pl);
        st = gather_count(ctx, pl);
        if (!st) {
            gather_sizes(pl, *it, &it->sizes);
            std::vector<Item*> one{it};
            if (!(st = arena_outputs(ctx, one)) && !(st = gather_emit(ctx, pl, it->d_coords, it->d_normals, it->d_conn)))
                st = copy_back(ctx, one, items.data(), alloc, user);
        }
        if (st) { it->status = st; if (!first) first = st; }
    }
    for (int32_t i = 0; i < n; ++i) sizes[i] = items[i].sizes;
    return first;
}

static kvsmc_status batch_items(kvsmc_context* ctx, kvsmc_request* reqs, int32_t n, bool emit)
{
    std::vector<Item> items((size_t)n);
    std::vector<Item*> ptrs;
    for (int32_t i = 0; i < n; ++i) {
        Item& it = items[i];
        it.vol = reqs[i].volume;
        it.params = reqs[i].params;
        it.d_coords = reqs[i].d_coords; it.coords_cap = reqs[i].coords_capacity;
        it.d_normals = reqs[i].d_normals; it.normals_cap = reqs[i].normals_capacity;
        it.d_conn = reqs[i].d_connections; it.conn_cap = reqs[i].connections_capacity;
        it.status = prepare(ctx, it);
        ptrs.push_back(&it);
    }
    kvsmc_status first = run_items(ctx, ptrs, emit);
    for (int32_t i = 0; i < n; ++i) {
        reqs[i].sizes = items[i].sizes;
        reqs[i].status = items[i].status;
        if (items[i].status && !first) first = items[i].status;
    }
    return first;
}

kvsmc_status kvsmc_count_batch(kvsmc_context* ctx, kvsmc_request* reqs, int32_t n)
{
    kvsmc_status st = use_device(ctx);
    if (st) return st;
    if ((!reqs && n) || n < 0) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "bad batch");
    return batch_items(ctx, reqs, n, false);
}

kvsmc_status kvsmc_extract_batch(kvsmc_context* ctx, kvsmc_request* reqs, int32_t n)
{
    kvsmc_status st = use_device(ctx);
    if (st) return st;
    if ((!reqs && n) || n < 0) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "bad batch");
    return batch_items(ctx, reqs, n, true);
}

static kvsmc_status selftest_run(kvsmc_context* ctx, bool cells, uint64_t n, uint64_t seed, uint64_t* tested,
                                 uint64_t* mismatches, uint64_t* fallbacks)
{
    kvsmc_status st = use_device(ctx);
    if (st) return st;
    if ((st = ensure_scratch(ctx, 256))) return st;
    unsigned long long* d = static_cast<unsigned long long*>(ctx->scratch);
    KVSMC_CUDA(ctx, cudaMemsetAsync(d, 0, 3 * sizeof(unsigned long long), ctx->stream));
    if (cells) KVSMC_CUDA(ctx, launch_selftest_cells(n, seed, d, launch_of(ctx)));
    else KVSMC_CUDA(ctx, launch_selftest(n, seed, d, launch_of(ctx)));
    KVSMC_CUDA(ctx, cudaMemcpyAsync(ctx->h_small, d, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream));
    KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (tested) *tested = ctx->h_small[0];
    if (mismatches) *mismatches = ctx->h_small[1];
    if (fallbacks) *fallbacks = ctx->h_small[2];
    return KVSMC_OK;
}

kvsmc_status kvsmc_selftest_interpolation(kvsmc_context* ctx, uint64_t n, uint64_t seed, uint64_t* tested,
                                          uint64_t* mismatches, uint64_t* fallbacks)
{
    return selftest_run(ctx, false, n, seed, tested, mismatches, fallbacks);
}

kvsmc_status kvsmc_selftest_cells(kvsmc_context* ctx, uint64_t n, uint64_t seed, uint64_t* tested,
                                  uint64_t* mismatches, uint64_t* fallbacks)
{
    return selftest_run(ctx, true, n, seed, tested, mismatches, fallbacks);
}

}  // extern "C"

namespace kvsmc_host {

kvsmc_status volume_create(kvsmc_context* ctx, kvsmc_dtype dtype, uint32_t nx, uint32_t ny, uint32_t nz,
                           kvsmc_volume** out)
{
    kvsmc_status st = check_shape(ctx, dtype, nx, ny, nz);
    if (st) return st;
    kvsmc_volume* v = new kvsmc_volume();
    if ((st = volume_alloc(ctx, dtype, nx, ny, nz, v))) {
        if (v->dev) cudaFree(v->dev);
        delete v;
        return st;
    }
    *out = v;
    return KVSMC_OK;
}

}  // namespace kvsmc_host
