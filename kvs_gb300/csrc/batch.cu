// batch.cu -- planning and launching of the streaming kernels for a batch of
// (volume, isolevel) requests: per value type present one count launch and one
// emit launch, plus the unit scan and the plane scan, whatever the number of
// volumes and isolevels.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>

#include "batch.h"

namespace kvsmc_host {

using kvsmc::StreamGroup;
using kvsmc::StreamIso;

namespace {

bool stream_dtype(int dt) { return dt == KVSMC_I8 || dt == KVSMC_I16 || dt == KVSMC_U8 || dt == KVSMC_U16 || dt == KVSMC_F32; }

}  // namespace

// FP32 fast-path constants of one request (see mc_interp.cuh).
kvsmc::FastIso make_fast(double iso, double vmin, double vmax, int dtype)
{
    kvsmc::FastIso f;
    std::memset(&f, 0, sizeof f);
    const kvsmc::Classifier c = make_classifier(iso);
    if (dtype == KVSMC_F32) {
        f.f_thr = c.f_thr;
    } else {
        // integer data: v > floor(iso) <=> float(v) > float(floor(iso)), |v| < 2^16
        long long t = c.i_thr;
        if (t > (1LL << 24)) t = 1LL << 24;
        if (t < -(1LL << 24)) t = -(1LL << 24);
        f.f_thr = (float)t;
    }
    f.ih = (float)iso;
    f.il = (float)(iso - (double)f.ih);
    const double rep = std::fabs(iso - ((double)f.ih + (double)f.il));
    float err = (float)rep;
    if ((double)err < rep) err = std::nextafter(err, INFINITY);
    f.iso_err = err;
    f.vmin_f = (float)vmin;
    f.vmax_f = (float)vmax;
    const double lim = 1.152921504606846976e18;  // 2^60
    f.fast_ok = std::isfinite(iso) && std::fabs(iso) <= lim && std::isfinite(vmin) && std::isfinite(vmax) &&
                std::fabs(vmin) <= lim && std::fabs(vmax) <= lim && (double)f.vmin_f == vmin &&
                (double)f.vmax_f == vmax && std::isfinite(f.ih) && std::isfinite(f.il);
    return f;
}

void bucket_params(float t0, float t1, float& bs, float& bo)
{
    // Any finite bs > 0 and finite bo give a monotone bucket map (which is all
    // the kernels rely on); these spread the thresholds [t0, t1] over buckets
    // 1 .. kStreamBuckets - 1.
    const double nb = (double)kvsmc::kStreamBuckets;
    const double span = (double)t1 - (double)t0;
    double s = (span > 0.0 && std::isfinite(span)) ? (1.0 - 2.0 / nb) / span : 1.0 / (1.0 + std::fabs((double)t0));
    if (!(s > 1.0e-30) || !(s < 1.0e30)) s = 1.0 / (1.0 + std::fabs((double)t0));
    double o = 1.0 / nb - (double)t0 * s;
    bs = (float)s;
    bo = (float)o;
    if (!(bs > 0.0f) || !std::isfinite(bs) || !std::isfinite(bo)) {
        bs = 1.0f;
        bo = 0.0f;
    }
}

uint64_t cap_triangles(const Item& it)
{
    const uint64_t a = it.d_coords ? it.coords_cap / 9 : 0, b = it.d_normals ? it.normals_cap / 3 : 0;
    return a < b ? a : b;
}

int stream_rows(uint32_t cx)
{
    // two 128-cell rows per warp when that leaves fewer idle lanes than one
    // 256-cell row (narrow volumes, or a last segment of at most 128 cells);
    // on a tie one row (fewer, longer units)
    const uint32_t w1 = (cx + 255) / 256 * 256, w2 = (cx + 127) / 128 * 128;
    return w2 < w1 ? 2 : 1;
}

kvsmc_tune_choice stream_shape(const kvsmc_context* ctx, const kvsmc::VolumeView& v)
{
    kvsmc_tune_choice c{};
    if (ctx->tune_forced) {
        c = ctx->tune_force;
        kvsmc_tune_entry e{};
        e.choice = c;
        e.dtype = v.dtype;
        e.size_class = kvsmc_size_class(v.nx, v.ny, v.nz);
        if (kvsmc_tune_resolve(&e, 1, (kvsmc_dtype)v.dtype, v.nx, v.ny, v.nz, &c) == KVSMC_OK) return c;
    }
    if (kvsmc_tune_resolve(ctx->tuning.data(), (int32_t)ctx->tuning.size(), (kvsmc_dtype)v.dtype, v.nx, v.ny, v.nz,
                           &c) != KVSMC_OK)
        kvsmc_tune_resolve(nullptr, 0, (kvsmc_dtype)v.dtype, v.nx, v.ny, v.nz, &c);
    return c;
}

uint32_t stream_zchunk(uint64_t warp_steps, int num_sms, int tasks_per_sm)
{
    const uint64_t want_tasks = (uint64_t)num_sms * (uint64_t)(tasks_per_sm > 0 ? tasks_per_sm : kDefaultTasksPerSm);
    uint64_t zc = (warp_steps + want_tasks - 1) / want_tasks;
    if (zc < 4) zc = 4;
    if (zc > 64) zc = 64;
    return (uint32_t)zc;
}

bool stream_eligible(const kvsmc_context* ctx, const Item& it)
{
    return it.params.mode == KVSMC_DUP_POLYGON_NORMAL && stream_volume_eligible(ctx, it);
}

bool stream_volume_eligible(const kvsmc_context* ctx, const Item& it)
{
    if (ctx->path != 0 || !it.vol) return false;
    const kvsmc::VolumeView& v = it.vol->view;
    if (!stream_dtype(v.dtype)) return false;
    if (v.nx < 2 || v.ny < 2 || v.nz < 2) return false;
    if (v.nx - 1 > (uint32_t)kvsmc::kStreamMaxCells) return false;
    // triangles of one (isolevel, z) plane must fit the u32 plane offsets
    if ((double)(v.nx - 1) * (double)(v.ny - 1) * 5.0 >= 4294967295.0) return false;
    const double iso = it.params.isolevel;
    if (!std::isfinite(iso) || std::fabs(iso) > 1.0e30) return false;
    return kvsmc::stream_shared_bytes(v.dtype, true, 1) <= (size_t)227 * 1024 &&
           kvsmc::stream_shared_bytes(v.dtype, true, 2) <= (size_t)227 * 1024;
}

void StreamBatch::plan_tables()
{
    // group by volume in request order, at most kStreamMaxIso per group
    std::vector<std::vector<Item*>> lists;
    std::map<kvsmc_volume*, size_t> open;
    for (Item* it : items) {
        auto f = open.find(it->vol);
        if (f == open.end() || lists[f->second].size() == (size_t)kvsmc::kStreamMaxIso) {
            open[it->vol] = lists.size();
            lists.push_back({});
            f = open.find(it->vol);
        }
        lists[f->second].push_back(it);
    }
    // one launch per (value type, rows per warp) present; the launch shape
    // of each volume from the context's tuning
    std::vector<std::pair<int, int>> kinds;
    std::map<const kvsmc_volume*, kvsmc_tune_choice> shape;
    for (auto& l : lists) shape[l[0]->vol] = stream_shape(ctx, l[0]->vol->view);
    // Under the built-in rules, a value type whose volumes mix one- and two-row
    // tasks takes two rows for all of them: one launch per type instead of two
    // (two-row tasks suit every width; on the uneven 200-volume batch this took
    // the replay from 10.06 to 9.17 ms).  Not for the shared-vertex count,
    // whose connection pass takes one-row groups only.
    if (!want_nodes && !ctx->tune_forced && ctx->tuning.empty()) {
        std::map<int, int> rows_seen;   // value type -> bit r set: some volume takes r rows
        for (auto& l : lists) rows_seen[(int)l[0]->vol->view.dtype] |= 1 << shape[l[0]->vol].rows;
        for (auto& l : lists)
            if (rows_seen[(int)l[0]->vol->view.dtype] == ((1 << 1) | (1 << 2))) shape[l[0]->vol].rows = 2;
    }
    auto kind_of = [&](const std::vector<Item*>& l) {
        return std::make_pair((int)l[0]->vol->view.dtype, (int)shape[l[0]->vol].rows);
    };
    // the largest volume (in cells) decides the launch-wide fields
    auto cells_of = [](const kvsmc::VolumeView& v) { return (uint64_t)(v.nx - 1) * (v.ny - 1) * (v.nz - 1); };
    const kvsmc_volume* largest = nullptr;
    for (auto& l : lists)
        if (!largest || cells_of(l[0]->vol->view) > cells_of(largest->view)) largest = l[0]->vol;
    scan_threads = largest ? shape[largest].scan_threads : 256;
    for (auto& l : lists)
        if (std::find(kinds.begin(), kinds.end(), kind_of(l)) == kinds.end()) kinds.push_back(kind_of(l));
    groups.clear();
    isos.clear();
    iso_item.clear();
    launches.clear();
    unit_elems = 0;
    scan_blocks = 0;
    iso_planes = 0;
    node_elems = 0;
    for (const auto& kd : kinds) {
        const int dt = kd.first, rows = kd.second;
        Launch1 L;
        L.dtype = dt;
        L.rows = rows;
        L.g0 = (int)groups.size();
        L.ntasks = 0;
        // one z-chunk for the whole launch: sized by all its warp steps, so a
        // batch of small volumes gets long tasks rather than many short ones
        uint64_t steps = 0;
        const kvsmc_volume* big = nullptr;
        for (auto& l : lists) {
            if (kind_of(l) != kd) continue;
            const kvsmc::VolumeView& v = l[0]->vol->view;
            steps += (uint64_t)(v.nz - 1) * ((v.ny - 1 + rows - 1) / rows) * segments_per_row(v, rows);
            if (!big || cells_of(v) > cells_of(big->view)) big = l[0]->vol;
        }
        const kvsmc_tune_choice& bs_shape = shape[big];
        L.ctas_per_sm = bs_shape.ctas_per_sm;
        const uint32_t zchunk = stream_zchunk(steps, ctx->num_sms, bs_shape.tasks_per_sm);
        for (auto& l : lists) {
            if (kind_of(l) != kd) continue;
            const kvsmc::VolumeView v = l[0]->vol->view;
            StreamGroup g;
            std::memset(&g, 0, sizeof g);
            g.vol = v;
            g.rows = (uint32_t)rows;
            const kvsmc_volume* vol = l[0]->vol;
            g.bricks = vol->bricks_valid ? vol->bricks : nullptr;
            g.brick_wpr = (v.nx - 1 + kvsmc::kBrickCells - 1) / kvsmc::kBrickCells;
            g.wpr = segments_per_row(v, rows);
            g.zchunk = zchunk;
            const uint32_t cz = v.nz - 1;
            g.task_begin = L.ntasks;
            L.ntasks += stream_tasks(v, rows, g.wpr, g.zchunk);
            g.seg_elems = (uint32_t)kvsmc::stream_row_elems(dt, rows);
            g.seg_copy_bytes = g.seg_elems * (uint32_t)kvsmc::dtype_size(dt);
            g.warp_smem_bytes = (uint32_t)kvsmc::stream_warp_smem_bytes(dt, true, rows);
            g.warp_smem_offset = (uint32_t)kvsmc::stream_warp_smem_offset();
            // isolevels sorted by threshold
            std::vector<std::pair<float, Item*>> sorted;
            for (Item* it : l) sorted.push_back({make_fast(it->params.isolevel, it->vmin, it->vmax, dt).f_thr, it});
            std::stable_sort(sorted.begin(), sorted.end(),
                             [](const std::pair<float, Item*>& a, const std::pair<float, Item*>& b) { return a.first < b.first; });
            g.iso_begin = (int32_t)isos.size();
            g.niso = (int32_t)sorted.size();
            bucket_params(sorted.front().first, sorted.back().first, g.bs, g.bo);
            g.unit_base = unit_elems;
            unit_elems += stream_units(v, g.wpr, g.niso);
            if (want_nodes && rows == 1 && g.wpr == (v.nx + 255) / 256) {
                g.node_units = (uint64_t)v.nz * v.ny * g.wpr;
                g.node_base = node_elems;
                node_elems += (uint64_t)g.niso * g.node_units;
            }
            g.plane_begin = scan_blocks;
            scan_blocks += cz;
            for (auto& pr : sorted) {
                Item* it = pr.second;
                StreamIso s;
                std::memset(&s, 0, sizeof s);
                s.f = make_fast(it->params.isolevel, it->vmin, it->vmax, dt);
                s.ip.iso = it->params.isolevel;
                s.ip.vmin = it->vmin;
                s.ip.vmax = it->vmax;
                for (int k = 0; k < 3; ++k) { s.ip.min_coord[k] = it->params.min_coord[k]; s.ip.scale[k] = it->params.scale[k]; }
                s.plane_index = iso_planes;
                iso_planes += cz;
                isos.push_back(s);
                iso_item.push_back(it);
            }
            groups.push_back(g);
        }
        L.ng = (int)groups.size() - L.g0;
        launches.push_back(L);
    }
}

size_t StreamBatch::scratch_bytes() const
{
    const size_t niso = isos.size();
    return 16 * 256 + align_up(groups.size() * sizeof(StreamGroup), 256) + align_up(niso * sizeof(StreamIso), 256) +
           align_up(unit_elems * 2, 256) + align_up(unit_elems * 4, 256) + align_up(iso_planes * 4, 256) +
           align_up(iso_planes * 8, 256) + align_up(kvsmc::scan_scratch_bytes(iso_planes), 256) +
           align_up(niso * 8, 256) + align_up(launches.size() * 16, 256) + align_up(kMaxParts * 8, 256) +
           align_up(node_elems * 4, 256) + 6 * 256;
}

void StreamBatch::carve(char* base)
{
    const size_t niso = isos.size();
    Carve cv{base};
    d_groups = cv.take<StreamGroup>(groups.size() * sizeof(StreamGroup));
    d_isos = cv.take<StreamIso>(niso * sizeof(StreamIso));
    d_unit_counts = cv.take<uint16_t>(unit_elems * 2);
    d_unit_offsets = cv.take<uint32_t>(unit_elems * 4);
    d_plane_totals = cv.take<uint32_t>(iso_planes * 4);
    d_plane_base = cv.take<uint64_t>(iso_planes * 8);
    d_scan = cv.take<char>(kvsmc::scan_scratch_bytes(iso_planes));
    d_totals = cv.take<uint64_t>(niso * 8);
    d_total = cv.take<uint64_t>(256);
    d_status = cv.take<int>(256);
    d_next = cv.take<unsigned long long>(launches.size() * 16);
    d_next_parts = cv.take<unsigned long long>(kMaxParts * 8);
    d_node_counts = node_elems ? cv.take<uint32_t>(node_elems * 4) : nullptr;
}

kvsmc_status StreamBatch::plan()
{
    plan_tables();
    kvsmc_status st = ensure_scratch(ctx, scratch_bytes());
    if (st) return st;
    carve(static_cast<char*>(ctx->scratch));
    return upload_tables();
}

kvsmc_status StreamBatch::upload_tables()
{
    const size_t bg = groups.size() * sizeof(StreamGroup), bi = isos.size() * sizeof(StreamIso);
    kvsmc_status st = ensure_stage(ctx, bg + bi + 64);
    if (st) return st;
    char* h = static_cast<char*>(ctx->h_stage);
    std::memcpy(h, groups.data(), bg);
    std::memcpy(h + bg, isos.data(), bi);
    KVSMC_CUDA(ctx, cudaMemcpyAsync(d_groups, h, bg, cudaMemcpyHostToDevice, ctx->stream));
    KVSMC_CUDA(ctx, cudaMemcpyAsync(d_isos, h + bg, bi, cudaMemcpyHostToDevice, ctx->stream));
    return KVSMC_OK;
}

kvsmc_status StreamBatch::count()
{
    const kvsmc::Launch L = launch_of(ctx);
    KVSMC_CUDA(ctx, cudaMemsetAsync(d_status, 0, sizeof(int), ctx->stream));
    // units the kernels skip as empty space keep these zeros
    KVSMC_CUDA(ctx, cudaMemsetAsync(d_unit_counts, 0, unit_elems * sizeof(uint16_t), ctx->stream));
    KVSMC_CUDA(ctx, cudaMemsetAsync(d_next, 0, launches.size() * 16, ctx->stream));
    if (node_elems) KVSMC_CUDA(ctx, cudaMemsetAsync(d_node_counts, 0, node_elems * 4, ctx->stream));
    // one count launch per (value type, rows) kind, side by side
    KVSMC_CUDA(ctx, fan_out(ctx, ctx->stream, launches.size(), [&](size_t i, cudaStream_t st) {
        const Launch1& l = launches[i];
        kvsmc::Launch Li = L;
        Li.stream = st;
        return kvsmc::launch_stream(false, l.dtype, l.rows, d_groups + l.g0, l.ng, l.ntasks, d_isos, d_unit_counts,
                                    nullptr, nullptr, d_status, d_next + 2 * i, Li, l.ctas_per_sm, 0,
                                    node_elems && l.rows == 1 ? d_node_counts : nullptr);
    }));
    KVSMC_CUDA(ctx, kvsmc::launch_unit_scan(d_groups, (int)groups.size(), scan_blocks, d_isos, d_unit_counts,
                                            d_unit_offsets, d_plane_totals, L, scan_threads));
    KVSMC_CUDA(ctx, kvsmc::launch_scan(d_plane_totals, d_plane_base, iso_planes, d_scan, d_total, L));
    KVSMC_CUDA(ctx, kvsmc::launch_iso_totals(d_isos, (int)isos.size(), d_plane_base, d_total, d_totals, L));
    // read back: status word, then one total per isolevel
    const size_t n = isos.size();
    kvsmc_status st = ensure_stage(ctx, (n + 2) * 8);
    if (st) return st;
    uint64_t* h = static_cast<uint64_t*>(ctx->h_stage);
    KVSMC_CUDA(ctx, cudaMemcpyAsync(h, d_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    KVSMC_CUDA(ctx, cudaMemcpyAsync(h + 1, d_totals, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
    KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    int status;
    std::memcpy(&status, h, sizeof(int));
    if (status) return fail(ctx, KVSMC_ERR_TIMEOUT, "streaming count: a shared-memory load did not complete");
    for (size_t i = 0; i < n; ++i) {
        Item* it = iso_item[i];
        const uint64_t t = h[1 + i];
        std::memset(&it->sizes, 0, sizeof it->sizes);
        it->sizes.ntriangles = t;
        it->sizes.nvertices = 3 * t;
        it->sizes.ncoords = 9 * t;
        it->sizes.nnormals = 3 * t;
        it->sizes.min_value = it->vmin;
        it->sizes.max_value = it->vmax;
        it->sizes.extracted = 1;
    }
    return KVSMC_OK;
}

kvsmc_status StreamBatch::emit()
{
    bool any = false;
    for (size_t i = 0; i < isos.size(); ++i) {
        Item* it = iso_item[i];
        const bool ok = it->emit && it->status == KVSMC_OK && it->sizes.ntriangles > 0;
        isos[i].coords = ok ? it->d_coords : nullptr;
        isos[i].normals = ok ? it->d_normals : nullptr;
        isos[i].cap_tris = ok ? cap_triangles(*it) : 0;
        any = any || ok;
    }
    if (!any) return KVSMC_OK;
    for (StreamGroup& g : groups) {
        g.skip_emit = 1;
        for (int k = 0; k < g.niso; ++k)
            if (isos[g.iso_begin + k].coords) g.skip_emit = 0;
    }
    kvsmc_status st = upload_tables();
    if (st) return st;
    const kvsmc::Launch L = launch_of(ctx);
    KVSMC_CUDA(ctx, fan_out(ctx, ctx->stream, launches.size(), [&](size_t i, cudaStream_t st) {
        const Launch1& l = launches[i];
        kvsmc::Launch Li = L;
        Li.stream = st;
        return kvsmc::launch_stream(true, l.dtype, l.rows, d_groups + l.g0, l.ng, l.ntasks, d_isos, d_unit_counts,
                                    d_unit_offsets, d_plane_base, d_status, d_next + 2 * i + 1, Li, l.ctas_per_sm);
    }));
    return KVSMC_OK;
}

kvsmc_status StreamBatch::emit_parts(int parts, const std::function<kvsmc_status(uint32_t, uint32_t, bool)>& after)
{
    if (groups.size() != 1 || launches.size() != 1 || parts <= 1) {
        kvsmc_status st = emit();
        return st ? st : after(0, 0, true);
    }
    bool any = false;
    for (size_t i = 0; i < isos.size(); ++i) {
        Item* it = iso_item[i];
        const bool ok = it->emit && it->status == KVSMC_OK && it->sizes.ntriangles > 0;
        isos[i].coords = ok ? it->d_coords : nullptr;
        isos[i].normals = ok ? it->d_normals : nullptr;
        isos[i].cap_tris = ok ? cap_triangles(*it) : 0;
        any = any || ok;
    }
    if (!any) return after(0, 0, true);
    groups[0].skip_emit = 0;
    kvsmc_status st = upload_tables();
    if (st) return st;
    // tasks are numbered z-chunk-major: a range of z-chunks is a range of tasks
    const StreamGroup& g = groups[0];
    const Launch1& l = launches[0];
    const uint32_t cz = g.vol.nz - 1;
    const uint64_t zchunks = (cz + g.zchunk - 1) / g.zchunk;
    const uint64_t per_chunk = l.ntasks / zchunks;
    if (parts > kMaxParts) parts = kMaxParts;
    if ((uint64_t)parts > zchunks) parts = (int)zchunks;
    KVSMC_CUDA(ctx, cudaMemsetAsync(d_next_parts, 0, kMaxParts * 8, ctx->stream));
    const kvsmc::Launch L = launch_of(ctx);
    uint64_t c0 = 0;
    for (int p = 0; p < parts; ++p) {
        const uint64_t c1 = zchunks * (uint64_t)(p + 1) / (uint64_t)parts;
        KVSMC_CUDA(ctx, kvsmc::launch_stream(true, l.dtype, l.rows, d_groups, 1, c1 * per_chunk, d_isos, d_unit_counts,
                                             d_unit_offsets, d_plane_base, d_status, d_next_parts + p, L,
                                             l.ctas_per_sm, c0 * per_chunk));
        const uint32_t z0 = (uint32_t)(c0 * g.zchunk);
        const uint32_t z1 = (uint32_t)(c1 * g.zchunk < cz ? c1 * g.zchunk : cz);
        if ((st = after(z0, z1, false))) return st;
        c0 = c1;
    }
    return KVSMC_OK;
}

kvsmc_status StreamBatch::finish()
{
    int* h = static_cast<int*>(ctx->h_stage);
    KVSMC_CUDA(ctx, cudaMemcpyAsync(h, d_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (*h) return fail(ctx, KVSMC_ERR_TIMEOUT, "streaming emit: a shared-memory load did not complete");
    return KVSMC_OK;
}

}  // namespace kvsmc_host
