// slice.cu -- kvs::SlicePlane on structured volumes, on the GPU.
//
// The reference (Source/Core/Visualization/Mapper/SlicePlane.cpp) runs
// marching cubes on the plane function p(x) = a x + b y + c z + d instead of
// the volume: a cell's case has bit k set iff p(corner k) > 0 in float
// (calculate_table_index, :802-818; substitute_plane_equation, :949-959,
// ((a x + b y) + c z) + d), triangles come from MarchingCubesTable in table
// order with vertices (e[i], e[i+2], e[i+1]) (:101-135), each vertex at
// (1 - r) v0 + r v1 with r = |p0 / (p1 - p0)| in float (interpolate_vertex,
// :986-995) then (v + min_coord) * scale; its colour is
// ColorMap::at(value) of the volume value interpolated with the same r in the
// value type's own arithmetic (interpolate_value, :1006-1031; ColorMap.cpp:
// 1043-1054, RGBColor::Mix, RGBColor(Vec3) rounding); one normal per triangle
// -((v2 - v0) x (v1 - v0)).  Cells in z, y, x order.
//
// Two passes: count (one thread per cell row (y, z); cases from the plane
// alone, only over the x-interval of cells the plane can cut, bounded
// conservatively in double), an exclusive scan of the row counts, then emit
// (a warp per 32 rows: the rows' cut cells 32 at a time, one per lane, and
// each batch's triangles one per lane; the volume read only at the corners
// of cut edges).
#include <cuda_runtime.h>

#include <cstring>

#include "context.h"
#include "slice_common.cuh"
#include "mc_tables.h"

namespace kvsmc {

namespace {

__constant__ uint64_t c_slice_tri[256] = MC_TRI_PACKED_INIT;
__constant__ uint8_t c_slice_ntri[256] = MC_NTRI_INIT;
__constant__ uint8_t c_slice_edge[12] = MC_EDGE_PACKED_INIT;

constexpr int kSliceThreads = 128;

__device__ __forceinline__ unsigned slice_case(const SliceJob& j, uint32_t x, uint32_t y, uint32_t z)
{
    const float fx = __uint2float_rn(x), fy = __uint2float_rn(y), fz = __uint2float_rn(z);
    const float x1 = __uint2float_rn(x + 1), y1 = __uint2float_rn(y + 1), z1 = __uint2float_rn(z + 1);
    unsigned c = 0;
    c |= (plane_at(j, fx, fy, fz) > 0.0f) ? 1u : 0u;
    c |= (plane_at(j, x1, fy, fz) > 0.0f) ? 2u : 0u;
    c |= (plane_at(j, x1, y1, fz) > 0.0f) ? 4u : 0u;
    c |= (plane_at(j, fx, y1, fz) > 0.0f) ? 8u : 0u;
    c |= (plane_at(j, fx, fy, z1) > 0.0f) ? 16u : 0u;
    c |= (plane_at(j, x1, fy, z1) > 0.0f) ? 32u : 0u;
    c |= (plane_at(j, x1, y1, z1) > 0.0f) ? 64u : 0u;
    c |= (plane_at(j, fx, y1, z1) > 0.0f) ? 128u : 0u;
    return c;
}

struct SliceVertex {
    float3 p;     // after (v + min_coord) * scale
    uchar3 rgb;
};

template <typename T>
__device__ __forceinline__ SliceVertex slice_vertex(const SliceJob& j, const T* vol, uint32_t x, uint32_t y,
                                                    uint32_t z, int e)
{
    const unsigned ep = c_slice_edge[e];
    const unsigned a = ep & 7u, b = ep >> 3;
    const uint32_t ax = x + (a & 1u), ay = y + ((a >> 1) & 1u), az = z + (a >> 2);
    const uint32_t bx = x + (b & 1u), by = y + ((b >> 1) & 1u), bz = z + (b >> 2);
    const float v0x = __uint2float_rn(ax), v0y = __uint2float_rn(ay), v0z = __uint2float_rn(az);
    const float v1x = __uint2float_rn(bx), v1y = __uint2float_rn(by), v1z = __uint2float_rn(bz);
    const float p0 = plane_at(j, v0x, v0y, v0z), p1 = plane_at(j, v1x, v1y, v1z);
    const float ratio = fabsf(__fdiv_rn(p0, __fsub_rn(p1, p0)));
    const float s = __fsub_rn(1.0f, ratio);
    SliceVertex o;
    const float vx = __fadd_rn(__fmul_rn(s, v0x), __fmul_rn(ratio, v1x));
    const float vy = __fadd_rn(__fmul_rn(s, v0y), __fmul_rn(ratio, v1y));
    const float vz = __fadd_rn(__fmul_rn(s, v0z), __fmul_rn(ratio, v1z));
    o.p.x = __fmul_rn(__fadd_rn(vx, j.min_coord[0]), j.scale[0]);
    o.p.y = __fmul_rn(__fadd_rn(vy, j.min_coord[1]), j.scale[1]);
    o.p.z = __fmul_rn(__fadd_rn(vz, j.min_coord[2]), j.scale[2]);
    const T va = vol[(uint64_t)az * j.vol.slice + (uint64_t)ay * j.vol.pitch + ax];
    const T vb = vol[(uint64_t)bz * j.vol.slice + (uint64_t)by * j.vol.pitch + bx];
    o.rgb = color_at(j, slice_value(va, vb, ratio));
    return o;
}

// The cells of row (y, z) the plane can cut: an interval [x0, x1] of x (x0 >
// x1: none).  Over a cell the plane ranges over [a x + min(0, a) + Bmin + Cmin
// + d, a x + max(0, a) + Bmax + Cmax + d] (B, C: b y', c z' over the cell's
// y', z'), exactly, in double (the products of float coefficients with
// integers below 2^24 are exact there).  The float evaluation
// ((a x + b y) + c z) + d of a node is within 2^-21 (|a| cx + |b| (y + 1) +
// |c| (z + 1) + |d|) of the exact value (four roundings of 2^-24 each, times
// 2), so a cell whose exact range lies beyond that margin on one side has
// all its corners on that side in float: case 0 or 255, no triangle.  The
// interval is padded by one cell for the double arithmetic of its ends.
__device__ __forceinline__ void row_interval(const SliceJob& j, uint32_t cx, uint32_t y, uint32_t z, int64_t& x0,
                                             int64_t& x1)
{
    const double a = j.coef[0], b = j.coef[1], c = j.coef[2], d = j.coef[3];
    const double by0 = b * (double)y, by1 = b * (double)(y + 1), cz0 = c * (double)z, cz1 = c * (double)(z + 1);
    const double m = 4.76837158203125e-07 * (fabs(a) * (double)cx + fabs(b) * (double)(y + 1) +
                                             fabs(c) * (double)(z + 1) + fabs(d)) + 1e-30;
    const double k1 = fmin(0.0, a) + fmin(by0, by1) + fmin(cz0, cz1) + d - m;   // low end <= margin: a x + k1 <= 0
    const double k2 = fmax(0.0, a) + fmax(by0, by1) + fmax(cz0, cz1) + d + m;   // high end > -margin: a x + k2 > 0
    x0 = 0;
    x1 = (int64_t)cx - 1;
    if (!(k1 == k1) || !(k2 == k2) || !(a == a)) return;   // NaN plane: every cell is evaluated
    if (a == 0.0) {
        if (!(k1 <= 0.0 && k2 > 0.0)) x1 = -1;
        return;
    }
    double lo, hi;   // x in [lo, hi] (open ends widened below)
    if (a > 0.0) { lo = -k2 / a; hi = -k1 / a; }
    else { lo = -k1 / a; hi = -k2 / a; }
    if (!(lo <= hi)) { x1 = -1; return; }
    const double cap = (double)cx;
    lo = fmax(lo, -2.0);
    hi = fmin(hi, cap + 1.0);
    const int64_t l = (int64_t)floor(lo) - 1, h = (int64_t)ceil(hi) + 1;
    x0 = l > 0 ? l : 0;
    x1 = h < (int64_t)cx - 1 ? h : (int64_t)cx - 1;
}

// One thread per cell row (y, z), rows in z, y order: the triangles of the
// cells of its interval (the interval's double arithmetic once per row).
__global__ void __launch_bounds__(kSliceThreads) k_slice_count(SliceJob j)
{
    const uint32_t cx = j.vol.nx - 1, cy = j.vol.ny - 1;
    for (uint64_t row = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; row < j.nrows;
         row += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t z = (uint32_t)(row / cy), y = (uint32_t)(row - (uint64_t)z * cy);
        int64_t x0, x1;
        row_interval(j, cx, y, z, x0, x1);
        uint32_t sum = 0;
        for (int64_t x = x0; x <= x1; ++x) sum += c_slice_ntri[slice_case(j, (uint32_t)x, y, z)];
        j.row_counts[row] = sum;
    }
}

template <typename T>
__global__ void __launch_bounds__(kSliceThreads) k_slice_emit(SliceJob j)
{
    const T* vol = static_cast<const T*>(j.vol.data);
    const uint32_t cx = j.vol.nx - 1, cy = j.vol.ny - 1;
    const unsigned lane = threadIdx.x & 31u;
    const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x / 32);
    // Each warp takes 32 consecutive rows; lane i works out row i's interval
    // and first output triangle.  The rows' cut cells, in row and x order,
    // are then taken 32 at a time (one cell per lane, whatever row it is in),
    // and each batch's triangles are spread over the lanes, so a row with
    // only a few cut cells does not leave most of the warp idle.
    for (uint64_t r0 = ((uint64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5)) * 32; r0 < j.nrows;
         r0 += warps * 32) {
        const uint64_t my = r0 + lane;
        int64_t mx0 = 0, mx1 = -1;
        uint64_t rowrun = 0;   // next output triangle of this lane's row
        uint32_t my_y = 0, my_z = 0;
        if (my < j.nrows) {
            my_z = (uint32_t)(my / cy);
            my_y = (uint32_t)(my - (uint64_t)my_z * cy);
            row_interval(j, cx, my_y, my_z, mx0, mx1);
            rowrun = j.row_offsets[my];
        }
        const uint32_t len = mx1 >= mx0 ? (uint32_t)(mx1 - mx0 + 1) : 0u;
        uint32_t linc = len;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, linc, o);
            if (lane >= (unsigned)o) linc += t;
        }
        const uint32_t lexc = linc - len;
        const uint32_t ltot = __shfl_sync(0xffffffffu, linc, 31);
        for (uint32_t b0 = 0; b0 < ltot; b0 += 32) {
            // ---- one cut cell per lane: its row (the lane owning it) and x
            const uint32_t item = b0 + lane;
            unsigned owner = 0;
#pragma unroll
            for (unsigned step = 16; step > 0; step >>= 1) {
                const uint32_t probe = __shfl_sync(0xffffffffu, linc, owner + step - 1);
                if (probe <= item) owner += step;
            }
            const int64_t ox0 = __shfl_sync(0xffffffffu, mx0, owner);
            const uint32_t oexc = __shfl_sync(0xffffffffu, lexc, owner);
            const uint32_t y = __shfl_sync(0xffffffffu, my_y, owner), z = __shfl_sync(0xffffffffu, my_z, owner);
            const uint64_t orun = __shfl_sync(0xffffffffu, rowrun, owner);
            const bool has = item < ltot;
            const uint32_t x = has ? (uint32_t)(ox0 + (int64_t)(item - oexc)) : 0u;
            const unsigned c = has ? slice_case(j, x, y, z) : 0u;
            const uint32_t n = c_slice_ntri[c];
            uint32_t ninc = n;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t t = __shfl_up_sync(0xffffffffu, ninc, o);
                if (lane >= (unsigned)o) ninc += t;
            }
            const uint32_t ntot = __shfl_sync(0xffffffffu, ninc, 31);
            // first triangle of this cell: its row's running count plus the
            // triangles of the row's earlier cells in this batch
            const uint32_t ofirst = oexc > b0 ? oexc - b0 : 0u;   // the row's first lane in the batch
            const uint32_t before = __shfl_sync(0xffffffffu, ninc, ofirst ? ofirst - 1 : 0);
            const uint64_t tbase = orun + (ninc - n) - (ofirst ? before : 0u);
            // every row's running count moves past its cells of this batch
            {
                const uint32_t f = lexc > b0 ? (lexc - b0 < 32u ? lexc - b0 : 32u) : 0u;
                const uint32_t e = linc > b0 ? (linc - b0 < 32u ? linc - b0 : 32u) : 0u;
                const uint32_t s_end = __shfl_sync(0xffffffffu, ninc, e ? e - 1 : 0);
                const uint32_t s_beg = __shfl_sync(0xffffffffu, ninc, f ? f - 1 : 0);
                if (e > f) rowrun += (uint64_t)(s_end - (f ? s_beg : 0u));
            }
            // ---- the batch's triangles, one per lane
            for (uint32_t first = 0; first < ntot; first += 32) {   // warp-uniform: every lane shuffles
                const uint32_t tri = first + lane;
                unsigned q = 0;
#pragma unroll
                for (unsigned step = 16; step > 0; step >>= 1) {
                    const uint32_t probe = __shfl_sync(0xffffffffu, ninc, q + step - 1);
                    if (probe <= tri) q += step;
                }
                const uint32_t q_inc = __shfl_sync(0xffffffffu, ninc, q);
                const uint32_t q_n = __shfl_sync(0xffffffffu, n, q);
                const unsigned q_c = __shfl_sync(0xffffffffu, c, q);
                const uint32_t qx = __shfl_sync(0xffffffffu, x, q);
                const uint32_t qy = __shfl_sync(0xffffffffu, y, q), qz = __shfl_sync(0xffffffffu, z, q);
                const uint64_t q_base = __shfl_sync(0xffffffffu, tbase, q);
                if (tri >= ntot) continue;
                const uint32_t k = tri - (q_inc - q_n);
                const uint64_t t = q_base + k;
                if (t >= j.cap_tris) continue;   // never past the outputs
                const uint64_t pk = c_slice_tri[q_c] >> (12 * k);
                const SliceVertex va = slice_vertex<T>(j, vol, qx, qy, qz, (int)(pk & 15u));
                const SliceVertex vb = slice_vertex<T>(j, vol, qx, qy, qz, (int)((pk >> 4) & 15u));
                const SliceVertex vd = slice_vertex<T>(j, vol, qx, qy, qz, (int)((pk >> 8) & 15u));
                float* o = j.coords + 9 * t;
                o[0] = va.p.x; o[1] = va.p.y; o[2] = va.p.z;
                o[3] = vb.p.x; o[4] = vb.p.y; o[5] = vb.p.z;
                o[6] = vd.p.x; o[7] = vd.p.y; o[8] = vd.p.z;
                uint8_t* col = j.colors + 9 * t;
                col[0] = va.rgb.x; col[1] = va.rgb.y; col[2] = va.rgb.z;
                col[3] = vb.rgb.x; col[4] = vb.rgb.y; col[5] = vb.rgb.z;
                col[6] = vd.rgb.x; col[7] = vd.rgb.y; col[8] = vd.rgb.z;
                const float3 nn = slice_normal(va.p, vb.p, vd.p);
                float* w = j.normals + 3 * t;
                w[0] = nn.x; w[1] = nn.y; w[2] = nn.z;
            }
        }
    }
}

// blocks for `units` work items of `per_block` each, at most 16 per SM
unsigned slice_grid(uint64_t units, uint64_t per_block, const Launch& L)
{
    const uint64_t blocks = (units + per_block - 1) / per_block;
    const uint64_t cap = (uint64_t)L.num_sms * 16;
    return (unsigned)(blocks < cap ? (blocks ? blocks : 1) : cap);
}

}  // namespace

cudaError_t launch_slice_count(const SliceJob& j, const Launch& L)
{
    if (j.nrows == 0) return cudaSuccess;
    prof_begin(L, "slice_count");
    k_slice_count<<<slice_grid(j.nrows, kSliceThreads, L), kSliceThreads, 0, L.stream>>>(j);
    prof_end(L);
    *L.counter += 1;
    return cudaGetLastError();
}

cudaError_t launch_slice_emit(const SliceJob& j, const Launch& L)
{
    if (j.nrows == 0) return cudaSuccess;
    prof_begin(L, "slice_emit");
    switch (j.vol.dtype) {
    case 0: k_slice_emit<int8_t><<<slice_grid(j.nrows, (kSliceThreads / 32) * 32, L), kSliceThreads, 0, L.stream>>>(j); break;
    case 1: k_slice_emit<int16_t><<<slice_grid(j.nrows, (kSliceThreads / 32) * 32, L), kSliceThreads, 0, L.stream>>>(j); break;
    case 2: k_slice_emit<int32_t><<<slice_grid(j.nrows, (kSliceThreads / 32) * 32, L), kSliceThreads, 0, L.stream>>>(j); break;
    case 3: k_slice_emit<long long><<<slice_grid(j.nrows, (kSliceThreads / 32) * 32, L), kSliceThreads, 0, L.stream>>>(j); break;
    case 4: k_slice_emit<uint8_t><<<slice_grid(j.nrows, (kSliceThreads / 32) * 32, L), kSliceThreads, 0, L.stream>>>(j); break;
    case 5: k_slice_emit<uint16_t><<<slice_grid(j.nrows, (kSliceThreads / 32) * 32, L), kSliceThreads, 0, L.stream>>>(j); break;
    case 6: k_slice_emit<uint32_t><<<slice_grid(j.nrows, (kSliceThreads / 32) * 32, L), kSliceThreads, 0, L.stream>>>(j); break;
    case 7: k_slice_emit<unsigned long long><<<slice_grid(j.nrows, (kSliceThreads / 32) * 32, L), kSliceThreads, 0, L.stream>>>(j); break;
    case 8: k_slice_emit<float><<<slice_grid(j.nrows, (kSliceThreads / 32) * 32, L), kSliceThreads, 0, L.stream>>>(j); break;
    case 9: k_slice_emit<double><<<slice_grid(j.nrows, (kSliceThreads / 32) * 32, L), kSliceThreads, 0, L.stream>>>(j); break;
    default: prof_end(L); return cudaErrorInvalidValue;
    }
    prof_end(L);
    *L.counter += 1;
    return cudaGetLastError();
}

}  // namespace kvsmc

namespace {

using kvsmc_host::fail;

// Count one slice on a resident volume (plan, count, scan; *ntri = total)
// into the context's scratch; slice_emit then writes it.  The job stays
// valid until the scratch is next used.
kvsmc_status slice_count_pass(kvsmc_context* ctx, kvsmc_volume* v, const kvsmc_slice_params* p, kvsmc::SliceJob& j,
                              uint64_t* ntri)
{
    using namespace kvsmc_host;
    *ntri = 0;
    std::memset(&j, 0, sizeof j);
    if (!p || !p->tf_table || p->tf_resolution < 1)
        return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "slice: bad parameters (colour table)");
    const kvsmc::VolumeView& vv = v->view;
    if (vv.nx < 2 || vv.ny < 2 || vv.nz < 2) return KVSMC_OK;   // no cells
    j.vol = vv;
    for (int k = 0; k < 4; ++k) j.coef[k] = p->coefficients[k];
    for (int k = 0; k < 3; ++k) { j.min_coord[k] = p->min_coord[k]; j.scale[k] = p->scale[k]; }
    j.tf_min = p->tf_min;
    j.tf_max = p->tf_max;
    j.tf_res = p->tf_resolution;
    j.nrows = (uint64_t)(vv.ny - 1) * (vv.nz - 1);
    const size_t bt = align_up((size_t)3 * j.tf_res, 256), bc = align_up(j.nrows * 4, 256),
                 bo = align_up(j.nrows * 8, 256), bs = align_up(kvsmc::scan_scratch_bytes(j.nrows), 256);
    kvsmc_status st = ensure_scratch(ctx, bt + bc + bo + bs + 256);
    if (st) return st;
    char* base = static_cast<char*>(ctx->scratch);
    uint8_t* d_table = reinterpret_cast<uint8_t*>(base);
    j.table = d_table;
    j.row_counts = reinterpret_cast<uint32_t*>(base + bt);
    j.row_offsets = reinterpret_cast<uint64_t*>(base + bt + bc);
    void* d_scan = base + bt + bc + bo;
    uint64_t* d_total = reinterpret_cast<uint64_t*>(base + bt + bc + bo + bs);
    if ((st = ensure_stage(ctx, (size_t)3 * j.tf_res))) return st;
    std::memcpy(ctx->h_stage, p->tf_table, (size_t)3 * j.tf_res);
    KVSMC_CUDA(ctx, cudaMemcpyAsync(d_table, ctx->h_stage, (size_t)3 * j.tf_res, cudaMemcpyHostToDevice, ctx->stream));
    const kvsmc::Launch L = launch_of(ctx);
    KVSMC_CUDA(ctx, kvsmc::launch_slice_count(j, L));
    KVSMC_CUDA(ctx, kvsmc::launch_scan(j.row_counts, j.row_offsets, j.nrows, d_scan, d_total, L));
    KVSMC_CUDA(ctx, cudaMemcpyAsync(ctx->h_small, d_total, sizeof(uint64_t), cudaMemcpyDeviceToHost, ctx->stream));
    KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *ntri = ctx->h_small[0];
    return KVSMC_OK;
}

kvsmc_status slice_emit(kvsmc_context* ctx, kvsmc::SliceJob& j, float* d_coords, uint8_t* d_colors, float* d_normals,
                        uint64_t cap)
{
    using namespace kvsmc_host;
    if (j.nrows == 0) return KVSMC_OK;
    j.coords = d_coords;
    j.colors = d_colors;
    j.normals = d_normals;
    j.cap_tris = cap;
    KVSMC_CUDA(ctx, kvsmc::launch_slice_emit(j, launch_of(ctx)));
    return KVSMC_OK;
}

}  // namespace

extern "C" {

kvsmc_status kvsmc_slice_count(kvsmc_context* ctx, kvsmc_volume* vol, const kvsmc_slice_params* p,
                               uint64_t* ntriangles)
{
    if (!ctx || !vol || !ntriangles) return KVSMC_ERR_INVALID_ARGUMENT;
    KVSMC_CUDA(ctx, cudaSetDevice(ctx->device));
    kvsmc::SliceJob j;
    return slice_count_pass(ctx, vol, p, j, ntriangles);
}

kvsmc_status kvsmc_slice_extract_device(kvsmc_context* ctx, kvsmc_volume* vol, const kvsmc_slice_params* p,
                                        float* d_coords, uint64_t coords_capacity, uint8_t* d_colors,
                                        uint64_t colors_capacity, float* d_normals, uint64_t normals_capacity,
                                        uint64_t* ntriangles)
{
    if (!ctx || !vol || !ntriangles) return KVSMC_ERR_INVALID_ARGUMENT;
    KVSMC_CUDA(ctx, cudaSetDevice(ctx->device));
    uint64_t n = 0;
    kvsmc::SliceJob j;
    kvsmc_status st = slice_count_pass(ctx, vol, p, j, &n);
    *ntriangles = n;
    if (st || n == 0) return st;
    const uint64_t cap = std::min(std::min(coords_capacity / 9, colors_capacity / 9), normals_capacity / 3);
    if (!d_coords || !d_colors || !d_normals || cap < n)
        return fail(ctx, KVSMC_ERR_CAPACITY, "slice: %llu triangles do not fit the outputs", (unsigned long long)n);
    st = slice_emit(ctx, j, d_coords, d_colors, d_normals, cap);
    if (!st) KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return st;
}

kvsmc_status kvsmc_slice_plane(kvsmc_context* ctx, kvsmc_volume* vol, const kvsmc_slice_params* p,
                               kvsmc_host_alloc_fn alloc, void* user, uint64_t* ntriangles)
{
    using namespace kvsmc_host;
    if (!ctx || !vol || !alloc || !ntriangles) return KVSMC_ERR_INVALID_ARGUMENT;
    KVSMC_CUDA(ctx, cudaSetDevice(ctx->device));
    uint64_t n = 0;
    kvsmc::SliceJob j;
    kvsmc_status st = slice_count_pass(ctx, vol, p, j, &n);
    *ntriangles = n;
    if (st || n == 0) return st;
    const size_t bc = align_up(n * 36, 256), bn = align_up(n * 12, 256), bk = align_up(n * 9, 256);
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
    float* dc = reinterpret_cast<float*>(base);
    float* dn = reinterpret_cast<float*>(base + bc);
    uint8_t* dk = reinterpret_cast<uint8_t*>(base + bc + bn);
    if ((st = slice_emit(ctx, j, dc, dk, dn, n))) return st;
    void* hc = alloc(user, 0, 9 * n);
    void* hn = hc ? alloc(user, 1, 3 * n) : nullptr;
    void* hk = hn ? alloc(user, 3, 9 * n) : nullptr;
    if (!hc || !hn || !hk) return fail(ctx, KVSMC_ERR_OUT_OF_MEMORY, "slice: host alloc");
    KVSMC_CUDA(ctx, cudaMemcpyAsync(hc, dc, n * 36, cudaMemcpyDeviceToHost, ctx->stream));
    KVSMC_CUDA(ctx, cudaMemcpyAsync(hn, dn, n * 12, cudaMemcpyDeviceToHost, ctx->stream));
    KVSMC_CUDA(ctx, cudaMemcpyAsync(hk, dk, n * 9, cudaMemcpyDeviceToHost, ctx->stream));
    KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return KVSMC_OK;
}

}  // extern "C"
