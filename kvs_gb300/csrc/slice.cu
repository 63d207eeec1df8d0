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
// Two passes over tiles of cell rows (one plane z, up to a few rows): count
// (cases from the plane alone, no volume read), an exclusive scan of the tile
// counts, then emit (block-wide scan of each cell's triangle count, the
// volume read only at the corners of cut edges).
#include <cuda_runtime.h>

#include <cstring>

#include "context.h"
#include "mc_tables.h"

namespace kvsmc {

namespace {

__constant__ uint64_t c_slice_tri[256] = MC_TRI_PACKED_INIT;
__constant__ uint8_t c_slice_ntri[256] = MC_NTRI_INIT;
__constant__ uint8_t c_slice_edge[12] = MC_EDGE_PACKED_INIT;

constexpr int kSliceThreads = 128;

__device__ __forceinline__ float plane_at(const SliceJob& j, float x, float y, float z)
{
    return __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(j.coef[0], x), __fmul_rn(j.coef[1], y)), __fmul_rn(j.coef[2], z)),
                     j.coef[3]);
}

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

// values[i0] + ratio * (values[i1] - values[i0]) with C++'s conversions for
// each value type; the result as the float ColorMap::at receives.
__device__ __forceinline__ float slice_value(int8_t a, int8_t b, float r)
{
    return __fadd_rn(__int2float_rn((int)a), __fmul_rn(r, __int2float_rn((int)b - (int)a)));
}
__device__ __forceinline__ float slice_value(uint8_t a, uint8_t b, float r)
{
    return __fadd_rn(__int2float_rn((int)a), __fmul_rn(r, __int2float_rn((int)b - (int)a)));
}
__device__ __forceinline__ float slice_value(int16_t a, int16_t b, float r)
{
    return __fadd_rn(__int2float_rn((int)a), __fmul_rn(r, __int2float_rn((int)b - (int)a)));
}
__device__ __forceinline__ float slice_value(uint16_t a, uint16_t b, float r)
{
    return __fadd_rn(__int2float_rn((int)a), __fmul_rn(r, __int2float_rn((int)b - (int)a)));
}
__device__ __forceinline__ float slice_value(int32_t a, int32_t b, float r)
{
    const int32_t d = (int32_t)((uint32_t)b - (uint32_t)a);   // two's-complement wrap
    return __fadd_rn(__int2float_rn(a), __fmul_rn(r, __int2float_rn(d)));
}
__device__ __forceinline__ float slice_value(uint32_t a, uint32_t b, float r)
{
    return __fadd_rn(__uint2float_rn(a), __fmul_rn(r, __uint2float_rn(b - a)));
}
__device__ __forceinline__ float slice_value(long long a, long long b, float r)
{
    const long long d = (long long)((unsigned long long)b - (unsigned long long)a);
    return __fadd_rn(__ll2float_rn(a), __fmul_rn(r, __ll2float_rn(d)));
}
__device__ __forceinline__ float slice_value(unsigned long long a, unsigned long long b, float r)
{
    return __fadd_rn(__ull2float_rn(a), __fmul_rn(r, __ull2float_rn(b - a)));
}
__device__ __forceinline__ float slice_value(float a, float b, float r)
{
    return __fadd_rn(a, __fmul_rn(r, __fsub_rn(b, a)));
}
__device__ __forceinline__ float slice_value(double a, double b, float r)
{
    return __double2float_rn(__dadd_rn(a, __dmul_rn((double)r, __dsub_rn(b, a))));
}

// ColorMap::at (ColorMap.cpp:1043-1054) with RGBColor::Mix and the
// RGBColor(Vec3) rounding (RGBColor.cpp:23-31, 125-134; Math::Round).
__device__ __forceinline__ uchar3 color_at(const SliceJob& j, float value)
{
    const float lo = j.tf_min, hi = j.tf_max;
    const float v0 = value <= lo ? lo : (value <= hi ? value : hi);
    const float r = (float)(j.tf_res - 1);
    const float v = __fmul_rn(__fdiv_rn(__fsub_rn(v0, lo), __fsub_rn(hi, lo)), r);
    // a NaN or out-of-range table position (undefined in the reference): entry 0
    const uint32_t s0 = (v >= 0.0f && v <= r) ? (uint32_t)v : 0u;
    const uint32_t s1 = (s0 + 1 < (uint32_t)j.tf_res) ? s0 + 1 : (uint32_t)j.tf_res - 1;
    const float t = (v >= 0.0f && v <= r) ? __fsub_rn(v, __uint2float_rn(s0)) : 0.0f;
    uint8_t out[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float a = __fdiv_rn(__uint2float_rn(j.table[3 * s0 + k]), 255.0f);
        const float b = __fdiv_rn(__uint2float_rn(j.table[3 * s1 + k]), 255.0f);
        float m = __fadd_rn(__fmul_rn(a, __fsub_rn(1.0f, t)), __fmul_rn(b, t));
        m = m <= 0.0f ? 0.0f : (m <= 1.0f ? m : 1.0f);
        const float x = __fmul_rn(m, 255.0f);
        out[k] = (uint8_t)__double2int_rz(__dadd_rn((double)x, 0.5));
    }
    return make_uchar3(out[0], out[1], out[2]);
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

// -((c - a) x (b - a)) (Vector3::cross, Matrix/Vector3.h; negation last)
__device__ __forceinline__ float3 slice_normal(float3 a, float3 b, float3 c)
{
    const float ux = __fsub_rn(c.x, a.x), uy = __fsub_rn(c.y, a.y), uz = __fsub_rn(c.z, a.z);
    const float vx = __fsub_rn(b.x, a.x), vy = __fsub_rn(b.y, a.y), vz = __fsub_rn(b.z, a.z);
    float3 n;
    n.x = -__fsub_rn(__fmul_rn(uy, vz), __fmul_rn(uz, vy));
    n.y = -__fsub_rn(__fmul_rn(uz, vx), __fmul_rn(ux, vz));
    n.z = -__fsub_rn(__fmul_rn(ux, vy), __fmul_rn(uy, vx));
    return n;
}

__device__ __forceinline__ void slice_tile(const SliceJob& j, uint64_t tile, uint32_t& z, uint32_t& y0, uint32_t& rows)
{
    z = (uint32_t)(tile / j.ytiles);
    y0 = (uint32_t)(tile - (uint64_t)z * j.ytiles) * j.rows;
    const uint32_t cy = j.vol.ny - 1;
    rows = (cy - y0) < j.rows ? (cy - y0) : j.rows;
}

// True when every node of the tile's cells (x in [0, cx], y in [y0, y0 + rows],
// z in [z, z + 1]) evaluates to the same side of the plane in float, so no
// cell of the tile is cut.  The plane is linear: its exact range over the box
// is taken at the box corners in double (the float products of the
// coefficients with integers below 2^24 are exact there); the float
// evaluation ((a x + b y) + c z) + d differs from the exact value by less
// than 2^-21 (|a| x_max + |b| y_max + |c| z_max + |d|) (four roundings of
// 2^-24 each), so a range beyond that margin decides every node's sign.
__device__ __forceinline__ bool tile_uncut(const SliceJob& j, uint32_t cx, uint32_t y0, uint32_t rows, uint32_t z)
{
    const double a = j.coef[0], b = j.coef[1], c = j.coef[2], d = j.coef[3];
    const double x0 = 0.0, x1 = (double)cx, ya = (double)y0, yb = (double)(y0 + rows), za = (double)z,
                 zb = (double)(z + 1);
    const double lo = (a < 0 ? a * x1 : a * x0) + (b < 0 ? b * yb : b * ya) + (c < 0 ? c * zb : c * za) + d;
    const double hi = (a < 0 ? a * x0 : a * x1) + (b < 0 ? b * ya : b * yb) + (c < 0 ? c * za : c * zb) + d;
    const double m = 4.76837158203125e-07 * (fabs(a) * x1 + fabs(b) * yb + fabs(c) * zb + fabs(d)) + 1e-30;
    return lo > m || hi < -m;
}

__device__ __forceinline__ uint32_t block_sum_u32(uint32_t v, uint32_t* ws)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) ws[warp] = v;
    __syncthreads();
    uint32_t t = 0;
    for (unsigned w = 0; w < blockDim.x / 32; ++w) t += ws[w];
    return t;
}

// Exclusive scan over the block; *total = the block's sum.
__device__ __forceinline__ uint32_t block_excl_u32(uint32_t v, uint32_t* ws, uint32_t* total)
{
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t inc = v;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= (unsigned)o) inc += t;
    }
    __syncthreads();
    if (lane == 31) ws[warp] = inc;
    __syncthreads();
    uint32_t before = 0, all = 0;
    for (unsigned w = 0; w < blockDim.x / 32; ++w) {
        before += w < warp ? ws[w] : 0u;
        all += ws[w];
    }
    *total = all;
    return before + inc - v;
}

__global__ void __launch_bounds__(kSliceThreads) k_slice_count(SliceJob j)
{
    __shared__ uint32_t ws[32];
    const uint32_t cx = j.vol.nx - 1;
    for (uint64_t tile = blockIdx.x; tile < j.tiles; tile += gridDim.x) {
        uint32_t z, y0, rows;
        slice_tile(j, tile, z, y0, rows);
        if (tile_uncut(j, cx, y0, rows, z)) {   // uniform across the block
            if (threadIdx.x == 0) j.tile_counts[tile] = 0;
            continue;
        }
        uint32_t sum = 0;
        for (uint32_t r = 0; r < rows; ++r)
            for (uint32_t x = threadIdx.x; x < cx; x += blockDim.x) sum += c_slice_ntri[slice_case(j, x, y0 + r, z)];
        const uint32_t t = block_sum_u32(sum, ws);
        if (threadIdx.x == 0) j.tile_counts[tile] = t;
    }
}

template <typename T>
__global__ void __launch_bounds__(kSliceThreads) k_slice_emit(SliceJob j)
{
    __shared__ uint32_t ws[32];
    const T* vol = static_cast<const T*>(j.vol.data);
    const uint32_t cx = j.vol.nx - 1;
    for (uint64_t tile = blockIdx.x; tile < j.tiles; tile += gridDim.x) {
        uint32_t z, y0, rows;
        slice_tile(j, tile, z, y0, rows);
        if (tile_uncut(j, cx, y0, rows, z)) continue;   // uniform across the block
        uint64_t running = j.tile_offsets[tile];
        for (uint32_t r = 0; r < rows; ++r) {
            const uint32_t y = y0 + r;
            for (uint32_t xc = 0; xc < cx; xc += blockDim.x) {
                const uint32_t x = xc + threadIdx.x;
                const unsigned c = x < cx ? slice_case(j, x, y, z) : 0u;
                const uint32_t n = c_slice_ntri[c];
                uint32_t tot;
                const uint32_t excl = block_excl_u32(n, ws, &tot);
                uint64_t t = running + excl;
                uint64_t pk = c_slice_tri[c];
                for (uint32_t k = 0; k < n; ++k, ++t, pk >>= 12) {
                    if (t >= j.cap_tris) break;   // never past the outputs
                    const SliceVertex a = slice_vertex<T>(j, vol, x, y, z, (int)(pk & 15u));
                    const SliceVertex b = slice_vertex<T>(j, vol, x, y, z, (int)((pk >> 4) & 15u));
                    const SliceVertex d = slice_vertex<T>(j, vol, x, y, z, (int)((pk >> 8) & 15u));
                    float* o = j.coords + 9 * t;
                    o[0] = a.p.x; o[1] = a.p.y; o[2] = a.p.z;
                    o[3] = b.p.x; o[4] = b.p.y; o[5] = b.p.z;
                    o[6] = d.p.x; o[7] = d.p.y; o[8] = d.p.z;
                    uint8_t* col = j.colors + 9 * t;
                    col[0] = a.rgb.x; col[1] = a.rgb.y; col[2] = a.rgb.z;
                    col[3] = b.rgb.x; col[4] = b.rgb.y; col[5] = b.rgb.z;
                    col[6] = d.rgb.x; col[7] = d.rgb.y; col[8] = d.rgb.z;
                    const float3 nn = slice_normal(a.p, b.p, d.p);
                    float* q = j.normals + 3 * t;
                    q[0] = nn.x; q[1] = nn.y; q[2] = nn.z;
                }
                running += tot;
            }
        }
    }
}

unsigned slice_grid(uint64_t tiles, const Launch& L)
{
    const uint64_t cap = (uint64_t)L.num_sms * 16;
    return (unsigned)(tiles < cap ? (tiles ? tiles : 1) : cap);
}

}  // namespace

cudaError_t launch_slice_count(const SliceJob& j, const Launch& L)
{
    if (j.tiles == 0) return cudaSuccess;
    prof_begin(L, "slice_count");
    k_slice_count<<<slice_grid(j.tiles, L), kSliceThreads, 0, L.stream>>>(j);
    prof_end(L);
    *L.counter += 1;
    return cudaGetLastError();
}

cudaError_t launch_slice_emit(const SliceJob& j, const Launch& L)
{
    if (j.tiles == 0) return cudaSuccess;
    prof_begin(L, "slice_emit");
    switch (j.vol.dtype) {
    case 0: k_slice_emit<int8_t><<<slice_grid(j.tiles, L), kSliceThreads, 0, L.stream>>>(j); break;
    case 1: k_slice_emit<int16_t><<<slice_grid(j.tiles, L), kSliceThreads, 0, L.stream>>>(j); break;
    case 2: k_slice_emit<int32_t><<<slice_grid(j.tiles, L), kSliceThreads, 0, L.stream>>>(j); break;
    case 3: k_slice_emit<long long><<<slice_grid(j.tiles, L), kSliceThreads, 0, L.stream>>>(j); break;
    case 4: k_slice_emit<uint8_t><<<slice_grid(j.tiles, L), kSliceThreads, 0, L.stream>>>(j); break;
    case 5: k_slice_emit<uint16_t><<<slice_grid(j.tiles, L), kSliceThreads, 0, L.stream>>>(j); break;
    case 6: k_slice_emit<uint32_t><<<slice_grid(j.tiles, L), kSliceThreads, 0, L.stream>>>(j); break;
    case 7: k_slice_emit<unsigned long long><<<slice_grid(j.tiles, L), kSliceThreads, 0, L.stream>>>(j); break;
    case 8: k_slice_emit<float><<<slice_grid(j.tiles, L), kSliceThreads, 0, L.stream>>>(j); break;
    case 9: k_slice_emit<double><<<slice_grid(j.tiles, L), kSliceThreads, 0, L.stream>>>(j); break;
    default: prof_end(L); return cudaErrorInvalidValue;
    }
    prof_end(L);
    *L.counter += 1;
    return cudaGetLastError();
}

}  // namespace kvsmc

namespace {

using kvsmc_host::fail;

// Plan, count and (when outputs are given) emit one slice on a resident
// volume; *ntri = the triangle count.  Outputs: device arrays of at least
// cap triangles (the emit never writes past them).
kvsmc_status slice_run(kvsmc_context* ctx, kvsmc_volume* v, const kvsmc_slice_params* p, float* d_coords,
                       uint8_t* d_colors, float* d_normals, uint64_t cap, bool emit, uint64_t* ntri)
{
    using namespace kvsmc_host;
    *ntri = 0;
    if (!p || (p->tf_resolution > 0 && !p->tf_table) || p->tf_resolution < 1)
        return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "slice: bad parameters (colour table)");
    const kvsmc::VolumeView& vv = v->view;
    if (vv.nx < 2 || vv.ny < 2 || vv.nz < 2) return KVSMC_OK;   // no cells
    kvsmc::SliceJob j;
    std::memset(&j, 0, sizeof j);
    j.vol = vv;
    for (int k = 0; k < 4; ++k) j.coef[k] = p->coefficients[k];
    for (int k = 0; k < 3; ++k) { j.min_coord[k] = p->min_coord[k]; j.scale[k] = p->scale[k]; }
    j.tf_min = p->tf_min;
    j.tf_max = p->tf_max;
    j.tf_res = p->tf_resolution;
    const uint32_t cx = vv.nx - 1, cy = vv.ny - 1, cz = vv.nz - 1;
    j.rows = std::max<uint32_t>(1, std::min<uint32_t>(cy, (2048 + cx - 1) / cx));
    j.ytiles = (cy + j.rows - 1) / j.rows;
    j.tiles = (uint64_t)cz * j.ytiles;
    const size_t bt = align_up((size_t)3 * j.tf_res, 256), bc = align_up(j.tiles * 4, 256),
                 bo = align_up(j.tiles * 8, 256), bs = align_up(kvsmc::scan_scratch_bytes(j.tiles), 256);
    kvsmc_status st = ensure_scratch(ctx, bt + bc + bo + bs + 256);
    if (st) return st;
    char* base = static_cast<char*>(ctx->scratch);
    uint8_t* d_table = reinterpret_cast<uint8_t*>(base);
    j.table = d_table;
    j.tile_counts = reinterpret_cast<uint32_t*>(base + bt);
    j.tile_offsets = reinterpret_cast<uint64_t*>(base + bt + bc);
    void* d_scan = base + bt + bc + bo;
    uint64_t* d_total = reinterpret_cast<uint64_t*>(base + bt + bc + bo + bs);
    if ((st = ensure_stage(ctx, (size_t)3 * j.tf_res))) return st;
    std::memcpy(ctx->h_stage, p->tf_table, (size_t)3 * j.tf_res);
    KVSMC_CUDA(ctx, cudaMemcpyAsync(d_table, ctx->h_stage, (size_t)3 * j.tf_res, cudaMemcpyHostToDevice, ctx->stream));
    const kvsmc::Launch L = launch_of(ctx);
    KVSMC_CUDA(ctx, kvsmc::launch_slice_count(j, L));
    KVSMC_CUDA(ctx, kvsmc::launch_scan(j.tile_counts, j.tile_offsets, j.tiles, d_scan, d_total, L));
    KVSMC_CUDA(ctx, cudaMemcpyAsync(ctx->h_small, d_total, sizeof(uint64_t), cudaMemcpyDeviceToHost, ctx->stream));
    KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *ntri = ctx->h_small[0];
    if (!emit || *ntri == 0) return KVSMC_OK;
    j.coords = d_coords;
    j.colors = d_colors;
    j.normals = d_normals;
    j.cap_tris = cap;
    KVSMC_CUDA(ctx, kvsmc::launch_slice_emit(j, L));
    return KVSMC_OK;
}

}  // namespace

extern "C" {

kvsmc_status kvsmc_slice_count(kvsmc_context* ctx, kvsmc_volume* vol, const kvsmc_slice_params* p,
                               uint64_t* ntriangles)
{
    if (!ctx || !vol || !ntriangles) return KVSMC_ERR_INVALID_ARGUMENT;
    KVSMC_CUDA(ctx, cudaSetDevice(ctx->device));
    return slice_run(ctx, vol, p, nullptr, nullptr, nullptr, 0, false, ntriangles);
}

kvsmc_status kvsmc_slice_extract_device(kvsmc_context* ctx, kvsmc_volume* vol, const kvsmc_slice_params* p,
                                        float* d_coords, uint64_t coords_capacity, uint8_t* d_colors,
                                        uint64_t colors_capacity, float* d_normals, uint64_t normals_capacity,
                                        uint64_t* ntriangles)
{
    if (!ctx || !vol || !ntriangles) return KVSMC_ERR_INVALID_ARGUMENT;
    KVSMC_CUDA(ctx, cudaSetDevice(ctx->device));
    uint64_t n = 0;
    kvsmc_status st = slice_run(ctx, vol, p, nullptr, nullptr, nullptr, 0, false, &n);
    *ntriangles = n;
    if (st || n == 0) return st;
    const uint64_t cap = std::min(std::min(coords_capacity / 9, colors_capacity / 9), normals_capacity / 3);
    if (!d_coords || !d_colors || !d_normals || cap < n)
        return fail(ctx, KVSMC_ERR_CAPACITY, "slice: %llu triangles do not fit the outputs", (unsigned long long)n);
    st = slice_run(ctx, vol, p, d_coords, d_colors, d_normals, cap, true, &n);
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
    kvsmc_status st = slice_run(ctx, vol, p, nullptr, nullptr, nullptr, 0, false, &n);
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
    if ((st = slice_run(ctx, vol, p, dc, dk, dn, n, true, &n))) return st;
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
