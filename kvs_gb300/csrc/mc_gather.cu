// mc_gather.cu -- the gather-form kernels: one thread per cell (or node),
// corner values fetched through the read-only cache.  They cover every mode
// and every dtype and define the layout of the intermediate buffers:
//
//   cell tile  = `cell_rows` consecutive cell rows of one z-slab, full x:
//                a contiguous range of the reference's linear cell order.
//   node tile  = `node_rows` consecutive node rows of one z-plane, full x.
//   rank word  = per 32 nodes of a node row: the x-, y- and z-edge crossing
//                flags (one bit per node each) and the id of the first
//                vertex in the word.  Vertex ids follow the reference's
//                numbering (node order, then x, y, z edge:
//                MarchingCubes.cpp:388-441), so id = word base + popcounts.
#include <cuda_runtime.h>

#include "mc_internal.h"

namespace kvsmc {

namespace {

__constant__ uint64_t c_tri_packed[256] = MC_TRI_PACKED_INIT;
__constant__ uint8_t c_ntri[256] = MC_NTRI_INIT;
__constant__ uint8_t c_edge_packed[12] = MC_EDGE_PACKED_INIT;

struct SmemTables {
    uint64_t tri[256];
    uint8_t ntri[256];
    uint8_t edge[16];
};

__device__ __forceinline__ void load_tables(SmemTables& t)
{
    for (unsigned i = threadIdx.x; i < 256; i += blockDim.x) {
        t.tri[i] = c_tri_packed[i];
        t.ntri[i] = c_ntri[i];
        if (i < 12) t.edge[i] = c_edge_packed[i];
    }
    __syncthreads();
}

constexpr int kThreads = 128;

int grid_for(uint64_t tiles, const Launch& L)
{
    const uint64_t cap = (uint64_t)L.num_sms * 16;
    uint64_t g = tiles < cap ? tiles : cap;
    return g == 0 ? 1 : (int)g;
}

// ------------------------------------------------------------ min / max

template <typename T> __device__ __forceinline__ bool is_nan(T) { return false; }
template <> __device__ __forceinline__ bool is_nan<float>(float v) { return v != v; }
template <> __device__ __forceinline__ bool is_nan<double>(double v) { return v != v; }

template <typename T>
struct MinMax {
    T lo, hi;
    unsigned long long ilo, ihi;
    int any;
};

// Combine so that the result equals the reference's sequential scan
// (StructuredVolumeObject.cpp:80-85): the first occurrence wins among equal
// values (this only matters for -0.0 vs +0.0).
template <typename T>
__device__ __forceinline__ void mm_combine(MinMax<T>& a, const MinMax<T>& b)
{
    if (!b.any) return;
    if (!a.any) { a = b; return; }
    if (b.lo < a.lo || (b.lo == a.lo && b.ilo < a.ilo)) { a.lo = b.lo; a.ilo = b.ilo; }
    if (b.hi > a.hi || (b.hi == a.hi && b.ihi < a.ihi)) { a.hi = b.hi; a.ihi = b.ihi; }
}

template <typename T>
__device__ void mm_block_reduce(MinMax<T>& m, MinMax<T>* sm)
{
    sm[threadIdx.x] = m;
    __syncthreads();
    for (unsigned s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            MinMax<T> a = sm[threadIdx.x];
            mm_combine(a, sm[threadIdx.x + s]);
            sm[threadIdx.x] = a;
        }
        __syncthreads();
    }
    m = sm[0];
}

template <typename T>
__global__ void __launch_bounds__(256) k_minmax_partial(VolumeView v, MinMax<T>* partial)
{
    __shared__ MinMax<T> sm[256];
    const T* d = static_cast<const T*>(v.data);
    const uint64_t rows = (uint64_t)v.ny * v.nz;
    const uint64_t per = (rows + gridDim.x - 1) / gridDim.x;
    const uint64_t r0 = (uint64_t)blockIdx.x * per;
    const uint64_t r1 = r0 + per < rows ? r0 + per : rows;
    MinMax<T> m;
    m.any = 0; m.lo = T(0); m.hi = T(0); m.ilo = m.ihi = 0;
    for (uint64_t row = r0; row < r1; ++row) {
        const uint64_t z = row / v.ny, y = row - z * v.ny;
        const T* p = d + y * v.pitch + z * v.slice;
        const unsigned long long lin = (unsigned long long)row * v.nx;
        for (uint32_t x = threadIdx.x; x < v.nx; x += blockDim.x) {
            const T val = __ldg(p + x);
            if (is_nan(val)) continue;
            const unsigned long long idx = lin + x;
            if (!m.any) { m.lo = m.hi = val; m.ilo = m.ihi = idx; m.any = 1; continue; }
            if (val < m.lo) { m.lo = val; m.ilo = idx; }
            if (val > m.hi) { m.hi = val; m.ihi = idx; }
        }
    }
    mm_block_reduce(m, sm);
    if (threadIdx.x == 0) partial[blockIdx.x] = m;
}

template <typename T>
__global__ void __launch_bounds__(256) k_minmax_final(VolumeView v, const MinMax<T>* partial, int n, double* out)
{
    __shared__ MinMax<T> sm[256];
    MinMax<T> m;
    m.any = 0; m.lo = T(0); m.hi = T(0); m.ilo = m.ihi = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) mm_combine(m, partial[i]);
    mm_block_reduce(m, sm);
    if (threadIdx.x == 0) {
        const T first = static_cast<const T*>(v.data)[0];
        if (is_nan(first) || !m.any) {
            // the scan starts at values[0]; a NaN there is never replaced
            out[0] = to_double(first);
            out[1] = to_double(first);
        } else {
            out[0] = to_double(m.lo);
            out[1] = to_double(m.hi);
        }
    }
}

// ------------------------------------------------------------ cell kernels

__device__ __forceinline__ void cell_tile(const Job& j, uint64_t tile, uint32_t& z, uint32_t& y0, uint32_t& rows)
{
    z = (uint32_t)(tile / j.cell_ytiles);
    const uint32_t yb = (uint32_t)(tile - (uint64_t)z * j.cell_ytiles);
    y0 = yb * j.cell_rows;
    const uint32_t cy = j.vol.ny - 1;
    rows = (cy - y0) < j.cell_rows ? (cy - y0) : j.cell_rows;
}

template <typename T>
__global__ void __launch_bounds__(kThreads) k_cell_count(Job j)
{
    __shared__ SmemTables tb;
    __shared__ uint32_t ws[33];
    load_tables(tb);
    const T* vol = static_cast<const T*>(j.vol.data);
    const uint32_t cx = j.vol.nx - 1;
    for (uint64_t tile = blockIdx.x; tile < j.cell_tiles; tile += gridDim.x) {
        uint32_t z, y0, rows;
        cell_tile(j, tile, z, y0, rows);
        uint32_t sum = 0;
        for (uint32_t r = 0; r < rows; ++r)
            for (uint32_t x = threadIdx.x; x < cx; x += blockDim.x)
                sum += tb.ntri[cell_case<T>(j, vol, x, y0 + r, z)];
        const uint32_t t = block_sum(sum, ws);
        if (threadIdx.x == 0) j.tile_counts[tile] = t;
    }
}

// Duplicated vertices + polygon normals (MarchingCubes.cpp:180-234).
template <typename T>
__global__ void __launch_bounds__(kThreads) k_emit_dup(Job j)
{
    __shared__ SmemTables tb;
    __shared__ uint32_t ws[33];
    load_tables(tb);
    const T* vol = static_cast<const T*>(j.vol.data);
    const uint32_t cx = j.vol.nx - 1;
    for (uint64_t tile = blockIdx.x; tile < j.cell_tiles; tile += gridDim.x) {
        uint32_t z, y0, rows;
        cell_tile(j, tile, z, y0, rows);
        uint64_t running = j.tile_offsets[tile];
        for (uint32_t r = 0; r < rows; ++r) {
            const uint32_t y = y0 + r;
            for (uint32_t xc = 0; xc < cx; xc += blockDim.x) {
                const uint32_t x = xc + threadIdx.x;
                const unsigned c = (x < cx) ? cell_case<T>(j, vol, x, y, z) : 0u;
                const uint32_t n = tb.ntri[c];
                uint32_t tot;
                const uint32_t excl = block_exclusive_scan(n, ws, &tot);
                uint64_t t = running + excl;
                uint64_t pk = tb.tri[c];
                for (uint32_t k = 0; k < n; ++k, ++t, pk >>= 12) {
                    const float3 a = cell_edge_vertex<T>(j, vol, tb.edge, x, y, z, (int)(pk & 15u));
                    const float3 b = cell_edge_vertex<T>(j, vol, tb.edge, x, y, z, (int)((pk >> 4) & 15u));
                    const float3 cc = cell_edge_vertex<T>(j, vol, tb.edge, x, y, z, (int)((pk >> 8) & 15u));
                    float* o = j.coords + 9 * t;
                    o[0] = a.x; o[1] = a.y; o[2] = a.z;
                    o[3] = b.x; o[4] = b.y; o[5] = b.z;
                    o[6] = cc.x; o[7] = cc.y; o[8] = cc.z;
                    const float3 nn = tri_normal(a, b, cc);
                    float* q = j.normals + 3 * t;
                    q[0] = nn.x; q[1] = nn.y; q[2] = nn.z;
                }
                running += tot;
            }
        }
    }
}

// ------------------------------------------------------------ node kernels

__device__ __forceinline__ void node_tile(const Job& j, uint64_t tile, uint32_t& z, uint32_t& y0, uint32_t& rows)
{
    z = (uint32_t)(tile / j.node_ytiles);
    const uint32_t yb = (uint32_t)(tile - (uint64_t)z * j.node_ytiles);
    y0 = yb * j.node_rows;
    rows = (j.vol.ny - y0) < j.node_rows ? (j.vol.ny - y0) : j.node_rows;
}

// Crossing flags of node (x,y,z): bit 0 x-edge, bit 1 y-edge, bit 2 z-edge,
// each only inside the grid (calculate_isopoints, MarchingCubes.cpp:401-441).
template <typename T>
__device__ __forceinline__ unsigned node_flags(const Job& j, const T* vol, uint32_t x, uint32_t y, uint32_t z)
{
    const uint64_t i0 = node_index<T>(j.vol, x, y, z);
    const bool b0 = above(j.cls, load(vol, i0));
    unsigned f = 0;
    if (x + 1 < j.vol.nx && above(j.cls, load(vol, i0 + 1)) != b0) f |= 1u;
    if (y + 1 < j.vol.ny && above(j.cls, load(vol, i0 + j.vol.pitch)) != b0) f |= 2u;
    if (z + 1 < j.vol.nz && above(j.cls, load(vol, i0 + j.vol.slice)) != b0) f |= 4u;
    return f;
}

template <typename T>
__global__ void __launch_bounds__(kThreads) k_node_count(Job j)
{
    __shared__ uint32_t ws[33];
    const T* vol = static_cast<const T*>(j.vol.data);
    for (uint64_t tile = blockIdx.x; tile < j.node_tiles; tile += gridDim.x) {
        uint32_t z, y0, rows;
        node_tile(j, tile, z, y0, rows);
        uint32_t sum = 0;
        for (uint32_t r = 0; r < rows; ++r)
            for (uint32_t x = threadIdx.x; x < j.vol.nx; x += blockDim.x)
                sum += __popc(node_flags<T>(j, vol, x, y0 + r, z));
        const uint32_t t = block_sum(sum, ws);
        if (threadIdx.x == 0) j.vtile_counts[tile] = t;
    }
}

// Shared vertex of node (x,y,z) along `axis`, interpolated from this lower
// node to the upper one (MarchingCubes.cpp:406,420,434).
template <typename T>
__device__ __forceinline__ float3 node_edge_vertex(const Job& j, const T* vol, uint32_t x, uint32_t y, uint32_t z, int axis)
{
    const uint64_t i0 = node_index<T>(j.vol, x, y, z);
    const uint64_t step = axis == 0 ? 1 : (axis == 1 ? j.vol.pitch : j.vol.slice);
    const double va = to_double(load(vol, i0));
    const double vb = to_double(load(vol, i0 + step));
    const float fx = __uint2float_rn(x), fy = __uint2float_rn(y), fz = __uint2float_rn(z);
    return interpolate_exact(j.ip, va, vb, fx, fy, fz,
                             axis == 0 ? __uint2float_rn(x + 1) : fx,
                             axis == 1 ? __uint2float_rn(y + 1) : fy,
                             axis == 2 ? __uint2float_rn(z + 1) : fz);
}

template <typename T>
__global__ void __launch_bounds__(kThreads) k_node_emit(Job j)
{
    __shared__ uint32_t ws[33];
    const T* vol = static_cast<const T*>(j.vol.data);
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t lt = (1u << lane) - 1u;
    for (uint64_t tile = blockIdx.x; tile < j.node_tiles; tile += gridDim.x) {
        uint32_t z, y0, rows;
        node_tile(j, tile, z, y0, rows);
        uint64_t running = j.vtile_offsets[tile];
        for (uint32_t r = 0; r < rows; ++r) {
            const uint32_t y = y0 + r;
            const uint64_t row = (uint64_t)z * j.vol.ny + y;
            for (uint32_t xc = 0; xc < j.vol.nx; xc += blockDim.x) {
                const uint32_t x = xc + threadIdx.x;
                const unsigned f = (x < j.vol.nx) ? node_flags<T>(j, vol, x, y, z) : 0u;
                const uint32_t bx = __ballot_sync(0xffffffffu, f & 1u);
                const uint32_t by = __ballot_sync(0xffffffffu, f & 2u);
                const uint32_t bz = __ballot_sync(0xffffffffu, f & 4u);
                const uint32_t wc = __popc(bx) + __popc(by) + __popc(bz);
                uint32_t tot;
                const uint32_t excl = block_exclusive_scan(lane == 0 ? wc : 0u, ws, &tot);
                const uint64_t wbase = running + __shfl_sync(0xffffffffu, excl, 0);
                const uint32_t word = (xc >> 5) + warp;
                if (lane == 0 && word < j.words_per_row)
                    j.rank[row * j.words_per_row + word] = make_uint4(bx, by, bz, (uint32_t)wbase);
                uint64_t id = wbase + __popc(bx & lt) + __popc(by & lt) + __popc(bz & lt);
                for (int axis = 0; axis < 3; ++axis) {
                    if (f & (1u << axis)) {
                        const float3 p = node_edge_vertex<T>(j, vol, x, y, z, axis);
                        float* o = j.coords + 3 * id;
                        o[0] = p.x; o[1] = p.y; o[2] = p.z;
                        ++id;
                    }
                }
                running += tot;
            }
        }
    }
}

// Vertex id of node (x,y,z)'s edge along `axis` from the rank words.
__device__ __forceinline__ uint32_t rank_id(const Job& j, uint32_t x, uint32_t y, uint32_t z, int axis)
{
    const uint64_t row = (uint64_t)z * j.vol.ny + y;
    const uint4 R = j.rank[row * j.words_per_row + (x >> 5)];
    const uint32_t bit = x & 31u, lt = (1u << bit) - 1u;
    uint32_t id = R.w + __popc(R.x & lt) + __popc(R.y & lt) + __popc(R.z & lt);
    if (axis >= 1) id += (R.x >> bit) & 1u;
    if (axis >= 2) id += (R.y >> bit) & 1u;
    return id;
}

// Vertex id of local edge e of cell (x,y,z): the edge's lower node and axis
// (the mapping of connect_isopoints, MarchingCubes.cpp:493-504).
__device__ __forceinline__ uint32_t cell_edge_id(const Job& j, const uint8_t* edge, uint32_t x, uint32_t y, uint32_t z, int e)
{
    const unsigned ep = edge[e];
    const unsigned a = ep & 7u, b = ep >> 3;
    const unsigned n = a & b, d = a ^ b;
    const int axis = d == 1u ? 0 : (d == 2u ? 1 : 2);
    return rank_id(j, x + (n & 1u), y + ((n >> 1) & 1u), z + (n >> 2), axis);
}

__device__ __forceinline__ float3 load_coord(const Job& j, uint32_t id)
{
    const float* p = j.coords + 3 * (uint64_t)id;
    return make_float3(p[0], p[1], p[2]);
}

// connect_isopoints (MarchingCubes.cpp:456-521) and, in the polygon-normal
// mode, calculate_normals_on_polygon (:531-560) from the stored coords.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_connect(Job j)
{
    __shared__ SmemTables tb;
    __shared__ uint32_t ws[33];
    load_tables(tb);
    const T* vol = static_cast<const T*>(j.vol.data);
    const uint32_t cx = j.vol.nx - 1;
    // polygon normals into the output (mode 1), or into the per-triangle
    // scratch the vertex normals are summed from (mode 2)
    float* const tri_out = j.mode == 1 ? j.normals : j.tri_normals;
    for (uint64_t tile = blockIdx.x; tile < j.cell_tiles; tile += gridDim.x) {
        uint32_t z, y0, rows;
        cell_tile(j, tile, z, y0, rows);
        uint64_t running = j.tile_offsets[tile];
        for (uint32_t r = 0; r < rows; ++r) {
            const uint32_t y = y0 + r;
            for (uint32_t xc = 0; xc < cx; xc += blockDim.x) {
                const uint32_t x = xc + threadIdx.x;
                const unsigned c = (x < cx) ? cell_case<T>(j, vol, x, y, z) : 0u;
                const uint32_t n = tb.ntri[c];
                uint32_t tot;
                const uint32_t excl = block_exclusive_scan(n, ws, &tot);
                uint64_t t = running + excl;
                uint64_t pk = tb.tri[c];
                for (uint32_t k = 0; k < n; ++k, ++t, pk >>= 12) {
                    const uint32_t i0 = cell_edge_id(j, tb.edge, x, y, z, (int)(pk & 15u));
                    const uint32_t i1 = cell_edge_id(j, tb.edge, x, y, z, (int)((pk >> 4) & 15u));
                    const uint32_t i2 = cell_edge_id(j, tb.edge, x, y, z, (int)((pk >> 8) & 15u));
                    uint32_t* o = j.connections + 3 * t;
                    o[0] = i0; o[1] = i1; o[2] = i2;
                    if (tri_out) {
                        const float3 nn = tri_normal(load_coord(j, i0), load_coord(j, i1), load_coord(j, i2));
                        float* q = tri_out + 3 * t;
                        q[0] = nn.x; q[1] = nn.y; q[2] = nn.z;
                    }
                }
                running += tot;
            }
        }
    }
}

// calculate_normals_on_vertex (MarchingCubes.cpp:569-605): every vertex's
// normal is the sum, from 0.0f and in triangle order, of the normals of the
// triangles that use it.  Float addition is not associative, so the order is
// kept: each triangle's normal is formed once (by the connection pass), the
// triangle ids of every vertex are placed into its own slots by atomics (in
// any order), and one thread per vertex sorts them and adds the normals in
// increasing triangle order.  A vertex lies on one cell edge, shared by at
// most four cells, and no case of the table puts one edge into more than five
// of its triangles, so a vertex has at most kVnMaxInc triangles: fixed slots,
// no count pass and no scan.  Slots 0-7 of a vertex fill one 32-byte sector
// of their own (v * 8 + s: a vertex's triangles, written close together in
// time, land in one sector, and the sum reads them with two 16-byte loads);
// slots 8-19, rarely used, follow slot-major (8 nvert + (s - 8) nvert + v).
// (connections hold vertex ids below nvert; an id at or above it, which
// consistent inputs never give, is skipped so nothing is touched out of
// range, and so is a slot past kVnMaxInc)
constexpr uint32_t kVnMaxInc = 20;   // 4 cells x 5 triangles of one cell on one edge

__device__ __forceinline__ uint64_t vn_slot(uint32_t s, uint64_t v, uint64_t nvert)
{
    return s < 8u ? 8 * v + s : (uint64_t)s * nvert + v;
}

// One incidence per lane, 32 consecutive ones per warp: lanes holding the
// same vertex (a cell's triangles share corners) take their slots with one
// atomic for the group.  (Four incidences per lane in flight measured slower:
// the pass is not bound by the atomics' latency.)
__global__ void __launch_bounds__(256) k_vn_fill(const uint32_t* __restrict__ conn, uint64_t ntri, uint64_t nvert,
                                                uint32_t* __restrict__ vcount, uint32_t* __restrict__ vlist)
{
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t lt = (1u << lane) - 1u;
    const uint64_t n = 3 * ntri;
    for (uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); i0 < n;
         i0 += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i = i0 + lane;
        const uint32_t v = i < n ? conn[i] : 0xffffffffu;
        const bool ok = v < nvert;
        const uint32_t grp = __match_any_sync(0xffffffffu, ok ? v : 0xffffffffu);
        const int leader = __ffs(grp) - 1;
        uint32_t base = 0;
        if (ok && (int)lane == leader) base = atomicAdd(vcount + v, (uint32_t)__popc(grp));
        base = __shfl_sync(0xffffffffu, base, leader);
        const uint32_t s = base + (uint32_t)__popc(grp & lt);
        if (ok && s < kVnMaxInc) vlist[vn_slot(s, v, nvert)] = (uint32_t)(i / 3);
    }
}

__global__ void __launch_bounds__(256) k_vn_sum(const uint32_t* __restrict__ vcount,
                                               const uint32_t* __restrict__ vlist, uint64_t nvert,
                                               const float* __restrict__ tri_normals, float* __restrict__ normals)
{
    for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nvert;
         v += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t n = min(vcount[v], kVnMaxInc);
        float sx = 0.0f, sy = 0.0f, sz = 0.0f;
        auto add = [&](uint32_t t) {
            sx = __fadd_rn(sx, tri_normals[3 * (uint64_t)t + 0]);
            sy = __fadd_rn(sy, tri_normals[3 * (uint64_t)t + 1]);
            sz = __fadd_rn(sz, tri_normals[3 * (uint64_t)t + 2]);
        };
        if (n <= 8u) {
            // the common case (four cells, a triangle or two each): a
            // 19-comparator sorting network in registers, missing entries
            // padded with the largest id
            const uint4* q = reinterpret_cast<const uint4*>(vlist + 8 * v);
            const uint4 lo = q[0], hi = n > 4u ? q[1] : make_uint4(0, 0, 0, 0);
            uint32_t d[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
#pragma unroll
            for (int i = 0; i < 8; ++i)
                if ((uint32_t)i >= n) d[i] = 0xffffffffu;
            auto cx = [&](int i, int k) {
                const uint32_t lo = min(d[i], d[k]), hi = max(d[i], d[k]);
                d[i] = lo;
                d[k] = hi;
            };
            cx(0, 1); cx(2, 3); cx(4, 5); cx(6, 7);
            cx(0, 2); cx(1, 3); cx(4, 6); cx(5, 7);
            cx(1, 2); cx(5, 6); cx(0, 4); cx(3, 7);
            cx(1, 5); cx(2, 6); cx(1, 4); cx(3, 6);
            cx(2, 4); cx(3, 5); cx(3, 4);
#pragma unroll
            for (int i = 0; i < 8; ++i)
                if ((uint32_t)i < n) add(d[i]);
        } else {
            uint32_t ids[kVnMaxInc];
            for (uint32_t i = 0; i < n; ++i) {
                // insertion sort while loading
                const uint32_t t = vlist[vn_slot(i, v, nvert)];
                uint32_t k = i;
                while (k > 0 && ids[k - 1] > t) {
                    ids[k] = ids[k - 1];
                    --k;
                }
                ids[k] = t;
            }
            for (uint32_t i = 0; i < n; ++i) add(ids[i]);
        }
        normals[3 * v + 0] = sx;
        normals[3 * v + 1] = sy;
        normals[3 * v + 2] = sz;
    }
}

// ------------------------------------------------------------ scan

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr uint64_t kScanTile = (uint64_t)kScanThreads * kScanItems;

__device__ __forceinline__ uint64_t block_exclusive_scan64(uint64_t v, uint64_t* ws, uint64_t* total)
{
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    uint64_t inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint64_t t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= (unsigned)o) inc += t;
    }
    if (lane == 31) ws[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        const uint64_t w = lane < nwarps ? ws[lane] : 0;
        uint64_t wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint64_t t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= (unsigned)o) wi += t;
        }
        if (lane < nwarps) ws[lane] = wi - w;
        if (lane == nwarps - 1) ws[32] = wi;
    }
    __syncthreads();
    const uint64_t r = ws[warp] + inc - v;
    *total = ws[32];
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const uint32_t* counts, uint64_t n, uint64_t* block_sums)
{
    __shared__ uint64_t ws[33];
    const uint64_t base = (uint64_t)blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanItems;
    uint64_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k)
        if (base + k < n) s += counts[base + k];
    uint64_t tot;
    block_exclusive_scan64(s, ws, &tot);
    if (threadIdx.x == 0) block_sums[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_top(uint64_t* block_sums, uint64_t nb, uint64_t* d_total)
{
    __shared__ uint64_t ws[33];
    uint64_t carry = 0;
    for (uint64_t base = 0; base < nb; base += blockDim.x) {
        const uint64_t i = base + threadIdx.x;
        const uint64_t v = i < nb ? block_sums[i] : 0;
        uint64_t tot;
        const uint64_t e = block_exclusive_scan64(v, ws, &tot);
        if (i < nb) block_sums[i] = carry + e;
        carry += tot;
    }
    if (threadIdx.x == 0) *d_total = carry;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_down(const uint32_t* counts, uint64_t n,
                                                           const uint64_t* block_prefix, uint64_t* offsets)
{
    __shared__ uint64_t ws[33];
    const uint64_t base = (uint64_t)blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint64_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = (base + k < n) ? counts[base + k] : 0u;
        s += v[k];
    }
    uint64_t tot;
    uint64_t e = block_exclusive_scan64(s, ws, &tot) + block_prefix[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < n) offsets[base + k] = e;
        e += v[k];
    }
}

}  // namespace

// ------------------------------------------------------------ host side

size_t dtype_size(int dtype)
{
    switch (dtype) {
    case 0: case 4: return 1;
    case 1: case 5: return 2;
    case 2: case 6: case 8: return 4;
    case 3: case 7: case 9: return 8;
    default: return 0;
    }
}

#define KVSMC_DTYPE_SWITCH(DT, ...)                          \
    switch (DT) {                                            \
    case 0: { using T = int8_t; __VA_ARGS__; } break;               \
    case 1: { using T = int16_t; __VA_ARGS__; } break;              \
    case 2: { using T = int32_t; __VA_ARGS__; } break;              \
    case 3: { using T = long long; __VA_ARGS__; } break;            \
    case 4: { using T = uint8_t; __VA_ARGS__; } break;              \
    case 5: { using T = uint16_t; __VA_ARGS__; } break;             \
    case 6: { using T = uint32_t; __VA_ARGS__; } break;             \
    case 7: { using T = unsigned long long; __VA_ARGS__; } break;   \
    case 8: { using T = float; __VA_ARGS__; } break;                \
    case 9: { using T = double; __VA_ARGS__; } break;               \
    default: return cudaErrorInvalidValue;                   \
    }

static int minmax_blocks(int num_sms) { return num_sms * 4; }

size_t minmax_scratch_bytes(int num_sms)
{
    return (size_t)minmax_blocks(num_sms) * sizeof(MinMax<double>) + 256;
}

cudaError_t launch_minmax(const VolumeView& v, void* scratch, double* d_out, const Launch& L)
{
    const int nb = minmax_blocks(L.num_sms);
    prof_begin(L, "minmax");
    KVSMC_DTYPE_SWITCH(v.dtype, {
        MinMax<T>* part = static_cast<MinMax<T>*>(scratch);
        k_minmax_partial<T><<<nb, 256, 0, L.stream>>>(v, part);
        k_minmax_final<T><<<1, 256, 0, L.stream>>>(v, part, nb, d_out);
    });
    prof_end(L);
    *L.counter += 2;
    return cudaGetLastError();
}

size_t scan_scratch_bytes(uint64_t n)
{
    const uint64_t nb = (n + kScanTile - 1) / kScanTile;
    return (size_t)(nb + 1) * sizeof(uint64_t);
}

cudaError_t launch_scan(const uint32_t* counts, uint64_t* offsets, uint64_t n, void* scratch,
                        uint64_t* d_total, const Launch& L)
{
    uint64_t nb = (n + kScanTile - 1) / kScanTile;
    if (nb == 0) nb = 1;
    uint64_t* bs = static_cast<uint64_t*>(scratch);
    prof_begin(L, "scan");
    k_scan_reduce<<<(unsigned)nb, kScanThreads, 0, L.stream>>>(counts, n, bs);
    k_scan_top<<<1, kScanThreads, 0, L.stream>>>(bs, nb, d_total);
    k_scan_down<<<(unsigned)nb, kScanThreads, 0, L.stream>>>(counts, n, bs, offsets);
    prof_end(L);
    *L.counter += 3;
    return cudaGetLastError();
}

cudaError_t launch_cell_count(const Job& j, const Launch& L)
{
    prof_begin(L, "gather_cell_count");
    KVSMC_DTYPE_SWITCH(j.vol.dtype, { k_cell_count<T><<<grid_for(j.cell_tiles, L), kThreads, 0, L.stream>>>(j); });
    prof_end(L);
    *L.counter += 1;
    return cudaGetLastError();
}

cudaError_t launch_emit_dup(const Job& j, const Launch& L)
{
    prof_begin(L, "gather_emit_dup");
    KVSMC_DTYPE_SWITCH(j.vol.dtype, { k_emit_dup<T><<<grid_for(j.cell_tiles, L), kThreads, 0, L.stream>>>(j); });
    prof_end(L);
    *L.counter += 1;
    return cudaGetLastError();
}

cudaError_t launch_node_count(const Job& j, const Launch& L)
{
    prof_begin(L, "gather_node_count");
    KVSMC_DTYPE_SWITCH(j.vol.dtype, { k_node_count<T><<<grid_for(j.node_tiles, L), kThreads, 0, L.stream>>>(j); });
    prof_end(L);
    *L.counter += 1;
    return cudaGetLastError();
}

cudaError_t launch_node_emit(const Job& j, const Launch& L)
{
    prof_begin(L, "gather_node_emit");
    KVSMC_DTYPE_SWITCH(j.vol.dtype, { k_node_emit<T><<<grid_for(j.node_tiles, L), kThreads, 0, L.stream>>>(j); });
    prof_end(L);
    *L.counter += 1;
    return cudaGetLastError();
}

cudaError_t launch_connect(const Job& j, const Launch& L)
{
    prof_begin(L, "gather_connect");
    KVSMC_DTYPE_SWITCH(j.vol.dtype, { k_connect<T><<<grid_for(j.cell_tiles, L), kThreads, 0, L.stream>>>(j); });
    prof_end(L);
    *L.counter += 1;
    return cudaGetLastError();
}

size_t vertex_normals_scratch_bytes(uint64_t ntri, uint64_t nvert)
{
    auto al = [](size_t v) { return (v + 255) / 256 * 256; };
    return al(12 * ntri) + al(4 * nvert) + al(4 * (size_t)kVnMaxInc * nvert);
}

void vertex_normals_carve(Job& j, uint64_t ntri, uint64_t nvert, void* scratch)
{
    auto al = [](size_t v) { return (v + 255) / 256 * 256; };
    char* p = static_cast<char*>(scratch);
    j.tri_normals = reinterpret_cast<float*>(p); p += al(12 * ntri);
    j.vcount = reinterpret_cast<uint32_t*>(p); p += al(4 * nvert);
    j.vlist = reinterpret_cast<uint32_t*>(p);
}

cudaError_t launch_vertex_normals(const Job& j, uint64_t ntri, uint64_t nvert, const Launch& L)
{
    const unsigned grid = (unsigned)L.num_sms * 8;
    cudaError_t e = cudaMemsetAsync(j.vcount, 0, 4 * nvert, L.stream);
    if (e != cudaSuccess) return e;
    prof_begin(L, "vn_fill");
    k_vn_fill<<<grid, 256, 0, L.stream>>>(j.connections, ntri, nvert, j.vcount, j.vlist);
    prof_end(L);
    prof_begin(L, "vn_sum");
    k_vn_sum<<<grid, 256, 0, L.stream>>>(j.vcount, j.vlist, nvert, j.tri_normals, j.normals);
    prof_end(L);
    *L.counter += 2;
    return cudaGetLastError();
}

}  // namespace kvsmc
