// cells.cu -- marching tetrahedra / hexahedra / pyramids / prisms on
// unstructured volumes, on the GPU.
//
// The reference mappers (Source/Core/Visualization/Mapper/MarchingTetrahedra.cpp,
// MarchingHexahedra.cpp, MarchingPyramid.cpp, MarchingPrism.cpp) share one
// structure, restated here once: cells in order; a cell's case has bit k set
// iff double(value of local node k) > isolevel (calculate_table_index), the
// local nodes being the cell's connections (hexahedra take connections 4-7
// then 0-3, MarchingHexahedra.cpp:105-112); pyramid cases 10, 11, 20, 21 are
// resolved by the sign of (iso - A) D + B C over the base's four values
// (calculate_special_table_index, MarchingPyramid.cpp:293-315); triangles
// come from the cell type's table in the mapper's vertex order (cell_tables.h);
// a vertex on the edge (n0, n1) is, in double, c0 + r (c1 - c0) per axis with
// r = |(iso - v0) / (v1 - v0)|, v clamped to the volume's [min, max], c1 - c0
// a float difference, then rounded to float (interpolate_vertex) -- here
// computed in FP32 double-float arithmetic with a rigorous error bound and
// taken only when no float rounding boundary lies within it (cell_axis),
// else by the FP64 sequence, so the bits are the reference's either way; one
// normal per triangle (v1 - v0) x (v2 - v0).  Duplicated vertices only (the
// reference's shared-vertex branch is not built, :164-206).
//
// Two passes over groups of 32 cells, a warp per group: count, an exclusive
// scan of the group counts, emit (a warp scan of each cell's triangle
// count); the emit pass skips the groups that counted no triangle without
// reading their cells.  A
// connection index outside the nodes sets a flag and reads node 0 instead.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "cell_tables.h"
#include "context.h"
#include "batch.h"
#include "mc_device.cuh"
#include "mc_interp.cuh"
#include "slice_common.cuh"

namespace kvsmc {

namespace {

__constant__ uint8_t c_tet_ntri[CELL_TETRA_CASES] = CELL_TETRA_NTRI_INIT;
__constant__ uint64_t c_tet_tri[CELL_TETRA_CASES] = CELL_TETRA_TRI_INIT;
__constant__ uint8_t c_tet_edge[CELL_TETRA_EDGES] = CELL_TETRA_EDGE_INIT;
__constant__ uint8_t c_hex_ntri[CELL_HEXA_CASES] = CELL_HEXA_NTRI_INIT;
__constant__ uint64_t c_hex_tri[CELL_HEXA_CASES] = CELL_HEXA_TRI_INIT;
__constant__ uint8_t c_hex_edge[CELL_HEXA_EDGES] = CELL_HEXA_EDGE_INIT;
__constant__ uint8_t c_pyr_ntri[CELL_PYRAMID_CASES] = CELL_PYRAMID_NTRI_INIT;
__constant__ uint64_t c_pyr_tri[CELL_PYRAMID_CASES] = CELL_PYRAMID_TRI_INIT;
__constant__ uint8_t c_pyr_edge[CELL_PYRAMID_EDGES] = CELL_PYRAMID_EDGE_INIT;
__constant__ uint8_t c_pri_ntri[CELL_PRISM_CASES] = CELL_PRISM_NTRI_INIT;
__constant__ uint64_t c_pri_tri[CELL_PRISM_CASES] = CELL_PRISM_TRI_INIT;
__constant__ uint8_t c_pri_edge[CELL_PRISM_EDGES] = CELL_PRISM_EDGE_INIT;

constexpr int kCellThreads = 256;
constexpr int kCountGroups = 4;    // 32-cell groups per warp step of the count pass

template <int CT> struct CellTraits;
template <> struct CellTraits<KVSMC_TETRAHEDRA> {
    static constexpr int kNodes = 4;
    __device__ static int node(int k) { return k; }
    __device__ static uint32_t ntri(unsigned c) { return c_tet_ntri[c]; }
    __device__ static uint64_t tri(unsigned c) { return c_tet_tri[c]; }
    __device__ static unsigned edge(int e) { return c_tet_edge[e]; }
};
template <> struct CellTraits<KVSMC_HEXAHEDRA> {
    static constexpr int kNodes = 8;
    __device__ static int node(int k) { return k < 4 ? k + 4 : k - 4; }   // MarchingHexahedra.cpp:105-112
    __device__ static uint32_t ntri(unsigned c) { return c_hex_ntri[c]; }
    __device__ static uint64_t tri(unsigned c) { return c_hex_tri[c]; }
    __device__ static unsigned edge(int e) { return c_hex_edge[e]; }
};
template <> struct CellTraits<KVSMC_PYRAMID> {
    static constexpr int kNodes = 5;
    __device__ static int node(int k) { return k; }
    __device__ static uint32_t ntri(unsigned c) { return c < CELL_PYRAMID_CASES ? c_pyr_ntri[c] : 0u; }
    __device__ static uint64_t tri(unsigned c) { return c < CELL_PYRAMID_CASES ? c_pyr_tri[c] : 0ull; }
    __device__ static unsigned edge(int e) { return c_pyr_edge[e]; }
};
template <> struct CellTraits<KVSMC_PRISM> {
    static constexpr int kNodes = 6;
    __device__ static int node(int k) { return k; }
    __device__ static uint32_t ntri(unsigned c) { return c_pri_ntri[c]; }
    __device__ static uint64_t tri(unsigned c) { return c_pri_tri[c]; }
    __device__ static unsigned edge(int e) { return c_pri_edge[e]; }
};

template <typename T> __device__ __forceinline__ double dval(const void* v, uint64_t i)
{
    return to_double(static_cast<const T*>(v)[i]);
}

// The cell's local node indices (checked against the node count): one or two
// 16-byte loads per cell when the connections allow it (tetrahedra,
// hexahedra on a 16-byte aligned array), else 32-bit loads.
template <int CT>
__device__ __forceinline__ void cell_nodes(const CellJob& j, uint64_t cell, uint32_t* nodes)
{
    using Tr = CellTraits<CT>;
    const uint32_t* conn = j.conn + (uint64_t)Tr::kNodes * cell;
    uint32_t raw[Tr::kNodes];
    if ((CT == KVSMC_TETRAHEDRA || CT == KVSMC_HEXAHEDRA) && j.conn_vec16) {
#pragma unroll
        for (int q = 0; q < Tr::kNodes / 4; ++q) {
            const uint4 w = __ldg(reinterpret_cast<const uint4*>(conn) + q);
            raw[4 * q] = w.x; raw[4 * q + 1] = w.y; raw[4 * q + 2] = w.z; raw[4 * q + 3] = w.w;
        }
    } else {
#pragma unroll
        for (int k = 0; k < Tr::kNodes; ++k) raw[k] = __ldg(conn + k);
    }
#pragma unroll
    for (int k = 0; k < Tr::kNodes; ++k) {
        uint32_t n = raw[Tr::node(k)];
        if (n >= j.nnodes) {
            atomicExch(j.bad_index, 1);
            n = 0;
        }
        nodes[k] = n;
    }
}

// The case: bit k iff double(value of local node k) > isolevel, decided
// without FP64 for float and up-to-32-bit integer values (Classifier).
template <int CT, typename T>
__device__ __forceinline__ unsigned case_of(const Classifier& cls, double iso, const T* v)
{
    using Tr = CellTraits<CT>;
    unsigned c = 0;
#pragma unroll
    for (int k = 0; k < Tr::kNodes; ++k) c |= above(cls, v[k]) ? (1u << k) : 0u;
    if (CT == KVSMC_PYRAMID && (c == 10u || c == 11u || c == 20u || c == 21u)) {
        // x / 4 as x * 0.25: the same correctly rounded result
        const double v1 = to_double(v[1]), v2 = to_double(v[2]);
        const double v3 = to_double(v[3]), v4 = to_double(v[4]);
        const double A = __dmul_rn(__dadd_rn(__dadd_rn(__dadd_rn(v1, v2), v3), v4), 0.25);
        const double B = __dmul_rn(__dsub_rn(__dadd_rn(__dadd_rn(-v1, v2), v3), v4), 0.25);
        const double C = __dmul_rn(__dadd_rn(__dadd_rn(__dsub_rn(-v1, v2), v3), v4), 0.25);
        const double D = __dmul_rn(__dsub_rn(__dadd_rn(__dsub_rn(v1, v2), v3), v4), 0.25);
        const double E = __dadd_rn(__dmul_rn(__dsub_rn(iso, A), D), __dmul_rn(B, C));
        if (c == 10u && E < 0) c = 32u;
        else if (c == 11u && E >= 0) c = 33u;
        else if (c == 20u && E >= 0) c = 34u;
        else if (c == 21u && E < 0) c = 35u;
    }
    return c;
}

// The cell's nodes and their values.
template <int CT, typename T>
__device__ __forceinline__ void cell_load(const CellJob& j, uint64_t cell, uint32_t* nodes, T* v)
{
    using Tr = CellTraits<CT>;
    cell_nodes<CT>(j, cell, nodes);
    const T* vals = static_cast<const T*>(j.values);
#pragma unroll
    for (int k = 0; k < Tr::kNodes; ++k) v[k] = __ldg(vals + nodes[k]);
}

template <int CT, typename T>
__device__ __forceinline__ unsigned cell_case(const CellJob& j, uint64_t cell, uint32_t* nodes)
{
    T v[CellTraits<CT>::kNodes];
    cell_load<CT, T>(j, cell, nodes, v);
    return case_of<CT, T>(j.cls, j.iso, v);
}

// The reference's FP64 sequence, out of line (it runs for the vertices the
// FP32 certificate cannot decide, and for 32/64-bit integer and double values).
template <typename T>
static __device__ __noinline__ float3 cell_vertex_exact(const CellJob& j, double iso, uint32_t n0, uint32_t n1)
{
    const double lo = j.vmin, hi = j.vmax;
    double v0 = dval<T>(j.values, n0), v1 = dval<T>(j.values, n1);
    v0 = v0 <= lo ? lo : (v0 <= hi ? v0 : hi);   // Math::Clamp
    v1 = v1 <= lo ? lo : (v1 <= hi ? v1 : hi);
    const double q = __ddiv_rn(__dsub_rn(iso, v0), __dsub_rn(v1, v0));
    const double r = q < 0.0 ? -q : q;
    const float* c0 = j.coords + 3 * (uint64_t)n0;
    const float* c1 = j.coords + 3 * (uint64_t)n1;
    float3 o;
    o.x = __double2float_rn(__dadd_rn((double)c0[0], __dmul_rn(r, (double)__fsub_rn(c1[0], c0[0]))));
    o.y = __double2float_rn(__dadd_rn((double)c0[1], __dmul_rn(r, (double)__fsub_rn(c1[1], c0[1]))));
    o.z = __double2float_rn(__dadd_rn((double)c0[2], __dmul_rn(r, (double)__fsub_rn(c1[2], c0[2]))));
    return o;
}

// Value types whose values are floats exactly (the FP32 certificate applies).
template <typename T> struct CellFast { static constexpr bool value = false; };
template <> struct CellFast<float> { static constexpr bool value = true; };
template <> struct CellFast<int8_t> { static constexpr bool value = true; };
template <> struct CellFast<int16_t> { static constexpr bool value = true; };
template <> struct CellFast<uint8_t> { static constexpr bool value = true; };
template <> struct CellFast<uint16_t> { static constexpr bool value = true; };

// interpolate_vertex: the FP32 certificate (cell_ratio / cell_axis), else FP64.
template <typename T>
__device__ __forceinline__ float3 cell_vertex(const CellJob& j, const FastIso& f, double iso, uint32_t n0, uint32_t n1)
{
    if constexpr (CellFast<T>::value) {
        const T* vals = static_cast<const T*>(j.values);
        const float v0 = clampf_ref((float)__ldg(vals + n0), f.vmin_f, f.vmax_f);
        const float v1 = clampf_ref((float)__ldg(vals + n1), f.vmin_f, f.vmax_f);
        const CellRatio c = cell_ratio(v0, v1, f);
        const float* c0 = j.coords + 3 * (uint64_t)n0;
        const float* c1 = j.coords + 3 * (uint64_t)n1;
        float3 o;
        const bool ox = cell_axis(c, __ldg(c0), __ldg(c1), o.x);
        const bool oy = cell_axis(c, __ldg(c0 + 1), __ldg(c1 + 1), o.y);
        const bool oz = cell_axis(c, __ldg(c0 + 2), __ldg(c1 + 2), o.z);
        if (ox && oy && oz) return o;
    }
    return cell_vertex_exact<T>(j, iso, n0, n1);
}

// Both passes work on groups of 32 consecutive cells, one warp per group
// (grid-stride over groups): the count pass writes each group's triangle
// count, the emit pass skips the groups that counted none without reading
// their cells and places the others' triangles by a warp scan.
template <int CT, typename T>
__global__ void __launch_bounds__(kCellThreads) k_cells_count(CellJob j)
{
    using Tr = CellTraits<CT>;
    const unsigned lane = threadIdx.x & 31u;
    const uint64_t warps = (uint64_t)gridDim.x * (kCellThreads / 32);
    const uint64_t groups = (j.ncells + 31) / 32;
    // kCountGroups groups per step (their loads in flight together)
    constexpr int G = kCountGroups;
    for (uint64_t g = ((uint64_t)blockIdx.x * (kCellThreads / 32) + (threadIdx.x >> 5)) * G; g < groups;
         g += warps * G) {
        uint32_t n[G];
#pragma unroll
        for (int q = 0; q < G; ++q) {
            const uint64_t c = (g + q) * 32 + lane;
            uint32_t nodes[Tr::kNodes];
            n[q] = c < j.ncells ? Tr::ntri(cell_case<CT, T>(j, c, nodes)) : 0u;
        }
#pragma unroll
        for (int q = 0; q < G; ++q) {
            const uint32_t t = __reduce_add_sync(0xffffffffu, n[q]);
            if (lane == 0 && g + q < groups) j.tile_counts[g + q] = t;
        }
    }
}

template <int CT, typename T>
__global__ void __launch_bounds__(kCellThreads) k_cells_emit(CellJob j)
{
    using Tr = CellTraits<CT>;
    // launched before the host knows the total: nothing is written unless all fits
    if (j.d_total && *j.d_total > j.cap_tris) return;
    const unsigned lane = threadIdx.x & 31u;
    const uint64_t warps = (uint64_t)gridDim.x * (kCellThreads / 32);
    const uint64_t groups = (j.ncells + 31) / 32;
    // a warp takes 32 groups at a time: one coalesced read of their counts,
    // then only the groups with triangles (ballot)
    for (uint64_t g0 = ((uint64_t)blockIdx.x * (kCellThreads / 32) + (threadIdx.x >> 5)) * 32; g0 < groups;
         g0 += warps * 32) {
        const uint64_t mine = g0 + lane;
        unsigned todo = __ballot_sync(0xffffffffu, mine < groups && j.tile_counts[mine] != 0);
        while (todo) {
        const uint64_t g = g0 + (unsigned)(__ffs(todo) - 1);
        todo &= todo - 1;
        const uint64_t cell = g * 32 + lane;
        uint32_t nodes[Tr::kNodes] = {};
        unsigned c = 0;
        uint32_t n = 0;
        if (cell < j.ncells) {
            c = cell_case<CT, T>(j, cell, nodes);
            n = Tr::ntri(c);
        }
        uint32_t inc = n;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= (unsigned)o) inc += y;
        }
        // the group's triangles spread over the lanes: lane l builds triangles
        // l, l + 32, ... of the group; its cell is the first lane whose
        // inclusive count exceeds the index (a 5-step search over shuffles)
        const uint32_t total = __shfl_sync(0xffffffffu, inc, 31);
        const uint64_t base = j.tile_offsets[g];
        for (uint32_t first = 0; first < total; first += 32) {   // warp-uniform: every lane shuffles
            const uint32_t tri = first + lane;
            unsigned lo = 0;
#pragma unroll
            for (unsigned step = 16; step > 0; step >>= 1) {
                const uint32_t probe = __shfl_sync(0xffffffffu, inc, lo + step - 1);
                if (probe <= tri) lo += step;
            }
            // lo: the owning lane (inc[lo] > tri, inc[lo - 1] <= tri)
            const uint32_t own_inc = __shfl_sync(0xffffffffu, inc, lo);
            const uint32_t own_n = __shfl_sync(0xffffffffu, n, lo);
            const unsigned own_c = __shfl_sync(0xffffffffu, c, lo);
            uint32_t own_nodes[Tr::kNodes];
#pragma unroll
            for (int k = 0; k < Tr::kNodes; ++k) own_nodes[k] = __shfl_sync(0xffffffffu, nodes[k], lo);
            const uint64_t t = base + tri;
            if (tri >= total || t >= j.cap_tris) continue;   // never past the group or the outputs
            const uint32_t k = tri - (own_inc - own_n);
            const uint64_t pk = Tr::tri(own_c) >> (12 * k);
            float3 v[3];
#pragma unroll
            for (int s = 0; s < 3; ++s) {
                const unsigned ed = Tr::edge((int)((pk >> (4 * s)) & 15u));
                v[s] = cell_vertex<T>(j, j.f, j.iso, own_nodes[ed & 15u], own_nodes[ed >> 4]);
            }
            float* o = j.out_coords + 9 * t;
            o[0] = v[0].x; o[1] = v[0].y; o[2] = v[0].z;
            o[3] = v[1].x; o[4] = v[1].y; o[5] = v[1].z;
            o[6] = v[2].x; o[7] = v[2].y; o[8] = v[2].z;
            const float3 nn = tri_normal(v[0], v[1], v[2]);
            float* q = j.out_normals + 3 * t;
            q[0] = nn.x; q[1] = nn.y; q[2] = nn.z;
        }
        }
    }
}

// ---- kvs::SlicePlane on unstructured volumes (SlicePlane.cpp:291-800):
// per cell type, a case from the plane's sign at the cell's node coordinates
// (calculate_*_table_index, :828-942; no pyramid re-mapping), the cell type's
// triangle table in table order [i], [i+1], [i+2] for all four types, each
// vertex (1 - r) v0 + r v1 with r = |p0 / (p1 - p0)| in float on the node
// coordinates (interpolate_vertex, :986-995, no coordinate transform), its
// colour ColorMap::at of the value interpolated with the same r in the value
// type's arithmetic (interpolate_value, :1043-1056), one normal
// -((v2 - v0) x (v1 - v0)).

template <int CT>
__device__ __forceinline__ float3 node_xyz(const CellJob& j, uint32_t n)
{
    const float* c = j.coords + 3 * (uint64_t)n;
    return make_float3(__ldg(c), __ldg(c + 1), __ldg(c + 2));
}

template <int CT>
__device__ __forceinline__ unsigned slice_cell_case(const CellJob& j, uint64_t cell, uint32_t* nodes)
{
    using Tr = CellTraits<CT>;
    cell_nodes<CT>(j, cell, nodes);
    unsigned c = 0;
#pragma unroll
    for (int k = 0; k < Tr::kNodes; ++k) {
        const float3 p = node_xyz<CT>(j, nodes[k]);
        c |= plane_at(j, p.x, p.y, p.z) > 0.0f ? (1u << k) : 0u;
    }
    return c;
}

template <int CT, typename T>
__global__ void __launch_bounds__(kCellThreads) k_cells_slice_count(CellJob j)
{
    using Tr = CellTraits<CT>;
    const unsigned lane = threadIdx.x & 31u;
    const uint64_t warps = (uint64_t)gridDim.x * (kCellThreads / 32);
    const uint64_t groups = (j.ncells + 31) / 32;
    for (uint64_t g = (uint64_t)blockIdx.x * (kCellThreads / 32) + (threadIdx.x >> 5); g < groups; g += warps) {
        const uint64_t cell = g * 32 + lane;
        uint32_t n = 0;
        if (cell < j.ncells) {
            uint32_t nodes[Tr::kNodes];
            n = Tr::ntri(slice_cell_case<CT>(j, cell, nodes));
        }
        const uint32_t t = __reduce_add_sync(0xffffffffu, n);
        if (lane == 0) j.tile_counts[g] = t;
    }
}

template <typename T>
__device__ __forceinline__ void slice_cell_vertex(const CellJob& j, uint32_t n0, uint32_t n1, float3& v, uchar3& rgb)
{
    const float3 a = node_xyz<0>(j, n0), b = node_xyz<0>(j, n1);
    const float p0 = plane_at(j, a.x, a.y, a.z), p1 = plane_at(j, b.x, b.y, b.z);
    const float r = fabsf(__fdiv_rn(p0, __fsub_rn(p1, p0)));
    const float s = __fsub_rn(1.0f, r);
    v.x = __fadd_rn(__fmul_rn(s, a.x), __fmul_rn(r, b.x));
    v.y = __fadd_rn(__fmul_rn(s, a.y), __fmul_rn(r, b.y));
    v.z = __fadd_rn(__fmul_rn(s, a.z), __fmul_rn(r, b.z));
    const T* vals = static_cast<const T*>(j.values);
    rgb = color_at(j, slice_value(vals[n0], vals[n1], r));
}

template <int CT, typename T>
__global__ void __launch_bounds__(kCellThreads) k_cells_slice_emit(CellJob j)
{
    using Tr = CellTraits<CT>;
    // hexahedra and pyramids are packed in the mappers' [i], [i+2], [i+1]
    // order; the slicer takes [i], [i+1], [i+2]
    constexpr bool kSwapped = CT == KVSMC_HEXAHEDRA || CT == KVSMC_PYRAMID;
    if (j.d_total && *j.d_total > j.cap_tris) return;
    const unsigned lane = threadIdx.x & 31u;
    const uint64_t warps = (uint64_t)gridDim.x * (kCellThreads / 32);
    const uint64_t groups = (j.ncells + 31) / 32;
    for (uint64_t g0 = ((uint64_t)blockIdx.x * (kCellThreads / 32) + (threadIdx.x >> 5)) * 32; g0 < groups;
         g0 += warps * 32) {
        const uint64_t mine = g0 + lane;
        unsigned todo = __ballot_sync(0xffffffffu, mine < groups && j.tile_counts[mine] != 0);
        while (todo) {
            const uint64_t g = g0 + (unsigned)(__ffs(todo) - 1);
            todo &= todo - 1;
            const uint64_t cell = g * 32 + lane;
            uint32_t nodes[Tr::kNodes] = {};
            unsigned c = 0;
            uint32_t n = 0;
            if (cell < j.ncells) {
                c = slice_cell_case<CT>(j, cell, nodes);
                n = Tr::ntri(c);
            }
            uint32_t inc = n;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= (unsigned)o) inc += y;
            }
            const uint32_t total = __shfl_sync(0xffffffffu, inc, 31);
            const uint64_t base = j.tile_offsets[g];
            for (uint32_t first = 0; first < total; first += 32) {   // warp-uniform: every lane shuffles
                const uint32_t tri = first + lane;
                unsigned lo = 0;
#pragma unroll
                for (unsigned step = 16; step > 0; step >>= 1) {
                    const uint32_t probe = __shfl_sync(0xffffffffu, inc, lo + step - 1);
                    if (probe <= tri) lo += step;
                }
                const uint32_t own_inc = __shfl_sync(0xffffffffu, inc, lo);
                const uint32_t own_n = __shfl_sync(0xffffffffu, n, lo);
                const unsigned own_c = __shfl_sync(0xffffffffu, c, lo);
                uint32_t own_nodes[Tr::kNodes];
#pragma unroll
                for (int k = 0; k < Tr::kNodes; ++k) own_nodes[k] = __shfl_sync(0xffffffffu, nodes[k], lo);
                const uint64_t t = base + tri;
                if (tri >= total || t >= j.cap_tris) continue;
                const uint32_t k = tri - (own_inc - own_n);
                const uint64_t pk = Tr::tri(own_c) >> (12 * k);
                float3 v[3];
                uchar3 rgb[3];
#pragma unroll
                for (int sl = 0; sl < 3; ++sl) {
                    const int src = kSwapped ? (sl == 0 ? 0 : 3 - sl) : sl;
                    const unsigned ed = Tr::edge((int)((pk >> (4 * src)) & 15u));
                    slice_cell_vertex<T>(j, own_nodes[ed & 15u], own_nodes[ed >> 4], v[sl], rgb[sl]);
                }
                float* o = j.out_coords + 9 * t;
                o[0] = v[0].x; o[1] = v[0].y; o[2] = v[0].z;
                o[3] = v[1].x; o[4] = v[1].y; o[5] = v[1].z;
                o[6] = v[2].x; o[7] = v[2].y; o[8] = v[2].z;
                uint8_t* q = j.out_colors + 9 * t;
                q[0] = rgb[0].x; q[1] = rgb[0].y; q[2] = rgb[0].z;
                q[3] = rgb[1].x; q[4] = rgb[1].y; q[5] = rgb[1].z;
                q[6] = rgb[2].x; q[7] = rgb[2].y; q[8] = rgb[2].z;
                const float3 nn = slice_normal(v[0], v[1], v[2]);
                float* w = j.out_normals + 3 * t;
                w[0] = nn.x; w[1] = nn.y; w[2] = nn.z;
            }
        }
    }
}

// ---- min/max over the cells' nodes (GetMinMaxValues with connections,
// UnstructuredVolumeObject.cpp:123-143): the scan starts at values[0] and
// then visits values[conn[p]] for every connection p in order; Min/Max keep
// the earlier value on ties and never take a NaN (a NaN values[0] stays).
template <typename T> struct CellMinMax {
    T lo, hi;
    unsigned long long ilo, ihi;   // scan positions (values[0] is position 0)
    int any;
};

template <typename T> __device__ __forceinline__ void cmm_combine(CellMinMax<T>& a, const CellMinMax<T>& b)
{
    if (!b.any) return;
    if (!a.any) { a = b; return; }
    if (b.lo < a.lo || (b.lo == a.lo && b.ilo < a.ilo)) { a.lo = b.lo; a.ilo = b.ilo; }
    if (b.hi > a.hi || (b.hi == a.hi && b.ihi < a.ihi)) { a.hi = b.hi; a.ihi = b.ihi; }
}

template <typename T> __device__ void cmm_block(CellMinMax<T>& m, CellMinMax<T>* sm)
{
    sm[threadIdx.x] = m;
    __syncthreads();
    for (unsigned s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            CellMinMax<T> a = sm[threadIdx.x];
            cmm_combine(a, sm[threadIdx.x + s]);
            sm[threadIdx.x] = a;
        }
        __syncthreads();
    }
    m = sm[0];
}

template <typename T>
__global__ void __launch_bounds__(kCellThreads) k_cells_minmax_partial(CellJob j, uint64_t nconn, CellMinMax<T>* partial)
{
    __shared__ CellMinMax<T> sm[kCellThreads];
    const T* vals = static_cast<const T*>(j.values);
    CellMinMax<T> m;
    m.any = 0; m.lo = T(0); m.hi = T(0); m.ilo = m.ihi = 0;
    const uint64_t per = (nconn + gridDim.x - 1) / gridDim.x;
    const uint64_t p0 = (uint64_t)blockIdx.x * per, p1 = p0 + per < nconn ? p0 + per : nconn;
    for (uint64_t p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
        const uint32_t n = j.conn[p];
        if (n >= j.nnodes) { atomicExch(j.bad_index, 1); continue; }
        const T v = vals[n];
        if (v != v) continue;
        const unsigned long long pos = p + 1;
        if (!m.any) { m.lo = m.hi = v; m.ilo = m.ihi = pos; m.any = 1; continue; }
        if (v < m.lo) { m.lo = v; m.ilo = pos; }
        if (v > m.hi) { m.hi = v; m.ihi = pos; }
    }
    cmm_block(m, sm);
    if (threadIdx.x == 0) partial[blockIdx.x] = m;
}

template <typename T>
__global__ void __launch_bounds__(kCellThreads) k_cells_minmax_final(CellJob j, const CellMinMax<T>* partial, int n, double* out)
{
    __shared__ CellMinMax<T> sm[kCellThreads];
    CellMinMax<T> m;
    m.any = 0; m.lo = T(0); m.hi = T(0); m.ilo = m.ihi = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) cmm_combine(m, partial[i]);
    cmm_block(m, sm);
    if (threadIdx.x == 0) {
        const T first = static_cast<const T*>(j.values)[0];
        if (first != first) {
            out[0] = out[1] = to_double(first);
            return;
        }
        CellMinMax<T> f;
        f.lo = f.hi = first; f.ilo = f.ihi = 0; f.any = 1;
        cmm_combine(f, m);
        out[0] = to_double(f.lo);
        out[1] = to_double(f.hi);
    }
}

// ---- bounding box (UnstructuredVolumeObject::updateMinMaxCoords,
// UnstructuredVolumeObject.cpp:396-466): per axis the fold
// Min(cur, x) = cur < x ? cur : x (Max alike) over the sequence
// [conn[0], conn[0], conn[1], ...] of node coordinates (the nodes in order
// when there are no connections), from its first element.  A NaN x is
// taken and the next element replaces it, ties keep the later element.  So
// the result is NaN when the last element is NaN, else the min (max) over
// the elements after the last NaN, the latest on ties (the sign of a zero).

__device__ __forceinline__ uint64_t bounds_node(const CellJob& j, uint64_t p, bool has_conn)
{
    return has_conn ? (p == 0 ? j.conn[0] : j.conn[p - 1]) : p;
}

__global__ void __launch_bounds__(kCellThreads) k_bounds_last_nan(CellJob j, uint64_t npos, int has_conn,
                                                                  unsigned long long* last_nan)
{
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < npos;
         p += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t n = bounds_node(j, p, has_conn != 0);
        if (n >= j.nnodes) { atomicExch(j.bad_index, 1); continue; }
        const float* c = j.coords + 3 * n;
#pragma unroll
        for (int ax = 0; ax < 3; ++ax)
            if (isnan(c[ax])) atomicMax(&last_nan[ax], (unsigned long long)(p + 1));
    }
}

struct BoundPart {
    float mn[3], mx[3];
    unsigned long long pmn[3], pmx[3];   // position + 1 (0: none)
};

__device__ __forceinline__ void bound_take(float& v, unsigned long long& pv, float w, unsigned long long pw, bool less)
{
    if (pw == 0) return;
    if (pv == 0 || (less ? w < v : w > v) || (w == v && pw > pv)) { v = w; pv = pw; }
}

__global__ void __launch_bounds__(kCellThreads) k_bounds_partial(CellJob j, uint64_t npos, int has_conn,
                                                                 const unsigned long long* last_nan, BoundPart* parts)
{
    __shared__ BoundPart sm[kCellThreads];
    BoundPart b;
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) { b.mn[ax] = b.mx[ax] = 0.0f; b.pmn[ax] = b.pmx[ax] = 0; }
    const uint64_t per = (npos + gridDim.x - 1) / gridDim.x;
    const uint64_t p0 = (uint64_t)blockIdx.x * per, p1 = p0 + per < npos ? p0 + per : npos;
    for (uint64_t p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
        const uint64_t n = bounds_node(j, p, has_conn != 0);
        if (n >= j.nnodes) continue;
        const float* c = j.coords + 3 * n;
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            if (p + 1 <= last_nan[ax]) continue;   // at or before the last NaN
            bound_take(b.mn[ax], b.pmn[ax], c[ax], p + 1, true);
            bound_take(b.mx[ax], b.pmx[ax], c[ax], p + 1, false);
        }
    }
    sm[threadIdx.x] = b;
    __syncthreads();
    for (unsigned st = blockDim.x / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st) {
            BoundPart a = sm[threadIdx.x];
            const BoundPart& o = sm[threadIdx.x + st];
#pragma unroll
            for (int ax = 0; ax < 3; ++ax) {
                bound_take(a.mn[ax], a.pmn[ax], o.mn[ax], o.pmn[ax], true);
                bound_take(a.mx[ax], a.pmx[ax], o.mx[ax], o.pmx[ax], false);
            }
            sm[threadIdx.x] = a;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) parts[blockIdx.x] = sm[0];
}

__global__ void __launch_bounds__(kCellThreads) k_bounds_final(CellJob j, uint64_t npos, int has_conn,
                                                               const unsigned long long* last_nan,
                                                               const BoundPart* parts, int nparts, float* out)
{
    __shared__ BoundPart sm[kCellThreads];
    BoundPart b;
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) { b.mn[ax] = b.mx[ax] = 0.0f; b.pmn[ax] = b.pmx[ax] = 0; }
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) {
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            bound_take(b.mn[ax], b.pmn[ax], parts[i].mn[ax], parts[i].pmn[ax], true);
            bound_take(b.mx[ax], b.pmx[ax], parts[i].mx[ax], parts[i].pmx[ax], false);
        }
    }
    sm[threadIdx.x] = b;
    __syncthreads();
    for (unsigned st = blockDim.x / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st) {
            BoundPart a = sm[threadIdx.x];
            const BoundPart& o = sm[threadIdx.x + st];
#pragma unroll
            for (int ax = 0; ax < 3; ++ax) {
                bound_take(a.mn[ax], a.pmn[ax], o.mn[ax], o.pmn[ax], true);
                bound_take(a.mx[ax], a.pmx[ax], o.mx[ax], o.pmx[ax], false);
            }
            sm[threadIdx.x] = a;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const uint64_t last = bounds_node(j, npos - 1, has_conn != 0);
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            if (last_nan[ax] == npos && last < j.nnodes) {
                // the last element is a NaN: the fold ends on it
                out[ax] = out[3 + ax] = j.coords[3 * last + ax];
            } else {
                out[ax] = sm[0].mn[ax];
                out[3 + ax] = sm[0].mx[ax];
            }
        }
    }
}

// ---- isolevel sweep: one count pass classifies every cell for all the
// isolevels (its connections and node values read once), one scan over the
// isolevels' group counts, one emit pass over (isolevel, 32 groups) items.

template <int CT, typename T>
__global__ void __launch_bounds__(kCellThreads) k_cells_sweep_count(CellJob j)
{
    using Tr = CellTraits<CT>;
    __shared__ CellIso s_iso[kCellSweepMax];
    for (int i = threadIdx.x; i < j.niso; i += blockDim.x) s_iso[i] = j.isos[i];
    __syncthreads();
    const unsigned lane = threadIdx.x & 31u;
    const uint64_t warps = (uint64_t)gridDim.x * (kCellThreads / 32);
    const uint64_t groups = (j.ncells + 31) / 32;
    for (uint64_t g = (uint64_t)blockIdx.x * (kCellThreads / 32) + (threadIdx.x >> 5); g < groups; g += warps) {
        const uint64_t cell = g * 32 + lane;
        const bool ok = cell < j.ncells;
        uint32_t nodes[Tr::kNodes];
        T v[Tr::kNodes];
        if (ok) cell_load<CT, T>(j, cell, nodes, v);
        for (int k = 0; k < j.niso; ++k) {
            const uint32_t n = ok ? Tr::ntri(case_of<CT, T>(s_iso[k].cls, s_iso[k].iso, v)) : 0u;
            const uint32_t t = __reduce_add_sync(0xffffffffu, n);
            if (lane == 0) j.tile_counts[(uint64_t)k * groups + g] = t;
        }
    }
}

template <int CT, typename T>
__global__ void __launch_bounds__(kCellThreads) k_cells_sweep_emit(CellJob j)
{
    using Tr = CellTraits<CT>;
    __shared__ CellIso s_iso[kCellSweepMax];
    for (int i = threadIdx.x; i < j.niso; i += blockDim.x) s_iso[i] = j.isos[i];
    __syncthreads();
    const unsigned lane = threadIdx.x & 31u;
    const uint64_t warps = (uint64_t)gridDim.x * (kCellThreads / 32);
    const uint64_t groups = (j.ncells + 31) / 32;
    const uint64_t nchunks = (groups + 31) / 32;
    const uint64_t items = nchunks * (uint64_t)j.niso;
    for (uint64_t it = (uint64_t)blockIdx.x * (kCellThreads / 32) + (threadIdx.x >> 5); it < items; it += warps) {
        const int k = (int)(it / nchunks);
        const uint64_t g0 = (it - (uint64_t)k * nchunks) * 32;
        const CellIso& I = s_iso[k];
        const uint32_t* counts = j.tile_counts + (uint64_t)k * groups;
        const uint64_t* offsets = j.tile_offsets + (uint64_t)k * groups;
        const uint64_t mine = g0 + lane;
        unsigned todo = __ballot_sync(0xffffffffu, mine < groups && counts[mine] != 0);
        while (todo) {
            const uint64_t g = g0 + (unsigned)(__ffs(todo) - 1);
            todo &= todo - 1;
            const uint64_t cell = g * 32 + lane;
            uint32_t nodes[Tr::kNodes] = {};
            unsigned c = 0;
            uint32_t n = 0;
            if (cell < j.ncells) {
                T v[Tr::kNodes];
                cell_load<CT, T>(j, cell, nodes, v);
                c = case_of<CT, T>(I.cls, I.iso, v);
                n = Tr::ntri(c);
            }
            uint32_t inc = n;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= (unsigned)o) inc += y;
            }
            const uint32_t total = __shfl_sync(0xffffffffu, inc, 31);
            const uint64_t base = offsets[g] - I.base;
            for (uint32_t first = 0; first < total; first += 32) {   // warp-uniform: every lane shuffles
                const uint32_t tri = first + lane;
                unsigned lo = 0;
#pragma unroll
                for (unsigned step = 16; step > 0; step >>= 1) {
                    const uint32_t probe = __shfl_sync(0xffffffffu, inc, lo + step - 1);
                    if (probe <= tri) lo += step;
                }
                const uint32_t own_inc = __shfl_sync(0xffffffffu, inc, lo);
                const uint32_t own_n = __shfl_sync(0xffffffffu, n, lo);
                const unsigned own_c = __shfl_sync(0xffffffffu, c, lo);
                uint32_t own_nodes[Tr::kNodes];
#pragma unroll
                for (int q = 0; q < Tr::kNodes; ++q) own_nodes[q] = __shfl_sync(0xffffffffu, nodes[q], lo);
                const uint64_t t = base + tri;
                if (tri >= total || t >= I.cap_tris) continue;
                const uint32_t kk = tri - (own_inc - own_n);
                const uint64_t pk = Tr::tri(own_c) >> (12 * kk);
                float3 vx[3];
#pragma unroll
                for (int sl = 0; sl < 3; ++sl) {
                    const unsigned ed = Tr::edge((int)((pk >> (4 * sl)) & 15u));
                    vx[sl] = cell_vertex<T>(j, I.f, I.iso, own_nodes[ed & 15u], own_nodes[ed >> 4]);
                }
                float* o = I.out_coords + 9 * t;
                o[0] = vx[0].x; o[1] = vx[0].y; o[2] = vx[0].z;
                o[3] = vx[1].x; o[4] = vx[1].y; o[5] = vx[1].z;
                o[6] = vx[2].x; o[7] = vx[2].y; o[8] = vx[2].z;
                const float3 nn = tri_normal(vx[0], vx[1], vx[2]);
                float* q = I.out_normals + 3 * t;
                q[0] = nn.x; q[1] = nn.y; q[2] = nn.z;
            }
        }
    }
}

// base[k] = the first scanned offset of isolevel k, base[niso] = the total.
__global__ void k_sweep_bases(const uint64_t* offsets, uint64_t groups, int niso, const uint64_t* total, uint64_t* out)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        for (int k = 0; k < niso; ++k) out[k] = groups ? offsets[(uint64_t)k * groups] : 0;
        out[niso] = *total;
    }
}

// Blocks of 8 warps, one warp per 32-cell group, at most 8 blocks per SM.
unsigned cell_grid(uint64_t groups, const Launch& L)
{
    const uint64_t blocks = (groups + kCellThreads / 32 - 1) / (kCellThreads / 32);
    const uint64_t cap = (uint64_t)L.num_sms * 8;
    return (unsigned)(blocks < cap ? (blocks ? blocks : 1) : cap);
}

#define KVSMC_CELL_SWITCH(CTV, DT, ...)                                                     \
    switch (CTV) {                                                                          \
    case KVSMC_TETRAHEDRA: { constexpr int CT = KVSMC_TETRAHEDRA; KVSMC_VALUE_SWITCH(DT, __VA_ARGS__); } break; \
    case KVSMC_HEXAHEDRA: { constexpr int CT = KVSMC_HEXAHEDRA; KVSMC_VALUE_SWITCH(DT, __VA_ARGS__); } break;   \
    case KVSMC_PYRAMID: { constexpr int CT = KVSMC_PYRAMID; KVSMC_VALUE_SWITCH(DT, __VA_ARGS__); } break;       \
    case KVSMC_PRISM: { constexpr int CT = KVSMC_PRISM; KVSMC_VALUE_SWITCH(DT, __VA_ARGS__); } break;           \
    default: return cudaErrorInvalidValue;                                                  \
    }

#define KVSMC_VALUE_SWITCH(DT, ...)                                 \
    switch (DT) {                                                   \
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
    default: return cudaErrorInvalidValue;                          \
    }

}  // namespace

cudaError_t launch_cells_count(const CellJob& j, const Launch& L)
{
    if (j.ncells == 0) return cudaSuccess;
    const uint64_t tiles = cells_tiles(j.ncells);
    prof_begin(L, "cells_count");
    KVSMC_CELL_SWITCH(j.cell_type, j.dtype,
                      { k_cells_count<CT, T><<<cell_grid(tiles, L), kCellThreads, 0, L.stream>>>(j); });
    prof_end(L);
    *L.counter += 1;
    return cudaGetLastError();
}

cudaError_t launch_cells_emit(const CellJob& j, const Launch& L)
{
    if (j.ncells == 0) return cudaSuccess;
    const uint64_t tiles = cells_tiles(j.ncells);
    prof_begin(L, "cells_emit");
    KVSMC_CELL_SWITCH(j.cell_type, j.dtype,
                      { k_cells_emit<CT, T><<<cell_grid(tiles, L), kCellThreads, 0, L.stream>>>(j); });
    prof_end(L);
    *L.counter += 1;
    return cudaGetLastError();
}


cudaError_t launch_cells_slice_count(const CellJob& j, const Launch& L)
{
    if (j.ncells == 0) return cudaSuccess;
    const uint64_t tiles = cells_tiles(j.ncells);
    prof_begin(L, "cells_slice_count");
    KVSMC_CELL_SWITCH(j.cell_type, j.dtype,
                      { k_cells_slice_count<CT, T><<<cell_grid(tiles, L), kCellThreads, 0, L.stream>>>(j); });
    prof_end(L);
    *L.counter += 1;
    return cudaGetLastError();
}

cudaError_t launch_cells_slice_emit(const CellJob& j, const Launch& L)
{
    if (j.ncells == 0) return cudaSuccess;
    const uint64_t tiles = cells_tiles(j.ncells);
    prof_begin(L, "cells_slice_emit");
    KVSMC_CELL_SWITCH(j.cell_type, j.dtype,
                      { k_cells_slice_emit<CT, T><<<cell_grid(tiles, L), kCellThreads, 0, L.stream>>>(j); });
    prof_end(L);
    *L.counter += 1;
    return cudaGetLastError();
}

cudaError_t launch_cells_sweep_count(const CellJob& j, const Launch& L)
{
    if (j.ncells == 0 || j.niso <= 0) return cudaSuccess;
    const uint64_t tiles = cells_tiles(j.ncells);
    prof_begin(L, "cells_sweep_count");
    KVSMC_CELL_SWITCH(j.cell_type, j.dtype,
                      { k_cells_sweep_count<CT, T><<<cell_grid(tiles, L), kCellThreads, 0, L.stream>>>(j); });
    prof_end(L);
    *L.counter += 1;
    return cudaGetLastError();
}

cudaError_t launch_cells_sweep_emit(const CellJob& j, const Launch& L)
{
    if (j.ncells == 0 || j.niso <= 0) return cudaSuccess;
    const uint64_t items = (cells_tiles(j.ncells) + 31) / 32 * (uint64_t)j.niso;
    prof_begin(L, "cells_sweep_emit");
    KVSMC_CELL_SWITCH(j.cell_type, j.dtype,
                      { k_cells_sweep_emit<CT, T><<<cell_grid(items * 32, L), kCellThreads, 0, L.stream>>>(j); });
    prof_end(L);
    *L.counter += 1;
    return cudaGetLastError();
}

cudaError_t launch_sweep_bases(const uint64_t* offsets, uint64_t groups, int niso, const uint64_t* total,
                               uint64_t* out, const Launch& L)
{
    k_sweep_bases<<<1, 32, 0, L.stream>>>(offsets, groups, niso, total, out);
    *L.counter += 1;
    return cudaGetLastError();
}

size_t cells_bounds_scratch_bytes(int num_sms) { return 64 + (size_t)num_sms * 4 * sizeof(BoundPart); }

cudaError_t launch_cells_bounds(const CellJob& j, bool has_conn, void* scratch, float* d_out, const Launch& L)
{
    const uint64_t npos = has_conn ? j.ncells * (uint64_t)(j.cell_type == KVSMC_TETRAHEDRA ? 4 : j.cell_type ==
                                                           KVSMC_HEXAHEDRA ? 8 : j.cell_type == KVSMC_PYRAMID ? 5 : 6) + 1
                                   : j.nnodes;
    if (npos == 0) return cudaSuccess;
    unsigned long long* last_nan = static_cast<unsigned long long*>(scratch);
    BoundPart* parts = reinterpret_cast<BoundPart*>(static_cast<char*>(scratch) + 64);
    const int nb = L.num_sms * 4;
    cudaError_t e = cudaMemsetAsync(last_nan, 0, 3 * sizeof(unsigned long long), L.stream);
    if (e != cudaSuccess) return e;
    prof_begin(L, "cells_bounds");
    k_bounds_last_nan<<<nb, kCellThreads, 0, L.stream>>>(j, npos, has_conn ? 1 : 0, last_nan);
    k_bounds_partial<<<nb, kCellThreads, 0, L.stream>>>(j, npos, has_conn ? 1 : 0, last_nan, parts);
    k_bounds_final<<<1, kCellThreads, 0, L.stream>>>(j, npos, has_conn ? 1 : 0, last_nan, parts, nb, d_out);
    prof_end(L);
    *L.counter += 3;
    return cudaGetLastError();
}

size_t cells_minmax_scratch_bytes(int num_sms) { return (size_t)num_sms * 4 * 64; }

cudaError_t launch_cells_minmax(const CellJob& j, void* scratch, double* d_out, const Launch& L)
{
    const uint64_t nconn = j.ncells * (uint64_t)(j.cell_type == KVSMC_TETRAHEDRA ? 4 : j.cell_type == KVSMC_HEXAHEDRA ? 8
                                                 : j.cell_type == KVSMC_PYRAMID ? 5 : 6);
    const int nb = L.num_sms * 4;
    prof_begin(L, "cells_minmax");
    KVSMC_VALUE_SWITCH(j.dtype, {
        static_assert(sizeof(CellMinMax<T>) <= 64, "partial slot");
        CellMinMax<T>* part = static_cast<CellMinMax<T>*>(scratch);
        k_cells_minmax_partial<T><<<nb, kCellThreads, 0, L.stream>>>(j, nconn, part);
        k_cells_minmax_final<T><<<1, kCellThreads, 0, L.stream>>>(j, part, nb, d_out);
    });
    prof_end(L);
    *L.counter += 2;
    return cudaGetLastError();
}

uint64_t cells_tiles(uint64_t ncells) { return (ncells + 31) / 32; }

}  // namespace kvsmc

namespace {

using kvsmc_host::fail;

int nodes_per_cell(int ct)
{
    return ct == KVSMC_TETRAHEDRA ? 4 : ct == KVSMC_HEXAHEDRA ? 8 : ct == KVSMC_PYRAMID ? 5 : ct == KVSMC_PRISM ? 6 : 0;
}

// kvs::Math::Equal (Utility/Math.h:135-138)
bool equal_abs(double a, double b)
{
    const double d = a - b;
    return (d < 0 ? -d : d) < 1.e-6;
}

kvsmc_status check_args(kvsmc_context* ctx, int cell_type, int dtype, uint64_t nnodes, const void* values,
                        const float* coords, const uint32_t* connections, uint64_t ncells)
{
    if (nodes_per_cell(cell_type) == 0)
        return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "cells: unknown cell type %d", cell_type);
    if (kvsmc::dtype_size(dtype) == 0) return fail(ctx, KVSMC_ERR_UNSUPPORTED_DTYPE, "cells: data type %d", dtype);
    if (nnodes == 0 || !values || !coords || (ncells && !connections))
        return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "cells: empty or null volume arrays");
    // the mappers hold node ids in int and loop cells with a UInt32 counter
    if (nnodes > 0x7fffffffull || ncells > 0xffffffffull)
        return fail(ctx, KVSMC_ERR_TOO_LARGE, "cells: %llu nodes / %llu cells beyond the 32-bit ids",
                    (unsigned long long)nnodes, (unsigned long long)ncells);
    return KVSMC_OK;
}

// The count pass's scratch (group counts, offsets, scan scratch, a tail for
// the total or the min/max) in the context's arena, and the bad-index flag.
struct CellsScratch {
    void* d_scan;
    uint64_t* d_tail;
    uint64_t tiles;      // 32-cell groups
    uint64_t nscan;      // scanned entries: groups x isolevels
    void* d_extra;       // sweep: isolevel records (kCellSweepMax) and bases (kCellSweepMax + 1)
};

kvsmc_status cells_prepare(kvsmc_context* ctx, kvsmc::CellJob& j, CellsScratch* sc, int niso = 1)
{
    using namespace kvsmc_host;
    if (!ctx->d_flag) KVSMC_CUDA(ctx, cudaMalloc(&ctx->d_flag, sizeof(int)));
    j.bad_index = ctx->d_flag;
    KVSMC_CUDA(ctx, cudaMemsetAsync(ctx->d_flag, 0, sizeof(int), ctx->stream));
    sc->tiles = kvsmc::cells_tiles(j.ncells);
    sc->nscan = sc->tiles * (uint64_t)niso;
    const size_t bc = align_up(sc->nscan * 4, 256), bo = align_up(sc->nscan * 8, 256),
                 bs = align_up(std::max(std::max(kvsmc::scan_scratch_bytes(sc->nscan),
                                                 kvsmc::cells_minmax_scratch_bytes(ctx->num_sms)),
                                        kvsmc::minmax_scratch_bytes(ctx->num_sms)), 256),
                 be = align_up(kvsmc::kCellSweepMax * sizeof(kvsmc::CellIso) + (kvsmc::kCellSweepMax + 1) * 8, 256);
    kvsmc_status st = ensure_scratch(ctx, bc + bo + bs + 256 + be);
    if (st) return st;
    char* base = static_cast<char*>(ctx->scratch);
    j.tile_counts = reinterpret_cast<uint32_t*>(base);
    j.tile_offsets = reinterpret_cast<uint64_t*>(base + bc);
    sc->d_scan = base + bc + bo;
    sc->d_tail = reinterpret_cast<uint64_t*>(base + bc + bo + bs);
    sc->d_extra = base + bc + bo + bs + 256;
    return KVSMC_OK;
}

int read_bad(kvsmc_context* ctx)
{
    int bad = 0;
    std::memcpy(&bad, ctx->h_small + 2, sizeof(int));
    return bad;
}

// Min/max (when not given) and the Math::Equal early exit.  *go is false
// when no cell is to be visited; sizes holds the range.
kvsmc_status cells_range(kvsmc_context* ctx, kvsmc::CellJob& j, const CellsScratch& sc, int32_t has_minmax,
                         double min_value, double max_value, kvsmc_sizes* sizes, bool* go)
{
    using namespace kvsmc_host;
    *go = false;
    const kvsmc::Launch L = launch_of(ctx);
    // MapperBase::setRange: the volume's min/max, computed when not set
    double vmin = min_value, vmax = max_value;
    if (!has_minmax) {
        if (j.ncells) {
            KVSMC_CUDA(ctx, kvsmc::launch_cells_minmax(j, sc.d_scan, reinterpret_cast<double*>(sc.d_tail), L));
        } else {
            // no connections: the scan runs over the nodes (UnstructuredVolumeObject.cpp:88-102)
            kvsmc::VolumeView v1;
            std::memset(&v1, 0, sizeof v1);
            v1.data = j.values;
            v1.dtype = j.dtype;
            v1.nx = (uint32_t)j.nnodes;
            v1.ny = v1.nz = 1;
            v1.pitch = v1.slice = j.nnodes;
            KVSMC_CUDA(ctx, kvsmc::launch_minmax(v1, sc.d_scan, reinterpret_cast<double*>(sc.d_tail), L));
        }
        KVSMC_CUDA(ctx, cudaMemcpyAsync(ctx->h_small, sc.d_tail, 2 * sizeof(double), cudaMemcpyDeviceToHost,
                                        ctx->stream));
        KVSMC_CUDA(ctx, cudaMemcpyAsync(ctx->h_small + 2, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        std::memcpy(&vmin, ctx->h_small, sizeof(double));
        std::memcpy(&vmax, ctx->h_small + 1, sizeof(double));
        if (read_bad(ctx)) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "cells: a connection index is >= nnodes");
    }
    sizes->min_value = vmin;
    sizes->max_value = vmax;
    if (equal_abs(vmin, vmax)) return KVSMC_OK;   // MarchingTetrahedra.cpp:118-119
    sizes->extracted = 1;
    if (j.ncells == 0) return KVSMC_OK;
    j.vmin = vmin;
    j.vmax = vmax;
    j.f = make_fast(j.iso, vmin, vmax, j.dtype);
    *go = true;
    return KVSMC_OK;
}

// Count and scan (total in sc.d_tail), and, when `emit` is set, the emit pass
// right behind them with the caller's capacity, guarded on the device by the
// total; then one read-back of the total and the flag.
kvsmc_status cells_passes(kvsmc_context* ctx, kvsmc::CellJob& j, const CellsScratch& sc, bool emit,
                          kvsmc_sizes* sizes)
{
    using namespace kvsmc_host;
    const kvsmc::Launch L = launch_of(ctx);
    KVSMC_CUDA(ctx, kvsmc::launch_cells_count(j, L));
    KVSMC_CUDA(ctx, kvsmc::launch_scan(j.tile_counts, j.tile_offsets, sc.nscan, sc.d_scan, sc.d_tail, L));
    if (emit) {
        j.d_total = sc.d_tail;
        KVSMC_CUDA(ctx, kvsmc::launch_cells_emit(j, L));
    }
    KVSMC_CUDA(ctx, cudaMemcpyAsync(ctx->h_small, sc.d_tail, sizeof(uint64_t), cudaMemcpyDeviceToHost, ctx->stream));
    KVSMC_CUDA(ctx, cudaMemcpyAsync(ctx->h_small + 2, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (read_bad(ctx)) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "cells: a connection index is >= nnodes");
    const uint64_t t = ctx->h_small[0];
    sizes->ntriangles = t;
    sizes->nvertices = 3 * t;
    sizes->ncoords = 9 * t;
    sizes->nnormals = 3 * t;
    return KVSMC_OK;
}

kvsmc::CellJob make_job(int cell_type, int dtype, const void* values, uint64_t nnodes, const float* coords,
                        const uint32_t* conn, uint64_t ncells, double isolevel)
{
    kvsmc::CellJob j;
    std::memset(&j, 0, sizeof j);
    j.cell_type = cell_type;
    j.dtype = dtype;
    j.values = values;
    j.nnodes = nnodes;
    j.coords = coords;
    j.conn = conn;
    j.ncells = ncells;
    j.iso = isolevel;
    j.cls = kvsmc_host::make_classifier(isolevel);
    j.conn_vec16 = (reinterpret_cast<uintptr_t>(conn) & 15u) == 0;
    return j;
}

}  // namespace

extern "C" {

kvsmc_status kvsmc_marching_cells_device(kvsmc_context* ctx, kvsmc_cell_type cell_type, const void* values,
                                         kvsmc_dtype dtype, uint64_t nnodes, const float* coords,
                                         const uint32_t* connections, uint64_t ncells, double isolevel,
                                         int32_t has_minmax, double min_value, double max_value, float* out_coords,
                                         uint64_t coords_capacity, float* out_normals, uint64_t normals_capacity,
                                         kvsmc_sizes* sizes)
{
    using namespace kvsmc_host;
    if (!ctx || !sizes) return KVSMC_ERR_INVALID_ARGUMENT;
    std::memset(sizes, 0, sizeof *sizes);
    kvsmc_status st = check_args(ctx, cell_type, dtype, nnodes, values, coords, connections, ncells);
    if (st) return st;
    KVSMC_CUDA(ctx, cudaSetDevice(ctx->device));
    kvsmc::CellJob j = make_job(cell_type, dtype, values, nnodes, coords, connections, ncells, isolevel);
    CellsScratch sc;
    bool go = false;
    if ((st = cells_prepare(ctx, j, &sc)) || (st = cells_range(ctx, j, sc, has_minmax, min_value, max_value, sizes,
                                                                &go)) || !go)
        return st;
    // emit behind the count when outputs are given (the kernel writes nothing
    // unless the total fits them): one host round trip per call
    const bool outs = out_coords && out_normals;
    j.out_coords = out_coords;
    j.out_normals = out_normals;
    j.cap_tris = outs ? std::min(coords_capacity / 9, normals_capacity / 3) : 0;
    if ((st = cells_passes(ctx, j, sc, outs, sizes))) return st;
    const uint64_t t = sizes->ntriangles;
    if (t > j.cap_tris && t > 0)
        return fail(ctx, KVSMC_ERR_CAPACITY, "cells: %llu triangles do not fit the outputs", (unsigned long long)t);
    return KVSMC_OK;
}

kvsmc_status kvsmc_marching_cells_host(kvsmc_context* ctx, kvsmc_cell_type cell_type, const void* values,
                                       kvsmc_dtype dtype, uint64_t nnodes, const float* coords,
                                       const uint32_t* connections, uint64_t ncells, double isolevel,
                                       int32_t has_minmax, double min_value, double max_value,
                                       kvsmc_host_alloc_fn alloc, void* user, kvsmc_sizes* sizes)
{
    using namespace kvsmc_host;
    if (!ctx || !alloc || !sizes) return KVSMC_ERR_INVALID_ARGUMENT;
    std::memset(sizes, 0, sizeof *sizes);
    kvsmc_status st = check_args(ctx, cell_type, dtype, nnodes, values, coords, connections, ncells);
    if (st) return st;
    KVSMC_CUDA(ctx, cudaSetDevice(ctx->device));
    const int npc = nodes_per_cell(cell_type);
    const size_t es = kvsmc::dtype_size(dtype);
    // inputs and outputs in one device allocation: values | coords | connections | outputs
    const size_t bv = align_up(nnodes * es, 256), bx = align_up(nnodes * 12, 256),
                 bk = align_up(std::max<uint64_t>(1, ncells * npc) * 4, 256);
    char* d_in = nullptr;
    float* d_out = nullptr;
    auto done = [&](kvsmc_status s) {
        cudaStreamSynchronize(ctx->stream);
        cudaFree(d_in);
        cudaFree(d_out);
        return s;
    };
    cudaError_t e = cudaMalloc(&d_in, bv + bx + bk);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_in, values, nnodes * es, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_in + bv, coords, nnodes * 12, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess && ncells)
        e = cudaMemcpyAsync(d_in + bv + bx, connections, ncells * npc * 4, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess)
        return done(fail(ctx, e == cudaErrorMemoryAllocation ? KVSMC_ERR_OUT_OF_MEMORY : KVSMC_ERR_CUDA,
                         "cells: %s", cudaGetErrorString(e)));
    kvsmc::CellJob j = make_job(cell_type, dtype, d_in, nnodes, reinterpret_cast<const float*>(d_in + bv),
                                reinterpret_cast<const uint32_t*>(d_in + bv + bx), ncells, isolevel);
    CellsScratch sc;
    bool go = false;
    if ((st = cells_prepare(ctx, j, &sc)) || (st = cells_range(ctx, j, sc, has_minmax, min_value, max_value, sizes,
                                                                &go)) || !go ||
        (st = cells_passes(ctx, j, sc, false, sizes)) || sizes->ntriangles == 0)
        return done(st);
    const uint64_t t = sizes->ntriangles;
    if ((e = cudaMalloc(&d_out, t * 12 * sizeof(float))) != cudaSuccess)
        return done(fail(ctx, KVSMC_ERR_OUT_OF_MEMORY, "cells: %s", cudaGetErrorString(e)));
    j.out_coords = d_out;
    j.out_normals = d_out + 9 * t;
    j.cap_tris = t;
    if ((e = kvsmc::launch_cells_emit(j, launch_of(ctx))) != cudaSuccess)
        return done(fail(ctx, KVSMC_ERR_CUDA, "cells: %s", cudaGetErrorString(e)));
    void* hc = alloc(user, 0, 9 * t);
    void* hn = hc ? alloc(user, 1, 3 * t) : nullptr;
    if (!hc || !hn) return done(fail(ctx, KVSMC_ERR_OUT_OF_MEMORY, "cells: host alloc"));
    e = cudaMemcpyAsync(hc, d_out, t * 9 * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hn, d_out + 9 * t, t * 3 * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return done(fail(ctx, KVSMC_ERR_CUDA, "cells: %s", cudaGetErrorString(e)));
    return done(KVSMC_OK);
}

kvsmc_status kvsmc_slice_cells_host(kvsmc_context* ctx, kvsmc_cell_type cell_type, const void* values,
                                    kvsmc_dtype dtype, uint64_t nnodes, const float* coords,
                                    const uint32_t* connections, uint64_t ncells, const kvsmc_slice_params* p,
                                    kvsmc_host_alloc_fn alloc, void* user, uint64_t* ntriangles)
{
    using namespace kvsmc_host;
    if (!ctx || !alloc || !ntriangles) return KVSMC_ERR_INVALID_ARGUMENT;
    *ntriangles = 0;
    if (!p || !p->tf_table || p->tf_resolution < 1)
        return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "slice: bad parameters (colour table)");
    kvsmc_status st = check_args(ctx, cell_type, dtype, nnodes, values, coords, connections, ncells);
    if (st) return st;
    KVSMC_CUDA(ctx, cudaSetDevice(ctx->device));
    if (ncells == 0) return KVSMC_OK;
    const int npc = nodes_per_cell(cell_type);
    const size_t es = kvsmc::dtype_size(dtype);
    // values | coords | connections | colour table in one device allocation
    const size_t bv = align_up(nnodes * es, 256), bx = align_up(nnodes * 12, 256), bk = align_up(ncells * npc * 4, 256),
                 bt = align_up((size_t)3 * p->tf_resolution, 256);
    char* d_in = nullptr;
    char* d_out = nullptr;
    auto done = [&](kvsmc_status s) {
        cudaStreamSynchronize(ctx->stream);
        cudaFree(d_in);
        cudaFree(d_out);
        return s;
    };
    cudaError_t e = cudaMalloc(&d_in, bv + bx + bk + bt);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_in, values, nnodes * es, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_in + bv, coords, nnodes * 12, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_in + bv + bx, connections, ncells * npc * 4, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_in + bv + bx + bk, p->tf_table, (size_t)3 * p->tf_resolution, cudaMemcpyHostToDevice,
                            ctx->stream);
    if (e != cudaSuccess)
        return done(fail(ctx, e == cudaErrorMemoryAllocation ? KVSMC_ERR_OUT_OF_MEMORY : KVSMC_ERR_CUDA,
                         "slice cells: %s", cudaGetErrorString(e)));
    kvsmc::CellJob j = make_job(cell_type, dtype, d_in, nnodes, reinterpret_cast<const float*>(d_in + bv),
                                reinterpret_cast<const uint32_t*>(d_in + bv + bx), ncells, 0.0);
    for (int k = 0; k < 4; ++k) j.coef[k] = p->coefficients[k];
    j.tf_min = p->tf_min;
    j.tf_max = p->tf_max;
    j.tf_res = p->tf_resolution;
    j.table = reinterpret_cast<const uint8_t*>(d_in + bv + bx + bk);
    CellsScratch sc;
    if ((st = cells_prepare(ctx, j, &sc))) return done(st);
    const kvsmc::Launch L = launch_of(ctx);
    e = kvsmc::launch_cells_slice_count(j, L);
    if (e == cudaSuccess) e = kvsmc::launch_scan(j.tile_counts, j.tile_offsets, sc.nscan, sc.d_scan, sc.d_tail, L);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ctx->h_small, sc.d_tail, sizeof(uint64_t), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ctx->h_small + 2, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return done(fail(ctx, KVSMC_ERR_CUDA, "slice cells: %s", cudaGetErrorString(e)));
    if (read_bad(ctx)) return done(fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "cells: a connection index is >= nnodes"));
    const uint64_t t = ctx->h_small[0];
    *ntriangles = t;
    if (t == 0) return done(KVSMC_OK);
    const size_t oc = align_up(t * 36, 256), on = align_up(t * 12, 256);
    if ((e = cudaMalloc(&d_out, oc + on + t * 9)) != cudaSuccess)
        return done(fail(ctx, KVSMC_ERR_OUT_OF_MEMORY, "slice cells: %s", cudaGetErrorString(e)));
    j.out_coords = reinterpret_cast<float*>(d_out);
    j.out_normals = reinterpret_cast<float*>(d_out + oc);
    j.out_colors = reinterpret_cast<uint8_t*>(d_out + oc + on);
    j.cap_tris = t;
    if ((e = kvsmc::launch_cells_slice_emit(j, L)) != cudaSuccess)
        return done(fail(ctx, KVSMC_ERR_CUDA, "slice cells: %s", cudaGetErrorString(e)));
    void* hc = alloc(user, 0, 9 * t);
    void* hn = hc ? alloc(user, 1, 3 * t) : nullptr;
    void* hk = hn ? alloc(user, 3, 9 * t) : nullptr;
    if (!hc || !hn || !hk) return done(fail(ctx, KVSMC_ERR_OUT_OF_MEMORY, "slice cells: host alloc"));
    e = cudaMemcpyAsync(hc, j.out_coords, t * 36, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hn, j.out_normals, t * 12, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hk, j.out_colors, t * 9, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return done(fail(ctx, KVSMC_ERR_CUDA, "slice cells: %s", cudaGetErrorString(e)));
    return done(KVSMC_OK);
}

kvsmc_status kvsmc_cells_bounds(kvsmc_context* ctx, kvsmc_cell_type cell_type, const float* coords, uint64_t nnodes,
                                const uint32_t* connections, uint64_t ncells, float* min_coord, float* max_coord)
{
    using namespace kvsmc_host;
    if (!ctx || !min_coord || !max_coord) return KVSMC_ERR_INVALID_ARGUMENT;
    const int npc = nodes_per_cell(cell_type);
    if (npc == 0) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "cells: unknown cell type %d", (int)cell_type);
    if (nnodes == 0 || !coords || (ncells && !connections))
        return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "cells: empty or null volume arrays");
    KVSMC_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t bx = align_up(nnodes * 12, 256), bk = align_up(std::max<uint64_t>(1, ncells * npc) * 4, 256);
    char* d_in = nullptr;
    auto done = [&](kvsmc_status st) {
        cudaStreamSynchronize(ctx->stream);
        cudaFree(d_in);
        return st;
    };
    cudaError_t e = cudaMalloc(&d_in, bx + bk);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_in, coords, nnodes * 12, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess && ncells)
        e = cudaMemcpyAsync(d_in + bx, connections, ncells * npc * 4, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess)
        return done(fail(ctx, e == cudaErrorMemoryAllocation ? KVSMC_ERR_OUT_OF_MEMORY : KVSMC_ERR_CUDA,
                         "cells bounds: %s", cudaGetErrorString(e)));
    kvsmc::CellJob j = make_job(cell_type, KVSMC_F32, nullptr, nnodes, reinterpret_cast<const float*>(d_in),
                                reinterpret_cast<const uint32_t*>(d_in + bx), ncells, 0.0);
    const size_t bs = align_up(kvsmc::cells_bounds_scratch_bytes(ctx->num_sms), 256);
    kvsmc_status st = ensure_scratch(ctx, bs + 256);
    if (st) return done(st);
    if (!ctx->d_flag) {
        if ((e = cudaMalloc(&ctx->d_flag, sizeof(int))) != cudaSuccess)
            return done(fail(ctx, KVSMC_ERR_OUT_OF_MEMORY, "cells bounds: %s", cudaGetErrorString(e)));
    }
    j.bad_index = ctx->d_flag;
    char* base = static_cast<char*>(ctx->scratch);
    float* d_out = reinterpret_cast<float*>(base + bs);
    e = cudaMemsetAsync(ctx->d_flag, 0, sizeof(int), ctx->stream);
    if (e == cudaSuccess) e = kvsmc::launch_cells_bounds(j, ncells > 0, base, d_out, launch_of(ctx));
    if (e == cudaSuccess) e = cudaMemcpyAsync(ctx->h_small, d_out, 6 * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream);
    // the six floats fill h_small[0..2]; the flag goes behind them
    if (e == cudaSuccess) e = cudaMemcpyAsync(ctx->h_small + 4, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return done(fail(ctx, KVSMC_ERR_CUDA, "cells bounds: %s", cudaGetErrorString(e)));
    int bad = 0;
    std::memcpy(&bad, ctx->h_small + 4, sizeof(int));
    if (bad) return done(fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "cells: a connection index is >= nnodes"));
    float out[6];
    std::memcpy(out, ctx->h_small, sizeof out);
    for (int k = 0; k < 3; ++k) {
        min_coord[k] = out[k];
        max_coord[k] = out[3 + k];
    }
    return done(KVSMC_OK);
}

kvsmc_status kvsmc_marching_cells_sweep_device(kvsmc_context* ctx, kvsmc_cell_type cell_type, const void* values,
                                               kvsmc_dtype dtype, uint64_t nnodes, const float* coords,
                                               const uint32_t* connections, uint64_t ncells,
                                               const double* isolevels, int32_t niso, int32_t has_minmax,
                                               double min_value, double max_value, float* const* out_coords,
                                               const uint64_t* coords_capacity, float* const* out_normals,
                                               const uint64_t* normals_capacity, kvsmc_sizes* sizes)
{
    using namespace kvsmc_host;
    if (!ctx || !isolevels || !sizes || niso < 1) return KVSMC_ERR_INVALID_ARGUMENT;
    if (niso > kvsmc::kCellSweepMax)
        return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "cells sweep: %d isolevels (at most %d)", (int)niso,
                    kvsmc::kCellSweepMax);
    std::memset(sizes, 0, sizeof(kvsmc_sizes) * (size_t)niso);
    kvsmc_status st = check_args(ctx, cell_type, dtype, nnodes, values, coords, connections, ncells);
    if (st) return st;
    KVSMC_CUDA(ctx, cudaSetDevice(ctx->device));
    kvsmc::CellJob j = make_job(cell_type, dtype, values, nnodes, coords, connections, ncells, isolevels[0]);
    CellsScratch sc;
    bool go = false;
    if ((st = cells_prepare(ctx, j, &sc, niso)) ||
        (st = cells_range(ctx, j, sc, has_minmax, min_value, max_value, &sizes[0], &go)))
        return st;
    for (int k = 1; k < niso; ++k) {
        sizes[k].min_value = sizes[0].min_value;
        sizes[k].max_value = sizes[0].max_value;
        sizes[k].extracted = sizes[0].extracted;
    }
    if (!go) return KVSMC_OK;
    std::vector<kvsmc::CellIso> isos((size_t)niso);
    for (int k = 0; k < niso; ++k) {
        kvsmc::CellIso& I = isos[k];
        std::memset(&I, 0, sizeof I);
        I.iso = isolevels[k];
        I.cls = make_classifier(isolevels[k]);
        I.f = make_fast(isolevels[k], j.vmin, j.vmax, j.dtype);
    }
    kvsmc::CellIso* d_isos = static_cast<kvsmc::CellIso*>(sc.d_extra);
    uint64_t* d_bases = reinterpret_cast<uint64_t*>(static_cast<char*>(sc.d_extra) +
                                                    kvsmc::kCellSweepMax * sizeof(kvsmc::CellIso));
    j.isos = d_isos;
    j.niso = niso;
    const kvsmc::Launch L = launch_of(ctx);
    KVSMC_CUDA(ctx, cudaMemcpyAsync(d_isos, isos.data(), sizeof(kvsmc::CellIso) * niso, cudaMemcpyHostToDevice,
                                    ctx->stream));
    KVSMC_CUDA(ctx, kvsmc::launch_cells_sweep_count(j, L));
    KVSMC_CUDA(ctx, kvsmc::launch_scan(j.tile_counts, j.tile_offsets, sc.nscan, sc.d_scan, sc.d_tail, L));
    KVSMC_CUDA(ctx, kvsmc::launch_sweep_bases(j.tile_offsets, sc.tiles, niso, sc.d_tail, d_bases, L));
    std::vector<uint64_t> bases((size_t)niso + 1);
    int bad = 0;
    KVSMC_CUDA(ctx, cudaMemcpyAsync(bases.data(), d_bases, 8 * ((size_t)niso + 1), cudaMemcpyDeviceToHost, ctx->stream));
    KVSMC_CUDA(ctx, cudaMemcpyAsync(&bad, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (bad) return fail(ctx, KVSMC_ERR_INVALID_ARGUMENT, "cells: a connection index is >= nnodes");
    bool fits = out_coords && out_normals && coords_capacity && normals_capacity;
    for (int k = 0; k < niso; ++k) {
        const uint64_t t = bases[k + 1] - bases[k];
        sizes[k].ntriangles = t;
        sizes[k].nvertices = 3 * t;
        sizes[k].ncoords = 9 * t;
        sizes[k].nnormals = 3 * t;
        if (t && (!fits || !out_coords[k] || !out_normals[k] || coords_capacity[k] < 9 * t ||
                  normals_capacity[k] < 3 * t))
            fits = false;
        isos[k].base = bases[k];
        isos[k].out_coords = fits ? out_coords[k] : nullptr;
        isos[k].out_normals = fits ? out_normals[k] : nullptr;
        isos[k].cap_tris = t;
    }
    if (!fits) return fail(ctx, KVSMC_ERR_CAPACITY, "cells sweep: the triangles do not fit the outputs");
    if (bases[niso] == 0) return KVSMC_OK;
    KVSMC_CUDA(ctx, cudaMemcpyAsync(d_isos, isos.data(), sizeof(kvsmc::CellIso) * niso, cudaMemcpyHostToDevice,
                                    ctx->stream));
    KVSMC_CUDA(ctx, kvsmc::launch_cells_sweep_emit(j, L));
    // the records' host copy must outlive the copies above
    KVSMC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return KVSMC_OK;
}

}  // extern "C"
