// mc_device.cuh -- device-side building blocks shared by the kernels.
//
// The arithmetic here restates, bit for bit, the per-cell steps of the
// reference kvs::MarchingCubes (Source/Core/Visualization/Mapper/MarchingCubes.cpp):
//   classification  double(v) > isolevel          (:300-316)
//   interpolation   interpolate_vertex<T> in FP64  (:327-356)
//   transform       (p + min_coord) * scale in FP32 (:168-173)
//   normal          (b - a) x (c - a) in FP32       (:227-228, Matrix/Vector3.h:479-485)
// Every FP operation is an explicit round-to-nearest intrinsic so that no
// multiply-add is contracted (the files are also built with --fmad=false).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "mc_tables.h"

namespace kvsmc {

// ----------------------------------------------------------------- descriptors

// A device-resident volume: rows padded to `pitch` elements (16-byte multiple),
// slices of pitch*ny elements, x fastest.
struct VolumeView {
    const void* data;
    uint32_t nx, ny, nz;
    int32_t dtype;
    uint64_t pitch;   // elements per row
    uint64_t slice;   // elements per slice
};

// Thresholds that make classification exact without FP64:
//   float data : v > f_thr   with f_thr = largest float <= isolevel
//   int data   : v > i_thr   with i_thr = floor(isolevel) (clamped)
//   64-bit int / double data: (double)v > isolevel
struct Classifier {
    double iso;
    float f_thr;
    int32_t pad;
    long long i_thr;
};

// Constants of the FP64 interpolation sequence of one request.
struct Interp {
    double iso;
    double vmin, vmax;      // clamp range (volume min/max or preset)
    float min_coord[3];     // volume->minObjectCoord()
    float scale[3];         // (max_coord - min_coord) / ncells
};

// One extraction request as the kernels see it.
struct Job {
    VolumeView vol;
    Classifier cls;
    Interp ip;
    int32_t mode;
    uint32_t cell_rows;     // cell rows (y) per cell tile
    uint32_t cell_ytiles;   // ceil((ny-1)/cell_rows)
    uint32_t node_rows;     // node rows per node tile
    uint32_t node_ytiles;   // ceil(ny/node_rows)
    uint32_t words_per_row; // ceil(nx/32) rank words per node row
    uint64_t cell_tiles;    // (nz-1)*cell_ytiles
    uint64_t node_tiles;    // nz*node_ytiles
    // scratch
    uint32_t* tile_counts;  // per cell tile triangle counts
    uint64_t* tile_offsets; // per cell tile first triangle
    uint32_t* vtile_counts; // per node tile vertex counts
    uint64_t* vtile_offsets;
    uint4* rank;            // per 32-node word: x/y/z crossing flags + first vertex id
    // outputs
    float* coords;
    float* normals;
    uint32_t* connections;
    // vertex normals (mode 2): per-triangle normals, then each vertex's
    // triangles (counts, scanned offsets, lists) for the ordered sums
    float* tri_normals;
    uint32_t* vcount;         // triangles per vertex
    uint32_t* vlist;          // their ids, slot-major (slot s of vertex v at s * nvert + v)
};

// ------------------------------------------------------------------- values

template <typename T> struct ValueTraits;
#define KVSMC_VT(T, CODE, FAST)                                             \
    template <> struct ValueTraits<T> {                                     \
        static constexpr int code = CODE;                                   \
        static constexpr int fast_cls = FAST;                               \
    };
KVSMC_VT(int8_t, 0, 1)
KVSMC_VT(int16_t, 1, 1)
KVSMC_VT(int32_t, 2, 1)
KVSMC_VT(long long, 3, 0)
KVSMC_VT(uint8_t, 4, 1)
KVSMC_VT(uint16_t, 5, 1)
KVSMC_VT(uint32_t, 6, 1)
KVSMC_VT(unsigned long long, 7, 0)
KVSMC_VT(float, 8, 1)
KVSMC_VT(double, 9, 0)
#undef KVSMC_VT

// static_cast<double>(v) as C++ does it (round to nearest for 64-bit ints).
__device__ __forceinline__ double to_double(int8_t v) { return (double)v; }
__device__ __forceinline__ double to_double(int16_t v) { return (double)v; }
__device__ __forceinline__ double to_double(int32_t v) { return (double)v; }
__device__ __forceinline__ double to_double(long long v) { return __ll2double_rn(v); }
__device__ __forceinline__ double to_double(uint8_t v) { return (double)v; }
__device__ __forceinline__ double to_double(uint16_t v) { return (double)v; }
__device__ __forceinline__ double to_double(uint32_t v) { return (double)v; }
__device__ __forceinline__ double to_double(unsigned long long v) { return __ull2double_rn(v); }
__device__ __forceinline__ double to_double(float v) { return (double)v; }
__device__ __forceinline__ double to_double(double v) { return v; }

// calculate_table_index's test `static_cast<double>(v) > isolevel` (MarchingCubes.cpp:306-313).
__device__ __forceinline__ bool above(const Classifier& c, float v) { return v > c.f_thr; }
__device__ __forceinline__ bool above(const Classifier& c, double v) { return v > c.iso; }
__device__ __forceinline__ bool above(const Classifier& c, int8_t v) { return (long long)v > c.i_thr; }
__device__ __forceinline__ bool above(const Classifier& c, int16_t v) { return (long long)v > c.i_thr; }
__device__ __forceinline__ bool above(const Classifier& c, int32_t v) { return (long long)v > c.i_thr; }
__device__ __forceinline__ bool above(const Classifier& c, uint8_t v) { return (long long)v > c.i_thr; }
__device__ __forceinline__ bool above(const Classifier& c, uint16_t v) { return (long long)v > c.i_thr; }
__device__ __forceinline__ bool above(const Classifier& c, uint32_t v) { return (long long)v > c.i_thr; }
__device__ __forceinline__ bool above(const Classifier& c, long long v) { return __ll2double_rn(v) > c.iso; }
__device__ __forceinline__ bool above(const Classifier& c, unsigned long long v) { return __ull2double_rn(v) > c.iso; }

template <typename T>
__device__ __forceinline__ T load(const T* p, uint64_t i) { return __ldg(p + i); }

template <typename T>
__device__ __forceinline__ uint64_t node_index(const VolumeView& v, uint32_t x, uint32_t y, uint32_t z)
{
    return (uint64_t)x + (uint64_t)y * v.pitch + (uint64_t)z * v.slice;
}

// Case index of cell (x,y,z); corner k at offset bits (dx | dy<<1 | dz<<2)
// in the reference's corner order 0:(0,0,0) 1:(1,0,0) 2:(1,1,0) 3:(0,1,0),
// 4..7 the same at z+1 (MarchingCubes.cpp:187-194).
template <typename T>
__device__ __forceinline__ unsigned cell_case(const Job& j, const T* vol, uint32_t x, uint32_t y, uint32_t z)
{
    const uint64_t i0 = node_index<T>(j.vol, x, y, z);
    const uint64_t p = j.vol.pitch, s = j.vol.slice;
    unsigned c = 0;
    c |= above(j.cls, load(vol, i0)) ? 1u : 0u;
    c |= above(j.cls, load(vol, i0 + 1)) ? 2u : 0u;
    c |= above(j.cls, load(vol, i0 + 1 + p)) ? 4u : 0u;
    c |= above(j.cls, load(vol, i0 + p)) ? 8u : 0u;
    c |= above(j.cls, load(vol, i0 + s)) ? 16u : 0u;
    c |= above(j.cls, load(vol, i0 + 1 + s)) ? 32u : 0u;
    c |= above(j.cls, load(vol, i0 + 1 + p + s)) ? 64u : 0u;
    c |= above(j.cls, load(vol, i0 + p + s)) ? 128u : 0u;
    return c;
}

// --------------------------------------------------------------- arithmetic

// kvs::Math::Clamp (Utility/Math.h:129-132)
__device__ __forceinline__ double clamp_ref(double a, double lo, double hi)
{
    return a <= lo ? lo : (a <= hi ? a : hi);
}

// interpolate_vertex<T> (MarchingCubes.cpp:327-356) then the (p + min) * scale
// lambda (:168-173).  a/b are the edge endpoints in the table's direction,
// va/vb their values.  Exact FP64 sequence, no contraction.
__device__ __forceinline__ float3 interpolate_exact(const Interp& j, double va, double vb,
                                                    float ax, float ay, float az,
                                                    float bx, float by, float bz)
{
    const double v0 = clamp_ref(va, j.vmin, j.vmax);
    const double v1 = clamp_ref(vb, j.vmin, j.vmax);
    const double q = __ddiv_rn(__dsub_rn(j.iso, v0), __dsub_rn(v1, v0));
    const double r = (q < 0.0) ? -q : q;            // kvs::Math::Abs
    const double s = __dsub_rn(1.0, r);
    const double px = __dadd_rn(__dmul_rn(s, (double)ax), __dmul_rn(r, (double)bx));
    const double py = __dadd_rn(__dmul_rn(s, (double)ay), __dmul_rn(r, (double)by));
    const double pz = __dadd_rn(__dmul_rn(s, (double)az), __dmul_rn(r, (double)bz));
    float3 o;
    o.x = __fmul_rn(__fadd_rn(__double2float_rn(px), j.min_coord[0]), j.scale[0]);
    o.y = __fmul_rn(__fadd_rn(__double2float_rn(py), j.min_coord[1]), j.scale[1]);
    o.z = __fmul_rn(__fadd_rn(__double2float_rn(pz), j.min_coord[2]), j.scale[2]);
    return o;
}

// Vertex of local edge `e` (0..11) of cell (x,y,z), interpolated in the
// direction of the reference's VertexID table (duplicated mode).
template <typename T>
__device__ __forceinline__ float3 cell_edge_vertex(const Job& j, const T* vol, const uint8_t* edge_packed,
                                                   uint32_t x, uint32_t y, uint32_t z, int e)
{
    const unsigned ep = edge_packed[e];
    const unsigned a = ep & 7u, b = ep >> 3;
    const uint32_t ax = x + (a & 1u), ay = y + ((a >> 1) & 1u), az = z + (a >> 2);
    const uint32_t bx = x + (b & 1u), by = y + ((b >> 1) & 1u), bz = z + (b >> 2);
    const double va = to_double(load(vol, node_index<T>(j.vol, ax, ay, az)));
    const double vb = to_double(load(vol, node_index<T>(j.vol, bx, by, bz)));
    return interpolate_exact(j.ip, va, vb, __uint2float_rn(ax), __uint2float_rn(ay), __uint2float_rn(az),
                             __uint2float_rn(bx), __uint2float_rn(by), __uint2float_rn(bz));
}

// (b - a) x (c - a), Vector3::cross (Matrix/Vector3.h:479-485).
__device__ __forceinline__ float3 tri_normal(float3 a, float3 b, float3 c)
{
    const float ux = __fsub_rn(b.x, a.x), uy = __fsub_rn(b.y, a.y), uz = __fsub_rn(b.z, a.z);
    const float vx = __fsub_rn(c.x, a.x), vy = __fsub_rn(c.y, a.y), vz = __fsub_rn(c.z, a.z);
    float3 n;
    n.x = __fsub_rn(__fmul_rn(uy, vz), __fmul_rn(uz, vy));
    n.y = __fsub_rn(__fmul_rn(uz, vx), __fmul_rn(ux, vz));
    n.z = __fsub_rn(__fmul_rn(ux, vy), __fmul_rn(uy, vx));
    return n;
}

// ------------------------------------------------------------ block helpers

// Exclusive scan of one uint32 per thread over the block; returns the
// thread's exclusive prefix, *total = block sum.  `warp_sums` holds
// blockDim/32 entries.  Contains __syncthreads.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* warp_sums, uint32_t* total)
{
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const unsigned nwarps = blockDim.x >> 5;
    uint32_t inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= (unsigned)o) inc += t;
    }
    if (lane == 31) warp_sums[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = (lane < nwarps) ? warp_sums[lane] : 0u;
        uint32_t wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= (unsigned)o) wi += t;
        }
        if (lane < nwarps) warp_sums[lane] = wi - w;   // exclusive per warp
        if (lane == nwarps - 1) warp_sums[32] = wi;    // block total
    }
    __syncthreads();
    const uint32_t r = warp_sums[warp] + inc - v;
    *total = warp_sums[32];
    __syncthreads();
    return r;
}

__device__ __forceinline__ uint32_t block_sum(uint32_t v, uint32_t* warp_sums)
{
    uint32_t t;
    block_exclusive_scan(v, warp_sums, &t);
    return t;
}

}  // namespace kvsmc
