// mc_snode.cu -- the shared-vertex modes' node passes as streaming kernels.
//
// calculate_isopoints (MarchingCubes.cpp:366-446) visits every node in z, y, x
// order and gives each of its x-, y- and z-edges (inside the grid) that the
// isolevel crosses a vertex, numbered in that order and interpolated from the
// node towards +axis.  Here a warp task is (a chunk of node planes, one node
// row, a 256-node segment); the warp walks the planes of its chunk with the
// row pair (y, y + 1) of planes z and z + 1 arriving in its shared-memory ring
// of three buffers through bulk copies (cp.async.bulk, bounded mbarrier
// waits), so each value is read from HBM once per pass.  A "node unit" =
// (plane z, row y, segment): the count pass writes its number of vertices,
// an exclusive scan over units in node order gives each unit's first vertex
// id, and the emit pass writes, per 32-node word, the x/y/z crossing flags and
// the word's first vertex id (the rank words the connection pass reads) and
// the vertices themselves (the exact FP32 path of mc_interp.cuh, the FP64
// sequence where it cannot decide).  Lane l takes the nodes l, l + 32, ...,
// l + 224 of the segment, so each 32-node word's flags are three ballots.
#include <cuda_runtime.h>

#include "mc_internal.h"
#include "mc_interp.cuh"
#include "mc_thermo.cuh"
#include "tma.cuh"

namespace kvsmc {

#define KVSMC_SN_SWITCH(DT, ...)                        \
    switch (DT) {                                       \
    case 0: { using T = int8_t; __VA_ARGS__; } break;   \
    case 1: { using T = int16_t; __VA_ARGS__; } break;  \
    case 4: { using T = uint8_t; __VA_ARGS__; } break;  \
    case 5: { using T = uint16_t; __VA_ARGS__; } break; \
    case 8: { using T = float; __VA_ARGS__; } break;    \
    default: return cudaErrorInvalidValue;              \
    }

namespace {

constexpr int kSnThreads = 256;
constexpr int kSnWarps = kSnThreads / 32;
constexpr uint32_t kSnSeg = 256;   // nodes per segment
constexpr unsigned FULL = 0xffffffffu;

// resident CTAs per SM the node emit pass is compiled for (registers per thread)
#ifndef KVSMC_SNODE_EMIT_CTAS
#define KVSMC_SNODE_EMIT_CTAS 3
#endif

__host__ __device__ __forceinline__ size_t sn_align(size_t v) { return (v + 127) / 128 * 128; }

template <typename T, bool EMIT>
__global__ void __launch_bounds__(kSnThreads, EMIT ? KVSMC_SNODE_EMIT_CTAS : 1)
    k_snode(Job j, FastIso f, uint32_t wprn, uint32_t zchunk, uint64_t ntasks, uint32_t row_elems,
            uint32_t copy_bytes, uint32_t* __restrict__ unit_counts, const uint64_t* __restrict__ unit_offsets,
            int* __restrict__ status, unsigned long long* __restrict__ next_task, uint32_t wait_polls)
{
    // count pass: writes unit_counts; emit pass: reads them with their scan
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const size_t plane_elems = 2 * (size_t)row_elems;
    unsigned char* wbase = smem_raw + (size_t)warp * (128 + sn_align(3 * plane_elems * sizeof(T)));
    uint64_t* bar = reinterpret_cast<uint64_t*>(wbase);
    T* ring = reinterpret_cast<T*>(wbase + 128);
    if (lane == 0) {
        for (int b = 0; b < 3; ++b) mbar_init(&bar[b], 1);
        fence_barrier_init();
    }
    __syncwarp();
    const uint32_t nx = j.vol.nx, ny = j.vol.ny, nz = j.vol.nz;
    const uint64_t pitch = j.vol.pitch, slice = j.vol.slice;
    const T* vol = static_cast<const T*>(j.vol.data);
    uint32_t ph = 0;   // per ring buffer: parity of its next completion
    for (;;) {
        unsigned long long tk = 0;
        if (lane == 0) tk = atomicAdd(next_task, 1ull);
        const uint64_t task = __shfl_sync(FULL, tk, 0);
        if (task >= ntasks) break;
        const uint32_t s = (uint32_t)(task % wprn);
        const uint32_t y = (uint32_t)((task / wprn) % ny);
        const uint32_t zc = (uint32_t)(task / ((uint64_t)wprn * ny));
        const uint32_t z0 = zc * zchunk;
        const uint32_t z1 = z0 + zchunk < nz ? z0 + zchunk : nz;            // node planes [z0, z1)
        const uint32_t nplanes = (z1 + 1 < nz ? z1 + 1 : nz) - z0;          // staged planes
        const uint32_t nrows = y + 1 < ny ? 2u : 1u;
        const uint64_t xoff = (uint64_t)s * kSnSeg;
        const uint64_t avail = (pitch - xoff) * sizeof(T);
        const uint32_t row_bytes = (uint32_t)(avail < copy_bytes ? avail : copy_bytes);
        auto issue = [&](uint32_t i) {
            const int b = (int)(i % 3u);
            T* dst = ring + (size_t)b * plane_elems;
            const T* src = vol + (uint64_t)(z0 + i) * slice + (uint64_t)y * pitch + xoff;
            mbar_arrive_expect_tx(&bar[b], nrows * row_bytes);
            for (uint32_t r = 0; r < nrows; ++r) bulk_copy_g2s(dst + r * row_elems, src + r * pitch, row_bytes, &bar[b]);
        };
        auto acquire = [&](uint32_t i) -> bool {
            const uint32_t b = i % 3u;
            const bool ok = mbar_wait(&bar[b], (ph >> b) & 1u, wait_polls);
            if (ok) ph ^= 1u << b;
            return ok;
        };
        __syncwarp();   // the previous task's reads of the ring are done
        if (lane == 0) {
            fence_proxy_async();
            for (uint32_t i = 0; i < nplanes && i < 3; ++i) issue(i);
        }
        uint32_t acq = 0;
        bool dead = false;
        uint32_t issued = 0;
        // emit: the unit's vertex count and first id, loaded one step ahead so
        // their latency hides behind a step's work; a unit without vertices
        // is skipped (no rank word of it is ever read)
        uint32_t next_n = 0;
        uint64_t next_base = 0;
        auto unit_of = [&](uint32_t zz) -> uint64_t { return ((uint64_t)zz * ny + y) * wprn + s; };
        if (EMIT) {
            next_n = unit_counts[unit_of(z0)];
            next_base = unit_offsets[unit_of(z0)];
        }
        for (uint32_t z = z0; z < z1; ++z) {
            const uint32_t st = z - z0;
            const uint32_t need = z + 1 < nz ? st + 1 : st;   // last plane staged this step
            const uint32_t n_now = next_n;
            const uint64_t base_now = next_base;
            if (EMIT && z + 1 < z1) {
                next_n = unit_counts[unit_of(z + 1)];
                next_base = unit_offsets[unit_of(z + 1)];
            }
            bool ok = true;
            while (ok && acq <= need) {
                ok = acquire(acq);
                if (ok) ++acq;
            }
            if (__any_sync(FULL, !ok)) {
                if (lane == 0) atomicExch(status, 1);
                dead = true;
                issued = st + 3 < nplanes ? st + 3 : nplanes;
                break;
            }
            if (EMIT && n_now == 0) {
                __syncwarp();
                if (lane == 0 && st + 3 < nplanes) {
                    fence_proxy_async();
                    issue(st + 3);
                }
                continue;
            }
            const T* ra = ring + (size_t)(st % 3u) * plane_elems;            // plane z, row y
            const T* rb = ra + row_elems;                                     // plane z, row y + 1
            const T* rz = ring + (size_t)((st + 1) % 3u) * plane_elems;      // plane z + 1, row y
            const bool has_y = y + 1 < ny, has_z = z + 1 < nz;
            uint32_t fx = 0, fy = 0, fz = 0;   // crossing flags of this lane's 8 nodes, bit i = node lane + 32 i
            uint32_t cnt = 0;
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const uint32_t xl = lane + 32u * i;
                const uint64_t x = xoff + xl;
                bool bx = false, by = false, bz = false;
                if (x < nx) {
                    const bool a0 = above(j.cls, ra[xl]);
                    bx = x + 1 < nx && above(j.cls, ra[xl + 1]) != a0;
                    by = has_y && above(j.cls, rb[xl]) != a0;
                    bz = has_z && above(j.cls, rz[xl]) != a0;
                }
                fx |= (uint32_t)bx << i;
                fy |= (uint32_t)by << i;
                fz |= (uint32_t)bz << i;
                cnt += (uint32_t)bx + (uint32_t)by + (uint32_t)bz;
            }
            const uint64_t unit = ((uint64_t)z * ny + y) * wprn + s;
            if (!EMIT) {
                const uint32_t tot = __reduce_add_sync(FULL, cnt);
                if (lane == 0) unit_counts[unit] = tot;
            } else {
                const uint64_t base = base_now;
                const uint64_t row = (uint64_t)z * ny + y;
                // per 32-node word i: its crossing flags (three ballots) and its first
                // vertex within the unit; items (node, axis) are numbered like the ids
                uint32_t wx[8], wy[8], wz[8], wrun[8];
                uint32_t total = 0;
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    wx[i] = __ballot_sync(FULL, (fx >> i) & 1u);
                    wy[i] = __ballot_sync(FULL, (fy >> i) & 1u);
                    wz[i] = __ballot_sync(FULL, (fz >> i) & 1u);
                    wrun[i] = total;
                    total += __popc(wx[i]) + __popc(wy[i]) + __popc(wz[i]);
                }
                // lane i < 8 writes word i's rank word
                {
                    uint32_t mx = 0, my = 0, mz = 0, mr = 0;
#pragma unroll
                    for (int i = 0; i < 8; ++i)
                        if ((int)lane == i) { mx = wx[i]; my = wy[i]; mz = wz[i]; mr = wrun[i]; }
                    const uint64_t word = (uint64_t)s * (kSnSeg / 32) + lane;
                    if (lane < 8 && word < j.words_per_row)
                        j.rank[row * j.words_per_row + word] = make_uint4(mx, my, mz, (uint32_t)(base + mr));
                }
                // the step's vertices spread over the lanes: item q has id base + q
                const float fyf = __uint2float_rn(y), fzf = __uint2float_rn(z);
                for (uint32_t q = lane; q < total; q += 32) {
                    // its word: the last i with wrun[i] <= q (words without items share
                    // the next word's start, so the last such i holds items)
                    int wi = 0;
                    uint32_t bx = wx[0], by = wy[0], bz = wz[0], r0 = wrun[0];
#pragma unroll
                    for (int i = 1; i < 8; ++i)
                        if (wrun[i] <= q) { wi = i; bx = wx[i]; by = wy[i]; bz = wz[i]; r0 = wrun[i]; }
                    const uint32_t r = q - r0;
                    // its node: the last lane L whose flags before it (all axes) are at most r
                    uint32_t lo = 0;
#pragma unroll
                    for (int k = 4; k >= 0; --k) {
                        const uint32_t mid = lo + (1u << k);
                        const uint32_t ltm = (1u << mid) - 1u;   // mid <= 31
                        if ((uint32_t)(__popc(bx & ltm) + __popc(by & ltm) + __popc(bz & ltm)) <= r) lo = mid;
                    }
                    const uint32_t L = lo;
                    const uint32_t ltl = (1u << L) - 1u;
                    uint32_t k = r - (__popc(bx & ltl) + __popc(by & ltl) + __popc(bz & ltl));   // k-th flag of node L
                    const uint32_t nf = ((bx >> L) & 1u) | (((by >> L) & 1u) << 1) | (((bz >> L) & 1u) << 2);
                    int axis = 0;
                    for (; axis < 3; ++axis)
                        if ((nf >> axis) & 1u) {
                            if (k == 0) break;
                            --k;
                        }
                    const uint32_t xl = L + 32u * wi;
                    const float ax = __uint2float_rn((uint32_t)xoff + xl);
                    const float v0 = (float)ra[xl];
                    const float v1 = (float)(axis == 0 ? ra[xl + 1] : (axis == 1 ? rb[xl] : rz[xl]));
                    const float bxf = axis == 0 ? __fadd_rn(ax, 1.0f) : ax;
                    const float byf = axis == 1 ? __fadd_rn(fyf, 1.0f) : fyf;
                    const float bzf = axis == 2 ? __fadd_rn(fzf, 1.0f) : fzf;
                    const float3 p = edge_vertex_fast(j.ip, f, v0, v1, ax, fyf, fzf, bxf, byf, bzf, axis);
                    float* o = j.coords + 3 * (base + q);
                    o[0] = p.x; o[1] = p.y; o[2] = p.z;
                }
            }
            // plane z is consumed: refill its buffer with plane z + 3
            __syncwarp();
            if (lane == 0 && st + 3 < nplanes) {
                fence_proxy_async();
                issue(st + 3);
            }
        }
        if (dead) {
            // wait (bounded, by its own limit) for the copies still in flight, then stop
            for (uint32_t i = acq; i < issued; ++i) {
                const uint32_t b = i % 3u;
                if (mbar_wait(&bar[b], (ph >> b) & 1u, 1u << 16)) ph ^= 1u << b;
            }
            break;
        }
        // a normal walk acquires every staged plane: the last step's (z1 < nz) or
        // none more (z1 == nz); keep the parity in step with what was issued
        while (acq < nplanes) {
            if (!acquire(acq)) break;
            ++acq;
        }
    }
}


// resident CTAs per SM the multi-isolevel node emit is compiled for
#ifndef KVSMC_SNODE_MULTI_CTAS
#define KVSMC_SNODE_MULTI_CTAS 3
#endif

// Per-warp tables of the multi-isolevel node emit: for each isolevel with
// vertices in the current node unit (active index m, in threshold order), its
// 32-node words' x/y/z crossing flags and first vertex within the unit, its
// first item of the step, the isolevel and the unit's first vertex id.
struct SnMulti {
    uint32_t fx[kStreamMaxIso * 8], fy[kStreamMaxIso * 8], fz[kStreamMaxIso * 8];
    uint32_t run[kStreamMaxIso * 8];
    uint32_t first[kStreamMaxIso];
    uint32_t iso[kStreamMaxIso];
    uint64_t base[kStreamMaxIso];
};

// Per-CTA tables: the thresholds' bucket map and the requests' constants.
struct SnMultiCta {
    ThermoTables th;
    NodeIso iso[kStreamMaxIso];
};

// calculate_isopoints for up to kStreamMaxIso requests on one volume in one
// pass: the same tasks, ring and numbering as k_snode<T, true>, but each node
// value is classified once for all the requests (threshold masks), the cut
// edges of request k are bit k of the masks' XORs, and the step's vertices of
// all the requests share the lanes.  Every request's ids and rank words are
// the ones its own node emit writes.
template <typename T>
__global__ void __launch_bounds__(kSnThreads, KVSMC_SNODE_MULTI_CTAS)
    k_snode_multi(VolumeView vol, const NodeIso* __restrict__ isos, int niso, float bs, float bo, uint32_t wprn,
                  uint32_t zchunk, uint64_t ntasks, uint32_t row_elems, uint32_t copy_bytes, uint32_t words_per_row,
                  int* __restrict__ status, unsigned long long* __restrict__ next_task, uint32_t wait_polls)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    SnMultiCta& C = *reinterpret_cast<SnMultiCta*>(smem_raw);
    const size_t plane_elems = 2 * (size_t)row_elems;
    const size_t ring_bytes = sn_align(3 * plane_elems * sizeof(T));
    unsigned char* wbase =
        smem_raw + sn_align(sizeof(SnMultiCta)) + (size_t)warp * (128 + ring_bytes + sn_align(sizeof(SnMulti)));
    uint64_t* bar = reinterpret_cast<uint64_t*>(wbase);
    T* ring = reinterpret_cast<T*>(wbase + 128);
    SnMulti& M = *reinterpret_cast<SnMulti*>(wbase + 128 + ring_bytes);
    if (warp == 0) {
        float t = 0.0f;
        if (lane < (unsigned)niso) t = isos[lane].f.f_thr;
        __shared__ float s_thr[kStreamMaxIso];
        if (lane < (unsigned)niso) s_thr[lane] = t;
        __syncwarp();
        thermo_build(C.th, s_thr, niso, bs, bo, lane);
    }
    for (unsigned i = threadIdx.x; i < (unsigned)niso; i += blockDim.x) C.iso[i] = isos[i];
    __syncthreads();   // the only CTA-wide barrier: the tables are read-only from here on
    if (lane == 0) {
        for (int b = 0; b < 3; ++b) mbar_init(&bar[b], 1);
        fence_barrier_init();
    }
    __syncwarp();
    const uint32_t nx = vol.nx, ny = vol.ny, nz = vol.nz;
    const uint64_t pitch = vol.pitch, slice = vol.slice;
    const T* vp = static_cast<const T*>(vol.data);
    uint32_t ph = 0;
    for (;;) {
        unsigned long long tk = 0;
        if (lane == 0) tk = atomicAdd(next_task, 1ull);
        const uint64_t task = __shfl_sync(FULL, tk, 0);
        if (task >= ntasks) break;
        const uint32_t s = (uint32_t)(task % wprn);
        const uint32_t y = (uint32_t)((task / wprn) % ny);
        const uint32_t zc = (uint32_t)(task / ((uint64_t)wprn * ny));
        const uint32_t z0 = zc * zchunk;
        const uint32_t z1 = z0 + zchunk < nz ? z0 + zchunk : nz;            // node planes [z0, z1)
        const uint32_t nplanes = (z1 + 1 < nz ? z1 + 1 : nz) - z0;          // staged planes
        const uint32_t nrows = y + 1 < ny ? 2u : 1u;
        const uint64_t xoff = (uint64_t)s * kSnSeg;
        const uint64_t avail = (pitch - xoff) * sizeof(T);
        const uint32_t row_bytes = (uint32_t)(avail < copy_bytes ? avail : copy_bytes);
        auto issue = [&](uint32_t i) {
            const int b = (int)(i % 3u);
            T* dst = ring + (size_t)b * plane_elems;
            const T* src = vp + (uint64_t)(z0 + i) * slice + (uint64_t)y * pitch + xoff;
            mbar_arrive_expect_tx(&bar[b], nrows * row_bytes);
            for (uint32_t r = 0; r < nrows; ++r) bulk_copy_g2s(dst + r * row_elems, src + r * pitch, row_bytes, &bar[b]);
        };
        auto acquire = [&](uint32_t i) -> bool {
            const uint32_t b = i % 3u;
            const bool ok = mbar_wait(&bar[b], (ph >> b) & 1u, wait_polls);
            if (ok) ph ^= 1u << b;
            return ok;
        };
        __syncwarp();   // the previous task's reads of the ring are done
        if (lane == 0) {
            fence_proxy_async();
            for (uint32_t i = 0; i < nplanes && i < 3; ++i) issue(i);
        }
        uint32_t acq = 0, issued = 0;
        bool dead = false;
        // lane k < niso: request k's vertex count and first id of the unit,
        // loaded one step ahead
        auto unit_of = [&](uint32_t zz) -> uint64_t { return ((uint64_t)zz * ny + y) * wprn + s; };
        uint32_t next_n = 0;
        uint64_t next_base = 0;
        if (lane < (unsigned)niso) {
            next_n = C.iso[lane].counts[unit_of(z0)];
            next_base = C.iso[lane].offsets[unit_of(z0)];
        }
        const float fyf = __uint2float_rn(y);
        for (uint32_t z = z0; z < z1; ++z) {
            const uint32_t st = z - z0;
            const uint32_t need = z + 1 < nz ? st + 1 : st;   // last plane staged this step
            const uint32_t n_now = next_n;
            const uint64_t base_now = next_base;
            if (z + 1 < z1 && lane < (unsigned)niso) {
                next_n = C.iso[lane].counts[unit_of(z + 1)];
                next_base = C.iso[lane].offsets[unit_of(z + 1)];
            }
            bool ok = true;
            while (ok && acq <= need) {
                ok = acquire(acq);
                if (ok) ++acq;
            }
            if (__any_sync(FULL, !ok)) {
                if (lane == 0) atomicExch(status, 1);
                dead = true;
                issued = st + 3 < nplanes ? st + 3 : nplanes;
                break;
            }
            const uint32_t act = __ballot_sync(FULL, lane < (unsigned)niso && n_now != 0);
            if (act) {
                const T* ra = ring + (size_t)(st % 3u) * plane_elems;            // plane z, row y
                const T* rb = ra + row_elems;                                     // plane z, row y + 1
                const T* rz = ring + (size_t)((st + 1) % 3u) * plane_elems;      // plane z + 1, row y
                const bool has_y = y + 1 < ny, has_z = z + 1 < nz;
                // per node lane + 32 i: the requests whose isolevel its x, y, z edges
                // cross (XOR of the two ends' masks), two nodes per word
                uint32_t CX[4] = {0, 0, 0, 0}, CY[4] = {0, 0, 0, 0}, CZ[4] = {0, 0, 0, 0};
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const uint32_t xl = lane + 32u * i;
                    const uint64_t x = xoff + xl;
                    uint32_t cx = 0, cy = 0, cz = 0;
                    if (x < nx) {
                        const uint32_t a = thermo_mask(C.th, niso, bs, bo, (float)ra[xl]);
                        if (x + 1 < nx) cx = a ^ thermo_mask(C.th, niso, bs, bo, (float)ra[xl + 1]);
                        if (has_y) cy = a ^ thermo_mask(C.th, niso, bs, bo, (float)rb[xl]);
                        if (has_z) cz = a ^ thermo_mask(C.th, niso, bs, bo, (float)rz[xl]);
                    }
                    CX[i >> 1] |= cx << (16 * (i & 1));
                    CY[i >> 1] |= cy << (16 * (i & 1));
                    CZ[i >> 1] |= cz << (16 * (i & 1));
                }
                const uint64_t row = (uint64_t)z * ny + y;
                uint32_t total = 0, nact = 0;
                for (uint32_t rem = act; rem; rem &= rem - 1) {
                    const uint32_t k = __ffs(rem) - 1;
                    const uint64_t base = __shfl_sync(FULL, base_now, k);
                    uint32_t wx[8], wy[8], wz[8], wrun[8];
                    uint32_t tot = 0;
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        const uint32_t sh = k + 16u * (uint32_t)(i & 1);
                        wx[i] = __ballot_sync(FULL, (CX[i >> 1] >> sh) & 1u);
                        wy[i] = __ballot_sync(FULL, (CY[i >> 1] >> sh) & 1u);
                        wz[i] = __ballot_sync(FULL, (CZ[i >> 1] >> sh) & 1u);
                        wrun[i] = tot;
                        tot += __popc(wx[i]) + __popc(wy[i]) + __popc(wz[i]);
                    }
                    // lane i < 8: word i's rank word, and the same words for the items below
                    uint32_t mx = 0, my = 0, mz = 0, mr = 0;
#pragma unroll
                    for (int i = 0; i < 8; ++i)
                        if ((int)lane == i) { mx = wx[i]; my = wy[i]; mz = wz[i]; mr = wrun[i]; }
                    if (lane < 8) {
                        const uint64_t word = (uint64_t)s * (kSnSeg / 32) + lane;
                        if (word < words_per_row)
                            C.iso[k].rank[row * words_per_row + word] = make_uint4(mx, my, mz, (uint32_t)(base + mr));
                        M.fx[nact * 8 + lane] = mx;
                        M.fy[nact * 8 + lane] = my;
                        M.fz[nact * 8 + lane] = mz;
                        M.run[nact * 8 + lane] = mr;
                    }
                    if (lane == 0) {
                        M.first[nact] = total;
                        M.iso[nact] = k;
                        M.base[nact] = base;
                    }
                    total += tot;
                    ++nact;
                }
                __syncwarp();
                // the step's vertices of all the requests spread over the lanes: item
                // q belongs to active request m (the last whose first item <= q)
                const float fzf = __uint2float_rn(z);
                for (uint32_t q = lane; q < total; q += 32) {
                    uint32_t m = 0;
#pragma unroll
                    for (uint32_t step = 8; step >= 1; step >>= 1)
                        if (m + step < nact && M.first[m + step] <= q) m += step;
                    const uint32_t r0q = q - M.first[m];
                    // its word: the last i with run[i] <= r0q (words without items share
                    // the next word's start, so the last such i holds items)
                    const uint4 ra4 = *reinterpret_cast<const uint4*>(&M.run[m * 8]);
                    const uint4 rb4 = *reinterpret_cast<const uint4*>(&M.run[m * 8 + 4]);
                    const uint32_t runs[8] = {ra4.x, ra4.y, ra4.z, ra4.w, rb4.x, rb4.y, rb4.z, rb4.w};
                    uint32_t wi = 0;
#pragma unroll
                    for (uint32_t i = 1; i < 8; ++i)
                        if (runs[i] <= r0q) wi = i;
                    const uint32_t bx = M.fx[m * 8 + wi], by = M.fy[m * 8 + wi], bz = M.fz[m * 8 + wi];
                    const uint32_t r = r0q - M.run[m * 8 + wi];
                    // its node: the last lane L whose flags before it (all axes) are at most r
                    uint32_t lo = 0;
#pragma unroll
                    for (int b = 4; b >= 0; --b) {
                        const uint32_t mid = lo + (1u << b);
                        const uint32_t ltm = (1u << mid) - 1u;   // mid <= 31
                        if ((uint32_t)(__popc(bx & ltm) + __popc(by & ltm) + __popc(bz & ltm)) <= r) lo = mid;
                    }
                    const uint32_t L = lo;
                    const uint32_t ltl = (1u << L) - 1u;
                    uint32_t kk = r - (__popc(bx & ltl) + __popc(by & ltl) + __popc(bz & ltl));   // kk-th flag of L
                    const uint32_t nf = ((bx >> L) & 1u) | (((by >> L) & 1u) << 1) | (((bz >> L) & 1u) << 2);
                    int axis = 0;
                    for (; axis < 3; ++axis)
                        if ((nf >> axis) & 1u) {
                            if (kk == 0) break;
                            --kk;
                        }
                    const uint32_t xl = L + 32u * wi;
                    const float ax = __uint2float_rn((uint32_t)xoff + xl);
                    const float v0 = (float)ra[xl];
                    const float v1 = (float)(axis == 0 ? ra[xl + 1] : (axis == 1 ? rb[xl] : rz[xl]));
                    const float bxf = axis == 0 ? __fadd_rn(ax, 1.0f) : ax;
                    const float byf = axis == 1 ? __fadd_rn(fyf, 1.0f) : fyf;
                    const float bzf = axis == 2 ? __fadd_rn(fzf, 1.0f) : fzf;
                    const NodeIso& I = C.iso[M.iso[m]];
                    const float3 p = edge_vertex_fast(I.ip, I.f, v0, v1, ax, fyf, fzf, bxf, byf, bzf, axis);
                    float* o = I.coords + 3 * (M.base[m] + r0q);
                    o[0] = p.x; o[1] = p.y; o[2] = p.z;
                }
            }
            // plane z is consumed: refill its buffer with plane z + 3
            __syncwarp();
            if (lane == 0 && st + 3 < nplanes) {
                fence_proxy_async();
                issue(st + 3);
            }
        }
        if (dead) {
            for (uint32_t i = acq; i < issued; ++i) {
                const uint32_t b = i % 3u;
                if (mbar_wait(&bar[b], (ph >> b) & 1u, 1u << 16)) ph ^= 1u << b;
            }
            break;
        }
        while (acq < nplanes) {
            if (!acquire(acq)) break;
            ++acq;
        }
    }
}

__constant__ uint64_t c_sc_tri[256] = MC_TRI_PACKED_INIT;
__constant__ uint8_t c_sc_ntri[256] = MC_NTRI_INIT;
__constant__ uint8_t c_sc_edge[12] = MC_EDGE_PACKED_INIT;

// Vertex id of node (x, y, z)'s edge along `axis` from the rank words.
__device__ __forceinline__ uint32_t sc_rank_id(const Job& j, uint32_t x, uint32_t y, uint32_t z, int axis)
{
    const uint4 R = j.rank[((uint64_t)z * j.vol.ny + y) * j.words_per_row + (x >> 5)];
    const uint32_t bit = x & 31u, lt = (1u << bit) - 1u;
    uint32_t id = R.w + __popc(R.x & lt) + __popc(R.y & lt) + __popc(R.z & lt);
    if (axis >= 1) id += (R.x >> bit) & 1u;
    if (axis >= 2) id += (R.y >> bit) & 1u;
    return id;
}

// connect_isopoints (MarchingCubes.cpp:456-521) on the streaming layout: a
// warp task is a cell task of the streaming count (one 256-cell row segment,
// a chunk of planes, row pair (y, y + 1) of planes z, z + 1 in its ring); the
// count pass's unit counts and scanned unit and plane offsets give every
// unit's first triangle, a warp scan each lane's.  Lane l takes cells 8 l ..
// 8 l + 7; per triangle (table order, vertices e[i], e[i+2], e[i+1]) the three
// vertex ids come from the rank words of the edges' lower nodes, and the
// polygon normal from the three vertices' coordinates (written by the node
// emit pass): into the normals (polygon normals) or the per-triangle scratch
// the vertex normals are summed from.  One isolevel per launch: isolevel
// iso_k of the streaming count's group `groups[0]` (whose counters hold all
// the group's isolevels, niso per unit).
template <typename T>
__global__ void __launch_bounds__(kSnThreads)
    k_sconnect(Job j, const StreamGroup* __restrict__ groups, const StreamIso* __restrict__ isos,
               const uint16_t* __restrict__ unit_counts, const uint32_t* __restrict__ unit_offsets,
               const uint64_t* __restrict__ plane_base, uint32_t iso_k, uint64_t ntasks, uint64_t nvert,
               uint64_t ntri, int* __restrict__ status, unsigned long long* __restrict__ next_task,
               uint32_t wait_polls)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ uint64_t s_tri[256];
    __shared__ uint8_t s_ntri[256];
    __shared__ uint8_t s_edge[16];
    const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    for (unsigned c = tid; c < 256; c += blockDim.x) {
        s_tri[c] = c_sc_tri[c];
        s_ntri[c] = c_sc_ntri[c];
        if (c < 12) s_edge[c] = c_sc_edge[c];
    }
    __syncthreads();
    const StreamGroup& G = groups[0];
    const uint32_t row_elems = G.seg_elems;
    const size_t plane_elems = 2 * (size_t)row_elems;
    unsigned char* wbase = smem_raw + (size_t)warp * (128 + sn_align(3 * plane_elems * sizeof(T)));
    uint64_t* bar = reinterpret_cast<uint64_t*>(wbase);
    T* ring = reinterpret_cast<T*>(wbase + 128);
    if (lane == 0) {
        for (int b = 0; b < 3; ++b) mbar_init(&bar[b], 1);
        fence_barrier_init();
    }
    __syncwarp();
    const uint32_t cx = G.vol.nx - 1, cy = G.vol.ny - 1, cz = G.vol.nz - 1;
    const uint32_t wpr = G.wpr;
    const uint64_t pitch = G.vol.pitch, slice = G.vol.slice;
    const T* vol = static_cast<const T*>(G.vol.data);
    const StreamIso& I = isos[G.iso_begin + iso_k];
    const uint32_t niso = (uint32_t)G.niso;
    const uint64_t first_plane = plane_base[I.plane_index];
    float* const tri_out = j.mode == 1 ? j.normals : j.tri_normals;
    uint32_t ph = 0;
    for (;;) {
        unsigned long long tk = 0;
        if (lane == 0) tk = atomicAdd(next_task, 1ull);
        const uint64_t task = __shfl_sync(FULL, tk, 0);
        if (task >= ntasks) break;
        const uint32_t seg = (uint32_t)(task % wpr);
        const uint32_t y = (uint32_t)((task / wpr) % cy);
        const uint32_t zc = (uint32_t)(task / ((uint64_t)wpr * cy));
        const uint32_t z0 = zc * G.zchunk;
        const uint32_t z1 = z0 + G.zchunk < cz ? z0 + G.zchunk : cz;   // cell planes [z0, z1)
        const uint32_t nplanes = z1 - z0 + 1;
        const uint64_t xoff = (uint64_t)seg * 256;
        const uint64_t avail = (pitch - xoff) * sizeof(T);
        const uint32_t row_bytes = (uint32_t)(avail < G.seg_copy_bytes ? avail : G.seg_copy_bytes);
        auto issue = [&](uint32_t i) {
            const int b = (int)(i % 3u);
            T* dst = ring + (size_t)b * plane_elems;
            const T* src = vol + (uint64_t)(z0 + i) * slice + (uint64_t)y * pitch + xoff;
            mbar_arrive_expect_tx(&bar[b], 2 * row_bytes);
            for (uint32_t r = 0; r < 2; ++r) bulk_copy_g2s(dst + r * row_elems, src + r * pitch, row_bytes, &bar[b]);
        };
        auto acquire = [&](uint32_t i) -> bool {
            const uint32_t b = i % 3u;
            const bool ok = mbar_wait(&bar[b], (ph >> b) & 1u, wait_polls);
            if (ok) ph ^= 1u << b;
            return ok;
        };
        __syncwarp();
        if (lane == 0) {
            fence_proxy_async();
            for (uint32_t i = 0; i < nplanes && i < 3; ++i) issue(i);
        }
        uint32_t acq = 0, issued = 0;
        bool dead = false;
        const uint32_t x0 = (uint32_t)xoff + 8 * lane;
        const int lim = (int)cx - (int)x0;   // cells of this lane inside the row (if < 8)
        // the unit's triangle count and first triangle, loaded one step ahead
        // so their latency hides behind a step's work
        auto unit_elem = [&](uint32_t zz) -> uint64_t {
            return G.unit_base + (((uint64_t)zz * cy + y) * wpr + seg) * niso + iso_k;
        };
        auto unit_first = [&](uint32_t zz) -> uint64_t {
            return plane_base[I.plane_index + zz] - first_plane + unit_offsets[unit_elem(zz)];
        };
        uint32_t next_count = unit_counts[unit_elem(z0)];
        uint64_t next_first = unit_first(z0);
        for (uint32_t z = z0; z < z1; ++z) {
            const uint32_t st = z - z0;
            const uint32_t count_now = next_count;
            const uint64_t tbase = next_first;
            if (z + 1 < z1) {
                next_count = unit_counts[unit_elem(z + 1)];
                next_first = unit_first(z + 1);
            }
            bool ok = true;
            while (ok && acq <= st + 1) {
                ok = acquire(acq);
                if (ok) ++acq;
            }
            if (__any_sync(FULL, !ok)) {
                if (lane == 0) atomicExch(status, 1);
                dead = true;
                issued = st + 3 < nplanes ? st + 3 : nplanes;
                break;
            }
            if (count_now != 0) {
                const T* a0 = ring + (size_t)(st % 3u) * plane_elems + 8 * lane;
                const T* a1 = a0 + row_elems;
                const T* b0 = ring + (size_t)((st + 1) % 3u) * plane_elems + 8 * lane;
                const T* b1 = b0 + row_elems;
                uint32_t m[4] = {0, 0, 0, 0};   // per staged row: node above bits of this lane's 9 nodes
#pragma unroll
                for (int k = 0; k < 9; ++k) {
                    m[0] |= (above(j.cls, a0[k]) ? 1u : 0u) << k;
                    m[1] |= (above(j.cls, a1[k]) ? 1u : 0u) << k;
                    m[2] |= (above(j.cls, b0[k]) ? 1u : 0u) << k;
                    m[3] |= (above(j.cls, b1[k]) ? 1u : 0u) << k;
                }
                // the 8 cells' cases (corners 0:(x,y,z) 1:(x+1,y,z) 2:(x+1,y+1,z)
                // 3:(x,y+1,z), 4..7 the same at z+1), byte i = cell i: byte b of
                // the word below holds case bit b of the 8 cells, and an 8x8 bit
                // transpose turns it into one case per byte
                uint64_t cw =
                    (uint64_t)((m[0] & 0xffu) | (((m[0] >> 1) & 0xffu) << 8) | (((m[1] >> 1) & 0xffu) << 16) |
                               ((m[1] & 0xffu) << 24)) |
                    ((uint64_t)((m[2] & 0xffu) | (((m[2] >> 1) & 0xffu) << 8) | (((m[3] >> 1) & 0xffu) << 16) |
                                ((m[3] & 0xffu) << 24))
                     << 32);
                uint64_t tt = (cw ^ (cw >> 7)) & 0x00AA00AA00AA00AAull;
                cw ^= tt ^ (tt << 7);
                tt = (cw ^ (cw >> 14)) & 0x0000CCCC0000CCCCull;
                cw ^= tt ^ (tt << 14);
                tt = (cw ^ (cw >> 28)) & 0x00000000F0F0F0F0ull;
                cw ^= tt ^ (tt << 28);
                if (lim < 8) cw &= lim <= 0 ? 0ull : (~0ull >> (64 - 8 * lim));   // cells past the row: none
                const uint32_t clo = (uint32_t)cw, chi = (uint32_t)(cw >> 32);     // cells 0-3, 4-7
                uint32_t n = 0;
#pragma unroll
                for (int i = 0; i < 8; ++i) n += s_ntri[((i < 4 ? clo : chi) >> (8 * (i & 3))) & 0xffu];
                uint32_t inc = n;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t t = __shfl_up_sync(FULL, inc, o);
                    if (lane >= (unsigned)o) inc += t;
                }
                const uint32_t total = __shfl_sync(FULL, inc, 31);
                // the step's triangles spread over the lanes: triangle q belongs to the
                // first lane whose inclusive count exceeds q (binary search over lanes)
                for (uint32_t q0 = 0; q0 < total; q0 += 32) {
                    const uint32_t q = q0 + lane;
                    uint32_t lo = 0;
#pragma unroll
                    for (int b = 4; b >= 0; --b) {
                        const uint32_t mid = lo + (1u << b) - 1u;
                        const uint32_t im = __shfl_sync(FULL, inc, mid);
                        if (im <= q) lo = mid + 1;
                    }
                    const uint32_t owner = lo < 32 ? lo : 31;
                    const uint32_t first = __shfl_sync(FULL, inc - n, owner);
                    const uint32_t olo = __shfl_sync(FULL, clo, owner), ohi = __shfl_sync(FULL, chi, owner);
                    uint32_t oc[8];
#pragma unroll
                    for (int i = 0; i < 8; ++i) oc[i] = ((i < 4 ? olo : ohi) >> (8 * (i & 3))) & 0xffu;
                    if (q < total) {
                        // the owner's cell and triangle of local triangle r
                        uint32_t r = q - first, ci = 0, c = oc[0];
#pragma unroll
                        for (int i = 0; i < 8; ++i) {
                            const uint32_t nt = s_ntri[oc[i]];
                            if (ci == (uint32_t)i && r >= nt) { r -= nt; ci = i + 1; }
                        }
#pragma unroll
                        for (int i = 0; i < 8; ++i) if ((uint32_t)i == ci) c = oc[i];
                        const uint64_t pk = s_tri[c] >> (12 * r);
                        const uint32_t x = (uint32_t)xoff + 8 * owner + ci;
                        const uint64_t t = tbase + q;
                        uint32_t id[3];
                        bool good = true;
#pragma unroll
                        for (int e = 0; e < 3; ++e) {
                            const unsigned ep = s_edge[(pk >> (4 * e)) & 15u];
                            const unsigned ca = ep & 7u, cb = ep >> 3;
                            const unsigned nd = ca & cb, d = ca ^ cb;   // lower node, axis bit
                            const int axis = d == 1u ? 0 : (d == 2u ? 1 : 2);
                            id[e] = sc_rank_id(j, x + (nd & 1u), y + ((nd >> 1) & 1u), z + (nd >> 2), axis);
                            good = good && id[e] < nvert;
                        }
                        if (t >= ntri) {
                            atomicExch(status, 2);   // never with the count's offsets; nothing written out of range
                            continue;
                        }
                        uint32_t* o = j.connections + 3 * t;
                        o[0] = id[0]; o[1] = id[1]; o[2] = id[2];
                        if (!good) {
                            atomicExch(status, 2);   // never with consistent rank words; nothing read out of range
                        } else if (tri_out) {
                            const float* p0 = j.coords + 3 * (uint64_t)id[0];
                            const float* p1 = j.coords + 3 * (uint64_t)id[1];
                            const float* p2 = j.coords + 3 * (uint64_t)id[2];
                            const float3 nn = tri_normal(make_float3(p0[0], p0[1], p0[2]),
                                                         make_float3(p1[0], p1[1], p1[2]),
                                                         make_float3(p2[0], p2[1], p2[2]));
                            float* qn = tri_out + 3 * t;
                            qn[0] = nn.x; qn[1] = nn.y; qn[2] = nn.z;
                        }
                    }
                }
            }
            __syncwarp();
            if (lane == 0 && st + 3 < nplanes) {
                fence_proxy_async();
                issue(st + 3);
            }
        }
        if (dead) {
            for (uint32_t i = acq; i < issued; ++i) {
                const uint32_t b = i % 3u;
                if (mbar_wait(&bar[b], (ph >> b) & 1u, 1u << 16)) ph ^= 1u << b;
            }
            break;
        }
    }
}


// ------------------------------------------------------------------
// connect_isopoints for up to kStreamMaxIso requests on one volume in one pass
// (the requests of one streaming count group): the cell tasks of k_sconnect,
// each cell classified once for all the requests by threshold masks, the
// step's active (cell, request) pairs taken 32 at a time, one lane per
// triangle.  Every request's connections and normals are the ones its own
// connection pass writes.

constexpr int kScPairCap = 128;   // listed (cell, request) pairs per warp at a time

struct ScMultiCta {
    ThermoTables th;
    ConnIso iso[kStreamMaxIso];
    uint64_t tri[256];   // per reference case: edges per triangle, 4 bits each
    uint8_t ntri[256];
    uint8_t edge[16];
};

struct ScMultiWarp {
    uint32_t pairs[kScPairCap];   // cell | request << 8 | corner code << 16
    uint32_t run[kStreamMaxIso];  // per request: triangles of the unit written so far this step
    uint32_t add[kStreamMaxIso];
    uint8_t item[32 * 5];         // triangle -> its pair's lane, one round
};

// Vertex id of node (x, y, z)'s edge along `axis` from a request's rank words.
__device__ __forceinline__ uint32_t sc_rank_id_of(const uint4* rank, uint32_t ny, uint32_t words_per_row, uint32_t x,
                                                  uint32_t y, uint32_t z, int axis)
{
    const uint4 R = rank[((uint64_t)z * ny + y) * words_per_row + (x >> 5)];
    const uint32_t bit = x & 31u, lt = (1u << bit) - 1u;
    uint32_t id = R.w + __popc(R.x & lt) + __popc(R.y & lt) + __popc(R.z & lt);
    if (axis >= 1) id += (R.x >> bit) & 1u;
    if (axis >= 2) id += (R.y >> bit) & 1u;
    return id;
}

template <typename T>
__global__ void __launch_bounds__(kSnThreads, 3)
    k_sconnect_multi(const StreamGroup* __restrict__ groups, const StreamIso* __restrict__ isos,
                     const ConnIso* __restrict__ conn, const uint16_t* __restrict__ unit_counts,
                     const uint32_t* __restrict__ unit_offsets, const uint64_t* __restrict__ plane_base,
                     uint64_t ntasks, int* __restrict__ status, unsigned long long* __restrict__ next_task,
                     uint32_t wait_polls)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const StreamGroup& G = groups[0];
    const int niso = G.niso;
    const float bs = G.bs, bo = G.bo;
    ScMultiCta& C = *reinterpret_cast<ScMultiCta*>(smem_raw);
    const uint32_t row_elems = G.seg_elems;
    const size_t plane_elems = 2 * (size_t)row_elems;
    const size_t ring_bytes = sn_align(3 * plane_elems * sizeof(T));
    unsigned char* wbase =
        smem_raw + sn_align(sizeof(ScMultiCta)) + (size_t)warp * (128 + ring_bytes + sn_align(sizeof(ScMultiWarp)));
    uint64_t* bar = reinterpret_cast<uint64_t*>(wbase);
    T* ring = reinterpret_cast<T*>(wbase + 128);
    ScMultiWarp& W = *reinterpret_cast<ScMultiWarp*>(wbase + 128 + ring_bytes);
    for (unsigned c = tid; c < 256; c += blockDim.x) {
        C.tri[c] = c_sc_tri[c];
        C.ntri[c] = c_sc_ntri[c];
        if (c < 12) C.edge[c] = c_sc_edge[c];
        if (c < (unsigned)niso) C.iso[c] = conn[c];
    }
    if (warp == 0) {
        __shared__ float s_thr[kStreamMaxIso];
        if (lane < (unsigned)niso) s_thr[lane] = isos[G.iso_begin + lane].f.f_thr;
        __syncwarp();
        thermo_build(C.th, s_thr, niso, bs, bo, lane);
    }
    __syncthreads();   // the only CTA-wide barrier: the tables are read-only from here on
    if (lane == 0) {
        for (int b = 0; b < 3; ++b) mbar_init(&bar[b], 1);
        fence_barrier_init();
    }
    if (lane < (unsigned)kStreamMaxIso) {
        W.run[lane] = 0;
        W.add[lane] = 0;
    }
    __syncwarp();
    const uint32_t nx = G.vol.nx, cx = G.vol.nx - 1, cy = G.vol.ny - 1, cz = G.vol.nz - 1;
    const uint32_t ny = G.vol.ny;
    const uint32_t wpr = G.wpr, words_per_row = (nx + 31) / 32;
    const uint64_t pitch = G.vol.pitch, slice = G.vol.slice;
    const T* vol = static_cast<const T*>(G.vol.data);
    const unsigned lt = (1u << lane) - 1u;
    // lane k < niso: request k's first (isolevel, z) plane of the scans
    const uint64_t my_plane = lane < (unsigned)niso ? isos[G.iso_begin + lane].plane_index : 0;
    const uint64_t my_plane0 = lane < (unsigned)niso ? plane_base[my_plane] : 0;
    const bool my_on = lane < (unsigned)niso && C.iso[lane].enabled;
    uint32_t ph = 0;
    for (;;) {
        unsigned long long tk = 0;
        if (lane == 0) tk = atomicAdd(next_task, 1ull);
        const uint64_t task = __shfl_sync(FULL, tk, 0);
        if (task >= ntasks) break;
        const uint32_t seg = (uint32_t)(task % wpr);
        const uint32_t y = (uint32_t)((task / wpr) % cy);
        const uint32_t zc = (uint32_t)(task / ((uint64_t)wpr * cy));
        const uint32_t z0 = zc * G.zchunk;
        const uint32_t z1 = z0 + G.zchunk < cz ? z0 + G.zchunk : cz;   // cell planes [z0, z1)
        const uint32_t nplanes = z1 - z0 + 1;
        const uint64_t xoff = (uint64_t)seg * 256;
        const uint64_t avail = (pitch - xoff) * sizeof(T);
        const uint32_t row_bytes = (uint32_t)(avail < G.seg_copy_bytes ? avail : G.seg_copy_bytes);
        auto issue = [&](uint32_t i) {
            const int b = (int)(i % 3u);
            T* dst = ring + (size_t)b * plane_elems;
            const T* src = vol + (uint64_t)(z0 + i) * slice + (uint64_t)y * pitch + xoff;
            mbar_arrive_expect_tx(&bar[b], 2 * row_bytes);
            for (uint32_t r = 0; r < 2; ++r) bulk_copy_g2s(dst + r * row_elems, src + r * pitch, row_bytes, &bar[b]);
        };
        auto acquire = [&](uint32_t i) -> bool {
            const uint32_t b = i % 3u;
            const bool ok = mbar_wait(&bar[b], (ph >> b) & 1u, wait_polls);
            if (ok) ph ^= 1u << b;
            return ok;
        };
        __syncwarp();
        if (lane == 0) {
            fence_proxy_async();
            for (uint32_t i = 0; i < nplanes && i < 3; ++i) issue(i);
        }
        uint32_t acq = 0, issued = 0;
        bool dead = false;
        const uint32_t xl = 8 * lane;                         // this lane's first cell in the segment
        const int lim = (int)cx - (int)((uint32_t)xoff + xl);  // its cells inside the row (if < 8)
        // lane k: request k's triangle count and first triangle of the unit, one step ahead
        auto unit_elem = [&](uint32_t zz) -> uint64_t {
            return G.unit_base + (((uint64_t)zz * cy + y) * wpr + seg) * niso + lane;
        };
        uint32_t next_n = my_on ? unit_counts[unit_elem(z0)] : 0u;
        uint64_t next_first = my_on ? plane_base[my_plane + z0] - my_plane0 + unit_offsets[unit_elem(z0)] : 0;
        for (uint32_t z = z0; z < z1; ++z) {
            const uint32_t st = z - z0;
            const uint32_t n_now = next_n;
            const uint64_t first_now = next_first;
            if (z + 1 < z1 && my_on) {
                next_n = unit_counts[unit_elem(z + 1)];
                next_first = plane_base[my_plane + z + 1] - my_plane0 + unit_offsets[unit_elem(z + 1)];
            }
            bool ok = true;
            while (ok && acq <= st + 1) {
                ok = acquire(acq);
                if (ok) ++acq;
            }
            if (__any_sync(FULL, !ok)) {
                if (lane == 0) atomicExch(status, 1);
                dead = true;
                issued = st + 3 < nplanes ? st + 3 : nplanes;
                break;
            }
            const uint32_t act_iso = __ballot_sync(FULL, n_now != 0) & ((1u << niso) - 1u);
            if (act_iso) {
                const T* pa = ring + (size_t)(st % 3u) * plane_elems;
                const T* pb = ring + (size_t)((st + 1) % 3u) * plane_elems;
                // threshold masks of this lane's 9 nodes in the 4 staged rows,
                // two nodes per word (node 2m low, 2m + 1 high; word 4 = node 8)
                uint32_t P[4][5];
#pragma unroll
                for (int r = 0; r < 4; ++r) {
                    const T* row = (r < 2 ? pa : pb) + (r & 1) * row_elems + xl;
                    uint32_t e[9];
#pragma unroll
                    for (int i = 0; i < 9; ++i) e[i] = thermo_mask(C.th, niso, bs, bo, (float)row[i]);
                    P[r][0] = e[0] | (e[1] << 16);
                    P[r][1] = e[2] | (e[3] << 16);
                    P[r][2] = e[4] | (e[5] << 16);
                    P[r][3] = e[6] | (e[7] << 16);
                    P[r][4] = e[8];
                }
                // per cell: the requests (with triangles in this unit) whose
                // isolevel lies between its lowest and highest corner
                const uint32_t want = act_iso | (act_iso << 16);
                uint32_t act[4];
                uint32_t m = 0;
#pragma unroll
                for (int w = 0; w < 4; ++w) {
                    const uint32_t co0 = P[0][w] | P[1][w] | P[2][w] | P[3][w];
                    const uint32_t co1 = P[0][w + 1] | P[1][w + 1] | P[2][w + 1] | P[3][w + 1];
                    const uint32_t ca0 = P[0][w] & P[1][w] & P[2][w] & P[3][w];
                    const uint32_t ca1 = P[0][w + 1] & P[1][w + 1] & P[2][w + 1] & P[3][w + 1];
                    const uint32_t o = co0 | __funnelshift_r(co0, co1, 16);
                    const uint32_t a = ca0 & __funnelshift_r(ca0, ca1, 16);
                    uint32_t keep = want;
                    if (2 * w >= lim) keep &= 0xffff0000u;
                    if (2 * w + 1 >= lim) keep &= 0x0000ffffu;
                    act[w] = o & ~a & keep;
                    m += __popc(act[w]);
                }
                uint32_t inc = m;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t t = __shfl_up_sync(FULL, inc, o);
                    if (lane >= (unsigned)o) inc += t;
                }
                const uint32_t npairs = __shfl_sync(FULL, inc, 31);
                const uint32_t my_first = inc - m;
                for (uint32_t fill0 = 0; fill0 < npairs; fill0 += kScPairCap) {
                    // this lane's pairs (cell order, then request) that fall into
                    // [fill0, fill0 + kScPairCap)
                    if (m && my_first < fill0 + kScPairCap && my_first + m > fill0) {
                        uint32_t slot = my_first;
#pragma unroll
                        for (int i = 0; i < 8; ++i) {
                            uint32_t am = (act[i >> 1] >> (16 * (i & 1))) & 0xffffu;
                            if (am) {
                                const uint32_t w0 = cell_word(P[0], i), w1 = cell_word(P[1], i);
                                const uint32_t w2 = cell_word(P[2], i), w3 = cell_word(P[3], i);
                                do {
                                    const uint32_t k = __ffs(am) - 1;
                                    am &= am - 1;
                                    if (slot >= fill0 && slot < fill0 + kScPairCap)
                                        W.pairs[slot - fill0] =
                                            (xl + i) | (k << 8) | (code_to_case(case_code(w0, w1, w2, w3, k)) << 16);
                                    ++slot;
                                } while (am);
                            }
                        }
                    }
                    __syncwarp();
                    const uint32_t nfill = npairs - fill0 < (uint32_t)kScPairCap ? npairs - fill0 : (uint32_t)kScPairCap;
                    for (uint32_t r0 = 0; r0 < nfill; r0 += 32) {
                        // one pair per lane; its first triangle: the request's running
                        // count in the unit plus the triangles of the earlier lanes with
                        // the same request
                        const uint32_t p = r0 + lane;
                        const bool has = p < nfill;
                        const uint32_t pe = has ? W.pairs[p] : 0u;
                        const uint32_t k = (pe >> 8) & 0xffu, cs = pe >> 16;
                        const uint32_t nt = has ? C.ntri[cs] : 0u;
                        const uint32_t grp = __match_any_sync(FULL, has ? (int)k : 32 + (int)lane);
                        uint32_t pre = 0, gtot = 0, tpre = 0, ntr = 0;
#pragma unroll
                        for (int bit = 0; bit < 3; ++bit) {
                            const uint32_t bm = __ballot_sync(FULL, (nt >> bit) & 1u);
                            pre += (uint32_t)__popc(bm & grp & lt) << bit;
                            gtot += (uint32_t)__popc(bm & grp) << bit;
                            tpre += (uint32_t)__popc(bm & lt) << bit;
                            ntr += (uint32_t)__popc(bm) << bit;
                        }
                        const uint64_t kfirst = __shfl_sync(FULL, first_now, k);
                        const uint64_t obase = kfirst + (has ? W.run[k] : 0u) + pre;
                        __syncwarp();
                        if (has && (31 - __clz(grp)) == (int)lane) W.add[k] = gtot;
                        for (uint32_t t = 0; t < nt; ++t) W.item[tpre + t] = (uint8_t)lane;
                        __syncwarp();
                        if (lane < (unsigned)kStreamMaxIso) {
                            W.run[lane] += W.add[lane];
                            W.add[lane] = 0;
                        }
                        __syncwarp();
                        for (uint32_t j0 = 0; j0 < ntr; j0 += 32) {
                            const uint32_t jj = j0 + lane;
                            const bool ht = jj < ntr;
                            const uint32_t q = ht ? W.item[jj] : 0u;
                            const uint32_t qe = __shfl_sync(FULL, pe, q);
                            const uint32_t qt = __shfl_sync(FULL, tpre, q);
                            const uint64_t qo = __shfl_sync(FULL, obase, q);
                            if (!ht) continue;
                            const uint32_t qk = (qe >> 8) & 0xffu, qc = qe >> 16;
                            const uint32_t t = jj - qt;
                            const uint64_t tt = qo + t;
                            const ConnIso& R = C.iso[qk];
                            const uint64_t pk = C.tri[qc] >> (12 * t);
                            const uint32_t x = (uint32_t)xoff + (qe & 0xffu);
                            uint32_t id[3];
                            bool good = true;
#pragma unroll
                            for (int e = 0; e < 3; ++e) {
                                const unsigned ep = C.edge[(pk >> (4 * e)) & 15u];
                                const unsigned ca = ep & 7u, cb = ep >> 3;
                                const unsigned nd = ca & cb, d = ca ^ cb;   // lower node, axis bit
                                const int axis = d == 1u ? 0 : (d == 2u ? 1 : 2);
                                id[e] = sc_rank_id_of(R.rank, ny, words_per_row, x + (nd & 1u), y + ((nd >> 1) & 1u),
                                                      z + (nd >> 2), axis);
                                good = good && id[e] < R.nvert;
                            }
                            if (tt >= R.ntri) {
                                atomicExch(status, 2);   // never with the count's offsets; nothing written out of range
                                continue;
                            }
                            uint32_t* o = R.connections + 3 * tt;
                            o[0] = id[0]; o[1] = id[1]; o[2] = id[2];
                            if (!good) {
                                atomicExch(status, 2);   // never with consistent rank words; nothing read out of range
                            } else if (R.tri_out) {
                                const float* p0 = R.coords + 3 * (uint64_t)id[0];
                                const float* p1 = R.coords + 3 * (uint64_t)id[1];
                                const float* p2 = R.coords + 3 * (uint64_t)id[2];
                                const float3 nn = tri_normal(make_float3(p0[0], p0[1], p0[2]),
                                                             make_float3(p1[0], p1[1], p1[2]),
                                                             make_float3(p2[0], p2[1], p2[2]));
                                float* qn = R.tri_out + 3 * tt;
                                qn[0] = nn.x; qn[1] = nn.y; qn[2] = nn.z;
                            }
                        }
                        __syncwarp();
                    }
                    __syncwarp();
                }
                if (lane < (unsigned)kStreamMaxIso) W.run[lane] = 0;
                __syncwarp();
            }
            __syncwarp();
            if (lane == 0 && st + 3 < nplanes) {
                fence_proxy_async();
                issue(st + 3);
            }
        }
        if (dead) {
            for (uint32_t i = acq; i < issued; ++i) {
                const uint32_t b = i % 3u;
                if (mbar_wait(&bar[b], (ph >> b) & 1u, 1u << 16)) ph ^= 1u << b;
            }
            break;
        }
    }
}

}  // namespace

size_t sconnect_shared_bytes(int dtype)
{
    const size_t es = dtype_size(dtype);
    const size_t plane = 2 * stream_row_elems(dtype, 1) * es;
    return (size_t)kSnWarps * (128 + sn_align(3 * plane));
}

cudaError_t launch_sconnect(const Job& j, const StreamGroup* d_groups, const StreamIso* d_isos,
                            const uint16_t* unit_counts, const uint32_t* unit_offsets, const uint64_t* plane_base,
                            uint32_t iso_k, uint64_t ntasks, uint64_t nvert, uint64_t ntri, int* status,
                            unsigned long long* next_task, const Launch& L)
{
    if (ntasks == 0) return cudaSuccess;
    const int dt = j.vol.dtype;
    const size_t smem = sconnect_shared_bytes(dt);
    KVSMC_SN_SWITCH(dt, {
        auto kern = k_sconnect<T>;
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        int per_sm = 0;
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kSnThreads, smem);
        if (e != cudaSuccess) return e;
        const uint64_t resident = (uint64_t)(per_sm > 0 ? per_sm : 1) * (uint64_t)L.num_sms;
        const uint64_t need = (ntasks + kSnWarps - 1) / kSnWarps;
        const uint64_t nctas = need < resident ? need : resident;
        prof_begin(L, "sconnect");
        kern<<<(unsigned)nctas, kSnThreads, smem, L.stream>>>(j, d_groups, d_isos, unit_counts, unit_offsets,
                                                                plane_base, iso_k, ntasks, nvert, ntri, status,
                                                                next_task, L.wait_polls[1]);
        prof_end(L);
    });
    *L.counter += 1;
    return cudaGetLastError();
}

size_t sconnect_multi_shared_bytes(int dtype)
{
    const size_t es = dtype_size(dtype);
    const size_t plane = 2 * stream_row_elems(dtype, 1) * es;
    return sn_align(sizeof(ScMultiCta)) + (size_t)kSnWarps * (128 + sn_align(3 * plane) + sn_align(sizeof(ScMultiWarp)));
}

cudaError_t launch_sconnect_multi(const StreamGroup* d_group, const StreamIso* d_isos, const ConnIso* d_conn, int dtype,
                                  const uint16_t* unit_counts, const uint32_t* unit_offsets, const uint64_t* plane_base,
                                  uint64_t ntasks, int* status, unsigned long long* next_task, const Launch& L)
{
    if (ntasks == 0) return cudaSuccess;
    const size_t smem = sconnect_multi_shared_bytes(dtype);
    KVSMC_SN_SWITCH(dtype, {
        auto kern = k_sconnect_multi<T>;
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        int per_sm = 0;
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kSnThreads, smem);
        if (e != cudaSuccess) return e;
        const uint64_t resident = (uint64_t)(per_sm > 0 ? per_sm : 1) * (uint64_t)L.num_sms;
        const uint64_t need = (ntasks + kSnWarps - 1) / kSnWarps;
        const uint64_t nctas = need < resident ? need : resident;
        prof_begin(L, "sconnect_multi");
        kern<<<(unsigned)nctas, kSnThreads, smem, L.stream>>>(d_group, d_isos, d_conn, unit_counts, unit_offsets,
                                                                plane_base, ntasks, status, next_task, L.wait_polls[1]);
        prof_end(L);
    });
    *L.counter += 1;
    return cudaGetLastError();
}

size_t snode_shared_bytes(int dtype)
{
    const size_t es = dtype_size(dtype);
    const size_t plane = 2 * stream_row_elems(dtype, 1) * es;
    return (size_t)kSnWarps * (128 + sn_align(3 * plane));
}

size_t snode_multi_shared_bytes(int dtype)
{
    const size_t es = dtype_size(dtype);
    const size_t plane = 2 * stream_row_elems(dtype, 1) * es;
    return sn_align(sizeof(SnMultiCta)) + (size_t)kSnWarps * (128 + sn_align(3 * plane) + sn_align(sizeof(SnMulti)));
}

cudaError_t launch_snode_multi(const VolumeView& vol, const NodeIso* d_isos, int niso, float bs, float bo,
                               uint32_t wprn, uint32_t zchunk, uint64_t ntasks, uint32_t words_per_row, int* status,
                               unsigned long long* next_task, const Launch& L)
{
    if (ntasks == 0) return cudaSuccess;
    if (niso < 1 || niso > kStreamMaxIso) return cudaErrorInvalidValue;
    const int dt = vol.dtype;
    const size_t smem = snode_multi_shared_bytes(dt);
    const uint32_t row_elems = (uint32_t)stream_row_elems(dt, 1);
    const uint32_t copy_bytes = row_elems * (uint32_t)dtype_size(dt);
    KVSMC_SN_SWITCH(dt, {
        auto kern = k_snode_multi<T>;
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        int per_sm = 0;
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kSnThreads, smem);
        if (e != cudaSuccess) return e;
        const uint64_t resident = (uint64_t)(per_sm > 0 ? per_sm : 1) * (uint64_t)L.num_sms;
        const uint64_t need = (ntasks + kSnWarps - 1) / kSnWarps;
        const uint64_t nctas = need < resident ? need : resident;
        prof_begin(L, "snode_emit_multi");
        kern<<<(unsigned)nctas, kSnThreads, smem, L.stream>>>(vol, d_isos, niso, bs, bo, wprn, zchunk, ntasks,
                                                                row_elems, copy_bytes, words_per_row, status,
                                                                next_task, L.wait_polls[1]);
        prof_end(L);
    });
    *L.counter += 1;
    return cudaGetLastError();
}

cudaError_t launch_snode(bool emit, const Job& j, const FastIso& f, uint32_t wprn, uint32_t zchunk, uint64_t ntasks,
                         uint32_t* unit_counts, const uint64_t* unit_offsets, int* status,
                         unsigned long long* next_task, const Launch& L)
{
    if (ntasks == 0) return cudaSuccess;
    const int dt = j.vol.dtype;
    const size_t smem = snode_shared_bytes(dt);
    const uint32_t row_elems = (uint32_t)stream_row_elems(dt, 1);
    const uint32_t copy_bytes = row_elems * (uint32_t)dtype_size(dt);
    KVSMC_SN_SWITCH(dt, {
        auto kern = emit ? k_snode<T, true> : k_snode<T, false>;
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        int per_sm = 0;
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kSnThreads, smem);
        if (e != cudaSuccess) return e;
        const uint64_t resident = (uint64_t)(per_sm > 0 ? per_sm : 1) * (uint64_t)L.num_sms;
        const uint64_t need = (ntasks + kSnWarps - 1) / kSnWarps;
        const uint64_t nctas = need < resident ? need : resident;
        prof_begin(L, emit ? "snode_emit" : "snode_count");
        kern<<<(unsigned)nctas, kSnThreads, smem, L.stream>>>(j, f, wprn, zchunk, ntasks, row_elems, copy_bytes,
                                                                unit_counts, unit_offsets, status, next_task,
                                                                L.wait_polls[emit ? 1 : 0]);
        prof_end(L);
    });
    *L.counter += 1;
    return cudaGetLastError();
}

}  // namespace kvsmc
