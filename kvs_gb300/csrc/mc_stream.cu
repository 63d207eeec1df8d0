// mc_stream.cu -- the streaming kernels: duplicated-vertex extraction of many
// (volume, isolevel) requests in two fused launches (count, emit).
//
// Work decomposition (one CTA = 16 warps):
//   * A CTA owns `rows` consecutive cell rows (a y-tile) of one volume and a
//     chunk of cell planes, and walks z.  Node planes arrive in shared memory
//     through TMA bulk copies (cp.async.bulk, one per node row) into a ring of
//     three buffers guarded by mbarriers, so every node row is read from HBM
//     once per pass while the next plane is in flight.
//   * Warp w handles a 256-cell segment of one row (8 cells per lane).  For
//     each cell it takes the min/max of the 8 corners and looks up the range
//     [lo, hi) of isolevels (sorted by threshold) the cell is active for: a
//     cell is active for t exactly when min <= t < max, and the lookup is a
//     bucket table plus exact compares.  Only active (cell, isolevel) pairs
//     are classified further.
//   * count: per-warp, per-isolevel triangle counts -> one count per
//     (isolevel, z, y-tile) tile, in the reference's linear cell order.
//   * emit: the warps of a z-step exchange their counts, so each warp knows
//     where its segment's triangles start for every isolevel; it then
//     compacts its active pairs (warp scan), interpolates each pair's edges
//     once (work spread over all lanes), and writes each triangle (one lane
//     per triangle) at its position: cells in linear order, table order
//     inside a cell, isolevels into their own arrays.
#include <cuda_runtime.h>

#include "mc_internal.h"
#include "mc_interp.cuh"

namespace kvsmc {

namespace {

constexpr int kWarps = kStreamThreads / 32;
constexpr int kLaneCells = 8;
constexpr int kSegCells = 32 * kLaneCells;
constexpr int kPairCap = 256;   // pair buffer entries per warp
constexpr int kEdgeCap = 96;    // vertex slots per warp and round
constexpr unsigned FULL = 0xffffffffu;

__constant__ uint64_t c_tri_packed[256] = MC_TRI_PACKED_INIT;
__constant__ uint8_t c_ntri[256] = MC_NTRI_INIT;
__constant__ uint16_t c_edge_mask[256] = MC_EDGE_MASK_INIT;
__constant__ uint8_t c_edge_packed[12] = MC_EDGE_PACKED_INIT;

// ------------------------------------------------------------ TMA + mbarrier

__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_barrier_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait: false after `limit` polls (each poll may suspend the thread
// for a while inside try_wait).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit)
{
    for (uint32_t i = 0; i < limit; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// ------------------------------------------------------------ value access

template <typename T> __device__ __forceinline__ float cls_value(T v) { return (float)v; }
template <> __device__ __forceinline__ float cls_value<float>(float v) { return v != v ? -INFINITY : v; }

// 8 consecutive values of a shared-memory row as floats (x0 multiple of 8).
template <typename T> __device__ __forceinline__ void load8(const T* row, uint32_t x0, float* o);
template <> __device__ __forceinline__ void load8<float>(const float* row, uint32_t x0, float* o)
{
    const float4 a = *reinterpret_cast<const float4*>(row + x0);
    const float4 b = *reinterpret_cast<const float4*>(row + x0 + 4);
    o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w; o[4] = b.x; o[5] = b.y; o[6] = b.z; o[7] = b.w;
}
template <> __device__ __forceinline__ void load8<uint16_t>(const uint16_t* row, uint32_t x0, float* o)
{
    const uint4 a = *reinterpret_cast<const uint4*>(row + x0);
    const uint32_t w[4] = {a.x, a.y, a.z, a.w};
#pragma unroll
    for (int i = 0; i < 4; ++i) { o[2 * i] = (float)(w[i] & 0xffffu); o[2 * i + 1] = (float)(w[i] >> 16); }
}
template <> __device__ __forceinline__ void load8<int16_t>(const int16_t* row, uint32_t x0, float* o)
{
    const uint4 a = *reinterpret_cast<const uint4*>(row + x0);
    const uint32_t w[4] = {a.x, a.y, a.z, a.w};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        o[2 * i] = (float)(int16_t)(w[i] & 0xffffu);
        o[2 * i + 1] = (float)(int16_t)(w[i] >> 16);
    }
}
template <> __device__ __forceinline__ void load8<uint8_t>(const uint8_t* row, uint32_t x0, float* o)
{
    const uint2 a = *reinterpret_cast<const uint2*>(row + x0);
#pragma unroll
    for (int i = 0; i < 4; ++i) { o[i] = (float)((a.x >> (8 * i)) & 255u); o[4 + i] = (float)((a.y >> (8 * i)) & 255u); }
}
template <> __device__ __forceinline__ void load8<int8_t>(const int8_t* row, uint32_t x0, float* o)
{
    const uint2 a = *reinterpret_cast<const uint2*>(row + x0);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        o[i] = (float)(int8_t)((a.x >> (8 * i)) & 255u);
        o[4 + i] = (float)(int8_t)((a.y >> (8 * i)) & 255u);
    }
}

// ------------------------------------------------------------ shared layout

struct Shared {
    uint64_t bar[3];
    uint64_t tri_packed[256];
    uint64_t wbase[kWarps][kStreamMaxIso];   // emit: first output triangle of each warp, per isolevel
    uint64_t tile_base[kStreamMaxIso];       // emit: first triangle of the current tile, per isolevel
    uint64_t iso_first[kStreamMaxIso];
    FastIso fast[kStreamMaxIso];
    Interp ip[kStreamMaxIso];
    float* coords[kStreamMaxIso];
    float* normals[kStreamMaxIso];
    uint64_t count_base[kStreamMaxIso];
    float thr[kStreamMaxIso];
    int32_t thr_bucket[kStreamMaxIso];
    uint32_t wcnt[kWarps][kStreamMaxIso];    // per-warp triangle counts of the current z-step
    uint32_t wrun[kWarps][kStreamMaxIso];    // emit: running triangle offset inside the warp's segment
    uint16_t edge_mask[256];
    uint8_t ntri[256];
    uint8_t edge_packed[16];
    uint8_t bucket[kStreamBuckets + 3];
    int32_t group;
    int32_t dead;
};

struct EmitShared {
    uint32_t pairs[kWarps][kPairCap];
    float3 vtx[kWarps][kEdgeCap];
};

// Monotone (non-decreasing) bucket of a value; thresholds and cell values go
// through exactly this function, so #{t < v} = #{t in lower buckets} + the
// exact compares inside v's own bucket.
__device__ __forceinline__ int bucket_of(const StreamGroup& G, float v)
{
    float fb = floorf(__fmul_rn(__fsub_rn(v, G.bt0), G.bscale));
    if (!(fb >= -1.0f)) fb = -1.0f;
    if (fb > (float)(kStreamBuckets + 1)) fb = (float)(kStreamBuckets + 1);
    return (int)fb;
}

// Number of thresholds strictly below v.
__device__ __forceinline__ int count_below(const Shared& S, const StreamGroup& G, float v)
{
    const int b = bucket_of(G, v);
    const unsigned e = S.bucket[b + 1];
    int k = (int)(e & 0x3fu);
    if (e & 0x80u) {
        while (k < G.niso && S.thr_bucket[k] == b && S.thr[k] < v) ++k;
    }
    return k;
}

__device__ __forceinline__ unsigned case_of(const float* a0, const float* a1, const float* b0, const float* b1, int i,
                                            float t)
{
    return (a0[i] > t ? 1u : 0u) | (a0[i + 1] > t ? 2u : 0u) | (a1[i + 1] > t ? 4u : 0u) | (a1[i] > t ? 8u : 0u) |
           (b0[i] > t ? 16u : 0u) | (b0[i + 1] > t ? 32u : 0u) | (b1[i + 1] > t ? 64u : 0u) |
           (b1[i] > t ? 128u : 0u);
}

template <typename T, bool EMIT>
__global__ void __launch_bounds__(kStreamThreads, 1)
    k_stream(const StreamGroup* __restrict__ groups, int ngroups, const StreamIso* __restrict__ isos,
             uint32_t* __restrict__ counts,
             const uint64_t* __restrict__ offsets, int* __restrict__ status)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    Shared& S = *reinterpret_cast<Shared*>(smem_raw);
    EmitShared* ES = reinterpret_cast<EmitShared*>(smem_raw + ((sizeof(Shared) + 127) / 128) * 128);
    const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;

    if (tid == 0) {
        int lo = 0, hi = ngroups - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (groups[mid].cta_begin <= blockIdx.x) lo = mid; else hi = mid - 1;
        }
        S.group = lo;
        S.dead = 0;
    }
    __syncthreads();
    const StreamGroup G = groups[S.group];
    const uint32_t cx = G.vol.nx - 1, cy = G.vol.ny - 1, cz = G.vol.nz - 1;
    const uint32_t local = blockIdx.x - G.cta_begin;
    const uint32_t ytile = local % G.ytiles, zc = local / G.ytiles;
    const uint32_t z0 = zc * G.zchunk;
    const uint32_t z1 = (z0 + G.zchunk < cz) ? z0 + G.zchunk : cz;   // cell planes [z0, z1)
    const uint32_t y0 = ytile * G.rows;
    const uint32_t rows_here = (cy - y0 < G.rows) ? cy - y0 : G.rows;
    const uint32_t nrows = rows_here + 1;                              // node rows per plane
    const uint64_t pitch = G.vol.pitch;
    const uint32_t row_bytes = (uint32_t)(pitch * sizeof(T));
    T* planes = reinterpret_cast<T*>(smem_raw + ((sizeof(Shared) + 127) / 128) * 128 +
                                     (EMIT ? ((sizeof(EmitShared) + 127) / 128) * 128 : 0));

    // tables
    for (unsigned i = tid; i < 256; i += blockDim.x) {
        S.tri_packed[i] = c_tri_packed[i];
        S.ntri[i] = c_ntri[i];
        S.edge_mask[i] = c_edge_mask[i];
        if (i < 12) S.edge_packed[i] = c_edge_packed[i];
    }
    if (tid < (unsigned)G.niso) {
        const StreamIso& I = isos[G.iso_begin + tid];
        S.fast[tid] = I.f;
        S.ip[tid] = I.ip;
        S.coords[tid] = I.coords;
        S.normals[tid] = I.normals;
        S.count_base[tid] = I.count_base;
        S.thr[tid] = I.f.f_thr;
        S.thr_bucket[tid] = bucket_of(G, I.f.f_thr);
        if (EMIT) S.iso_first[tid] = offsets[I.count_base];
    }
    __syncthreads();
    // bucket table: entry b+1 = #{thresholds in buckets < b} | 0x80 if bucket b holds one
    for (unsigned i = tid; i < kStreamBuckets + 3; i += blockDim.x) {
        const int b = (int)i - 1;
        unsigned below = 0, has = 0;
        for (int k = 0; k < G.niso; ++k) {
            below += S.thr_bucket[k] < b ? 1u : 0u;
            has |= S.thr_bucket[k] == b ? 1u : 0u;
        }
        S.bucket[i] = (uint8_t)(below | (has << 7));
    }
    for (unsigned i = tid; i < kWarps * kStreamMaxIso; i += blockDim.x) {
        (&S.wcnt[0][0])[i] = 0;
        (&S.wrun[0][0])[i] = 0;
    }
    if (tid == 0) {
        for (int b = 0; b < 3; ++b) mbar_init(&S.bar[b], 1);
        fence_barrier_init();
    }
    __syncthreads();

    auto issue = [&](uint32_t plane_index /* node plane z0 + i */) {
        const uint32_t i = plane_index - z0;
        const int b = (int)(i % 3u);
        T* dst = planes + (size_t)b * G.plane_elems;
        const T* src = static_cast<const T*>(G.vol.data) + (uint64_t)plane_index * G.vol.slice + (uint64_t)y0 * pitch;
        mbar_arrive_expect_tx(&S.bar[b], row_bytes * nrows);
        for (uint32_t r = 0; r < nrows; ++r) bulk_copy_g2s(dst + (size_t)r * pitch, src + (uint64_t)r * pitch, row_bytes, &S.bar[b]);
    };
    if (tid == 0) {
        for (uint32_t p = z0; p <= z1 && p < z0 + 3; ++p) issue(p);
    }

    const uint32_t wpr = G.wpr;
    const uint32_t row_l = warp / wpr, seg = warp % wpr;
    const bool warp_active = row_l < rows_here && seg * kSegCells < cx && warp < wpr * G.rows;
    const uint32_t xb = seg * kSegCells + lane * kLaneCells;
    const unsigned lt = (1u << lane) - 1u;

    uint32_t s_break = 0;
    for (uint32_t z = z0; z < z1; ++z) {
        const uint32_t s = z - z0;
        // wait for node planes z and z+1
        if (!mbar_wait(&S.bar[s % 3u], (s / 3u) & 1u, 1u << 22) ||
            !mbar_wait(&S.bar[(s + 1) % 3u], ((s + 1) / 3u) & 1u, 1u << 22)) {
            S.dead = 1;
        }
        __syncthreads();
        if (S.dead) {
            if (tid == 0) atomicExch(status, 1);
            s_break = s;
            break;
        }
        const T* pa = planes + (size_t)(s % 3u) * G.plane_elems;
        const T* pb = planes + (size_t)((s + 1) % 3u) * G.plane_elems;

        // ---------------- phase 1: classify, per-warp counts
        float a0[9], a1[9], b0[9], b1[9];
        uint32_t lohi[kLaneCells / 2] = {0, 0, 0, 0};
        if (warp_active) {
            const T* ra0 = pa + (size_t)row_l * pitch;
            const T* ra1 = ra0 + pitch;
            const T* rb0 = pb + (size_t)row_l * pitch;
            const T* rb1 = rb0 + pitch;
            load8<T>(ra0, xb, a0);
            load8<T>(ra1, xb, a1);
            load8<T>(rb0, xb, b0);
            load8<T>(rb1, xb, b1);
            float n0 = __shfl_down_sync(FULL, a0[0], 1), n1 = __shfl_down_sync(FULL, a1[0], 1);
            float n2 = __shfl_down_sync(FULL, b0[0], 1), n3 = __shfl_down_sync(FULL, b1[0], 1);
            if (lane == 31) {
                n0 = (float)ra0[xb + 8]; n1 = (float)ra1[xb + 8];
                n2 = (float)rb0[xb + 8]; n3 = (float)rb1[xb + 8];
            }
            a0[8] = n0; a1[8] = n1; b0[8] = n2; b1[8] = n3;
            if constexpr (std::is_same<T, float>::value) {
                // NaN classifies as "not above" for every threshold, like -inf
#pragma unroll
                for (int i = 0; i < 9; ++i) {
                    a0[i] = cls_value<float>(a0[i]);
                    a1[i] = cls_value<float>(a1[i]);
                    b0[i] = cls_value<float>(b0[i]);
                    b1[i] = cls_value<float>(b1[i]);
                }
            }
#pragma unroll
            for (int i = 0; i < kLaneCells; ++i) {
                if (xb + i >= cx) continue;
                const float mn = fminf(fminf(fminf(a0[i], a0[i + 1]), fminf(a1[i], a1[i + 1])),
                                       fminf(fminf(b0[i], b0[i + 1]), fminf(b1[i], b1[i + 1])));
                const float mx = fmaxf(fmaxf(fmaxf(a0[i], a0[i + 1]), fmaxf(a1[i], a1[i + 1])),
                                       fmaxf(fmaxf(b0[i], b0[i + 1]), fmaxf(b1[i], b1[i + 1])));
                const int lo = count_below(S, G, mn);
                const int hi = count_below(S, G, mx);
                lohi[i >> 1] |= (uint32_t)(lo | (hi << 8)) << (16 * (i & 1));
                for (int k = lo; k < hi; ++k) {
                    const unsigned c = case_of(a0, a1, b0, b1, i, S.thr[k]);
                    atomicAdd(&S.wcnt[warp][k], (uint32_t)S.ntri[c]);
                }
            }
        }
        __syncthreads();

        if (!EMIT) {
            // one count per (isolevel, z, y-tile)
            if (tid < (unsigned)G.niso) {
                uint32_t t = 0;
                for (int w = 0; w < kWarps; ++w) t += S.wcnt[w][tid];
                counts[S.count_base[tid] + (uint64_t)z * G.ytiles + ytile] = t;
            }
            __syncthreads();
            for (unsigned i = tid; i < kWarps * kStreamMaxIso; i += blockDim.x) (&S.wcnt[0][0])[i] = 0;
        } else {
            // ---------------- phase 2: warp bases, compaction, vertices, triangles
            if (warp_active && lane < (unsigned)G.niso) {
                const uint64_t tb = offsets[S.count_base[lane] + (uint64_t)z * G.ytiles + ytile] - S.iso_first[lane];
                uint64_t b = tb;
                for (unsigned w = 0; w < warp; ++w) b += S.wcnt[w][lane];
                S.wbase[warp][lane] = b;
                S.wrun[warp][lane] = 0;
            }
            __syncwarp();
            if (warp_active) {
                // pairs of this lane, in (cell, isolevel) order
                uint32_t m = 0;
#pragma unroll
                for (int i = 0; i < kLaneCells; ++i) {
                    const uint32_t e = (lohi[i >> 1] >> (16 * (i & 1))) & 0xffffu;
                    m += (e >> 8) - (e & 0xffu);
                }
                uint32_t inc = m;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t t = __shfl_up_sync(FULL, inc, o);
                    if (lane >= (unsigned)o) inc += t;
                }
                const uint32_t npairs = __shfl_sync(FULL, inc, 31);
                const uint32_t my_first = inc - m;
                uint32_t* pbuf = ES->pairs[warp];
                float3* vbuf = ES->vtx[warp];
                const uint32_t ybase = y0 + row_l;
                for (uint32_t fill0 = 0; fill0 < npairs; fill0 += kPairCap) {
                    // write this lane's pairs that fall into [fill0, fill0 + kPairCap)
                    uint32_t slot = my_first;
#pragma unroll
                    for (int i = 0; i < kLaneCells; ++i) {
                        const uint32_t e = (lohi[i >> 1] >> (16 * (i & 1))) & 0xffffu;
                        for (uint32_t k = e & 0xffu; k < (e >> 8); ++k, ++slot) {
                            if (slot >= fill0 && slot < fill0 + kPairCap) {
                                const unsigned c = case_of(a0, a1, b0, b1, i, S.thr[k]);
                                pbuf[slot - fill0] = (uint32_t)(lane * kLaneCells + i) | (k << 8) | (c << 16);
                            }
                        }
                    }
                    __syncwarp();
                    const uint32_t nfill = (npairs - fill0 < (uint32_t)kPairCap) ? npairs - fill0 : (uint32_t)kPairCap;
                    for (uint32_t r0 = 0; r0 < nfill;) {
                        const uint32_t p = r0 + lane;
                        const bool has = p < nfill;
                        const uint32_t pe = has ? pbuf[p] : 0u;
                        const uint32_t cell = pe & 0xffu, k = (pe >> 8) & 0xffu, cs = pe >> 16;
                        uint32_t em = has ? S.edge_mask[cs] : 0u;
                        uint32_t ne = __popc(em);
                        uint32_t einc = ne;
#pragma unroll
                        for (int o = 1; o < 32; o <<= 1) {
                            const uint32_t t = __shfl_up_sync(FULL, einc, o);
                            if (lane >= (unsigned)o) einc += t;
                        }
                        const bool join = has && einc <= (uint32_t)kEdgeCap;
                        const uint32_t nround = __popc(__ballot_sync(FULL, join));
                        uint32_t nt = join ? S.ntri[cs] : 0u;
                        if (!join) { ne = 0; em = 0; }
                        const uint32_t ebase = einc - ne;
                        uint32_t tinc = nt;
#pragma unroll
                        for (int o = 1; o < 32; o <<= 1) {
                            const uint32_t t = __shfl_up_sync(FULL, tinc, o);
                            if (lane >= (unsigned)o) tinc += t;
                        }
                        const uint32_t tbase = tinc - nt;
                        const uint32_t ttot = __shfl_sync(FULL, tinc, nround - 1);
                        const uint32_t etot = __shfl_sync(FULL, einc, nround - 1);
                        // per-isolevel offsets in cell order
                        const int key = join ? (int)k : 64 + (int)lane;
                        const uint32_t grp = __match_any_sync(FULL, key);
                        uint32_t pre = 0, gtot = 0;
#pragma unroll
                        for (int bit = 0; bit < 3; ++bit) {
                            const uint32_t bm = __ballot_sync(FULL, (nt >> bit) & 1u);
                            pre += (uint32_t)__popc(bm & grp & lt) << bit;
                            gtot += (uint32_t)__popc(bm & grp) << bit;
                        }
                        const uint32_t run = join ? S.wrun[warp][k] : 0u;
                        __syncwarp();
                        if (join && (31 - __clz(grp)) == (int)lane) S.wrun[warp][k] = run + gtot;
                        const uint64_t obase = join ? S.wbase[warp][k] + run + pre : 0ull;
                        __syncwarp();
                        // vertices: one lane per (pair, edge)
                        for (uint32_t b0i = 0; b0i < etot; b0i += 32) {
                            const uint32_t it = b0i + lane;
                            uint32_t q = 0;
#pragma unroll
                            for (int step = 16; step >= 1; step >>= 1) {
                                const uint32_t cand = q + step;
                                const uint32_t v = __shfl_sync(FULL, ebase, cand & 31u);
                                if (cand < nround && v <= it) q = cand;
                            }
                            const uint32_t em_q = __shfl_sync(FULL, em, q);
                            const uint32_t eb_q = __shfl_sync(FULL, ebase, q);
                            const uint32_t cell_q = __shfl_sync(FULL, cell, q);
                            const uint32_t k_q = __shfl_sync(FULL, k, q);
                            if (it < etot) {
                                const int e = __fns(em_q, 0, (int)(it - eb_q) + 1);
                                const unsigned ep = S.edge_packed[e];
                                const unsigned ca = ep & 7u, cb = ep >> 3;
                                const uint32_t x = seg * kSegCells + cell_q;
                                const T* sa = ((ca >> 2) ? pb : pa) + (size_t)(row_l + ((ca >> 1) & 1u)) * pitch + x + (ca & 1u);
                                const T* sb = ((cb >> 2) ? pb : pa) + (size_t)(row_l + ((cb >> 1) & 1u)) * pitch + x + (cb & 1u);
                                const unsigned d = ca ^ cb;
                                const int axis = d == 1u ? 0 : (d == 2u ? 1 : 2);
                                vbuf[it] = edge_vertex_fast(
                                    S.ip[k_q], S.fast[k_q], (float)*sa, (float)*sb,
                                    __uint2float_rn(x + (ca & 1u)), __uint2float_rn(ybase + ((ca >> 1) & 1u)),
                                    __uint2float_rn(z + (ca >> 2)), __uint2float_rn(x + (cb & 1u)),
                                    __uint2float_rn(ybase + ((cb >> 1) & 1u)), __uint2float_rn(z + (cb >> 2)), axis);
                            }
                        }
                        __syncwarp();
                        // triangles: one lane per triangle
                        for (uint32_t b0i = 0; b0i < ttot; b0i += 32) {
                            const uint32_t it = b0i + lane;
                            uint32_t q = 0;
#pragma unroll
                            for (int step = 16; step >= 1; step >>= 1) {
                                const uint32_t cand = q + step;
                                const uint32_t v = __shfl_sync(FULL, tbase, cand & 31u);
                                if (cand < nround && v <= it) q = cand;
                            }
                            const uint32_t em_q = __shfl_sync(FULL, em, q);
                            const uint32_t eb_q = __shfl_sync(FULL, ebase, q);
                            const uint32_t tb_q = __shfl_sync(FULL, tbase, q);
                            const uint32_t cs_q = __shfl_sync(FULL, cs, q);
                            const uint32_t k_q = __shfl_sync(FULL, k, q);
                            const uint64_t ob_q = __shfl_sync(FULL, obase, q);
                            if (it < ttot) {
                                const uint32_t ti = it - tb_q;
                                const uint64_t pk = S.tri_packed[cs_q] >> (12 * ti);
                                const uint32_t e0 = (uint32_t)pk & 15u, e1 = (uint32_t)(pk >> 4) & 15u,
                                               e2 = (uint32_t)(pk >> 8) & 15u;
                                const float3 A = vbuf[eb_q + __popc(em_q & ((1u << e0) - 1u))];
                                const float3 B = vbuf[eb_q + __popc(em_q & ((1u << e1) - 1u))];
                                const float3 C = vbuf[eb_q + __popc(em_q & ((1u << e2) - 1u))];
                                const float3 n = tri_normal(A, B, C);
                                const uint64_t o = ob_q + ti;
                                float* pc = S.coords[k_q];
                                if (pc) {
                                    float* oc = pc + 9 * o;
                                    oc[0] = A.x; oc[1] = A.y; oc[2] = A.z;
                                    oc[3] = B.x; oc[4] = B.y; oc[5] = B.z;
                                    oc[6] = C.x; oc[7] = C.y; oc[8] = C.z;
                                    float* on = S.normals[k_q] + 3 * o;
                                    on[0] = n.x; on[1] = n.y; on[2] = n.z;
                                }
                            }
                        }
                        __syncwarp();
                        r0 += nround;
                    }
                }
            }
            __syncthreads();
            for (unsigned i = tid; i < kWarps * kStreamMaxIso; i += blockDim.x) (&S.wcnt[0][0])[i] = 0;
        }
        // plane z is consumed: refill its buffer with plane z + 3
        __syncthreads();
        if (tid == 0 && z + 3 <= z1) issue(z + 3);
    }
    // After a normal walk every issued plane has been waited for.  After a
    // timeout, wait (bounded) for the copies still in flight before leaving,
    // so no bulk copy lands in shared memory this CTA no longer owns.
    if (S.dead && tid == 0) {
        // planes s_break .. s_break + 2 (those issued) may still be landing
        const uint32_t last = z1 - z0;
        for (uint32_t i = s_break; i <= last && i < s_break + 3; ++i)
            mbar_wait(&S.bar[i % 3u], (i / 3u) & 1u, 1u << 16);
    }
    __syncthreads();
}

__global__ void k_iso_totals(const StreamIso* isos, int n, const uint64_t* offsets, const uint64_t* d_total,
                             uint64_t* totals)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t first = offsets[isos[i].count_base];
    const uint64_t next = (i + 1 < n) ? offsets[isos[i + 1].count_base] : *d_total;
    totals[i] = next - first;
}

}  // namespace

size_t stream_shared_bytes(size_t plane_bytes, bool emit)
{
    size_t s = ((sizeof(Shared) + 127) / 128) * 128;
    if (emit) s += ((sizeof(EmitShared) + 127) / 128) * 128;
    return s + 3 * plane_bytes;
}

size_t stream_plane_offset(bool emit)
{
    size_t s = ((sizeof(Shared) + 127) / 128) * 128;
    if (emit) s += ((sizeof(EmitShared) + 127) / 128) * 128;
    return s;
}

#define KVSMC_STREAM_SWITCH(DT, ...)                    \
    switch (DT) {                                       \
    case 0: { using T = int8_t; __VA_ARGS__; } break;   \
    case 1: { using T = int16_t; __VA_ARGS__; } break;  \
    case 4: { using T = uint8_t; __VA_ARGS__; } break;  \
    case 5: { using T = uint16_t; __VA_ARGS__; } break; \
    case 8: { using T = float; __VA_ARGS__; } break;    \
    default: return cudaErrorInvalidValue;              \
    }

cudaError_t launch_stream(bool emit, int dtype, const StreamGroup* d_groups, int ngroups, uint32_t nctas,
                          size_t smem_bytes, const StreamIso* d_isos, uint32_t* d_counts, const uint64_t* d_offsets,
                          int* d_status, const Launch& L)
{
    KVSMC_STREAM_SWITCH(dtype, {
        auto kern = emit ? k_stream<T, true> : k_stream<T, false>;
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes);
        if (e != cudaSuccess) return e;
        prof_begin(L, emit ? "stream_emit" : "stream_count");
        kern<<<nctas, kStreamThreads, smem_bytes, L.stream>>>(d_groups, ngroups, d_isos, d_counts, d_offsets,
                                                              d_status);
        prof_end(L);
    });
    *L.counter += 1;
    return cudaGetLastError();
}

cudaError_t launch_iso_totals(const StreamIso* d_isos, int n, const uint64_t* d_offsets, const uint64_t* d_total,
                              uint64_t* d_totals, const Launch& L)
{
    prof_begin(L, "iso_totals");
    k_iso_totals<<<(n + 127) / 128, 128, 0, L.stream>>>(d_isos, n, d_offsets, d_total, d_totals);
    prof_end(L);
    *L.counter += 1;
    return cudaGetLastError();
}

}  // namespace kvsmc
