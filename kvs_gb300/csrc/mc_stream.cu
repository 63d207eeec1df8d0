// mc_stream.cu -- the streaming kernels: duplicated-vertex extraction of many
// (volume, isolevel) requests in fused launches (count, unit scan, emit).
//
// Work decomposition: every warp is an independent worker.
//   * A warp task = (volume, z-chunk, cell row y, 256-cell x-segment).  The
//     warp walks z through its chunk.  Its two node rows (y, y+1) of each node
//     plane arrive in the warp's own shared-memory ring of three buffers
//     through TMA bulk copies (cp.async.bulk, issued by lane 0, completion on
//     a per-buffer mbarrier), so a plane is read from HBM once per pass and
//     the next one is in flight while the warp works.  No CTA-wide barrier:
//     warps never wait for each other.
//   * Each lane owns 8 consecutive cells.  Per cell: min/max of the 8 corners
//     and the range [lo, hi) of isolevels (sorted by threshold) for which
//     min <= t < max -- exactly the isolevels for which the cell has a
//     surface -- from a monotone bucket table plus exact compares.  Only
//     active (cell, isolevel) pairs are classified further.
//   * A "unit" = (z, y, segment): a contiguous piece of the reference's linear
//     cell order.  The count kernel writes one u16 triangle count per (unit,
//     isolevel); the unit-scan kernel turns them into u32 offsets inside each
//     (isolevel, z) plane plus one total per plane; a scan of the plane totals
//     gives each plane's first triangle.  So an emitting warp knows where its
//     unit's triangles start for every isolevel without talking to any other
//     warp.
//   * Emit: the warp compacts its active pairs (warp scan), groups lanes by
//     isolevel with __match_any_sync (per-isolevel offsets from bit-sliced
//     ballots), interpolates each pair's edges once (one lane per edge, the
//     exact FP32 path of mc_interp.cuh), then writes each triangle (one lane
//     per triangle) at its position: cells in linear order, table order
//     inside a cell, each isolevel into its own arrays.
#include <cuda_runtime.h>

#include "mc_internal.h"
#include "mc_interp.cuh"

namespace kvsmc {

namespace {

constexpr int kWarps = kStreamThreads / 32;
constexpr int kLaneCells = 8;
constexpr int kSegCells = 32 * kLaneCells;
constexpr int kPairCap = 128;   // pair buffer entries per warp
constexpr int kEdgeCap = 96;    // vertex slots per warp and round
constexpr int kTriCap = 160;    // triangles per round (32 pairs x 5)
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

__device__ __forceinline__ void fence_proxy_async()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
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

// Bounded wait: false after `limit` polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit)
{
    for (uint32_t i = 0; i < limit; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// ------------------------------------------------------------ value access

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

// Per-CTA tables (filled once, read-only afterwards).
struct Tables {
    uint64_t tri_packed[256];
    uint16_t edge_mask[256];
    uint8_t ntri[256];
    uint8_t edge_packed[16];
};

// Per-warp state.
struct WarpState {
    uint64_t bar[3];
    float thr[kStreamMaxIso];
    int32_t thr_bucket[kStreamMaxIso];
    uint32_t cnt[kStreamMaxIso];             // count: triangles of the current unit
    uint32_t add[kStreamMaxIso];             // emit: per-isolevel advance of the current round
    uint8_t bucket[kStreamBuckets + 3];
};

struct WarpEmit {
    uint32_t pairs[kPairCap];
    uint16_t edge_map[kEdgeCap];             // vertex slot -> pair lane | edge rank << 5
    uint8_t tri_map[kTriCap];                // triangle of the round -> pair lane | index << 5
    float3 vtx[kEdgeCap];
};

__host__ __device__ __forceinline__ size_t align128(size_t v) { return (v + 127) / 128 * 128; }

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
__device__ __forceinline__ int count_below(const WarpState& W, int niso, const StreamGroup& G, float v)
{
    const int b = bucket_of(G, v);
    const unsigned e = W.bucket[b + 1];
    int k = (int)(e & 0x3fu);
    if (e & 0x80u) {
        while (k < niso && W.thr_bucket[k] == b && W.thr[k] < v) ++k;
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

__device__ __forceinline__ uint32_t warp_inclusive_scan(uint32_t v, unsigned lane)
{
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(FULL, v, o);
        if (lane >= (unsigned)o) v += t;
    }
    return v;
}

// Locate a warp's task: group (binary search), then (z-chunk, row, segment).
__device__ __forceinline__ int find_group(const StreamGroup* groups, int ngroups, uint64_t task)
{
    int lo = 0, hi = ngroups - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (groups[mid].task_begin <= task) lo = mid; else hi = mid - 1;
    }
    return lo;
}

template <typename T, bool EMIT>
__global__ void __launch_bounds__(kStreamThreads)
    k_stream(const StreamGroup* __restrict__ groups, int ngroups, uint64_t ntasks, const StreamIso* __restrict__ isos,
             uint16_t* __restrict__ unit_counts, const uint32_t* __restrict__ unit_offsets,
             const uint64_t* __restrict__ plane_base, int* __restrict__ status)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    Tables& TB = *reinterpret_cast<Tables*>(smem_raw);
    for (unsigned i = tid; i < 256; i += blockDim.x) {
        TB.tri_packed[i] = c_tri_packed[i];
        TB.ntri[i] = c_ntri[i];
        TB.edge_mask[i] = c_edge_mask[i];
        if (i < 12) TB.edge_packed[i] = c_edge_packed[i];
    }
    __syncthreads();   // the only CTA-wide barrier: tables are read-only from here on

    const uint64_t task = (uint64_t)blockIdx.x * kWarps + warp;
    if (task >= ntasks) return;
    const StreamGroup& G = groups[find_group(groups, ngroups, task)];
    const uint64_t local = task - G.task_begin;
    const uint32_t cx = G.vol.nx - 1, cy = G.vol.ny - 1, cz = G.vol.nz - 1;
    const uint32_t seg = (uint32_t)(local % G.wpr);
    const uint32_t y = (uint32_t)((local / G.wpr) % cy);
    const uint32_t zc = (uint32_t)(local / ((uint64_t)G.wpr * cy));
    const uint32_t z0 = zc * G.zchunk;
    const uint32_t z1 = (z0 + G.zchunk < cz) ? z0 + G.zchunk : cz;   // cell planes [z0, z1)
    const int niso = G.niso;

    // per-warp shared memory: state, then (emit) buffers, then the row ring
    // (the same layout as stream_warp_smem_bytes on the host)
    const size_t wstride = align128(sizeof(WarpState)) + (EMIT ? align128(sizeof(WarpEmit)) : 0) +
                           align128((size_t)3 * 2 * G.seg_elems * sizeof(T));
    unsigned char* wbase = smem_raw + align128(sizeof(Tables)) + (size_t)warp * wstride;
    WarpState& W = *reinterpret_cast<WarpState*>(wbase);
    WarpEmit* WE = reinterpret_cast<WarpEmit*>(wbase + align128(sizeof(WarpState)));
    T* ring = reinterpret_cast<T*>(wbase + align128(sizeof(WarpState)) + (EMIT ? align128(sizeof(WarpEmit)) : 0));
    const uint64_t pitch = G.vol.pitch;
    const uint64_t xoff = (uint64_t)seg * kSegCells;
    const uint32_t row_elems = G.seg_elems;              // staged elements per row
    // bytes copied per row: 257 values rounded up to 16 bytes, or up to the end
    // of the (16-byte padded) row for the last segment
    const uint64_t avail = (pitch - xoff) * sizeof(T);
    const uint32_t row_bytes = (uint32_t)(avail < G.seg_copy_bytes ? avail : G.seg_copy_bytes);

    if (lane < (unsigned)niso) {
        const float t = isos[G.iso_begin + lane].f.f_thr;
        W.thr[lane] = t;
        W.thr_bucket[lane] = bucket_of(G, t);
        W.cnt[lane] = 0;
        W.add[lane] = 0;
    }
    __syncwarp();
    for (unsigned i = lane; i < kStreamBuckets + 3; i += 32) {
        const int b = (int)i - 1;
        unsigned below = 0, has = 0;
        for (int k = 0; k < niso; ++k) {
            below += W.thr_bucket[k] < b ? 1u : 0u;
            has |= W.thr_bucket[k] == b ? 1u : 0u;
        }
        W.bucket[i] = (uint8_t)(below | (has << 7));
    }
    if (lane == 0) {
        for (int b = 0; b < 3; ++b) mbar_init(&W.bar[b], 1);
        fence_barrier_init();
    }
    __syncwarp();

    const T* vol = static_cast<const T*>(G.vol.data);
    auto issue = [&](uint32_t plane) {
        const uint32_t i = plane - z0;
        const int b = (int)(i % 3u);
        T* dst = ring + (size_t)b * 2 * row_elems;
        const T* src = vol + (uint64_t)plane * G.vol.slice + (uint64_t)y * pitch + xoff;
        mbar_arrive_expect_tx(&W.bar[b], 2 * row_bytes);
        bulk_copy_g2s(dst, src, row_bytes, &W.bar[b]);
        bulk_copy_g2s(dst + row_elems, src + pitch, row_bytes, &W.bar[b]);
    };
    if (lane == 0) {
        for (uint32_t p = z0; p <= z1 && p < z0 + 3; ++p) issue(p);
    }

    const uint32_t xl = lane * kLaneCells;              // first cell of this lane inside the segment
    const uint32_t xb = (uint32_t)xoff + xl;            // its x
    const unsigned lt = (1u << lane) - 1u;
    bool dead = false;
    uint32_t s_break = 0;

    for (uint32_t z = z0; z < z1; ++z) {
        const uint32_t s = z - z0;
        bool ok = mbar_wait(&W.bar[s % 3u], (s / 3u) & 1u, 1u << 22);
        ok = ok && mbar_wait(&W.bar[(s + 1) % 3u], ((s + 1) / 3u) & 1u, 1u << 22);
        if (__any_sync(FULL, !ok)) {
            if (lane == 0) atomicExch(status, 1);
            dead = true;
            s_break = s;
            break;
        }
        const T* ra0 = ring + (size_t)(s % 3u) * 2 * row_elems;
        const T* ra1 = ra0 + row_elems;
        const T* rb0 = ring + (size_t)((s + 1) % 3u) * 2 * row_elems;
        const T* rb1 = rb0 + row_elems;
        const uint64_t unit = ((uint64_t)z * cy + y) * G.wpr + seg;

        // ---------------- phase 1: classify (lo/hi isolevel range per cell)
        float a0[9], a1[9], b0[9], b1[9];
        load8<T>(ra0, xl, a0);
        load8<T>(ra1, xl, a1);
        load8<T>(rb0, xl, b0);
        load8<T>(rb1, xl, b1);
        a0[8] = (float)ra0[xl + 8];
        a1[8] = (float)ra1[xl + 8];
        b0[8] = (float)rb0[xl + 8];
        b1[8] = (float)rb1[xl + 8];
        if constexpr (std::is_same<T, float>::value) {
            // NaN classifies as "not above" for every threshold, like -inf
#pragma unroll
            for (int i = 0; i < 9; ++i) {
                a0[i] = a0[i] != a0[i] ? -INFINITY : a0[i];
                a1[i] = a1[i] != a1[i] ? -INFINITY : a1[i];
                b0[i] = b0[i] != b0[i] ? -INFINITY : b0[i];
                b1[i] = b1[i] != b1[i] ? -INFINITY : b1[i];
            }
        }
        uint32_t lohi[kLaneCells / 2] = {0, 0, 0, 0};
        uint32_t m = 0;
#pragma unroll
        for (int i = 0; i < kLaneCells; ++i) {
            if (xb + i >= cx) continue;
            const float mn = fminf(fminf(fminf(a0[i], a0[i + 1]), fminf(a1[i], a1[i + 1])),
                                   fminf(fminf(b0[i], b0[i + 1]), fminf(b1[i], b1[i + 1])));
            const float mx = fmaxf(fmaxf(fmaxf(a0[i], a0[i + 1]), fmaxf(a1[i], a1[i + 1])),
                                   fmaxf(fmaxf(b0[i], b0[i + 1]), fmaxf(b1[i], b1[i + 1])));
            const int lo = count_below(W, niso, G, mn);
            const int hi = count_below(W, niso, G, mx);
            lohi[i >> 1] |= (uint32_t)(lo | (hi << 8)) << (16 * (i & 1));
            m += (uint32_t)(hi - lo);
            if (!EMIT) {
                for (int k = lo; k < hi; ++k) atomicAdd(&W.cnt[k], (uint32_t)TB.ntri[case_of(a0, a1, b0, b1, i, W.thr[k])]);
            }
        }

        if (!EMIT) {
            __syncwarp();
            if (lane < (unsigned)niso) {
                unit_counts[G.unit_base + unit * niso + lane] = (uint16_t)W.cnt[lane];
                W.cnt[lane] = 0;
            }
        } else {
            // ---------------- phase 2: positions, compaction, vertices, triangles
            // lane k holds the next output triangle of isolevel k for this unit
            uint64_t run = 0;
            if (lane < (unsigned)niso) {
                const StreamIso& I = isos[G.iso_begin + lane];
                run = plane_base[I.plane_index + z] - plane_base[I.plane_index] +
                      unit_offsets[G.unit_base + unit * niso + lane];
            }
            const uint32_t inc = warp_inclusive_scan(m, lane);
            const uint32_t npairs = __shfl_sync(FULL, inc, 31);
            const uint32_t my_first = inc - m;
            uint32_t* pbuf = WE->pairs;
            for (uint32_t fill0 = 0; fill0 < npairs; fill0 += kPairCap) {
                // this lane's pairs that fall into [fill0, fill0 + kPairCap)
                uint32_t slot = my_first;
#pragma unroll
                for (int i = 0; i < kLaneCells; ++i) {
                    const uint32_t e = (lohi[i >> 1] >> (16 * (i & 1))) & 0xffffu;
                    for (uint32_t k = e & 0xffu; k < (e >> 8); ++k, ++slot) {
                        if (slot >= fill0 && slot < fill0 + kPairCap) {
                            const unsigned c = case_of(a0, a1, b0, b1, i, W.thr[k]);
                            pbuf[slot - fill0] = (uint32_t)(xl + i) | (k << 8) | (c << 16);
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
                    uint32_t em = has ? TB.edge_mask[cs] : 0u;
                    uint32_t ne = __popc(em);
                    const uint32_t einc = warp_inclusive_scan(ne, lane);
                    const bool join = has && einc <= (uint32_t)kEdgeCap;
                    const uint32_t nround = __popc(__ballot_sync(FULL, join));
                    const uint32_t nt = join ? TB.ntri[cs] : 0u;
                    if (!join) { ne = 0; em = 0; }
                    const uint32_t ebase = einc - ne;
                    const uint32_t tinc = warp_inclusive_scan(nt, lane);
                    const uint32_t tbase = tinc - nt;
                    const uint32_t ttot = __shfl_sync(FULL, tinc, nround - 1);
                    const uint32_t etot = __shfl_sync(FULL, einc, nround - 1);
                    // per-isolevel position of this pair's first triangle (cell order)
                    const int key = join ? (int)k : 64 + (int)lane;
                    const uint32_t grp = __match_any_sync(FULL, key);
                    uint32_t pre = 0, gtot = 0;
#pragma unroll
                    for (int bit = 0; bit < 3; ++bit) {
                        const uint32_t bm = __ballot_sync(FULL, (nt >> bit) & 1u);
                        pre += (uint32_t)__popc(bm & grp & lt) << bit;
                        gtot += (uint32_t)__popc(bm & grp) << bit;
                    }
                    const uint64_t run_k = __shfl_sync(FULL, run, k & 31u);
                    const uint64_t obase = run_k + pre;
                    if (join && (31 - __clz(grp)) == (int)lane) W.add[k] = gtot;
                    // expansion maps: vertex slot -> (pair, edge rank), triangle -> (pair, index)
                    for (uint32_t j = 0; j < ne; ++j) WE->edge_map[ebase + j] = (uint16_t)(lane | (j << 5));
                    for (uint32_t j = 0; j < nt; ++j) WE->tri_map[tbase + j] = (uint8_t)(lane | (j << 5));
                    __syncwarp();
                    if (lane < (unsigned)niso) {
                        run += W.add[lane];
                        W.add[lane] = 0;
                    }
                    // vertices: one lane per (pair, edge)
                    for (uint32_t b = 0; b < etot; b += 32) {
                        const uint32_t it = b + lane;
                        const bool v = it < etot;
                        const uint32_t mp = v ? (uint32_t)WE->edge_map[it] : 0u;
                        const uint32_t q = mp & 31u, j = mp >> 5;
                        const uint32_t em_q = __shfl_sync(FULL, em, q);
                        const uint32_t cell_q = __shfl_sync(FULL, cell, q);
                        const uint32_t k_q = __shfl_sync(FULL, k, q);
                        if (v) {
                            const int e = __fns(em_q, 0, (int)j + 1);
                            const unsigned ep = TB.edge_packed[e];
                            const unsigned ca = ep & 7u, cb = ep >> 3;
                            const T* sa = ((ca >> 2) ? rb0 : ra0) + ((ca >> 1) & 1u) * row_elems + cell_q + (ca & 1u);
                            const T* sb = ((cb >> 2) ? rb0 : ra0) + ((cb >> 1) & 1u) * row_elems + cell_q + (cb & 1u);
                            const unsigned d = ca ^ cb;
                            const int axis = d == 1u ? 0 : (d == 2u ? 1 : 2);
                            const uint32_t x = (uint32_t)xoff + cell_q;
                            const StreamIso& I = isos[G.iso_begin + k_q];
                            WE->vtx[it] = edge_vertex_fast(
                                I.ip, I.f, (float)*sa, (float)*sb, __uint2float_rn(x + (ca & 1u)),
                                __uint2float_rn(y + ((ca >> 1) & 1u)), __uint2float_rn(z + (ca >> 2)),
                                __uint2float_rn(x + (cb & 1u)), __uint2float_rn(y + ((cb >> 1) & 1u)),
                                __uint2float_rn(z + (cb >> 2)), axis);
                        }
                    }
                    __syncwarp();
                    // triangles: one lane per triangle
                    for (uint32_t b = 0; b < ttot; b += 32) {
                        const uint32_t it = b + lane;
                        const bool v = it < ttot;
                        const uint32_t mp = v ? (uint32_t)WE->tri_map[it] : 0u;
                        const uint32_t q = mp & 31u, ti = mp >> 5;
                        const uint32_t em_q = __shfl_sync(FULL, em, q);
                        const uint32_t eb_q = __shfl_sync(FULL, ebase, q);
                        const uint32_t cs_q = __shfl_sync(FULL, cs, q);
                        const uint32_t k_q = __shfl_sync(FULL, k, q);
                        const uint64_t ob_q = __shfl_sync(FULL, obase, q);
                        if (v) {
                            const uint64_t pk = TB.tri_packed[cs_q] >> (12 * ti);
                            const uint32_t e0 = (uint32_t)pk & 15u, e1 = (uint32_t)(pk >> 4) & 15u,
                                           e2 = (uint32_t)(pk >> 8) & 15u;
                            const float3 A = WE->vtx[eb_q + __popc(em_q & ((1u << e0) - 1u))];
                            const float3 B = WE->vtx[eb_q + __popc(em_q & ((1u << e1) - 1u))];
                            const float3 C = WE->vtx[eb_q + __popc(em_q & ((1u << e2) - 1u))];
                            const float3 n = tri_normal(A, B, C);
                            const StreamIso& I = isos[G.iso_begin + k_q];
                            float* pc = I.coords;
                            if (pc) {
                                const uint64_t o = ob_q + ti;
                                float* oc = pc + 9 * o;
                                oc[0] = A.x; oc[1] = A.y; oc[2] = A.z;
                                oc[3] = B.x; oc[4] = B.y; oc[5] = B.z;
                                oc[6] = C.x; oc[7] = C.y; oc[8] = C.z;
                                float* on = I.normals + 3 * o;
                                on[0] = n.x; on[1] = n.y; on[2] = n.z;
                            }
                        }
                    }
                    __syncwarp();
                    r0 += nround;
                }
                __syncwarp();
            }
        }
        // plane z is consumed: refill its buffer with plane z + 3
        __syncwarp();
        if (lane == 0 && z + 3 <= z1) {
            fence_proxy_async();
            issue(z + 3);
        }
    }
    // After a normal walk every issued plane has been waited for.  After a
    // timeout, wait (bounded) for the copies still in flight before leaving,
    // so no bulk copy lands in shared memory this warp no longer owns.
    if (dead && lane == 0) {
        const uint32_t last = z1 - z0;
        for (uint32_t i = s_break; i <= last && i < s_break + 3; ++i)
            mbar_wait(&W.bar[i % 3u], (i / 3u) & 1u, 1u << 16);
    }
}

// One CTA per (group, z): for every isolevel of the group, the exclusive scan
// of its unit counts over the plane's units (rows y, segments x) -> u32
// offsets inside the plane, and the plane's total.
constexpr int kScanUnitThreads = 256;

__global__ void __launch_bounds__(kScanUnitThreads)
    k_unit_scan(const StreamGroup* __restrict__ groups, int ngroups, const StreamIso* __restrict__ isos,
                const uint16_t* __restrict__ unit_counts, uint32_t* __restrict__ unit_offsets,
                uint32_t* __restrict__ plane_totals)
{
    __shared__ uint32_t ws[33];
    __shared__ int s_g;
    if (threadIdx.x == 0) {
        int lo = 0, hi = ngroups - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (groups[mid].plane_begin <= blockIdx.x) lo = mid; else hi = mid - 1;
        }
        s_g = lo;
    }
    __syncthreads();
    const StreamGroup& G = groups[s_g];
    const uint32_t z = blockIdx.x - G.plane_begin;
    const uint64_t U = (uint64_t)(G.vol.ny - 1) * G.wpr;
    const int niso = G.niso;
    const uint64_t base = G.unit_base + (uint64_t)z * U * niso;
    for (int k = 0; k < niso; ++k) {
        uint32_t running = 0;
        for (uint64_t u0 = 0; u0 < U; u0 += blockDim.x) {
            const uint64_t u = u0 + threadIdx.x;
            const uint32_t c = u < U ? unit_counts[base + u * niso + k] : 0u;
            uint32_t tot;
            const uint32_t e = block_exclusive_scan(c, ws, &tot);
            if (u < U) unit_offsets[base + u * niso + k] = running + e;
            running += tot;
        }
        if (threadIdx.x == 0) plane_totals[isos[G.iso_begin + k].plane_index + z] = running;
    }
}

// Triangles of every isolevel: the difference of its first plane's offset and
// the next isolevel's (or the grand total).
__global__ void k_iso_totals(const StreamIso* isos, int n, const uint64_t* plane_base, const uint64_t* d_total,
                             uint64_t* totals)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t first = plane_base[isos[i].plane_index];
    const uint64_t next = (i + 1 < n) ? plane_base[isos[i + 1].plane_index] : *d_total;
    totals[i] = next - first;
}

}  // namespace

size_t stream_warp_smem_bytes(int dtype, bool emit)
{
    const size_t es = dtype_size(dtype);
    const size_t row = ((257 * es + 15) / 16) * 16;
    return align128(sizeof(WarpState)) + (emit ? align128(sizeof(WarpEmit)) : 0) + align128(3 * 2 * row);
}

size_t stream_row_elems(int dtype)
{
    const size_t es = dtype_size(dtype);
    return ((257 * es + 15) / 16) * 16 / es;
}

size_t stream_warp_smem_offset() { return align128(sizeof(Tables)); }

size_t stream_shared_bytes(int dtype, bool emit)
{
    return stream_warp_smem_offset() + (size_t)kWarps * stream_warp_smem_bytes(dtype, emit);
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

cudaError_t launch_stream(bool emit, int dtype, const StreamGroup* d_groups, int ngroups, uint64_t ntasks,
                          const StreamIso* d_isos, uint16_t* d_unit_counts, const uint32_t* d_unit_offsets,
                          const uint64_t* d_plane_base, int* d_status, const Launch& L)
{
    if (ntasks == 0) return cudaSuccess;
    const size_t smem = stream_shared_bytes(dtype, emit);
    const uint64_t nctas = (ntasks + kWarps - 1) / kWarps;
    KVSMC_STREAM_SWITCH(dtype, {
        auto kern = emit ? k_stream<T, true> : k_stream<T, false>;
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        prof_begin(L, emit ? "stream_emit" : "stream_count");
        kern<<<(unsigned)nctas, kStreamThreads, smem, L.stream>>>(d_groups, ngroups, ntasks, d_isos, d_unit_counts,
                                                                   d_unit_offsets, d_plane_base, d_status);
        prof_end(L);
    });
    *L.counter += 1;
    return cudaGetLastError();
}

cudaError_t launch_unit_scan(const StreamGroup* d_groups, int ngroups, uint32_t nplanes, const StreamIso* d_isos,
                             const uint16_t* d_unit_counts, uint32_t* d_unit_offsets, uint32_t* d_plane_totals,
                             const Launch& L)
{
    if (nplanes == 0) return cudaSuccess;
    prof_begin(L, "unit_scan");
    k_unit_scan<<<nplanes, kScanUnitThreads, 0, L.stream>>>(d_groups, ngroups, d_isos, d_unit_counts, d_unit_offsets,
                                                            d_plane_totals);
    prof_end(L);
    *L.counter += 1;
    return cudaGetLastError();
}

cudaError_t launch_iso_totals(const StreamIso* d_isos, int n, const uint64_t* d_plane_base, const uint64_t* d_total,
                              uint64_t* d_totals, const Launch& L)
{
    prof_begin(L, "iso_totals");
    k_iso_totals<<<(n + 127) / 128, 128, 0, L.stream>>>(d_isos, n, d_plane_base, d_total, d_totals);
    prof_end(L);
    *L.counter += 1;
    return cudaGetLastError();
}

}  // namespace kvsmc
