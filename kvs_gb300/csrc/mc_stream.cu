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
//   * Classification works on each node's isolevel index q = #{thresholds < v}
//     (isolevels sorted by threshold; a monotone bucket table plus exact
//     compares in the rare shared bucket).  Since v > t_k exactly when q > k,
//     a cell is active for isolevel k exactly when min(q) <= k < max(q) over
//     its 8 corners, and its case bits are (q_c > k).  Each lane owns 8
//     consecutive cells; q of the new plane's nodes is computed once per
//     step and carried (packed bytes) to the next step.
//   * A "unit" = (z, y, segment): a contiguous piece of the reference's linear
//     cell order.  The count kernel writes one u16 triangle count per (unit,
//     isolevel); the unit-scan kernel turns them into u32 offsets inside each
//     (isolevel, z) plane plus one total per plane; a scan of the plane totals
//     gives each plane's first triangle.  So an emitting warp knows where its
//     unit's triangles start for every isolevel without talking to any other
//     warp.
//   * Emit: the warp compacts its active pairs in (cell, isolevel) order (warp
//     scan), then takes them 32 at a time, one pair per lane: lanes of the
//     same isolevel are grouped with __match_any_sync and bit-sliced ballots
//     give each pair's output position; each lane interpolates its pair's
//     edges once (the exact FP32 path of mc_interp.cuh) into its own column
//     of a shared-memory vertex table and writes the pair's triangles, cells
//     in linear order, table order inside a cell, each isolevel into its own
//     arrays.
#include <cstddef>

#include <cuda_runtime.h>

#include "mc_internal.h"
#include "mc_interp.cuh"
#include "mc_thermo.cuh"
#include "tma.cuh"

#ifndef KVSMC_VERTS_PER_LANE
#define KVSMC_VERTS_PER_LANE 1
#endif
// launch shape of the emit kernel: warps per CTA, resident CTAs per SM it is
// compiled for (registers per thread), vertex items per round (shared memory)
#ifndef KVSMC_EMIT_WARPS
#define KVSMC_EMIT_WARPS 8
#endif
#ifndef KVSMC_EMIT_CTAS
#define KVSMC_EMIT_CTAS 2
#endif
#ifndef KVSMC_EMIT_MAX_VERTS
#define KVSMC_EMIT_MAX_VERTS 192
#endif

namespace kvsmc {

namespace {

constexpr int kWarps = kStreamThreads / 32;
constexpr int kEmitThreads = 32 * KVSMC_EMIT_WARPS;
constexpr int kEmitWarps = KVSMC_EMIT_WARPS;
constexpr int kLaneCells = 8;
constexpr int kSegCells = 32 * kLaneCells;
constexpr int kPairCap = 128;   // pair buffer entries per warp
constexpr unsigned FULL = 0xffffffffu;

__constant__ uint64_t c_tri_packed[256] = MC_TRI_PACKED_INIT;
__constant__ uint8_t c_ntri[256] = MC_NTRI_INIT;
__constant__ uint16_t c_edge_mask[256] = MC_EDGE_MASK_INIT;
__constant__ uint8_t c_edge_packed[12] = MC_EDGE_PACKED_INIT;

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

constexpr int kMaxVerts = KVSMC_EMIT_MAX_VERTS;   // vertex items of one round (rounds end before it is exceeded)
static_assert(kMaxVerts >= 12 && kMaxVerts <= 256, "a round holds one pair's 12 edges; item maps are 8-bit");
constexpr int kMaxTris = 32 * 5;           // triangle items of one round (5 per pair at most)
constexpr int kVertsPerLane = KVSMC_VERTS_PER_LANE;   // vertex items per lane per pass

// Per-CTA tables, indexed by the corner code of case_code() (not by the
// reference's case number: the code -> case permutation is applied when the
// tables are filled).
struct Tables {
    // per triangle in emission order, its three corners' positions in the
    // pair's vertex list (the rank of each corner's edge among the used
    // edges), 4 bits each, 12 bits per triangle
    uint64_t tri_slots[256];
    uint64_t edge_list[256];    // the used edges in increasing order, 4 bits each
    // per edge: corner A's offsets (dx, dy, dz) and corner B's offset along
    // the edge's axis, as floats (0 or 1)
    float4 edge_geo[12];
    // per ring phase p (plane z in ring buffer p) and edge: element offsets
    // from the warp's ring of corner A (bits 0-13) and corner B (bits 14-27)
    // for the cell at row 0, x 0 of the segment; the edge's axis in bits 28-29
    uint32_t edge_off[3][12];
    uint16_t edge_mask[256];
    uint8_t ntri[256];
};
// ring offsets: 3 planes x at most 3 node rows x at most kSegCells + 16 elements
static_assert(3 * 3 * (kSegCells + 16) < (1 << 14), "edge_off packs ring offsets into 14 bits");

// Per-warp state.
struct WarpState {
    uint64_t bar[3];
    float thr[kStreamMaxIso];
    int32_t thr_bucket[kStreamMaxIso];
    uint32_t cnt[32];                        // count: triangles of the current units, [row][isolevel]
    uint32_t add[32];                        // emit: per-(row, isolevel) advance of the current round
    // bucket -> (thermometer mask of the thresholds in lower buckets | kMultiThr,
    //            bits of the bucket's first threshold, +inf when it has none)
    uint2 lut[kLut];
};

// Per-warp emit buffers: the unit's pairs, and for one round the vertex pool
// (one entry per (pair, used edge)) and the item -> pair maps.
// An isolevel's constants as the emit loops read them (copied from the
// group's StreamIso entries when a warp starts on a group).
struct __align__(16) IsoConst {
    FastIso f;
    float mc[3], sc[3];   // min_coord, scale
    float* coords;
    float* normals;
    uint64_t cap_tris;
};

struct WarpEmit {
    IsoConst ic[kStreamMaxIso];
    uint32_t pairs_round[32];   // this round's pair entry and vertex base per lane
    uint32_t vpre_round[32];
    uint32_t pairs[kPairCap];
    float4 pv[kMaxVerts];   // vertex pool: x, y, z, unused (one 16-byte access per vertex)
    uint8_t item_v[kMaxVerts];
    uint8_t item_t[kMaxTris];
};

__device__ __forceinline__ void store_vertex(WarpEmit* WE, uint32_t j, float3 v)
{
    WE->pv[j] = make_float4(v.x, v.y, v.z, 0.0f);
}

__device__ __forceinline__ float3 load_vertex(const WarpEmit* WE, uint32_t j)
{
    const float4 v = WE->pv[j];
    return make_float3(v.x, v.y, v.z);
}

// One triangle's 9 coordinates and 3 normal components, as the 8-byte
// stores the addresses allow: a word whose address is 8-byte aligned pairs
// with the next one, the odd word out is stored alone (the first word when
// the array starts off an 8-byte boundary, else the last).  Seven stores
// instead of twelve; the values are chosen by selects, so lanes with either
// alignment run the same instructions.
__device__ __forceinline__ void store_triangle(float* oc, float* on, float3 A, float3 B, float3 C, float3 n)
{
    const bool ho = (reinterpret_cast<uintptr_t>(oc) & 4u) != 0;
    *(ho ? oc : oc + 8) = ho ? A.x : C.z;
    float2* p2 = reinterpret_cast<float2*>(ho ? oc + 1 : oc);
    p2[0] = make_float2(ho ? A.y : A.x, ho ? A.z : A.y);
    p2[1] = make_float2(ho ? B.x : A.z, ho ? B.y : B.x);
    p2[2] = make_float2(ho ? B.z : B.y, ho ? C.x : B.z);
    p2[3] = make_float2(ho ? C.y : C.x, ho ? C.z : C.y);
    const bool hn = (reinterpret_cast<uintptr_t>(on) & 4u) != 0;
    *(hn ? on : on + 2) = hn ? n.x : n.z;
    *reinterpret_cast<float2*>(hn ? on + 1 : on) = make_float2(hn ? n.y : n.x, hn ? n.z : n.y);
}

// An isolevel's interpolation constants in registers, read from its IsoConst
// with four 16-byte loads.
struct IsoRegs {
    FastIso f;
    float mc[3], sc[3];
};

static_assert(offsetof(IsoConst, f) == 0 && sizeof(FastIso) == 32 && offsetof(IsoConst, mc) == 32 &&
                  offsetof(IsoConst, sc) == 44 && sizeof(IsoConst) % 16 == 0,
              "load_iso reads IsoConst as four float4");

__device__ __forceinline__ IsoRegs load_iso(const IsoConst& c)
{
    const float4* p = reinterpret_cast<const float4*>(&c);
    const float4 a = p[0], b = p[1], m = p[2], n = p[3];
    IsoRegs r;
    r.f.ih = a.x;
    r.f.il = a.y;
    r.f.iso_err = a.z;
    r.f.f_thr = a.w;
    r.f.vmin_f = b.x;
    r.f.vmax_f = b.y;
    r.f.fast_ok = __float_as_int(b.z);
    r.f.pad = 0;
    r.mc[0] = m.x;
    r.mc[1] = m.y;
    r.mc[2] = m.z;
    r.sc[0] = m.w;
    r.sc[1] = n.x;
    r.sc[2] = n.y;
    return r;
}

// One vertex item: where its edge's two corner values sit in the warp's ring,
// the edge's axis, corner A's coordinates and corner B's coordinate along the
// axis.  qe = the pair entry (warp cell | isolevel << 8 | code << 16), r = the
// edge's rank among the code's used edges, phase = ring buffer of plane z.
struct EdgeItem {
    uint32_t oa, ob;
    int axis;
    float ax, ay, az, b;
};

template <int SEG_SHIFT>
__device__ __forceinline__ EdgeItem edge_item(const Tables& TB, uint32_t qe, uint32_t r, uint32_t phase,
                                              uint32_t row_elems, uint64_t xoff, float fy, float fz)
{
    const uint32_t qh = (qe & 0xffu) >> SEG_SHIFT, cell = qe & ((1u << SEG_SHIFT) - 1u);
    const uint32_t e = (uint32_t)(TB.edge_list[qe >> 16] >> (4 * (r & 15u))) & 15u;
    const uint32_t ow = TB.edge_off[phase][e];
    const float4 g = TB.edge_geo[e];
    const uint32_t base = qh * row_elems + cell;
    EdgeItem it;
    it.oa = (ow & 0x3fffu) + base;
    it.ob = ((ow >> 14) & 0x3fffu) + base;
    it.axis = (int)(ow >> 28);
    // corner coordinates: integers below 2^24, exact as floats
    const float fx = __uint2float_rn((uint32_t)xoff + cell);
    const float fyh = __fadd_rn(fy, qh ? 1.0f : 0.0f);
    it.ax = __fadd_rn(fx, g.x);
    it.ay = __fadd_rn(fyh, g.y);
    it.az = __fadd_rn(fz, g.z);
    it.b = __fadd_rn(it.axis == 0 ? fx : (it.axis == 1 ? fyh : fz), g.w);
    return it;
}

__host__ __device__ __forceinline__ size_t align128(size_t v) { return (v + 127) / 128 * 128; }

// Thermometer masks of the 9 nodes x0 .. x0+8 of a staged row: bit k set when
// the value is above isolevel k's threshold (v > t_k; thresholds sorted, so
// the set bits are 0 .. q-1), packed two nodes per word (node 2m in the low
// half of word m, node 2m+1 in the high half; word 4 holds node 8).  A bucket
// holding one threshold needs one compare (branch-free); only a bucket holding
// several takes the exact loop.
template <typename T>
__device__ __forceinline__ void row_masks(const T* row, uint32_t x0, const WarpState& W, int niso, float bs, float bo,
                                          uint32_t* P)
{
    float v[9];
    load8<T>(row, x0, v);
    v[8] = (float)row[x0 + 8];
    uint32_t e[9];
    uint32_t any = 0;
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const uint2 l = W.lut[bucket_index(v[i], bs, bo)];
        e[i] = (v[i] > __int_as_float((int)l.y)) ? 2u * l.x + 1u : l.x;
        any |= l.x;
    }
    if (any & kMultiThr) {
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            const uint32_t b = bucket_index(v[i], bs, bo);
            const uint32_t lx = W.lut[b].x;
            if (lx & kMultiThr) {
                int k = __popc(lx & 0xffffu);
                while (k < niso && (uint32_t)W.thr_bucket[k] == b && W.thr[k] < v[i]) ++k;
                e[i] = (1u << k) - 1u;
            }
        }
    }
    P[0] = __byte_perm(e[0], e[1], 0x5410);
    P[1] = __byte_perm(e[2], e[3], 0x5410);
    P[2] = __byte_perm(e[4], e[5], 0x5410);
    P[3] = __byte_perm(e[6], e[7], 0x5410);
    P[4] = e[8];
}

// Thermometer mask of one value (the per-node rule of row_masks).
__device__ __forceinline__ uint32_t value_mask(const WarpState& W, int niso, float bs, float bo, float v)
{
    const uint32_t b = bucket_index(v, bs, bo);
    const uint2 l = W.lut[b];
    uint32_t e = (v > __int_as_float((int)l.y)) ? 2u * l.x + 1u : l.x;
    if (l.x & kMultiThr) {
        int k = __popc(l.x & 0xffffu);
        while (k < niso && (uint32_t)W.thr_bucket[k] == b && W.thr[k] < v) ++k;
        e = (1u << k) - 1u;
    }
    return e & 0xffffu;
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

// R = cell rows per warp task (1 or 2).  With R = 2, lanes 0-15 take row y
// and lanes 16-31 row y+1, each over a 128-cell segment, so narrow volumes
// keep every lane busy and a node row is staged for 1.5 cell rows, not 2.
//
// Persistent: the grid holds as many CTAs as fit on the GPU and every warp
// takes tasks from `next_task` (one atomicAdd per task) until they run out,
// so warps that skip empty tasks go on at once instead of idling in a CTA
// whose other warps still run.  Tasks come out in increasing order; the
// group's isolevel tables are rebuilt when a warp crosses a group boundary.
//
// NODES (count pass, one row per task): the pass also counts, per isolevel,
// the vertices of the shared-vertex modes' node units (plane, node row,
// 256-node segment): the cut x, y and z edges from each node to its upper
// neighbours, the edges whose two ends' threshold masks differ.  A task of
// cell row y counts node row y at its planes; on the last cell row also node
// row y + 1, on the last cell plane also the last node plane.  Groups with
// node_units == 0 are not counted.
template <typename T, bool EMIT, int R, bool NODES = false>
__global__ void __launch_bounds__(EMIT ? kEmitThreads : kStreamThreads, EMIT ? KVSMC_EMIT_CTAS : 3)
    k_stream(const StreamGroup* __restrict__ groups, int ngroups, uint64_t ntasks, const StreamIso* __restrict__ isos,
             uint16_t* __restrict__ unit_counts, const uint32_t* __restrict__ unit_offsets,
             const uint64_t* __restrict__ plane_base, int* __restrict__ status,
             unsigned long long* __restrict__ next_task, uint32_t wait_polls, uint64_t task0,
             uint32_t* __restrict__ node_counts)
{
    static_assert(!NODES || (!EMIT && R == 1), "node counts come from one-row count tasks");
    constexpr int LPR = 32 / R;                 // lanes per cell row
    constexpr int SEG = kSegCells / R;          // cells per row segment
    constexpr int SEG_SHIFT = R == 1 ? 8 : 7;   // log2(SEG)
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    Tables& TB = *reinterpret_cast<Tables*>(smem_raw);
    // per-warp shared memory: state, then (emit) buffers, then the row ring
    // (the same layout as stream_warp_smem_bytes on the host; one value type
    // and one rows-per-task per launch, so one layout for all groups)
    const uint32_t row_elems = groups[0].seg_elems;      // staged elements per row
    const uint32_t plane_elems = (R + 1) * row_elems;
    for (unsigned code = tid; code < 256; code += blockDim.x) {
        const uint32_t cs = code_to_case(code);
        TB.ntri[code] = c_ntri[cs];
        const uint32_t em = c_edge_mask[cs];
        TB.edge_mask[code] = (uint16_t)em;
        if (EMIT) {
            uint64_t list = 0;
            int n = 0;
            for (int e = 0; e < 12; ++e)
                if ((em >> e) & 1u) list |= (uint64_t)e << (4 * n++);
            TB.edge_list[code] = list;
            const uint64_t tp = c_tri_packed[cs];
            uint64_t slots = 0;
            for (int c = 0; c < 3 * (int)c_ntri[cs]; ++c) {
                const uint32_t e = (uint32_t)(tp >> (4 * c)) & 15u;
                slots |= (uint64_t)__popc(em & ((1u << e) - 1u)) << (4 * c);
            }
            TB.tri_slots[code] = slots;
        }
        if (EMIT && code < 36) {
            const uint32_t e = code % 12u, ph = code / 12u;
            const uint32_t ep = c_edge_packed[e], c0 = ep & 7u, c1 = ep >> 3, d = c0 ^ c1;
            const uint32_t axis = d == 1u ? 0u : (d == 2u ? 1u : 2u);
            auto corner = [&](uint32_t c) -> uint32_t {
                const uint32_t buf = (c >> 2) ? (ph + 1u) % 3u : ph;   // plane z + 1 or z
                return buf * plane_elems + ((c >> 1) & 1u) * row_elems + (c & 1u);
            };
            TB.edge_off[ph][e] = corner(c0) | (corner(c1) << 14) | (axis << 28);
            if (ph == 0)
                TB.edge_geo[e] = make_float4((c0 & 1u) ? 1.0f : 0.0f, (c0 & 2u) ? 1.0f : 0.0f,
                                             (c0 & 4u) ? 1.0f : 0.0f, (c1 & d) ? 1.0f : 0.0f);
        }
    }
    __syncthreads();   // the only CTA-wide barrier: tables are read-only from here on

    const size_t wstride = align128(sizeof(WarpState)) + (EMIT ? align128(sizeof(WarpEmit)) : 0) +
                           align128((size_t)3 * plane_elems * sizeof(T));
    unsigned char* wbase = smem_raw + align128(sizeof(Tables)) + (size_t)warp * wstride;
    WarpState& W = *reinterpret_cast<WarpState*>(wbase);
    WarpEmit* WE = reinterpret_cast<WarpEmit*>(wbase + align128(sizeof(WarpState)));
    T* ring = reinterpret_cast<T*>(wbase + align128(sizeof(WarpState)) + (EMIT ? align128(sizeof(WarpEmit)) : 0));
    if (lane == 0) {
        for (int b = 0; b < 3; ++b) mbar_init(&W.bar[b], 1);
        fence_barrier_init();
    }
    W.cnt[lane] = 0;
    W.add[lane] = 0;
    __syncwarp();

    uint32_t ph = 0;     // per ring buffer: parity of its next completion
    int gcur = -1;       // group whose tables are in W
    for (;;) {
    unsigned long long tk = 0;
    if (lane == 0) tk = atomicAdd(next_task, 1ull);
    const uint64_t task = task0 + __shfl_sync(FULL, tk, 0);
    if (task >= ntasks) break;
    int gi = gcur;
    if (gi < 0 || task < groups[gi].task_begin || (gi + 1 < ngroups && task >= groups[gi + 1].task_begin))
        gi = find_group(groups, ngroups, task);
    const StreamGroup& G = groups[gi];
    const uint64_t local = task - G.task_begin;
    const uint32_t cx = G.vol.nx - 1, cy = G.vol.ny - 1, cz = G.vol.nz - 1;
    const uint32_t wpr = G.wpr;
    const uint32_t cyr = (cy + R - 1) / R;   // row groups
    const uint32_t seg = (uint32_t)(local % wpr);
    const uint32_t y = (uint32_t)((local / wpr) % cyr) * R;
    const uint32_t zc = (uint32_t)(local / ((uint64_t)wpr * cyr));
    const uint32_t z0 = zc * G.zchunk;
    const uint32_t z1 = (z0 + G.zchunk < cz) ? z0 + G.zchunk : cz;   // cell planes [z0, z1)
    const int niso = G.niso;
    const float bs = G.bs, bo = G.bo;
    const int iso_begin = G.iso_begin;
    const uint64_t unit_base = G.unit_base;
    const uint32_t nrows = (y + R + 1 <= G.vol.ny) ? R + 1 : G.vol.ny - y;   // node rows staged per plane
    const uint64_t pitch = G.vol.pitch;
    const uint64_t slice = G.vol.slice;
    const uint64_t xoff = (uint64_t)seg * SEG;
    // bytes copied per row: SEG + 1 values rounded up to 16 bytes, or up to the
    // end of the (16-byte padded) row for the last segment
    const uint64_t avail = (pitch - xoff) * sizeof(T);
    const uint32_t row_bytes = (uint32_t)(avail < G.seg_copy_bytes ? avail : G.seg_copy_bytes);
    const T* vol = static_cast<const T*>(G.vol.data);

    if (EMIT && G.skip_emit) continue;   // nothing of this group is written in this launch
    if (gi != gcur) {
        // the group's thresholds and bucket table
        if (lane < (unsigned)niso) {
            const StreamIso& I = isos[iso_begin + lane];
            const float t = I.f.f_thr;
            W.thr[lane] = t;
            W.thr_bucket[lane] = (int32_t)bucket_index(t, bs, bo);
            if (EMIT) {
                IsoConst& c = WE->ic[lane];
                c.f = I.f;
                for (int a = 0; a < 3; ++a) { c.mc[a] = I.ip.min_coord[a]; c.sc[a] = I.ip.scale[a]; }
                c.coords = I.coords;
                c.normals = I.normals;
                c.cap_tris = I.cap_tris;
            }
        }
        __syncwarp();
        for (unsigned b = lane; b < (unsigned)kLut; b += 32) {
            uint32_t below = 0, in = 0;
            for (int k = 0; k < niso; ++k) {
                below += (uint32_t)W.thr_bucket[k] < b ? 1u : 0u;
                in += (uint32_t)W.thr_bucket[k] == b ? 1u : 0u;
            }
            const float first = in ? W.thr[below] : __int_as_float(0x7f800000);
            W.lut[b] = make_uint2(((1u << below) - 1u) | (in > 1 ? kMultiThr : 0u), (uint32_t)__float_as_int(first));
        }
        __syncwarp();
        gcur = gi;
    }

    // empty space: a brick whose node min and max have the same mask (no
    // threshold between them) holds no active cell for any isolevel
    const float2* bricks = G.bricks;
    const uint32_t nby = (cy + 1) / 2;
    auto brick_empty = [&](uint32_t z) -> bool {
        const float2* row = bricks + ((uint64_t)(z / kBrickPlanes) * nby + (y >> 1)) * G.brick_wpr;
        float2 mm;
        if (R == 2) {
            mm = row[seg];   // a 128-cell segment is one brick
        } else {
            const uint32_t b0 = 2 * seg;   // a 256-cell segment spans bricks b0 and b0 + 1
            mm = row[b0];
            if (b0 + 1 < G.brick_wpr) {
                const float2 m1 = row[b0 + 1];
                mm.x = fminf(mm.x, m1.x);
                mm.y = fmaxf(mm.y, m1.y);
            }
        }
        return value_mask(W, niso, bs, bo, mm.x) == value_mask(W, niso, bs, bo, mm.y);
    };
    if (bricks) {
        bool all_empty = true;
        for (uint32_t z = z0; z < z1 && all_empty; z = (z / kBrickPlanes + 1) * kBrickPlanes) all_empty = brick_empty(z);
        if (all_empty) continue;   // nothing to count or emit (counts are zeroed before the count pass)
    }

    // plane i of this task goes to ring buffer i % 3
    auto issue = [&](uint32_t i) {
        const int b = (int)(i % 3u);
        T* dst = ring + (size_t)b * plane_elems;
        const T* src = vol + (uint64_t)(z0 + i) * slice + (uint64_t)y * pitch + xoff;
        mbar_arrive_expect_tx(&W.bar[b], nrows * row_bytes);
        for (uint32_t r = 0; r < nrows; ++r) bulk_copy_g2s(dst + r * row_elems, src + r * pitch, row_bytes, &W.bar[b]);
    };
    // wait (bounded) for plane i; on success the buffer's parity advances
    auto acquire = [&](uint32_t i) -> bool {
        const uint32_t b = i % 3u;
        const bool ok = mbar_wait(&W.bar[b], (ph >> b) & 1u, wait_polls);
        if (ok) ph ^= 1u << b;
        return ok;
    };
    const uint32_t nplanes = z1 - z0 + 1;
    __syncwarp();   // the previous task's reads of the ring are done
    if (lane == 0) {
        fence_proxy_async();
        for (uint32_t i = 0; i < nplanes && i < 3; ++i) issue(i);
    }
    const uint32_t half = lane / LPR;                     // this lane's row: y + half
    const uint32_t xl = (lane % LPR) * kLaneCells;        // first cell of this lane inside the segment
    const bool row_ok = y + half < cy;
    // cells of this lane inside the volume (if < 8)
    const int lim = row_ok ? (int)cx - (int)((uint32_t)xoff + xl) : 0;
    const unsigned lt = (1u << lane) - 1u;
    const float fy = __uint2float_rn(y);
    bool dead = false;
    uint32_t acq = 0;          // planes of this task acquired so far
    uint32_t issued = 0;       // planes of this task issued when a wait timed out
    uint32_t PA0[5], PA1[5];   // masks of plane z, this lane's rows (carried from the previous step)
    bool pa_valid = false;
    bool brick_skip = false;   // the current brick is empty
    // emit: whether this lane's (row, isolevel) unit of step z has triangles,
    // loaded one step ahead so the load's latency hides behind a step's work
    const uint32_t uh = lane >> 4, uk = lane & 15u;
    const bool u_lane = EMIT && uh < (uint32_t)R && uk < (uint32_t)niso && y + uh < cy;
    auto unit_nonzero = [&](uint32_t zz) -> bool {
        return u_lane && unit_counts[unit_base + (((uint64_t)zz * cy + y + uh) * wpr + seg) * niso + uk] != 0;
    };
    bool next_any = EMIT ? unit_nonzero(z0) : false;

    for (uint32_t z = z0; z < z1; ++z) {
        const uint32_t s = z - z0;
        // step s needs planes s and s + 1
        bool ok = true;
        while (ok && acq <= s + 1) {
            ok = acquire(acq);
            if (ok) ++acq;
        }
        if (__any_sync(FULL, !ok)) {
            if (lane == 0) atomicExch(status, 1);
            dead = true;
            issued = (s + 3 < nplanes) ? s + 3 : nplanes;   // 3 at the start + one per finished step
            break;
        }
        const T* pa = ring + (size_t)(s % 3u) * plane_elems;         // plane z
        const T* pb = ring + (size_t)((s + 1) % 3u) * plane_elems;   // plane z + 1
        const uint32_t phase = s % 3u;
        const T* ra0 = pa + half * row_elems;
        const T* ra1 = ra0 + row_elems;
        const T* rb0 = pb + half * row_elems;
        const T* rb1 = rb0 + row_elems;
        const float fz = __uint2float_rn(z);
        if (bricks && (s == 0 || z % kBrickPlanes == 0)) brick_skip = brick_empty(z);
        bool skip = brick_skip;
        if (EMIT) {
            // the count pass found no triangle in this step's units: nothing to emit
            const bool any = next_any;
            next_any = z + 1 < z1 ? unit_nonzero(z + 1) : false;
            if (!skip) skip = !__any_sync(FULL, any);
        }
        if (skip) {
            pa_valid = false;
            __syncwarp();
            if (lane == 0 && s + 3 < nplanes) {
                fence_proxy_async();
                issue(s + 3);
            }
            continue;
        }

        // ---------------- phase 1: node masks, per-cell active isolevels
        if (!pa_valid) {
            row_masks<T>(ra0, xl, W, niso, bs, bo, PA0);
            row_masks<T>(ra1, xl, W, niso, bs, bo, PA1);
        }
        uint32_t PB0[5], PB1[5];
        row_masks<T>(rb0, xl, W, niso, bs, bo, PB0);
        row_masks<T>(rb1, xl, W, niso, bs, bo, PB1);
        // per node column: OR / AND of the 4 corners' masks (thermometer codes:
        // OR = the highest, AND = the lowest); per cell: the isolevels whose
        // threshold lies between its lowest and highest corner
        uint32_t co[5], ca[5];
#pragma unroll
        for (int w = 0; w < 5; ++w) {
            co[w] = PA0[w] | PA1[w] | PB0[w] | PB1[w];
            ca[w] = PA0[w] & PA1[w] & PB0[w] & PB1[w];
        }
        uint32_t act[4];
        uint32_t m = 0;
#pragma unroll
        for (int w = 0; w < 4; ++w) {
            const uint32_t o = co[w] | __funnelshift_r(co[w], co[w + 1], 16);
            const uint32_t a = ca[w] & __funnelshift_r(ca[w], ca[w + 1], 16);
            act[w] = o & ~a;
        }
        if (lim < kLaneCells) {
            // cells past the last one of the row, or rows past the last: none
#pragma unroll
            for (int w = 0; w < 4; ++w) {
                const uint32_t keep = (2 * w < lim ? 0xffffu : 0u) | (2 * w + 1 < lim ? 0xffff0000u : 0u);
                act[w] &= keep;
            }
        }
#pragma unroll
        for (int w = 0; w < 4; ++w) m += __popc(act[w]);

        if (!EMIT) {
            // count: one u16 per (unit, isolevel); counters [row][isolevel]
            if (__any_sync(FULL, m != 0)) {
#pragma unroll
                for (int i = 0; i < kLaneCells; ++i) {
                    uint32_t am = (act[i >> 1] >> (16 * (i & 1))) & 0xffffu;
                    if (am) {
                        const uint32_t w0 = cell_word(PA0, i), w1 = cell_word(PA1, i);
                        const uint32_t w2 = cell_word(PB0, i), w3 = cell_word(PB1, i);
                        do {
                            const uint32_t k = __ffs(am) - 1;
                            am &= am - 1;
                            atomicAdd(&W.cnt[half * 16 + k], (uint32_t)TB.ntri[case_code(w0, w1, w2, w3, k)]);
                        } while (am);
                    }
                }
                __syncwarp();
                if (NODES && G.node_units) {
                    // (a node edge that is cut for isolevel k belongs to a cell active
                    // for k, so a step without active cells has no vertices either)
                    const int nlim = (int)G.vol.nx - (int)((uint32_t)xoff + xl);   // this lane's nodes in the row
                    // vertices of node row (plane zn, row yn): masks Pn, and the rows
                    // across its y edges (Py) and z edges (Pz) when it has them
                    auto node_unit = [&](const uint32_t* Pn, const uint32_t* Py, const uint32_t* Pz, bool has_y,
                                         bool has_z, uint32_t zn, uint32_t yn) {
                        uint32_t X[4], Y[4], Z[4], U = 0;
#pragma unroll
                        for (int w = 0; w < 4; ++w) {
                            // halves: nodes 2w (low) and 2w + 1 (high)
                            const uint32_t vn = (2 * w < nlim ? 0xffffu : 0u) | (2 * w + 1 < nlim ? 0xffff0000u : 0u);
                            const uint32_t vx =
                                (2 * w + 1 < nlim ? 0xffffu : 0u) | (2 * w + 2 < nlim ? 0xffff0000u : 0u);
                            X[w] = (Pn[w] ^ __funnelshift_r(Pn[w], Pn[w + 1], 16)) & vx;
                            Y[w] = has_y ? (Pn[w] ^ Py[w]) & vn : 0u;
                            Z[w] = has_z ? (Pn[w] ^ Pz[w]) & vn : 0u;
                            U |= X[w] | Y[w] | Z[w];
                        }
                        uint32_t am = (U | (U >> 16)) & 0xffffu;
                        if (!__any_sync(FULL, am != 0)) return;
                        while (am) {
                            const uint32_t k = __ffs(am) - 1;
                            am &= am - 1;
                            const uint32_t mk = 0x10001u << k;
                            uint32_t c = 0;
#pragma unroll
                            for (int w = 0; w < 4; ++w) c += __popc(X[w] & mk) + __popc(Y[w] & mk) + __popc(Z[w] & mk);
                            atomicAdd(&W.add[k], c);
                        }
                        __syncwarp();
                        if (lane < (unsigned)niso) {
                            const uint64_t un = ((uint64_t)zn * G.vol.ny + yn) * wpr + seg;
                            node_counts[G.node_base + (uint64_t)lane * G.node_units + un] = W.add[lane];
                            W.add[lane] = 0;
                        }
                        __syncwarp();
                    };
                    const bool last_row = y + 1 == cy, last_plane = z + 1 == cz;
                    node_unit(PA0, PA1, PB0, true, true, z, y);
                    if (last_row) node_unit(PA1, PA1, PB1, false, true, z, y + 1);
                    if (last_plane) node_unit(PB0, PB1, PB0, true, false, z + 1, y);
                    if (last_row && last_plane) node_unit(PB1, PB1, PB1, false, false, z + 1, y + 1);
                }
            }
            const uint32_t h = lane >> 4, k = lane & 15u;
            if (h < (uint32_t)R && k < (uint32_t)niso && y + h < cy) {
                const uint64_t unit = ((uint64_t)z * cy + y + h) * wpr + seg;
                unit_counts[unit_base + unit * niso + k] = (uint16_t)W.cnt[lane];
                W.cnt[lane] = 0;
            }
        } else {
            // ---------------- phase 2: pairs, positions, vertices, triangles
            const uint32_t inc = warp_inclusive_scan(m, lane);
            const uint32_t npairs = __shfl_sync(FULL, inc, 31);
            if (npairs) {
                // lane 16 h + k holds the next output triangle of isolevel k in row y + h
                uint64_t run = 0;
                {
                    const uint32_t h = lane >> 4, k = lane & 15u;
                    if (h < (uint32_t)R && k < (uint32_t)niso && y + h < cy) {
                        const StreamIso& I = isos[iso_begin + k];
                        const uint64_t unit = ((uint64_t)z * cy + y + h) * wpr + seg;
                        run = plane_base[I.plane_index + z] - plane_base[I.plane_index] +
                              unit_offsets[unit_base + unit * niso + k];
                    }
                }
                const uint32_t my_first = inc - m;
                uint32_t* pbuf = WE->pairs;
                for (uint32_t fill0 = 0; fill0 < npairs; fill0 += kPairCap) {
                    // this lane's pairs (cell order, then isolevel) that fall into
                    // [fill0, fill0 + kPairCap): warp cell | isolevel << 8 | code << 16
                    // (warp cell = lane * 8 + i: row half in its high bit when R = 2)
                    if (m && my_first < fill0 + kPairCap && my_first + m > fill0) {
                        uint32_t slot = my_first;
#pragma unroll
                        for (int i = 0; i < kLaneCells; ++i) {
                            uint32_t am = (act[i >> 1] >> (16 * (i & 1))) & 0xffffu;
                            if (am) {
                                const uint32_t w0 = cell_word(PA0, i), w1 = cell_word(PA1, i);
                                const uint32_t w2 = cell_word(PB0, i), w3 = cell_word(PB1, i);
                                do {
                                    const uint32_t k = __ffs(am) - 1;
                                    am &= am - 1;
                                    if (slot >= fill0 && slot < fill0 + kPairCap)
                                        pbuf[slot - fill0] = (lane * kLaneCells + i) | (k << 8) |
                                                             (case_code(w0, w1, w2, w3, k) << 16);
                                    ++slot;
                                } while (am);
                            }
                        }
                    }
                    __syncwarp();
                    const uint32_t nfill = (npairs - fill0 < (uint32_t)kPairCap) ? npairs - fill0 : (uint32_t)kPairCap;
                    for (uint32_t r0 = 0, taken = 0; r0 < nfill; r0 += taken) {
                        // ---- one pair per lane, as many as the vertex pool holds
                        const uint32_t p = r0 + lane;
                        bool has = p < nfill;
                        const uint32_t pe0 = has ? pbuf[p] : 0u;
                        const uint32_t ne0 = has ? (uint32_t)__popc(TB.edge_mask[pe0 >> 16]) : 0u;
                        uint32_t vpre = 0;
#pragma unroll
                        for (int bit = 0; bit < 4; ++bit)
                            vpre += (uint32_t)__popc(__ballot_sync(FULL, (ne0 >> bit) & 1u) & lt) << bit;
                        has = has && vpre + ne0 <= (uint32_t)kMaxVerts;   // a suffix of lanes waits
                        taken = (uint32_t)__popc(__ballot_sync(FULL, has));
                        const uint32_t nv = __shfl_sync(FULL, vpre + ne0, taken - 1);
                        const uint32_t pe = has ? pe0 : 0u;
                        const uint32_t k = (pe >> 8) & 0xffu, code = pe >> 16;
                        const uint32_t rk = ((pe & 0xffu) >> SEG_SHIFT) * 16 + k;   // (row, isolevel) slot
                        const uint32_t nt = has ? TB.ntri[code] : 0u;
                        const uint32_t ne = has ? ne0 : 0u;
                        // output position of the pair's first triangle: pairs are in
                        // cell order, so it is the (row, isolevel)'s running count plus
                        // the triangles of the earlier lanes of the same (row, isolevel)
                        const int key = has ? (int)rk : 64 + (int)lane;
                        const uint32_t grp = __match_any_sync(FULL, key);
                        uint32_t pre = 0, gtot = 0, tpre = 0, ntr = 0;
#pragma unroll
                        for (int bit = 0; bit < 3; ++bit) {
                            const uint32_t bm = __ballot_sync(FULL, (nt >> bit) & 1u);
                            pre += (uint32_t)__popc(bm & grp & lt) << bit;
                            gtot += (uint32_t)__popc(bm & grp) << bit;
                            tpre += (uint32_t)__popc(bm & lt) << bit;
                            ntr += (uint32_t)__popc(bm) << bit;
                        }
                        const uint64_t obase = __shfl_sync(FULL, run, rk & 31u) + pre;
                        if (has && (31 - __clz(grp)) == (int)lane) W.add[rk] = gtot;
                        // item -> pair maps of this round
                        WE->pairs_round[lane] = pe;
                        WE->vpre_round[lane] = vpre;
                        for (uint32_t r = 0; r < ne; ++r) WE->item_v[vpre + r] = (uint8_t)lane;
                        for (uint32_t t = 0; t < nt; ++t) WE->item_t[tpre + t] = (uint8_t)lane;
                        __syncwarp();
                        run += W.add[lane];
                        W.add[lane] = 0;
                        // ---- vertices: one (pair, used edge) per lane, edges in increasing order;
                        // kVertsPerLane items per lane per pass, their arithmetic branch-free so
                        // it interleaves; an edge the FP32 path cannot certify (rare) takes the
                        // exact FP64 sequence afterwards
                        for (uint32_t j0 = 0; j0 < nv; j0 += 32 * kVertsPerLane) {
                            uint32_t fail = 0;   // bit u: item u of this lane needs the FP64 path
#pragma unroll
                            for (int u = 0; u < kVertsPerLane; ++u) {
                                const uint32_t j = j0 + 32 * u + lane;
                                const bool hv = j < nv;
                                const uint32_t q = hv ? WE->item_v[j] : 0u;
                                const uint32_t qe = __shfl_sync(FULL, pe, q);
                                const uint32_t qv = __shfl_sync(FULL, vpre, q);
                                const EdgeItem it = edge_item<SEG_SHIFT>(TB, qe, j - qv, phase, row_elems, xoff, fy, fz);
                                const IsoRegs I = load_iso(WE->ic[(qe >> 8) & 0xffu]);
                                float3 v;
                                const bool ok = edge_vertex_axis_try(I.f, I.mc, I.sc, (float)ring[it.oa],
                                                                     (float)ring[it.ob], it.ax, it.ay, it.az, it.axis,
                                                                     it.b, v);
                                if (hv) {
                                    store_vertex(WE, j, v);
                                    if (!ok) fail |= 1u << u;
                                }
                            }
                            if (__any_sync(FULL, fail != 0)) {
                                for (int u = 0; u < kVertsPerLane; ++u) {
                                    if (!((fail >> u) & 1u)) continue;
                                    const uint32_t j = j0 + 32 * u + lane;
                                    const uint32_t q = WE->item_v[j];
                                    const uint32_t qe = WE->pairs_round[q], qv = WE->vpre_round[q];
                                    const uint32_t qk = (qe >> 8) & 0xffu;
                                    const EdgeItem it = edge_item<SEG_SHIFT>(TB, qe, j - qv, phase, row_elems, xoff, fy, fz);
                                    const IsoRegs I = load_iso(WE->ic[qk]);
                                    const float3 v = edge_vertex_axis(I.f, I.mc, I.sc, isos[iso_begin + qk].ip,
                                                                      (float)ring[it.oa], (float)ring[it.ob], it.ax,
                                                                      it.ay, it.az, it.axis, it.b);
                                    store_vertex(WE, j, v);
                                }
                            }
                        }
                        __syncwarp();
                        // ---- triangles: one (pair, triangle) per lane, table order
                        for (uint32_t j0 = 0; j0 < ntr; j0 += 32) {
                            const uint32_t j = j0 + lane;
                            const bool ht = j < ntr;
                            const uint32_t q = ht ? WE->item_t[j] : 0u;
                            const uint32_t qe = __shfl_sync(FULL, pe, q);
                            const uint32_t qv = __shfl_sync(FULL, vpre, q);
                            const uint32_t qt = __shfl_sync(FULL, tpre, q);
                            const uint64_t qo = __shfl_sync(FULL, obase, q);
                            if (ht) {
                                const uint32_t qk = (qe >> 8) & 0xffu, qc = qe >> 16;
                                const uint32_t t = j - qt;
                                const uint32_t sl = (uint32_t)(TB.tri_slots[qc] >> (12 * t));
                                const uint32_t s0 = qv + (sl & 15u), s1 = qv + ((sl >> 4) & 15u), s2 = qv + ((sl >> 8) & 15u);
                                const float3 A = load_vertex(WE, s0);
                                const float3 B = load_vertex(WE, s1);
                                const float3 C = load_vertex(WE, s2);
                                const float3 n = tri_normal(A, B, C);
                                const IsoConst& IC = WE->ic[qk];
                                float* const pc = IC.coords;
                                if (pc && qo + t < IC.cap_tris)
                                    store_triangle(pc + 9 * (qo + t), IC.normals + 3 * (qo + t), A, B, C, n);
                            }
                        }
                        __syncwarp();
                    }
                    __syncwarp();
                }
            }
        }
        // plane z+1's masks are plane z's at the next step
#pragma unroll
        for (int w = 0; w < 5; ++w) { PA0[w] = PB0[w]; PA1[w] = PB1[w]; }
        pa_valid = true;
        // plane z is consumed: refill its buffer with plane z + 3
        __syncwarp();
        if (lane == 0 && s + 3 < nplanes) {
            fence_proxy_async();
            issue(s + 3);
        }
    }
    if (dead) {
        // After a timeout, wait (bounded, by its own limit whatever the plane
        // waits' limit) for the copies still in flight before leaving, so no
        // bulk copy lands in shared memory this warp no longer uses; then stop
        // taking tasks.  (A normal walk acquires every plane it issued.)
        for (uint32_t i = acq; i < issued; ++i) {
            const uint32_t b = i % 3u;
            if (mbar_wait(&W.bar[b], (ph >> b) & 1u, 1u << 16)) ph ^= 1u << b;
        }
        break;
    }
    }   // task loop
}

// Brick min/max: one warp per brick, lanes across its node rows.
template <typename T>
__global__ void __launch_bounds__(256)
    k_bricks(VolumeView v, uint32_t seg_cells, uint32_t wpr, uint32_t nby, uint64_t nbricks, float2* __restrict__ out)
{
    const uint64_t b = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned lane = threadIdx.x & 31u;
    if (b >= nbricks) return;
    const uint32_t seg = (uint32_t)(b % wpr);
    const uint32_t by = (uint32_t)((b / wpr) % nby);
    const uint32_t bz = (uint32_t)(b / ((uint64_t)wpr * nby));
    const uint32_t cx = v.nx - 1, cy = v.ny - 1, cz = v.nz - 1;
    const uint32_t x0 = seg * seg_cells, x1 = min(x0 + seg_cells, cx);
    const uint32_t y0 = 2 * by, y1 = min(y0 + 2, cy);
    const uint32_t z0 = bz * kBrickPlanes, z1 = min(z0 + kBrickPlanes, cz);
    const T* d = static_cast<const T*>(v.data);
    float lo = __int_as_float(0x7f800000), hi = __int_as_float(0xff800000);
    bool nan = false;
    for (uint32_t z = z0; z <= z1; ++z)
        for (uint32_t y = y0; y <= y1; ++y) {
            const T* row = d + (uint64_t)z * v.slice + (uint64_t)y * v.pitch;
            for (uint32_t x = x0 + lane; x <= x1; x += 32) {
                const float f = (float)row[x];
                nan |= f != f;
                lo = fminf(lo, f);
                hi = fmaxf(hi, f);
            }
        }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lo = fminf(lo, __shfl_xor_sync(FULL, lo, o));
        hi = fmaxf(hi, __shfl_xor_sync(FULL, hi, o));
    }
    nan = __any_sync(FULL, nan);
    if (lane == 0)
        out[b] = nan ? make_float2(__int_as_float(0xff800000), __int_as_float(0x7f800000)) : make_float2(lo, hi);
}

// One CTA per (group, z): for every isolevel of the group, the exclusive scan
// of its unit counts over the plane's units (rows y, segments x) -> u32
// offsets inside the plane, and the plane's total.  Counts are stored
// [unit][isolevel]; the plane is walked in tiles of NT units, each staged
// through shared memory with coalesced loads and stores, one unit per thread
// and all isolevels scanned at once.
template <int NT>
__global__ void __launch_bounds__(NT)
    k_unit_scan(const StreamGroup* __restrict__ groups, int ngroups, const StreamIso* __restrict__ isos,
                const uint16_t* __restrict__ unit_counts, uint32_t* __restrict__ unit_offsets,
                uint32_t* __restrict__ plane_totals)
{
    constexpr int NW = NT / 32;
    __shared__ uint16_t sc[NT * kStreamMaxIso];
    __shared__ uint32_t so[NT * kStreamMaxIso];
    __shared__ uint32_t wsum[NW][kStreamMaxIso];
    __shared__ int s_g;
    const unsigned tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    if (tid == 0) {
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

    uint32_t carry[kStreamMaxIso];
#pragma unroll
    for (int k = 0; k < kStreamMaxIso; ++k) carry[k] = 0;
    for (uint64_t t0 = 0; t0 < U; t0 += NT) {
        const uint32_t n = (uint32_t)(U - t0 < (uint64_t)NT ? U - t0 : (uint64_t)NT);
        const uint32_t nel = n * (uint32_t)niso;
        const uint16_t* src = unit_counts + base + t0 * niso;
        for (uint32_t i = tid; i < nel; i += NT) sc[i] = src[i];
        __syncthreads();
        uint32_t c[kStreamMaxIso], ex[kStreamMaxIso];
#pragma unroll
        for (int k = 0; k < kStreamMaxIso; ++k) {
            c[k] = (k < niso && tid < n) ? sc[tid * niso + k] : 0u;
            uint32_t v = c[k];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
                if (lane >= (unsigned)o) v += t;
            }
            if (lane == 31) wsum[warp][k] = v;
            ex[k] = v - c[k];
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kStreamMaxIso; ++k) {
            if (k < niso) {
                uint32_t before = 0, all = 0;
#pragma unroll
                for (int w = 0; w < NW; ++w) {
                    const uint32_t x = wsum[w][k];
                    before += (w < (int)warp) ? x : 0u;
                    all += x;
                }
                if (tid < n) so[tid * niso + k] = carry[k] + before + ex[k];
                carry[k] += all;
            }
        }
        __syncthreads();
        uint32_t* dst = unit_offsets + base + t0 * niso;
        for (uint32_t i = tid; i < nel; i += NT) dst[i] = so[i];
        __syncthreads();
    }
    if (tid < (unsigned)niso) {
#pragma unroll
        for (int k = 0; k < kStreamMaxIso; ++k)
            if (k == (int)tid) plane_totals[isos[G.iso_begin + k].plane_index + z] = carry[k];
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

size_t stream_row_elems(int dtype, int rows)
{
    const size_t es = dtype_size(dtype);
    return ((((size_t)kSegCells / rows + 1) * es + 15) / 16) * 16 / es;
}

size_t stream_warp_smem_bytes(int dtype, bool emit, int rows)
{
    const size_t plane = (size_t)(rows + 1) * stream_row_elems(dtype, rows) * dtype_size(dtype);
    return align128(sizeof(WarpState)) + (emit ? align128(sizeof(WarpEmit)) : 0) + align128(3 * plane);
}

size_t stream_warp_smem_offset() { return align128(sizeof(Tables)); }

size_t stream_shared_bytes(int dtype, bool emit, int rows)
{
    return stream_warp_smem_offset() + (size_t)(emit ? kEmitWarps : kWarps) * stream_warp_smem_bytes(dtype, emit, rows);
}

uint64_t brick_count(const VolumeView& v)
{
    const uint64_t seg = kBrickCells;
    const uint64_t wpr = (v.nx - 1 + seg - 1) / seg;
    const uint64_t nby = (v.ny - 1 + 1) / 2, nbz = (v.nz - 1 + kBrickPlanes - 1) / kBrickPlanes;
    return wpr * nby * nbz;
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

cudaError_t launch_stream(bool emit, int dtype, int rows, const StreamGroup* d_groups, int ngroups, uint64_t ntasks,
                          const StreamIso* d_isos, uint16_t* d_unit_counts, const uint32_t* d_unit_offsets,
                          const uint64_t* d_plane_base, int* d_status, unsigned long long* d_next_task,
                          const Launch& L, int ctas_per_sm, uint64_t task0, uint32_t* d_node_counts)
{
    if (ntasks <= task0) return cudaSuccess;
    if (rows != 1 && rows != 2) return cudaErrorInvalidValue;
    const size_t smem = stream_shared_bytes(dtype, emit, rows);
    const int threads = emit ? kEmitThreads : kStreamThreads;
    const uint64_t need = (ntasks - task0 + threads / 32 - 1) / (threads / 32);
    KVSMC_STREAM_SWITCH(dtype, {
        auto kern = emit ? (rows == 1 ? k_stream<T, true, 1> : k_stream<T, true, 2>)
                         : (rows == 1 ? (d_node_counts ? k_stream<T, false, 1, true> : k_stream<T, false, 1>)
                                      : k_stream<T, false, 2>);
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                     (int)cudaSharedmemCarveoutMaxShared);
        int per_sm = 0;
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
        if (e != cudaSuccess) return e;
        if (ctas_per_sm > 0 && ctas_per_sm < per_sm) per_sm = ctas_per_sm;
        // persistent: as many CTAs as are resident at once (never more than the tasks need)
        const uint64_t resident = (uint64_t)(per_sm > 0 ? per_sm : 1) * (uint64_t)L.num_sms;
        const uint64_t nctas = need < resident ? need : resident;
        prof_begin(L, emit ? "stream_emit" : "stream_count");
        kern<<<(unsigned)nctas, threads, smem, L.stream>>>(d_groups, ngroups, ntasks, d_isos, d_unit_counts,
                                                           d_unit_offsets, d_plane_base, d_status, d_next_task,
                                                           L.wait_polls[emit ? 1 : 0], task0,
                                                           emit ? nullptr : d_node_counts);
        prof_end(L);
    });
    *L.counter += 1;
    return cudaGetLastError();
}

cudaError_t launch_bricks(const VolumeView& v, float2* out, const Launch& L)
{
    const uint64_t n = brick_count(v);
    if (n == 0) return cudaSuccess;
    const uint32_t seg = kBrickCells;
    const uint32_t wpr = (v.nx - 1 + seg - 1) / seg, nby = (v.ny - 1 + 1) / 2;
    const unsigned blocks = (unsigned)((n * 32 + 255) / 256);
    KVSMC_STREAM_SWITCH(v.dtype, {
        prof_begin(L, "bricks");
        k_bricks<T><<<blocks, 256, 0, L.stream>>>(v, seg, wpr, nby, n, out);
        prof_end(L);
    });
    *L.counter += 1;
    return cudaGetLastError();
}

cudaError_t launch_unit_scan(const StreamGroup* d_groups, int ngroups, uint32_t nplanes, const StreamIso* d_isos,
                             const uint16_t* d_unit_counts, uint32_t* d_unit_offsets, uint32_t* d_plane_totals,
                             const Launch& L, int scan_threads)
{
    if (nplanes == 0) return cudaSuccess;
    prof_begin(L, "unit_scan");
    switch (scan_threads) {
    case 64:
        k_unit_scan<64><<<nplanes, 64, 0, L.stream>>>(d_groups, ngroups, d_isos, d_unit_counts, d_unit_offsets,
                                                      d_plane_totals);
        break;
    case 128:
        k_unit_scan<128><<<nplanes, 128, 0, L.stream>>>(d_groups, ngroups, d_isos, d_unit_counts, d_unit_offsets,
                                                        d_plane_totals);
        break;
    case 0:
    case 256:
        k_unit_scan<256><<<nplanes, 256, 0, L.stream>>>(d_groups, ngroups, d_isos, d_unit_counts, d_unit_offsets,
                                                        d_plane_totals);
        break;
    default:
        prof_end(L);
        return cudaErrorInvalidValue;
    }
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
