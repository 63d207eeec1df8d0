// mc_thermo.cuh -- threshold ("thermometer") masks of node values for up to
// kStreamMaxIso isolevels of one volume at once, and the cells' corner codes
// built from them.
//
// With the isolevels' thresholds sorted (t_0 <= t_1 <= ...), a value's mask
// has bit k set when v > t_k, so its set bits are 0 .. q-1.  A bucket index
// floor(kStreamBuckets * sat(v * bs + bo)) is monotone in v; a lookup table
// per bucket holds the mask of the thresholds in lower buckets and the
// bucket's first threshold, so one float compare finishes the mask; only a
// bucket holding two or more thresholds runs an exact loop.  NaN saturates to
// bucket 0 and is above no threshold, as in the reference's double compare.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "mc_internal.h"

namespace kvsmc {

constexpr int kLut = kStreamBuckets + 1;   // bucket indices 0 .. kStreamBuckets
constexpr uint32_t kMultiThr = 1u << 31;   // LUT flag: two or more thresholds lie in this bucket

// Monotone (non-decreasing) bucket of a value in [0, kStreamBuckets]:
// floor(kStreamBuckets * sat(v * bs + bo)).  Thresholds and node values go
// through exactly this function, so a threshold in a lower bucket than v is
// below v, one in a higher bucket is not, and only a shared bucket needs an
// exact compare.  NaN saturates to 0 (the fma's .sat flushes NaN to +0).
__device__ __forceinline__ uint32_t bucket_index(float v, float bs, float bo)
{
    float u;
    asm("fma.rn.sat.f32 %0, %1, %2, %3;" : "=f"(u) : "f"(v), "f"(bs), "f"(bo));
    // u * NB + 2^23 rounded down: 2^23 + floor(u * NB) exactly
    const float t = __fmaf_rd(u, (float)kStreamBuckets, 8388608.0f);
    return (uint32_t)__float_as_int(t) - 0x4B000000u;
}

// A group's threshold tables (shared memory).
struct ThermoTables {
    float thr[kStreamMaxIso];
    int32_t thr_bucket[kStreamMaxIso];
    // bucket -> (thermometer mask of the thresholds in lower buckets | kMultiThr,
    //            bits of the bucket's first threshold, +inf when it has none)
    uint2 lut[kLut];
};

// Fill W from the sorted thresholds t[0 .. niso): called by all 32 lanes of
// one warp (the caller synchronizes before W is read by others).
__device__ __forceinline__ void thermo_build(ThermoTables& W, const float* t, int niso, float bs, float bo,
                                             unsigned lane)
{
    if (lane < (unsigned)niso) {
        W.thr[lane] = t[lane];
        W.thr_bucket[lane] = (int32_t)bucket_index(t[lane], bs, bo);
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
}

// The mask of one value: bit k set when v > t_k.
__device__ __forceinline__ uint32_t thermo_mask(const ThermoTables& W, int niso, float bs, float bo, float v)
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

// The row word of cell i (0..7): node i in the low half, node i+1 in the high half.
__device__ __forceinline__ uint32_t cell_word(const uint32_t* P, int i)
{
    return (i & 1) ? __funnelshift_r(P[i >> 1], P[(i >> 1) + 1], 16) : P[i >> 1];
}

// Corner code of a cell for isolevel k from its four row words (plane z rows
// y, y+1 = a0, a1; plane z+1 = b0, b1): bit r = row r's node i above, bit
// 4 + r = row r's node i+1 above.
__device__ __forceinline__ uint32_t case_code(uint32_t a0, uint32_t a1, uint32_t b0, uint32_t b1, uint32_t k)
{
    const uint32_t m0 = (a0 >> k) & 0x10001u, m1 = (a1 >> k) & 0x10001u;
    const uint32_t m2 = (b0 >> k) & 0x10001u, m3 = (b1 >> k) & 0x10001u;
    const uint32_t x = m0 | (m1 << 1) | (m2 << 2) | (m3 << 3);
    return (x & 0xfu) | ((x >> 12) & 0xf0u);
}

// The reference's case number of a corner code: bit c = corner c above, with
// corners (x,y,z) 0:(0,0,0) 1:(1,0,0) 2:(1,1,0) 3:(0,1,0) 4:(0,0,1) 5:(1,0,1)
// 6:(1,1,1) 7:(0,1,1) (MarchingCubes.cpp:187-194).
__device__ __forceinline__ uint32_t code_to_case(uint32_t c)
{
    return (c & 1u) | (((c >> 4) & 1u) << 1) | (((c >> 5) & 1u) << 2) | (((c >> 1) & 1u) << 3) |
           (((c >> 2) & 1u) << 4) | (((c >> 6) & 1u) << 5) | (((c >> 7) & 1u) << 6) | (((c >> 3) & 1u) << 7);
}

}  // namespace kvsmc
