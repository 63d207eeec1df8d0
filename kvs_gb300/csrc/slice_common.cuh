// slice_common.cuh -- the plane function, value interpolation, colour and
// normal of kvs::SlicePlane (Source/Core/Visualization/Mapper/SlicePlane.cpp),
// shared by the structured (slice.cu) and unstructured (cells.cu) slicers.
// plane_at / color_at take any job with coef[4] / tf_min, tf_max, tf_res, table.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace kvsmc {

// substitute_plane_equation (SlicePlane.cpp:949-975): ((a x + b y) + c z) + d in float
template <typename J>
__device__ __forceinline__ float plane_at(const J& j, float x, float y, float z)
{
    return __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(j.coef[0], x), __fmul_rn(j.coef[1], y)), __fmul_rn(j.coef[2], z)),
                     j.coef[3]);
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
template <typename J>
__device__ __forceinline__ uchar3 color_at(const J& j, float value)
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
        // Math::Round: (int)(x + 0.5) in double for x in [0, 255], i.e. the
        // integer part plus one when the (exact) fraction is at least 1/2
        const float ip = truncf(x);
        out[k] = (uint8_t)((int)ip + (__fsub_rn(x, ip) >= 0.5f ? 1 : 0));
    }
    return make_uchar3(out[0], out[1], out[2]);
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

}  // namespace kvsmc
