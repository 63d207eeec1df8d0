// selftest.cu -- on-device check of the FP32 interpolation path against the
// FP64 sequence of the reference, on random edges (diagnostic entry point).
#include <cuda_runtime.h>

#include "mc_internal.h"
#include "mc_interp.cuh"

namespace kvsmc {

namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t x)
{
    x ^= x >> 33; x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ull;
    x ^= x >> 33;
    return x;
}

__device__ __forceinline__ double unit(uint64_t h) { return (double)(h >> 11) * (1.0 / 9007199254740992.0); }

// One random straddling edge per index; several value distributions.
__global__ void k_selftest(uint64_t n, uint64_t seed, unsigned long long* counters)
{
    unsigned long long mism = 0, fall = 0, tested = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t h0 = mix64(seed * 0x9e3779b97f4a7c15ull + i);
        const uint64_t h1 = mix64(h0 + 1), h2 = mix64(h0 + 2), h3 = mix64(h0 + 3);
        const int kind = (int)(h0 % 10);
        double iso;
        float va, vb;
        if (kind == 0) {          // float data in [0,1], double isolevel
            va = (float)unit(h1); vb = (float)unit(h2); iso = unit(h3);
        } else if (kind == 1) {   // float data, float isolevel
            va = (float)unit(h1); vb = (float)unit(h2); iso = (double)(float)unit(h3);
        } else if (kind == 2) {   // uint8-like data, isolevel k + 0.5 or k
            va = (float)(h1 & 255); vb = (float)(h2 & 255); iso = (double)(h3 & 255) + ((h3 >> 8) & 1 ? 0.5 : 0.0);
        } else if (kind == 3) {   // uint16-like data, random double isolevel
            va = (float)(h1 & 65535); vb = (float)(h2 & 65535); iso = unit(h3) * 65535.0;
        } else if (kind == 4) {   // close values (small denominators)
            va = (float)unit(h1); vb = __int_as_float(__float_as_int(va) + (int)(h2 & 15) - 7);
            iso = (double)va + ((double)vb - (double)va) * unit(h3);
        } else if (kind == 5) {   // isolevel just above v0 (small numerators)
            va = (float)unit(h1); vb = (float)unit(h2);
            iso = (double)fminf(va, vb) + unit(h3) * 1e-9;
        } else if (kind == 6) {   // wide dynamic range
            va = (float)((unit(h1) - 0.5) * 2e6); vb = (float)((unit(h2) - 0.5) * 2e6); iso = (unit(h3) - 0.5) * 2e6;
        } else if (kind == 7) {   // ratio near 1/2 (midpoint-prone)
            va = (float)(h1 & 1023); vb = va + 1.0f; iso = (double)va + 0.5 + (unit(h3) - 0.5) * 1e-12;
        } else if (kind == 8) {   // close values, ratio near 0 or 1 (vertices on power-of-two coordinates below)
            va = (float)unit(h1); vb = __int_as_float(__float_as_int(va) + (int)(h2 & 3) + 1);
            const double t = unit(h3) * 1e-6;
            iso = ((h3 >> 60) & 1) ? (double)va + ((double)vb - (double)va) * t
                                   : (double)vb - ((double)vb - (double)va) * t;
        } else {                  // isolevel a double just off a float value, close values
            va = (float)unit(h1); vb = __int_as_float(__float_as_int(va) + 1);
            iso = (double)va + ((double)vb - (double)va) * unit(h3) * 1e-3;
        }
        const float f_iso = (float)iso;
        float thr = f_iso;
        if ((double)thr > iso) thr = nextafterf(thr, -INFINITY);
        const bool b0 = va > thr, b1 = vb > thr;
        if (b0 == b1) continue;
        FastIso f;
        f.ih = f_iso;
        f.il = (float)(iso - (double)f.ih);
        const double rep = iso - ((double)f.ih + (double)f.il);
        f.iso_err = (float)fabs(rep) * 1.0001f;
        f.f_thr = thr;
        f.vmin_f = -3.0e38f; f.vmax_f = 3.0e38f;
        f.fast_ok = 1; f.pad = 0;
        Interp j;
        j.iso = iso;
        j.vmin = -3.0e38; j.vmax = 3.0e38;
        for (int k = 0; k < 3; ++k) { j.min_coord[k] = 0.0f; j.scale[k] = 1.0f; }
        const int axis = (int)((h3 >> 20) % 3);
        // kinds 8 and 9: the edge starts or ends on a power of two
        const float a = kind >= 8 ? (float)(1u << ((h3 >> 24) & 10)) - (((h3 >> 50) & 1) ? 1.0f : 0.0f)
                                  : (float)((h3 >> 24) & 2047);
        const bool rev = (h3 >> 40) & 1;
        float ax = (float)((h2 >> 30) & 2047), ay = (float)((h2 >> 41) & 2047), az = (float)((h1 >> 30) & 2047);
        float bx = ax, by = ay, bz = az;
        float* pa = axis == 0 ? &ax : (axis == 1 ? &ay : &az);
        float* pb = axis == 0 ? &bx : (axis == 1 ? &by : &bz);
        *pa = rev ? a + 1.0f : a;
        *pb = rev ? a : a + 1.0f;
        const float3 ex = interpolate_exact(j, (double)va, (double)vb, ax, ay, az, bx, by, bz);
        // every certified FP32 path must agree with the FP64 sequence where it
        // claims certainty: fast_axis (and edge_vertex_fast, which falls back)
        // and fast_axis_bf (the streaming kernels' branch-free form)
        const float want = axis == 0 ? ex.x : (axis == 1 ? ex.y : ex.z);
        float r, rb;
        const float v0 = va, v1 = vb;
        const bool ok = fast_axis(v0, v1, *pa, *pb, f, r);
        const bool okb = fast_axis_bf(v0, v1, *pa, *pb, f, rb);
        const float3 fv = edge_vertex_fast(j, f, va, vb, ax, ay, az, bx, by, bz, axis);
        ++tested;
        if (!okb) ++fall;
        if (__float_as_int(ex.x) != __float_as_int(fv.x) || __float_as_int(ex.y) != __float_as_int(fv.y) ||
            __float_as_int(ex.z) != __float_as_int(fv.z) ||
            (ok && __float_as_int(r) != __float_as_int(want)) || (okb && __float_as_int(rb) != __float_as_int(want)))
            ++mism;
    }
    atomicAdd(&counters[0], tested);
    atomicAdd(&counters[1], mism);
    atomicAdd(&counters[2], fall);
}

// The unstructured mappers' vertex on random float endpoints: the FP32
// certificate (cell_ratio / cell_axis) against the FP64 sequence
// RN32(RN64(c0 + RN64(|RN64(RN64(iso - v0) / RN64(v1 - v0))| * RN32(c1 - c0)))).
__global__ void k_selftest_cells(uint64_t n, uint64_t seed, unsigned long long* counters)
{
    unsigned long long mism = 0, fall = 0, tested = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t h0 = mix64(seed * 0x9e3779b97f4a7c15ull + i + 0x5bd1e995ull);
        const uint64_t h1 = mix64(h0 + 1), h2 = mix64(h0 + 2), h3 = mix64(h0 + 3), h4 = mix64(h0 + 4);
        const int vk = (int)(h0 % 6), ck = (int)((h0 >> 8) % 7);
        double iso;
        float va, vb;
        if (vk == 0) {            // float data, double isolevel
            va = (float)unit(h1); vb = (float)unit(h2); iso = unit(h3);
        } else if (vk == 1) {     // int-like data, isolevel k + 0.5 or k
            va = (float)(h1 & 255); vb = (float)(h2 & 255); iso = (double)(h3 & 255) + ((h3 >> 8) & 1 ? 0.5 : 0.0);
        } else if (vk == 2) {     // close values
            va = (float)unit(h1); vb = __int_as_float(__float_as_int(va) + (int)(h2 & 15) - 7);
            iso = (double)va + ((double)vb - (double)va) * unit(h3);
        } else if (vk == 3) {     // ratio near 0, 1/2 or 1
            va = (float)(h1 & 1023); vb = va + 1.0f;
            const double t = ((h3 >> 60) & 3) == 0 ? 1e-9 * unit(h3) : (((h3 >> 60) & 3) == 1 ? 0.5 : 1.0 - 1e-9 * unit(h3));
            iso = (double)va + t;
        } else if (vk == 4) {     // isolevel exactly a value (r = 0)
            va = (float)unit(h1); vb = (float)unit(h2); iso = (double)va;
        } else {                  // wide range, negative values
            va = (float)((unit(h1) - 0.5) * 2e6); vb = (float)((unit(h2) - 0.5) * 2e6); iso = (unit(h3) - 0.5) * 2e6;
        }
        float c0, c1;
        const float u0 = (float)unit(h4), u1 = (float)unit(mix64(h4));
        if (ck == 0) {            // grid-like coordinates with jitter
            c0 = (float)((h4 >> 20) & 255) + u0 * 0.4f - 0.2f; c1 = c0 + 1.0f + u1 * 0.4f - 0.2f;
        } else if (ck == 1) {     // small magnitudes of both signs
            c0 = (u0 - 0.5f) * 1e-3f; c1 = (u1 - 0.5f) * 1e-3f;
        } else if (ck == 2) {     // large magnitudes
            c0 = (u0 - 0.5f) * 2e20f; c1 = (u1 - 0.5f) * 2e20f;
        } else if (ck == 3) {     // equal coordinates (d = 0), zeros included
            c0 = ((h4 >> 40) & 1) ? 0.0f : (u0 - 0.5f) * 100.0f; c1 = c0;
        } else if (ck == 4) {     // crossing zero
            c0 = -u0 * 10.0f; c1 = u1 * 10.0f;
        } else if (ck == 5) {     // near powers of two
            c0 = (float)(1u << ((h4 >> 20) & 15)); c1 = c0 - 1.0f + u1 * 2.0f;
        } else {                  // arbitrary float bit patterns of moderate exponent
            c0 = __int_as_float((int)(0x30000000u + (uint32_t)(h4 & 0x1fffffffu)));
            c1 = __int_as_float((int)(0x30000000u + (uint32_t)((h4 >> 29) & 0x1fffffffu)));
            if ((h4 >> 62) & 1) c0 = -c0;
        }
        const float f_iso = (float)iso;
        float thr = f_iso;
        if ((double)thr > iso) thr = nextafterf(thr, -INFINITY);
        if ((va > thr) == (vb > thr)) continue;
        FastIso f;
        f.ih = f_iso;
        f.il = (float)(iso - (double)f.ih);
        const double rep = iso - ((double)f.ih + (double)f.il);
        f.iso_err = (float)fabs(rep) * 1.0001f;
        f.f_thr = thr;
        f.vmin_f = -3.0e38f; f.vmax_f = 3.0e38f;
        f.fast_ok = 1; f.pad = 0;
        const double q = __ddiv_rn(__dsub_rn(iso, (double)va), __dsub_rn((double)vb, (double)va));
        const double r = q < 0.0 ? -q : q;
        const float want = __double2float_rn(__dadd_rn((double)c0, __dmul_rn(r, (double)__fsub_rn(c1, c0))));
        const CellRatio cr = cell_ratio(va, vb, f);
        float got;
        const bool ok = cell_axis(cr, c0, c1, got);
        ++tested;
        if (!ok) ++fall;
        else if (__float_as_int(got) != __float_as_int(want)) ++mism;
    }
    atomicAdd(&counters[0], tested);
    atomicAdd(&counters[1], mism);
    atomicAdd(&counters[2], fall);
}

}  // namespace

cudaError_t launch_selftest(uint64_t n, uint64_t seed, unsigned long long* d_counters, const Launch& L)
{
    k_selftest<<<L.num_sms * 8, 256, 0, L.stream>>>(n, seed, d_counters);
    *L.counter += 1;
    return cudaGetLastError();
}

cudaError_t launch_selftest_cells(uint64_t n, uint64_t seed, unsigned long long* d_counters, const Launch& L)
{
    k_selftest_cells<<<L.num_sms * 8, 256, 0, L.stream>>>(n, seed, d_counters);
    *L.counter += 1;
    return cudaGetLastError();
}

}  // namespace kvsmc
