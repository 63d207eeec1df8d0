// mc_interp.cuh -- exact edge interpolation without FP64 on the common path.
//
// The reference interpolates in FP64 and rounds to float
// (interpolate_vertex<T>, MarchingCubes.cpp:327-356):
//     r = |RN64(RN64(iso - v0) / RN64(v1 - v0))|,  X = RN64(RN64(RN64(1-r)*a) + RN64(r*b))
//     F = RN32(X)
// GB300 runs FP64 at 1/58 of the FP32 rate (measured: 0.63 T DFMA/s, 61 G DDIV/s),
// so the kernels compute F with FP32 "double-float" arithmetic (Knuth's
// TwoSum, Dekker's product via FMA, one Newton correction for the quotient:
// the classic error-free transformations) and a rigorous error bound E, and
// accept the FP32 answer only when no float rounding boundary lies within E
// of it.  Otherwise (about one vertex in 10^6) they run the exact FP64
// sequence.  Either way the float bits equal the reference's.
//
// Why it is exact (a, b = edge endpoint coordinates, integers < 2^24;
// v0, v1 = clamped endpoint values, exactly representable as float):
//  * The endpoints straddle the isolevel in the reference's double test, so
//    RN64(iso - v0) and RN64(v1 - v0) have equal signs and |num| <= |den|:
//    r lies in [0, 1].
//  * Constant axes (a == b == c): (1-r)*c + r*c evaluated in FP64 is within
//    3*2^-53 |c| of c, so RN32 gives c exactly.  No work is needed.
//  * Varying axis (b = a +- 1): with R = (iso - v0)/(v1 - v0) in exact
//    arithmetic, |X - (a + (b-a) R)| <= 2^-51 (max(|a|,|b|) + 1)   (E_D).
//    The double-float Y approximates a + (b-a) R within
//        E_Y = 2^-40 |q| + err(num)/|den| + 2^-23 |y_lo|
//    The quotient starts from the hardware reciprocal approximation
//    (rcp.approx, relative error below 2^-22 assumed, twice its documented
//    1 ulp), q1 = nh * inv, and takes one residual correction q2 = rho * inv
//    with rho = num - q1 * den formed from exact FMA products; then
//    |q1 + q2 - num/den| < 1.5 * 2^-43 |R|, below the 2^-40 |q| term with a
//    factor 5 of slack.  If every real in [Y - E, Y + E], E = E_Y + E_D,
//    rounds to the same float, that float is RN32(X) = F.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "mc_device.cuh"

namespace kvsmc {

// Per-request constants of the fast path (computed on the host).
struct FastIso {
    float ih, il;        // iso ~ ih + il
    float iso_err;       // upper bound of |iso - (ih + il)|
    float f_thr;         // largest float <= iso: v > f_thr <=> double(v) > iso
    float vmin_f, vmax_f;// the clamp range as floats (exact when fast_ok)
    int32_t fast_ok;     // 0: always take the FP64 sequence
    int32_t pad;
};

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ float clampf_ref(float a, float lo, float hi)
{
    return a <= lo ? lo : (a <= hi ? a : hi);
}

// Distance from x + e (x > 0 a normal float, |e| below half its gaps) to the
// nearer of x's two rounding boundaries: half the gap to the next float above
// less e, or half the gap to the next float below plus e.  Both sides count:
// at a power of two the gap below is half the gap above.
__device__ __forceinline__ float rounding_margin(float x, float e)
{
    const int ib = __float_as_int(x);
    const float hi = __fmul_rn(__fsub_rn(__int_as_float(ib + 1), x), 0.5f);
    const float lo = __fmul_rn(__fsub_rn(x, __int_as_float(ib - 1)), 0.5f);
    return fminf(__fsub_rn(hi, e), __fadd_rn(lo, e));
}

// The varying-axis coordinate RN32(X) for an edge from coordinate a (value
// v0) to b = a + d (value v1), d = +-1.  Returns false when the FP32 path
// cannot decide; `out` is then unspecified.
__device__ __forceinline__ bool fast_axis(float v0, float v1, float a, float b, const FastIso& f, float& out)
{
    // num = iso - v0 as a double-float (nh, nl); err_num bounds its error.
    float s, e;
    two_sum(f.ih, -v0, s, e);
    const float e2 = __fadd_rn(e, f.il);
    float nh, nl;
    two_sum(s, e2, nh, nl);
    if (nh == 0.0f && nl == 0.0f && f.iso_err == 0.0f) {
        // iso == v0 exactly: r = 0 and the reference returns a exactly
        out = a;
        return true;
    }
    const float err_num = __fadd_rn(f.iso_err, __fmul_rn(fabsf(e2), 1.1920929e-07f));  // + 2^-23 |e2|
    // den = v1 - v0 exactly as (dh, dl).
    float dh, dl;
    two_sum(v1, -v0, dh, dl);
    const float adh = fabsf(dh);
    if (!(adh >= 8.67361738e-19f) || !(adh <= 1.15292150e+18f)) return false;  // 2^-60 .. 2^60
    // q = num / den: q1 from the approximate reciprocal, then one residual correction.
    float inv;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(inv) : "f"(dh));
    const float q1 = __fmul_rn(nh, inv);
    const float p = __fmul_rn(q1, dh);
    const float pe = __fmaf_rn(q1, dh, -p);
    const float p2 = __fmul_rn(q1, dl);
    const float pe2 = __fmaf_rn(q1, dl, -p2);
    const float rho = __fsub_rn(__fadd_rn(__fsub_rn(__fsub_rn(nh, p), pe), __fsub_rn(nl, p2)), pe2);
    const float q2 = __fmul_rn(rho, inv);
    const float aq = fabsf(q1);
    if (!(aq <= 1.5f)) return false;
    // Y = a + d*(q1 + q2) as (yh, yl).
    const bool up = b > a;
    const float dq1 = up ? q1 : -q1, dq2 = up ? q2 : -q2;
    float ya, yb;
    two_sum(a, dq1, ya, yb);
    const float yb2 = __fadd_rn(yb, dq2);
    float yh, yl;
    two_sum(ya, yb2, yh, yl);
    // E = E_R + rounding of yb2 + E_D, each with slack.
    const float m = fmaxf(a, b);
    float E = __fmul_rn(aq, 9.09494702e-13f);                                   // 2^-40 |q|
    E = __fadd_rn(E, __fmul_rn(__fmul_rn(err_num, fabsf(inv)), 1.0001f));      // err(num)/|den| (inv within 2^-22)
    E = __fadd_rn(E, __fmul_rn(fabsf(yb2), 1.1920929e-07f));                    // 2^-23 |yb2|
    E = __fadd_rn(E, __fmul_rn(__fadd_rn(m, 1.0f), 8.8817842e-16f));            // 2^-50 (M + 1)
    E = __fmul_rn(E, 1.001f);
    if (!(yh > 0.0f) || !(yh < 3.0e7f)) {
        // Y at (or below) zero: exact only if the double-float is exactly 0
        if (yh == 0.0f && yl == 0.0f && E < 1.0e-30f) { out = 0.0f; return true; }
        return false;
    }
    const float dist = rounding_margin(yh, yl);
    if (!(dist > E)) return false;
    out = yh;
    return true;
}

// fast_axis without branches: every step is computed and the result is
// selected, so independent edges' arithmetic can interleave in one thread.
// Same accepted results as fast_axis (the cases it returns early on come out
// as selects; out is meaningless when the result is false).
__device__ __forceinline__ bool fast_axis_bf(float v0, float v1, float a, float b, const FastIso& f, float& out)
{
    float s, e;
    two_sum(f.ih, -v0, s, e);
    const float e2 = __fadd_rn(e, f.il);
    float nh, nl;
    two_sum(s, e2, nh, nl);
    const bool at_v0 = nh == 0.0f && nl == 0.0f && f.iso_err == 0.0f;   // iso == v0: r = 0, X = a
    const float err_num = __fadd_rn(f.iso_err, __fmul_rn(fabsf(e2), 1.1920929e-07f));
    float dh, dl;
    two_sum(v1, -v0, dh, dl);
    const float adh = fabsf(dh);
    const bool den_ok = adh >= 8.67361738e-19f && adh <= 1.15292150e+18f;   // 2^-60 .. 2^60
    float inv;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(inv) : "f"(dh));
    const float q1 = __fmul_rn(nh, inv);
    const float p = __fmul_rn(q1, dh);
    const float pe = __fmaf_rn(q1, dh, -p);
    const float p2 = __fmul_rn(q1, dl);
    const float pe2 = __fmaf_rn(q1, dl, -p2);
    const float rho = __fsub_rn(__fadd_rn(__fsub_rn(__fsub_rn(nh, p), pe), __fsub_rn(nl, p2)), pe2);
    const float q2 = __fmul_rn(rho, inv);
    const float aq = fabsf(q1);
    const bool up = b > a;
    const float dq1 = up ? q1 : -q1, dq2 = up ? q2 : -q2;
    // a + dq1 exactly as (ya, yb) by Dekker's Fast2Sum: a is an integer
    // coordinate (0, or at least 1 in magnitude) and |dq1| <= 1.5 on every
    // accepted result, so a == 0 or exponent(a) >= exponent(dq1)
    const float ya = __fadd_rn(a, dq1);
    const float yb = __fsub_rn(dq1, __fsub_rn(ya, a));
    const float yb2 = __fadd_rn(yb, dq2);
    float yh, yl;
    two_sum(ya, yb2, yh, yl);
    const float m = fmaxf(a, b);
    float E = __fmul_rn(aq, 9.09494702e-13f);
    E = __fadd_rn(E, __fmul_rn(__fmul_rn(err_num, fabsf(inv)), 1.0001f));
    E = __fadd_rn(E, __fmul_rn(fabsf(yb2), 1.1920929e-07f));
    E = __fadd_rn(E, __fmul_rn(__fadd_rn(m, 1.0f), 8.8817842e-16f));
    E = __fmul_rn(E, 1.001f);
    const float dist = rounding_margin(yh, yl);
    const bool pos_ok = yh > 0.0f && yh < 3.0e7f && dist > E;
    const bool zero_ok = yh == 0.0f && yl == 0.0f && E < 1.0e-30f;
    const bool ok = at_v0 || (den_ok && aq <= 1.5f && (pos_ok || zero_ok));
    out = at_v0 ? a : (zero_ok ? 0.0f : yh);
    return ok;
}

// The fast path of edge_vertex_axis without branches: the vertex, and
// whether it is certain (false: run edge_vertex_axis for this edge).
__device__ __forceinline__ bool edge_vertex_axis_try(const FastIso& f, const float* min_coord, const float* scale,
                                                     float va, float vb, float ax, float ay, float az, int axis,
                                                     float b, float3& o)
{
    const float a = axis == 0 ? ax : (axis == 1 ? ay : az);
    const float v0 = clampf_ref(va, f.vmin_f, f.vmax_f);
    const float v1 = clampf_ref(vb, f.vmin_f, f.vmax_f);
    float r;
    const bool ok = fast_axis_bf(v0, v1, a, b, f, r) && f.fast_ok != 0 && ((v0 > f.f_thr) != (v1 > f.f_thr));
    const float px = axis == 0 ? r : ax, py = axis == 1 ? r : ay, pz = axis == 2 ? r : az;
    o.x = __fmul_rn(__fadd_rn(px, min_coord[0]), scale[0]);
    o.y = __fmul_rn(__fadd_rn(py, min_coord[1]), scale[1]);
    o.z = __fmul_rn(__fadd_rn(pz, min_coord[2]), scale[2]);
    return ok;
}

// The FP64 sequence, kept out of line: it runs for about one vertex in 10^5
// and would otherwise hold FP64 registers in the hot loop.
static __device__ __noinline__ float3 interpolate_exact_slow(const Interp& j, float va, float vb, float ax, float ay,
                                                             float az, float bx, float by, float bz)
{
    return interpolate_exact(j, (double)va, (double)vb, ax, ay, az, bx, by, bz);
}

// Vertex of an edge from corner A = (ax, ay, az) (value va) to the corner one
// step along `axis` (0, 1, 2), whose coordinate there is `b` (a +- 1).  Same
// result as edge_vertex_fast; the callers pass integer coordinates as floats
// and the fast path's constants (f, min_coord, scale) from wherever they keep
// them.
__device__ __forceinline__ float3 edge_vertex_axis(const FastIso& f, const float* min_coord, const float* scale,
                                                   const Interp& j, float va, float vb, float ax, float ay, float az,
                                                   int axis, float b)
{
    bool ok = f.fast_ok != 0;
    float r = 0.0f;
    const float a = axis == 0 ? ax : (axis == 1 ? ay : az);
    if (ok) {
        const float v0 = clampf_ref(va, f.vmin_f, f.vmax_f);
        const float v1 = clampf_ref(vb, f.vmin_f, f.vmax_f);
        ok = (v0 > f.f_thr) != (v1 > f.f_thr);
        if (ok) ok = fast_axis(v0, v1, a, b, f, r);
    }
    if (ok) {
        const float px = axis == 0 ? r : ax, py = axis == 1 ? r : ay, pz = axis == 2 ? r : az;
        float3 o;
        o.x = __fmul_rn(__fadd_rn(px, min_coord[0]), scale[0]);
        o.y = __fmul_rn(__fadd_rn(py, min_coord[1]), scale[1]);
        o.z = __fmul_rn(__fadd_rn(pz, min_coord[2]), scale[2]);
        return o;
    }
    // j (the FP64 constants, same min_coord and scale) is read only here
    const float bx = axis == 0 ? b : ax, by = axis == 1 ? b : ay, bz = axis == 2 ? b : az;
    return interpolate_exact_slow(j, va, vb, ax, ay, az, bx, by, bz);
}

// Vertex of an edge whose endpoints differ along `axis` (0, 1, 2): A = (ax,
// ay, az) with value va, B with value vb (both raw values as float).  `j`
// carries the FP64 constants for the fallback.  Output after the
// (p + min_coord) * scale transform.
__device__ __forceinline__ float3 edge_vertex_fast(const Interp& j, const FastIso& f, float va, float vb,
                                                   float ax, float ay, float az, float bx, float by, float bz,
                                                   int axis)
{
    bool ok = f.fast_ok != 0;
    float r = 0.0f;
    if (ok) {
        const float v0 = clampf_ref(va, f.vmin_f, f.vmax_f);
        const float v1 = clampf_ref(vb, f.vmin_f, f.vmax_f);
        ok = (v0 > f.f_thr) != (v1 > f.f_thr);
        // one inlined copy of the varying-axis computation for all three axes
        // (lanes of a warp interpolate edges of different directions)
        const float a = axis == 0 ? ax : (axis == 1 ? ay : az);
        const float b = axis == 0 ? bx : (axis == 1 ? by : bz);
        if (ok) ok = fast_axis(v0, v1, a, b, f, r);
    }
    if (ok) {
        const float px = axis == 0 ? r : ax, py = axis == 1 ? r : ay, pz = axis == 2 ? r : az;
        float3 o;
        o.x = __fmul_rn(__fadd_rn(px, j.min_coord[0]), j.scale[0]);
        o.y = __fmul_rn(__fadd_rn(py, j.min_coord[1]), j.scale[1]);
        o.z = __fmul_rn(__fadd_rn(pz, j.min_coord[2]), j.scale[2]);
        return o;
    }
    return interpolate_exact_slow(j, va, vb, ax, ay, az, bx, by, bz);
}

// ------------------------------------------------------------------ cells
//
// The unstructured mappers' vertex (interpolate_vertex, e.g.
// MarchingTetrahedra.cpp:325-346) on arbitrary float endpoints c0, c1:
//     r = |RN64(RN64(iso - v0) / RN64(v1 - v0))|,  d = RN32(c1 - c0)
//     X = RN64(c0 + RN64(r * d)),  F = RN32(X)
// With R = (iso - v0) / (v1 - v0) exactly and |R| <= 1.5:
//     |X - (c0 + d |R|)| <= 2^-53 (|c0| + 8 |d|) <= 2^-50 (|c0| + |d|)   (E_D)
// (three roundings in r, one in r d, one in the sum).  The FP32 path forms
// r = q1 + q2 as fast_axis does (|r - |R|| <= EQ = 2^-40 |q1| + err_num/|den|),
// d r1 exactly by FMA, d r2 and two additions rounded (2^-23 of each), and
// Y = yh + yl by TwoSum: |Y - (c0 + d |R|)| <= |d| EQ + 2^-23 (|p2| + |t1| + |t|).
// If no float rounding boundary lies within E = (E_Y + E_D) 1.001 of Y, F = yh.

// The ratio part shared by the three axes of one vertex.
struct CellRatio {
    float r1, r2;   // |R| ~ r1 + r2
    float eq;       // bound of |r1 + r2 - |R||
    int ok;         // the FP32 path may be used (denominator in range, |R| <= 1.5)
    int zero;       // iso == v0 exactly: R = 0
};

__device__ __forceinline__ CellRatio cell_ratio(float v0, float v1, const FastIso& f)
{
    CellRatio c;
    float s, e;
    two_sum(f.ih, -v0, s, e);
    const float e2 = __fadd_rn(e, f.il);
    float nh, nl;
    two_sum(s, e2, nh, nl);
    const float err_num = __fadd_rn(f.iso_err, __fmul_rn(fabsf(e2), 1.1920929e-07f));
    float dh, dl;
    two_sum(v1, -v0, dh, dl);
    const float adh = fabsf(dh);
    const bool den_ok = adh >= 8.67361738e-19f && adh <= 1.15292150e+18f;   // 2^-60 .. 2^60
    float inv;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(inv) : "f"(dh));
    const float q1 = __fmul_rn(nh, inv);
    const float p = __fmul_rn(q1, dh);
    const float pe = __fmaf_rn(q1, dh, -p);
    const float p2 = __fmul_rn(q1, dl);
    const float pe2 = __fmaf_rn(q1, dl, -p2);
    const float rho = __fsub_rn(__fadd_rn(__fsub_rn(__fsub_rn(nh, p), pe), __fsub_rn(nl, p2)), pe2);
    const float q2 = __fmul_rn(rho, inv);
    const float aq = fabsf(q1);
    const bool neg = q1 < 0.0f;
    c.r1 = neg ? -q1 : q1;
    c.r2 = neg ? -q2 : q2;
    c.eq = __fmul_rn(__fadd_rn(__fmul_rn(aq, 9.09494702e-13f), __fmul_rn(__fmul_rn(err_num, fabsf(inv)), 1.0001f)),
                     1.001f);
    c.zero = nh == 0.0f && nl == 0.0f && f.iso_err == 0.0f;
    c.ok = f.fast_ok && den_ok && aq <= 1.5f;
    return c;
}

// F for one axis, or false when the FP32 path cannot decide.
__device__ __forceinline__ bool cell_axis(const CellRatio& c, float c0, float c1, float& out)
{
    const float d = __fsub_rn(c1, c0);
    const float ad = fabsf(d), ac = fabsf(c0);
    const bool in_range = ad <= 1.26765060e+30f && ac <= 1.26765060e+30f;   // 2^100
    const bool pos_zero = __float_as_uint(c0) == 0u;   // c0 = +0: +0 + (+-0) = +0
    if (c.zero) {
        // r = +-0: X = c0 + (+-0) = c0, except for c0 = -0
        out = c0;
        return c.ok && in_range && (c0 != 0.0f || pos_zero);
    }
    if (d == 0.0f && pos_zero) {
        // r finite: r d = +-0 and X = +0
        out = 0.0f;
        return c.ok && in_range;
    }
    const float p1 = __fmul_rn(d, c.r1);
    const float pe1 = __fmaf_rn(d, c.r1, -p1);
    const float p2 = __fmul_rn(d, c.r2);
    float s, e;
    two_sum(c0, p1, s, e);
    const float t1 = __fadd_rn(e, pe1);
    const float t = __fadd_rn(t1, p2);
    float yh, yl;
    two_sum(s, t, yh, yl);
    float E = __fmul_rn(ad, c.eq);
    E = __fadd_rn(E, __fmul_rn(__fadd_rn(__fadd_rn(fabsf(p2), fabsf(t1)), fabsf(t)), 1.1920929e-07f));  // 2^-23
    E = __fadd_rn(E, __fmul_rn(__fadd_rn(ac, ad), 8.8817842e-16f));                                       // 2^-50
    E = __fmul_rn(E, 1.001f);
    const float ay = fabsf(yh);
    const bool y_ok = ay >= 7.88860905e-31f && ay <= 1.26765060e+30f;   // 2^-100 .. 2^100
    const float dist = yh > 0.0f ? rounding_margin(yh, yl) : rounding_margin(-yh, -yl);
    out = yh;
    return c.ok && in_range && y_ok && dist > E;
}

}  // namespace kvsmc
